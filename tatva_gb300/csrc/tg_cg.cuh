// CG building blocks shared by the vector kernels (linalg.cu) and the fused grid
// iteration (grid.cu): device-scalar slots, compensated FP32 dot accumulation, the
// fixed-order CTA reduction and the last-arriving-CTA pattern.
#pragma once

#include "tg_common.cuh"

namespace tg {

constexpr int DOT_CHUNKS = 2048;
constexpr int DOT_THREADS = 256;
// SCAL_TOL2: the squared residual tolerance of the running CG; SCAL_DONE: set by the
// update when |r|^2 <= SCAL_TOL2 (the iteration's launches then return at once, so a
// captured block of iterations stops doing work when the solve has converged inside
// it); SCAL_ITERS: iterations performed.  Slots 5 and 7: true-residual norms.
constexpr int SCAL_RZ = 0, SCAL_PQ = 1, SCAL_ALPHA = 2, SCAL_BETA = 3, SCAL_RR = 4,
              SCAL_FLAG = 6, SCAL_TOL2 = 8, SCAL_DONE = 9, SCAL_ITERS = 10, SCAL_N = 12;

// ------------------------------------------------------------------ dot accumulators
// FP32 vectors: each thread accumulates x_i y_i as an unevaluated pair (hi, lo) of
// floats -- the product is split exactly with an FMA and added with a two-sum, so the
// thread's partial keeps about 48 bits -- and only the per-thread partials enter the
// FP64 tree reduction.  (This GPU's FP64 rate is a small fraction of FP32: per-element
// FP64 conversions and multiply-adds made the dots several times slower than their
// memory traffic.)  FP64 vectors accumulate in FP64.
template <class T>
struct DotAcc;
template <>
struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float a, float b) {
    const float pr = a * b;
    const float pe = fmaf(a, b, -pr);
    const float s = hi + pr;
    const float bp = s - hi;
    const float err = (hi - (s - bp)) + (pr - bp);
    hi = s;
    lo += err + pe;
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};
template <>
struct DotAcc<double> {
  double v = 0.0;
  __device__ __forceinline__ void add(double a, double b) { v += a * b; }
  __device__ __forceinline__ double value() const { return v; }
};

// ------------------------------------------------------------------ reductions
// Sum of one value per thread of the CTA into out[k] (thread 0 writes): a fixed tree
// (shuffles inside each warp, then the warps' sums in warp order), so the result does
// not depend on timing.  Ends with a barrier: the CTA may call it again.
template <int K, int NT = DOT_THREADS>
__device__ __forceinline__ void block_reduce_store(double (&v)[K], double* __restrict__ out) {
  constexpr int NW = NT / 32;
  __shared__ double sh[K][NW];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0) sh[k][warp] = v[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double a = sh[k][0];
#pragma unroll
      for (int w = 1; w < NW; ++w) a += sh[k][w];
      out[k] = a;
    }
  }
  __syncthreads();
}

// Called by every thread after thread 0 stored this CTA's partials: true in the CTA
// that arrives last, which then sees every CTA's partials (read them with __ldcg).
// That CTA resets the ticket for the next launch.  An arrival counter, no waiting.
// Only thread 0's partial has to be visible before its arrival, so only thread 0
// fences: a fence in every thread waited for all of the CTA's output stores.
__device__ __forceinline__ bool last_cta(unsigned* ticket) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
    if (last) *ticket = 0u;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

}  // namespace tg
