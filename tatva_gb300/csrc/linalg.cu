// Sparse and vector kernels (K7, K8) and the device-resident solvers built on them.
//
// The reference has no solver: users compose jax.scipy.sparse.linalg.cg with the
// matrix-free HVP (README.md:93).  Here:
//   * CSR SpMV (layout of ColoredMatrix.to_csr, tatva/sparse/base.py:76-81)
//   * deterministic FP64 dot products: a fixed partition (one chunk per 2048 entries,
//     at most DOT_CHUNKS chunks) and a fixed tree order, independent of the GPU and of
//     the launch, so repeated solves are bitwise identical
//   * Jacobi-preconditioned CG whose scalars never leave the device; `check_every`
//     iterations are captured once in a CUDA graph and replayed between host
//     convergence checks; every loop is bounded by max_iter
//   * mixed precision: FP32 CG inner solves (FP32 HVP, FP64 dots), FP64 iterative
//     refinement on the true residual b - A64 x.
#include <cmath>
#include <vector>

#include "tg_cg.cuh"
#include "tg_common.cuh"
#include "tg_dispatch.cuh"
#include "tg_internal.h"

namespace tg {

// Chunk count of the fixed partition of an n-vector: one chunk per 8192 entries, at
// most DOT_CHUNKS (about five CTAs per SM for the largest vectors here, one wave; the
// count depends on n only).
__host__ __device__ inline int dot_chunks(int64_t n) {
  const int64_t c = (n + 8191) / 8192;
  return (int)(c < 1 ? 1 : (c > DOT_CHUNKS ? DOT_CHUNKS : c));
}

// fixed partition into gridDim.x (= dot_chunks(n)) chunks whose starts are multiples
// of 4 elements
__device__ __forceinline__ void chunk_range(int64_t n, int64_t& i0, int64_t& i1) {
  const int64_t nc = gridDim.x;
  const int64_t chunk = (((n + nc - 1) / nc) + 3) & ~int64_t(3);
  i0 = min(n, (int64_t)blockIdx.x * chunk);
  i1 = min(n, i0 + chunk);
}

// 16-byte vector access of 4 consecutive values (4-aligned index, 16-byte aligned base)
__device__ __forceinline__ void ldv(const float* p, float (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ldv(const double* p, double (&v)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0];
  const double2 b = reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void stv(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void stv(double* p, const double (&v)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}

template <class T>
__global__ void __launch_bounds__(DOT_THREADS)
    dot_partial_kernel(const T* __restrict__ x, const T* __restrict__ y, int64_t n,
                       double* __restrict__ part) {
  int64_t i0, i1;
  chunk_range(n, i0, i1);
  const int64_t iv = i0 + ((i1 - i0) & ~int64_t(3));
  DotAcc<T> acc;
#pragma unroll 4
  for (int64_t i = i0 + 4 * threadIdx.x; i < iv; i += 4 * DOT_THREADS) {
    T a[4], b[4];
    ldv(x + i, a);
    ldv(y + i, b);
#pragma unroll
    for (int k = 0; k < 4; ++k) acc.add(a[k], b[k]);
  }
  for (int64_t i = iv + threadIdx.x; i < i1; i += DOT_THREADS) acc.add(x[i], y[i]);
  double v[1] = {acc.value()};
  block_reduce_store<1>(v, part + blockIdx.x);
}

// sums nchunks partials (stride K) into out[k]
template <int K>
__global__ void __launch_bounds__(DOT_THREADS)
    dot_final_kernel(const double* __restrict__ part, double* __restrict__ out, int nchunks) {
  double v[K];
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = 0.0;
  for (int b = threadIdx.x; b < nchunks; b += DOT_THREADS)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] += part[b * K + k];
  block_reduce_store<K>(v, out);
}

// ------------------------------------------------------------------ vector kernels
template <class T>
__global__ void axpby_kernel(int64_t n, double a, const T* __restrict__ x, double b,
                             T* __restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = (T)(a * (double)x[i] + b * (double)y[i]);
}

template <class Ti, class To>
__global__ void convert_kernel(const Ti* __restrict__ in, To* __restrict__ out, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (To)in[i];
}

// ------------------------------------------------------------------ CSR
// SPMV_LANES lanes per row (4 rows per warp): the finite-element rows here hold 7 to
// 81 entries, for which a whole warp per row leaves most lanes idle.  Fixed lane
// count and reduction tree: the result does not depend on the launch.
constexpr int SPMV_LANES = 8;
template <class T>
__global__ void spmv_kernel(int64_t n_rows, const int32_t* __restrict__ indptr,
                            const int32_t* __restrict__ indices, const T* __restrict__ data,
                            const T* __restrict__ x, T* __restrict__ y) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / SPMV_LANES;
  const int lane = threadIdx.x & (SPMV_LANES - 1);
  const bool live = row < n_rows;
  T acc = T(0);
  if (live) {
    const int k0 = __ldg(indptr + row), k1 = __ldg(indptr + row + 1);
    int k = k0 + lane;
    for (; k + SPMV_LANES < k1; k += 2 * SPMV_LANES) {
      const T a0 = __ldg(data + k), a1 = __ldg(data + k + SPMV_LANES);
      const T x0 = x[__ldg(indices + k)], x1 = x[__ldg(indices + k + SPMV_LANES)];
      acc += a0 * x0;
      acc += a1 * x1;
    }
    if (k < k1) acc += __ldg(data + k) * x[__ldg(indices + k)];
  }
#pragma unroll
  for (int o = SPMV_LANES / 2; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o, SPMV_LANES);
  if (live && lane == 0) y[row] = acc;
}

// node blocks of a 3-dof-per-node CSR pattern: one thread per node (the last thread
// writes node_ptr[n_nodes]); any row triple not of the blocked form raises the flag
__global__ void node_blocks3_kernel(int64_t n_nodes, const int32_t* __restrict__ indptr,
                                    const int32_t* __restrict__ indices,
                                    int32_t* __restrict__ nptr, int32_t* __restrict__ nidx,
                                    int32_t* __restrict__ not_blocked) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i > n_nodes) return;
  const int32_t r0 = indptr[3 * i];
  if (r0 % 9 != 0) {
    *not_blocked = 1;
    return;
  }
  nptr[i] = r0 / 9;
  if (i == n_nodes) return;
  const int32_t L = indptr[3 * i + 1] - r0;
  bool good = (L % 3 == 0) && (indptr[3 * i + 2] - indptr[3 * i + 1] == L) &&
              (indptr[3 * i + 3] - indptr[3 * i + 2] == L);
  for (int32_t m = 0; good && m < L / 3; ++m) {
    const int32_t j3 = indices[r0 + 3 * m];
    good = (j3 % 3 == 0);
    for (int a = 0; good && a < 3; ++a)
      for (int b = 0; b < 3; ++b) good = good && indices[r0 + a * L + 3 * m + b] == j3 + b;
    if (good) nidx[r0 / 9 + m] = j3 / 3;
  }
  if (!good) *not_blocked = 1;
}

// y = A x over node blocks: SPMV3_LANES lanes per node, each lane a strided subset of
// the node's neighbour blocks, the three row sums reduced over the lanes in a fixed tree.
// Eight lanes: on the Kuhn tangent (15 blocks per node) sixteen lanes, one block each,
// measured 9 % slower (129.5 against 119.1 us at 121 M nonzeros).
constexpr int SPMV3_LANES = 8;
template <class T>
__global__ void spmv_blocks3_kernel(int64_t n_nodes, const int32_t* __restrict__ indptr,
                                    const int32_t* __restrict__ nptr,
                                    const int32_t* __restrict__ nidx, const T* __restrict__ data,
                                    const T* __restrict__ x, T* __restrict__ y) {
  const int64_t node = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / SPMV3_LANES;
  const int lane = threadIdx.x & (SPMV3_LANES - 1);
  const bool live = node < n_nodes;
  T s0 = T(0), s1 = T(0), s2 = T(0);
  if (live) {
    const int32_t b0 = __ldg(nptr + node), deg = __ldg(nptr + node + 1) - b0;
    const int64_t r0 = __ldg(indptr + 3 * node);
    const int64_t L = 3 * (int64_t)deg;
    for (int32_t m = lane; m < deg; m += SPMV3_LANES) {
      const int64_t j = __ldg(nidx + b0 + m);
      const T x0 = x[3 * j], x1 = x[3 * j + 1], x2 = x[3 * j + 2];
      const T* v = data + r0 + 3 * m;
      s0 += __ldg(v) * x0 + __ldg(v + 1) * x1 + __ldg(v + 2) * x2;
      s1 += __ldg(v + L) * x0 + __ldg(v + L + 1) * x1 + __ldg(v + L + 2) * x2;
      s2 += __ldg(v + 2 * L) * x0 + __ldg(v + 2 * L + 1) * x1 + __ldg(v + 2 * L + 2) * x2;
    }
  }
#pragma unroll
  for (int o = SPMV3_LANES / 2; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o, SPMV3_LANES);
    s1 += __shfl_down_sync(0xffffffffu, s1, o, SPMV3_LANES);
    s2 += __shfl_down_sync(0xffffffffu, s2, o, SPMV3_LANES);
  }
  if (live && lane == 0) {
    y[3 * node] = s0;
    y[3 * node + 1] = s1;
    y[3 * node + 2] = s2;
  }
}

template <class T>
__global__ void csr_diag_kernel(int64_t n_rows, const int32_t* __restrict__ indptr,
                                const int32_t* __restrict__ indices, const T* __restrict__ data,
                                T* __restrict__ diag) {
  const int64_t row = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= n_rows) return;
  T d = T(0);
  for (int k = indptr[row]; k < indptr[row + 1]; ++k)
    if (indices[k] == row) d = data[k];
  diag[row] = d;
}

template <class T>
__global__ void csr_dirichlet_kernel(int64_t n_rows, const int32_t* __restrict__ indptr,
                                     const int32_t* __restrict__ indices,
                                     const uint8_t* __restrict__ fixed, T* __restrict__ data) {
  const int64_t row = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (row >= n_rows) return;
  const bool rf = fixed[row] != 0;
  for (int k = indptr[row] + lane; k < indptr[row + 1]; k += 32) {
    const int c = indices[k];
    if (rf) data[k] = (c == row) ? T(1) : T(0);
    else if (fixed[c]) data[k] = T(0);
  }
}

// ------------------------------------------------------------------ CG kernels
// dinv = 1 / diag (once per restart: the iterations multiply)
template <class T>
__global__ void inv_kernel(int64_t n, const T* __restrict__ diag, T* __restrict__ dinv) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dinv[i] = T(1) / diag[i];
}

// p = z = r dinv, partials of (r.z, r.r)
template <class T>
__global__ void __launch_bounds__(DOT_THREADS)
    cg_init_kernel(int64_t n, const T* __restrict__ r, const T* __restrict__ dinv,
                   T* __restrict__ p, double* __restrict__ part) {
  int64_t i0, i1;
  chunk_range(n, i0, i1);
  const int64_t iv = i0 + ((i1 - i0) & ~int64_t(3));
  DotAcc<T> a0, a1;
  for (int64_t i = i0 + 4 * threadIdx.x; i < iv; i += 4 * DOT_THREADS) {
    T rr[4], dd[4], zz[4];
    ldv(r + i, rr);
    ldv(dinv + i, dd);
#pragma unroll
    for (int k = 0; k < 4; ++k) zz[k] = rr[k] * dd[k];
#pragma unroll
    for (int k = 0; k < 4; ++k) a0.add(rr[k], zz[k]);
#pragma unroll
    for (int k = 0; k < 4; ++k) a1.add(rr[k], rr[k]);
    stv(p + i, zz);
  }
  for (int64_t i = iv + threadIdx.x; i < i1; i += DOT_THREADS) {
    const T ri = r[i];
    const T zi = ri * dinv[i];
    p[i] = zi;
    a0.add(ri, zi);
    a1.add(ri, ri);
  }
  double v[2] = {a0.value(), a1.value()};
  block_reduce_store<2>(v, part + 2 * blockIdx.x);
}

// scal[RZ] = rz, scal[RR] = rr from the two-slot partials
__global__ void cg_init_final_kernel(const double* __restrict__ part, double* __restrict__ scal,
                                     int nchunks) {
  double v[2] = {0.0, 0.0};
  for (int b = threadIdx.x; b < nchunks; b += DOT_THREADS) {
    v[0] += part[2 * b];
    v[1] += part[2 * b + 1];
  }
  __shared__ double out[2];
  block_reduce_store<2>(v, out);
  __syncthreads();
  if (threadIdx.x == 0) {
    scal[SCAL_RZ] = out[0];
    scal[SCAL_RR] = out[1];
    scal[SCAL_FLAG] = 0.0;
    scal[SCAL_DONE] = 0.0;
    scal[SCAL_ITERS] = 0.0;
  }
}

// partials of p.q; the last CTA adds them (fixed order) and sets
// alpha = rz / pq (breakdown flag on pq <= 0 or non-finite)
template <class T>
__global__ void __launch_bounds__(DOT_THREADS)
    cg_pq_kernel(const T* __restrict__ p, const T* __restrict__ q, int64_t n,
                 double* __restrict__ part, double* __restrict__ scal, unsigned* ticket) {
  if (scal[SCAL_DONE] != 0.0) return;
  int64_t i0, i1;
  chunk_range(n, i0, i1);
  const int64_t iv = i0 + ((i1 - i0) & ~int64_t(3));
  DotAcc<T> acc;
#pragma unroll 4
  for (int64_t i = i0 + 4 * threadIdx.x; i < iv; i += 4 * DOT_THREADS) {
    T a[4], b[4];
    ldv(p + i, a);
    ldv(q + i, b);
#pragma unroll
    for (int k = 0; k < 4; ++k) acc.add(a[k], b[k]);
  }
  for (int64_t i = iv + threadIdx.x; i < i1; i += DOT_THREADS) acc.add(p[i], q[i]);
  double v[1] = {acc.value()};
  block_reduce_store<1>(v, part + blockIdx.x);
  if (!last_cta(ticket)) return;
  double w[1] = {0.0};
  for (int b = threadIdx.x; b < (int)gridDim.x; b += DOT_THREADS) w[0] += __ldcg(part + b);
  __shared__ double out[1];
  block_reduce_store<1>(w, out);
  if (threadIdx.x == 0) {
    const double pq = out[0];
    scal[SCAL_PQ] = pq;
    const bool bad = !(pq > 0.0) || !isfinite(pq) || scal[SCAL_FLAG] != 0.0;
    if (bad) scal[SCAL_FLAG] = 1.0;
    scal[SCAL_ALPHA] = bad ? 0.0 : scal[SCAL_RZ] / pq;
  }
}

// x += alpha p; r -= alpha q; partials of (r.z, r.r) with z = r dinv; the last CTA
// adds them (fixed order) and sets beta = rz_new / rz, rz = rz_new, rr
template <class T>
__global__ void __launch_bounds__(DOT_THREADS)
    cg_update_kernel(int64_t n, double* __restrict__ scal, T* __restrict__ x,
                     T* __restrict__ r, const T* __restrict__ p, const T* __restrict__ q,
                     const T* __restrict__ dinv, double* __restrict__ part, unsigned* ticket) {
  if (scal[SCAL_DONE] != 0.0) return;
  int64_t i0, i1;
  chunk_range(n, i0, i1);
  const int64_t iv = i0 + ((i1 - i0) & ~int64_t(3));
  const T alpha = (T)scal[SCAL_ALPHA];
  DotAcc<T> a0, a1;
#pragma unroll 2
  for (int64_t i = i0 + 4 * threadIdx.x; i < iv; i += 4 * DOT_THREADS) {
    T xx[4], pp[4], rr[4], qq[4], dd[4], zz[4];
    ldv(x + i, xx);
    ldv(p + i, pp);
    ldv(r + i, rr);
    ldv(q + i, qq);
    ldv(dinv + i, dd);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      xx[k] += alpha * pp[k];
      rr[k] = rr[k] - alpha * qq[k];
      zz[k] = rr[k] * dd[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) a0.add(rr[k], zz[k]);
#pragma unroll
    for (int k = 0; k < 4; ++k) a1.add(rr[k], rr[k]);
    stv(x + i, xx);
    stv(r + i, rr);
  }
  for (int64_t i = iv + threadIdx.x; i < i1; i += DOT_THREADS) {
    x[i] += alpha * p[i];
    const T ri = r[i] - alpha * q[i];
    r[i] = ri;
    a0.add(ri, ri * dinv[i]);
    a1.add(ri, ri);
  }
  double v[2] = {a0.value(), a1.value()};
  block_reduce_store<2>(v, part + 2 * blockIdx.x);
  if (!last_cta(ticket)) return;
  double w[2] = {0.0, 0.0};
  for (int b = threadIdx.x; b < (int)gridDim.x; b += DOT_THREADS) {
    w[0] += __ldcg(part + 2 * b);
    w[1] += __ldcg(part + 2 * b + 1);
  }
  __shared__ double out[2];
  block_reduce_store<2>(w, out);
  if (threadIdx.x == 0) {
    const double rz_new = out[0];
    const bool bad = scal[SCAL_FLAG] != 0.0 || !isfinite(rz_new);
    if (bad) scal[SCAL_FLAG] = 1.0;
    scal[SCAL_BETA] = bad ? 0.0 : rz_new / scal[SCAL_RZ];
    if (!bad) scal[SCAL_RZ] = rz_new;
    scal[SCAL_RR] = out[1];
    scal[SCAL_ITERS] += 1.0;
    if (out[1] <= scal[SCAL_TOL2]) scal[SCAL_DONE] = 1.0;
  }
}

// p = r dinv + beta p
template <class T>
__global__ void cg_p_kernel(int64_t n, const double* __restrict__ scal, const T* __restrict__ r,
                            const T* __restrict__ dinv, T* __restrict__ p) {
  if (scal[SCAL_DONE] != 0.0) return;
  const int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
  const T beta = (T)scal[SCAL_BETA];
  if (i + 3 < n) {
    T rr[4], dd[4], pp[4];
    ldv(r + i, rr);
    ldv(dinv + i, dd);
    ldv(p + i, pp);
#pragma unroll
    for (int k = 0; k < 4; ++k) pp[k] = rr[k] * dd[k] + beta * pp[k];
    stv(p + i, pp);
  } else {
    for (int64_t j = i; j < n; ++j) p[j] = r[j] * dinv[j] + beta * p[j];
  }
}

// Reliable update of the inner recursion (the mixed solver, when the direction is
// kept): r holds the new residual in the new unit, p the last direction in the old
// unit, scale = |r_old| / |r_new| takes it over.  The direction is made orthogonal to
// the new residual again (the recursive residual it was conjugated against has been
// replaced) and extended as in a CG step:
//   p <- dinv r + beta (scale p - c r),  c = scale (p.r) / (r.r),
//   beta = (r.dinv r) / (rz_k scale^2),
// rz_k being the r.z that the last direction was built from (rz / beta, as the update
// kernel that stopped the recursion left them).  Pass 1: partials of p.r and r.r
// (part2, two per chunk) and of r.dinv r (part1).
template <class T>
__global__ void __launch_bounds__(DOT_THREADS)
    cg_resume_partial_kernel(int64_t n, const T* __restrict__ r, const T* __restrict__ dinv,
                             const T* __restrict__ p, double* __restrict__ part2,
                             double* __restrict__ part1) {
  int64_t i0, i1;
  chunk_range(n, i0, i1);
  DotAcc<T> apr, arr, arz;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += DOT_THREADS) {
    const T ri = r[i];
    apr.add(p[i], ri);
    arr.add(ri, ri);
    arz.add(ri, ri * dinv[i]);
  }
  double v[3] = {apr.value(), arr.value(), arz.value()};
  __shared__ double out[3];
  block_reduce_store<3>(v, out);
  __syncthreads();
  if (threadIdx.x == 0) {
    part2[2 * blockIdx.x] = out[0];
    part2[2 * blockIdx.x + 1] = out[1];
    part1[blockIdx.x] = out[2];
  }
}

// the chunk partials added in a fixed order; coef = {beta scale, -beta c}.  A direction
// that cannot be continued (no usable rz_k, a zero or non-finite product) gives beta =
// 0, i.e. p = dinv r, the restart of the recursion.
__global__ void cg_resume_final_kernel(const double* __restrict__ part2,
                                       const double* __restrict__ part1, int nchunks,
                                       double scale, double* __restrict__ scal,
                                       double* __restrict__ coef) {
  double w[3] = {0.0, 0.0, 0.0};
  for (int b = threadIdx.x; b < nchunks; b += DOT_THREADS) {
    w[0] += part2[2 * b];
    w[1] += part2[2 * b + 1];
    w[2] += part1[b];
  }
  __shared__ double out[3];
  block_reduce_store<3>(w, out);
  __syncthreads();
  if (threadIdx.x == 0) {
    const double pr = out[0], rr = out[1], rz = out[2];
    const double beta_k = scal[SCAL_BETA];
    const double rz_k = beta_k > 0.0 ? scal[SCAL_RZ] / beta_k : 0.0;
    const bool ok = rz_k > 0.0 && isfinite(rz_k) && rr > 0.0 && rz > 0.0 && isfinite(pr) &&
                    isfinite(rz) && scale > 0.0 && isfinite(scale);
    const double beta = ok ? rz / (rz_k * scale * scale) : 0.0;
    const double c = ok ? scale * pr / rr : 0.0;
    coef[0] = beta * scale;
    coef[1] = -beta * c;
    scal[SCAL_RZ] = rz;
    scal[SCAL_RR] = rr;
    scal[SCAL_FLAG] = 0.0;
    scal[SCAL_DONE] = 0.0;
    scal[SCAL_ITERS] = 0.0;
  }
}

template <class T>
__global__ void cg_resume_p_kernel(int64_t n, const double* __restrict__ coef,
                                   const T* __restrict__ r, const T* __restrict__ dinv,
                                   T* __restrict__ p) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const T a = (T)coef[0], c = (T)coef[1];
  const T ri = r[i];
  p[i] = ri * dinv[i] + a * p[i] + c * ri;
}

// out = (T)(r64 / |r64|) and x += |r64| d, the scale and its reciprocal passed in
// (an FP64 square root or division per element costs more than the memory traffic on
// this GPU's FP64 pipe)
template <class T>
__global__ void scale_down_kernel(int64_t n, const double* __restrict__ r64, double inv_s,
                                  T* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = (T)(r64[i] * inv_s);
}
template <class T>
__global__ void scale_up_add_kernel(int64_t n, const T* __restrict__ d, double s,
                                    double* __restrict__ x) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] += s * (double)d[i];
}

// ------------------------------------------------------------------ operator description
inline int op_values(const tg_operator_desc* op) {
  const int D = (op->elem == TG_TRI3) ? 2 : 3;
  if (op->mat.kind == TG_LINEAR_ELASTIC) return D;
  if (op->mat.kind == TG_NEO_HOOKEAN) return 3;
  return 1;
}
inline int64_t op_ndofs(const tg_operator_desc* op) {
  return op->csr_data ? op->n_rows : op->n_nodes * op_values(op);
}
inline size_t prec_size(int prec) { return prec == TG_F32 ? 4 : 8; }
inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

struct Carve {
  char* base;
  size_t off = 0;
  void* take(size_t bytes) {
    void* p = base + off;
    off += align256(bytes);
    return p;
  }
};

}  // namespace tg

using namespace tg;

// ============================================================================ C ABI
extern "C" int tg_spmv(int prec, int64_t n_rows, const int32_t* indptr, const int32_t* indices,
                       const void* data, const void* x, void* y, void* stream) {
  if (n_rows < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n_rows == 0) return TG_OK;
  TG_TRY(check_ptr(indptr, "indptr"));
  TG_TRY(check_ptr(indices, "indices"));
  TG_TRY(check_ptr(data, "data"));
  TG_TRY(check_ptr(x, "x"));
  TG_TRY(check_ptr(y, "y"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    spmv_kernel<T><<<grid_for(n_rows * SPMV_LANES, 256), 256, 0, as_stream(stream)>>>(
        n_rows, indptr, indices, (const T*)data, (const T*)x, (T*)y);
    return launch_check("tg_spmv");
  });
}

extern "C" int tg_csr_node_blocks3(int64_t n_rows, const int32_t* indptr, const int32_t* indices,
                                   int32_t* node_ptr, int32_t* node_indices, int32_t* not_blocked,
                                   void* stream) {
  if (n_rows < 0 || n_rows % 3 != 0) return set_error(TG_ERR_VALUE, "n_rows must be a multiple of 3");
  TG_TRY(check_ptr(indptr, "indptr"));
  TG_TRY(check_ptr(node_ptr, "node_ptr"));
  TG_TRY(check_ptr(not_blocked, "not_blocked"));
  const int64_t nn = n_rows / 3;
  node_blocks3_kernel<<<grid_for(nn + 1, 256), 256, 0, as_stream(stream)>>>(
      nn, indptr, indices, node_ptr, node_indices, not_blocked);
  return launch_check("tg_csr_node_blocks3");
}

extern "C" int tg_spmv_blocks3(int prec, int64_t n_rows, const int32_t* indptr,
                               const int32_t* node_ptr, const int32_t* node_indices,
                               const void* data, const void* x, void* y, void* stream) {
  if (n_rows < 0 || n_rows % 3 != 0) return set_error(TG_ERR_VALUE, "n_rows must be a multiple of 3");
  if (n_rows == 0) return TG_OK;
  TG_TRY(check_ptr(indptr, "indptr"));
  TG_TRY(check_ptr(node_ptr, "node_ptr"));
  TG_TRY(check_ptr(node_indices, "node_indices"));
  TG_TRY(check_ptr(data, "data"));
  TG_TRY(check_ptr(x, "x"));
  TG_TRY(check_ptr(y, "y"));
  const int64_t nn = n_rows / 3;
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    spmv_blocks3_kernel<T><<<grid_for(nn * SPMV3_LANES, 256), 256, 0, as_stream(stream)>>>(
        nn, indptr, node_ptr, node_indices, (const T*)data, (const T*)x, (T*)y);
    return launch_check("tg_spmv_blocks3");
  });
}

extern "C" int tg_csr_diagonal(int prec, int64_t n_rows, const int32_t* indptr,
                               const int32_t* indices, const void* data, void* diag,
                               void* stream) {
  if (n_rows < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n_rows == 0) return TG_OK;
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    csr_diag_kernel<T><<<grid_for(n_rows, 256), 256, 0, as_stream(stream)>>>(
        n_rows, indptr, indices, (const T*)data, (T*)diag);
    return launch_check("tg_csr_diagonal");
  });
}

extern "C" int tg_csr_apply_dirichlet(int prec, int64_t n_rows, const int32_t* indptr,
                                      const int32_t* indices, const uint8_t* fixed, void* data,
                                      void* stream) {
  if (n_rows < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n_rows == 0 || fixed == nullptr) return TG_OK;
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    csr_dirichlet_kernel<T><<<grid_for(n_rows * 32, 256), 256, 0, as_stream(stream)>>>(
        n_rows, indptr, indices, fixed, (T*)data);
    return launch_check("tg_csr_apply_dirichlet");
  });
}

// The vector kernels read and write four entries at a time (16-byte loads and
// stores); a caller's pointer at an odd offset would fault, so it is refused here.
static int check_align16(const void* p, const char* fn, const char* what) {
  if (reinterpret_cast<uintptr_t>(p) % 16 != 0)
    return set_error(TG_ERR_VALUE,
                     "%s: %s must be 16-byte aligned (address %p); copy the vector into a "
                     "fresh buffer first",
                     fn, what, p);
  return TG_OK;
}

extern "C" size_t tg_dot_workspace_bytes(void) { return (size_t)DOT_CHUNKS * 2 * sizeof(double); }

extern "C" int tg_dot(int prec, const void* x, const void* y, int64_t n, double* out_dev,
                      void* workspace, size_t workspace_bytes, void* stream) {
  if (n < 0) return set_error(TG_ERR_VALUE, "negative size");
  TG_TRY(check_ptr(out_dev, "out"));
  TG_TRY(check_align16(x, "tg_dot", "x"));
  TG_TRY(check_align16(y, "tg_dot", "y"));
  if (workspace_bytes < tg_dot_workspace_bytes())
    return set_error(TG_ERR_WORKSPACE, "tg_dot: workspace too small");
  cudaStream_t st = as_stream(stream);
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    dot_partial_kernel<T><<<dot_chunks(n), DOT_THREADS, 0, st>>>((const T*)x, (const T*)y, n,
                                                              (double*)workspace);
    dot_final_kernel<1><<<1, DOT_THREADS, 0, st>>>((const double*)workspace, out_dev, dot_chunks(n));
    return launch_check("tg_dot");
  });
}

extern "C" int tg_axpby(int prec, int64_t n, double a, const void* x, double b, void* y,
                        void* stream) {
  if (n < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n == 0) return TG_OK;
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    axpby_kernel<T><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(n, a, (const T*)x, b, (T*)y);
    return launch_check("tg_axpby");
  });
}

extern "C" int tg_convert(int prec_in, const void* in, int prec_out, void* out, int64_t n,
                          void* stream) {
  if (n < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n == 0) return TG_OK;
  return dispatch_prec(prec_in, [&](auto ti) -> int {
    using Ti = decltype(ti);
    return dispatch_prec(prec_out, [&](auto to) -> int {
      using To = decltype(to);
      convert_kernel<Ti, To><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>((const Ti*)in,
                                                                              (To*)out, n);
      return launch_check("tg_convert");
    });
  });
}

extern "C" size_t tg_operator_workspace_bytes(const tg_operator_desc* op) {
  if (!op || op->csr_data) return 0;
  return tg_apply_workspace_bytes(op->elem, op->prec, op->mat.kind, op->plan);
}

extern "C" int tg_operator_apply(const tg_operator_desc* op, const void* x, void* y,
                                 void* workspace, size_t workspace_bytes, void* stream) {
  TG_TRY(check_ptr(op, "op"));
  if (op->csr_data) {
    if (op->csr_node_ptr && op->csr_node_indices)
      return tg_spmv_blocks3(op->prec, op->n_rows, op->csr_indptr, op->csr_node_ptr,
                             op->csr_node_indices, op->csr_data, x, y, stream);
    return tg_spmv(op->prec, op->n_rows, op->csr_indptr, op->csr_indices, op->csr_data, x, y,
                   stream);
  }
  return tg_apply(op->elem, op->prec, TG_MODE_HVP, &op->mat, op->plan, op->coords, op->n_nodes,
                  op->u, x, op->fixed, y, workspace, workspace_bytes, stream);
}

// ----------------------------------------------------------------------------- CG
namespace tg {

struct CgBuffers {
  void *r, *p, *q, *dinv, *apply_ws;
  bool grid;  // structured-brick linear elasticity: the HVP launch also forms p.q
  uint8_t* nmask;  // grid: the Dirichlet mask packed to one byte per node (or NULL)
  double *part, *scal;
  unsigned* ticket;  // [2] last-CTA arrival counters of the p.q and update kernels
  size_t apply_bytes;
  // the captured run of check_every iterations: its buffers and operator are the same
  // for every restart of one solve, so it is instantiated once per solve call (the
  // caller destroys it with cg_release)
  cudaGraphExec_t exec = nullptr;
  int graph_len = 0;
};

static void cg_release(CgBuffers& B) {
  if (B.exec) cudaGraphExecDestroy(B.exec);
  B.exec = nullptr;
  B.graph_len = 0;
}

// releases the solve's CUDA graph on every return path of a solve entry point
struct CgGraphGuard {
  CgBuffers& b;
  ~CgGraphGuard() { cg_release(b); }
};

// The operator is linear elasticity on a structured brick whose plan carries the grid:
// the CG's HVP runs as the grid stencil and forms p.q and alpha in the same launch.
static bool grid_op(const tg_operator_desc* op) {
  return !op->csr_data && op->plan && op->elem == TG_HEX8 && op->mat.kind == TG_LINEAR_ELASTIC &&
         op->mat.elem_param == nullptr && op->plan->grid_nodes[0] > 0 &&
         (int64_t)op->plan->grid_nodes[0] * op->plan->grid_nodes[1] * op->plan->grid_nodes[2] ==
             op->n_nodes &&
         grid_cg_ctas(op->plan) > 0;
}

static int64_t cg_part_doubles(const tg_operator_desc* op) {
  const int64_t g = grid_op(op) ? grid_cg_ctas(op->plan) : 0;
  return g > 2 * DOT_CHUNKS ? g : 2 * DOT_CHUNKS;
}

static size_t cg_bytes(const tg_operator_desc* op) {
  const int64_t n = op_ndofs(op);
  const size_t vs = align256((size_t)n * prec_size(op->prec));
  const size_t mask_bytes = (grid_op(op) && op->fixed) ? align256((size_t)op->n_nodes) : 0;
  return 4 * vs + mask_bytes + align256(tg_operator_workspace_bytes(op)) +
         align256((size_t)cg_part_doubles(op) * sizeof(double)) +
         align256(SCAL_N * sizeof(double)) + align256(2 * sizeof(unsigned));
}

static CgBuffers cg_carve(const tg_operator_desc* op, void* ws) {
  Carve c{(char*)ws};
  const int64_t n = op_ndofs(op);
  CgBuffers b;
  const size_t vb = (size_t)n * prec_size(op->prec);
  b.grid = grid_op(op);
  b.r = c.take(vb);
  b.p = c.take(vb);
  b.dinv = c.take(vb);
  b.q = c.take(vb);
  b.nmask = (b.grid && op->fixed) ? (uint8_t*)c.take((size_t)op->n_nodes) : nullptr;
  b.apply_bytes = tg_operator_workspace_bytes(op);
  b.apply_ws = c.take(b.apply_bytes);
  b.part = (double*)c.take((size_t)cg_part_doubles(op) * sizeof(double));
  b.scal = (double*)c.take(SCAL_N * sizeof(double));
  b.ticket = (unsigned*)c.take(2 * sizeof(unsigned));
  return b;
}

// dinv = 1/diag and the recursion's residual r = b - A x; the direction is left as it
// is.  Grid CG with fixed dofs: x = b and dinv = 0 on them first (grid_cg_fixed), so r,
// z and p stay exactly zero there and the iterations' HVP masks only its output rows.
template <class T>
static int cg_residual(const tg_operator_desc* op, const T* bvec, T* x, const T* diag,
                       CgBuffers& B, cudaStream_t st) {
  const int64_t n = op_ndofs(op);
  inv_kernel<T><<<grid_for(n, 256), 256, 0, st>>>(n, diag, (T*)B.dinv);
  if (B.nmask) {
    TG_TRY(pack_node_mask(op->fixed, op->n_nodes, B.nmask, st));
    TG_TRY(grid_cg_fixed(op->prec, op->n_nodes, B.nmask, bvec, x, B.dinv, st));
  }
  TG_TRY(tg_operator_apply(op, x, B.r, B.apply_ws, B.apply_bytes, st));
  axpby_kernel<T><<<grid_for(n, 256), 256, 0, st>>>(n, 1.0, bvec, -1.0, (T*)B.r);
  return launch_check("cg residual");
}

// cg_residual, then p = r dinv ; scal <- (rz, rr); arrival counters zeroed
template <class T>
static int cg_restart(const tg_operator_desc* op, const T* bvec, T* x, const T* diag,
                      CgBuffers& B, cudaStream_t st) {
  const int64_t n = op_ndofs(op);
  TG_TRY(cg_residual<T>(op, bvec, x, diag, B, st));
  cg_init_kernel<T><<<dot_chunks(n), DOT_THREADS, 0, st>>>(n, (const T*)B.r, (const T*)B.dinv,
                                                        (T*)B.p, B.part);
  cg_init_final_kernel<<<1, DOT_THREADS, 0, st>>>(B.part, B.scal, dot_chunks(n));
  TG_TRY(cuda_check(cudaMemsetAsync(B.ticket, 0, 2 * sizeof(unsigned), st), "cg: counters"));
  return launch_check("cg restart");
}

template <class T>
static int cg_iteration(const tg_operator_desc* op, T* x, const T* diag, CgBuffers& B,
                        cudaStream_t st) {
  const int64_t n = op_ndofs(op);
  if (B.grid) {  // q = A p with p.q and alpha in the same launch
    TG_TRY(launch_grid_hvp_dot(op->plan, op->prec, op->mat.p0, op->mat.p1, B.p, B.nmask, B.q,
                               B.scal, B.part, B.ticket, st));
  } else {
    TG_TRY(tg_operator_apply(op, B.p, B.q, B.apply_ws, B.apply_bytes, st));
    cg_pq_kernel<T><<<dot_chunks(n), DOT_THREADS, 0, st>>>((const T*)B.p, (const T*)B.q, n,
                                                        B.part, B.scal, B.ticket);
  }
  cg_update_kernel<T><<<dot_chunks(n), DOT_THREADS, 0, st>>>(n, B.scal, x, (T*)B.r,
                                                          (const T*)B.p, (const T*)B.q,
                                                          (const T*)B.dinv, B.part, B.ticket + 1);
  cg_p_kernel<T><<<grid_for((n + 3) / 4, 256), 256, 0, st>>>(n, B.scal, (const T*)B.r,
                                                          (const T*)B.dinv, (T*)B.p);
  return launch_check("cg iteration");
}

static int read_scalars(const double* dev, double* host, cudaStream_t st) {
  TG_TRY(cuda_check(cudaMemcpyAsync(host, dev, SCAL_N * sizeof(double), cudaMemcpyDeviceToHost, st),
                    "cg: read scalars"));
  return cuda_check(cudaStreamSynchronize(st), "cg: synchronize");
}

// Runs CG from the current x until sqrt(rr) <= tol_abs (recursive residual) or the
// iteration budget is spent.  Returns TG_OK, TG_ERR_NOT_CONVERGED or TG_ERR_BREAKDOWN.
// resume: the recursion's residual, direction and scalars were set by the caller
// (a reliable update) instead of a restart from x.
template <class T>
static int cg_run(const tg_operator_desc* op, const T* bvec, T* x, const T* diag, double tol_abs,
                  int max_iter, int check_every, CgBuffers& B, cudaStream_t st, int* iters,
                  bool resume = false) {
  double h[SCAL_N];
  if (!resume) TG_TRY(cg_restart<T>(op, bvec, x, diag, B, st));
  const double tol2 = tol_abs * tol_abs;  // the update kernel's stopping test
  TG_TRY(cuda_check(cudaMemcpyAsync(B.scal + SCAL_TOL2, &tol2, sizeof(double),
                                    cudaMemcpyHostToDevice, st),
                    "cg: tolerance"));
  TG_TRY(read_scalars(B.scal, h, st));
  *iters = 0;
  if (!std::isfinite(h[SCAL_RR])) return set_error(TG_ERR_BREAKDOWN, "cg: non-finite residual");
  if (std::sqrt(h[SCAL_RR]) <= tol_abs) return TG_OK;
  check_every = check_every < 1 ? 1 : check_every;
  cudaGraphExec_t& exec = B.exec;
  int& graph_len = B.graph_len;
  const bool can_capture = (st != nullptr) && (st != cudaStreamLegacy) && (st != cudaStreamPerThread);
  int rc = TG_OK;
  bool done = false;
  while (*iters < max_iter) {
    const int k = (max_iter - *iters) < check_every ? (max_iter - *iters) : check_every;
    const int before = *iters;
    if (can_capture && k == check_every) {
      if (!exec || graph_len != k) {
        cudaGraph_t graph;
        rc = cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cg: capture");
        if (rc != TG_OK) break;
        int rci = TG_OK;
        for (int i = 0; i < k && rci == TG_OK; ++i) rci = cg_iteration<T>(op, x, diag, B, st);
        cudaError_t ec = cudaStreamEndCapture(st, &graph);
        if (rci != TG_OK) { rc = rci; break; }
        rc = cuda_check(ec, "cg: end capture");
        if (rc != TG_OK) break;
        if (exec) cudaGraphExecDestroy(exec);
        rc = cuda_check(cudaGraphInstantiate(&exec, graph, 0), "cg: instantiate");
        cudaGraphDestroy(graph);
        if (rc != TG_OK) { exec = nullptr; break; }
        graph_len = k;
      }
      rc = cuda_check(cudaGraphLaunch(exec, st), "cg: graph launch");
      if (rc != TG_OK) break;
    } else {
      for (int i = 0; i < k && rc == TG_OK; ++i) rc = cg_iteration<T>(op, x, diag, B, st);
      if (rc != TG_OK) break;
    }
    rc = read_scalars(B.scal, h, st);
    if (rc != TG_OK) break;
    *iters = (int)h[SCAL_ITERS];  // iterations that ran (a converged block stops early)
    if (h[SCAL_FLAG] != 0.0 || !std::isfinite(h[SCAL_RR])) {
      rc = set_error(TG_ERR_BREAKDOWN, "cg: breakdown (p.Ap <= 0 or non-finite) after %d iterations", *iters);
      break;
    }
    done = h[SCAL_DONE] != 0.0 || std::sqrt(h[SCAL_RR]) <= tol_abs;
    if (done) break;
    if (*iters == before) {  // no iteration ran although the solve has not converged
      rc = set_error(TG_ERR_BREAKDOWN, "cg: no progress after %d iterations", *iters);
      break;
    }
  }
  if (rc != TG_OK) return rc;
  if (!done)
    return set_error(TG_ERR_NOT_CONVERGED, "cg: not converged in %d iterations", *iters);
  return TG_OK;
}

template <class T>
static int true_residual_norm(const tg_operator_desc* op, const T* bvec, const T* x,
                              CgBuffers& B, cudaStream_t st, double* rn, double* bn) {
  const int64_t n = op_ndofs(op);
  TG_TRY(tg_operator_apply(op, x, B.r, B.apply_ws, B.apply_bytes, st));
  axpby_kernel<T><<<grid_for(n, 256), 256, 0, st>>>(n, 1.0, bvec, -1.0, (T*)B.r);
  dot_partial_kernel<T><<<dot_chunks(n), DOT_THREADS, 0, st>>>((const T*)B.r, (const T*)B.r, n, B.part);
  dot_final_kernel<1><<<1, DOT_THREADS, 0, st>>>(B.part, B.scal + 5, dot_chunks(n));
  dot_partial_kernel<T><<<dot_chunks(n), DOT_THREADS, 0, st>>>(bvec, bvec, n, B.part);
  dot_final_kernel<1><<<1, DOT_THREADS, 0, st>>>(B.part, B.scal + 7, dot_chunks(n));
  TG_TRY(launch_check("true residual"));
  double h[SCAL_N];
  TG_TRY(read_scalars(B.scal, h, st));
  *rn = std::sqrt(h[5]);
  *bn = std::sqrt(h[7]);
  return TG_OK;
}

}  // namespace tg

extern "C" size_t tg_cg_workspace_bytes(const tg_operator_desc* op) {
  return op ? cg_bytes(op) : 0;
}

extern "C" int tg_cg_solve(const tg_operator_desc* op, const void* b, void* x, const void* diag,
                           double rtol, int max_iter, int check_every, void* workspace,
                           size_t workspace_bytes, tg_solve_stats* stats, void* stream) {
  TG_TRY(check_ptr(op, "op"));
  TG_TRY(check_ptr(b, "b"));
  TG_TRY(check_ptr(x, "x"));
  TG_TRY(check_ptr(diag, "diag"));
  TG_TRY(check_align16(b, "tg_cg_solve", "b"));
  TG_TRY(check_align16(x, "tg_cg_solve", "x"));
  if (workspace_bytes < cg_bytes(op)) return set_error(TG_ERR_WORKSPACE, "tg_cg_solve: workspace too small");
  if (!(rtol > 0.0) || max_iter < 0) return set_error(TG_ERR_VALUE, "bad rtol / max_iter");
  cudaStream_t st = as_stream(stream);
  CgBuffers B = cg_carve(op, workspace);
  CgGraphGuard guard{B};
  return dispatch_prec(op->prec, [&](auto t) -> int {
    using T = decltype(t);
    double rn = 0, bn = 0;
    TG_TRY(true_residual_norm<T>(op, (const T*)b, (const T*)x, B, st, &rn, &bn));
    int total = 0, rc = TG_OK;
    const double tol = rtol * bn;
    // restart on the true residual until it meets the tolerance (bounded by max_iter)
    for (int restart = 0; restart < 8 && rn > tol && total < max_iter; ++restart) {
      int it = 0;
      rc = cg_run<T>(op, (const T*)b, (T*)x, (const T*)diag, 0.5 * tol, max_iter - total,
                     check_every, B, st, &it);
      total += it;
      TG_TRY(true_residual_norm<T>(op, (const T*)b, (const T*)x, B, st, &rn, &bn));
      if (rc != TG_OK) break;
    }
    if (stats) {
      stats->iterations = total;
      stats->outer = 0;
      stats->rel_res = bn > 0 ? rn / bn : rn;
    }
    if (rc == TG_OK && rn > tol) rc = set_error(TG_ERR_NOT_CONVERGED, "tg_cg_solve: not converged");
    if (stats) stats->status = rc;
    return rc;
  });
}

// ----------------------------------------------------------------------------- mixed
extern "C" size_t tg_mixed_workspace_bytes(const tg_operator_desc* op64,
                                           const tg_operator_desc* op32) {
  if (!op64 || !op32) return 0;
  const int64_t n = op_ndofs(op64);
  return cg_bytes(op32) + align256(tg_operator_workspace_bytes(op64)) +
         align256((size_t)n * sizeof(double)) + 3 * align256((size_t)n * sizeof(float)) +
         align256(DOT_CHUNKS * sizeof(double)) + align256(8 * sizeof(double));
}

extern "C" int tg_mixed_solve(const tg_operator_desc* op64, const tg_operator_desc* op32,
                              const double* b, double* x, const double* diag64, double rtol,
                              double inner_rtol, int max_outer, int max_inner, int check_every,
                              void* workspace, size_t workspace_bytes, tg_solve_stats* stats,
                              void* stream) {
  TG_TRY(check_ptr(op64, "op64"));
  TG_TRY(check_ptr(op32, "op32"));
  TG_TRY(check_ptr(b, "b"));
  TG_TRY(check_ptr(x, "x"));
  TG_TRY(check_ptr(diag64, "diag64"));
  TG_TRY(check_align16(b, "tg_mixed_solve", "b"));
  if (op64->prec != TG_F64 || op32->prec != TG_F32)
    return set_error(TG_ERR_TYPE, "tg_mixed_solve: op64 must be FP64 and op32 FP32");
  const int64_t n = op_ndofs(op64);
  if (op_ndofs(op32) != n) return set_error(TG_ERR_VALUE, "tg_mixed_solve: operator sizes differ");
  if (workspace_bytes < tg_mixed_workspace_bytes(op64, op32))
    return set_error(TG_ERR_WORKSPACE, "tg_mixed_solve: workspace too small");
  cudaStream_t st = as_stream(stream);
  Carve c{(char*)workspace};
  CgBuffers B = cg_carve(op32, c.take(cg_bytes(op32)));
  CgGraphGuard guard{B};
  const size_t ab64 = tg_operator_workspace_bytes(op64);
  void* aws64 = c.take(ab64);
  double* r64 = (double*)c.take(n * sizeof(double));
  float* r32 = (float*)c.take(n * sizeof(float));
  float* d32 = (float*)c.take(n * sizeof(float));
  float* diag32 = (float*)c.take(n * sizeof(float));
  double* part = (double*)c.take(DOT_CHUNKS * sizeof(double));
  double* sc = (double*)c.take(8 * sizeof(double));

  convert_kernel<double, float><<<grid_for(n, 256), 256, 0, st>>>(diag64, diag32, n);
  // |b|^2
  dot_partial_kernel<double><<<dot_chunks(n), DOT_THREADS, 0, st>>>(b, b, n, part);
  dot_final_kernel<1><<<1, DOT_THREADS, 0, st>>>(part, sc + 1, dot_chunks(n));
  TG_TRY(launch_check("mixed: setup"));
  int total_inner = 0, outer = 0, rc = TG_OK;
  double rn = 0.0, bn = 0.0, rn_prev = 0.0;
  double h[8];
  // inner_rtol >= 0.01: reliable updates.  The inner recursion keeps its direction
  // from one FP64 residual replacement to the next (re-orthogonalised against the new
  // residual, cg_resume_*), so the Krylov information outlives the replacement; the
  // replacements have to come often for that (every 10x reduction by default).
  // Smaller inner_rtol: each refinement restarts the inner CG from d = 0.
  const bool keep_direction = inner_rtol >= 0.01;
  bool have_direction = false;
  for (;;) {
    // true residual r64 = b - A64 x in FP64
    TG_TRY(tg_operator_apply(op64, x, r64, aws64, ab64, st));
    axpby_kernel<double><<<grid_for(n, 256), 256, 0, st>>>(n, 1.0, b, -1.0, r64);
    dot_partial_kernel<double><<<dot_chunks(n), DOT_THREADS, 0, st>>>(r64, r64, n, part);
    dot_final_kernel<1><<<1, DOT_THREADS, 0, st>>>(part, sc, dot_chunks(n));
    TG_TRY(launch_check("mixed: residual"));
    TG_TRY(cuda_check(cudaMemcpyAsync(h, sc, 8 * sizeof(double), cudaMemcpyDeviceToHost, st), "mixed: read"));
    TG_TRY(cuda_check(cudaStreamSynchronize(st), "mixed: sync"));
    rn = std::sqrt(h[0]);
    bn = std::sqrt(h[1]);
    if (!std::isfinite(rn)) { rc = set_error(TG_ERR_BREAKDOWN, "mixed: non-finite residual"); break; }
    if (rn <= rtol * bn || bn == 0.0) break;
    if (outer >= max_outer) { rc = set_error(TG_ERR_NOT_CONVERGED, "mixed: not converged after %d refinements", outer); break; }
    // inner FP32 solve A32 d = r64 / |r64|, d0 = 0
    scale_down_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(n, r64, 1.0 / rn, r32);
    TG_TRY(cuda_check(cudaMemsetAsync(d32, 0, n * sizeof(float), st), "mixed: zero"));
    int it = 0;
    // the inner solve needs to reduce |r| only as far as the target still requires
    // (with a factor-2 margin): the last refinement is not solved to inner_rtol
    double itol = 0.5 * rtol * bn / rn;
    itol = itol < inner_rtol ? inner_rtol : (itol > 0.5 ? 0.5 : itol);
    const bool resume = keep_direction && have_direction;
    if (resume) {  // the recursion continues on the new residual (d = 0 again)
      TG_TRY(cg_residual<float>(op32, r32, d32, diag32, B, st));
      const int nc = dot_chunks(n);
      cg_resume_partial_kernel<float><<<nc, DOT_THREADS, 0, st>>>(
          n, (const float*)B.r, (const float*)B.dinv, (const float*)B.p, B.part, part);
      cg_resume_final_kernel<<<1, DOT_THREADS, 0, st>>>(B.part, part, nc, rn_prev / rn, B.scal,
                                                        sc + 2);
      cg_resume_p_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(
          n, sc + 2, (const float*)B.r, (const float*)B.dinv, (float*)B.p);
      TG_TRY(cuda_check(cudaMemsetAsync(B.ticket, 0, 2 * sizeof(unsigned), st), "mixed: counters"));
      TG_TRY(launch_check("mixed: reliable update"));
    }
    const int irc = cg_run<float>(op32, r32, d32, diag32, itol, max_inner, check_every, B, st,
                                  &it, resume);
    total_inner += it;
    if (irc == TG_ERR_BREAKDOWN) { rc = irc; break; }
    if (irc != TG_OK && irc != TG_ERR_NOT_CONVERGED) { rc = irc; break; }
    // the direction can be carried on only from a recursion that stopped in its update
    // kernel (beta and rz of its last step are then in the scalars)
    have_direction = irc == TG_OK && it > 0;
    rn_prev = rn;
    // x += |r64| d
    scale_up_add_kernel<float><<<grid_for(n, 256), 256, 0, st>>>(n, d32, rn, x);
    TG_TRY(launch_check("mixed: update"));
    ++outer;
  }
  if (stats) {
    stats->status = rc;
    stats->iterations = total_inner;
    stats->outer = outer;
    stats->rel_res = bn > 0 ? rn / bn : rn;
  }
  return rc;
}
