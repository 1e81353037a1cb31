// Batched solves of many independent sparse SPD systems in one persistent launch.
//
// The reference has no batched solver: a user loops over meshes and calls
// jax.scipy.sparse.linalg.cg on each (README.md:93).  Here every system is one
// mesh's assembled, Dirichlet-reduced CSR matrix (tatva.sparse.jacfwd output,
// tatva/sparse/base.py:139-176), converted once to a per-system ELLPACK layout:
// column-major (entry k of local row i at k * n_rows + i) with 16-bit local column
// ids, so that one thread per row reads coalesced.
//
// One CTA solves one system at a time, start to finish, and then takes the next one
// from a device counter (systems ordered largest first).  The search direction p
// lives in shared memory, so the SpMV gathers hit shared memory; the other vectors
// stay in global memory (the working set of the systems in flight fits in L2).
// Each system runs FP32 Jacobi-preconditioned CG on the residual direction
// r64 / |r64| and FP64 iterative refinement on the true residual b - A64 x, until
// |b - A64 x| <= rtol |b|.  Dots accumulate as exact-product float pairs per thread
// and are reduced in FP64 in a fixed order, so each system's result depends only on
// its own data and the block size -- not on which CTA took it, nor on what else ran.
// Every loop is bounded by max_outer / max_inner; no CTA waits on another.
#include <cmath>
#include <map>
#include <mutex>

#include "tg_common.cuh"
#include "tg_dispatch.cuh"

namespace tg {
namespace {

constexpr int BATCH_MAX_ROWS = 49152;  // shared-memory p: 192 KB
constexpr int RU = 4;                  // rows per thread in flight in the CG passes

struct BatchArgs {
  tg_batch_desc d;
  const double* b;
  double* x;
  float* q;
  float* r;
  float* dv;
  float* idiag;
  double* r64;
  int* counter;
  double rtol, inner_rtol;
  int max_outer, max_inner;
  int32_t* iters;
  int32_t* outer;
  double* rel_res;
  int32_t* status;
};

struct Acc2 {  // float pair with exact products (two-sum + FMA split)
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

// Sum of K per-thread values over the block in a fixed order; every thread gets the
// result.  `buf` alternates between two halves so that one barrier per reduction
// suffices (a half is rewritten only after the next reduction's barrier).
template <int NT, int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* buf, int& flip) {
  constexpr int NW = NT / 32;
  double* h = buf + flip * (NW * 4);
  flip ^= 1;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double t = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    v[k] = t;
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) h[w * 4 + k] = v[k];
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < NW; ++j) s += h[j * 4 + k];
    v[k] = s;
  }
}

template <int NT>
__device__ void solve_system(const BatchArgs& a, int sys, float* p, double* red, int& flip) {
  const int tid = threadIdx.x;
  const int64_t r0 = a.d.row_ofs[sys];
  const int n = (int)(a.d.row_ofs[sys + 1] - r0);
  const int W = a.d.ell_width[sys];
  const int64_t e0 = a.d.ell_ofs[sys];
  const uint16_t* __restrict__ col = a.d.ell_col + e0;
  const float* __restrict__ v32 = a.d.ell_val32 + e0;
  const double* __restrict__ v64 = a.d.ell_val64 + e0;
  const double* __restrict__ b = a.b + r0;
  double* __restrict__ x = a.x + r0;
  float* __restrict__ q = a.q + r0;
  float* __restrict__ r = a.r + r0;
  float* __restrict__ dv = a.dv + r0;
  float* __restrict__ idg = a.idiag + r0;
  double* __restrict__ r64 = a.r64 + r0;

  if (n < 0 || n > a.d.max_rows || W < 0) {  // inconsistent description: skip the system
    if (tid == 0) {
      a.iters[sys] = 0;
      a.outer[sys] = 0;
      a.rel_res[sys] = 1.0;
      a.status[sys] = TG_ERR_VALUE;
    }
    __syncthreads();
    return;
  }
  // set-up: inverse diagonal, x = 0, r64 = b, |b|^2
  double s2[2] = {0.0, 0.0};
  for (int i = tid; i < n; i += NT) {
    float dg = 0.f;
    for (int k = 0; k < W; ++k)
      if (col[(int64_t)k * n + i] == i) dg += v32[(int64_t)k * n + i];
    if (!(dg > 0.f)) s2[1] += 1.0;
    idg[i] = 1.f / dg;
    x[i] = 0.0;
    const double bi = b[i];
    r64[i] = bi;
    s2[0] += bi * bi;
  }
  block_sum<NT, 2>(s2, red, flip);
  const double nb = sqrt(s2[0]);
  int status = TG_OK, it_total = 0, n_outer = 0;
  double rel = 0.0;
  if (s2[1] > 0.0) {
    status = TG_ERR_BREAKDOWN;  // a non-positive diagonal entry: not SPD
    rel = 1.0;
  } else if (nb > 0.0) {
    double rn = nb;
    for (;;) {
      rel = rn / nb;
      if (rel <= a.rtol) break;
      if (n_outer >= a.max_outer) { status = TG_ERR_NOT_CONVERGED; break; }
      ++n_outer;
      // inner FP32 CG on A d = r64 / |r64|
      const double inv_rn = 1.0 / rn;
      Acc2 rz_acc, rr_acc;
      for (int i = tid; i < n; i += NT) {
        const float ri = (float)(r64[i] * inv_rn);
        const float zi = ri * idg[i];
        r[i] = ri;
        dv[i] = 0.f;
        p[i] = zi;
        rz_acc.add(ri, zi);
        rr_acc.add(ri, ri);
      }
      double t2[2] = {rz_acc.value(), rr_acc.value()};
      block_sum<NT, 2>(t2, red, flip);  // also publishes p
      double rz = t2[0];
      const double rr0 = t2[1];
      const double stop = a.inner_rtol * a.inner_rtol * rr0;
      bool broke = false;
      for (int it = 0; it < a.max_inner; ++it) {
        // rows i0, i0 + NT, ..., i0 + (RU-1) NT together: their loads are independent,
        // so RU rows' worth of L2 requests are in flight at once.  Accumulation order
        // (rows in increasing i per thread, entries in increasing k) is unchanged.
        Acc2 pq_acc;
        for (int i0 = tid; i0 < n; i0 += RU * NT) {
          float sv[RU];
#pragma unroll
          for (int u = 0; u < RU; ++u) sv[u] = 0.f;
          for (int k = 0; k < W; ++k) {
            float av[RU];
            uint16_t cv[RU];
#pragma unroll
            for (int u = 0; u < RU; ++u) {
              const int i = i0 + u * NT;
              const int64_t e = (int64_t)k * n + (i < n ? i : 0);
              av[u] = v32[e];
              cv[u] = col[e];
            }
#pragma unroll
            for (int u = 0; u < RU; ++u)
              if (i0 + u * NT < n) sv[u] = fmaf(av[u], p[cv[u]], sv[u]);
          }
#pragma unroll
          for (int u = 0; u < RU; ++u) {
            const int i = i0 + u * NT;
            if (i < n) {
              q[i] = sv[u];
              pq_acc.add(p[i], sv[u]);
            }
          }
        }
        double t1[1] = {pq_acc.value()};
        block_sum<NT, 1>(t1, red, flip);
        const double pq = t1[0];
        ++it_total;
        if (!(pq > 0.0) || !isfinite(pq)) { broke = true; break; }
        const float alpha = (float)(rz / pq);
        Acc2 rz2, rr2;
        for (int i0 = tid; i0 < n; i0 += RU * NT) {
          float dvv[RU], qv[RU], rv[RU], gv[RU];
#pragma unroll
          for (int u = 0; u < RU; ++u) {
            const int i = i0 + u * NT < n ? i0 + u * NT : i0;
            dvv[u] = dv[i];
            qv[u] = q[i];
            rv[u] = r[i];
            gv[u] = idg[i];
          }
#pragma unroll
          for (int u = 0; u < RU; ++u) {
            const int i = i0 + u * NT;
            if (i < n) {
              dv[i] = fmaf(alpha, p[i], dvv[u]);
              const float ri = fmaf(-alpha, qv[u], rv[u]);
              r[i] = ri;
              const float zi = ri * gv[u];
              rz2.add(ri, zi);
              rr2.add(ri, ri);
            }
          }
        }
        double t3[2] = {rz2.value(), rr2.value()};
        block_sum<NT, 2>(t3, red, flip);
        if (!isfinite(t3[1])) { broke = true; break; }
        if (t3[1] <= stop) break;
        const float beta = (float)(t3[0] / rz);
        rz = t3[0];
#pragma unroll 4
        for (int i = tid; i < n; i += NT) p[i] = fmaf(beta, p[i], r[i] * idg[i]);
        __syncthreads();
      }
      if (broke) { status = TG_ERR_BREAKDOWN; break; }
      // refinement: x += |r64| d, r64 = b - A64 x (FP64)
      for (int i = tid; i < n; i += NT) x[i] += rn * (double)dv[i];
      __syncthreads();
      double u2[1] = {0.0};
      for (int i = tid; i < n; i += NT) {
        double s = b[i];
        for (int k = 0; k < W; ++k) {
          const int64_t e = (int64_t)k * n + i;
          s -= v64[e] * x[col[e]];
        }
        r64[i] = s;
        u2[0] += s * s;
      }
      block_sum<NT, 1>(u2, red, flip);
      rn = sqrt(u2[0]);
      if (!isfinite(rn)) { status = TG_ERR_BREAKDOWN; break; }
    }
  }
  if (tid == 0) {
    a.iters[sys] = it_total;
    a.outer[sys] = n_outer;
    a.rel_res[sys] = rel;
    a.status[sys] = status;
  }
  __syncthreads();  // p, red and the system index are reused by the next system
}

template <int NT>
__global__ void __launch_bounds__(NT) batch_solve_kernel(BatchArgs a) {
  extern __shared__ __align__(16) float p[];
  __shared__ double red[2 * (NT / 32) * 4];
  __shared__ int s_next;
  int flip = 0;
  for (;;) {
    if (threadIdx.x == 0) s_next = atomicAdd(a.counter, 1);
    __syncthreads();
    const int k = s_next;
    __syncthreads();
    if (k >= a.d.n_systems) break;
    solve_system<NT>(a, a.d.order[k], p, red, flip);
  }
}

// ELL conversion: thread per global row (row -> system by binary search on row_ofs)
__global__ void ell_from_csr_kernel(tg_batch_desc d, int64_t n_rows, const int32_t* __restrict__ indptr,
                                    const int32_t* __restrict__ indices,
                                    const double* __restrict__ data, uint16_t* col, float* v32,
                                    double* v64, int* bad) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_rows) return;
  int lo = 0, hi = d.n_systems;  // largest s with row_ofs[s] <= g
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (d.row_ofs[mid] <= g) lo = mid; else hi = mid;
  }
  const int s = lo;
  const int64_t r0 = d.row_ofs[s];
  const int n = (int)(d.row_ofs[s + 1] - r0);
  const int i = (int)(g - r0);
  const int W = d.ell_width[s];
  const int64_t e0 = d.ell_ofs[s];
  const int j0 = indptr[g], len = indptr[g + 1] - j0;
  if (len > W) { atomicExch(bad, 1); return; }
  for (int k = 0; k < W; ++k) {
    const int64_t e = e0 + (int64_t)k * n + i;
    if (k < len) {
      const int64_t c = (int64_t)indices[j0 + k] - r0;
      if (c < 0 || c >= n) {  // a coupling between two systems: not block diagonal
        atomicExch(bad, 2);
        col[e] = (uint16_t)i;
        v32[e] = 0.f;
        v64[e] = 0.0;
        continue;
      }
      col[e] = (uint16_t)c;
      v64[e] = data[j0 + k];
      v32[e] = (float)data[j0 + k];
    } else {
      col[e] = (uint16_t)i;
      v32[e] = 0.f;
      v64[e] = 0.0;
    }
  }
}

int desc_check(const tg_batch_desc* d) {
  if (!d) return set_error(TG_ERR_VALUE, "batch description must not be NULL");
  if (d->n_systems < 0) return set_error(TG_ERR_VALUE, "n_systems must be >= 0");
  if (d->max_rows < 0 || d->max_rows > BATCH_MAX_ROWS)
    return set_error(TG_ERR_UNSUPPORTED, "batched solve: a system has %d rows; at most %d are supported",
                     d->max_rows, BATCH_MAX_ROWS);
  if (d->n_systems > 0) {
    TG_TRY(check_ptr(d->row_ofs, "row_ofs"));
    TG_TRY(check_ptr(d->ell_ofs, "ell_ofs"));
    TG_TRY(check_ptr(d->ell_width, "ell_width"));
    TG_TRY(check_ptr(d->ell_col, "ell_col"));
    TG_TRY(check_ptr(d->ell_val32, "ell_val32"));
    TG_TRY(check_ptr(d->ell_val64, "ell_val64"));
  }
  return TG_OK;
}

}  // namespace
}  // namespace tg

using namespace tg;

extern "C" int tg_batch_ell_from_csr(const tg_batch_desc* desc, int64_t n_rows,
                                     const int32_t* indptr, const int32_t* indices,
                                     const double* data, int32_t* bad_flag, void* stream) {
  TG_TRY(desc_check(desc));
  if (n_rows < 0) return set_error(TG_ERR_VALUE, "n_rows must be >= 0");
  if (n_rows == 0) return TG_OK;
  TG_TRY(check_ptr(indptr, "indptr"));
  TG_TRY(check_ptr(indices, "indices"));
  TG_TRY(check_ptr(data, "data"));
  TG_TRY(check_ptr(bad_flag, "bad_flag"));
  ell_from_csr_kernel<<<grid_for(n_rows, 256), 256, 0, as_stream(stream)>>>(
      *desc, n_rows, indptr, indices, data, const_cast<uint16_t*>(desc->ell_col),
      const_cast<float*>(desc->ell_val32), const_cast<double*>(desc->ell_val64), bad_flag);
  return launch_check("tg_batch_ell_from_csr");
}

extern "C" size_t tg_batch_workspace_bytes(int64_t n_rows) {
  const size_t n = (size_t)(n_rows > 0 ? n_rows : 0);
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  return al(4 * n * sizeof(float)) + al(n * sizeof(double)) + 256;
}

extern "C" int tg_batch_solve(const tg_batch_desc* desc, int64_t n_rows, const double* b, double* x,
                              double rtol, double inner_rtol, int max_outer, int max_inner,
                              int threads, int ctas_per_sm, void* workspace, size_t workspace_bytes,
                              int32_t* iters, int32_t* outer, double* rel_res, int32_t* status,
                              void* stream) {
  TG_TRY(desc_check(desc));
  if (n_rows < 0) return set_error(TG_ERR_VALUE, "n_rows must be >= 0");
  if (!(rtol > 0.0) || !(inner_rtol > 0.0) || inner_rtol >= 1.0)
    return set_error(TG_ERR_VALUE, "need rtol > 0 and 0 < inner_rtol < 1");
  if (max_outer < 0 || max_inner <= 0) return set_error(TG_ERR_VALUE, "bad iteration limits");
  if (workspace_bytes < tg_batch_workspace_bytes(n_rows))
    return set_error(TG_ERR_WORKSPACE, "tg_batch_solve: workspace too small");
  if (desc->n_systems == 0) return TG_OK;
  TG_TRY(check_ptr(desc->order, "order"));
  TG_TRY(check_ptr(b, "b"));
  TG_TRY(check_ptr(x, "x"));
  TG_TRY(check_ptr(iters, "iters"));
  TG_TRY(check_ptr(outer, "outer"));
  TG_TRY(check_ptr(rel_res, "rel_res"));
  TG_TRY(check_ptr(status, "status"));
  TG_TRY(check_ptr(workspace, "workspace"));
  const size_t n = (size_t)n_rows;
  auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
  char* w = (char*)workspace;
  BatchArgs a;
  a.d = *desc;
  a.b = b;
  a.x = x;
  a.q = (float*)w;
  a.r = a.q + n;
  a.dv = a.r + n;
  a.idiag = a.dv + n;
  a.r64 = (double*)(w + al(4 * n * sizeof(float)));
  a.counter = (int*)(w + al(4 * n * sizeof(float)) + al(n * sizeof(double)));
  a.rtol = rtol;
  a.inner_rtol = inner_rtol;
  a.max_outer = max_outer;
  a.max_inner = max_inner;
  a.iters = iters;
  a.outer = outer;
  a.rel_res = rel_res;
  a.status = status;
  cudaStream_t st = as_stream(stream);
  TG_TRY(cuda_check(cudaMemsetAsync(a.counter, 0, sizeof(int), st), "tg_batch_solve: counter reset"));
  const size_t smem = (size_t)std::max(desc->max_rows, 1) * sizeof(float);
  int dev = 0, sms = 0;
  TG_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  TG_TRY(cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "SM count"));
  auto go = [&](auto kern, int nt) -> int {
    {
      // the attribute only grows: graphs captured with larger systems stay launchable
      static std::mutex mu;
      static std::map<std::pair<const void*, int>, size_t> attr;
      std::lock_guard<std::mutex> g(mu);
      size_t& cur = attr[std::make_pair((const void*)kern, dev)];
      if (smem > cur) {
        TG_TRY(cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                          "tg_batch_solve: shared memory attribute"));
        cur = smem;
      }
    }
    int per_sm = 0;
    TG_TRY(cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, smem),
                      "tg_batch_solve: occupancy"));
    if (per_sm <= 0) return set_error(TG_ERR_UNSUPPORTED, "tg_batch_solve: kernel does not fit on an SM");
    const int want = ctas_per_sm > 0 ? std::min(ctas_per_sm, per_sm) : per_sm;
    const int grid = std::max(1, std::min(desc->n_systems, sms * want));
    kern<<<grid, nt, smem, st>>>(a);
    return launch_check("tg_batch_solve");
  };
  switch (threads) {
    case 128: return go(batch_solve_kernel<128>, 128);
    case 256: return go(batch_solve_kernel<256>, 256);
    case 512: return go(batch_solve_kernel<512>, 512);
    default: return set_error(TG_ERR_VALUE, "threads must be 128, 256 or 512");
  }
}
