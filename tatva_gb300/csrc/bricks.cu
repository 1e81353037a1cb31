// Continuous batching of structured-brick solves: many mixed-precision Jacobi-CG
// solves of linear-elastic Hex8 bricks (each one a request of the request loop, i.e.
// the matrix-free solve a reference user runs with the jax.jvp(jax.grad(E)) HVP,
// README.md:93) advance together, one launch per CG step for all of them.
//
// Slots.  A batch holds up to TG_BRICK_MAX_SLOTS solves.  A slot's configuration
// (brick size, stencil coefficients in FP32 and FP64, vector pointers) and its
// control state live in device memory; the host writes them once at admission.
// Every launch takes a table, by value in its parameters, of the slots it covers and
// the first CTA of each: a CTA finds its slot by binary search, so bricks of any
// sizes share one launch and each brick keeps the CTA decomposition it has alone.
//
// Per slot, on the device (the CTA that arrives last in a slot's launch decides):
//   REFINE: x += s d (after an inner solve); r64 = b - A64 x and |r64| in FP64 (the
//           grid stencil with the residual epilogue); converged (|r64| <= rtol |b|)
//           -> DONE, refinement budget spent -> FAILED, else restart the inner solve:
//           r = r64 / |r64| in FP32, d = 0, p = r / diag -> RUN.
//   RUN:    one Jacobi-CG step in FP32: q = A32 p with p.q and alpha (grid stencil),
//           d += alpha p, r -= alpha q with r.z, r.r and beta, p = z + beta p; inner
//           tolerance reached (or the inner budget spent) -> REFINE.
// A step is the refinement launches followed by `iterations` CG steps, for every
// slot in use; a slot whose phase does not match a launch leaves it at once.  The
// host only admits (writes a slot) and polls (reads the per-slot states) between
// steps.  A slot's arithmetic depends on its own data alone -- fixed CTA
// decomposition, fixed-order dot reductions, no atomics on values -- so a solve
// gives the same bits alone and in any mix.
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "tg_dispatch.cuh"
#include "tg_grid.cuh"

namespace tg {
namespace {

constexpr int BR_MAX = TG_BRICK_MAX_SLOTS;
constexpr int PH_FREE = TG_BRICK_FREE, PH_REFINE = TG_BRICK_REFINE, PH_RUN = TG_BRICK_RUN,
              PH_DONE = TG_BRICK_DONE, PH_FAILED = TG_BRICK_FAILED;

struct BrickSlot {
  GridCoef<float> c32;
  GridCoef<double> c64;
  int64_t n_nodes, n_dofs;
  int grid_ctas, chunks;
  const double* b;
  double* x;
  const uint8_t* fixed;  // one byte per dof (or NULL)
  double* r64;
  float *r, *d, *p, *q, *dinv;
  uint8_t* nmask;  // one byte per node, bit a: dof 3 n + a fixed
  double* part;
  double rtol, inner_rtol;
  double tol2_inner;  // of the running inner solve (set at each refinement)
  int max_outer, max_inner;
  // written on the device
  double scal[SCAL_N];
  double s;   // |r64| of the current refinement: the scale of d
  double bn;  // |b|
  unsigned ticket[4];  // arrival counters: HVP, update, residual, restart
  int inner_iters;
};

struct Launch {
  int n;
  int slot[BR_MAX];
  int off[BR_MAX + 1];
};

__device__ __forceinline__ int find_entry(const Launch& L, int b) {
  int lo = 0, hi = L.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (L.off[mid] <= b) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// chunk b of nc of [0, n), starts at multiples of 4
__device__ __forceinline__ void chunk_of(int64_t n, int b, int nc, int64_t& i0, int64_t& i1) {
  const int64_t chunk = (((n + nc - 1) / nc) + 3) & ~int64_t(3);
  i0 = min(n, (int64_t)b * chunk);
  i1 = min(n, i0 + chunk);
}

// true in the CTA of a slot's launch that arrives last (count CTAs); resets the counter
// (thread 0 stored the CTA's partial and alone fences before arriving)
__device__ __forceinline__ bool last_of(unsigned* ticket, int count) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(ticket, 1u);
    last = (t == (unsigned)count - 1u);
    if (last) *ticket = 0u;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

// sum of part[stride * i + k], i < count, k < K, in a fixed order (thread 0 gets it)
template <int K, int NT>
__device__ __forceinline__ void sum_parts(const double* part, int count, double (&out)[K]) {
  double w[K];
#pragma unroll
  for (int k = 0; k < K; ++k) w[k] = 0.0;
  for (int i = threadIdx.x; i < count; i += NT)
#pragma unroll
    for (int k = 0; k < K; ++k) w[k] += __ldcg(part + K * i + k);
  __shared__ double sh[K];
  block_reduce_store<K, NT>(w, sh);
#pragma unroll
  for (int k = 0; k < K; ++k) out[k] = sh[k];
}

// the entry, slot and CTA index of this CTA in the launch (recomputed from the launch
// table where keeping them live would cost registers)
__device__ __forceinline__ void reslot(const Launch& L, int& e, int& s, BrickSlot*& S, int& b,
                                       int& count, BrickSlot* slots) {
  e = find_entry(L, blockIdx.x);
  s = L.slot[e];
  S = slots + s;
  b = blockIdx.x - L.off[e];
  count = L.off[e + 1] - L.off[e];
}

template <class T>
__device__ __forceinline__ void copy_words(T* dst, const T* src) {
  static_assert(sizeof(T) % 4 == 0, "word copy");
  const unsigned* s = reinterpret_cast<const unsigned*>(src);
  unsigned* d = reinterpret_cast<unsigned*>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(T) / 4); i += blockDim.x) d[i] = s[i];
}

__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x;
  v[1] = t.y;
  v[2] = t.z;
  v[3] = t.w;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

// ------------------------------------------------------------------ admission
// node mask, Jacobi inverse diagonal (FP64 sum of the element diagonals of the cells
// around the node, rounded to FP32) and x = 0; on fixed dofs x = b (the identity rows of
// the masked system) and a zero inverse diagonal, so that the inner CG's r, z, p and d
// stay exactly zero there and its HVP masks only the output rows
__global__ void __launch_bounds__(256) brick_admit_kernel(const __grid_constant__ Launch L,
                                                          BrickSlot* __restrict__ slots) {
  const int e = find_entry(L, blockIdx.x);
  BrickSlot* S = slots + L.slot[e];
  const int b = blockIdx.x - L.off[e], count = L.off[e + 1] - L.off[e];
  int64_t j0, j1;
  chunk_of(S->n_nodes, b, count, j0, j1);
  const int nx = S->c64.nx, ny = S->c64.ny, nz = S->c64.nz;
  const uint8_t* fixed = S->fixed;
  for (int64_t g = j0 + threadIdx.x; g < j1; g += blockDim.x) {
    const int bits = fixed ? mask_bits<MASK_DOF>(fixed, g) : 0;
    S->nmask[g] = (uint8_t)bits;
    const int x = (int)(g % nx), y = (int)((g / nx) % ny), z = (int)(g / ((int64_t)nx * ny));
    for (int a = 0; a < 3; ++a) {
      float dv = 0.0f;
      if (!(bits >> a & 1)) {
        double sum = 0.0;
        for (int o = 0; o < 8; ++o) {  // cell whose corner o is this node
          const int cx = x - (o & 1), cy = y - ((o >> 1) & 1), cz = z - (o >> 2);
          if (cx >= 0 && cy >= 0 && cz >= 0 && cx < nx - 1 && cy < ny - 1 && cz < nz - 1)
            sum += S->c64.ke[o][o][a][a];
        }
        dv = 1.0f / (float)sum;
      }
      S->dinv[3 * g + a] = dv;
      S->x[3 * g + a] = (bits >> a & 1) ? S->b[3 * g + a] : 0.0;
    }
  }
}

// ------------------------------------------------------------------ refinement
// x += s d after an inner solve
__global__ void __launch_bounds__(256) brick_xupdate_kernel(const __grid_constant__ Launch L,
                                                            const BrickSlot* __restrict__ slots,
                                                            const tg_brick_state* __restrict__ st) {
  const int e = find_entry(L, blockIdx.x);
  const int s = L.slot[e];
  if (st[s].phase != PH_REFINE || st[s].outer == 0) return;
  const BrickSlot* S = slots + s;
  int64_t i0, i1;
  chunk_of(S->n_dofs, blockIdx.x - L.off[e], L.off[e + 1] - L.off[e], i0, i1);
  const double sc = S->s;
  double* x = S->x;
  const float* d = S->d;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) x[i] += sc * (double)d[i];
}

// r64 = b - A64 x (FP64 grid stencil, Dirichlet rows identity) and |r64|; the slot's
// last CTA decides: DONE, FAILED, or a restart of the inner solve at scale |r64|
__global__ void __launch_bounds__(GR_THREADS, 2)
    brick_resid_kernel(const __grid_constant__ Launch L, BrickSlot* __restrict__ slots,
                       tg_brick_state* __restrict__ st) {
  __shared__ GridCoef<double> P;
  __shared__ double4 sm[2 * GR_PLANE];
  int e = find_entry(L, blockIdx.x);
  int s = L.slot[e];
  if (st[s].phase != PH_REFINE) return;
  BrickSlot* S = slots + s;
  int b = blockIdx.x - L.off[e], count = L.off[e + 1] - L.off[e];
  copy_words(&P, &S->c64);
  __syncthreads();
  GridDotAcc<double> dot;
  {
    const double* x = S->x;
    if (b < P.n_boundary_ctas)
      grid_boundary<double, TG_MODE_HVP, MASK_NODE, true, EPI_RESID>(
          P, (int64_t)b * GR_BNODES, x, x, S->nmask, S->r64, reinterpret_cast<double*>(sm), dot,
          S->b);
    else if (b < P.n_boundary_ctas + P.n_xface_ctas)
      grid_xface<double, TG_MODE_HVP, MASK_NODE, true, EPI_RESID>(
          P, b - P.n_boundary_ctas, x, x, S->nmask, S->r64, sm, dot, S->b);
    else
      grid_interior<double, TG_MODE_HVP, MASK_NODE, true, EPI_RESID>(
          P, b - P.n_boundary_ctas - P.n_xface_ctas, x, x, S->nmask, S->r64, sm, dot, S->b);
  }
  double v[1] = {dot.value()};
  reslot(L, e, s, S, b, count, slots);
  block_reduce_store<1, GR_THREADS>(v, S->part + b);
  if (!last_of(&S->ticket[2], count)) return;
  double rr[1];
  sum_parts<1, GR_THREADS>(S->part, count, rr);
  if (threadIdx.x == 0) {
    const double rn = sqrt(rr[0]);
    tg_brick_state& q = st[s];
    if (q.outer == 0) S->bn = rn;  // x = 0: the residual is b itself
    const double bn = S->bn;
    q.rel_res = bn > 0.0 ? rn / bn : rn;
    if (!isfinite(rn)) {
      q.phase = PH_FAILED;
      q.status = TG_ERR_BREAKDOWN;
    } else if (rn <= S->rtol * bn || bn == 0.0) {
      q.phase = PH_DONE;
      q.status = TG_OK;
    } else if (q.outer >= S->max_outer) {
      q.phase = PH_FAILED;
      q.status = TG_ERR_NOT_CONVERGED;
    } else {
      S->s = rn;
      // the next inner solve reduces |r| only as far as the target still requires
      // (factor-2 margin), at least by inner_rtol
      double itol = 0.5 * S->rtol * bn / rn;
      itol = itol < S->inner_rtol ? S->inner_rtol : (itol > 0.5 ? 0.5 : itol);
      S->tol2_inner = itol * itol;
    }
  }
}

// r = r64 / |r64| (FP32), d = 0, p = z = r dinv, (r.z, r.r); last CTA: scalars, RUN
__global__ void __launch_bounds__(DOT_THREADS)
    brick_restart_kernel(const __grid_constant__ Launch L, BrickSlot* __restrict__ slots,
                         tg_brick_state* __restrict__ st) {
  const int e = find_entry(L, blockIdx.x);
  const int s = L.slot[e];
  if (st[s].phase != PH_REFINE) return;
  BrickSlot* S = slots + s;
  const int b = blockIdx.x - L.off[e], count = L.off[e + 1] - L.off[e];
  int64_t i0, i1;
  chunk_of(S->n_dofs, b, count, i0, i1);
  const double inv_s = 1.0 / S->s;  // one division per thread, not per element
  const double* r64 = S->r64;
  float *r = S->r, *d = S->d, *p = S->p;
  const float* dinv = S->dinv;
  DotAcc<float> a0, a1;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += DOT_THREADS) {
    const float ri = (float)(r64[i] * inv_s);
    const float zi = ri * dinv[i];
    r[i] = ri;
    d[i] = 0.0f;
    p[i] = zi;
    a0.add(ri, zi);
    a1.add(ri, ri);
  }
  double v[2] = {a0.value(), a1.value()};
  block_reduce_store<2, DOT_THREADS>(v, S->part + 2 * b);
  if (!last_of(&S->ticket[3], count)) return;
  double w[2];
  sum_parts<2, DOT_THREADS>(S->part, count, w);
  if (threadIdx.x == 0) {
    S->scal[SCAL_RZ] = w[0];
    S->scal[SCAL_RR] = w[1];
    S->scal[SCAL_FLAG] = 0.0;
    S->inner_iters = 0;
    st[s].outer += 1;
    st[s].phase = PH_RUN;
  }
}

// ------------------------------------------------------------------ one CG step
// q = A32 p (grid stencil, Dirichlet rows identity) with p.q; last CTA: alpha
__global__ void __launch_bounds__(GR_THREADS, TG_GRID_MINB)
    brick_hvp_kernel(const __grid_constant__ Launch L, BrickSlot* __restrict__ slots,
                     tg_brick_state* __restrict__ st) {
  __shared__ GridCoef<float> P;
  __shared__ float4 sm[2 * GR_PLANE];
  int e = find_entry(L, blockIdx.x);
  int s = L.slot[e];
  if (st[s].phase != PH_RUN) return;
  BrickSlot* S = slots + s;
  int b = blockIdx.x - L.off[e], count = L.off[e + 1] - L.off[e];
  copy_words(&P, &S->c32);
  __syncthreads();
  GridDotAcc<float> dot;
  {
    const float* p = S->p;
    if (b < P.n_boundary_ctas)
      grid_boundary<float, TG_MODE_HVP, MASK_NODE_OUT, true>(P, (int64_t)b * GR_BNODES, p, p,
                                                             S->nmask, S->q,
                                                             reinterpret_cast<float*>(sm), dot);
    else if (b < P.n_boundary_ctas + P.n_xface_ctas)
      grid_xface<float, TG_MODE_HVP, MASK_NODE_OUT, true>(P, b - P.n_boundary_ctas, p, p,
                                                          S->nmask, S->q, sm, dot);
    else
      grid_interior<float, TG_MODE_HVP, MASK_NODE_OUT, true>(
          P, b - P.n_boundary_ctas - P.n_xface_ctas, p, p, S->nmask, S->q, sm, dot);
  }
  double v[1] = {dot.value()};
  reslot(L, e, s, S, b, count, slots);  // recomputed: not held in registers across the sweep
  block_reduce_store<1, GR_THREADS>(v, S->part + b);
  if (!last_of(&S->ticket[0], count)) return;
  double w[1];
  sum_parts<1, GR_THREADS>(S->part, count, w);
  if (threadIdx.x == 0) {
    const double pq = w[0];
    S->scal[SCAL_PQ] = pq;
    if (!(pq > 0.0) || !isfinite(pq)) {
      S->scal[SCAL_ALPHA] = 0.0;
      st[s].phase = PH_FAILED;
      st[s].status = TG_ERR_BREAKDOWN;
    } else {
      S->scal[SCAL_ALPHA] = S->scal[SCAL_RZ] / pq;
    }
  }
}

// d += alpha p; r -= alpha q; (r.z, r.r) with z = r dinv; last CTA: beta, rz, and the
// inner stopping test (|r| <= inner tolerance or the inner budget spent -> REFINE)
__global__ void __launch_bounds__(DOT_THREADS)
    brick_update_kernel(const __grid_constant__ Launch L, BrickSlot* __restrict__ slots,
                        tg_brick_state* __restrict__ st) {
  const int e = find_entry(L, blockIdx.x);
  const int s = L.slot[e];
  if (st[s].phase != PH_RUN) return;
  BrickSlot* S = slots + s;
  const int b = blockIdx.x - L.off[e], count = L.off[e + 1] - L.off[e];
  int64_t i0, i1;
  chunk_of(S->n_dofs, b, count, i0, i1);
  const int64_t iv = i0 + ((i1 - i0) & ~int64_t(3));
  const float alpha = (float)S->scal[SCAL_ALPHA];
  float *d = S->d, *r = S->r;
  const float *p = S->p, *q = S->q, *dinv = S->dinv;
  DotAcc<float> a0, a1;
#pragma unroll 2
  for (int64_t i = i0 + 4 * threadIdx.x; i < iv; i += 4 * DOT_THREADS) {
    float dd[4], pp[4], rr[4], qq[4], di[4];
    ld4(d + i, dd);
    ld4(p + i, pp);
    ld4(r + i, rr);
    ld4(q + i, qq);
    ld4(dinv + i, di);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      dd[k] += alpha * pp[k];
      rr[k] = rr[k] - alpha * qq[k];
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) a0.add(rr[k], rr[k] * di[k]);
#pragma unroll
    for (int k = 0; k < 4; ++k) a1.add(rr[k], rr[k]);
    st4(d + i, dd);
    st4(r + i, rr);
  }
  for (int64_t i = iv + threadIdx.x; i < i1; i += DOT_THREADS) {
    d[i] += alpha * p[i];
    const float ri = r[i] - alpha * q[i];
    r[i] = ri;
    a0.add(ri, ri * dinv[i]);
    a1.add(ri, ri);
  }
  double v[2] = {a0.value(), a1.value()};
  block_reduce_store<2, DOT_THREADS>(v, S->part + 2 * b);
  if (!last_of(&S->ticket[1], count)) return;
  double w[2];
  sum_parts<2, DOT_THREADS>(S->part, count, w);
  if (threadIdx.x == 0) {
    const double rz_new = w[0], rr = w[1];
    tg_brick_state& o = st[s];
    o.iterations += 1;
    S->inner_iters += 1;
    S->scal[SCAL_RR] = rr;
    if (!isfinite(rz_new) || !isfinite(rr)) {
      o.phase = PH_FAILED;
      o.status = TG_ERR_BREAKDOWN;
    } else {
      S->scal[SCAL_BETA] = rz_new / S->scal[SCAL_RZ];
      S->scal[SCAL_RZ] = rz_new;
      if (rr <= S->tol2_inner || S->inner_iters >= S->max_inner) o.phase = PH_REFINE;
    }
  }
}

// p = r dinv + beta p
__global__ void __launch_bounds__(DOT_THREADS) brick_p_kernel(const __grid_constant__ Launch L,
                                                              const BrickSlot* __restrict__ slots,
                                                              const tg_brick_state* __restrict__ st) {
  const int e = find_entry(L, blockIdx.x);
  const int s = L.slot[e];
  if (st[s].phase != PH_RUN) return;
  const BrickSlot* S = slots + s;
  int64_t i0, i1;
  chunk_of(S->n_dofs, blockIdx.x - L.off[e], L.off[e + 1] - L.off[e], i0, i1);
  const int64_t iv = i0 + ((i1 - i0) & ~int64_t(3));
  const float beta = (float)S->scal[SCAL_BETA];
  const float *r = S->r, *dinv = S->dinv;
  float* p = S->p;
  for (int64_t i = i0 + 4 * threadIdx.x; i < iv; i += 4 * DOT_THREADS) {
    float rr[4], di[4], pp[4];
    ld4(r + i, rr);
    ld4(dinv + i, di);
    ld4(p + i, pp);
#pragma unroll
    for (int k = 0; k < 4; ++k) pp[k] = rr[k] * di[k] + beta * pp[k];
    st4(p + i, pp);
  }
  for (int64_t i = iv + threadIdx.x; i < i1; i += DOT_THREADS) p[i] = r[i] * dinv[i] + beta * p[i];
}

// ------------------------------------------------------------------ host
int brick_chunks(int64_t n_dofs) {
  const int64_t c = (n_dofs + 8191) / 8192;
  return (int)(c < 1 ? 1 : (c > DOT_CHUNKS ? DOT_CHUNKS : c));
}

int64_t brick_grid_ctas(const int32_t nodes[3]) {
  GridCoef<float> P;
  const double h[3] = {1.0, 1.0, 1.0};
  return grid_setup_dims<float>(nodes, h, 1.0, 1.0, P, true);
}

size_t brick_part_doubles(const int32_t nodes[3]) {
  const int64_t n = 3 * (int64_t)nodes[0] * nodes[1] * nodes[2];
  const int64_t g = brick_grid_ctas(nodes), c = 2 * (int64_t)brick_chunks(n);
  return (size_t)(g > c ? g : c);
}

inline size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace
}  // namespace tg

using namespace tg;

struct tg_brick_batch {
  int device = 0;
  tg::BrickSlot* d_slots = nullptr;
  tg_brick_state* d_state = nullptr;
  tg_brick_state* h_state = nullptr;  // pinned
  bool used[TG_BRICK_MAX_SLOTS] = {};
  int grid_ctas[TG_BRICK_MAX_SLOTS] = {};
  int chunks[TG_BRICK_MAX_SLOTS] = {};
  std::vector<int> admitted;
  // the last step's launches as a CUDA graph, replayed while the slots in use and the
  // step length stay the same (a new admission or a release changes the tables)
  cudaGraphExec_t exec = nullptr;
  std::vector<int> exec_slots;
  int exec_iterations = -1;
  bool exec_stale = true;  // set by every admission (a slot may come back with another size)
};

extern "C" size_t tg_brick_workspace_bytes(const int32_t nodes[3]) {
  if (!nodes || nodes[0] < 2 || nodes[1] < 2 || nodes[2] < 2) return 0;
  const int64_t nn = (int64_t)nodes[0] * nodes[1] * nodes[2], n = 3 * nn;
  return al256((size_t)n * 8) + 5 * al256((size_t)n * 4) + al256((size_t)nn) +
         al256(brick_part_doubles(nodes) * sizeof(double));
}

extern "C" int tg_brick_batch_create(tg_brick_batch** out) {
  TG_TRY(check_ptr(out, "out"));
  *out = nullptr;
  auto* bt = new (std::nothrow) tg_brick_batch();
  if (!bt) return set_error(TG_ERR_VALUE, "tg_brick_batch_create: out of host memory");
  int rc = cuda_check(cudaGetDevice(&bt->device), "brick batch: device");
  if (rc == TG_OK)
    rc = cuda_check(cudaMalloc(&bt->d_slots, BR_MAX * sizeof(BrickSlot)), "brick batch: slots");
  if (rc == TG_OK)
    rc = cuda_check(cudaMalloc(&bt->d_state, BR_MAX * sizeof(tg_brick_state)), "brick batch: states");
  if (rc == TG_OK)
    rc = cuda_check(cudaMallocHost(&bt->h_state, BR_MAX * sizeof(tg_brick_state)), "brick batch: host states");
  if (rc == TG_OK)
    rc = cuda_check(cudaMemset(bt->d_state, 0, BR_MAX * sizeof(tg_brick_state)), "brick batch: clear");
  if (rc != TG_OK) {
    tg_brick_batch_destroy(bt);
    return rc;
  }
  *out = bt;
  return TG_OK;
}

extern "C" void tg_brick_batch_destroy(tg_brick_batch* bt) {
  if (!bt) return;
  if (bt->d_slots) cudaFree(bt->d_slots);
  if (bt->d_state) cudaFree(bt->d_state);
  if (bt->h_state) cudaFreeHost(bt->h_state);
  if (bt->exec) cudaGraphExecDestroy(bt->exec);
  delete bt;
}

extern "C" int tg_brick_admit(tg_brick_batch* bt, const tg_brick_request* req, void* stream,
                              int* slot_out) {
  TG_TRY(check_ptr(bt, "batch"));
  TG_TRY(check_ptr(req, "request"));
  TG_TRY(check_ptr(slot_out, "slot_out"));
  *slot_out = -1;
  TG_TRY(check_ptr(req->b, "b"));
  TG_TRY(check_ptr(req->x, "x"));
  TG_TRY(check_ptr(req->workspace, "workspace"));
  const int32_t* nd = req->nodes;
  if (nd[0] < 2 || nd[1] < 2 || nd[2] < 2)
    return set_error(TG_ERR_VALUE, "tg_brick_admit: a brick needs at least 2 nodes per axis");
  if (!(req->h[0] > 0.0 && req->h[1] > 0.0 && req->h[2] > 0.0))
    return set_error(TG_ERR_VALUE, "tg_brick_admit: spacings must be positive");
  if (!(req->rtol > 0.0) || !(req->inner_rtol > 0.0) || req->max_outer < 0 || req->max_inner < 1)
    return set_error(TG_ERR_VALUE, "tg_brick_admit: bad tolerances or budgets");
  const size_t need = tg_brick_workspace_bytes(nd);
  if (req->workspace_bytes < need)
    return set_error(TG_ERR_WORKSPACE, "tg_brick_admit: workspace of %zu bytes, %zu needed",
                     req->workspace_bytes, need);
  if (((uintptr_t)req->workspace & 255u) != 0)
    return set_error(TG_ERR_VALUE, "tg_brick_admit: workspace must be 256-byte aligned");
  if (((uintptr_t)req->b & 7u) != 0 || ((uintptr_t)req->x & 7u) != 0)
    return set_error(TG_ERR_VALUE, "tg_brick_admit: b and x must be 8-byte aligned");
  int dev = -1;
  TG_TRY(cuda_check(cudaGetDevice(&dev), "brick admit: device"));
  if (dev != bt->device)
    return set_error(TG_ERR_VALUE, "tg_brick_admit: the batch belongs to device %d", bt->device);
  int s = -1;
  for (int i = 0; i < BR_MAX; ++i)
    if (!bt->used[i]) {
      s = i;
      break;
    }
  if (s < 0) return set_error(TG_ERR_VALUE, "tg_brick_admit: no free slot");

  BrickSlot h;
  std::memset(&h, 0, sizeof(h));
  const int64_t g32 = grid_setup_dims<float>(nd, req->h, req->mu, req->lam, h.c32, true);
  const int64_t g64 = grid_setup_dims<double>(nd, req->h, req->mu, req->lam, h.c64, true);
  if (g32 <= 0 || g64 != g32 || g32 > 0x3fffffff)
    return set_error(TG_ERR_VALUE, "tg_brick_admit: brick too large");
  h.n_nodes = (int64_t)nd[0] * nd[1] * nd[2];
  h.n_dofs = 3 * h.n_nodes;
  h.grid_ctas = (int)g32;
  h.chunks = brick_chunks(h.n_dofs);
  h.b = req->b;
  h.x = req->x;
  h.fixed = req->fixed;
  char* w = (char*)req->workspace;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    void* p = w + off;
    off += al256(bytes);
    return p;
  };
  h.r64 = (double*)take((size_t)h.n_dofs * 8);
  h.r = (float*)take((size_t)h.n_dofs * 4);
  h.d = (float*)take((size_t)h.n_dofs * 4);
  h.p = (float*)take((size_t)h.n_dofs * 4);
  h.q = (float*)take((size_t)h.n_dofs * 4);
  h.dinv = (float*)take((size_t)h.n_dofs * 4);
  h.nmask = (uint8_t*)take((size_t)h.n_nodes);
  h.part = (double*)take(brick_part_doubles(nd) * sizeof(double));
  h.rtol = req->rtol;
  h.inner_rtol = req->inner_rtol;
  h.tol2_inner = req->inner_rtol * req->inner_rtol;
  h.max_outer = req->max_outer;
  h.max_inner = req->max_inner;
  tg_brick_state q;
  std::memset(&q, 0, sizeof(q));
  q.phase = PH_REFINE;
  cudaStream_t st = as_stream(stream);
  // ordered after every launch already queued on the stream that reads this slot
  TG_TRY(cuda_check(cudaMemcpyAsync(bt->d_slots + s, &h, sizeof(h), cudaMemcpyHostToDevice, st),
                    "brick admit: slot"));
  TG_TRY(cuda_check(cudaMemcpyAsync(bt->d_state + s, &q, sizeof(q), cudaMemcpyHostToDevice, st),
                    "brick admit: state"));
  bt->used[s] = true;
  bt->grid_ctas[s] = h.grid_ctas;
  bt->chunks[s] = h.chunks;
  bt->admitted.push_back(s);
  bt->exec_stale = true;
  *slot_out = s;
  return TG_OK;
}

namespace {
// launch table over the given slots with per-slot CTA counts
Launch make_launch(const std::vector<int>& slots, const int* ctas, int64_t* total) {
  Launch L;
  std::memset(&L, 0, sizeof(L));
  L.n = (int)slots.size();
  int64_t t = 0;
  for (int i = 0; i < L.n; ++i) {
    L.slot[i] = slots[i];
    L.off[i] = (int)t;
    t += ctas[slots[i]];
  }
  L.off[L.n] = (int)t;
  *total = t;
  return L;
}
}  // namespace

extern "C" int tg_brick_step(tg_brick_batch* bt, int iterations, void* stream) {
  TG_TRY(check_ptr(bt, "batch"));
  if (iterations < 0) return set_error(TG_ERR_VALUE, "tg_brick_step: iterations < 0");
  std::vector<int> active;
  for (int i = 0; i < BR_MAX; ++i)
    if (bt->used[i]) active.push_back(i);
  if (active.empty()) return TG_OK;
  cudaStream_t st = as_stream(stream);
  int64_t ng = 0, nc = 0, na = 0;
  const Launch Lg = make_launch(active, bt->grid_ctas, &ng);
  const Launch Lc = make_launch(active, bt->chunks, &nc);
  if (ng > 0x7fffffff) return set_error(TG_ERR_VALUE, "tg_brick_step: too many CTAs");
  if (!bt->admitted.empty()) {
    const Launch La = make_launch(bt->admitted, bt->chunks, &na);
    brick_admit_kernel<<<(unsigned)na, 256, 0, st>>>(La, bt->d_slots);
    bt->admitted.clear();
    TG_TRY(launch_check("tg_brick_step: admission"));
  }
  auto enqueue = [&]() {
    brick_xupdate_kernel<<<(unsigned)nc, 256, 0, st>>>(Lc, bt->d_slots, bt->d_state);
    brick_resid_kernel<<<(unsigned)ng, GR_THREADS, 0, st>>>(Lg, bt->d_slots, bt->d_state);
    brick_restart_kernel<<<(unsigned)nc, DOT_THREADS, 0, st>>>(Lc, bt->d_slots, bt->d_state);
    for (int it = 0; it < iterations; ++it) {
      brick_hvp_kernel<<<(unsigned)ng, GR_THREADS, 0, st>>>(Lg, bt->d_slots, bt->d_state);
      brick_update_kernel<<<(unsigned)nc, DOT_THREADS, 0, st>>>(Lc, bt->d_slots, bt->d_state);
      brick_p_kernel<<<(unsigned)nc, DOT_THREADS, 0, st>>>(Lc, bt->d_slots, bt->d_state);
    }
  };
  const bool can_capture = st != nullptr && st != cudaStreamLegacy && st != cudaStreamPerThread;
  if (!can_capture) {
    enqueue();
    return launch_check("tg_brick_step");
  }
  if (!bt->exec || bt->exec_stale || bt->exec_slots != active ||
      bt->exec_iterations != iterations) {
    cudaGraph_t graph;
    TG_TRY(cuda_check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal),
                      "brick step: capture"));
    enqueue();
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ee = cudaStreamEndCapture(st, &graph);
    TG_TRY(cuda_check(le, "brick step: launches"));
    TG_TRY(cuda_check(ee, "brick step: end capture"));
    bool updated = false;
    if (bt->exec) {  // same number of launches: update the parameters in place
      cudaGraphExecUpdateResultInfo info;
      updated = bt->exec_iterations == iterations &&
                cudaGraphExecUpdate(bt->exec, graph, &info) == cudaSuccess;
      if (!updated) {
        cudaGetLastError();
        cudaGraphExecDestroy(bt->exec);
        bt->exec = nullptr;
      }
    }
    int rc = TG_OK;
    if (!updated) rc = cuda_check(cudaGraphInstantiate(&bt->exec, graph, 0), "brick step: instantiate");
    cudaGraphDestroy(graph);
    if (rc != TG_OK) {
      bt->exec = nullptr;
      return rc;
    }
    bt->exec_slots = active;
    bt->exec_iterations = iterations;
    bt->exec_stale = false;
  }
  return cuda_check(cudaGraphLaunch(bt->exec, st), "brick step: graph launch");
}

extern "C" int tg_brick_poll(tg_brick_batch* bt, tg_brick_state* out, int n_out, void* stream) {
  TG_TRY(check_ptr(bt, "batch"));
  TG_TRY(check_ptr(out, "out"));
  if (n_out < BR_MAX) return set_error(TG_ERR_VALUE, "tg_brick_poll: out needs %d entries", BR_MAX);
  cudaStream_t st = as_stream(stream);
  TG_TRY(cuda_check(cudaMemcpyAsync(bt->h_state, bt->d_state, BR_MAX * sizeof(tg_brick_state),
                                    cudaMemcpyDeviceToHost, st),
                    "brick poll: read"));
  TG_TRY(cuda_check(cudaStreamSynchronize(st), "brick poll: synchronize"));
  for (int i = 0; i < BR_MAX; ++i) {
    if (!bt->used[i]) {
      std::memset(out + i, 0, sizeof(tg_brick_state));
      out[i].phase = PH_FREE;
      continue;
    }
    out[i] = bt->h_state[i];
    if (out[i].phase == PH_DONE || out[i].phase == PH_FAILED) bt->used[i] = false;
  }
  return TG_OK;
}
