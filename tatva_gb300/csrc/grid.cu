// Structured-brick linear-elastic Hex8 residual / HVP launches (the stencil and its
// tiling are in tg_grid.cuh).
#include "tg_grid.cuh"

namespace tg {

// pack the per-dof mask into one byte per node
__global__ void pack_node_mask_kernel(const uint8_t* __restrict__ fixed, int64_t n_nodes,
                                      uint8_t* __restrict__ out) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < n_nodes) out[g] = (uint8_t)mask_bits<MASK_DOF>(fixed, g);
}

// Jacobi diagonal of the brick's operator: per dof, the sum of the element matrix's
// diagonal entry over the cells that exist around the node (the element-by-element sum
// of the reference's Hessian diagonal); fixed dofs get 1, the identity rows of the
// Dirichlet-masked operator.
template <class T>
__global__ void grid_diag_kernel(const __grid_constant__ GridCoef<T> P,
                                 const uint8_t* __restrict__ fixed, T* __restrict__ y) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t plane = (int64_t)P.nx * P.ny;
  if (g >= plane * P.nz) return;
  const int x = (int)(g % P.nx), yy = (int)((g / P.nx) % P.ny), z = (int)(g / plane);
  const int bits = fixed ? mask_bits<MASK_DOF>(fixed, g) : 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    T sum = T(0);
#pragma unroll
    for (int o = 0; o < 8; ++o) {  // cell whose corner o is this node
      const int cx = x - (o & 1), cy = yy - ((o >> 1) & 1), cz = z - (o >> 2);
      if (cx >= 0 && cy >= 0 && cz >= 0 && cx < P.nx - 1 && cy < P.ny - 1 && cz < P.nz - 1)
        sum += P.ke[o][o][a][a];
    }
    y[3 * g + a] = (bits >> a & 1) ? T(1) : sum;
  }
}

// Device scalars and partials of the CG dot that a DOT launch produces.
struct GridDot {
  double* scal;    // SCAL_* slots: reads RZ and FLAG, writes PQ, ALPHA, FLAG
  double* part;    // one partial per CTA
  unsigned* ticket;  // zeroed arrival counter (reset by the last CTA)
};

// DOT: the launch also forms p.q of its input p and output q (every dof: the HVP's
// fixed rows are the identity, so they add p^2) -- per CTA in a fixed order, the CTAs'
// partials added by the CTA that arrives last in index order -- and stores
// alpha = rz / (p.q) for the CG update (breakdown flag when p.q <= 0 or not finite).
template <class T, int MODE, int MK, bool DOT>
__global__ void __launch_bounds__(GR_THREADS, sizeof(T) == 4 ? TG_GRID_MINB : 2)
    grid_le_kernel(const __grid_constant__ GridCoef<T> P, const T* __restrict__ in,
                   const T* __restrict__ vin, const uint8_t* __restrict__ fixed,
                   T* __restrict__ y, const GridDot D) {
  using V4 = typename Vec4<T>::type;
  __shared__ V4 sm[2 * GR_PLANE];
  if constexpr (DOT) {
    if (D.scal[SCAL_DONE] != 0.0) return;  // the CG converged earlier in this block
  }
  GridDotAcc<T> dot;
  // boundary CTAs first: they start with the first wave and overlap the interior tiles
  const int b = blockIdx.x;
  if (b < P.n_boundary_ctas) {
    grid_boundary<T, MODE, MK, DOT>(P, (int64_t)b * GR_BNODES, in, vin, fixed, y,
                                      reinterpret_cast<T*>(sm), dot);
  } else if (b < P.n_boundary_ctas + P.n_xface_ctas) {
    grid_xface<T, MODE, MK, DOT>(P, b - P.n_boundary_ctas, in, vin, fixed, y, sm, dot);
  } else {
    grid_interior<T, MODE, MK, DOT>(P, b - P.n_boundary_ctas - P.n_xface_ctas, in, vin, fixed,
                                    y, sm, dot);
  }
  if constexpr (DOT) {
    double v[1] = {dot.value()};
    block_reduce_store<1, GR_THREADS>(v, D.part + blockIdx.x);
    if (!last_cta(D.ticket)) return;
    double w[1] = {0.0};
    for (int i = threadIdx.x; i < (int)gridDim.x; i += GR_THREADS) w[0] += __ldcg(D.part + i);
    __shared__ double out[1];
    block_reduce_store<1, GR_THREADS>(w, out);
    if (threadIdx.x == 0) {
      const double pq = out[0];
      D.scal[SCAL_PQ] = pq;
      const bool bad = !(pq > 0.0) || !isfinite(pq) || D.scal[SCAL_FLAG] != 0.0;
      if (bad) D.scal[SCAL_FLAG] = 1.0;
      D.scal[SCAL_ALPHA] = bad ? 0.0 : D.scal[SCAL_RZ] / pq;
    }
  }
}

template <class T>
static int launch_grid_le_t(const tg_block_plan* plan, int mode, const T* u, const T* v,
                            const uint8_t* fixed, T* y, double mu, double lam,
                            cudaStream_t st) {
  GridCoef<T> P;
  const int64_t n = grid_setup<T>(plan, mu, lam, P);
  if (n < 0) return set_error(TG_ERR_VALUE, "grid too large");
  if (n == 0) return TG_OK;
  if (mode == TG_MODE_DIAG) {
    const int64_t nn = (int64_t)P.nx * P.ny * P.nz;
    grid_diag_kernel<T><<<grid_for(nn, 256), 256, 0, st>>>(P, fixed, y);
    return launch_check("grid diagonal kernel");
  }
  const T* in = (mode == TG_MODE_HVP) ? v : u;
  const unsigned grid = (unsigned)n;
  const GridDot D{nullptr, nullptr, nullptr};
  if (mode == TG_MODE_HVP) {
    if (fixed)
      grid_le_kernel<T, TG_MODE_HVP, MASK_DOF, false><<<grid, GR_THREADS, 0, st>>>(P, in, v, fixed,
                                                                                  y, D);
    else
      grid_le_kernel<T, TG_MODE_HVP, MASK_NONE, false><<<grid, GR_THREADS, 0, st>>>(P, in, v,
                                                                                   fixed, y, D);
  } else if (fixed) {
    grid_le_kernel<T, TG_MODE_RESIDUAL, MASK_DOF, false><<<grid, GR_THREADS, 0, st>>>(
        P, in, v, fixed, y, D);
  } else {
    grid_le_kernel<T, TG_MODE_RESIDUAL, MASK_NONE, false><<<grid, GR_THREADS, 0, st>>>(
        P, in, v, fixed, y, D);
  }
  return launch_check("grid linear-elastic kernel");
}

int64_t grid_cg_ctas(const tg_block_plan* plan) {
  GridCoef<float> P;
  return grid_setup<float>(plan, 1.0, 1.0, P);
}

// The grid CG's handling of fixed dofs: x = b there (the identity rows of the masked
// system) and a zero inverse diagonal, so that z, p and the updates of x and r are
// exactly zero on them and the HVP of p needs no input mask.
template <class T>
__global__ void grid_cg_fixed_kernel(int64_t n_nodes, const uint8_t* __restrict__ nmask,
                                     const T* __restrict__ b, T* __restrict__ x,
                                     T* __restrict__ dinv) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n_nodes) return;
  const int m = nmask[g];
  if (!m) return;
#pragma unroll
  for (int d = 0; d < 3; ++d)
    if (m >> d & 1) {
      x[3 * g + d] = b[3 * g + d];
      dinv[3 * g + d] = T(0);
    }
}

int grid_cg_fixed(int prec, int64_t n_nodes, const uint8_t* nmask, const void* b, void* x,
                  void* dinv, cudaStream_t st) {
  if (prec == TG_F32)
    grid_cg_fixed_kernel<float><<<grid_for(n_nodes, 256), 256, 0, st>>>(
        n_nodes, nmask, (const float*)b, (float*)x, (float*)dinv);
  else
    grid_cg_fixed_kernel<double><<<grid_for(n_nodes, 256), 256, 0, st>>>(
        n_nodes, nmask, (const double*)b, (double*)x, (double*)dinv);
  return launch_check("grid CG fixed dofs");
}

int pack_node_mask(const uint8_t* fixed, int64_t n_nodes, uint8_t* out, cudaStream_t st) {
  pack_node_mask_kernel<<<grid_for(n_nodes, 256), 256, 0, st>>>(fixed, n_nodes, out);
  return launch_check("pack node mask");
}

int launch_grid_hvp_dot(const tg_block_plan* plan, int prec, double mu, double lam,
                        const void* p, const uint8_t* node_mask, void* q, double* scal,
                        double* part, unsigned* ticket, cudaStream_t st) {
  auto go = [&](auto t) -> int {
    using T = decltype(t);
    GridCoef<T> P;
    const int64_t n = grid_setup<T>(plan, mu, lam, P);
    if (n <= 0) return set_error(TG_ERR_VALUE, "grid CG: empty or too large grid");
    const GridDot D{scal, part, ticket};
    const T* in = (const T*)p;
    if (node_mask)  // p is zero on the fixed dofs (grid_cg_fixed): only the rows are masked
      grid_le_kernel<T, TG_MODE_HVP, MASK_NODE_OUT, true><<<(unsigned)n, GR_THREADS, 0, st>>>(
          P, in, in, node_mask, (T*)q, D);
    else
      grid_le_kernel<T, TG_MODE_HVP, MASK_NONE, true><<<(unsigned)n, GR_THREADS, 0, st>>>(
          P, in, in, node_mask, (T*)q, D);
    return launch_check("grid HVP with p.q");
  };
  return prec == TG_F32 ? go(0.f) : go(0.0);
}

int launch_grid_le(const tg_block_plan* plan, int prec, int mode, const void* u, const void* v,
                   const uint8_t* fixed, void* y, double mu, double lam, cudaStream_t st) {
  if (mode != TG_MODE_HVP && mode != TG_MODE_RESIDUAL && mode != TG_MODE_DIAG)
    return TG_ERR_UNSUPPORTED;
  if (plan->grid_nodes[0] < 2 || plan->grid_nodes[1] < 2 || plan->grid_nodes[2] < 2)
    return TG_ERR_UNSUPPORTED;
  if (prec == TG_F32)
    return launch_grid_le_t<float>(plan, mode, (const float*)u, (const float*)v, fixed,
                                   (float*)y, mu, lam, st);
  return launch_grid_le_t<double>(plan, mode, (const double*)u, (const double*)v, fixed,
                                  (double*)y, mu, lam, st);
}

}  // namespace tg
