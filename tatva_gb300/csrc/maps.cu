// Operator maps: eval / grad / integration weights / integrate / deterministic sums /
// gather and the reverse-mode transposes (K1-K3).
//
// Reference semantics (tatva/operator.py):
//   eval                     :358-377  out[e,q,v]   = sum_a N_a(xi_q) u[conn[e,a], v]
//   grad                     :379-397  out[e,q,v,d] = sum_a dN_a/dx_d u[conn[e,a], v]
//   get_integration_weights  :172-192  out[e,q]     = detJ(e,q) * w_q
//   _integrate_quad_array    :344-356  out[e,v]     = sum_q quad[e,q,v] w[e,q]
//   integrate                :307-319  sum over elements
#include "tg_common.cuh"
#include "tg_dispatch.cuh"

namespace tg {

constexpr int TPB_T = 256;

// ------------------------------------------------------------------ eval
template <int ET, class T>
__global__ void eval_kernel(const T* __restrict__ nodal, int V, const int32_t* __restrict__ conn,
                            int64_t n_elems, T* __restrict__ out) {
  using E = Elem<ET>;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = n_elems * E::Q * V;
  if (tid >= total) return;
  const int v = (int)(tid % V);
  const int64_t eq = tid / V;
  const int q = (int)(eq % E::Q);
  const int64_t e = eq / E::Q;
  T acc = T(0);
#pragma unroll
  for (int a = 0; a < E::NN; ++a) {
    const int64_t n = __ldg(conn + e * E::NN + a);
    acc += E::template N<T>(q, a) * nodal[n * V + v];
  }
  out[tid] = acc;
}

// ------------------------------------------------------------------ gather coords
template <int ET, class T>
__device__ __forceinline__ void gather_coords(const T* __restrict__ coords,
                                              const int32_t* __restrict__ conn, int64_t e,
                                              T (&X)[Elem<ET>::NN][Elem<ET>::D],
                                              int (&nid)[Elem<ET>::NN]) {
  using E = Elem<ET>;
#pragma unroll
  for (int a = 0; a < E::NN; ++a) {
    nid[a] = __ldg(conn + e * E::NN + a);
#pragma unroll
    for (int d = 0; d < E::D; ++d) X[a][d] = coords[(int64_t)nid[a] * E::D + d];
  }
}

// ------------------------------------------------------------------ grad
template <int ET, class T>
__global__ void grad_kernel(const T* __restrict__ nodal, const T* __restrict__ coords, int V,
                            const int32_t* __restrict__ conn, int64_t n_elems,
                            T* __restrict__ out) {
  using E = Elem<ET>;
  constexpr int NN = E::NN, D = E::D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  T X[NN][D];
  int nid[NN];
  gather_coords<ET, T>(coords, conn, e, X, nid);
  if (V <= 3) {  // the element's values loaded once, not once per quadrature point
    T U[NN][3];
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
      for (int v = 0; v < 3; ++v) U[a][v] = v < V ? nodal[(int64_t)nid[a] * V + v] : T(0);
#pragma unroll
    for (int q = 0; q < E::Q; ++q) {
      T G[NN][D];
      qp_geometry<ET, T>(q, X, G);
      T* o = out + ((e * E::Q + q) * V) * D;
#pragma unroll
      for (int v = 0; v < 3; ++v) {
        if (v >= V) break;
        T g[D];
#pragma unroll
        for (int d = 0; d < D; ++d) g[d] = T(0);
#pragma unroll
        for (int a = 0; a < NN; ++a)
#pragma unroll
          for (int d = 0; d < D; ++d) g[d] += G[a][d] * U[a][v];
#pragma unroll
        for (int d = 0; d < D; ++d) o[v * D + d] = g[d];
      }
    }
    return;
  }
#pragma unroll
  for (int q = 0; q < E::Q; ++q) {
    T G[NN][D];
    qp_geometry<ET, T>(q, X, G);
    T* o = out + ((e * E::Q + q) * V) * D;
    for (int v = 0; v < V; ++v) {
      T g[D];
#pragma unroll
      for (int d = 0; d < D; ++d) g[d] = T(0);
#pragma unroll
      for (int a = 0; a < NN; ++a) {
        const T u = nodal[(int64_t)nid[a] * V + v];
#pragma unroll
        for (int d = 0; d < D; ++d) g[d] += G[a][d] * u;
      }
#pragma unroll
      for (int d = 0; d < D; ++d) o[v * D + d] = g[d];
    }
  }
}

// ------------------------------------------------------------------ Hex8 modal form
// The trilinear map of a Hex8 cell is x(xi) = sum_m c_m xi^m over the eight monomials
// m of {1, xi1, xi2, xi1 xi2, xi3, xi1 xi3, xi2 xi3, xi1 xi2 xi3} (bit k of m: factor
// xi_{k+1}), with c_m = 1/8 sum_a (prod_{k in m} s_{a,k}) x_a for the corner signs
// s_{a,k} of tatva/element/base.py:478-491.  Then
//   dx/dxi1 = c_1 + c_3 xi2 + c_5 xi3 + c_7 xi2 xi3   (and cyclically),
// so J at a quadrature point costs 3 FMAs per entry instead of an 8-term sum, and the
// same transform of the nodal values gives their reference gradient.  The transform
// is a 3-stage butterfly over the corners in binary order (reference node a is binary
// corner {0,1,3,2,4,5,7,6}[a]).  GB300's FP64 pipe bounds these FP64 maps, so the
// operation count is what sets their time.  A parallelepiped cell has c_3 = c_5 =
// c_6 = c_7 = 0 exactly: its J is the same at every point and is inverted once
// (bitwise what the per-point evaluation gives).
__host__ __device__ constexpr int hex_bin(int a) { return a ^ ((a >> 1) & 1); }

// corners (reference order) -> modes c_m, C components, in place
template <class T, int C>
__device__ __forceinline__ void hex_modes(T (&v)[8][C]) {
  T w[8][C];
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int c = 0; c < C; ++c) w[hex_bin(a)][c] = v[a][c];
#pragma unroll
  for (int k = 1; k < 8; k <<= 1)
#pragma unroll
    for (int b = 0; b < 8; ++b)
      if (!(b & k))
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const T x = w[b][c], y = w[b | k][c];
          w[b][c] = x + y;
          w[b | k][c] = y - x;
        }
#pragma unroll
  for (int m = 0; m < 8; ++m)
#pragma unroll
    for (int c = 0; c < C; ++c) v[m][c] = w[m][c] * T(0.125);
}

// adjoint of hex_modes: mode weights -> corner (reference order) contributions
template <class T, int C>
__device__ __forceinline__ void hex_modes_adjoint(T (&w)[8][C], T (&out)[8][C]) {
#pragma unroll
  for (int k = 1; k < 8; k <<= 1)
#pragma unroll
    for (int b = 0; b < 8; ++b)
      if (!(b & k))
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const T x = w[b][c], y = w[b | k][c];
          w[b][c] = x - y;
          w[b | k][c] = x + y;
        }
#pragma unroll
  for (int a = 0; a < 8; ++a)
#pragma unroll
    for (int c = 0; c < C; ++c) out[a][c] = w[hex_bin(a)][c] * T(0.125);
}

// d/dxi_i of the modal field at xi: D[i][c]
template <class T, int C>
__device__ __forceinline__ void hex_dxi(const T (&m)[8][C], const T (&xi)[3], T (&D)[3][C]) {
  const T x12 = xi[0] * xi[1], x13 = xi[0] * xi[2], x23 = xi[1] * xi[2];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    D[0][c] = fma(m[7][c], x23, fma(m[5][c], xi[2], fma(m[3][c], xi[1], m[1][c])));
    D[1][c] = fma(m[7][c], x13, fma(m[6][c], xi[2], fma(m[3][c], xi[0], m[2][c])));
    D[2][c] = fma(m[7][c], x12, fma(m[6][c], xi[1], fma(m[5][c], xi[0], m[4][c])));
  }
}

template <class T>
__device__ __forceinline__ void hex_qp(int q, T (&xi)[3]) {
  const T g = T(HEX_GAUSS);
#pragma unroll
  for (int i = 0; i < 3; ++i) xi[i] = Elem<TG_HEX8>::s(q, i) > 0 ? g : -g;
}

template <class T>
__device__ __forceinline__ bool hex_affine(const T (&mx)[8][3]) {
  bool z = true;
#pragma unroll
  for (int c = 0; c < 3; ++c)
    z = z && mx[3][c] == T(0) && mx[5][c] == T(0) && mx[6][c] == T(0) && mx[7][c] == T(0);
  return z;
}

// out[e, q, v, d] = sum_i Ji[d][i] dU_v/dxi_i
template <class T>
__global__ void __launch_bounds__(128) hex_grad_kernel(const T* __restrict__ nodal,
                                                       const T* __restrict__ coords, int V,
                                                       const int32_t* __restrict__ conn,
                                                       int64_t n_elems, T* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  T mx[8][3];
  int nid[8];
  gather_coords<TG_HEX8, T>(coords, conn, e, mx, nid);
  hex_modes<T, 3>(mx);
  const bool affine = hex_affine(mx);
  T Ji[3][3];
  if (affine) {
    T xi[3] = {T(0), T(0), T(0)}, J[3][3];
    hex_dxi<T, 3>(mx, xi, J);
    inv3(J, Ji);
  }
  for (int v0 = 0; v0 < V; v0 += 3) {
    const int nv = (V - v0) < 3 ? (V - v0) : 3;
    T mu[8][3];
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int k = 0; k < 3; ++k) mu[a][k] = k < nv ? nodal[(int64_t)nid[a] * V + v0 + k] : T(0);
    hex_modes<T, 3>(mu);
#pragma unroll 1
    for (int q = 0; q < 8; ++q) {
      T xi[3];
      hex_qp<T>(q, xi);
      if (!affine) {
        T J[3][3];
        hex_dxi<T, 3>(mx, xi, J);
        inv3(J, Ji);
      }
      T H[3][3];  // H[i][k] = dU_k/dxi_i
      hex_dxi<T, 3>(mu, xi, H);
      T* o = out + ((e * 8 + q) * V + v0) * 3;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k < nv) {
#pragma unroll
          for (int d = 0; d < 3; ++d)
            o[k * 3 + d] = fma(Ji[d][2], H[2][k], fma(Ji[d][1], H[1][k], Ji[d][0] * H[0][k]));
        }
      }
    }
  }
}

// contrib[e, a, v] = sum_q sum_d dN_a/dx_d flux[e, q, v, d]
//                 = sum_q sum_i dN_a/dxi_i F_i,  F_i = sum_d Ji[d][i] flux[e, q, v, d],
// accumulated in the modal basis and returned to the corners by the adjoint transform
template <class T>
__global__ void __launch_bounds__(128)
    hex_grad_transpose_elem_kernel(const T* __restrict__ flux, const T* __restrict__ coords,
                                   int V, const int32_t* __restrict__ conn, int64_t n_elems,
                                   T* __restrict__ contrib) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  T mx[8][3];
  int nid[8];
  gather_coords<TG_HEX8, T>(coords, conn, e, mx, nid);
  hex_modes<T, 3>(mx);
  const bool affine = hex_affine(mx);
  T Ji[3][3];
  if (affine) {
    T xi[3] = {T(0), T(0), T(0)}, J[3][3];
    hex_dxi<T, 3>(mx, xi, J);
    inv3(J, Ji);
  }
  for (int v0 = 0; v0 < V; v0 += 3) {
    const int nv = (V - v0) < 3 ? (V - v0) : 3;
    T w[8][3];
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
      for (int k = 0; k < 3; ++k) w[m][k] = T(0);
#pragma unroll 1
    for (int q = 0; q < 8; ++q) {
      T xi[3];
      hex_qp<T>(q, xi);
      if (!affine) {
        T J[3][3];
        hex_dxi<T, 3>(mx, xi, J);
        inv3(J, Ji);
      }
      const T* f = flux + ((e * 8 + q) * V + v0) * 3;
      const T x12 = xi[0] * xi[1], x13 = xi[0] * xi[2], x23 = xi[1] * xi[2];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k < nv) {
          const T f0 = f[k * 3], f1 = f[k * 3 + 1], f2 = f[k * 3 + 2];
          T F[3];
#pragma unroll
          for (int i = 0; i < 3; ++i) F[i] = fma(Ji[2][i], f2, fma(Ji[1][i], f1, Ji[0][i] * f0));
          // adjoint of hex_dxi
          w[1][k] += F[0];
          w[2][k] += F[1];
          w[4][k] += F[2];
          w[3][k] = fma(F[0], xi[1], fma(F[1], xi[0], w[3][k]));
          w[5][k] = fma(F[0], xi[2], fma(F[2], xi[0], w[5][k]));
          w[6][k] = fma(F[1], xi[2], fma(F[2], xi[1], w[6][k]));
          w[7][k] = fma(F[0], x23, fma(F[1], x13, fma(F[2], x12, w[7][k])));
        }
      }
    }
    T c[8][3];
    hex_modes_adjoint<T, 3>(w, c);
#pragma unroll
    for (int a = 0; a < 8; ++a)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (k < nv) contrib[(e * 8 + a) * V + v0 + k] = c[a][k];
  }
}

// ------------------------------------------------------------------ weights
template <int ET, class T>
__global__ void weights_kernel(const T* __restrict__ coords, const int32_t* __restrict__ conn,
                               int64_t n_elems, T* __restrict__ out) {
  using E = Elem<ET>;
  constexpr int NN = E::NN, D = E::D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  T X[NN][D];
  int nid[NN];
  gather_coords<ET, T>(coords, conn, e, X, nid);
#pragma unroll
  for (int q = 0; q < E::Q; ++q) {
    T G[NN][D];
    const T det = qp_geometry<ET, T>(q, X, G);
    out[e * E::Q + q] = det * E::template w<T>(q);
  }
}

// ------------------------------------------------------------------ integrate quad array
template <class T>
__global__ void integrate_quad_kernel(const T* __restrict__ quad, const T* __restrict__ w,
                                      int64_t n_elems, int Q, int V, T* __restrict__ out) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n_elems * V) return;
  const int v = (int)(tid % V);
  const int64_t e = tid / V;
  T acc = T(0);
  for (int q = 0; q < Q; ++q) acc += quad[(e * Q + q) * V + v] * w[e * Q + q];
  out[tid] = acc;
}

// ------------------------------------------------------------------ deterministic row sums
// Stage 1: a fixed number of chunks (independent of the GPU), each summed by one
// block in a fixed strided + tree order, accumulated in FP64.  Stage 2: one block
// sums the chunk partials in a fixed tree order.
constexpr int SUM_CHUNKS = 512;
constexpr int SUM_THREADS = 256;

template <class T>
__global__ void __launch_bounds__(SUM_THREADS)
    rowsum_stage1(const T* __restrict__ in, int64_t n_rows, int V, double* __restrict__ part) {
  __shared__ double sh[SUM_THREADS];
  const int64_t chunk = (n_rows + SUM_CHUNKS - 1) / SUM_CHUNKS;
  const int64_t r0 = blockIdx.x * chunk;
  const int64_t r1 = min(n_rows, r0 + chunk);
  for (int v = 0; v < V; ++v) {
    double acc = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += SUM_THREADS) acc += (double)in[r * V + v];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = SUM_THREADS / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x * V + v] = sh[0];
    __syncthreads();
  }
}

template <class T>
__global__ void __launch_bounds__(SUM_THREADS)
    rowsum_stage2(const double* __restrict__ part, int V, T* __restrict__ out) {
  __shared__ double sh[SUM_THREADS];
  for (int v = 0; v < V; ++v) {
    double acc = 0.0;
    for (int b = threadIdx.x; b < SUM_CHUNKS; b += SUM_THREADS) acc += part[b * V + v];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int s = SUM_THREADS / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[v] = (T)sh[0];
    __syncthreads();
  }
}

// ------------------------------------------------------------------ gather
template <class T>
__global__ void gather_nodal_kernel(const T* __restrict__ nodal, int V,
                                    const int32_t* __restrict__ conn, int64_t n_entries,
                                    T* __restrict__ out) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n_entries * V) return;
  const int v = (int)(tid % V);
  const int64_t k = tid / V;
  out[tid] = nodal[(int64_t)__ldg(conn + k) * V + v];
}

// ------------------------------------------------------------------ transposes
// Phase 1: element e's contribution to each of its nodes, c[e][a][v] = sum_q sum_d
// dNdX[e,q,d,a] flux[e,q,v,d], with the geometry of each quadrature point formed once
// (values in groups of up to 3 per pass, so that the sums stay in registers).
template <int ET, class T>
__global__ void grad_transpose_elem_kernel(const T* __restrict__ flux, const T* __restrict__ coords,
                                           int V, const int32_t* __restrict__ conn,
                                           int64_t n_elems, T* __restrict__ contrib) {
  using E = Elem<ET>;
  constexpr int NN = E::NN, D = E::D;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  T X[NN][D];
  int nid[NN];
  gather_coords<ET, T>(coords, conn, e, X, nid);
  for (int v0 = 0; v0 < V; v0 += 3) {
    const int nv = (V - v0) < 3 ? (V - v0) : 3;
    T c[NN][3];
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
      for (int k = 0; k < 3; ++k) c[a][k] = T(0);
    // Not unrolled: the Hex8 geometry of eight points at once does not fit in registers.
#pragma unroll 1
    for (int q = 0; q < E::Q; ++q) {
      T G[NN][D];
      qp_geometry<ET, T>(q, X, G);
      const T* f = flux + ((e * E::Q + q) * V + v0) * D;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k < nv) {
          T fk[D];
#pragma unroll
          for (int d = 0; d < D; ++d) fk[d] = f[k * D + d];
#pragma unroll
          for (int a = 0; a < NN; ++a) {
            T s = G[a][0] * fk[0];
#pragma unroll
            for (int d = 1; d < D; ++d) s += G[a][d] * fk[d];
            c[a][k] += s;
          }
        }
      }
    }
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (k < nv) contrib[(e * NN + a) * V + v0 + k] = c[a][k];
  }
}

// Phase 2: out[n] = the contributions of node n's incident (element, corner) pairs, in
// the order of the incidence CSR (increasing element): deterministic.
template <class T>
__global__ void grad_transpose_node_kernel(const T* __restrict__ contrib, int64_t n_nodes, int V,
                                           const int32_t* __restrict__ inc_ptr,
                                           const int32_t* __restrict__ inc_idx,
                                           T* __restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_nodes * V) return;
  const int64_t n = i / V;
  const int v = (int)(i - n * V);
  T s = T(0);
  for (int k = __ldg(inc_ptr + n); k < __ldg(inc_ptr + n + 1); ++k)
    s += contrib[(int64_t)__ldg(inc_idx + k) * V + v];
  out[i] = s;
}

template <int ET, class T>
__global__ void eval_transpose_kernel(const T* __restrict__ quad, int64_t n_nodes, int V,
                                      const int32_t* __restrict__ inc_ptr,
                                      const int32_t* __restrict__ inc_idx, T* __restrict__ out) {
  using E = Elem<ET>;
  const int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= n_nodes) return;
  for (int v = 0; v < V; ++v) {
    T acc = T(0);
    for (int k = inc_ptr[n]; k < inc_ptr[n + 1]; ++k) {
      const int ea = inc_idx[k];
      const int64_t e = ea / E::NN;
      const int a = ea % E::NN;
      for (int q = 0; q < E::Q; ++q) acc += E::template N<T>(q, a) * quad[(e * E::Q + q) * V + v];
    }
    out[n * V + v] = acc;
  }
}

template <class T>
__global__ void integrate_quad_transpose_kernel(const T* __restrict__ g, const T* __restrict__ w,
                                                int64_t n_elems, int Q, int V,
                                                T* __restrict__ out) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n_elems * Q * V) return;
  const int v = (int)(tid % V);
  const int64_t eq = tid / V;
  const int64_t e = eq / Q;
  out[tid] = g[e * V + v] * w[eq];
}

template <class T>
__global__ void scatter_nodal_kernel(const T* __restrict__ vals, int64_t n_nodes, int V,
                                     const int32_t* __restrict__ inc_ptr,
                                     const int32_t* __restrict__ inc_idx, T* __restrict__ out) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n_nodes * V) return;
  const int v = (int)(tid % V);
  const int64_t n = tid / V;
  T acc = T(0);
  for (int k = inc_ptr[n]; k < inc_ptr[n + 1]; ++k) acc += vals[(int64_t)inc_idx[k] * V + v];
  out[tid] = acc;
}

}  // namespace tg

using namespace tg;

extern "C" int tg_integrate_quad_transpose(int prec, const void* g, const void* weights,
                                           int64_t n_elems, int n_quad, int n_vals, void* out,
                                           void* stream) {
  TG_TRY(check_sizes(n_elems, 0, n_vals));
  if (n_quad <= 0) return set_error(TG_ERR_VALUE, "n_quad must be positive");
  if (n_elems == 0) return TG_OK;
  TG_TRY(check_ptr(g, "g"));
  TG_TRY(check_ptr(weights, "weights"));
  TG_TRY(check_ptr(out, "out"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    const int64_t total = n_elems * n_quad * n_vals;
    integrate_quad_transpose_kernel<T><<<grid_for(total, TPB_T), TPB_T, 0, as_stream(stream)>>>(
        (const T*)g, (const T*)weights, n_elems, n_quad, n_vals, (T*)out);
    return launch_check("tg_integrate_quad_transpose");
  });
}

extern "C" int tg_scatter_nodal(int prec, const void* vals, int64_t n_nodes, int n_vals,
                                int nodes_per_elem, const int32_t* inc_ptr,
                                const int32_t* inc_idx, void* out, void* stream) {
  (void)nodes_per_elem;
  TG_TRY(check_sizes(0, n_nodes, n_vals));
  if (n_nodes == 0) return TG_OK;
  TG_TRY(check_ptr(inc_ptr, "inc_ptr"));
  TG_TRY(check_ptr(out, "out"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    scatter_nodal_kernel<T><<<grid_for(n_nodes * n_vals, TPB_T), TPB_T, 0, as_stream(stream)>>>(
        (const T*)vals, n_nodes, n_vals, inc_ptr, inc_idx, (T*)out);
    return launch_check("tg_scatter_nodal");
  });
}

static constexpr int TPB = 256;

extern "C" int tg_eval(int elem, int prec, const void* nodal, int64_t n_nodes, int n_vals,
                       const int32_t* conn, int64_t n_elems, void* out, void* stream) {
  TG_TRY(check_sizes(n_elems, n_nodes, n_vals));
  if (n_elems == 0) return TG_OK;
  TG_TRY(check_ptr(nodal, "nodal"));
  TG_TRY(check_ptr(conn, "conn"));
  TG_TRY(check_ptr(out, "out"));
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_prec(prec, [&](auto t) -> int {
      using T = decltype(t);
      const int64_t total = n_elems * Elem<ET>::Q * n_vals;
      eval_kernel<ET, T><<<grid_for(total, TPB), TPB, 0, as_stream(stream)>>>(
          (const T*)nodal, n_vals, conn, n_elems, (T*)out);
      return launch_check("tg_eval");
    });
  });
}

extern "C" int tg_grad(int elem, int prec, const void* nodal, const void* coords, int64_t n_nodes,
                       int n_vals, const int32_t* conn, int64_t n_elems, void* out, void* stream) {
  TG_TRY(check_sizes(n_elems, n_nodes, n_vals));
  if (n_elems == 0) return TG_OK;
  TG_TRY(check_ptr(nodal, "nodal"));
  TG_TRY(check_ptr(coords, "coords"));
  TG_TRY(check_ptr(conn, "conn"));
  TG_TRY(check_ptr(out, "out"));
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_prec(prec, [&](auto t) -> int {
      using T = decltype(t);
      if constexpr (ET == TG_HEX8)
        hex_grad_kernel<T><<<grid_for(n_elems, 128), 128, 0, as_stream(stream)>>>(
            (const T*)nodal, (const T*)coords, n_vals, conn, n_elems, (T*)out);
      else
        grad_kernel<ET, T><<<grid_for(n_elems, 128), 128, 0, as_stream(stream)>>>(
            (const T*)nodal, (const T*)coords, n_vals, conn, n_elems, (T*)out);
      return launch_check("tg_grad");
    });
  });
}

extern "C" int tg_integration_weights(int elem, int prec, const void* coords, int64_t n_nodes,
                                      const int32_t* conn, int64_t n_elems, void* out,
                                      void* stream) {
  TG_TRY(check_sizes(n_elems, n_nodes, 1));
  if (n_elems == 0) return TG_OK;
  TG_TRY(check_ptr(coords, "coords"));
  TG_TRY(check_ptr(conn, "conn"));
  TG_TRY(check_ptr(out, "out"));
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_prec(prec, [&](auto t) -> int {
      using T = decltype(t);
      weights_kernel<ET, T><<<grid_for(n_elems, 128), 128, 0, as_stream(stream)>>>(
          (const T*)coords, conn, n_elems, (T*)out);
      return launch_check("tg_integration_weights");
    });
  });
}

extern "C" int tg_integrate_quad(int prec, const void* quad, const void* weights, int64_t n_elems,
                                 int n_quad, int n_vals, void* out, void* stream) {
  TG_TRY(check_sizes(n_elems, 0, n_vals));
  if (n_quad <= 0) return set_error(TG_ERR_VALUE, "n_quad must be positive");
  if (n_elems == 0) return TG_OK;
  TG_TRY(check_ptr(quad, "quad"));
  TG_TRY(check_ptr(weights, "weights"));
  TG_TRY(check_ptr(out, "out"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    integrate_quad_kernel<T><<<grid_for(n_elems * n_vals, TPB), TPB, 0, as_stream(stream)>>>(
        (const T*)quad, (const T*)weights, n_elems, n_quad, n_vals, (T*)out);
    return launch_check("tg_integrate_quad");
  });
}

extern "C" size_t tg_sum_rows_workspace_bytes(int prec, int n_vals) {
  (void)prec;
  return (size_t)SUM_CHUNKS * (size_t)(n_vals > 0 ? n_vals : 1) * sizeof(double);
}

extern "C" int tg_sum_rows(int prec, const void* in, int64_t n_rows, int n_vals, void* out,
                           void* workspace, size_t workspace_bytes, void* stream) {
  if (n_rows < 0 || n_vals <= 0) return set_error(TG_ERR_VALUE, "bad sizes for tg_sum_rows");
  TG_TRY(check_ptr(out, "out"));
  if (workspace_bytes < tg_sum_rows_workspace_bytes(prec, n_vals))
    return set_error(TG_ERR_WORKSPACE, "tg_sum_rows: workspace too small");
  if (n_rows > 0) TG_TRY(check_ptr(in, "in"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    rowsum_stage1<T><<<SUM_CHUNKS, SUM_THREADS, 0, as_stream(stream)>>>(
        (const T*)in, n_rows, n_vals, (double*)workspace);
    rowsum_stage2<T><<<1, SUM_THREADS, 0, as_stream(stream)>>>((const double*)workspace, n_vals,
                                                               (T*)out);
    return launch_check("tg_sum_rows");
  });
}

extern "C" int tg_gather_nodal(int prec, const void* nodal, int64_t n_nodes, int n_vals,
                               const int32_t* conn, int64_t n_elems, int nodes_per_elem,
                               void* out, void* stream) {
  TG_TRY(check_sizes(n_elems, n_nodes, n_vals));
  if (nodes_per_elem <= 0) return set_error(TG_ERR_VALUE, "nodes_per_elem must be positive");
  if (n_elems == 0) return TG_OK;
  TG_TRY(check_ptr(nodal, "nodal"));
  TG_TRY(check_ptr(conn, "conn"));
  TG_TRY(check_ptr(out, "out"));
  const int64_t entries = n_elems * nodes_per_elem;
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    gather_nodal_kernel<T><<<grid_for(entries * n_vals, TPB), TPB, 0, as_stream(stream)>>>(
        (const T*)nodal, n_vals, conn, entries, (T*)out);
    return launch_check("tg_gather_nodal");
  });
}

extern "C" size_t tg_grad_transpose_workspace_bytes(int elem, int prec, int64_t n_elems,
                                                    int n_vals) {
  const int NN = elem == TG_TRI3 ? 3 : (elem == TG_TET4 ? 4 : 8);
  if (n_elems <= 0 || n_vals <= 0) return 0;
  return (size_t)n_elems * NN * n_vals * (prec == TG_F32 ? 4 : 8);
}

extern "C" int tg_grad_transpose(int elem, int prec, const void* flux, const void* coords,
                                 int64_t n_nodes, int n_vals, const int32_t* conn,
                                 int64_t n_elems, const int32_t* inc_ptr, const int32_t* inc_idx,
                                 void* out, void* workspace, size_t workspace_bytes,
                                 void* stream) {
  TG_TRY(check_sizes(n_elems, n_nodes, n_vals));
  if (n_nodes == 0) return TG_OK;
  if (workspace_bytes < tg_grad_transpose_workspace_bytes(elem, prec, n_elems, n_vals))
    return set_error(TG_ERR_WORKSPACE, "tg_grad_transpose: workspace too small (%zu < %zu)",
                     workspace_bytes, tg_grad_transpose_workspace_bytes(elem, prec, n_elems, n_vals));
  TG_TRY(check_ptr(coords, "coords"));
  TG_TRY(check_ptr(inc_ptr, "inc_ptr"));
  TG_TRY(check_ptr(out, "out"));
  if (n_elems > 0) {
    TG_TRY(check_ptr(flux, "flux"));
    TG_TRY(check_ptr(conn, "conn"));
    TG_TRY(check_ptr(inc_idx, "inc_idx"));
  }
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_prec(prec, [&](auto t) -> int {
      using T = decltype(t);
      if (n_elems > 0) {
        if constexpr (ET == TG_HEX8)
          hex_grad_transpose_elem_kernel<T><<<grid_for(n_elems, 128), 128, 0,
                                              as_stream(stream)>>>(
              (const T*)flux, (const T*)coords, n_vals, conn, n_elems, (T*)workspace);
        else
          grad_transpose_elem_kernel<ET, T><<<grid_for(n_elems, 128), 128, 0,
                                              as_stream(stream)>>>(
              (const T*)flux, (const T*)coords, n_vals, conn, n_elems, (T*)workspace);
      }
      grad_transpose_node_kernel<T><<<grid_for(n_nodes * n_vals, 256), 256, 0,
                                      as_stream(stream)>>>((const T*)workspace, n_nodes, n_vals,
                                                           inc_ptr, inc_idx, (T*)out);
      return launch_check("tg_grad_transpose");
    });
  });
}

extern "C" int tg_eval_transpose(int elem, int prec, const void* quad, int64_t n_nodes,
                                 int n_vals, const int32_t* conn, int64_t n_elems,
                                 const int32_t* inc_ptr, const int32_t* inc_idx, void* out,
                                 void* stream) {
  (void)conn;
  TG_TRY(check_sizes(n_elems, n_nodes, n_vals));
  if (n_nodes == 0) return TG_OK;
  TG_TRY(check_ptr(inc_ptr, "inc_ptr"));
  TG_TRY(check_ptr(out, "out"));
  if (n_elems > 0) {
    TG_TRY(check_ptr(quad, "quad"));
    TG_TRY(check_ptr(inc_idx, "inc_idx"));
  }
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_prec(prec, [&](auto t) -> int {
      using T = decltype(t);
      eval_transpose_kernel<ET, T><<<grid_for(n_nodes, 128), 128, 0, as_stream(stream)>>>(
          (const T*)quad, n_nodes, n_vals, inc_ptr, inc_idx, (T*)out);
      return launch_check("tg_eval_transpose");
    });
  });
}
