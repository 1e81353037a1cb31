// Colored compressed Hessian (K6) and its decompression into CSR values.
//
// Reference (tatva/sparse/base.py):
//   colored_jacobian_batch (:230-270): Jc[:, c] = jvp(grad E, u, seed_c),
//        seed_c = (colors == c) as 1.0 / 0.0  (:259), Jc has shape (N, C) (:268-270)
//   compute_rows_cols (:108-136): rows = repeat(arange(N), diff(indptr)),
//        col_colors = colors[indices]
//   jacfwd decompression (:173): data = Jc[rows, col_colors]
//
// Jc is computed here from element tangents instead of C full HVPs:
//   Jc[i, c] = sum_e sum_{(b,k) in e : color(dof(b,k)) = c} K_e[(a,i), (b,k)]
// which equals sum_{j: color j = c} H[i, j] because every element-local dof pair is
// inside the pattern.  Each thread owns one (element, node a) row block; elements
// are processed one element colour per launch (no two elements of a launch share a
// node), so the read-modify-write of Jc rows is race-free and its order is fixed.
#include "tg_common.cuh"
#include "tg_dispatch.cuh"
#include "tg_materials.cuh"

namespace tg {

template <int ET, int MAT, class T>
__global__ void compressed_hessian_kernel(const T* __restrict__ coords,
                                          const int32_t* __restrict__ conn,
                                          const T* __restrict__ u, T p0, T p1,
                                          const T* __restrict__ eparam,
                                          const int32_t* __restrict__ order, int n_in_color,
                                          const int32_t* __restrict__ dof_colors, int n_colors,
                                          T* __restrict__ Jc) {
  using E = Elem<ET>;
  using L = Law<MAT, E::D, T>;
  constexpr int NN = E::NN, D = E::D, V = L::V;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= n_in_color * NN) return;
  const int a = tid % NN;
  const int64_t e = __ldg(order + tid / NN);
  T X[NN][D], U[NN][V];
  int nid[NN];
#pragma unroll
  for (int b = 0; b < NN; ++b) {
    nid[b] = __ldg(conn + e * NN + b);
#pragma unroll
    for (int d = 0; d < D; ++d) X[b][d] = coords[(int64_t)nid[b] * D + d];
#pragma unroll
    for (int i = 0; i < V; ++i) U[b][i] = L::LINEAR ? T(0) : u[(int64_t)nid[b] * V + i];
  }
  const L law(eparam ? eparam[e] : p0, p1);
  T acc[V][NN * V];
#pragma unroll
  for (int i = 0; i < V; ++i)
#pragma unroll
    for (int c = 0; c < NN * V; ++c) acc[i][c] = T(0);
#pragma unroll
  for (int q = 0; q < E::Q; ++q) {
    T G[NN][D];
    const T wd = qp_geometry<ET, T>(q, X, G) * E::template w<T>(q);
    T H[V][D];
#pragma unroll
    for (int i = 0; i < V; ++i)
#pragma unroll
      for (int d = 0; d < D; ++d) {
        T s = T(0);
        if constexpr (!L::LINEAR) {
#pragma unroll
          for (int b = 0; b < NN; ++b) s += G[b][d] * U[b][i];
        }
        H[i][d] = s;
      }
    const auto lin = law.linearize(H);
    T ga[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      ga[d] = G[0][d];
#pragma unroll
      for (int b = 1; b < NN; ++b)
        if (b == a) ga[d] = G[b][d];
    }
#pragma unroll
    for (int b = 0; b < NN; ++b)
#pragma unroll
      for (int k = 0; k < V; ++k) {
        T dH[V][D], dP[V][D];
#pragma unroll
        for (int kk = 0; kk < V; ++kk)
#pragma unroll
          for (int d = 0; d < D; ++d) dH[kk][d] = (kk == k) ? G[b][d] : T(0);
        lin.dflux(dH, dP);
#pragma unroll
        for (int i = 0; i < V; ++i) {
          T s = T(0);
#pragma unroll
          for (int d = 0; d < D; ++d) s += dP[i][d] * ga[d];
          acc[i][b * V + k] += wd * s;
        }
      }
  }
  int na = nid[0];
#pragma unroll
  for (int b = 1; b < NN; ++b)
    if (b == a) na = nid[b];
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const int64_t row = (int64_t)na * V + i;
#pragma unroll
    for (int b = 0; b < NN; ++b)
#pragma unroll
      for (int k = 0; k < V; ++k) {
        const int col = __ldg(dof_colors + (int64_t)nid[b] * V + k);
        Jc[row * n_colors + col] += acc[i][b * V + k];
      }
  }
}

template <class T>
__global__ void fill_kernel(T* __restrict__ x, int64_t n, T val) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = val;
}

__global__ void rows_cols_kernel(const int32_t* __restrict__ indptr,
                                 const int32_t* __restrict__ indices,
                                 const int32_t* __restrict__ colors, int64_t n_rows,
                                 int32_t* __restrict__ rows, int32_t* __restrict__ col_colors) {
  // one warp per row
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) / 32;
  const int lane = threadIdx.x & 31;
  if (w >= n_rows) return;
  const int k0 = indptr[w], k1 = indptr[w + 1];
  for (int k = k0 + lane; k < k1; k += 32) {
    rows[k] = (int32_t)w;
    col_colors[k] = __ldg(colors + __ldg(indices + k));
  }
}

template <class T>
__global__ void decompress_kernel(const T* __restrict__ Jc, int n_colors,
                                  const int32_t* __restrict__ rows,
                                  const int32_t* __restrict__ col_colors, int64_t nnz,
                                  T* __restrict__ data) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  data[k] = Jc[(int64_t)__ldg(rows + k) * n_colors + __ldg(col_colors + k)];
}

template <class T>
__global__ void seeds_kernel(const int32_t* __restrict__ colors, int64_t n, int c0, int nc,
                             T* __restrict__ seeds) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * nc) return;
  const int j = (int)(t / n);
  const int64_t i = t % n;
  seeds[t] = (__ldg(colors + i) == c0 + j) ? T(1) : T(0);
}

template <class T>
__global__ void set_column_kernel(const T* __restrict__ col, int64_t n, int n_colors, int c,
                                  T* __restrict__ Jc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) Jc[i * n_colors + c] = col[i];
}

template <class F>
int dispatch_mat2(int kind, F&& f) {
  switch (kind) {
    case TG_POISSON: return f(IntC<TG_POISSON>{});
    case TG_LINEAR_ELASTIC: return f(IntC<TG_LINEAR_ELASTIC>{});
    case TG_NEO_HOOKEAN: return f(IntC<TG_NEO_HOOKEAN>{});
    default: return set_error(TG_ERR_VALUE, "unknown material kind %d", kind);
  }
}

}  // namespace tg

using namespace tg;

extern "C" int tg_compressed_hessian(int elem, int prec, const tg_material* mat,
                                     const void* coords, int64_t n_nodes, const int32_t* conn,
                                     int64_t n_elems, const void* u, const int32_t* elem_order,
                                     const int32_t* elem_color_ptr_host, int n_elem_colors,
                                     const int32_t* dof_colors, int n_colors, void* Jc,
                                     void* stream) {
  TG_TRY(check_ptr(mat, "mat"));
  TG_TRY(check_sizes(n_elems, n_nodes, 1));
  TG_TRY(check_ptr(Jc, "Jc"));
  if (n_colors <= 0) return set_error(TG_ERR_VALUE, "n_colors must be positive");
  if (n_elem_colors < 0) return set_error(TG_ERR_VALUE, "n_elem_colors must be >= 0");
  cudaStream_t st = as_stream(stream);
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_mat2(mat->kind, [&](auto mk) -> int {
      constexpr int MAT = decltype(mk)::value;
      if constexpr (MAT == TG_NEO_HOOKEAN && Elem<ET>::D != 3) {
        return set_error(TG_ERR_UNSUPPORTED, "Neo-Hookean needs a 3D element");
      } else {
        return dispatch_prec(prec, [&](auto t) -> int {
          using T = decltype(t);
          constexpr int V = LawDims<MAT, Elem<ET>::D>::V;
          const int64_t total = n_nodes * V * (int64_t)n_colors;
          fill_kernel<T><<<grid_for(total, 256), 256, 0, st>>>((T*)Jc, total, T(0));
          TG_TRY(launch_check("tg_compressed_hessian: zero"));
          if (n_elems == 0) return TG_OK;
          TG_TRY(check_ptr(coords, "coords"));
          TG_TRY(check_ptr(conn, "conn"));
          TG_TRY(check_ptr(elem_order, "elem_order"));
          TG_TRY(check_ptr(elem_color_ptr_host, "elem_color_ptr"));
          TG_TRY(check_ptr(dof_colors, "dof_colors"));
          if (!Law<MAT, Elem<ET>::D, T>::LINEAR) TG_TRY(check_ptr(u, "u"));
          for (int c = 0; c < n_elem_colors; ++c) {
            const int k0 = elem_color_ptr_host[c], k1 = elem_color_ptr_host[c + 1];
            const int cnt = k1 - k0;
            if (cnt <= 0) continue;
            compressed_hessian_kernel<ET, MAT, T>
                <<<grid_for((int64_t)cnt * Elem<ET>::NN, 128), 128, 0, st>>>(
                    (const T*)coords, conn, (const T*)u, (T)mat->p0, (T)mat->p1,
                    (const T*)mat->elem_param, elem_order + k0, cnt, dof_colors, n_colors,
                    (T*)Jc);
            TG_TRY(launch_check("tg_compressed_hessian"));
          }
          return TG_OK;
        });
      }
    });
  });
}

extern "C" int tg_rows_cols(const int32_t* indptr, const int32_t* indices, const int32_t* colors,
                            int64_t n_rows, int64_t nnz, int32_t* rows, int32_t* col_colors,
                            void* stream) {
  if (n_rows < 0 || nnz < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n_rows == 0 || nnz == 0) return TG_OK;
  TG_TRY(check_ptr(indptr, "indptr"));
  TG_TRY(check_ptr(indices, "indices"));
  TG_TRY(check_ptr(colors, "colors"));
  TG_TRY(check_ptr(rows, "rows"));
  TG_TRY(check_ptr(col_colors, "col_colors"));
  rows_cols_kernel<<<grid_for(n_rows * 32, 256), 256, 0, as_stream(stream)>>>(
      indptr, indices, colors, n_rows, rows, col_colors);
  return launch_check("tg_rows_cols");
}

extern "C" int tg_decompress(int prec, const void* Jc, int n_colors, const int32_t* rows,
                             const int32_t* col_colors, int64_t nnz, void* data, void* stream) {
  if (nnz < 0 || n_colors <= 0) return set_error(TG_ERR_VALUE, "bad sizes for tg_decompress");
  if (nnz == 0) return TG_OK;
  TG_TRY(check_ptr(Jc, "Jc"));
  TG_TRY(check_ptr(rows, "rows"));
  TG_TRY(check_ptr(col_colors, "col_colors"));
  TG_TRY(check_ptr(data, "data"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    decompress_kernel<T><<<grid_for(nnz, 256), 256, 0, as_stream(stream)>>>(
        (const T*)Jc, n_colors, rows, col_colors, nnz, (T*)data);
    return launch_check("tg_decompress");
  });
}

extern "C" int tg_color_seeds(int prec, const int32_t* colors, int64_t n, int c0, int nc,
                              void* seeds, void* stream) {
  if (n < 0 || nc < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n == 0 || nc == 0) return TG_OK;
  TG_TRY(check_ptr(colors, "colors"));
  TG_TRY(check_ptr(seeds, "seeds"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    seeds_kernel<T><<<grid_for(n * nc, 256), 256, 0, as_stream(stream)>>>(colors, n, c0, nc,
                                                                            (T*)seeds);
    return launch_check("tg_color_seeds");
  });
}

extern "C" int tg_set_column(int prec, const void* col, int64_t n, int n_colors, int c, void* Jc,
                             void* stream) {
  if (n < 0 || n_colors <= 0 || c < 0 || c >= n_colors)
    return set_error(TG_ERR_VALUE, "bad arguments for tg_set_column");
  if (n == 0) return TG_OK;
  TG_TRY(check_ptr(col, "col"));
  TG_TRY(check_ptr(Jc, "Jc"));
  return dispatch_prec(prec, [&](auto t) -> int {
    using T = decltype(t);
    set_column_kernel<T><<<grid_for(n, 256), 256, 0, as_stream(stream)>>>((const T*)col, n,
                                                                          n_colors, c, (T*)Jc);
    return launch_check("tg_set_column");
  });
}
