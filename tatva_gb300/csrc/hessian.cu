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
// inside the pattern.  Node-centric: a thread owns one node's V rows of Jc and adds the
// row blocks of the node's incident (element, corner) pairs in incidence order
// (ascending element): deterministic, no atomics, no colouring of the elements.  With
// a distance-2 colouring each colour occurs at most once per row, so a row is a dense
// vector over the colours; the thread accumulates it in shared memory and the CTA
// writes its consecutive nodes' rows as one contiguous, coalesced block of Jc.
#include "tg_common.cuh"
#include "tg_dispatch.cuh"
#include "tg_materials.cuh"

namespace tg {

// Row block K_e[(a, i), (b, k)] (i, k < V, b < NN) of element e's tangent at u,
// acc[i][b V + k]; nid: the element's nodes
template <int ET, int MAT, class T>
__device__ __forceinline__ void element_row_block(
    const T* __restrict__ coords, const int32_t* __restrict__ conn, const T* __restrict__ u,
    T p0, T p1, const T* __restrict__ eparam, int64_t e, int a,
    T (&acc)[Law<MAT, Elem<ET>::D, T>::V][Elem<ET>::NN * Law<MAT, Elem<ET>::D, T>::V],
    int (&nid)[Elem<ET>::NN]) {
  using E = Elem<ET>;
  using L = Law<MAT, E::D, T>;
  constexpr int NN = E::NN, D = E::D, V = L::V;
  T X[NN][D], U[NN][V];
#pragma unroll
  for (int b = 0; b < NN; ++b) {
    nid[b] = __ldg(conn + e * NN + b);
#pragma unroll
    for (int d = 0; d < D; ++d) X[b][d] = coords[(int64_t)nid[b] * D + d];
#pragma unroll
    for (int i = 0; i < V; ++i) U[b][i] = L::LINEAR ? T(0) : u[(int64_t)nid[b] * V + i];
  }
  const L law(eparam ? eparam[e] : p0, p1);
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
}

// Thread t of the CTA owns node n0 + t.  ACC_SMEM: its V x C row block sits in shared
// memory at row t (stride V C + 1 words: conflict-free for the CTA's row-major write);
// otherwise (too many colours for shared memory) it accumulates in its own rows of
// Jc, which the caller zeroed.
template <int ET, int MAT, class T, bool ACC_SMEM>
__global__ void compressed_hessian_kernel(const T* __restrict__ coords,
                                          const int32_t* __restrict__ conn,
                                          const T* __restrict__ u, T p0, T p1,
                                          const T* __restrict__ eparam, int64_t n_nodes,
                                          const int32_t* __restrict__ inc_ptr,
                                          const int32_t* __restrict__ inc_idx,
                                          const int32_t* __restrict__ dof_colors, int n_colors,
                                          T* __restrict__ Jc) {
  using E = Elem<ET>;
  using L = Law<MAT, E::D, T>;
  constexpr int NN = E::NN, V = L::V;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sm = reinterpret_cast<T*>(smem_raw);
  const int row_words = V * n_colors;
  const int stride = row_words + 1;
  const int64_t n0 = (int64_t)blockIdx.x * blockDim.x;
  const int64_t n = n0 + threadIdx.x;
  T* acc_row = ACC_SMEM ? sm + (int64_t)threadIdx.x * stride : Jc + n * row_words;
  if (ACC_SMEM)
    for (int k = 0; k < row_words; ++k) acc_row[k] = T(0);
  if (n < n_nodes) {
    for (int j = __ldg(inc_ptr + n); j < __ldg(inc_ptr + n + 1); ++j) {
      const int ea = __ldg(inc_idx + j);
      const int64_t e = ea / NN;
      const int a = ea - (int)(e * NN);
      T rb[V][NN * V];
      int nid[NN];
      element_row_block<ET, MAT, T>(coords, conn, u, p0, p1, eparam, e, a, rb, nid);
#pragma unroll
      for (int b = 0; b < NN; ++b)
#pragma unroll
        for (int k = 0; k < V; ++k) {
          const int col = __ldg(dof_colors + (int64_t)nid[b] * V + k);
#pragma unroll
          for (int i = 0; i < V; ++i) acc_row[i * n_colors + col] += rb[i][b * V + k];
        }
    }
  }
  if (ACC_SMEM) {
    __syncthreads();
    // rows of nodes n0 .. n0 + blockDim.x - 1 are one contiguous block of Jc
    const int64_t rows_here = (n_nodes - n0) < (int64_t)blockDim.x ? (n_nodes - n0) : blockDim.x;
    const int64_t total = rows_here * row_words;
    T* out = Jc + n0 * row_words;
    for (int64_t k = threadIdx.x; k < total; k += blockDim.x) {
      const int t = (int)(k / row_words);
      out[k] = sm[(int64_t)t * stride + (k - (int64_t)t * row_words)];
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
                                     int64_t n_elems, const void* u, const int32_t* inc_ptr,
                                     const int32_t* inc_idx, const int32_t* dof_colors,
                                     int n_colors, void* Jc, void* stream) {
  TG_TRY(check_ptr(mat, "mat"));
  TG_TRY(check_sizes(n_elems, n_nodes, 1));
  TG_TRY(check_ptr(Jc, "Jc"));
  if (n_colors <= 0) return set_error(TG_ERR_VALUE, "n_colors must be positive");
  if (n_nodes == 0) return TG_OK;
  TG_TRY(check_ptr(inc_ptr, "inc_ptr"));
  if (n_elems > 0) {
    TG_TRY(check_ptr(coords, "coords"));
    TG_TRY(check_ptr(conn, "conn"));
    TG_TRY(check_ptr(inc_idx, "inc_idx"));
    TG_TRY(check_ptr(dof_colors, "dof_colors"));
  }
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
          if (!Law<MAT, Elem<ET>::D, T>::LINEAR && n_elems > 0) TG_TRY(check_ptr(u, "u"));
          // threads per CTA (a multiple of 32, <= 128): the most resident threads per
          // SM that shared memory allows (each thread holds one node's row block)
          const size_t row_bytes = ((size_t)V * n_colors + 1) * sizeof(T);
          int dev = 0, sm_bytes = 0, cta_bytes = 0;
          TG_TRY(cuda_check(cudaGetDevice(&dev), "tg_compressed_hessian: device"));
          TG_TRY(cuda_check(cudaDeviceGetAttribute(&sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev),
                            "tg_compressed_hessian: shared memory per SM"));
          TG_TRY(cuda_check(cudaDeviceGetAttribute(&cta_bytes, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                            "tg_compressed_hessian: shared memory per CTA"));
          int nt = 0, best = 0;
          for (int cand = 128; cand >= 32; cand -= 32) {
            const size_t need = (size_t)cand * row_bytes;
            if (need > (size_t)cta_bytes) continue;
            const int resident = (int)((size_t)sm_bytes / (need + 1024)) * cand;
            if (resident > best) {
              best = resident;
              nt = cand;
            }
          }
          if (nt == 0) nt = 32;
          const unsigned grid = (unsigned)((n_nodes + nt - 1) / nt);
          if (best > 0) {
            const size_t smem = (size_t)nt * row_bytes;
            auto kern = compressed_hessian_kernel<ET, MAT, T, true>;
            TG_TRY(cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)smem),
                              "tg_compressed_hessian: shared memory"));
            kern<<<grid, nt, smem, st>>>((const T*)coords, conn, (const T*)u, (T)mat->p0,
                                         (T)mat->p1, (const T*)mat->elem_param, n_nodes, inc_ptr,
                                         inc_idx, dof_colors, n_colors, (T*)Jc);
          } else {
            const int64_t total = n_nodes * V * (int64_t)n_colors;
            fill_kernel<T><<<grid_for(total, 256), 256, 0, st>>>((T*)Jc, total, T(0));
            compressed_hessian_kernel<ET, MAT, T, false><<<grid, 32, 0, st>>>(
                (const T*)coords, conn, (const T*)u, (T)mat->p0, (T)mat->p1,
                (const T*)mat->elem_param, n_nodes, inc_ptr, inc_idx, dof_colors, n_colors,
                (T*)Jc);
          }
          return launch_check("tg_compressed_hessian");
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
