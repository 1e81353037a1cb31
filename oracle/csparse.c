/* Oracle (test infrastructure only): plain-C restatement of the reference's sparsity
 * pattern and distance-2 colouring, for sizes where the numpy / pure-Python oracle in
 * sparse.py takes too long (millions of dofs).  Nothing in the product links it.
 *
 *   oracle_pattern   tatva/sparse/_extraction.py:37-102 (_create_sparse_structure):
 *                    every (row dof, col dof) pair of every element, made unique and
 *                    sorted by row * N + col (np.unique), dof = node * ndpn + comp.
 *                    Computed here row by row: the columns of a row are the dofs of
 *                    every node of every element that holds the row's node, sorted and
 *                    made unique -- the same set, in the same order.
 *   oracle_d2_colors tatva/sparse/_coloring.py:27-48 (A2 = A @ A, the distance-2
 *                    neighbours of row i are the columns of the rows j in A's row i),
 *                    :136-153 (natural order: colour i = the smallest colour not taken
 *                    by an already coloured distance-2 neighbour), :270-283.
 *
 * Build: cc -O2 -shared -fPIC oracle/csparse.c -o oracle/_build/liboracle_sparse.so
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static int cmp_i32(const void* a, const void* b) {
  const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* Node -> element incidence (CSR).  Returns 0, or -1 when out of memory. */
static int incidence(const int32_t* conn, int64_t n_elems, int npe, int64_t n_nodes,
                     int64_t** ptr_out, int32_t** idx_out) {
  int64_t* ptr = (int64_t*)calloc((size_t)n_nodes + 1, sizeof(int64_t));
  int32_t* idx = (int32_t*)malloc((size_t)(n_elems * npe) * sizeof(int32_t));
  int64_t* fill = (int64_t*)calloc((size_t)n_nodes, sizeof(int64_t));
  if (!ptr || !idx || !fill) {
    free(ptr); free(idx); free(fill);
    return -1;
  }
  for (int64_t e = 0; e < n_elems; ++e)
    for (int a = 0; a < npe; ++a) ptr[conn[e * npe + a] + 1]++;
  for (int64_t n = 0; n < n_nodes; ++n) ptr[n + 1] += ptr[n];
  for (int64_t e = 0; e < n_elems; ++e)
    for (int a = 0; a < npe; ++a) {
      const int32_t n = conn[e * npe + a];
      idx[ptr[n] + fill[n]++] = (int32_t)e;
    }
  free(fill);
  *ptr_out = ptr;
  *idx_out = idx;
  return 0;
}

/* Pass 1 (indices == NULL): row lengths into indptr (n_dofs + 1 entries, prefix sums).
 * Pass 2: column indices of every row into indices (indptr[n_dofs] entries). */
int oracle_pattern(const int32_t* conn, int64_t n_elems, int npe, int64_t n_nodes, int ndpn,
                   int64_t* indptr, int32_t* indices) {
  int64_t* iptr;
  int32_t* iidx;
  if (incidence(conn, n_elems, npe, n_nodes, &iptr, &iidx)) return -1;
  int64_t cap = 64;
  int32_t* nodes = (int32_t*)malloc((size_t)cap * sizeof(int32_t));
  if (!nodes) {
    free(iptr); free(iidx);
    return -1;
  }
  if (!indices) indptr[0] = 0;
  for (int64_t n = 0; n < n_nodes; ++n) {
    int64_t m = 0;
    const int64_t need = (iptr[n + 1] - iptr[n]) * npe;
    if (need > cap) {
      cap = need;
      int32_t* t = (int32_t*)realloc(nodes, (size_t)cap * sizeof(int32_t));
      if (!t) {
        free(nodes); free(iptr); free(iidx);
        return -1;
      }
      nodes = t;
    }
    for (int64_t k = iptr[n]; k < iptr[n + 1]; ++k)
      for (int a = 0; a < npe; ++a) nodes[m++] = conn[(int64_t)iidx[k] * npe + a];
    qsort(nodes, (size_t)m, sizeof(int32_t), cmp_i32);
    int64_t u = 0;
    for (int64_t k = 0; k < m; ++k)
      if (u == 0 || nodes[k] != nodes[u - 1]) nodes[u++] = nodes[k];
    for (int c = 0; c < ndpn; ++c) {
      const int64_t row = n * ndpn + c;
      if (!indices) {
        indptr[row + 1] = indptr[row] + u * ndpn;
      } else {
        int32_t* out = indices + indptr[row];
        for (int64_t k = 0; k < u; ++k)
          for (int d = 0; d < ndpn; ++d) *out++ = (int32_t)(nodes[k] * ndpn + d);
      }
    }
  }
  free(nodes);
  free(iptr);
  free(iidx);
  return 0;
}

/* Natural-order greedy distance-2 colouring of the CSR pattern; returns the number of
 * colours, or -1 when out of memory. */
int oracle_d2_colors(const int64_t* indptr, const int32_t* indices, int64_t n, int32_t* colors) {
  int64_t cap = 1024;
  int64_t* stamp = (int64_t*)malloc((size_t)cap * sizeof(int64_t));
  if (!stamp) return -1;
  for (int64_t c = 0; c < cap; ++c) stamp[c] = -1;
  for (int64_t i = 0; i < n; ++i) colors[i] = -1;
  int32_t ncol = 0;
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t a = indptr[i]; a < indptr[i + 1]; ++a) {
      const int32_t j = indices[a];
      for (int64_t b = indptr[j]; b < indptr[j + 1]; ++b) {
        const int32_t c = colors[indices[b]];
        if (c >= 0) stamp[c] = i;
      }
    }
    int32_t c = 0;
    while (c < cap && stamp[c] == i) ++c;
    if (c == cap) {
      int64_t* t = (int64_t*)realloc(stamp, (size_t)(2 * cap) * sizeof(int64_t));
      if (!t) {
        free(stamp);
        return -1;
      }
      stamp = t;
      for (int64_t k = cap; k < 2 * cap; ++k) stamp[k] = -1;
      cap *= 2;
    }
    colors[i] = c;
    if (c + 1 > ncol) ncol = c + 1;
  }
  free(stamp);
  return ncol;
}
