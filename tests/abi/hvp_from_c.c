/* Drives the C ABI of libtatva_gb300 from plain C: no Python, no PyTorch.
 *
 * Builds a structured Hex8 brick on the host, an element-block plan (HOST setup
 * entry points), copies the plan to the device with the CUDA runtime, applies the
 * linear-elastic HVP in FP64 with tg_apply, and checks the result against a host
 * evaluation of y = K v for a linear field v, where K v can be written down:
 * for v = A x (constant strain) the interior rows of K v vanish.  Also runs the
 * FP32 HVP and checks it against the FP64 one.  Prints "ok" and returns 0 on success.
 *
 * Build: nvcc -x cu -I include tests/abi/hvp_from_c.c -L tatva_gb300 -ltatva_gb300
 */
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "tatva_gb300.h"

#define CK(x)                                                              \
  do {                                                                     \
    cudaError_t e_ = (x);                                                  \
    if (e_ != cudaSuccess) {                                               \
      fprintf(stderr, "%s:%d %s\n", __FILE__, __LINE__, cudaGetErrorString(e_)); \
      return 2;                                                            \
    }                                                                      \
  } while (0)
#define TG(x)                                                              \
  do {                                                                     \
    int r_ = (x);                                                          \
    if (r_ != TG_OK) {                                                     \
      fprintf(stderr, "%s:%d tg error %d: %s\n", __FILE__, __LINE__, r_, tg_last_error()); \
      return 3;                                                            \
    }                                                                      \
  } while (0)

static void* dcopy(const void* h, size_t bytes) {
  void* d = NULL;
  if (cudaMalloc(&d, bytes ? bytes : 16) != cudaSuccess) return NULL;
  if (bytes) cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice);
  return d;
}

int main(void) {
  const int n = 12, nx = n + 1;
  const int64_t nn = (int64_t)nx * nx * nx, ne = (int64_t)n * n * n, ndof = 3 * nn;
  double* X = (double*)malloc(sizeof(double) * 3 * nn);
  int32_t* conn = (int32_t*)malloc(sizeof(int32_t) * 8 * ne);
  for (int k = 0; k < nx; ++k)
    for (int j = 0; j < nx; ++j)
      for (int i = 0; i < nx; ++i) {
        const int64_t g = i + (int64_t)nx * (j + (int64_t)nx * k);
        X[3 * g] = (double)i / n;
        X[3 * g + 1] = (double)j / n;
        X[3 * g + 2] = (double)k / n;
      }
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const int64_t e = i + (int64_t)n * (j + (int64_t)n * k);
        const int32_t n0 = i + nx * (j + nx * k), sx = 1, sy = nx, sz = nx * nx;
        const int32_t c[8] = {n0, n0 + sx, n0 + sx + sy, n0 + sy,
                              n0 + sz, n0 + sx + sz, n0 + sx + sy + sz, n0 + sy + sz};
        memcpy(conn + 8 * e, c, sizeof c);
      }

  /* plan on the host, then to the device */
  void* h = NULL;
  TG(tg_plan_build(TG_HEX8, conn, ne, nn, X, 3, 512, 4096, &h));
  int64_t sz[13];
  TG(tg_plan_sizes(h, sz));
  const int64_t nb = sz[0], nel = sz[1], ncol = sz[2], nloc = sz[3], nsh = sz[4], npart = sz[5];
  int32_t *bep = malloc(4 * (nb + 1)), *bcp = malloc(4 * (nb + 1)), *cof = malloc(4 * (ncol + 1));
  int32_t *bnp = malloc(4 * (nb + 1)), *eid = malloc(4 * (nel + 1)), *lg = malloc(4 * (nloc + 1));
  int32_t *ls = malloc(4 * (nloc + 1)), *lsm = malloc(4 * (nloc + 1)), *shn = malloc(4 * (nsh + 1));
  int32_t *shp = malloc(4 * (nsh + 2)), *shs = malloc(4 * (npart + 1));
  uint16_t* lc = malloc(2 * (8 * nel + 8));
  TG(tg_plan_export(h, bep, bcp, cof, bnp, lc, eid, lg, ls, lsm, shn, shp, shs));
  tg_block_plan p;
  memset(&p, 0, sizeof p);
  p.n_blocks = (int32_t)nb;
  p.n_elems = (int32_t)nel;
  p.nodes_per_elem_padded = (int32_t)sz[8];
  p.max_local_nodes = (int32_t)sz[6];
  p.n_shared = (int32_t)nsh;
  p.n_partials = (int32_t)npart;
  p.threads = 128;
  p.n_affine_blocks = (int32_t)sz[9];
  p.n_diag_blocks = (int32_t)sz[10];
  p.max_block_elems = (int32_t)sz[11];
  p.n_lattice_blocks = (int32_t)sz[12];
  p.blk_elem_ptr = dcopy(bep, 4 * (nb + 1));
  p.blk_color_ptr = dcopy(bcp, 4 * (nb + 1));
  p.color_ofs = dcopy(cof, 4 * ncol);
  p.blk_node_ptr = dcopy(bnp, 4 * (nb + 1));
  p.lconn = dcopy(lc, 2 * 8 * nel);
  p.elem_id = dcopy(eid, 4 * nel);
  p.lnode_gid = dcopy(lg, 4 * nloc);
  p.lnode_slot = dcopy(ls, 4 * nloc);
  p.lnode_smem = dcopy(lsm, 4 * nloc);
  p.shared_node = dcopy(shn, 4 * nsh);
  p.shared_ptr = dcopy(shp, 4 * (nsh + 1));
  p.shared_slots = dcopy(shs, 4 * npart);
  tg_plan_free(h);

  /* v = A x with a constant matrix A: interior rows of K v vanish */
  const double A[9] = {0.3, -0.2, 0.1, 0.05, 0.4, -0.3, -0.1, 0.2, 0.25};
  double* v = (double*)malloc(sizeof(double) * ndof);
  for (int64_t g = 0; g < nn; ++g)
    for (int r = 0; r < 3; ++r)
      v[3 * g + r] = A[3 * r] * X[3 * g] + A[3 * r + 1] * X[3 * g + 1] + A[3 * r + 2] * X[3 * g + 2];
  tg_material m;
  memset(&m, 0, sizeof m);
  m.kind = TG_LINEAR_ELASTIC;
  m.p0 = 0.7;
  m.p1 = 1.3;
  double *dX = dcopy(X, 8 * 3 * nn), *dv = dcopy(v, 8 * ndof), *dy = NULL;
  CK(cudaMalloc((void**)&dy, 8 * ndof));
  const size_t wsb = tg_apply_workspace_bytes(TG_HEX8, TG_F64, TG_LINEAR_ELASTIC, &p);
  void* ws = NULL;
  CK(cudaMalloc(&ws, wsb ? wsb : 16));
  TG(tg_apply(TG_HEX8, TG_F64, TG_MODE_HVP, &m, &p, dX, nn, NULL, dv, NULL, dy, ws, wsb, NULL));
  CK(cudaDeviceSynchronize());
  double* y = (double*)malloc(8 * ndof);
  CK(cudaMemcpy(y, dy, 8 * ndof, cudaMemcpyDeviceToHost));
  double ymax = 0, interior = 0;
  for (int k = 0; k < nx; ++k)
    for (int j = 0; j < nx; ++j)
      for (int i = 0; i < nx; ++i) {
        const int64_t g = i + (int64_t)nx * (j + (int64_t)nx * k);
        const int in = i > 0 && j > 0 && k > 0 && i < n && j < n && k < n;
        for (int r = 0; r < 3; ++r) {
          ymax = fmax(ymax, fabs(y[3 * g + r]));
          if (in) interior = fmax(interior, fabs(y[3 * g + r]));
        }
      }

  /* FP32 HVP of the same field */
  float *X32 = malloc(4 * 3 * nn), *v32 = malloc(4 * ndof), *y32 = malloc(4 * ndof);
  for (int64_t i = 0; i < 3 * nn; ++i) X32[i] = (float)X[i];
  for (int64_t i = 0; i < ndof; ++i) v32[i] = (float)v[i];
  float *dX32 = dcopy(X32, 4 * 3 * nn), *dv32 = dcopy(v32, 4 * ndof), *dy32 = NULL;
  CK(cudaMalloc((void**)&dy32, 4 * ndof));
  const size_t wsb32 = tg_apply_workspace_bytes(TG_HEX8, TG_F32, TG_LINEAR_ELASTIC, &p);
  TG(tg_apply(TG_HEX8, TG_F32, TG_MODE_HVP, &m, &p, dX32, nn, NULL, dv32, NULL, dy32, ws, wsb32,
              NULL));
  CK(cudaDeviceSynchronize());
  CK(cudaMemcpy(y32, dy32, 4 * ndof, cudaMemcpyDeviceToHost));
  double d32 = 0;
  for (int64_t i = 0; i < ndof; ++i) d32 = fmax(d32, fabs((double)y32[i] - y[i]));

  printf("n_blocks %lld ymax %.3e interior %.3e fp32-fp64 %.3e\n", (long long)nb, ymax, interior,
         d32);
  if (!(ymax > 1e-3) || interior > 1e-12 * ymax || d32 > 1e-5 * ymax) {
    printf("FAILED\n");
    return 1;
  }
  printf("ok\n");
  return 0;
}
