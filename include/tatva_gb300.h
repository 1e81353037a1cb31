/*
 * tatva_gb300 -- C ABI of the GB300 (sm_103a) finite-element hot path.
 *
 * Plain C: device pointers, sizes, an opaque cudaStream_t passed as void*, and an
 * int status.  No allocation happens on compute calls: every temporary lives in
 * caller-provided workspace whose size is reported by a *_workspace_bytes query.
 * Setup routines marked HOST take host pointers and run on the CPU.
 *
 * Each entry point names the reference (smec-ethz/tatva 0.11.1) interface it
 * replaces.  In the reference these are Python/JAX functions; a JAX host binds
 * the compute entry points as XLA FFI custom calls (the stream argument is the
 * XLA stream), a PyTorch host (tatva_gb300 package) binds them through ctypes.
 *
 * Conventions
 *   elem   TG_TRI3 | TG_TET4 | TG_HEX8   (node orders of tatva/element/base.py)
 *   prec   TG_F32 | TG_F64               (every float buffer of a call has this type)
 *   nodal arrays are (n_nodes, n_vals) row-major; dof = node*n_vals + comp
 *   quadrature arrays are (n_elems, n_quad, ...) row-major, reference QP order
 *   conn is int32 (n_elems, nodes_per_element), as tatva/mesh.py:205
 */
#ifndef TATVA_GB300_H
#define TATVA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define TG_API __attribute__((visibility("default")))
#else
#define TG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------- status codes (mapped to Python exceptions by the host) ---- */
enum {
  TG_OK = 0,
  TG_ERR_VALUE = 1,         /* ValueError   (tatva/operator.py:143-168)      */
  TG_ERR_TYPE = 2,          /* TypeError    (tatva/operator.py:156-157)      */
  TG_ERR_CUDA = 3,          /* RuntimeError                                  */
  TG_ERR_UNSUPPORTED = 4,   /* NotImplementedError                           */
  TG_ERR_NOT_CONVERGED = 5, /* solver hit max_iter before the tolerance      */
  TG_ERR_WORKSPACE = 6,     /* workspace smaller than the *_workspace_bytes  */
  TG_ERR_BREAKDOWN = 7,     /* CG breakdown (p.Ap <= 0) or non-finite value  */
};

enum { TG_TRI3 = 0, TG_TET4 = 1, TG_HEX8 = 2 };
enum { TG_F32 = 0, TG_F64 = 1 };
enum { TG_POISSON = 0, TG_LINEAR_ELASTIC = 1, TG_NEO_HOOKEAN = 2 };
enum { TG_MODE_RESIDUAL = 0, TG_MODE_HVP = 1, TG_MODE_DIAG = 2 };

/* last error message of the calling thread ("" if none) */
TG_API const char* tg_last_error(void);
TG_API int tg_version(void);
/* number of SMs of the current device (0 when no device) */
TG_API int tg_device_sm_count(void);
/* Streams of this library's CUDA runtime: for hosts whose stream handles are not
 * valid in it (the legacy default stream, NULL, is valid everywhere).          */
TG_API int tg_stream_create(void** stream);
TG_API int tg_stream_destroy(void* stream);
TG_API int tg_stream_synchronize(void* stream);
TG_API int tg_device_synchronize(void);

/* ============================================================================
 * Operator maps (K1-K3).  Replaces tatva/operator.py Operator.eval (:358-377),
 * Operator.grad (:379-397), get_integration_weights (:172-192),
 * _integrate_quad_array (:344-356), integrate (:307-319), and the reverse-mode
 * transposes of the gather nodal_values[mesh.elements] (:221,256).
 * ========================================================================== */

/* out (E,Q,V) = sum_a N_a(xi_q) nodal[conn[e,a], :]            operator.py:358-377 */
TG_API int tg_eval(int elem, int prec, const void* nodal, int64_t n_nodes, int n_vals,
            const int32_t* conn, int64_t n_elems, void* out, void* stream);

/* out (E,Q,V,D) = grad of nodal at QPs (value dims first, spatial last)
 *                                                  operator.py:379-397, base.py:99-115 */
TG_API int tg_grad(int elem, int prec, const void* nodal, const void* coords, int64_t n_nodes,
            int n_vals, const int32_t* conn, int64_t n_elems, void* out, void* stream);

/* out (E,Q) = detJ * w_q                                        operator.py:172-192 */
TG_API int tg_integration_weights(int elem, int prec, const void* coords, int64_t n_nodes,
                           const int32_t* conn, int64_t n_elems, void* out, void* stream);

/* out (E,V) = sum_q quad[e,q,:] * weights[e,q]      ("eq...,eq->e...") operator.py:344-356 */
TG_API int tg_integrate_quad(int prec, const void* quad, const void* weights, int64_t n_elems,
                      int n_quad, int n_vals, void* out, void* stream);

/* out (V) = sum over rows of in (R,V): deterministic fixed-order two-stage sum.
 * Replaces jnp.sum(res, axis=0) of Operator.integrate (operator.py:318-319).     */
TG_API size_t tg_sum_rows_workspace_bytes(int prec, int n_vals);
TG_API int tg_sum_rows(int prec, const void* in, int64_t n_rows, int n_vals, void* out,
                void* workspace, size_t workspace_bytes, void* stream);

/* out (E,n_e,V) = nodal[conn]  (the gather of Operator.map, operator.py:255-258) */
TG_API int tg_gather_nodal(int prec, const void* nodal, int64_t n_nodes, int n_vals,
                    const int32_t* conn, int64_t n_elems, int nodes_per_elem, void* out,
                    void* stream);

/* (E,Q,V) out[e,q,:] = g[e,:] * weights[e,q]: transpose of tg_integrate_quad */
TG_API int tg_integrate_quad_transpose(int prec, const void* g, const void* weights,
                                       int64_t n_elems, int n_quad, int n_vals, void* out,
                                       void* stream);
/* out (N,V) = sum over incident (e,a) of vals[e,a,:]: transpose of tg_gather_nodal */
TG_API int tg_scatter_nodal(int prec, const void* vals, int64_t n_nodes, int n_vals,
                            int nodes_per_elem, const int32_t* inc_ptr, const int32_t* inc_idx,
                            void* out, void* stream);

/* Transposes (reverse-mode AD of grad / eval; no reference function: the
 * reference gets them from XLA's transpose of the gather at operator.py:221).
 * out (N,V) = sum over incident (e,a) of sum_q sum_d dNdX[e,q,d,a] flux[e,q,:,d]
 * The node->(e*n_e+a) incidence CSR comes from tg_node_incidence (HOST) and fixes
 * the summation order: the result is deterministic.  tg_grad_transpose forms each
 * element's contribution to its nodes once (workspace of
 * tg_grad_transpose_workspace_bytes: n_elems * nodes_per_elem * n_vals values),
 * then sums them per node in incidence order.                                   */
TG_API size_t tg_grad_transpose_workspace_bytes(int elem, int prec, int64_t n_elems, int n_vals);
TG_API int tg_grad_transpose(int elem, int prec, const void* flux, const void* coords,
                      int64_t n_nodes, int n_vals, const int32_t* conn, int64_t n_elems,
                      const int32_t* inc_ptr, const int32_t* inc_idx, void* out,
                      void* workspace, size_t workspace_bytes, void* stream);
TG_API int tg_eval_transpose(int elem, int prec, const void* quad, int64_t n_nodes, int n_vals,
                      const int32_t* conn, int64_t n_elems, const int32_t* inc_ptr,
                      const int32_t* inc_idx, void* out, void* stream);

/* ============================================================================
 * Fused element assembly (K4 residual, K5 HVP, Jacobi diagonal) over a
 * deterministic element-block plan.  Replaces jax.grad(E) and
 * jax.jvp(jax.grad(E)) of the energies on the hot path (README.md:93,
 * tatva/sparse/base.py:257-265): Poisson 1/2 kappa|grad u|^2 - f u, linear
 * elastic 1/2 sigma:eps, Neo-Hookean mu/2(I1-3-2lnJ)+lambda/2(lnJ)^2
 * (tests/test_sparse_tracer.py:101-113).
 * ========================================================================== */

/* Element-block plan: elements grouped into spatially compact blocks; each block
 * stages its nodes in shared memory, accumulates element results in block-local
 * element-colour order, writes nodes it owns alone and leaves partial sums for
 * nodes shared with other blocks, which a second pass adds in fixed order.   */
typedef struct tg_block_plan {
  int32_t n_blocks;
  int32_t n_elems;
  int32_t nodes_per_elem_padded; /* stride of lconn (4 for Tri3/Tet4, 8 for Hex8) */
  int32_t max_local_nodes;       /* shared-memory sizing                          */
  int32_t n_shared;              /* nodes touched by more than one block          */
  int32_t n_partials;            /* partial-sum slots                             */
  int32_t threads;               /* threads per block (64/128/256; 0 = 256)       */
  int32_t n_affine_blocks;       /* Hex8: blocks [0, n_affine_blocks) hold only
                                    parallelepipeds (exactly, in FP32 and FP64)      */
  int32_t n_diag_blocks;         /* Hex8: blocks [0, n_diag_blocks) hold only
                                    axis-aligned boxes (a prefix of the affine ones) */
  int32_t max_block_elems;       /* largest element count of a block                */
  const int32_t* blk_elem_ptr;   /* [n_blocks+1] element range of block b         */
  const int32_t* blk_color_ptr;  /* [n_blocks+1] range of b's entries in color_ofs*/
  const int32_t* color_ofs;      /* per block: colour boundaries, relative         */
  const int32_t* blk_node_ptr;   /* [n_blocks+1] range of b's local nodes          */
  const uint16_t* lconn;         /* [n_elems*stride] block-local connectivity      */
  const int32_t* elem_id;        /* [n_elems] original element id                  */
  const int32_t* lnode_gid;      /* [sum L_b] global node id                       */
  const int32_t* lnode_slot;     /* [sum L_b] -1: owned alone, else partial slot   */
  const int32_t* lnode_smem;     /* [sum L_b] shared-memory slot of the local node */
  const int32_t* shared_node;    /* [n_shared] global node id                      */
  const int32_t* shared_ptr;     /* [n_shared+1]                                   */
  const int32_t* shared_slots;   /* [n_partials] slots in summation order; NULL:
                                  * identity (the k-th partial sits in slot k)    */
  /* optional, FP32 linear elasticity on Hex8 boxes: [3][n_elems] edge terms
   * 4(x1-x0), 4(y3-y0), 4(z4-z0) of the element positions of the box blocks, filled
   * by tg_plan_box_geometry; NULL: the kernel computes them from coordinates.     */
  const float* box_geom32;
  int32_t n_lattice_blocks;      /* Hex8: blocks [0, n_lattice_blocks) (a prefix of
                                    the box blocks) hold 8 x 8 x 8 boxes on 9 x 9 x 9
                                    local nodes numbered l = i + 9 j + 81 k, element
                                    corner a at (i,j,k) + (0,0,0) (1,0,0) (1,1,0)
                                    (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1); 0: none */
  int32_t reserved0;
  /* Hex8 structured brick (tg_grid_detect): nodes per axis Nx, Ny, Nz with node id
   * i + Nx (j + Ny k), uniform spacing grid_h along each axis, one element per cell
   * in the reference corner order.  Linear-elastic residual / HVP then run as a
   * stencil over the grid (no element data read).  grid_nodes[0] = 0: not a brick. */
  int32_t grid_nodes[3];
  int32_t grid_reserved;
  double grid_h[3];
} tg_block_plan;

/* Material parameters.  kind = TG_POISSON: p0 = kappa, p1 = f (source);
 * TG_LINEAR_ELASTIC: p0 = mu, p1 = lambda; TG_NEO_HOOKEAN: p0 = mu, p1 = lambda.
 * elem_param (optional, prec-typed, (n_elems,) in ORIGINAL element order) replaces
 * p0 per element (per-element conductivity through Operator.map's
 * element_quantity, tatva/operator.py:255-258).                                  */
typedef struct tg_material {
  int32_t kind;
  int32_t reserved;
  double p0, p1, p2, p3;
  const void* elem_param;
} tg_material;

/* HOST: build a plan.  conn/coords are host arrays (coords FP64, dim = 2 or 3).
 * block_elems: target elements per block; max_local_nodes: cap (<= 65535).   */
TG_API int tg_plan_build(int elem, const int32_t* conn, int64_t n_elems, int64_t n_nodes,
                  const double* coords, int dim, int block_elems, int max_local_nodes,
                  void** handle);
/* sizes[0..12] = n_blocks, n_elems, color_ofs_len, total_local_nodes, n_shared,
 * n_partials, max_local_nodes, max_block_colors, stride, n_affine_blocks,
 * n_diag_blocks, max_block_elems, n_lattice_blocks.  Local node l of a block lives in shared-memory
 * slot lnode_smem[l] < 8 ceil(L_b / 8), chosen so that the nodes one quarter-warp
 * reads at an element corner fall in distinct bank quads; lconn stores slots.   */
TG_API int tg_plan_sizes(const void* handle, int64_t* sizes);
TG_API int tg_plan_export(const void* handle, int32_t* blk_elem_ptr, int32_t* blk_color_ptr,
                   int32_t* color_ofs, int32_t* blk_node_ptr, uint16_t* lconn,
                   int32_t* elem_id, int32_t* lnode_gid, int32_t* lnode_slot,
                   int32_t* lnode_smem, int32_t* shared_node, int32_t* shared_ptr,
                   int32_t* shared_slots);
TG_API void tg_plan_free(void* handle);
/* HOST: is a Hex8 mesh a structured brick?  nodes[3] = (Nx, Ny, Nz) and h[3] = the
 * spacing per axis when node n sits at (X[i], Y[j], Z[k]) for n = i + Nx (j + Ny k),
 * the spacing along each axis is uniform (to 1e-13 relative), and the elements are the
 * (Nx-1)(Ny-1)(Nz-1) cells, each once, with the corner order of the reference
 * Hexahedron8 (tatva/element/base.py:478-491); nodes = (0, 0, 0) otherwise.  The
 * result goes into tg_block_plan.grid_nodes / grid_h.  No reference counterpart: it
 * selects the stencil schedule of the same HVP (jax.jvp(jax.grad(E)), README.md:93). */
TG_API int tg_grid_detect(int elem, const int32_t* conn, int64_t n_elems, int64_t n_nodes,
                          const double* coords, int dim, int32_t* nodes, double* h);
/* Fill box_geom32 (device, 3 * n_elems floats) from FP32 coordinates and the int32
 * connectivity; identical in every bit to what the kernel derives from coordinates. */
TG_API int tg_plan_box_geometry(const tg_block_plan* plan, const float* coords, const int32_t* conn,
                                float* out, void* stream);

/* y = mode(u, v) over the plan:
 *   RESIDUAL  y = dE/du (u)               v unused
 *   HVP       y = d2E/du2 (u) . v         u unused for linear laws (may be NULL)
 *   DIAG      y = diag d2E/du2 (u)        v unused
 * fixed (optional, (n_nodes*V) uint8): Dirichlet mask with the semantics of
 * Lifter.reduce_adjoint/Fixed (tatva/lifter/base.py:235-251,
 * lifter/constraints.py:312-318): inputs v are read as 0 on fixed dofs and the
 * output on fixed dofs is 0 (RESIDUAL), v (HVP, identity block) or 1 (DIAG).
 * coords must have precision prec.  Workspace: tg_apply_workspace_bytes.
 * Entries of y that belong to nodes no element references are not written.      */
TG_API size_t tg_apply_workspace_bytes(int elem, int prec, int mat_kind, const tg_block_plan* plan);
TG_API int tg_apply(int elem, int prec, int mode, const tg_material* mat, const tg_block_plan* plan,
             const void* coords, int64_t n_nodes, const void* u, const void* v,
             const uint8_t* fixed, void* y, void* workspace, size_t workspace_bytes,
             void* stream);
/* tg_apply without a workspace argument, for callers that may not allocate device
 * memory (a custom call running inside a runtime that owns the device heap, or a
 * loop where cudaMalloc's device synchronisation is not acceptable).  No counterpart
 * in the reference: it exists only for this C ABI.  The partial slots live in one
 * fixed array of TG_NOALLOC_SCRATCH_BYTES per device inside the library; plans whose
 * tg_apply_workspace_bytes exceed it are rejected with TG_ERR_WORKSPACE.  Nothing in
 * the array needs to start at zero (each slot is written before it is read).  The
 * first call in a CUDA context looks the array's address up and caches it under the
 * context's id (a device reset gives a new context and a fresh lookup): make that
 * call before any stream capture.  Calls that overlap on the GPU share the array and
 * race; calls ordered on one stream are safe.  Allocates nothing.              */
#define TG_NOALLOC_SCRATCH_BYTES (8u << 20)
TG_API int tg_apply_noalloc(int elem, int prec, int mode, const tg_material* mat,
                            const tg_block_plan* plan, const void* coords, int64_t n_nodes,
                            const void* u, const void* v, const uint8_t* fixed, void* y,
                            void* stream);
/* Per-element energies (n_elems,) in original element order (E(u) before the sum). */
TG_API int tg_energy_per_element(int elem, int prec, const tg_material* mat, const void* coords,
                          int64_t n_nodes, const int32_t* conn, int64_t n_elems,
                          const void* u, void* out, void* stream);

/* ============================================================================
 * Batched solves: many independent SPD systems (one per mesh) in one persistent
 * launch.  No single counterpart in the reference, where a user loops over meshes
 * and calls jax.scipy.sparse.linalg.cg per mesh (README.md:93) on the matrix that
 * tatva.sparse.jacfwd assembles (tatva/sparse/base.py:139-176).
 *
 * The systems are the diagonal blocks of one block-diagonal CSR matrix (rows
 * row_ofs[s] .. row_ofs[s+1]-1 couple only among themselves), stored per system as
 * column-major ELLPACK of width ell_width[s] starting at entry ell_ofs[s]: entry k of
 * local row i at ell_ofs[s] + k * n_s + i, 16-bit local column ids, padding entries
 * (value 0) point at the row itself.                                          */
typedef struct tg_batch_desc {
  int32_t n_systems;
  int32_t max_rows;           /* largest n_s (<= 49152) */
  const int64_t* row_ofs;     /* (n_systems + 1) */
  const int64_t* ell_ofs;     /* (n_systems) */
  const int32_t* ell_width;   /* (n_systems) */
  const int32_t* order;       /* (n_systems) order in which CTAs take systems */
  const uint16_t* ell_col;
  const float* ell_val32;
  const double* ell_val64;
} tg_batch_desc;
/* Fill ell_col / ell_val32 / ell_val64 (written through the descriptor's pointers)
 * from the block-diagonal CSR (int32 indptr/indices, FP64 data).  *bad_flag (device
 * int, zeroed by the caller) becomes 1 when a row is longer than its system's width
 * and 2 when a row couples to another system.                                  */
TG_API int tg_batch_ell_from_csr(const tg_batch_desc* desc, int64_t n_rows, const int32_t* indptr,
                                 const int32_t* indices, const double* data, int32_t* bad_flag,
                                 void* stream);
TG_API size_t tg_batch_workspace_bytes(int64_t n_rows);
/* Solve A_s x_s = b_s for every system (x overwritten, starting from 0): FP32
 * Jacobi-CG inner solves on r64/|r64| to inner_rtol, FP64 refinement on the true
 * residual until |b - A64 x| <= rtol |b|.  One CTA of `threads` (128, 256, 512)
 * threads per system at a time, at most ctas_per_sm CTAs per SM (0: as many as fit).
 * Per system (device arrays): total inner iterations, refinements, final relative
 * residual, status (TG_OK, TG_ERR_NOT_CONVERGED, TG_ERR_BREAKDOWN, TG_ERR_VALUE).
 * The result of a system does not depend on the other systems in the batch.    */
TG_API int tg_batch_solve(const tg_batch_desc* desc, int64_t n_rows, const double* b, double* x,
                          double rtol, double inner_rtol, int max_outer, int max_inner,
                          int threads, int ctas_per_sm, void* workspace, size_t workspace_bytes,
                          int32_t* iters, int32_t* outer, double* rel_res, int32_t* status,
                          void* stream);

/* ============================================================================
 * Colored compressed Hessian (K6) and CSR decompression.  Replaces
 * tatva/sparse/base.py compute_rows_cols (:108-136), colored_jacobian_batch
 * (:230-270) and the decompression data = Jc[rows, col_colors] of jacfwd /
 * linearized_jacfwd (:173, :224).
 * ========================================================================== */

/* Jc (n_nodes*V, n_colors) row-major, overwritten:
 *   Jc[i, c] = sum_{j : dof_colors[j] == c} H[i, j],  H = d2E/du2(u)
 * computed from element tangents: each node's rows sum the row blocks of its
 * incident (element, corner) pairs in the order of the incidence CSR inc_ptr /
 * inc_idx (tg_node_incidence, device copies): deterministic.  Decompression
 * (tg_decompress) needs dof_colors to be a distance-2 colouring (each colour at
 * most once per row of the pattern).                                             */
TG_API int tg_compressed_hessian(int elem, int prec, const tg_material* mat, const void* coords,
                          int64_t n_nodes, const int32_t* conn, int64_t n_elems,
                          const void* u, const int32_t* inc_ptr, const int32_t* inc_idx,
                          const int32_t* dof_colors, int n_colors, void* Jc, void* stream);
/* rows[k] = row of nonzero k; col_colors[k] = colors[indices[k]]   base.py:108-136 */
TG_API int tg_rows_cols(const int32_t* indptr, const int32_t* indices, const int32_t* colors,
                 int64_t n_rows, int64_t nnz, int32_t* rows, int32_t* col_colors,
                 void* stream);
/* data[k] = Jc[rows[k], col_colors[k]]                              base.py:173 */
TG_API int tg_decompress(int prec, const void* Jc, int n_colors, const int32_t* rows,
                  const int32_t* col_colors, int64_t nnz, void* data, void* stream);
/* seeds (nc, n): seeds[j, i] = (colors[i] == c0 + j) ? 1 : 0         base.py:259 */
TG_API int tg_color_seeds(int prec, const int32_t* colors, int64_t n, int c0, int nc, void* seeds,
                   void* stream);
/* Jc[:, c] = col  (assemble one compressed column from a JVP)      base.py:268-270 */
TG_API int tg_set_column(int prec, const void* col, int64_t n, int n_colors, int c, void* Jc,
                  void* stream);

/* ============================================================================
 * Sparse / vector kernels (K7, K8) for solvers composed on top of the path
 * (the reference has no solver; users call jax.scipy.sparse.linalg.cg).
 * ========================================================================== */

/* y = A x, CSR (int32 indptr/indices), data/x/y of precision prec */
TG_API int tg_spmv(int prec, int64_t n_rows, const int32_t* indptr, const int32_t* indices,
            const void* data, const void* x, void* y, void* stream);
/* Node blocks of a CSR matrix with 3 dofs per node (pattern_from_mesh with
 * n_dofs_per_node = 3, dof = 3 node + c, sparse/_extraction.py:57-60): the three rows
 * of node i list the same neighbour nodes, each as 3 consecutive columns.  Writes
 * node_ptr[n_rows/3 + 1] and node_indices[nnz/9] (neighbour node ids); sets the
 * device int *not_blocked to 1 if the pattern has another form (leaves it otherwise).
 * Device buffers; n_rows must be a multiple of 3.                               */
TG_API int tg_csr_node_blocks3(int64_t n_rows, const int32_t* indptr, const int32_t* indices,
                               int32_t* node_ptr, int32_t* node_indices, int32_t* not_blocked,
                               void* stream);
/* y = A x over the node blocks of tg_csr_node_blocks3: reads one neighbour id per
 * 3 x 3 block instead of one column index per entry; data stays in CSR order.   */
TG_API int tg_spmv_blocks3(int prec, int64_t n_rows, const int32_t* indptr,
                           const int32_t* node_ptr, const int32_t* node_indices,
                           const void* data, const void* x, void* y, void* stream);
/* CSR diagonal (Jacobi) */
TG_API int tg_csr_diagonal(int prec, int64_t n_rows, const int32_t* indptr, const int32_t* indices,
                    const void* data, void* diag, void* stream);
/* out_dev[0] = sum x_i y_i accumulated in FP64, deterministic (fixed partition
 * and tree order independent of the GPU).  out_dev is a device double.  x and y
 * are read with 16-byte vector loads: both must be 16-byte aligned, else
 * TG_ERR_VALUE (a slice at an odd element offset must be copied first).      */
TG_API size_t tg_dot_workspace_bytes(void);
TG_API int tg_dot(int prec, const void* x, const void* y, int64_t n, double* out_dev,
           void* workspace, size_t workspace_bytes, void* stream);
/* y = a*x + b*y (a, b host doubles) */
TG_API int tg_axpby(int prec, int64_t n, double a, const void* x, double b, void* y, void* stream);
/* out = in converted to prec_out */
TG_API int tg_convert(int prec_in, const void* in, int prec_out, void* out, int64_t n, void* stream);

/* Solver statistics (filled by the solve entry points). */
typedef struct tg_solve_stats {
  int32_t status;       /* TG_OK / TG_ERR_NOT_CONVERGED / TG_ERR_BREAKDOWN */
  int32_t iterations;   /* total (inner) CG iterations                      */
  int32_t outer;        /* refinement steps (mixed solve)                   */
  int32_t reserved;
  double rel_res;       /* final FP64 true relative residual ||b-Ax||/||b|| */
} tg_solve_stats;

/* Description of an operator A: either matrix-free, A = d2E/du2(u) restricted by
 * the Dirichlet mask (tg_apply in HVP mode), or, when csr_data != NULL, an
 * assembled CSR matrix of n_rows rows (Dirichlet rows/columns already applied
 * with tg_csr_apply_dirichlet).                                              */
typedef struct tg_operator_desc {
  int32_t elem;
  int32_t prec;
  tg_material mat;
  const tg_block_plan* plan;
  const void* coords;    /* precision prec */
  int64_t n_nodes;
  const void* u;         /* linearisation point (nonlinear laws), precision prec */
  const uint8_t* fixed;  /* Dirichlet mask or NULL */
  int64_t n_rows;
  const int32_t* csr_indptr;
  const int32_t* csr_indices;
  const void* csr_data;  /* precision prec */
  /* optional node blocks of the CSR pattern (tg_csr_node_blocks3); when both are
   * set the SpMV is tg_spmv_blocks3                                              */
  const int32_t* csr_node_ptr;
  const int32_t* csr_node_indices;
} tg_operator_desc;

/* Dirichlet rows/columns of an assembled matrix: for fixed rows data = (col == row);
 * entries in fixed columns of free rows are zeroed.                          */
TG_API int tg_csr_apply_dirichlet(int prec, int64_t n_rows, const int32_t* indptr,
                           const int32_t* indices, const uint8_t* fixed, void* data,
                           void* stream);
/* y = A x for an operator description (one HVP or SpMV).                    */
TG_API size_t tg_operator_workspace_bytes(const tg_operator_desc* op);
TG_API int tg_operator_apply(const tg_operator_desc* op, const void* x, void* y, void* workspace,
                      size_t workspace_bytes, void* stream);

/* Jacobi-preconditioned CG, all vectors of precision op->prec, scalars and dot
 * products in FP64 on the device.  Solves A x = b from the given x.  The loop runs
 * `check_every` iterations per CUDA graph replay between host convergence checks
 * and never exceeds max_iter; the stopping test itself runs on the device after
 * every iteration, so the result does not depend on check_every.  On a structured
 * brick with a Dirichlet mask, x is set to b on the fixed dofs first (the identity
 * rows of the masked system).  b and x must be 16-byte aligned (vector loads and
 * stores), else TG_ERR_VALUE.                                                  */
TG_API size_t tg_cg_workspace_bytes(const tg_operator_desc* op);
TG_API int tg_cg_solve(const tg_operator_desc* op, const void* b, void* x, const void* diag,
                double rtol, int max_iter, int check_every, void* workspace,
                size_t workspace_bytes, tg_solve_stats* stats, void* stream);

/* Mixed precision: FP32 Jacobi-CG inner solves on op32 (FP32 HVP, FP64 dots),
 * FP64 iterative refinement with the true residual r = b - A64 x on op64.
 * b, x, diag64 are FP64; converges to ||b - A64 x|| <= rtol ||b||.  b must be
 * 16-byte aligned (vector loads), else TG_ERR_VALUE.  Each inner solve reduces its
 * residual by inner_rtol (less on the last one).  inner_rtol >= 0.01: reliable
 * updates, the inner CG keeps its search direction across the FP64 residual
 * replacements (re-orthogonalised against the new residual; 0.1 recommended);
 * smaller values restart the inner CG at every refinement.  max_outer bounds the
 * replacements.                                                               */
TG_API size_t tg_mixed_workspace_bytes(const tg_operator_desc* op64, const tg_operator_desc* op32);
TG_API int tg_mixed_solve(const tg_operator_desc* op64, const tg_operator_desc* op32,
                   const double* b, double* x, const double* diag64, double rtol,
                   double inner_rtol, int max_outer, int max_inner, int check_every,
                   void* workspace, size_t workspace_bytes, tg_solve_stats* stats,
                   void* stream);

/* ============================================================================
 * Continuous batching of structured-brick solves (request loop).  No reference
 * counterpart: each request is the matrix-free solve of README.md:93 (FP32 grid
 * HVP inner Jacobi-CG, FP64 refinement on the true residual, as tg_mixed_solve on
 * a brick), and up to TG_BRICK_MAX_SLOTS of them advance together, one launch per
 * CG step for all.  A request's result is bitwise the same alone and in any mix.
 * ========================================================================== */
#define TG_BRICK_MAX_SLOTS 64
/* slot phases */
#define TG_BRICK_FREE 0
#define TG_BRICK_REFINE 1 /* FP64 residual / restart pending */
#define TG_BRICK_RUN 2    /* inner FP32 CG running */
#define TG_BRICK_DONE 3   /* converged: status TG_OK */
#define TG_BRICK_FAILED 4 /* status TG_ERR_NOT_CONVERGED or TG_ERR_BREAKDOWN */

/* A linear-elastic Hex8 brick of nodes[0] x nodes[1] x nodes[2] nodes, node id
 * i + nx (j + ny k), corner order of tatva/element/base.py:478-491, spacings h,
 * Lame parameters mu, lam.  b: FP64 right-hand side (3 dofs per node, interleaved);
 * x: FP64 solution (written: zero at admission, then the iterate); fixed: one byte
 * per dof, nonzero = Dirichlet (identity row, value 0), or NULL.  b, x and fixed
 * stay owned by the caller and must live until the slot is polled DONE / FAILED;
 * workspace: tg_brick_workspace_bytes(nodes) bytes, 256-byte aligned, likewise.
 * Converges to ||b - A x|| <= rtol ||b||; each inner solve stops at relative
 * residual inner_rtol or max_inner iterations; at most max_outer inner solves.   */
typedef struct tg_brick_request {
  int32_t nodes[3];
  int32_t reserved;
  double h[3];
  double mu, lam;
  const double* b;
  double* x;
  const uint8_t* fixed;
  void* workspace;
  size_t workspace_bytes;
  double rtol, inner_rtol;
  int32_t max_outer, max_inner;
} tg_brick_request;

typedef struct tg_brick_state {
  int32_t phase;      /* TG_BRICK_* */
  int32_t status;     /* TG_OK / TG_ERR_NOT_CONVERGED / TG_ERR_BREAKDOWN when finished */
  int32_t iterations; /* inner CG iterations so far */
  int32_t outer;      /* inner solves started */
  double rel_res;     /* ||b - A x|| / ||b|| at the last refinement */
} tg_brick_state;

typedef struct tg_brick_batch tg_brick_batch;

/* The batch belongs to the current device; create / destroy allocate and free its
 * slot table (not hot calls).                                                   */
TG_API int tg_brick_batch_create(tg_brick_batch** out);
TG_API void tg_brick_batch_destroy(tg_brick_batch* batch);
TG_API size_t tg_brick_workspace_bytes(const int32_t nodes[3]);
/* Takes the lowest free slot (TG_ERR_VALUE when all are taken); the solve starts
 * at the next tg_brick_step.  Stream-ordered: the slot is written after the work
 * already queued on `stream`.                                                   */
TG_API int tg_brick_admit(tg_brick_batch* batch, const tg_brick_request* req, void* stream,
                          int* slot);
/* Enqueues one step for every slot in use: the refinement launches, then
 * `iterations` CG steps (three launches each).  Does not synchronize.  The step is
 * captured as a CUDA graph and replayed while the slots in use and `iterations`
 * stay the same (a stream that cannot be captured gets plain launches).         */
TG_API int tg_brick_step(tg_brick_batch* batch, int iterations, void* stream);
/* Synchronizes `stream` and writes the state of all TG_BRICK_MAX_SLOTS slots to
 * out (n_out >= TG_BRICK_MAX_SLOTS); slots reported DONE or FAILED are released
 * (reported once, FREE afterwards).                                             */
TG_API int tg_brick_poll(tg_brick_batch* batch, tg_brick_state* out, int n_out, void* stream);

/* ============================================================================
 * HOST setup (H1).  Replaces tatva/sparse/_extraction.py _create_sparse_structure
 * / pattern_from_mesh (:37-102), tatva_coloring.distance2_colors as restated by
 * tatva/sparse/_coloring.py (:27-48, :136-153, :270-283).
 * ========================================================================== */

/* CSR pattern of the dof-level matrix, identical (bit-exact) to
 * _create_sparse_structure: rows/cols sorted, dof = node*ndpn + comp.        */
TG_API int tg_pattern_build(const int32_t* conn, int64_t n_elems, int nodes_per_elem,
                     int64_t n_nodes, int n_dofs_per_node, void** handle);
TG_API int tg_pattern_nnz(const void* handle, int64_t* nnz);
TG_API int tg_pattern_export(const void* handle, int32_t* indptr, int32_t* indices);
TG_API void tg_pattern_free(void* handle);

/* Natural-order greedy distance-2 colouring of the CSR pattern (A @ A
 * neighbourhoods; smallest unused colour), bit-exact with
 * tatva/sparse/_coloring.py greedy_coloring(get_distance2_adjacency(...)).    */
TG_API int tg_distance2_colors(const int32_t* indptr, const int32_t* indices, int64_t n,
                        int32_t* colors, int32_t* n_colors);

/* Greedy natural-order element colouring (elements sharing a node differ).
 * order (n_elems): elements sorted by colour (stable); color_ptr (<= 129).   */
TG_API int tg_element_colors(const int32_t* conn, int64_t n_elems, int nodes_per_elem,
                      int64_t n_nodes, int32_t* colors, int32_t* order,
                      int32_t* color_ptr, int32_t* n_colors);

/* node -> (e*nodes_per_elem + a) incidence CSR, entries in increasing e.    */
TG_API int tg_node_incidence(const int32_t* conn, int64_t n_elems, int nodes_per_elem,
                      int64_t n_nodes, int32_t* ptr, int32_t* idx);

#ifdef __cplusplus
}
#endif
#endif /* TATVA_GB300_H */
