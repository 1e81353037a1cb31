// Entry points shared between translation units of the library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>

#include "tatva_gb300.h"

namespace tg {

// FP32 linear-elastic Hex8 residual / HVP over the plan's all-parallelepiped blocks
// [0, n_affine_blocks); returns TG_ERR_UNSUPPORTED (nothing launched) when the plan
// does not fit the kernel's staging limits.
int launch_hex_le_f32x2(const tg_block_plan* plan, int mode, const float* coords, const float* u,
                        const float* v, const uint8_t* fixed, float* y, float* partials,
                        float mu, float lam, cudaStream_t st);

// Linear-elastic Hex8 residual / HVP on a structured brick (plan->grid_nodes set) as a
// stencil over the grid; TG_ERR_UNSUPPORTED (nothing launched) for other modes or plans.
int launch_grid_le(const tg_block_plan* plan, int prec, int mode, const void* u, const void* v,
                   const uint8_t* fixed, void* y, double mu, double lam, cudaStream_t st);

// HVP q = A p on a structured brick with the CG dot: alpha = rz / (p . q) into scal
// (SCAL_* slots of the CG), through per-CTA partials in part (grid_cg_ctas(plan)
// doubles) and a zeroed arrival counter ticket.
int64_t grid_cg_ctas(const tg_block_plan* plan);
// node_mask: NULL, or one byte per node, bit d set when dof 3 n + d is fixed
// (pack_node_mask from the C ABI's per-dof mask).
int launch_grid_hvp_dot(const tg_block_plan* plan, int prec, double mu, double lam,
                        const void* p, const uint8_t* node_mask, void* q, double* scal,
                        double* part, unsigned* ticket, cudaStream_t st);
int pack_node_mask(const uint8_t* fixed, int64_t n_nodes, uint8_t* out, cudaStream_t st);
// x = b and dinv = 0 on the fixed dofs of a packed node mask (the grid CG)
int grid_cg_fixed(int prec, int64_t n_nodes, const uint8_t* nmask, const void* b, void* x,
                  void* dinv, cudaStream_t st);

}  // namespace tg
