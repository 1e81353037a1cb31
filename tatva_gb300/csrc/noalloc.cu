// tg_apply_noalloc: the residual / HVP / diagonal of tg_apply with its scratch taken
// from a fixed array that lives in the library's own device image instead of a
// caller-provided workspace.
//
// Who needs it: callers that are not allowed to allocate device memory at the point
// where they run the operator.  Examples are a handler invoked from inside another
// runtime that owns the device heap (an XLA/JAX custom call, whose buffers all come
// from that runtime's pool and which must not grow the process's footprint behind its
// back), and latency-critical loops where cudaMalloc / cudaFree would synchronise the
// device and stall every stream in flight.  Such callers can pass tg_apply a workspace
// only if someone allocated one for them earlier; this entry point removes that need
// for plans whose scratch fits in TG_NOALLOC_SCRATCH_BYTES.
//
// The scratch holds the plan's partial slots (one value per dof of every node that
// several element blocks touch).  Every call writes each slot it reads before reading
// it, so nothing in the array has to start at zero and the previous call's leftovers
// never reach the result.  All calls in the process share the one array per device:
// two calls whose kernels overlap on the GPU (different streams, no ordering between
// them) race on it and give wrong results.  Calls issued on one stream are ordered and
// safe.
//
// First call in a CUDA context: the array's device address is looked up with
// cudaGetSymbolAddress, with that context's device current, and cached under the
// context's id (cuCtxGetId, reached through cudaGetDriverEntryPointByVersion, so the
// library needs no link to the driver library).  A device reset, or another context
// made current on the same device, has a new id: the next call looks the address up
// again instead of using one from a module that no longer exists.  That lookup (and
// the lazy load of the library's device code it can trigger) is set-up work, so make
// the first call on each device, and the first after a reset, before any stream
// capture begins.
#include <cuda.h>

#include <mutex>

#include "tg_common.cuh"

namespace tg {
namespace {

constexpr int kMaxDevices = 64;

// 8 MiB of partial slots: 2M FP32 or 1M FP64 values.
static __device__ __align__(256) unsigned char g_noalloc_scratch[TG_NOALLOC_SCRATCH_BYTES];

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

std::mutex g_setup_mutex;
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;
struct Cached {
  unsigned long long ctx_id;
  void* ptr;
};
Cached g_scratch[kMaxDevices] = {};

// Id of the context current on the calling thread (the primary context of `dev` after
// cudaGetDevice has made sure one exists).  Called with g_setup_mutex held.
int current_context_id(unsigned long long* id) {
  if (!g_ctx_current || !g_ctx_id) {
    void* f0 = nullptr;
    void* f1 = nullptr;
    cudaDriverEntryPointQueryResult q0, q1;
    TG_TRY(cuda_check(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000,
                                                       cudaEnableDefault, &q0),
                      "tg_apply_noalloc: driver entry point cuCtxGetCurrent"));
    TG_TRY(cuda_check(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000,
                                                       cudaEnableDefault, &q1),
                      "tg_apply_noalloc: driver entry point cuCtxGetId"));
    if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
      return set_error(TG_ERR_UNSUPPORTED,
                       "tg_apply_noalloc: the driver does not provide cuCtxGetCurrent / cuCtxGetId");
    g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f0);
    g_ctx_id = reinterpret_cast<CtxGetIdFn>(f1);
  }
  CUcontext ctx = nullptr;
  if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx)
    return set_error(TG_ERR_CUDA, "tg_apply_noalloc: no current CUDA context");
  if (g_ctx_id(ctx, id) != CUDA_SUCCESS)
    return set_error(TG_ERR_CUDA, "tg_apply_noalloc: cuCtxGetId failed");
  return TG_OK;
}

// Returns the scratch address in the current context, looking it up on first use in
// that context.
int scratch_on_current_device(void** out) {
  int dev = -1;
  TG_TRY(cuda_check(cudaGetDevice(&dev), "tg_apply_noalloc: cudaGetDevice"));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(TG_ERR_UNSUPPORTED, "tg_apply_noalloc: device ordinal %d >= %d", dev,
                     kMaxDevices);
  // re-selecting the current device makes its primary context current (CUDA >= 12
  // initialises it here) so that the context query below has one to name
  TG_TRY(cuda_check(cudaSetDevice(dev), "tg_apply_noalloc: cudaSetDevice"));
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  unsigned long long id = 0;
  TG_TRY(current_context_id(&id));
  if (!g_scratch[dev].ptr || g_scratch[dev].ctx_id != id) {
    void* p = nullptr;
    TG_TRY(cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                      "tg_apply_noalloc: cudaGetSymbolAddress of the scratch array"));
    if (!p) return set_error(TG_ERR_CUDA, "tg_apply_noalloc: scratch array has no address");
    g_scratch[dev] = Cached{id, p};
  }
  *out = g_scratch[dev].ptr;
  return TG_OK;
}

}  // namespace
}  // namespace tg

using namespace tg;

extern "C" int tg_apply_noalloc(int elem, int prec, int mode, const tg_material* mat,
                                const tg_block_plan* plan, const void* coords, int64_t n_nodes,
                                const void* u, const void* v, const uint8_t* fixed, void* y,
                                void* stream) {
  if (!plan) return set_error(TG_ERR_VALUE, "plan must not be NULL");
  if (plan->n_partials < 0) return set_error(TG_ERR_VALUE, "corrupt plan");
  if (!mat) return set_error(TG_ERR_VALUE, "mat must not be NULL");
  const size_t need = tg_apply_workspace_bytes(elem, prec, mat->kind, plan);
  if (need > (size_t)TG_NOALLOC_SCRATCH_BYTES)
    return set_error(TG_ERR_WORKSPACE,
                     "tg_apply_noalloc: plan needs %zu bytes of scratch for its %d shared-node "
                     "slots, above the fixed maximum of %zu bytes; use tg_apply with a "
                     "workspace of tg_apply_workspace_bytes()",
                     need, plan->n_partials, (size_t)TG_NOALLOC_SCRATCH_BYTES);
  void* scratch = nullptr;
  TG_TRY(scratch_on_current_device(&scratch));
  return tg_apply(elem, prec, mode, mat, plan, coords, n_nodes, u, v, fixed, y, scratch,
                  (size_t)TG_NOALLOC_SCRATCH_BYTES, stream);
}
