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
// First call on a device: the array's device address is looked up with
// cudaGetSymbolAddress, with that device current, and cached per device.  That lookup
// (and the lazy load of the library's device code it can trigger) is set-up work, so
// make the first call on each device before any stream capture begins.
#include <mutex>

#include "tg_common.cuh"

namespace tg {
namespace {

constexpr int kMaxDevices = 64;

// 8 MiB of partial slots: 2M FP32 or 1M FP64 values.
static __device__ __align__(256) unsigned char g_noalloc_scratch[TG_NOALLOC_SCRATCH_BYTES];

std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

// Returns the scratch address on the current device, looking it up on first use.
int scratch_on_current_device(void** out) {
  int dev = -1;
  TG_TRY(cuda_check(cudaGetDevice(&dev), "tg_apply_noalloc: cudaGetDevice"));
  if (dev < 0 || dev >= kMaxDevices)
    return set_error(TG_ERR_UNSUPPORTED, "tg_apply_noalloc: device ordinal %d >= %d", dev,
                     kMaxDevices);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    TG_TRY(cuda_check(cudaGetSymbolAddress(&p, g_noalloc_scratch),
                      "tg_apply_noalloc: cudaGetSymbolAddress of the scratch array"));
    if (!p) return set_error(TG_ERR_CUDA, "tg_apply_noalloc: scratch array has no address");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
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
