// Host-side dispatch from the C ABI's runtime enums to template instantiations.
#pragma once

#include <type_traits>

#include "tg_common.cuh"

namespace tg {

template <int V>
using IntC = std::integral_constant<int, V>;

template <class F>
int dispatch_elem(int elem, F&& f) {
  switch (elem) {
    case TG_TRI3: return f(IntC<TG_TRI3>{});
    case TG_TET4: return f(IntC<TG_TET4>{});
    case TG_HEX8: return f(IntC<TG_HEX8>{});
    default: return set_error(TG_ERR_VALUE, "unknown element type %d", elem);
  }
}

template <class F>
int dispatch_prec(int prec, F&& f) {
  switch (prec) {
    case TG_F32: return f(float{});
    case TG_F64: return f(double{});
    default: return set_error(TG_ERR_TYPE, "unknown precision %d", prec);
  }
}

inline int check_ptr(const void* p, const char* name) {
  if (p == nullptr) return set_error(TG_ERR_VALUE, "%s must not be NULL", name);
  return TG_OK;
}

inline int check_sizes(int64_t n_elems, int64_t n_nodes, int n_vals) {
  if (n_elems < 0 || n_nodes < 0) return set_error(TG_ERR_VALUE, "negative size");
  if (n_vals <= 0) return set_error(TG_ERR_VALUE, "n_vals must be positive");
  if (n_elems > INT32_MAX || n_nodes > INT32_MAX)
    return set_error(TG_ERR_VALUE, "sizes above 2^31-1 are not supported");
  return TG_OK;
}

}  // namespace tg
