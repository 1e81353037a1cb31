// Shared device code: element traits, per-quadrature-point geometry, error helpers.
//
// Element tables follow tatva/element/base.py:
//   Tri3          base.py:245-265   N = [1-x-y, x, y], 1-point rule (1/3,1/3), w = 1/2
//   Tetrahedron4  base.py:448-472   N = [1-x-y-z, x, y, z], 1-point rule (1/4,..), w = 1/6
//   Hexahedron8   base.py:475-568   trilinear, nodes in the order of :478-491,
//                                   2x2x2 Gauss at +-1/sqrt(3) in the order of :497-508
// Jacobian J = dN/dxi @ X (J[i][j] = dx_j/dxi_i), dN/dX = inv(J) @ dN/dxi
// (base.py:90-115).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tatva_gb300.h"

namespace tg {

// ---------------------------------------------------------------- errors (host)
int set_error(int code, const char* fmt, ...);
int cuda_check(cudaError_t e, const char* where);
inline int launch_check(const char* where) { return cuda_check(cudaGetLastError(), where); }
inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

#define TG_TRY(expr)              \
  do {                            \
    int _tg_rc = (expr);          \
    if (_tg_rc != TG_OK) return _tg_rc; \
  } while (0)

// 1/sqrt(3) exactly as the reference evaluates it in FP64 (1 / jnp.sqrt(3)).
constexpr double HEX_GAUSS = 0x1.279a74590331dp-1;

constexpr int grid_for(int64_t n, int block) {
  return (int)((n + block - 1) / block);
}

// ---------------------------------------------------------------- element traits
template <int ET>
struct Elem;

template <>
struct Elem<TG_TRI3> {
  static constexpr int NN = 3, D = 2, Q = 1, NPAD = 4;
  static constexpr bool SIMPLEX = true;
  template <class T>
  __host__ __device__ static T w(int) { return T(0.5); }
  template <class T>
  __host__ __device__ static T N(int, int a) {
    const T t = T(1.0 / 3);
    return a == 0 ? (T(1) - t - t) : t;
  }
  // dN/dxi_i of node a (constant)
  template <class T>
  __host__ __device__ static T dN(int, int i, int a) {
    return a == 0 ? T(-1) : ((a - 1) == i ? T(1) : T(0));
  }
};

template <>
struct Elem<TG_TET4> {
  static constexpr int NN = 4, D = 3, Q = 1, NPAD = 4;
  static constexpr bool SIMPLEX = true;
  template <class T>
  __host__ __device__ static T w(int) { return T(1.0 / 6); }
  template <class T>
  __host__ __device__ static T N(int, int a) {
    const T t = T(1.0 / 4);
    return a == 0 ? (T(1) - t - t - t) : t;
  }
  template <class T>
  __host__ __device__ static T dN(int, int i, int a) {
    return a == 0 ? T(-1) : ((a - 1) == i ? T(1) : T(0));
  }
};

template <>
struct Elem<TG_HEX8> {
  static constexpr int NN = 8, D = 3, Q = 8, NPAD = 8;
  static constexpr bool SIMPLEX = false;
  // sign of reference coordinate i of node a (base.py:478-491); QPs use the same
  // sign pattern scaled by 1/sqrt(3) (base.py:497-508).
  __host__ __device__ static constexpr int s(int a, int i) {
    return i == 0 ? (((a & 3) == 1 || (a & 3) == 2) ? 1 : -1)
                  : (i == 1 ? (((a & 3) >= 2) ? 1 : -1) : (a >= 4 ? 1 : -1));
  }
  template <class T>
  __host__ __device__ static T w(int) { return T(1); }
  // factor (1 +- xi_i) of node a at quadrature point q
  template <class T>
  __host__ __device__ static T f(int q, int a, int i) {
    const T g = T(HEX_GAUSS);
    return s(a, i) * s(q, i) > 0 ? T(1) + g : T(1) - g;
  }
  template <class T>
  __host__ __device__ static T N(int q, int a) {
    return T(0.125) * (f<T>(q, a, 0) * f<T>(q, a, 1) * f<T>(q, a, 2));
  }
  template <class T>
  __host__ __device__ static T dN(int q, int i, int a) {
    const int j = (i == 0) ? 1 : 0;
    const int k = (i == 2) ? 1 : 2;
    return T(0.125) * (T(s(a, i)) * (f<T>(q, a, j) * f<T>(q, a, k)));
  }
};

// ---------------------------------------------------------------- small linear algebra
template <class T>
__device__ __forceinline__ T inv2(const T (&J)[2][2], T (&Ji)[2][2]) {
  const T det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
  const T r = T(1) / det;
  Ji[0][0] = J[1][1] * r;
  Ji[0][1] = -J[0][1] * r;
  Ji[1][0] = -J[1][0] * r;
  Ji[1][1] = J[0][0] * r;
  return det;
}

template <class T>
__device__ __forceinline__ T inv3(const T (&J)[3][3], T (&Ji)[3][3]) {
  const T c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
  const T c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
  const T c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
  const T det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
  const T r = T(1) / det;
  Ji[0][0] = c00 * r;
  Ji[1][0] = c01 * r;
  Ji[2][0] = c02 * r;
  Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * r;
  Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * r;
  Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * r;
  Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * r;
  Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * r;
  Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * r;
  return det;
}

template <class T, int D>
__device__ __forceinline__ T invD(const T (&J)[D][D], T (&Ji)[D][D]);
template <>
__device__ __forceinline__ float invD<float, 2>(const float (&J)[2][2], float (&Ji)[2][2]) { return inv2(J, Ji); }
template <>
__device__ __forceinline__ double invD<double, 2>(const double (&J)[2][2], double (&Ji)[2][2]) { return inv2(J, Ji); }
template <>
__device__ __forceinline__ float invD<float, 3>(const float (&J)[3][3], float (&Ji)[3][3]) { return inv3(J, Ji); }
template <>
__device__ __forceinline__ double invD<double, 3>(const double (&J)[3][3], double (&Ji)[3][3]) { return inv3(J, Ji); }

// Physical shape-function gradients at quadrature point q:
// G[a][k] = dN_a/dx_k = sum_i inv(J)[k][i] dN_a/dxi_i; returns det(J).
template <int ET, class T>
__device__ __forceinline__ T qp_geometry(int q, const T (&X)[Elem<ET>::NN][Elem<ET>::D],
                                         T (&G)[Elem<ET>::NN][Elem<ET>::D]) {
  using E = Elem<ET>;
  constexpr int NN = E::NN, D = E::D;
  T J[D][D];
  if constexpr (E::SIMPLEX) {
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) J[i][j] = X[i + 1][j] - X[0][j];
  } else {
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        T acc = T(0);
#pragma unroll
        for (int a = 0; a < NN; ++a) acc += E::template dN<T>(q, i, a) * X[a][j];
        J[i][j] = acc;
      }
  }
  T Ji[D][D];
  const T det = invD<T, D>(J, Ji);
  if constexpr (E::SIMPLEX) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      T s0 = T(0);
#pragma unroll
      for (int i = 0; i < D; ++i) {
        G[i + 1][k] = Ji[k][i];
        s0 -= Ji[k][i];
      }
      G[0][k] = s0;
    }
  } else {
#pragma unroll
    for (int a = 0; a < NN; ++a)
#pragma unroll
      for (int k = 0; k < D; ++k) {
        T acc = T(0);
#pragma unroll
        for (int i = 0; i < D; ++i) acc += Ji[k][i] * E::template dN<T>(q, i, a);
        G[a][k] = acc;
      }
  }
  return det;
}

// ---------------------------------------------------------------- vector loads of lconn
template <int NPAD>
__device__ __forceinline__ void load_lconn(const uint16_t* __restrict__ p, int (&l)[NPAD]);
template <>
__device__ __forceinline__ void load_lconn<4>(const uint16_t* __restrict__ p, int (&l)[4]) {
  const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
  l[0] = v.x & 0xffff; l[1] = v.x >> 16; l[2] = v.y & 0xffff; l[3] = v.y >> 16;
}
template <>
__device__ __forceinline__ void load_lconn<8>(const uint16_t* __restrict__ p, int (&l)[8]) {
  const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
  l[0] = v.x & 0xffff; l[1] = v.x >> 16; l[2] = v.y & 0xffff; l[3] = v.y >> 16;
  l[4] = v.z & 0xffff; l[5] = v.z >> 16; l[6] = v.w & 0xffff; l[7] = v.w >> 16;
}

// The packed row as loaded (one 8- or 16-byte load), for a load issued well before
// the row is unpacked (the next chunk's row, fetched while this chunk computes).
template <int NPAD>
struct LconnRaw;
template <>
struct LconnRaw<4> {
  uint2 v;
  __device__ __forceinline__ void load(const uint16_t* __restrict__ p) {
    v = __ldg(reinterpret_cast<const uint2*>(p));
  }
  __device__ __forceinline__ void unpack(int (&l)[4]) const {
    l[0] = v.x & 0xffff; l[1] = v.x >> 16; l[2] = v.y & 0xffff; l[3] = v.y >> 16;
  }
};
template <>
struct LconnRaw<8> {
  uint4 v;
  __device__ __forceinline__ void load(const uint16_t* __restrict__ p) {
    v = __ldg(reinterpret_cast<const uint4*>(p));
  }
  __device__ __forceinline__ void unpack(int (&l)[8]) const {
    l[0] = v.x & 0xffff; l[1] = v.x >> 16; l[2] = v.y & 0xffff; l[3] = v.y >> 16;
    l[4] = v.z & 0xffff; l[5] = v.z >> 16; l[6] = v.w & 0xffff; l[7] = v.w >> 16;
  }
};

}  // namespace tg
