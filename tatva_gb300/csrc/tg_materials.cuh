// Material laws on the hot path, in closed form (the reference differentiates user
// JAX energies with jax.grad / jax.jvp; these are the same derivatives written out).
//
//   Poisson        psi = 1/2 kappa |H|^2 - f u                (H = grad u, V = 1)
//   LinearElastic  psi = 1/2 sigma:eps, eps = sym H, sigma = 2 mu eps + lambda tr(eps) I
//                  (tests/test_sparse.py:12-30, tests/test_sparse_benchmark.py:59-78)
//   NeoHookean     psi = mu/2 (I1 - 3 - 2 ln J) + lambda/2 (ln J)^2, F = I + H
//                  (tests/test_sparse_tracer.py:101-113)
//
// Each law provides: energy density, flux P = dpsi/dH, and a linearisation object
// whose dflux(dH) = d2psi/dH2 : dH (used for the HVP, the Jacobi diagonal and the
// element tangents).
#pragma once

#include "tg_common.cuh"

namespace tg {

template <int MAT, int D>
struct LawDims;
template <int D>
struct LawDims<TG_POISSON, D> { static constexpr int V = 1; };
template <int D>
struct LawDims<TG_LINEAR_ELASTIC, D> { static constexpr int V = D; };
template <int D>
struct LawDims<TG_NEO_HOOKEAN, D> { static constexpr int V = 3; };

template <int MAT, int D, class T>
struct Law;

// ------------------------------------------------------------------- Poisson
template <int D, class T>
struct Law<TG_POISSON, D, T> {
  static constexpr int V = 1;
  static constexpr bool LINEAR = true;
  T k, f;
  __device__ Law(T p0, T p1) : k(p0), f(p1) {}
  __device__ T energy(const T (&H)[1][D], T uq) const {
    T s = T(0);
#pragma unroll
    for (int d = 0; d < D; ++d) s += H[0][d] * H[0][d];
    return T(0.5) * k * s - f * uq;
  }
  __device__ void flux(const T (&H)[1][D], T (&P)[1][D]) const {
#pragma unroll
    for (int d = 0; d < D; ++d) P[0][d] = k * H[0][d];
  }
  struct Lin {
    T k;
    __device__ void dflux(const T (&dH)[1][D], T (&dP)[1][D]) const {
#pragma unroll
      for (int d = 0; d < D; ++d) dP[0][d] = k * dH[0][d];
    }
  };
  __device__ Lin linearize(const T (&)[1][D]) const { return Lin{k}; }
  __device__ T source() const { return f; }
};

// ------------------------------------------------------------------- linear elastic
template <int D, class T>
struct Law<TG_LINEAR_ELASTIC, D, T> {
  static constexpr int V = D;
  static constexpr bool LINEAR = true;
  T mu, lam;
  __device__ Law(T p0, T p1) : mu(p0), lam(p1) {}
  __device__ static void stress(T mu, T lam, const T (&H)[D][D], T (&P)[D][D]) {
    T tr = T(0);
#pragma unroll
    for (int i = 0; i < D; ++i) tr += H[i][i];
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) P[i][j] = mu * (H[i][j] + H[j][i]);
#pragma unroll
    for (int i = 0; i < D; ++i) P[i][i] += lam * tr;
  }
  __device__ T energy(const T (&H)[D][D], T) const {
    T ee = T(0), tr = T(0);
#pragma unroll
    for (int i = 0; i < D; ++i) {
      tr += H[i][i];
#pragma unroll
      for (int j = 0; j < D; ++j) {
        const T e = T(0.5) * (H[i][j] + H[j][i]);
        ee += e * e;
      }
    }
    return mu * ee + T(0.5) * lam * tr * tr;
  }
  __device__ void flux(const T (&H)[D][D], T (&P)[D][D]) const { stress(mu, lam, H, P); }
  struct Lin {
    T mu, lam;
    __device__ void dflux(const T (&dH)[D][D], T (&dP)[D][D]) const { stress(mu, lam, dH, dP); }
  };
  __device__ Lin linearize(const T (&)[D][D]) const { return Lin{mu, lam}; }
  __device__ T source() const { return T(0); }
};

// ------------------------------------------------------------------- Neo-Hookean (3D)
template <class T>
struct Law<TG_NEO_HOOKEAN, 3, T> {
  static constexpr int V = 3;
  static constexpr bool LINEAR = false;
  T mu, lam;
  __device__ Law(T p0, T p1) : mu(p0), lam(p1) {}
  __device__ static T deformation(const T (&H)[3][3], T (&F)[3][3], T (&FiT)[3][3]) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) F[i][j] = H[i][j] + (i == j ? T(1) : T(0));
    T Fi[3][3];
    const T J = inv3(F, Fi);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) FiT[i][j] = Fi[j][i];
    return J;
  }
  __device__ T energy(const T (&H)[3][3], T) const {
    T F[3][3], FiT[3][3];
    const T J = deformation(H, F, FiT);
    T I1 = T(0);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) I1 += F[i][j] * F[i][j];
    const T lnJ = log(J);
    return T(0.5) * mu * (I1 - T(3) - T(2) * lnJ) + T(0.5) * lam * lnJ * lnJ;
  }
  // P = mu (F - F^-T) + lambda ln J F^-T
  __device__ void flux(const T (&H)[3][3], T (&P)[3][3]) const {
    T F[3][3], FiT[3][3];
    const T J = deformation(H, F, FiT);
    const T c = lam * log(J);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) P[i][j] = mu * (F[i][j] - FiT[i][j]) + c * FiT[i][j];
  }
  // dP = mu dH + (mu - lambda ln J) F^-T dH^T F^-T + lambda tr(F^-1 dH) F^-T
  struct Lin {
    T mu, c1, lam;
    T FiT[3][3];
    __device__ void dflux(const T (&dH)[3][3], T (&dP)[3][3]) const {
      T tr = T(0);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) tr += FiT[a][b] * dH[a][b];
      // M = dH^T F^-T  -> M[b][J] = sum_a dH[a][b] FiT[a][J]
      T M[3][3];
#pragma unroll
      for (int b = 0; b < 3; ++b)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          T s = T(0);
#pragma unroll
          for (int a = 0; a < 3; ++a) s += dH[a][b] * FiT[a][j];
          M[b][j] = s;
        }
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          T s = T(0);
#pragma unroll
          for (int b = 0; b < 3; ++b) s += FiT[i][b] * M[b][j];
          dP[i][j] = mu * dH[i][j] + c1 * s + lam * tr * FiT[i][j];
        }
    }
  };
  __device__ Lin linearize(const T (&H)[3][3]) const {
    Lin L;
    T F[3][3];
    const T J = deformation(H, F, L.FiT);
    L.mu = mu;
    L.lam = lam;
    L.c1 = mu - lam * log(J);
    return L;
  }
  __device__ T source() const { return T(0); }
};

}  // namespace tg
