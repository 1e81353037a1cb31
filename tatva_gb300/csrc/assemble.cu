// Fused element assembly over an element-block plan: residual (K4), Hessian-vector
// product (K5) and Jacobi diagonal, for Tri3 / Tet4 / Hex8 and the Poisson, linear
// elastic and Neo-Hookean laws, in FP32 or FP64.
//
// Reference semantics: y = jax.grad(E)(u) and y = jax.jvp(jax.grad(E), (u,), (v,))[1]
// for E(u) = op.integrate(psi(op.grad(u))) (README.md:93, tatva/sparse/base.py:257-265),
// i.e. gather (operator.py:221) -> per-QP law -> scatter-add (XLA's transpose of the
// gather).
//
// Determinism without float atomics: every CTA owns one block of spatially compact
// elements and stages the block's nodes in shared memory.  It computes a chunk of
// elements (one per thread) into registers, then adds the chunk's results into shared
// memory colour by colour (no two elements of a colour share a node, so the adds do
// not race).  Last it writes the nodes it owns alone straight to y and the nodes
// shared with other blocks to partial-sum slots.  A second kernel adds each shared node's
// partials in the fixed slot order.  The summation order is fixed by the plan, so
// the result is bitwise reproducible.
//
// Hex8 fast path: for an affine (parallelepiped) element and a law that is quadratic
// in grad u (linear elasticity, Poisson), the 2x2x2 Gauss sum is evaluated exactly in
// the orthogonal monomial basis {1, x, y, z, yz, xz, xy} of grad u: the nodal values
// are taken to modal coefficients with an 8-point Walsh-Hadamard transform, the law is
// applied once per monomial (with the Gauss weight sum_q M(xi_q)^2 of that monomial),
// and the result returns through the transposed transform.  The Gauss rule integrates these
// products exactly, so the result equals the per-QP evaluation up to rounding, at
// roughly 1/8 of the flops.  Non-affine elements take the per-QP path.
#include <map>
#include <mutex>

#include "tg_common.cuh"
#include "tg_dispatch.cuh"
#include "tg_internal.h"
#include "tg_materials.cuh"

namespace tg {

constexpr int APPLY_MAX_THREADS = 256;
// nodes a thread stages (and writes back) per pass of the general block kernel; Tri3
// keeps one: its element is so small that the staging registers would set the
// occupancy
template <int ET>
constexpr int apply_sb() { return ET == TG_TRI3 ? 1 : 4; }



template <int ET, int MAT>
struct Supported {
  static constexpr bool value = !(MAT == TG_NEO_HOOKEAN && Elem<ET>::D != 3);
};

// ------------------------------------------------------------------ generic per-QP element
template <int ET, int MAT, class T, int MODE>
__device__ __forceinline__ void element_generic(
    const Law<MAT, Elem<ET>::D, T>& law, const T (&X)[Elem<ET>::NN][Elem<ET>::D],
    const T (&U)[Elem<ET>::NN][LawDims<MAT, Elem<ET>::D>::V],
    const T (&W)[Elem<ET>::NN][LawDims<MAT, Elem<ET>::D>::V],
    T (&Y)[Elem<ET>::NN][LawDims<MAT, Elem<ET>::D>::V]) {
  using E = Elem<ET>;
  using L = Law<MAT, E::D, T>;
  constexpr int NN = E::NN, D = E::D, V = L::V;
#pragma unroll
  for (int a = 0; a < NN; ++a)
#pragma unroll
    for (int i = 0; i < V; ++i) Y[a][i] = T(0);
  // Hex8: the eight quadrature points run as a loop (the per-point constants are a
  // few selects); unrolled, the Hex8 element held ~200 registers and two CTAs per SM
  constexpr int QUNROLL = (E::Q > 4) ? 1 : E::Q;
#pragma unroll QUNROLL
  for (int q = 0; q < E::Q; ++q) {
    T G[NN][D];
    const T wd = qp_geometry<ET, T>(q, X, G) * E::template w<T>(q);
    T H[V][D];
    if constexpr (MODE == TG_MODE_RESIDUAL || !L::LINEAR) {
#pragma unroll
      for (int i = 0; i < V; ++i)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          T s = T(0);
#pragma unroll
          for (int a = 0; a < NN; ++a) s += G[a][d] * U[a][i];
          H[i][d] = s;
        }
    }
    if constexpr (MODE == TG_MODE_RESIDUAL) {
      T P[V][D];
      law.flux(H, P);
#pragma unroll
      for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int i = 0; i < V; ++i) {
          T s = T(0);
#pragma unroll
          for (int d = 0; d < D; ++d) s += P[i][d] * G[a][d];
          Y[a][i] += wd * s;
        }
      if constexpr (MAT == TG_POISSON) {
        const T f = law.source();
#pragma unroll
        for (int a = 0; a < NN; ++a) Y[a][0] -= wd * f * E::template N<T>(q, a);
      }
    } else if constexpr (MODE == TG_MODE_HVP) {
      const auto lin = law.linearize(H);
      T dH[V][D], dP[V][D];
#pragma unroll
      for (int i = 0; i < V; ++i)
#pragma unroll
        for (int d = 0; d < D; ++d) {
          T s = T(0);
#pragma unroll
          for (int a = 0; a < NN; ++a) s += G[a][d] * W[a][i];
          dH[i][d] = s;
        }
      lin.dflux(dH, dP);
#pragma unroll
      for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int i = 0; i < V; ++i) {
          T s = T(0);
#pragma unroll
          for (int d = 0; d < D; ++d) s += dP[i][d] * G[a][d];
          Y[a][i] += wd * s;
        }
    } else {  // diagonal of the element tangent
      const auto lin = law.linearize(H);
#pragma unroll
      for (int a = 0; a < NN; ++a)
#pragma unroll
        for (int i = 0; i < V; ++i) {
          T dH[V][D], dP[V][D];
#pragma unroll
          for (int k = 0; k < V; ++k)
#pragma unroll
            for (int d = 0; d < D; ++d) dH[k][d] = (k == i) ? G[a][d] : T(0);
          lin.dflux(dH, dP);
          T s = T(0);
#pragma unroll
          for (int d = 0; d < D; ++d) s += dP[i][d] * G[a][d];
          Y[a][i] += wd * s;
        }
    }
  }
}

// ------------------------------------------------------------------ Hex8 affine modal path
// node a <-> tensor index t = bx + 2 by + 4 bz (bits of the reference coordinates)
__host__ __device__ constexpr int hex_t(int a) { return (a == 2) ? 3 : (a == 3) ? 2 : (a == 6) ? 7 : (a == 7) ? 6 : a; }

// in place: m[S] = sum_t v_t prod_{i in S} s_i(t), S = bit set over (x, y, z)
template <class T>
__device__ __forceinline__ void hadamard8(T (&m)[8]) {
#pragma unroll
  for (int h = 1; h < 8; h <<= 1)
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (!(t & h)) {
        const T a = m[t], b = m[t | h];
        m[t] = b + a;
        m[t | h] = b - a;
      }
}

// transpose of hadamard8 (its matrix is not symmetric: entries are products of
// (2 bit - 1) signs): y_t = sum_S m[S] prod_{i in S} s_i(t)
template <class T>
__device__ __forceinline__ void hadamard8_t(T (&m)[8]) {
#pragma unroll
  for (int h = 1; h < 8; h <<= 1)
#pragma unroll
    for (int t = 0; t < 8; ++t)
      if (!(t & h)) {
        const T a = m[t], b = m[t | h];
        m[t] = a - b;
        m[t | h] = a + b;
      }
}

template <class T>
__device__ __forceinline__ bool hex_affine_geometry(const T (&X)[8][3], T (&R)[3][3], T& detJm) {
  T Jm[3][3];
  bool affine = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    T m[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) m[hex_t(a)] = X[a][k];
    hadamard8(m);
    Jm[0][k] = m[1];
    Jm[1][k] = m[2];
    Jm[2][k] = m[4];
    affine = affine && (m[3] == T(0)) && (m[5] == T(0)) && (m[6] == T(0)) && (m[7] == T(0));
  }
  detJm = inv3(Jm, R);
  return affine;
}

// one monomial mode of a vector law: G[i][j] (direction i, component j; only the
// directions flagged in MASK are non-zero) -> F[j][i] = d psi / d G[i][j], scaled.
template <class T, int MASK, int V, int MAT>
__device__ __forceinline__ void modal_flux(const T (&R)[3][3], const T (&G)[3][V], T mu, T lam,
                                           T (&F)[V][3]) {
  T H[V][3];
#pragma unroll
  for (int j = 0; j < V; ++j)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      T s = T(0);
#pragma unroll
      for (int i = 0; i < 3; ++i)
        if (MASK & (1 << i)) s += R[k][i] * G[i][j];
      H[j][k] = s;
    }
  T P[V][3];
  if constexpr (MAT == TG_LINEAR_ELASTIC) {
    Law<TG_LINEAR_ELASTIC, 3, T>::stress(mu, lam, H, P);
  } else {
#pragma unroll
    for (int k = 0; k < 3; ++k) P[0][k] = mu * H[0][k];
  }
#pragma unroll
  for (int j = 0; j < V; ++j)
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (MASK & (1 << i)) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) s += P[j][k] * R[k][i];
        F[j][i] = s;
      } else {
        F[j][i] = T(0);
      }
    }
}

// Linear elasticity, monomial carried by two reference directions p < q with
// coefficient vectors gp, gq (over components): with r_a = R[:, a] and the metric
// Gm = R^T R,  F_p = sigma r_p,  F_q = sigma r_q  where
// sigma = mu (H + H^T) + lam tr(H) I,  H = gp r_p^T + gq r_q^T, written out through
// the dot products g.r and Gm (no 3x3 products).
template <class T, int P, int Q>
__device__ __forceinline__ void le_two_dir(const T (&R)[3][3], const T (&Gm)[3][3],
                                           const T (&gp)[3], const T (&gq)[3], T mu, T lam,
                                           T (&Fp)[3], T (&Fq)[3]) {
  T a_pp = T(0), a_pq = T(0), a_qp = T(0), a_qq = T(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    a_pp += gp[k] * R[k][P];
    a_pq += gp[k] * R[k][Q];
    a_qp += gq[k] * R[k][P];
    a_qq += gq[k] * R[k][Q];
  }
  const T lt = lam * (a_pp + a_qq);
  const T c1 = mu * Gm[P][P], c2 = mu * Gm[P][Q], c3 = mu * a_pp + lt, c4 = mu * a_qp;
  const T d2 = mu * Gm[Q][Q], d3 = mu * a_pq, d4 = mu * a_qq + lt;
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Fp[j] = c1 * gp[j] + c2 * gq[j] + c3 * R[j][P] + c4 * R[j][Q];
    Fq[j] = c2 * gp[j] + d2 * gq[j] + d3 * R[j][P] + d4 * R[j][Q];
  }
}

// y = dE/du for psi quadratic in grad u (LE: mu, lam; Poisson: kappa in mu), affine hex.
// W holds the nodal values the quadratic form acts on.  Returns the element
// Jacobian determinant (unscaled: det(8 J)).
template <int MAT, class T>
__device__ __forceinline__ void hex_modal_apply(const T (&R)[3][3], T detJm, T mu, T lam,
                                                const T (&W)[8][LawDims<MAT, 3>::V],
                                                T (&Y)[8][LawDims<MAT, 3>::V]) {
  constexpr int V = LawDims<MAT, 3>::V;
  const T g2 = T(HEX_GAUSS) * T(HEX_GAUSS);
  // detJ * sum_q M(xi_q)^2 for the three monomial classes (w_q = 1, detJ = detJm/512)
  const T s0 = detJm * T(1.0 / 64);
  const T s1 = s0 * g2;
  const T s2 = s1 * g2;
  T M[V][8];
#pragma unroll
  for (int j = 0; j < V; ++j) {
#pragma unroll
    for (int a = 0; a < 8; ++a) M[j][hex_t(a)] = W[a][j];
    hadamard8(M[j]);
  }
  T dM[V][8];
  {
    T G[3][V], F[V][3];
#pragma unroll
    for (int j = 0; j < V; ++j) { G[0][j] = M[j][1]; G[1][j] = M[j][2]; G[2][j] = M[j][4]; }
    modal_flux<T, 7, V, MAT>(R, G, mu * s0, lam * s0, F);
#pragma unroll
    for (int j = 0; j < V; ++j) {
      dM[j][0] = T(0);
      dM[j][1] = F[j][0];
      dM[j][2] = F[j][1];
      dM[j][4] = F[j][2];
    }
  }
  if constexpr (MAT == TG_LINEAR_ELASTIC) {
    T Gm[3][3];
#pragma unroll
    for (int a2 = 0; a2 < 3; ++a2)
#pragma unroll
      for (int b2 = a2; b2 < 3; ++b2) {
        T acc = T(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) acc += R[k][a2] * R[k][b2];
        Gm[a2][b2] = acc;
        Gm[b2][a2] = acc;
      }
    const T mu1 = mu * s1, lam1 = lam * s1;
    T g12[3], g13[3], g23[3], g123[3], Fp[3], Fq[3];
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      g12[j] = M[j][3];
      g13[j] = M[j][5];
      g23[j] = M[j][6];
      g123[j] = M[j][7];
    }
    // monomial x: directions (y, z) carry (M12, M13)
    le_two_dir<T, 1, 2>(R, Gm, g12, g13, mu1, lam1, Fp, Fq);
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][3] = Fp[j]; dM[j][5] = Fq[j]; }
    // monomial y: directions (x, z) carry (M12, M23)
    le_two_dir<T, 0, 2>(R, Gm, g12, g23, mu1, lam1, Fp, Fq);
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][3] += Fp[j]; dM[j][6] = Fq[j]; }
    // monomial z: directions (x, y) carry (M13, M23)
    le_two_dir<T, 0, 1>(R, Gm, g13, g23, mu1, lam1, Fp, Fq);
#pragma unroll
    for (int j = 0; j < 3; ++j) { dM[j][5] += Fp[j]; dM[j][6] += Fq[j]; }
    // monomials yz, xz, xy (direction x, y, z carries M123):
    // sum_i [mu Gm_ii g + (mu + lam)(g.r_i) r_i] = mu tr(Gm) g + (mu + lam) R R^T g
    const T mu2 = mu * s2, ml2 = (mu + lam) * s2;
    const T trG = Gm[0][0] + Gm[1][1] + Gm[2][2];
    T h[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < 3; ++k) acc += R[k][i] * g123[k];
      h[i] = acc;
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T acc = T(0);
#pragma unroll
      for (int i = 0; i < 3; ++i) acc += R[j][i] * h[i];
      dM[j][7] = mu2 * trG * g123[j] + ml2 * acc;
    }
  } else {
  {  // monomial x: directions (y, z) carry (M12, M13)
      T G[3][V], F[V][3];
  #pragma unroll
      for (int j = 0; j < V; ++j) { G[0][j] = T(0); G[1][j] = M[j][3]; G[2][j] = M[j][5]; }
      modal_flux<T, 6, V, MAT>(R, G, mu * s1, lam * s1, F);
  #pragma unroll
      for (int j = 0; j < V; ++j) { dM[j][3] = F[j][1]; dM[j][5] = F[j][2]; }
    }
    {  // monomial y: directions (x, z) carry (M12, M23)
      T G[3][V], F[V][3];
  #pragma unroll
      for (int j = 0; j < V; ++j) { G[0][j] = M[j][3]; G[1][j] = T(0); G[2][j] = M[j][6]; }
      modal_flux<T, 5, V, MAT>(R, G, mu * s1, lam * s1, F);
  #pragma unroll
      for (int j = 0; j < V; ++j) { dM[j][3] += F[j][0]; dM[j][6] = F[j][2]; }
    }
    {  // monomial z: directions (x, y) carry (M13, M23)
      T G[3][V], F[V][3];
  #pragma unroll
      for (int j = 0; j < V; ++j) { G[0][j] = M[j][5]; G[1][j] = M[j][6]; G[2][j] = T(0); }
      modal_flux<T, 3, V, MAT>(R, G, mu * s1, lam * s1, F);
  #pragma unroll
      for (int j = 0; j < V; ++j) { dM[j][5] += F[j][0]; dM[j][6] += F[j][1]; }
    }
    {  // monomials yz, xz, xy: direction x, y, z carries M123
      T G[3][V], F[V][3];
  #pragma unroll
      for (int j = 0; j < V; ++j) { G[0][j] = M[j][7]; G[1][j] = T(0); G[2][j] = T(0); }
      modal_flux<T, 1, V, MAT>(R, G, mu * s2, lam * s2, F);
  #pragma unroll
      for (int j = 0; j < V; ++j) dM[j][7] = F[j][0];
  #pragma unroll
      for (int j = 0; j < V; ++j) { G[0][j] = T(0); G[1][j] = M[j][7]; }
      modal_flux<T, 2, V, MAT>(R, G, mu * s2, lam * s2, F);
  #pragma unroll
      for (int j = 0; j < V; ++j) dM[j][7] += F[j][1];
  #pragma unroll
      for (int j = 0; j < V; ++j) { G[1][j] = T(0); G[2][j] = M[j][7]; }
      modal_flux<T, 4, V, MAT>(R, G, mu * s2, lam * s2, F);
  #pragma unroll
      for (int j = 0; j < V; ++j) dM[j][7] += F[j][2];
    }
  }
#pragma unroll
  for (int j = 0; j < V; ++j) {
    hadamard8_t(dM[j]);
#pragma unroll
    for (int a = 0; a < 8; ++a) Y[a][j] = dM[j][hex_t(a)];
  }
}

// ------------------------------------------------------------------ per-element dispatch
// Kernels instantiated with AFFINE = true run only on blocks whose elements the host
// verified to be exact parallelepipeds (tg_plan_build replays the coordinate
// transform below bit for bit in FP32 and FP64); they use the modal evaluation.
template <int ET, int MAT, int MODE>
struct HasAffinePath {
  static constexpr bool value = ET == TG_HEX8 &&
                                (MAT == TG_LINEAR_ELASTIC || MAT == TG_POISSON) &&
                                MODE != TG_MODE_DIAG;
};

// Linear elasticity on an axis-aligned box: R = diag(r) (r_k = 1 / Jm_kk), so every
// product with R is one multiply and the Gram matrix is diag(r_k^2).  Same monomial
// algebra as hex_modal_apply, with the zeros of R removed (about a third of the
// arithmetic, which bounds the FP64 kernel on this GPU).
template <class T, int P, int Q>
__device__ __forceinline__ void le_two_dir_box(const T (&r)[3], const T (&rr)[3], const T (&gp)[3],
                                               const T (&gq)[3], T mu, T lam, T (&Fp)[3],
                                               T (&Fq)[3]) {
  const T a_pp = gp[P] * r[P], a_pq = gp[Q] * r[Q];
  const T a_qp = gq[P] * r[P], a_qq = gq[Q] * r[Q];
  const T lt = lam * (a_pp + a_qq);
  const T c1 = mu * rr[P], d2 = mu * rr[Q];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    Fp[j] = c1 * gp[j];
    Fq[j] = d2 * gq[j];
  }
  Fp[P] += (mu * a_pp + lt) * r[P];
  Fp[Q] += (mu * a_qp) * r[Q];
  Fq[P] += (mu * a_pq) * r[P];
  Fq[Q] += (mu * a_qq + lt) * r[Q];
}

template <class T>
__device__ __forceinline__ void hex_le_modal_box(const T (&r)[3], T detJm, T mu, T lam,
                                                 const T (&W)[8][3], T (&Y)[8][3]) {
  const T g2 = T(HEX_GAUSS) * T(HEX_GAUSS);
  const T s0 = detJm * T(1.0 / 64);
  const T s1 = s0 * g2;
  const T s2 = s1 * g2;
  T M[3][8];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
#pragma unroll
    for (int a = 0; a < 8; ++a) M[j][hex_t(a)] = W[a][j];
    hadamard8(M[j]);
  }
  T dM[3][8];
  {  // constant monomial: directions (x, y, z) carry (M1, M2, M4)
    T H[3][3];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) H[j][k] = r[k] * M[j][1 << k];
    const T m0 = mu * s0;
    const T lt = (lam * s0) * (H[0][0] + H[1][1] + H[2][2]);
    T Pm[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      Pm[i][i] = m0 * (H[i][i] + H[i][i]) + lt;
#pragma unroll
      for (int j = i + 1; j < 3; ++j) {
        Pm[i][j] = m0 * (H[i][j] + H[j][i]);
        Pm[j][i] = Pm[i][j];
      }
    }
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      dM[j][0] = T(0);
      dM[j][1] = Pm[j][0] * r[0];
      dM[j][2] = Pm[j][1] * r[1];
      dM[j][4] = Pm[j][2] * r[2];
    }
  }
  const T rr[3] = {r[0] * r[0], r[1] * r[1], r[2] * r[2]};
  const T mu1 = mu * s1, lam1 = lam * s1;
  T g12[3], g13[3], g23[3], Fp[3], Fq[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    g12[j] = M[j][3];
    g13[j] = M[j][5];
    g23[j] = M[j][6];
  }
  le_two_dir_box<T, 1, 2>(r, rr, g12, g13, mu1, lam1, Fp, Fq);  // monomial x
#pragma unroll
  for (int j = 0; j < 3; ++j) { dM[j][3] = Fp[j]; dM[j][5] = Fq[j]; }
  le_two_dir_box<T, 0, 2>(r, rr, g12, g23, mu1, lam1, Fp, Fq);  // monomial y
#pragma unroll
  for (int j = 0; j < 3; ++j) { dM[j][3] += Fp[j]; dM[j][6] = Fq[j]; }
  le_two_dir_box<T, 0, 1>(r, rr, g13, g23, mu1, lam1, Fp, Fq);  // monomial z
#pragma unroll
  for (int j = 0; j < 3; ++j) { dM[j][5] += Fp[j]; dM[j][6] += Fq[j]; }
  // yz, xz, xy: (mu tr(Gm) + (mu + lam) r_j^2) M123_j
  const T a = (mu * s2) * (rr[0] + rr[1] + rr[2]), ml2 = (mu + lam) * s2;
#pragma unroll
  for (int j = 0; j < 3; ++j) dM[j][7] = (ml2 * rr[j] + a) * M[j][7];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    hadamard8_t(dM[j]);
#pragma unroll
    for (int a8 = 0; a8 < 8; ++a8) Y[a8][j] = dM[j][hex_t(a8)];
  }
}

template <int ET, int MAT, class T, int MODE, bool AFFINE>
__device__ __forceinline__ void element_apply(
    T p0, T p1, const T (&X)[Elem<ET>::NN][Elem<ET>::D],
    const T (&U)[Elem<ET>::NN][LawDims<MAT, Elem<ET>::D>::V],
    const T (&W)[Elem<ET>::NN][LawDims<MAT, Elem<ET>::D>::V],
    T (&Y)[Elem<ET>::NN][LawDims<MAT, Elem<ET>::D>::V]) {
  using E = Elem<ET>;
  if constexpr (AFFINE) {
    static_assert(HasAffinePath<ET, MAT, MODE>::value, "no affine path for this law / mode");
    T R[3][3], detJm;
    hex_affine_geometry(X, R, detJm);
    const T lam = (MAT == TG_LINEAR_ELASTIC) ? p1 : T(0);
    if constexpr (MODE == TG_MODE_RESIDUAL) {
      hex_modal_apply<MAT, T>(R, detJm, p0, lam, U, Y);
      if constexpr (MAT == TG_POISSON) {
        // -f int N_a = -f detJ (sum_q N_a(xi_q) = 1 for the 2x2x2 rule)
        const T fd = p1 * detJm * T(1.0 / 512);
#pragma unroll
        for (int a = 0; a < 8; ++a) Y[a][0] -= fd;
      }
    } else {
      hex_modal_apply<MAT, T>(R, detJm, p0, lam, W, Y);
    }
  } else {
    const Law<MAT, E::D, T> law(p0, p1);
    element_generic<ET, MAT, T, MODE>(law, X, U, W, Y);
  }
}

// ------------------------------------------------------------------ block kernel
template <int ET, int MAT, class T, int MODE>
struct ApplyCfg {
  using E = Elem<ET>;
  static constexpr int D = E::D, V = LawDims<MAT, D>::V;
  static constexpr bool LINEAR = Law<MAT, D, T>::LINEAR;
  static constexpr bool NEED_U = (MODE == TG_MODE_RESIDUAL) || !LINEAR;
  static constexpr bool NEED_W = (MODE == TG_MODE_HVP);
  static constexpr int WORDS_PER_NODE = D + (NEED_U ? V : 0) + (NEED_W ? V : 0) + V;
};

template <int ET, int MAT, class T, int MODE, bool AFFINE>
__global__ void __launch_bounds__(APPLY_MAX_THREADS)
    block_apply_kernel(const tg_block_plan p, int block0, const T* __restrict__ coords,
                       const T* __restrict__ u, const T* __restrict__ v,
                       const uint8_t* __restrict__ fixed, T* __restrict__ y,
                       T* __restrict__ partials, T p0, T p1, const T* __restrict__ eparam) {
  using C = ApplyCfg<ET, MAT, T, MODE>;
  using E = Elem<ET>;
  constexpr int NN = E::NN, D = C::D, V = C::V, NPAD = E::NPAD, SB = apply_sb<ET>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);

  const int b = block0 + blockIdx.x;
  const int n0 = p.blk_node_ptr[b];
  const int nl = p.blk_node_ptr[b + 1] - n0;
  const int nl8 = (nl + 7) & ~7;  // local node l lives in shared-memory slot lnode_smem[l] < nl8
  T* Xs = smem;
  T* Us = Xs + nl8 * D;
  T* Ws = Us + (C::NEED_U ? nl8 * V : 0);
  T* Ys = Ws + (C::NEED_W ? nl8 * V : 0);

  // staging: SB nodes per thread and pass, every node's global id loaded
  // before any of the gathers that depend on it
  for (int l0 = threadIdx.x; l0 < nl; l0 += SB * blockDim.x) {
    int64_t g[SB];
    int q[SB];
#pragma unroll
    for (int k = 0; k < SB; ++k) {
      const int l = l0 + k * blockDim.x;
      g[k] = (l < nl) ? (int64_t)__ldg(p.lnode_gid + n0 + l) : -1;
      q[k] = (l < nl) ? __ldg(p.lnode_smem + n0 + l) : 0;
    }
    T xv[SB][D], uv[SB][V], wv[SB][V];
#pragma unroll
    for (int k = 0; k < SB; ++k) {
      if (g[k] < 0) continue;
#pragma unroll
      for (int d = 0; d < D; ++d) xv[k][d] = coords[g[k] * D + d];
#pragma unroll
      for (int i = 0; i < V; ++i) {
        const int64_t dof = g[k] * V + i;
        if constexpr (C::NEED_U) uv[k][i] = u[dof];
        if constexpr (C::NEED_W) wv[k][i] = (fixed && fixed[dof]) ? T(0) : v[dof];
      }
    }
#pragma unroll
    for (int k = 0; k < SB; ++k) {
      if (g[k] < 0) continue;
#pragma unroll
      for (int d = 0; d < D; ++d) Xs[q[k] * D + d] = xv[k][d];
#pragma unroll
      for (int i = 0; i < V; ++i) {
        if constexpr (C::NEED_U) Us[q[k] * V + i] = uv[k][i];
        if constexpr (C::NEED_W) Ws[q[k] * V + i] = wv[k][i];
        Ys[q[k] * V + i] = T(0);
      }
    }
  }
  __syncthreads();

  // Every thread computes one element of the current chunk of blockDim.x elements
  // into registers (no barrier), then the chunk's results are added into shared
  // memory one element colour at a time (elements of a colour share no node).  The
  // elements are stored by colour, so the additions at every node come in the plan's
  // colour order, as in a colour-by-colour sweep, while no thread idles through the
  // element work of a small colour.
  const int e_base = p.blk_elem_ptr[b];
  const int ne = p.blk_elem_ptr[b + 1] - e_base;
  const int c_last = p.blk_color_ptr[b + 1] - 1;
  const int nt = blockDim.x;
  int c_first = p.blk_color_ptr[b];  // first colour that still has elements at or after k0
  LconnRaw<NPAD> next;  // the row of this thread's element in the next chunk
  if ((int)threadIdx.x < ne) next.load(p.lconn + (int64_t)(e_base + threadIdx.x) * NPAD);
  for (int k0 = 0; k0 < ne; k0 += nt) {
    const int k = k0 + threadIdx.x;
    const bool act = k < ne;
    int lc[NPAD];
    T Y[NN][V];
    if (act) next.unpack(lc);
    if (k + nt < ne) next.load(p.lconn + (int64_t)(e_base + k + nt) * NPAD);
    if (act) {
      const int e = e_base + k;
      T X[NN][D], U[NN][V], W[NN][V];
#pragma unroll
      for (int a = 0; a < NN; ++a) {
#pragma unroll
        for (int d = 0; d < D; ++d) X[a][d] = Xs[lc[a] * D + d];
#pragma unroll
        for (int i = 0; i < V; ++i) {
          U[a][i] = C::NEED_U ? Us[lc[a] * V + i] : T(0);
          W[a][i] = C::NEED_W ? Ws[lc[a] * V + i] : T(0);
        }
      }
      const T kp = eparam ? eparam[__ldg(p.elem_id + e)] : p0;
      element_apply<ET, MAT, T, MODE, AFFINE>(kp, p1, X, U, W, Y);
    }
    while (c_first < c_last && p.color_ofs[c_first + 1] <= k0) ++c_first;
    for (int c = c_first; c < c_last; ++c) {
      const int lo = max(p.color_ofs[c], k0);
      const int hi = min(p.color_ofs[c + 1], k0 + nt);
      if (lo >= k0 + nt) break;  // the same decision in every thread of the block
      if (lo >= hi) continue;
      if (act && k >= lo && k < hi) {
#pragma unroll
        for (int a = 0; a < NN; ++a)
#pragma unroll
          for (int i = 0; i < V; ++i) Ys[lc[a] * V + i] += Y[a][i];
      }
      __syncthreads();
    }
  }

  // write-back: owned-alone nodes to y, shared nodes to their partial slot; the ids of
  // SB nodes are loaded before their stores
  for (int l0 = threadIdx.x; l0 < nl; l0 += SB * blockDim.x) {
    int64_t g[SB];
    int slot[SB], q[SB];
#pragma unroll
    for (int k = 0; k < SB; ++k) {
      const int l = l0 + k * blockDim.x;
      const bool in = l < nl;
      g[k] = in ? (int64_t)__ldg(p.lnode_gid + n0 + l) : -1;
      slot[k] = in ? __ldg(p.lnode_slot + n0 + l) : 0;
      q[k] = in ? __ldg(p.lnode_smem + n0 + l) : 0;
    }
#pragma unroll
    for (int k = 0; k < SB; ++k) {
      if (g[k] < 0) continue;
      if (slot[k] < 0) {
#pragma unroll
        for (int i = 0; i < V; ++i) {
          const int64_t dof = g[k] * V + i;
          T val = Ys[q[k] * V + i];
          if (fixed && fixed[dof])
            val = (MODE == TG_MODE_HVP) ? v[dof] : (MODE == TG_MODE_DIAG ? T(1) : T(0));
          y[dof] = val;
        }
      } else {
#pragma unroll
        for (int i = 0; i < V; ++i) partials[(int64_t)slot[k] * V + i] = Ys[q[k] * V + i];
      }
    }
  }
}

template <class T, int V, int MODE>
__global__ void shared_reduce_kernel(const tg_block_plan p, const T* __restrict__ partials,
                                     const T* __restrict__ v, const uint8_t* __restrict__ fixed,
                                     T* __restrict__ y) {
  // launched as a programmatic dependent of the block kernel: wait until that grid has
  // finished and its partial sums are visible (no-op for an ordinary launch)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= p.n_shared) return;
  const int64_t g = p.shared_node[s];
  T acc[V];
#pragma unroll
  for (int i = 0; i < V; ++i) acc[i] = T(0);
  const int k1 = p.shared_ptr[s + 1];
  for (int k = p.shared_ptr[s]; k < k1; ++k) {
    const int64_t slot = p.shared_slots ? p.shared_slots[k] : k;
#pragma unroll
    for (int i = 0; i < V; ++i) acc[i] += partials[slot * V + i];
  }
#pragma unroll
  for (int i = 0; i < V; ++i) {
    const int64_t dof = g * V + i;
    T val = acc[i];
    if (fixed && fixed[dof])
      val = (MODE == TG_MODE_HVP) ? v[dof] : (MODE == TG_MODE_DIAG ? T(1) : T(0));
    y[dof] = val;
  }
}

// ------------------------------------------------------------------ affine Hex8 kernel
// Dedicated kernel for blocks of host-verified parallelepipeds (LE / Poisson, residual
// or HVP).  Every node occupies one 4-wide slot (x, y, z, 0) / (v0, v1, v2, 0) in
// shared memory, so each node access is a single 16-byte (FP32) or two 16-byte (FP64)
// shared-memory operations; slots are XOR-swizzled within groups of 8 to spread the
// bank quads of the nodes that one quarter-warp touches.  The element geometry comes
// from the three edge vectors at node 0 (exact for a parallelepiped).

template <class T>
__device__ __forceinline__ void ld4(const T* p, T& a, T& b, T& c, T& d);
template <>
__device__ __forceinline__ void ld4<float>(const float* p, float& a, float& b, float& c,
                                           float& d) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  a = v.x; b = v.y; c = v.z; d = v.w;
}
template <>
__device__ __forceinline__ void ld4<double>(const double* p, double& a, double& b, double& c,
                                            double& d) {
  const double2 v0 = reinterpret_cast<const double2*>(p)[0];
  const double2 v1 = reinterpret_cast<const double2*>(p)[1];
  a = v0.x; b = v0.y; c = v1.x; d = v1.y;
}
template <class T>
__device__ __forceinline__ void st4(T* p, T a, T b, T c, T d);
template <>
__device__ __forceinline__ void st4<float>(float* p, float a, float b, float c, float d) {
  *reinterpret_cast<float4*>(p) = make_float4(a, b, c, d);
}
template <>
__device__ __forceinline__ void st4<double>(double* p, double a, double b, double c, double d) {
  reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
  reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}

template <int MAT, int MODE>
struct AffineCfg {
  static constexpr int V = LawDims<MAT, 3>::V;
  static constexpr int FW = (V == 3) ? 4 : 1;  // words per field slot
  // X (4) + field (FW) + Y (FW) words per node
  static constexpr int WORDS_PER_NODE = 4 + 2 * FW;
};

template <int MAT, class T, int MODE>
__global__ void __launch_bounds__(APPLY_MAX_THREADS)
    affine_hex_kernel(const tg_block_plan p, const T* __restrict__ coords,
                      const T* __restrict__ u, const T* __restrict__ v,
                      const uint8_t* __restrict__ fixed, T* __restrict__ y,
                      T* __restrict__ partials, T p0, T p1, const T* __restrict__ eparam) {
  using C = AffineCfg<MAT, MODE>;
  constexpr int V = C::V, FW = C::FW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* smem = reinterpret_cast<T*>(smem_raw);
  const int b = blockIdx.x;
  const int n0 = p.blk_node_ptr[b];
  const int nl = p.blk_node_ptr[b + 1] - n0;
  const int nl8 = (nl + 7) & ~7;
  T* XS = smem;             // nl8 * 4
  T* FS = XS + nl8 * 4;     // nl8 * FW  (u for the residual, v for the HVP)
  T* YS = FS + nl8 * FW;    // nl8 * FW
  const T* fin = (MODE == TG_MODE_RESIDUAL) ? u : v;
  const int nt = blockDim.x;

  // ---- stage the block's nodes (4 nodes per thread per pass, independent loads)
  for (int l0 = threadIdx.x; l0 < nl; l0 += 4 * nt) {
    int64_t g[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int l = l0 + k * nt;
      g[k] = (l < nl) ? (int64_t)__ldg(p.lnode_gid + n0 + l) : 0;
    }
    T xv[4][3], fv[4][V];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int l = l0 + k * nt;
      if (l < nl) {
#pragma unroll
        for (int d = 0; d < 3; ++d) xv[k][d] = coords[g[k] * 3 + d];
#pragma unroll
        for (int i = 0; i < V; ++i) {
          const int64_t dof = g[k] * V + i;
          T val = fin[dof];
          if (MODE == TG_MODE_HVP && fixed && fixed[dof]) val = T(0);
          fv[k][i] = val;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int l = l0 + k * nt;
      if (l < nl) {
        const int q = __ldg(p.lnode_smem + n0 + l);
        st4<T>(XS + q * 4, xv[k][0], xv[k][1], xv[k][2], T(0));
        if constexpr (FW == 4) {
          st4<T>(FS + q * 4, fv[k][0], fv[k][1], fv[k][2], T(0));
          st4<T>(YS + q * 4, T(0), T(0), T(0), T(0));
        } else {
          FS[q] = fv[k][0];
          YS[q] = T(0);
        }
      }
    }
  }
  __syncthreads();

  // ---- elements: every thread computes one element of the current chunk into
  // registers (no barrier), then the chunk's results are added into shared memory
  // one element colour at a time (elements of a colour share no node), so the
  // order of the additions at every node is the plan's colour order.
  const T lam = (MAT == TG_LINEAR_ELASTIC) ? p1 : T(0);
  const int e_base = p.blk_elem_ptr[b];
  const int ne = p.blk_elem_ptr[b + 1] - e_base;
  const int c_begin = p.blk_color_ptr[b];
  const int c_last = p.blk_color_ptr[b + 1] - 1;
  const bool box = b < p.n_diag_blocks;
  for (int k0 = 0; k0 < ne; k0 += nt) {
    const int k = k0 + threadIdx.x;
    const bool act = k < ne;
    T Y[8][V];
    int q[8];
    if (act) {
      const int e = e_base + k;
      int lc[8];
      load_lconn<8>(p.lconn + (int64_t)e * 8, lc);
#pragma unroll
      for (int a = 0; a < 8; ++a) q[a] = lc[a];
      // geometry: Jm = 8 J, rows 4 (x_1 - x_0), 4 (x_3 - x_0), 4 (x_4 - x_0)
      T Jm[3][3], pad;
      {
        T x0[3], xe[3];
        ld4<T>(XS + q[0] * 4, x0[0], x0[1], x0[2], pad);
        const int ed[3] = {1, 3, 4};
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          ld4<T>(XS + q[ed[i]] * 4, xe[0], xe[1], xe[2], pad);
#pragma unroll
          for (int d = 0; d < 3; ++d) Jm[i][d] = T(4) * (xe[d] - x0[d]);
        }
      }
      T W[8][V];
#pragma unroll
      for (int a = 0; a < 8; ++a) {
        if constexpr (FW == 4) {
          ld4<T>(FS + q[a] * 4, W[a][0], W[a][1], W[a][2], pad);
        } else {
          W[a][0] = FS[q[a]];
        }
      }
      const T k0p = eparam ? eparam[__ldg(p.elem_id + e)] : p0;
      bool done_box = false;
      if constexpr (MAT == TG_LINEAR_ELASTIC) {
        if (box) {  // axis-aligned box (host-verified for the whole block)
          const T r[3] = {T(1) / Jm[0][0], T(1) / Jm[1][1], T(1) / Jm[2][2]};
          hex_le_modal_box<T>(r, Jm[0][0] * Jm[1][1] * Jm[2][2], k0p, lam, W, Y);
          done_box = true;
        }
      }
      if (!done_box) {
        T R[3][3];
        const T detJm = inv3(Jm, R);
        hex_modal_apply<MAT, T>(R, detJm, k0p, lam, W, Y);
      }
      if constexpr (MODE == TG_MODE_RESIDUAL && MAT == TG_POISSON) {
        T Rn[3][3];
        const T detJm = inv3(Jm, Rn);
        const T fd = p1 * detJm * T(1.0 / 512);
#pragma unroll
        for (int a = 0; a < 8; ++a) Y[a][0] -= fd;
      }
    }
    for (int c = c_begin; c < c_last; ++c) {
      const int lo = max(p.color_ofs[c], k0);
      const int hi = min(p.color_ofs[c + 1], k0 + nt);
      if (lo >= hi) continue;  // the same decision in every thread of the block
      if (act && k >= lo && k < hi) {
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          if constexpr (FW == 4) {
            T y0, y1, y2, pad;
            ld4<T>(YS + q[a] * 4, y0, y1, y2, pad);
            st4<T>(YS + q[a] * 4, y0 + Y[a][0], y1 + Y[a][1], y2 + Y[a][2], T(0));
          } else {
            YS[q[a]] += Y[a][0];
          }
        }
      }
      __syncthreads();
    }
  }

  // ---- write back: owned-alone nodes to y, shared nodes to their partial slot
  for (int l0 = threadIdx.x; l0 < nl; l0 += 2 * nt) {
    int64_t g[2];
    int slot[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int l = l0 + k * nt;
      g[k] = (l < nl) ? (int64_t)__ldg(p.lnode_gid + n0 + l) : 0;
      slot[k] = (l < nl) ? __ldg(p.lnode_slot + n0 + l) : 0;
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      const int l = l0 + k * nt;
      if (l >= nl) continue;
      T yv[4];
      const int ql = __ldg(p.lnode_smem + n0 + l);
      if constexpr (FW == 4) {
        ld4<T>(YS + ql * 4, yv[0], yv[1], yv[2], yv[3]);
      } else {
        yv[0] = YS[ql];
      }
      if (slot[k] < 0) {
#pragma unroll
        for (int i = 0; i < V; ++i) {
          const int64_t dof = g[k] * V + i;
          T val = yv[i];
          if (fixed && fixed[dof]) val = (MODE == TG_MODE_HVP) ? v[dof] : T(0);
          y[dof] = val;
        }
      } else {
#pragma unroll
        for (int i = 0; i < V; ++i) partials[(int64_t)slot[k] * V + i] = yv[i];
      }
    }
  }
}

// ------------------------------------------------------------------ energy per element
template <int ET, int MAT, class T>
__global__ void energy_kernel(const T* __restrict__ coords, const int32_t* __restrict__ conn,
                              int64_t n_elems, const T* __restrict__ u, T p0, T p1,
                              const T* __restrict__ eparam, T* __restrict__ out) {
  using E = Elem<ET>;
  constexpr int NN = E::NN, D = E::D, V = LawDims<MAT, D>::V;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_elems) return;
  T X[NN][D], U[NN][V];
#pragma unroll
  for (int a = 0; a < NN; ++a) {
    const int64_t n = __ldg(conn + e * NN + a);
#pragma unroll
    for (int d = 0; d < D; ++d) X[a][d] = coords[n * D + d];
#pragma unroll
    for (int i = 0; i < V; ++i) U[a][i] = u[n * V + i];
  }
  const Law<MAT, D, T> law(eparam ? eparam[e] : p0, p1);
  T acc = T(0);
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
#pragma unroll
        for (int a = 0; a < NN; ++a) s += G[a][d] * U[a][i];
        H[i][d] = s;
      }
    T uq = T(0);
#pragma unroll
    for (int a = 0; a < NN; ++a) uq += E::template N<T>(q, a) * U[a][0];
    acc += wd * law.energy(H, uq);
  }
  out[e] = acc;
}

// ------------------------------------------------------------------ host side
template <int MAT, class F>
int dispatch_mat_impl(F&& f) {
  return f(IntC<MAT>{});
}

template <class F>
int dispatch_mat(int kind, F&& f) {
  switch (kind) {
    case TG_POISSON: return f(IntC<TG_POISSON>{});
    case TG_LINEAR_ELASTIC: return f(IntC<TG_LINEAR_ELASTIC>{});
    case TG_NEO_HOOKEAN: return f(IntC<TG_NEO_HOOKEAN>{});
    default: return set_error(TG_ERR_VALUE, "unknown material kind %d", kind);
  }
}

template <class F>
int dispatch_mode(int mode, F&& f) {
  switch (mode) {
    case TG_MODE_RESIDUAL: return f(IntC<TG_MODE_RESIDUAL>{});
    case TG_MODE_HVP: return f(IntC<TG_MODE_HVP>{});
    case TG_MODE_DIAG: return f(IntC<TG_MODE_DIAG>{});
    default: return set_error(TG_ERR_VALUE, "unknown mode %d", mode);
  }
}

// raise the dynamic shared-memory limit of a kernel once per (kernel, device)
inline int ensure_smem(const void* fn, size_t smem) {
  if (smem <= 48 * 1024) return TG_OK;
  {
    int dev = 0, optin = 0;
    TG_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
    TG_TRY(cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev),
                      "shared memory limit"));
    if (smem > (size_t)optin)
      return set_error(TG_ERR_VALUE,
                       "plan needs %zu bytes of shared memory per block, the device allows %d: "
                       "build the plan with fewer elements or local nodes per block",
                       smem, optin);
  }
  static std::mutex mu;
  static std::map<std::pair<const void*, int>, size_t> done;
  int dev = 0;
  TG_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
  std::lock_guard<std::mutex> g(mu);
  auto key = std::make_pair(fn, dev);
  auto it = done.find(key);
  if (it != done.end() && it->second >= smem) return TG_OK;
  TG_TRY(cuda_check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                    "tg_apply: shared memory attribute"));
  done[key] = smem;
  return TG_OK;
}

inline int plan_check(const tg_block_plan* p, int elem) {
  if (!p) return set_error(TG_ERR_VALUE, "plan must not be NULL");
  if (p->n_blocks < 0 || p->n_elems < 0) return set_error(TG_ERR_VALUE, "corrupt plan");
  const int npad = (elem == TG_HEX8) ? 8 : 4;
  if (p->nodes_per_elem_padded != npad)
    return set_error(TG_ERR_VALUE, "plan was built for another element type");
  if (p->threads != 0 && p->threads != 64 && p->threads != 128 && p->threads != 256)
    return set_error(TG_ERR_VALUE, "plan.threads must be 0, 64, 128 or 256");
  if (p->max_local_nodes < 0 || p->max_local_nodes > 65535)
    return set_error(TG_ERR_VALUE, "plan.max_local_nodes out of range");
  return TG_OK;
}

}  // namespace tg

using namespace tg;

extern "C" size_t tg_apply_workspace_bytes(int elem, int prec, int mat_kind,
                                           const tg_block_plan* plan) {
  if (!plan) return 0;
  int V = 1;
  const int D = (elem == TG_TRI3) ? 2 : 3;
  if (mat_kind == TG_LINEAR_ELASTIC) V = D;
  if (mat_kind == TG_NEO_HOOKEAN) V = 3;
  const size_t sz = (prec == TG_F32) ? 4 : 8;
  return (size_t)plan->n_partials * V * sz;
}

extern "C" int tg_apply(int elem, int prec, int mode, const tg_material* mat,
                        const tg_block_plan* plan, const void* coords, int64_t n_nodes,
                        const void* u, const void* v, const uint8_t* fixed, void* y,
                        void* workspace, size_t workspace_bytes, void* stream) {
  TG_TRY(plan_check(plan, elem));
  TG_TRY(check_ptr(mat, "mat"));
  TG_TRY(check_ptr(y, "y"));
  if (n_nodes <= 0) return set_error(TG_ERR_VALUE, "n_nodes must be positive");
  if (workspace_bytes < tg_apply_workspace_bytes(elem, prec, mat->kind, plan))
    return set_error(TG_ERR_WORKSPACE, "tg_apply: workspace too small (%zu < %zu)",
                     workspace_bytes, tg_apply_workspace_bytes(elem, prec, mat->kind, plan));
  if (plan->n_blocks == 0) return TG_OK;
  TG_TRY(check_ptr(coords, "coords"));
  cudaStream_t st = as_stream(stream);
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_mat(mat->kind, [&](auto mk) -> int {
      constexpr int MAT = decltype(mk)::value;
      if constexpr (!Supported<ET, MAT>::value) {
        return set_error(TG_ERR_UNSUPPORTED, "material %d is not available for element %d", MAT, ET);
      } else {
        return dispatch_prec(prec, [&](auto t) -> int {
          using T = decltype(t);
          return dispatch_mode(mode, [&](auto md) -> int {
            constexpr int MODE = decltype(md)::value;
            using C = ApplyCfg<ET, MAT, T, MODE>;
            if (C::NEED_U && !u) return set_error(TG_ERR_VALUE, "u must not be NULL for this mode");
            if (C::NEED_W && !v) return set_error(TG_ERR_VALUE, "v must not be NULL for HVP");
            const size_t smem =
                (size_t)((plan->max_local_nodes + 7) & ~7) * C::WORDS_PER_NODE * sizeof(T);
            const int threads = plan->threads ? plan->threads : 256;
            const int n_aff = HasAffinePath<ET, MAT, MODE>::value ? plan->n_affine_blocks : 0;
            if (n_aff < 0 || n_aff > plan->n_blocks)
              return set_error(TG_ERR_VALUE, "plan.n_affine_blocks out of range");
            if constexpr (ET == TG_HEX8 && MAT == TG_LINEAR_ELASTIC &&
                          (MODE == TG_MODE_HVP || MODE == TG_MODE_RESIDUAL ||
                           MODE == TG_MODE_DIAG)) {
              // structured brick: the stencil schedule over the grid
              if (plan->grid_nodes[0] > 0 && mat->elem_param == nullptr &&
                  (int64_t)plan->grid_nodes[0] * plan->grid_nodes[1] * plan->grid_nodes[2] ==
                      n_nodes) {
                const int rcg = launch_grid_le(plan, prec, MODE, u, v, fixed, y, mat->p0,
                                               mat->p1, st);
                if (rcg != TG_ERR_UNSUPPORTED) return rcg;
              }
            }
            if constexpr (HasAffinePath<ET, MAT, MODE>::value) {
              bool done = false;
              if constexpr (std::is_same<T, float>::value && MAT == TG_LINEAR_ELASTIC) {
                if (n_aff > 0 && mat->elem_param == nullptr) {
                  const int rc5 = launch_hex_le_f32x2(plan, MODE, (const float*)coords,
                                                      (const float*)u, (const float*)v, fixed,
                                                      (float*)y, (float*)workspace,
                                                      (float)mat->p0, (float)mat->p1, st);
                  if (rc5 == TG_OK) done = true;
                  else if (rc5 != TG_ERR_UNSUPPORTED) return rc5;
                }
              }
              if (n_aff > 0 && !done) {
                const int nl8 = (plan->max_local_nodes + 7) & ~7;
                const size_t smem_a = (size_t)nl8 * AffineCfg<MAT, MODE>::WORDS_PER_NODE * sizeof(T);
                auto ka = affine_hex_kernel<MAT, T, MODE>;
                TG_TRY(ensure_smem((const void*)ka, smem_a));
                ka<<<n_aff, threads, smem_a, st>>>(
                    *plan, (const T*)coords, (const T*)u, (const T*)v, fixed, (T*)y,
                    (T*)workspace, (T)mat->p0, (T)mat->p1, (const T*)mat->elem_param);
                TG_TRY(launch_check("tg_apply: affine block kernel"));
              }
            }
            if (plan->n_blocks - n_aff > 0) {
              auto kg = block_apply_kernel<ET, MAT, T, MODE, false>;
              TG_TRY(ensure_smem((const void*)kg, smem));
              kg<<<plan->n_blocks - n_aff, threads, smem, st>>>(
                  *plan, n_aff, (const T*)coords, (const T*)u, (const T*)v, fixed, (T*)y,
                  (T*)workspace, (T)mat->p0, (T)mat->p1, (const T*)mat->elem_param);
            }
            TG_TRY(launch_check("tg_apply: block kernel"));
            if (plan->n_shared > 0) {
              // programmatic dependent launch: the reduce grid is set up while the block
              // kernel drains, and its griddepcontrol.wait orders it after that kernel
              cudaLaunchConfig_t cfg = {};
              cfg.gridDim = dim3((unsigned)grid_for(plan->n_shared, 256));
              cfg.blockDim = dim3(256);
              cfg.dynamicSmemBytes = 0;
              cfg.stream = st;
              cudaLaunchAttribute attr[1];
              attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
              attr[0].val.programmaticStreamSerializationAllowed = 1;
              cfg.attrs = attr;
              cfg.numAttrs = 1;
              TG_TRY(cuda_check(cudaLaunchKernelEx(&cfg, shared_reduce_kernel<T, C::V, MODE>, *plan,
                                                   (const T*)workspace, (const T*)v, fixed, (T*)y),
                                "tg_apply: shared reduce"));
            }
            return TG_OK;
          });
        });
      }
    });
  });
}

extern "C" int tg_energy_per_element(int elem, int prec, const tg_material* mat,
                                     const void* coords, int64_t n_nodes, const int32_t* conn,
                                     int64_t n_elems, const void* u, void* out, void* stream) {
  TG_TRY(check_ptr(mat, "mat"));
  TG_TRY(check_sizes(n_elems, n_nodes, 1));
  if (n_elems == 0) return TG_OK;
  TG_TRY(check_ptr(coords, "coords"));
  TG_TRY(check_ptr(conn, "conn"));
  TG_TRY(check_ptr(u, "u"));
  TG_TRY(check_ptr(out, "out"));
  return dispatch_elem(elem, [&](auto et) -> int {
    constexpr int ET = decltype(et)::value;
    return dispatch_mat(mat->kind, [&](auto mk) -> int {
      constexpr int MAT = decltype(mk)::value;
      if constexpr (!Supported<ET, MAT>::value) {
        return set_error(TG_ERR_UNSUPPORTED, "material %d is not available for element %d", MAT, ET);
      } else {
        return dispatch_prec(prec, [&](auto t) -> int {
          using T = decltype(t);
          energy_kernel<ET, MAT, T><<<grid_for(n_elems, 128), 128, 0, as_stream(stream)>>>(
              (const T*)coords, conn, n_elems, (const T*)u, (T)mat->p0, (T)mat->p1,
              (const T*)mat->elem_param, (T*)out);
          return launch_check("tg_energy_per_element");
        });
      }
    });
  });
}
