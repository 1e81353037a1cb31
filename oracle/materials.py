"""Material laws and their derivatives (oracle, test infrastructure only).

The reference expresses energies as user JAX code and differentiates them with
``jax.grad`` / ``jax.jvp`` (``README.md:93``, ``tatva/sparse/base.py:257-265``).
The energies on the hot path are restated here in closed form:

* Poisson           psi = 1/2 kappa |grad u|^2 - f u
                    (Poisson configuration of the benchmark; kappa may be per element)
* linear elastic    psi = 1/2 sigma:eps, eps = sym(grad u),
                    sigma = 2 mu eps + lambda tr(eps) I
                    (``tests/test_sparse.py:12-30``, ``tests/test_sparse_benchmark.py:30-78``)
* Neo-Hookean       psi = mu/2 (I1 - 3 - 2 ln J) + lambda/2 (ln J)^2, F = I + grad u
                    (``tests/test_sparse_tracer.py:101-113``)

For each: energy density, first derivative P = d psi / d(grad u) (the flux),
its directional derivative dP[dH], and the fourth-order tangent A.
Element residual / HVP / tangent use the quadrature of ``oracle.operator``.
"""

from __future__ import annotations

import numpy as np

from .operator import OracleOperator


def lame_from_young(E, nu):
    """mu = E/2(1+nu), lambda = E nu/((1+nu)(1-2nu))  (tests/test_sparse_benchmark.py:35-43)."""
    mu = E / 2 / (1 + nu)
    lmbda = E * nu / (1 - 2 * nu) / (1 + nu)
    return mu, lmbda


class Poisson:
    name = "poisson"
    n_values = 1

    def __init__(self, kappa=1.0, f=0.0):
        self.kappa = kappa  # scalar or (E,) per-element
        self.f = f

    def _k(self, H):
        k = np.asarray(self.kappa, dtype=np.float64)
        return k[:, None] if k.ndim == 1 else k

    def density(self, H, u_q):
        # H: (E,Q,1,D) ; u_q: (E,Q,1)
        g2 = np.sum(H[:, :, 0, :] ** 2, axis=-1)
        return 0.5 * self._k(H) * g2 - self.f * u_q[..., 0]

    def flux(self, H):
        k = self._k(H)
        return (k[..., None, None] if np.ndim(k) else k) * H

    def dflux(self, H, dH):
        return self.flux(dH)

    def tangent(self, H):
        E, Q, _, D = H.shape
        k = np.broadcast_to(np.asarray(self._k(H), dtype=np.float64), (E, Q))
        A = np.zeros((E, Q, 1, D, 1, D))
        for d in range(D):
            A[:, :, 0, d, 0, d] = k
        return A

    def source(self):
        return self.f


class LinearElastic:
    name = "linear_elastic"

    def __init__(self, mu, lmbda, dim=3):
        self.mu, self.lmbda, self.dim = mu, lmbda, dim
        self.n_values = dim

    def density(self, H, u_q=None):
        eps = 0.5 * (H + np.swapaxes(H, -1, -2))
        tr = np.trace(eps, axis1=-2, axis2=-1)
        return self.mu * np.sum(eps * eps, axis=(-2, -1)) + 0.5 * self.lmbda * tr**2

    def flux(self, H):
        eps = 0.5 * (H + np.swapaxes(H, -1, -2))
        tr = np.trace(eps, axis1=-2, axis2=-1)
        eye = np.eye(H.shape[-1])
        return 2 * self.mu * eps + self.lmbda * tr[..., None, None] * eye

    def dflux(self, H, dH):
        return self.flux(dH)

    def tangent(self, H):
        D = H.shape[-1]
        I = np.eye(D)
        A = self.mu * (np.einsum("ik,jl->ijkl", I, I) + np.einsum("il,jk->ijkl", I, I))
        A = A + self.lmbda * np.einsum("ij,kl->ijkl", I, I)
        return np.broadcast_to(A, H.shape[:2] + A.shape).copy()

    def source(self):
        return 0.0


class NeoHookean:
    name = "neo_hookean"
    n_values = 3

    def __init__(self, mu, lmbda):
        self.mu, self.lmbda = mu, lmbda

    def density(self, H, u_q=None):
        F = np.eye(3) + H
        J = np.linalg.det(F)
        I1 = np.sum(F * F, axis=(-2, -1))
        lnJ = np.log(J)
        return 0.5 * self.mu * (I1 - 3 - 2 * lnJ) + 0.5 * self.lmbda * lnJ**2

    def flux(self, H):
        F = np.eye(3) + H
        J = np.linalg.det(F)
        FinvT = np.swapaxes(np.linalg.inv(F), -1, -2)
        return self.mu * (F - FinvT) + self.lmbda * np.log(J)[..., None, None] * FinvT

    def dflux(self, H, dH):
        F = np.eye(3) + H
        J = np.linalg.det(F)
        Finv = np.linalg.inv(F)
        FinvT = np.swapaxes(Finv, -1, -2)
        lnJ = np.log(J)[..., None, None]
        tr = np.einsum("...ab,...ba->...", Finv, dH)[..., None, None]
        term = FinvT @ np.swapaxes(dH, -1, -2) @ FinvT
        return self.mu * dH + (self.mu - self.lmbda * lnJ) * term + self.lmbda * tr * FinvT

    def tangent(self, H):
        F = np.eye(3) + H
        J = np.linalg.det(F)
        Fi = np.linalg.inv(F)
        lnJ = np.log(J)
        I = np.eye(3)
        A = self.mu * np.einsum("ik,jl->ijkl", I, I)[None, None]
        A = A + (self.mu - self.lmbda * lnJ)[..., None, None, None, None] * np.einsum(
            "...li,...jk->...ijkl", Fi, Fi
        )
        A = A + self.lmbda * np.einsum("...ji,...lk->...ijkl", Fi, Fi)
        return A

    def source(self):
        return 0.0


# ---------------------------------------------------------------------------
# element-level assembly (gather -> QP law -> scatter), numpy reference
# ---------------------------------------------------------------------------


def _as_nodal(op: OracleOperator, u, nv):
    u = np.asarray(u)
    return u.reshape(op.coords.shape[0], nv) if nv > 1 else u.reshape(-1, 1)


def energy(op: OracleOperator, law, u):
    nv = law.n_values
    U = _as_nodal(op, u, nv)
    H = op.grad(U)  # (E,Q,nv,D)
    uq = op.eval(U)  # (E,Q,nv)
    dens = law.density(H, uq) if law.name == "poisson" else law.density(H)
    return op.integrate(dens)


def residual(op: OracleOperator, law, u):
    """jax.grad(E)(u) in closed form: r_a = sum_q w detJ (P . dN_a - f N_a)."""
    nv = law.n_values
    U = _as_nodal(op, u, nv)
    H = op.grad(U)
    P = law.flux(H)  # (E,Q,nv,D)
    w = op.get_integration_weights()
    r = op.grad_transpose(P * w[:, :, None, None])
    src = law.source()
    if np.any(src != 0):
        f = np.broadcast_to(np.asarray(src, dtype=np.float64), w.shape) if np.ndim(src) else src
        r = r - op.eval_transpose((f * w)[:, :, None])
    return r.reshape(-1)


def hvp(op: OracleOperator, law, u, v):
    """jax.jvp(jax.grad(E), (u,), (v,))[1] in closed form."""
    nv = law.n_values
    V = _as_nodal(op, v, nv)
    dH = op.grad(V)
    if u is None:  # linear laws: the HVP does not depend on u (linearised at u = 0)
        H = np.zeros(dH.shape)
    else:
        H = op.grad(_as_nodal(op, u, nv))
    dP = law.dflux(H, dH)
    w = op.get_integration_weights()
    return op.grad_transpose(dP * w[:, :, None, None]).reshape(-1)


def element_tangents(op: OracleOperator, law, u):
    """K_e[(a,i),(b,k)] = sum_q w detJ dNdX[a,J] A[i,J,k,L] dNdX[b,L]  -> (E, n*nv, n*nv)."""
    nv = law.n_values
    U = _as_nodal(op, u, nv)
    H = op.grad(U)
    A = law.tangent(H)  # (E,Q,nv,D,nv,D)
    dNdX, detJ = op.geometry()
    w = detJ * op.qw[None, :]
    K = np.einsum("eq,eqJa,eqiJkL,eqLb->eaibk", w, dNdX, A, dNdX)
    E, n = K.shape[0], K.shape[1]
    return K.reshape(E, n * nv, n * nv)


def assemble_dense(op: OracleOperator, Ke, nv):
    n_dofs = op.coords.shape[0] * nv
    dofs = (op.elements[:, :, None] * nv + np.arange(nv)).reshape(op.n_elements, -1)
    K = np.zeros((n_dofs, n_dofs))
    for e in range(op.n_elements):
        K[np.ix_(dofs[e], dofs[e])] += Ke[e]
    return K


def assemble_csr_data(op: OracleOperator, Ke, nv, indptr, indices):
    """Values of sum_e P_e^T K_e P_e on a given CSR pattern (zeros where absent)."""
    import scipy.sparse as sps

    n_dofs = op.coords.shape[0] * nv
    dofs = (op.elements[:, :, None] * nv + np.arange(nv)).reshape(op.n_elements, -1)
    m = dofs.shape[1]
    rows = np.repeat(dofs, m, axis=1).ravel()
    cols = np.tile(dofs, (1, m)).ravel()
    K = sps.coo_matrix((Ke.ravel(), (rows, cols)), shape=(n_dofs, n_dofs)).tocsr()
    K.sum_duplicates()
    K.sort_indices()
    pat = sps.csr_matrix((np.ones(len(indices)), indices, indptr), shape=(n_dofs, n_dofs))
    # pick K values at the pattern positions
    out = np.asarray(K[pat.nonzero()]).ravel()
    r, c = pat.nonzero()
    order = np.lexsort((c, r))
    data = np.empty(len(indices))
    data[order] = out[order]
    return data
