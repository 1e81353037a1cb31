"""A numpy model of the mixed solver's two refinement schemes (tg_mixed_solve).

FP32 operator and vectors, FP64 dot products, Jacobi preconditioner, on the clamped
brick's FP64 stiffness from the oracle's element tangents.  Both schemes reach the
FP64 relative residual 1e-10.  The reliable-update scheme keeps the inner CG's
direction across the FP64 residual replacements and needs fewer inner iterations than
restarting at each refinement.  After each replacement the re-orthogonalised direction
satisfies p.r = r.z again, the property a CG step's length relies on.  This is a model
of the algorithm the CUDA solver runs (cg_resume_* kernels), not a test of the kernels.
"""

import numpy as np
import scipy.sparse as sps

from oracle import elements as oe
from oracle import materials as omat
from oracle import operator as oop
from tatva_gb300.problems import clamped_brick

RTOL = 1e-10


def _system(n):
    P = clamped_brick(n, "cpu")
    c, e = P["mesh"].coords_host(), P["mesh"].elements_host()
    op = oop.OracleOperator(c, e, oe.Hexahedron8())
    law = omat.LinearElastic(*omat.lame_from_young(1.0, 0.3))
    nd = c.shape[0] * 3
    Ke = omat.element_tangents(op, law, np.zeros(nd))
    dofs = (e[:, :, None] * 3 + np.arange(3)).reshape(len(e), -1)
    rows = np.repeat(dofs, dofs.shape[1], axis=1).ravel()
    cols = np.tile(dofs, (1, dofs.shape[1])).ravel()
    K = sps.csr_matrix((Ke.reshape(len(e), -1).ravel(), (rows, cols)), shape=(nd, nd))
    free = ~P["fixed"].numpy().astype(bool)
    A = K[free][:, free].tocsr()
    return A, P["b"].numpy()[free]


def _dot(a, b):
    return float(np.dot(a.astype(np.float64), b.astype(np.float64)))


class Model:
    def __init__(self, A, b):
        self.A, self.b = A, b
        self.A32 = A.astype(np.float32)
        self.dinv32 = (1.0 / A.diagonal()).astype(np.float32)
        self.bn = np.linalg.norm(b)

    def true_residual(self, x):
        r = self.b - self.A @ x
        return r, np.linalg.norm(r)

    def solve(self, inner_rtol, keep_direction, max_outer=50, max_inner=5000):
        """The refinement loop of tg_mixed_solve; returns (inner iterations, rel-res,
        max |p.r - r.z| / r.z seen right after a reliable update)."""
        x = np.zeros_like(self.b)
        r64, s = self.true_residual(x)
        p = rz = None
        total, worst = 0, 0.0
        for _ in range(max_outer):
            if s <= RTOL * self.bn:
                break
            r = (r64 / s).astype(np.float32)
            d = np.zeros_like(r)
            z = self.dinv32 * r
            if keep_direction and p is not None:
                scale = s_prev / s
                ps = (p.astype(np.float64) * scale).astype(np.float32)
                c = np.float32(_dot(ps, r) / _dot(r, r))
                ps = ps - c * r  # orthogonal to the new residual
                rz_new = _dot(r, z)
                beta = rz_new / (rz_k * scale * scale)
                p = z + np.float32(beta) * ps
                rz = rz_new
                worst = max(worst, abs(_dot(p, r) - rz) / rz)
            else:
                p, rz = z.copy(), _dot(r, z)
            tol = min(max(inner_rtol, 0.5 * RTOL * self.bn / s), 0.5)
            for _ in range(max_inner):
                q = self.A32 @ p
                a = np.float32(rz / _dot(p, q))
                d += a * p
                r -= a * q
                total += 1
                z = self.dinv32 * r
                rz_k, rz = rz, _dot(r, z)
                if np.sqrt(_dot(r, r)) <= tol:
                    break  # stopped in the update: p is the last direction, rz_k its r.z
                p = z + np.float32(rz / rz_k) * p
            x += s * d.astype(np.float64)
            s_prev = s
            r64, s = self.true_residual(x)
        return total, s / self.bn, worst


def test_reliable_updates_need_fewer_inner_iterations():
    m = Model(*_system(12))
    restarted, rel_r, _ = m.solve(1e-4, keep_direction=False)
    reliable, rel_k, worst = m.solve(0.1, keep_direction=True)
    assert rel_r <= RTOL and rel_k <= RTOL
    assert reliable < 0.95 * restarted, (reliable, restarted)
    assert worst < 1e-5, worst
