"""A two-field Compound energy through the kernels: displacement u (Neo-Hookean) and
temperature theta (Poisson with per-element conductivity) stacked per node on a
jittered Kuhn Tet4 mesh, E(s) = E_NH(s.u) + E_P(s.theta).

Residual, HVP and the colored sparse Hessian on the pattern of
pattern_from_compound (tatva/sparse/_extraction.py:117-245) against the oracle,
FP64 <= 1e-12 relative (max-norm); the Dirichlet mask in the compound layout.
"""

import numpy as np
import pytest
import torch

from oracle import elements as oe
from oracle import materials as omat
from oracle import mesh as om
from oracle import operator as oop
from tatva_gb300 import Mesh, Operator, element, materials, sparse
from tatva_gb300.compound import Compound, CompoundEnergy, FieldSize, field, pattern_from_compound

pytestmark = pytest.mark.gpu

TOL = 1e-12


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_two_field_compound_residual_hvp_hessian(cuda):
    c, e = om.kuhn_box((1, 1, 1), (3, 4, 3), origin=(0, 0, 0))
    c = om.jitter_interior(c, 0.25, 0.2, seed=2)
    mesh = Mesh(c, e, device=cuda)

    class State(Compound, mesh=mesh):
        u = field((FieldSize.AUTO, 3))
        theta = field((FieldSize.AUTO,))

    op = Operator(mesh, element.Tetrahedron4())
    kappa = np.random.default_rng(5).lognormal(0.0, 1.0, e.shape[0])
    energy = CompoundEnergy(State, u=materials.NeoHookean(op, 1.0, 10.0),
                            theta=materials.Poisson(op, kappa, 0.7))
    rng = np.random.default_rng(6)
    s = 0.02 * rng.standard_normal(State.size)
    v = rng.standard_normal(State.size)
    iu, it = State.u.indices(), State.theta.indices()

    oo = oop.OracleOperator(c, e, oe.Tetrahedron4())
    nh, po = omat.NeoHookean(1.0, 10.0), omat.Poisson(kappa, 0.7)
    r_ref = np.zeros(State.size)
    r_ref[iu] = omat.residual(oo, nh, s[iu])
    r_ref[it] = omat.residual(oo, po, s[it])
    h_ref = np.zeros(State.size)
    h_ref[iu] = omat.hvp(oo, nh, s[iu], v[iu])
    h_ref[it] = omat.hvp(oo, po, s[it], v[it])

    st = torch.as_tensor(s, device=cuda)
    vt = torch.as_tensor(v, device=cuda)
    assert rel(energy.residual(State(st)), r_ref) < TOL
    assert rel(energy.hvp(st, vt), h_ref) < TOL
    # Dirichlet mask in the compound layout: the x = 0 nodes' u and theta held
    fixed = np.zeros(State.size, np.uint8)
    left = np.nonzero(c[:, 0] == 0.0)[0]
    fixed[State.u[left].reshape(-1)] = 1
    fixed[State.theta[left].reshape(-1)] = 1
    fm = torch.as_tensor(fixed, device=cuda)
    rm = r_ref.copy()
    rm[fixed.astype(bool)] = 0.0
    assert rel(energy.residual(st, fixed=fm), rm) < TOL

    # colored Hessian on the compound pattern
    cm = sparse.ColoredMatrix.from_csr(pattern_from_compound(State), device=cuda)
    H = sparse.jacfwd(energy.residual, cm)(st)
    n = State.size
    K = np.zeros((n, n))
    Ku = omat.assemble_dense(oo, omat.element_tangents(oo, nh, s[iu]), 3)
    Kt = omat.assemble_dense(oo, omat.element_tangents(oo, po, s[it]), 1)
    K[np.ix_(iu, iu)] = Ku
    K[np.ix_(it, it)] = Kt
    dense = H.to_dense().cpu().numpy()
    assert rel(dense, K) < TOL  # an entry outside the pattern would be missing here
