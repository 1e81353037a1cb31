"""Device solvers composed on the hot path: FP64 Jacobi-CG, mixed FP32/FP64 iterative
refinement, CSR CG on the colored Hessian and Newton, against the CPU oracle.
Failure statuses are produced on the host side (iteration budget, an indefinite
operator): no GPU fault, trap or hang is involved."""

import numpy as np
import pytest
import torch

from oracle import elements as oe
from oracle import materials as omat
from oracle import mesh as om
from oracle import operator as oop
from oracle import solvers as osol
from tatva_gb300 import BreakdownError, Mesh, NotConvergedError, Operator, element, materials
from tatva_gb300 import solvers, sparse
from tatva_gb300.lifter import Fixed, Lifter

pytestmark = pytest.mark.gpu


def _brick_problem(n, cuda):
    c, e = om.brick(n, n, n)
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    en = materials.LinearElastic.from_young(op, 1.0, 0.3)
    nn = c.shape[0]
    fixed = np.zeros(nn * 3, np.uint8)
    left = np.where(c[:, 0] == 0.0)[0]
    for k in range(3):
        fixed[left * 3 + k] = 1
    b = np.zeros(nn * 3)
    right = np.where(c[:, 0] == 1.0)[0]
    b[right * 3] = 1e-3 / len(right)
    return c, e, op, en, torch.as_tensor(fixed, device=cuda), torch.as_tensor(b, device=cuda)


def _oracle_solution(c, e, en, fixed, b):
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    law = omat.LinearElastic(en.p0, en.p1)
    f = fixed.cpu().numpy().astype(bool)

    def apply(x):
        xm = x.copy()
        xm[f] = 0
        y = omat.hvp(oo, law, None, xm)
        y[f] = x[f]
        return y

    Kd = np.diag(omat.assemble_dense(oo, omat.element_tangents(oo, law, np.zeros(len(f))), 3))
    Kd = Kd.copy()
    Kd[f] = 1.0
    x, _ = osol.jacobi_cg(apply, b.cpu().numpy(), Kd, rtol=1e-12)
    return x, apply


def test_cg_fp64_matches_oracle(cuda):
    c, e, op, en, fixed, b = _brick_problem(6, cuda)
    res = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=10)
    assert res.converged and res.rel_res <= 1e-10, res.message
    xo, apply = _oracle_solution(c, e, en, fixed, b)
    x = res.x.cpu().numpy()
    assert np.max(np.abs(x - xo)) / np.max(np.abs(xo)) < 1e-8
    r = b.cpu().numpy() - apply(x)
    assert np.linalg.norm(r) / np.linalg.norm(b.cpu().numpy()) <= 1.0001e-10


def test_mixed_precision_reaches_fp64_tolerance(cuda):
    c, e, op, en, fixed, b = _brick_problem(8, cuda)
    res = solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10, inner_rtol=1e-4, check_every=10)
    assert res.converged and res.rel_res <= 1e-10, res.message
    assert res.outer >= 1
    xo, apply = _oracle_solution(c, e, en, fixed, b)
    r = b.cpu().numpy() - apply(res.x.cpu().numpy())
    assert np.linalg.norm(r) / np.linalg.norm(b.cpu().numpy()) <= 1.0001e-10


def test_cg_deterministic_and_graph_replay(cuda):
    c, e, op, en, fixed, b = _brick_problem(5, cuda)
    r1 = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=7)
    r2 = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=7)
    assert r1.iterations == r2.iterations
    assert torch.equal(r1.x, r2.x)


def test_cg_not_converged_status(cuda):
    c, e, op, en, fixed, b = _brick_problem(6, cuda)
    with pytest.raises(NotConvergedError):
        solvers.cg(en, b, fixed=fixed, rtol=1e-12, maxiter=3, check_every=1)
    res = solvers.cg(en, b, fixed=fixed, rtol=1e-12, maxiter=3, check_every=1,
                     raise_on_fail=False)
    assert not res.converged and res.iterations <= 3


def test_cg_breakdown_status_on_indefinite_operator(cuda):
    """A negative Lame parameter makes the operator indefinite: CG reports breakdown
    through its status, the context stays usable."""
    c, e, op, en, fixed, b = _brick_problem(4, cuda)
    bad = materials.LinearElastic(op, -1.0, 0.0)
    diag = torch.ones(bad.n_dofs, dtype=torch.float64, device=cuda)
    with pytest.raises(BreakdownError):
        solvers.cg(bad, b, fixed=fixed, rtol=1e-10, maxiter=200, check_every=1, diag=diag)
    res = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=10)
    assert res.converged


def test_poisson_unit_square_cg(cuda):
    """Configuration 1: unit square 64x64, f = 1, u = 0 on the boundary, CG to 1e-12."""
    m = Mesh.unit_square(64, 64, device=cuda)
    op = Operator(m, element.Tri3())
    en = materials.Poisson(op, 1.0, 1.0)
    c = m.coords_host()
    bnd = np.where((c[:, 0] == 0) | (c[:, 0] == 1) | (c[:, 1] == 0) | (c[:, 1] == 1))[0]
    lifter = Lifter(m.n_nodes, Fixed(bnd))
    u0 = torch.zeros(m.n_nodes, dtype=torch.float64, device=cuda)
    rhs = -en.residual(u0, fixed=lifter)  # = int f N_a on free dofs
    res = solvers.cg(en, rhs, fixed=lifter, rtol=1e-12, check_every=25)
    assert res.converged and res.rel_res <= 1e-12
    # max of the discrete solution of -lap u = 1 on the unit square ~ 0.0737
    assert abs(float(res.x.max()) - 0.07367) < 1e-3
    r = en.residual(res.x, fixed=lifter)
    assert float(r.norm() / rhs.norm()) <= 1.0001e-12


def test_csr_cg_on_colored_hessian(cuda):
    c, e, op, en, fixed, b = _brick_problem(4, cuda)
    cm = sparse.ColoredMatrix.from_csr(sparse.pattern_from_mesh(op.mesh, 3), device=cuda)
    K = sparse.jacfwd(en.residual, cm)(torch.zeros(en.n_dofs, dtype=torch.float64, device=cuda))
    r_csr = solvers.csr_cg(K, b, fixed=fixed, rtol=1e-10)
    r_mf = solvers.cg(en, b, fixed=fixed, rtol=1e-10)
    assert r_csr.converged and r_mf.converged
    x1, x2 = r_csr.x.cpu().numpy(), r_mf.x.cpu().numpy()
    assert np.max(np.abs(x1 - x2)) / np.max(np.abs(x2)) < 1e-8


def test_newton_neo_hookean_stretch(cuda):
    """Small configuration-3 analogue: Kuhn Tet4 box, Neo-Hookean mu=1 lambda=10,
    10% stretch in 2 load steps; FP32 colored tangent, FP64 residual and update."""
    n = 3
    m = Mesh.kuhn_box(n, n, n, device=cuda)
    op = Operator(m, element.Tetrahedron4())
    en = materials.NeoHookean(op, 1.0, 10.0)
    c = m.coords_host()
    left = np.where(c[:, 0] == 0.0)[0]
    right = np.where(c[:, 0] == 1.0)[0]
    dofs = np.concatenate([left * 3, left * 3 + 1, left * 3 + 2, right * 3, right * 3 + 1,
                           right * 3 + 2])
    cm = sparse.ColoredMatrix.from_csr(sparse.pattern_from_mesh(m, 3), device=cuda)
    u = torch.zeros(en.n_dofs, dtype=torch.float64, device=cuda)
    for step in (1, 2):
        stretch = 0.05 * step
        vals = np.zeros(len(dofs))
        vals[3 * len(left): 4 * len(left)] = stretch
        lifter = Lifter(en.n_dofs, Fixed(dofs, vals))
        u = lifter.lift(lifter.reduce(u), u)
        res = solvers.newton(en, u, lifter, colored_matrix=cm, rtol=1e-10, max_iter=20)
        assert res.converged, res.history
        u = res.x
    # oracle check of the equilibrium: reduced residual of the solution is ~0
    oo = oop.OracleOperator(c, m.elements_host(), oe.Tetrahedron4())
    r = omat.residual(oo, omat.NeoHookean(1.0, 10.0), u.cpu().numpy())
    r[dofs] = 0
    assert np.linalg.norm(r) < 1e-9


def test_solvers_accept_right_hand_sides_at_odd_offsets(cuda):
    """A right-hand side that is a slice of a larger buffer (data at an offset that is
    not a multiple of 16 bytes) is copied by the wrappers; the C ABI refuses such a
    pointer on the host, before any launch, with TG_ERR_VALUE."""
    import ctypes

    from tatva_gb300 import _lib
    from tatva_gb300._device import ptr, workspace

    c, e, op, en, fixed, b = _brick_problem(4, cuda)
    n = en.n_dofs
    big = torch.zeros(n + 1, dtype=torch.float64, device=cuda)
    big[1:] = b
    b_odd = big[1:]
    assert b_odd.data_ptr() % 16 != 0
    r_ref = solvers.cg(en, b, fixed=fixed, rtol=1e-10)
    r_odd = solvers.cg(en, b_odd, fixed=fixed, rtol=1e-10)
    assert r_odd.converged and torch.equal(r_odd.x, r_ref.x)
    m_ref = solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10)
    m_odd = solvers.mixed_cg(en, b_odd, fixed=fixed, rtol=1e-10)
    assert m_odd.converged and torch.equal(m_odd.x, m_ref.x)
    # the raw entry points: refused on the host (no kernel runs)
    desc, keep = en.operator_desc(None, fixed, torch.float64)
    x_odd = torch.zeros(n + 1, dtype=torch.float64, device=cuda)[1:]
    diag = torch.ones(n, dtype=torch.float64, device=cuda)
    nb = _lib.lib().tg_cg_workspace_bytes(ctypes.byref(desc))
    ws = workspace(nb, cuda)
    st = _lib.SolveStats()
    rc = _lib.lib().tg_cg_solve(ctypes.byref(desc), ptr(b_odd), ptr(torch.zeros_like(b)),
                                ptr(diag), 1e-10, 10, 5, ptr(ws), nb, ctypes.byref(st),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.TG_ERR_VALUE and "16-byte aligned" in _lib.lib().tg_last_error().decode()
    rc = _lib.lib().tg_cg_solve(ctypes.byref(desc), ptr(b), ptr(x_odd), ptr(diag), 1e-10, 10, 5,
                                ptr(ws), nb, ctypes.byref(st),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.TG_ERR_VALUE
    out = torch.zeros(1, dtype=torch.float64, device=cuda)
    dws = workspace(_lib.lib().tg_dot_workspace_bytes(), cuda)
    rc = _lib.lib().tg_dot(_lib.TG_F64, ptr(b_odd), ptr(b), n, ptr(out), ptr(dws),
                           _lib.lib().tg_dot_workspace_bytes(),
                           torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.TG_ERR_VALUE
    del keep
