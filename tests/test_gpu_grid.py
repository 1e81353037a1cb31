"""The structured-brick stencil schedule of the linear-elastic Hex8 residual / HVP
(``grid_le_kernel``) against the oracle and against the element-block kernels that
the same plan runs with the stencil switched off.

Tolerances (relative max-norm): FP64 <= 1e-12 against the oracle and <= 1e-13
between the two FP64 schedules; FP32 <= 1e-5 against the FP64 oracle.
"""

import numpy as np
import pytest
import torch

from oracle import elements as oe
from oracle import materials as omat
from oracle import mesh as om
from oracle import operator as oop
from tatva_gb300 import Mesh, Operator, element, materials

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
SWAP64_TOL = 1e-13
F32_TOL = 1e-5
MU, LAM = 0.7, 1.9


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _setup(shape, lengths, cuda, seed=0):
    c, e = om.brick(*shape, lengths=lengths)
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    en = materials.LinearElastic(op, MU, LAM)
    assert en.plan().grid, en.plan().stats()
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(en.n_dofs)
    u = 0.01 * rng.standard_normal(en.n_dofs)
    fixed = np.zeros(en.n_dofs, np.uint8)
    fixed[rng.random(en.n_dofs) < 0.1] = 1  # scattered fixed dofs, not only whole nodes
    fixed.reshape(-1, 3)[c[:, 0] == c[:, 0].min()] = 1  # and a clamped face
    return c, e, en, v, u, fixed


def _oracle(c, e, v, u, fixed):
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    law = omat.LinearElastic(MU, LAM)
    f = fixed.astype(bool)
    yo = omat.hvp(oo, law, None, np.where(f, 0.0, v))
    yo[f] = v[f]
    ro = omat.residual(oo, law, u)
    ro[f] = 0.0
    return omat.hvp(oo, law, None, v), omat.residual(oo, law, u), yo, ro


SHAPES = [((1, 1, 1), (1.0, 1.0, 1.0)),      # boundary CTAs only
          ((2, 3, 4), (0.5, 0.9, 1.3)),      # one interior node layer in x
          ((7, 5, 6), (0.7, 0.5, 1.2)),      # anisotropic spacing
          ((33, 9, 17), (1.0, 0.3, 0.5)),    # partial tiles in x, y and z
          ((40, 20, 36), (4.0, 2.0, 3.6))]   # several tiles per axis


@pytest.mark.parametrize("shape,lengths", SHAPES)
def test_grid_hvp_and_residual_fp64_fp32(cuda, shape, lengths):
    c, e, en, v, u, fixed = _setup(shape, lengths, cuda)
    yo, ro, yom, rom = _oracle(c, e, v, u, fixed)
    f = torch.as_tensor(fixed, device=cuda)
    for dtype, tol in ((torch.float64, F64_TOL), (torch.float32, F32_TOL)):
        vt = torch.as_tensor(v, dtype=dtype, device=cuda)
        ut = torch.as_tensor(u, dtype=dtype, device=cuda)
        assert rel(en.hvp(None, vt), yo) < tol, dtype
        assert rel(en.residual(ut), ro) < tol, dtype
        assert rel(en.hvp(None, vt, fixed=f), yom) < tol, dtype
        assert rel(en.residual(ut, fixed=f), rom) < tol, dtype


def test_grid_matches_element_blocks_and_is_deterministic(cuda):
    c, e, en, v, u, fixed = _setup((24, 17, 19), (2.4, 1.7, 1.9), cuda, seed=3)
    plan = en.plan()
    f = torch.as_tensor(fixed, device=cuda)
    vt = torch.as_tensor(v, device=cuda)
    a, b = en.hvp(None, vt, fixed=f), en.hvp(None, vt, fixed=f)
    assert torch.equal(a, b)
    plan.grid = False
    try:
        ref = en.hvp(None, vt, fixed=f)
    finally:
        plan.grid = True
    assert rel(a, ref) < SWAP64_TOL
    v32 = vt.float()
    a32, b32 = en.hvp(None, v32), en.hvp(None, v32)
    assert torch.equal(a32, b32)
    assert rel(a32, en.hvp(None, vt)) < F32_TOL


def test_grid_brick_128_properties(cuda):
    """The 128^3 brick of the benchmark through the stencil: symmetry (w.Kv = v.Kw),
    linearity and FP32 against FP64, at full size."""
    c, e = om.brick(128, 128, 128)
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    en = materials.LinearElastic.from_young(op, 1.0, 0.3)
    assert en.plan().grid
    g = torch.Generator(device=cuda).manual_seed(5)
    v = torch.randn(en.n_dofs, dtype=torch.float64, device=cuda, generator=g)
    w = torch.randn(en.n_dofs, dtype=torch.float64, device=cuda, generator=g)
    kv, kw = en.hvp(None, v), en.hvp(None, w)
    s1, s2 = float(w @ kv), float(v @ kw)
    assert abs(s1 - s2) <= 1e-12 * (abs(s1) + abs(s2))
    assert rel(en.hvp(None, 2.0 * v - 3.0 * w), 2.0 * kv - 3.0 * kw) < 1e-13
    assert rel(en.hvp(None, v.float()), kv) < F32_TOL


@pytest.mark.parametrize("check_every", [10, 7])
def test_grid_cg_matches_element_cg_and_is_deterministic(cuda, check_every):
    """CG on the grid stencil (the HVP launch also forms p.q and alpha) against the CG
    on the element-block HVP: same tolerance reached, same solution to 1e-8; FP64 and
    mixed precision; repeated solves bitwise equal (check_every 10 and 7)."""
    from tatva_gb300 import solvers

    c, e = om.brick(20, 12, 10, lengths=(2.0, 1.2, 1.0))
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    en = materials.LinearElastic.from_young(op, 1.0, 0.3)
    plan = en.plan()
    assert plan.grid
    fixed = np.zeros(en.n_dofs, np.uint8)
    fixed.reshape(-1, 3)[c[:, 0] == 0.0] = 1
    fixed = torch.as_tensor(fixed, device=cuda)
    b = torch.zeros(en.n_dofs, dtype=torch.float64, device=cuda)
    b.view(-1, 3)[torch.as_tensor(c[:, 0] == 2.0, device=cuda), 0] = 1e-3
    r1 = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=check_every)
    r2 = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=check_every)
    m1 = solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10, check_every=check_every)
    m2 = solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10, check_every=check_every)
    assert r1.converged and m1.converged and r1.rel_res <= 1e-10 and m1.rel_res <= 1e-10
    assert torch.equal(r1.x, r2.x) and torch.equal(m1.x, m2.x)
    plan.grid = False
    try:
        e1 = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=check_every)
        em = solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10, check_every=check_every)
    finally:
        plan.grid = True
    assert e1.converged and em.converged
    ref = e1.x.cpu().numpy()
    for res in (r1, m1, em):
        assert rel(res.x, ref) < 1e-8


def test_grid_diagonal_matches_element_blocks_and_oracle(cuda):
    """Jacobi diagonal on the grid (per node, the element diagonal summed over the cells
    around it; fixed dofs 1) against the element-block schedule and the oracle's sum
    of element-tangent diagonals."""
    c, e, en, v, u, fixed = _setup((7, 5, 6), (0.7, 0.5, 1.2), cuda)
    f = torch.as_tensor(fixed, device=cuda)
    ut = torch.zeros(en.n_dofs, dtype=torch.float64, device=cuda)
    d_grid = en.diagonal(ut, f)
    plan = en.plan()
    plan.grid = False
    try:
        d_el = en.diagonal(ut, f)
    finally:
        plan.grid = True
    assert rel(d_grid, d_el) < SWAP64_TOL
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    Ke = omat.element_tangents(oo, omat.LinearElastic(MU, LAM), np.zeros(en.n_dofs))
    dofs = (e[:, :, None] * 3 + np.arange(3)).reshape(e.shape[0], -1)
    d = np.zeros(en.n_dofs)
    np.add.at(d, dofs.ravel(), np.einsum("eii->ei", Ke).ravel())
    d[fixed == 1] = 1.0
    assert rel(d_grid, d) < F64_TOL
    assert rel(en.diagonal(ut.float(), f), d) < F32_TOL


def test_grid_cg_with_prescribed_values_on_fixed_dofs(cuda):
    """Right-hand side nonzero on fixed dofs (the masked system's identity rows give
    x = b there) with scattered fixed dofs: the grid CG starts those dofs at b and
    keeps its direction zero on them; FP64 and mixed CG against the element-block CG,
    solution to 1e-8, x = b on the fixed dofs exactly."""
    from tatva_gb300 import solvers

    c, e = om.brick(14, 9, 11, lengths=(1.4, 0.9, 1.1))
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    en = materials.LinearElastic.from_young(op, 1.0, 0.35)
    plan = en.plan()
    assert plan.grid
    rng = np.random.default_rng(8)
    fixed = np.zeros(en.n_dofs, np.uint8)
    fixed.reshape(-1, 3)[c[:, 0] == 0.0] = 1
    fixed[rng.random(en.n_dofs) < 0.03] = 1
    fixed = torch.as_tensor(fixed, device=cuda)
    b = torch.as_tensor(1e-3 * rng.standard_normal(en.n_dofs), device=cuda)
    f = fixed.bool()
    r64 = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=10)
    rmx = solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10, check_every=10)
    assert r64.converged and rmx.converged
    plan.grid = False
    try:
        ref = solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=10)
    finally:
        plan.grid = True
    assert ref.converged
    for res in (r64, rmx):
        assert torch.equal(res.x[f], b[f])
        assert rel(res.x, ref.x) < 1e-8


def test_cg_result_does_not_depend_on_the_check_interval(cuda):
    """The stopping test runs on the device after every iteration (a converged block of
    captured iterations stops working), so iteration counts are exact and the solution
    is bitwise the same whatever the host's check interval."""
    from tatva_gb300 import solvers

    c, e = om.brick(12, 10, 8, lengths=(1.2, 1.0, 0.8))
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    en = materials.LinearElastic.from_young(op, 1.0, 0.3)
    fixed = np.zeros(en.n_dofs, np.uint8)
    fixed.reshape(-1, 3)[c[:, 0] == 0.0] = 1
    fixed = torch.as_tensor(fixed, device=cuda)
    b = torch.as_tensor(np.random.default_rng(4).standard_normal(en.n_dofs) * 1e-3, device=cuda)
    b[fixed.bool()] = 0.0
    runs = [solvers.cg(en, b, fixed=fixed, rtol=1e-10, check_every=k) for k in (4, 10, 50)]
    assert all(r.converged for r in runs)
    assert len({r.iterations for r in runs}) == 1
    assert all(torch.equal(r.x, runs[0].x) for r in runs[1:])
    mixed = [solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10, check_every=k) for k in (6, 50)]
    assert mixed[0].iterations == mixed[1].iterations and torch.equal(mixed[0].x, mixed[1].x)
