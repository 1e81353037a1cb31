"""The FP32 Hex8 lattice kernel (8 x 8 x 8 box blocks, register and lane-shuffle
accumulation) against the oracle and against the colour-ordered box kernel that the
same plan runs when its lattice blocks are switched off.

Tolerances: relative max-norm error <= 1e-5 against the FP64 oracle (FP32
arithmetic); <= 2e-6 between the two FP32 kernels, which evaluate every element law
bit for bit alike and differ only in the order of the node sums.
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

F32_TOL = 1e-5
SWAP_TOL = 2e-6


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def graded_brick(n, seed=0):
    """n^3 brick with uneven spacing along each axis (distinct edge lengths per layer)."""
    rng = np.random.default_rng(seed)
    c, e = om.brick(n, n, n, lengths=(float(n),) * 3)
    for d in range(3):
        lines = np.cumsum(np.r_[0.0, 0.5 + rng.random(n)])
        c[:, d] = lines[np.rint(c[:, d]).astype(int)]
    return c, e


def _run(c, e, cuda, fixed=None, block_elems=512):
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    plan = op.plan(block_elems, 4096, 128)
    plan.grid = False  # element blocks even where the mesh is a uniform brick
    en = materials.LinearElastic(op, 0.7, 1.9)
    en.use_plan(plan)
    rng = np.random.default_rng(3)
    v = torch.as_tensor(rng.standard_normal(en.n_dofs), dtype=torch.float32, device=cuda)
    u = torch.as_tensor(0.01 * rng.standard_normal(en.n_dofs), dtype=torch.float32, device=cuda)
    fm = None if fixed is None else torch.as_tensor(fixed, device=cuda)
    y, r = en.hvp(None, v, fixed=fm), en.residual(u, fixed=fm)
    saved = plan.struct.n_lattice_blocks
    try:
        plan.struct.n_lattice_blocks = 0  # the same blocks through the box kernel
        y0, r0 = en.hvp(None, v, fixed=fm), en.residual(u, fixed=fm)
    finally:
        plan.struct.n_lattice_blocks = saved
    return plan, v, u, y, r, y0, r0


def _oracle(c, e, v, u, fixed=None):
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    law = omat.LinearElastic(0.7, 1.9)
    v = v.double().cpu().numpy()
    u = u.double().cpu().numpy()
    if fixed is None:
        return omat.hvp(oo, law, None, v), omat.residual(oo, law, u)
    f = fixed.astype(bool)
    yo = omat.hvp(oo, law, None, np.where(f, 0.0, v))
    yo[f] = v[f]
    ro = omat.residual(oo, law, u)
    ro[f] = 0.0
    return yo, ro


def test_lattice_hvp_and_residual(cuda):
    c, e = graded_brick(16)
    plan, v, u, y, r, y0, r0 = _run(c, e, cuda)
    assert plan.sizes["n_lattice_blocks"] == plan.sizes["n_blocks"] == 8
    yo, ro = _oracle(c, e, v, u)
    assert rel(y, yo) < F32_TOL and rel(r, ro) < F32_TOL
    assert rel(y, y0) < SWAP_TOL and rel(r, r0) < SWAP_TOL


def test_lattice_dirichlet_mask(cuda):
    c, e = graded_brick(16, seed=1)
    fixed = np.zeros(c.shape[0] * 3, np.uint8)
    side = np.where(c[:, 0] == c[:, 0].min())[0]
    fixed[(side[:, None] * 3 + np.arange(3)).ravel()] = 1
    fixed[3 * np.where(c[:, 2] == c[:, 2].max())[0] + 1] = 1  # one component on another face
    plan, v, u, y, r, y0, r0 = _run(c, e, cuda, fixed)
    assert plan.sizes["n_lattice_blocks"] == 8
    yo, ro = _oracle(c, e, v, u, fixed)
    assert rel(y, yo) < F32_TOL and rel(r, ro) < F32_TOL
    assert rel(y, y0) < SWAP_TOL and rel(r, r0) < SWAP_TOL


def test_lattice_permuted_node_numbering(cuda):
    """Global node ids in random order: the plan numbers a lattice block's local nodes
    by grid position, so the blocks still take the lattice kernel."""
    c, e = graded_brick(16, seed=2)
    perm = np.random.default_rng(4).permutation(c.shape[0])
    inv = np.argsort(perm)
    c, e = c[perm], inv[e]
    plan, v, u, y, r, y0, r0 = _run(c, e, cuda)
    assert plan.sizes["n_lattice_blocks"] == 8
    yo, ro = _oracle(c, e, v, u)
    assert rel(y, yo) < F32_TOL and rel(r, ro) < F32_TOL
    assert rel(y, y0) < SWAP_TOL


def test_lattice_mixed_with_general_blocks(cuda):
    """A moved interior node turns the blocks around it into general blocks; the rest
    stay lattice blocks, and the shared nodes between the two kinds add up."""
    c, e = graded_brick(16, seed=3)
    g = np.argmin(np.linalg.norm(c - c.mean(axis=0) - 0.3, axis=1))
    c = c.copy()
    c[g] += np.array([0.11, -0.07, 0.05])
    plan, v, u, y, r, y0, r0 = _run(c, e, cuda)
    assert 0 < plan.sizes["n_lattice_blocks"] < plan.sizes["n_blocks"]
    yo, ro = _oracle(c, e, v, u)
    assert rel(y, yo) < F32_TOL and rel(r, ro) < F32_TOL


def test_lattice_many_blocks_per_cta_and_bitwise_repeat(cuda):
    """More lattice blocks than resident CTAs (each CTA walks several blocks through
    the double-buffered pipeline); two calls give the same bits."""
    c, e = om.brick(128, 64, 64)  # 1024 blocks, above the 608 resident CTAs of a GB300
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    plan = op.plan(512, 4096, 128)
    plan.grid = False  # a uniform brick: without this the stencil schedule runs it
    assert plan.sizes["n_lattice_blocks"] == plan.sizes["n_blocks"] == 1024
    en = materials.LinearElastic(op, 0.7, 1.9)
    en.use_plan(plan)
    g = torch.Generator(device=cuda).manual_seed(1)
    v = torch.randn(en.n_dofs, dtype=torch.float32, device=cuda, generator=g)
    a, b = en.hvp(None, v), en.hvp(None, v)
    assert torch.equal(a, b)
    y64 = en.hvp(None, v.double())
    assert rel(a, y64) < F32_TOL


def test_lattice_and_box_blocks_on_uneven_sides(cuda):
    """Sides that are not multiples of 8: the full 8 x 8 x 8 cubes run the lattice kernel,
    the partial cubes the colour-ordered box kernel, in the same HVP."""
    rng = np.random.default_rng(7)
    shape = (20, 12, 10)
    c, e = om.brick(*shape, lengths=tuple(float(s) for s in shape))
    for d in range(3):
        lines = np.cumsum(np.r_[0.0, 0.5 + rng.random(shape[d])])
        c[:, d] = lines[np.rint(c[:, d]).astype(int)]
    plan, v, u, y, r, y0, r0 = _run(c, e, cuda)
    assert plan.sizes["n_lattice_blocks"] == 2
    assert plan.sizes["n_diag_blocks"] == plan.sizes["n_blocks"] > 2
    yo, ro = _oracle(c, e, v, u)
    assert rel(y, yo) < F32_TOL and rel(r, ro) < F32_TOL
    assert rel(y, y0) < SWAP_TOL and rel(r, r0) < SWAP_TOL
