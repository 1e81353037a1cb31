"""Size-independent properties at the full benchmark sizes, where the oracle would
take too long: the 128^3 Hex8 brick (2,097,152 elements, 6,440,067 dofs).

* the HVP is symmetric: v.(K w) = w.(K v)
* the HVP is linear: K(a v + w) = a K v + K w
* the quadratic energy is consistent with the HVP: E(u) = 1/2 u.(K u) (linear elasticity)
* the FP32 kernels (grid stencil; lattice and box element blocks) agree with FP64
Tolerances: FP64 1e-12 relative; FP32 results against FP64 2e-5 relative (max-norm).
"""

import pytest
import torch

from tatva_gb300 import _lib
from tatva_gb300.problems import clamped_brick

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def brick(cuda):
    return clamped_brick(128, cuda)


def _rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


def test_full_size_hvp_symmetry_linearity_energy(brick):
    en = brick["energy"]
    g = torch.Generator(device="cpu").manual_seed(0)
    n = en.n_dofs
    v = torch.randn(n, generator=g, dtype=torch.float64).cuda()
    w = torch.randn(n, generator=g, dtype=torch.float64).cuda()
    Kv, Kw = en.hvp(None, v), en.hvp(None, w)
    s1, s2 = float(torch.dot(v, Kw)), float(torch.dot(w, Kv))
    assert abs(s1 - s2) <= 1e-12 * abs(s1) * 10
    a = 0.37
    assert _rel(en.hvp(None, a * v + w), a * Kv + Kw) < 1e-12
    u = 1e-3 * v
    E = float(en.value(u))
    assert abs(E - 0.5 * float(torch.dot(u, en.hvp(None, u)))) <= 1e-11 * abs(E)


def test_full_size_fp32_box_kernel_vs_fp64(brick):
    en = brick["energy"]
    plan = en.plan()
    assert plan.sizes["n_diag_blocks"] == plan.sizes["n_blocks"]
    g = torch.Generator(device="cpu").manual_seed(1)
    v = torch.randn(en.n_dofs, generator=g, dtype=torch.float64).cuda()
    y64 = en.hvp(None, v)
    y32 = en.hvp(None, v.float())
    assert _rel(y32.double(), y64) < 2e-5
    r64 = en.residual(1e-3 * v, fixed=brick["fixed"])
    r32 = en.residual((1e-3 * v).float(), fixed=brick["fixed"])
    assert _rel(r32.double(), r64) < 2e-5
    # the element-block kernels of the same plan (the brick runs the grid stencil by
    # default): FP32 lattice / box kernel against FP64, and the no-staging box kernel
    # (plan edge terms) bit for bit equal to the staging one
    assert plan.grid
    plan.grid = False
    saved = plan.struct.box_geom32
    try:
        y32b = en.hvp(None, v.float())
        assert _rel(y32b.double(), y64) < 2e-5
        n_lat = plan.struct.n_lattice_blocks
        plan.struct.n_lattice_blocks = 0
        y32g = en.hvp(None, v.float())
        plan.struct.box_geom32 = None
        y32x = en.hvp(None, v.float())
        plan.struct.n_lattice_blocks = n_lat
    finally:
        plan.struct.box_geom32 = saved
        plan.grid = True
    assert torch.equal(y32g, y32x)
