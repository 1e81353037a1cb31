"""tg_apply_noalloc (scratch in a fixed device array of the library, no allocation)
against tg_apply (caller-provided workspace), called straight through the C ABI.

Each case makes two calls in a row with different inputs, so the second call runs
on the scratch left behind by the first; both must agree with tg_apply to the
tolerances of the parity tests (1e-12 FP64, 2e-5 FP32, relative max-norm).
This file is collected last so that it also runs after every other kernel of the
library has used the device.
"""

import ctypes

import numpy as np
import pytest
import torch

from oracle import mesh as om
from tatva_gb300 import Mesh, Operator, _lib, element, materials
from tatva_gb300._device import prec_of, ptr, stream

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 2e-5


def rel(a, b):
    a, b = a.double().cpu().numpy(), b.double().cpu().numpy()
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _noalloc(en, mode, u, v, fixed, y):
    dtype = (u if u is not None else v).dtype
    plan = en.plan()
    m = en.material(dtype)
    return _lib.lib().tg_apply_noalloc(
        en.op.element.tg_id, prec_of(dtype), mode, ctypes.byref(m), plan.ref(),
        ptr(en.op.coords_as(dtype)), en.op.n_nodes, ptr(u), ptr(v), ptr(fixed), ptr(y), stream())


def _cases(cuda):
    c, e = om.brick(10, 8, 6)
    box = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    cj = om.jitter_interior(c, 0.1, 0.2, seed=3)
    jit = Operator(Mesh(cj, e, device=cuda), element.Hexahedron8())
    ct, et = om.kuhn_box((1, 1, 1), (5, 4, 6), origin=(0, 0, 0))
    tet = Operator(Mesh(ct, et, device=cuda), element.Tetrahedron4())
    # two full 8 x 8 x 8 cubes: the FP32 plan has lattice blocks, whose kernel writes
    # its partial slots in its own order, on scratch left behind by the other plans
    cl, el = om.brick(16, 8, 8)
    lat = Operator(Mesh(cl, el, device=cuda), element.Hexahedron8())
    lat.plan().grid = False  # a uniform brick: keep the element blocks and their slots
    return [("hex8 box LE", materials.LinearElastic(box, 0.8, 1.3), c),
            ("hex8 jittered LE", materials.LinearElastic(jit, 0.8, 1.3), cj),
            ("tet4 NH", materials.NeoHookean(tet, 1.0, 10.0), ct),
            ("hex8 lattice LE", materials.LinearElastic(lat, 0.8, 1.3), cl)]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_noalloc_apply_matches_tg_apply_two_calls(cuda, dtype):
    tol = F64_TOL if dtype == torch.float64 else F32_TOL
    g = torch.Generator(device="cpu").manual_seed(7)
    for name, en, coords in _cases(cuda):
        if name == "hex8 lattice LE" and dtype == torch.float32:
            assert en.plan().stats()["n_lattice_blocks"] > 0, en.plan().stats()
        n = en.n_dofs
        fixed = torch.zeros(n, dtype=torch.uint8)
        fixed.view(-1, 3)[torch.as_tensor(coords[:, 0] == coords[:, 0].min())] = 1
        fixed = fixed.to(cuda)
        for mode in (_lib.TG_MODE_RESIDUAL, _lib.TG_MODE_HVP, _lib.TG_MODE_DIAG):
            for call in range(2):  # second call reuses the scratch of the first
                u = (1e-2 * torch.randn(n, generator=g, dtype=torch.float64)).to(cuda, dtype)
                v = torch.randn(n, generator=g, dtype=torch.float64).to(cuda, dtype)
                vv = v if mode == _lib.TG_MODE_HVP else None
                mask = fixed if call == 1 else None
                want = en.apply(mode, u, vv, mask)
                got = torch.full_like(want, float("nan"))
                rc = _noalloc(en, mode, u, vv, mask, got)
                assert rc == _lib.TG_OK, _lib.lib().tg_last_error().decode()
                torch.cuda.synchronize()
                assert torch.isfinite(got).all(), (name, mode, call)
                assert rel(got, want) < tol, (name, mode, call, rel(got, want))


def test_noalloc_rejects_plans_above_the_scratch_limit(cuda):
    c, e = om.brick(4, 4, 4)
    en = materials.LinearElastic(Operator(Mesh(c, e, device=cuda), element.Hexahedron8()), 1.0, 1.0)
    real = en.plan().struct
    fake = _lib.BlockPlan.from_buffer_copy(real)
    limit = 8 << 20
    fake.n_partials = limit // (3 * 8) + 1  # one FP64 3-dof slot too many
    u = torch.zeros(en.n_dofs, dtype=torch.float64, device=cuda)
    y = torch.zeros_like(u)
    m = en.material(torch.float64)
    rc = _lib.lib().tg_apply_noalloc(
        _lib.TG_HEX8, _lib.TG_F64, _lib.TG_MODE_RESIDUAL, ctypes.byref(m), ctypes.byref(fake),
        ptr(en.op.coords_as(torch.float64)), en.op.n_nodes, ptr(u), None, None, ptr(y), stream())
    assert rc == _lib.TG_ERR_WORKSPACE
    msg = _lib.lib().tg_last_error().decode()
    assert "fixed maximum of 8388608 bytes" in msg, msg
    # the largest plan that fits is accepted (checked on the host only: not launched)
    fake.n_partials = limit // (3 * 8)
    assert _lib.lib().tg_apply_workspace_bytes(_lib.TG_HEX8, _lib.TG_F64, _lib.TG_LINEAR_ELASTIC,
                                               ctypes.byref(fake)) <= limit
