"""Parity of the CUDA path (through the C ABI) with the oracle and the reference goldens.

Tolerances: FP64 results agree with the reference to <= 1e-12 relative (max-norm);
FP32 results are reported against the FP64 oracle with the bound stated per test.
"""

import numpy as np
import pytest
import torch

from oracle import elements as oe
from oracle import materials as omat
from oracle import mesh as om
from oracle import operator as oop
from oracle import sparse as osp
from tatva_gb300 import Mesh, Operator, element, materials, sparse

pytestmark = pytest.mark.gpu

ELS = {"tri3": (element.Tri3, oe.Tri3), "tet4": (element.Tetrahedron4, oe.Tetrahedron4),
       "hex8": (element.Hexahedron8, oe.Hexahedron8)}
MESHES = {"tri": "tri3", "tet": "tet4", "hexj": "hex8", "hexa": "hex8"}
F64_TOL = 1e-12
F32_TOL = 2e-5


def rel(a, b):
    a = a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)
    b = b.detach().cpu().numpy() if isinstance(b, torch.Tensor) else np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _op(golden, key, cuda):
    m = Mesh(golden[f"{key}_coords"], golden[f"{key}_elements"], device=cuda)
    return Operator(m, ELS[MESHES[key]][0]())


def _t(x, cuda, dtype=torch.float64):
    return torch.as_tensor(np.asarray(x), dtype=dtype, device=cuda)


# ------------------------------------------------------------------ maps
@pytest.mark.parametrize("key", list(MESHES))
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_maps_match_reference(golden, cuda, key, dtype):
    op = _op(golden, key, cuda)
    tol = F64_TOL if dtype == torch.float64 else F32_TOL
    for s in ("s", "v"):
        u = _t(golden[f"{key}_u{s}"], cuda, dtype)
        assert rel(op.eval(u), golden[f"{key}_eval_{s}"]) < tol
        assert rel(op.grad(u), golden[f"{key}_grad_{s}"]) < tol
        assert rel(op.integrate_per_element(u), golden[f"{key}_int_pe_{s}"]) < tol
        assert rel(op.integrate(u), golden[f"{key}_int_pe_{s}"].sum(0)) < tol
    assert rel(op.get_integration_weights(), golden[f"{key}_weights"]) < F64_TOL


def test_reference_operator_known_answers(cuda):
    """tests/test_operator.py:14-178 through the CUDA path."""
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    op = Operator(Mesh(nodes, np.array([[0, 1, 2], [0, 2, 3]], np.int32), device=cuda),
                  element.Tri3())
    np.testing.assert_allclose(op.eval(_t([0.0, 1.0, 2.0, 3.0], cuda)).cpu(), [[1.0], [5.0 / 3.0]])
    np.testing.assert_allclose(op.grad(_t(nodes @ np.array([2.0, 3.0]), cuda)).cpu(),
                               [[[2.0, 3.0]], [[2.0, 3.0]]])
    ones = torch.ones(4, dtype=torch.float64, device=cuda)
    np.testing.assert_allclose(op.integrate_per_element(ones).cpu(), [0.5, 0.5])
    np.testing.assert_allclose(op.integrate(ones).cpu(), 1.0)
    np.testing.assert_allclose(op.integrate_per_element(torch.full((2, 1), 4.0, device=cuda,
                                                                   dtype=torch.float64)).cpu(),
                               [2.0, 2.0])
    np.testing.assert_allclose(op.integrate(2.5).cpu(), 2.5)
    vals = torch.arange(4.0, dtype=torch.float64, device=cuda)
    f = op.map(lambda xi, ev: ev.sum() + xi.sum())(vals)
    np.testing.assert_allclose(f.cpu(), [[3 + 2 / 3], [5 + 2 / 3]])
    g = op.map(lambda xi, ev, b: ev.sum() + b + xi[0], element_quantity=(1,))(
        vals, _t([10.0, 20.0], cuda))
    np.testing.assert_allclose(g.cpu(), [[13 + 1 / 3], [25 + 1 / 3]])
    np.testing.assert_allclose(op.map_over_elements(lambda ev: ev.sum())(vals).cpu(), [3.0, 5.0])


def test_operator_validation_errors(cuda):
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0]])
    with pytest.raises(ValueError, match="outside the mesh"):
        Operator(Mesh(nodes, np.array([[0, 1, 3]], np.int32), device=cuda), element.Tri3())
    with pytest.raises(ValueError, match="negative"):
        Operator(Mesh(nodes, np.array([[0, -1, 2]], np.int32), device=cuda), element.Tri3())
    with pytest.raises(TypeError):
        Mesh(nodes, np.array([[0.0, 1.0, 2.0]]), device=cuda)


# ------------------------------------------------------------------ fused energies
def _energies(op, dim):
    out = [("poisson", materials.Poisson(op, 1.7, 0.9), omat.Poisson(1.7, 0.9)),
           ("linear_elastic", materials.LinearElastic(op, 0.8, 1.3),
            omat.LinearElastic(0.8, 1.3, dim))]
    if dim == 3:
        out.append(("neo_hookean", materials.NeoHookean(op, 1.0, 10.0), omat.NeoHookean(1.0, 10.0)))
    return out


@pytest.mark.parametrize("key", list(MESHES))
def test_fused_residual_hvp_fp64(golden, cuda, key):
    op = _op(golden, key, cuda)
    oo = oop.OracleOperator(golden[f"{key}_coords"], golden[f"{key}_elements"],
                            ELS[MESHES[key]][1]())
    for kind, en, law in _energies(op, op.dim):
        u, v = golden[f"{key}_{kind}_u"], golden[f"{key}_{kind}_v"]
        ut, vt = _t(u, cuda), _t(v, cuda)
        assert rel(en.residual(ut), golden[f"{key}_{kind}_residual"]) < F64_TOL, kind
        assert rel(en.hvp(ut, vt), omat.hvp(oo, law, u, v)) < F64_TOL, kind
        assert rel(en.value(ut), golden[f"{key}_{kind}_energy_pe"].sum()) < F64_TOL, kind
        Kd = np.diag(omat.assemble_dense(oo, omat.element_tangents(oo, law, u), en.n_values))
        assert rel(en.diagonal(ut), Kd) < F64_TOL, kind


@pytest.mark.parametrize("key", list(MESHES))
def test_fused_residual_hvp_fp32(golden, cuda, key):
    """FP32 kernels (FP32 coordinates and arithmetic) against the FP64 oracle."""
    op = _op(golden, key, cuda)
    oo = oop.OracleOperator(golden[f"{key}_coords"], golden[f"{key}_elements"],
                            ELS[MESHES[key]][1]())
    for kind, en, law in _energies(op, op.dim):
        u, v = golden[f"{key}_{kind}_u"], golden[f"{key}_{kind}_v"]
        ut, vt = _t(u, cuda, torch.float32), _t(v, cuda, torch.float32)
        assert rel(en.residual(ut), golden[f"{key}_{kind}_residual"]) < 1e-4, kind
        assert rel(en.hvp(ut, vt), omat.hvp(oo, law, u, v)) < 1e-4, kind


@pytest.mark.parametrize("shape,jitter", [((6, 5, 4), 0.0), ((5, 4, 6), 0.2)])
@pytest.mark.parametrize("kind", ["linear_elastic", "poisson", "neo_hookean"])
def test_hex_brick_affine_and_general(cuda, shape, jitter, kind):
    """Affine bricks take the modal fast path, jittered bricks the per-QP path."""
    c, e = om.brick(*shape, lengths=(1.2, 0.9, 1.1))
    if jitter:
        c = om.jitter_interior(c, 1.0 / max(shape), jitter, seed=4)
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    en, law = {"linear_elastic": (materials.LinearElastic(op, 0.7, 1.9), omat.LinearElastic(0.7, 1.9)),
               "poisson": (materials.Poisson(op, 1.3, 0.6), omat.Poisson(1.3, 0.6)),
               "neo_hookean": (materials.NeoHookean(op, 1.0, 10.0), omat.NeoHookean(1.0, 10.0))}[kind]
    rng = np.random.default_rng(9)
    n = c.shape[0] * en.n_values
    u, v = 0.03 * rng.standard_normal(n), rng.standard_normal(n)
    assert rel(en.residual(_t(u, cuda)), omat.residual(oo, law, u)) < F64_TOL
    assert rel(en.hvp(_t(u, cuda), _t(v, cuda)), omat.hvp(oo, law, u, v)) < F64_TOL
    assert rel(en.hvp(_t(u, cuda, torch.float32), _t(v, cuda, torch.float32)),
               omat.hvp(oo, law, u, v)) < 1e-4
    if kind == "linear_elastic" and not jitter:
        # a uniform brick: the stencil schedule above; the modal element path here
        plan = en.plan()
        assert plan.grid
        plan.grid = False
        try:
            assert rel(en.residual(_t(u, cuda)), omat.residual(oo, law, u)) < F64_TOL
            assert rel(en.hvp(_t(u, cuda), _t(v, cuda)), omat.hvp(oo, law, u, v)) < F64_TOL
            assert rel(en.hvp(_t(u, cuda, torch.float32), _t(v, cuda, torch.float32)),
                       omat.hvp(oo, law, u, v)) < 1e-4
        finally:
            plan.grid = True


@pytest.mark.parametrize("elem", ["tet4", "hex8"])
def test_general_kernel_results_do_not_depend_on_the_cta_size(cuda, elem):
    """The per-QP block kernel adds every node's element contributions in the plan's
    colour order, whatever the number of threads per CTA: the same blocks run with
    64, 128 and 256 threads give the same bits (FP32 and FP64), and the oracle's
    values.  Kuhn tets and a jittered (non-affine) Hex8 brick, Neo-Hookean."""
    if elem == "tet4":
        m = Mesh.kuhn_box(7, 6, 5, device="cpu")
        c, e = om.jitter_interior(m.coords_host(), 1.0 / 7, 0.2, seed=2), m.elements_host()
        el, oel = element.Tetrahedron4(), oe.Tetrahedron4()
    else:
        c, e = om.brick(9, 8, 7)
        c = om.jitter_interior(c, 1.0 / 9, 0.2, seed=3)
        el, oel = element.Hexahedron8(), oe.Hexahedron8()
    op = Operator(Mesh(c, e, device=cuda), el)
    oo = oop.OracleOperator(c, e, oel)
    en, law = materials.NeoHookean(op, 1.0, 10.0), omat.NeoHookean(1.0, 10.0)
    rng = np.random.default_rng(6)
    n = en.n_dofs
    u, v = 0.01 * rng.standard_normal(n), rng.standard_normal(n)
    want = omat.hvp(oo, law, u, v)
    for dtype, tol in ((torch.float64, F64_TOL), (torch.float32, 1e-4)):
        out = []
        for threads in (64, 128, 256):
            plan = op.plan(96, 4096, threads)
            assert plan.sizes["n_blocks"] > 1 and plan.sizes["n_affine_blocks"] == 0
            en.use_plan(plan)
            out.append(en.hvp(_t(u, cuda, dtype), _t(v, cuda, dtype)))
        en.use_plan(None)
        assert torch.equal(out[0], out[1]) and torch.equal(out[0], out[2]), dtype
        assert rel(out[0], want) < tol, dtype


def test_hex_box_geometry_path_is_bitwise_equal(cuda):
    """FP32 box kernel with the plan's precomputed edge terms (box_geom32) equals the
    kernel that derives them from staged coordinates, bit for bit; both match the
    oracle.  Uneven box sizes so that the edge terms differ per element."""
    xs = np.cumsum(np.r_[0.0, np.linspace(0.5, 1.5, 9)])
    c, e = om.brick(9, 7, 6)
    c = c * np.array([9.0, 7.0, 6.0])
    c[:, 0] = xs[np.rint(c[:, 0]).astype(int)]
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    plan = op.plan(128, 4096, 128)
    assert plan.sizes["n_diag_blocks"] == plan.sizes["n_blocks"] and plan.box_geom32 is not None
    en = materials.LinearElastic(op, 0.7, 1.9)
    en.use_plan(plan)
    rng = np.random.default_rng(5)
    v = _t(rng.standard_normal(en.n_dofs), cuda, torch.float32)
    u = _t(0.01 * rng.standard_normal(en.n_dofs), cuda, torch.float32)
    y_geo, r_geo = en.hvp(None, v), en.residual(u)
    saved = plan.struct.box_geom32
    try:
        plan.struct.box_geom32 = None
        y_x, r_x = en.hvp(None, v), en.residual(u)
    finally:
        plan.struct.box_geom32 = saved
    assert torch.equal(y_geo, y_x) and torch.equal(r_geo, r_x)
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    law = omat.LinearElastic(0.7, 1.9)
    assert rel(y_geo, omat.hvp(oo, law, None, v.double().cpu().numpy())) < 1e-5


@pytest.mark.parametrize("kind", ["linear_elastic", "poisson"])
def test_hex_sheared_parallelepipeds_modal_path(cuda, kind):
    """A sheared brick with dyadic shear factors: every element is an exact
    parallelepiped in FP32 and FP64, so all blocks take the modal kernel with a full
    (non-diagonal) Jacobian."""
    c, e = om.brick(6, 5, 7, lengths=(6.0, 5.0, 7.0))  # integer grid
    A = np.array([[1.0, 0.25, -0.125], [0.5, 1.0, 0.25], [0.0, -0.375, 1.0]]) / 8
    c = c @ A.T  # dyadic shear: exact in FP32 and FP64
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    assert op.plan().sizes["n_affine_blocks"] == op.plan().sizes["n_blocks"]
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    en, law = {"linear_elastic": (materials.LinearElastic(op, 0.7, 1.9), omat.LinearElastic(0.7, 1.9)),
               "poisson": (materials.Poisson(op, 1.3, 0.6), omat.Poisson(1.3, 0.6))}[kind]
    rng = np.random.default_rng(2)
    n = c.shape[0] * en.n_values
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    assert rel(en.residual(_t(u, cuda)), omat.residual(oo, law, u)) < F64_TOL
    assert rel(en.hvp(None, _t(v, cuda)), omat.hvp(oo, law, u, v)) < F64_TOL
    assert rel(en.hvp(None, _t(v, cuda, torch.float32)), omat.hvp(oo, law, u, v)) < 1e-5


def test_unit_square_poisson_c1_size(cuda):
    """Configuration-1 size (64x64 Tri3, f=1): residual of u and HVP vs the oracle."""
    c, e = om.unit_square(64, 64)
    op = Operator(Mesh(c, e, device=cuda), element.Tri3())
    oo = oop.OracleOperator(c, e, oe.Tri3())
    en, law = materials.Poisson(op, 1.0, 1.0), omat.Poisson(1.0, 1.0)
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal(c.shape[0]), rng.standard_normal(c.shape[0])
    assert rel(en.residual(_t(u, cuda)), omat.residual(oo, law, u)) < F64_TOL
    assert rel(en.hvp(None, _t(v, cuda)), omat.hvp(oo, law, u, v)) < F64_TOL


def test_per_element_conductivity(cuda):
    c, e = om.unit_square(10, 7)
    rng = np.random.default_rng(3)
    kappa = rng.lognormal(0.0, 1.0, e.shape[0])
    op = Operator(Mesh(c, e, device=cuda), element.Tri3())
    oo = oop.OracleOperator(c, e, oe.Tri3())
    en, law = materials.Poisson(op, _t(kappa, cuda), 1.0), omat.Poisson(kappa, 1.0)
    u = rng.standard_normal(c.shape[0])
    assert rel(en.residual(_t(u, cuda)), omat.residual(oo, law, u)) < F64_TOL
    assert rel(en.value(_t(u, cuda)), omat.energy(oo, law, u)) < F64_TOL


def test_dirichlet_mask_semantics(cuda):
    """Residual rows of fixed dofs are 0 (Fixed.apply_transpose); the HVP is the identity
    there and reads fixed inputs as 0 (reduced operator of Lifter)."""
    c, e = om.brick(3, 3, 3)
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    en, law = materials.LinearElastic(op, 1.0, 1.5), omat.LinearElastic(1.0, 1.5)
    n = c.shape[0] * 3
    fixed = np.zeros(n, np.uint8)
    fixed[np.repeat(np.where(c[:, 0] == 0)[0] * 3, 3) + np.tile(np.arange(3), (c[:, 0] == 0).sum())] = 1
    rng = np.random.default_rng(0)
    u, v = rng.standard_normal(n), rng.standard_normal(n)
    fm = torch.as_tensor(fixed, device=cuda)
    r = en.residual(_t(u, cuda), fixed=fm).cpu().numpy()
    ro = omat.residual(oo, law, u)
    ro[fixed == 1] = 0
    assert rel(r, ro) < F64_TOL
    y = en.hvp(None, _t(v, cuda), fixed=fm).cpu().numpy()
    vm = v.copy()
    vm[fixed == 1] = 0
    yo = omat.hvp(oo, law, u, vm)
    yo[fixed == 1] = v[fixed == 1]
    assert rel(y, yo) < F64_TOL


def test_determinism_bitwise(cuda):
    c, e = om.kuhn_box((1, 1, 1), (8, 7, 6), origin=(0, 0, 0))
    op = Operator(Mesh(c, e, device=cuda), element.Tetrahedron4())
    en = materials.NeoHookean(op, 1.0, 10.0)
    g = torch.Generator(device=cuda).manual_seed(0)
    u = 0.02 * torch.randn(en.n_dofs, dtype=torch.float64, device=cuda, generator=g)
    v = torch.randn(en.n_dofs, dtype=torch.float64, device=cuda, generator=g)
    a, b = en.hvp(u, v), en.hvp(u, v)
    assert torch.equal(a, b)
    assert torch.equal(en.residual(u), en.residual(u))
    assert torch.equal(op.integrate(u[: op.n_nodes]), op.integrate(u[: op.n_nodes]))


# ------------------------------------------------------------------ autograd path
@pytest.mark.parametrize("key", ["tri", "tet", "hexj"])
def test_autograd_energy_matches_reference(golden, cuda, key):
    """User energy written with op.grad / op.integrate; torch autograd through the
    transpose kernels reproduces jax.grad (complex-step golden) and jax.jvp."""
    op = _op(golden, key, cuda)
    dim = op.dim
    u = _t(golden[f"{key}_linear_elastic_u"], cuda).requires_grad_(True)
    v = _t(golden[f"{key}_linear_elastic_v"], cuda)
    mu, lm = 0.8, 1.3

    def energy(uf):
        H = op.grad(uf.view(-1, dim))
        eps = 0.5 * (H + H.transpose(-1, -2))
        tr = eps.diagonal(dim1=-2, dim2=-1).sum(-1)
        return op.integrate(mu * (eps * eps).sum((-2, -1)) + 0.5 * lm * tr * tr)

    (g,) = torch.autograd.grad(energy(u), u, create_graph=True)
    assert rel(g, golden[f"{key}_linear_elastic_residual"]) < F64_TOL
    (hv,) = torch.autograd.grad(g, u, v)
    assert rel(hv, golden[f"{key}_linear_elastic_hvp"]) < F64_TOL
    # Poisson with the -f u term through op.eval
    up = _t(golden[f"{key}_poisson_u"], cuda).requires_grad_(True)

    def poisson(x):
        return op.integrate(0.5 * 1.7 * (op.grad(x) ** 2).sum(-1) - 0.9 * op.eval(x))

    (gp,) = torch.autograd.grad(poisson(up), up)
    assert rel(gp, golden[f"{key}_poisson_residual"]) < F64_TOL


# ------------------------------------------------------------------ sparse Hessian
def test_reference_sparse_case(golden, cuda):
    """tests/test_sparse.py:48-80 through the CUDA path: fused and generic colored
    Jacobians both equal the dense Hessian; linearized_jacfwd returns the residual."""
    m = Mesh.unit_square(8, 8, device=cuda)
    op = Operator(m, element.Tri3())
    en = materials.LinearElastic(op, 1.0, 0.0)
    csr = sparse.pattern_from_mesh(m, 2)
    np.testing.assert_array_equal(csr.indices, golden["sq8_pat2_indices"])
    cm = sparse.ColoredMatrix.from_csr(csr, device=cuda)
    np.testing.assert_array_equal(cm.colors.cpu().numpy(), golden["sq8_pat2_colors"])
    u0 = torch.zeros(m.n_nodes * 2, dtype=torch.float64, device=cuda)
    K = golden["sq8_le_dense_K"]
    K_fused = sparse.jacfwd(en.residual, cm, color_batch_size=10)(u0)
    assert rel(K_fused.to_dense(), K) < F64_TOL

    def total_energy(u_flat):
        H = op.grad(u_flat.view(-1, 2))
        eps = 0.5 * (H + H.transpose(-1, -2))
        return op.integrate((eps * eps).sum((-2, -1)))

    def grad_fn(x):
        x = x.detach().requires_grad_(True) if not x.requires_grad else x
        (g,) = torch.autograd.grad(total_energy(x), x, create_graph=True)
        return g

    K_generic = sparse.jacfwd(grad_fn, cm, color_batch_size=10)(u0)
    np.testing.assert_allclose(K_generic.to_dense().cpu().numpy(), K, rtol=1e-7, atol=1e-13)
    primal, K_lin = sparse.linearized_jacfwd(en.residual, cm, color_batch_size=10)(u0)
    assert rel(K_lin.to_dense(), K) < F64_TOL
    assert float(primal.abs().max()) == 0.0
    rows, cols = sparse.compute_rows_cols(cm)
    r, cc = osp.compute_rows_cols(csr.indptr, csr.indices, golden["sq8_pat2_colors"])
    np.testing.assert_array_equal(rows.cpu().numpy(), r)
    np.testing.assert_array_equal(cols.cpu().numpy(), cc)


@pytest.mark.parametrize("key", ["tet", "hexj"])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_colored_hessian_neo_hookean(golden, cuda, key, dtype):
    op = _op(golden, key, cuda)
    oo = oop.OracleOperator(golden[f"{key}_coords"], golden[f"{key}_elements"],
                            ELS[MESHES[key]][1]())
    en, law = materials.NeoHookean(op, 1.0, 10.0), omat.NeoHookean(1.0, 10.0)
    u = golden[f"{key}_neo_hookean_u"]
    csr = sparse.pattern_from_mesh(op.mesh, 3)
    cm = sparse.ColoredMatrix.from_csr(csr, device=cuda)
    K = sparse.jacfwd(en.residual, cm)(_t(u, cuda, dtype))
    data = omat.assemble_csr_data(oo, omat.element_tangents(oo, law, u), 3, csr.indptr, csr.indices)
    assert rel(K.data, data) < (F64_TOL if dtype == torch.float64 else 1e-4)
    # the compressed matrix equals the colour sums of the dense Hessian
    Kd = omat.assemble_dense(oo, omat.element_tangents(oo, law, u), 3)
    colors = cm.colors.cpu().numpy()
    Jc = np.stack([Kd[:, colors == c].sum(1) for c in range(colors.max() + 1)], 1)
    Jc_gpu = en.compressed_hessian(_t(u, cuda, dtype), cm.colors, cm.n_colors)
    assert rel(Jc_gpu, Jc) < (F64_TOL if dtype == torch.float64 else 1e-4)


@pytest.mark.parametrize("key", ["hexj", "hexa"])
def test_operator_project_matches_oracle(golden, cuda, key):
    """Operator.project (operator.py:523-554, utils.py:118-262): scalar and vector
    quadrature fields, with and without a lifter, vs the oracle's direct solve."""
    from oracle.operator import project as oproject
    from tatva_gb300.lifter import Fixed, Lifter

    c, e = golden[f"{key}_coords"], golden[f"{key}_elements"]
    op = Operator(Mesh(c, e, device=cuda), ELS[MESHES[key]][0]())
    oo = oop.OracleOperator(c, e, ELS[MESHES[key]][1]())
    xq = op.eval(torch.as_tensor(c, device=cuda))  # (E, Q, D) physical QP coordinates
    fs = torch.sin(3 * xq[..., 0]) + xq[..., 1] ** 2
    fv = torch.stack([fs, xq[..., 0] * xq[..., 1]], dim=-1)
    for field in (fs, fv):
        got = op.project(field)
        want = oproject(oo, field.cpu().numpy())
        assert rel(got, want) < 1e-10
    bnd = np.where(np.isclose(c[:, 0], c[:, 0].min()))[0]
    lifter = Lifter(c.shape[0], Fixed(bnd, 0.5))
    got = op.project(fs, lifter=lifter)
    want = oproject(oo, fs.cpu().numpy(), fixed_nodes=bnd, fixed_values=np.full(len(bnd), 0.5))
    assert rel(got, want) < 1e-10


def test_nodes_without_elements(cuda):
    """Ragged input: a mesh whose node list holds nodes that no element uses (the
    reference's gradient is zero there)."""
    c, e = om.brick(3, 2, 2)
    c = np.vstack([c, [[5.0, 5.0, 5.0], [6.0, 5.0, 5.0]]])  # two unused nodes at the end
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    oo = oop.OracleOperator(c, e, oe.Hexahedron8())
    en, law = materials.LinearElastic(op, 0.7, 1.9), omat.LinearElastic(0.7, 1.9)
    rng = np.random.default_rng(3)
    u, v = 0.01 * rng.standard_normal(c.shape[0] * 3), rng.standard_normal(c.shape[0] * 3)
    for dt, tol in ((torch.float64, F64_TOL), (torch.float32, 1e-5)):
        r = en.residual(_t(u, cuda, dt))
        h = en.hvp(None, _t(v, cuda, dt))
        assert rel(r, omat.residual(oo, law, u)) < tol
        assert rel(h, omat.hvp(oo, law, u, v)) < tol
        assert torch.count_nonzero(r[-6:]) == 0 and torch.count_nonzero(h[-6:]) == 0
    fixed = torch.zeros(c.shape[0] * 3, dtype=torch.uint8, device=cuda)
    fixed[-3:] = 1
    h = en.hvp(None, _t(v, cuda), fixed=fixed)
    assert torch.equal(h[-3:], _t(v, cuda)[-3:]) and torch.count_nonzero(h[-6:-3]) == 0


def test_empty_mesh(cuda):
    """Empty input: the reference rejects a mesh without elements
    (operator.py:154-155, "Mesh must contain at least one element."), and so does the
    Operator here; the C ABI itself accepts an empty element list (nothing to do)."""
    c = np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0]])
    e = np.zeros((0, 8), np.int32)
    with pytest.raises(ValueError, match="at least one element"):
        Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    from tatva_gb300 import _lib
    from tatva_gb300._device import ptr, stream

    u = torch.ones(6, dtype=torch.float64, device=cuda)
    out = torch.full((0, 8, 3), 7.0, dtype=torch.float64, device=cuda)
    assert _lib.lib().tg_eval(_lib.TG_HEX8, _lib.TG_F64, ptr(u), 2, 3, None, 0, ptr(out),
                              stream()) == _lib.TG_OK



def test_periodic_reduced_residual_and_hessian(cuda):
    """x-periodic Poisson on the unit square with the bottom row fixed: the reduced
    residual reduce_adjoint(r(lift(u_r))) and the reduced Hessian P^T K P (on the
    adapt_sparsity pattern) match the oracle."""
    import scipy.sparse as sps

    from oracle import lifter as olf
    from tatva_gb300.lifter import Fixed, Lifter, Periodic

    n = 8
    c, e = om.unit_square(n, n)
    left = np.where(np.isclose(c[:, 0], 0.0))[0]
    right = np.where(np.isclose(c[:, 0], 1.0))[0]
    left, right = left[np.argsort(c[left, 1])], right[np.argsort(c[right, 1])]
    bottom = np.setdiff1d(np.where(np.isclose(c[:, 1], 0.0))[0], right)
    N = c.shape[0]
    lf = Lifter(N, Periodic(right, left), Fixed(bottom, 0.25))
    ol = olf.Lifter(N, olf.Periodic(right, left), olf.Fixed(bottom, 0.25))
    op = Operator(Mesh(c, e, device=cuda), element.Tri3())
    oo = oop.OracleOperator(c, e, oe.Tri3())
    en, law = materials.Poisson(op, 1.3, 1.0), omat.Poisson(1.3, 1.0)
    rng = np.random.default_rng(4)
    ur = rng.standard_normal(lf.size_reduced)
    u0 = np.zeros(N)
    r = lf.reduce_adjoint(en.residual(lf.lift(_t(ur, cuda), _t(u0, cuda))))
    ro = ol.reduce_adjoint(omat.residual(oo, law, ol.lift(ur, u0)))
    assert rel(r, ro) < F64_TOL
    # reduced Hessian: P^T K P with the lifting matrix P (slaves copy their masters)
    cm = sparse.ColoredMatrix.from_csr(sparse.pattern_from_mesh(op.mesh, 1), device=cuda)
    K = sparse.jacfwd(en.residual, cm)(_t(u0, cuda)).to_csr()
    free = ol.free_dofs
    P = sps.lil_matrix((N, free.size))
    P[free, np.arange(free.size)] = 1.0
    col_of = {d: i for i, d in enumerate(free)}
    for s_, m_ in zip(right, left):
        if m_ in col_of:
            P[s_, col_of[m_]] = 1.0
    Kr = (P.T @ K @ P).tocsr()
    pat = lf.adapt_sparsity(sparse.pattern_from_mesh(op.mesh, 1))
    assert set(zip(*Kr.nonzero())) <= set(zip(*pat.nonzero()))
    Ke = omat.element_tangents(oo, law, u0)
    Ko = omat.assemble_dense(oo, Ke, 1)
    Kro = P.T.toarray() @ Ko @ P.toarray()
    assert np.abs(Kr.toarray() - Kro).max() / np.abs(Kro).max() < F64_TOL


def test_spmv_node_blocks3(cuda):
    """SpMV over the node blocks of a 3-dof-per-node pattern equals the row-CSR SpMV
    (FP64: same products, other summation order); a pattern of another form is
    reported as not blocked."""
    from tatva_gb300 import _lib, solvers
    from tatva_gb300._device import ptr

    c, e = om.kuhn_box((1, 1, 1), (6, 5, 4), origin=(0, 0, 0))
    pat = osp.pattern_from_mesh(c, e, 3)
    cm = sparse.ColoredMatrix.from_csr(pat, device=cuda)
    rng = np.random.default_rng(2)
    data = torch.as_tensor(rng.standard_normal(cm.nnz), device=cuda)
    x = torch.as_tensor(rng.standard_normal(cm.shape[0]), device=cuda)
    blocks = solvers.node_blocks3(cm)
    assert blocks is not None
    st = torch.cuda.current_stream().cuda_stream
    y_csr, y_blk = torch.empty_like(x), torch.empty_like(x)
    _lib.call("tg_spmv", _lib.TG_F64, cm.shape[0], ptr(cm.indptr), ptr(cm.indices), ptr(data),
              ptr(x), ptr(y_csr), st)
    _lib.call("tg_spmv_blocks3", _lib.TG_F64, cm.shape[0], ptr(cm.indptr), ptr(blocks[0]),
              ptr(blocks[1]), ptr(data), ptr(x), ptr(y_blk), st)
    A = pat.astype(np.float64)
    A.data = data.cpu().numpy()
    assert rel(y_blk, A @ x.cpu().numpy()) < F64_TOL
    assert rel(y_blk, y_csr) < F64_TOL
    # 6 rows of 3 entries (nnz 18) whose row triples differ: not blocked
    import scipy.sparse as sps

    rows = np.repeat(np.arange(6), 3)
    cols = (rows + np.tile(np.arange(3), 6)) % 6
    pat2 = sps.csr_matrix((np.ones(18), (rows, cols)), shape=(6, 6))
    pat2.sort_indices()
    assert solvers.node_blocks3(sparse.ColoredMatrix.from_csr(pat2, device=cuda)) is None
