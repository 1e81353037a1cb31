"""The CPU oracle against the reference: golden fixtures produced by executing the
reference's own modules (tests/golden/make_golden.py) and the known answers of the
reference's tests (tests/test_operator.py, test_element.py, test_sparse.py,
test_lifter.py).  No GPU."""

import numpy as np
import pytest

from oracle import elements as oe
from oracle import lifter as olift
from oracle import materials as omat
from oracle import mesh as om
from oracle import operator as oop
from oracle import sparse as osp

ELS = {"tri3": oe.Tri3, "tet4": oe.Tetrahedron4, "hex8": oe.Hexahedron8}
MESHES = {"tri": "tri3", "tet": "tet4", "hexj": "hex8", "hexa": "hex8"}


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


# ------------------------------------------------------------------ elements
@pytest.mark.parametrize("name", list(ELS))
def test_element_tables_match_reference(golden, name):
    e = ELS[name]()
    N, dN, qw = e.tables()
    np.testing.assert_array_equal(e.quad_points, golden[f"{name}_qp"])
    np.testing.assert_array_equal(qw, golden[f"{name}_qw"])
    np.testing.assert_array_equal(N, golden[f"{name}_N"])
    np.testing.assert_array_equal(dN, golden[f"{name}_dN"])
    X, U = golden[f"{name}_el_X"], golden[f"{name}_el_U"]
    gr = np.stack([e.gradient(x, U, X) for x in e.quad_points])
    assert rel(gr, golden[f"{name}_el_grad"]) < 1e-14


# tests/test_element.py:45-149: exact gradients of linear fields, atol 1e-12
@pytest.mark.parametrize("name", list(ELS))
def test_linear_field_gradients_exact(name):
    e = ELS[name]()
    coords = e.reference_nodes()
    d = coords.shape[1]
    rng = np.random.default_rng(0)
    a = np.arange(2.0, 2.0 + d)
    for xi in e.quad_points:
        np.testing.assert_allclose(e.gradient(xi, coords @ a, coords), a, atol=1e-12)
    A = rng.standard_normal((d, d))
    u = np.einsum("ij,kj->ki", A, coords)
    for xi in e.quad_points:
        np.testing.assert_allclose(e.gradient(xi, u, coords), A, atol=1e-12)
    B = rng.standard_normal((2, 2, d))
    T = np.einsum("ijk,nk->nij", B, coords)
    for xi in e.quad_points:
        np.testing.assert_allclose(e.gradient(xi, T, coords), B, atol=1e-12)


# ------------------------------------------------------------------ operator
def test_reference_operator_known_answers():
    """tests/test_operator.py:14-143 (two-triangle unit square)."""
    nodes = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    elements = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int32)
    op = oop.OracleOperator(nodes, elements, oe.Tri3())
    np.testing.assert_allclose(op.eval(np.array([0.0, 1.0, 2.0, 3.0])), [[1.0], [5.0 / 3.0]])
    np.testing.assert_allclose(op.grad(nodes @ np.array([2.0, 3.0])), [[[2.0, 3.0]], [[2.0, 3.0]]])
    np.testing.assert_allclose(op.integrate_per_element(np.ones(4)), [0.5, 0.5])
    np.testing.assert_allclose(op.integrate(np.ones(4)), 1.0)
    np.testing.assert_allclose(op.integrate_per_element(np.full((2, 1), 4.0)), [2.0, 2.0])
    vals = np.arange(4.0)
    f = op.map(lambda xi, ev: np.sum(ev) + np.sum(xi))(vals)
    np.testing.assert_allclose(f, [[3 + 2 / 3], [5 + 2 / 3]])
    g = op.map(lambda xi, ev, b: np.sum(ev) + b + xi[0], element_quantity=(1,))(
        vals, np.array([10.0, 20.0]))
    np.testing.assert_allclose(g, [[13 + 1 / 3], [25 + 1 / 3]])
    np.testing.assert_allclose(op.map_over_elements(np.sum)(vals), [3.0, 5.0])


@pytest.mark.parametrize("key", list(MESHES))
def test_operator_maps_match_reference(golden, key):
    op = oop.OracleOperator(golden[f"{key}_coords"], golden[f"{key}_elements"],
                            ELS[MESHES[key]]())
    for s in ("s", "v"):
        u = golden[f"{key}_u{s}"]
        assert rel(op.eval(u), golden[f"{key}_eval_{s}"]) < 1e-14
        assert rel(op.grad(u), golden[f"{key}_grad_{s}"]) < 1e-13
        assert rel(op.integrate_per_element(u), golden[f"{key}_int_pe_{s}"]) < 1e-13
    assert rel(op.get_integration_weights(), golden[f"{key}_weights"]) < 1e-13


def test_mesh_generator_matches_reference(golden):
    for nx, ny in ((3, 2), (8, 8)):
        c, e = om.unit_square(nx, ny)
        np.testing.assert_array_equal(c, golden[f"usq_{nx}x{ny}_coords"])
        np.testing.assert_array_equal(e, golden[f"usq_{nx}x{ny}_elements"])


# ------------------------------------------------------------------ pattern & colouring
@pytest.mark.parametrize("key", list(MESHES))
def test_pattern_colors_rows_bit_exact(golden, key):
    c, e = golden[f"{key}_coords"], golden[f"{key}_elements"]
    for ndpn in ((1, 2, 3) if c.shape[1] == 3 else (1, 2)):
        csr = osp.pattern_from_mesh(c, e, ndpn)
        np.testing.assert_array_equal(csr.indptr, golden[f"{key}_pat{ndpn}_indptr"])
        np.testing.assert_array_equal(csr.indices, golden[f"{key}_pat{ndpn}_indices"])
        col = osp.distance2_colors(csr.indptr, csr.indices, csr.shape[0])
        np.testing.assert_array_equal(col, golden[f"{key}_pat{ndpn}_colors"])
        r, cc = osp.compute_rows_cols(csr.indptr, csr.indices, col)
        np.testing.assert_array_equal(r, golden[f"{key}_pat{ndpn}_rows"])
        np.testing.assert_array_equal(cc, golden[f"{key}_pat{ndpn}_colcolors"])
        assert osp.check_distance2(csr.indptr, csr.indices, col)


# ------------------------------------------------------------------ derivatives
def _laws(dim):
    out = [("poisson", omat.Poisson(1.7, 0.9)), ("linear_elastic", omat.LinearElastic(0.8, 1.3, dim))]
    if dim == 3:
        out.append(("neo_hookean", omat.NeoHookean(1.0, 10.0)))
    return out


@pytest.mark.parametrize("key", list(MESHES))
def test_energy_residual_hvp_match_reference(golden, key):
    c = golden[f"{key}_coords"]
    op = oop.OracleOperator(c, golden[f"{key}_elements"], ELS[MESHES[key]]())
    for kind, law in _laws(c.shape[1]):
        u, v = golden[f"{key}_{kind}_u"], golden[f"{key}_{kind}_v"]
        assert rel(omat.energy(op, law, u), golden[f"{key}_{kind}_energy_pe"].sum()) < 1e-13
        # complex-step golden: exact to rounding
        assert rel(omat.residual(op, law, u), golden[f"{key}_{kind}_residual"]) < 1e-13
        # NH golden is a Richardson difference of complex-step gradients (~1e-11)
        tol = 1e-10 if kind == "neo_hookean" else 1e-13
        assert rel(omat.hvp(op, law, u, v), golden[f"{key}_{kind}_hvp"]) < tol


def test_hvp_is_derivative_of_residual_complex_step():
    """The oracle HVP equals the complex-step derivative of the oracle residual."""
    c, e = om.kuhn_box((1, 1, 1), (2, 2, 2), origin=(0, 0, 0))
    c = om.jitter_interior(c, 0.5, 0.15, seed=3)
    op = oop.OracleOperator(c, e, oe.Tetrahedron4())
    rng = np.random.default_rng(5)
    law = omat.NeoHookean(1.0, 10.0)
    u, v = 0.05 * rng.standard_normal(c.shape[0] * 3), rng.standard_normal(c.shape[0] * 3)
    h = 1e-30
    cs = np.imag(omat.residual(op, law, u + 1j * h * v)) / h
    assert rel(omat.hvp(op, law, u, v), cs) < 1e-13


def test_reference_sparse_hessian_case(golden):
    """tests/test_sparse.py:48-80: Tri3 8x8, 2-dof elasticity mu=1, lambda=0; colored
    compressed Hessian + decompression equals the dense Hessian."""
    c, e = om.unit_square(8, 8)
    op = oop.OracleOperator(c, e, oe.Tri3())
    law = omat.LinearElastic(1.0, 0.0, 2)
    csr = osp.pattern_from_mesh(c, e, 2)
    np.testing.assert_array_equal(csr.indices, golden["sq8_pat2_indices"])
    colors = osp.distance2_colors(csr.indptr, csr.indices, csr.shape[0])
    np.testing.assert_array_equal(colors, golden["sq8_pat2_colors"])
    n = csr.shape[0]
    u0 = np.zeros(n)
    Jc = osp.colored_jacobian(lambda s: omat.hvp(op, law, u0, s), n, colors)
    r, cc = osp.compute_rows_cols(csr.indptr, csr.indices, colors)
    data = osp.decompress(Jc, r, cc)
    import scipy.sparse as sps

    K = sps.csr_matrix((data, csr.indices, csr.indptr), shape=(n, n)).toarray()
    np.testing.assert_allclose(K, golden["sq8_le_dense_K"], rtol=1e-7, atol=1e-13)
    Ke = omat.element_tangents(op, law, u0)
    np.testing.assert_allclose(omat.assemble_dense(op, Ke, 2), golden["sq8_le_dense_K"],
                               rtol=1e-7, atol=1e-13)


def test_element_tangent_matches_hvp_neo_hookean():
    c, e = om.brick(2, 2, 1)
    c = om.jitter_interior(c, 0.5, 0.1, seed=1)
    op = oop.OracleOperator(c, e, oe.Hexahedron8())
    law = omat.NeoHookean(1.0, 10.0)
    rng = np.random.default_rng(2)
    u, v = 0.05 * rng.standard_normal(c.shape[0] * 3), rng.standard_normal(c.shape[0] * 3)
    K = omat.assemble_dense(op, omat.element_tangents(op, law, u), 3)
    assert rel(K @ v, omat.hvp(op, law, u, v)) < 1e-13
    assert rel(K, K.T) < 1e-13


# ------------------------------------------------------------------ lifter
def test_lifter_known_answers():
    """tests/test_lifter.py:11-20 and the Fixed semantics (constraints.py:312-318)."""
    lf = olift.Lifter(4)
    np.testing.assert_array_equal(lf.lift_from_zeros(np.arange(4.0)), np.arange(4.0))
    lf = olift.Lifter(6, olift.Fixed(np.array([0, 5]), 0.0))
    full = lf.lift_from_zeros(np.array([10.0, 20.0, 30.0, 40.0]))
    np.testing.assert_array_equal(full, [0, 10, 20, 30, 40, 0])
    np.testing.assert_array_equal(lf.reduce(full), [10, 20, 30, 40])
    np.testing.assert_array_equal(lf.reduce_adjoint(np.arange(6.0)), [1, 2, 3, 4])
    lf2 = olift.Lifter(6, olift.Fixed(np.array([0, 5]), np.array([0.0, 1.0])))
    np.testing.assert_array_equal(lf2.lift_from_zeros(np.zeros(4)), [0, 0, 0, 0, 0, 1])


@pytest.mark.parametrize("key", ["hexj", "hexa"])
def test_oracle_projection_reproduces_fe_fields(golden, key):
    """The L2 projection of the quadrature values of a nodal field is that field
    (utils.py:118-262 solves M x = int N field).  Hex8's 2x2x2 Gauss rule integrates
    the mass matrix exactly; the one-point rules of Tri3/Tet4 give a rank-deficient
    element mass matrix, for which the property does not hold."""
    from oracle import elements as oe
    from oracle import operator as oop

    c, e = golden[f"{key}_coords"], golden[f"{key}_elements"]
    el = oe.Hexahedron8()
    oo = oop.OracleOperator(c, e, el)
    rng = np.random.default_rng(1)
    u = rng.standard_normal((c.shape[0], 2))
    x = oop.project(oo, oo.eval(u))
    np.testing.assert_allclose(x, u, rtol=0, atol=1e-11 * np.abs(u).max())
