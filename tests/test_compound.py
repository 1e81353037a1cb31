"""Compound states and pattern_from_compound (host side, CPU).

Known answers restate the reference's tests/test_compound.py (layout, access,
stacking, AUTO nodal sizing); the sparsity of a single nodal field equals
pattern_from_mesh, and mixed fields follow _extraction.py:117-245.
"""

import numpy as np
import pytest
import torch

from oracle import mesh as om
from tatva_gb300 import Mesh, sparse
from tatva_gb300.compound import (Compound, CompoundError, FieldSize, FieldType, Nodal, field,
                                  pattern_from_compound, stack_fields)


class SimpleState(Compound):
    u = field((2, 3))
    phi = field((2,))


@stack_fields("u", "v", axis=-1)
class StackedState(Compound):
    u = field((2, 2))
    v = field((2, 2))
    w = field((2,))


@pytest.mark.parametrize("cls", [SimpleState, StackedState])
def test_size_and_zero_init(cls):
    s = cls()
    assert s.arr.shape == (cls.size,) and torch.count_nonzero(s.arr) == 0


def test_access_assignment_iteration():
    s = SimpleState()
    assert SimpleState.size == 8
    u = torch.arange(6.0).reshape(2, 3)
    s = s.at("u").set(u).at("phi").set(torch.tensor([10.0, 20.0]))
    assert torch.equal(s.u, u) and torch.equal(s.phi, torch.tensor([10.0, 20.0]))
    assert torch.equal(s.arr[:6], u.flatten()) and torch.equal(s.arr[6:], torch.tensor([10.0, 20.0]))
    assert len(s) == 2 and [c.shape for c in s] == [(2, 3), (2,)]
    np.testing.assert_array_equal(SimpleState.u[1], [3, 4, 5])
    np.testing.assert_array_equal(SimpleState.u[:, 1], [1, 4])
    np.testing.assert_array_equal(np.atleast_1d(SimpleState.phi[1]), [7])
    t = SimpleState(torch.arange(8.0)) + SimpleState(2 * torch.arange(8.0))
    assert torch.equal(t.arr, 3 * torch.arange(8.0))
    with pytest.raises(AttributeError):
        s.at("nope")


def test_stacked_layout():
    s = StackedState(torch.arange(float(StackedState.size)))
    assert torch.equal(s.u, torch.tensor([[0.0, 1.0], [4.0, 5.0]]))
    assert torch.equal(s.v, torch.tensor([[2.0, 3.0], [6.0, 7.0]]))
    assert torch.equal(s.w, torch.tensor([8.0, 9.0]))
    np.testing.assert_array_equal(StackedState.u[1], [4, 5])
    np.testing.assert_array_equal(StackedState.v[0], [2, 3])


def test_auto_sized_nodal_fields():
    c, e = om.unit_square(4, 1)  # 10 nodes
    mesh = Mesh(c, e, device="cpu")

    class MyState(Compound, mesh=mesh):
        param1 = field(shape=(5,))
        u = field(shape=(FieldSize.AUTO, 3))
        phi = field(shape=(FieldSize.AUTO,))
        param2 = field(shape=(2,))

    s = MyState()
    assert [n for n, _ in MyState.fields] == ["param1", "u", "phi", "param2"]
    p1, u, phi, p2 = s
    assert (p1.shape, u.shape, phi.shape, p2.shape) == ((5,), (10, 3), (10,), (2,))
    assert MyState.size == 47
    np.testing.assert_array_equal(MyState.u.indices(), [i * 4 + j for i in range(10) for j in range(3)])
    np.testing.assert_array_equal(MyState.phi.indices(), [i * 4 + 3 for i in range(10)])
    np.testing.assert_array_equal(MyState.param1.indices(), np.arange(40, 45))
    np.testing.assert_array_equal(MyState.param2.indices(), np.arange(45, 47))
    with pytest.raises(CompoundError):
        class NoMesh(Compound):  # noqa: F841
            u = field(shape=(FieldSize.AUTO,))


def test_pattern_single_nodal_field_equals_mesh_pattern():
    c, e = om.unit_square(5, 4)
    mesh = Mesh(c, e, device="cpu")

    class S(Compound, mesh=mesh):
        u = field(shape=(FieldSize.AUTO, 2))

    got = pattern_from_compound(S)
    want = sparse.pattern_from_mesh(mesh, 2)
    np.testing.assert_array_equal(got.indptr, want.indptr)
    np.testing.assert_array_equal(got.indices, want.indices)


def test_pattern_mixed_fields_and_blocks():
    c, e = om.unit_square(3, 3)
    mesh = Mesh(c, e, device="cpu")
    N = c.shape[0]

    class S(Compound, mesh=mesh):
        u = field(shape=(FieldSize.AUTO, 2))
        p = field(shape=(FieldSize.AUTO,))
        lam = field(shape=(3,))

    with pytest.warns(UserWarning):
        P = pattern_from_compound(S)
    assert P.shape == (S.size, S.size) and S.size == 3 * N + 3
    # u and p dofs of one element couple; the 3 extra dofs only to themselves
    el = e[0]
    ud = S.u[el].reshape(-1)
    pd = S.p[el].reshape(-1)
    dense = P.toarray()
    assert dense[np.ix_(ud, pd)].all() and dense[np.ix_(pd, ud)].all()
    lam = S.lam.indices()
    assert (dense[lam][:, lam] == np.eye(3)).all() and dense[lam].sum() == 3
    with pytest.warns(UserWarning):
        blocks = pattern_from_compound(S, block_wise=True)
    assert len(blocks) == 2 and blocks[0][0].shape == (3 * N, 3 * N) and blocks[1][1].shape == (3, 3)


def _golden_classes():
    from tatva_gb300.compound import Nodal

    ct, et = om.kuhn_box((1, 1, 1), (2, 2, 1), origin=(0, 0, 0))
    mt = Mesh(ct, et, device="cpu")
    cq, eq = om.unit_square(3, 2)
    mq = Mesh(cq, eq, device="cpu")

    class TwoNodal(Compound, mesh=mt):
        u = field((FieldSize.AUTO, 3))
        theta = field((FieldSize.AUTO,))

    class NodalAndLocal(Compound, mesh=mt):
        u = field((FieldSize.AUTO, 3))
        p = field((5,))

    class PartialNodal(Compound, mesh=mq):
        u = field((FieldSize.AUTO, 2))
        lam = field((4,), field_type=Nodal(node_ids=np.array([0, 3, 5, 11])))

    return {"two_nodal": TwoNodal, "nodal_local": NodalAndLocal, "partial_nodal": PartialNodal}


@pytest.mark.parametrize("name", ["two_nodal", "nodal_local", "partial_nodal"])
def test_layout_and_pattern_bit_exact_vs_reference(name):
    """Field index maps, pattern_from_compound and its block-wise split equal the
    reference's own (tests/golden/compound_golden.npz, written by make_golden.py from
    tatva/compound/__init__.py and tatva/sparse/_extraction.py:117-245)."""
    import os
    import warnings

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "compound_golden.npz"))
    cls = _golden_classes()[name]
    assert cls.size == int(g[f"{name}_size"])
    for fname, f in cls.fields:
        assert np.array_equal(np.asarray(f.indices(slice(None))).reshape(-1),
                              g[f"{name}_field_{fname}"]), fname
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        pat = pattern_from_compound(cls)
        blocks = pattern_from_compound(cls, block_wise=True)
    assert np.array_equal(pat.indptr, g[f"{name}_indptr"])
    assert np.array_equal(pat.indices, g[f"{name}_indices"])
    shapes = np.array([[b.shape[0], b.shape[1], b.nnz] for row in blocks for b in row])
    assert np.array_equal(shapes, g[f"{name}_block_shapes"])
