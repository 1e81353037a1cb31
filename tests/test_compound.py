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
