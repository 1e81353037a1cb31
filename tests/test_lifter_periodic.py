"""Periodic constraints, adapt_sparsity and the lifted decorator (CPU tensors).

Known answers restate the reference's tests/test_lifter.py:25-42 and
tests/test_lifter_residual.py:7-77; sparsity patterns are compared bit for bit with
the oracle's restatement of constraints.py:184-221 / base.py:281-331.
"""

import numpy as np
import pytest
import torch

from oracle import lifter as olf
from oracle import mesh as om
from oracle import sparse as osp
from tatva_gb300 import Mesh, sparse
from tatva_gb300.lifter import Fixed, Lifter, LifterError, Periodic, lifted


def _t(a):
    return torch.as_tensor(np.asarray(a, dtype=np.float64))


def test_dirichlet_and_periodic_lift():
    lf = Lifter(6, Fixed([0, 5]), Periodic(dofs=[2], master_dofs=[1]))
    u = lf.lift_from_zeros(_t([10.0, 20.0, 30.0]))
    np.testing.assert_array_equal(u.numpy(), [0.0, 10.0, 10.0, 20.0, 30.0, 0.0])
    np.testing.assert_array_equal(lf.reduce(u).numpy(), [10.0, 20.0, 30.0])


def test_reduce_adjoint_periodic_and_mixed():
    lf = Lifter(4, Periodic(dofs=[2], master_dofs=[1]))
    np.testing.assert_array_equal(lf.reduce_adjoint(_t([10.0, 20.0, 30.0, 40.0])).numpy(),
                                  [10.0, 50.0, 40.0])
    lf2 = Lifter(4, Periodic(dofs=[2], master_dofs=[1]), Fixed([3], 0.0))
    np.testing.assert_array_equal(lf2.reduce_adjoint(_t([10.0, 20.0, 30.0, 40.0])).numpy(),
                                  [10.0, 50.0])


def test_lifted_decorator():
    lf = Lifter(4, Periodic(dofs=[2], master_dofs=[1]))

    @lifted(argnums=0, output="dual")
    def residual(u):
        return u * 2.0

    np.testing.assert_array_equal(residual(lf, _t([1.0, 2.0, 3.0])).numpy(), [2.0, 8.0, 6.0])

    @lifted(argnums=0, output="primal")
    def twice(u):
        return u * 2.0

    np.testing.assert_array_equal(twice(Lifter(4, Fixed([0, 3])), _t([10.0, 20.0])).numpy(),
                                  [20.0, 40.0])
    with pytest.raises(LifterError):
        residual(lf, _t([1.0, 2.0]))


def test_periodic_with_shared_masters_matches_oracle():
    rng = np.random.default_rng(0)
    dofs = np.array([7, 3, 9, 12, 5])
    masters = np.array([1, 1, 2, 1, 2])  # several slaves per master
    r = rng.standard_normal(14)
    u = rng.standard_normal(14)
    lf = Lifter(14, Periodic(dofs, masters), Fixed([0], 0.5))
    ol = olf.Lifter(14, olf.Periodic(dofs, masters), olf.Fixed([0], 0.5))
    np.testing.assert_allclose(lf.reduce_adjoint(_t(r)).numpy(), ol.reduce_adjoint(r),
                               rtol=0, atol=1e-15)
    ur = u[ol.free_dofs]
    np.testing.assert_array_equal(lf.lift(_t(ur), _t(u)).numpy(), ol.lift(ur, u))


@pytest.mark.parametrize("ndpn", [1, 2])
def test_adapt_sparsity_periodic_bit_exact(ndpn):
    """x-periodic unit square (right column slaved to the left one) with the bottom
    row fixed: the reduced pattern equals the oracle's M^T S M restatement."""
    n = 6
    c, e = om.unit_square(n, n)
    left = np.where(np.isclose(c[:, 0], 0.0))[0]
    right = np.where(np.isclose(c[:, 0], 1.0))[0]
    left = left[np.argsort(c[left, 1])]
    right = right[np.argsort(c[right, 1])]
    bottom = np.where(np.isclose(c[:, 1], 0.0))[0]
    sl = (right[:, None] * ndpn + np.arange(ndpn)).ravel()
    ms = (left[:, None] * ndpn + np.arange(ndpn)).ravel()
    fx = (bottom[:, None] * ndpn + np.arange(ndpn)).ravel()
    fx = np.setdiff1d(fx, sl)
    csr = sparse.pattern_from_mesh(Mesh(c, e, device="cpu"), ndpn)
    got = Lifter(c.shape[0] * ndpn, Periodic(sl, ms), Fixed(fx)).adapt_sparsity(csr)
    ocsr = osp.pattern_from_mesh(c, e, ndpn)
    want = olf.Lifter(c.shape[0] * ndpn, olf.Periodic(sl, ms), olf.Fixed(fx)).adapt_sparsity(ocsr)
    got.sort_indices()
    want.sort_indices()
    np.testing.assert_array_equal(got.indptr, want.indptr)
    np.testing.assert_array_equal(got.indices, want.indices)
    # the master columns inherit the slave couplings
    assert got.nnz > csr[Lifter(c.shape[0] * ndpn, Periodic(sl, ms), Fixed(fx)).free_dofs.numpy()][
        :, Lifter(c.shape[0] * ndpn, Periodic(sl, ms), Fixed(fx)).free_dofs.numpy()].nnz
