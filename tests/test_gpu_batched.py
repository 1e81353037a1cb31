"""Batched multi-mesh Poisson solve (one persistent launch) against the oracle.

Each mesh's solution is checked against a direct solve of the oracle-assembled
FP64 system (element tangents of psi = 1/2 kappa_e |grad u|^2 - f u, zero
Dirichlet values on the boundary): relative error <= 1e-8 at rel-res 1e-10.
A mesh's result must not depend on the batch it is solved in: bitwise equal alone
and in the batch, and between repeated solves and graph replays.
"""

import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla
import torch

from oracle import elements as oe
from oracle import materials as omat
from oracle import mesh as om
from oracle import operator as oop
from oracle import sparse as osp
from tatva_gb300 import batched

pytestmark = pytest.mark.gpu

SIDES = [3, 9, 5, 16, 4, 12, 7, 24]


def _meshes(seed=0, sides=SIDES):
    rng = np.random.default_rng(seed)
    meshes, kappas = [], []
    for n in sides:
        c, e = om.unit_square(n, n)
        meshes.append((c, e))
        kappas.append(rng.lognormal(0.0, 1.0, size=e.shape[0]))
    return meshes, kappas


def _oracle_solution(c, e, kappa, f=1.0):
    op = oop.OracleOperator(c, e, oe.Tri3())
    law = omat.Poisson(kappa, f)
    Ke = omat.element_tangents(op, law, np.zeros(c.shape[0]))
    ocsr = osp.pattern_from_mesh(c, e, 1)
    data = omat.assemble_csr_data(op, Ke, 1, ocsr.indptr, ocsr.indices)
    K = sps.csr_matrix((data, ocsr.indices, ocsr.indptr), shape=(c.shape[0],) * 2)
    b = -omat.residual(op, law, np.zeros(c.shape[0]))
    fixed = batched.boundary_nodes_tri3(e, c.shape[0])
    free = ~fixed
    x = np.zeros(c.shape[0])
    x[free] = spla.spsolve(K[free][:, free].tocsc(), b[free])
    return x


def test_batched_poisson_matches_oracle(cuda):
    meshes, kappas = _meshes()
    sysm, b, info = batched.poisson_batch(meshes, kappas, f=1.0, device=cuda)
    res = sysm.solve(b, rtol=1e-10, inner_rtol=1e-3)
    assert res.converged, res.status
    assert np.all(res.rel_res <= 1e-10)
    assert np.all(res.refinements >= 1)
    xs = sysm.split(res.x)
    for (c, e), k, x in zip(meshes, kappas, xs):
        xr = _oracle_solution(c, e, k)
        err = np.max(np.abs(x.cpu().numpy() - xr)) / np.max(np.abs(xr))
        assert err < 1e-8, err


def test_batched_result_independent_of_the_batch(cuda):
    meshes, kappas = _meshes(seed=1)
    sysm, b, _ = batched.poisson_batch(meshes, kappas, device=cuda)
    full = sysm.split(sysm.solve(b).x)
    again = sysm.split(sysm.solve(b).x)
    for s in (0, 3, 7):
        alone, b1, _ = batched.poisson_batch([meshes[s]], [kappas[s]], device=cuda)
        x1 = alone.solve(b1).x
        assert torch.equal(x1, full[s]), s
    for a, z in zip(full, again):
        assert torch.equal(a, z)
    # reversed batch order: same per-mesh bits
    rsys, rb, _ = batched.poisson_batch(meshes[::-1], kappas[::-1], device=cuda)
    rev = rsys.split(rsys.solve(rb).x)[::-1]
    for a, z in zip(full, rev):
        assert torch.equal(a, z)


@pytest.mark.parametrize("threads", [128, 256, 512])
def test_batched_graph_replay_and_block_sizes(cuda, threads):
    meshes, kappas = _meshes(seed=2, sides=[6, 11, 20, 3])
    sysm, b, _ = batched.poisson_batch(meshes, kappas, device=cuda)
    bb = b.to(torch.float64).contiguous()
    x = torch.empty_like(bb)
    g = sysm.capture(bb, x, threads=threads, ctas_per_sm=1)
    g.replay()
    torch.cuda.synchronize()
    r1 = sysm.result(x.clone())
    assert r1.converged and np.all(r1.rel_res <= 1e-10)
    x.fill_(7.0)
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(x, r1.x)


def test_batched_limits_and_statuses(cuda):
    meshes, kappas = _meshes(seed=3, sides=[5, 8])
    sysm, b, _ = batched.poisson_batch(meshes, kappas, device=cuda)
    res = sysm.solve(b, max_outer=0)
    assert np.all(res.status == 5) and np.all(res.rel_res == 1.0)
    zero = torch.zeros_like(b)
    res0 = sysm.solve(zero)
    assert res0.converged and torch.count_nonzero(res0.x) == 0
    with pytest.raises(ValueError):
        sysm.solve(b, inner_rtol=2.0)
