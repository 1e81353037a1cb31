"""Parity with the oracle at the full sizes of the benchmark configurations.

The kernels run on the whole mesh; the oracle evaluates the same quantity at a
seeded sample of nodes (rows), from the elements that hold them -- which is all
that a node's entry depends on -- so that it finishes in seconds at these sizes.

* 128^3 Hex8 brick (6,440,067 dofs): FP64 residual and HVP <= 1e-12 relative,
  FP32 <= 1e-5, with and without the clamped-face Dirichlet mask.
* Kuhn 96^3 Tet4 block, interior jitter 0.2h, Neo-Hookean mu = 1, lambda = 10
  (2,738,019 dofs, 121,188,969 nonzeros, 90 colours): FP64 residual, HVP and colored
  Hessian values at the sampled rows <= 1e-12; compute_rows_cols bit-exact over all
  nonzeros.  The pattern and colouring at this size are compared bit for bit on the
  host (tests/test_host_setup.py).
* 4096 random unit squares of the batched configuration, solved in one launch:
  a seeded sample of 256 meshes against oracle direct solves, <= 1e-8 at rel-res 1e-10.
Relative errors are max-norm over the sampled entries over the max of the oracle's.
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
from tatva_gb300 import Mesh, Operator, batched, element, materials, sparse
from tatva_gb300.problems import clamped_brick, stretched_kuhn

pytestmark = pytest.mark.gpu

F64_TOL = 1e-12
F32_TOL = 1e-5


def rel(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _sample_nodes(n_nodes, k, seed, extra=()):
    rng = np.random.default_rng(seed)
    s = np.unique(np.concatenate([rng.choice(n_nodes, size=k, replace=False),
                                  np.asarray(extra, dtype=np.int64)]))
    return s


def _sub_operator(c, e, nodes, elem):
    """Oracle operator on the elements that hold any sampled node."""
    mark = np.zeros(c.shape[0], bool)
    mark[nodes] = True
    sel = np.nonzero(mark[e].any(axis=1))[0]
    return oop.OracleOperator(c, e[sel], elem), sel


def _dofs(nodes, nv=3):
    return (np.asarray(nodes)[:, None] * nv + np.arange(nv)).reshape(-1)


def test_brick_128_fp64_fp32_vs_oracle_sample(cuda):
    n = 128
    P = clamped_brick(n, cuda)
    en, fixed = P["energy"], P["fixed"]
    c, e = P["mesh"].coords_host(), P["mesh"].elements_host()
    nn = c.shape[0]
    corners = [0, n, (n + 1) * n, (n + 1) ** 2 - 1, nn - 1]
    nodes = _sample_nodes(nn, 3000, seed=11, extra=corners)
    op, _ = _sub_operator(c, e, nodes, oe.Hexahedron8())
    law = omat.LinearElastic(en.p0, en.p1)
    rng = np.random.default_rng(12)
    v = rng.standard_normal(en.n_dofs)
    u = 1e-3 * rng.standard_normal(en.n_dofs)
    d = _dofs(nodes)
    f = fixed.cpu().numpy().astype(bool)
    yo = omat.hvp(op, law, None, v)[d]
    ro = omat.residual(op, law, u)[d]
    yom = omat.hvp(op, law, None, np.where(f, 0.0, v))[d]
    yom[f[d]] = v[d][f[d]]
    for dtype, tol in ((torch.float64, F64_TOL), (torch.float32, F32_TOL)):
        vt = torch.as_tensor(v, dtype=dtype, device=cuda)
        ut = torch.as_tensor(u, dtype=dtype, device=cuda)
        assert rel(en.hvp(None, vt).cpu().numpy()[d], yo) < tol, dtype
        assert rel(en.residual(ut).cpu().numpy()[d], ro) < tol, dtype
        assert rel(en.hvp(None, vt, fixed=fixed).cpu().numpy()[d], yom) < tol, dtype


@pytest.fixture(scope="module")
def kuhn96(cuda):
    P = stretched_kuhn(96, cuda)
    c, e = P["coords"], P["mesh"].elements_host()
    ux = 0.1 * c[:, 0]  # 10 % stretch along x plus a small seeded perturbation
    rng = np.random.default_rng(21)
    u = np.zeros(c.shape[0] * 3)
    u[0::3] = ux
    u += 1e-4 * rng.standard_normal(u.size)
    return P, c, e, u


def test_kuhn96_neo_hookean_residual_hvp_vs_oracle_sample(kuhn96, cuda):
    P, c, e, u = kuhn96
    en = P["energy"]
    nodes = _sample_nodes(c.shape[0], 2000, seed=13, extra=[0, c.shape[0] - 1])
    op, _ = _sub_operator(c, e, nodes, oe.Tetrahedron4())
    law = omat.NeoHookean(1.0, 10.0)
    v = np.random.default_rng(14).standard_normal(u.size)
    d = _dofs(nodes)
    ut = torch.as_tensor(u, device=cuda)
    assert rel(en.residual(ut).cpu().numpy()[d], omat.residual(op, law, u)[d]) < F64_TOL
    assert rel(en.hvp(ut, torch.as_tensor(v, device=cuda)).cpu().numpy()[d],
               omat.hvp(op, law, u, v)[d]) < F64_TOL


def test_kuhn96_colored_hessian_vs_oracle_sample(kuhn96, cuda):
    P, c, e, u = kuhn96
    en = P["energy"]
    cm = sparse.ColoredMatrix.from_csr(sparse.pattern_from_mesh(P["mesh"], 3), device=cuda)
    assert cm.n_colors == 90 and cm.nnz == 121188969
    H = sparse.jacfwd(en.residual, cm)(torch.as_tensor(u, device=cuda))
    indptr = H.indptr.cpu().numpy().astype(np.int64)
    indices = H.indices.cpu().numpy()
    # compute_rows_cols over every nonzero (sparse/base.py:108-136)
    rows, col_colors = sparse.compute_rows_cols(cm)
    colors = cm.colors.cpu().numpy()
    assert np.array_equal(rows.cpu().numpy(), np.repeat(np.arange(indptr.size - 1), np.diff(indptr)))
    assert np.array_equal(col_colors.cpu().numpy(), colors[indices])
    # values of the sampled rows from the oracle's element tangents
    nodes = _sample_nodes(c.shape[0], 1500, seed=15, extra=[0, c.shape[0] - 1])
    op, _ = _sub_operator(c, e, nodes, oe.Tetrahedron4())
    Ke = omat.element_tangents(op, omat.NeoHookean(1.0, 10.0), u)
    edofs = (op.elements[:, :, None] * 3 + np.arange(3)).reshape(op.n_elements, -1)
    m = edofs.shape[1]
    r_all = np.repeat(edofs, m, axis=1).ravel()
    c_all = np.tile(edofs, (1, m)).ravel()
    d = _dofs(nodes)
    keep = np.isin(r_all, d)
    N = u.size
    K = sps.coo_matrix((Ke.ravel()[keep], (r_all[keep], c_all[keep])), shape=(N, N)).tocsr()
    K.sum_duplicates()
    data = H.data.cpu().numpy()
    got, want = [], []
    for r in d:
        k0, k1 = indptr[r], indptr[r + 1]
        got.append(data[k0:k1])
        row = K.getrow(r)
        dense = dict(zip(row.indices, row.data))
        assert set(dense) <= set(indices[k0:k1].tolist())
        want.append(np.array([dense.get(j, 0.0) for j in indices[k0:k1]]))
    assert rel(np.concatenate(got), np.concatenate(want)) < F64_TOL


def test_batched_4096_sample_vs_oracle(cuda):
    meshes, kappas, sides = batched.random_unit_squares(4096, seed=0)
    sysm, b, info = batched.poisson_batch(meshes, kappas, f=1.0, device=cuda)
    res = sysm.solve(b, rtol=1e-10)
    assert res.converged and np.all(res.rel_res <= 1e-10)
    xs = sysm.split(res.x)
    pick = np.random.default_rng(16).choice(len(meshes), size=256, replace=False)
    for i in pick:
        c, e = meshes[i]
        op = oop.OracleOperator(c, e, oe.Tri3())
        law = omat.Poisson(kappas[i], 1.0)
        Ke = omat.element_tangents(op, law, np.zeros(c.shape[0]))
        dofs = e
        m = dofs.shape[1]
        K = sps.coo_matrix((Ke.ravel(), (np.repeat(dofs, m, axis=1).ravel(),
                                         np.tile(dofs, (1, m)).ravel())),
                           shape=(c.shape[0],) * 2).tocsr()
        rhs = -omat.residual(op, law, np.zeros(c.shape[0]))
        free = ~batched.boundary_nodes_tri3(e, c.shape[0])
        xo = np.zeros(c.shape[0])
        xo[free] = spla.spsolve(K[free][:, free].tocsc(), rhs[free])
        x = xs[i].cpu().numpy() if isinstance(xs[i], torch.Tensor) else np.asarray(xs[i])
        assert rel(x, xo) < 1e-8, (i, sides[i])
