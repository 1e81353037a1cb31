"""Host-side setup of the C ABI (pattern, colouring, incidence, block plan) against
the reference goldens and the oracle.  Runs on the CPU (no GPU compute)."""

import ctypes

import numpy as np
import pytest
import scipy.sparse as sps

from oracle import mesh as om
from oracle import sparse as osp
from tatva_gb300 import Mesh, _lib, sparse
from tatva_gb300.plan import BlockPlan

MESHES = ["tri", "tet", "hexj", "hexa"]


@pytest.mark.parametrize("key", MESHES)
def test_pattern_and_colors_bit_exact_vs_reference(golden, key):
    c, e = golden[f"{key}_coords"], golden[f"{key}_elements"]
    m = Mesh(c, e, device="cpu")
    for ndpn in ((1, 2, 3) if c.shape[1] == 3 else (1, 2)):
        csr = sparse.pattern_from_mesh(m, ndpn)
        assert csr.data.dtype == np.int8 and csr.indices.dtype == np.int32
        np.testing.assert_array_equal(csr.indptr, golden[f"{key}_pat{ndpn}_indptr"])
        np.testing.assert_array_equal(csr.indices, golden[f"{key}_pat{ndpn}_indices"])
        col = sparse.distance2_colors(csr.indptr, csr.indices, csr.shape[0])
        np.testing.assert_array_equal(col, golden[f"{key}_pat{ndpn}_colors"])


def test_mesh_generator_bit_exact_vs_reference(golden):
    for nx, ny in ((3, 2), (8, 8)):
        m = Mesh.unit_square(nx, ny, device="cpu")
        np.testing.assert_array_equal(m.coords.numpy(), golden[f"usq_{nx}x{ny}_coords"])
        np.testing.assert_array_equal(m.elements.numpy(), golden[f"usq_{nx}x{ny}_elements"])


@pytest.mark.parametrize("case", ["tri64", "kuhn6", "brick8", "kuhn_jit5"])
def test_pattern_and_colors_vs_oracle_larger(case):
    """Larger meshes than the goldens: C++ setup == numpy restatement, bit for bit."""
    if case == "tri64":
        c, e = om.unit_square(64, 64)
        ndpn, ncol = 1, 9  # configuration-1 mesh: 9 colours
    elif case == "kuhn6":
        c, e = om.kuhn_box((1, 1, 1), (6, 6, 6), origin=(0, 0, 0))
        ndpn, ncol = 3, None
    elif case == "brick8":
        c, e = om.brick(8, 8, 8)
        ndpn, ncol = 3, 81
    else:
        c, e = om.kuhn_box((1, 1, 1), (5, 4, 3), origin=(0, 0, 0))
        ndpn, ncol = 2, None
    m = Mesh(c, e, device="cpu")
    csr = sparse.pattern_from_mesh(m, ndpn)
    ocsr = osp.pattern_from_mesh(c, e, ndpn)
    np.testing.assert_array_equal(csr.indptr, ocsr.indptr)
    np.testing.assert_array_equal(csr.indices, ocsr.indices)
    col = sparse.distance2_colors(csr.indptr, csr.indices, csr.shape[0])
    if csr.shape[0] <= 6000:
        ocol = osp.distance2_colors(ocsr.indptr, ocsr.indices, ocsr.shape[0])
        np.testing.assert_array_equal(col, ocol)
    assert osp.check_distance2(csr.indptr, csr.indices, col)
    if ncol is not None:
        assert col.max() + 1 == ncol


def test_coloring_of_general_patterns():
    """Unsymmetric / irregular CSR input (from_csr accepts any pattern): the grouped
    C++ greedy equals the row-by-row restatement."""
    rng = np.random.default_rng(0)
    for n, dens in ((40, 0.05), (200, 0.02), (300, 0.01)):
        A = sps.random(n, n, density=dens, random_state=rng, format="csr")
        A = (A + sps.eye(n)).tocsr()
        A.sort_indices()
        # duplicate some rows to exercise the identical-row groups
        rows = [A.getrow(i) for i in range(n)]
        for i in range(1, n, 7):
            rows[i] = rows[i - 1]
        B = sps.vstack(rows).tocsr()
        B.sort_indices()
        col = sparse.distance2_colors(B.indptr, B.indices, n)
        ocol = osp.distance2_colors(B.indptr, B.indices, n)
        np.testing.assert_array_equal(col, ocol)


def test_colored_matrix_from_csr_host(golden):
    csr = sparse.pattern_from_mesh(Mesh.unit_square(8, 8, device="cpu"), 2)
    cm = sparse.ColoredMatrix.from_csr(csr, device="cpu")
    np.testing.assert_array_equal(cm.colors.numpy(), golden["sq8_pat2_colors"])
    assert cm.shape == (162, 162) and cm.n_colors == int(golden["sq8_pat2_colors"].max()) + 1
    back = cm.to_csr()
    np.testing.assert_array_equal(back.indices, csr.indices)


@pytest.mark.parametrize("elem,case,block", [(2, "brick", 512), (2, "brick", 100),
                                              (1, "kuhn", 777), (0, "tri", 300)])
def test_block_plan_invariants(elem, case, block):
    if case == "brick":
        c, e = om.brick(9, 7, 6)
        c = om.jitter_interior(c, 0.1, 0.2, seed=0)
    elif case == "kuhn":
        c, e = om.kuhn_box((1, 1, 1), (6, 5, 7), origin=(0, 0, 0))
    else:
        c, e = om.unit_square(23, 17)
    p = BlockPlan(elem, e, c, "cpu", block_elems=block, max_local_nodes=4096)
    h, s = p.host, p.sizes
    npe, npad = e.shape[1], s["stride"]
    E = e.shape[0]
    # every element exactly once
    np.testing.assert_array_equal(np.sort(h["elem_id"][:E]), np.arange(E))
    covered_slots = []
    for b in range(s["n_blocks"]):
        e0, e1 = h["blk_elem_ptr"][b], h["blk_elem_ptr"][b + 1]
        n0, n1 = h["blk_node_ptr"][b], h["blk_node_ptr"][b + 1]
        assert e1 - e0 <= block
        gid = h["lnode_gid"][n0:n1]
        assert np.all(np.diff(gid) > 0)  # sorted unique
        smem = h["lnode_smem"][n0:n1]
        nl = n1 - n0
        assert len(np.unique(smem)) == nl and smem.min() >= 0 and smem.max() < 8 * ((nl + 7) // 8)
        inv = np.full(8 * ((nl + 7) // 8), -1)
        inv[smem] = np.arange(nl)
        for k in range(e0, e1):
            lc = h["lconn"][k * npad:k * npad + npe].astype(np.int64)  # shared-memory slots
            np.testing.assert_array_equal(gid[inv[lc]], e[h["elem_id"][k]])
        # colour classes: no two elements of one colour share a node
        c0, c1 = h["blk_color_ptr"][b], h["blk_color_ptr"][b + 1]
        ofs = h["color_ofs"][c0:c1]
        assert ofs[0] == 0 and ofs[-1] == e1 - e0
        for a, z in zip(ofs[:-1], ofs[1:]):
            nodes = np.concatenate([e[h["elem_id"][e0 + k]] for k in range(a, z)])
            assert len(np.unique(nodes)) == len(nodes)
        # owned-alone nodes really are touched only by this block
        slots = h["lnode_slot"][n0:n1]
        blk_elems = set(h["elem_id"][e0:e1].tolist())
        for g_, sl in zip(gid, slots):
            touching = set(np.where((e == g_).any(axis=1))[0].tolist())
            if sl < 0:
                assert touching <= blk_elems
            else:
                assert not touching <= blk_elems
                covered_slots.append(sl)
    # shared-node CSR lists every slot once, in block order
    assert sorted(covered_slots) == list(range(s["n_partials"]))
    assert h["shared_ptr"][-1] == s["n_partials"] if s["n_shared"] else True


def test_general_blocks_spread_warp_accesses_over_the_banks():
    """The general block kernel reads scalar node records (word d of a node at slot x 3
    + d for Tet4), one wavefront per warp when the 32 lanes' slots differ modulo 32.
    On a Kuhn plan, a warp's access at one element corner must need well under the
    3.1 wavefronts that a modulo-8 placement gave (a random one gives ~3.5); the
    placement reaches ~2.2 here."""
    c, e = om.kuhn_box((1, 1, 1), (12, 12, 12), origin=(0, 0, 0))
    p = BlockPlan(_lib.TG_TET4, e, c, "cpu", block_elems=2048, max_local_nodes=4096)
    h, s = p.host, p.sizes
    npad = s["stride"]

    def wavefronts(words):
        banks = words % 32
        return max(len(np.unique(words[banks == b])) for b in np.unique(banks))

    w = []
    for b in range(s["n_blocks"]):
        e0, e1 = h["blk_elem_ptr"][b], h["blk_elem_ptr"][b + 1]
        lc = h["lconn"][e0 * npad:e1 * npad].reshape(-1, npad)[:, :4].astype(np.int64)
        for g0 in range(0, e1 - e0, 32):
            w += [wavefronts(3 * lc[g0:g0 + 32, a]) for a in range(4)]
    assert s["n_blocks"] > 1 and np.mean(w) < 2.5, np.mean(w)


def test_affine_hex_blocks_spread_16_byte_accesses_over_the_bank_groups():
    """The affine Hex8 kernels read 16-byte node records: a warp's access is served
    in four 8-lane phases, each free of conflicts when its lanes' slots differ modulo
    8.  On the box (non-lattice) blocks of a brick the plan's placement needs about
    5.3 wavefronts per 32-lane access at one element corner (4 = conflict-free); a
    random placement of the same slots needs about 10."""
    c, e = om.brick(18, 14, 12, lengths=(1.0, 0.8, 0.7))
    p = BlockPlan(_lib.TG_HEX8, e, c, "cpu", block_elems=512, max_local_nodes=4096)
    h, s = p.host, p.sizes
    npad = s["stride"]
    assert s["n_affine_blocks"] > s["n_lattice_blocks"]

    def wavefronts(slots):
        groups = [slots[q:q + 8] % 8 for q in range(0, len(slots), 8)]
        return sum(np.bincount(g).max() for g in groups)

    w = []
    for b in range(s["n_lattice_blocks"], s["n_affine_blocks"]):
        e0, e1 = h["blk_elem_ptr"][b], h["blk_elem_ptr"][b + 1]
        lc = h["lconn"][e0 * npad:e1 * npad].reshape(-1, npad)[:, :8].astype(np.int64)
        for g0 in range(0, e1 - e0, 32):
            w += [wavefronts(lc[g0:g0 + 32, a]) for a in range(8)]
    assert np.mean(w) < 6.5, np.mean(w)


def test_element_colors_and_incidence():
    c, e = om.kuhn_box((1, 1, 1), (4, 3, 5), origin=(0, 0, 0))
    E, npe = e.shape
    L = _lib.lib()
    colors = np.zeros(E, np.int32)
    order = np.zeros(E, np.int32)
    cptr = np.zeros(129, np.int32)
    nc = ctypes.c_int32()
    _lib.check(L.tg_element_colors(e.ctypes.data, E, npe, c.shape[0], colors.ctypes.data,
                                   order.ctypes.data, cptr.ctypes.data, ctypes.byref(nc)))
    np.testing.assert_array_equal(colors, osp.element_colors(e, c.shape[0]))
    for k in range(nc.value):
        sel = order[cptr[k]:cptr[k + 1]]
        assert np.all(colors[sel] == k) and np.all(np.diff(sel) > 0)
    ip = np.zeros(c.shape[0] + 1, np.int32)
    ix = np.zeros(E * npe, np.int32)
    _lib.check(L.tg_node_incidence(e.ctypes.data, E, npe, c.shape[0], ip.ctypes.data,
                                   ix.ctypes.data))
    for n in range(0, c.shape[0], 7):
        ent = ix[ip[n]:ip[n + 1]]
        assert np.all(e.reshape(-1)[ent] == n) and np.all(np.diff(ent) > 0)
        assert len(ent) == np.sum(e == n)


def test_batch_helpers_boundary_and_concat():
    from tatva_gb300 import batched

    c, e = om.unit_square(5, 3)
    mask = batched.boundary_nodes_tri3(e, c.shape[0])
    geo = (np.isclose(c[:, 0], 0) | np.isclose(c[:, 0], 1) | np.isclose(c[:, 1], 0)
           | np.isclose(c[:, 1], 1))
    np.testing.assert_array_equal(mask, geo)
    c2, e2 = om.unit_square(2, 2)
    cc, ee, nofs, eofs = batched.concat_meshes([(c, e), (c2, e2)])
    assert list(nofs) == [0, c.shape[0], c.shape[0] + c2.shape[0]]
    assert list(eofs) == [0, e.shape[0], e.shape[0] + e2.shape[0]]
    np.testing.assert_array_equal(ee[e.shape[0]:], e2 + c.shape[0])
    meshes, kappas, sides = batched.random_unit_squares(64, seed=5)
    assert sides.min() >= 8 and sides.max() <= 96 and len(meshes) == 64
    assert all(k.shape[0] == 2 * n * n for k, n in zip(kappas, sides))


def test_synthetic_request_stream():
    from tatva_gb300 import serving

    reqs = serving.synthetic_requests(2000, rate=2000.0, seed=0)
    arr = np.array([r.arrival for r in reqs])
    assert arr[0] == 0.0 and np.all(np.diff(arr) >= 0)
    assert 0.8 < (len(arr) - 1) / arr[-1] / 2000.0 < 1.2
    assert {r.side for r in reqs} == {16, 24, 32, 48, 64}
    assert all(0.2 <= r.poisson <= 0.45 for r in reqs)


@pytest.mark.parametrize("shape,n_lat,n_blocks", [((16, 16, 16), 8, 8), ((20, 20, 20), 8, 27),
                                                   ((24, 16, 8), 6, 6), ((12, 12, 12), 1, 8)])
def test_lattice_blocks_of_structured_bricks(shape, n_lat, n_blocks):
    """Structured bricks (any spacing per axis): every full 8 x 8 x 8 cube of cells is
    one lattice block, local nodes in grid order l = i + 9 j + 81 k; other cells form
    blocks of their own.  Node numbering does not matter; a moved node does."""
    rng = np.random.default_rng(0)
    c, e = om.brick(*shape, lengths=tuple(float(s) for s in shape))
    for d in range(3):  # uneven spacing per axis
        lines = np.cumsum(np.r_[0.0, 0.5 + rng.random(shape[d])])
        c[:, d] = lines[np.rint(c[:, d]).astype(int)]
    perm = rng.permutation(c.shape[0])
    c, e = c[perm], np.argsort(perm)[e]
    p = BlockPlan(_lib.TG_HEX8, e, c, "cpu", block_elems=512, threads=128)
    assert p.sizes["n_lattice_blocks"] == n_lat and p.sizes["n_blocks"] == n_blocks
    bnp, gid = p.host["blk_node_ptr"], p.host["lnode_gid"]
    for b in range(n_lat):
        x = c[gid[bnp[b]:bnp[b + 1]]].reshape(9, 9, 9, 3)  # [k][j][i]
        assert np.all(np.diff(x[..., 0], axis=2) > 0) and np.all(np.diff(x[..., 1], axis=1) > 0)
        assert np.all(np.diff(x[..., 2], axis=0) > 0)
        assert np.all(x[..., 0] == x[0, 0, :, 0]) and np.all(x[..., 2] == x[:, :1, :1, 2])
    c2 = c.copy()
    c2[np.argmin(np.linalg.norm(c2 - c2.mean(axis=0), axis=1))] += 0.01
    p2 = BlockPlan(_lib.TG_HEX8, e, c2, "cpu", block_elems=512, threads=128)
    assert p2.sizes["n_lattice_blocks"] < max(n_lat, 1)


def _detect(c, e, elem=_lib.TG_HEX8):
    gn = (ctypes.c_int32 * 3)()
    gh = (ctypes.c_double * 3)()
    c = np.ascontiguousarray(c, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.int32)
    _lib.check(_lib.lib().tg_grid_detect(elem, e.ctypes.data, e.shape[0], c.shape[0],
                                         c.ctypes.data, c.shape[1], gn, gh))
    return tuple(gn), tuple(gh)


def test_grid_detect_structured_bricks():
    """Structured bricks (node id i + Nx (j + Ny k), uniform spacing per axis, each cell
    once with the reference corner order) are recognised; anything else is not."""
    c, e = om.brick(7, 5, 6, lengths=(0.7, 0.5, 1.2))
    n, h = _detect(c, e)
    assert n == (8, 6, 7) and np.allclose(h, (0.1, 0.1, 0.2), rtol=1e-14)
    # element order does not matter
    perm = np.random.default_rng(0).permutation(e.shape[0])
    assert _detect(c, e[perm])[0] == (8, 6, 7)
    # one cell: all nodes on the boundary
    assert _detect(*om.brick(1, 1, 1))[0] == (2, 2, 2)
    # not bricks: uneven spacing, jitter, renumbered nodes, rotated corner order,
    # a missing or repeated cell, a Tet4 mesh
    cg = c.copy()
    cg[:, 0] = np.where(c[:, 0] > 0.35, c[:, 0] + 0.01 * (c[:, 0] - 0.35), c[:, 0])
    assert _detect(cg, e)[0] == (0, 0, 0)
    assert _detect(om.jitter_interior(c, 0.1, 0.2, seed=1), e)[0] == (0, 0, 0)
    p = np.random.default_rng(1).permutation(c.shape[0])
    inv = np.empty_like(p)
    inv[p] = np.arange(p.size)
    assert _detect(c[p], inv[e])[0] == (0, 0, 0)
    assert _detect(c, np.roll(e, 1, axis=1))[0] == (0, 0, 0)
    e2 = e.copy()
    e2[3] = e2[4]
    assert _detect(c, e2)[0] == (0, 0, 0)
    ck, ek = om.kuhn_box((1, 1, 1), (3, 3, 3), origin=(0, 0, 0))
    assert _detect(ck, ek, _lib.TG_TET4)[0] == (0, 0, 0)
    # the plan carries the result, and can switch the stencil schedule off
    plan = BlockPlan(_lib.TG_HEX8, e, c, "cpu")
    assert plan.grid and tuple(plan.struct.grid_nodes) == (8, 6, 7)
    plan.grid = False
    assert not plan.grid and tuple(plan.struct.grid_nodes) == (0, 0, 0)
    plan.grid = True
    assert tuple(plan.struct.grid_nodes) == (8, 6, 7)


def test_pattern_and_colors_bit_exact_at_kuhn96():
    """The Neo-Hookean configuration's full size (Kuhn 96^3 Tet4, 2,738,019 dofs,
    121,188,969 nonzeros): pattern and natural-order distance-2 colouring bit for bit
    against the oracle's C restatement of _extraction.py:37-102 and
    _coloring.py:27-48, 136-153 (the Python oracle's loops are too slow at this size;
    the C restatement equals it on the small cases of this file)."""
    from oracle import cbuild

    c, e = om.kuhn_box((1, 1, 1), (96, 96, 96), origin=(0, 0, 0))
    ip, ix = cbuild.pattern(e, c.shape[0], 3)
    csr = sparse.pattern_from_mesh(Mesh(c, e, device="cpu"), 3)
    assert ix.size == 121188969
    assert np.array_equal(csr.indptr, ip) and np.array_equal(csr.indices, ix)
    del csr
    colors = cbuild.d2_colors(ip, ix)
    got = sparse.distance2_colors(ip.astype(np.int32), ix, ip.size - 1)
    assert int(colors.max()) + 1 == 90
    assert np.array_equal(np.asarray(got), colors)


@pytest.mark.parametrize("case", ["tri", "hex", "tet"])
def test_c_oracle_equals_python_oracle(case):
    from oracle import cbuild

    c, e, nd = {"tri": om.unit_square(9, 7) + (1,), "hex": om.brick(3, 4, 2) + (3,),
                "tet": om.kuhn_box((1, 1, 1), (4, 3, 5), origin=(0, 0, 0)) + (3,)}[case]
    ip, ix = cbuild.pattern(e, c.shape[0], nd)
    ref = osp.pattern_from_mesh(c, e, nd)
    assert np.array_equal(ip, ref.indptr) and np.array_equal(ix, ref.indices)
    assert np.array_equal(cbuild.d2_colors(ip, ix),
                          osp.distance2_colors(ref.indptr, ref.indices, ref.shape[0]))
