"""Element-block plan on the device (see ``tg_block_plan`` in include/tatva_gb300.h).

Built once per (mesh, element, tuning) on the host by ``tg_plan_build`` and copied
to the GPU.  The plan fixes the order of every floating-point addition of the
fused residual / HVP kernels, which makes them deterministic.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

# Defaults measured on GB300 (HVP, graph-timed): Tri3 Poisson 1024^2 best at 2048 / 256,
# Kuhn Tet4 96^3 at 2048 / 128 (34 colours per block: fewer threads keep more of them
# busy in each colour pass), Hex8 box bricks at 512 elements per block -- on structured
# bricks each full 8 x 8 x 8 cube of cells is then a lattice block (sizes
# "n_lattice_blocks"), which the FP32 linear-elastic kernels sum without colouring.
DEFAULT_BLOCK_ELEMS = {_lib.TG_TRI3: 2048, _lib.TG_TET4: 2048, _lib.TG_HEX8: 512}
DEFAULT_THREADS = {_lib.TG_TRI3: 256, _lib.TG_TET4: 128, _lib.TG_HEX8: 128}
DEFAULT_MAX_LOCAL = 4096


class BlockPlan:
    def __init__(self, elem_id: int, elements: np.ndarray, coords: np.ndarray, device,
                 block_elems: int | None = None, max_local_nodes: int = DEFAULT_MAX_LOCAL,
                 threads: int = 256):
        L = _lib.lib()
        self.elem = elem_id
        self.block_elems = int(block_elems or DEFAULT_BLOCK_ELEMS[elem_id])
        self.max_local_nodes = int(max_local_nodes)
        conn = np.ascontiguousarray(elements, dtype=np.int32)
        xyz = np.ascontiguousarray(coords, dtype=np.float64)
        h = ctypes.c_void_p()
        _lib.check(L.tg_plan_build(elem_id, conn.ctypes.data, conn.shape[0], xyz.shape[0],
                                   xyz.ctypes.data, xyz.shape[1], self.block_elems,
                                   self.max_local_nodes, ctypes.byref(h)))
        try:
            sizes = np.zeros(13, dtype=np.int64)
            _lib.check(L.tg_plan_sizes(h, sizes.ctypes.data))
            nb, ne, ncol, nloc, nsh, npart, maxl, maxc, npad, naff, ndiag, maxe, nlat = (
                int(x) for x in sizes)
            host = {
                "blk_elem_ptr": np.zeros(nb + 1, np.int32),
                "blk_color_ptr": np.zeros(nb + 1, np.int32),
                "color_ofs": np.zeros(max(ncol, 1), np.int32),
                "blk_node_ptr": np.zeros(nb + 1, np.int32),
                "lconn": np.zeros(max(ne * npad, 8), np.uint16),
                "elem_id": np.zeros(max(ne, 1), np.int32),
                "lnode_gid": np.zeros(max(nloc, 1), np.int32),
                "lnode_slot": np.zeros(max(nloc, 1), np.int32),
                "lnode_smem": np.zeros(max(nloc, 1), np.int32),
                "shared_node": np.zeros(max(nsh, 1), np.int32),
                "shared_ptr": np.zeros(nsh + 1, np.int32),
                "shared_slots": np.zeros(max(npart, 1), np.int32),
            }
            order = ["blk_elem_ptr", "blk_color_ptr", "color_ofs", "blk_node_ptr", "lconn",
                     "elem_id", "lnode_gid", "lnode_slot", "lnode_smem", "shared_node",
                     "shared_ptr", "shared_slots"]
            _lib.check(L.tg_plan_export(h, *[host[k].ctypes.data for k in order]))
        finally:
            L.tg_plan_free(h)
        self.host = host
        self.sizes = dict(n_blocks=nb, n_elems=ne, color_ofs=ncol, local_nodes=nloc,
                          n_shared=nsh, n_partials=npart, max_local_nodes=maxl,
                          max_block_colors=maxc, stride=npad, n_affine_blocks=naff,
                          n_diag_blocks=ndiag, max_block_elems=maxe, n_lattice_blocks=nlat)
        self.device = torch.device(device)
        self.dev = {k: torch.from_numpy(v).to(self.device) for k, v in host.items()}
        s = _lib.BlockPlan()
        s.n_blocks, s.n_elems, s.nodes_per_elem_padded = nb, ne, npad
        s.max_local_nodes, s.n_shared, s.n_partials = maxl, nsh, npart
        s.threads = int(threads)
        s.n_affine_blocks = naff
        s.n_diag_blocks = ndiag
        s.max_block_elems = maxe
        s.n_lattice_blocks = nlat
        for k in order:
            setattr(s, k, self.dev[k].data_ptr())
        if np.array_equal(host["shared_slots"][:npart], np.arange(npart, dtype=np.int32)):
            s.shared_slots = None  # identity: the reduce reads partials in slot order
        # structured brick: the linear-elastic residual / HVP run as a grid stencil
        gn = (ctypes.c_int32 * 3)()
        gh = (ctypes.c_double * 3)()
        _lib.check(L.tg_grid_detect(elem_id, conn.ctypes.data, conn.shape[0], xyz.shape[0],
                                    xyz.ctypes.data, xyz.shape[1], gn, gh))
        self.grid_nodes = tuple(int(x) for x in gn)
        self.grid_h = tuple(float(x) for x in gh)
        s.grid_nodes[:] = self.grid_nodes
        s.grid_h[:] = self.grid_h
        self.struct = s
        self.box_geom32 = None
        if elem_id == _lib.TG_HEX8 and ndiag > 0 and self.device.type == "cuda":
            # edge terms of the box elements for the FP32 box kernel (no coordinate staging)
            x32 = torch.as_tensor(xyz, dtype=torch.float32, device=self.device)
            c32 = torch.as_tensor(conn, device=self.device)
            self.box_geom32 = torch.empty(3 * ne, dtype=torch.float32, device=self.device)
            _lib.call("tg_plan_box_geometry", ctypes.byref(s), x32.data_ptr(), c32.data_ptr(),
                      self.box_geom32.data_ptr(), torch.cuda.current_stream(self.device).cuda_stream)
            s.box_geom32 = self.box_geom32.data_ptr()

    @property
    def threads(self) -> int:
        return int(self.struct.threads)

    @threads.setter
    def threads(self, t: int) -> None:
        self.struct.threads = int(t)

    def ref(self):
        return ctypes.byref(self.struct)

    @property
    def grid(self) -> bool:
        """True when the stencil schedule of a structured brick is in use."""
        return self.struct.grid_nodes[0] > 0

    @grid.setter
    def grid(self, on: bool) -> None:
        """Switch the structured-brick stencil schedule off (element blocks for every
        mode) or back on, when the mesh is a brick."""
        self.struct.grid_nodes[:] = self.grid_nodes if on else (0, 0, 0)

    def stats(self) -> dict:
        s = dict(self.sizes)
        s.update(block_elems=self.block_elems, threads=self.threads, grid=self.grid,
                 shared_fraction=self.sizes["n_partials"] / max(self.sizes["local_nodes"], 1))
        return s
