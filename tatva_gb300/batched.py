"""Many independent meshes solved together in one persistent launch.

The reference solves one mesh at a time: a user assembles ``tatva.sparse.jacfwd``
(tatva/sparse/base.py:139-176) or uses the matrix-free HVP (README.md:93) and calls
``jax.scipy.sparse.linalg.cg`` per mesh.  Here a batch of meshes becomes one
disconnected mesh, its Hessian is assembled once by the colored compressed-Hessian
kernels, Dirichlet rows/columns are reduced on the device, and every mesh's diagonal
block is solved by ``tg_batch_solve``: one CTA per mesh at a time, FP32 CG inner
solves with FP64 iterative refinement on the true residual, until
``|b - A x| <= rtol |b|`` per mesh.  The solve can be captured once in a CUDA graph
(``BatchedSystems.capture``) and replayed.

``poisson_batch`` builds the batched Poisson problem
``psi = 1/2 kappa_e |grad u|^2 - f u`` with per-element conductivity (an
``element_quantity`` in the reference's ``Operator.map``, operator.py:255-258) and
zero Dirichlet values on each mesh's boundary.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, sparse
from ._device import ptr, require_cuda, stream, workspace
from .element import Tri3
from .materials import Poisson
from .mesh import Mesh
from .operator import Operator

MAX_ROWS = 49152


@dataclass
class BatchResult:
    x: torch.Tensor           # (n_rows,) FP64, all systems
    iterations: np.ndarray    # inner FP32 CG iterations per system
    refinements: np.ndarray   # FP64 refinement steps per system
    rel_res: np.ndarray       # final |b - A x| / |b| per system
    status: np.ndarray        # 0 converged, 5 not converged, 7 breakdown
    seconds: float = 0.0

    @property
    def converged(self) -> bool:
        return bool(np.all(self.status == _lib.TG_OK))


def boundary_nodes_tri3(elements: np.ndarray, n_nodes: int) -> np.ndarray:
    """Nodes on edges that belong to exactly one triangle (topological boundary)."""
    el = np.asarray(elements, dtype=np.int64)
    e = np.concatenate([el[:, [0, 1]], el[:, [1, 2]], el[:, [2, 0]]])
    e.sort(axis=1)
    key = e[:, 0] * n_nodes + e[:, 1]
    uniq, cnt = np.unique(key, return_counts=True)
    b = uniq[cnt == 1]
    mask = np.zeros(n_nodes, dtype=bool)
    mask[b // n_nodes] = True
    mask[b % n_nodes] = True
    return mask


class BatchedSystems:
    """Block-diagonal SPD matrix (one block per system) in the per-system ELL layout
    of ``tg_batch_solve``, built from a CSR matrix (FP64 data on the device)."""

    def __init__(self, indptr: torch.Tensor, indices: torch.Tensor, data: torch.Tensor,
                 row_ofs: np.ndarray):
        require_cuda(data)
        dev = data.device
        self.device = dev
        row_ofs = np.asarray(row_ofs, dtype=np.int64)
        self.n_systems = len(row_ofs) - 1
        self.n_rows = int(row_ofs[-1])
        sizes = np.diff(row_ofs)
        if sizes.max(initial=0) > MAX_ROWS:
            raise NotImplementedError(f"a system has {sizes.max()} rows; at most {MAX_ROWS}")
        ip = indptr.cpu().numpy().astype(np.int64)
        lens = np.diff(ip)
        width = np.zeros(self.n_systems, np.int32)
        nonempty = sizes > 0
        if nonempty.any():
            width[nonempty] = np.maximum.reduceat(lens, row_ofs[:-1][nonempty])
        ell_ofs = np.zeros(self.n_systems, np.int64)
        ell_ofs[1:] = np.cumsum(sizes * width)[:-1]
        n_ell = int((sizes * width).sum())
        order = np.argsort(-(sizes * width), kind="stable").astype(np.int32)
        self.sizes, self.width, self.order = sizes, width, order
        self.row_ofs = torch.from_numpy(row_ofs).to(dev)
        self.ell_ofs = torch.from_numpy(ell_ofs).to(dev)
        self.ell_width = torch.from_numpy(width).to(dev)
        self.order_d = torch.from_numpy(order).to(dev)
        self.ell_col = torch.empty(max(n_ell, 1), dtype=torch.int16, device=dev)
        self.ell_val32 = torch.empty(max(n_ell, 1), dtype=torch.float32, device=dev)
        self.ell_val64 = torch.empty(max(n_ell, 1), dtype=torch.float64, device=dev)
        d = _lib.BatchDesc()
        d.n_systems = self.n_systems
        d.max_rows = int(sizes.max(initial=0))
        d.row_ofs, d.ell_ofs = self.row_ofs.data_ptr(), self.ell_ofs.data_ptr()
        d.ell_width, d.order = self.ell_width.data_ptr(), self.order_d.data_ptr()
        d.ell_col, d.ell_val32 = self.ell_col.data_ptr(), self.ell_val32.data_ptr()
        d.ell_val64 = self.ell_val64.data_ptr()
        self.desc = d
        bad = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("tg_batch_ell_from_csr", ctypes.byref(d), self.n_rows, ptr(indptr.contiguous()),
                  ptr(indices.contiguous()), ptr(data.to(torch.float64).contiguous()), ptr(bad),
                  stream())
        flag = int(bad.item())
        if flag == 1:
            raise ValueError("a CSR row is longer than its system's ELL width")
        if flag == 2:
            raise ValueError("the matrix is not block diagonal: a row couples two systems")
        self._ws_bytes = _lib.lib().tg_batch_workspace_bytes(self.n_rows)
        self._ws = workspace(self._ws_bytes, dev)
        self.iters = torch.zeros(self.n_systems, dtype=torch.int32, device=dev)
        self.outer = torch.zeros(self.n_systems, dtype=torch.int32, device=dev)
        self.rel = torch.zeros(self.n_systems, dtype=torch.float64, device=dev)
        self.status = torch.zeros(self.n_systems, dtype=torch.int32, device=dev)
        self.threads, self.ctas_per_sm = 256, 0

    @property
    def ell_bytes(self) -> int:
        """Bytes of matrix data read by one FP32 CG iteration over all systems."""
        return int(self.ell_val32.numel()) * 6

    def launch(self, b: torch.Tensor, x: torch.Tensor, *, rtol=1e-10, inner_rtol=1e-3,
               max_outer=60, max_inner=20000, threads=None, ctas_per_sm=None) -> None:
        """Enqueue the batched solve on the current stream (graph-capturable)."""
        _lib.call("tg_batch_solve", ctypes.byref(self.desc), self.n_rows, ptr(b), ptr(x),
                  float(rtol), float(inner_rtol), int(max_outer), int(max_inner),
                  int(threads or self.threads),
                  int(self.ctas_per_sm if ctas_per_sm is None else ctas_per_sm),
                  ptr(self._ws), self._ws_bytes, ptr(self.iters), ptr(self.outer), ptr(self.rel),
                  ptr(self.status), stream())

    def result(self, x: torch.Tensor, seconds: float = 0.0) -> BatchResult:
        return BatchResult(x, self.iters.cpu().numpy(), self.outer.cpu().numpy(),
                           self.rel.cpu().numpy(), self.status.cpu().numpy(), seconds)

    def solve(self, b: torch.Tensor, **kw) -> BatchResult:
        bb = b.reshape(-1).to(torch.float64).contiguous()
        if bb.numel() != self.n_rows:
            raise ValueError(f"b has {bb.numel()} entries, the batch {self.n_rows} rows")
        x = torch.empty_like(bb)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        self.launch(bb, x, **kw)
        ev1.record()
        ev1.synchronize()
        return self.result(x, ev0.elapsed_time(ev1) * 1e-3)

    def capture(self, b: torch.Tensor, x: torch.Tensor, **kw) -> torch.cuda.CUDAGraph:
        """One CUDA graph holding the whole batched solve (counter reset + the
        persistent kernel); replay it to solve again with the contents of b."""
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.launch(b, x, **kw)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(b, x, **kw)
        return g

    def split(self, x: torch.Tensor) -> list[torch.Tensor]:
        ro = self.row_ofs.cpu().numpy()
        return [x[ro[s]:ro[s + 1]] for s in range(self.n_systems)]


def concat_meshes(meshes):
    """One disconnected mesh from [(coords, elements), ...]; returns coords, elements,
    node offsets, element offsets."""
    nodes = [np.asarray(c, dtype=np.float64) for c, _ in meshes]
    elems = [np.asarray(e, dtype=np.int64) for _, e in meshes]
    nofs = np.zeros(len(meshes) + 1, np.int64)
    nofs[1:] = np.cumsum([c.shape[0] for c in nodes])
    eofs = np.zeros(len(meshes) + 1, np.int64)
    eofs[1:] = np.cumsum([e.shape[0] for e in elems])
    coords = np.concatenate(nodes)
    elements = np.concatenate([e + o for e, o in zip(elems, nofs[:-1])]).astype(np.int32)
    return coords, elements, nofs, eofs


def random_unit_squares(count: int, n_min: int = 8, n_max: int = 96, seed: int = 0,
                        sigma: float = 1.0):
    """``count`` Tri3 unit-square meshes with side n = round(exp(U(ln n_min, ln n_max)))
    and per-element conductivity lognormal(0, sigma), from numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    sides = np.rint(np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=count))).astype(int)
    cache, meshes, kappas = {}, [], []
    for n in sides:
        if n not in cache:
            m = Mesh.unit_square(int(n), int(n), device="cpu")
            cache[n] = (m.coords_host(), m.elements_host())
        c, e = cache[n]
        meshes.append((c, e))
        kappas.append(rng.lognormal(0.0, sigma, size=e.shape[0]))
    return meshes, kappas, sides


def poisson_batch(meshes, kappas=None, f: float = 1.0, fixed=None, device=None):
    """Assemble the batched Tri3 Poisson problem.

    meshes: [(coords (n,2), elements (m,3)), ...]; kappas: per-element conductivities
    per mesh (None: 1); fixed: per-mesh boolean node masks (None: topological boundary).
    Returns (BatchedSystems, b (FP64, zero on fixed dofs), info dict)."""
    coords, elements, nofs, eofs = concat_meshes(meshes)
    dev = torch.device(device) if device is not None else torch.device("cuda")
    mesh = Mesh(coords, elements, device=dev)
    op = Operator(mesh, Tri3())
    if kappas is None:
        kap = np.ones(elements.shape[0])
    else:
        kap = np.concatenate([np.asarray(k, dtype=np.float64).reshape(-1) for k in kappas])
    en = Poisson(op, kap, f)
    if fixed is None:
        fixed = [boundary_nodes_tri3(e, c.shape[0]) for c, e in meshes]
    mask_np = np.concatenate([np.asarray(m, dtype=bool) for m in fixed]).astype(np.uint8)
    mask = torch.from_numpy(mask_np).to(dev)
    csr = sparse.pattern_from_mesh(mesh, 1)
    cm = sparse.ColoredMatrix.from_csr(csr, device=dev)
    u0 = torch.zeros(mesh.n_nodes, dtype=torch.float64, device=dev)
    H = sparse.jacfwd(en.residual, cm)(u0)
    data = H.data.contiguous()
    _lib.call("tg_csr_apply_dirichlet", _lib.TG_F64, mesh.n_nodes, ptr(H.indptr), ptr(H.indices),
              ptr(mask), ptr(data), stream())
    # b = f int N_a: element integrals summed per node in increasing element order
    # (node incidence), so a mesh gets the same bits alone and inside any batch
    w = op._weights_raw(torch.float64)
    b = op._eval_t_raw((float(f) * w).contiguous(), ())
    b = torch.where(mask.bool(), torch.zeros_like(b), b).contiguous()
    systems = BatchedSystems(H.indptr, H.indices, data, nofs)
    info = dict(n_meshes=len(meshes), n_rows=int(nofs[-1]), n_elements=int(eofs[-1]),
                nnz=int(H.indices.numel()), n_colors=cm.n_colors)
    return systems, b, info


__all__ = ["BatchResult", "BatchedSystems", "boundary_nodes_tri3", "concat_meshes",
           "poisson_batch", "random_unit_squares"]
