"""Sparsity patterns, distance-2 colouring and colored sparse Jacobians.

Drop-in for ``tatva.sparse`` (tatva/sparse/__init__.py):

* ``pattern_from_mesh(mesh, n_dofs_per_node)`` -> ``scipy.sparse.csr_matrix`` (int8
  ones), identical to ``_create_sparse_structure`` (tatva/sparse/_extraction.py:37-102);
  built by the host C++ routine ``tg_pattern_build``.
* ``ColoredMatrix`` (tatva/sparse/base.py:37-105) with ``from_csr`` colouring by
  ``tg_distance2_colors`` (natural-order greedy, tatva/sparse/_coloring.py:136-153),
  ``to_csr`` / ``to_dense`` / ``to_bcsr`` / ``to_bcoo`` (torch sparse tensors stand
  in for jax.experimental.sparse).
* ``compute_rows_cols`` (base.py:108-136) -> ``tg_rows_cols``.
* ``jacfwd(fn, cm, color_batch_size=None)`` and ``linearized_jacfwd`` (base.py:139-227):
  - ``fn`` a fused energy residual (``energy.residual`` or the ``Energy`` itself):
    the compressed Jacobian comes from element tangents (``tg_compressed_hessian``);
  - any other differentiable torch function: one JVP per colour with the seeds of
    ``colored_jacobian_batch`` (base.py:230-270), JVPs through torch autograd's
    double-backward (``torch.autograd.functional.jvp``).
  Decompression ``data = Jc[rows, col_colors]`` (base.py:173) is ``tg_decompress``.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass, field, replace
from typing import Callable

import numpy as np
import scipy.sparse as sps
import torch

from . import _lib
from ._device import default_device, prec_of, ptr, require_cuda, stream
from .mesh import Mesh


def pattern_from_mesh(mesh: Mesh, n_dofs_per_node: int) -> sps.csr_matrix:
    el = mesh.elements_host()
    n_nodes = mesh.n_nodes
    L = _lib.lib()
    h = ctypes.c_void_p()
    _lib.check(L.tg_pattern_build(el.ctypes.data, el.shape[0], el.shape[1], n_nodes,
                                  int(n_dofs_per_node), ctypes.byref(h)))
    try:
        nnz = ctypes.c_int64()
        _lib.check(L.tg_pattern_nnz(h, ctypes.byref(nnz)))
        n = n_nodes * int(n_dofs_per_node)
        indptr = np.zeros(n + 1, np.int32)
        indices = np.zeros(max(nnz.value, 1), np.int32)
        _lib.check(L.tg_pattern_export(h, indptr.ctypes.data, indices.ctypes.data))
    finally:
        L.tg_pattern_free(h)
    indices = indices[: nnz.value]
    data = np.ones(nnz.value, dtype=np.int8)
    return sps.csr_matrix((data, indices, indptr), shape=(n, n))


def distance2_colors(indptr, indices, n_dofs: int) -> np.ndarray:
    ip = np.ascontiguousarray(np.asarray(indptr), dtype=np.int32)
    ix = np.ascontiguousarray(np.asarray(indices), dtype=np.int32)
    colors = np.zeros(max(int(n_dofs), 1), np.int32)
    nc = ctypes.c_int32()
    _lib.call("tg_distance2_colors", ip.ctypes.data, ix.ctypes.data, int(n_dofs),
              colors.ctypes.data, ctypes.byref(nc))
    return colors[: int(n_dofs)]


@dataclass(frozen=True)
class ColoredMatrix:
    data: torch.Tensor = field(repr=False)
    indptr: torch.Tensor = field(repr=False)
    indices: torch.Tensor = field(repr=False)
    shape: tuple
    colors: torch.Tensor = field(repr=False)

    @classmethod
    def from_csr(cls, csr_matrix: sps.csr_matrix, colors=None, device=None) -> "ColoredMatrix":
        dev = torch.device(device) if device is not None else default_device()
        indptr = np.ascontiguousarray(csr_matrix.indptr, dtype=np.int32)
        indices = np.ascontiguousarray(csr_matrix.indices, dtype=np.int32)
        if colors is None:
            colors = distance2_colors(indptr, indices, csr_matrix.shape[0])
        colors = np.ascontiguousarray(np.asarray(colors), dtype=np.int32)
        data = np.asarray(csr_matrix.data)
        return cls(
            data=torch.as_tensor(data, device=dev),
            indptr=torch.as_tensor(indptr, device=dev),
            indices=torch.as_tensor(indices, device=dev),
            shape=tuple(int(s) for s in csr_matrix.shape),
            colors=torch.as_tensor(colors, device=dev),
        )

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])

    @property
    def n_colors(self) -> int:
        return int(self.colors.max().item()) + 1 if self.colors.numel() else 0

    def to_csr(self) -> sps.csr_matrix:
        return sps.csr_matrix(
            (self.data.detach().cpu().numpy(), self.indices.cpu().numpy(),
             self.indptr.cpu().numpy()), shape=self.shape)

    def to_dense(self) -> torch.Tensor:
        return torch.as_tensor(self.to_csr().toarray(), device=self.data.device)

    def to_bcsr(self) -> torch.Tensor:
        return torch.sparse_csr_tensor(self.indptr.to(torch.int64), self.indices.to(torch.int64),
                                       self.data, size=self.shape)

    def to_bcoo(self) -> torch.Tensor:
        return self.to_bcsr().to_sparse_coo()


def compute_rows_cols(cm: ColoredMatrix):
    """rows[k], col_colors[k] of every stored entry (tatva/sparse/base.py:108-136)."""
    require_cuda(cm.indptr)
    rows = torch.empty(cm.nnz, dtype=torch.int32, device=cm.indptr.device)
    cols = torch.empty(cm.nnz, dtype=torch.int32, device=cm.indptr.device)
    _lib.call("tg_rows_cols", ptr(cm.indptr), ptr(cm.indices), ptr(cm.colors), cm.shape[0],
              cm.nnz, ptr(rows), ptr(cols), stream())
    return rows, cols


def decompress(Jc: torch.Tensor, rows: torch.Tensor, col_colors: torch.Tensor) -> torch.Tensor:
    require_cuda(Jc)
    Jc = Jc.contiguous()
    data = torch.empty(rows.shape[0], dtype=Jc.dtype, device=Jc.device)
    _lib.call("tg_decompress", prec_of(Jc.dtype), ptr(Jc), Jc.shape[1], ptr(rows),
              ptr(col_colors), rows.shape[0], ptr(data), stream())
    return data


def _fused_energy(fn):
    from .compound import CompoundEnergy
    from .materials import Energy

    if isinstance(fn, (Energy, CompoundEnergy)):
        return fn
    owner = getattr(fn, "__self__", None)
    if isinstance(owner, (Energy, CompoundEnergy)) and getattr(fn, "__name__", "") == "residual":
        return owner
    return None


def colored_jacobian(fn: Callable, u: torch.Tensor, colors: torch.Tensor, n_colors: int,
                     color_batch_size: int | None = None, *args, **kwargs) -> torch.Tensor:
    """Jc (N, C) with Jc[:, c] = J(u) seed_c (tatva/sparse/base.py:230-270)."""
    energy = _fused_energy(fn)
    if energy is not None and not args and not kwargs:
        return energy.compressed_hessian(u, colors, n_colors)
    n = u.numel()
    bs = int(color_batch_size or n_colors)
    Jc = torch.empty((n, n_colors), dtype=u.dtype, device=u.device)
    for c0 in range(0, n_colors, bs):
        nc = min(bs, n_colors - c0)
        seeds = torch.empty((nc, n), dtype=u.dtype, device=u.device)
        _lib.call("tg_color_seeds", prec_of(u.dtype), ptr(colors), n, c0, nc, ptr(seeds),
                  stream())
        for j in range(nc):
            seed = seeds[j].view(u.shape)
            _, col = torch.autograd.functional.jvp(lambda x: fn(x, *args, **kwargs), u, seed)
            col = col.detach().contiguous().view(-1)
            _lib.call("tg_set_column", prec_of(u.dtype), ptr(col), n, n_colors, c0 + j,
                      ptr(Jc), stream())
    return Jc


def jacfwd(fn: Callable, colored_matrix: ColoredMatrix, *, color_batch_size: int | None = None):
    """Sparse Jacobian of ``fn`` on the pattern of ``colored_matrix`` (base.py:139-176)."""
    nb_colors = colored_matrix.n_colors
    rows, col_colors = compute_rows_cols(colored_matrix)

    def _wrapped_jacfwd(u: torch.Tensor, *args, **kwargs) -> ColoredMatrix:
        Jc = colored_jacobian(fn, u, colored_matrix.colors, nb_colors, color_batch_size, *args,
                              **kwargs)
        return replace(colored_matrix, data=decompress(Jc, rows, col_colors))

    return _wrapped_jacfwd


def linearized_jacfwd(fn: Callable, colored_matrix: ColoredMatrix, *,
                      color_batch_size: int | None = None):
    """Like ``jacfwd`` but also returns fn(u) (base.py:179-227)."""
    jac = jacfwd(fn, colored_matrix, color_batch_size=color_batch_size)

    def _wrapped_linearized(u: torch.Tensor, *args, **kwargs):
        primal = fn(u, *args, **kwargs)
        if isinstance(primal, torch.Tensor):
            primal = primal.detach()
        return primal, jac(u, *args, **kwargs)

    return _wrapped_linearized


def pattern_from_compound(compound_cls, block_wise: bool = False):
    """Sparsity of a ``Compound`` state on its mesh (tatva/sparse/_extraction.py:117-245)."""
    from .compound import pattern_from_compound as _pfc

    return _pfc(compound_cls, block_wise=block_wise)


__all__ = ["ColoredMatrix", "compute_rows_cols", "decompress", "distance2_colors", "jacfwd",
           "linearized_jacfwd", "pattern_from_compound", "pattern_from_mesh"]
