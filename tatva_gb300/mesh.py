"""Mesh container and structured generators.

``Mesh(coords, elements)`` mirrors ``tatva/mesh.py:53-85`` (coords (n_nodes, dim),
elements (n_elements, nodes_per_element) int32).  Arrays live as torch tensors on
the GPU (coords FP64, connectivity int32); host copies are kept for the setup
routines (pattern, colouring, block plans), which run on the CPU.

Generators:
  * ``unit_square`` / ``rectangle`` (Tri3): the reference's ``_rectangle_triangular``
    (``tatva/mesh.py:180-205``): node id ``i*(n_y+1)+j``, triangles ``[n0,n1,n3]``,
    ``[n0,n3,n2]``.
  * ``brick`` (Hex8): structured box, node order of ``Hexahedron8`` (base.py:478-491),
    node id ``i + j*(nx+1) + k*(nx+1)*(ny+1)`` (no reference counterpart).
  * ``kuhn_box`` (Tet4): six tetrahedra per cell in the order of the reference's
    Kuhn-box fixture (``tests/test_sparse_tracer.py:29-70``), on ``[origin, origin+L]``.
"""

from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Any

import numpy as np
import torch

from ._device import default_device


def _as_tensor(a, dtype, device):
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(np.asarray(a)), dtype=dtype, device=device)


@dataclass(frozen=True, eq=False)
class Mesh:
    coords: torch.Tensor
    """Coordinates of the mesh nodes, shape (n_nodes, n_dim), FP64."""
    elements: torch.Tensor
    """Connectivity, shape (n_elements, nodes_per_element), int32."""
    _host: dict = field(default_factory=dict, repr=False, compare=False)

    def __init__(self, coords, elements, device=None):
        dev = torch.device(device) if device is not None else (
            coords.device if isinstance(coords, torch.Tensor) else default_device())
        if isinstance(elements, torch.Tensor) and elements.dtype.is_floating_point:
            raise TypeError("Mesh element connectivity must contain integer indices.")
        if not isinstance(elements, torch.Tensor):
            el = np.asarray(elements)
            if el.size and not np.issubdtype(el.dtype, np.integer):
                raise TypeError("Mesh element connectivity must contain integer indices.")
        object.__setattr__(self, "coords", _as_tensor(coords, torch.float64, dev))
        object.__setattr__(self, "elements", _as_tensor(elements, torch.int32, dev))
        object.__setattr__(self, "_host", {})

    # ---------------------------------------------------------------- host copies
    def coords_host(self) -> np.ndarray:
        if "coords" not in self._host:
            self._host["coords"] = np.ascontiguousarray(self.coords.detach().cpu().numpy())
        return self._host["coords"]

    def elements_host(self) -> np.ndarray:
        if "elements" not in self._host:
            self._host["elements"] = np.ascontiguousarray(
                self.elements.detach().cpu().numpy().astype(np.int32))
        return self._host["elements"]

    @property
    def n_nodes(self) -> int:
        return int(self.coords.shape[0])

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[0])

    @property
    def dim(self) -> int:
        return int(self.coords.shape[1])

    def _replace(self, **changes: Any) -> "Mesh":
        c = changes.get("coords", self.coords)
        e = changes.get("elements", self.elements)
        return Mesh(c, e)

    def set_coords(self, new_coords) -> "Mesh":
        return Mesh(new_coords, self.elements)

    def to(self, device) -> "Mesh":
        return Mesh(self.coords.to(device), self.elements.to(device))

    # ---------------------------------------------------------------- generators
    @classmethod
    def unit_square(cls, n_x: int, n_y: int, *, type="triangle", dim: int = 2, device=None):
        return cls.rectangle((0.0, 1.0), (0.0, 1.0), n_x, n_y, type=type, dim=dim, device=device)

    @classmethod
    def rectangle(cls, x, y, n_x: int, n_y: int, *, type="triangle", dim: int = 2, device=None):
        t = getattr(type, "value", type)
        if t != "triangle":
            raise NotImplementedError(f"Element type {type} not implemented.")
        xv_, yv_ = np.linspace(x[0], x[1], n_x + 1), np.linspace(y[0], y[1], n_y + 1)
        xv, yv = np.meshgrid(xv_, yv_, indexing="ij")
        coords = np.stack([xv.ravel(), yv.ravel()], axis=-1)
        i, j = np.meshgrid(np.arange(n_x), np.arange(n_y), indexing="ij")
        i, j = i.ravel(), j.ravel()
        n0 = i * (n_y + 1) + j
        n1 = (i + 1) * (n_y + 1) + j
        n2 = i * (n_y + 1) + j + 1
        n3 = (i + 1) * (n_y + 1) + j + 1
        el = np.stack([np.stack([n0, n1, n3], 1), np.stack([n0, n3, n2], 1)], 1).reshape(-1, 3)
        if dim == 3:
            coords = np.hstack([coords, np.zeros((coords.shape[0], 1))])
        return cls(coords, el.astype(np.int32), device=device)

    @classmethod
    def brick(cls, nx: int, ny: int, nz: int, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0),
              device=None):
        xr = np.linspace(origin[0], origin[0] + lengths[0], nx + 1)
        yr = np.linspace(origin[1], origin[1] + lengths[1], ny + 1)
        zr = np.linspace(origin[2], origin[2] + lengths[2], nz + 1)
        Z, Y, X = np.meshgrid(zr, yr, xr, indexing="ij")
        coords = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
        sx, sy, sz = 1, nx + 1, (nx + 1) * (ny + 1)
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        n0 = (i * sx + j * sy + k * sz).ravel().astype(np.int64)
        el = np.stack([n0, n0 + sx, n0 + sx + sy, n0 + sy,
                       n0 + sz, n0 + sx + sz, n0 + sx + sy + sz, n0 + sy + sz], axis=1)
        return cls(coords, el.astype(np.int32), device=device)

    @classmethod
    def kuhn_box(cls, nx: int, ny: int, nz: int, lengths=(1.0, 1.0, 1.0),
                 origin=(0.0, 0.0, 0.0), device=None):
        xr = np.linspace(origin[0], origin[0] + lengths[0], nx + 1)
        yr = np.linspace(origin[1], origin[1] + lengths[1], ny + 1)
        zr = np.linspace(origin[2], origin[2] + lengths[2], nz + 1)
        Z, Y, X = np.meshgrid(zr, yr, xr, indexing="ij")
        coords = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
        sx, sy, sz = 1, nx + 1, (nx + 1) * (ny + 1)
        k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
        n0 = (i * sx + j * sy + k * sz).ravel().astype(np.int64)
        n1, n2 = n0 + sx, n0 + sy
        n3, n4 = n2 + sx, n0 + sz
        n5, n6 = n4 + sx, n4 + sy
        n7 = n6 + sx
        tets = [(n0, n1, n3, n7), (n0, n1, n7, n5), (n0, n5, n7, n4),
                (n0, n3, n2, n7), (n0, n2, n6, n7), (n0, n6, n4, n7)]
        el = np.stack([np.stack(t, axis=-1) for t in tets], axis=1).reshape(-1, 4)
        return cls(coords, el.astype(np.int32), device=device)


def jitter_interior(coords: np.ndarray, h: float, amplitude: float, seed: int,
                    tol: float = 1e-12) -> np.ndarray:
    """Uniform(+-amplitude*h) displacement of interior nodes, numpy default_rng(seed)."""
    rng = np.random.default_rng(seed)
    lo, hi = coords.min(axis=0), coords.max(axis=0)
    interior = np.all((coords > lo + tol) & (coords < hi - tol), axis=1)
    out = coords.copy()
    d = rng.uniform(-amplitude * h, amplitude * h, size=coords.shape)
    out[interior] += d[interior]
    return out
