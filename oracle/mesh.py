"""Structured mesh generators (oracle, test infrastructure only).

* unit_square / rectangle (Tri3): restates ``tatva/mesh.py:146-205``
  (``elements.append([n0, n1, n3]); elements.append([n0, n3, n2])``, node id
  ``i*(n_y+1)+j``, int32 connectivity).
* kuhn_box (Tet4): restates the 6-tet split of
  ``tests/test_sparse_tracer.py:29-70`` (node id ``i + j*(nx+1) + k*(nx+1)*(ny+1)``).
* brick (Hex8): new (the reference has no 3D generator); each cell's nodes follow
  ``Hexahedron8._reference_nodes`` (``tatva/element/base.py:478-491``), node id
  ``i + j*(nx+1) + k*(nx+1)*(ny+1)``.
"""

from __future__ import annotations

import numpy as np


def rectangle_tri(x=(0.0, 1.0), y=(0.0, 1.0), n_x=1, n_y=1):
    xv_, yv_ = np.linspace(x[0], x[1], n_x + 1), np.linspace(y[0], y[1], n_y + 1)
    xv, yv = np.meshgrid(xv_, yv_, indexing="ij")
    coords = np.stack([xv.ravel(), yv.ravel()], axis=-1)
    i, j = np.meshgrid(np.arange(n_x), np.arange(n_y), indexing="ij")
    i, j = i.ravel(), j.ravel()
    n0 = i * (n_y + 1) + j
    n1 = (i + 1) * (n_y + 1) + j
    n2 = i * (n_y + 1) + j + 1
    n3 = (i + 1) * (n_y + 1) + j + 1
    t1 = np.stack([n0, n1, n3], axis=1)
    t2 = np.stack([n0, n3, n2], axis=1)
    elements = np.stack([t1, t2], axis=1).reshape(-1, 3)
    return coords, elements.astype(np.int32)


def unit_square(n_x, n_y):
    return rectangle_tri((0.0, 1.0), (0.0, 1.0), n_x, n_y)


def kuhn_box(lengths=(1.0, 1.0, 1.0), nb_elems=(1, 1, 1), origin=None):
    """6-tet Kuhn split, following tests/test_sparse_tracer.py:29-70 (centred x/y)."""
    lx, ly, lz = lengths
    nx, ny, nz = nb_elems
    if origin is None:
        xr = np.linspace(-lx / 2, lx / 2, nx + 1)
        yr = np.linspace(-ly / 2, ly / 2, ny + 1)
        zr = np.linspace(0, lz, nz + 1)
    else:
        xr = np.linspace(origin[0], origin[0] + lx, nx + 1)
        yr = np.linspace(origin[1], origin[1] + ly, ny + 1)
        zr = np.linspace(origin[2], origin[2] + lz, nz + 1)
    Z, Y, X = np.meshgrid(zr, yr, xr, indexing="ij")
    coords = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
    sx, sy, sz = 1, nx + 1, (nx + 1) * (ny + 1)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    n0 = (i * sx + j * sy + k * sz).ravel()
    n1 = n0 + sx
    n2 = n0 + sy
    n3 = n2 + sx
    n4 = n0 + sz
    n5 = n4 + sx
    n6 = n4 + sy
    n7 = n6 + sx
    tets = [
        (n0, n1, n3, n7),
        (n0, n1, n7, n5),
        (n0, n5, n7, n4),
        (n0, n3, n2, n7),
        (n0, n2, n6, n7),
        (n0, n6, n4, n7),
    ]
    el = np.stack([np.stack(t, axis=-1) for t in tets], axis=1).reshape(-1, 4)
    return coords, el.astype(np.int32)


def brick(nx, ny, nz, lengths=(1.0, 1.0, 1.0), origin=(0.0, 0.0, 0.0)):
    xr = np.linspace(origin[0], origin[0] + lengths[0], nx + 1)
    yr = np.linspace(origin[1], origin[1] + lengths[1], ny + 1)
    zr = np.linspace(origin[2], origin[2] + lengths[2], nz + 1)
    Z, Y, X = np.meshgrid(zr, yr, xr, indexing="ij")
    coords = np.stack([X, Y, Z], axis=-1).reshape(-1, 3)
    sx, sy, sz = 1, nx + 1, (nx + 1) * (ny + 1)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    n0 = (i * sx + j * sy + k * sz).ravel()
    el = np.stack(
        [n0, n0 + sx, n0 + sx + sy, n0 + sy,
         n0 + sz, n0 + sx + sz, n0 + sx + sy + sz, n0 + sy + sz],
        axis=1,
    )
    return coords, el.astype(np.int32)


def jitter_interior(coords, h, amplitude, seed, boundary_tol=1e-12):
    """Uniform(+-amplitude*h) jitter of interior nodes with numpy's default_rng(seed)."""
    rng = np.random.default_rng(seed)
    lo, hi = coords.min(axis=0), coords.max(axis=0)
    interior = np.all((coords > lo + boundary_tol) & (coords < hi - boundary_tol), axis=1)
    out = coords.copy()
    d = rng.uniform(-amplitude * h, amplitude * h, size=coords.shape)
    out[interior] += d[interior]
    return out
