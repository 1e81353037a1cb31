"""Synthetic benchmark problems built from the public API.

``clamped_brick``: Hex8 linear elasticity on the structured brick [0,1]^3 with n^3
cells, 2x2x2 Gauss, clamped face x = 0 and a uniform traction t e_x on x = 1.
The reference has no surface operator (a Quad4 face Jacobian is not square,
tatva/element/base.py:90-93), so the traction enters as consistent nodal forces:
each face cell of area h^2 gives h^2/4 to each of its four corner nodes.
"""

from __future__ import annotations

import numpy as np
import torch

from .element import Hexahedron8
from .materials import LinearElastic
from .mesh import Mesh
from .operator import Operator


def clamped_brick(n: int, device, traction: float = 1e-3, young: float = 1.0,
                  poisson: float = 0.3) -> dict:
    mesh = Mesh.brick(n, n, n, device=device)
    op = Operator(mesh, Hexahedron8())
    en = LinearElastic.from_young(op, young, poisson)
    c = mesh.coords_host()
    nn = c.shape[0]
    fixed = np.zeros(nn * 3, np.uint8)
    left = np.where(c[:, 0] == 0.0)[0]
    for k in range(3):
        fixed[left * 3 + k] = 1
    b = np.zeros(nn * 3)
    h = 1.0 / n
    right = np.where(c[:, 0] == 1.0)[0]
    jy = np.rint(c[right, 1] / h).astype(int)
    jz = np.rint(c[right, 2] / h).astype(int)
    mult = (np.where((jy == 0) | (jy == n), 1, 2) * np.where((jz == 0) | (jz == n), 1, 2))
    b[right * 3] = traction * (h * h / 4) * mult
    return dict(mesh=mesh, op=op, energy=en, fixed=torch.as_tensor(fixed, device=device),
                b=torch.as_tensor(b, device=device), n_nodes=nn, n_elems=mesh.n_elements)




def stretched_kuhn(n: int, device, jitter: float = 0.2, seed: int = 0, mu: float = 1.0,
                   lmbda: float = 10.0) -> dict:
    """Neo-Hookean Tet4 block: Kuhn 6-tet split of [0,1]^3 with n^3 cells (the node
    and tet order of the reference's Kuhn-box fixture, tests/test_sparse_tracer.py:29-70),
    interior nodes displaced by U(+-jitter h) from numpy default_rng(seed); the faces
    x = 0 and x = 1 are held, x = 1 moved along x by the prescribed stretch."""
    from .element import Tetrahedron4
    from .materials import NeoHookean
    from .mesh import jitter_interior

    m0 = Mesh.kuhn_box(n, n, n, device="cpu")
    c = jitter_interior(m0.coords_host(), 1.0 / n, jitter, seed=seed) if jitter else m0.coords_host()
    mesh = Mesh(c, m0.elements_host(), device=device)
    op = Operator(mesh, Tetrahedron4())
    en = NeoHookean(op, mu, lmbda)
    left = np.where(c[:, 0] == 0.0)[0]
    right = np.where(c[:, 0] == 1.0)[0]
    dofs = np.concatenate([left * 3, left * 3 + 1, left * 3 + 2,
                           right * 3, right * 3 + 1, right * 3 + 2])

    def values(stretch: float) -> np.ndarray:
        v = np.zeros(len(dofs))
        v[3 * len(left): 4 * len(left)] = stretch
        return v

    return dict(mesh=mesh, op=op, energy=en, coords=c, dofs=dofs, values=values,
                n_nodes=c.shape[0], n_elems=mesh.n_elements)


__all__ = ["clamped_brick", "stretched_kuhn"]
