"""Element definitions (oracle, test infrastructure only).

Restates ``tatva/element/base.py``:
  * Element.get_jacobian / gradient / interpolate   base.py:90-115
  * Tri3                                            base.py:245-265
  * Tetrahedron4                                    base.py:448-472
  * Hexahedron8                                     base.py:475-568
Quadrature points and node orders are kept in the reference's order.
"""

from __future__ import annotations

import numpy as np


class OracleElement:
    name: str
    n_nodes: int
    dim: int

    def reference_nodes(self) -> np.ndarray:
        raise NotImplementedError

    def quadrature(self) -> tuple[np.ndarray, np.ndarray]:
        raise NotImplementedError

    def shape_function(self, xi: np.ndarray) -> np.ndarray:
        raise NotImplementedError

    def shape_function_derivative(self, xi: np.ndarray) -> np.ndarray:
        """(dim, n_nodes) derivative w.r.t. local coordinates."""
        raise NotImplementedError

    @property
    def quad_points(self) -> np.ndarray:
        return self.quadrature()[0]

    @property
    def quad_weights(self) -> np.ndarray:
        return self.quadrature()[1]

    # base.py:90-93
    def get_jacobian(self, xi, nodal_coords):
        dNdr = self.shape_function_derivative(xi)
        J = dNdr @ nodal_coords
        return J, np.linalg.det(J)

    # base.py:95-97
    def interpolate(self, xi, nodal_values, nodal_coords=None):
        N = self.shape_function(xi)
        return np.einsum("n,n...->...", N, nodal_values)

    # base.py:99-115 ("dn,n...->...d": value dims first, spatial dim last)
    def gradient(self, xi, nodal_values, nodal_coords):
        dNdr = self.shape_function_derivative(xi)
        J = dNdr @ nodal_coords
        dNdX = np.linalg.inv(J) @ dNdr
        return np.einsum("dn,n...->...d", dNdX, nodal_values)

    # tables evaluated at the default quadrature points: N (Q, n), dN (Q, d, n)
    def tables(self):
        qp, qw = self.quadrature()
        N = np.stack([self.shape_function(x) for x in qp])
        dN = np.stack([self.shape_function_derivative(x) for x in qp])
        return N, dN, qw


class Tri3(OracleElement):
    """base.py:245-265."""

    name, n_nodes, dim = "tri3", 3, 2

    def reference_nodes(self):
        return np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])

    def quadrature(self):
        return np.array([[1.0 / 3, 1.0 / 3]]), np.array([1.0 / 2])

    def shape_function(self, xi):
        x1, x2 = xi
        return np.array([1.0 - x1 - x2, x1, x2])

    def shape_function_derivative(self, xi=None):
        return np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]]).T


class Tetrahedron4(OracleElement):
    """base.py:448-472."""

    name, n_nodes, dim = "tet4", 4, 3

    def reference_nodes(self):
        return np.array(
            [[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]
        )

    def quadrature(self):
        return np.array([[1.0 / 4, 1.0 / 4, 1.0 / 4]]), np.array([1.0 / 6])

    def shape_function(self, xi):
        a, b, c = xi
        return np.array([1.0 - a - b - c, a, b, c])

    def shape_function_derivative(self, xi=None):
        return np.array(
            [[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]
        ).T


class Hexahedron8(OracleElement):
    """base.py:475-568.  Node order base.py:478-491, 2x2x2 Gauss order base.py:497-508."""

    name, n_nodes, dim = "hex8", 8, 3

    SIGNS = np.array(
        [
            [-1, -1, -1],
            [1, -1, -1],
            [1, 1, -1],
            [-1, 1, -1],
            [-1, -1, 1],
            [1, -1, 1],
            [1, 1, 1],
            [-1, 1, 1],
        ],
        dtype=np.float64,
    )

    def reference_nodes(self):
        return self.SIGNS.copy()

    def quadrature(self):
        a = 1 / np.sqrt(3)
        return self.SIGNS * a, np.ones(8)

    def shape_function(self, xi):
        s = self.SIGNS
        return (1 / 8) * np.prod(1.0 + s * np.asarray(xi)[None, :], axis=1)

    def shape_function_derivative(self, xi):
        s = self.SIGNS
        f = 1.0 + s * np.asarray(xi)[None, :]  # (8, 3)
        d = np.empty((3, 8))
        d[0] = s[:, 0] * f[:, 1] * f[:, 2]
        d[1] = s[:, 1] * f[:, 0] * f[:, 2]
        d[2] = s[:, 2] * f[:, 0] * f[:, 1]
        return d / 8


ELEMENTS = {"tri3": Tri3, "tet4": Tetrahedron4, "hex8": Hexahedron8}


def element_for(n_nodes: int, dim: int) -> OracleElement:
    if (n_nodes, dim) == (3, 2):
        return Tri3()
    if (n_nodes, dim) == (4, 3):
        return Tetrahedron4()
    if (n_nodes, dim) == (8, 3):
        return Hexahedron8()
    raise ValueError(f"no oracle element with {n_nodes} nodes in {dim}D")
