"""Element types (host-side description; the arithmetic runs in the CUDA kernels).

Mirrors ``tatva/element/base.py``: ``Tri3`` (:245-265), ``Tetrahedron4`` (:448-472),
``Hexahedron8`` (:475-568) with the same node orders and default quadrature
(points and weights in the reference's order).  ``shape_function`` /
``shape_function_derivative`` are provided as numpy for inspection; the kernels
hard-code the same tables.  Custom quadrature rules are not supported by the
kernels and raise ``NotImplementedError``.
"""

from __future__ import annotations

import numpy as np

from . import _lib


class Element:
    """Base class; elements are immutable static descriptions."""

    tg_id: int
    n_nodes: int
    dim: int

    def __init__(self, quad_points=None, quad_weights=None):
        if quad_points is not None or quad_weights is not None:
            raise NotImplementedError(
                "custom quadrature rules are not available in the GB300 kernels; "
                "the default rule of the reference element is used"
            )
        self.quad_points, self.quad_weights = self._default_quadrature()

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self))

    def __repr__(self):
        return f"{type(self).__name__}()"

    @property
    def n_quad(self) -> int:
        return int(self.quad_weights.shape[0])

    def _reference_nodes(self) -> np.ndarray:
        raise NotImplementedError

    def _default_quadrature(self):
        raise NotImplementedError

    def shape_function(self, xi) -> np.ndarray:
        raise NotImplementedError

    def shape_function_derivative(self, xi=None) -> np.ndarray:
        raise NotImplementedError


class Tri3(Element):
    """3-node linear triangle (tatva/element/base.py:245-265)."""

    tg_id, n_nodes, dim = _lib.TG_TRI3, 3, 2

    def _reference_nodes(self):
        return np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])

    def _default_quadrature(self):
        return np.array([[1.0 / 3, 1.0 / 3]]), np.array([1.0 / 2])

    def shape_function(self, xi):
        x1, x2 = xi
        return np.array([1.0 - x1 - x2, x1, x2])

    def shape_function_derivative(self, xi=None):
        return np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]]).T


class Tetrahedron4(Element):
    """4-node linear tetrahedron (tatva/element/base.py:448-472)."""

    tg_id, n_nodes, dim = _lib.TG_TET4, 4, 3

    def _reference_nodes(self):
        return np.array([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])

    def _default_quadrature(self):
        return np.array([[1.0 / 4, 1.0 / 4, 1.0 / 4]]), np.array([1.0 / 6])

    def shape_function(self, xi):
        a, b, c = xi
        return np.array([1.0 - a - b - c, a, b, c])

    def shape_function_derivative(self, xi=None):
        return np.array([[-1.0, -1.0, -1.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]]).T


class Hexahedron8(Element):
    """8-node trilinear hexahedron, 2x2x2 Gauss (tatva/element/base.py:475-568)."""

    tg_id, n_nodes, dim = _lib.TG_HEX8, 8, 3
    _SIGNS = np.array(
        [[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
         [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]],
        dtype=np.float64,
    )

    def _reference_nodes(self):
        return self._SIGNS.copy()

    def _default_quadrature(self):
        return self._SIGNS * (1 / np.sqrt(3)), np.ones(8)

    def shape_function(self, xi):
        return (1 / 8) * np.prod(1.0 + self._SIGNS * np.asarray(xi)[None, :], axis=1)

    def shape_function_derivative(self, xi):
        s = self._SIGNS
        f = 1.0 + s * np.asarray(xi)[None, :]
        return np.stack(
            [s[:, 0] * f[:, 1] * f[:, 2], s[:, 1] * f[:, 0] * f[:, 2], s[:, 2] * f[:, 0] * f[:, 1]]
        ) / 8


# reference class names
Tet4 = Tetrahedron4
Hex8 = Hexahedron8

__all__ = ["Element", "Tri3", "Tetrahedron4", "Hexahedron8", "Tet4", "Hex8"]
