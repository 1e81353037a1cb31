"""Operator maps (oracle, test infrastructure only).

Restates ``tatva/operator.py``:
  * get_integration_weights          operator.py:172-192  (einsum "eq,q->eq")
  * _vmap_over_elements_and_quads    operator.py:194-223  (gather nodal[elements])
  * map / map_over_elements          operator.py:225-305
  * integrate / integrate_per_element / _integrate_quad_array  operator.py:307-356
  * eval / grad                      operator.py:358-397
All arithmetic is vectorised numpy over elements in FP64 (complex inputs are
accepted so that complex-step derivatives can be taken through it).
"""

from __future__ import annotations

import numpy as np

from .elements import OracleElement


class OracleOperator:
    def __init__(self, coords, elements, element: OracleElement):
        self.coords = np.asarray(coords, dtype=np.float64)
        self.elements = np.asarray(elements)
        self.element = element
        self.N, self.dN, self.qw = element.tables()  # (Q,n), (Q,d,n), (Q,)

    @property
    def n_elements(self):
        return self.elements.shape[0]

    def geometry(self):
        """Per (e,q): dNdX (E,Q,d,n) and detJ (E,Q).  element/base.py:90-115.
        Computed once per operator (coordinates and connectivity are fixed)."""
        if getattr(self, "_geometry", None) is None:
            X = self.coords[self.elements]  # (E, n, d)
            J = np.einsum("qdn,enk->eqdk", self.dN, X)
            detJ = np.linalg.det(J)
            Jinv = np.linalg.inv(J)
            dNdX = np.einsum("eqkd,qdn->eqkn", Jinv, self.dN)
            self._geometry = (dNdX, detJ)
        return self._geometry

    def get_integration_weights(self):
        _, detJ = self.geometry()
        return np.einsum("eq,q->eq", detJ, self.qw)

    def eval(self, nodal_values):
        u = np.asarray(nodal_values)
        ue = u[self.elements]  # (E, n, ...)
        return np.einsum("qn,en...->eq...", self.N, ue)

    def grad(self, nodal_values):
        u = np.asarray(nodal_values)
        ue = u[self.elements]
        dNdX, _ = self.geometry()
        return np.einsum("eqdn,en...->eq...d", dNdX, ue)

    def _integrate_quad_array(self, quad_values):
        return np.einsum("eq...,eq->e...", quad_values, self.get_integration_weights())

    def integrate_per_element(self, arg):
        if np.isscalar(arg) or np.ndim(arg) == 0:
            vals = np.full((self.n_elements, self.qw.shape[0]), float(arg))
            return self._integrate_quad_array(vals)
        arg = np.asarray(arg)
        if arg.shape[0] == self.n_elements:
            return self._integrate_quad_array(arg)
        return self._integrate_quad_array(self.eval(arg))

    def integrate(self, arg):
        return np.sum(self.integrate_per_element(arg), axis=0)

    def map(self, func, *, element_quantity=()):
        """operator.py:225-266: func(xi, *element_values) at each (e,q)."""

        def _mapped(*values):
            xs = [
                np.asarray(v)[self.elements] if i not in element_quantity else np.asarray(v)
                for i, v in enumerate(values)
            ]
            out = []
            for e in range(self.n_elements):
                out.append(np.stack([np.asarray(func(xi, *[x[e] for x in xs]))
                                     for xi in self.element.quad_points]))
            return np.stack(out)

        return _mapped

    def map_over_elements(self, func, *, element_quantity=()):
        def _mapped(*values):
            xs = [
                np.asarray(v)[self.elements] if i not in element_quantity else np.asarray(v)
                for i, v in enumerate(values)
            ]
            return np.stack([np.asarray(func(*[x[e] for x in xs]))
                             for e in range(self.n_elements)])

        return _mapped

    # transposes used for reverse-mode AD of eval / grad
    def grad_transpose(self, flux, n_nodes=None):
        """nodal[a] += sum_q sum_d dNdX[e,q,d,a] * flux[e,q,...,d]."""
        n_nodes = n_nodes or self.coords.shape[0]
        dNdX, _ = self.geometry()
        contrib = np.einsum("eqdn,eq...d->en...", dNdX, flux)
        return _scatter_add(self.elements, contrib, n_nodes)

    def eval_transpose(self, quad_values, n_nodes=None):
        n_nodes = n_nodes or self.coords.shape[0]
        contrib = np.einsum("qn,eq...->en...", self.N, quad_values)
        return _scatter_add(self.elements, contrib, n_nodes)


def _scatter_add(elements, contrib, n_nodes):
    """out[elements[e, a]] += contrib[e, a, ...], the adds in (e, a) order (the order of
    np.add.at, done per trailing component with np.bincount, which is much faster)."""
    idx = np.asarray(elements).reshape(-1)
    flat = contrib.reshape(idx.size, -1)
    out = np.zeros((n_nodes, flat.shape[1]), dtype=contrib.dtype)
    for c in range(flat.shape[1]):
        col = flat[:, c]
        if np.iscomplexobj(col):
            out[:, c] = (np.bincount(idx, weights=col.real, minlength=n_nodes)
                         + 1j * np.bincount(idx, weights=col.imag, minlength=n_nodes))
        else:
            out[:, c] = np.bincount(idx, weights=col, minlength=n_nodes)
    return out.reshape((n_nodes,) + contrib.shape[2:])


def project(op: OracleOperator, field, fixed_nodes=None, fixed_values=None):
    """L2 projection of a quadrature field onto the nodal space, following
    make_project_function / _make_projection / _solve_projection
    (tatva/utils.py:118-262): M x = b with the consistent mass matrix
    M_ab = sum_e int N_a N_b and b_a = int N_a field, solved per field component
    (the coupled vector system is M (x) I); with a lifter (nodes ``fixed_nodes``)
    the reduced system M_ff x_f = b_f is solved and the fixed nodes take their
    prescribed values (Lifter.lift_from_zeros, tatva/lifter/base.py:223-229)."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla

    field = np.asarray(field, dtype=np.float64)
    E, Q = field.shape[:2]
    vshape = field.shape[2:]
    F = field.reshape(E, Q, -1)
    nn = op.coords.shape[0]
    _, detJ = op.geometry()
    w = detJ * op.qw[None, :]
    Me = np.einsum("eq,qa,qb->eab", w, op.N, op.N)
    rows = np.repeat(op.elements, op.elements.shape[1], axis=1).ravel()
    cols = np.tile(op.elements, (1, op.elements.shape[1])).ravel()
    M = sps.coo_matrix((Me.ravel(), (rows, cols)), shape=(nn, nn)).tocsr()
    b = op.eval_transpose(F * w[:, :, None])  # (nn, C)
    free = np.ones(nn, dtype=bool)
    if fixed_nodes is not None:
        free[np.asarray(fixed_nodes)] = False
    x = np.zeros_like(b)
    Mf = M[free][:, free].tocsc()
    for c in range(b.shape[1]):
        x[free, c] = spla.spsolve(Mf, b[free, c])
    if fixed_nodes is not None:
        x[~free] = 0.0 if fixed_values is None else np.asarray(fixed_values).reshape(-1, 1)
    return x.reshape((nn,) + vshape)
