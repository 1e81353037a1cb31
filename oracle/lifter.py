"""Dirichlet lift / reduce (oracle, test infrastructure only).

Restates ``tatva/lifter/base.py``:
  * _compute_sizes (free = setdiff(arange, unique(constrained)))  base.py:268-279
  * lift            base.py:201-221   (u.at[free].set(u_r) then constraints)
  * lift_from_zeros base.py:223-229
  * reduce          base.py:231-233   (u[free])
  * reduce_adjoint  base.py:235-251   (constraints' transposes, then [free])
and ``Fixed`` (``tatva/lifter/constraints.py:290-318``): lift sets values,
transpose zeroes the residual on the fixed dofs; ``Periodic``
(``constraints.py:184-221``): lift copies the master values, transpose adds the
slave residuals to the masters and zeroes the slaves, sparsity M^T S M with
M = I + (slave, master) entries; ``adapt_sparsity`` = augment then [free][:, free]
(``base.py:281-331``).
"""

from __future__ import annotations

import numpy as np


class Fixed:
    def __init__(self, dofs, values=None):
        self.dofs = np.asarray(dofs, dtype=np.int64)
        self.values = 0.0 if values is None else values

    def apply_lift(self, u):
        u = u.copy()
        u[self.dofs] = self.values
        return u

    def apply_transpose(self, r):
        r = r.copy()
        r[self.dofs] = 0.0
        return r


class Periodic:
    def __init__(self, dofs, master_dofs):
        self.dofs = np.asarray(dofs, dtype=np.int64)
        self.master_dofs = np.asarray(master_dofs, dtype=np.int64)

    def apply_lift(self, u):
        u = u.copy()
        u[self.dofs] = u[self.master_dofs]
        return u

    def apply_transpose(self, r):
        r = r.copy()
        np.add.at(r, self.master_dofs, r[self.dofs])
        r[self.dofs] = 0.0
        return r

    def augment_sparsity(self, S):
        import scipy.sparse as sps

        n = S.shape[0]
        rows = np.concatenate([np.arange(n), self.dofs])
        cols = np.concatenate([np.arange(n), self.master_dofs])
        M = sps.csr_matrix((np.ones(rows.shape[0], dtype=np.int8), (rows, cols)), shape=(n, n))
        A = M.T @ (S.astype(np.int8) @ M)
        A.data = np.ones_like(A.data, dtype=np.int8)
        return A.tocsr()


class Lifter:
    def __init__(self, size, *constraints):
        self.size = size
        self.constraints = constraints
        if constraints:
            c = np.unique(np.concatenate([k.dofs for k in constraints]))
            self.free_dofs = np.setdiff1d(np.arange(size), c, assume_unique=True)
            self.constrained_dofs = c
        else:
            self.free_dofs = np.arange(size)
            self.constrained_dofs = np.array([], dtype=np.int64)
        self.size_reduced = self.free_dofs.size

    def lift(self, u_reduced, u_full):
        u = np.array(u_full, dtype=np.result_type(u_full, u_reduced), copy=True)
        u[self.free_dofs] = u_reduced
        for c in self.constraints:
            u = c.apply_lift(u)
        return u

    def lift_from_zeros(self, u_reduced):
        return self.lift(u_reduced, np.zeros(self.size, dtype=np.asarray(u_reduced).dtype))

    def reduce(self, u_full):
        return np.asarray(u_full)[self.free_dofs]

    def reduce_adjoint(self, r_full):
        r = np.asarray(r_full)
        for c in reversed(self.constraints):
            r = c.apply_transpose(r)
        return r[self.free_dofs]

    def augment_sparsity(self, S):
        for c in self.constraints:
            if hasattr(c, "augment_sparsity"):
                S = c.augment_sparsity(S)
        return S

    def adapt_sparsity(self, S):
        A = self.augment_sparsity(S)
        return A[self.free_dofs][:, self.free_dofs]
