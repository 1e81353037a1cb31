"""Dirichlet lift / reduce between full and free-dof vectors.

Mirrors ``tatva/lifter/base.py`` ``Lifter`` with ``Fixed`` constraints
(``tatva/lifter/constraints.py:290-318``):

* free dofs = setdiff(arange(size), unique(constrained))     base.py:268-279
* ``lift(u_reduced, u_full)``: u_full[free] = u_reduced, then each constraint's
  lift (Fixed: u[dofs] = values)                             base.py:201-221
* ``lift_from_zeros``                                         base.py:223-229
* ``reduce(u_full)`` = u_full[free]                           base.py:231-233
* ``reduce_adjoint(r_full)``: constraints' transposes in reverse order (Fixed:
  r[dofs] = 0), then [free]                                   base.py:235-251
* ``adapt_sparsity`` for Fixed = pattern[free][:, free]       base.py:281-331

* ``Periodic(dofs, master_dofs)`` (constraints.py:184-221): lift copies the master
  values into the slave dofs; the transpose adds the slave residuals to their masters
  (in a fixed order, so the result is deterministic) and zeroes the slaves; its
  sparsity is M^T S M with M = I + (slave, master) entries.
* ``lifted`` decorator (base.py:428-507).

``fixed_mask()`` exposes the constrained dofs as the uint8 mask consumed by the
fused kernels and the device solvers: exact for ``Fixed`` constraints (the reduced
operator is the masked one); with ``Periodic`` constraints the reduced residual and
operator come from ``reduce_adjoint(f(lift(.)))``.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sps
import torch

from ._device import default_device


class LifterError(Exception):
    """Raised for inconsistent lifter use (tatva/lifter/common.py)."""


class Fixed:
    def __init__(self, dofs, values=None):
        self.dofs = np.asarray(dofs.cpu() if isinstance(dofs, torch.Tensor) else dofs,
                               dtype=np.int64).reshape(-1)
        self.values = 0.0 if values is None else values

    def apply_lift(self, u: torch.Tensor) -> torch.Tensor:
        idx = torch.as_tensor(self.dofs, device=u.device)
        vals = self.values
        if isinstance(vals, (int, float)):
            return u.index_fill(0, idx, float(vals))
        vals = torch.as_tensor(np.asarray(vals.cpu() if isinstance(vals, torch.Tensor) else vals),
                               dtype=u.dtype, device=u.device)
        return u.index_put((idx,), vals.expand(idx.shape))

    def apply_transpose(self, r: torch.Tensor) -> torch.Tensor:
        idx = torch.as_tensor(self.dofs, device=r.device)
        return r.index_fill(0, idx, 0.0)

    def __hash__(self):
        return hash((self.dofs.tobytes(), str(self.values)))


class Periodic:
    def __init__(self, dofs, master_dofs):
        def _np(a):
            return np.asarray(a.cpu() if isinstance(a, torch.Tensor) else a, dtype=np.int64).reshape(-1)

        self.dofs = _np(dofs)
        self.master_dofs = _np(master_dofs)
        if self.dofs.shape != self.master_dofs.shape:
            raise LifterError("Periodic: dofs and master_dofs must have the same length")
        # occurrence rank of each slave among the slaves of its master: the transpose adds
        # the slaves in rounds of distinct masters, so no two adds hit one entry at once
        order = np.argsort(self.master_dofs, kind="stable")
        rank = np.zeros(self.dofs.size, dtype=np.int64)
        m_sorted = self.master_dofs[order]
        start = np.r_[0, np.flatnonzero(np.diff(m_sorted)) + 1] if m_sorted.size else np.array([], int)
        for a, b in zip(start, np.r_[start[1:], m_sorted.size] if m_sorted.size else []):
            rank[order[a:b]] = np.arange(b - a)
        self._rounds = [np.flatnonzero(rank == k) for k in range(int(rank.max(initial=-1)) + 1)]
        self._dev: dict = {}

    def _on(self, name, arr, device):
        key = (name, str(device))
        if key not in self._dev:
            self._dev[key] = torch.as_tensor(arr, device=device)
        return self._dev[key]

    def apply_lift(self, u: torch.Tensor) -> torch.Tensor:
        d = self._on("d", self.dofs, u.device)
        m = self._on("m", self.master_dofs, u.device)
        return u.index_put((d,), u[m])

    def apply_transpose(self, r: torch.Tensor) -> torch.Tensor:
        d = self._on("d", self.dofs, r.device)
        out = r
        for k, sel in enumerate(self._rounds):
            s = self._on(f"s{k}", self.dofs[sel], r.device)
            mk = self._on(f"m{k}", self.master_dofs[sel], r.device)
            out = out.index_add(0, mk, r[s])  # masters distinct within a round
        return out.index_fill(0, d, 0.0)

    def augment_sparsity(self, sparsity: sps.csr_matrix) -> sps.csr_matrix:
        n = sparsity.shape[0]
        rows = np.concatenate([np.arange(n), self.dofs])
        cols = np.concatenate([np.arange(n), self.master_dofs])
        M = sps.csr_matrix((np.ones(rows.shape[0], dtype=np.int8), (rows, cols)), shape=(n, n))
        A = M.T @ (sparsity.astype(np.int8) @ M)
        A.data = np.ones_like(A.data, dtype=np.int8)
        return A.tocsr()

    def __hash__(self):
        return hash((self.dofs.tobytes(), self.master_dofs.tobytes()))


class Lifter:
    def __init__(self, size: int, *constraints):
        self.size = int(size)
        self.constraints = tuple(constraints)
        if self.constraints:
            c = np.unique(np.concatenate([k.dofs for k in self.constraints]))
            free = np.setdiff1d(np.arange(self.size), c, assume_unique=True)
        else:
            c = np.array([], dtype=np.int64)
            free = np.arange(self.size)
        self._free_np, self._cons_np = free, c
        self.size_reduced = int(free.size)
        self._dev: dict = {}

    def _on(self, name, arr, device):
        key = (name, str(device))
        if key not in self._dev:
            self._dev[key] = torch.as_tensor(arr, device=device)
        return self._dev[key]

    @property
    def free_dofs(self) -> torch.Tensor:
        return self._on("free", self._free_np, default_device())

    @property
    def constrained_dofs(self) -> torch.Tensor:
        return self._on("cons", self._cons_np, default_device())

    def add(self, condition) -> "Lifter":
        return Lifter(self.size, *self.constraints, condition)

    def lift(self, u_reduced: torch.Tensor, u_full: torch.Tensor) -> torch.Tensor:
        free = self._on("free", self._free_np, u_full.device)
        u = u_full.clone()
        u[free] = u_reduced.to(u.dtype)
        for cond in self.constraints:
            u = cond.apply_lift(u)
        return u

    def lift_from_zeros(self, u_reduced: torch.Tensor) -> torch.Tensor:
        return self.lift(u_reduced, torch.zeros(self.size, dtype=u_reduced.dtype,
                                                device=u_reduced.device))

    def reduce(self, u_full: torch.Tensor) -> torch.Tensor:
        return u_full[self._on("free", self._free_np, u_full.device)]

    def reduce_adjoint(self, r_full: torch.Tensor) -> torch.Tensor:
        for cond in reversed(self.constraints):
            r_full = cond.apply_transpose(r_full)
        return r_full[self._on("free", self._free_np, r_full.device)]

    def fixed_mask(self, device=None) -> torch.Tensor:
        device = device or default_device()
        key = ("mask", str(device))
        if key not in self._dev:
            m = np.zeros(self.size, dtype=np.uint8)
            m[self._cons_np] = 1
            self._dev[key] = torch.as_tensor(m, device=device)
        return self._dev[key]

    def fixed_values(self, dtype=torch.float64, device=None) -> torch.Tensor:
        """Full vector holding the prescribed values on constrained dofs, 0 elsewhere."""
        device = device or default_device()
        return self.lift_from_zeros(torch.zeros(self.size_reduced, dtype=dtype, device=device))

    def reduce_sparsity(self, sparsity: sps.csr_matrix) -> sps.csr_matrix:
        return sparsity[self._free_np][:, self._free_np]

    def augment_sparsity(self, sparsity: sps.csr_matrix) -> sps.csr_matrix:
        if sparsity.shape[0] < self.size:
            extra = np.full(self.size - sparsity.shape[0], sparsity.indptr[-1],
                            dtype=sparsity.indptr.dtype)
            sparsity = sps.csr_matrix((sparsity.data, sparsity.indices,
                                       np.concatenate([sparsity.indptr, extra])),
                                      shape=(self.size, self.size))
        for cond in self.constraints:
            if hasattr(cond, "augment_sparsity"):
                sparsity = cond.augment_sparsity(sparsity)
        return sparsity

    def adapt_sparsity(self, sparsity: sps.csr_matrix) -> sps.csr_matrix:
        return self.reduce_sparsity(self.augment_sparsity(sparsity))


def lifted(fn=None, *, argnums=0, output=None):
    """Decorator: the wrapped function takes a ``Lifter`` first; the arguments in
    ``argnums`` are reduced vectors lifted with ``lift_from_zeros``; the output is
    reduced with ``reduce`` (``output="primal"``) or ``reduce_adjoint`` (``"dual"``)
    (tatva/lifter/base.py:428-507)."""
    argnums = (argnums,) if isinstance(argnums, int) else tuple(argnums)
    if fn is None:
        return lambda f: lifted(f, argnums=argnums, output=output)

    def lifted_fn(lifter, *args, **kwargs):
        largs = list(args)
        for i, a in enumerate(args):
            if i not in argnums:
                continue
            if not isinstance(a, torch.Tensor):
                raise LifterError(f"Argument {i} is not an Array and cannot be lifted by the lifter")
            if tuple(a.shape) != (lifter.size_reduced,):
                raise LifterError(f"Argument {i} has shape {tuple(a.shape)} but expected "
                                  f"{(lifter.size_reduced,)} for lifting")
            largs[i] = lifter.lift_from_zeros(a)
        out = fn(*largs, **kwargs)
        if output:
            if not isinstance(out, torch.Tensor):
                raise LifterError("Output is not an Array and cannot be reduced by the lifter")
            if output == "primal":
                return lifter.reduce(out)
            if output == "dual":
                return lifter.reduce_adjoint(out)
            raise LifterError(f"Invalid value for output: {output}")
        return out

    return lifted_fn


__all__ = ["Fixed", "Lifter", "LifterError", "Periodic", "lifted"]
