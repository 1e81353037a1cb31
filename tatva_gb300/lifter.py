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

``fixed_mask()`` exposes the constrained dofs as the uint8 mask consumed by the
fused kernels and the device solvers.  Periodic constraints are not part of this
build.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sps
import torch

from ._device import default_device


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


class Lifter:
    def __init__(self, size: int, *constraints: Fixed):
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

    def add(self, condition: Fixed) -> "Lifter":
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
        return sparsity

    def adapt_sparsity(self, sparsity: sps.csr_matrix) -> sps.csr_matrix:
        return self.reduce_sparsity(self.augment_sparsity(sparsity))
