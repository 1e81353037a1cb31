"""Energies of the hot path with fused residual / HVP / tangent kernels.

In the reference a user writes ``E(u) = op.integrate(psi(op.grad(u)))`` and gets the
residual from ``jax.grad(E)``, the matrix-free Hessian-vector product from
``jax.jvp(jax.grad(E), (u,), (v,))`` (README.md:93) and the sparse Hessian from
``tatva.sparse.jacfwd(jax.grad(E), cm)`` (tatva/sparse/base.py:139-176).  For the
three energies on the hot path these derivatives are available here as fused
gather -> QP law -> scatter kernels:

* ``Poisson(op, kappa, f)``      psi = 1/2 kappa |grad u|^2 - f u  (kappa scalar or
                                 per element, as an ``element_quantity``)
* ``LinearElastic(op, mu, lmbda)`` psi = 1/2 sigma:eps  (tests/test_sparse.py:12-30)
* ``NeoHookean(op, mu, lmbda)``  psi = mu/2 (I1-3-2 ln J) + lambda/2 (ln J)^2
                                 (tests/test_sparse_tracer.py:101-113)

The kernel precision follows the dtype of ``u`` (float32 or float64).  Vectors
are flat ``(n_nodes * n_values,)`` with dof = node * n_values + component
(tests/test_sparse.py:52) or shaped ``(n_nodes, n_values)``; outputs keep the
input shape.  A Dirichlet mask (``fixed``: uint8 per dof, or a ``Lifter``) gives
the reduced operator of ``Lifter.reduce_adjoint`` / ``Fixed``
(tatva/lifter/base.py:235-251, constraints.py:312-318): residual rows of fixed
dofs are 0, the HVP acts as the identity there.
"""

from __future__ import annotations

import ctypes
from numbers import Number

import numpy as np
import torch

from . import _lib
from ._device import prec_of, ptr, require_cuda, stream, workspace
from .operator import Operator, _sum_rows_raw


def lame_from_young(E: float, nu: float):
    """mu = E/2(1+nu), lambda = E nu/((1+nu)(1-2nu))  (tests/test_sparse_benchmark.py:35-43)."""
    return E / 2 / (1 + nu), E * nu / (1 - 2 * nu) / (1 + nu)


class Energy:
    kind: int = -1
    name = "energy"

    def __init__(self, op: Operator, p0, p1: float = 0.0):
        self.op = op
        self._elem_param = None
        if isinstance(p0, Number):
            self.p0 = float(p0)
        else:
            t = torch.as_tensor(p0, dtype=torch.float64, device=op.device).contiguous()
            if t.shape != (op.n_elements,):
                raise ValueError(f"per-element parameter must have shape ({op.n_elements},)")
            self._elem_param = {torch.float64: t}
            self.p0 = float("nan")
        self.p1 = float(p1)
        self._ws: dict = {}
        self._plan_override = None
        if self.kind == _lib.TG_NEO_HOOKEAN and op.dim != 3:
            raise NotImplementedError("the Neo-Hookean energy is implemented for 3D elements")

    # ------------------------------------------------------------------ helpers
    @property
    def n_values(self) -> int:
        if self.kind == _lib.TG_POISSON:
            return 1
        if self.kind == _lib.TG_LINEAR_ELASTIC:
            return self.op.dim
        return 3

    @property
    def n_dofs(self) -> int:
        return self.op.n_nodes * self.n_values

    def plan(self):
        return self._plan_override if self._plan_override is not None else self.op.plan()

    def use_plan(self, plan) -> None:
        self._plan_override = plan

    def material(self, dtype) -> _lib.Material:
        m = _lib.Material()
        m.kind = self.kind
        m.p0 = self.p0 if self._elem_param is None else 0.0
        m.p1 = self.p1
        if self._elem_param is not None:
            if dtype not in self._elem_param:
                self._elem_param[dtype] = self._elem_param[torch.float64].to(dtype)
            m.elem_param = self._elem_param[dtype].data_ptr()
        return m

    def _flat(self, u: torch.Tensor) -> torch.Tensor:
        if u.numel() != self.n_dofs:
            raise ValueError(f"expected {self.n_dofs} dofs, got tensor of shape {tuple(u.shape)}")
        require_cuda(u)
        return u.contiguous().view(-1)

    def _workspace(self, dtype, plan):
        key = (dtype, id(plan))
        nb = _lib.lib().tg_apply_workspace_bytes(self.op.element.tg_id, prec_of(dtype), self.kind,
                                                 plan.ref())
        if key not in self._ws or self._ws[key][1] < nb:
            self._ws[key] = (workspace(nb, self.op.device), nb)
        return self._ws[key]

    @staticmethod
    def _mask(fixed, like: torch.Tensor):
        if fixed is None:
            return None
        if hasattr(fixed, "fixed_mask"):
            fixed = fixed.fixed_mask(like.device)
        if fixed.dtype != torch.uint8 or fixed.numel() != like.numel():
            raise ValueError("fixed must be a uint8 mask with one entry per dof")
        return fixed.contiguous()

    def apply(self, mode: int, u, v=None, fixed=None, out=None) -> torch.Tensor:
        ref = u if u is not None else v
        dtype = ref.dtype
        prec = prec_of(dtype)
        uf = self._flat(u) if u is not None else None
        vf = self._flat(v) if v is not None else None
        if uf is not None and vf is not None and uf.dtype != vf.dtype:
            raise TypeError("u and v must have the same dtype")
        plan = self.plan()
        y = out if out is not None else torch.empty(self.n_dofs, dtype=dtype, device=ref.device)
        ws, nb = self._workspace(dtype, plan)
        mask = self._mask(fixed, y)
        m = self.material(dtype)
        _lib.call("tg_apply", self.op.element.tg_id, prec, mode, ctypes.byref(m), plan.ref(),
                  ptr(self.op.coords_as(dtype)), self.op.n_nodes, ptr(uf), ptr(vf), ptr(mask),
                  ptr(y), ptr(ws), nb, stream())
        orphans = self.op.unused_nodes()
        if orphans.numel():
            # rows of nodes without elements: zero, with the Dirichlet rule on fixed dofs
            nv = self.n_values
            dofs = (orphans[:, None] * nv + torch.arange(nv, device=y.device)).reshape(-1)
            val = torch.zeros(dofs.numel(), dtype=y.dtype, device=y.device)
            if mask is not None:
                fx = mask[dofs].bool()
                if mode == _lib.TG_MODE_HVP:
                    val = torch.where(fx, vf[dofs], val)
                elif mode == _lib.TG_MODE_DIAG:
                    val = torch.where(fx, torch.ones_like(val), val)
            y[dofs] = val
        return y.view(ref.shape) if out is None else y

    # ------------------------------------------------------------------ public API
    def residual(self, u: torch.Tensor, fixed=None) -> torch.Tensor:
        """dE/du at u (jax.grad(E)(u))."""
        return self.apply(_lib.TG_MODE_RESIDUAL, u, None, fixed)

    def hvp(self, u: torch.Tensor | None, v: torch.Tensor, fixed=None) -> torch.Tensor:
        """d2E/du2(u) . v (jax.jvp(jax.grad(E), (u,), (v,))[1]); u may be None for
        linear laws."""
        if u is None and self.kind == _lib.TG_NEO_HOOKEAN:
            raise ValueError("the Neo-Hookean HVP needs the linearisation point u")
        return self.apply(_lib.TG_MODE_HVP, u, v, fixed)

    def diagonal(self, u: torch.Tensor, fixed=None) -> torch.Tensor:
        """diag of d2E/du2(u) (Jacobi preconditioner)."""
        return self.apply(_lib.TG_MODE_DIAG, u, None, fixed)

    def energy_per_element(self, u: torch.Tensor) -> torch.Tensor:
        uf = self._flat(u)
        out = torch.empty(self.op.n_elements, dtype=uf.dtype, device=uf.device)
        m = self.material(uf.dtype)
        _lib.call("tg_energy_per_element", self.op.element.tg_id, prec_of(uf.dtype),
                  ctypes.byref(m), ptr(self.op.coords_as(uf.dtype)), self.op.n_nodes,
                  ptr(self.op.mesh.elements), self.op.n_elements, ptr(uf), ptr(out), stream())
        return out

    def value(self, u: torch.Tensor) -> torch.Tensor:
        """E(u) = op.integrate(psi(op.grad(u))) with a deterministic element sum."""
        return _sum_rows_raw(self.energy_per_element(u))

    __call__ = value

    def element_colors(self):
        """Greedy element colouring (host), cached on the operator."""
        key = "ecol"
        if key not in self.op._cache:
            el = self.op.mesh.elements_host()
            E, npe = el.shape
            colors = np.zeros(E, np.int32)
            order = np.zeros(E, np.int32)
            cptr = np.zeros(129, np.int32)
            nc = ctypes.c_int32()
            _lib.call("tg_element_colors", el.ctypes.data, E, npe, self.op.n_nodes,
                      colors.ctypes.data, order.ctypes.data, cptr.ctypes.data, ctypes.byref(nc))
            self.op._cache[key] = (torch.from_numpy(order).to(self.op.device),
                                   cptr[: nc.value + 1].copy(), nc.value)
        return self.op._cache[key]

    def compressed_hessian(self, u: torch.Tensor, colors: torch.Tensor, n_colors: int,
                           dtype=None) -> torch.Tensor:
        """Jc (n_dofs, n_colors): Jc[i, c] = sum_{j: colors[j] = c} H[i, j]
        (tatva/sparse/base.py:230-270), from element tangents."""
        dtype = dtype or u.dtype
        uf = self._flat(u).to(dtype)
        ip, ii = self.op.incidence()
        Jc = torch.empty((self.n_dofs, n_colors), dtype=dtype, device=uf.device)
        m = self.material(dtype)
        _lib.call("tg_compressed_hessian", self.op.element.tg_id, prec_of(dtype), ctypes.byref(m),
                  ptr(self.op.coords_as(dtype)), self.op.n_nodes, ptr(self.op.mesh.elements),
                  self.op.n_elements, ptr(uf), ptr(ip), ptr(ii), ptr(colors), int(n_colors),
                  ptr(Jc), stream())
        return Jc

    def operator_desc(self, u, fixed=None, dtype=torch.float64):
        """tg_operator_desc for the device solvers (keeps referenced tensors alive)."""
        d = _lib.OperatorDesc()
        d.elem = self.op.element.tg_id
        d.prec = prec_of(dtype)
        d.mat = self.material(dtype)
        plan = self.plan()
        d.plan = ctypes.addressof(plan.struct)
        coords = self.op.coords_as(dtype)
        d.coords = coords.data_ptr()
        d.n_nodes = self.op.n_nodes
        keep = [plan, coords]
        if u is not None:
            uu = self._flat(u).to(dtype).contiguous()
            d.u = uu.data_ptr()
            keep.append(uu)
        if fixed is not None:
            mk = self._mask(fixed, torch.empty(self.n_dofs, device=self.op.device))
            d.fixed = mk.data_ptr()
            keep.append(mk)
        return d, keep


class Poisson(Energy):
    kind = _lib.TG_POISSON
    name = "poisson"

    def __init__(self, op: Operator, kappa=1.0, f: float = 0.0):
        super().__init__(op, kappa, f)


class LinearElastic(Energy):
    kind = _lib.TG_LINEAR_ELASTIC
    name = "linear_elastic"

    def __init__(self, op: Operator, mu: float, lmbda: float):
        super().__init__(op, mu, lmbda)

    @classmethod
    def from_young(cls, op: Operator, E: float, nu: float):
        mu, lm = lame_from_young(E, nu)
        return cls(op, mu, lm)


class NeoHookean(Energy):
    kind = _lib.TG_NEO_HOOKEAN
    name = "neo_hookean"

    def __init__(self, op: Operator, mu: float, lmbda: float):
        super().__init__(op, mu, lmbda)
