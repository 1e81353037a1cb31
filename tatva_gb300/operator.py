"""Operator: quadrature maps over a mesh, executed by the sm_103a kernels.

Drop-in for ``tatva/operator.py`` ``Operator`` (:77-554) on torch tensors:

=============================  =================================================
reference (tatva/operator.py)  here
=============================  =================================================
``eval`` (:358-377)            ``tg_eval``                     (E,Q,...)
``grad`` (:379-397)            ``tg_grad``                     (E,Q,...,D)
``get_integration_weights``    ``tg_integration_weights``      (E,Q)
(:172-192)
``integrate_per_element``      ``tg_integrate_quad``           (E,...)
(:321-356)
``integrate`` (:307-319)       ``tg_sum_rows`` (deterministic FP64 accumulation)
``map`` / ``map_over_elements``  ``tg_gather_nodal`` + ``torch.func.vmap`` of the
(:225-305)                     user function over elements (and quadrature points)
``quads`` (:512-521)           ``eval(mesh.coords)``
=============================  =================================================

Reverse-mode AD: ``eval``, ``grad``, the quadrature integration, the element sum
and the gather are ``torch.autograd.Function``s whose backward passes are the
transpose kernels (``tg_eval_transpose``, ``tg_grad_transpose``,
``tg_integrate_quad_transpose``, ``tg_scatter_nodal``); each transpose's backward
is the forward map again, so double backward (Hessian-vector products through
``torch.autograd``) works on user energies written with these maps.

Validation follows ``Operator.__check_init__`` (:132-170): ``ValueError`` /
``TypeError`` with the reference's messages.
"""

from __future__ import annotations

import dataclasses

import math
from numbers import Number
from typing import Callable, Sequence

import numpy as np
import torch

from . import _lib
from ._device import prec_of, ptr, require_cuda, stream, workspace
from .element import Element
from .mesh import Mesh


class Operator:
    def __init__(self, mesh: Mesh, element: Element, batch_size: int | None = None,
                 cache_weights: bool = False):
        self.mesh = mesh
        self.element = element
        self.cache_weights = bool(cache_weights)
        self.__check_init__()
        self.batch_size = int(batch_size) if batch_size is not None else mesh.n_elements
        self._cache: dict = {}
        if self.cache_weights and mesh.coords.is_cuda:
            self._cache[("w", torch.float64)] = self._weights_raw(torch.float64)

    # ------------------------------------------------------------------ checks
    def __check_init__(self) -> None:
        coords, elements = self.mesh.coords, self.mesh.elements
        if coords.ndim != 2:
            raise ValueError("Mesh coordinates must be a 2D array shaped (n_nodes, n_dim).")
        if coords.shape[0] == 0:
            raise ValueError("Mesh must contain at least one node.")
        if elements.ndim != 2:
            raise ValueError(
                "Mesh elements must be a 2D array shaped (n_elements, n_nodes_per_element).")
        if elements.shape[0] == 0:
            raise ValueError("Mesh must contain at least one element.")
        if elements.dtype.is_floating_point:
            raise TypeError("Mesh element connectivity must contain integer indices.")
        el = self.mesh.elements_host()
        if el.min() < 0:
            raise ValueError("Mesh element connectivity contains negative node indices.")
        if el.max() >= coords.shape[0]:
            raise ValueError(
                "Mesh element connectivity references nodes outside the mesh coordinates array.")
        if elements.shape[1] != self.element.n_nodes:
            raise ValueError(
                f"{type(self.element).__name__} has {self.element.n_nodes} nodes, the mesh "
                f"elements have {elements.shape[1]}")
        if coords.shape[1] != self.element.dim:
            raise ValueError(
                f"{type(self.element).__name__} needs {self.element.dim}D coordinates, the "
                f"mesh has {coords.shape[1]}D")

    # ------------------------------------------------------------------ basics
    @property
    def n_elements(self) -> int:
        return self.mesh.n_elements

    @property
    def n_nodes(self) -> int:
        return self.mesh.n_nodes

    @property
    def n_quad(self) -> int:
        return self.element.n_quad

    @property
    def dim(self) -> int:
        return self.element.dim

    @property
    def device(self):
        return self.mesh.coords.device

    def coords_as(self, dtype) -> torch.Tensor:
        if dtype == torch.float64:
            return self.mesh.coords
        key = ("coords", dtype)
        if key not in self._cache:
            c = torch.empty(self.mesh.coords.shape, dtype=dtype, device=self.device)
            require_cuda(c)
            _lib.call("tg_convert", _lib.TG_F64, ptr(self.mesh.coords), prec_of(dtype), ptr(c),
                      c.numel(), stream())
            self._cache[key] = c
        return self._cache[key]

    def incidence(self):
        """node -> (e*n_e + a) CSR on the device (host-built, ascending e)."""
        if "inc" not in self._cache:
            el = self.mesh.elements_host()
            ptr_h = np.zeros(self.n_nodes + 1, np.int32)
            idx_h = np.zeros(max(el.size, 1), np.int32)
            _lib.call("tg_node_incidence", el.ctypes.data, el.shape[0], el.shape[1],
                      self.n_nodes, ptr_h.ctypes.data, idx_h.ctypes.data)
            self._cache["inc"] = (torch.from_numpy(ptr_h).to(self.device),
                                  torch.from_numpy(idx_h).to(self.device))
        return self._cache["inc"]

    def plan(self, block_elems: int | None = None, max_local_nodes: int | None = None,
             threads: int | None = None):
        """Element-block plan of the fused kernels (cached per tuning)."""
        from . import autotune
        from .plan import BlockPlan, DEFAULT_MAX_LOCAL, DEFAULT_THREADS

        if block_elems is None and max_local_nodes is None and threads is None:
            cfg = autotune.lookup(self)
            if cfg == (None, None, None) and self.element.tg_id == _lib.TG_HEX8:
                # Hex8: 512-element blocks suit the parallelepiped kernels; meshes whose
                # blocks are mostly general (per-QP path) run faster with 1024 / 128
                p512 = self.plan(512, DEFAULT_MAX_LOCAL, DEFAULT_THREADS[_lib.TG_HEX8])
                if 2 * p512.sizes["n_affine_blocks"] >= p512.sizes["n_blocks"]:
                    return p512
                return self.plan(1024, DEFAULT_MAX_LOCAL, 128)
            block_elems, max_local_nodes, threads = cfg
        threads = threads or DEFAULT_THREADS[self.element.tg_id]
        key = ("plan", block_elems, max_local_nodes or DEFAULT_MAX_LOCAL, threads)
        if key not in self._cache:
            self._cache[key] = BlockPlan(self.element.tg_id, self.mesh.elements_host(),
                                         self.mesh.coords_host(), self.device,
                                         block_elems=block_elems,
                                         max_local_nodes=max_local_nodes or DEFAULT_MAX_LOCAL,
                                         threads=threads)
        return self._cache[key]

    def unused_nodes(self) -> torch.Tensor:
        """Nodes that no element references (cached); the fused kernels do not write
        their entries."""
        key = "unused_nodes"
        if key not in self._cache:
            used = np.zeros(self.n_nodes, dtype=bool)
            used[self.mesh.elements_host().reshape(-1)] = True
            self._cache[key] = torch.as_tensor(np.where(~used)[0], device=self.device)
        return self._cache[key]

    def _nodal_shape(self, u: torch.Tensor):
        if u.ndim == 0 or u.shape[0] != self.n_nodes:
            raise ValueError(
                f"nodal values must have leading dimension n_nodes={self.n_nodes}, "
                f"got shape {tuple(u.shape)}")
        vshape = tuple(u.shape[1:])
        return vshape, int(math.prod(vshape)) if vshape else 1

    # ------------------------------------------------------------------ raw kernels
    def _eval_raw(self, u: torch.Tensor) -> torch.Tensor:
        require_cuda(u)
        u = u.contiguous()
        vshape, V = self._nodal_shape(u)
        out = torch.empty((self.n_elements, self.n_quad) + vshape, dtype=u.dtype,
                          device=u.device)
        _lib.call("tg_eval", self.element.tg_id, prec_of(u.dtype), ptr(u), self.n_nodes, V,
                  ptr(self.mesh.elements), self.n_elements, ptr(out), stream())
        return out

    def _grad_raw(self, u: torch.Tensor) -> torch.Tensor:
        require_cuda(u)
        u = u.contiguous()
        vshape, V = self._nodal_shape(u)
        out = torch.empty((self.n_elements, self.n_quad) + vshape + (self.dim,), dtype=u.dtype,
                          device=u.device)
        _lib.call("tg_grad", self.element.tg_id, prec_of(u.dtype), ptr(u),
                  ptr(self.coords_as(u.dtype)), self.n_nodes, V, ptr(self.mesh.elements),
                  self.n_elements, ptr(out), stream())
        return out

    def _grad_t_raw(self, flux: torch.Tensor, vshape) -> torch.Tensor:
        require_cuda(flux)
        flux = flux.contiguous()
        V = int(math.prod(vshape)) if vshape else 1
        out = torch.empty((self.n_nodes,) + tuple(vshape), dtype=flux.dtype, device=flux.device)
        ip, ii = self.incidence()
        nb = _lib.lib().tg_grad_transpose_workspace_bytes(self.element.tg_id,
                                                          prec_of(flux.dtype), self.n_elements, V)
        ws = torch.empty(max(int(nb), 1), dtype=torch.uint8, device=flux.device)
        _lib.call("tg_grad_transpose", self.element.tg_id, prec_of(flux.dtype), ptr(flux),
                  ptr(self.coords_as(flux.dtype)), self.n_nodes, V, ptr(self.mesh.elements),
                  self.n_elements, ptr(ip), ptr(ii), ptr(out), ptr(ws), nb, stream())
        return out

    def _eval_t_raw(self, q: torch.Tensor, vshape) -> torch.Tensor:
        require_cuda(q)
        q = q.contiguous()
        V = int(math.prod(vshape)) if vshape else 1
        out = torch.empty((self.n_nodes,) + tuple(vshape), dtype=q.dtype, device=q.device)
        ip, ii = self.incidence()
        _lib.call("tg_eval_transpose", self.element.tg_id, prec_of(q.dtype), ptr(q),
                  self.n_nodes, V, ptr(self.mesh.elements), self.n_elements, ptr(ip), ptr(ii),
                  ptr(out), stream())
        return out

    def _weights_raw(self, dtype) -> torch.Tensor:
        out = torch.empty((self.n_elements, self.n_quad), dtype=dtype, device=self.device)
        require_cuda(out)
        _lib.call("tg_integration_weights", self.element.tg_id, prec_of(dtype),
                  ptr(self.coords_as(dtype)), self.n_nodes, ptr(self.mesh.elements),
                  self.n_elements, ptr(out), stream())
        return out

    def _weights(self, dtype) -> torch.Tensor:
        key = ("w", dtype)
        if key in self._cache:
            return self._cache[key]
        w = self._weights_raw(dtype)
        if self.cache_weights:
            self._cache[key] = w
        return w

    def _intq_raw(self, quad: torch.Tensor) -> torch.Tensor:
        require_cuda(quad)
        quad = quad.contiguous()
        if quad.ndim < 2 or quad.shape[0] != self.n_elements or quad.shape[1] != self.n_quad:
            raise ValueError(
                f"quadrature values must be shaped (n_elements={self.n_elements}, "
                f"n_quad={self.n_quad}, ...), got {tuple(quad.shape)}")
        vshape = tuple(quad.shape[2:])
        V = int(math.prod(vshape)) if vshape else 1
        w = self._weights(quad.dtype)
        out = torch.empty((self.n_elements,) + vshape, dtype=quad.dtype, device=quad.device)
        _lib.call("tg_integrate_quad", prec_of(quad.dtype), ptr(quad), ptr(w), self.n_elements,
                  self.n_quad, V, ptr(out), stream())
        return out

    def _intq_t_raw(self, g: torch.Tensor) -> torch.Tensor:
        g = g.contiguous()
        vshape = tuple(g.shape[1:])
        V = int(math.prod(vshape)) if vshape else 1
        w = self._weights(g.dtype)
        out = torch.empty((self.n_elements, self.n_quad) + vshape, dtype=g.dtype, device=g.device)
        _lib.call("tg_integrate_quad_transpose", prec_of(g.dtype), ptr(g), ptr(w),
                  self.n_elements, self.n_quad, V, ptr(out), stream())
        return out

    def _gather_raw(self, u: torch.Tensor) -> torch.Tensor:
        require_cuda(u)
        u = u.contiguous()
        vshape, V = self._nodal_shape(u)
        npe = self.element.n_nodes
        out = torch.empty((self.n_elements, npe) + vshape, dtype=u.dtype, device=u.device)
        _lib.call("tg_gather_nodal", prec_of(u.dtype), ptr(u), self.n_nodes, V,
                  ptr(self.mesh.elements), self.n_elements, npe, ptr(out), stream())
        return out

    def _scatter_raw(self, vals: torch.Tensor, vshape) -> torch.Tensor:
        vals = vals.contiguous()
        V = int(math.prod(vshape)) if vshape else 1
        out = torch.empty((self.n_nodes,) + tuple(vshape), dtype=vals.dtype, device=vals.device)
        ip, ii = self.incidence()
        _lib.call("tg_scatter_nodal", prec_of(vals.dtype), ptr(vals), self.n_nodes, V,
                  self.element.n_nodes, ptr(ip), ptr(ii), ptr(out), stream())
        return out

    # ------------------------------------------------------------------ public maps
    def eval(self, nodal_values: torch.Tensor) -> torch.Tensor:
        """(E, Q, ...) values at the quadrature points (operator.py:358-377)."""
        return _Eval.apply(nodal_values, self) if _needs_grad(nodal_values) else \
            self._eval_raw(nodal_values)

    def grad(self, nodal_values: torch.Tensor) -> torch.Tensor:
        """(E, Q, ..., D) gradients at the quadrature points (operator.py:379-397)."""
        return _Grad.apply(nodal_values, self) if _needs_grad(nodal_values) else \
            self._grad_raw(nodal_values)

    def get_integration_weights(self) -> torch.Tensor:
        """(E, Q) detJ * w_q in FP64 (operator.py:172-192)."""
        return self._weights(torch.float64)

    def _integrate_quad_array(self, quad_values: torch.Tensor) -> torch.Tensor:
        return _IntQ.apply(quad_values, self) if _needs_grad(quad_values) else \
            self._intq_raw(quad_values)

    def integrate_per_element(self, arg) -> torch.Tensor:
        """Per-element integrals of a numeric, nodal or quadrature array (operator.py:321-342)."""
        if isinstance(arg, Number) or (isinstance(arg, torch.Tensor) and arg.ndim == 0):
            quad = torch.full((self.n_elements, self.n_quad), float(arg), dtype=torch.float64,
                              device=self.device)
            return self._integrate_quad_array(quad)
        if not isinstance(arg, torch.Tensor):
            arg = torch.as_tensor(np.asarray(arg), device=self.device)
        if arg.shape[0] == self.n_elements:
            return self._integrate_quad_array(arg)
        return self._integrate_quad_array(self.eval(arg))

    def integrate(self, arg) -> torch.Tensor:
        """Integral over the mesh (operator.py:307-319), summed deterministically."""
        per = self.integrate_per_element(arg)
        return _SumRows.apply(per) if _needs_grad(per) else _sum_rows_raw(per)

    def quads(self) -> torch.Tensor:
        """Quadrature points in physical coordinates (operator.py:512-521)."""
        return self.eval(self.mesh.coords)

    def map(self, func: Callable, *, element_quantity: Sequence[int] = ()) -> Callable:
        """func(xi, *element_values) at every (element, quadrature point) (operator.py:225-266).

        Nodal arguments are gathered per element by ``tg_gather_nodal``; ``func`` is
        vectorised with ``torch.func.vmap`` over quadrature points and elements.
        """
        qp = torch.as_tensor(self.element.quad_points, dtype=torch.float64, device=self.device)

        def _mapped(*values, **kwargs):
            xs = tuple(self._gather(v) if i not in element_quantity else v
                       for i, v in enumerate(values))

            def per_element(*ev):
                return torch.func.vmap(lambda xi: func(xi, *ev, **kwargs))(qp)

            return torch.func.vmap(per_element)(*xs)

        return _mapped

    def map_over_elements(self, func: Callable, *,
                          element_quantity: Sequence[int] = ()) -> Callable:
        """func(*element_values) per element (operator.py:268-305)."""

        def _mapped(*values, **kwargs):
            xs = tuple(self._gather(v) if i not in element_quantity else v
                       for i, v in enumerate(values))
            return torch.func.vmap(lambda *ev: func(*ev, **kwargs))(*xs)

        return _mapped

    def _gather(self, v: torch.Tensor) -> torch.Tensor:
        return _Gather.apply(v, self) if _needs_grad(v) else self._gather_raw(v)

    def interpolate(self, arg, points):
        raise NotImplementedError(
            "Operator.interpolate (point location) is not part of the GB300 hot path")

    def project(self, field: torch.Tensor, colored_matrix=None, lifter=None,
                rtol: float = 1e-13) -> torch.Tensor:
        """L2 projection of a quadrature field (E, Q, ...) onto the nodes
        (operator.py:523-554, tatva/utils.py:118-262): M x = b with the consistent mass
        matrix M_ab = int N_a N_b, assembled on the scalar pattern by the colored
        Jacobian kernels (one mass-operator application per colour), and
        b_a = int N_a field, solved per component by device CG to ``rtol`` (the
        reference uses a sparse direct solve).  With a ``lifter`` (scalar dofs = nodes)
        the reduced system is solved and constrained nodes take the lifter's values
        (Lifter.lift_from_zeros)."""
        from . import sparse, solvers

        require_cuda(field)
        f = field.to(torch.float64).contiguous()
        if f.ndim < 2 or f.shape[0] != self.n_elements or f.shape[1] != self.n_quad:
            raise ValueError(f"field must be shaped (n_elements={self.n_elements}, "
                             f"n_quad={self.n_quad}, ...), got {tuple(field.shape)}")
        nn = self.n_nodes
        if colored_matrix is not None and colored_matrix.shape[0] % nn:
            raise ValueError("colored matrix size is not a multiple of the number of nodes")
        if lifter is not None and lifter.size != nn:
            raise NotImplementedError("projection with a lifter needs one dof per node")
        vshape = tuple(f.shape[2:])
        F = f.reshape(self.n_elements, self.n_quad, -1)
        key = "proj_mass"
        if key not in self._cache:
            cm = sparse.ColoredMatrix.from_csr(sparse.pattern_from_mesh(self.mesh, 1),
                                               device=self.device)
            w = self._weights(torch.float64)

            def mass(u):
                return self._eval_t_raw((self._eval_raw(u.contiguous()) * w).contiguous(), ())

            Jc = torch.empty((nn, cm.n_colors), dtype=torch.float64, device=self.device)
            for c in range(cm.n_colors):
                Jc[:, c] = mass((cm.colors == c).to(torch.float64))
            rows, cols = sparse.compute_rows_cols(cm)
            M = dataclasses.replace(cm, data=sparse.decompress(Jc, rows, cols))
            self._cache[key] = M
        M = self._cache[key]
        w = self._weights(torch.float64)
        mask = lifter.fixed_mask(self.device) if lifter is not None else None
        out = torch.empty((nn, F.shape[2]), dtype=torch.float64, device=self.device)
        for c in range(F.shape[2]):
            b = self._eval_t_raw((F[:, :, c] * w).contiguous(), ())
            if mask is not None:
                b = torch.where(mask.bool(), torch.zeros_like(b), b)
            r = solvers.csr_cg(M, b, fixed=mask, rtol=rtol, maxiter=10000, check_every=10)
            out[:, c] = r.x
        if lifter is not None:
            for k in range(F.shape[2]):
                out[:, k] = lifter.lift(lifter.reduce(out[:, k]), out[:, k])
        return out.reshape((nn,) + vshape)

    def _replace(self, **changes):
        kw = dict(mesh=self.mesh, element=self.element, batch_size=self.batch_size,
                  cache_weights=self.cache_weights)
        kw.update(changes)
        return Operator(**kw)


# ---------------------------------------------------------------------- autograd
def _needs_grad(t) -> bool:
    return isinstance(t, torch.Tensor) and t.requires_grad and torch.is_grad_enabled()


def _sum_rows_raw(per: torch.Tensor) -> torch.Tensor:
    require_cuda(per)
    per = per.contiguous()
    vshape = tuple(per.shape[1:])
    V = int(math.prod(vshape)) if vshape else 1
    out = torch.empty(vshape, dtype=per.dtype, device=per.device)
    nb = _lib.lib().tg_sum_rows_workspace_bytes(prec_of(per.dtype), V)
    ws = workspace(nb, per.device)
    _lib.call("tg_sum_rows", prec_of(per.dtype), ptr(per), per.shape[0], V, ptr(out), ptr(ws),
              nb, stream())
    return out


class _Eval(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, op):
        ctx.op, ctx.vshape = op, tuple(u.shape[1:])
        return op._eval_raw(u)

    @staticmethod
    def backward(ctx, g):
        return _EvalT.apply(g, ctx.op, ctx.vshape), None


class _EvalT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, q, op, vshape):
        ctx.op = op
        return op._eval_t_raw(q, vshape)

    @staticmethod
    def backward(ctx, h):
        return _Eval.apply(h, ctx.op), None, None


class _Grad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, op):
        ctx.op, ctx.vshape = op, tuple(u.shape[1:])
        return op._grad_raw(u)

    @staticmethod
    def backward(ctx, g):
        return _GradT.apply(g, ctx.op, ctx.vshape), None


class _GradT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, flux, op, vshape):
        ctx.op = op
        return op._grad_t_raw(flux, vshape)

    @staticmethod
    def backward(ctx, h):
        return _Grad.apply(h, ctx.op), None, None


class _IntQ(torch.autograd.Function):
    @staticmethod
    def forward(ctx, quad, op):
        ctx.op = op
        return op._intq_raw(quad)

    @staticmethod
    def backward(ctx, g):
        return _IntQT.apply(g, ctx.op), None


class _IntQT(torch.autograd.Function):
    @staticmethod
    def forward(ctx, g, op):
        ctx.op = op
        return op._intq_t_raw(g)

    @staticmethod
    def backward(ctx, h):
        return _IntQ.apply(h, ctx.op), None


class _SumRows(torch.autograd.Function):
    @staticmethod
    def forward(ctx, per):
        ctx.n = per.shape[0]
        return _sum_rows_raw(per)

    @staticmethod
    def backward(ctx, g):
        return g.unsqueeze(0).expand((ctx.n,) + tuple(g.shape))


class _Gather(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, op):
        ctx.op, ctx.vshape = op, tuple(u.shape[1:])
        return op._gather_raw(u)

    @staticmethod
    def backward(ctx, g):
        return _Scatter.apply(g, ctx.op, ctx.vshape), None


class _Scatter(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vals, op, vshape):
        ctx.op = op
        return op._scatter_raw(vals, vshape)

    @staticmethod
    def backward(ctx, h):
        return _Gather.apply(h, ctx.op), None, None
