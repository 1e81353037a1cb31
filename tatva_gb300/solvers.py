"""Device-resident solvers composed on the hot-path kernels.

The reference ships no solver; users call ``jax.scipy.sparse.linalg.cg`` with the
matrix-free HVP (README.md:93) or a sparse factorisation of the colored Hessian.
These wrappers drive the native solvers of the C ABI:

* ``cg``        Jacobi-preconditioned CG on the fused HVP (FP32 or FP64 vectors,
                FP64 dot products), ``tg_cg_solve``
* ``mixed_cg``  FP32 HVP + FP32 CG inner solves with FP64 iterative refinement on the
                true residual (FP64 HVP), ``tg_mixed_solve``
* ``csr_cg``    CG on an assembled CSR matrix (``tg_spmv``; ``tg_spmv_blocks3`` for
  3-dof-per-node patterns)
* ``newton``    load-stepped Newton: FP64 residual and update, colored sparse tangent
                (``sparse.jacfwd`` of the residual, optionally in FP32), CSR CG inner solve

All scalars stay on the GPU; the host reads one small vector every
``check_every`` iterations, which run as one captured CUDA graph.
"""

from __future__ import annotations

import ctypes
import time
import weakref
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._device import aligned16, prec_of, ptr, require_cuda, workspace


@dataclass
class SolveResult:
    x: torch.Tensor
    iterations: int
    outer: int
    rel_res: float
    status: int
    seconds: float
    history: list = field(default_factory=list)
    message: str = ""

    @property
    def converged(self) -> bool:
        return self.status == _lib.TG_OK


_STREAMS: dict = {}


def solver_stream(device=None) -> torch.cuda.Stream:
    """A non-default stream (graph capture is not allowed on the legacy stream)."""
    dev = torch.device(device or "cuda")
    key = str(dev)
    if key not in _STREAMS:
        _STREAMS[key] = torch.cuda.Stream(device=dev)
    return _STREAMS[key]


def _run(fn, device, raise_on_fail):
    st = solver_stream(device)
    cur = torch.cuda.current_stream(device)
    st.wait_stream(cur)
    stats = _lib.SolveStats()
    t0 = time.perf_counter()
    with torch.cuda.stream(st):
        rc = fn(st.cuda_stream, ctypes.byref(stats))
    cur.wait_stream(st)
    torch.cuda.synchronize(device)
    dt = time.perf_counter() - t0
    msg = _lib.lib().tg_last_error().decode(errors="replace") if rc != _lib.TG_OK else ""
    if rc != _lib.TG_OK and raise_on_fail:
        raise _lib._EXC.get(rc, RuntimeError)(msg)
    return stats, rc, dt, msg


def cg(energy, b: torch.Tensor, x0: torch.Tensor | None = None, *, u=None, fixed=None,
       rtol: float = 1e-10, maxiter: int = 100000, check_every: int = 50, dtype=None,
       diag: torch.Tensor | None = None, raise_on_fail: bool = True) -> SolveResult:
    """Solve d2E/du2(u) x = b (masked by ``fixed``) with Jacobi-CG in ``dtype``."""
    dtype = dtype or b.dtype
    require_cuda(b)
    n = energy.n_dofs
    bb = aligned16(b.reshape(-1).to(dtype).contiguous())
    x = (x0.reshape(-1).to(dtype).clone() if x0 is not None
         else torch.zeros(n, dtype=dtype, device=b.device))
    desc, keep = energy.operator_desc(u, fixed, dtype)
    if diag is None:
        uu = u if u is not None else torch.zeros(n, dtype=dtype, device=b.device)
        diag = energy.diagonal(uu.to(dtype), fixed)
    diag = diag.reshape(-1).to(dtype).contiguous()
    nb = _lib.lib().tg_cg_workspace_bytes(ctypes.byref(desc))
    ws = workspace(nb, b.device)

    def go(st, stats):
        return _lib.lib().tg_cg_solve(ctypes.byref(desc), ptr(bb), ptr(x), ptr(diag), rtol,
                                      int(maxiter), int(check_every), ptr(ws), nb, stats, st)

    stats, rc, dt, msg = _run(go, b.device, raise_on_fail)
    del keep
    return SolveResult(x.view(b.shape), stats.iterations, 0, stats.rel_res, rc, dt, message=msg)


def mixed_cg(energy, b: torch.Tensor, x0: torch.Tensor | None = None, *, u=None, fixed=None,
             rtol: float = 1e-10, inner_rtol: float = 0.1, max_outer: int = 50,
             max_inner: int = 100000, check_every: int = 50,
             raise_on_fail: bool = True) -> SolveResult:
    """FP32 inner CG + FP64 iterative refinement to ||b - A64 x|| <= rtol ||b||.

    ``inner_rtol`` is the FP32 residual reduction between two FP64 residual
    replacements; from 0.01 up the inner CG keeps its search direction across them
    (reliable updates), below it restarts at each refinement."""
    require_cuda(b)
    n = energy.n_dofs
    bb = aligned16(b.reshape(-1).to(torch.float64).contiguous())
    x = (x0.reshape(-1).to(torch.float64).clone() if x0 is not None
         else torch.zeros(n, dtype=torch.float64, device=b.device))
    d64, k64 = energy.operator_desc(u, fixed, torch.float64)
    d32, k32 = energy.operator_desc(u, fixed, torch.float32)
    uu = u if u is not None else torch.zeros(n, dtype=torch.float64, device=b.device)
    diag = energy.diagonal(uu.to(torch.float64), fixed).reshape(-1).contiguous()
    nb = _lib.lib().tg_mixed_workspace_bytes(ctypes.byref(d64), ctypes.byref(d32))
    ws = workspace(nb, b.device)

    def go(st, stats):
        return _lib.lib().tg_mixed_solve(ctypes.byref(d64), ctypes.byref(d32), ptr(bb), ptr(x),
                                         ptr(diag), rtol, inner_rtol, int(max_outer),
                                         int(max_inner), int(check_every), ptr(ws), nb, stats,
                                         st)

    stats, rc, dt, msg = _run(go, b.device, raise_on_fail)
    del k64, k32
    return SolveResult(x.view(b.shape), stats.iterations, stats.outer, stats.rel_res, rc, dt,
                       message=msg)


# id of a pattern's indices tensor -> (weak reference to it, node blocks or None)
_BLOCKS3: dict = {}


def node_blocks3(cm):
    """Node blocks of a 3-dof-per-node CSR pattern (``tg_csr_node_blocks3``), computed
    once per pattern (per indices tensor); None when the pattern is not of that form."""
    hit = _BLOCKS3.get(id(cm.indices))
    if hit is not None and hit[0]() is cm.indices:
        return hit[1]
    for k in [k for k, (ref, _) in _BLOCKS3.items() if ref() is None]:
        del _BLOCKS3[k]
    n, nnz = cm.shape[0], cm.nnz
    res = None
    if n > 0 and n % 3 == 0 and nnz % 9 == 0:
        dev = cm.indices.device
        nptr = torch.empty(n // 3 + 1, dtype=torch.int32, device=dev)
        nidx = torch.empty(max(nnz // 9, 1), dtype=torch.int32, device=dev)
        flag = torch.zeros(1, dtype=torch.int32, device=dev)
        _lib.call("tg_csr_node_blocks3", n, ptr(cm.indptr), ptr(cm.indices), ptr(nptr),
                  ptr(nidx), ptr(flag), torch.cuda.current_stream(dev).cuda_stream)
        if int(flag.item()) == 0:
            res = (nptr, nidx)
    _BLOCKS3[id(cm.indices)] = (weakref.ref(cm.indices), res)
    return res


def csr_cg(cm, b: torch.Tensor, x0=None, *, fixed=None, rtol: float = 1e-8,
           maxiter: int = 100000, check_every: int = 50, raise_on_fail: bool = True,
           apply_dirichlet: bool = True) -> SolveResult:
    """Jacobi-CG on the CSR matrix ``cm`` (a ColoredMatrix with data); vectors take the
    dtype of ``cm.data``.  Fixed rows/columns are replaced by the identity."""
    dtype = cm.data.dtype
    require_cuda(b, cm.data)
    n = cm.shape[0]
    data = cm.data.contiguous()
    mask = None
    if fixed is not None:
        mask = fixed.fixed_mask(b.device) if hasattr(fixed, "fixed_mask") else fixed
        if apply_dirichlet:
            data = data.clone()
            _lib.call("tg_csr_apply_dirichlet", prec_of(dtype), n, ptr(cm.indptr),
                      ptr(cm.indices), ptr(mask), ptr(data), torch.cuda.current_stream().cuda_stream)
    bb = aligned16(b.reshape(-1).to(dtype).contiguous())
    x = (x0.reshape(-1).to(dtype).clone() if x0 is not None
         else torch.zeros(n, dtype=dtype, device=b.device))
    diag = torch.empty(n, dtype=dtype, device=b.device)
    _lib.call("tg_csr_diagonal", prec_of(dtype), n, ptr(cm.indptr), ptr(cm.indices), ptr(data),
              ptr(diag), torch.cuda.current_stream().cuda_stream)
    desc = _lib.OperatorDesc()
    desc.prec = prec_of(dtype)
    desc.n_rows = n
    desc.csr_indptr, desc.csr_indices, desc.csr_data = (cm.indptr.data_ptr(),
                                                        cm.indices.data_ptr(), data.data_ptr())
    blocks = node_blocks3(cm)
    if blocks is not None:  # 3 dofs per node: one neighbour id per 3 x 3 block
        desc.csr_node_ptr, desc.csr_node_indices = blocks[0].data_ptr(), blocks[1].data_ptr()
    nb = _lib.lib().tg_cg_workspace_bytes(ctypes.byref(desc))
    ws = workspace(nb, b.device)

    def go(st, stats):
        return _lib.lib().tg_cg_solve(ctypes.byref(desc), ptr(bb), ptr(x), ptr(diag), rtol,
                                      int(maxiter), int(check_every), ptr(ws), nb, stats, st)

    stats, rc, dt, msg = _run(go, b.device, raise_on_fail)
    return SolveResult(x.view(b.shape), stats.iterations, 0, stats.rel_res, rc, dt, message=msg)


def newton(energy, u0: torch.Tensor, lifter, *, colored_matrix=None, rtol: float = 1e-10,
           max_iter: int = 25, tangent_dtype=torch.float32, cg_rtol: float | None = None,
           forcing: str = "adaptive", eta_max: float = 1e-2,
           external_force: torch.Tensor | None = None) -> SolveResult:
    """Newton for min E(u) - f.u with Dirichlet values from ``lifter`` (FP64 residual and
    update; colored sparse tangent in ``tangent_dtype``; CSR CG inner solve).

    Inner tolerance: ``forcing="fixed"`` solves every step to ``cg_rtol`` (default 1e-6);
    ``"adaptive"`` uses the Eisenstat-Walker rule eta_k = 0.9 (|F_k| / |F_{k-1}|)^2
    (safeguarded, at most ``eta_max``), never tighter than needed for the final
    tolerance nor than 10 machine epsilons of the tangent precision.

    ``u0`` must already carry the prescribed values on the constrained dofs."""
    from . import sparse

    if colored_matrix is None:
        colored_matrix = sparse.ColoredMatrix.from_csr(
            sparse.pattern_from_mesh(energy.op.mesh, energy.n_values), device=u0.device)
    mask = lifter.fixed_mask(u0.device)
    u = u0.reshape(-1).to(torch.float64).clone()
    fext = None if external_force is None else external_force.reshape(-1).to(torch.float64)
    jac = sparse.jacfwd(energy.residual, colored_matrix)
    t0 = time.perf_counter()
    hist = []
    r0n = None
    status = _lib.TG_ERR_NOT_CONVERGED
    it = 0
    total_cg = 0
    if forcing not in ("fixed", "adaptive"):
        raise ValueError("forcing must be 'fixed' or 'adaptive'")
    eta_floor = 10.0 * float(torch.finfo(tangent_dtype).eps)
    eta_prev, rn_prev = None, None
    for it in range(max_iter + 1):
        r = energy.residual(u, fixed=mask)
        if fext is not None:
            r = r - torch.where(mask.bool(), torch.zeros_like(fext), fext)
        rn = float(torch.linalg.vector_norm(r).item())
        r0n = rn if r0n is None else r0n
        ref = float(torch.linalg.vector_norm(fext).item()) if fext is not None else r0n
        hist.append(rn)
        if rn <= rtol * max(ref, 1e-300) or rn == 0.0:
            status = _lib.TG_OK
            break
        if it == max_iter:
            break
        if forcing == "fixed":
            eta = 1e-6 if cg_rtol is None else cg_rtol
        else:
            if rn_prev is None:
                eta = eta_max
            else:
                eta = 0.9 * (rn / rn_prev) ** 2
                guard = 0.9 * eta_prev ** 2
                if guard > 0.1:
                    eta = max(eta, guard)
                eta = min(eta, eta_max)
            eta = max(eta, 0.5 * rtol * max(ref, 1e-300) / rn, eta_floor)
        eta_prev, rn_prev = eta, rn
        K = jac(u.to(tangent_dtype))
        sol = csr_cg(K, -r, fixed=mask, rtol=eta, raise_on_fail=False)
        total_cg += sol.iterations
        if sol.status == _lib.TG_ERR_BREAKDOWN or not bool(torch.isfinite(sol.x).all()):
            status = _lib.TG_ERR_BREAKDOWN  # indefinite tangent: stop, keep the last iterate
            break
        u = u + sol.x.to(torch.float64)
    torch.cuda.synchronize()
    res = SolveResult(u.view(u0.shape), total_cg, it, hist[-1] / max(hist[0], 1e-300), status,
                      time.perf_counter() - t0, hist)
    return res
