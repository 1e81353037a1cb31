"""Request loop for Hex8 linear-elastic solves with continuous batching.

The reference has no serving layer; each request here is what a reference user
would run once: a matrix-free solve of a clamped brick under traction with the
jax.jvp(jax.grad(E)) HVP (README.md:93), to relative residual 1e-10.

* Resident state: one ``BrickModel`` per brick side holds the mesh, operator,
  element-block plan, Dirichlet mask and unit-traction load on the device; a
  request only adds its vectors and solver workspace.
* Slots: ``slots`` worker threads, each with its own CUDA stream.  A free slot
  takes the oldest request that has arrived, if the HBM budget has room for its
  vectors and workspace; otherwise it waits until a finishing solve returns memory.
  Requests that arrive while others are running are admitted as soon as a slot and
  memory are free, and their kernels overlap with the running solves on the device.
* Each solve is ``tg_mixed_solve`` on the slot's stream: FP32 HVP inner CG, FP64
  refinement on the true residual.  Its arithmetic depends only on its own data
  (deterministic kernels, no data shared between requests), so a result is the
  same alone and in the mix.
* Reported: per-request queueing, service and end-to-end latency (from arrival);
  p50 / p99 latency and solves/s over the run.
"""

from __future__ import annotations

import ctypes
import threading
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._device import ptr
from .materials import LinearElastic
from .problems import clamped_brick


@dataclass
class SolveRequest:
    rid: int
    arrival: float    # seconds after the start of the run
    side: int         # brick of side^3 Hex8 cells
    young: float
    poisson: float
    traction: float


@dataclass
class SolveRecord:
    rid: int
    side: int
    arrival: float
    start: float
    end: float
    status: int
    iterations: int
    refinements: int
    rel_res: float
    slot: int
    x: torch.Tensor | None = field(default=None, repr=False)

    @property
    def latency(self) -> float:
        return self.end - self.arrival


def synthetic_requests(n: int, rate: float = 2000.0, sides=(16, 24, 32, 48, 64),
                       seed: int = 0) -> list[SolveRequest]:
    """Poisson arrivals (mean ``rate`` per second), side uniform in ``sides``,
    E ~ lognormal(0, 0.5), nu ~ U[0.2, 0.45], traction magnitude ~ U[0.5, 1.5] 1e-3."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n)
    arrival = np.cumsum(gaps) - gaps[0]
    side = rng.choice(np.asarray(sides), size=n)
    young = rng.lognormal(0.0, 0.5, size=n)
    nu = rng.uniform(0.2, 0.45, size=n)
    tr = rng.uniform(0.5, 1.5, size=n) * 1e-3
    return [SolveRequest(i, float(arrival[i]), int(side[i]), float(young[i]), float(nu[i]),
                         float(tr[i])) for i in range(n)]


class BrickModel:
    """Device-resident mesh, operator, plan, mask and unit-traction load of one side."""

    def __init__(self, side: int, device):
        P = clamped_brick(side, device, traction=1.0)
        self.side = side
        self.op = P["op"]
        self.fixed = P["fixed"]
        self.f_unit = P["b"]
        self.n_dofs = self.f_unit.numel()
        # build the cached plan and coordinate copies once, before any thread uses them
        self.op.plan()
        self.op.coords_as(torch.float32)
        self.op.coords_as(torch.float64)
        en = LinearElastic.from_young(self.op, 1.0, 0.3)
        d64, _ = en.operator_desc(None, self.fixed, torch.float64)
        d32, _ = en.operator_desc(None, self.fixed, torch.float32)
        self.ws_bytes = int(_lib.lib().tg_mixed_workspace_bytes(ctypes.byref(d64), ctypes.byref(d32)))
        # b, x, diag (FP64), the FP32 mask-free copies made by operator_desc, workspace
        self.bytes_per_solve = self.ws_bytes + 5 * 8 * self.n_dofs


class Server:
    def __init__(self, device=None, slots: int = 16, hbm_budget: int = 16 << 30,
                 rtol: float = 1e-10, inner_rtol: float = 1e-4, check_every: int = 50,
                 max_outer: int = 50, max_inner: int = 200000, keep_solutions: bool = False):
        self.device = torch.device(device or "cuda")
        self.slots = int(slots)
        self.hbm_budget = int(hbm_budget)
        self.rtol, self.inner_rtol = rtol, inner_rtol
        self.check_every, self.max_outer, self.max_inner = check_every, max_outer, max_inner
        self.keep_solutions = keep_solutions
        self.models: dict[int, BrickModel] = {}
        self.streams = [torch.cuda.Stream(device=self.device) for _ in range(self.slots)]

    def model(self, side: int) -> BrickModel:
        if side not in self.models:
            self.models[side] = BrickModel(side, self.device)
        return self.models[side]

    def warm(self, sides) -> None:
        for s in sorted(set(int(v) for v in sides)):
            m = self.model(s)
            if m.bytes_per_solve > self.hbm_budget:
                raise ValueError(f"a side-{s} solve needs {m.bytes_per_solve} bytes, above the "
                                 f"HBM budget of {self.hbm_budget}")
            self._solve(SolveRequest(-1, 0.0, s, 1.0, 0.3, 1e-3), 0)

    # ------------------------------------------------------------------ one solve
    def _solve(self, req: SolveRequest, slot: int):
        m = self.models[req.side]
        st = self.streams[slot]
        with torch.cuda.stream(st):
            en = LinearElastic.from_young(m.op, req.young, req.poisson)
            b = m.f_unit * req.traction
            x = torch.zeros(m.n_dofs, dtype=torch.float64, device=self.device)
            d64, k64 = en.operator_desc(None, m.fixed, torch.float64)
            d32, k32 = en.operator_desc(None, m.fixed, torch.float32)
            diag = en.diagonal(torch.zeros_like(x), m.fixed).reshape(-1).contiguous()
            ws = torch.empty(max(m.ws_bytes, 1), dtype=torch.uint8, device=self.device)
            stats = _lib.SolveStats()
            rc = _lib.lib().tg_mixed_solve(
                ctypes.byref(d64), ctypes.byref(d32), ptr(b), ptr(x), ptr(diag), self.rtol,
                self.inner_rtol, self.max_outer, self.max_inner, self.check_every, ptr(ws),
                m.ws_bytes, ctypes.byref(stats), st.cuda_stream)
            st.synchronize()
            del k64, k32
        if rc not in (_lib.TG_OK, _lib.TG_ERR_NOT_CONVERGED, _lib.TG_ERR_BREAKDOWN):
            _lib.check(rc)
        return x, rc, stats

    # ------------------------------------------------------------------ the loop
    def run(self, requests, realtime: bool = True) -> "ServeReport":
        """Serve ``requests`` (arrival times relative to the start of the run)."""
        self.warm(r.side for r in requests)
        torch.cuda.synchronize(self.device)
        queue = deque(sorted(requests, key=lambda r: (r.arrival, r.rid)))
        cond = threading.Condition()
        used = [0]
        records: list[SolveRecord] = []
        errors: list[BaseException] = []
        t0 = time.perf_counter()

        def worker(slot: int):
            while True:
                with cond:
                    while True:
                        if not queue or errors:
                            return
                        req = queue[0]
                        need = self.models[req.side].bytes_per_solve
                        now = time.perf_counter() - t0
                        if realtime and req.arrival > now:
                            cond.wait(timeout=req.arrival - now)
                            continue
                        if used[0] + need > self.hbm_budget:
                            cond.wait(timeout=0.05)
                            continue
                        queue.popleft()
                        used[0] += need
                        break
                start = time.perf_counter() - t0
                try:
                    x, rc, stats = self._solve(req, slot)
                except BaseException as ex:  # noqa: BLE001 - reported to the caller
                    with cond:
                        errors.append(ex)
                        used[0] -= need
                        cond.notify_all()
                    return
                end = time.perf_counter() - t0
                rec = SolveRecord(req.rid, req.side, req.arrival, start, end, rc,
                                  stats.iterations, stats.outer, stats.rel_res, slot,
                                  x if self.keep_solutions else None)
                del x
                with cond:
                    records.append(rec)
                    used[0] -= need
                    cond.notify_all()

        threads = [threading.Thread(target=worker, args=(i,), daemon=True)
                   for i in range(self.slots)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise errors[0]
        records.sort(key=lambda r: r.rid)
        return ServeReport(records, self.slots, self.hbm_budget)


@dataclass
class ServeReport:
    records: list
    slots: int
    hbm_budget: int

    def summary(self) -> dict:
        lat = np.array([r.latency for r in self.records])
        svc = np.array([r.end - r.start for r in self.records])
        wait = np.array([r.start - r.arrival for r in self.records])
        first = min(r.arrival for r in self.records)
        last = max(r.end for r in self.records)
        ok = sum(1 for r in self.records if r.status == _lib.TG_OK)
        return {
            "requests": len(self.records),
            "converged": ok,
            "solves_per_s": len(self.records) / (last - first),
            "makespan_s": last - first,
            "p50_latency_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_latency_ms": float(np.percentile(lat, 99) * 1e3),
            "p50_service_ms": float(np.percentile(svc, 50) * 1e3),
            "p99_service_ms": float(np.percentile(svc, 99) * 1e3),
            "mean_queue_ms": float(wait.mean() * 1e3),
            "max_rel_res": float(max(r.rel_res for r in self.records)),
            "slots": self.slots,
            "hbm_budget_bytes": self.hbm_budget,
        }


__all__ = ["BrickModel", "ServeReport", "Server", "SolveRecord", "SolveRequest",
           "synthetic_requests"]
