"""Request loop for Hex8 linear-elastic solves with continuous batching.

The reference has no serving layer; each request here is what a reference user
would run once: a matrix-free solve of a clamped brick under traction with the
jax.jvp(jax.grad(E)) HVP (README.md:93), to relative residual 1e-10.

* Resident state: one ``BrickModel`` per brick side holds the Dirichlet mask and
  the unit-traction load on the device (the brick's stencil needs no mesh data);
  a request adds its right-hand side, solution and solver workspace.
* Continuous batching: all running solves advance together in the brick batch
  engine (``tg_brick_*``): one launch per CG step for every request in flight,
  whatever its size.  Between steps the loop admits the oldest arrived requests
  into free slots while the HBM budget has room for their vectors and workspace,
  and retires the finished ones -- a request that arrives while others run joins
  them at the next step, and its work shares the launches with theirs.
* Each solve is FP32 grid-stencil Jacobi-CG inner solves with FP64 refinement on
  the true residual, decided per request on the device.  A request's arithmetic
  depends only on its own data (fixed CTA decomposition, fixed-order reductions,
  no data shared between requests), so a result is the same alone and in the mix.
* Reported: per-request queueing, service and end-to-end latency (from arrival);
  p50 / p99 latency and solves/s over the run.
"""

from __future__ import annotations

import ctypes
import time
from collections import deque
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from .materials import lame_from_young
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
    """Device-resident Dirichlet mask and unit-traction load of one brick side."""

    def __init__(self, side: int, device):
        P = clamped_brick(side, device, traction=1.0)
        plan = P["op"].plan()
        if not plan.grid:
            raise ValueError(f"the side-{side} brick is not a structured grid")
        self.side = side
        self.nodes = tuple(plan.grid_nodes)
        self.h = tuple(plan.grid_h)
        self.fixed = P["fixed"]
        self.f_unit = P["b"]
        self.n_dofs = self.f_unit.numel()
        arr = (ctypes.c_int32 * 3)(*self.nodes)
        self.ws_bytes = int(_lib.lib().tg_brick_workspace_bytes(arr))
        # b and x (FP64) beside the workspace
        self.bytes_per_solve = self.ws_bytes + 2 * 8 * self.n_dofs


class BrickBatch:
    """The ``tg_brick_*`` engine: up to 64 solves in flight on one device."""

    def __init__(self, device):
        self.device = torch.device(device)
        with torch.cuda.device(self.device):
            h = ctypes.c_void_p()
            _lib.check(_lib.lib().tg_brick_batch_create(ctypes.byref(h)))
        self.handle = h
        self.states = (_lib.BrickState * _lib.TG_BRICK_MAX_SLOTS)()

    def admit(self, req: _lib.BrickRequest, stream) -> int:
        slot = ctypes.c_int()
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().tg_brick_admit(self.handle, ctypes.byref(req), stream.cuda_stream,
                                                 ctypes.byref(slot)))
        return slot.value

    def step(self, iterations: int, stream) -> None:
        _lib.check(_lib.lib().tg_brick_step(self.handle, int(iterations), stream.cuda_stream))

    def poll(self, stream):
        _lib.check(_lib.lib().tg_brick_poll(self.handle, self.states, _lib.TG_BRICK_MAX_SLOTS,
                                            stream.cuda_stream))
        return self.states

    def close(self) -> None:
        if self.handle:
            _lib.lib().tg_brick_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


class Server:
    """Continuous-batching request loop.  ``slots`` (<= 64) solves run together;
    ``step_iterations`` CG steps run between two polls of the batch."""

    def __init__(self, device=None, slots: int = 64, hbm_budget: int = 16 << 30,
                 rtol: float = 1e-10, inner_rtol: float = 1e-4, step_iterations: int = 20,
                 max_outer: int = 50, max_inner: int = 200000, keep_solutions: bool = False):
        self.device = torch.device(device or "cuda")
        if not 1 <= int(slots) <= _lib.TG_BRICK_MAX_SLOTS:
            raise ValueError(f"slots must be in [1, {_lib.TG_BRICK_MAX_SLOTS}]")
        self.slots = int(slots)
        self.hbm_budget = int(hbm_budget)
        self.rtol, self.inner_rtol = rtol, inner_rtol
        self.step_iterations = int(step_iterations)
        self.max_outer, self.max_inner = max_outer, max_inner
        self.keep_solutions = keep_solutions
        self.models: dict[int, BrickModel] = {}
        self.stream = torch.cuda.Stream(device=self.device)
        self.batch = BrickBatch(self.device)

    def model(self, side: int) -> BrickModel:
        if side not in self.models:
            self.models[side] = BrickModel(side, self.device)
        return self.models[side]

    def warm(self, sides) -> None:
        """Build the models and run one solve of each side (loads every kernel)."""
        sides = sorted(set(int(v) for v in sides))
        for s in sides:
            m = self.model(s)
            if m.bytes_per_solve > self.hbm_budget:
                raise ValueError(f"a side-{s} solve needs {m.bytes_per_solve} bytes, above the "
                                 f"HBM budget of {self.hbm_budget}")
        self._loop([SolveRequest(-1 - i, 0.0, s, 1.0, 0.3, 1e-3) for i, s in enumerate(sides)],
                   realtime=False)

    def solve_alone(self, req: SolveRequest) -> SolveRecord:
        """One request with the batch to itself."""
        keep = self.keep_solutions
        self.keep_solutions = True
        try:
            return self._loop([SolveRequest(req.rid, 0.0, req.side, req.young, req.poisson,
                                            req.traction)], realtime=False)[0]
        finally:
            self.keep_solutions = keep

    # ------------------------------------------------------------------ the loop
    def _request(self, req: SolveRequest):
        m = self.models[req.side]
        mu, lam = lame_from_young(req.young, req.poisson)
        b = m.f_unit * req.traction
        x = torch.empty(m.n_dofs, dtype=torch.float64, device=self.device)
        ws = torch.empty(max(m.ws_bytes, 1), dtype=torch.uint8, device=self.device)
        r = _lib.BrickRequest()
        r.nodes[:] = m.nodes
        r.h[:] = m.h
        r.mu, r.lam = float(mu), float(lam)
        r.b, r.x, r.fixed = b.data_ptr(), x.data_ptr(), m.fixed.data_ptr()
        r.workspace, r.workspace_bytes = ws.data_ptr(), m.ws_bytes
        r.rtol, r.inner_rtol = self.rtol, self.inner_rtol
        r.max_outer, r.max_inner = self.max_outer, self.max_inner
        return r, (b, x, ws)

    def _loop(self, requests, realtime: bool) -> list:
        queue = deque(sorted(requests, key=lambda r: (r.arrival, r.rid)))
        for s in set(r.side for r in queue):
            self.model(s)
        st = self.stream
        torch.cuda.synchronize(self.device)
        running: dict[int, tuple] = {}  # slot -> (request, start, need, tensors)
        used = 0
        records = []
        t0 = time.perf_counter()
        with torch.cuda.stream(st):
            while queue or running:
                now = time.perf_counter() - t0
                while (queue and len(running) < self.slots
                       and (not realtime or queue[0].arrival <= now)):
                    req = queue[0]
                    need = self.models[req.side].bytes_per_solve
                    if used + need > self.hbm_budget:
                        if not running:
                            raise ValueError(f"request {req.rid} needs {need} bytes, above the "
                                             f"HBM budget of {self.hbm_budget}")
                        break
                    queue.popleft()
                    r, tensors = self._request(req)
                    slot = self.batch.admit(r, st)
                    running[slot] = (req, now, need, tensors)
                    used += need
                if not running:
                    time.sleep(max(0.0, min(queue[0].arrival - now, 0.01)))
                    continue
                self.batch.step(self.step_iterations, st)
                states = self.batch.poll(st)
                end = time.perf_counter() - t0
                for slot in list(running):
                    sv = states[slot]
                    if sv.phase not in (_lib.TG_BRICK_DONE, _lib.TG_BRICK_FAILED):
                        continue
                    req, start, need, (b, x, ws) = running.pop(slot)
                    used -= need
                    records.append(SolveRecord(req.rid, req.side, req.arrival, start, end,
                                               int(sv.status), int(sv.iterations),
                                               int(sv.outer), float(sv.rel_res), slot,
                                               x if self.keep_solutions else None))
        records.sort(key=lambda r: r.rid)
        return records

    def run(self, requests, realtime: bool = True) -> "ServeReport":
        """Serve ``requests`` (arrival times relative to the start of the run)."""
        self.warm(r.side for r in requests)
        records = self._loop(requests, realtime)
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


__all__ = ["BrickBatch", "BrickModel", "ServeReport", "Server", "SolveRecord", "SolveRequest",
           "synthetic_requests"]
