"""Benchmark: Hex8 linear-elastic solve to FP64 relative residual 1e-10 on a 128^3 brick.

Workload (the reference's Hex8 configuration): structured Hex8 brick 128x128x128
(2,097,152 elements, 2,146,689 nodes, 6,440,067 dofs), 2x2x2 Gauss, E = 1.0,
nu = 0.3, clamped x = 0 face, uniform normal traction 1e-3 on x = 1.

* step: one Jacobi-preconditioned CG solve of that system from x = 0 to
  ||b - A x|| <= 1e-10 ||b||, the residual evaluated in FP64.  The solve is the
  mixed-precision one of the public API (``solvers.mixed_cg``): FP32 matrix-free HVP
  and inner CG vectors, FP64 true residual, refinement update and dot products; the
  inner CG keeps its direction across the FP64 residual replacements (reliable
  updates, one per 10x reduction with the default ``--inner-rtol 0.1``).
  The L2 is flushed (256 MiB write) before every solve; the solve's own working set
  (about 280 MB of vectors) is larger than the L2 anyway.
* value: solves per second over the K timed solves (CUDA events on the solver's
  stream), summed over ranks (replicas).
* e2e: the same solve through the public API with the right-hand side copied from
  pinned host memory and the solution copied back inside the timed region.
* roofline: the solve's dominant kernel, the FP32 HVP (captured once as a CUDA graph
  and replayed with the L2 flushed before every launch): algorithmic bytes per HVP
  (x read + y written + int32 connectivity + coordinates: 2*4*N_dof + 4*8*E +
  4*3*N_nodes = 144.39 MB) over its measured time, against the measured HBM copy
  bandwidth; ``traffic`` is the HVP's DRAM bytes per launch from the committed ncu
  summary of the same kernels.
* extras: the plain FP64 Jacobi-CG solve of the same system (the reference user's
  algorithm, on the GPU), FP32 and FP64 HVP rates, the batched Poisson solve, the
  request loop and the Neo-Hookean Newton run.
* cpu_baseline: the numpy restatement (oracle) of one FP64 Jacobi-CG iteration on the
  same 128^3 system over all host cores, times the FP64 solver's iteration count.

``--impl reference`` times the same CPU restatement of the FP64 Jacobi-CG iteration
(the reference itself needs JAX, which is not installable here) on the same 128^3
system and reports solves/s = 1 / (seconds per iteration x iterations to 1e-10).
``--driver NAME`` runs one of the workload drivers that the ncu summaries under
profiles/ were taken on (see ``run_driver``).

Multi-GPU: replicas only (each rank runs the same workload on its own GPU).
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Hex8 HVP GDOF/s; solves/s & p99 latency at rel-res 1e-10, mixed vs FP64"
UNIT = "solves/s"
N_CELLS = 128
RTOL = 1e-10
# Jacobi-CG iterations that the FP64 solver needs on the clamped 128^3 brick to reach
# rel-res 1e-10 (tg_cg_solve, measured on GB300 with convergence checks every 10
# iterations).  The CPU arm runs the same FP64 algorithm, so it needs the same count;
# timing the whole CPU solve (hours) is replaced by iterations x seconds per iteration.
FP64_CG_ITERATIONS = {128: 1000}
TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "hex8_hvp_f32_brick128_traffic.md")


def workload_config(n: int) -> dict:
    """The config block both arms print (identical, so the arms can be matched)."""
    return {"workload": f"hex8 linear elasticity, structured brick {n}^3 ({n ** 3} elements, "
                        f"{3 * (n + 1) ** 3} dofs), 2x2x2 Gauss, E=1 nu=0.3, clamped x=0, "
                        "traction 1e-3 on x=1; Jacobi-CG solve to FP64 rel-res 1e-10",
            "cells_per_side": n, "dofs": 3 * (n + 1) ** 3, "rtol": RTOL}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_value(path, key):
    """``key: value`` line of a committed ncu summary, or None."""
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        import tempfile

        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clocks unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ----------------------------------------------------------------------------- CPU arm
class CpuBrickCg:
    """FP64 Jacobi-CG on the clamped n^3 brick with the oracle (numpy) HVP, the
    elements split into contiguous layers over a pool of spawned worker processes.

    The brick's elements are numbered layer by layer (k slowest), so each worker's
    element range touches one contiguous slab of nodes.  Coordinates, connectivity and
    the input vector are shared with the workers through shared memory; a worker
    returns only its slab of the product."""

    def __init__(self, n_cells: int, processes: int):
        import multiprocessing as mp

        from oracle import materials as omat
        from oracle import mesh as om

        c, e = om.brick(n_cells, n_cells, n_cells)
        nn = c.shape[0]
        self.ndof = 3 * nn
        mu, lm = omat.lame_from_young(1.0, 0.3)
        fixed = np.zeros(self.ndof, bool)
        left = np.where(c[:, 0] == 0.0)[0]
        for k in range(3):
            fixed[left * 3 + k] = True
        self.fixed = fixed
        b = np.zeros(self.ndof)
        h = 1.0 / n_cells
        right = np.where(c[:, 0] == 1.0)[0]
        jy = np.rint(c[right, 1] / h).astype(int)
        jz = np.rint(c[right, 2] / h).astype(int)
        mult = (np.where((jy == 0) | (jy == n_cells), 1, 2)
                * np.where((jz == 0) | (jz == n_cells), 1, 2))
        b[right * 3] = 1e-3 * (h * h / 4) * mult
        self.b = b
        self.processes = max(1, int(processes))
        self.shm = {}
        self.v = self._shared("v", np.zeros(self.ndof))
        self._shared("c", c)
        self._shared("e", e)
        self.tasks = []
        for ch in np.array_split(np.arange(e.shape[0]), self.processes):
            e0, e1 = int(ch[0]), int(ch[-1]) + 1
            lo, hi = int(e[e0:e1].min()), int(e[e0:e1].max()) + 1
            self.tasks.append((e0, e1, lo, hi))
        spec = {k: (m.name, a.shape, a.dtype.str) for k, (m, a) in self.shm.items()}
        self.pool = mp.get_context("spawn").Pool(self.processes, initializer=_cpu_pool_init,
                                                 initargs=(spec, mu, lm))
        # Jacobi diagonal: element tangent diagonals of the law, summed per dof
        diag = np.zeros(self.ndof)
        for (lo, part) in self.pool.map(_cpu_pool_diag, self.tasks):
            diag[3 * lo: 3 * lo + part.size] += part
        self.dinv = np.where(fixed, 1.0, 1.0 / np.where(fixed, 1.0, diag))

    def _shared(self, name, arr):
        from multiprocessing import shared_memory

        m = shared_memory.SharedMemory(create=True, size=max(arr.nbytes, 1))
        a = np.ndarray(arr.shape, dtype=arr.dtype, buffer=m.buf)
        a[...] = arr
        self.shm[name] = (m, a)
        return a

    def apply(self, p):
        """A p with the Dirichlet rows of the identity (fixed inputs read as 0)."""
        self.v[:] = np.where(self.fixed, 0.0, p)
        y = np.zeros(self.ndof)
        for (lo, part) in self.pool.map(_cpu_pool_hvp, self.tasks):
            y[3 * lo: 3 * lo + part.size] += part
        y[self.fixed] = p[self.fixed]
        return y

    def start(self):
        """CG state at x = 0: r = b, z = dinv r, p = z."""
        self.x = np.zeros(self.ndof)
        self.r = self.b.copy()
        z = self.dinv * self.r
        self.p = z
        self.rz = float(self.r @ z)

    def iteration(self):
        q = self.apply(self.p)
        alpha = self.rz / float(self.p @ q)
        self.x += alpha * self.p
        self.r -= alpha * q
        z = self.dinv * self.r
        rz = float(self.r @ z)
        self.p = z + (rz / self.rz) * self.p
        self.rz = rz

    def time_iterations(self, warmup: int, steps: int) -> float:
        self.start()
        for _ in range(warmup):
            self.iteration()
        t0 = time.perf_counter()
        for _ in range(steps):
            self.iteration()
        return (time.perf_counter() - t0) / max(steps, 1)

    def close(self):
        self.pool.close()
        self.pool.join()
        for m, _ in self.shm.values():
            m.close()
            m.unlink()
        self.shm = {}


_CPU = {}


def _cpu_pool_init(spec, mu, lm):
    from multiprocessing import shared_memory

    from oracle import materials as omat

    arrs, keep = {}, []
    for k, (name, shape, dt) in spec.items():
        m = shared_memory.SharedMemory(name=name)
        keep.append(m)
        arrs[k] = np.ndarray(shape, dtype=np.dtype(dt), buffer=m.buf)
    _CPU.update(arrs, keep=keep, law=omat.LinearElastic(mu, lm), ops={})


def _cpu_op(task):
    from oracle import elements as oe
    from oracle import operator as oop

    if task not in _CPU["ops"]:
        e0, e1, lo, hi = task
        _CPU["ops"][task] = oop.OracleOperator(_CPU["c"][lo:hi], _CPU["e"][e0:e1] - lo,
                                               oe.Hexahedron8())
    return _CPU["ops"][task]


def _cpu_pool_diag(task):
    """Diagonal of the linear-elastic element tangents, summed per dof:
    K[(a,i),(a,i)] = sum_q w detJ (mu |grad N_a|^2 + (lambda + mu) (d_i N_a)^2)."""
    op = _cpu_op(task)
    law = _CPU["law"]
    dNdX, detJ = op.geometry()  # (E,Q,3,n), (E,Q)
    w = detJ * op.qw[None, :]
    g2 = dNdX ** 2
    de = (law.mu * np.einsum("eq,eqdn->en", w, g2)[:, :, None]
          + (law.lmbda + law.mu) * np.einsum("eq,eqdn->end", w, g2))  # (E, n, 3)
    lo, hi = task[2], task[3]
    from oracle.operator import _scatter_add

    return lo, _scatter_add(op.elements, de, hi - lo).reshape(-1)


def _cpu_pool_hvp(task):
    from oracle import materials as omat

    op = _cpu_op(task)
    lo, hi = task[2], task[3]
    return lo, omat.hvp(op, _CPU["law"], None, _CPU["v"][3 * lo: 3 * hi])


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    n = args.size
    cores = os.cpu_count() or 1
    cpu = CpuBrickCg(n, cores)
    sec = cpu.time_iterations(args.warmup, args.steps)
    cpu.close()
    its = FP64_CG_ITERATIONS.get(n)
    note = ""
    if its is None:  # sizes without a measured count: the O(n) growth of Jacobi-CG
        its = int(round(FP64_CG_ITERATIONS[N_CELLS] * n / N_CELLS))
        note = " (iteration count scaled from the 128^3 measurement)"
    solve_s = sec * its
    value = 1.0 / solve_s
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": solve_s * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": workload_config(n),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"numpy restatement of FP64 Jacobi-CG on the {n}^3 brick "
                                   f"({cpu.ndof} dofs): {args.steps} timed iterations "
                                   f"(HVP over {cores} processes, vectors in the parent) at "
                                   f"{sec:.3f} s each, x {its} iterations to rel-res 1e-10"
                                   + note},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "seconds_per_iteration": sec, "iterations_per_solve": its,
        "note": "the reference (JAX) cannot be installed offline; its CPU path, "
                "jax.scipy.sparse.linalg.cg with the jax.jvp(jax.grad(E)) HVP in FP64, is "
                "represented by the numpy restatement of the same iteration",
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- GPU arm
def _hvp_timing(en, v, y, flush, steps, warmup, dev):
    """Mean CUDA-event time (ms) of one HVP replayed from a CUDA graph, the L2 flushed
    before every launch; events on the replaying stream."""
    import torch

    from tatva_gb300 import _lib

    st = torch.cuda.current_stream(dev)
    side = torch.cuda.Stream(device=dev)
    side.wait_stream(st)
    with torch.cuda.stream(side):
        en.apply(_lib.TG_MODE_HVP, None, v, out=y)
    st.wait_stream(side)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        en.apply(_lib.TG_MODE_HVP, None, v, out=y)
    for _ in range(warmup):
        flush.fill_(1.0)
        graph.replay()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(steps)]
    for i in range(steps):
        flush.fill_(float(i))
        evs[i][0].record(st)
        graph.replay()
        evs[i][1].record(st)
    torch.cuda.synchronize()
    return float(np.mean([a.elapsed_time(b) for a, b in evs])), graph


def run_ours(args):
    import torch

    from tatva_gb300 import autotune, replicas, solvers
    from tatva_gb300.problems import clamped_brick

    ws, rank, local = replicas.world()
    torch.cuda.set_device(local)
    replicas.init("nccl")
    dev = torch.device("cuda", local)
    n = args.size
    P = clamped_brick(n, dev, traction=1e-3)
    en = P["energy"]
    ndof = en.n_dofs
    tune = autotune.tune(en, dtype=torch.float32) if args.autotune else None
    if not args.autotune and args.block_elems:
        en.use_plan(P["op"].plan(args.block_elems, 4096, args.threads))
    plan = en.plan()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    b, fixed = P["b"], P["fixed"]
    sst = solvers.solver_stream(dev)
    hvp_launches = 1 if plan.grid else (2 if plan.sizes["n_shared"] > 0 else 1)

    # ---- the dominant kernel: FP32 HVP (roofline), and the FP64 HVP
    g = torch.Generator(device=dev).manual_seed(1234 + rank)
    v = torch.randn(ndof, dtype=torch.float32, device=dev, generator=g)
    y = torch.empty_like(v)
    hvp_ms, _ = _hvp_timing(en, v, y, flush, max(args.steps, 20), args.warmup, dev)
    v64, y64 = v.double(), torch.empty(ndof, dtype=torch.float64, device=dev)
    hvp64_ms, _ = _hvp_timing(en, v64, y64, flush, 5, 2, dev)

    def mixed():
        return solvers.mixed_cg(en, b, fixed=fixed, rtol=RTOL, inner_rtol=args.inner_rtol,
                                max_inner=args.max_iter, check_every=args.check_every,
                                raise_on_fail=False)

    # ---- headline: mixed-precision solves, device-timed on the solver's stream
    for _ in range(args.warmup):
        flush.fill_(1.0)
        r = mixed()
    torch.cuda.synchronize()
    replicas.barrier()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    results = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))
            evs[i][0].record(sst)
            results.append(mixed())
            evs[i][1].record(sst)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    clocks = clk.summary()
    clocks["window"] = "nvidia-smi every 200 ms over the timed solves"
    ms = [a.elapsed_time(bb) for a, bb in evs]
    replicas.barrier()
    ms_step = replicas.max_over_ranks(float(np.mean(ms)))
    value = replicas.sum_over_ranks(1.0) / (ms_step * 1e-3)
    conv = all(rr.converged and rr.rel_res <= RTOL for rr in results)
    inner = results[-1].iterations
    outer = results[-1].outer
    # launches per mixed solve: per inner iteration 3 kernels on a structured brick (the
    # HVP with p.q, the update, the direction), else the HVP plus 3 CG kernels; per
    # refinement the FP64 HVP, 3 residual/norm kernels, the scale-down, the inner
    # residual (HVP + 2 kernels, + 2 for the packed Dirichlet mask on a brick), the
    # direction (2 kernels at a restart, 3 at a reliable update) and the update; 3
    # set-up kernels, and the Jacobi diagonal
    per_inner = 3 if plan.grid else hvp_launches + 3
    resumes = max(outer - 1, 0) if args.inner_rtol >= 0.01 else 0
    launches_per_solve = (inner * per_inner + (outer + 1) * (hvp_launches + 3)
                          + outer * (hvp_launches + 6 + (2 if plan.grid else 0)) + resumes
                          + 3 + hvp_launches)

    # ---- e2e through the public API: each step's own right-hand side (the traction
    # scaled per step) from pinned host memory, its solution back to pinned host memory
    e2e_steps = max(1, min(args.steps, 5))
    b_cpu = b.cpu()
    bhs = [torch.empty(ndof, dtype=torch.float64, pin_memory=True) for _ in range(e2e_steps + 1)]
    for k, bk in enumerate(bhs):
        bk.copy_(b_cpu * (1.0 + 0.1 * k))
    xhs = [torch.empty(ndof, dtype=torch.float64, pin_memory=True) for _ in range(e2e_steps + 1)]
    cur = torch.cuda.current_stream(dev)
    e2e_res = []

    def e2e_step(k):
        bd = bhs[k].to(dev, non_blocking=True)
        rr = solvers.mixed_cg(en, bd, fixed=fixed, rtol=RTOL, inner_rtol=args.inner_rtol,
                              max_inner=args.max_iter, check_every=args.check_every,
                              raise_on_fail=False)
        xhs[k].copy_(rr.x, non_blocking=True)
        return rr

    e2e_step(e2e_steps)  # warm-up on its own input
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(cur)
    for k in range(e2e_steps):
        e2e_res.append(e2e_step(k))
    e.record(cur)
    torch.cuda.synchronize()
    e2e_ms = replicas.max_over_ranks(s.elapsed_time(e) / e2e_steps)
    e2e_value = replicas.sum_over_ranks(1.0) / (e2e_ms * 1e-3)
    e2e_converged = all(r.converged and r.rel_res <= RTOL for r in e2e_res)

    # ---- the plain FP64 solve (the reference user's algorithm) on the GPU
    fp64 = None
    if args.fp64_solves:
        solvers.cg(en, b, fixed=fixed, rtol=RTOL, maxiter=args.max_iter,
                   check_every=args.check_every, raise_on_fail=False)
        ts = []
        for _ in range(args.fp64_solves):
            flush.fill_(2.0)
            s.record(sst)
            r64 = solvers.cg(en, b, fixed=fixed, rtol=RTOL, maxiter=args.max_iter,
                             check_every=args.check_every, raise_on_fail=False)
            e.record(sst)
            torch.cuda.synchronize()
            ts.append(s.elapsed_time(e))
        fp64 = {"ms_per_solve": float(np.mean(ts)), "solves_per_s": 1e3 / float(np.mean(ts)),
                "iterations": r64.iterations, "rel_res": r64.rel_res,
                "converged": r64.converged, "dtype": "f64",
                "mixed_speedup": float(np.mean(ts)) / ms_step}

    # ---- roofline of the HVP
    nn, ne = P["n_nodes"], P["n_elems"]
    alg_bytes = 2 * 4 * ndof + 4 * 8 * ne + 4 * 3 * nn
    peak, peak_kind = _peaks()
    achieved = alg_bytes / (hvp_ms * 1e-3) / 1e9
    traffic = _profile_value(TRAFFIC_PROFILE, "traffic_bytes_per_hvp_128") if n == N_CELLS else None
    replicas.barrier()
    if rank != 0:
        return

    cpu = None
    if not args.no_cpu_baseline:
        its = fp64["iterations"] if fp64 else FP64_CG_ITERATIONS.get(n, 1000)
        cores = os.cpu_count() or 1
        cb = CpuBrickCg(n, cores)
        sec = cb.time_iterations(1, args.cpu_iterations)
        cb.close()
        cpu = {"value": 1.0 / (sec * its), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"numpy restatement of FP64 Jacobi-CG on the same {n}^3 system: "
                         f"{args.cpu_iterations} iterations (HVP over {cores} processes) at "
                         f"{sec:.3f} s each, x {its} iterations (the FP64 solver's count)"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "precision": "FP32 HVP and inner CG vectors; FP64 true residual, refinement update "
                     "and every dot product; each solve stops at FP64 rel-res <= 1e-10",
        "inner_rtol": args.inner_rtol,
        "data": "synthetic", "config": workload_config(n),
        "l2": "flushed before every solve (256 MiB write); solve working set > L2",
        "converged": conv, "rel_res": results[-1].rel_res, "inner_iterations": inner,
        "refinements": outer,
        "gpu_launches": args.steps * launches_per_solve,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": ndof * 8,
                "d2h_bytes_per_step": ndof * 8, "ms_per_step": e2e_ms,
                "inputs": f"{e2e_steps} distinct right-hand sides (traction x 1.0 .. "
                          f"{1.0 + 0.1 * (e2e_steps - 1):.1f}), each its own pinned buffer",
                "converged": e2e_converged},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "kernel": "FP32 HVP",
                     "ms": hvp_ms, "peak_source": peak_kind, "algorithmic_bytes": alg_bytes},
        "clocks": clocks,
        "cpu_baseline": cpu,
        "fp64_solve": fp64,
        "hvp": {"f32_ms": hvp_ms, "f32_gdof_s": ndof / (hvp_ms * 1e-3) / 1e9,
                "f64_ms": hvp64_ms, "f64_gdof_s": ndof / (hvp64_ms * 1e-3) / 1e9,
                "launches_per_hvp": hvp_launches},
        "plan": {k: plan.stats()[k] for k in ("grid", "block_elems", "threads", "n_blocks",
                                              "shared_fraction", "n_lattice_blocks")},
        "wall_s_timed_region": wall,
    }
    if tune:
        line["autotune"] = tune
    if args.kernels:
        line["maps"] = bench_maps(P, dev)
    if args.batched:
        line["batched"] = bench_batched(dev, args)
    if args.serving:
        line["serving"] = bench_serving(dev, args)
    if args.newton:
        line["newton"] = bench_newton(dev, args)
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- extras
def _time_ms(fn, reps=5, warm=2):
    """Mean CUDA-event time (ms) of fn() on the current stream, after warm-up calls."""
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def _roofline(nbytes, ms, what):
    peak, kind = _peaks()
    gbs = nbytes / (ms * 1e-3) / 1e9
    return {"ms": ms, "algorithmic_bytes": int(nbytes), "achieved_gbs": gbs, "peak_gbs": peak,
            "frac": gbs / peak, "peak_source": kind, "bytes": what}


def bench_maps(P, dev):
    """Operator.grad and its transpose (the reverse-mode gather / scatter of
    tatva/operator.py:194-223, 379-397) in FP64 on the 128^3 brick: every (element,
    quadrature point) gradient materialised, as the reference does."""
    import torch

    op = P["op"]
    E, N = P["n_elems"], P["n_nodes"]
    u = torch.randn((N, 3), dtype=torch.float64, device=dev)
    g = op._grad_raw(u)
    out = {}
    ms = _time_ms(lambda: op._grad_raw(u))
    out["grad_f64"] = _roofline(4 * 8 * E + 8 * 3 * N * 2 + 8 * 72 * E, ms,
                                "int32 connectivity, FP64 coordinates and nodal values in, "
                                "FP64 (E, 8, 3, 3) gradients out")
    ms = _time_ms(lambda: op._grad_t_raw(g, (3,)))
    out["grad_transpose_f64"] = _roofline(8 * 72 * E + 4 * 8 * E + 8 * 3 * N * 2 + 4 * (N + 1 + 8 * E),
                                          ms, "FP64 (E, 8, 3, 3) flux, connectivity, coordinates and "
                                              "node incidence in, FP64 nodal values out")
    del g
    return out


def bench_c3_kernels(P, en, cm, dev):
    """The Neo-Hookean configuration's kernels at Kuhn 96^3: the general-path FP32 HVP,
    the FP32 colored compressed Hessian (sparse/base.py:230-270), its decompression
    (base.py:173) and the node-block SpMV of the CG on the tangent."""
    import torch

    from tatva_gb300 import _lib, sparse, solvers
    from tatva_gb300._device import ptr, stream

    N, E = P["n_nodes"], P["n_elems"]
    nd = en.n_dofs
    g = torch.Generator(device=dev).manual_seed(3)
    u = (1e-3 * torch.randn(nd, generator=g, device=dev, dtype=torch.float64)).float()
    v = torch.randn(nd, generator=g, device=dev, dtype=torch.float64).float()
    out = {}
    ms = _time_ms(lambda: en.hvp(u, v))
    out["hvp_nh_f32"] = _roofline(3 * 4 * nd + 4 * 4 * E + 4 * 3 * N, ms,
                                  "u and v read, y written (FP32), int32 connectivity, "
                                  "FP32 coordinates")
    C = cm.n_colors
    ms = _time_ms(lambda: en.compressed_hessian(u, cm.colors, C), reps=3, warm=1)
    out["compressed_hessian_f32"] = _roofline(4 * nd * C + 4 * nd + 4 * 4 * E + 4 * 3 * N + 4 * nd, ms,
                                              "Jc (n_dofs x colours) written, u, colours, "
                                              "connectivity, coordinates read")
    Jc = en.compressed_hessian(u, cm.colors, C)
    rows, cols = sparse.compute_rows_cols(cm)
    ms = _time_ms(lambda: sparse.decompress(Jc, rows, cols), reps=3, warm=1)
    out["decompress_f32"] = _roofline(16 * cm.nnz, ms, "rows, colour of the column, one Jc "
                                                       "value read and one value written per entry")
    del Jc, rows, cols
    data = torch.randn(cm.nnz, generator=g, device=dev, dtype=torch.float32)
    blocks = solvers.node_blocks3(cm)
    y = torch.empty_like(v)
    if blocks is not None:
        nptr, nidx = blocks
        ms = _time_ms(lambda: _lib.call("tg_spmv_blocks3", _lib.TG_F32, nd, ptr(cm.indptr),
                                        ptr(nptr), ptr(nidx), ptr(data), ptr(v), ptr(y),
                                        stream()))
        out["spmv_blocks3_f32"] = _roofline(4 * cm.nnz + 4 * nidx.numel() + 4 * (nptr.numel() + nd + 1)
                                            + 2 * 4 * nd, ms,
                                            "FP32 values, one neighbour id per 3 x 3 block, "
                                            "row and block pointers, x read and y written")
    out["nnz"], out["n_colors"] = cm.nnz, C
    return out


BATCH_TRAFFIC_PROFILE = os.path.join(ROOT, "profiles", "batch_solve_poisson_4096.md")


def bench_batched(dev, args):
    """Batched Tri3 Poisson: 4096 unit squares, side log-uniform in [8, 96], lognormal(0, 1)
    conductivity per element, f = 1, zero Dirichlet; one persistent launch per solve
    (CUDA graph), FP32 CG + FP64 refinement to rel-res 1e-10 per mesh."""
    import torch

    from tatva_gb300 import autotune, batched

    t0 = time.perf_counter()
    meshes, kappas, sides = batched.random_unit_squares(args.batched, seed=0)
    sysm, b, info = batched.poisson_batch(meshes, kappas, device=dev)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    tune = autotune.tune_batch(sysm, b)
    x = torch.empty_like(b)
    g = sysm.capture(b, x)
    g.replay()
    torch.cuda.synchronize()
    ms = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        g.replay()
        e1.record()
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    r = sysm.result(x)
    t = float(np.median(ms)) * 1e-3
    alg = float(np.sum(r.iterations.astype(np.float64) * sysm.sizes * (6.0 * sysm.width + 36.0)))
    peak, kind = _peaks()
    out = {"workload": f"{len(meshes)} Tri3 unit squares, n log-uniform in [8,96], kappa "
                       "lognormal(0,1) per element, f=1, zero Dirichlet, rel-res 1e-10",
           "rows": info["n_rows"], "elements": info["n_elements"], "nnz": info["nnz"],
           "solves_per_s": len(meshes) / t, "ms_per_batch": t * 1e3, "setup_s": setup_s,
           "converged": int(np.sum(r.status == 0)), "max_rel_res": float(r.rel_res.max()),
           "mean_inner_iterations": float(r.iterations.mean()),
           "max_inner_iterations": int(r.iterations.max()),
           "mean_refinements": float(r.refinements.mean()),
           "threads": sysm.threads, "ctas_per_sm": sysm.ctas_per_sm, "autotune": tune,
           "gpu_launches_per_batch": 1}
    # DRAM bytes of one batched launch (ncu, committed summary) over the measured time:
    # the HBM fraction.  The inner-iteration byte count is mostly served by the L2
    # (systems in flight fit in it) and is reported separately as an L2-inclusive rate.
    dram = _profile_value(BATCH_TRAFFIC_PROFILE, f"dram_bytes_per_batch_{len(meshes)}")
    rf = {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": kind,
          "l2_inclusive_gbs": alg / t / 1e9, "l2_inclusive_bytes": alg,
          "note": "achieved = DRAM bytes of one launch (ncu) / measured time; "
                  "l2_inclusive counts 6 B per ELL entry + 36 B of vector traffic per row "
                  "and inner iteration, most of it served by the L2"}
    if dram:
        rf.update(achieved=dram / t / 1e9, frac=dram / t / 1e9 / peak, traffic=dram)
    out["roofline"] = rf
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = _cpu_batched_sample(meshes, kappas, args.cpu_seconds)
    return out


def _cpu_batched_sample(meshes, kappas, budget_s):
    import scipy.sparse as sps

    from oracle import elements as oe
    from oracle import materials as omat
    from oracle import operator as oop
    from oracle import solvers as osol
    from oracle import sparse as osp
    from tatva_gb300.batched import boundary_nodes_tri3

    done, spent, wall0 = 0, 0.0, time.perf_counter()
    for (c, e), k in zip(meshes, kappas):
        op = oop.OracleOperator(c, e, oe.Tri3())
        law = omat.Poisson(k, 1.0)
        Ke = omat.element_tangents(op, law, np.zeros(c.shape[0]))
        pat = osp.pattern_from_mesh(c, e, 1)
        data = omat.assemble_csr_data(op, Ke, 1, pat.indptr, pat.indices)
        K = sps.csr_matrix((data, pat.indices, pat.indptr), shape=(c.shape[0],) * 2)
        fixed = boundary_nodes_tri3(e, c.shape[0])
        free = np.where(~fixed)[0]
        Kf = K[free][:, free].tocsr()
        b = -omat.residual(op, law, np.zeros(c.shape[0]))[free]
        t0 = time.perf_counter()
        osol.jacobi_cg(lambda z: Kf @ z, b, Kf.diagonal(), rtol=1e-10)
        spent += time.perf_counter() - t0
        done += 1
        if spent >= budget_s or time.perf_counter() - wall0 >= 2 * budget_s:
            break
    return {"value": done / spent, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"first {done} meshes of the same seeded batch, numpy/scipy FP64 "
                      "Jacobi-CG to rel-res 1e-10 (assembly not timed)"}


def bench_serving(dev, args):
    """Request loop: Poisson arrivals (mean 2000/s) of Hex8 linear-elastic solves on
    bricks of side in {16,24,32,48,64}; E lognormal(0,0.5), nu U[0.2,0.45], traction
    U[0.5,1.5]e-3; mixed-precision solve to rel-res 1e-10."""
    from tatva_gb300 import serving

    reqs = serving.synthetic_requests(args.serving, rate=2000.0, seed=0)
    srv = serving.Server(dev, slots=args.slots, hbm_budget=args.hbm_budget << 30,
                         step_iterations=args.step_iterations)
    rep = srv.run(reqs, realtime=True)
    out = {"workload": f"{len(reqs)} requests, Poisson arrivals mean 2000/s, Hex8 LE bricks "
                       "side in {16,24,32,48,64}, mixed precision to rel-res 1e-10"}
    out.update(rep.summary())
    # the offered load above is far beyond one GPU's capacity, so its latencies are
    # queueing; the same mix at ~80 % of the measured capacity shows the service-bound
    # latencies
    rate = 0.8 * out["solves_per_s"]
    reqs2 = serving.synthetic_requests(max(40, args.serving // 2), rate=rate, seed=1)
    rep2 = srv.run(reqs2, realtime=True)
    out["at_80pct_capacity"] = dict(rep2.summary(), rate_per_s=rate)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = _cpu_serving_sample()
    return out


def _cpu_serving_sample():
    from oracle import elements as oe
    from oracle import materials as omat
    from oracle import operator as oop
    from oracle import solvers as osol
    from tatva_gb300.problems import clamped_brick

    P = clamped_brick(16, "cpu", traction=1e-3)
    c, e = P["mesh"].coords_host(), P["mesh"].elements_host()
    op = oop.OracleOperator(c, e, oe.Hexahedron8())
    mu, lm = omat.lame_from_young(1.0, 0.3)
    law = omat.LinearElastic(mu, lm)
    fixed = P["fixed"].numpy().astype(bool)
    b = np.where(fixed, 0.0, P["b"].numpy())

    def apply(z):
        zz = np.where(fixed, 0.0, z)
        y = omat.hvp(op, law, None, zz)
        return np.where(fixed, z, y)

    cols = np.zeros_like(b)
    ndof = b.size
    # Jacobi diagonal from unit probes of the element tangents
    Ke = omat.element_tangents(op, law, np.zeros(ndof))
    dofs = (e[:, :, None] * 3 + np.arange(3)).reshape(e.shape[0], -1)
    np.add.at(cols, dofs.ravel(), np.einsum("eii->ei", Ke).ravel())
    diag = np.where(fixed, 1.0, cols)
    t0 = time.perf_counter()
    osol.jacobi_cg(apply, b, diag, rtol=1e-10)
    dt = time.perf_counter() - t0
    return {"value": 1.0 / dt, "unit": "solves/s", "cores": 1, "kind": "port",
            "sample": f"one side-16 request (E=1, nu=0.3; {ndof} dofs), numpy FP64 matrix-free "
                      f"Jacobi-CG to rel-res 1e-10, {dt:.1f} s"}


def bench_newton(dev, args):
    """Neo-Hookean Tet4 (Kuhn split of n^3 cells, interior jitter +-0.2h, mu=1, lambda=10),
    20% uniaxial stretch in load steps; Newton with FP64 residual/update and the FP32
    colored sparse tangent, CSR CG inner solves (Eisenstat-Walker tolerances)."""
    import torch

    from tatva_gb300 import sparse, solvers
    from tatva_gb300.lifter import Fixed, Lifter
    from tatva_gb300.problems import stretched_kuhn

    n, steps = args.newton, args.newton_steps
    t0 = time.perf_counter()
    P = stretched_kuhn(n, dev)
    en, c = P["energy"], P["coords"]
    cm = sparse.ColoredMatrix.from_csr(sparse.pattern_from_mesh(P["mesh"], 3), device=dev)
    def load_step(step, u):
        """One load step: exact lift of the affine predictor, then Newton to 1e-10."""
        lifter = Lifter(en.n_dofs, Fixed(P["dofs"], P["values"](0.2 * step / steps)))
        du = torch.zeros_like(u)
        du.view(-1, 3)[:, 0] = torch.as_tensor(c[:, 0] * (0.2 / steps), device=dev)
        u = lifter.lift(lifter.reduce(u + du), u + du)  # affine predictor, exact lift
        return solvers.newton(en, u, lifter, colored_matrix=cm, rtol=1e-10, max_iter=30)

    # warm-up, untimed: the whole first load step from u = 0, exactly as the timed loop
    # runs it (builds the element plan and loads every kernel the loop uses -- torch's
    # and this library's kernels are loaded on first use, seconds after other large
    # work in the process); the timed run then starts again from u = 0
    load_step(1, torch.zeros(en.n_dofs, dtype=torch.float64, device=dev))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    u = torch.zeros(en.n_dofs, dtype=torch.float64, device=dev)
    hist, newton_its, cg_its = [], 0, 0
    t1 = time.perf_counter()
    for step in range(1, steps + 1):
        ts = time.perf_counter()
        res = load_step(step, u)
        torch.cuda.synchronize()
        hist.append({"step": step, "newton": res.outer, "cg": res.iterations,
                     "rel_res": res.rel_res, "converged": res.converged,
                     "seconds": time.perf_counter() - ts})
        newton_its += res.outer
        cg_its += res.iterations
        u = res.x
        if not res.converged:
            break
    total = time.perf_counter() - t1
    out = {"workload": f"Neo-Hookean Tet4, Kuhn {n}^3 ({P['n_elems']} tets, {en.n_dofs} dofs), "
                       f"jitter 0.2h, 20% stretch in {steps} load steps, rel-res 1e-10 per step",
           "seconds": total, "setup_s": setup_s, "newton_iterations": newton_its,
           "cg_iterations": cg_its, "nnz": cm.nnz, "n_colors": cm.n_colors,
           "converged_steps": sum(1 for h in hist if h["converged"]),
           "dof_newton_iterations_per_s": en.n_dofs * newton_its / total, "steps": hist}
    if args.kernels:
        out["kernels"] = bench_c3_kernels(P, en, cm, dev)
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = _cpu_newton_sample()
    return out


def _cpu_newton_sample(n=10):
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla

    from oracle import elements as oe
    from oracle import materials as omat
    from oracle import operator as oop
    from oracle import sparse as osp
    from tatva_gb300.problems import stretched_kuhn

    P = stretched_kuhn(n, "cpu")
    c, e = P["coords"], P["mesh"].elements_host()
    op = oop.OracleOperator(c, e, oe.Tetrahedron4())
    law = omat.NeoHookean(1.0, 10.0)
    pat = osp.pattern_from_mesh(c, e, 3)
    nd = c.shape[0] * 3
    dofs = P["dofs"]
    free = np.setdiff1d(np.arange(nd), dofs)
    u = np.zeros(nd)
    u[0::3] = c[:, 0] * 0.02
    u[dofs] = P["values"](0.02)
    its, t0 = 0, time.perf_counter()
    r0 = None
    for _ in range(30):
        r = omat.residual(op, law, u)[free]
        rn = np.linalg.norm(r)
        r0 = rn if r0 is None else r0
        if rn <= 1e-10 * r0:
            break
        Ke = omat.element_tangents(op, law, u)
        data = omat.assemble_csr_data(op, Ke, 3, pat.indptr, pat.indices)
        K = sps.csr_matrix((data, pat.indices, pat.indptr), shape=(nd, nd))[free][:, free]
        u[free] -= spla.spsolve(K.tocsc(), r)
        its += 1
    dt = time.perf_counter() - t0
    return {"value": nd * its / dt, "unit": "dof-Newton-iterations/s", "cores": 1, "kind": "port",
            "sample": f"one 2% load step on a Kuhn {n}^3 block ({nd} dofs): {its} Newton "
                      f"iterations, numpy element tangents + scipy sparse direct solve, {dt:.1f} s"}


# ----------------------------------------------------------------------------- drivers
def run_driver(args):
    """Workload drivers that the ncu summaries under profiles/ were captured on:

    * ``brick`` / ``kuhn`` / ``kuhn-le``: ``--repeats`` fused HVPs (``--prec``) of the
      clamped brick (``--size`` cells per side), the Neo-Hookean Kuhn block, or the same
      Kuhn mesh with the linear-elastic law;
    * ``brick-cg``: ``--repeats`` Jacobi-CG iterations on the clamped brick;
    * ``mixed``: ``--repeats`` mixed-precision solves of the clamped brick to rel-res
      1e-10 (the headline's solve);
    * ``batch``: the seeded random unit-square batch of ``--batched`` meshes, solved
      ``--repeats`` times;
    * ``serve``: ``--slots`` requests of the seeded serving mix admitted into one brick
      batch, then ``--repeats`` steps of ``--step-iterations`` CG steps (all in flight);
    * ``kernels``: the map kernels on the brick of ``--size`` cells and the Neo-Hookean
      kernels (HVP, compressed Hessian, decompression, node-block SpMV) on the Kuhn
      block of ``--newton`` cells, as the bench's roofline legs run them."""
    import torch

    from tatva_gb300 import _lib, solvers
    from tatva_gb300.materials import LinearElastic
    from tatva_gb300.problems import clamped_brick, stretched_kuhn

    dtype = torch.float64 if args.prec == "f64" else torch.float32
    name, n, reps = args.driver, args.size, args.repeats
    if name == "batch":
        from tatva_gb300 import batched

        meshes, kappas, _ = batched.random_unit_squares(args.batched, seed=0)
        systems, b, info = batched.poisson_batch(meshes, kappas, device="cuda")
        res = None
        for _ in range(reps):
            res = systems.solve(b)
        print(dict(info, converged=res.converged, max_rel_res=float(res.rel_res.max()),
                   seconds=res.seconds))
        return
    if name == "kernels":
        from tatva_gb300 import sparse

        Pb = clamped_brick(n, "cuda")
        maps = bench_maps(Pb, torch.device("cuda"))
        del Pb
        Pk = stretched_kuhn(args.newton, "cuda")
        cm = sparse.ColoredMatrix.from_csr(sparse.pattern_from_mesh(Pk["mesh"], 3), device="cuda")
        ker = bench_c3_kernels(Pk, Pk["energy"], cm, torch.device("cuda"))
        print(json.dumps({"maps": maps, "kernels": ker}))
        return
    if name == "serve":
        from tatva_gb300 import serving

        srv = serving.Server("cuda", slots=args.slots, hbm_budget=64 << 30,
                             step_iterations=args.step_iterations)
        reqs = serving.synthetic_requests(args.slots, seed=0)
        keep = []
        st = srv.stream
        with torch.cuda.stream(st):
            for rq in reqs:
                srv.model(rq.side)
                r, t = srv._request(rq)
                srv.batch.admit(r, st)
                keep.append(t)
            srv.batch.step(args.step_iterations, st)  # admission, first refinement, warm-up
            srv.batch.poll(st)
            t0 = time.perf_counter()
            for _ in range(reps):
                srv.batch.step(args.step_iterations, st)
            states = srv.batch.poll(st)
            dt = time.perf_counter() - t0
        dofs = sum(srv.models[r.side].n_dofs for r in reqs)
        running = sum(1 for s in states if s.phase == _lib.TG_BRICK_RUN)
        its = reps * args.step_iterations
        print(json.dumps({"driver": "serve", "requests": len(reqs), "dofs_in_flight": dofs,
                          "running_at_end": running, "iterations": its,
                          "us_per_iteration": 1e6 * dt / its,
                          "ns_per_dof_iteration": 1e9 * dt / its / dofs}))
        return
    if name == "mixed":
        P = clamped_brick(n, "cuda")
        for _ in range(reps):
            r = solvers.mixed_cg(P["energy"], P["b"], fixed=P["fixed"], rtol=RTOL,
                                 inner_rtol=args.inner_rtol, check_every=args.check_every)
        torch.cuda.synchronize()
        print(json.dumps({"driver": "mixed", "dofs": P["energy"].n_dofs,
                          "inner_iterations": r.iterations, "refinements": r.outer,
                          "rel_res": r.rel_res}))
        return
    if name == "brick-cg":
        P = clamped_brick(n, "cuda")
        bb = P["b"].to(dtype)
        solvers.cg(P["energy"], bb, fixed=P["fixed"], dtype=dtype, rtol=1e-30, maxiter=reps,
                   check_every=min(reps, 50), raise_on_fail=False)  # warm-up, graph build
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = solvers.cg(P["energy"], bb, fixed=P["fixed"], dtype=dtype, rtol=1e-30,
                       maxiter=reps, check_every=min(reps, 50), raise_on_fail=False)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        print(name, n, P["energy"].n_dofs, r.iterations,
              f"{1e6 * dt / max(r.iterations, 1):.1f} us/it")
        return
    if name == "brick":
        P = clamped_brick(n, "cuda")
        en, u = P["energy"], None
    elif name in ("kuhn", "kuhn-le"):
        P = stretched_kuhn(n, "cuda")
        en = P["energy"] if name == "kuhn" else LinearElastic(P["op"], 1.0, 1.0)
        u = None if name != "kuhn" else torch.zeros(en.n_dofs, dtype=dtype, device="cuda")
    else:
        raise SystemExit(f"unknown driver {name}")
    v = torch.ones(en.n_dofs, dtype=dtype, device="cuda")
    y = torch.empty_like(v)
    for _ in range(reps):
        en.apply(_lib.TG_MODE_HVP, u, v, out=y)
    torch.cuda.synchronize()
    print(name, n, en.n_dofs, float(y.abs().sum()))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10, help="timed solves")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=N_CELLS)
    ap.add_argument("--autotune", type=int, default=1)
    ap.add_argument("--block-elems", type=int, default=0, help="plan when --autotune 0")
    ap.add_argument("--threads", type=int, default=256, help="plan when --autotune 0")
    ap.add_argument("--max-iter", type=int, default=20000)
    ap.add_argument("--inner-rtol", type=float, default=0.1,
                    help="mixed solve: FP32 reduction between FP64 residual replacements")
    ap.add_argument("--check-every", type=int, default=50)
    ap.add_argument("--fp64-solves", type=int, default=2, help="timed FP64 solves (0: skip)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--cpu-iterations", type=int, default=2)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batched", type=int, default=4096, help="meshes in the batched solve (0: skip)")
    ap.add_argument("--serving", type=int, default=400, help="requests in the serving run (0: skip)")
    ap.add_argument("--slots", type=int, default=64, help="serving: solves in flight (<= 64)")
    ap.add_argument("--step-iterations", type=int, default=20,
                    help="serving: CG steps of the batch between two polls")
    ap.add_argument("--newton", type=int, default=96, help="Kuhn cells per side (0: skip)")
    ap.add_argument("--newton-steps", type=int, default=10)
    ap.add_argument("--hbm-budget", type=int, default=32, help="serving HBM budget, GiB")
    ap.add_argument("--kernels", type=int, default=1,
                    help="time the map, Hessian and SpMV kernels beside the solve (0: skip)")
    ap.add_argument("--driver", default="", help="run a profiling workload driver instead")
    ap.add_argument("--repeats", type=int, default=3, help="driver repetitions")
    ap.add_argument("--prec", default="f32", choices=["f32", "f64"], help="driver precision")
    args = ap.parse_args()
    if args.driver:
        run_driver(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
