"""Autotuner for the element-block plan (elements per block, threads per block).

``tune(energy)`` times the fused HVP of ``energy`` for every candidate plan with
CUDA events on the current stream and records the fastest configuration for the
(element type, mesh size) of its operator; ``Operator.plan()`` then uses it.
Results are kept per process (and can be saved to / loaded from JSON).
"""

from __future__ import annotations

import json

import torch

from . import _lib

_TABLE: dict = {}

DEFAULT_CANDIDATES = {
    _lib.TG_TRI3: [(1024, 4096, 128), (2048, 4096, 256), (4096, 4096, 256)],
    _lib.TG_TET4: [(1024, 4096, 64), (2048, 4096, 128), (2048, 4096, 256), (4096, 8192, 256)],
    _lib.TG_HEX8: [(512, 4096, 128), (512, 4096, 256), (1024, 4096, 128), (1024, 4096, 256),
                   (2048, 4096, 256), (4096, 8192, 256)],
}


def _key(op):
    return (op.element.tg_id, op.n_elements)


def lookup(op):
    return _TABLE.get(_key(op), (None, None, None))


def record(op, cfg) -> None:
    _TABLE[_key(op)] = tuple(cfg)


def tune(energy, dtype=torch.float32, candidates=None, reps: int = 20, warmup: int = 3):
    """Time the HVP for each candidate (block_elems, max_local_nodes, threads)."""
    op = energy.op
    cands = candidates or DEFAULT_CANDIDATES[op.element.tg_id]
    n = energy.n_dofs
    g = torch.Generator(device=op.device).manual_seed(0)
    v = torch.randn(n, dtype=dtype, device=op.device, generator=g)
    u = torch.zeros(n, dtype=dtype, device=op.device)
    results = []
    saved = energy._plan_override
    try:
        for cfg in cands:
            plan = op.plan(*cfg)
            energy.use_plan(plan)
            y = torch.empty_like(v)
            try:
                energy.apply(_lib.TG_MODE_HVP, u, v, out=y)
            except ValueError:
                continue  # infeasible (e.g. shared memory) for this law / precision
            for _ in range(warmup):
                energy.apply(_lib.TG_MODE_HVP, u, v, out=y)
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            s.record()
            for _ in range(reps):
                energy.apply(_lib.TG_MODE_HVP, u, v, out=y)
            e.record()
            torch.cuda.synchronize()
            results.append((s.elapsed_time(e) / reps, cfg, plan.stats()))
    finally:
        energy.use_plan(saved)
    if not results:
        raise RuntimeError("no feasible plan among the autotune candidates")
    results.sort(key=lambda r: r[0])
    record(op, results[0][1])
    return [dict(ms=r[0], block_elems=r[1][0], max_local_nodes=r[1][1], threads=r[1][2],
                 **{k: v for k, v in r[2].items() if k in ("n_blocks", "shared_fraction",
                                                          "max_block_colors")})
            for r in results]


def save(path: str) -> None:
    with open(path, "w") as f:
        json.dump([[list(k), list(v)] for k, v in _TABLE.items()], f)


def load(path: str) -> None:
    with open(path) as f:
        for k, v in json.load(f):
            _TABLE[tuple(k)] = tuple(v)


def tune_batch(systems, b, candidates=((128, 0), (256, 0), (512, 0), (256, 2), (512, 2)),
               **solve_kw):
    """Pick threads per CTA and CTAs per SM of ``tg_batch_solve`` by timing one full
    batched solve per candidate; the choice is stored on ``systems``."""
    bb = b.reshape(-1).to(torch.float64).contiguous()
    x = torch.empty_like(bb)
    results = []
    for threads, cps in candidates:
        systems.launch(bb, x, threads=threads, ctas_per_sm=cps, **solve_kw)  # warm
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        systems.launch(bb, x, threads=threads, ctas_per_sm=cps, **solve_kw)
        e.record()
        e.synchronize()
        results.append((s.elapsed_time(e), threads, cps))
    results.sort()
    systems.threads, systems.ctas_per_sm = results[0][1], results[0][2]
    return [dict(ms=r[0], threads=r[1], ctas_per_sm=r[2]) for r in results]
