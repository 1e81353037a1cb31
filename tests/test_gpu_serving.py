"""Request loop: continuous batching of Hex8 elasticity solves.

Each request's solution must be the same alone and in the mix -- bitwise, since the
kernels are deterministic and requests share no data -- and reach the FP64 relative
residual 1e-10.  Admission must respect the HBM budget, and requests must overlap
on the device when slots and memory allow.
"""

import pytest
import torch

from tatva_gb300 import serving

pytestmark = pytest.mark.gpu


def _overlaps(recs):
    return [(a.rid, b.rid) for i, a in enumerate(recs) for b in recs[i + 1:]
            if a.start < b.end and b.start < a.end]


def test_results_same_alone_and_in_the_mix(cuda):
    reqs = serving.synthetic_requests(10, rate=5000.0, sides=(4, 6, 8), seed=3)
    srv = serving.Server(cuda, slots=3, keep_solutions=True)
    rep = srv.run(reqs, realtime=False)
    assert len(rep.records) == 10
    assert all(r.status == 0 for r in rep.records)
    assert all(r.rel_res <= 1e-10 for r in rep.records)
    assert _overlaps(rep.records), "no two requests ran at the same time"
    alone = serving.Server(cuda, slots=1, keep_solutions=True)
    alone.warm(r.side for r in reqs)
    for req, rec in zip(reqs, rep.records):
        x, rc, stats = alone._solve(req, 0)
        assert rc == 0
        assert torch.equal(x, rec.x), req.rid
    s = rep.summary()
    assert s["converged"] == 10 and s["p99_latency_ms"] >= s["p50_latency_ms"] > 0


def test_admission_respects_the_hbm_budget(cuda):
    reqs = serving.synthetic_requests(8, rate=1e5, sides=(6, 10), seed=4)
    probe = serving.Server(cuda, slots=1)
    probe.warm([6, 10])
    need = {s: probe.models[s].bytes_per_solve for s in (6, 10)}
    budget = int(need[10] * 1.5)  # one side-10 solve at a time, never two
    srv = serving.Server(cuda, slots=4, hbm_budget=budget)
    rep = srv.run(reqs, realtime=False)
    assert all(r.status == 0 for r in rep.records)
    events = sorted([(r.start, need[r.side]) for r in rep.records]
                    + [(r.end, -need[r.side]) for r in rep.records], key=lambda t: (t[0], t[1]))
    used = 0
    for _, d in events:
        used += d
        assert used <= budget
    with pytest.raises(ValueError):
        serving.Server(cuda, slots=1, hbm_budget=need[6] // 2).warm([6])
