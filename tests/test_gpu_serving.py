"""Request loop and the brick batch engine it runs on (continuous batching of
Hex8 elasticity solves).

Each request's solution must be the same alone and in the mix -- bitwise, since the
kernels are deterministic and requests share no data -- and reach the FP64 relative
residual 1e-10, checked against the oracle's FP64 operator (<= 2e-10: the engine's
own residual is the GPU stencil's, equal to the oracle's to ~1e-15 relative).
Admission must respect the HBM budget, and requests must overlap on the device when
slots and memory allow.  The engine's state machine is checked on bricks of uneven
axes and spacings against the single-solve mixed-precision CG (same system, solution
to 1e-8), and its refinement budget reports NOT_CONVERGED when spent.
"""

import ctypes

import numpy as np
import pytest
import torch

from oracle import elements as oe
from oracle import materials as omat
from oracle import mesh as om
from oracle import operator as oop
from tatva_gb300 import Mesh, Operator, _lib, element, materials, serving, solvers
from tatva_gb300.problems import clamped_brick

pytestmark = pytest.mark.gpu


def _overlaps(recs):
    return [(a.rid, b.rid) for i, a in enumerate(recs) for b in recs[i + 1:]
            if a.start < b.end and b.start < a.end]


def _oracle_rel_res(req, x):
    P = clamped_brick(req.side, "cpu", traction=1.0)
    c, e = P["mesh"].coords_host(), P["mesh"].elements_host()
    op = oop.OracleOperator(c, e, oe.Hexahedron8())
    law = omat.LinearElastic(*omat.lame_from_young(req.young, req.poisson))
    fixed = P["fixed"].numpy().astype(bool)
    b = P["b"].numpy() * req.traction
    xv = x.cpu().numpy()
    y = omat.hvp(op, law, None, np.where(fixed, 0.0, xv))
    y[fixed] = xv[fixed]
    return float(np.linalg.norm(b - y) / np.linalg.norm(b))


def test_results_same_alone_and_in_the_mix(cuda):
    reqs = serving.synthetic_requests(10, rate=5000.0, sides=(4, 6, 8), seed=3)
    srv = serving.Server(cuda, slots=3, keep_solutions=True, step_iterations=7)
    rep = srv.run(reqs, realtime=False)
    assert len(rep.records) == 10
    assert all(r.status == 0 for r in rep.records)
    assert all(r.rel_res <= 1e-10 for r in rep.records)
    assert _overlaps(rep.records), "no two requests ran at the same time"
    alone = serving.Server(cuda, slots=1, keep_solutions=True, step_iterations=7)
    alone.warm(r.side for r in reqs)
    for req, rec in zip(reqs, rep.records):
        a = alone.solve_alone(req)
        assert a.status == 0
        assert torch.equal(a.x, rec.x), req.rid
        assert a.iterations == rec.iterations and a.refinements == rec.refinements
    for req, rec in list(zip(reqs, rep.records))[:4]:
        assert _oracle_rel_res(req, rec.x) <= 2e-10, req.rid
    s = rep.summary()
    assert s["converged"] == 10 and s["p99_latency_ms"] >= s["p50_latency_ms"] > 0


def test_the_step_length_does_not_change_results(cuda):
    """A request's bits do not depend on how many CG steps run between polls."""
    reqs = serving.synthetic_requests(5, rate=1e5, sides=(5, 7), seed=9)
    out = []
    for k in (1, 13):
        srv = serving.Server(cuda, slots=4, keep_solutions=True, step_iterations=k)
        out.append(srv.run(reqs, realtime=False).records)
    for a, b in zip(*out):
        assert torch.equal(a.x, b.x) and a.iterations == b.iterations


def test_admission_respects_the_hbm_budget(cuda):
    reqs = serving.synthetic_requests(8, rate=1e5, sides=(6, 10), seed=4)
    probe = serving.Server(cuda, slots=1)
    need = {s: probe.model(s).bytes_per_solve for s in (6, 10)}
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


def _brick_problem(cuda, shape, lengths, young, nu, seed):
    c, e = om.brick(*shape, lengths=lengths)
    op = Operator(Mesh(c, e, device=cuda), element.Hexahedron8())
    en = materials.LinearElastic.from_young(op, young, nu)
    plan = en.plan()
    assert plan.grid
    n = en.n_dofs
    fixed = np.zeros(n, np.uint8)
    fixed.reshape(-1, 3)[c[:, 0] == c[:, 0].min()] = 1
    fixed[np.random.default_rng(seed).random(n) < 0.05] = 1  # scattered single dofs too
    b = np.random.default_rng(seed + 1).standard_normal(n) * 1e-3
    b[fixed == 1] = 0.0
    return en, plan, torch.as_tensor(fixed, device=cuda), torch.as_tensor(b, device=cuda)


def _engine_solve(cuda, items, max_outer=50, inner_rtol=1e-4, step=11):
    """Admit all items into one batch and step until every slot is finished."""
    bt = serving.BrickBatch(cuda)
    st = torch.cuda.Stream(device=cuda)
    keep, slots = [], []
    with torch.cuda.stream(st):
        for en, plan, fixed, b in items:
            x = torch.empty_like(b)
            nodes = (ctypes.c_int32 * 3)(*plan.grid_nodes)
            wsb = int(_lib.lib().tg_brick_workspace_bytes(nodes))
            ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
            r = _lib.BrickRequest()
            r.nodes[:] = plan.grid_nodes
            r.h[:] = plan.grid_h
            r.mu, r.lam = en.p0, en.p1
            r.b, r.x, r.fixed = b.data_ptr(), x.data_ptr(), fixed.data_ptr()
            r.workspace, r.workspace_bytes = ws.data_ptr(), wsb
            r.rtol, r.inner_rtol, r.max_outer, r.max_inner = 1e-10, inner_rtol, max_outer, 100000
            slots.append(bt.admit(r, st))
            keep.append((x, ws))
        done = {}
        for _ in range(100000):
            bt.step(step, st)
            states = bt.poll(st)
            for s in slots:
                if s not in done and states[s].phase in (_lib.TG_BRICK_DONE, _lib.TG_BRICK_FAILED):
                    sv = states[s]
                    done[s] = (sv.status, sv.iterations, sv.outer, sv.rel_res)
            if len(done) == len(slots):
                break
    bt.close()
    return [(keep[i][0], done[s]) for i, s in enumerate(slots)]


def test_engine_on_uneven_bricks_matches_the_mixed_solver(cuda):
    items = [_brick_problem(cuda, (9, 5, 7), (1.8, 0.5, 1.4), 1.3, 0.25, 0),
             _brick_problem(cuda, (33, 9, 17), (1.0, 0.3, 0.5), 0.7, 0.4, 1),
             _brick_problem(cuda, (2, 3, 4), (0.5, 0.9, 1.3), 2.0, 0.3, 2)]
    res = _engine_solve(cuda, items)
    for (en, plan, fixed, b), (x, (status, its, outer, rr)) in zip(items, res):
        assert status == _lib.TG_OK and rr <= 1e-10 and outer >= 1
        ref = solvers.mixed_cg(en, b, fixed=fixed, rtol=1e-10)
        assert ref.converged
        err = float((x - ref.x).abs().max() / ref.x.abs().max())
        assert err < 1e-8, err
        assert torch.all(x[fixed.bool()] == 0)


def test_engine_reports_a_spent_refinement_budget(cuda):
    items = [_brick_problem(cuda, (9, 5, 7), (1.8, 0.5, 1.4), 1.3, 0.25, 0)]
    [(x, (status, its, outer, rr))] = _engine_solve(cuda, items, max_outer=1)
    assert status == _lib.TG_ERR_NOT_CONVERGED and outer == 1 and 1e-10 < rr < 1e-2


def test_engine_rejects_bad_admissions_and_a_full_batch(cuda):
    """Host-side checks of the C ABI: workspace size and alignment, brick size, a full
    batch (64 slots), and the poll buffer length; the batch stays usable after each."""
    bt = serving.BrickBatch(cuda)
    st = torch.cuda.Stream(device=cuda)
    nodes = (3, 3, 3)
    wsb = int(_lib.lib().tg_brick_workspace_bytes((ctypes.c_int32 * 3)(*nodes)))
    n = 3 * 27
    b = torch.zeros(n, dtype=torch.float64, device=cuda)
    keep = []

    def req(ws_bytes=wsb, offset=0, nd=nodes):
        x = torch.empty(n, dtype=torch.float64, device=cuda)
        ws = torch.empty(wsb + 512, dtype=torch.uint8, device=cuda)
        keep.append((x, ws))
        r = _lib.BrickRequest()
        r.nodes[:] = nd
        r.h[:] = (0.5, 0.5, 0.5)
        r.mu, r.lam = 1.0, 1.0
        r.b, r.x, r.fixed = b.data_ptr(), x.data_ptr(), None
        r.workspace, r.workspace_bytes = ws.data_ptr() + offset, ws_bytes
        r.rtol, r.inner_rtol, r.max_outer, r.max_inner = 1e-10, 1e-4, 10, 1000
        return r

    with torch.cuda.stream(st):
        with pytest.raises(RuntimeError):  # workspace too small
            bt.admit(req(ws_bytes=wsb - 1), st)
        with pytest.raises(ValueError):  # workspace not 256-byte aligned
            bt.admit(req(offset=16), st)
        with pytest.raises(ValueError):  # a brick needs 2 nodes per axis
            bt.admit(req(nd=(1, 3, 3)), st)
        slots = [bt.admit(req(), st) for _ in range(_lib.TG_BRICK_MAX_SLOTS)]
        assert sorted(slots) == list(range(_lib.TG_BRICK_MAX_SLOTS))
        with pytest.raises(ValueError):  # no free slot
            bt.admit(req(), st)
        short = (_lib.BrickState * 8)()
        assert _lib.lib().tg_brick_poll(bt.handle, short, 8, st.cuda_stream) == _lib.TG_ERR_VALUE
        # b = 0: every solve is converged at its first residual
        bt.step(3, st)
        states = bt.poll(st)
        assert all(states[s].phase == _lib.TG_BRICK_DONE and states[s].status == 0 for s in slots)
        states = bt.poll(st)
        assert all(s.phase == _lib.TG_BRICK_FREE for s in states)
        assert bt.admit(req(), st) == 0
    bt.close()
