"""Continuous-batching server: every request's result is the same alone and
in the mix (bitwise: each request's kernels are deterministic and their
launch shapes depend on the request alone), HBM-budget admission, limits."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mix(Q):
    """Small requests of all three kinds (seeded, deterministic)."""
    S, L, D = 0, 1, 2
    return [
        dict(kind=S, n=512, rows=256, xi=3.0, seed=11, model=0, ftol=1e-8),
        dict(kind=S, n=2048, rows=256, xi=6.0, seed=12, model=1, ftol=1e-8),
        dict(kind=L, n=1024, rows=256, xi=4.0, seed=13, model=1, steps=400, temperature=0.3,
             dt=0.01, driving_force=0.5),
        dict(kind=D, n=512, rows=64, xi=4.0, seed=14, f_step=0.1, f_max=4.0, bisect_rtol=1e-4,
             max_sweeps=3000),
        dict(kind=S, n=1000, rows=256, xi=2.5, seed=15, model=0, ftol=1e-8),
        dict(kind=L, n=4096, rows=256, xi=3.0, seed=16, model=0, steps=300, temperature=0.1,
             dt=0.01),
    ]


def _run(Q, reqs, inflight, budget=20e9, one_at_a_time=False):
    srv = Q.Server(hbm_budget_bytes=budget, max_inflight=inflight)
    outs, ids = {}, []
    lines = [np.zeros(r["n"]) for r in reqs]
    try:
        for k, r in enumerate(reqs):
            ids.append(srv.submit(h_out=lines[k], **r))
            if one_at_a_time:
                srv.drain(600)
        srv.drain(600)
        for resp in srv.poll():
            outs[resp["id"]] = resp
    finally:
        srv.close()
    return [outs[i] for i in ids], lines


def test_results_same_alone_and_in_mix(Q):
    reqs = _mix(Q)
    mix, lines_mix = _run(Q, reqs, inflight=len(reqs))
    alone, lines_alone = _run(Q, reqs, inflight=1, one_at_a_time=True)
    for r, a, b, la, lb in zip(reqs, mix, alone, lines_mix, lines_alone):
        assert a["status"] == 0 and b["status"] == 0, (a, b)
        assert a["value"] == b["value"] and a["iterations"] == b["iterations"], (r, a, b)
        assert np.array_equal(la, lb)
        if r["kind"] == 0:
            assert a["converged"] and a["max_force"] < 1e-8
        if r["kind"] == 2:
            assert a["converged"] and a["value"] > 0
    # in the mix, later requests started before earlier ones finished
    starts = sorted(m["t_start"] for m in mix)
    ends = sorted(m["t_end"] for m in mix)
    assert starts[-1] < ends[-1] and starts[1] < ends[0]


def test_budget_admission_and_limits(Q):
    reqs = [dict(kind=0, n=1024, rows=256, xi=4.0, seed=20 + k, ftol=1e-8) for k in range(3)]
    # a budget that fits one request at a time still completes everything
    one = 1024 * 256 * 28 + 1024 * 320 + (1 << 20)
    res, _ = _run(Q, reqs, inflight=3, budget=one * 1.5)
    assert all(r["status"] == 0 for r in res)
    # requests are admitted one at a time: no two run concurrently
    spans = sorted((r["t_start"], r["t_end"]) for r in res)
    for (s0, e0), (s1, e1) in zip(spans, spans[1:]):
        assert s1 >= e0 - 1e-6
    srv = Q.Server(hbm_budget_bytes=1e6, max_inflight=1)
    try:
        with pytest.raises(Q.QewError):
            srv.submit(kind=0, n=4096, rows=256, xi=4.0, seed=1)
        with pytest.raises(ValueError):
            srv.submit(kind=2, n=513, rows=64, xi=4.0, seed=1)
        # a force ramp of more than 1e9 steps would hold a worker for ever
        with pytest.raises(ValueError):
            srv.submit(kind=2, n=512, rows=64, xi=4.0, seed=1, f_step=1e-12, f_max=40.0,
                       bisect_rtol=1e-3, max_sweeps=100)
        # the device loop's workspace holds lines of at most 16384 points
        for bad in (-1, 16385):
            with pytest.raises(ValueError):
                srv.set_lane_limit(bad)
    finally:
        srv.close()


@pytest.mark.parametrize("limit,specs", [
    (None, [(512, 3.0, 21, 0), (1000, 2.5, 22, 1), (1536, 5.0, 23, 0), (2046, 4.0, 24, 1)]),
    (16384, [(4096, 3.0, 25, 1), (9000, 6.0, 26, 0), (16384, 4.0, 27, 0)])])
def test_static_lane_equals_ensemble(Q, limit, specs):
    """Static requests up to the lane limit (2048 points by default, raised to
    16384 here for long lines) go to the device-resident loop; each result is
    the one-line ensemble solve's (same field, same settings) bit for bit."""
    import torch
    reqs = [dict(kind=0, n=n, rows=256, xi=xi, seed=sd, model=m, ftol=1e-8)
            for n, xi, sd, m in specs]
    srv = Q.Server(hbm_budget_bytes=20e9, max_inflight=2)
    if limit is not None:
        srv.set_lane_limit(limit)
    lines = [np.zeros(r["n"]) for r in reqs]
    try:
        ids = [srv.submit(h_out=lines[k], **r) for k, r in enumerate(reqs)]
        srv.drain(600)
        got = {r["id"]: r for r in srv.poll()}
        stats = srv.lane_stats()
    finally:
        srv.close()
    assert stats["available"] and stats["served"] == len(reqs) and stats["launches"] >= 1
    lp = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=20000, precondition=True, ls_fallback=True)
    for (n, xi, sd, m), k, h in zip(specs, ids, lines):
        f = Q.FilteredNoise.generated(n, 256, float(n), 256.0, 1.0, xi, xi, sd,
                                      store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
        p = Q.Params(float(n), 1.0, 0.0, Q.Model(m))
        he = torch.zeros(n, dtype=torch.float64, device="cuda")
        re = Q.ensemble_minimize([(he, p, f, 0.5 / xi ** 2)], lp, ftol_fp32=2e-5)[0]
        assert got[k]["status"] == 0 and got[k]["iterations"] == re.iterations
        assert np.array_equal(h, he.cpu().numpy())
        assert got[k]["converged"] and got[k]["max_force"] < 1e-8
