"""The configurations at their own sizes, checked through properties that do
not depend on size (the oracle is too slow there):
  * C2 (L = 16384, 16384^2 field): a blocked line is a fixed point of the
    construction up to its stopping tolerances -- every site's velocity is
    <= 0 up to the root tolerance's effect, and a second rk_block from it
    blocks again at once;
  * C1 (L = 65536, 65536 x 4096 field, arclength, f = 0.5): the
    device-resident run equals the step-by-step form;
  * C3 (L up to 16384, 256-row fields): ensemble lines meet max|g| < 1e-8
    under an independent FP64 gradient evaluation.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def npy(t):
    return t.detach().cpu().numpy()


def test_c2_blocked_line_is_a_fixed_point(Q):
    import torch
    n = ny = 16384
    f = Q.FilteredNoise.generated(n, ny, float(n), float(ny), 1.0, 4.0, 4.0, 2)
    p = Q.Params(float(n), 1.0, 0.05, Q.Model.Linear)
    rp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * ny, max_sweeps=200000)
    h = torch.full((n,), 0.5 * ny, dtype=torch.float64, device="cuda")
    r = Q.rk_block(h, p, f, rp)
    assert r.blocked
    v = npy(Q.rk_site_velocity(h, p, f))
    # a site stops within root_tol of its velocity zero: |v| there is at most
    # root_tol times the local slope of v (elastic 2/dx^2 plus the field's)
    assert np.max(v) <= 1e-7
    # the construction stopped once a sweep moved the line by less than
    # sweep_tol in total: restarting from there blocks again at once, moving
    # the line by no more than those residual amounts
    h2 = h.clone()
    r2 = Q.rk_block(h2, p, f, rp)
    assert r2.blocked and r2.sweeps <= 100
    assert float((h2 - h).abs().max()) <= 100 * rp.sweep_tol


def test_c1_resident_run_equals_steps_at_full_size(Q):
    import torch
    n, ny = 65536, 4096
    f = Q.FilteredNoise.generated(n, ny, float(n), float(ny), 1.0, 4.0, 4.0, 1)
    p = Q.Params(float(n), 1.0, 0.5, Q.Model.Arclength)
    steps = 200
    T = 0.5 * (1.0 - np.arange(steps) / 1e5)
    drift = np.full(steps, 0.01)
    diff = np.sqrt(2.0 * T * 0.01)
    h1 = torch.full((n,), 0.5 * ny, dtype=torch.float64, device="cuda")
    h2 = h1.clone()
    d1, d2 = Q.LangevinDynamics(n, 1), Q.LangevinDynamics(n, 1)
    d1.run(h1, p, f, drift, diff)
    for k in range(steps):
        d2.step(h2, p, f, drift[k], diff[k])
    a, b = npy(h1), npy(h2)
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(a))


def test_c3_lines_meet_the_tolerance(Q):
    import torch
    rng = np.random.default_rng(3)
    lines, specs = [], []
    for k in range(48):
        L = int(round(np.exp(rng.uniform(np.log(256), np.log(16384))) / 2)) * 2
        xi = float(rng.uniform(2, 8))
        model = Q.Model(int(rng.integers(0, 2)))
        f = Q.FilteredNoise.generated(L, 256, float(L), 256.0, 1.0, xi, xi, 1000 + k,
                                      store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
        p = Q.Params(float(L), 1.0, 0.0, model)
        h = torch.zeros(L, dtype=torch.float64, device="cuda")
        lines.append((h, p, f, 0.5 / xi ** 2))
        specs.append((h, p, f))
    lp = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=20000, precondition=True, ls_fallback=True)
    res = Q.ensemble_minimize(lines, lp, ftol_fp32=2e-5)
    for r, (h, p, f) in zip(res, specs):
        assert r.converged
        g = npy(Q.gradient(h, p, f))
        assert np.max(np.abs(g)) < 1e-8
