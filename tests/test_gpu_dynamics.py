"""GPU Langevin step against the oracle (trajectory parity given identical
increments) and the reference's dynamics tests (test_dynamics.cpp)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import band_limited_field

pytestmark = pytest.mark.gpu


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def npy(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("model", [0, 1])
def test_trajectory_matches_oracle_with_increments(Q, O, model):
    n, ny, Lx, Ly = 512, 64, 51.2, 6.4
    fld = band_limited_field(n, ny, Lx, Ly, 1.0, 0.4, 3)
    f = Q.FilteredNoise(fld, Lx, Ly)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    rng = np.random.default_rng(11)
    h0 = 3.2 + rng.standard_normal(n) * 0.1
    xi = rng.standard_normal((200, n))
    p = Q.Params(Lx, 1.0, 0.5, Q.Model(model))
    po = O.params(Lx, 1.0, 0.5, model)
    dyn = Q.LangevinDynamics(n, 1)
    h = t64(h0)
    ho = h0.copy()
    dt, T = 0.01, 0.3
    for s in range(200):
        drift, diff = dt, np.sqrt(2 * T * dt) if s % 7 else 0.0
        dyn.step_with_increments(h, p, f, drift, diff, t64(xi[s]))
        O.langevin_step(ho, po, of, drift, diff, xi[s])
    assert np.max(np.abs(npy(h) - ho)) <= 1e-12 * np.max(np.abs(ho))


def test_philox_increments_match_oracle(Q, O):
    n = 10001
    dyn = Q.LangevinDynamics(n, 12345)
    z = npy(dyn.peek_increments())
    zo = O.philox_normals(12345, 0, n)
    assert np.max(np.abs(z - zo)) < 1e-13
    h = t64(np.zeros(n))
    dyn.step(h, Q.Params(float(n)), Q.ZeroNoise(), 0.1, 0.5)
    assert dyn.steps == 1
    assert np.max(np.abs(npy(h) - 0.5 * zo)) < 1e-13
    z1 = npy(dyn.peek_increments())
    assert np.max(np.abs(z1 - O.philox_normals(12345, 1, n))) < 1e-13


def test_zero_temperature_descent(Q):
    """test_dynamics.cpp:44-65."""
    n = 64
    p = Q.Params(float(n), 1.0, 0.0, Q.Model.Linear)
    well = Q.HarmonicWell(4.0, 0.0)
    h = t64(np.random.default_rng(1).uniform(-0.5, 0.5, n))
    dyn = Q.LangevinDynamics(n, 0)
    e_prev = Q.objective(h, p, well)
    for _ in range(2000):
        dyn.step(h, p, well, 0.05, 0.0)
        e = Q.objective(h, p, well)
        assert e <= e_prev + 1e-12
        e_prev = e
    assert e_prev < 1e-6


def test_force_shifts_equilibrium(Q):
    """test_dynamics.cpp:106-130."""
    n, k, y0, fdr = 32, 4.0, 0.2, 0.6
    p = Q.Params(float(n), 1.0, fdr, Q.Model.Linear)
    h = t64(np.zeros(n))
    dyn = Q.LangevinDynamics(n, 0)
    for _ in range(5000):
        dyn.step(h, p, Q.HarmonicWell(k, y0), 0.05, 0.0)
    assert np.max(np.abs(npy(h) - (y0 + fdr / k))) < 1e-6


def test_zero_diffusion_ignores_seed(Q):
    """test_dynamics.cpp:137-161 (bitwise)."""
    n = 48
    p = Q.Params(float(n), 1.0, 0.3, Q.Model.Linear)
    well = Q.HarmonicWell(4.0, 0.1)
    h0 = np.random.default_rng(5).uniform(-0.5, 0.5, n)
    h1, h2 = t64(h0), t64(h0)
    d1, d2 = Q.LangevinDynamics(n, 111), Q.LangevinDynamics(n, 999)
    for _ in range(50):
        d1.step(h1, p, well, 0.05, 0.0)
        d2.step(h2, p, well, 0.05, 0.0)
    assert np.array_equal(npy(h1), npy(h2))


def test_equipartition(Q):
    """test_dynamics.cpp:70-99: <E> = (N/2) kT within 10% (shorter run)."""
    n = 16
    p = Q.Params(float(n), 1.0, 0.0, Q.Model.Linear)
    well = Q.HarmonicWell(4.0, 0.0)
    drift, kT = 0.02, 0.05
    diff = np.sqrt(2 * drift * kT)
    h = t64(np.zeros(n))
    dyn = Q.LangevinDynamics(n, 2024)
    for _ in range(4000):
        dyn.step(h, p, well, drift, diff)
    es = []
    for s in range(40000):
        dyn.step(h, p, well, drift, diff)
        if s % 4 == 0:
            es.append(Q.objective(h, p, well))
    mean_e = float(np.mean(es))
    assert abs(mean_e - 0.5 * n * kT) < 0.1 * 0.5 * n * kT, mean_e


@pytest.mark.parametrize("model", [0, 1])
def test_resident_run_matches_step_loop(Q, model):
    """qew_langevin_run == the same schedule stepped one call at a time
    (same Philox increments; FP64 within 1e-12 relative)."""
    n, ny, Lx, Ly = 1000, 64, 100.0, 6.4
    f = Q.FilteredNoise(band_limited_field(n, ny, Lx, Ly, 1.0, 0.4, 3), Lx, Ly)
    p = Q.Params(Lx, 1.0, 0.3, Q.Model(model))
    rng = np.random.default_rng(2)
    h0 = 3.2 + 0.1 * rng.standard_normal(n)
    steps = 301
    drift = np.full(steps, 0.01)
    diff = np.sqrt(2 * np.linspace(0.4, 0.0, steps) * 0.01)
    diff[::7] = 0.0
    d1, d2 = Q.LangevinDynamics(n, 5), Q.LangevinDynamics(n, 5)
    h1, h2 = t64(h0), t64(h0)
    for k in range(steps):
        d1.step(h1, p, f, drift[k], diff[k])
    d2.run(h2, p, f, drift, diff)
    assert d1.steps == d2.steps
    a, b = npy(h1), npy(h2)
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(a))


@pytest.mark.parametrize("edge", [False, True])
def test_resident_run_fp32(Q, edge):
    """FP32-gather run (16 taps, or 4 from the x-filtered store): deterministic
    part close to FP64, FP32 normals N(0,1)."""
    n, ny = 4096, 64
    store = Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32 | (Q.QEW_STORE_FP32_EDGE if edge else 0)
    f = Q.FilteredNoise(band_limited_field(n, ny, float(n), float(ny), 1.0, 4.0, 8),
                        float(n), float(ny), store=store)
    p = Q.Params(float(n), 1.0, 0.2, Q.Model.Arclength)
    h0 = 32 + np.cumsum(np.random.default_rng(1).standard_normal(n)) * 0.01
    a, b = t64(h0), t64(h0)
    sched = np.full(200, 0.05)
    Q.LangevinDynamics(n, 1).run(a, p, f, sched, np.zeros(200))
    Q.LangevinDynamics(n, 1).run(b, p, f, sched, np.zeros(200), precision=Q.QEW_PREC_FP32_SPLIT)
    assert np.max(np.abs(npy(a) - npy(b))) < 1e-4
    zero = Q.FilteredNoise(np.zeros((n, ny)), float(n), float(ny), store=store)
    h = t64(np.zeros(n))
    Q.LangevinDynamics(n, 9).run(h, Q.Params(float(n), 0.0, 0.0), zero, [0.0], [1.0],
                                 precision=Q.QEW_PREC_FP32_SPLIT)
    z = npy(h)
    assert abs(z.mean()) < 0.05 and abs(z.std() - 1.0) < 0.05
