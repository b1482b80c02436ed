"""The reference's seeded field and its three drivers on the GPU.

* FilteredNoise's seeded constructor against the oracle's restatement
  (std::mt19937_64 phases, inverse FFT2, std scaling, prefilter);
* static_sweep / dynamic_anneal / depinning_ramp against the reference's
  driver tests (tests/test_executables.cpp:59-190) and against the same loops
  written out over this library's single-line solvers;
* the executables end to end: console lines and the output key contract.
"""
from __future__ import annotations

import math
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
PI = 3.14159265358979323846


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def npy(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("nx, ny, Lx, Ly, amp, xi, seed", [
    (64, 32, 1.0, 1.0, 1.0, 0.1, 1),
    (48, 40, 3.2, 1.0, 0.7, 0.2, 12345),
    (30, 18, 2.0, 1.5, 1.3, 0.15, 7),
])
def test_seeded_field_matches_oracle(Q, O, nx, ny, Lx, Ly, amp, xi, seed):
    """filtered_noise.cpp:25-82 then :92-136; FFT rounding only (1e-12)."""
    f = Q.FilteredNoise.seeded(nx, ny, Lx, Ly, amp, xi, xi, seed)
    ref = O.prefilter(O.seeded_field(nx, ny, Lx, Ly, amp, xi, xi, seed))
    got = f.coefficients()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_mt19937_64_known_answer(O):
    """[rand.predef]: the 10000th output of a default-constructed mt19937_64."""
    assert int(O.mt64_outputs(5489, 10000)[-1]) == 9981545732273789042


def test_static_sweep_zero_noise(Q):
    """test_executables.cpp:59-91: the flat start is the minimum; Larkin map."""
    c = Q.StaticConfig(model=Q.Model.Linear, amplitude=1.3, xi=0.1, Lx=1.0, Ly=1.0, nx=16,
                       ny=8, pinning_lengths_over_xi=(0.1, 1.0, 4.0), ftol=1e-8, max_iter=2000)
    prof = Q.static_sweep(c, Q.ZeroNoise())
    assert len(prof) == 3
    for k, p in enumerate(prof):
        assert p.pinning_length_over_xi == c.pinning_lengths_over_xi[k]
        assert abs(p.line_tension - c.pinning_lengths_over_xi[k] ** 1.5 * c.amplitude) < 1e-12
        assert p.h.shape == (16,) and p.result.converged
        assert np.ptp(p.h) < 1e-9 and np.max(np.abs(p.h - 0.5)) < 1e-9


@pytest.mark.parametrize("model", [0, 1])
def test_static_sweep_equals_one_solve_per_ratio(Q, model):
    """The batched sweep equals lbfgs_minimize called per ratio with the
    driver's settings (qew_runs.h:74-100), line for line."""
    nx, ny, Lx, Ly, xi = 256, 64, 8.0, 1.0, 0.1
    f = Q.FilteredNoise.seeded(nx, ny, Lx, Ly, 1.0, xi, xi, 3)
    c = Q.StaticConfig(model=Q.Model(model), xi=xi, Lx=Lx, Ly=Ly, nx=nx, ny=ny,
                       pinning_lengths_over_xi=(0.3, 1.0, 3.0, 10.0), ftol=1e-6, max_iter=3000)
    prof = Q.static_sweep(c, f)
    for p in prof:
        h = t64(np.full(nx, 0.5 * Ly))
        lp = Q.LbfgsParams(ftol=c.ftol, max_iter=c.max_iter, precondition=True,
                           precond_shift=0.5 * (Lx / nx) * 1.0 / xi ** 2)
        r = Q.lbfgs_minimize(h, Q.Params(Lx, p.line_tension, 0.0, Q.Model(model)), f, lp)
        assert r.iterations == p.result.iterations and r.converged == p.result.converged
        assert np.max(np.abs(npy(h) - p.h)) <= 1e-12 * np.max(np.abs(p.h))
        assert p.result.converged and p.result.max_force < 1e-6


def test_dynamic_anneal_timestep_and_snapshots(Q):
    """test_executables.cpp:94-132."""
    c = Q.DynamicConfig(model=Q.Model.Linear, amplitude=1.0, xi=0.1, pinning_length_over_xi=0.1,
                        Lx=1.0, Ly=1.0, nx=32, ny=8, tau=1.0, tl_start=0.01, tl_end=0.0001,
                        total_time=200.0)
    r = Q.dynamic_anneal(c, Q.ZeroNoise())
    fac = c.xi / max(c.tl_start, c.tl_end)
    assert abs(r.dt - min(0.1, c.tau / 10 * min(fac, fac * fac))) < 1e-12
    assert abs(r.line_tension - c.pinning_length_over_xi ** 1.5 * c.amplitude) < 1e-12
    assert len(r.snapshots) >= 2
    assert abs(r.snapshots[0].t - 10 * r.dt) < r.dt
    for a, b in zip(r.snapshots, r.snapshots[1:]):
        assert b.t > a.t and abs(b.t / a.t - 10.0) < 0.5
    for s in r.snapshots:
        assert s.h.shape == (32,) and np.all(np.isfinite(s.h))
    assert r.snapshots[-1].t <= r.total_time


@pytest.mark.parametrize("model", [0, 1])
def test_dynamic_anneal_equals_step_loop(Q, model):
    """The driver's device-resident runs equal the reference's loop
    (qew_runs.h:161-175) written out over LangevinDynamics.step."""
    nx, ny, Lx, Ly, xi = 128, 64, 2.0, 1.0, 0.1
    f = Q.FilteredNoise.seeded(nx, ny, Lx, Ly, 1.0, xi, xi, 4)
    c = Q.DynamicConfig(model=Q.Model(model), xi=xi, pinning_length_over_xi=0.5,
                        driving_force=0.2, Lx=Lx, Ly=Ly, nx=nx, ny=ny, seed=9, total_time=3.0)
    r = Q.dynamic_anneal(c, f)
    dyn = Q.LangevinDynamics(nx, c.seed + 1)
    h = t64(np.full(nx, 0.5 * Ly))
    p = Q.Params(Lx, r.line_tension, c.driving_force, Q.Model(model))
    t, next_save, tl, snaps = 0.0, 10 * r.dt, c.tl_start, []
    while t < c.total_time:
        dyn.step(h, p, f, tl * r.dt / (c.tau * c.amplitude), tl * math.sqrt(2 * r.dt / c.tau))
        tl = c.tl_start + (c.tl_end - c.tl_start) * (t / c.total_time)
        t += r.dt
        if t > next_save - r.dt / 2:
            snaps.append((t, npy(h).copy()))
            next_save *= 10
    assert r.steps == dyn.steps and len(snaps) == len(r.snapshots)
    for (ta, ha), s in zip(snaps, r.snapshots):
        assert ta == s.t
        assert np.max(np.abs(ha - s.h)) <= 1e-12 * np.max(np.abs(ha))


def test_depinning_ramp_brackets_fc(Q):
    """test_executables.cpp:135-190 (washboard, f_c = A k)."""
    A, k = 0.1, 2 * PI
    lam = 2 * PI / k
    rp = Q.RkParams(dstep=lam / 100, max_advance=lam, root_tol=1e-11, sweep_tol=1e-8,
                    runaway=3 * lam, max_sweeps=20000)
    c = Q.DepinningConfig(model=Q.Model.Linear, amplitude=1.0, pinning_length_over_xi=1.0,
                          Lx=8.0, Ly=1.0, nx=8, ny=8, f_step=0.2, f_max=2.0, rp=rp)
    r = Q.depinning_ramp(c, Q.SinusoidNoise(A, k))
    assert abs(r.line_tension - 1.0) < 1e-12
    assert r.steps[0].result.blocked and r.steps[0].f == 0.0
    last = r.steps[-1]
    assert not last.result.blocked and last.result.runaway and last.h is None
    assert abs(r.f_c_upper_bound - last.f) < 1e-9
    assert 0 < r.f_c_upper_bound <= c.f_max
    assert r.f_c_upper_bound - c.f_step <= A * k <= r.f_c_upper_bound + 1e-9
    for st in r.steps:
        if st.result.blocked:
            assert st.h.shape == (8,)
    assert r.f_c == -1.0  # no bisection asked


def test_depinning_ramp_bisection(Q):
    """The added bisection narrows the ramp's bracket onto f_c = A k."""
    A, k = 0.1, 2 * PI
    lam = 2 * PI / k
    rp = Q.RkParams(dstep=lam / 100, max_advance=lam, root_tol=1e-12, sweep_tol=1e-10,
                    runaway=3 * lam, max_sweeps=100000)
    c = Q.DepinningConfig(model=Q.Model.Linear, pinning_length_over_xi=1.0, Lx=8.0, Ly=1.0,
                          nx=8, ny=8, f_step=0.2, f_max=2.0, rp=rp, bisect_rtol=1e-6)
    r = Q.depinning_ramp(c, Q.SinusoidNoise(A, k))
    lo, hi = r.f_c_bracket
    assert lo < hi and hi - lo <= 1e-6 * hi and r.bisect_blocks > 0
    assert abs(r.f_c - A * k) < 2e-3 * A * k


def test_depinning_ramp_equals_rk_block_loop(Q):
    """On a seeded field the ramp equals rk_block called per force, restarting
    from the previous configuration (qew_runs.h:226-241)."""
    nx, ny, Lx, Ly, xi = 128, 64, 4.0, 1.0, 0.1
    f = Q.FilteredNoise.seeded(nx, ny, Lx, Ly, 1.0, xi, xi, 5)
    rp = Q.RkParams(dstep=0.5 * Ly / ny, max_advance=Ly, root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2 * Ly, max_sweeps=50000)
    c = Q.DepinningConfig(model=Q.Model.Linear, pinning_length_over_xi=5.0, Lx=Lx, Ly=Ly, nx=nx,
                          ny=ny, f_step=2.0, f_max=200.0, rp=rp)
    r = Q.depinning_ramp(c, f)
    assert len(r.steps) >= 2 and not r.steps[-1].result.blocked
    h = t64(np.full(nx, 0.5 * Ly))
    for st in r.steps:
        res = Q.rk_block(h, Q.Params(Lx, r.line_tension, st.f, Q.Model.Linear), f, rp)
        assert res.sweeps == st.result.sweeps and res.blocked == st.result.blocked
        if st.result.blocked:
            assert np.array_equal(npy(h), st.h)


def test_depinning_odd_length_rejected(Q):
    c = Q.DepinningConfig(nx=17, rp=Q.RkParams(0.01, 1.0, 1e-10, 1e-9, 2.0, 100))
    with pytest.raises(ValueError):
        Q.depinning_ramp(c, Q.SinusoidNoise())


@pytest.mark.parametrize("f_step", [0.0, -0.1, float("nan")])
def test_depinning_unbounded_ramp_rejected(Q, f_step):
    """k * f_step <= f_max never ends for f_step <= 0 (f_max >= 0): rejected
    instead of ramping forever; f_max < 0 runs no force at all."""
    rp = Q.RkParams(0.01, 1.0, 1e-10, 1e-9, 2.0, 100)
    with pytest.raises(ValueError, match="f_step|bad arguments"):
        Q.depinning_ramp(Q.DepinningConfig(nx=8, ny=8, f_step=f_step, f_max=1.0, rp=rp),
                         Q.SinusoidNoise())
    if f_step == 0.0:
        r = Q.depinning_ramp(Q.DepinningConfig(nx=8, ny=8, f_step=f_step, f_max=-1.0, rp=rp),
                             Q.SinusoidNoise())
        assert r.steps == [] and r.f_c_upper_bound == -1


def _run(exe, *args, cwd):
    from qew_gb300 import build
    r = subprocess.run([build.executable(exe), *args], capture_output=True, text=True, cwd=cwd,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return r.stdout


def test_executable_static_end_to_end(Q, tmp_path):
    out = _run("qew_static", "--model", "linear", "--nx", "256", "--ny", "64", "--Lx", "8",
               "--pinning_lengths", "1,10", "--ftol", "1e-8", "--seed", "3", cwd=tmp_path)
    assert out.count("converged") == 2 and "wrote static_linear.npz" in out
    z = np.load(tmp_path / "static_linear.npz")
    assert float(z["physical_size"]) == 8.0
    f = Q.FilteredNoise.seeded(256, 64, 8.0, 1.0, 1.0, 0.1, 0.1, 3)
    prof = Q.static_sweep(Q.StaticConfig(model=Q.Model.Linear, Lx=8.0, nx=256, ny=64,
                                         pinning_lengths_over_xi=(1.0, 10.0), ftol=1e-8), f)
    for p, key in zip(prof, ("pinning_length=1", "pinning_length=10")):
        assert np.array_equal(z["driving_force=0/%s/h" % key], p.h)
        assert float(z["driving_force=0/%s/pinning_length" % key]) == p.pinning_length_over_xi


def test_executable_dynamic_and_depinning(Q, tmp_path):
    out = _run("qew_dynamic", "--nx", "128", "--ny", "64", "--total_time", "2", "--output",
               "d.npz", cwd=tmp_path)
    assert out.startswith("dt=") and "saved t=" in out
    z = np.load(tmp_path / "d.npz")
    keys = [k for k in z.files if k.endswith("/h")]
    assert keys and all(k.startswith("timestep=") and "/driving_force=0/line_tension=0.0316/" in k
                        for k in keys)
    out = _run("qew_depinning", "--model", "linear", "--nx", "64", "--ny", "32", "--f_step", "2",
               "--f_max", "100", "--max_sweeps", "20000", "--bisect_rtol", "1e-4", cwd=tmp_path)
    assert "blocked" in out and "f_c=" in out
    z = np.load(tmp_path / "depinning_linear.npz")
    assert "driving_force=0/h" in z.files and "f_c_upper_bound" in z.files and "f_c" in z.files
    fc_ub = float(z["f_c_upper_bound"])
    assert fc_ub - 2.0 <= float(z["f_c"]) <= fc_ub


def test_executable_analysis_keys(Q, tmp_path):
    """--analysis 1 adds ell, acf, q, psd beside every profile (the datasets of
    the reference's post-processing), equal to line_statistics of that profile."""
    import torch
    _run("qew_static", "--model", "linear", "--nx", "128", "--ny", "32", "--Lx", "4",
         "--pinning_lengths", "2", "--analysis", "1", "--output", "s.npz", cwd=tmp_path)
    z = np.load(tmp_path / "s.npz")
    pre = "driving_force=0/pinning_length=2"
    for key in ("ell", "acf", "q", "psd"):
        assert z[pre + "/" + key].shape == (65,)
    ell, acf, q, psd = (t.cpu().numpy() for t in Q.line_statistics(
        torch.as_tensor(z[pre + "/h"], device="cuda"), 4.0))
    assert np.array_equal(z[pre + "/acf"], acf) and np.array_equal(z[pre + "/psd"], psd)
    assert np.array_equal(z[pre + "/ell"], ell) and np.array_equal(z[pre + "/q"], q)


def test_cpp_face_runs(Q, tmp_path):
    """The C++ face (include/qew_gpu.hpp) used as a reference caller would:
    solvers, drivers, std::invalid_argument on odd n, Error statuses."""
    from test_cli import build_hpp_probe
    exe = build_hpp_probe(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout and r.stdout.count("ok ") == 8
