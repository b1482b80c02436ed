"""CPU oracle pinned against the reference's golden vectors and known answers.

Every case here restates a test of the reference suite (file:line in each
docstring), with the reference's tolerance, against the oracle. The GPU tests
then compare the CUDA path with this oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import band_limited_field

PI = 3.14159265358979323846


def test_prefilter_matches_scipy_grid_wrap(O, noise_golden):
    """The FFT prefilter equals SciPy's spline_filter(mode='grid-wrap')
    (filtered_noise.h:59-62; gen_golden.py:40)."""
    coef = O.prefilter(noise_golden["field"])
    assert np.max(np.abs(coef - noise_golden["coef_scipy"])) < 1e-12


def test_sample_matches_scipy_golden(O, noise_golden):
    """test_filtered_noise.cpp:286-324: value 1e-7, derivatives 1e-4."""
    g = noise_golden
    assert bool(g["verified_bytes"]), "fixture not byte-verified against the reference"
    f = O.BSplineField(g["field"], float(g["Lx"]), float(g["Ly"]))
    v, dvdx, dvdy = O.sample(f, g["x"], g["y"])
    assert np.max(np.abs(v - g["v"])) < 1e-7
    assert np.max(np.abs(dvdx - g["dvdx"])) < 1e-4
    assert np.max(np.abs(dvdy - g["dvdy"])) < 1e-4


def test_lbfgs_matches_scipy_golden(O, lbfgs_golden):
    """test_lbfgs.cpp:309-349: preconditioned, ftol 1e-8, e within 1e-5 rel of
    the reference's committed SciPy minimum."""
    g = lbfgs_golden
    f = O.BSplineField(g["field"], float(g["Lx"]), float(g["Ly"]))
    p = O.params(float(g["Lx"]), float(g["line_tension"]), 0.0, 0)
    h = g["h0"].copy()
    r = O.lbfgs_minimize(h, p, f, O.lbfgs_default_params(ftol=1e-8, precondition=1))
    assert r.converged
    e = O.objective(h, p, f)
    e_ref = float(g["e_min_ref"])
    assert np.isfinite(e_ref)
    assert abs(e - e_ref) <= 1e-5 * abs(e_ref) + 1e-6


def test_nodes_reproduced(O):
    """test_filtered_noise.cpp:118-143."""
    nx, ny, Lx, Ly = 64, 48, 3.2, 1.0
    field = band_limited_field(nx, ny, Lx, Ly, 1.5, 0.15, 3)
    f = O.BSplineField(field, Lx, Ly)
    ii, jj = np.meshgrid(np.arange(0, nx, 5), np.arange(0, ny, 5), indexing="ij")
    v, _, _ = O.sample(f, ii.ravel() * (Lx / nx), jj.ravel() * (Ly / ny))
    assert np.max(np.abs(v - field[ii.ravel(), jj.ravel()])) < 1e-9


def test_periodic_wrap(O):
    """test_filtered_noise.cpp:238-281: shifts by whole periods are exact."""
    nx, ny, Lx, Ly = 48, 40, 2.5, 1.3
    f = O.BSplineField(band_limited_field(nx, ny, Lx, Ly, 1.0, 0.25, 17), Lx, Ly)
    rng = np.random.default_rng(123)
    x, y = rng.uniform(0, Lx, 60), rng.uniform(0, Ly, 60)
    base = O.sample(f, x, y)
    for sx, sy in [(1, 0), (0, 1), (-1, 0), (0, -1), (3, -2), (-5, 7), (-13, -11)]:
        s = O.sample(f, x + sx * Lx, y + sy * Ly)
        for a, b in zip(base, s):
            assert np.max(np.abs(a - b)) < 1e-9


@pytest.mark.parametrize("model", [0, 1])
def test_gradient_matches_fd_analytic(O, model):
    """test_qew_model.cpp:44-100 (AnalyticNoise, tolerance 1e-6)."""
    n = 64
    p = O.params(float(n), 1.0, 0.37, model)
    nz = O.AnalyticNoise()
    h = np.random.default_rng(12345).uniform(0, 1, n)
    g = O.gradient(h, p, nz)
    eps = 1e-6
    fd = np.empty(n)
    for j in range(n):
        hp, hm = h.copy(), h.copy()
        hp[j] += eps
        hm[j] -= eps
        fd[j] = (O.objective(hp, p, nz) - O.objective(hm, p, nz)) / (2 * eps)
    assert np.max(np.abs(fd - g)) < 1e-6


@pytest.mark.parametrize("model", [0, 1])
def test_gradient_matches_fd_bspline(O, model):
    """test_filtered_noise.cpp:187-230 (real field, tolerance 1e-5)."""
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    f = O.BSplineField(band_limited_field(nx, ny, Lx, Ly, 0.5, 0.3, 11), Lx, Ly)
    p = O.params(Lx, 0.5, 0.1, model)
    h = np.random.default_rng(7).uniform(0.2 * Ly, 0.8 * Ly, nx)
    g = O.gradient(h, p, f)
    eps = 1e-6
    fd = np.empty(nx)
    for j in range(nx):
        hp, hm = h.copy(), h.copy()
        hp[j] += eps
        hm[j] -= eps
        fd[j] = (O.objective(hp, p, f) - O.objective(hm, p, f)) / (2 * eps)
    assert np.max(np.abs(fd - g)) < 1e-5


def test_flat_line_energy(O):
    """test_qew_model.cpp:110-132: E = L (v0 - f c) to 1e-12."""
    n, L, c, v0, fdr = 50, 3.0, 0.7, 1.25, 0.4
    for model in (0, 1):
        e = O.objective(np.full(n, c), O.params(L, 2.3, fdr, model), O.ConstNoise(v0))
        assert abs(e - L * (v0 - fdr * c)) < 1e-12


def test_sinusoid_linear_energy(O):
    """test_qew_model.cpp:140-163: closed-form discrete elastic energy."""
    n, lt, a = 32, 1.7, 0.9
    h = a * np.sin(2 * PI * np.arange(n) / n)
    e = O.objective(h, O.params(float(n), lt, 0.0, 0), O.ConstNoise(0.0))
    assert abs(e - (lt * a * a * n / 2) * (1 - np.cos(2 * PI / n))) < 1e-10


def test_precond_matches_numpy_fft(O):
    """The preconditioner is irfft(rfft(q)/eig) with kokkos-fft normalisation
    (lbfgs.h:117-118, 138-145, 173-180)."""
    for n in (1, 2, 7, 64, 100, 1024):
        q = np.random.default_rng(n).standard_normal(n)
        d = O.precond_apply(q, 1.3, 5.0, 0.2)
        k = np.arange(n // 2 + 1)
        eig = (1.3 / (5.0 / n)) * 4 * np.sin(PI * k / n) ** 2 + 0.2
        ref = np.fft.irfft(np.fft.rfft(q) / eig, n)
        assert np.max(np.abs(d - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))


def test_lbfgs_reference_cases(O):
    """test_lbfgs.cpp:68-124, 128-141, 150-188: flat relaxation, harmonic
    minimum (both models), non-convergence flag, curvature skip, LS give-up."""
    n = 128
    h = 0.5 + 0.3 * np.cos(4 * PI * np.arange(n) / n)
    r = O.lbfgs_minimize(h, O.params(float(n), 1.0, 0.0, 0), O.ZeroNoise(),
                         O.lbfgs_default_params(ftol=1e-9))
    assert r.converged and np.ptp(h) < 1e-6
    for model in (0, 1):
        h = np.zeros(96)
        r = O.lbfgs_minimize(h, O.params(96.0, 1.0, 0.0, model), O.HarmonicWell(2.0, 0.5),
                             O.lbfgs_default_params(ftol=1e-9))
        assert r.converged and np.max(np.abs(h - 0.5)) < 1e-6
    h = np.zeros(96)
    r = O.lbfgs_minimize(h, O.params(96.0, 1.0, 0.0, 0), O.HarmonicWell(2.0, 0.5),
                         O.lbfgs_default_params(ftol=1e-12, max_iter=1))
    assert not r.converged and r.max_force >= 1e-12
    h = np.zeros(16)
    r = O.lbfgs_minimize(h, O.params(16.0, 1.0, 0.0, 0), O.HarmonicWell(2.0, 0.5),
                         O.lbfgs_default_params(ftol=1e-8, max_iter=20000, curvature_eps=1e30))
    assert r.n_curvature_skips > 0 and r.converged and np.max(np.abs(h - 0.5)) < 1e-6
    h = np.zeros(32)
    r = O.lbfgs_minimize(h, O.params(32.0, 1.0, 0.0, 0), O.HarmonicWell(2.0, 0.5),
                         O.lbfgs_default_params(ftol=1e-9, max_ls=0))
    assert not r.converged and r.iterations == 0 and r.n_ls_restarts == 0


def test_rk_washboard_fc(O):
    """test_rosso_krauth.cpp:51-89: f_c = A k recovered by bisection to 2%."""
    n, A, k = 16, 0.1, 2 * PI
    lam = 2 * PI / k
    nz = O.SinusoidNoise(A, k)
    rp = O.rk_params(lam / 200, lam, 1e-12, 1e-11, 3 * lam, 100000)

    def blocks(f):
        return O.rk_block(np.zeros(n), O.params(float(n), 1.0, f, 0), nz, rp).blocked

    lo, hi = 0.0, 2 * A * k
    assert blocks(lo) and not blocks(hi)
    for _ in range(40):
        m = 0.5 * (lo + hi)
        if blocks(m):
            lo = m
        else:
            hi = m
    assert abs(0.5 * (lo + hi) - A * k) < 0.02 * A * k


def test_rk_velocity_is_minus_gradient(O):
    """test_rosso_krauth.cpp:94-141: rk_site_velocity == -gradient to 1e-12."""
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    f = O.BSplineField(band_limited_field(nx, ny, Lx, Ly, 0.7, 0.2, 13), Lx, Ly)
    h = np.random.default_rng(21).uniform(0.1 * Ly, 0.9 * Ly, nx)
    for model in (0, 1):
        p = O.params(Lx, 1.3, 0.4, model)
        g = O.gradient(h, p, f)
        dx = Lx / nx
        v = np.array([O.rk_site_velocity(i, nx, dx, 1.3, 0.4, model, h[i], h[i - 1],
                                         h[(i + 1) % nx], f) for i in range(nx)])
        assert np.max(np.abs(v + g)) < 1e-12


def test_rk_odd_length_rejected(O):
    """test_rosso_krauth.cpp:296-313."""
    with pytest.raises(ValueError):
        O.rk_block(np.zeros(17), O.params(17.0, 1.0, 0.0, 0), O.SinusoidNoise(),
                   O.rk_params(0.01, 1.0, 1e-10, 1e-9, 3.0))


def test_philox_normals_moments(O):
    """Philox4x32-10 + Box-Muller increments are N(0,1)."""
    z = np.concatenate([O.philox_normals(1, s, 4096) for s in range(64)])
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1) < 0.01
    assert abs(np.mean(z ** 4) - 3.0) < 0.1
    a, b = O.philox_normals(7, 3, 1000), O.philox_normals(7, 3, 1000)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, O.philox_normals(7, 4, 1000))


def test_oracle_fire_reference_cases(O):
    """The reference's FIRE known answers (tests/test_fire.cpp) on the oracle."""
    import math
    n = 128
    h = 0.5 + 0.3 * np.cos(4 * np.pi * np.arange(n) / n)
    r = O.fire_minimize(h, O.params(float(n), 1.0, 0.0, 0), O.ZeroNoise(),
                        O.fire_params(0.1, ftol=1e-9))
    assert r.converged and r.max_force < 1e-9 and np.ptp(h) < 1e-6
    n = 96
    h = np.zeros(n)
    r = O.fire_minimize(h, O.params(float(n), 1.0, 0.0, 0), O.HarmonicWell(2.0, 0.5),
                        O.fire_params(0.1 * math.sqrt(1.0), ftol=1e-9))
    assert r.converged and np.max(np.abs(h - 0.5)) < 1e-6
    h = np.zeros(64)
    r = O.fire_minimize(h, O.params(64.0, 1.0, 0.0, 0), O.HarmonicWell(2.0, 0.5),
                        O.fire_params(0.1, ftol=1e-12, max_iter=3))
    assert not r.converged and r.iterations == 3


def test_x_filtered_store_identity(O):
    """The x-filtered store's algebra: on a line with one point per field
    column, the midpoint of edge e sits at x = (e + 1/2) dx, where the cubic
    B-spline x weights are 1/48, 23/48, 23/48, 1/48. The per-column x sums
    E[e, j] = sum_a w_a c[e - 1 + a, j], weighted along y, reproduce the
    oracle's 16-tap value and dV/dy there (to rounding, the sum's order
    aside)."""
    nx, ny, Lx, Ly = 64, 16, 64.0, 8.0
    rng = np.random.default_rng(11)
    fld = rng.standard_normal((nx, ny))
    of = O.BSplineField(fld, Lx, Ly)
    c = of.coef                                  # [nx][ny], y fastest
    w = np.array([1.0, 23.0, 23.0, 1.0]) / 48.0
    E = sum(w[a] * np.roll(c, 1 - a, axis=0) for a in range(4))   # E[e] uses c[e-1+a]
    dx, dy = Lx / nx, Ly / ny
    e = np.repeat(np.arange(nx - 1), 5)          # every edge but the wrap edge
    y = rng.uniform(-2 * Ly, 3 * Ly, e.size)     # rows wrap on both sides
    gy = y / dy
    iy = np.floor(gy).astype(int)
    t = gy - iy
    wy = np.stack([(1 - t) ** 3, 3 * t ** 3 - 6 * t ** 2 + 4, -3 * t ** 3 + 3 * t ** 2 + 3 * t + 1,
                   t ** 3]) / 6.0
    dwy = np.stack([-0.5 * (1 - t) ** 2, 1.5 * t ** 2 - 2 * t, -1.5 * t ** 2 + t + 0.5, 0.5 * t ** 2])
    rows = [(iy - 1 + b) % ny for b in range(4)]
    v = sum(wy[b] * E[e, rows[b]] for b in range(4))
    dvdy = sum(dwy[b] * E[e, rows[b]] for b in range(4)) / dy
    vo, _, dvdyo = O.sample(of, (e + 0.5) * dx, y)
    assert np.max(np.abs(v - vo)) <= 1e-13 * np.max(np.abs(vo))
    assert np.max(np.abs(dvdy - dvdyo)) <= 1e-13 * np.max(np.abs(dvdyo))


def test_cell_polynomial_store_identity(O):
    """The FP64 cell-polynomial store's algebra: inside row cell j the
    x-filtered interpolant at x = (e + 1/2) dx is the cubic
    v0 + dy t (q0 + t (q1/2 + t q2/3)) with dV/dy = q0 + t (q1 + t q2), whose
    coefficients are fixed combinations of the x sums E of rows j-1 .. j+2.
    Evaluated that way it reproduces the oracle's 16-tap value and dV/dy (to
    rounding; the sum's order aside), including rows that wrap."""
    nx, ny, Lx, Ly = 64, 16, 64.0, 5.6                    # dy = 0.35: not a power of two
    rng = np.random.default_rng(12)
    fld = rng.standard_normal((nx, ny))
    of = O.BSplineField(fld, Lx, Ly)
    c = of.coef                                           # [nx][ny], y fastest
    w = np.array([1.0, 23.0, 23.0, 1.0]) / 48.0
    E = sum(w[a] * np.roll(c, 1 - a, axis=0) for a in range(4))
    dx, dy = Lx / nx, Ly / ny
    Eb = [np.roll(E, 1 - b, axis=1) for b in range(4)]    # Eb[b][e, j] = E[e, j - 1 + b]
    q0 = 0.5 * (Eb[2] - Eb[0]) / dy
    q1 = ((Eb[0] + Eb[2]) - 2.0 * Eb[1]) / dy
    q2 = 0.5 * ((Eb[3] - Eb[0]) + 3.0 * (Eb[1] - Eb[2])) / dy
    v0 = (Eb[0] + 4.0 * Eb[1] + Eb[2]) / 6.0
    e = np.repeat(np.arange(nx - 1), 7)
    y = rng.uniform(-2 * Ly, 3 * Ly, e.size)
    gy = y / dy
    iy = np.floor(gy).astype(int)
    t = gy - iy
    j = iy % ny
    dv = q0[e, j] + t * (q1[e, j] + t * q2[e, j])
    v = v0[e, j] + dy * t * (q0[e, j] + t * (0.5 * q1[e, j] + t * q2[e, j] / 3.0))
    vo, _, dvo = O.sample(of, (e + 0.5) * dx, y)
    assert np.max(np.abs(v - vo)) <= 1e-13 * np.max(np.abs(vo))
    assert np.max(np.abs(dv - dvo)) <= 1e-13 * np.max(np.abs(dvo))


def test_oracle_dynamics_known_answers(O):
    """The oracle's Langevin step against the reference's dynamics known
    answers (test_dynamics.cpp:40-161), harmonic trough k = 4, linear model,
    dx = 1; the oracle takes the N(0,1) increments from the caller."""
    rng = np.random.default_rng(0)
    # T = 0 is gradient descent: the energy never rises and relaxes to 0 (44-65)
    n = 64
    p, well = O.params(float(n), 1.0, 0.0, 0), O.HarmonicWell(4.0, 0.0)
    h = rng.uniform(-0.5, 0.5, n)
    zero = np.zeros(n)
    e_prev = O.objective(h, p, well)
    for _ in range(2000):
        O.langevin_step(h, p, well, 0.05, 0.0, zero)
        e = O.objective(h, p, well)
        assert e <= e_prev + 1e-12
        e_prev = e
    assert e_prev < 1e-6
    # a driving force shifts the equilibrium to y0 + f/k (106-130)
    n, k, y0, f = 32, 4.0, 0.2, 0.6
    p, well = O.params(float(n), 1.0, f, 0), O.HarmonicWell(k, y0)
    h = np.zeros(n)
    for _ in range(5000):
        O.langevin_step(h, p, well, 0.05, 0.0, np.zeros(n))
    assert np.max(np.abs(h - (y0 + f / k))) < 1e-6
    # diff = 0 ignores the increments entirely (137-161)
    n = 48
    p, well = O.params(float(n), 1.0, 0.3, 0), O.HarmonicWell(4.0, 0.1)
    h1 = rng.uniform(-0.5, 0.5, n)
    h2 = h1.copy()
    for _ in range(50):
        O.langevin_step(h1, p, well, 0.05, 0.0, rng.standard_normal(n))
        O.langevin_step(h2, p, well, 0.05, 0.0, rng.standard_normal(n))
    assert np.array_equal(h1, h2)


def test_oracle_equipartition(O):
    """<E> = (N/2) kT with kT = diff^2 / (2 drift) (test_dynamics.cpp:70-99),
    within 10 %, on a shorter run than the reference's."""
    n, drift, kT = 16, 0.02, 0.05
    diff = np.sqrt(2 * drift * kT)
    p, well = O.params(float(n), 1.0, 0.0, 0), O.HarmonicWell(4.0, 0.0)
    rng = np.random.default_rng(2024)
    h = np.zeros(n)
    n_equil, n_sample, block = 5000, 60000, 5000
    for _ in range(n_equil // block):
        for xi in rng.standard_normal((block, n)):
            O.langevin_step(h, p, well, drift, diff, xi)
    total = 0.0
    for _ in range(n_sample // block):
        for xi in rng.standard_normal((block, n)):
            O.langevin_step(h, p, well, drift, diff, xi)
            total += O.objective(h, p, well)
    mean_e, expected = total / n_sample, 0.5 * n * kT
    assert abs(mean_e - expected) < 0.1 * expected, mean_e


def test_oracle_seeded_field_amplitude_and_band_limit(O):
    """The seeded generator's known answer (test_filtered_noise.cpp:68-111): the
    field's population std is the amplitude, and its Fourier modes outside the
    correlation ellipse (fx xi_x)^2 + (fy xi_y)^2 > 1 vanish."""
    nx, ny, Lx, Ly, amp, xi_x, xi_y = 128, 96, 4.0, 1.0, 2.0, 0.2, 0.1
    f = O.seeded_field(nx, ny, Lx, Ly, amp, xi_x, xi_y, 42)
    assert f.shape == (nx, ny)
    assert abs(f.std() - amp) < 1e-10
    mag = np.abs(np.fft.fft2(f))
    fx = np.fft.fftfreq(nx, d=Lx / nx)[:, None]
    fy = np.fft.fftfreq(ny, d=Ly / ny)[None, :]
    masked = (fx * xi_x) ** 2 + (fy * xi_y) ** 2 > 1.0
    assert masked.any() and (~masked).sum() > 1
    assert mag[masked].max() < 1e-8 * mag.max()


def _seeded_bspline(O, nx, ny, Lx, Ly, amp, xi, seed):
    """FilteredNoise(nx, ny, Lx, Ly, amp, xi, xi, seed) of the reference."""
    return O.BSplineField(O.seeded_field(nx, ny, Lx, Ly, amp, xi, xi, seed), Lx, Ly)


def _max_site_velocity(O, h, p, f):
    return float(np.max(-O.gradient(h, p, f)))


def test_rk_blocked_config_forward_and_arrested(O):
    """test_rosso_krauth.cpp:143-186 (linear) and 250-291 (arclength): the
    blocked line lies forward of the flat start and no site has a positive
    velocity."""
    for (amp, seed, lt, force, model) in ((0.5, 7, 1.0, 0.0, 0), (0.6, 29, 1.2, 0.1, 1)):
        nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
        f = _seeded_bspline(O, nx, ny, Lx, Ly, amp, 0.2, seed)
        p = O.params(Lx, lt, force, model)
        h = np.full(nx, 0.5 * Ly)
        h0 = h.copy()
        r = O.rk_block(h, p, f, O.rk_params(0.5 * Ly / ny, Ly, 1e-11, 1e-9, 3 * Ly, 200000))
        assert r.blocked
        assert np.all(h >= h0 - 1e-12)
        assert _max_site_velocity(O, h, p, f) < 1e-6


def test_rk_deterministic(O):
    """test_rosso_krauth.cpp:189-216: the same force and start give the same
    blocked line, bit for bit (arclength, f = 0.3)."""
    nx, ny, Lx, Ly = 48, 48, 2.4, 1.0
    f = _seeded_bspline(O, nx, ny, Lx, Ly, 0.5, 0.2, 9)
    p = O.params(Lx, 1.5, 0.3, 1)
    rp = O.rk_params(0.5 * Ly / ny, Ly, 1e-11, 1e-9, 5 * Ly, 200000)
    a, b = np.full(nx, 0.5 * Ly), np.full(nx, 0.5 * Ly)
    O.rk_block(a, p, f, rp)
    O.rk_block(b, p, f, rp)
    assert np.array_equal(a, b)


def test_rk_runaway_flag(O):
    """test_rosso_krauth.cpp:223-248: at twice the washboard's f_c the sweep
    reports runaway (not merely not blocked) past the runaway distance."""
    n, A, k = 16, 0.1, 2 * PI
    lam = 2 * PI / k
    p = O.params(float(n), 1.0, 2.0 * A * k, 0)
    rp = O.rk_params(lam / 200, lam, 1e-12, 1e-11, 3 * lam, 100000)
    r = O.rk_block(np.zeros(n), p, O.SinusoidNoise(A, k), rp)
    assert r.runaway and not r.blocked
    assert r.mean_h > rp.runaway


def test_lbfgs_restart_fast_fire_and_preconditioner(O):
    """test_lbfgs.cpp:200-304 on the oracle: a clamped line search (max_ls = 3)
    takes the restart branch where the normal budget converges without one; a
    quadratic converges in < 200 iterations; L-BFGS and FIRE reach the same
    minimum to 1e-5; the preconditioner converges a stiff line (Gamma = 50,
    dx = 0.01) in < 300 iterations, fewer than without it."""
    import math
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    f = _seeded_bspline(O, nx, ny, Lx, Ly, 2.0, 0.15, 3)
    p = O.params(Lx, 0.5, 0.0, 0)
    h = np.full(nx, 0.5 * Ly)
    r = O.lbfgs_minimize(h, p, f, O.lbfgs_default_params(ftol=1e-6, max_iter=50000, max_ls=3))
    assert r.n_ls_restarts > 0
    h = np.full(nx, 0.5 * Ly)
    r = O.lbfgs_minimize(h, p, f, O.lbfgs_default_params(ftol=1e-6, max_iter=50000, max_ls=30))
    assert r.converged and r.n_ls_restarts == 0

    n = 128
    h = np.zeros(n)
    r = O.lbfgs_minimize(h, O.params(float(n), 1.0, 0.0, 0), O.HarmonicWell(1.0, 0.3),
                         O.lbfgs_default_params(ftol=1e-8))
    assert r.converged and r.iterations < 200

    n = 96
    p = O.params(float(n), 1.0, 0.0, 0)
    init = np.random.default_rng(3).uniform(0.0, 1.0, n)
    a, b = init.copy(), init.copy()
    O.lbfgs_minimize(a, p, O.HarmonicWell(1.5, 0.4), O.lbfgs_default_params(ftol=1e-9))
    O.fire_minimize(b, p, O.HarmonicWell(1.5, 0.4), O.fire_params(0.1 * math.sqrt(1.0), ftol=1e-9))
    assert np.max(np.abs(a - b)) < 1e-5

    nx, ny, Lx, Ly = 256, 64, 2.56, 1.0
    f = _seeded_bspline(O, nx, ny, Lx, Ly, 0.3, 0.2, 5)
    p = O.params(Lx, 50.0, 0.0, 0)
    h = np.full(nx, 0.5 * Ly)
    r = O.lbfgs_minimize(h, p, f, O.lbfgs_default_params(ftol=1e-6, max_iter=5000,
                                                         precondition=1))
    assert r.converged and r.iterations < 300
    h = np.full(nx, 0.5 * Ly)
    r2 = O.lbfgs_minimize(h, p, f, O.lbfgs_default_params(ftol=1e-6, max_iter=5000,
                                                          precondition=0))
    assert r.iterations < r2.iterations


def test_oracle_fire_lowers_energy_and_is_deterministic(O):
    """test_fire.cpp:108-160 on the oracle: FIRE does not raise the energy
    (arclength, random start) and identical inputs give identical results."""
    import math
    n = 96
    p = O.params(float(n), 1.0, 0.0, 1)
    well = O.HarmonicWell(1.5, 0.6)
    h = np.random.default_rng(1).uniform(0.0, 1.0, n)
    e0 = O.objective(h, p, well)
    O.fire_minimize(h, p, well, O.fire_params(0.1 * math.sqrt(1.0), ftol=1e-9))
    assert O.objective(h, p, well) <= e0 + 1e-12
    n = 64
    p = O.params(float(n), 1.0, 0.0, 0)
    well = O.HarmonicWell(1.0, 0.5)
    init = 0.3 * np.sin(2 * np.pi * np.arange(n) / n)
    a, b = init.copy(), init.copy()
    fp = O.fire_params(0.1, ftol=1e-10)
    r1, r2 = O.fire_minimize(a, p, well, fp), O.fire_minimize(b, p, well, fp)
    assert r1.iterations == r2.iterations and np.array_equal(a, b)
