"""GPU Rosso-Krauth construction against the oracle and the reference's tests
(test_rosso_krauth.cpp)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import band_limited_field, gaussian_field

pytestmark = pytest.mark.gpu
PI = 3.14159265358979323846


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def npy(t):
    return t.detach().cpu().numpy()


def rkp(Q, dstep, max_adv, root_tol, sweep_tol, runaway, max_sweeps=200000):
    return Q.RkParams(dstep, max_adv, root_tol, sweep_tol, runaway, max_sweeps)


def test_velocity_is_minus_gradient(Q):
    """test_rosso_krauth.cpp:94-141: 1e-12."""
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    f = Q.FilteredNoise(band_limited_field(nx, ny, Lx, Ly, 0.7, 0.2, 13), Lx, Ly)
    h = t64(np.random.default_rng(21).uniform(0.1, 0.9, nx))
    for model in (Q.Model.Linear, Q.Model.Arclength):
        p = Q.Params(Lx, 1.3, 0.4, model)
        v = npy(Q.rk_site_velocity(h, p, f))
        g = npy(Q.gradient(h, p, f))
        assert np.max(np.abs(v + g)) < 1e-12


@pytest.mark.parametrize("model", [0, 1])
def test_rk_block_matches_oracle(Q, O, model):
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    fld = band_limited_field(nx, ny, Lx, Ly, 0.5, 0.2, 7)
    f = Q.FilteredNoise(fld, Lx, Ly)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    for fdr in (0.0, 0.3):
        h = t64(np.full(nx, 0.5))
        r = Q.rk_block(h, Q.Params(Lx, 1.0, fdr, Q.Model(model)), f,
                       rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly))
        ho = np.full(nx, 0.5)
        ro = O.rk_block(ho, O.params(Lx, 1.0, fdr, model), of,
                        O.rk_params(0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly))
        assert r.blocked == bool(ro.blocked) and r.runaway == bool(ro.runaway)
        assert r.sweeps == ro.sweeps
        assert np.max(np.abs(npy(h) - ho)) < 1e-12
        # the reference-exact arithmetic: the oracle's line bit for bit
        he = t64(np.full(nx, 0.5))
        re = Q.rk_block(he, Q.Params(Lx, 1.0, fdr, Q.Model(model)), f,
                        rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly),
                        precision=Q.QEW_PREC_FP64_REFERENCE)
        assert re.sweeps == ro.sweeps and np.array_equal(npy(he), ho)


def test_blocked_is_forward_and_arrested(Q):
    """test_rosso_krauth.cpp:145-186."""
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    f = Q.FilteredNoise(band_limited_field(nx, ny, Lx, Ly, 0.5, 0.2, 7), Lx, Ly)
    p = Q.Params(Lx, 1.0, 0.0, Q.Model.Linear)
    h = t64(np.full(nx, 0.5))
    r = Q.rk_block(h, p, f, rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly))
    assert r.blocked
    assert np.all(npy(h) >= 0.5 - 1e-12)
    assert np.max(-npy(Q.gradient(h, p, f))) < 1e-6


def test_arclength_blocks(Q):
    """test_rosso_krauth.cpp:255-291."""
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    f = Q.FilteredNoise(band_limited_field(nx, ny, Lx, Ly, 0.6, 0.2, 29), Lx, Ly)
    p = Q.Params(Lx, 1.2, 0.1, Q.Model.Arclength)
    h = t64(np.full(nx, 0.5))
    r = Q.rk_block(h, p, f, rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly))
    assert r.blocked and np.max(-npy(Q.gradient(h, p, f))) < 1e-6


def test_deterministic(Q):
    """test_rosso_krauth.cpp:189-216 (bitwise)."""
    nx, ny, Lx, Ly = 48, 48, 2.4, 1.0
    f = Q.FilteredNoise(band_limited_field(nx, ny, Lx, Ly, 0.5, 0.2, 9), Lx, Ly)
    p = Q.Params(Lx, 1.5, 0.3, Q.Model.Arclength)
    rp = rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 5 * Ly)
    h1, h2 = t64(np.full(nx, 0.5)), t64(np.full(nx, 0.5))
    Q.rk_block(h1, p, f, rp)
    Q.rk_block(h2, p, f, rp)
    assert np.array_equal(npy(h1), npy(h2))


def test_washboard_fc_and_runaway(Q):
    """test_rosso_krauth.cpp:51-89 and 223-248."""
    n, A, k = 16, 0.1, 2 * PI
    lam = 2 * PI / k
    nz = Q.SinusoidNoise(A, k)
    rp = rkp(Q, lam / 200, lam, 1e-12, 1e-11, 3 * lam, 100000)

    def blocks(fdr):
        return Q.rk_block(t64(np.zeros(n)), Q.Params(float(n), 1.0, fdr, Q.Model.Linear), nz,
                          rp).blocked

    lo, hi = 0.0, 2 * A * k
    assert blocks(lo) and not blocks(hi)
    for _ in range(40):
        m = 0.5 * (lo + hi)
        if blocks(m):
            lo = m
        else:
            hi = m
    assert abs(0.5 * (lo + hi) - A * k) < 0.02 * A * k
    h = t64(np.zeros(n))
    r = Q.rk_block(h, Q.Params(float(n), 1.0, 2 * A * k, Q.Model.Linear), nz, rp)
    assert r.runaway and not r.blocked and r.mean_h > rp.runaway


def test_odd_length_rejected(Q):
    """test_rosso_krauth.cpp:296-313: ValueError where the reference throws."""
    with pytest.raises(ValueError, match="even"):
        Q.rk_block(t64(np.zeros(17)), Q.Params(17.0), Q.SinusoidNoise(),
                   rkp(Q, 0.01, 1.0, 1e-10, 1e-9, 3.0))


def test_bisect_matches_oracle(Q, O):
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    fld = band_limited_field(nx, ny, Lx, Ly, 0.5, 0.2, 7)
    f = Q.FilteredNoise(fld, Lx, Ly)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    rp = rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly, 50000)
    orp = O.rk_params(0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly, 50000)
    h = t64(np.full(nx, 0.5))
    p = Q.Params(Lx, 1.0, 0.0, Q.Model.Linear)
    assert Q.rk_block(h, p, f, rp).blocked
    ho = npy(h).copy()
    fc, flo, fhi, nb = Q.depinning_bisect(h, p, f, rp, 0.0, 4.0, rtol=1e-6, max_steps=60)
    fco, flo_o, fhi_o, nbo = O.depinning_bisect(ho, O.params(Lx, 1.0, 0.0, 0), of, orp, 0.0, 4.0,
                                                1e-6, 60)
    assert abs(fc - fco) <= 1e-6 * fco
    assert np.max(np.abs(npy(h) - ho)) < 1e-6


@pytest.mark.parametrize("model", [0, 1])
def test_resident_equals_plain_bitwise(Q, model):
    """The persistent kernel and the host-driven loop run the same per-site
    arithmetic: identical lines and verdicts."""
    nx, ny, Lx, Ly = 128, 64, 6.4, 1.0
    f = Q.FilteredNoise(band_limited_field(nx, ny, Lx, Ly, 0.6, 0.2, 31), Lx, Ly)
    rp = rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly)
    for fdr in (0.0, 0.25, 5.0):
        p = Q.Params(Lx, 1.1, fdr, Q.Model(model))
        h1, h2 = t64(np.full(nx, 0.5)), t64(np.full(nx, 0.5))
        r1 = Q.rk_block(h1, p, f, rp, form=Q.QEW_RK_PLAIN)
        r2 = Q.rk_block(h2, p, f, rp, form=Q.QEW_RK_RESIDENT)
        assert (r1.blocked, r1.runaway, r1.sweeps) == (r2.blocked, r2.runaway, r2.sweeps)
        assert np.array_equal(npy(h1), npy(h2))


def test_fp32_velocity_form_close_to_fp64(Q):
    nx, ny, Lx, Ly = 256, 64, 12.8, 1.0
    f = Q.FilteredNoise(band_limited_field(nx, ny, Lx, Ly, 0.5, 0.2, 5), Lx, Ly,
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
    rp = rkp(Q, 0.5 / ny, Ly, 1e-10, 1e-8, 3 * Ly)
    p = Q.Params(Lx, 1.0, 0.1, Q.Model.Linear)
    h64, h32 = t64(np.full(nx, 0.5)), t64(np.full(nx, 0.5))
    r64 = Q.rk_block(h64, p, f, rp)
    r32 = Q.rk_block(h32, p, f, rp, precision=Q.QEW_PREC_FP32_SPLIT)
    assert r64.blocked and r32.blocked
    assert np.max(np.abs(npy(h64) - npy(h32))) < 1e-4


def test_bisect_fp32_close_to_fp64(Q):
    nx, ny, Lx, Ly = 64, 64, 3.2, 1.0
    f = Q.FilteredNoise(band_limited_field(nx, ny, Lx, Ly, 0.5, 0.2, 7), Lx, Ly,
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
    rp = rkp(Q, 0.5 / ny, Ly, 1e-11, 1e-9, 3 * Ly, 50000)
    p = Q.Params(Lx, 1.0, 0.0, Q.Model.Linear)
    ha, hb = t64(np.full(nx, 0.5)), t64(np.full(nx, 0.5))
    assert Q.rk_block(ha, p, f, rp).blocked
    hb.copy_(ha)
    fa = Q.depinning_bisect(ha, p, f, rp, 0.0, 4.0, rtol=1e-6, max_steps=60)[0]
    fb = Q.depinning_bisect(hb, p, f, rp, 0.0, 4.0, rtol=1e-6, max_steps=60,
                            precision=Q.QEW_PREC_FP32_SPLIT)[0]
    assert abs(fa - fb) < 1e-4 * fa


@pytest.mark.parametrize("n", [4096, 16384, 32768])
def test_resident_equals_plain_bitwise_long_lines(Q, n):
    """Long lines take the other search widths of the resident kernel (8-lane
    groups, lane-pair evaluations, one thread per site): still the plain
    form's lines and verdicts, bit for bit."""
    ny = 64
    f = Q.FilteredNoise(gaussian_field(n, ny, 3.0, n % 97), float(n), float(ny))
    rp = rkp(Q, 0.5, float(ny), 1e-10, 1e-8, 2.0 * ny, 60)
    rng = np.random.default_rng(n)
    h0 = ny / 2 + np.cumsum(rng.standard_normal(n)) * 0.05
    for fdr in (0.05, 0.3):
        p = Q.Params(float(n), 1.0, fdr, Q.Model.Linear)
        h1, h2 = t64(h0), t64(h0)
        r1 = Q.rk_block(h1, p, f, rp, form=Q.QEW_RK_PLAIN)
        r2 = Q.rk_block(h2, p, f, rp, form=Q.QEW_RK_RESIDENT)
        assert (r1.blocked, r1.runaway, r1.sweeps) == (r2.blocked, r2.runaway, r2.sweeps)
        assert np.array_equal(npy(h1), npy(h2))
