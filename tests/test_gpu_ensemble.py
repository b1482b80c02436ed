"""Batched ensemble statics and the on-device field generator."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import band_limited_field

pytestmark = pytest.mark.gpu
FTOL = 1e-8


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def npy(t):
    return t.detach().cpu().numpy()


def test_generated_field_statistics(Q):
    nx, ny, xi = 512, 256, 4.0
    store = Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32
    f = Q.FilteredNoise.generated(nx, ny, float(nx), float(ny), 1.0, xi, xi, 7, store=store)
    g = Q.FilteredNoise.generated(nx, ny, float(nx), float(ny), 1.0, xi, xi, 7, store=store)
    h = Q.FilteredNoise.generated(nx, ny, float(nx), float(ny), 1.0, xi, xi, 8, store=store)
    c, cg, ch = f.coefficients(), g.coefficients(), h.coefficients()
    assert np.array_equal(c, cg)                 # deterministic in the seed
    assert not np.allclose(c, ch)
    # the field itself is the interpolant at the nodes
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    v = npy(f.sample(ii.ravel().astype(float), jj.ravel().astype(float))[0]).reshape(nx, ny)
    assert abs(v.std() - 1.0) < 1e-9              # population std = amplitude
    assert abs(v.mean()) < 0.2
    # Gaussian correlation exp(-r^2 / (4 xi^2)) of a Gaussian filter of std xi
    r = 4
    corr = np.mean((v - v.mean()) * (np.roll(v, r, axis=0) - v.mean())) / v.var()
    assert abs(corr - np.exp(-r * r / (4 * xi * xi))) < 0.1


def _c3_lines(Q, count, seed, lmin=256, lmax=2048, edge=False):
    rng = np.random.default_rng(seed)
    lines = []
    store = Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32 | (Q.QEW_STORE_FP32_EDGE if edge else 0)
    for k in range(count):
        L = int(round(np.exp(rng.uniform(np.log(lmin), np.log(lmax))) / 2)) * 2
        xi = rng.uniform(2, 8)
        model = Q.Model(int(rng.integers(0, 2)))
        f = Q.FilteredNoise.generated(L, 256, float(L), 256.0, 1.0, xi, xi, 1000 + k, store=store)
        h = t64(np.zeros(L))
        lines.append((h, Q.Params(float(L), 1.0, 0.0, model), f, 0.5 / xi ** 2))
    return lines


@pytest.mark.parametrize("ftol32, edge", [(0.0, False), (2e-5, False), (2e-5, True)])
def test_ensemble_reaches_fp64_tolerance(Q, ftol32, edge):
    lines = _c3_lines(Q, 48, 3, edge=edge)
    lp = Q.LbfgsParams(m=10, ftol=FTOL, max_iter=20000, precondition=True, ls_fallback=True)
    res = Q.ensemble_minimize(lines, lp, ftol_fp32=ftol32)
    for (h, p, f, _), r in zip(lines, res):
        assert r.converged, r
        g = npy(Q.gradient(h, p, f))      # independent FP64 check of the final line
        assert np.max(np.abs(g)) < FTOL


def test_ensemble_matches_single_line_solver(Q, O):
    """On stiff lines with weak disorder (a unique minimum) the ensemble, the
    single-line resident solver and the oracle reach the same minimiser."""
    rng = np.random.default_rng(5)
    lines, ref = [], []
    for k, n in enumerate([96, 256, 500, 1024]):
        Lx, Ly = n * 0.01, 1.0
        fld = band_limited_field(n, 64, Lx, Ly, 0.3, 0.2, 10 + k)
        f = Q.FilteredNoise(fld, Lx, Ly, store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
        p = Q.Params(Lx, 20.0, 0.0, Q.Model(k % 2))
        h0 = 0.5 + 0.01 * rng.standard_normal(n)
        lines.append((t64(h0), p, f, 0.0))
        ref.append((h0, p, f, fld, Lx, Ly))
    lp = Q.LbfgsParams(m=10, ftol=1e-9, max_iter=20000, precondition=True, ls_fallback=True)
    res = Q.ensemble_minimize(lines, lp, ftol_fp32=1e-5)
    for (h, p, f, _), r, (h0, _, _, fld, Lx, Ly) in zip(lines, res, ref):
        assert r.converged
        hs = t64(h0)
        rs = Q.lbfgs_minimize(hs, p, f, lp)
        assert rs.converged
        assert np.max(np.abs(npy(h) - npy(hs))) < 1e-6
        of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
        ho = h0.copy()
        ro = O.lbfgs_minimize(ho, O.params(Lx, p.line_tension, 0.0, int(p.model)), of,
                              O.lbfgs_default_params(m=10, ftol=1e-9, max_iter=20000,
                                                     precondition=1, ls_fallback=1))
        assert ro.converged and np.max(np.abs(npy(h) - ho)) < 1e-6


def test_ensemble_rejects_missing_fp32(Q):
    f = Q.FilteredNoise(band_limited_field(64, 32, 3.2, 1.0, 1.0, 0.3, 1), 3.2, 1.0)
    lines = [(t64(np.zeros(64)), Q.Params(3.2), f, 0.0)]
    with pytest.raises(ValueError, match="FP32"):
        Q.ensemble_minimize(lines, Q.LbfgsParams(), ftol_fp32=1e-5)


@pytest.mark.parametrize("form", [0, 1])
def test_fallback_reaches_1e8_where_armijo_stalls(Q, O, form):
    """A C3-shaped line on which the reference's Armijo search alone stalls
    above 1e-8: with the fallback both GPU forms and the oracle converge."""
    from conftest import gaussian_field
    L, xi = 4096, 2.56
    fld = gaussian_field(L, 256, xi, 4096)
    f = Q.FilteredNoise(fld, float(L), 256.0)
    p = Q.Params(float(L), 1.0, 0.0, Q.Model.Linear)
    lp = Q.LbfgsParams(m=10, ftol=FTOL, max_iter=20000, precondition=True,
                       precond_shift=0.5 / xi ** 2, ls_fallback=True)
    h = t64(np.zeros(L))
    r = Q.lbfgs_minimize(h, p, f, lp, form=form)
    assert r.converged and np.max(np.abs(npy(Q.gradient(h, p, f)))) < FTOL
