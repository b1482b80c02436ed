"""Depinning threshold parity: f_c, the critical configuration and every
block's verdict against the oracle's restatement of the reference.

Near f_c most bisection blocks end at max_sweeps (their verdict: not
blocked), so the measured f_c is the force where "blocked within max_sweeps"
flips, and any difference in the dynamics' rounding can move it. The
reference-exact precision (QEW_PREC_FP64_REFERENCE) evaluates the reference's
expressions in its order with its roundings (true divisions, no fused
multiply-adds), as the oracle does (built with -ffp-contract=off): gradients,
velocities and every sweep's line are then equal bit for bit, and so are the
verdict sequence, f_c and the critical line. The bar of the configurations,
f_c within 1e-10 relative, is asserted; equality is what these runs show.

The knobs are those of the depinning configuration (dstep 0.5 cell,
max_advance = rows, runaway = 2 rows, root_tol 1e-10, sweep_tol 1e-8, force
ramp by 0.05 from a flat line at rows/2, then bisection to 1e-10 relative)
on an L x L Gaussian field (xi = 4 cells, seed 2, unit variance, grid
spacing 1), linear elasticity, Gamma = 1; max_sweeps is cut so the oracle
finishes in tens of seconds.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import band_limited_field, gaussian_field

pytestmark = pytest.mark.gpu


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def npy(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("shape", [(96, 40, 4.8, 1.3), (512, 64, 512.0, 64.0), (1000, 48, 1000.0, 12.0)])
def test_reference_exact_gradient_is_the_oracles(Q, O, model, shape):
    """gradient() at QEW_PREC_FP64_REFERENCE equals the oracle's, bit for bit
    (other spacings, heights folded from outside the field)."""
    nx, ny, Lx, Ly = shape
    fld = band_limited_field(nx, ny, Lx, Ly, 1.0, 0.25 * Ly, nx + ny)
    f = Q.FilteredNoise(fld, Lx, Ly)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    rng = np.random.default_rng(model + nx)
    h = rng.uniform(-Ly, 2 * Ly, nx)
    p = Q.Params(Lx, 1.3, 0.21, Q.Model(model))
    g = npy(Q.gradient(t64(h), p, f, precision=Q.QEW_PREC_FP64_REFERENCE))
    assert np.array_equal(g, O.gradient(h, O.params(Lx, 1.3, 0.21, model), of))


@pytest.mark.parametrize("form", ["plain", "resident"])
@pytest.mark.parametrize("model", [0, 1])
def test_reference_exact_rk_block_is_the_oracles(Q, O, form, model):
    """rk_block at QEW_PREC_FP64_REFERENCE: the oracle's line, sweep count and
    verdict, bit for bit, below and above the threshold."""
    n, ny = 256, 64
    fld = gaussian_field(n, ny, 4.0, 17)
    f = Q.FilteredNoise(fld, float(n), float(ny))
    of = O.BSplineField(fld, float(n), float(ny), coef=f.coefficients())
    rp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * ny, max_sweeps=3000)
    orp = O.rk_params(0.5, float(ny), 1e-10, 1e-8, 2.0 * ny, 3000)
    fm = Q.QEW_RK_PLAIN if form == "plain" else Q.QEW_RK_RESIDENT
    h = np.full(n, 0.5 * ny)
    for fdr in (0.0, 0.05, 0.1, 0.4):
        hg, ho = t64(h), h.copy()
        r = Q.rk_block(hg, Q.Params(float(n), 1.0, fdr, Q.Model(model)), f, rp, form=fm,
                       precision=Q.QEW_PREC_FP64_REFERENCE)
        ro = O.rk_block(ho, O.params(float(n), 1.0, fdr, model), of, orp)
        assert (r.blocked, r.runaway, r.sweeps) == (bool(ro.blocked), bool(ro.runaway), ro.sweeps)
        assert np.array_equal(npy(hg), ho), fdr
        if r.blocked:
            h = ho


def _ramp(step, blocked_of, fstep, fmax):
    """Force ramp (qew_runs.h:224-241): the last blocked force and the first
    that is not, with each block's verdict."""
    verdicts, k, f_lo = [], 0, None
    while k * fstep <= fmax:
        v = step(k * fstep)
        verdicts.append(v)
        if not blocked_of(v):
            return f_lo, k * fstep, verdicts
        f_lo = k * fstep
        k += 1
    return f_lo, None, verdicts


@pytest.mark.parametrize("L,ramp_sweeps,bisect_sweeps", [(512, 5000, 5000), (2048, 20000, 2000)])
def test_fc_matches_oracle_depinning_knobs(Q, O, L, ramp_sweeps, bisect_sweeps):
    """Ramp and bisection on both sides from the same field: identical ramp
    and bisection verdicts, f_c within 1e-10 relative (here: equal), and the
    critical (last blocked) line equal. (At L = 2048 the flat start needs
    more sweeps to block than the bisection is given.)"""
    fld = gaussian_field(L, L, 4.0, 2)
    f = Q.FilteredNoise(fld, float(L), float(L))
    of = O.BSplineField(fld, float(L), float(L), coef=f.coefficients())
    rp = Q.RkParams(dstep=0.5, max_advance=float(L), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * L, max_sweeps=ramp_sweeps)
    orp = O.rk_params(0.5, float(L), 1e-10, 1e-8, 2.0 * L, ramp_sweeps)
    REFP = Q.QEW_PREC_FP64_REFERENCE

    hg = t64(np.full(L, 0.5 * L))
    ho = np.full(L, 0.5 * L)

    def gpu_step(fk):
        work = hg.clone()
        r = Q.rk_block(work, Q.Params(float(L), 1.0, fk, Q.Model.Linear), f, rp, precision=REFP)
        if r.blocked:
            hg.copy_(work)
        return (r.blocked, r.runaway, r.sweeps)

    def cpu_step(fk):
        work = ho.copy()
        r = O.rk_block(work, O.params(float(L), 1.0, fk, 0), of, orp)
        if r.blocked:
            ho[:] = work
        return (bool(r.blocked), bool(r.runaway), r.sweeps)

    g_lo, g_hi, gv = _ramp(gpu_step, lambda v: v[0], 0.05, 5.0)
    c_lo, c_hi, cv = _ramp(cpu_step, lambda v: v[0], 0.05, 5.0)
    assert gv == cv
    assert (g_lo, g_hi) == (c_lo, c_hi) and g_lo is not None and g_hi is not None
    assert np.array_equal(npy(hg), ho)

    rp.max_sweeps = bisect_sweeps
    orp.max_sweeps = bisect_sweeps
    h_start = ho.copy()
    rg = Q.depinning_bisect_report(hg, Q.Params(float(L), 1.0, 0.0, Q.Model.Linear), f, rp,
                                   g_lo, g_hi, rtol=1e-10, max_steps=64, precision=REFP)
    fco, flo_o, fhi_o, vo, sweeps_o = O.depinning_bisect_verdicts(
        ho, O.params(float(L), 1.0, 0.0, 0), of, orp, c_lo, c_hi, 1e-10, 64)
    assert rg.verdicts == vo
    assert rg.sweeps == sweeps_o
    assert abs(rg.f_c - fco) <= 1e-10 * fco
    assert (rg.f_lo, rg.f_hi) == (flo_o, fhi_o)
    assert np.array_equal(npy(hg), ho)                     # the critical configuration
    assert (rg.f_hi - rg.f_lo) <= 1e-10 * rg.f_hi
    assert rg.n_blocked + rg.n_runaway + rg.n_timeout == rg.blocks == len(vo)
    # The default FP64 path (fused multiply-adds, weights by multiplication)
    # from the same blocked start: its velocities differ from the reference's
    # in the last bits, yet here too the verdicts and f_c are the oracle's.
    hd = t64(h_start)
    rd = Q.depinning_bisect_report(hd, Q.Params(float(L), 1.0, 0.0, Q.Model.Linear), f, rp,
                                   g_lo, g_hi, rtol=1e-10, max_steps=64)
    assert rd.verdicts == vo
    assert abs(rd.f_c - fco) <= 1e-10 * fco
    assert np.max(np.abs(npy(hd) - ho)) <= 1e-9   # critical lines within root_tol-scale bounds
