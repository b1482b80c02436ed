"""FP64 gradient on the cell-polynomial store (QEW_STORE_FP64_POLY) against
the FP64 oracle.

Bar: energy and gradient within 1e-12 relative (to the largest magnitude of
the compared vector), the FP64 parity bar. The store re-associates the
reference's tensor sum, so it is not bitwise equal to the reference's order;
against the reference-order kernel on the same field it agrees to 1e-13.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import band_limited_field, gaussian_field

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def npy(t):
    return t.detach().cpu().numpy()


def close(a, b, rtol=RTOL):
    scale = max(float(np.max(np.abs(b))), 1e-300)
    err = float(np.max(np.abs(np.asarray(a) - np.asarray(b))))
    assert err <= rtol * scale, "max err %.3e vs scale %.3e" % (err, scale)


def poly_field(Q, fld, Lx, Ly):
    return Q.FilteredNoise(fld, Lx, Ly, store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY)


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("shape", [(1, 8, 1.0, 8.0), (2, 8, 2.0, 8.0), (3, 5, 3.0, 5.0),
                                   (96, 40, 4.8, 1.3), (257, 33, 257.0, 33.0),
                                   (1000, 48, 1000.0, 12.0), (4096, 64, 4096.0, 64.0)])
def test_poly_gradient_matches_oracle(Q, O, model, shape):
    """One point per field column, power-of-two and other row spacings,
    heights that leave [0, Ly) on both sides (the reference's fold)."""
    nx, ny, Lx, Ly = shape
    fld = band_limited_field(nx, ny, Lx, Ly, 1.0, 0.3 * Ly, nx + 7 * ny)
    f = poly_field(Q, fld, Lx, Ly)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    rng = np.random.default_rng(nx + model)
    h = rng.uniform(-1.5 * Ly, 2.5 * Ly, nx)
    h[::7] = rng.uniform(0, Ly, h[::7].size)
    p = Q.Params(Lx, 1.3, 0.37, Q.Model(model))
    po = O.params(Lx, 1.3, 0.37, model)
    go = O.gradient(h, po, of)
    g = npy(Q.gradient(t64(h), p, f))
    close(g, go)
    # the reference-order kernel on the same field
    gr = npy(Q.gradient(t64(h), p, f, precision=Q.QEW_PREC_FP64_REFERENCE))
    close(g, gr, 1e-13)
    close(gr, go)


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("scale", [1.0, 0.25, 3.0])
def test_poly_zero_force_form_is_the_general_form(Q, O, model, scale):
    """At f = 0 with dx/2 a power of two the store gather forms (dx/2) dv on
    each edge by moving dv's exponent; the gradient equals, bit for bit, the
    general form's at a force too small to change any sum (1e-300): with
    dx/2 = 2^k the general combine fma(dx/2, S, -dx f) is an exact scaling
    plus a negligible term. Both match the oracle at f = 0 to the bar. (At
    dx = 3 the general form runs at f = 0 as well; there the product 1.5 S
    is not exact, so the tiny force may tip a rounding tie and only the
    oracle bar applies.)"""
    import torch
    nx, ny = 3000, 40
    Lx = nx * scale
    fld = gaussian_field(nx, ny, 3.0, 31)
    f = poly_field(Q, fld, Lx, float(ny))
    of = O.BSplineField(fld, Lx, float(ny), coef=f.coefficients())
    rng = np.random.default_rng(model + 11)
    h = ny / 2 + np.cumsum(rng.standard_normal(nx)) * 0.4
    h -= np.linspace(0, h[-1] - h[0], nx)
    h[:8] = [0.0, -0.0, 1e-310, 2.0, 2.0, -3.5, 1e6, 0.5]
    hb = t64(np.stack([h, h[::-1].copy()]))
    g0 = Q.gradient_batch(hb, Q.Params(Lx, 1.2, 0.0, Q.Model(model)), f)
    gt = Q.gradient_batch(hb, Q.Params(Lx, 1.2, 1e-300, Q.Model(model)), f)
    if scale != 3.0:
        assert torch.equal(g0.view(torch.int64), gt.view(torch.int64))
    close(npy(g0[0]), O.gradient(h, O.params(Lx, 1.2, 0.0, model), of))


def test_poly_cell_boundaries_and_special_heights(Q, O):
    """Heights on exact cell boundaries, zero, tiny and negative values, and
    far outside the field: the bit-level floor/fraction agrees with the
    reference's floor and fold (the results match the oracle to the bar)."""
    nx, ny = 512, 32
    Lx, Ly = float(nx), 8.0  # dy = 0.25
    fld = gaussian_field(nx, ny, 3.0, 21)
    f = poly_field(Q, fld, Lx, Ly)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    rng = np.random.default_rng(5)
    specials = np.array([0.0, -0.0, 5e-324, 1e-310, 1e-300, 0.125, 0.25, 0.375, 7.75, 7.999999,
                         8.0, 8.25, -0.25, -1e-17, 1e-17, 1e6, -1e6, 0.5, 3.0, 4.0])
    h = rng.uniform(0, Ly, nx)
    h[: specials.size] = specials
    h[100:200] = np.round(h[100:200] * 4) / 4       # midpoints on cell boundaries
    for model in (0, 1):
        p = Q.Params(Lx, 0.9, -0.2, Q.Model(model))
        po = O.params(Lx, 0.9, -0.2, model)
        close(npy(Q.gradient(t64(h), p, f)), O.gradient(h, po, of))


def test_poly_batch_equals_single_lines(Q):
    """The batched persistent launch gives every line what a per-line call
    gives, bit for bit, for batches shorter and longer than one wave."""
    import torch
    nx, ny = 3000, 48
    f = poly_field(Q, gaussian_field(nx, ny, 4.0, 2), float(nx), float(ny))
    rng = np.random.default_rng(9)
    for count in (1, 3, 17):
        h = t64(ny / 2 + np.cumsum(rng.standard_normal((count, nx)), axis=1) * 0.3)
        for model in (0, 1):
            p = Q.Params(float(nx), 1.0, 0.1, Q.Model(model))
            gb = Q.gradient_batch(h, p, f)
            for k in range(count):
                assert torch.equal(gb[k], Q.gradient(h[k].contiguous(), p, f))
    # a field without the store: the batch is one reference-order launch per line
    f2 = Q.FilteredNoise(gaussian_field(nx, ny, 4.0, 2), float(nx), float(ny))
    h = t64(ny / 2 + rng.standard_normal((2, nx)))
    p = Q.Params(float(nx), 1.0, 0.1, Q.Model.Linear)
    gb = Q.gradient_batch(h, p, f2)
    for k in range(2):
        assert torch.equal(gb[k], Q.gradient(h[k].contiguous(), p, f2))


def test_poly_other_lines_ignore_the_store(Q):
    """A line that does not have one point per field column (n != nx, or a
    different physical length) takes the reference-order kernel, bitwise."""
    import torch
    nx, ny = 600, 32
    fld = gaussian_field(nx, ny, 3.0, 4)
    fp = poly_field(Q, fld, float(nx), float(ny))
    f0 = Q.FilteredNoise(fld, float(nx), float(ny))
    rng = np.random.default_rng(1)
    for n, P in ((500, float(nx)), (600, 300.0)):
        h = t64(rng.uniform(0, ny, n))
        p = Q.Params(P, 1.0, 0.0, Q.Model.Linear)
        assert torch.equal(Q.gradient(h, p, fp), Q.gradient(h, p, f0))


def test_poly_store_needs_fp64(Q):
    with pytest.raises(ValueError, match="QEW_STORE_FP64_POLY needs QEW_STORE_FP64"):
        Q.FilteredNoise(np.zeros((16, 8)), 16.0, 8.0,
                        store=Q.QEW_STORE_FP32 | Q.QEW_STORE_FP64_POLY)


def test_poly_full_size_line(Q, O):
    """A 2^20-point line on a 2^20 x 64 field, both models, against the
    OpenMP oracle on the same (downloaded) coefficients."""
    import torch
    n, ny = 1 << 20, 64
    rng = np.random.default_rng(6)
    fld = rng.standard_normal((n, ny))
    f = poly_field(Q, fld, float(n), float(ny))
    of = O.BSplineField(fld, float(n), float(ny), coef=f.coefficients())
    h = 32 + np.cumsum(rng.standard_normal(n)) * 0.05
    for model in (0, 1):
        p = Q.Params(float(n), 1.0, 0.3, Q.Model(model))
        g = npy(Q.gradient(t64(h), p, f))
        close(g, O.gradient(h, O.params(float(n), 1.0, 0.3, model), of, omp=True))
    del f
    torch.cuda.empty_cache()


def test_host_batch_mapped_and_copied_agree(Q):
    """qew_gradient_host_batch with pinned host buffers runs the kernels on
    the mapped host memory (no copies); with a pageable output it takes the
    copy pipeline. Both give exactly the device-resident gradient, for every
    precision."""
    import torch
    nx, ny = 2048, 32
    f = Q.FilteredNoise(gaussian_field(nx, ny, 3.0, 8), float(nx), float(ny),
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY | Q.QEW_STORE_FP32)
    rng = np.random.default_rng(12)
    count = 5
    h = torch.as_tensor(ny / 2 + rng.standard_normal((count, nx))).pin_memory().numpy()
    for model in (0, 1):
        p = Q.Params(float(nx), 1.1, 0.05, Q.Model(model))
        for prec in (Q.QEW_PREC_FP64, Q.QEW_PREC_FP64_REFERENCE, Q.QEW_PREC_FP32_SPLIT):
            pinned = torch.empty((count, nx), dtype=torch.float64).pin_memory().numpy()
            Q.gradient_host_batch(h, p, f, pinned, precision=prec)
            pageable = Q.gradient_host_batch(h, p, f, np.empty((count, nx)), precision=prec)
            dev = npy(Q.gradient_batch(t64(h), p, f, precision=prec)) \
                if prec != Q.QEW_PREC_FP32_SPLIT else \
                np.stack([npy(Q.gradient(t64(h[k]), p, f, precision=prec)) for k in range(count)])
            assert np.array_equal(pinned, dev)
            assert np.array_equal(pageable, dev)
            one = torch.empty(nx, dtype=torch.float64).pin_memory().numpy()
            Q.gradient_host(h[2].copy(), p, f, one, precision=prec)
            assert np.array_equal(one, dev[2])


def test_poly_objective_and_solvers_match_oracle(Q, O):
    """The store serves every FP64 consumer of the field on such a line: the
    energy (the polynomial's value), the site velocities of the Rosso-Krauth
    construction, a Langevin step with given increments and a preconditioned
    L-BFGS solve agree with the oracle's reference-order arithmetic."""
    nx, ny = 1024, 64
    fld = gaussian_field(nx, ny, 4.0, 31)
    f = poly_field(Q, fld, float(nx), float(ny))
    of = O.BSplineField(fld, float(nx), float(ny), coef=f.coefficients())
    rng = np.random.default_rng(4)
    h = ny / 2 + np.cumsum(rng.standard_normal(nx)) * 0.2
    h -= np.linspace(0, h[-1] - h[0], nx)
    for model in (0, 1):
        p = Q.Params(float(nx), 1.2, 0.15, Q.Model(model))
        po = O.params(float(nx), 1.2, 0.15, model)
        e, eo = Q.objective(t64(h), p, f), O.objective(h, po, of)
        assert abs(e - eo) <= 1e-12 * abs(eo)
        v = npy(Q.rk_site_velocity(t64(h), p, f))
        close(v, -O.gradient(h, po, of))
        xi = rng.standard_normal(nx)
        hl = t64(h)
        Q.LangevinDynamics(nx, 1).step_with_increments(hl, p, f, 0.01, 0.05, t64(xi))
        ho = h.copy()
        O.langevin_step(ho, po, of, 0.01, 0.05, xi)
        close(npy(hl), ho)
    p = Q.Params(float(nx), 1.0, 0.0, Q.Model.Linear)
    lp = Q.LbfgsParams(m=10, ftol=1e-8, max_iter=2000, precondition=True, precond_shift=0.03,
                       ls_fallback=True)
    hg = t64(np.full(nx, ny / 2))
    r = Q.lbfgs_minimize(hg, p, f, lp)
    ho = np.full(nx, ny / 2)
    ro = O.lbfgs_minimize(ho, O.params(float(nx), 1.0, 0.0, 0), of,
                          O.lbfgs_default_params(m=10, ftol=1e-8, max_iter=2000, precondition=1,
                                                 precond_shift=0.03, ls_fallback=1))
    assert r.converged and ro.converged
    assert np.max(np.abs(npy(hg) - ho)) < 1e-7
    e, eo = Q.objective(hg, p, f), O.objective(ho, O.params(float(nx), 1.0, 0.0, 0), of)
    assert abs(e - eo) <= 1e-12 * abs(eo)


def test_poly_rk_block_close_to_reference_order(Q, O):
    """Rosso-Krauth sweeps on the store: the oracle's verdict, the sweep count
    within one, lines within rounding-level distances."""
    n, ny = 512, 64
    fld = gaussian_field(n, ny, 4.0, 41)
    f = poly_field(Q, fld, float(n), float(ny))
    of = O.BSplineField(fld, float(n), float(ny), coef=f.coefficients())
    rp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * ny, max_sweeps=3000)
    orp = O.rk_params(0.5, float(ny), 1e-10, 1e-8, 2.0 * ny, 3000)
    for fdr in (0.0, 0.05):
        hg = t64(np.full(n, ny / 2))
        r = Q.rk_block(hg, Q.Params(float(n), 1.0, fdr, Q.Model.Linear), f, rp)
        ho = np.full(n, ny / 2)
        ro = O.rk_block(ho, O.params(float(n), 1.0, fdr, 0), of, orp)
        assert (r.blocked, r.runaway) == (bool(ro.blocked), bool(ro.runaway))
        assert abs(r.sweeps - ro.sweeps) <= 1
        assert np.max(np.abs(npy(hg) - ho)) < 1e-8
