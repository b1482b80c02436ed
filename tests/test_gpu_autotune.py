"""The launch-shape autotuner: every candidate shape of each tuned kernel
gives bitwise-identical results, and tuning (which times the candidates on
the call's own work) leaves the call's results as the default shape's."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_field

pytestmark = pytest.mark.gpu


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _each_candidate(ctx, kernel, n_cand, fn):
    outs = []
    try:
        for c in range(n_cand):
            ctx.force_tune_candidate(kernel, c)
            outs.append(fn())
    finally:
        ctx.force_tune_candidate(kernel, -1)
    return outs


def test_gradient_candidates_bitwise_equal(Q):
    import torch
    nx, ny, count = 5000, 48, 3
    fld = gaussian_field(nx, ny, 4.0, 12)
    f = Q.FilteredNoise(fld, float(nx), float(ny),
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY | Q.QEW_STORE_FP32 |
                        Q.QEW_STORE_FP32_EDGE)
    ctx = f.ctx
    rng = np.random.default_rng(2)
    h = t64(ny / 2 + np.cumsum(rng.standard_normal((count, nx)), axis=1) * 0.3)
    cells = torch.empty((count, nx), dtype=torch.int32, device="cuda")
    fracs = torch.empty((count, nx), dtype=torch.float32, device="cuda")
    for k in range(count):
        c, fr = Q.split_heights(h[k].contiguous(), f)
        cells[k].copy_(c)
        fracs[k].copy_(fr)
    for model in (0, 1):
        p = Q.Params(float(nx), 1.1, 0.2, Q.Model(model))
        outs = _each_candidate(ctx, Q.QEW_TUNE_GRADIENT_POLY, 9,
                               lambda: Q.gradient_batch(h, p, f).clone())
        tuned = Q.gradient_batch(h, p, f)
        for o in outs[1:] + [tuned]:
            assert torch.equal(o, outs[0])
        outs = _each_candidate(ctx, Q.QEW_TUNE_GRADIENT_SPLIT, 6,
                               lambda: Q.gradient_split_batch(cells, fracs, p, f).clone())
        tuned = Q.gradient_split_batch(cells, fracs, p, f)
        for o in outs[1:] + [tuned]:
            assert torch.equal(o, outs[0])
    rep = Q.tune_report()
    assert "k_gradient_poly" in rep and "k_gradient_split_persist" in rep


def test_gradient_candidates_on_special_heights(Q):
    """Every launch shape of the store gather, bitwise, on heights that take
    its exceptional paths: zeros of both signs, opposite signs (cancelling
    midpoint sums), subnormals, exact negatives of a neighbour, values far
    outside the field, and ties of the rounding."""
    import torch
    nx, ny = 4096, 32
    f = Q.FilteredNoise(gaussian_field(nx, ny, 3.0, 8), float(nx), float(ny),
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY)
    ctx = f.ctx
    rng = np.random.default_rng(4)
    h = rng.uniform(-ny, 2 * ny, nx)
    h[0:64:2] = 0.0
    h[1:64:2] = -0.0
    h[64:128] = rng.choice([5e-324, 1e-310, -1e-310, 2.2250738585072014e-308], 64)
    h[129:256:2] = -h[128:255:2]                              # a + b == 0 exactly
    h[256:512] = np.round(h[256:512] * 2 ** 20) / 2 ** 20      # short mantissas: exact sums
    h[512:520] = [1.0, 2.0 ** -53, 1.0, 3 * 2.0 ** -53, 1e12, -1e12, 1e6, -1e6]
    ht = t64(h).reshape(1, nx)
    for model in (0, 1):
        p = Q.Params(float(nx), 1.3, 0.1, Q.Model(model))
        outs = _each_candidate(ctx, Q.QEW_TUNE_GRADIENT_POLY, 9,
                               lambda: Q.gradient_batch(ht, p, f).clone())
        for c, o in enumerate(outs[1:], 1):  # bit patterns (a NaN equals itself)
            assert torch.equal(o.view(torch.int64), outs[0].view(torch.int64)), c


@pytest.mark.parametrize("n", [512, 8192])
def test_rk_search_candidates_bitwise_equal(Q, n):
    import torch
    ny = 64
    f = Q.FilteredNoise(gaussian_field(n, ny, 4.0, n % 31), float(n), float(ny))
    ctx = f.ctx
    rp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * ny, max_sweeps=300)
    h0 = t64(ny / 2 + np.cumsum(np.random.default_rng(n).standard_normal(n)) * 0.05)
    p = Q.Params(float(n), 1.0, 0.1, Q.Model.Linear)

    def run():
        h = h0.clone()
        r = Q.rk_block(h, p, f, rp)
        return h, (r.blocked, r.runaway, r.sweeps)

    outs = _each_candidate(ctx, Q.QEW_TUNE_RK_SEARCH, 3, run)
    tuned = run()
    for h, v in outs[1:] + [tuned]:
        assert v == outs[0][1]
        assert torch.equal(h, outs[0][0])
    assert "k_rk_resident" in Q.tune_report()


def _langevin_lines(Q, ctx, n, p, f, precision, steps=37, seed=3):
    import torch
    rng = np.random.default_rng(n)
    h0 = 0.5 * f.Ly + 0.2 * rng.standard_normal(n) if hasattr(f, "Ly") else \
        0.3 * rng.standard_normal(n)
    drift = np.full(steps, 0.01)
    diff = np.sqrt(2 * np.linspace(0.3, 0.05, steps) * 0.01)
    diff[::5] = 0.0  # deterministic steps leave the Philox counter where it is

    def run():
        h = t64(h0)
        d = Q.LangevinDynamics(n, seed, ctx=ctx)
        d.run(h, p, f, drift, diff, precision=precision)
        return h.clone(), d.steps
    outs = _each_candidate(ctx, Q.QEW_TUNE_LANGEVIN_RUN, 10, run)
    for c, (h, k) in enumerate(outs[1:], 1):
        assert k == outs[0][1]
        assert torch.equal(h.view(torch.int64), outs[0][0].view(torch.int64)), c


@pytest.mark.parametrize("model", [0, 1])
def test_langevin_run_candidates_bitwise_equal(Q, model):
    """One grid barrier per step or K in {8, 16, 32} steps per barrier at
    1, 2 or 4 CTAs per SM: the same line, bit for bit, after 37 steps (the
    last round partial), on the 16-tap FP64 gather, the cell-polynomial
    store and the FP32 split gather."""
    n, ny = 4096, 64
    fld = gaussian_field(n, ny, 3.0, 40)
    f16 = Q.FilteredNoise(fld, float(n), float(ny), store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
    fpoly = Q.FilteredNoise(fld, float(n), float(ny),
                            store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP64_POLY)
    ctx = f16.ctx
    p = Q.Params(float(n), 1.1, 0.3, Q.Model(model))
    _langevin_lines(Q, ctx, n, p, f16, Q.QEW_PREC_FP64)
    _langevin_lines(Q, ctx, n, p, fpoly, Q.QEW_PREC_FP64)
    _langevin_lines(Q, ctx, n, p, f16, Q.QEW_PREC_FP32_SPLIT)
    # a line that is not one point per field column: the generic gather
    f2 = Q.FilteredNoise(gaussian_field(1000, 48, 4.0, 41), 100.0, 4.8)
    _langevin_lines(Q, ctx, 1000, Q.Params(100.0, 1.0, 0.2, Q.Model(model)), f2,
                    Q.QEW_PREC_FP64)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 130])
def test_langevin_run_candidates_tiny_rings(Q, n):
    """Rings shorter than a round's halo: the shared-memory region wraps the
    ring several times and every copy of a site evolves alike."""
    f = Q.SinusoidNoise(0.3, 1.7)
    _langevin_lines(Q, f.ctx, n, Q.Params(float(n), 0.9, 0.1, Q.Model.Linear), f,
                    Q.QEW_PREC_FP64)
