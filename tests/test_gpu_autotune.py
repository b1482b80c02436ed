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
