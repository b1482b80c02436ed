"""FP32 split-index gather against the FP64 oracle.

Stated error of the precision change (gradient): max |g_split - g_fp64| <=
2e-6 * (the largest term magnitude of the gradient, dx * (|F_el| + |dV/dy| +
|f|)), from FP32 coefficients, weights and sums.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import band_limited_field, gaussian_field

pytestmark = pytest.mark.gpu
TOL = 2e-6


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def npy(t):
    return t.detach().cpu().numpy()


def term_scale(O, h, po, of):
    """Largest magnitude among the gradient's terms (elastic, pinning, force)."""
    g_el = O.gradient(h, po, O.ZeroNoise())      # elastic + force only
    g = O.gradient(h, po, of)
    return max(np.max(np.abs(g_el)), np.max(np.abs(g - g_el)), 1e-300)


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("shape", [(1024, 64, 1024), (1000, 48, 1000), (777, 40, 500),
                                   (300, 32, 901)])
def test_split_gradient_error_bound(Q, O, model, shape):
    nx, ny, n = shape
    Lx, Ly = float(nx), float(ny)
    fld = gaussian_field(nx, ny, 3.0, nx + ny)
    f = Q.FilteredNoise(fld, Lx, Ly, store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
    of = O.BSplineField(fld, Lx, Ly, coef=f.coefficients())
    rng = np.random.default_rng(n)
    h = ny / 2 + np.cumsum(rng.standard_normal(n)) * 0.2
    h -= np.linspace(0, h[-1] - h[0], n)  # keep it roughly periodic
    p = Q.Params(Lx, 1.0, 0.2, Q.Model(model))
    po = O.params(Lx, 1.0, 0.2, model)
    go = O.gradient(h, po, of)
    scale = term_scale(O, h, po, of)
    g64 = npy(Q.gradient(t64(h), p, f, precision=Q.QEW_PREC_FP32_SPLIT))
    assert np.max(np.abs(g64 - go)) <= TOL * scale
    cell, frac = Q.split_heights(t64(h), f)
    g32 = npy(Q.gradient_split(cell, frac, p, f)).astype(np.float64)
    assert np.max(np.abs(g32 - go)) <= TOL * scale
    assert np.array_equal(g32, g64)


def test_split_join_roundtrip(Q):
    n, ny = 4096, 64
    f = Q.FilteredNoise(np.random.default_rng(0).standard_normal((n, ny)), float(n), 6.4,
                        store=Q.QEW_STORE_FP32)
    h = np.random.default_rng(1).uniform(-50, 50, n)
    cell, frac = Q.split_heights(t64(h), f)
    c, fr = npy(cell), npy(frac)
    assert np.all((fr >= 0) & (fr < 1))
    assert np.array_equal(c, np.floor(h / 0.1).astype(np.int32))
    back = npy(Q.join_heights(cell, frac, f))
    assert np.max(np.abs(back - h)) < 1e-6 * 0.1


def test_split_full_size(Q, O):
    """L = 2^20 on a 2^20 x 64 field against the OpenMP oracle, with and
    without the x-filtered store."""
    import torch
    n, ny = 1 << 20, 64
    fld = np.random.default_rng(3).standard_normal((n, ny))
    f = Q.FilteredNoise(fld, float(n), float(ny),
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32 | Q.QEW_STORE_FP32_EDGE)
    of = O.BSplineField(fld, float(n), float(ny), coef=f.coefficients())
    rng = np.random.default_rng(4)
    h = 32 + np.cumsum(rng.standard_normal(n)) * 0.02
    po = O.params(float(n), 1.0, 0.1, 0)
    go = O.gradient(h, po, of, omp=True)
    g_el = O.gradient(h, po, O.ZeroNoise(), omp=True)
    scale = max(np.max(np.abs(g_el)), np.max(np.abs(go - g_el)))
    p = Q.Params(float(n), 1.0, 0.1)
    cell, frac = Q.split_heights(t64(h), f)
    g = npy(Q.gradient_split(cell, frac, p, f)).astype(np.float64)
    assert np.max(np.abs(g - go)) <= TOL * scale
    del f
    torch.cuda.empty_cache()
    f16 = Q.FilteredNoise(fld, float(n), float(ny), store=Q.QEW_STORE_FP32)
    g16 = npy(Q.gradient_split(cell, frac, p, f16)).astype(np.float64)
    assert np.max(np.abs(g16 - go)) <= TOL * scale
    del f16
    torch.cuda.empty_cache()


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("n, ny, rough", [
    (4096, 64, 0.2),    # smooth line, interior rows
    (4096, 16, 30.0),   # rough line wrapping the rows many times
    (1001, 24, 1.0),    # odd n: the wrap edge sits at x = (n-1)/2 exactly (fx = 0)
    (1000, 4, 0.5),     # four rows: every stencil wraps in y
])
def test_split_edge_store_error_bound(Q, O, model, n, ny, rough):
    """The x-filtered store (4 taps per edge) meets the same bound against the
    FP64 oracle as the 16-tap form, and the two FP32 forms agree to it."""
    Lx = float(n)
    fld = gaussian_field(n, ny, 3.0, n + 7 * ny)
    fe = Q.FilteredNoise(fld, Lx, float(ny),
                         store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32 | Q.QEW_STORE_FP32_EDGE)
    f16 = Q.FilteredNoise(fld, Lx, float(ny), store=Q.QEW_STORE_FP32)
    of = O.BSplineField(fld, Lx, float(ny), coef=fe.coefficients())
    rng = np.random.default_rng(n * ny)
    h = ny / 2 + np.cumsum(rng.standard_normal(n)) * rough * 0.1 + 0.3 * ny * np.sin(
        np.linspace(0, 2 * np.pi, n, endpoint=False))
    p = Q.Params(Lx, 0.9, 0.02, Q.Model(model))
    po = O.params(Lx, 0.9, 0.02, model)
    go = O.gradient(h, po, of)
    scale = term_scale(O, h, po, of)
    cell, frac = Q.split_heights(t64(h), fe)
    ge = npy(Q.gradient_split(cell, frac, p, fe)).astype(np.float64)
    g16 = npy(Q.gradient_split(cell, frac, p, f16)).astype(np.float64)
    assert np.max(np.abs(ge - go)) <= TOL * scale
    assert np.max(np.abs(ge - g16)) <= TOL * scale
    # FP64 heights in: the same kernel splits them itself
    g64 = npy(Q.gradient(t64(h), p, fe, precision=Q.QEW_PREC_FP32_SPLIT)).astype(np.float32)
    assert np.array_equal(g64.astype(np.float64), ge)


def test_split_edge_store_ignored_off_grid(Q):
    """A line whose points do not match the field columns uses the 16-tap form:
    the x-filtered store changes nothing there."""
    nx, ny, n = 2048, 48, 3000
    fld = gaussian_field(nx, ny, 3.0, 5)
    fe = Q.FilteredNoise(fld, float(nx), float(ny), store=Q.QEW_STORE_FP32 | Q.QEW_STORE_FP32_EDGE)
    f16 = Q.FilteredNoise(fld, float(nx), float(ny), store=Q.QEW_STORE_FP32)
    h = t64(ny / 2 + np.cumsum(np.random.default_rng(2).standard_normal(n)) * 0.05)
    p = Q.Params(float(nx), 1.0, 0.0)
    cell, frac = Q.split_heights(h, fe)
    assert np.array_equal(npy(Q.gradient_split(cell, frac, p, fe)),
                          npy(Q.gradient_split(cell, frac, p, f16)))


@pytest.mark.parametrize("n, count", [(5000, 5), (150001, 9)])
def test_split_edge_store_batch(Q, O, n, count):
    """Batched lines on the x-filtered store (the persistent launch: a ragged
    last tile; at 150001 x 9 more tiles than resident CTAs, so CTAs loop):
    bitwise equal to one line per call, and within the bound of the oracle."""
    import torch
    ny = 48
    fld = gaussian_field(n, ny, 3.0, 17)
    f = Q.FilteredNoise(fld, float(n), float(ny),
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32 | Q.QEW_STORE_FP32_EDGE)
    of = O.BSplineField(fld, float(n), float(ny), coef=f.coefficients())
    rng = np.random.default_rng(n + count)
    hs = [ny / 2 + np.cumsum(rng.standard_normal(n)) * 0.1 for _ in range(count)]
    sp = [Q.split_heights(t64(h), f) for h in hs]
    cells = torch.stack([c for c, _ in sp]).contiguous()
    fracs = torch.stack([fr for _, fr in sp]).contiguous()
    for model in (0, 1):
        p = Q.Params(float(n), 0.8, 0.05, Q.Model(model))
        po = O.params(float(n), 0.8, 0.05, model)
        gb = npy(Q.gradient_split_batch(cells, fracs, p, f))
        for k in (0, count // 2, count - 1):
            assert np.array_equal(gb[k], npy(Q.gradient_split(sp[k][0], sp[k][1], p, f)))
            go = O.gradient(hs[k], po, of, omp=True)
            g_el = O.gradient(hs[k], po, O.ZeroNoise(), omp=True)
            scale = max(np.max(np.abs(g_el)), np.max(np.abs(go - g_el)))
            assert np.max(np.abs(gb[k].astype(np.float64) - go)) <= TOL * scale


def test_edge_store_needs_fp32(Q):
    with pytest.raises(ValueError, match="FP32_EDGE"):
        Q.FilteredNoise(gaussian_field(64, 16, 3.0, 1), 64.0, 16.0,
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32_EDGE)


def test_split_needs_fp32_storage(Q):
    f = Q.FilteredNoise(band_limited_field(64, 32, 3.2, 1.0, 1.0, 0.3, 1), 3.2, 1.0)
    with pytest.raises(ValueError, match="FP32"):
        Q.gradient(t64(np.zeros(64)), Q.Params(3.2), f, precision=Q.QEW_PREC_FP32_SPLIT)


def test_split_batch_equals_single_lines(Q):
    import torch
    n, ny, count = 5000, 48, 5
    f = Q.FilteredNoise(gaussian_field(n, ny, 3.0, 8), float(n), float(ny),
                        store=Q.QEW_STORE_FP32)
    rng = np.random.default_rng(9)
    hs = [t64(ny / 2 + np.cumsum(rng.standard_normal(n)) * 0.1) for _ in range(count)]
    sp = [Q.split_heights(h, f) for h in hs]
    cells = torch.stack([c for c, _ in sp]).contiguous()
    fracs = torch.stack([fr for _, fr in sp]).contiguous()
    for model in (Q.Model.Linear, Q.Model.Arclength):
        p = Q.Params(float(n), 0.8, 0.05, model)
        gb = npy(Q.gradient_split_batch(cells, fracs, p, f))
        for k in range(count):
            gk = npy(Q.gradient_split(sp[k][0], sp[k][1], p, f))
            assert np.array_equal(gb[k], gk)


@pytest.mark.parametrize("model", [0, 1])
@pytest.mark.parametrize("n, nx, ny, rough", [
    (4096, 4096, 64, 0.2),     # shared grid, smooth line
    (4096, 4096, 64, 30.0),    # rough line wrapping around the field many times
    (3000, 2048, 48, 0.5),     # line and field grids differ
    (2048, 2046, 40, 0.3),     # odd row pitch
])
def test_split_heights_form_equals_fp64_input_form(Q, model, n, nx, ny, rough):
    """Split heights -> FP32 gradient equals the same gather fed FP64 heights
    (split inside the kernel), bitwise after rounding its FP64 output to FP32,
    including the interior fast path, the wrap-around stencils and both
    x-geometries."""
    Lx = float(nx)
    f = Q.FilteredNoise(gaussian_field(nx, ny, 3.0, 21), Lx, float(ny),
                        store=Q.QEW_STORE_FP64 | Q.QEW_STORE_FP32)
    rng = np.random.default_rng(n + nx)
    h = t64(ny / 2 + np.cumsum(rng.standard_normal(n)) * rough * 0.1 + 0.3 * ny * np.sin(
        np.linspace(0, 2 * np.pi, n, endpoint=False)))
    p = Q.Params(Lx, 0.9, 0.02, Q.Model(model))
    cell, frac = Q.split_heights(h, f)
    g_split = npy(Q.gradient_split(cell, frac, p, f))
    g_in64 = npy(Q.gradient(h, p, f, precision=Q.QEW_PREC_FP32_SPLIT)).astype(np.float32)
    assert np.array_equal(g_split, g_in64)
