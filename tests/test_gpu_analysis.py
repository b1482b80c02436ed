"""Roughness statistics (ell, acf, q, psd) on the GPU against their
definitions evaluated directly with numpy (the definitions are stated in
include/qew_gpu.h, qew_line_statistics)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def direct(h, L):
    n = h.size
    dx = L / n
    nh = n // 2 + 1
    k = np.arange(nh)
    acf = np.array([np.mean((np.roll(h, -j) - h) ** 2) for j in k])
    H = np.array([np.sum(h * np.exp(-2j * np.pi * np.arange(n) * j / n)) for j in k])
    return k * dx, acf, 2 * np.pi * k / L, dx / n * np.abs(H) ** 2


@pytest.mark.parametrize("n, L", [(64, 6.4), (150, 1.0), (1000, 37.0)])
def test_statistics_match_definitions(Q, n, L):
    import torch
    rng = np.random.default_rng(n)
    hs = np.cumsum(rng.standard_normal((3, n)), axis=1) * 0.1 + 0.5
    hs -= np.linspace(0, 1, n)[None, :] * (hs[:, -1:] - hs[:, :1])  # make them near periodic
    ell, acf, q, psd = (t.cpu().numpy() for t in Q.line_statistics(
        torch.as_tensor(hs, device="cuda"), L))
    for k in range(3):
        e, a, qq, p = direct(hs[k], L)
        np.testing.assert_allclose(ell, e, rtol=1e-15, atol=0)
        np.testing.assert_allclose(qq, q, rtol=1e-15, atol=0)
        scale = np.max(a)
        assert np.max(np.abs(acf[k] - a)) <= 1e-12 * scale
        assert np.max(np.abs(psd[k] - p)) <= 1e-12 * np.max(p)


def test_flat_line_and_single_mode(Q):
    import torch
    n, L = 128, 12.8
    flat = torch.full((n,), 0.7, dtype=torch.float64, device="cuda")
    _, acf, _, psd = Q.line_statistics(flat, L)
    assert float(acf.abs().max()) < 1e-14 and float(psd[1:].abs().max()) < 1e-24
    x = np.arange(n) * L / n
    A, m = 0.3, 5
    wave = torch.as_tensor(A * np.sin(2 * np.pi * m * x / L), device="cuda")
    ell, acf, q, psd = (t.cpu().numpy() for t in Q.line_statistics(wave, L))
    # acf of a sine: A^2 (1 - cos(q_m ell)); all power in mode m: psd_m = dx n A^2 / 4
    np.testing.assert_allclose(acf, A * A * (1 - np.cos(2 * np.pi * m * ell / L)), atol=1e-13)
    assert abs(psd[m] - (L / n) * n * A * A / 4) < 1e-12
    assert np.max(np.delete(psd, m)) < 1e-20
