"""Shared test configuration.

Tests marked ``gpu`` need a CUDA device and call the CUDA library through its C
ABI; everything else runs on the CPU (oracle checks, host logic, the ABI's
symbol table). The oracle under ``oracle/`` is the checker only.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        have_gpu = torch.cuda.is_available()
    except Exception:
        have_gpu = False
    if have_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def O():
    """The CPU oracle (built on first use)."""
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def noise_golden():
    return dict(np.load(os.path.join(GOLDEN, "noise_golden.npz")))


@pytest.fixture(scope="session")
def lbfgs_golden():
    return dict(np.load(os.path.join(GOLDEN, "lbfgs_golden.npz")))


@pytest.fixture(scope="session")
def Q():
    """The GPU package, with its library built (gpu tests only)."""
    from qew_gb300 import build
    build.build()
    import qew_gb300
    return qew_gb300


def band_limited_field(nx, ny, Lx, Ly, amplitude, xi, seed):
    """Random-phase band-limited field as in the reference's fixture generator
    (random phases masked to the correlation disc, inverse FFT, std scaling)."""
    dx, dy = Lx / nx, Ly / ny
    rng = np.random.default_rng(seed)
    fx = np.fft.fftfreq(nx) / dx
    fy = np.fft.fftfreq(ny) / dy
    FX, FY = np.meshgrid(fx, fy, indexing="ij")
    A = np.exp(1j * rng.uniform(0, 2 * np.pi, (nx, ny)))
    A[(FX * xi) ** 2 + (FY * xi) ** 2 > 1] = 0
    f = np.real(np.fft.ifft2(A))
    return f * (amplitude / np.std(f))


def gaussian_field(nx, ny, xi_cells, seed):
    """Synthetic benchmark field: seeded white noise, Gaussian filter of
    correlation length xi (in cells) in Fourier space, unit variance."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nx, ny))
    kx = np.fft.fftfreq(nx)[:, None]
    ky = np.fft.rfftfreq(ny)[None, :]
    filt = np.exp(-0.5 * (2 * np.pi * xi_cells) ** 2 * (kx ** 2 + ky ** 2))
    f = np.fft.irfft2(np.fft.rfft2(w) * filt, s=(nx, ny))
    return (f - 0.0) / f.std()
