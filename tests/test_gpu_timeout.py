"""The bounded grid-barrier waits of the persistent cooperative kernels run
out, report QEW_ERR_TIMEOUT and leave the context usable.

The fault is injected through the context's barrier limits: one CTA of the
launch leaves at its first barrier without arriving, and the others' waits
give up after 2^14 polls (about a millisecond) instead of 2^26. Nothing
hangs: every CTA returns, the host reads the barrier's error word, and the
next launch on the same context (default limits) gives the result of a
fresh run.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import gaussian_field

pytestmark = pytest.mark.gpu
SHORT = 1 << 14


def t64(a):
    import torch
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("cand", [0, 5])
def test_langevin_run_barrier_times_out_then_recovers(Q, cand):
    """One grid barrier per step (candidate 0: 32 CTAs of 256 sites) and 16
    steps per barrier at 2 CTAs per SM (candidate 5: 128 CTAs of 64 sites)."""
    import torch
    n, ny = 8192, 64
    f = Q.FilteredNoise(gaussian_field(n, ny, 4.0, 3), float(n), float(ny))
    p = Q.Params(float(n), 1.0, 0.2, Q.Model.Arclength)
    drift, diff = np.full(50, 0.01), np.full(50, 0.05)
    h0 = t64(ny / 2 + np.random.default_rng(1).standard_normal(n))
    ctx = f.ctx
    try:
        ctx.force_tune_candidate(Q.QEW_TUNE_LANGEVIN_RUN, cand)
        try:
            ctx.set_barrier_limits(SHORT, 3)
            dyn = Q.LangevinDynamics(n, 7)
            with pytest.raises(Q.QewError, match="timed out"):
                dyn.run(h0.clone(), p, f, drift, diff)
        finally:
            ctx.set_barrier_limits(0, -1)
        # the same object and context afterwards: the run a fresh object gives
        h1, h2 = h0.clone(), h0.clone()
        dyn.run(h1, p, f, drift, diff)
        Q.LangevinDynamics(n, 7).run(h2, p, f, drift, diff)
        assert torch.equal(h1, h2)
    finally:
        ctx.force_tune_candidate(Q.QEW_TUNE_LANGEVIN_RUN, -1)


def test_rk_block_barrier_times_out_then_recovers(Q):
    import torch
    n, ny = 1024, 64
    f = Q.FilteredNoise(gaussian_field(n, ny, 4.0, 5), float(n), float(ny))
    rp = Q.RkParams(dstep=0.5, max_advance=float(ny), root_tol=1e-10, sweep_tol=1e-8,
                    runaway=2.0 * ny, max_sweeps=500)
    p = Q.Params(float(n), 1.0, 0.05, Q.Model.Linear)
    h0 = t64(np.full(n, ny / 2))
    ctx = f.ctx
    try:
        ctx.set_barrier_limits(SHORT, 0)
        with pytest.raises(Q.QewError, match="timed out"):
            Q.rk_block(h0.clone(), p, f, rp)
    finally:
        ctx.set_barrier_limits(0, -1)
    h1, h2 = h0.clone(), h0.clone()
    r1 = Q.rk_block(h1, p, f, rp)
    r2 = Q.rk_block(h2, p, f, rp, form=Q.QEW_RK_PLAIN)
    assert (r1.blocked, r1.sweeps) == (r2.blocked, r2.sweeps)
    assert torch.equal(h1, h2)
