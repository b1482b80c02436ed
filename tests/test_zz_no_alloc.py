"""The allocation-free energy entry point, called through the C ABI.

qew_objective_noalloc exists for callers that cannot call cudaMalloc where
they need the energy (cudaMalloc/cudaFree may synchronise the whole device,
and a process whose device memory is reserved up front gets out-of-memory
from any extra allocation); its reduction scratch is a static device array.
This file is collected last on purpose: a failure here leaves every other
test already run. It must pass alone in a fresh process and after the rest.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import gaussian_field

pytestmark = pytest.mark.gpu
RTOL = 1e-12  # the energy tolerance of the other parity tests


def test_noalloc_objective_matches_objective_twice(Q):
    import torch
    from qew_gb300 import _capi
    lib = _capi.load()
    n_max = _capi.QEW_NOALLOC_MAX_N
    fld = gaussian_field(4096, 64, 3.0, 11)
    noise = Q.FilteredNoise(fld, 4096.0, 64.0)
    stream = torch.cuda.current_stream().cuda_stream
    rng = np.random.default_rng(3)
    # two calls in a row: the full-size line, then a shorter line whose CTA
    # count differs (the shared scratch keeps the first call's partials)
    cases = [(n_max, Q.Params(4096.0, 1.3, 0.2, Q.Model.Linear)),
             (3001, Q.Params(4096.0, 0.7, -0.1, Q.Model.Arclength))]
    out = torch.empty(2, dtype=torch.float64, device="cuda")
    for k, (n, p) in enumerate(cases):
        h = torch.as_tensor(32 + np.cumsum(rng.standard_normal(n)) * 0.05, device="cuda")
        pc = p.c()
        st = lib.qew_objective_noalloc(noise.h, C.c_void_p(h.data_ptr()), n, C.byref(pc),
                                       C.c_void_p(out.data_ptr() + 8 * k), C.c_void_p(stream))
        assert st == _capi.QEW_OK
        torch.cuda.synchronize()
        got = float(out[k].item())
        want = Q.objective(h, p, noise)
        assert abs(got - want) <= RTOL * abs(want), (n, got, want)
    # sizes beyond the static scratch are rejected
    h = torch.zeros(n_max + 2, dtype=torch.float64, device="cuda")
    pc = cases[0][1].c()
    st = lib.qew_objective_noalloc(noise.h, C.c_void_p(h.data_ptr()), n_max + 2, C.byref(pc),
                                   C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert st == _capi.QEW_ERR_INVALID
