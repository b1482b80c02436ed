"""The bounds-checked build (-DQEW_BOUNDS_CHECK): every field gather and the
gradient kernels' shared-memory indices are range-checked on the device. Its
library is built here, then the cases of tests/bounds_check_cases.py run on
it in a fresh process: no index may leave its array, and the results keep
the parity bars (1e-12 FP64, 2e-6 of the gradient scale for FP32)."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bounds_checked_build_has_no_out_of_range_index(Q):
    from qew_gb300 import build
    lib = build.build(variant="bounds_check")
    assert os.path.exists(lib)
    env = dict(os.environ, QEW_GB300_VARIANT="bounds_check")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "bounds_check_cases.py")],
                       capture_output=True, text=True, timeout=900, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    rep = out["report"]
    assert rep is not None, "the checked build was not the one loaded"
    assert rep["count"] == 0, rep
    for name, err in out["errors"].items():
        bar = 2e-6 if name.startswith("fp32") else 1e-12
        assert err <= bar, (name, err)
    assert out["lbfgs_converged"] and out["ensemble_converged"]


def test_normal_build_has_no_bounds_report(Q):
    assert Q.bounds_check_report() is None
