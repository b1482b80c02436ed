"""NVTX ranges: every compute entry point opens a range named for itself and
closes it on every return path. An injection library (tests/native/
nvtx_count.c, loaded through NVTX_INJECTION64_PATH) records the ranges while
a fresh process calls entry points with arguments they reject before any
device work, so no GPU is needed."""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CALLS = r"""
import ctypes as C
from qew_gb300 import _capi
lib = _capi.load()
assert lib.qew_gradient_prec(None, None, None, 0, None, 0, None) != 0
assert lib.qew_gradient_batch(None, None, 1, None, 1, None, 0, None) != 0
assert lib.qew_objective(None, None, None, 0, None, None) != 0
assert lib.qew_rk_block(None, None, None, 0, None, None, None) != 0
assert lib.qew_lbfgs_minimize_form(None, None, None, 0, None, None, 0, None) != 0
assert lib.qew_depinning_bisect_ex(None, None, None, 0, None, None, 0.0, 1.0, 1e-10, 1, 0,
                                   None, None) != 0
"""


@pytest.fixture(scope="module")
def injection(tmp_path_factory):
    from qew_gb300 import build
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    out = str(tmp_path_factory.mktemp("nvtx") / "libnvtx_count.so")
    subprocess.run([cc, "-shared", "-fPIC", "-O1",
                    "-I" + os.path.join(build._cuda_home(), "include"),
                    os.path.join(ROOT, "tests", "native", "nvtx_count.c"), "-o", out], check=True)
    build.build()
    return out


def test_entry_points_open_and_close_named_ranges(injection, tmp_path):
    log = tmp_path / "ranges.txt"
    env = dict(os.environ, NVTX_INJECTION64_PATH=injection, QEW_NVTX_LOG=str(log))
    subprocess.run([sys.executable, "-c", CALLS], check=True, cwd=ROOT, env=env, timeout=300)
    lines = log.read_text().splitlines()
    pushes = [ln.split(" ", 1)[1] for ln in lines if ln.startswith("push ")]
    assert pushes == ["qew_gradient_prec", "qew_gradient_batch", "qew_objective", "qew_rk_block",
                      "qew_lbfgs_minimize_form", "qew_depinning_bisect_ex"]
    depth = 0
    for ln in lines:  # every range closes before the next opens
        depth += 1 if ln.startswith("push ") else -1
        assert depth in (0, 1)
    assert depth == 0
