"""The C-ABI library builds for sm_103a, loads, and exports every function the
public header declares (no compute calls: this runs without a GPU)."""
from __future__ import annotations

import ctypes
import subprocess

from qew_gb300 import _capi, build


def test_library_builds_and_exports_header_symbols():
    path = build.build()
    lib = ctypes.CDLL(path)
    declared = _capi.header_symbols()
    assert len(declared) >= 30
    missing = [s for s in declared if not hasattr(lib, s)]
    assert not missing, "declared but not exported: %s" % missing
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln and "qew_" in ln}
    assert set(declared) <= exported


def test_binding_table_covers_header():
    assert set(_capi._SIGS) == set(_capi.header_symbols())


def test_status_strings():
    lib = _capi.load(build.build())
    assert lib.qew_status_string(0) == b"ok"
    assert b"even" in lib.qew_status_string(_capi.QEW_ERR_ODD_LENGTH)
