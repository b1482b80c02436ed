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


def test_header_constants_match_python_mirror():
    """Every enum constant and numeric #define of the public headers has the
    same value in the Python mirror, and the mirror defines each one the
    bindings use."""
    import re

    import qew_gb300 as Q
    txt = "".join(open(h).read() for h in _capi.HEADERS)
    consts = {}
    for body in re.findall(r"\benum\s*\{([^}]*)\}", txt):
        body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
        for name, val in re.findall(r"\b(QEW_[A-Z0-9_]+)\s*=\s*(-?\d+)", body):
            consts[name] = int(val)
    for name, val in re.findall(r"^#define\s+(QEW_[A-Z0-9_]+)\s+(-?\d+)\s*$", txt, re.M):
        consts[name] = int(val)
    assert len(consts) >= 28
    mirrored = {k: v for k, v in consts.items() if hasattr(_capi, k)}
    for name, val in mirrored.items():
        assert getattr(_capi, name) == val, name
    need = [k for k in consts if k.startswith(("QEW_ERR_", "QEW_STORE_", "QEW_PREC_", "QEW_FIELD_",
                                               "QEW_REQ_", "QEW_RK_", "QEW_LBFGS_"))]
    assert set(need) <= set(mirrored), sorted(set(need) - set(mirrored))
    assert int(Q.Model.Linear) == consts["QEW_MODEL_LINEAR"]
    assert int(Q.Model.Arclength) == consts["QEW_MODEL_ARCLENGTH"]
