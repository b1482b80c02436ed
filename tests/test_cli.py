"""The executables' option reader and output writers, on the CPU.

Mirrors the reference's parser tests (tests/test_cli.cpp) and the key-string
contract of its writers (tests/test_executables.cpp:50-56, 199-289) through a
small probe program compiled from tests/native/cli_io_probe.cpp, and checks
that the built executables answer --help and reject bad command lines with
exit status 2 before touching a GPU.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "qew_gb300", "csrc", "cli")


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    out = str(tmp_path_factory.mktemp("probe") / "cli_io_probe")
    subprocess.run([cxx, "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), "-I" + CLI,
                    os.path.join(ROOT, "tests", "native", "cli_io_probe.cpp"), "-o", out],
                   check=True)
    return out


def _parse(probe, *args):
    r = subprocess.run([probe, *args], capture_output=True, text=True,
                       env=dict(os.environ, QEW_PROBE="parse"))
    vals = dict(line.split("=", 1) for line in r.stdout.splitlines() if "=" in line)
    return r.returncode, vals


def test_defaults_kept_when_absent(probe):
    rc, v = _parse(probe)
    assert rc == 0 and v["help"] == "0"
    assert v["nx"] == "4096" and float(v["ftol"]) == 1e-6 and v["seed"] == "1"
    assert v["model"] == "arclength"
    assert [float(x) for x in v["pinning_lengths"].split(",")] == [0.01, 0.1, 1.0]


def test_overrides_both_spellings(probe):
    rc, v = _parse(probe, "--nx", "8192", "--ftol=1e-8", "--model", "linear")
    assert rc == 0 and v["nx"] == "8192" and float(v["ftol"]) == 1e-8 and v["model"] == "linear"


def test_negative_value_is_not_a_flag(probe):
    rc, v = _parse(probe, "--driving_force", "-1.5")
    assert rc == 0 and float(v["driving_force"]) == -1.5


def test_comma_list(probe):
    rc, v = _parse(probe, "--pinning_lengths", "0.1,1,10,100")
    assert rc == 0
    assert [float(x) for x in v["pinning_lengths"].split(",")] == [0.1, 1.0, 10.0, 100.0]
    rc, v = _parse(probe, "--pinning_lengths", ",,")
    assert rc == 2 and "empty list" in v["error"]


def test_help_flag(probe):
    assert _parse(probe, "--help")[1]["help"] == "1"
    assert _parse(probe, "-h")[1]["help"] == "1"


@pytest.mark.parametrize("args, msg", [
    (("--bogus", "3"), "unknown option"),
    (("--nx", "abc"), "cannot parse"),
    (("--ftol", "1.0x"), "cannot parse"),
    (("--nx",), "needs a value"),
    (("positional",), "unexpected argument"),
    (("--=3",), "empty option name"),
])
def test_bad_command_lines_rejected(probe, args, msg):
    rc, v = _parse(probe, *args)
    assert rc == 2 and msg in v["error"]


def test_key_formatter(probe):
    r = subprocess.run([probe], capture_output=True, text=True, env=dict(os.environ, QEW_PROBE="fmt"))
    assert r.stdout.strip() == "0|0.1|100|1|0.8"


def test_writers_keys_and_values(probe, tmp_path):
    subprocess.run([probe, str(tmp_path)], check=True, env=dict(os.environ, QEW_PROBE="write"))
    s = np.load(tmp_path / "static.npz")
    assert float(s["physical_size"]) == 4.0
    pre = "driving_force=0/pinning_length=0.1"
    assert list(s[pre + "/h"]) == [1.0, 2.0, 3.0, 4.0]
    assert float(s[pre + "/pinning_length"]) == 0.1
    d = np.load(tmp_path / "dynamic.npz")
    pre = "timestep=1/driving_force=0/line_tension=2"
    assert list(d[pre + "/h"]) == [5.0, 6.0]
    assert float(d[pre + "/pinning_length"]) == 0.1
    p = np.load(tmp_path / "depinning.npz")
    assert list(p["driving_force=0/h"]) == [0.5, 0.5, 0.5]
    assert float(p["driving_force=0/pinning_length"]) == 5.0
    assert "driving_force=0.8/h" not in p.files  # the runaway force stores no profile
    assert float(p["f_c_upper_bound"]) == 0.8
    assert "f_c" not in p.files


def _exe(name):
    from qew_gb300 import build
    path = build.executable(name)
    if not os.path.exists(path):
        pytest.skip("executables not built")
    return path


@pytest.mark.parametrize("name", ["qew_static", "qew_dynamic", "qew_depinning"])
def test_executables_help_and_usage_errors(name):
    exe = _exe(name)
    r = subprocess.run([exe, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith(name)
    for bad in (["--bogus", "1"], ["--nx", "abc"], ["--model", "elastic"], ["--output", "x.h5"]):
        r = subprocess.run([exe, *bad], capture_output=True, text=True, timeout=60)
        assert r.returncode == 2, (bad, r.stderr)
        assert r.stderr.startswith(name + ": ") and "--model" in r.stderr  # message + usage


def build_hpp_probe(out_dir):
    """Compile tests/native/hpp_probe.cpp against include/qew_gpu.hpp and the
    built library (host compiler + CUDA runtime for the caller's buffers)."""
    from qew_gb300 import build
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    if not os.path.exists(build.LIB):
        pytest.skip("library not built")
    cuda = build._cuda_home()
    out = os.path.join(str(out_dir), "hpp_probe")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "native", "hpp_probe.cpp"), "-o", out,
                    "-L" + build.OUT_DIR, "-lqew_gb300", "-Wl,-rpath," + build.OUT_DIR,
                    "-L" + os.path.join(cuda, "lib64"), "-lcudart",
                    "-Wl,-rpath," + os.path.join(cuda, "lib64")], check=True)
    return out


def test_cpp_face_compiles_and_links(tmp_path):
    """include/qew_gpu.hpp: the reference's signatures over the C ABI build
    against the library (it runs in tests/test_gpu_runs.py)."""
    assert os.path.exists(build_hpp_probe(tmp_path))


def _npy(probe, path):
    r = subprocess.run([probe, str(path)], capture_output=True, text=True,
                       env=dict(os.environ, QEW_PROBE="npy"))
    return r.returncode, dict(ln.split("=", 1) for ln in r.stdout.splitlines() if "=" in ln)


def test_field_file_reader(probe, tmp_path):
    """The --field_file reader: float64 C-order 2-D .npy (header versions 1
    and 2), shape and values as numpy wrote them; anything else rejected."""
    a = np.random.default_rng(0).standard_normal((7, 5))
    np.save(tmp_path / "f.npy", a)
    rc, v = _npy(probe, tmp_path / "f.npy")
    assert rc == 0 and (v["rows"], v["cols"]) == ("7", "5")
    assert float(v["first"]) == a[0, 0] and float(v["last"]) == a[-1, -1]
    assert abs(float(v["sum"]) - a.sum()) < 1e-12
    with open(tmp_path / "v2.npy", "wb") as fh:
        np.lib.format.write_array(fh, a, version=(2, 0))
    rc, v = _npy(probe, tmp_path / "v2.npy")
    assert rc == 0 and (v["rows"], v["cols"]) == ("7", "5")
    bad = {
        "f32.npy": a.astype(np.float32), "fortran.npy": np.asfortranarray(a),
        "one_d.npy": a.ravel(), "three_d.npy": a.reshape(7, 5, 1), "big_endian.npy": a.astype(">f8"),
    }
    for name, arr in bad.items():
        np.save(tmp_path / name, arr)
        rc, v = _npy(probe, tmp_path / name)
        assert rc == 2 and "error" in v, name
    raw = (tmp_path / "f.npy").read_bytes()
    (tmp_path / "short.npy").write_bytes(raw[:-8])
    (tmp_path / "text.npy").write_bytes(b"not an array")
    for name in ("short.npy", "text.npy", "missing.npy"):
        rc, v = _npy(probe, tmp_path / name)
        assert rc == 2 and "error" in v, name


@pytest.mark.parametrize("name", ["qew_static", "qew_dynamic", "qew_depinning"])
def test_executables_field_file_and_rows_errors(name, tmp_path):
    """--field_file / --rows mistakes end with exit 2, the message and the
    usage, before any GPU work."""
    exe = _exe(name)
    np.save(tmp_path / "f.npy", np.zeros((4, 3)))
    cases = [
        (["--rows", "16", "--ny", "8"], "--rows"),
        (["--rows", "16", "--Ly", "2"], "--rows"),
        (["--rows", "0"], "--rows"),
        (["--field_file", str(tmp_path / "missing.npy")], "cannot open"),
        (["--field_file", str(tmp_path / "f.npy"), "--nx", "5"], "has shape (4, 3)"),
        (["--field_file", str(tmp_path / "f.npy"), "--rows", "8"], "has shape (4, 3)"),
    ]
    for args, msg in cases:
        r = subprocess.run([exe, *args], capture_output=True, text=True, timeout=60)
        assert r.returncode == 2, (args, r.stderr)
        assert msg in r.stderr and "--field_file" in r.stderr, (args, r.stderr)
