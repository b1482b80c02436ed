"""Build the GB300 qEW CUDA library in-tree.

Compiles every ``csrc/*.cu`` for sm_103a with nvcc (in parallel, one object
per translation unit) and links ``_lib/libqew_gb300.so``, which exports the C
ABI declared in ``include/qew_gpu.h`` and ``include/qew_runs.h``. cudart is
linked statically; cuFFT (the host-driven comparator form of L-BFGS and the
seeded field's inverse transform) dynamically, with an rpath to the toolkit's
library directory. Then builds the three simulation executables
(``csrc/cli/*.cpp``, host C++ over that library) into ``_lib/bin``.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libqew_gb300.so")
BIN_DIR = os.path.join(OUT_DIR, "bin")
CLI_DIR = os.path.join(CSRC, "cli")
EXECUTABLES = ("qew_static", "qew_dynamic", "qew_depinning")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xcompiler", "-Wall", "-Xcompiler", "-Wno-unknown-pragmas"]


def _cuda_home() -> str:
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    raise RuntimeError("nvcc not found")


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h")) +
            glob.glob(os.path.join(CLI_DIR, "*.h")))


def executable(name: str) -> str:
    """Path of one of the built simulation executables."""
    return os.path.join(BIN_DIR, name)


def _build_executables(force: bool) -> None:
    os.makedirs(BIN_DIR, exist_ok=True)
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the executables")

    def one(name):
        src = os.path.join(CLI_DIR, name + ".cpp")
        out = executable(name)
        if not force and os.path.exists(out) and not _stale(out, [src, LIB]):
            return out
        tmp = out + ".tmp%d" % os.getpid()
        cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I" + INCLUDE, "-I" + CLI_DIR, src, "-o", tmp,
               "-L" + OUT_DIR, "-lqew_gb300", "-Wl,-rpath,$ORIGIN/.."]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("g++ failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        os.replace(tmp, out)
        return out

    with cf.ThreadPoolExecutor(len(EXECUTABLES)) as ex:
        list(ex.map(one, EXECUTABLES))


def _stale(lib: str, srcs) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    return any(os.path.getmtime(s) > t for s in list(srcs) + _headers() + [__file__])


def build(force: bool = False, verbose: bool = False, extra_flags=None,
          variant: str = "") -> str:
    """Build the library (variant "bounds_check": the range-checked build in
    _lib/bounds_check/, without the executables)."""
    if variant:
        if variant != "bounds_check":
            raise ValueError("unknown build variant %r" % variant)
        return _build_lib(force, verbose, list(extra_flags or []) + ["-DQEW_BOUNDS_CHECK"],
                          os.path.join(OUT_DIR, variant), executables=False)
    return _build_lib(force, verbose, extra_flags, OUT_DIR, executables=True)


def _build_lib(force, verbose, extra_flags, out_dir, executables) -> str:
    lib_path = os.path.join(out_dir, "libqew_gb300.so")
    obj_dir = os.path.join(out_dir, "obj")
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    if not force and not _stale(lib_path, srcs):
        if executables:
            _build_executables(force)
        return lib_path
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(obj_dir, exist_ok=True)
    flags = ARCH + NVCC_FLAGS + ["-I" + INCLUDE] + list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(obj_dir, os.path.basename(src) + ".o")
        cmd = [nvcc] + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj

    workers = min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(compile_one, srcs))
    libdir = os.path.join(cuda, "lib64")
    tmp = lib_path + ".tmp%d" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + [
        "-L" + libdir, "-lcufft", "-Xlinker", "-rpath," + libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib_path)
    if executables:
        _build_executables(True)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                variant="bounds_check" if "--bounds-check" in sys.argv else ""))
