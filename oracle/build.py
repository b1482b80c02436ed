"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/qew_oracle.c`` into ``oracle/_build/libqew_oracle.so`` with
gcc. ``-ffp-contract=off`` keeps every a*b+c as two rounded operations, as in
the reference's ISO C++20 build, on both x86-64 and aarch64; ``-fopenmp``
enables the thread-parallel gradient used as the timed CPU baseline.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libqew_oracle.so")
SOURCES = [os.path.join(HERE, "qew_oracle.c")]


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = SOURCES + [os.path.join(HERE, "qew_oracle.h")]
    return any(os.path.getmtime(s) > t for s in deps)


def build(force: bool = False) -> str:
    """Compile the oracle shared library if missing or stale; return its path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fopenmp", "-Wall", "-Wno-unknown-pragmas", "-o", tmp] + SOURCES + ["-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
