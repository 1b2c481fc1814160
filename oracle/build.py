"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/necstar_oracle.cpp`` — the C++ restatement of the
reference's Rust path — into ``oracle/_build/libnecstar_oracle.so``.  The
reference itself is Rust and cannot be compiled here (no cargo/rustc), so no
``oracle/_ref`` build exists.

``-ffp-contract=off`` keeps the FP64 rounding of the reference's f64
arithmetic (Rust never contracts a·b+c into an FMA; GCC does by default on
aarch64).
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "necstar_oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnecstar_oracle.so")


def command(out: str = LIB) -> list[str]:
    return [
        os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-ffp-contract=off",
        "-fPIC", "-shared", "-pthread", "-Wall", "-o", out, SRC,
    ]


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.run(command(tmp), check=True)
    os.replace(tmp, LIB)
    return LIB


def popen() -> subprocess.Popen:
    """Start the build without waiting (used to overlap with the CUDA build)."""
    os.makedirs(OUT_DIR, exist_ok=True)
    return subprocess.Popen(command())


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
