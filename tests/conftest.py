"""Shared fixtures: repo root on sys.path, the `gpu` marker, circuit helpers."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from stab_decomp_simulator_rust_gb300.workloads import OP, Xoshiro256ss  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on the GB300 box)")


def random_full_circuit(n: int, num_clifford: int, num_t: int, seed: int) -> np.ndarray:
    """Random circuit over every gate kind the compiler accepts (H, X, Y, Z, S,
    Sdg, SqrtX, SqrtXdg, CX, CZ, Swap; T and Tdg at uniform positions), in the
    spirit of random_circuit_with_t_gate (crates/necstar/src/test_utils/mod.rs:121-208)."""
    rng = Xoshiro256ss(seed)
    one = [OP[k] for k in ("H", "X", "Y", "Z", "S", "SDG", "SQRT_X", "SQRT_XDG")]
    two = [OP[k] for k in ("CX", "CZ", "SWAP")]
    gates = []
    for _ in range(num_clifford):
        kinds = len(one) + (len(two) if n >= 2 else 0)
        k = rng.below(kinds)
        if k < len(one):
            gates.append((one[k], rng.below(n), 0, 0))
        else:
            a = rng.below(n)
            b = rng.below(n - 1)
            if b >= a:
                b += 1
            gates.append((two[k - len(one)], a, b, 0))
    for _ in range(num_t):
        pos = rng.below(len(gates) + 1)
        op = OP["T"] if rng.below(2) == 0 else OP["TDG"]
        gates.insert(pos, (op, rng.below(n), 0, 0))
    return np.asarray(gates, dtype=np.uint32).reshape(-1, 4)


def toffoli_gates() -> np.ndarray:
    """The Toffoli-state circuit of tests/test_state_calculation.py:37-65."""
    H, T, TDG, CX = OP["H"], OP["T"], OP["TDG"], OP["CX"]
    g = [(H, 0), (H, 1), (H, 2), (CX, 1, 2), (TDG, 2), (CX, 0, 2), (T, 2), (CX, 1, 2), (TDG, 2), (CX, 0, 2),
         (T, 1), (T, 2), (CX, 0, 1), (H, 2), (T, 0), (TDG, 1), (CX, 0, 1)]
    return np.asarray([tuple(x) + (0,) * (4 - len(x)) for x in g], dtype=np.uint32)


@pytest.fixture(scope="session")
def oracle():
    from oracle import build, pyoracle
    build.build()
    return pyoracle


@pytest.fixture(scope="session")
def host_pkg():
    """The product package with its library loaded, for entry points that do
    host work only (no GPU call)."""
    from stab_decomp_simulator_rust_gb300 import _ffi, build
    build.build()
    _ffi.load()
    import stab_decomp_simulator_rust_gb300 as pkg
    return pkg


@pytest.fixture(scope="session")
def gpu_pkg():
    """The product package with its CUDA library loaded (built if missing)."""
    from stab_decomp_simulator_rust_gb300 import _ffi, build
    build.build()
    _ffi.load()
    import stab_decomp_simulator_rust_gb300 as pkg
    return pkg
