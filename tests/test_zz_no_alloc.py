"""nsg_exp_value_noalloc — ⟨P⟩ for callers that cannot allocate device memory.

Those callers (a process whose GPU memory is fully reserved by another
allocator, a latency-critical loop where cudaMalloc/cudaFree would
synchronise the device) get the same value as nsg_exp_value from one static
16 MiB device scratch array.  This file is collected last so that a run that
stops at the first failure has already run every other test; it passes both
alone in a fresh process and after the rest of the suite.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from stab_decomp_simulator_rust_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-9  # the tolerance of the other expectation-value tests


def _noalloc(lib, state, pauli):
    out = C.c_double()
    a = pauli.abi()
    rc = lib.nsg_exp_value_noalloc(state._h, C.byref(a), C.byref(out))
    return rc, out.value


def test_noalloc_matches_exp_value_twice(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import _ffi
    lib = _ffi.load()
    n = 40
    gates = W.random_clifford_t_circuit(n, 1500, 12, 7)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    paulis = [gpu_pkg.PauliString.dense(p) for p in W.random_dense_paulis(n, 2, 70)]
    for p in paulis:  # two calls in a row share (and reuse) the scratch
        want = st.exp_value(p)
        rc, got = _noalloc(lib, st, p)
        assert rc == 0, (rc, lib.nsg_last_error_message())
        assert abs(got - want) <= TOL * max(1.0, abs(want)), (got, want)


def test_noalloc_small_state_twice(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import _ffi
    lib = _ffi.load()
    st = gpu_pkg.QuantumState.from_gates(16, W.random_clifford_t_circuit(16, 300, 6, 8))
    p = gpu_pkg.PauliString.from_str("Z0 X3 Y7")
    want = st.exp_value(p)
    for _ in range(2):
        rc, got = _noalloc(lib, st, p)
        assert rc == 0 and abs(got - want) <= TOL * max(1.0, abs(want)), (rc, got, want)


def test_noalloc_rejects_states_above_its_limit(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import _ffi
    lib = _ffi.load()
    st = gpu_pkg.QuantumState.from_gates(12, W.random_clifford_t_circuit(12, 200, 36, 9))  # χ ≤ 26244
    assert st.stabilizer_rank > 8192
    rc, _ = _noalloc(lib, st, gpu_pkg.PauliString.from_str("Z0"))
    assert rc == _ffi.header_constants()["NSG_ERR_BUFFER_TOO_SMALL"]
    assert b"8192" in lib.nsg_last_error_message()
