"""Failure detection without a GPU fault.

The pair kernel's only waits are bounded polls of the mbarriers its bulk
copies complete (they stand where the reference would panic or hang:
form/resolve_superposition.rs:121, form/discard.rs:140,155 become status
words, a wait that never ends becomes NSG_ERR_TIMEOUT).  The test hook
nsg_debug_set_wait makes the first ket barrier of every chunk expect more
bytes than its copy delivers, with a short poll limit: the copy lands, the
phase stays open, the wait runs out, the warp records the timeout, waits for
its prefetch and leaves.  No address is invalid and no copy is in flight
when the kernel ends; the next call on the same state must succeed.
"""
from __future__ import annotations

import numpy as np
import pytest

from stab_decomp_simulator_rust_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,t", [(40, 10), (24, 9)])  # 64- and 32-bit rows
def test_bounded_wait_times_out_then_recovers(gpu_pkg, n, t):
    from stab_decomp_simulator_rust_gb300 import NecstarError, _ffi
    L = _ffi.load()
    codes = _ffi.header_constants()
    st = gpu_pkg.QuantumState.from_gates(n, W.random_clifford_t_circuit(n, 20 * n, t, 77))
    paulis = [gpu_pkg.PauliString.dense(p) for p in W.random_dense_paulis(n, 4, 78)]
    want = st.exp_values(paulis)
    _ffi.check(L.nsg_debug_set_wait(1 << 10, 16))
    try:
        with pytest.raises(NecstarError) as e:
            st.exp_values(paulis)
        assert e.value.code == codes["NSG_ERR_TIMEOUT"]
    finally:
        _ffi.check(L.nsg_debug_set_wait(0, 0))
    got = st.exp_values(paulis)  # the state and the context stay usable
    np.testing.assert_array_equal(got, want)
    assert abs(st.norm() - 1.0) < 1e-9


def test_wait_hook_argument_range(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import _ffi
    L = _ffi.load()
    assert L.nsg_debug_set_wait(0, 4096) == _ffi.header_constants()["NSG_ERR_INVALID_ARGUMENT"]
    _ffi.check(L.nsg_debug_set_wait(0, 0))
