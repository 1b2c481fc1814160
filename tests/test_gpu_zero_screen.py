"""The zero test on compiled states (nsg_zero_screen): the same answer as the
circuit-level test, carried through Clifford gates, clones and term
selections, dropped by projection, and sound against the pair sums."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_full_circuit

pytestmark = pytest.mark.gpu


def _paulis(pkg, n, count, seed):
    rng = np.random.default_rng(seed)
    return [pkg.PauliString.dense(rng.integers(0, 4, n).astype(np.uint8)) for _ in range(count)]


@pytest.mark.parametrize("n,nt,seed", [(8, 6, 401), (24, 10, 402), (40, 12, 403)])
def test_state_screen_follows_gates_and_is_sound(gpu_pkg, n, nt, seed):
    pkg = gpu_pkg
    gates = random_full_circuit(n, 20 * n, nt, seed)
    extra = random_full_circuit(n, 40, 0, seed + 1)
    ps = _paulis(pkg, n, 48, seed)
    st = pkg.QuantumState.from_gates(n, gates)
    want = pkg.zero_screen_circuit(n, gates, ps)
    np.testing.assert_array_equal(st.zero_screen(ps), want)
    many = pkg.QuantumState.from_gates_many([(n, gates)])[0]
    np.testing.assert_array_equal(many.zero_screen(ps), want)
    # gates one at a time (row kernel) and as a list (warp kernel)
    for i in range(0, 10):
        st.apply_gates(extra[i:i + 1])
    st.apply_gates(extra[10:])
    want2 = pkg.zero_screen_circuit(n, np.concatenate([gates, extra]), ps)
    np.testing.assert_array_equal(st.zero_screen(ps), want2)
    vals = st.exp_values(ps)
    assert np.all(vals[want2] == 0.0)
    np.testing.assert_array_equal(st.clone().zero_screen(ps), want2)
    np.testing.assert_array_equal(st.select(list(range(0, st.stabilizer_rank, 2))).zero_screen(ps), want2)
    st.project_unnormalized(0, False)
    assert not st.zero_screen(ps).any()  # unknown after a projection


def test_screened_evaluation_matches_the_pair_sums(gpu_pkg):
    """exp_values / exp_values_multi with screen=True give the same values as
    without: exact zeros where the test decides every observable of a state."""
    pkg = gpu_pkg
    from stab_decomp_simulator_rust_gb300 import workloads as W
    cs = W.batch_circuits()[:24]
    states = pkg.QuantumState.from_gates_many([(n, g) for n, g, _ in cs])
    pl = [[pkg.PauliString.dense(p) for p in ps] for _, _, ps in cs]
    want = pkg.exp_values_multi(states, pl, pkg.PRECISION_FP64)
    got = pkg.exp_values_multi(states, pl, pkg.PRECISION_FP64, screen=True)
    skipped = 0
    for s, ps, w, g in zip(states, pl, want, got):
        # a batch of other states may split the pair sums into other tasks: the last bits may differ
        np.testing.assert_allclose(g, w, rtol=1e-12, atol=1e-15)
        np.testing.assert_array_equal(s.exp_values(ps, screen=True), s.exp_values(ps))
        skipped += int(s.zero_screen(ps).all())
    assert skipped > 0
