"""GPU sampling and measurement against the oracle's exact marginals.

The reference's seeded streams come from ChaCha12 (rand_chacha 0.3.1), which
is not in the repository, so seeded outcomes are compared as distributions
(total-variation distance within a multinomial tolerance), as the reference's
own statistical tests do (stabilizer_decomposed_state/sampling.rs:198-254,
measurement.rs:181-216).  Both sampling strategies are covered: the marginal
pass (≤ 8 qubits) and the per-node projection tree (more qubits).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_full_circuit, toffoli_gates

pytestmark = pytest.mark.gpu


def tvd(counts: dict, probs: dict, shots: int) -> float:
    keys = set(counts) | set(probs)
    return 0.5 * sum(abs(counts.get(k, 0) / shots - probs.get(k, 0.0)) for k in keys)


def tvd_bound(support: int, shots: int) -> float:
    # E[TVD] ≤ ½·Σ sqrt(p(1-p)/N) ≤ ½·sqrt(K/N); allow a generous multiple.
    return 3.0 * 0.5 * np.sqrt(support / shots) + 1e-3


def test_toffoli_sampling_known_answer(gpu_pkg):
    # sampling.rs:198-254: outcomes 000, 001, 010, 111 (bit i = qubit i), each 1/4
    st = gpu_pkg.QuantumState.from_gates(3, toffoli_gates())
    shots = 20000
    vals, cnts = st.sample_raw([0, 1, 2], shots, seed=7)
    got = dict(zip(vals, cnts))
    assert set(got) <= {0b000, 0b001, 0b010, 0b111}
    assert sum(cnts) == shots
    for k in (0b000, 0b001, 0b010, 0b111):
        assert abs(got.get(k, 0) / shots - 0.25) < 0.02
    # string form: character i is qargs[i] (here q2, q1, q0)
    d = st.sample([2, 1, 0], 1000, seed=3)
    assert set(d) <= {"000", "001", "010", "111"} and sum(d.values()) == 1000


@pytest.mark.parametrize("n,nc,nt,seed,qargs", [
    (6, 150, 8, 201, [0, 3, 5]),           # marginal pass
    (9, 200, 10, 202, [8, 1, 4, 6, 2, 0]),  # unsorted qargs, marginal pass
    (10, 250, 9, 203, list(range(8))),      # 8 qubits: the largest marginal pass
    (10, 250, 9, 204, list(range(10))),     # 10 qubits: projection tree
    (40, 300, 8, 205, [39, 0, 17, 22]),     # wide state
])
def test_sampling_matches_marginal(gpu_pkg, oracle, n, nc, nt, seed, qargs):
    gates = random_full_circuit(n, nc, nt, seed)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    marg = ref.marginal(qargs)
    shots = 40000
    vals, cnts = st.sample_raw(qargs, shots, seed=seed)
    assert sum(cnts) == shots
    for v in vals:  # never an outcome of probability 0
        assert marg.get(v, 0.0) > 1e-12, v
    got = dict(zip(vals, cnts))
    support = sum(1 for p in marg.values() if p > 0)
    assert tvd(got, marg, shots) < tvd_bound(support, shots)


def test_sampling_seed_determinism(gpu_pkg):
    gates = random_full_circuit(7, 150, 8, 211)
    st = gpu_pkg.QuantumState.from_gates(7, gates)
    a = st.sample_raw([0, 1, 2, 3], 5000, seed=11)
    b = st.sample_raw([0, 1, 2, 3], 5000, seed=11)
    c = st.sample_raw([0, 1, 2, 3], 5000, seed=12)
    assert a == b
    assert a != c
    # the tree path is deterministic too
    t1 = st.sample_raw(list(range(7)), 3000, seed=5)
    t2 = st.sample_raw(list(range(7)), 3000, seed=5)
    assert t1 == t2


def test_measure_distribution_and_collapse(gpu_pkg, oracle):
    n, gates = 5, random_full_circuit(5, 120, 6, 221)
    ref = oracle.OracleState.from_circuit(n, gates)
    marg = ref.marginal([1, 3])
    counts: dict = {}
    trials = 400
    for t in range(trials):
        st = gpu_pkg.QuantumState.from_gates(n, gates)
        bits = st.measure([1, 3], seed=1000 + t)
        k = int(bits[0]) | (int(bits[1]) << 1)
        counts[k] = counts.get(k, 0) + 1
        assert marg.get(k, 0.0) > 1e-12
        if t < 10:  # the state collapsed: measuring again repeats the outcome
            again = st.measure([1, 3], seed=5)
            assert again == bits
            assert abs(st.norm() - 1.0) < 1e-9
    assert tvd(counts, marg, trials) < tvd_bound(len(marg), trials)


def test_measure_all_known_answer(gpu_pkg):
    # tests/test_state_simulation.py:82-105: the Toffoli state collapses to one of four basis states
    for i in range(6):
        st = gpu_pkg.QuantumState.from_gates(3, toffoli_gates())
        bits = st.measure_all(seed=bytes([i]) * 32)
        k = sum(int(b) << j for j, b in enumerate(bits))
        assert k in (0, 1, 2, 7)
        sv = st.to_statevector()
        assert abs(abs(sv[k]) - 1.0) < 1e-9


def test_measure_draws_the_reference_stream(gpu_pkg, oracle):
    # measure() takes one rng.gen::<f64>() per measured qubit from
    # StdRng::from_seed(seed) and returns 1 iff the draw is not below
    # p0 / (p0 + p1) (measurement.rs:34-103).  On |+⟩^n every p0 is 1/2, so
    # the outcomes are fixed by the stream alone.
    from conftest import OP
    n = 12
    plus = [(OP["H"], q, 0, 0) for q in range(n)]
    for s in range(6):
        seed = bytes([17 * s + 1]) * 32
        st = gpu_pkg.QuantumState.from_gates(n, plus)
        u = oracle.random_doubles(seed, n)
        assert st.measure(list(range(n)), seed=seed) == [bool(x >= 0.5) for x in u]
    # On Clifford+T states the outcomes equal the oracle's for the same seed.
    for n, nc, nt, gseed in ((6, 150, 7, 231), (9, 220, 9, 232)):
        gates = random_full_circuit(n, nc, nt, gseed)
        qargs = list(range(n))[::-1]
        for s in range(4):
            seed = (gseed * 1000 + s).to_bytes(8, "little") + bytes(24)
            ref = oracle.OracleState.from_circuit(n, gates)
            st = gpu_pkg.QuantumState.from_gates(n, gates)
            assert st.measure(qargs, seed=seed) == ref.measure(qargs, seed)
