"""GPU parity of the batched forms: many observables and many states of
uneven width and rank in one persistent pair launch (nsg_exp_value_multi,
nsg_exp_value_batch beyond 256 observables), FP64 and mixed accumulation,
against the oracle's exact sums to 1e-9."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_full_circuit
from stab_decomp_simulator_rust_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-9


def close(a, b, tol=TOL):
    return abs(a - b) <= tol * max(1.0, abs(b))


def oracle_values(oracle, n, gates, paulis):
    """The oracle's exact ⟨P⟩ (its exact accumulator over the full χ² sum, rows on all host threads)."""
    ref = oracle.OracleState.from_circuit(n, gates)
    ops = [(0, p.ops, None) if p.kind == 0 else (1, p.ops, p.qubits) for p in paulis]
    _, exact = ref.exp_value_counts(ops, 192, 512)
    return list(exact)


# widths on both sides of the 32-bit / 64-bit row boundary, uneven T counts
BATCH = [(3, 60, 4, 101), (12, 200, 9, 102), (31, 400, 8, 103), (32, 400, 10, 104), (33, 400, 7, 105),
         (40, 500, 12, 106), (64, 700, 9, 107), (8, 100, 0, 108), (20, 300, 11, 109)]


@pytest.mark.parametrize("precision", [0, 1])
def test_multi_matches_oracle(gpu_pkg, oracle, precision):
    states, plists, expect = [], [], []
    for idx, (n, nc, nt, seed) in enumerate(BATCH):
        gates = random_full_circuit(n, nc, nt, seed)
        rng = np.random.default_rng(seed)
        k = [5, 17, 40, 1, 3, 33, 2, 4, 0][idx]  # uneven observable counts, one state with none
        paulis = [gpu_pkg.PauliString.dense(rng.integers(0, 4, n)) for _ in range(k)]
        states.append(gpu_pkg.QuantumState.from_gates(n, gates))
        plists.append(paulis)
        expect.append(oracle_values(oracle, n, gates, paulis))
    got = gpu_pkg.exp_values_multi(states, plists, precision)
    assert [len(g) for g in got] == [len(p) for p in plists]
    for c, (g, e) in enumerate(zip(got, expect)):
        for o, (x, y) in enumerate(zip(g, e)):
            assert close(x, y), (c, o, x, y)
    # the per-state batched call gives the same values
    for c, st in enumerate(states):
        if plists[c]:
            single = st.exp_values(plists[c], precision)
            assert np.all(np.abs(single - got[c]) <= TOL * np.maximum(1.0, np.abs(single)))


def test_batch_beyond_256_observables(gpu_pkg, oracle):
    n, gates = 10, random_full_circuit(10, 200, 8, 111)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    rng = np.random.default_rng(111)
    paulis = [gpu_pkg.PauliString.dense(rng.integers(0, 4, n)) for _ in range(300)]
    got = st.exp_values(paulis)
    pick = [0, 1, 255, 256, 257, 299]
    ex = oracle_values(oracle, n, gates, [paulis[i] for i in pick])
    for i, e in zip(pick, ex):
        assert close(got[i], e), (i, got[i], e)
    # identical observables in both units give identical values
    rep = st.exp_values([paulis[3]] * 260)
    assert np.all(rep == rep[0])


def test_multi_batching_workload_subset(gpu_pkg, oracle):
    """Circuits of the 512-circuit batching workload (n ~ U[8, 64], t ~ U[4, 32],
    20·n Clifford gates, 16 observables each) whose oracle sums finish quickly."""
    circuits = W.batch_circuits()
    picked = []
    for n, gates, paulis in circuits[:60]:
        t = int((np.asarray(gates)[:, 0] == 11).sum())
        if t <= 17:
            picked.append((n, gates, paulis))
    assert len(picked) >= 10
    states = [gpu_pkg.QuantumState.from_gates(n, g) for n, g, _ in picked]
    plists = [[gpu_pkg.PauliString.dense(p) for p in ps] for _, _, ps in picked]
    got64 = gpu_pkg.exp_values_multi(states, plists, 0)
    gotmx = gpu_pkg.exp_values_multi(states, plists, 1)
    for c, (n, g, _) in enumerate(picked):
        ex = oracle_values(oracle, n, g, plists[c])
        for o, e in enumerate(ex):
            assert close(got64[c][o], e), (c, o, got64[c][o], e)
            assert close(gotmx[c][o], e), (c, o, gotmx[c][o], e)


def test_multi_argument_checks(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import NecstarError
    a = gpu_pkg.QuantumState.from_gates(3, random_full_circuit(3, 20, 2, 5))
    with pytest.raises(NecstarError) as e:
        gpu_pkg.exp_values_multi([a], [[gpu_pkg.PauliString.from_str("ZZ")]])
    assert e.value.code == 11
    assert gpu_pkg.exp_values_multi([], []) == []
    with pytest.raises(ValueError):
        gpu_pkg.exp_values_multi([a], [])


def test_states_from_circuits_equal_single_compiles(gpu_pkg):
    """The batched compile gives, circuit by circuit, the terms of nsg_state_from_circuit."""
    circuits = [(n, g) for n, g, _ in W.batch_circuits()[:24]]
    circuits.append((70, random_full_circuit(70, 300, 5, 41)))  # width 75: two-word rows while compiling
    many = gpu_pkg.QuantumState.from_gates_many(circuits)
    assert len(many) == len(circuits)
    for (n, g), st in zip(circuits, many):
        one = gpu_pkg.QuantumState.from_gates(n, g)
        a, b = st.export_terms(), one.export_terms()
        for k in ("G", "F", "M", "gamma", "v", "s", "phase", "coef_phase", "coef_r"):
            assert np.array_equal(a[k], b[k]), (n, k)
    assert gpu_pkg.QuantumState.from_gates_many([]) == []


def test_states_from_circuits_reports_the_failing_circuit(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import NecstarError
    good = W.random_clifford_t_circuit(5, 40, 2, 3)
    bad = np.asarray([[W.OP["CX"], 1, 1, 0]], np.uint32)
    with pytest.raises(NecstarError) as e:
        gpu_pkg.QuantumState.from_gates_many([(5, good), (5, good), (5, bad)])
    assert e.value.code == 14 and e.value.args3[2] == 2
    with pytest.raises(NecstarError) as e:
        gpu_pkg.QuantumState.from_gates_many([(5, good), (0, good)])
    assert e.value.code == 2 and e.value.args3[2] == 1
