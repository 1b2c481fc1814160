"""The CPU oracle pinned against the reference's own known-answer tests.

Each test cites the reference test it restates.  The reference (Rust) cannot
be built here, so these KATs plus an independent dense statevector simulator
(restated from crates/stabilizer-ch-form-rust/tests/common/mod.rs:108-200)
are what pin the oracle; the GPU path is then checked against the oracle.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from conftest import random_full_circuit, toffoli_gates

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "kats.json")
H, X, Y, Z, S, SDG, SX, SXDG, CX, CZ, SWAP, T, TDG, CCX = range(14)


def g(*rows):
    return np.asarray([tuple(r) + (0,) * (4 - len(r)) for r in rows], dtype=np.uint32).reshape(-1, 4)


@pytest.fixture(scope="module")
def kats():
    with open(GOLDEN) as f:
        return json.load(f)


def test_t_tensor_statevectors(oracle, kats):
    # crates/necstar/src/state/magic_states/t_state.rs:113-121 (t = 1..11)
    one = np.array([2 ** -0.5, 0.5 + 0.5j])
    ref = one
    for t in range(1, 12):
        st = oracle.OracleState.t_tensor(t)
        assert np.abs(st.to_statevector() - ref).max() < 1e-8, t
        assert st.stabilizer_rank == kats["t_tensor_rank"][str(t)]
        ref = np.kron(ref, one) if t < 11 else ref


def test_t_tensor_rank_recursion(oracle):
    # χ_T(t) = 2·χ_cat(t), χ_cat(m) = 3·χ_cat(m-4) for m ≥ 7 (cat_state.rs:162-188)
    cat = {1: 1, 2: 1, 3: 2, 4: 2, 5: 3, 6: 3}
    for m in range(7, 25):
        cat[m] = 3 * cat[m - 4]
    for t in (12, 16, 20, 24):
        assert oracle.OracleState.t_tensor(t).stabilizer_rank == 2 * cat[t]


def test_toffoli_state(oracle, kats):
    # stabilizer_decomposed_state/exp_value.rs:68-97; tests/test_state_calculation.py:68-82
    st = oracle.OracleState.from_circuit(3, toffoli_gates())
    ref, ex = st.exp_value(0, [0, 0, 3])  # "ZII" little-endian
    assert abs(ref - kats["toffoli"]["ZII"]) < 1e-10 and abs(ex - 0.5) < 1e-15
    ref, ex = st.exp_value(0, [0, 0, 0])
    assert abs(ref - 1.0) < 1e-10 and abs(ex - 1.0) < 1e-15
    sv = st.to_statevector()
    want = np.zeros(8, complex)
    want[kats["toffoli"]["support"]] = 0.5
    assert np.abs(sv - want).max() < 1e-10
    with pytest.raises(ValueError):
        st.exp_value(0, [3, 3, 0, 0])  # length mismatch


def test_state_initialization(oracle, kats):
    # tests/test_state_initialization.py:5-22
    st = oracle.OracleState.from_circuit(2, g((H, 0), (T, 0), (CX, 0, 1)))
    assert st.stabilizer_rank == kats["init"]["rank"]
    sv = st.to_statevector()
    want = np.array([complex(*c) for c in kats["init"]["statevector"]])
    assert np.abs(sv - want).max() < 1e-10
    assert abs(st.norm()[0] - 1.0) < 1e-10
    with pytest.raises(ValueError):
        oracle.OracleState.from_circuit(2, g((H, 0), (T, 3), (CX, 0, 1)))


def test_doctest_values(oracle, kats):
    # crates/necstar/src/state/mod.rs doctests
    d = kats["doctests"]
    st = oracle.OracleState.from_circuit(2, g((H, 0), (CX, 0, 1), (T, 0)))
    sv = st.to_statevector()
    assert abs(sv[0] - d["h_cx_t_amp0"]) < 1e-6 and abs(sv[3] - complex(*d["h_cx_t_amp3"])) < 1e-6
    a = oracle.OracleState.from_circuit(1, g((H, 0)))
    b = oracle.OracleState.from_circuit(1, g((X, 0)))
    ip, _ = a.inner_product(b)
    assert abs(ip - d["plus_minus_ip"]) < 1e-6
    bell = oracle.OracleState.from_circuit(2, g((H, 0), (CX, 0, 1)))
    assert abs(bell.exp_value(0, [3, 3])[0] - 1.0) < 1e-6
    pb = bell.clone()
    pb.project_normalized(0, False)
    assert abs(pb.norm()[0] - 1.0) < 1e-6 and abs(pb.to_statevector()[0] - 1.0) < 1e-6
    ub = bell.clone()
    ub.project_unnormalized(0, False)
    assert abs(ub.norm()[0] - d["bell_unnormalized_norm"]) < 1e-6


def test_gate_api(oracle):
    # crates/stabilizer-ch-form-rust/tests/gate_api.rs:6-61
    d = oracle.chform_run(1, g((H, 0)))
    assert np.abs(d["sv"] - np.array([2 ** -0.5, 2 ** -0.5])).max() < 1e-8
    d = oracle.chform_run(2, g((H, 0), (CX, 0, 1)))
    assert np.abs(d["sv"] - np.array([2 ** -0.5, 0, 0, 2 ** -0.5])).max() < 1e-8
    with pytest.raises(oracle.OracleError) as e:
        oracle.chform_run(2, g((H, 2)))
    assert e.value.code == 1 and e.value.args3[:2] == (2, 2)
    with pytest.raises(oracle.OracleError) as e:
        oracle.chform_run(2, g((CX, 0, 2)))
    assert e.value.code == 1 and e.value.args3[:2] == (2, 2)
    with pytest.raises(oracle.OracleError) as e:
        oracle.chform_run(2, g((CX, 1, 1)))
    assert e.value.code == 14 and e.value.args3[0] == 1


@pytest.mark.parametrize("n,seed", [(n, s) for n in (1, 2, 3, 4, 6, 8) for s in range(3)])
def test_clifford_chform_vs_dense(oracle, n, seed):
    # crates/stabilizer-ch-form-rust/tests/random_state.rs:5-91 (seeded here)
    gates = random_full_circuit(n, 60 * n, 0, 1000 + 17 * n + seed)
    d = oracle.chform_run(n, gates)
    ref = oracle.dense_simulate(n, gates)
    assert np.abs(d["sv"] - ref).max() < 1e-8


@pytest.mark.parametrize("n,nc,nt,seed", [(2, 20, 2, 1), (3, 40, 4, 2), (4, 60, 6, 3), (5, 100, 10, 4),
                                          (6, 100, 10, 5), (7, 150, 7, 6), (8, 150, 8, 7)])
def test_clifford_t_statevector_vs_dense(oracle, n, nc, nt, seed):
    # the compiled decomposition equals the circuit's statevector
    gates = random_full_circuit(n, nc, nt, seed)
    st = oracle.OracleState.from_circuit(n, gates)
    assert np.abs(st.to_statevector() - oracle.dense_simulate(n, gates)).max() < 1e-8


@pytest.mark.parametrize("i", range(5))
def test_inner_product_vs_statevector(oracle, i):
    # stabilizer_decomposed_state/inner_product.rs:61-82
    g1 = random_full_circuit(6, 100, 10, 42 + i)
    g2 = random_full_circuit(6, 100, 10, 123 + i)
    a, b = oracle.OracleState.from_circuit(6, g1), oracle.OracleState.from_circuit(6, g2)
    ip, ex = a.inner_product(b)
    naive = np.vdot(a.to_statevector(), b.to_statevector())
    assert abs(ip - naive) < 1e-8 and abs(ex - naive) < 1e-8


@pytest.mark.parametrize("i", range(8))
def test_projection_vs_statevector(oracle, i):
    # stabilizer_decomposed_state/projection.rs:112-181
    n = 5
    gates = random_full_circuit(n, 100, 10, i)
    st = oracle.OracleState.from_circuit(n, gates)
    sv = st.to_statevector()
    q, outcome = i % n, (i % 2) == 1
    mask = np.array([((k >> q) & 1) == outcome for k in range(1 << n)])
    st.project_unnormalized(q, outcome)
    assert np.abs(st.to_statevector() - np.where(mask, sv, 0)).max() < 1e-8


def test_projection_edge_cases(oracle):
    # projection.rs:244-323
    det = oracle.OracleState.from_circuit(2, g((H, 0), (S, 0), (CZ, 0, 1)))
    before = det.to_statevector()
    det.project_unnormalized(1, False)
    assert np.abs(det.to_statevector() - before).max() < 1e-12
    imp = oracle.OracleState.from_circuit(2, g((H, 0), (CZ, 0, 1)))
    with pytest.raises(oracle.OracleError) as e:
        imp.project_normalized(1, True)
    assert e.value.code == 9 and e.value.args3[:2] == (1, 1)
    imp = oracle.OracleState.from_circuit(2, g((H, 0), (CZ, 0, 1)))
    imp.project_unnormalized(1, True)
    assert imp.norm()[0] == 0.0
    with pytest.raises(oracle.OracleError) as e:
        oracle.OracleState.from_circuit(2, g((H, 0))).project_normalized(2, True)
    assert e.value.code == 1 and e.value.args3[:2] == (2, 2)


def test_discard_keeps_statevector(oracle):
    # form/discard.rs:193-229 and stabilizer_decomposed_state/discard.rs:20-44
    for i in range(6):
        n = 5
        gates = random_full_circuit(n, 80, 6, 300 + i)
        st = oracle.OracleState.from_circuit(n, gates)
        q = n - 1 - (i % n)
        st.project_unnormalized(q, False)
        sv = st.to_statevector()
        if st.stabilizer_rank == 0:
            continue
        st.discard(q)
        after = st.to_statevector()
        keep = np.array([((k >> q) & 1) == 0 for k in range(1 << n)])
        assert np.abs(sv[keep] - after).max() < 1e-8


def test_marginal_matches_statevector(oracle):
    n = 5
    gates = random_full_circuit(n, 100, 8, 77)
    st = oracle.OracleState.from_circuit(n, gates)
    probs = np.abs(st.to_statevector()) ** 2
    qargs = [3, 0, 4]
    marg = st.marginal(qargs)
    for outc, p in marg.items():
        want = sum(probs[k] for k in range(1 << n)
                   if all(((k >> q) & 1) == ((outc >> i) & 1) for i, q in enumerate(qargs)))
        assert abs(p - want) < 1e-10
    assert abs(sum(marg.values()) - 1.0) < 1e-10


def test_sampling_toffoli_marginal(oracle):
    # stabilizer_decomposed_state/sampling.rs:198-254: four equiprobable outcomes
    st = oracle.OracleState.from_circuit(3, toffoli_gates())
    marg = st.marginal([0, 1, 2])
    assert sorted(marg) == [0b000, 0b001, 0b010, 0b111]
    assert all(abs(p - 0.25) < 1e-12 for p in marg.values())


def test_measure_collapses(oracle):
    # tests/test_state_simulation.py:82-105
    for i in range(6):
        st = oracle.OracleState.from_circuit(3, toffoli_gates())
        bits = st.measure([0, 1, 2], seed=bytes([i]) * 32)
        k = sum(int(b) << j for j, b in enumerate(bits))
        assert k in (0, 1, 2, 7)
        sv = st.to_statevector()
        assert abs(abs(sv[k]) - 1.0) < 1e-9


def test_reference_order_fp64_close_to_exact(oracle):
    gates = random_full_circuit(8, 200, 12, 5)
    st = oracle.OracleState.from_circuit(8, gates)
    rng = np.random.default_rng(0)
    for _ in range(4):
        p = rng.integers(0, 4, 8)
        ref, ex = st.exp_value(0, p)
        assert abs(ref - ex) < 1e-12


@pytest.mark.parametrize("seed", [61, 62, 63])
def test_kron_vs_statevectors(oracle, seed):
    # stabilizer_decomposed_state/kron.rs:27-45: the kron state's statevector is the
    # tensor product of the factors' (qubits of the second factor after the first's)
    ga = random_full_circuit(3, 40, 3, seed)
    gb = random_full_circuit(4, 50, 2, seed + 10)
    a = oracle.OracleState.from_circuit(3, ga)
    b = oracle.OracleState.from_circuit(4, gb)
    k = a.kron(b)
    assert k.num_qubits == 7 and k.stabilizer_rank == a.stabilizer_rank * b.stabilizer_rank
    assert np.abs(k.to_statevector() - np.kron(b.to_statevector(), a.to_statevector())).max() < 1e-9
    assert np.abs(k.to_statevector() - np.kron(oracle.dense_simulate(4, gb), oracle.dense_simulate(3, ga))).max() < 1e-9


def test_measure_uses_the_seeded_stream(oracle):
    # measurement.rs:34-103: one rng.gen::<f64>() per measured qubit, outcome 1 iff the draw is not
    # below p0/(p0+p1); on |+⟩^n every p0 is 1/2, so the outcomes are the stream's.
    n = 10
    plus = g(*[(H, q) for q in range(n)])
    for s in range(5):
        seed = bytes([3 * s + 2]) * 32
        st = oracle.OracleState.from_circuit(n, plus)
        u = oracle.random_doubles(seed, n)
        assert st.measure(list(range(n)), seed) == [bool(x >= 0.5) for x in u]


def test_toffoli_state_statevector(oracle):
    """construct_toffoli_state (magic_states/toffoli_state.rs:5-9): (|000⟩ + |100⟩ + |010⟩ + |111⟩)/2,
    qubit 0 first in the text form, i.e. the little-endian indices 0, 1, 2, 7."""
    sv = oracle.OracleState.toffoli_tensor(1).to_statevector()
    want = np.zeros(8, complex)
    want[[0, 1, 2, 7]] = 0.5
    assert np.abs(sv - want).max() < 1e-12
    two = oracle.OracleState.toffoli_tensor(2)
    assert (two.num_qubits, two.stabilizer_rank) == (6, 4)
    assert np.abs(two.to_statevector() - np.kron(want, want)).max() < 1e-12  # kron puts the new factor on top
    with pytest.raises(ValueError):
        oracle.OracleState.toffoli_tensor(0)
