"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tableaux, γ, v, s, Z8 phases and coefficient exponents must be bit-exact;
every pair value ⟨S_i|P|S_j⟩ must be the exact (k, r) of the oracle;
expectation values, norms and inner products must agree with the oracle's
exact sums to 1e-9 (absolute, and relative for |value| > 1).
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_full_circuit, toffoli_gates
from stab_decomp_simulator_rust_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-9
FIELDS = ("G", "F", "M", "gamma", "v", "s", "phase", "coef_phase", "coef_r")


def close(a, b, tol=TOL):
    return abs(a - b) <= tol * max(1.0, abs(b))


def assert_same_terms(dg, dr):
    assert dg["n"] == dr["n"]
    assert len(dg["phase"]) == len(dr["phase"])
    for k in FIELDS:
        assert np.array_equal(dg[k], dr[k]), f"field {k} differs"


CASES = [
    (1, 5, 0, 11), (2, 30, 1, 12), (3, 60, 3, 13), (5, 100, 6, 14), (6, 100, 10, 15),
    (8, 200, 7, 16), (12, 300, 9, 17), (20, 500, 12, 18), (31, 400, 8, 19), (33, 500, 10, 20),
    (40, 800, 14, 21), (50, 600, 16, 22), (64, 700, 12, 23),
]


@pytest.mark.parametrize("n,nc,nt,seed", CASES)
def test_compile_bit_exact(gpu_pkg, oracle, n, nc, nt, seed):
    gates = random_full_circuit(n, nc, nt, seed)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    assert st.num_qubits == ref.num_qubits
    assert st.stabilizer_rank == ref.stabilizer_rank
    assert_same_terms(st.export_terms(), ref.export_terms())


def test_compile_wide_ancillas_bit_exact(gpu_pkg, oracle):
    # n + t > 64: the compile kernel runs with two-word rows
    n, t = 40, 30
    gates = W.random_clifford_t_circuit(n, 600, t, 99)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    assert_same_terms(st.export_terms(), ref.export_terms())


def test_small_benchmark_circuit_bit_exact(gpu_pkg, oracle):
    cfg = W.SMALL_N16
    g = W.random_clifford_t_circuit(cfg["n"], cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    st = gpu_pkg.QuantumState.from_gates(cfg["n"], g)
    ref = oracle.OracleState.from_circuit(cfg["n"], g)
    assert_same_terms(st.export_terms(), ref.export_terms())


def test_small_benchmark_outputs(gpu_pkg, oracle):
    """The outputs asked of the n = 16 workload: ⟨Z₀⟩; the amplitude ⟨0¹⁶|ψ⟩, which the reference
    obtains as from_circuit(QuantumCircuit::new(16)).inner_product(ψ) (state/mod.rs:165-172);
    and sample(0..15, 1024), whose bit-0 frequency and total parity follow ⟨Z₀⟩ and ⟨Z^{⊗16}⟩."""
    cfg = W.SMALL_N16
    n = cfg["n"]
    g = W.random_clifford_t_circuit(n, cfg["num_clifford"], cfg["num_t"], cfg["seed"])
    st = gpu_pkg.QuantumState.from_gates(n, g)
    ref = oracle.OracleState.from_circuit(n, g)
    z0 = [3] + [0] * (n - 1)
    _, want_z0 = ref.exp_value(0, z0)
    got_z0 = st.exp_value(gpu_pkg.PauliString.dense(z0))
    assert close(got_z0, want_z0)
    empty = np.zeros((0, 4), np.uint32)
    amp = gpu_pkg.QuantumState.from_gates(n, empty).inner_product(st)
    _, want_amp = oracle.OracleState.from_circuit(n, empty).inner_product(ref)
    assert abs(amp - want_amp) <= TOL
    assert abs(amp - st.to_statevector()[0]) <= TOL
    shots = 1024
    vals, cnts = st.sample_raw(list(range(n)), shots, seed=16)
    assert sum(cnts) == shots
    probs = np.abs(st.to_statevector()) ** 2
    assert all(probs[v] > 1e-12 for v in vals)
    zall = st.exp_value(gpu_pkg.PauliString.dense([3] * n))
    f0 = sum(c for v, c in zip(vals, cnts) if not v & 1) / shots
    fpar = sum(c for v, c in zip(vals, cnts) if bin(v).count("1") % 2 == 0) / shots
    assert abs(f0 - (1 + got_z0) / 2) < 5 * 0.5 / shots ** 0.5
    assert abs(fpar - (1 + zall) / 2) < 5 * 0.5 / shots ** 0.5


@pytest.mark.parametrize("t", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 16, 21, 24])
def test_device_t_tensor_bit_exact(gpu_pkg, oracle, t):
    """The device expansion of |T⟩^{⊗t} (t_state.rs:29-71): every term, phase and
    coefficient in the oracle's order."""
    dg = gpu_pkg.QuantumState.debug_t_tensor(t).export_terms()
    dr = oracle.OracleState.t_tensor(t).export_terms()
    assert_same_terms(dg, dr)


@pytest.mark.parametrize("n,nc,nt,seed", [(3, 40, 4, 31), (6, 100, 10, 32), (12, 200, 8, 33),
                                          (33, 300, 7, 34), (40, 400, 9, 35)])
def test_pair_values_exact(gpu_pkg, oracle, n, nc, nt, seed):
    gates = random_full_circuit(n, nc, nt, seed)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    chi = st.stabilizer_rank
    rng = np.random.default_rng(seed)
    paulis = [None, rng.integers(0, 4, n)]
    for p in paulis:
        k, r = st.debug_pair_values(None if p is None else gpu_pkg.PauliString.dense(p))
        for i in range(chi):
            for j in range(chi):
                z, kk, rr = ref.pair_scalar(i, j, None if p is None else (0, p, None))
                if z:
                    assert k[i, j] == 255, (i, j)
                else:
                    assert (k[i, j], r[i, j]) == (kk, rr), (i, j, k[i, j], r[i, j], kk, rr)


def test_toffoli_known_answers(gpu_pkg):
    # tests/test_state_calculation.py:68-82, stabilizer_decomposed_state/exp_value.rs:68-88
    PS = gpu_pkg.PauliString
    st = gpu_pkg.QuantumState.from_gates(3, toffoli_gates())
    assert close(st.exp_value(PS.from_str("ZII")), 0.5)
    assert close(st.exp_value(PS.from_str("III")), 1.0)
    assert close(st.norm(), 1.0)
    sv = st.to_statevector()
    ref = np.zeros(8, complex)
    ref[[0, 1, 2, 7]] = 0.5
    assert np.abs(sv - ref).max() < 1e-10
    with pytest.raises(ValueError):
        st.exp_value(PS.from_str("ZZIIII"))
    with pytest.raises(ValueError):
        st.exp_value(PS.from_str("Z0 Y2 X4"))
    with pytest.raises(ValueError):
        st.exp_value(PS.from_str("ZI"))


def test_state_initialization_known_answers(gpu_pkg):
    # tests/test_state_initialization.py:5-22
    c = gpu_pkg.QuantumCircuit(2)
    c.apply_h(0)
    c.apply_t(0)
    c.apply_cx(0, 1)
    st = gpu_pkg.QuantumState.from_circuit(c)
    assert st.num_qubits == 2 and st.stabilizer_rank == 2
    ref = [1 / 2 ** 0.5, 0.0, 0.0, 0.5 + 0.5j]
    for a, b in zip(st.to_statevector(), ref):
        assert abs(a - b) < 1e-10
    assert abs(st.norm() - 1.0) < 1e-10
    assert str(st) == "QuantumState(num_qubits=2, stabilizer_rank=2)"
    bad = gpu_pkg.QuantumCircuit(2)
    bad.apply_h(0)
    bad.apply_t(3)
    bad.apply_cx(0, 1)
    with pytest.raises(ValueError):
        gpu_pkg.QuantumState.from_circuit(bad)


@pytest.mark.parametrize("n,nc,nt,seed", [(5, 100, 10, 41), (8, 150, 12, 42), (16, 300, 10, 43),
                                          (30, 500, 12, 44), (40, 600, 14, 45), (64, 800, 10, 46)])
def test_exp_values_match_oracle(gpu_pkg, oracle, n, nc, nt, seed):
    gates = random_full_circuit(n, nc, nt, seed)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    rng = np.random.default_rng(seed)
    dense = [rng.integers(0, 4, n) for _ in range(5)] + [np.zeros(n, int)]
    paulis = [gpu_pkg.PauliString.dense(p) for p in dense]
    sparse = gpu_pkg.PauliString.sparse([3, 1, 2], [0, n // 2, n - 1]) if n >= 3 else None
    if sparse is not None:
        paulis.append(sparse)
    got_batch = st.exp_values(paulis)
    got_mixed = st.exp_values(paulis, precision=gpu_pkg.PRECISION_MIXED)
    for idx, p in enumerate(paulis):
        if p.kind == 0:
            _, ex = ref.exp_value(0, p.ops)
        else:
            _, ex = ref.exp_value(1, p.ops, p.qubits)
        single = st.exp_value(p)
        assert close(single, ex), (idx, single, ex)
        assert close(got_batch[idx], ex), (idx, got_batch[idx], ex)
        assert close(got_mixed[idx], ex), (idx, got_mixed[idx], ex)


@pytest.mark.parametrize("n,nc,nt,seed", [(4, 80, 5, 51), (10, 200, 8, 52), (40, 500, 10, 53)])
def test_norm_and_inner_product(gpu_pkg, oracle, n, nc, nt, seed):
    g1 = random_full_circuit(n, nc, nt, seed)
    g2 = random_full_circuit(n, nc, nt, seed + 1000)
    a, b = gpu_pkg.QuantumState.from_gates(n, g1), gpu_pkg.QuantumState.from_gates(n, g2)
    ra, rb = oracle.OracleState.from_circuit(n, g1), oracle.OracleState.from_circuit(n, g2)
    assert close(a.norm(), ra.norm()[1] ** 0.5)
    ip = a.inner_product(b)
    _, ex = ra.inner_product(rb)
    assert abs(ip - ex) <= TOL * max(1.0, abs(ex)), (ip, ex)
    ip2 = b.inner_product(a)
    assert abs(ip2 - ex.conjugate()) <= TOL * max(1.0, abs(ex))
    # ⟨0^n|ψ⟩ through the inner product (the amplitude output of the small benchmark)
    z = gpu_pkg.QuantumState.from_gates(n, np.zeros((0, 4), np.uint32))
    rz = oracle.OracleState.from_circuit(n, np.zeros((0, 4), np.uint32))
    amp = z.inner_product(a)
    _, amp_ex = rz.inner_product(ra)
    assert abs(amp - amp_ex) <= TOL


@pytest.mark.parametrize("n,nc,nt,seed", [(5, 100, 10, 61), (9, 150, 8, 62), (12, 200, 6, 63)])
def test_statevector_matches_oracle(gpu_pkg, oracle, n, nc, nt, seed):
    gates = random_full_circuit(n, nc, nt, seed)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    sv = st.to_statevector()
    dense = oracle.dense_simulate(n, gates)
    assert np.abs(sv - dense).max() < 1e-9


@pytest.mark.parametrize("n,nc,nt,seed", [(5, 100, 10, 71), (8, 150, 8, 72), (40, 400, 10, 73)])
def test_project_and_discard_bit_exact(gpu_pkg, oracle, n, nc, nt, seed):
    gates = random_full_circuit(n, nc, nt, seed)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    rng = np.random.default_rng(seed)
    for step in range(3):
        q = int(rng.integers(0, st.num_qubits))
        outcome = bool(rng.integers(0, 2))
        st.project_unnormalized(q, outcome)
        ref.project_unnormalized(q, outcome)
        assert_same_terms(st.export_terms(), ref.export_terms())
        # discard a qubit that is |0> after projecting it (discard.rs precondition)
        q2 = int(rng.integers(0, st.num_qubits))
        st.project_unnormalized(q2, False)
        ref.project_unnormalized(q2, False)
        if st.stabilizer_rank == 0:
            break
        st.discard(q2)
        ref.discard(q2)
        assert_same_terms(st.export_terms(), ref.export_terms())


def test_project_normalized_values(gpu_pkg, oracle):
    # projection.rs:140-181: projected statevector against the oracle
    for i in range(12):
        n = 5
        gates = random_full_circuit(n, 100, 10, 123 + i)
        st = gpu_pkg.QuantumState.from_gates(n, gates)
        ref = oracle.OracleState.from_circuit(n, gates)
        q, outcome = (i + 1) % n, (i % 2) == 0
        try:
            ref.project_normalized(q, outcome)
            ok = True
        except ValueError:
            ok = False
        if ok:
            st.project_normalized(q, outcome)
            assert np.abs(st.to_statevector() - ref.to_statevector()).max() < 1e-9
        else:
            with pytest.raises(ValueError):
                st.project_normalized(q, outcome)


def test_project_impossible_norm_zero(gpu_pkg):
    # projection.rs:258-293
    c = gpu_pkg.QuantumCircuit(2)
    c.apply_h(0)
    c.apply_cz(0, 1)
    st = gpu_pkg.QuantumState.from_circuit(c)
    with pytest.raises(ValueError):
        st.project_normalized(1, True)
    st = gpu_pkg.QuantumState.from_circuit(c)
    st.project_unnormalized(1, True)
    assert st.norm() == 0.0


@pytest.mark.parametrize("n,nc,nt,seed", [(6, 100, 8, 81), (40, 300, 8, 82)])
def test_apply_gates_bit_exact(gpu_pkg, oracle, n, nc, nt, seed):
    gates = random_full_circuit(n, nc, nt, seed)
    extra = random_full_circuit(n, 60, 0, seed + 7)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    st.apply_gates(extra)
    ref.apply_gates(extra)
    assert_same_terms(st.export_terms(), ref.export_terms())
    with pytest.raises(ValueError):
        st.apply_gates(np.asarray([[11, 0, 0, 0]], np.uint32))  # T on a compiled state


@pytest.mark.parametrize("n,nt,seed", [(6, 8, 91), (40, 8, 92), (70, 6, 93)])
def test_apply_gates_one_by_one_bit_exact(gpu_pkg, oracle, n, nt, seed):
    """Gate-by-gate calls — a single gate without H, or a short list of them,
    goes through the row kernel (one thread per term), lists with H through
    the warp kernel — leave the terms of the whole list applied at once
    (rows of one and two 64-bit words)."""
    gates = random_full_circuit(n, 120, nt, seed)
    extra = random_full_circuit(n, 90, 0, seed + 7)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    i = 0
    while i < len(extra):
        k = 3 if i % 4 == 0 else 1
        st.apply_gates(extra[i:i + k])
        i += k
    ref.apply_gates(extra)
    assert_same_terms(st.export_terms(), ref.export_terms())


def test_error_codes(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import NecstarError
    QS, PS = gpu_pkg.QuantumState, gpu_pkg.PauliString
    with pytest.raises(NecstarError) as e:
        QS.from_gates(2, np.asarray([[0, 2, 0, 0]], np.uint32))
    assert e.value.code == 1 and e.value.args3[:2] == (2, 2)
    with pytest.raises(NecstarError) as e:
        QS.from_gates(2, np.asarray([[8, 1, 1, 0]], np.uint32))
    assert e.value.code == 14 and e.value.args3[0] == 1
    with pytest.raises(NecstarError) as e:
        QS.from_gates(2, np.asarray([[13, 0, 1, 0]], np.uint32))
    assert e.value.code == 13
    with pytest.raises(NecstarError) as e:
        QS.from_gates(0, np.zeros((0, 4), np.uint32))
    assert e.value.code == 2
    st = QS.from_gates(3, toffoli_gates())
    with pytest.raises(NecstarError) as e:
        st.sample([0, 1, 3], 100)
    assert e.value.code == 1 and e.value.args3[:2] == (3, 3)
    with pytest.raises(NecstarError) as e:
        st.sample([0, 1, 1], 100)
    assert e.value.code == 10 and e.value.args3[0] == 1
    with pytest.raises(NecstarError) as e:
        st.sample([], 100)
    assert e.value.code == 12
    small = QS.from_gates(2, np.asarray([[0, 0, 0, 0]], np.uint32))
    with pytest.raises(NecstarError) as e:
        st.inner_product(small)
    assert e.value.code == 6
    with pytest.raises(NecstarError) as e:
        st.discard(3)
    assert e.value.code == 1
    with pytest.raises(NecstarError) as e:
        st.exp_value(PS.from_str("ZZZZ"))
    assert e.value.code == 11 and e.value.args3[:2] == (3, 4)


@pytest.mark.parametrize("n,nc,nt,seed", [(1, 0, 0, 401), (1, 6, 3, 402), (2, 10, 0, 403), (2, 12, 4, 404),
                                          (3, 20, 7, 405)])
def test_tiny_states_every_pauli(gpu_pkg, oracle, n, nc, nt, seed):
    """Widths 1-3, with and without T gates (χ = 1 included): every dense Pauli,
    the norm, ⟨0ⁿ|ψ⟩ and the statevector against the oracle."""
    import itertools
    gates = random_full_circuit(n, nc, nt, seed) if nc + nt else np.zeros((0, 4), np.uint32)
    st = gpu_pkg.QuantumState.from_gates(n, gates)
    ref = oracle.OracleState.from_circuit(n, gates)
    ops_all = [np.asarray(o, np.uint8) for o in itertools.product(range(4), repeat=n)]
    got = st.exp_values([gpu_pkg.PauliString.dense(o) for o in ops_all])
    for o, g in zip(ops_all, got):
        _, ex = ref.exp_value(0, o)
        assert close(g, ex), (o, g, ex)
    assert close(st.norm(), ref.norm()[1] ** 0.5)
    z = gpu_pkg.QuantumState.from_gates(n, np.zeros((0, 4), np.uint32))
    rz = oracle.OracleState.from_circuit(n, np.zeros((0, 4), np.uint32))
    amp = z.inner_product(st)
    _, amp_ex = rz.inner_product(ref)
    assert abs(amp - amp_ex) <= TOL
    assert np.allclose(st.to_statevector(), ref.to_statevector(), atol=1e-12)


@pytest.mark.parametrize("na,nb,seed", [(1, 1, 81), (3, 5, 82), (20, 12, 83), (30, 34, 84), (40, 24, 85),
                                        (64, 64, 86)])
def test_state_kron_bit_exact(gpu_pkg, oracle, na, nb, seed):
    """A ⊗ B on the device (stabilizer_decomposed_state/kron.rs:7-22): every term equal
    to the oracle's, in i-major order; ⟨P_A ⊗ P_B⟩ = ⟨P_A⟩·⟨P_B⟩."""
    ga = random_full_circuit(na, 12 * na, 3, seed)
    gb = random_full_circuit(nb, 12 * nb, 2, seed + 100)
    a = gpu_pkg.QuantumState.from_gates(na, ga)
    b = gpu_pkg.QuantumState.from_gates(nb, gb)
    k = a.kron(b)
    assert k.num_qubits == na + nb and k.stabilizer_rank == a.stabilizer_rank * b.stabilizer_rank
    rk = oracle.OracleState.from_circuit(na, ga).kron(oracle.OracleState.from_circuit(nb, gb))
    assert_same_terms(k.export_terms(), rk.export_terms())
    if na + nb <= 64:
        rng = np.random.default_rng(seed)
        for _ in range(3):
            pa, pb = rng.integers(0, 4, na), rng.integers(0, 4, nb)
            P = gpu_pkg.PauliString.dense
            want = a.exp_value(P(pa)) * b.exp_value(P(pb))
            assert close(k.exp_value(P(np.concatenate([pa, pb]))), want)
    if na + nb <= 10:
        assert np.abs(k.to_statevector() - np.kron(b.to_statevector(), a.to_statevector())).max() < 1e-9
    k.apply_h(na + nb - 1)  # the product is an ordinary state
    if na + nb <= 64:  # pair sums need n ≤ 64
        assert close(k.norm(), 1.0)


def test_state_kron_global_factors(gpu_pkg):
    ga, gb = toffoli_gates(), random_full_circuit(2, 20, 2, 87)
    a = gpu_pkg.QuantumState.from_gates(3, ga)
    b = gpu_pkg.QuantumState.from_gates(2, gb)
    a.project_normalized(0, True)  # global factor ≠ 1
    b.project_unnormalized(1, False)
    k = a.kron(b)
    assert np.abs(k.to_statevector() - np.kron(b.to_statevector(), a.to_statevector())).max() < 1e-9
    e = gpu_pkg.QuantumState.from_gates(1, []).kron(a)
    assert np.abs(e.to_statevector() - np.kron(a.to_statevector(), [1, 0])).max() < 1e-9
    with pytest.raises(gpu_pkg.NecstarError) as err:
        gpu_pkg.QuantumState.from_gates(100, []).kron(gpu_pkg.QuantumState.from_gates(29, []))
    assert err.value.code == 105


@pytest.mark.parametrize("n", [1, 5, 20, 40, 64])
def test_random_clifford_states_bit_exact(gpu_pkg, oracle, n):
    """QuantumCircuit.random_clifford followed by T gates, compiled on the device:
    terms equal the oracle's; ⟨P⟩ agrees with the oracle's exact value."""
    c = gpu_pkg.QuantumCircuit.random_clifford(n, seed=1000 + n)
    rng = np.random.default_rng(n)
    for q in rng.integers(0, n, 4):
        c.apply_t(int(q))
    c.append(gpu_pkg.QuantumCircuit.random_clifford(n, seed=2000 + n))
    st = gpu_pkg.QuantumState.from_circuit(c)
    ref = oracle.OracleState.from_circuit(n, c.gate_array())
    assert_same_terms(st.export_terms(), ref.export_terms())
    ops = rng.integers(0, 4, n)
    _, want = ref.exp_value(0, ops)
    assert close(st.exp_value(gpu_pkg.PauliString.dense(ops)), want)


def test_qasm_circuit_known_answer(gpu_pkg):
    # the Toffoli-state circuit of tests/test_state_calculation.py:37-65 read from OpenQASM: ⟨ZII⟩ = 0.5
    text = "\n".join(["OPENQASM 2.0;", 'include "qelib1.inc";', "qreg q[3];", "h q[0];", "h q[1];", "h q[2];",
                      "cx q[1], q[2];", "tdg q[2];", "cx q[0], q[2];", "t q[2];", "cx q[1], q[2];", "tdg q[2];",
                      "cx q[0], q[2];", "t q[1];", "t q[2];", "cx q[0], q[1];", "h q[2];", "t q[0];", "tdg q[1];",
                      "cx q[0], q[1];", "measure q[0] -> c[0];"])
    c = gpu_pkg.QuantumCircuit.from_qasm_str(text)
    assert np.array_equal(c.gate_array(), toffoli_gates())
    st = gpu_pkg.QuantumState.from_circuit(c)
    assert close(st.exp_value(gpu_pkg.PauliString.from_str("ZII")), 0.5)
    assert close(st.norm(), 1.0)


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8])
def test_toffoli_tensor_state_bit_exact(gpu_pkg, oracle, k):
    """|Toffoli⟩^{⊗k} (magic_states/toffoli_state.rs:12-40): every term equal to the oracle's."""
    st = gpu_pkg.QuantumState.toffoli_tensor(k)
    ref = oracle.OracleState.toffoli_tensor(k)
    assert (st.num_qubits, st.stabilizer_rank) == (3 * k, 2 ** k)
    assert_same_terms(st.export_terms(), ref.export_terms())
    if k <= 2:
        assert np.abs(st.to_statevector() - ref.to_statevector()).max() < 1e-12
    assert close(st.norm(), 1.0)


def test_toffoli_tensor_state_limits(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import NecstarError
    with pytest.raises(NecstarError) as e:
        gpu_pkg.QuantumState.toffoli_tensor(0)
    assert e.value.code == 2
    with pytest.raises(NecstarError) as e:
        gpu_pkg.QuantumState.toffoli_tensor(22)
    assert e.value.code == 105
