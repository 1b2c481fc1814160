"""The common-stabilizer zero test (nsg_zero_screen_circuit, host only).

Soundness is the whole contract: an observable the test calls zero must have
a zero term for every pair of the compiled state, which the oracle checks
pair by pair (pair_scalar) on small circuits of every gate kind.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_full_circuit

def _paulis(pkg, n, count, seed):
    rng = np.random.default_rng(seed)
    out = [pkg.PauliString.dense(np.zeros(n, np.uint8))]
    out += [pkg.PauliString.dense(rng.integers(0, 4, n).astype(np.uint8)) for _ in range(count)]
    out += [pkg.PauliString.dense(np.eye(n, dtype=np.uint8)[q] * 3) for q in range(n)]  # Z_q
    out += [pkg.PauliString.dense(np.eye(n, dtype=np.uint8)[q] * 1) for q in range(n)]  # X_q
    return out


@pytest.mark.parametrize("n,nc,nt,seed", [(3, 30, 2, 301), (4, 40, 3, 302), (5, 60, 4, 303), (6, 80, 5, 304),
                                          (8, 120, 6, 305), (7, 50, 1, 306), (6, 40, 0, 307)])
def test_screen_zero_means_every_pair_term_zero(host_pkg, oracle, n, nc, nt, seed):
    pkg = host_pkg
    gates = random_full_circuit(n, nc, nt, seed)
    ps = _paulis(pkg, n, 24, seed)
    zero = pkg.zero_screen_circuit(n, gates, ps)
    assert not zero[0]  # the identity: ⟨I⟩ is the squared norm
    ref = oracle.OracleState.from_circuit(n, gates)
    chi = ref.stabilizer_rank
    flagged = 0
    for p, z in zip(ps, zero):
        if not z:
            continue
        flagged += 1
        for i in range(chi):
            for j in range(chi):
                assert ref.pair_scalar(i, j, (0, p.ops, None))[0], (i, j, p)
        assert ref.exp_value(0, p.ops)[1] == 0.0
    if nt == 0:  # a stabilizer state: every P outside ±its stabilizer group has ⟨P⟩ = 0, all caught
        for p, z in zip(ps, zero):
            if not z:
                assert abs(ref.exp_value(0, p.ops)[1]) == pytest.approx(1.0)
    assert flagged > 0


def test_screen_on_the_batching_workload(host_pkg):
    """The test decides most of the workload's observables (16 dense random Paulis per circuit)."""
    pkg = host_pkg
    from stab_decomp_simulator_rust_gb300 import workloads as W
    cs = W.batch_circuits()[:64]
    tot = dec = 0
    for n, g, ps in cs:
        z = pkg.zero_screen_circuit(n, g, [pkg.PauliString.dense(p) for p in ps])
        tot += len(z)
        dec += int(z.sum())
    assert dec > tot // 2, (dec, tot)


def test_screen_errors(host_pkg):
    pkg = host_pkg
    from stab_decomp_simulator_rust_gb300 import NecstarError
    g = random_full_circuit(4, 20, 2, 9)
    with pytest.raises(NecstarError) as e:
        pkg.zero_screen_circuit(4, g, [pkg.PauliString.dense(np.zeros(5, np.uint8))])
    codes = pkg._ffi.header_constants()
    assert e.value.code == codes["NSG_ERR_INVALID_PAULI_STRING_LENGTH"]
    with pytest.raises(NecstarError):
        pkg.zero_screen_circuit(4, np.asarray([[13, 0, 1, 2]], np.uint32), [])  # CCX is not supported
    with pytest.raises(NecstarError) as e:
        pkg.zero_screen_circuit(70, np.zeros((0, 4), np.uint32), [])
    assert e.value.code == codes["NSG_ERR_TOO_WIDE"]


def test_screen_dense_and_sparse_agree(host_pkg):
    """A Pauli given sparse (qubits and ops) is screened like the same Pauli given dense."""
    pkg = host_pkg
    n = 12
    g = random_full_circuit(n, 150, 5, 311)
    rng = np.random.default_rng(311)
    dense, sparse = [], []
    for _ in range(40):
        ops = rng.integers(0, 4, n).astype(np.uint8)
        dense.append(pkg.PauliString.dense(ops))
        q = np.flatnonzero(ops).astype(np.uint32)
        sparse.append(pkg.PauliString.sparse(ops[q], q))
    np.testing.assert_array_equal(pkg.zero_screen_circuit(n, g, dense), pkg.zero_screen_circuit(n, g, sparse))


def test_screen_without_t_gates_is_the_stabilizer_group(host_pkg, oracle):
    """With no T gate the state is one stabilizer state: P is decided zero
    exactly when it is not ± an element of its stabilizer group."""
    pkg = host_pkg
    n = 5
    g = random_full_circuit(n, 60, 0, 312)
    ref = oracle.OracleState.from_circuit(n, g)
    every = [pkg.PauliString.dense(np.array([(k >> (2 * q)) & 3 for q in range(n)], np.uint8))
             for k in range(4 ** n)]
    z = pkg.zero_screen_circuit(n, g, every)
    for p, zz in zip(every, z):
        v = ref.exp_value(0, p.ops)[1]
        assert zz == (v == 0.0), (p, v)
