"""Host-side logic that needs no GPU: the C ABI library loads and exports every
declared symbol, Pauli/gate/circuit parsing mirrors the reference's Python
tests, seeds convert like python/src/utils.rs, and the workload generator is
deterministic."""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def test_library_exports_every_header_symbol(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import _ffi
    lib = _ffi.load()
    names = _ffi.header_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", _ffi._build.LIB], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert set(names) <= exported, set(names) - exported
    assert lib.nsg_version().decode().startswith("necstar-gb300")


def test_null_arguments_are_errors_not_crashes(gpu_pkg):
    from stab_decomp_simulator_rust_gb300 import _ffi
    lib = _ffi.load()
    consts = _ffi.header_constants()
    assert lib.nsg_num_qubits(None, None) == consts["NSG_ERR_INVALID_ARGUMENT"]
    assert lib.nsg_state_from_circuit(2, None, 3, None) == consts["NSG_ERR_INVALID_ARGUMENT"]
    args = (C.c_int64 * 3)()
    assert lib.nsg_last_error_args(args) == 0


def test_error_numbering_shared_with_oracle():
    from stab_decomp_simulator_rust_gb300 import _ffi
    c = _ffi.header_constants()
    assert c["NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS"] == 1 and c["NSG_ERR_DUPLICATE_QUBIT_INDICES"] == 14
    assert c["NSG_ERR_IMPOSSIBLE_PROJECTION"] == 9 and c["NSG_ERR_DEVICE_INVARIANT"] == 101


def test_pauli_dense():
    # tests/test_pauli_string.py:5-19
    from stab_decomp_simulator_rust_gb300 import PauliString
    p = PauliString.from_str("IXYZ")
    assert str(p) == "IXYZ" and repr(p) == "PauliString('IXYZ')" and not p.is_identity
    assert list(p.ops) == [3, 2, 1, 0]  # little-endian: qubit 0 is the rightmost character
    for bad in ("IXYZA", "IXY1", "I X Y Z", "xyz"):
        with pytest.raises(ValueError):
            PauliString.from_str(bad)


def test_pauli_sparse():
    # tests/test_pauli_string.py:22-41
    from stab_decomp_simulator_rust_gb300 import PauliString
    p = PauliString.from_str("X1 Y3 Z0")
    assert str(p) == "X1 Y3 Z0" and repr(p) == "PauliString('X1 Y3 Z0')" and not p.is_identity
    assert str(PauliString.from_str("x1 y3 z0")) == "X1 Y3 Z0"
    for bad in ("X1 Y3 A0", "X1 Y3 Z", "X1 Y3 Z-1", "X1 Y3 Z1.5", "X1 Y3 Z1"):
        with pytest.raises(ValueError):
            PauliString.from_str(bad)


def test_pauli_identity():
    # tests/test_pauli_string.py:44-52
    from stab_decomp_simulator_rust_gb300 import PauliString
    for s in ("", "I"):
        p = PauliString.from_str(s)
        assert str(p) == "I" and repr(p) == "PauliString('I')" and p.is_identity


def test_gates():
    # tests/test_gate.py:4-43
    from stab_decomp_simulator_rust_gb300 import QuantumGate as G
    x = G.x(0)
    assert x.name == "X" and x.qubits == [0] and str(x) == "X(0)" and repr(x) == "<QuantumGate: X(0)>"
    cx = G.cx(1, 2)
    assert cx.name == "CX" and cx.qubits == [1, 2] and str(cx) == "CX(1, 2)"
    cl = [G.h(0), G.x(1), G.y(2), G.z(3), G.s(4), G.sdg(5), G.sqrt_x(6), G.sqrt_xdg(7), G.cx(8, 9), G.cz(10, 11),
          G.swap(12, 13)]
    assert all(g.is_clifford() for g in cl) and not any(g.is_t_type() for g in cl)
    tt = [G.t(0), G.tdg(1)]
    assert all(g.is_t_type() for g in tt) and not any(g.is_clifford() for g in tt)


def test_circuit_builder():
    from stab_decomp_simulator_rust_gb300 import QuantumCircuit, QuantumGate
    c = QuantumCircuit(3)
    c.apply_h(0)
    c.apply_cx(0, 1)
    c.apply_t(2)
    c.apply_ccx(0, 1, 2)
    c.apply_gate(QuantumGate.sdg(1))
    assert c.num_qubits == 3 and c.num_gates == 5
    assert [str(g) for g in c.gates] == ["H(0)", "CX(0, 1)", "T(2)", "CCX(0, 1, 2)", "Sdg(1)"]
    arr = c.gate_array()
    assert arr.shape == (5, 4) and arr.dtype == np.uint32
    with pytest.raises(ValueError):
        c.apply_gate("cx", [0])


def test_seed_bytes():
    # python/src/utils.rs:4-39
    from stab_decomp_simulator_rust_gb300.state import seed_bytes
    assert seed_bytes(None) is None
    b = seed_bytes(42)
    assert b.tolist() == [42] + [0] * 31
    big = (1 << 70) + 5
    assert bytes(seed_bytes(big)) == big.to_bytes(32, "little")
    assert bytes(seed_bytes(bytes(range(32)))) == bytes(range(32))
    with pytest.raises(ValueError):
        seed_bytes(b"short")
    with pytest.raises(TypeError):
        seed_bytes(1.5)


def test_workloads_deterministic():
    from stab_decomp_simulator_rust_gb300 import workloads as W
    a = W.random_clifford_t_circuit(40, 4000, 24, 2)
    b = W.random_clifford_t_circuit(40, 4000, 24, 2)
    assert np.array_equal(a, b) and a.shape == (4024, 4)
    ops = a[:, 0]
    assert (ops == W.OP["T"]).sum() == 24
    assert set(np.unique(ops)) <= {W.OP["H"], W.OP["S"], W.OP["CX"], W.OP["T"]}
    cx = a[ops == W.OP["CX"]]
    assert np.all(cx[:, 1] != cx[:, 2]) and a[:, 1:3].max() < 40
    h = hashlib.sha256(a.tobytes()).hexdigest()
    assert h == hashlib.sha256(W.random_clifford_t_circuit(40, 4000, 24, 2).tobytes()).hexdigest()
    ps = W.random_dense_paulis(40, 64, 102)
    assert len(ps) == 64 and all(len(p) == 40 and p.max() <= 3 for p in ps)
    sp = W.random_sparse_paulis(60, 16, 1, 8, 3)
    assert all(1 <= len(o) <= 8 and len(set(q.tolist())) == len(q) and o.min() >= 1 for o, q in sp)


def test_xoshiro_reference_stream():
    # xoshiro256** seeded through SplitMix64: the first outputs for seed 0
    from stab_decomp_simulator_rust_gb300.workloads import Xoshiro256ss
    r = Xoshiro256ss(0)
    first = [r.next() for _ in range(3)]
    r2 = Xoshiro256ss(0)
    assert first == [r2.next() for _ in range(3)]
    assert len(set(first)) == 3 and all(0 <= x < 1 << 64 for x in first)
    counts = [0] * 5
    for _ in range(5000):
        counts[r.below(5)] += 1
    assert min(counts) > 850


def test_host_tensor_expansion_matches_oracle(oracle, tmp_path):
    """The product's host |T⟩^{⊗t} expansion (csrc/chform_host.hpp) is bit-exact
    with the oracle's construct_t_tensor_state restatement."""
    src = tmp_path / "tt.cpp"
    src.write_text(
        '#include "chform_host.hpp"\n#include <cstdio>\n#include <cstdlib>\nusing namespace nsg;\n'
        'int main(int c, char** v) { int t = atoi(v[1]); HostDecomp d = t_tensor_state(t);\n'
        ' printf("%zu\\n", d.terms.size());\n'
        ' for (size_t i = 0; i < d.terms.size(); i++) { const HostCH& h = d.terms[i];\n'
        '  for (int r = 0; r < t; r++) printf("%llu %llu %llu %d ", (unsigned long long)h.G[r].w[0],'
        ' (unsigned long long)h.F[r].w[0], (unsigned long long)h.M[r].w[0], h.gam[r]);\n'
        '  printf("%llu %llu %d %d %d\\n", (unsigned long long)h.v[0], (unsigned long long)h.s[0], h.phase,'
        ' d.coef[i].k, d.coef[i].r); } }\n')
    exe = tmp_path / "tt"
    csrc = os.path.join(ROOT, "stab_decomp_simulator_rust_gb300", "csrc")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", csrc, "-o", str(exe), str(src)], check=True)
    for t in (1, 2, 3, 5, 7, 9, 12, 16):
        lines = subprocess.run([str(exe), str(t)], capture_output=True, text=True, check=True).stdout.split("\n")
        ref = oracle.OracleState.t_tensor(t)
        d = ref.export_terms()
        chi = int(lines[0])
        assert chi == ref.stabilizer_rank
        w = 1 << np.arange(t, dtype=np.uint64)
        for i in range(chi):
            vals = list(map(int, lines[1 + i].split()))
            for r in range(t):
                gg, ff, mm, gm = vals[4 * r:4 * r + 4]
                assert gg == int((d["G"][i, r].astype(np.uint64) * w).sum())
                assert ff == int((d["F"][i, r].astype(np.uint64) * w).sum())
                assert mm == int((d["M"][i, r].astype(np.uint64) * w).sum())
                assert 2 * gm == int(d["gamma"][i, r])
            v, s, ph, k, rr = vals[4 * t:]
            assert v == int((d["v"][i].astype(np.uint64) * w).sum())
            assert s == int((d["s"][i].astype(np.uint64) * w).sum())
            assert (ph, k, rr) == (int(d["phase"][i]), int(d["coef_phase"][i]), int(d["coef_r"][i]))
