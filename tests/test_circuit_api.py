"""Circuit ingestion and random Clifford circuits (host side, no GPU).

* The reference's circuit tests (tests/test_circuit.py, crates/necstar/src/
  circuit/parser.rs:233-325, circuit/mod.rs doctests) against the Python
  mirror: gate names, QASM text in both directions, tensor/append, Display.
* The seeded stream: the library's and the oracle's ChaCha blocks against the
  published ChaCha known answers, and their streams against each other.
* random_clifford: the library's circuit equals the oracle's restatement of
  crates/stabilizer-ch-form-rust/src/circuit/random_clifford.rs gate for gate,
  and the circuits are uniform over the Clifford group (n = 1: all 24
  elements up to phase; n = 2: all 60 stabilizer states U|00⟩), checked with
  the oracle's dense simulator.
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def nec(gpu_pkg):
    return gpu_pkg


# ---------------------------------------------------------------- tests/test_circuit.py
def test_circuit_initialization_and_gates(nec):
    c = nec.QuantumCircuit(2)
    assert c.num_qubits == 2 and len(c.gates) == 0
    c.apply_h(0)
    c.apply_cx(0, 1)
    assert [(g.name, g.qubits) for g in c.gates] == [("H", [0]), ("CX", [0, 1])]


def test_gate_application_by_name(nec):
    c = nec.QuantumCircuit(2)
    c.apply_gate("x", [1])
    c.apply_gate("cz", [0, 1])
    c.apply_gate("CNOT", [1, 0])
    c.apply_gate("SqrtXdg", [0])
    assert [(g.name, g.qubits) for g in c.gates] == [("X", [1]), ("CZ", [0, 1]), ("CX", [1, 0]), ("SqrtXdg", [0])]
    with pytest.raises(ValueError, match="Unknown gate name: 'invalid_gate'"):
        c.apply_gate("invalid_gate", [0])
    with pytest.raises(ValueError, match="Unknown gate name: 'ccx'"):  # not reachable by name
        c.apply_gate("ccx", [0, 1, 2])
    with pytest.raises(ValueError, match=r"CX gate requires 2 qubit indices \(control, target\)\."):
        c.apply_gate("cx", [0])
    with pytest.raises(ValueError, match="H gate requires 1 qubit index."):
        c.apply_gate("h", [0, 1])


def test_random_clifford_basics(nec):
    c = nec.QuantumCircuit.random_clifford(3, seed=42)
    assert c.num_qubits == 3 and len(c.gates) > 0
    a = nec.QuantumCircuit.random_clifford(4, seed=12345678901234567890)
    b = nec.QuantumCircuit.random_clifford(4, seed=12345678901234567890)
    assert [(g.name, g.qubits) for g in a.gates] == [(g.name, g.qubits) for g in b.gates]
    assert nec.QuantumCircuit.random_clifford(4, seed=(1 << 256) - 1).num_qubits == 4
    with pytest.raises(OverflowError):
        nec.QuantumCircuit.random_clifford(4, seed=1 << 300)
    with pytest.raises(OverflowError):
        nec.QuantumCircuit.random_clifford(4, seed=-1)
    assert len({str(nec.QuantumCircuit.random_clifford(5)) for _ in range(10)}) > 1
    e = nec.QuantumCircuit.random_clifford(0, seed=1)
    assert e.num_qubits == 0 and e.num_gates == 0
    with pytest.raises(OverflowError):
        nec.QuantumCircuit.random_clifford(-1)


def test_from_qasm_str(nec):
    text = '\nOPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2];\nh q[0];\ncx q[0], q[1];\nt q[1];\n'
    c = nec.QuantumCircuit.from_qasm_str(text)
    assert c.num_qubits == 2 and [g.name for g in c.gates] == ["H", "CX", "T"]


def test_from_qasm_str_invalid(nec):
    bad_gate = '\nOPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2];\nt q[1];\nrx(pi/4) q[0];\n'
    with pytest.raises(ValueError) as e:
        nec.QuantumCircuit.from_qasm_str(bad_gate)
    assert str(e.value) == ("Failed to parse QASM string: QASM parsing error: "
                            "Unrecognized or malformed line: rx(pi/4) q[0];")
    bad_syntax = '\nOPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2]\nh q[0]\n'
    with pytest.raises(ValueError):
        nec.QuantumCircuit.from_qasm_str(bad_syntax)


def test_to_qasm_str_exact(nec):
    # parser.rs:233-250 (no trailing newline) and tests/test_circuit.py
    c = nec.QuantumCircuit(2)
    c.apply_z(0)
    c.apply_cx(0, 1)
    c.apply_t(0)
    assert c.to_qasm_str("q") == 'OPENQASM 2.0;\ninclude "qelib1.inc";\nqreg q[2];\nz q[0];\ncx q[0], q[1];\nt q[0];'


def test_qasm_roundtrip_every_gate(nec, tmp_path):
    c = nec.QuantumCircuit(5)
    for f in ("h", "x", "y", "z", "s", "sdg", "sqrt_x", "sqrt_xdg", "t", "tdg"):
        getattr(c, "apply_" + f)(3)
    c.apply_cx(0, 4)
    c.apply_cz(1, 2)
    c.apply_swap(4, 0)
    c.apply_ccx(0, 1, 2)
    d = nec.QuantumCircuit.from_qasm_str(c.to_qasm_str("reg_1"))
    assert d.num_qubits == 5 and [g.row() for g in d.gates] == [g.row() for g in c.gates]
    path = str(tmp_path / "c.qasm")
    c.to_qasm_file(path, "q")
    e = nec.QuantumCircuit.from_qasm_file(path)
    assert [g.row() for g in e.gates] == [g.row() for g in c.gates]
    assert "sx q[3];" in c.to_qasm_str("q") and "ccx q[0], q[1], q[2];" in c.to_qasm_str("q")


def test_qasm_reader_rules(nec, capfd):
    Q = nec.QuantumCircuit.from_qasm_str
    # comments, blank lines, CRLF line ends, whitespace, measure (ignored with a warning)
    c = Q('// header\r\nOPENQASM 2.0;\r\n\r\n  qreg  data [ 3 ] ;\r\n  h data[2] ;\r\nmeasure data[0] -> c[0];\r\n')
    assert c.num_qubits == 3 and [str(g) for g in c.gates] == ["H(2)"]
    assert "[Warning] Line 6: `measure` operation is ignored by the parser." in capfd.readouterr().err
    # matching is a search inside the line: only the first statement of a line is read
    c = Q("qreg q[2];\nx q[0]; h q[1];")
    assert [str(g) for g in c.gates] == ["X(0)"]

    def err(text):
        with pytest.raises(ValueError) as e:
            Q(text)
        return str(e.value).split("QASM parsing error: ", 1)[1]

    assert err("qreg q[2];\nqreg r[1];") == "Multiple qreg declarations are not supported."
    assert err("h q[0];") == "qreg declaration not found in QASM string."
    assert err("") == "qreg declaration not found in QASM string."
    assert err("qreg q[2];\ncreg c[2];") == "Unrecognized or malformed line: creg c[2];"
    assert err("qreg q[2];\ncy q[0], q[1];") == "Unrecognized or malformed line: cy q[0], q[1];"
    assert err("qreg q[3];\ncx q[0], q[1], q[2];") == "Unrecognized or malformed line: cx q[0], q[1], q[2];"
    assert err("qreg q[2];\nh q[99999999999999999999];") == (
        "Invalid qubit index in line: 'h q[99999999999999999999];' (number too large to fit in target type)")
    assert err("qreg q[٣];") == "Invalid qreg size in line: 'qreg q[٣];' (invalid digit found in string)"
    # indices are not checked against the register (the compiler checks them)
    assert Q("qreg q[1];\nh q[7];").gates[0].qubits == [7]


def test_qasm_file_errors(nec, tmp_path):
    missing = str(tmp_path / "missing.qasm")
    with pytest.raises(FileNotFoundError) as e:
        nec.QuantumCircuit.from_qasm_file(missing)
    assert str(e.value) == (f"Failed to read QASM file: QASM parsing error: Failed to read file '{missing}': "
                            "No such file or directory (os error 2)")
    assert isinstance(e.value, ValueError) and e.value.code == 19
    bad = tmp_path / "bad.qasm"
    bad.write_bytes(b"qreg q[1];\n\xff\xfe")
    with pytest.raises(FileNotFoundError, match="stream did not contain valid UTF-8"):
        nec.QuantumCircuit.from_qasm_file(str(bad))
    nog = tmp_path / "noreg.qasm"
    nog.write_text("h q[0];\n")
    with pytest.raises(FileNotFoundError, match="qreg declaration not found"):
        nec.QuantumCircuit.from_qasm_file(str(nog))
    with pytest.raises(ValueError) as e:
        nec.QuantumCircuit(1).to_qasm_file(str(tmp_path / "no_dir" / "x.qasm"), "q")
    assert str(e.value).startswith("Failed to write QASM file: IO error: No such file or directory (os error 2)")


def test_append_tensor_display(nec):
    a = nec.QuantumCircuit(2)
    a.apply_h(0)
    b = nec.QuantumCircuit(2)
    b.apply_cx(0, 1)
    b.apply_t(0)
    a.append(b)
    assert a.num_qubits == 2 and [str(g) for g in a.gates] == ["H(0)", "CX(0, 1)", "T(0)"]
    c1 = nec.QuantumCircuit(2)
    c1.apply_h(0)
    c2 = nec.QuantumCircuit(3)
    c2.apply_cx(0, 1)
    c2.apply_t(2)
    c2.apply_ccx(0, 1, 2)
    t = c1.tensor(c2)
    assert t.num_qubits == 5
    assert [str(g) for g in t.gates] == ["H(0)", "CX(2, 3)", "T(4)", "CCX(2, 3, 4)"]
    d = nec.QuantumCircuit(2)
    d.apply_h(0)
    d.apply_cx(0, 1)
    d.apply_t(1)
    assert str(d) == "QuantumCircuit(num_qubits=2) [H(0), CX(0, 1), T(1)]"
    assert str(nec.QuantumCircuit(3)) == "QuantumCircuit(num_qubits=3) []"


# ---------------------------------------------------------------- the seeded stream
SIGMA = [0x61707865, 0x3320646E, 0x79622D32, 0x6B206574]
# ChaCha20, zero key and nonce, block 0 (RFC 7539 appendix A.1, test vector #1)
KAT_ZERO_20 = ("76b8e0ada0f13d90405d6ae55386bd28bdd219b8a08ded1aa836efcc8b770dc7"
               "da41597c5157488d7724e03fb8d84a376a43b8f41518a11cc387b669b2ee6586")
# ChaCha20 block function test vector (RFC 7539 §2.3.2): key 00..1f, counter 1, nonce 00000009 0000004a 00000000
KAT_BLOCK_20 = ("10f1e7e4d13b5915500fdd1fa32071c4c7d1f4c733c068030422aa9ac3d46c4e"
                "d2826446079faa0914c2d705d98b02a2b5129cd1de164eb9cbd083e8a2503c4e")
# ChaCha with 12 rounds, zero key and IV, block 0 (eSTREAM ChaCha test vectors)
KAT_ZERO_12 = ("9bf49a6a0755f953811fce125f2683d50429c3bb49e074147e0089a52eae155f"
               "0564f879d27ae3c02ce82834acfa8c793a629f2ca0de6919610be82f411326be")


def _kat_inputs():
    key = list(struct.unpack("<8I", bytes(range(32))))
    nonce = list(struct.unpack("<3I", bytes.fromhex("000000090000004a00000000")))
    return [(SIGMA + [0] * 12, 20, KAT_ZERO_20), (SIGMA + key + [1] + nonce, 20, KAT_BLOCK_20),
            (SIGMA + [0] * 12, 12, KAT_ZERO_12)]


def _hex(words) -> str:
    return b"".join(struct.pack("<I", int(w)) for w in words).hex()


def test_chacha_known_answers(nec):
    from stab_decomp_simulator_rust_gb300 import _ffi
    from oracle import pyoracle as po
    L = _ffi.load()
    for words, rounds, want in _kat_inputs():
        inp = (C.c_uint32 * 16)(*words)
        out = (C.c_uint32 * 16)()
        assert L.nsg_debug_chacha_block(inp, rounds, out) == 0
        assert _hex(out) == want
        assert _hex(po.chacha_block(words, rounds)) == want


def test_stream_layout_and_conversions(nec):
    """The stream is block 0, 1, 2, … of 12-round ChaCha keyed by the seed
    (64-bit counter in words 12-13), and a double is the top 53 bits of two
    consecutive words (low word first) × 2^-53."""
    from stab_decomp_simulator_rust_gb300 import _ffi
    from oracle import pyoracle as po
    L = _ffi.load()
    for seed in (bytes(32), bytes(range(32)), bytes([0xA5]) * 32):
        w = (C.c_uint32 * 80)()
        assert L.nsg_random_words(seed, w, 80) == 0
        words = np.array(list(w), dtype=np.uint32)
        assert np.array_equal(words, po.random_words(seed, 80))
        key = list(struct.unpack("<8I", seed))
        for blk in range(5):
            ref = po.chacha_block(SIGMA + key + [blk, 0, 0, 0], 12)
            assert words[16 * blk:16 * blk + 16].tolist() == ref
        d = po.random_doubles(seed, 40)
        u64 = words[0::2].astype(np.uint64) | (words[1::2].astype(np.uint64) << np.uint64(32))
        assert np.array_equal(d, (u64 >> np.uint64(11)).astype(np.float64) * 2.0 ** -53)
    assert _hex(po.random_words(bytes(32), 16)) == KAT_ZERO_12


# ---------------------------------------------------------------- random_clifford
def _seeds():
    out = []
    for k in range(12):
        out.append((k * 2654435761).to_bytes(8, "little") + bytes(24) if k % 2 else bytes([k]) * 32)
    return out


@pytest.mark.parametrize("n", list(range(0, 14)) + [31, 40, 64])
def test_random_clifford_matches_oracle(nec, n):
    from oracle import pyoracle as po
    from stab_decomp_simulator_rust_gb300.state import seed_bytes
    for seed in _seeds():
        c = nec.QuantumCircuit.random_clifford(n, seed=seed)
        want = po.random_clifford(n, seed)
        got = c.gate_array()
        assert np.array_equal(got, want), (n, seed)
        assert c.num_gates <= 2 * n * n + 3 * n and all(g.is_clifford() for g in c.gates)
    # Python seeds map to the same 32 bytes (python/src/utils.rs)
    a = nec.QuantumCircuit.random_clifford(n, seed=987654321).gate_array()
    assert np.array_equal(a, po.random_clifford(n, bytes(seed_bytes(987654321))))


def _ray_key(v: np.ndarray) -> tuple:
    i = int(np.argmax(np.abs(v) > 1e-9))
    v = v * (abs(v[i]) / v[i])
    return tuple(np.round(np.concatenate([v.real, v.imag]), 6).tolist())


def _chi2_ok(counts: dict, classes: int, samples: int) -> bool:
    from scipy.stats import chi2
    exp = samples / classes
    stat = sum((c - exp) ** 2 / exp for c in counts.values()) + (classes - len(counts)) * exp
    return chi2.sf(stat, classes - 1) > 1e-5


def test_random_clifford_uniform_one_qubit(nec):
    from oracle import pyoracle as po
    counts: dict = {}
    samples = 2400
    for k in range(samples):
        g = [x.row() for x in nec.QuantumCircuit.random_clifford(1, seed=k).gates]
        a = po.dense_simulate(1, g)
        b = po.dense_simulate(1, [nec.QuantumGate.h(0).row()] + g)  # U|+⟩
        key = (_ray_key(a), _ray_key(b))
        counts[key] = counts.get(key, 0) + 1
    assert len(counts) == 24  # every single-qubit Clifford up to phase
    assert _chi2_ok(counts, 24, samples)


def test_random_clifford_uniform_two_qubit_states(nec):
    from oracle import pyoracle as po
    counts: dict = {}
    samples = 6000
    for k in range(samples):
        g = nec.QuantumCircuit.random_clifford(2, seed=10_000 + k).gate_array()
        key = _ray_key(po.dense_simulate(2, g))
        counts[key] = counts.get(key, 0) + 1
    assert len(counts) == 60  # every two-qubit stabilizer state
    assert _chi2_ok(counts, 60, samples)


def test_random_clifford_abi_arguments(nec):
    """nsg_random_clifford / nsg_random_words argument handling (no device work)."""
    from stab_decomp_simulator_rust_gb300 import _ffi
    L = _ffi.load()
    consts = _ffi.header_constants()
    nout = C.c_size_t(7)
    assert L.nsg_random_clifford(3, None, None, 0, None) == consts["NSG_ERR_INVALID_ARGUMENT"]
    assert L.nsg_random_clifford(0, None, None, 0, C.byref(nout)) == 0 and nout.value == 0
    small = (C.c_uint32 * 16)()
    assert L.nsg_random_clifford(3, bytes(32), small, 4, C.byref(nout)) == consts["NSG_ERR_BUFFER_TOO_SMALL"]
    args = (C.c_int64 * 3)()
    L.nsg_last_error_args(args)
    assert list(args)[:2] == [2 * 9 + 9, 4]
    assert L.nsg_random_words(None, small, 4) == consts["NSG_ERR_INVALID_ARGUMENT"]
    assert L.nsg_random_words(bytes(32), None, 0) == 0
    inp = (C.c_uint32 * 16)()
    for bad in (0, 3, -2, 66):
        assert L.nsg_debug_chacha_block(inp, bad, small) == consts["NSG_ERR_INVALID_ARGUMENT"]
