"""ctypes binding of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Used by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` to check and time against.  The product package never imports this module.
Gate lists are numpy ``uint32`` arrays of shape (N, 4) = (op, q0, q1, q2) with
the opcodes of ``include/necstar_gpu.h``; Pauli strings are
``(kind, ops, qubits)`` triples (kind 0 dense little-endian, 1 sparse).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class Gate(C.Structure):
    _fields_ = [("op", C.c_uint32), ("q0", C.c_uint32), ("q1", C.c_uint32), ("q2", C.c_uint32)]


class PauliABI(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("len", C.c_uint32),
                ("ops", C.POINTER(C.c_uint8)), ("qubits", C.POINTER(C.c_uint32))]


class OracleError(ValueError):
    def __init__(self, code: int, msg: str, args3):
        super().__init__(f"oracle error {code}: {msg} {list(args3)}")
        self.code = code
        self.args3 = tuple(args3)


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        u8p = C.POINTER(C.c_uint8)
        L.orc_last_error_message.restype = C.c_char_p
        L.orc_state_from_circuit.argtypes = [C.c_uint32, C.c_void_p, C.c_size_t, C.POINTER(vp)]
        L.orc_t_tensor_state.argtypes = [C.c_uint32, C.POINTER(vp)]
        L.orc_cat_state.argtypes = [C.c_uint32, C.POINTER(vp)]
        L.orc_state_from_terms.argtypes = [C.c_uint32, C.c_uint64] + [C.c_void_p] * 10 + [C.c_void_p, C.POINTER(vp)]
        L.orc_state_free.argtypes = [vp]
        L.orc_state_clone.argtypes = [vp, C.POINTER(vp)]
        L.orc_state_kron.argtypes = [vp, vp, C.POINTER(vp)]
        L.orc_num_qubits.argtypes = [vp, C.POINTER(C.c_uint32)]
        L.orc_stabilizer_rank.argtypes = [vp, C.POINTER(C.c_uint64)]
        L.orc_export_terms.argtypes = [vp] + [C.c_void_p] * 11
        L.orc_apply_gates.argtypes = [vp, C.c_void_p, C.c_size_t]
        L.orc_exp_value.argtypes = [vp, C.POINTER(PauliABI), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_norm.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_inner_product.argtypes = [vp, vp, C.c_void_p, C.c_void_p]
        L.orc_pair_scalar.argtypes = [vp, C.c_uint64, C.c_uint64, C.POINTER(PauliABI),
                                      C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int64)]
        L.orc_project_unnormalized.argtypes = [vp, C.c_uint32, C.c_int32]
        L.orc_project_normalized.argtypes = [vp, C.c_uint32, C.c_int32]
        L.orc_discard.argtypes = [vp, C.c_uint32]
        L.orc_measure.argtypes = [vp, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]
        L.orc_random_clifford.argtypes = [C.c_uint32, C.c_void_p, C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]
        L.orc_random_words.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.orc_random_doubles.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t]
        L.orc_chacha_block.argtypes = [C.c_void_p, C.c_int32, C.c_void_p]
        L.orc_marginal.argtypes = [vp, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p, C.c_size_t,
                                   C.POINTER(C.c_size_t)]
        L.orc_to_statevector.argtypes = [vp, C.c_void_p, C.c_size_t]
        L.orc_dense_simulate.argtypes = [C.c_uint32, C.c_void_p, C.c_size_t, C.c_void_p]
        L.orc_chform_run.argtypes = [C.c_uint32, C.c_void_p, C.c_size_t] + [C.c_void_p] * 8
        L.orc_time_pairs.argtypes = [vp, C.POINTER(PauliABI), C.c_uint64, C.c_uint64, C.c_int32,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.orc_t_tensor_terms.argtypes = [C.c_uint32, C.c_void_p, C.c_size_t, C.POINTER(vp)]
        L.orc_t_tensor_rank.argtypes = [C.c_uint32, C.POINTER(C.c_uint64)]
        L.orc_toffoli_tensor_state.argtypes = [C.c_uint32, C.POINTER(vp)]
        L.orc_compile_terms.argtypes = [C.c_uint32, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_int32,
                                        C.c_void_p, C.POINTER(vp)]
        L.orc_exp_value_counts.argtypes = [vp, C.POINTER(PauliABI), C.c_size_t, C.c_int32, C.c_int64, C.c_int64,
                                           C.c_void_p, C.c_void_p]
        L.orc_counts_value.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _check(rc: int):
    if rc != 0:
        L = lib()
        args = (C.c_int64 * 3)()
        L.orc_last_error_args(args)
        raise OracleError(rc, (L.orc_last_error_message() or b"").decode(), list(args))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def gates_array(gates) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(gates, dtype=np.uint32).reshape(-1, 4))
    return a


def pauli_abi(kind: int, ops, qubits=None):
    """Returns (struct, keepalive)."""
    o = np.ascontiguousarray(np.asarray(ops, dtype=np.uint8))
    q = np.ascontiguousarray(np.asarray(qubits if qubits is not None else [], dtype=np.uint32))
    st = PauliABI(kind, len(o), o.ctypes.data_as(C.POINTER(C.c_uint8)),
                  q.ctypes.data_as(C.POINTER(C.c_uint32)) if len(q) else None)
    return st, (o, q)


class OracleState:
    """A stabilizer-decomposed state held by the oracle."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle) if not isinstance(handle, C.c_void_p) else handle

    def __del__(self):
        try:
            if self._h:
                lib().orc_state_free(self._h)
        except Exception:
            pass

    # ---- construction
    @staticmethod
    def from_circuit(n: int, gates) -> "OracleState":
        g = gates_array(gates)
        h = C.c_void_p()
        _check(lib().orc_state_from_circuit(n, _ptr(g), len(g), C.byref(h)))
        return OracleState(h)

    @staticmethod
    def t_tensor(t: int) -> "OracleState":
        h = C.c_void_p()
        _check(lib().orc_t_tensor_state(t, C.byref(h)))
        return OracleState(h)

    @staticmethod
    def toffoli_tensor(k: int) -> "OracleState":
        """construct_toffoli_tensor_state (magic_states/toffoli_state.rs:12-40)."""
        h = C.c_void_p()
        _check(lib().orc_toffoli_tensor_state(k, C.byref(h)))
        return OracleState(h)

    @staticmethod
    def cat(t: int) -> "OracleState":
        h = C.c_void_p()
        _check(lib().orc_cat_state(t, C.byref(h)))
        return OracleState(h)

    @staticmethod
    def t_tensor_terms(t: int, tidx) -> "OracleState":
        """Terms tidx of |T⟩^{⊗t}, each built on its own (the cat recursion for one term)."""
        ti = np.ascontiguousarray(tidx, dtype=np.int64)
        h = C.c_void_p()
        _check(lib().orc_t_tensor_terms(t, _ptr(ti), len(ti), C.byref(h)))
        return OracleState(h)

    @staticmethod
    def compile_terms(n: int, gates, tidx, threads: int = 0):
        """The compile loop over the T-tensor terms `tidx` only (compiler/mod.rs:92-131).

        Returns (state of the kept terms in tidx order, kept flags)."""
        g = gates_array(gates)
        ti = np.ascontiguousarray(tidx, dtype=np.int64)
        kept = np.zeros(len(ti), np.uint8)
        h = C.c_void_p()
        _check(lib().orc_compile_terms(n, _ptr(g), len(g), _ptr(ti), len(ti), threads or (os.cpu_count() or 1),
                                       _ptr(kept), C.byref(h)))
        return OracleState(h), kept.astype(bool)

    @staticmethod
    def from_terms(d: dict) -> "OracleState":
        n = int(d["n"])
        chi = int(len(d["phase"]))
        arrs = [np.ascontiguousarray(d[k], dtype=np.uint8) for k in ("G", "F", "M", "gamma", "v", "s", "phase", "coef_phase")]
        r = np.ascontiguousarray(d["coef_r"], dtype=np.int32)
        z = np.ascontiguousarray(d["coef_zero"], dtype=np.uint8)
        gf = np.ascontiguousarray(d.get("global_factor", [1.0, 0.0]), dtype=np.float64)
        h = C.c_void_p()
        _check(lib().orc_state_from_terms(n, chi, *[_ptr(a) for a in arrs], _ptr(r), _ptr(z), _ptr(gf), C.byref(h)))
        return OracleState(h)

    def kron(self, other: "OracleState") -> "OracleState":
        """StabilizerDecomposedState::kron (stabilizer_decomposed_state/kron.rs:7-22)."""
        h = C.c_void_p()
        _check(lib().orc_state_kron(self._h, other._h, C.byref(h)))
        return OracleState(h)

    def clone(self) -> "OracleState":
        h = C.c_void_p()
        _check(lib().orc_state_clone(self._h, C.byref(h)))
        return OracleState(h)

    # ---- queries
    @property
    def num_qubits(self) -> int:
        v = C.c_uint32()
        lib().orc_num_qubits(self._h, C.byref(v))
        return v.value

    @property
    def stabilizer_rank(self) -> int:
        v = C.c_uint64()
        lib().orc_stabilizer_rank(self._h, C.byref(v))
        return v.value

    def export_terms(self) -> dict:
        n, chi = self.num_qubits, self.stabilizer_rank
        d = {
            "n": n,
            "G": np.zeros((chi, n, n), np.uint8), "F": np.zeros((chi, n, n), np.uint8),
            "M": np.zeros((chi, n, n), np.uint8), "gamma": np.zeros((chi, n), np.uint8),
            "v": np.zeros((chi, n), np.uint8), "s": np.zeros((chi, n), np.uint8),
            "phase": np.zeros(chi, np.uint8), "coef_phase": np.zeros(chi, np.uint8),
            "coef_r": np.zeros(chi, np.int32), "coef_zero": np.zeros(chi, np.uint8),
            "global_factor": np.zeros(2, np.float64),
        }
        keys = ("G", "F", "M", "gamma", "v", "s", "phase", "coef_phase", "coef_r", "coef_zero", "global_factor")
        _check(lib().orc_export_terms(self._h, *[_ptr(d[k]) for k in keys]))
        return d

    # ---- pair sums
    def exp_value(self, kind: int, ops, qubits=None):
        """Returns (reference-order FP64 value, exact value)."""
        st, keep = pauli_abi(kind, ops, qubits)
        out, ex = C.c_double(), C.c_double()
        _check(lib().orc_exp_value(self._h, C.byref(st), C.byref(out), C.byref(ex)))
        return out.value, ex.value

    def exp_value_counts(self, paulis, m_off: int, bins: int, threads: int = 0):
        """Exact accumulator of exp_value for several Paulis ((kind, ops, qubits) triples):
        signed counts of pair-term real parts per power of √2 (shape (nobs, bins), index
        m + m_off for sign·2^(-m/2)) and each exact value."""
        abis, keep = [], []
        for p in paulis:
            st, k = pauli_abi(*p)
            abis.append(st)
            keep.append(k)
        arr = (PauliABI * max(1, len(abis)))(*abis)
        counts = np.zeros((len(abis), bins), np.int64)
        exact = np.zeros(len(abis), np.float64)
        _check(lib().orc_exp_value_counts(self._h, arr, len(abis), threads or (os.cpu_count() or 1), m_off, bins,
                                          _ptr(counts), _ptr(exact)))
        return counts, exact

    def norm(self):
        out, ex = C.c_double(), C.c_double()
        _check(lib().orc_norm(self._h, C.byref(out), C.byref(ex)))
        return out.value, ex.value

    def inner_product(self, other: "OracleState"):
        out = np.zeros(2)
        ex = np.zeros(2)
        _check(lib().orc_inner_product(self._h, other._h, _ptr(out), _ptr(ex)))
        return complex(out[0], out[1]), complex(ex[0], ex[1])

    def pair_scalar(self, i: int, j: int, pauli=None):
        """⟨S_i| P |S_j⟩ as (zero, k, r)."""
        z, k, r = C.c_int32(), C.c_int32(), C.c_int64()
        if pauli is None:
            _check(lib().orc_pair_scalar(self._h, i, j, None, C.byref(z), C.byref(k), C.byref(r)))
        else:
            st, keep = pauli_abi(*pauli)
            _check(lib().orc_pair_scalar(self._h, i, j, C.byref(st), C.byref(z), C.byref(k), C.byref(r)))
        return bool(z.value), k.value, r.value

    # ---- projection etc.
    def apply_gates(self, gates):
        g = gates_array(gates)
        _check(lib().orc_apply_gates(self._h, _ptr(g), len(g)))

    def project_unnormalized(self, q: int, outcome: bool):
        _check(lib().orc_project_unnormalized(self._h, q, int(bool(outcome))))

    def project_normalized(self, q: int, outcome: bool):
        _check(lib().orc_project_normalized(self._h, q, int(bool(outcome))))

    def discard(self, q: int):
        _check(lib().orc_discard(self._h, q))

    def measure(self, qargs, seed: bytes | None = None):
        q = np.ascontiguousarray(qargs, dtype=np.uint32)
        out = np.zeros(len(q), np.uint8)
        sd = np.frombuffer(seed, dtype=np.uint8).copy() if seed is not None else None
        _check(lib().orc_measure(self._h, _ptr(q), len(q), _ptr(sd) if sd is not None else None, _ptr(out)))
        return [bool(x) for x in out]

    def marginal(self, qargs) -> dict:
        q = np.ascontiguousarray(qargs, dtype=np.uint32)
        cap = 1 << min(len(q), 20)
        outc = np.zeros(cap, np.uint64)
        probs = np.zeros(cap, np.float64)
        nout = C.c_size_t()
        _check(lib().orc_marginal(self._h, _ptr(q), len(q), _ptr(outc), _ptr(probs), cap, C.byref(nout)))
        return {int(outc[i]): float(probs[i]) for i in range(min(nout.value, cap))}

    def to_statevector(self) -> np.ndarray:
        n = self.num_qubits
        out = np.zeros(2 << n, np.float64)
        _check(lib().orc_to_statevector(self._h, _ptr(out), 1 << n))
        return out[0::2] + 1j * out[1::2]

    def time_pairs(self, kind, ops, qubits, num_pairs: int, seed: int, threads: int):
        st, keep = pauli_abi(kind, ops, qubits)
        sec, cs = C.c_double(), C.c_double()
        _check(lib().orc_time_pairs(self._h, C.byref(st), num_pairs, seed, threads, C.byref(sec), C.byref(cs)))
        return sec.value, cs.value


def t_tensor_rank(t: int) -> int:
    v = C.c_uint64()
    _check(lib().orc_t_tensor_rank(t, C.byref(v)))
    return v.value


def counts_value(counts, m_off: int) -> float:
    """Σ_m counts[m + m_off]·2^(-m/2), evaluated exactly by the oracle."""
    c = np.ascontiguousarray(counts, dtype=np.int64)
    v = C.c_double()
    _check(lib().orc_counts_value(_ptr(c), m_off, len(c), C.byref(v)))
    return v.value


def random_clifford(n: int, seed: bytes | None) -> np.ndarray:
    """CliffordCircuit::random_clifford (random_clifford.rs:177-212) as gate rows (op, q0, q1, q2)."""
    cap = 2 * n * n + 3 * n + 1
    out = np.zeros((cap, 4), np.uint32)
    sd = np.frombuffer(seed, dtype=np.uint8).copy() if seed is not None else None
    nout = C.c_size_t()
    _check(lib().orc_random_clifford(n, _ptr(sd) if sd is not None else None, _ptr(out), cap, C.byref(nout)))
    return out[:nout.value].copy()


def random_words(seed: bytes, count: int) -> np.ndarray:
    """The first `count` 32-bit words of StdRng::from_seed(seed)."""
    sd = np.frombuffer(seed, dtype=np.uint8).copy()
    out = np.zeros(count, np.uint32)
    _check(lib().orc_random_words(_ptr(sd), _ptr(out), count))
    return out


def random_doubles(seed: bytes, count: int) -> np.ndarray:
    """The first `count` rng.gen::<f64>() draws of StdRng::from_seed(seed)."""
    sd = np.frombuffer(seed, dtype=np.uint8).copy()
    out = np.zeros(count, np.float64)
    _check(lib().orc_random_doubles(_ptr(sd), _ptr(out), count))
    return out


def chacha_block(words, rounds: int) -> list[int]:
    w = np.ascontiguousarray(words, dtype=np.uint32)
    out = np.zeros(16, np.uint32)
    _check(lib().orc_chacha_block(_ptr(w), rounds, _ptr(out)))
    return [int(x) for x in out]


def dense_simulate(n: int, gates) -> np.ndarray:
    g = gates_array(gates)
    out = np.zeros(2 << n, np.float64)
    _check(lib().orc_dense_simulate(n, _ptr(g), len(g), _ptr(out)))
    return out[0::2] + 1j * out[1::2]


def chform_run(n: int, gates, want_sv: bool = True) -> dict:
    g = gates_array(gates)
    d = {"G": np.zeros((n, n), np.uint8), "F": np.zeros((n, n), np.uint8), "M": np.zeros((n, n), np.uint8),
         "gamma": np.zeros(n, np.uint8), "v": np.zeros(n, np.uint8), "s": np.zeros(n, np.uint8),
         "phase": np.zeros(1, np.uint8)}
    sv = np.zeros(2 << n, np.float64) if want_sv else None
    _check(lib().orc_chform_run(n, _ptr(g), len(g), *[_ptr(d[k]) for k in ("G", "F", "M", "gamma", "v", "s", "phase")],
                                _ptr(sv) if sv is not None else None))
    if sv is not None:
        d["sv"] = sv[0::2] + 1j * sv[1::2]
    return d
