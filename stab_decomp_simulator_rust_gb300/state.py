"""QuantumState — the compiled stabilizer decomposition, resident on the GPU.

Method names, arguments and errors mirror the reference's Python class
(python/necstar/state.pyi:9-379 over python/src/state.rs:13-222): every
failure raises ValueError (here NecstarError, a ValueError subclass carrying
the status code).  All work runs in libnecstar_gpu.so; the batched form
``exp_values`` evaluates many observables in one pass over the χ² pairs.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _ffi
from ._ffi import check
from .circuit import QuantumCircuit, QuantumGate, gate_rows
from .pauli import PauliString

PRECISION_FP64 = 0
PRECISION_MIXED = 1
EXACT_BINS = 512
EXACT_M_OFFSET = 192


def counts_to_xy(counts, m_offset: int = EXACT_M_OFFSET):
    """The exact sum Σ_m counts[m + m_offset]·2^(-m/2) as X + Y/√2 with X, Y
    dyadic rationals (even and odd m), returned as (X, Y) Fractions."""
    from fractions import Fraction
    X = Fraction(0)
    Y = Fraction(0)
    c = np.asarray(counts, dtype=np.int64)
    for b in np.flatnonzero(c).tolist():
        m = b - m_offset
        e = m // 2 if m % 2 == 0 else (m - 1) // 2
        v = Fraction(int(c[b])) / Fraction(2) ** e if e >= 0 else Fraction(int(c[b]) * 2 ** (-e))
        if m % 2 == 0:
            X += v
        else:
            Y += v
    return X, Y


def xy_to_float(X, Y, scale=1.0) -> float:
    """scale·(X + Y/√2) rounded once: √2 is taken to 400 bits, far below the
    last bit of a double."""
    import math
    from fractions import Fraction
    if X == 0 and Y == 0:
        return 0.0
    P = 400
    s2 = math.isqrt(2 << (2 * P))  # floor(√2·2^P)
    return float((X * s2 + Y * (1 << P)) / s2 * Fraction(scale))


def counts_to_value(counts, m_offset: int = EXACT_M_OFFSET, scale: float = 1.0) -> float:
    """scale·Σ_m counts[m + m_offset]·2^(-m/2), rounded once from its exact value."""
    X, Y = counts_to_xy(counts, m_offset)
    return xy_to_float(X, Y, scale)


def seed_bytes(seed) -> np.ndarray | None:
    """Python seed → 32 bytes (python/src/utils.rs:4-39)."""
    if seed is None:
        return None
    if isinstance(seed, (bytes, bytearray)):
        if len(seed) != 32:
            raise ValueError(f"Seed must be 32 bytes, got {len(seed)}")
        return np.frombuffer(bytes(seed), dtype=np.uint8).copy()
    if isinstance(seed, int):
        if 0 <= seed < (1 << 64):
            b = seed.to_bytes(8, "little") + bytes(24)
        else:
            b = seed.to_bytes(32, "little")
        return np.frombuffer(b, dtype=np.uint8).copy()
    raise TypeError("Seed must be an integer or 32 bytes")


def _p(a: np.ndarray | None):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _pauli_array(paulis):
    """The ABI array of a list of PauliString (and the list, which keeps their buffers alive)."""
    paulis = list(paulis)
    arr = (_ffi.PauliABI * max(len(paulis), 1))()
    for i, p in enumerate(paulis):
        arr[i] = p.abi()
    return arr, paulis


def zero_screen_circuit(num_qubits: int, gates, paulis) -> np.ndarray:
    """The common-stabilizer zero test for a circuit, without compiling it
    (nsg_zero_screen_circuit; host work only): True where ⟨P⟩ = 0 exactly on the
    circuit's compiled state, False where the test does not decide."""
    rows = gate_rows(gates)
    arr, keep = _pauli_array(paulis)
    out = np.zeros(len(keep), np.uint8)
    check(_ffi.load().nsg_zero_screen_circuit(num_qubits, _p(rows), len(rows), arr, len(keep), _p(out)))
    return out.astype(bool)


class QuantumState:
    def __init__(self, handle: C.c_void_p):
        self._h = handle

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _ffi.load().nsg_state_free(h)
            except Exception:
                pass
            self._h = None

    # ---- construction
    @staticmethod
    def from_circuit(circuit: QuantumCircuit) -> "QuantumState":
        return QuantumState.from_gates(circuit.num_qubits, circuit.gate_array())

    @staticmethod
    def from_gates(num_qubits: int, gates) -> "QuantumState":
        L = _ffi.load()
        rows = gate_rows(gates)
        h = C.c_void_p()
        check(L.nsg_state_from_circuit(num_qubits, _p(rows), len(rows), C.byref(h)))
        return QuantumState(h)

    @staticmethod
    def from_gates_many(circuits) -> list["QuantumState"]:
        """Compiles many circuits in one call (nsg_states_from_circuits): ``circuits``
        is a list of (num_qubits, gates); every compile is queued before any wait."""
        L = _ffi.load()
        rows = [gate_rows(g) for _, g in circuits]
        k = len(rows)
        nq = np.asarray([int(n) for n, _ in circuits], dtype=np.uint32)
        ng = np.asarray([len(r) for r in rows], dtype=np.uint64)
        gp = (C.c_void_p * max(k, 1))(*[r.ctypes.data for r in rows])
        hs = (C.c_void_p * max(k, 1))()
        check(L.nsg_states_from_circuits(k, _p(nq), gp, _p(ng), hs))
        return [QuantumState(C.c_void_p(hs[i])) for i in range(k)]

    @staticmethod
    def toffoli_tensor(num_tensors: int) -> "QuantumState":
        """|Toffoli⟩^{⊗k} on 3k qubits, 2^k terms (construct_toffoli_tensor_state,
        crates/necstar/src/state/magic_states/toffoli_state.rs:12-40)."""
        h = C.c_void_p()
        check(_ffi.load().nsg_toffoli_tensor_state(num_tensors, C.byref(h)))
        return QuantumState(h)

    @staticmethod
    def debug_t_tensor(t: int) -> "QuantumState":
        """The device expansion of |T⟩^{⊗t} as a state (terms in the reference's order)."""
        h = C.c_void_p()
        check(_ffi.load().nsg_debug_t_tensor(t, C.byref(h)))
        return QuantumState(h)

    @staticmethod
    def from_terms(d: dict) -> "QuantumState":
        """Build from a term dump (the layout of ``export_terms``)."""
        L = _ffi.load()
        n = int(d["n"])
        chi = int(len(d["phase"]))
        u8 = lambda k: np.ascontiguousarray(d[k], dtype=np.uint8)
        arrs = [u8(k) for k in ("G", "F", "M", "gamma", "v", "s", "phase", "coef_phase")]
        r = np.ascontiguousarray(d["coef_r"], dtype=np.int32)
        z = np.ascontiguousarray(d.get("coef_zero", np.zeros(chi)), dtype=np.uint8)
        gf = np.ascontiguousarray(d.get("global_factor", [1.0, 0.0]), dtype=np.float64)
        h = C.c_void_p()
        check(L.nsg_state_from_terms(n, chi, *[_p(a) for a in arrs], _p(r), _p(z), _p(gf), C.byref(h)))
        return QuantumState(h)

    def clone(self) -> "QuantumState":
        h = C.c_void_p()
        check(_ffi.load().nsg_state_clone(self._h, C.byref(h)))
        return QuantumState(h)

    def kron(self, other: "QuantumState") -> "QuantumState":
        """|self⟩ ⊗ |other⟩ (other's qubits after self's), computed on the device term by term
        (StabilizerDecomposedState::kron, stabilizer_decomposed_state/kron.rs:7-22)."""
        h = C.c_void_p()
        check(_ffi.load().nsg_state_kron(self._h, other._h, C.byref(h)))
        return QuantumState(h)

    def set_stream(self, cuda_stream: int | None) -> None:
        """Run this state's work on a caller-owned cudaStream_t (an integer handle)."""
        check(_ffi.load().nsg_state_set_stream(self._h, C.c_void_p(cuda_stream or 0)))

    # ---- properties
    @property
    def num_qubits(self) -> int:
        v = C.c_uint32()
        check(_ffi.load().nsg_num_qubits(self._h, C.byref(v)))
        return v.value

    @property
    def stabilizer_rank(self) -> int:
        v = C.c_uint64()
        check(_ffi.load().nsg_stabilizer_rank(self._h, C.byref(v)))
        return v.value

    def __str__(self) -> str:
        return f"QuantumState(num_qubits={self.num_qubits}, stabilizer_rank={self.stabilizer_rank})"

    # ---- pair sums
    def exp_value(self, pauli_string: PauliString) -> float:
        out = C.c_double()
        a = pauli_string.abi()
        check(_ffi.load().nsg_exp_value(self._h, C.byref(a), C.byref(out)))
        return out.value

    def exp_values(self, paulis, precision: int = PRECISION_FP64, screen: bool = False) -> np.ndarray:
        """Batched expectation values: one pass over the pairs for all observables.
        screen=True (opt-in): when the common-stabilizer test (zero_screen)
        decides every observable, return the exact zeros without the pair pass."""
        paulis = list(paulis)
        if screen and paulis and self.zero_screen(paulis).all():
            return np.zeros(len(paulis), np.float64)
        arr = (_ffi.PauliABI * max(len(paulis), 1))()
        for i, p in enumerate(paulis):
            arr[i] = p.abi()
        out = np.zeros(len(paulis), np.float64)
        check(_ffi.load().nsg_exp_value_batch(self._h, arr, len(paulis), precision, _p(out)))
        return out

    def exp_value_counts(self, paulis):
        """The exact accumulator of ⟨P⟩ for each observable: (counts of shape
        (nobs, EXACT_BINS) — signed numbers of pair terms with real part
        2^(-m/2) at index m + EXACT_M_OFFSET — and the scale |g|²)."""
        paulis = list(paulis)
        arr = (_ffi.PauliABI * max(len(paulis), 1))()
        for i, p in enumerate(paulis):
            arr[i] = p.abi()
        counts = np.zeros((len(paulis), EXACT_BINS), np.int64)
        scale = C.c_double()
        check(_ffi.load().nsg_exp_value_counts(self._h, arr, len(paulis), _p(counts), C.byref(scale)))
        return counts, scale.value

    def zero_screen(self, paulis) -> np.ndarray:
        """Observables with ⟨P⟩ = 0 exactly by the common-stabilizer test
        (nsg_zero_screen): True = provably zero, False = not decided.  No pair
        work; exp_value does not use it."""
        arr, keep = _pauli_array(paulis)
        out = np.zeros(len(keep), np.uint8)
        check(_ffi.load().nsg_zero_screen(self._h, arr, len(keep), _p(out)))
        return out.astype(bool)

    def exp_values_exact(self, paulis) -> np.ndarray:
        """⟨P⟩ rounded once from the exact sum of every pair term."""
        counts, scale = self.exp_value_counts(paulis)
        return np.asarray([counts_to_value(c, EXACT_M_OFFSET, scale) for c in counts], np.float64)

    def select(self, indices) -> "QuantumState":
        """A new state of the terms `indices` (strictly ascending), same global factor."""
        idx = np.ascontiguousarray(list(indices), dtype=np.uint64)
        h = C.c_void_p()
        check(_ffi.load().nsg_state_select(self._h, _p(idx), len(idx), C.byref(h)))
        return QuantumState(h)

    def inner_product(self, other: "QuantumState") -> complex:
        out = np.zeros(2, np.float64)
        check(_ffi.load().nsg_inner_product(self._h, other._h, _p(out)))
        return complex(out[0], out[1])

    def norm(self) -> float:
        out = C.c_double()
        check(_ffi.load().nsg_norm(self._h, C.byref(out)))
        return out.value

    # ---- projection / measurement
    def project_normalized(self, qubit: int, outcome: bool) -> None:
        check(_ffi.load().nsg_project_normalized(self._h, qubit, int(bool(outcome))))

    def project_unnormalized(self, qubit: int, outcome: bool) -> None:
        check(_ffi.load().nsg_project_unnormalized(self._h, qubit, int(bool(outcome))))

    def discard(self, qubit: int) -> None:
        check(_ffi.load().nsg_discard(self._h, qubit))

    def measure(self, qargs, seed=None) -> list[bool]:
        q = np.ascontiguousarray(list(qargs), dtype=np.uint32)
        out = np.zeros(max(len(q), 1), np.uint8)
        check(_ffi.load().nsg_measure(self._h, _p(q), len(q), _p(seed_bytes(seed)), _p(out)))
        return [bool(x) for x in out[:len(q)]]

    def measure_all(self, seed=None) -> list[bool]:
        n = self.num_qubits
        out = np.zeros(max(n, 1), np.uint8)
        check(_ffi.load().nsg_measure_all(self._h, _p(seed_bytes(seed)), _p(out)))
        return [bool(x) for x in out[:n]]

    def sample_raw(self, qargs, shots: int, seed=None):
        """Returns (outcomes as Python ints with bit i ↔ qargs[i], counts)."""
        L = _ffi.load()
        q = np.ascontiguousarray(list(qargs), dtype=np.uint32)
        cap = int(min(max(shots, 1), 1 << 20))
        while True:
            outc = np.zeros(2 * cap, np.uint64)
            cnts = np.zeros(cap, np.uint64)
            nout = C.c_size_t()
            rc = L.nsg_sample(self._h, _p(q), len(q), shots, _p(seed_bytes(seed)), _p(outc), _p(cnts), cap,
                              C.byref(nout))
            if rc == 104 and nout.value > cap:  # NSG_ERR_BUFFER_TOO_SMALL
                cap = nout.value
                continue
            check(rc)
            k = nout.value
            vals = [int(outc[2 * i]) | (int(outc[2 * i + 1]) << 64) for i in range(k)]
            return vals, [int(c) for c in cnts[:k]]

    def sample(self, qargs, shots: int, seed=None) -> dict[str, int]:
        """Counts keyed by outcome strings: character i is qargs[i] (python/src/state.rs:64-90)."""
        qargs = list(qargs)
        vals, cnts = self.sample_raw(qargs, shots, seed)
        k = len(qargs)
        return {"".join("1" if (v >> i) & 1 else "0" for i in range(k)): c for v, c in zip(vals, cnts)}

    # ---- gates
    def apply_gate(self, gate: QuantumGate) -> None:
        self.apply_gates([gate])

    def apply_gates(self, gates) -> None:
        rows = gate_rows(gates)
        check(_ffi.load().nsg_apply_gates(self._h, _p(rows), len(rows)))

    def apply_x(self, q): self.apply_gate(QuantumGate.x(q))
    def apply_y(self, q): self.apply_gate(QuantumGate.y(q))
    def apply_z(self, q): self.apply_gate(QuantumGate.z(q))
    def apply_h(self, q): self.apply_gate(QuantumGate.h(q))
    def apply_s(self, q): self.apply_gate(QuantumGate.s(q))
    def apply_sdg(self, q): self.apply_gate(QuantumGate.sdg(q))
    def apply_sqrt_x(self, q): self.apply_gate(QuantumGate.sqrt_x(q))
    def apply_sqrt_xdg(self, q): self.apply_gate(QuantumGate.sqrt_xdg(q))
    def apply_cx(self, c, t): self.apply_gate(QuantumGate.cx(c, t))
    def apply_cz(self, a, b): self.apply_gate(QuantumGate.cz(a, b))
    def apply_swap(self, a, b): self.apply_gate(QuantumGate.swap(a, b))

    def debug_pair_values(self, pauli: PauliString | None = None):
        """Exact ⟨S_i|P|S_j⟩ for all pairs: (k, r) arrays of shape (χ, χ); k = 255 means 0."""
        chi = self.stabilizer_rank
        k = np.zeros((chi, chi), np.uint8)
        r = np.zeros((chi, chi), np.int32)
        if pauli is None:
            check(_ffi.load().nsg_debug_pair_values(self._h, None, _p(k), _p(r)))
        else:
            a = pauli.abi()
            check(_ffi.load().nsg_debug_pair_values(self._h, C.byref(a), _p(k), _p(r)))
        return k, r

    # ---- dense views (tests)
    def to_statevector(self) -> np.ndarray:
        n = self.num_qubits
        out = np.zeros(2 << n if n < 28 else 2, np.float64)
        check(_ffi.load().nsg_to_statevector(self._h, _p(out), 1 << n if n < 28 else 1))
        return out[0::2] + 1j * out[1::2]

    def export_terms(self) -> dict:
        """Every term as bool bytes (the parity-dump / checkpoint format)."""
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
        check(_ffi.load().nsg_export_terms(self._h, *[_p(d[k]) for k in keys]))
        return d


def compile_keep(num_qubits: int, gates) -> np.ndarray:
    """Per term of the T-tensor expansion, whether compilation keeps it (the
    compiled state's term i is the i-th kept term)."""
    L = _ffi.load()
    rows = gate_rows(gates)
    nt = C.c_uint64()
    rc = L.nsg_debug_compile_keep(num_qubits, _p(rows), len(rows), None, 0, C.byref(nt))
    if rc not in (0, 104):
        check(rc)
    keep = np.zeros(max(nt.value, 1), np.uint8)
    check(L.nsg_debug_compile_keep(num_qubits, _p(rows), len(rows), _p(keep), len(keep), C.byref(nt)))
    return keep[:nt.value].astype(bool)


def set_pair_tiling(chunk: int = 0, tasks_per_warp: int = 0) -> None:
    """Tiling of direct pair sums in this process (0 = default)."""
    check(_ffi.load().nsg_set_pair_tiling(chunk, tasks_per_warp))


def _multi_args(states, paulis_per_state):
    states = list(states)
    groups = [list(g) for g in paulis_per_state]
    if len(groups) != len(states):
        raise ValueError(f"got {len(states)} states but {len(groups)} observable lists")
    offs = np.zeros(len(states) + 1, np.uint64)
    for c, g in enumerate(groups):
        offs[c + 1] = offs[c] + len(g)
    total = int(offs[-1])
    arr = (_ffi.PauliABI * max(total, 1))()
    k = 0
    for g in groups:
        for p in g:
            arr[k] = p.abi()
            k += 1
    hs = (C.c_void_p * max(len(states), 1))(*[s._h for s in states])
    return states, groups, offs, total, arr, hs


class BatchPlan:
    """A captured batched evaluation (nsg_plan_*): the work of
    ``exp_values_multi`` recorded once in a CUDA graph and replayed by
    ``run()``.  Each run reads the states' current terms, so gates applied in
    place are seen; projection, discard, measurement or freeing a state makes
    ``run()`` raise.  Creation picks the pair-kernel variant by timing it on a
    sample of the plan's work (or takes it from the tuning cache)."""

    def __init__(self, states, paulis_per_state, precision: int = PRECISION_FP64):
        states, groups, offs, total, arr, hs = _multi_args(states, paulis_per_state)
        self._states = states  # keep the handles alive as long as the plan
        self._groups = groups  # and the Pauli storage the ABI structs point into
        self._offs = offs
        self._out = np.zeros(max(total, 1), np.float64)
        h = C.c_void_p()
        check(_ffi.load().nsg_plan_create(hs, len(states), arr, _p(offs), precision, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                _ffi.load().nsg_plan_free(h)
            except Exception:
                pass
            self._h = None

    def run(self) -> list[np.ndarray]:
        check(_ffi.load().nsg_plan_run(self._h, _p(self._out)))
        o = self._offs
        return [self._out[int(o[c]):int(o[c + 1])].copy() for c in range(len(self._states))]

    @property
    def tiling(self) -> dict:
        """Per row width (32- and 64-bit rows; 0 where the plan has none): kets per chunk,
        tasks per resident warp, kernel variant; and whether creation timed candidates."""
        chunk, tpw, minb = (C.c_int32 * 2)(), (C.c_int32 * 2)(), (C.c_int32 * 2)()
        timed = C.c_int32()
        check(_ffi.load().nsg_plan_info(self._h, chunk, tpw, minb, C.byref(timed)))
        out = {"timed": bool(timed.value)}
        for w, name in ((0, "rows32"), (1, "rows64")):
            out[f"chunk_{name}"] = chunk[w]
            out[f"tasks_per_warp_{name}"] = tpw[w]
            out[f"minb_{name}"] = minb[w]
        return out


def exp_values_multi(states, paulis_per_state, precision: int = PRECISION_FP64,
                     screen: bool = False) -> list[np.ndarray]:
    """⟨P⟩ for many states at once: observables ``paulis_per_state[c]`` on
    ``states[c]``, every pair sum in one persistent launch (one per row width:
    ≤ 32 and > 32 qubits).  Returns one array per state, each value as
    ``states[c].exp_values(paulis_per_state[c], precision)`` gives it.
    screen=True (opt-in): states whose every observable the common-stabilizer
    test (QuantumState.zero_screen) decides get the exact zeros without a pair
    sum; the others are summed as usual."""
    if screen:
        states, paulis_per_state = list(states), [list(p) for p in paulis_per_state]
        done = [bool(ps) and s.zero_screen(ps).all() for s, ps in zip(states, paulis_per_state)]
        rest = [c for c in range(len(states)) if not done[c]]
        out = [np.zeros(len(ps), np.float64) for ps in paulis_per_state]
        if rest:
            got = exp_values_multi([states[c] for c in rest], [paulis_per_state[c] for c in rest], precision)
            for k, c in enumerate(rest):
                out[c] = got[k]
        return out
    states, groups, offs, total, arr, hs = _multi_args(states, paulis_per_state)
    out = np.zeros(max(total, 1), np.float64)
    check(_ffi.load().nsg_exp_value_multi(hs, len(states), arr, _p(offs), precision, _p(out)))
    return [out[int(offs[c]):int(offs[c + 1])].copy() for c in range(len(states))]
