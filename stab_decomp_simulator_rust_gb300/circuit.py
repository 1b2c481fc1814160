"""QuantumCircuit / QuantumGate — the circuit blueprint handed to QuantumState.

Mirrors the reference's Python surface (python/necstar/circuit.pyi,
python/necstar/gate.pyi; Rust crates/necstar/src/circuit/mod.rs:53-56 and
circuit/gates.rs:7-42).  A circuit is a gate list; the gate opcodes are those
of include/necstar_gpu.h.  Nothing is validated here: like the reference,
qubit indices are checked when the circuit is compiled.

Circuit ingestion follows crates/necstar/src/circuit/parser.rs: an OpenQASM
2.0 subset read line by line (one register, the gates h x y z s sdg sx sxdg
t tdg cx cz swap ccx, ``measure`` lines ignored with a warning, anything
else an error) and written back in the same form; ``random_clifford`` draws
a uniformly random Clifford circuit with the library's seeded generator.
"""
from __future__ import annotations

import ctypes as C
import re
import sys

import numpy as np

from ._ffi import NecstarError
from .workloads import OP

_NAMES = {v: k for k, v in OP.items()}
_DISPLAY = {"H": "H", "X": "X", "Y": "Y", "Z": "Z", "S": "S", "SDG": "Sdg", "SQRT_X": "SqrtX",
            "SQRT_XDG": "SqrtXdg", "CX": "CX", "CZ": "CZ", "SWAP": "Swap", "T": "T", "TDG": "Tdg", "CCX": "CCX"}
_ARITY = {"H": 1, "X": 1, "Y": 1, "Z": 1, "S": 1, "SDG": 1, "SQRT_X": 1, "SQRT_XDG": 1,
          "CX": 2, "CZ": 2, "SWAP": 2, "T": 1, "TDG": 1, "CCX": 3}
# QuantumCircuit.apply_gate(name, qubits) of the Python layer
# (python/src/circuit.rs:90-186): case-insensitive names, the arity message
# of each gate; CCX is not reachable by name there.
_BY_NAME = {"h": ("H", "H gate requires 1 qubit index."), "x": ("X", "X gate requires 1 qubit index."),
            "y": ("Y", "Y gate requires 1 qubit index."), "z": ("Z", "Z gate requires 1 qubit index."),
            "s": ("S", "S gate requires 1 qubit index."), "sdg": ("SDG", "Sdg gate requires 1 qubit index."),
            "sqrtx": ("SQRT_X", "SqrtX gate requires 1 qubit index."),
            "sqrtxdg": ("SQRT_XDG", "SqrtXdg gate requires 1 qubit index."),
            "t": ("T", "T gate requires 1 qubit index."), "tdg": ("TDG", "Tdg gate requires 1 qubit index."),
            "cx": ("CX", "CX gate requires 2 qubit indices (control, target)."),
            "cnot": ("CX", "CX gate requires 2 qubit indices (control, target)."),
            "cz": ("CZ", "CZ gate requires 2 qubit indices."), "swap": ("SWAP", "SWAP gate requires 2 qubit indices.")}
# OpenQASM mnemonics (QuantumGate::to_qasm_str, crates/necstar/src/circuit/gates.rs:235-257)
_QASM = {"H": "h", "X": "x", "Y": "y", "Z": "z", "S": "s", "SDG": "sdg", "SQRT_X": "sx", "SQRT_XDG": "sxdg",
         "T": "t", "TDG": "tdg", "CX": "cx", "CZ": "cz", "SWAP": "swap", "CCX": "ccx"}
_FROM_QASM = {v: k for k, v in _QASM.items()}


class QuantumGate:
    """One gate: opcode and qubits (QuantumGate, crates/necstar/src/circuit/gates.rs:7-42)."""

    __slots__ = ("op", "_q")

    def __init__(self, op: int, qubits):
        self.op = int(op)
        self._q = tuple(int(q) for q in qubits)

    @property
    def qubits(self) -> list[int]:
        return list(self._q)

    @property
    def name(self) -> str:
        return _DISPLAY[_NAMES[self.op]]

    def is_clifford(self) -> bool:
        return self.op <= OP["SWAP"]

    def is_t_type(self) -> bool:
        return self.op in (OP["T"], OP["TDG"])

    is_t_type_gate = is_t_type

    def row(self) -> tuple[int, int, int, int]:
        q = list(self._q) + [0, 0, 0]
        return (self.op, q[0], q[1], q[2])

    def __eq__(self, other) -> bool:
        return isinstance(other, QuantumGate) and self.op == other.op and self._q == other._q

    def __str__(self) -> str:  # QuantumGate Display (crates/necstar/src/circuit/gates.rs:329-347)
        return f"{self.name}({', '.join(map(str, self._q))})"

    def __repr__(self) -> str:
        return f"<QuantumGate: {self}>"

    # constructors (python/necstar/gate.pyi)
    @staticmethod
    def h(q): return QuantumGate(OP["H"], (q,))
    @staticmethod
    def x(q): return QuantumGate(OP["X"], (q,))
    @staticmethod
    def y(q): return QuantumGate(OP["Y"], (q,))
    @staticmethod
    def z(q): return QuantumGate(OP["Z"], (q,))
    @staticmethod
    def s(q): return QuantumGate(OP["S"], (q,))
    @staticmethod
    def sdg(q): return QuantumGate(OP["SDG"], (q,))
    @staticmethod
    def sqrt_x(q): return QuantumGate(OP["SQRT_X"], (q,))
    @staticmethod
    def sqrt_xdg(q): return QuantumGate(OP["SQRT_XDG"], (q,))
    @staticmethod
    def cx(c, t): return QuantumGate(OP["CX"], (c, t))
    @staticmethod
    def cz(a, b): return QuantumGate(OP["CZ"], (a, b))
    @staticmethod
    def swap(a, b): return QuantumGate(OP["SWAP"], (a, b))
    @staticmethod
    def t(q): return QuantumGate(OP["T"], (q,))
    @staticmethod
    def tdg(q): return QuantumGate(OP["TDG"], (q,))
    @staticmethod
    def ccx(c1, c2, t): return QuantumGate(OP["CCX"], (c1, c2, t))


def gate_rows(gates) -> np.ndarray:
    """Gate list → uint32 array (N, 4) for the C ABI."""
    if isinstance(gates, np.ndarray):
        return np.ascontiguousarray(gates, dtype=np.uint32).reshape(-1, 4)
    rows = [g.row() if isinstance(g, QuantumGate) else tuple(g) for g in gates]
    return np.asarray(rows, dtype=np.uint32).reshape(-1, 4)


class QuantumCircuit:
    """Gate-list blueprint (QuantumCircuit, crates/necstar/src/circuit/mod.rs:53-56)."""

    def __init__(self, num_qubits: int):
        self._n = int(num_qubits)
        self._rows: list[tuple[int, int, int, int]] = []

    @staticmethod
    def from_gate_array(num_qubits: int, rows: np.ndarray) -> "QuantumCircuit":
        c = QuantumCircuit(num_qubits)
        c._rows = [tuple(int(x) for x in r) for r in np.asarray(rows).reshape(-1, 4)]
        return c

    @property
    def num_qubits(self) -> int:
        return self._n

    @property
    def num_gates(self) -> int:
        return len(self._rows)

    @property
    def gates(self) -> list[QuantumGate]:
        return [QuantumGate(r[0], r[1:1 + _ARITY[_NAMES[r[0]]]]) for r in self._rows]

    def gate_array(self) -> np.ndarray:
        return np.asarray(self._rows, dtype=np.uint32).reshape(-1, 4)

    def apply_gate(self, gate, qubits=None) -> None:
        """``apply_gate(name, qubits)`` (python/necstar/circuit.pyi:141) or ``apply_gate(QuantumGate)``."""
        if isinstance(gate, QuantumGate):
            self._rows.append(gate.row())
            return
        entry = _BY_NAME.get(str(gate).lower())
        if entry is None:
            raise ValueError(f"Unknown gate name: '{gate}'")
        key, arity_msg = entry
        qs = [int(q) for q in (qubits or [])]
        if any(q < 0 for q in qs):
            raise OverflowError("can't convert negative int to unsigned")
        if len(qs) != _ARITY[key]:
            raise ValueError(arity_msg)
        self._rows.append(QuantumGate(OP[key], qs).row())

    def apply_gates(self, gates) -> None:
        for g in gates:
            self.apply_gate(g)

    def append(self, other: "QuantumCircuit") -> None:
        self._rows.extend(other._rows)

    def apply_h(self, q): self._rows.append((OP["H"], q, 0, 0))
    def apply_x(self, q): self._rows.append((OP["X"], q, 0, 0))
    def apply_y(self, q): self._rows.append((OP["Y"], q, 0, 0))
    def apply_z(self, q): self._rows.append((OP["Z"], q, 0, 0))
    def apply_s(self, q): self._rows.append((OP["S"], q, 0, 0))
    def apply_sdg(self, q): self._rows.append((OP["SDG"], q, 0, 0))
    def apply_sqrt_x(self, q): self._rows.append((OP["SQRT_X"], q, 0, 0))
    def apply_sqrt_xdg(self, q): self._rows.append((OP["SQRT_XDG"], q, 0, 0))
    def apply_t(self, q): self._rows.append((OP["T"], q, 0, 0))
    def apply_tdg(self, q): self._rows.append((OP["TDG"], q, 0, 0))
    def apply_cx(self, c, t): self._rows.append((OP["CX"], c, t, 0))
    def apply_cz(self, a, b): self._rows.append((OP["CZ"], a, b, 0))
    def apply_swap(self, a, b): self._rows.append((OP["SWAP"], a, b, 0))
    def apply_ccx(self, c1, c2, t): self._rows.append((OP["CCX"], c1, c2, t))

    def tensor(self, other: "QuantumCircuit") -> "QuantumCircuit":
        """self ⊗ other: other's gates act on qubits shifted by self.num_qubits
        (QuantumCircuit::tensor, crates/necstar/src/circuit/mod.rs:253-270)."""
        c = QuantumCircuit(self._n + other._n)
        off = self._n
        c._rows = list(self._rows)
        for op, q0, q1, q2 in other._rows:
            k = _ARITY[_NAMES[op]]
            c._rows.append((op, q0 + off, q1 + off if k > 1 else q1, q2 + off if k > 2 else q2))
        return c

    # ---- OpenQASM 2.0 (crates/necstar/src/circuit/parser.rs) ----
    @staticmethod
    def from_qasm_str(qasm: str) -> "QuantumCircuit":
        """parser.rs:17-186; every failure is a ValueError "Failed to parse QASM string: …"
        (python/src/circuit.rs:53-60)."""
        try:
            return _parse_qasm(qasm)
        except _QasmError as e:
            raise _qasm_exc(NecstarError, f"Failed to parse QASM string: {e}") from None

    @staticmethod
    def from_qasm_file(path: str) -> "QuantumCircuit":
        """parser.rs:191-201; every failure (unreadable file or bad content) is a
        FileNotFoundError "Failed to read QASM file: …" (python/src/circuit.rs:43-51)."""
        try:
            try:
                with open(path, "rb") as f:
                    raw = f.read()
            except OSError as e:
                raise _QasmError(f"Failed to read file '{path}': {_os_message(e)}") from None
            try:
                text = raw.decode("utf-8")
            except UnicodeDecodeError:
                raise _QasmError(f"Failed to read file '{path}': stream did not contain valid UTF-8") from None
            return _parse_qasm(text)
        except _QasmError as e:
            raise _qasm_exc(QasmFileError, f"Failed to read QASM file: {e}") from None

    def to_qasm_str(self, reg_name: str) -> str:
        """parser.rs:203-214: header, register, one line per gate, no final newline."""
        lines = ["OPENQASM 2.0;", 'include "qelib1.inc";', f"qreg {reg_name}[{self._n}];"]
        for op, q0, q1, q2 in self._rows:
            name = _NAMES[op]
            args = [q0, q1, q2][:_ARITY[name]]
            lines.append(f"{_QASM[name]} " + ", ".join(f"{reg_name}[{q}]" for q in args) + ";")
        return "\n".join(lines)

    def to_qasm_file(self, path: str, reg_name: str) -> None:
        """parser.rs:221-230; a write failure is a ValueError "Failed to write QASM file: IO error: …"."""
        text = self.to_qasm_str(reg_name)
        try:
            with open(path, "wb") as f:
                f.write(text.encode("utf-8"))
        except OSError as e:
            raise NecstarError(_IO_ERR, f"Failed to write QASM file: IO error: {_os_message(e)}", [-1, -1, -1]) \
                from None

    @staticmethod
    def random_clifford(n: int, seed=None) -> "QuantumCircuit":
        """A uniformly random n-qubit Clifford circuit (QuantumCircuit::random_clifford,
        crates/necstar/src/circuit/mod.rs:289-291): the Bravyi–Maslov canonical form drawn
        by nsg_random_clifford from the seeded stream (seeds as in python/src/utils.rs)."""
        from . import _ffi
        from .state import seed_bytes
        n = int(n)
        if n < 0:
            raise OverflowError("can't convert negative int to unsigned")
        sd = seed_bytes(seed)
        cap = 2 * n * n + 3 * n
        out = np.zeros((max(cap, 1), 4), dtype=np.uint32)
        nout = C.c_size_t()
        _ffi.check(_ffi.load().nsg_random_clifford(
            n, sd.ctypes.data_as(C.c_void_p) if sd is not None else None,
            out.ctypes.data_as(C.c_void_p), cap, C.byref(nout)))
        return QuantumCircuit.from_gate_array(n, out[:nout.value])

    def __str__(self) -> str:  # QuantumCircuit Display (crates/necstar/src/circuit/mod.rs:326-338)
        return f"QuantumCircuit(num_qubits={self._n}) [" + ", ".join(str(g) for g in self.gates) + "]"

    __repr__ = __str__


# ---------------------------------------------------------------------------
# OpenQASM 2.0 reader (parser.rs:17-186).  Each line is trimmed; blank lines,
# "//" comments and lines starting with OPENQASM or include are skipped; a
# qreg declaration (exactly one) sets the width; "measure" lines are ignored
# with a warning on stderr; otherwise the line must contain a 3-, 2- or
# 1-qubit gate application of a known name (tried in that order) or it is an
# error.  Matching is a search within the line, as the reference's regexes do.
_IDENT = r"[a-zA-Z][a-zA-Z0-9_]*"
_QREG = re.compile(r"qreg\s+(" + _IDENT + r")\s*\[\s*(\d+)\s*\]\s*;")


def _gate_pattern(k: int) -> re.Pattern:
    arg = r"(" + _IDENT + r")\[(\d+)\]"
    return re.compile(r"([a-z_]+)\s+" + r",\s*".join([arg] * k) + r"\s*;")


_GATE_RE = {k: _gate_pattern(k) for k in (3, 2, 1)}
# Unicode White_Space (Rust's str::trim)
_WS = "\t\n\x0b\x0c\r \x85\xa0\u1680\u2000\u2001\u2002\u2003\u2004\u2005\u2006\u2007\u2008\u2009\u200a" \
      "\u2028\u2029\u202f\u205f\u3000"
_QASM_ERR = 19  # NSG_ERR_QASM_PARSING
_IO_ERR = 20    # NSG_ERR_IO


class _QasmError(Exception):
    def __str__(self) -> str:  # Error::QasmParsingError Display (crates/necstar/src/error/mod.rs:73)
        return f"QASM parsing error: {self.args[0]}"


def _os_message(e: OSError) -> str:  # std::io::Error Display for an OS error
    return f"{e.strerror} (os error {e.errno})" if e.errno is not None else str(e)


def _usize(text: str, line: str, what: str) -> int:
    """`str::parse::<usize>()` with its failure messages."""
    if not text.isascii():
        raise _QasmError(f"Invalid {what} in line: '{line}' (invalid digit found in string)")
    v = int(text)
    if v >= 1 << 64:
        raise _QasmError(f"Invalid {what} in line: '{line}' (number too large to fit in target type)")
    return v


def _parse_qasm(qasm: str) -> "QuantumCircuit":
    n = None
    rows = []
    for num, raw in enumerate(qasm.split("\n")):
        line = raw.strip(_WS)
        if not line or line.startswith("//") or line.startswith("OPENQASM") or line.startswith("include"):
            continue
        m = _QREG.search(line)
        if m:
            if n is not None:
                raise _QasmError("Multiple qreg declarations are not supported.")
            n = _usize(m.group(2), line, "qreg size")
            continue
        if line.startswith("measure"):
            sys.stderr.write(f"[Warning] Line {num + 1}: `measure` operation is ignored by the parser.\n")
            continue
        done = False
        for k in (3, 2, 1):
            m = _GATE_RE[k].search(line)
            if not m:
                continue
            key = _FROM_QASM.get(m.group(1))
            if key is None or _ARITY[key] != k:
                continue
            qs = [_usize(m.group(3 + 2 * a), line, "qubit index") for a in range(k)] + [0] * (3 - k)
            rows.append((OP[key], qs[0], qs[1], qs[2]))
            done = True
            break
        if not done:
            raise _QasmError(f"Unrecognized or malformed line: {line}")
    if n is None:
        raise _QasmError("qreg declaration not found in QASM string.")
    return QuantumCircuit.from_gate_array(n, np.asarray(rows, dtype=np.uint64).reshape(-1, 4))


def _qasm_exc(cls, message: str):
    return cls(_QASM_ERR, message, [-1, -1, -1])


class QasmFileError(NecstarError, FileNotFoundError):
    """from_qasm_file's failure: a FileNotFoundError like the reference's Python layer
    (python/src/circuit.rs:45-47), and a NecstarError like every other failure here."""
