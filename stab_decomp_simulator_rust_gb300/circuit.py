"""QuantumCircuit / QuantumGate — the circuit blueprint handed to QuantumState.

Mirrors the reference's Python surface (python/necstar/circuit.pyi,
python/necstar/gate.pyi; Rust crates/necstar/src/circuit/mod.rs:53-56 and
circuit/gates.rs:7-42).  A circuit is a gate list; the gate opcodes are those
of include/necstar_gpu.h.  Nothing is validated here: like the reference,
qubit indices are checked when the circuit is compiled.
"""
from __future__ import annotations

import numpy as np

from .workloads import OP

_NAMES = {v: k for k, v in OP.items()}
_DISPLAY = {"H": "H", "X": "X", "Y": "Y", "Z": "Z", "S": "S", "SDG": "Sdg", "SQRT_X": "SqrtX",
            "SQRT_XDG": "SqrtXdg", "CX": "CX", "CZ": "CZ", "SWAP": "Swap", "T": "T", "TDG": "Tdg", "CCX": "CCX"}
_ARITY = {"H": 1, "X": 1, "Y": 1, "Z": 1, "S": 1, "SDG": 1, "SQRT_X": 1, "SQRT_XDG": 1,
          "CX": 2, "CZ": 2, "SWAP": 2, "T": 1, "TDG": 1, "CCX": 3}
_ALIASES = {"h": "H", "x": "X", "y": "Y", "z": "Z", "s": "S", "sdg": "SDG", "sx": "SQRT_X", "sqrt_x": "SQRT_X",
            "sxdg": "SQRT_XDG", "sqrt_xdg": "SQRT_XDG", "cx": "CX", "cnot": "CX", "cz": "CZ", "swap": "SWAP",
            "t": "T", "tdg": "TDG", "ccx": "CCX", "toffoli": "CCX"}


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
        """``apply_gate(QuantumGate)`` or ``apply_gate(name, qubits)`` (circuit.pyi:141)."""
        if isinstance(gate, QuantumGate):
            self._rows.append(gate.row())
            return
        key = _ALIASES.get(str(gate).lower(), str(gate).upper())
        if key not in OP:
            raise ValueError(f"Unknown gate name: {gate}")
        qs = list(qubits or [])
        if len(qs) != _ARITY[key]:
            raise ValueError(f"Gate {gate} expects {_ARITY[key]} qubits, got {len(qs)}")
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

    def __str__(self) -> str:
        return f"QuantumCircuit(num_qubits={self._n}, num_gates={len(self._rows)})"
