"""PauliString — dense ("IXYZ", little-endian) or sparse ("X1 Y3") observables.

Parsing follows PauliString's FromStr
(crates/stabilizer-ch-form-rust/src/types/pauli/mod.rs:51-143): an empty
string or "I" is the identity (sparse, no terms); a string containing digits
is sparse ("X1 y3": case-insensitive op + qubit, whitespace separated, no
repeated qubit); otherwise dense over {I, X, Y, Z}, reversed so that the
rightmost character acts on qubit 0.
"""
from __future__ import annotations

import ctypes as C
import re

import numpy as np

from ._ffi import NecstarError, PauliABI

I, X, Y, Z = 0, 1, 2, 3
_CH = {"I": I, "X": X, "Y": Y, "Z": Z}
_TERM = re.compile(r"^([XYZxyz])(\d+)$")
DENSE, SPARSE = 0, 1
_PARSE_ERR = 17  # NSG_ERR_PAULI_STRING_PARSING


class PauliString:
    __slots__ = ("kind", "ops", "qubits", "_keep")

    def __init__(self, kind: int, ops, qubits=None):
        self.kind = int(kind)
        self.ops = np.ascontiguousarray(np.asarray(ops, dtype=np.uint8))
        self.qubits = np.ascontiguousarray(np.asarray(qubits if qubits is not None else [], dtype=np.uint32))

    @staticmethod
    def identity() -> "PauliString":
        return PauliString(SPARSE, [], [])

    @staticmethod
    def dense(ops) -> "PauliString":
        """Little-endian ops list (ops[q] acts on qubit q)."""
        return PauliString(DENSE, ops)

    @staticmethod
    def sparse(ops, qubits) -> "PauliString":
        return PauliString(SPARSE, ops, qubits)

    @staticmethod
    def from_str(s: str) -> "PauliString":
        t = s.strip()
        if t == "" or t.lower() == "i":
            return PauliString.identity()
        if any(c.isdigit() for c in t):
            ops, qs, seen = [], [], set()
            for term in t.split():
                m = _TERM.match(term)
                if not m:
                    raise NecstarError(_PARSE_ERR, f"Invalid Pauli string format: invalid sparse Pauli term: "
                                                   f"'{term}' in string: '{t}'", [-1, -1, -1])
                q = int(m.group(2))
                if q in seen:
                    raise NecstarError(_PARSE_ERR, f"Invalid Pauli string format: duplicate Pauli operator on qubit "
                                                   f"{q} in string: '{t}'", [q, -1, -1])
                seen.add(q)
                ops.append(_CH[m.group(1).upper()])
                qs.append(q)
            return PauliString(SPARSE, ops, qs)
        ops = []
        for i, ch in enumerate(t):
            if ch not in _CH:
                raise NecstarError(_PARSE_ERR, f"Invalid Pauli string format: invalid character '{ch}' at position "
                                               f"{i} in dense PauliString", [i, -1, -1])
            ops.append(_CH[ch])
        return PauliString(DENSE, ops[::-1])

    @property
    def is_identity(self) -> bool:
        return bool(np.all(self.ops == I))

    def abi(self) -> PauliABI:
        return PauliABI(self.kind, len(self.ops), self.ops.ctypes.data_as(C.POINTER(C.c_uint8)),
                        self.qubits.ctypes.data_as(C.POINTER(C.c_uint32)) if len(self.qubits) else None)

    def __str__(self) -> str:
        inv = "IXYZ"
        if self.kind == SPARSE and len(self.ops) == 0:
            return "I"
        if self.kind == DENSE:
            return "".join(inv[o] for o in self.ops[::-1])
        return " ".join(f"{inv[o]}{q}" for o, q in zip(self.ops, self.qubits))

    def __repr__(self) -> str:
        return f"PauliString('{self}')"
