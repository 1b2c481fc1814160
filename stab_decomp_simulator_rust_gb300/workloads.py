"""Seeded synthetic workloads (circuits and Pauli observables).

The reference names no public benchmark suite; its benchmark configurations
are random Clifford+T circuits generated from a fixed seed.  This module is
the project's documented generator for them:

* PRNG: xoshiro256** (Blackman & Vigna) whose four state words come from
  SplitMix64 applied to the seed; ``below(m)`` is Lemire's unbiased
  multiply-shift bounded draw.
* Circuits: ``num_clifford`` gates drawn uniformly from {H, S, CX} with
  uniform qubits (CX on a uniform ordered distinct pair), then ``num_t``
  T gates inserted one after another at uniform positions of the current
  list (0 .. len) on uniform qubits.  Start state |0^n⟩.
* Observables: dense Paulis with each qubit uniform in {I, X, Y, Z}, or
  sparse weight-k Paulis (k uniform in [kmin, kmax], support a uniform
  k-subset, ops uniform in {X, Y, Z}).

Gate lists are ``numpy.uint32`` arrays of shape (N, 4) = (op, q0, q1, q2)
with the opcodes of ``include/necstar_gpu.h``.
"""
from __future__ import annotations

import numpy as np

MASK64 = (1 << 64) - 1

OP = {
    "H": 0, "X": 1, "Y": 2, "Z": 3, "S": 4, "SDG": 5, "SQRT_X": 6, "SQRT_XDG": 7,
    "CX": 8, "CZ": 9, "SWAP": 10, "T": 11, "TDG": 12, "CCX": 13,
}


class Xoshiro256ss:
    def __init__(self, seed: int):
        x = seed & MASK64
        self.s = []
        for _ in range(4):
            x = (x + 0x9E3779B97F4A7C15) & MASK64
            z = x
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
            self.s.append(z ^ (z >> 31))

    @staticmethod
    def _rotl(x: int, k: int) -> int:
        return ((x << k) | (x >> (64 - k))) & MASK64

    def next(self) -> int:
        s = self.s
        r = (self._rotl((s[1] * 5) & MASK64, 7) * 9) & MASK64
        t = (s[1] << 17) & MASK64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = self._rotl(s[3], 45)
        return r

    def below(self, m: int) -> int:
        """Uniform integer in [0, m) (Lemire's method with rejection)."""
        if m <= 0:
            raise ValueError("m must be positive")
        while True:
            x = self.next()
            prod = x * m
            lo = prod & MASK64
            if lo >= m or lo >= ((1 << 64) - m) % m:
                return prod >> 64


def random_clifford_t_circuit(n: int, num_clifford: int, num_t: int, seed: int) -> np.ndarray:
    """{H, S, CX} random circuit with T gates inserted at uniform positions."""
    rng = Xoshiro256ss(seed)
    gates: list[tuple[int, int, int, int]] = []
    for _ in range(num_clifford):
        kind = rng.below(3) if n >= 2 else rng.below(2)
        if kind == 0:
            gates.append((OP["H"], rng.below(n), 0, 0))
        elif kind == 1:
            gates.append((OP["S"], rng.below(n), 0, 0))
        else:
            c = rng.below(n)
            t = rng.below(n - 1)
            if t >= c:
                t += 1
            gates.append((OP["CX"], c, t, 0))
    for _ in range(num_t):
        pos = rng.below(len(gates) + 1)
        q = rng.below(n)
        gates.insert(pos, (OP["T"], q, 0, 0))
    return np.asarray(gates, dtype=np.uint32).reshape(-1, 4)


def random_dense_paulis(n: int, count: int, seed: int) -> list[np.ndarray]:
    """Dense Paulis, each qubit uniform in {I, X, Y, Z} (little-endian ops)."""
    rng = Xoshiro256ss(seed)
    return [np.asarray([rng.below(4) for _ in range(n)], dtype=np.uint8) for _ in range(count)]


def random_sparse_paulis(n: int, count: int, kmin: int, kmax: int, seed: int):
    """Sparse Paulis of weight k ~ U[kmin, kmax] on uniform supports, ops in {X,Y,Z}.

    Returns a list of (ops, qubits) pairs with qubits ascending."""
    rng = Xoshiro256ss(seed)
    out = []
    for _ in range(count):
        k = kmin + rng.below(kmax - kmin + 1)
        pool = list(range(n))
        sup = []
        for i in range(k):  # partial Fisher-Yates
            j = i + rng.below(n - i)
            pool[i], pool[j] = pool[j], pool[i]
            sup.append(pool[i])
        sup.sort()
        ops = [1 + rng.below(3) for _ in range(k)]
        out.append((np.asarray(ops, dtype=np.uint8), np.asarray(sup, dtype=np.uint32)))
    return out


# The five benchmark configurations of the path, by what they are.
SMALL_N16 = dict(n=16, num_clifford=1000, num_t=6, seed=1)           # plain method, CPU-runnable
PLAIN_N40 = dict(n=40, num_clifford=4000, num_t=24, seed=2, num_paulis=64)
PRECISION_N60 = dict(n=60, num_clifford=6000, num_t=36, seed=3, num_paulis=256)
BATCH_512 = dict(num_circuits=512, nmin=8, nmax=64, tmin=4, tmax=32, gates_per_qubit=20,
                 num_paulis=16, seed=4)
PROJECT_N64 = dict(n=64, num_clifford=8000, num_t=40, seed=5, num_project=8, shots=1_000_000)


def batch_circuits(cfg: dict = BATCH_512):
    """Circuits of the batching workload: n ~ U[nmin, nmax], t ~ U[tmin, tmax],
    20·n {H,S,CX} gates; circuit c is seeded with seed·1_000_003 + c."""
    out = []
    for c in range(cfg["num_circuits"]):
        rng = Xoshiro256ss(cfg["seed"] * 1_000_003 + c)
        n = cfg["nmin"] + rng.below(cfg["nmax"] - cfg["nmin"] + 1)
        t = cfg["tmin"] + rng.below(cfg["tmax"] - cfg["tmin"] + 1)
        gates = random_clifford_t_circuit(n, cfg["gates_per_qubit"] * n, t, rng.next())
        paulis = random_dense_paulis(n, cfg["num_paulis"], rng.next())
        out.append((n, gates, paulis))
    return out
