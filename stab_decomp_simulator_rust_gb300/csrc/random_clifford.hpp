// random_clifford.hpp — uniformly random n-qubit Clifford circuits
// (QuantumCircuit::random_clifford, crates/necstar/src/circuit/mod.rs:289-291
// → crates/stabilizer-ch-form-rust/src/circuit/random_clifford.rs:177-212).
//
// Method: Bravyi & Maslov, "Hadamard-free circuits expose the structure of
// the Clifford group", IEEE Trans. Inf. Theory 67, 5800 (2021),
// arXiv:2003.09412: U = F1·H·S·F2 with (h, S) drawn from the quantum Mallows
// distribution and F1, F2 Hadamard-free layers whose free entries are fair
// bits (rules C1–C5 of Theorem 1 restrict F1).  To give the same circuit as
// the reference for the same seed, the draws happen in the reference's order
// and the gates are emitted in its order (random_clifford.rs:7-175):
//   1. per position i: one uniform double for the Mallows step;
//   2. n bits for the Z part and n bits for the X part of F2's Pauli layer;
//   3. per i: F2's diagonal bit, then (if h_i) F1's diagonal bit;
//   4. per i > j: F2's symmetric CZ bit, F2's CNOT bit, then F1's CZ bit and
//      F1's CNOT bit where the rules allow them;
// and the circuit is F2 (CNOTs, then S/CZ, then Paulis), the permutation as
// SWAPs, the Hadamards, then F1 (CNOTs, then S/CZ).
#pragma once

#include <cmath>
#include <cstdint>
#include <utility>
#include <vector>

#include "host_rng.hpp"
#include "necstar_gpu.h"

namespace nsg {

// Upper bound on the gate count for n qubits: two layers of at most
// n(n-1)/2 CNOTs, n(n-1)/2 CZs and n S gates, n Paulis, n-1 SWAPs, n H.
inline uint64_t random_clifford_max_gates(uint64_t n) { return n == 0 ? 0 : 2 * n * n + 3 * n; }

struct CliffordLayer {
    uint32_t n;
    std::vector<uint8_t> cz;    // symmetric, n×n; diagonal = S
    std::vector<uint8_t> cnot;  // below the diagonal: (i, j), i > j → CX(j, i)
    explicit CliffordLayer(uint32_t n_) : n(n_), cz((size_t)n_ * n_, 0), cnot((size_t)n_ * n_, 0) {}
    uint8_t& z(uint32_t i, uint32_t j) { return cz[(size_t)i * n + j]; }
    uint8_t& c(uint32_t i, uint32_t j) { return cnot[(size_t)i * n + j]; }
};

inline void emit_layer(CliffordLayer& L, std::vector<nsg_gate>& out) {
    const uint32_t n = L.n;
    for (uint32_t j = 0; j < n; j++)
        for (uint32_t i = j + 1; i < n; i++)
            if (L.c(i, j)) out.push_back({NSG_GATE_CX, j, i, 0});
    for (uint32_t i = 0; i < n; i++) {
        if (L.z(i, i)) out.push_back({NSG_GATE_S, i, 0, 0});
        for (uint32_t j = 0; j < i; j++)
            if (L.z(i, j)) out.push_back({NSG_GATE_CZ, i, j, 0});
    }
}

// The quantum Mallows step for a block of m remaining positions: a ∈ [1, 2m]
// with P(a) ∝ 2^{-a} by inverting the distribution function
// (arXiv:2003.09412, Algorithm 1 / Lemma 6); a ≤ m sets h and picks the a-th
// remaining index, otherwise h = 0 and the (2m + 1 - a)-th.
inline void mallows_step(double r, uint64_t m, uint8_t& h, uint64_t& pick_1based) {
    const double val = r * (std::pow(4.0, (double)m) - 1.0) + 1.0;
    const double cl = std::ceil(std::log2(val));
    // ceil(log2) as an integer with a saturating conversion (NaN → 0, which
    // only r = 0 with 4^m = ∞ produces); a ≤ 0 is clamped to 1.
    const uint64_t ci = std::isnan(cl) ? 0 : (cl >= 18446744073709551616.0 ? UINT64_MAX : (uint64_t)cl);
    const uint64_t a = ci >= 2 * m + 1 ? 1 : 2 * m + 1 - ci;
    if (a <= m) {
        h = 1;
        pick_1based = a;
    } else {
        h = 0;
        pick_1based = 2 * m - a + 1;  // 0 only for r = 0 exactly
    }
}

inline std::vector<nsg_gate> random_clifford_gates(uint32_t n, HostRng& rng) {
    std::vector<nsg_gate> out;
    if (n == 0) return out;
    std::vector<uint8_t> h(n, 0);
    std::vector<uint32_t> perm(n, 0), avail(n);
    for (uint32_t i = 0; i < n; i++) avail[i] = i;
    for (uint32_t i = 0; i < n; i++) {
        const uint64_t m = n - i;
        uint64_t k;
        mallows_step(rng.uniform(), m, h[i], k);
        if (k >= 1 && k - 1 < avail.size()) {
            perm[i] = avail[k - 1];
            avail.erase(avail.begin() + (k - 1));
        } else {  // a rounding edge: the last remaining index
            perm[i] = avail.back();
            avail.pop_back();
        }
    }
    CliffordLayer F1(n), F2(n);
    std::vector<uint8_t> pz(n), px(n);
    for (uint32_t i = 0; i < n; i++) pz[i] = (uint8_t)rng.bit();
    for (uint32_t i = 0; i < n; i++) px[i] = (uint8_t)rng.bit();
    for (uint32_t i = 0; i < n; i++) {
        F2.z(i, i) = (uint8_t)rng.bit();
        if (h[i]) F1.z(i, i) = (uint8_t)rng.bit();
    }
    for (uint32_t i = 1; i < n; i++) {
        for (uint32_t j = 0; j < i; j++) {
            const uint8_t b = (uint8_t)rng.bit();
            F2.z(i, j) = F2.z(j, i) = b;
            F2.c(i, j) = (uint8_t)rng.bit();
            const bool hi = h[i] != 0, hj = h[j] != 0;
            const uint32_t si = perm[i], sj = perm[j];
            if (((si < sj || hj) && hi) || (hj && sj < si)) {  // C1, C2: a free CZ in F1
                const uint8_t c = (uint8_t)rng.bit();
                F1.z(i, j) = F1.z(j, i) = c;
            }
            if ((si < sj || hj) && (si > sj || !hi) && (hj || !hi))  // C3–C5: a free CNOT in F1
                F1.c(i, j) = (uint8_t)rng.bit();
        }
    }
    emit_layer(F2, out);
    for (uint32_t i = 0; i < n; i++) {
        if (pz[i] && px[i]) out.push_back({NSG_GATE_Y, i, 0, 0});
        else if (pz[i]) out.push_back({NSG_GATE_Z, i, 0, 0});
        else if (px[i]) out.push_back({NSG_GATE_X, i, 0, 0});
    }
    std::vector<uint32_t> at(n);  // at[pos] = index currently at pos
    for (uint32_t i = 0; i < n; i++) at[i] = i;
    for (uint32_t i = 0; i < n; i++) {
        if (at[i] == perm[i]) continue;
        uint32_t j = i + 1;
        while (at[j] != perm[i]) j++;  // positions < i are final, so j > i
        out.push_back({NSG_GATE_SWAP, i, j, 0});
        std::swap(at[i], at[j]);
    }
    for (uint32_t i = 0; i < n; i++)
        if (h[i]) out.push_back({NSG_GATE_H, i, 0, 0});
    emit_layer(F1, out);
    return out;
}

}  // namespace nsg
