// kernels_pairs.cu — the χ² pair sums behind exp_value, norm and
// inner_product (crates/necstar/src/state/stabilizer_decomposed_state/
// {exp_value,norm,inner_product}.rs).
//
// Every pair value ⟨A|P|B⟩ between two CH-form terms is an exact
// e^{iπk/4}·2^{-r/2} (or 0) — a canonical number, so any exact method gives
// the reference's (k, r).  The reference computes it by Gauss-eliminating A
// to |0^n⟩ (a recorded list of O(n²) gates, form/inner_product.rs:52-123)
// and replaying that list on a clone of B.  Here the same quantity is an
// exponential sum evaluated in A's frame:
//
//   |A⟩ = φ_A U_A U_{H,A}|s_A⟩,  V = U_A^{-1} (tableau precomputed per A)
//   ⟨A|P|B⟩ = conj(φ_A)·μ_{A,P}·⟨x_{A,P}| U_{H,A}·D·U_{H,B}|s_B⟩·φ_B,  D = V·U_B
//
// with (x_{A,P}, μ_{A,P}) the Pauli seen from A's frame (precomputed per
// (A, P)).  D is control-type, so ⟨y|D U_{H,B}|s_B⟩ = ω^{ph_B}·2^{-|v_B|/2}·
// i^{γ_D·y}·(-1)^{Q(y) + (yF_D)·(v_B∧s_B)}·δ((yF_D ⊕ s_B)∧¬v_B = 0) with
// the quadratic form Q(y) = Σ_{p<r} y_p y_r K[r][p] + Σ_p y_p K[p][p],
// K = M_D·F_Dᵀ (arXiv:1808.00128 eqs. 48-55).  ⟨x|U_{H,A} sums that over
// the 2^{|v_A|} points y = x' ⊕ z, x' = x∧¬v_A, z ∈ span(v_A), which is a
// sum of i^{L·z}·(-1)^{zᵀJz} under |¬v_B| linear constraints.  It is reduced
// variable by variable (constraints by substitution, then each variable
// summed out: an odd L_j gives √2·ω^{±1} and a rank-one update of J, an even
// one gives 2·δ(linear form) and a substitution; variables no longer coupled
// to any other factor out and are summed out all at once), O(rank J) steps of
// O(1) word operations per lane.  The pivots, J and the low bits of L are the same for
// every observable, so one warp reduces one pair for up to 256 observables
// at once, each lane tracking the per-observable high bits of L, the phase
// and the constraint right-hand sides of its observables.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cstdint>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>

#include "device_state.hpp"
#include "warp_chform.cuh"

namespace nsg {
namespace {

using dev::FULL;
using dev::popc;
using dev::ffs0;
using dev::shfl;

constexpr int FWARPS = 4;  // warps per block in the frame kernels
constexpr int PWARPS = 4;  // warps per block in the pair kernel

__device__ __forceinline__ double pow2i(int e) {  // exact 2^e for |e| < 1022
    return __longlong_as_double((long long)(e + 1023) << 52);
}

// ---- bra frames ----------------------------------------------------------------
// For U with tableau (G, F, M, γ) (U^{-1} Z_p U = Z(G_p), U^{-1} X_p U =
// i^{γ_p} X(F_p) Z(M_p), F G^T = I), the inverse V = U^{-1} has
//   G_V = F^T,  F_V = G^T,  M_V = G^T M F^T,
//   γ_V[p] = -Σ_{q∈x} γ_q + 2·Σ_{q<r∈x} M_q·F_r  (mod 4),  x = column p of G.
__global__ void __launch_bounds__(FWARPS * 32) frames_kernel(TermsView tv, FrameView fr) {
    __shared__ uint64_t sF[FWARPS][64], sG[FWARPS][64], sM[FWARPS][64];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t term = (int64_t)blockIdx.x * FWARPS + wid;
    if (term >= tv.chi) return;
    const int n = tv.n;
    for (int r = lane; r < 64; r += 32) {
        size_t idx = ((size_t)term * tv.R + r) * tv.W;  // word 0 of row r (n ≤ 64)
        sF[wid][r] = tv.F[idx];
        sG[wid][r] = tv.G[idx];
        sM[wid][r] = tv.M[idx];
    }
    __syncwarp();
    const uint64_t gl = tv.GL[term * tv.W], gh = tv.GH[term * tv.W];
    uint32_t b0[2], b1[2];
    for (int k = 0; k < 2; k++) {
        int p = 32 * k + lane;
        uint64_t x = 0, gv = 0, y = 0, mv = 0;
        int cnt = 0, gsum = 0;
        if (p < n) {
            for (int q = 0; q < n; q++) {
                x |= ((sG[wid][q] >> p) & 1ULL) << q;
                gv |= ((sF[wid][q] >> p) & 1ULL) << q;
            }
            for (int q = 0; q < n; q++) {
                if ((x >> q) & 1ULL) {
                    cnt += __popcll(y & sF[wid][q]);
                    y ^= sM[wid][q];
                }
            }
            gsum = __popcll(x & gl) + 2 * __popcll(x & gh);
            for (int c = 0; c < n; c++) mv |= (uint64_t)(__popcll(y & sF[wid][c]) & 1) << c;
        }
        int gV = (-gsum + 2 * cnt) & 3;
        size_t o = (size_t)term * 64 + p;
        fr.GV[o] = gv;
        fr.FV[o] = x;
        fr.MV[o] = mv;
        b0[k] = __ballot_sync(FULL, (p < n) && (gV & 1));
        b1[k] = __ballot_sync(FULL, (p < n) && ((gV >> 1) & 1));
    }
    if (lane == 0) {
        fr.GVL[term] = (uint64_t)b0[0] | ((uint64_t)b0[1] << 32);
        fr.GVH[term] = (uint64_t)b1[0] | ((uint64_t)b1[1] << 32);
    }
}

// ---- Pauli frames ----------------------------------------------------------------
// P = i^{ny} X(px) Z(pz).  U_A^{-1} P U_A = i^{ny} λ(px) X(a) Z(b), a = px·F,
// b = px·M ⊕ pz·G, λ(px) = i^{Σγ_q} (-1)^{Σ_{q<r} M_q·F_r}.  Conjugating by
// U_{H,A} swaps X/Z on v_A (sign (-1)^{|a∧b∧v|}); then ⟨s_A|X(a')Z(b') =
// (-1)^{(s_A⊕a')·b'}⟨s_A⊕a'|.  Output x = s_A⊕a' and k = Z8 phase of
// conj(φ_A)·μ.
__global__ void __launch_bounds__(FWARPS * 32) pauli_frames_kernel(TermsView tv, const DevPauli* __restrict__ P,
                                                                  int nobs, uint64_t* __restrict__ xout,
                                                                  uint8_t* __restrict__ kout) {
    __shared__ uint64_t sF[FWARPS][64], sG[FWARPS][64], sM[FWARPS][64];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t term = (int64_t)blockIdx.x * FWARPS + wid;
    if (term >= tv.chi) return;
    const int n = tv.n;
    for (int r = lane; r < 64; r += 32) {
        size_t idx = ((size_t)term * tv.R + r) * tv.W;
        sF[wid][r] = tv.F[idx];
        sG[wid][r] = tv.G[idx];
        sM[wid][r] = tv.M[idx];
    }
    __syncwarp();
    const uint64_t gl = tv.GL[term * tv.W], gh = tv.GH[term * tv.W], vA = tv.V[term * tv.W], sA = tv.S[term * tv.W];
    const int phA = tv.phase[term];
    for (int o = lane; o < nobs; o += 32) {
        DevPauli pl = P[o];
        uint64_t a = 0, macc = 0;
        int cnt = 0;
        for (int q = 0; q < n; q++) {
            if ((pl.px >> q) & 1ULL) {
                cnt += __popcll(macc & sF[wid][q]);
                macc ^= sM[wid][q];
                a ^= sF[wid][q];
            }
        }
        uint64_t b = macc;
        for (int q = 0; q < n; q++)
            if ((pl.pz >> q) & 1ULL) b ^= sG[wid][q];
        int gsum = __popcll(pl.px & gl) + 2 * __popcll(pl.px & gh);
        int sign2 = __popcll(a & b & vA);
        uint64_t d = (a ^ b) & vA;
        uint64_t a2 = a ^ d, b2 = b ^ d;
        uint64_t x = sA ^ a2;
        int sign3 = __popcll(x & b2);
        int kmu = (2 * (pl.ny + gsum) + 4 * ((cnt + sign2 + sign3) & 1)) & 7;
        xout[(size_t)term * nobs + o] = x;
        kout[(size_t)term * nobs + o] = (uint8_t)((kmu - phA) & 7);
    }
}

// ---- pair kernel ---------------------------------------------------------------
template <typename Word>
__device__ __forceinline__ Word lowbits(uint64_t x) {
    return (Word)x;
}

// Re / Im of e^{iπk/4}·2^{-r/2} as (sign, m): value = sign·2^{-m/2}.
__device__ __forceinline__ void re_part(int k, int r, int& sgn, int& m) {
    switch (k & 7) {
        case 0: sgn = 1; m = r; break;
        case 4: sgn = -1; m = r; break;
        case 1: case 7: sgn = 1; m = r + 1; break;
        case 3: case 5: sgn = -1; m = r + 1; break;
        default: sgn = 0; m = 0; break;
    }
}
__device__ __forceinline__ void im_part(int k, int r, int& sgn, int& m) {
    switch (k & 7) {
        case 2: sgn = 1; m = r; break;
        case 6: sgn = -1; m = r; break;
        case 1: case 3: sgn = 1; m = r + 1; break;
        case 5: case 7: sgn = -1; m = r + 1; break;
        default: sgn = 0; m = 0; break;
    }
}

// Lane accumulators.  FP64 mode: plain FP64 sums of the exact terms within a
// chunk, folded into double-double partials per chunk.  Mixed mode: the same
// double registers hold an FP32 (hi, lo) pair each, accumulated with a
// compensated two-sum relative to a per-chunk power-of-two base 2^{-base}
// (exact scaling), widened to FP64 once per chunk.
__device__ __forceinline__ double pack_f2(float hi, float lo) {
    return __hiloint2double(__float_as_int(hi), __float_as_int(lo));
}
__device__ __forceinline__ void unpack_f2(double d, float& hi, float& lo) {
    hi = __int_as_float(__double2hiint(d));
    lo = __int_as_float(__double2loint(d));
}
__device__ __forceinline__ void two_sum_f(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void two_sum_d(double a, double b, double& s, double& e) {
    s = a + b;
    double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Per-lane, per-chunk accumulator of exact terms sign·2^{-e} in classes
// 0 = Re even, 1 = Re odd (×√½), 2 = Im even, 3 = Im odd.
template <int NG, int NA>
struct ChunkAcc {
    double a[NG][NA];
    int base[NG];
    __device__ __forceinline__ void reset() {
#pragma unroll
        for (int g = 0; g < NG; g++) {
#pragma unroll
            for (int c = 0; c < NA; c++) a[g][c] = 0.0;
            base[g] = INT_MIN;
        }
    }
    __device__ __forceinline__ void flush_group(int g, double* pp, bool mixed) {
#pragma unroll
        for (int c = 0; c < NA; c++) {
            double val = a[g][c];
            if (mixed) {
                float hi, lo;
                unpack_f2(val, hi, lo);
                val = (base[g] == INT_MIN) ? 0.0 : ((double)hi + (double)lo) * pow2i(-base[g]);
            }
            double s, err;
            two_sum_d(pp[2 * c], val, s, err);
            pp[2 * c] = s;
            pp[2 * c + 1] += err;
            a[g][c] = 0.0;
        }
        base[g] = INT_MIN;
    }
    __device__ __forceinline__ void add(int g, int cls, int sgn, int e, bool mixed, double* pp) {
        if (!mixed) {
            const double t = sgn * pow2i(-e);
#pragma unroll
            for (int c = 0; c < NA; c++)
                if (c == cls) a[g][c] += t;
            return;
        }
        if (base[g] == INT_MIN) base[g] = e;
        int d = base[g] - e;  // 2^{-e} = 2^{-base}·2^{d}
        if (d > 100 || d < -100) {
            flush_group(g, pp, true);
            base[g] = e;
            d = 0;
        }
        const float t = (float)sgn * __int_as_float((d + 127) << 23);
#pragma unroll
        for (int c = 0; c < NA; c++) {
            if (c == cls) {
                float hi, lo, sum, err;
                unpack_f2(a[g][c], hi, lo);
                two_sum_f(hi, t, sum, err);
                a[g][c] = pack_f2(sum, __fadd_rn(lo, err));
            }
        }
    }
};

// ---- term tables ----------------------------------------------------------------
// Per term B, Four-Russians tables (the 16 XOR combinations of each group of
// four rows) of three matrices the pair kernel multiplies by:
//   F        the tableau's F rows,
//   P        P[c] = the bits r > c of K[c]  (ordered-sign matrix),
//   K        K[c][r] = parity(M_c·F_r), i.e. K = M·F^T,
// then a 48-byte trailer with the term's scalars (KetTrailer), and last the
// table of G, which the pair kernel reads when the term is the bra.  Layout
// per term: [ngrp][16][F, P, K] Words (the three entries of one index side
// by side, so one address serves three loads), trailer, [G][ngrp][16] Words; one bulk
// copy of the first part brings everything the kernel reads of a ket.  ngrp
// is ⌈n/4⌉ rounded up to an even count: the padding group is all zeros, so
// the pair kernel looks groups up two at a time with no mask.
struct KetTrailer {
    uint64_t gl, gh, v, s;  // γ planes, v, s (low word)
    uint8_t phase, coef_k, pad0, pad1;
    int32_t coef_r;
    uint64_t pad2;
};
static_assert(sizeof(KetTrailer) == 48, "trailer size");

template <typename Word>
__global__ void __launch_bounds__(FWARPS * 32) ket_tables_kernel(TermsView tv, int ngrp, size_t stride,
                                                                 unsigned char* __restrict__ out) {
    __shared__ Word sR[FWARPS][4][64];  // F, P, K, G
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t term = (int64_t)blockIdx.x * FWARPS + wid;
    if (term >= tv.chi) return;
    const int n = tv.n;
    for (int r = lane; r < 64; r += 32) {
        size_t idx = ((size_t)term * tv.R + r) * tv.W;
        sR[wid][0][r] = (Word)tv.F[idx];
        sR[wid][2][r] = (Word)tv.M[idx];  // M, replaced by K below
        sR[wid][3][r] = (Word)tv.G[idx];
    }
    __syncwarp();
    Word kr[2];
    for (int t = 0; t < 2; t++) {
        const int c = lane + 32 * t;
        Word k = 0;
        if (c < n) {
            const Word mc = sR[wid][2][c];
            for (int r = 0; r < n; r++) k |= (Word)(popc<Word>(mc & sR[wid][0][r]) & 1) << r;
        }
        kr[t] = k;
    }
    __syncwarp();
    for (int t = 0; t < 2; t++) {
        const int c = lane + 32 * t;
        if (c < 8 * (int)sizeof(Word)) {
            sR[wid][2][c] = kr[t];
            sR[wid][1][c] = (c + 1 < 8 * (int)sizeof(Word)) ? (kr[t] & ~(((Word)1 << (c + 1)) - 1)) : (Word)0;
        } else {
            sR[wid][2][c] = 0;
            sR[wid][1][c] = 0;
        }
    }
    __syncwarp();
    const int per = ngrp * 16;
    unsigned char* base = out + (size_t)term * stride;
    Word* dst = (Word*)base;
    Word* gdst = (Word*)(base + 3 * per * sizeof(Word) + sizeof(KetTrailer));
    for (int e = lane; e < 4 * per; e += 32) {
        const int mat = e / per, g = (e / 16) % ngrp, idx = e & 15;
        Word acc = 0;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int row = 4 * g + b;
            if (((idx >> b) & 1) && row < n) acc ^= sR[wid][mat][row];
        }
        if (mat < 3) dst[(g * 16 + idx) * 3 + mat] = acc;
        else gdst[e - 3 * per] = acc;
    }
    if (lane == 0) {
        KetTrailer t;
        t.gl = tv.GL[term * tv.W];
        t.gh = tv.GH[term * tv.W];
        t.v = tv.V[term * tv.W];
        t.s = tv.S[term * tv.W];
        t.phase = tv.phase[term];
        t.coef_k = tv.coef_k[term];
        t.pad0 = t.pad1 = 0;
        t.coef_r = tv.coef_r[term];
        t.pad2 = 0;
        *(KetTrailer*)(dst + 3 * per) = t;
    }
}

// ---- pair kernel ---------------------------------------------------------------
// Shared memory per warp: two ket buffers (double-buffered bulk copies of the
// next ket's tables), the bra's G table, the composed F and J rows (for the
// per-observable start values), and one mbarrier per ket buffer.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One elected lane: arm the barrier for `bytes` (+ `extra`, a test hook that
// leaves the phase incomplete after the copy has landed) and start the bulk
// copy of `bytes`.
__device__ __forceinline__ void tma_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                         uint32_t extra = 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes + extra)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Bounded wait on a barrier phase; false if the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    for (uint32_t it = 0; it < limit; it++) {
        uint32_t done;
        asm volatile(
            "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

template <typename Word>
__device__ __forceinline__ int parity(Word x) {
    return popc<Word>(x) & 1;
}

template <typename Word, int RPL>
__device__ __forceinline__ int nib(const Word x, int g) {  // 4-bit group g of a row
    return (int)((x >> (4 * g)) & 15);
}

// 32×32 bit-matrix transpose across a warp (lane l holds row l; returns row
// l of the transpose): five rounds of block swaps between lanes l and l^j.
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
    const uint32_t m[5] = {0x0000ffffu, 0x00ff00ffu, 0x0f0f0f0fu, 0x33333333u, 0x55555555u};
#pragma unroll
    for (int t = 0; t < 5; t++) {
        const int j = 16 >> t;
        const uint32_t y = __shfl_xor_sync(FULL, x, j);
        x = (lane & j) ? ((x & ~m[t]) | ((y >> j) & m[t])) : ((x & m[t]) | ((y << j) & ~m[t]));
    }
    return x;
}

// Transpose of a strictly lower-triangular matrix held as rows (lane, slot):
// one word per row for n ≤ 32, rows l and l+32 for n ≤ 64 (the upper-right
// 32×32 block is zero).
__device__ __forceinline__ void transpose_lower(const uint32_t (&L)[1], uint32_t (&T)[1], int lane) {
    T[0] = transpose32(L[0], lane);
}
__device__ __forceinline__ void transpose_lower(const uint64_t (&L)[2], uint64_t (&T)[2], int lane) {
    const uint32_t a = transpose32((uint32_t)L[0], lane);          // rows 0-31, cols 0-31
    const uint32_t c = transpose32((uint32_t)L[1], lane);          // rows 32-63, cols 0-31
    const uint32_t dd = transpose32((uint32_t)(L[1] >> 32), lane); // rows 32-63, cols 32-63
    T[0] = (uint64_t)a | ((uint64_t)c << 32);
    T[1] = (uint64_t)dd << 32;
}

// Bit `lane` of half k of a row mask (the lane's own row in slot k), tested on
// the 32-bit half that holds it.
template <typename Word>
__device__ __forceinline__ bool own_bit(Word x, int k, uint32_t lbit) {
    return ((uint32_t)(sizeof(Word) == 8 ? ((uint64_t)x >> (32 * k)) : (uint64_t)x) & lbit) != 0;
}

template <typename Word, int RPL>
__device__ __forceinline__ Word row_of(const Word (&R)[RPL], int q) {  // row q, from its lane
    return shfl<Word>((RPL > 1 && q >= 32) ? R[RPL - 1] : R[0], q & 31);
}

// The exponential sum Σ_z i^{L·z}·(-1)^{Σ_{a<b} J_ab z_a z_b} over the alive
// variables is reduced one variable at a time.  L = L0 + 2·h (mod 4): the low
// bits L0, the matrix J and the pivots are shared by all observables; the high
// bits split into a shared part hs and a per-observable part h[g].
//
// expand(T): multiply by i^{±τ}, τ = ⊕_{a∈T} z_a, using
// τ = Σ_a z_a − 2·Σ_{a<b} z_a z_b (mod 4): J ^= T·Tᵀ off the diagonal and
// L_a ± 1 on T (the per-observable part of the carry is applied by the caller).
template <typename Word, int RPL>
__device__ __forceinline__ void g_expand(Word (&J)[RPL], Word& hs, Word& L0, Word T, const Word (&own)[RPL]) {
    const uint32_t lbit = (uint32_t)own[0];
#pragma unroll
    for (int k = 0; k < RPL; k++)
        if (own_bit<Word>(T, k, lbit)) J[k] ^= T ^ own[k];  // own bit set in T: flip every other bit of T
    hs ^= T & ~L0;
    L0 ^= T;
}

// Calls f(slot, q) for the highest (HIGHEST) or lowest set bit of m ≠ 0:
// slot (a std::integral_constant) is the row slot that holds that row, q its
// bit within the slot's 32 bits.  Knowing the slot at compile time lets every
// test and update on that bit run on the one 32-bit half that holds it.
template <typename Word, bool HIGHEST, typename F>
__device__ __forceinline__ void on_bit(Word m, F&& f) {
    if constexpr (sizeof(Word) == 8) {
        const uint32_t hi = (uint32_t)((uint64_t)m >> 32), lo = (uint32_t)m;
        if (HIGHEST ? hi != 0 : lo == 0)
            f(std::integral_constant<int, 1>{}, HIGHEST ? 31 - __clz(hi) : __ffs(hi) - 1);
        else
            f(std::integral_constant<int, 0>{}, HIGHEST ? 31 - __clz(lo) : __ffs(lo) - 1);
    } else {
        f(std::integral_constant<int, 0>{}, HIGHEST ? 31 - __clz((uint32_t)m) : __ffs((uint32_t)m) - 1);
    }
}

// subst: eliminate z_k = c ⊕ lp·z (c per observable) from the form; k is
// bit q of row slot H (k = 32·H + q).
template <typename Word, int RPL, int NG, int H>
__device__ __forceinline__ void g_subst(int q, Word lp, const bool (&c)[NG], Word (&J)[RPL], Word& hs, Word& L0,
                                        Word& alive, Word (&h)[NG], int (&ph)[NG], const Word (&own)[RPL]) {
    const Word kb = (Word)(1u << q) << (32 * H);
    const Word R = shfl<Word>(J[H], q) & alive & ~kb;
#pragma unroll
    for (int k = 0; k < RPL; k++) {  // z_k·(R·z) → (lp·z)(R·z): J ^= lp·Rᵀ + R·lpᵀ
        const uint32_t lbit = (uint32_t)own[0];
        Word u = 0;
        if (own_bit<Word>(lp, k, lbit)) u ^= R;
        if (own_bit<Word>(R, k, lbit)) u ^= lp;
        J[k] ^= u;
    }
    hs ^= lp & R;  // its diagonal terms z_a² = z_a
    const bool lowk = (L0 & kb) != 0, hsk = (hs & kb) != 0;
    alive &= ~kb;
#pragma unroll
    for (int g = 0; g < NG; g++) {
        if (c[g]) h[g] ^= R;
        const bool hb = hsk ^ ((h[g] & kb) != 0);
        if (!lowk) {  // (-1)^{hb·(c ⊕ lp·z)}
            if (hb && c[g]) ph[g] += 4;
            if (hb) h[g] ^= lp;
        } else {  // i^{L_k·(c ⊕ lp·z)} = i^{L_k c}·i^{±lp·z}
            if (c[g]) ph[g] += hb ? 6 : 2;
            if (hb == c[g]) h[g] ^= lp;
        }
    }
    if (lowk) g_expand<Word, RPL>(J, hs, L0, lp, own);
}

template <typename Word>
__device__ __forceinline__ int fls0(Word x);  // index of the highest set bit
template <>
__device__ __forceinline__ int fls0<uint32_t>(uint32_t x) { return 31 - __clz(x); }

// The alive variables coupled to no other alive variable, one ballot per row
// slot.  They factor out together: an even L gives 2·δ(hb = 0) (IE), an odd
// one √2·ω^{1-2hb} (IO).
template <typename Word, int RPL>
__device__ __forceinline__ Word isolated(const Word (&J)[RPL], Word alive, const Word (&own)[RPL]) {
    Word iso = 0;
#pragma unroll
    for (int k = 0; k < RPL; k++)
        iso |= (Word)__ballot_sync(FULL, own_bit<Word>(alive, k, (uint32_t)own[0]) && !(J[k] & alive & ~own[k]))
               << (32 * k);
    return iso;
}

// Variables e just joined IE: an observable whose high bit hb (hs ^ h) is set
// on one of them has a zero term, whatever the rest of the sum (those bits
// never change again).  True when every observable of the warp is zero
// (zero[] is set on unused lanes), so the pair can stop: with many random
// observables a pair often ends this way before its last rounds.
template <typename Word, int NG>
__device__ __forceinline__ bool all_zero_after(bool (&zero)[NG], Word hs, const Word (&h)[NG], Word e) {
    if (!e) return false;  // nothing new (e is warp-uniform)
    bool dead = true;
#pragma unroll
    for (int g = 0; g < NG; g++) {
        zero[g] |= ((hs ^ h[g]) & e) != 0;
        dead &= zero[g];
    }
    return __all_sync(FULL, dead);
}

// Sums out alive variables while one is left in `until` (the summation rounds
// of the pair kernel).  A variable removed from `alive` keeps its bits of hs,
// h and L0 from then on (every later update is masked by alive), so the
// factors that depend only on its own bits are taken at the end: IE collects
// summed-out variables with even L (a factor 2·δ(hb = 0)), IO those with odd L
// (a factor √2·ω^{1-2hb}).  HIGH: pivots (and substituted variables) are the
// highest candidates instead of the lowest.
// Returns true when every observable's term became zero (the pair is done).
template <typename Word, int RPL, int NG, bool HIGH>
__device__ __forceinline__ bool sum_out(Word (&J)[RPL], Word& hs, Word& L0, Word& alive, Word& IE, Word& IO, int& r,
                                        Word (&h)[NG], int (&ph)[NG], bool (&zero)[NG], const Word (&own)[RPL],
                                        const Word until) {
    while (alive & until) {
        // the next variable, with even L if there is one (an even step removes
        // two variables, which leaves fewer steps in all)
        const Word cand = alive & until;
        const Word even = cand & ~L0;
        int jq;
        Word jb, S;
        if constexpr (HIGH && sizeof(Word) == 8) {  // candidates are in rows 32..63 only
            const uint32_t e32 = (uint32_t)((uint64_t)even >> 32), c32 = (uint32_t)((uint64_t)cand >> 32);
            const int q = 31 - __clz(e32 ? e32 : c32);
            jq = 32 + q;
            jb = (Word)(1u << q) << 32;
            S = shfl<Word>(J[RPL - 1], q) & alive & ~jb;
        } else {
            jq = HIGH ? fls0<Word>(even ? even : cand) : ffs0<Word>(even ? even : cand);
            jb = (Word)1 << jq;
            S = row_of<Word, RPL>(J, jq) & alive & ~jb;
        }
        if (!S) {
            // it is isolated (coupled to no other alive variable): all isolated
            // variables factor out together, found by one ballot.  An elimination
            // never touches an isolated variable (its row and column are zero
            // among the alive ones), so they can wait until a pivot is one of them.
            const Word iso = isolated<Word, RPL>(J, alive, own);
            IE |= iso & ~L0;
            IO |= iso & L0;
            alive &= ~iso;
            if (all_zero_after<Word, NG>(zero, hs, h, iso & ~L0)) return true;
            continue;
        }
        alive &= ~jb;
        if (L0 & jb) {  // 1 + i^{L_j}(-1)^{S·z} = √2·ω^{±1}·i^{∓S·z}
            IO |= jb;
#pragma unroll
            for (int g = 0; g < NG; g++)
                if ((hs ^ h[g]) & jb) h[g] ^= S;
            g_expand<Word, RPL>(J, hs, L0, S, own);
        } else {  // 1 + (-1)^{hb + S·z} = 2·δ(S·z = hb), S ≠ 0 here
            r -= 2;
            bool hb[NG];
            const bool hsj = (hs & jb) != 0;
#pragma unroll
            for (int g = 0; g < NG; g++) hb[g] = hsj ^ ((h[g] & jb) != 0);
            on_bit<Word, HIGH>(S, [&](auto slot, int q) {
                constexpr int H = decltype(slot)::value;
                g_subst<Word, RPL, NG, H>(q, S ^ ((Word)(1u << q) << (32 * H)), hb, J, hs, L0, alive, h, ph, own);
            });
        }
    }
    return false;
}

// MINB: blocks per SM the register allocation must allow (the register cap is
// 65536 / (128·MINB)); the launch picks it per workload (fewer blocks leave
// more registers for many observables per lane).
// Exact mode: one signed count per (observable, power of √2) in global
// memory (integer atomics, so the result does not depend on the schedule);
// a lane merges consecutive terms of one observable that fall in the same bin.
__device__ __forceinline__ void exact_flush(unsigned long long* bins, int& bin, int& cnt) {
    if (cnt) atomicAdd(bins + bin, (unsigned long long)(long long)cnt);
    cnt = 0;
}
__device__ __forceinline__ void exact_add(unsigned long long* bins, int& bin, int& cnt, int m, int v, int* status) {
    const int b = m + kExactMOffset;
    if (b < 0 || b >= kExactBins) {
        atomicOr(status, DS_RANGE);
        return;
    }
    if (b != bin) {
        exact_flush(bins, bin, cnt);
        bin = b;
    }
    cnt += v;
}

template <typename Word, int RPL, int NG, int MINB, bool EXACT>
__global__ void __launch_bounds__(PWARPS * 32, MINB) pair_kernel(MultiLaunch p) {
    constexpr int GMAX = (8 * sizeof(Word)) / 4;  // groups of four rows (8 or 16)
    // Unrolling of the table-lookup loops: full for 32-bit rows and for one
    // observable group; for 64-bit rows with more groups partial, less with
    // more observables per lane (code size and registers; from launch timings
    // at n = 40 and 60 and on the 512-circuit workload).  The lookups go two
    // groups at a time (ngrp is even), so each accumulator takes one
    // three-input XOR per 32-bit half for two table entries.
    constexpr int UNROLL_COMP = sizeof(Word) == 4 ? GMAX : (NG == 1 ? GMAX : (NG <= 2 ? 4 : 2));
    constexpr int UNROLL_BRA = sizeof(Word) == 4 ? GMAX : (NG <= 2 ? GMAX : 2);
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gwarp = blockIdx.x * PWARPS + wid;
    unsigned char* wbase = smem_raw + (size_t)wid * p.warp_smem;
    Word* tb0 = (Word*)wbase;
    Word* tb1 = (Word*)(wbase + p.tab_bytes_max);
    Word* tbA = (Word*)(wbase + 2 * p.tab_bytes_max);  // the bra's G table
    Word* sF = (Word*)(wbase + 2 * p.tab_bytes_max + p.bra_bytes_max);
    Word* sJ = sF + 64;
    uint64_t* bars = (uint64_t*)(sJ + 64);
    if (lane == 0) {
        mbar_init(&bars[0]);
        mbar_init(&bars[1]);
        fence_mbar_init();
    }
    __syncwarp();
    uint32_t par0 = 0, par1 = 0;  // next phase parity per buffer

    Word own[RPL];  // this lane's row bits
#pragma unroll
    for (int k = 0; k < RPL; k++) own[k] = (Word)1 << (32 * k + lane);

    // current descriptor
    int ds = -1;
    const PairDesc* d = nullptr;
    const unsigned char* ktab = nullptr;
    uint32_t tab_bytes = 0;
    int n = 0, ngrp = 0, nobs = 0;
    int64_t chiB = 0;
    bool tri = true, cplx = false;

    int64_t cur_i = -1;
    Word FV[RPL], MV[RPL];
    uint32_t gamV = 0;
    Word vA = 0;
    int kcA = 0, rcA = 0;
    Word xs[NG];
    int ks[NG];
    int buf = 0;
    bool timed_out = false;
    const uint32_t polls = p.poll_limit ? p.poll_limit : (1u << 22);

    // Work queue: the first task of every warp is its own index, the next
    // ones come from a global counter.  A task is a run of at most
    // task_chunks chunks inside one descriptor and owns one record (so the
    // sums do not depend on which warp ran which task).
    int64_t task = gwarp;
    while (task < p.total_tasks && !timed_out) {
        if (ds < 0 || task >= p.task_begin[ds + 1]) {  // enter the descriptor that owns the task
            int lo = ds < 0 ? 0 : ds, hi = p.num_descs;
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (p.task_begin[mid] <= task) lo = mid;
                else hi = mid;
            }
            ds = lo;
            d = p.descs + ds;
            ktab = (const unsigned char*)d->ktab;
            tab_bytes = d->ket_bytes;
            n = d->A.n;
            ngrp = d->ngrp;
            nobs = d->nobs;
            chiB = d->B.chi;
            tri = d->triangular != 0;
            cplx = d->complex_out != 0;
            cur_i = -1;
        }
        const int64_t tl = task - p.task_begin[ds];
        const int64_t c0 = tl * p.task_chunks, c1 = min(c0 + (int64_t)p.task_chunks, d->nchunks);
        double* rec = p.records + d->rec0 + tl * (int64_t)nobs * 8;  // this task's record
        for (int64_t lc = c0; lc < c1 && !timed_out; lc++) {
            // Ket-major order: chunk lc is bra i against the ket block kb (kets
            // kb·chunk .. +chunk), all bras of one block consecutive, so the warps
            // working at one time share a few blocks of ket tables in L2.
            int64_t i, j0, j1;
            if (tri) {  // block kb pairs with bras 0 .. min(kb·chunk + chunk, χ) - 1 (i ≤ j)
                int64_t lo = 0, hi = d->nblk;
                while (hi - lo > 1) {
                    int64_t mid = (lo + hi) >> 1;
                    if (d->blk_chunk_off[mid] <= lc) lo = mid;
                    else hi = mid;
                }
                i = lc - d->blk_chunk_off[lo];
                j0 = max(i, lo * (int64_t)p.chunk);
                j1 = min((lo + 1) * (int64_t)p.chunk, chiB);
            } else {  // every block pairs with all χ_A bras
                const int64_t kb = lc / d->A.chi;
                i = lc - kb * d->A.chi;
                j0 = kb * (int64_t)p.chunk;
                j1 = min(j0 + (int64_t)p.chunk, chiB);
            }
            if (i != cur_i) {  // a new bra: its frame rows, scalars, Pauli frames and G table
                cur_i = i;
                const FrameView& fr = d->fr;
#pragma unroll
                for (int k = 0; k < RPL; k++) {
                    size_t o = (size_t)i * 64 + 32 * k + lane;
                    FV[k] = (Word)fr.FV[o];
                    MV[k] = (Word)fr.MV[o];
                }
                const uint64_t gvl = fr.GVL[i], gvh = fr.GVH[i];
                gamV = 0;
#pragma unroll
                for (int k = 0; k < RPL; k++) {
                    const int r = 32 * k + lane;
                    gamV |= (uint32_t)(((gvl >> r) & 1) | (((gvh >> r) & 1) << 1)) << (2 * k);
                }
                const TermsView& A = d->A;
                vA = (Word)A.V[i * A.W];
                kcA = A.coef_k[i];
                rcA = A.coef_r[i];
#pragma unroll
                for (int g = 0; g < NG; g++) {
                    const int o = 32 * g + lane;
                    xs[g] = (o < nobs) ? (Word)d->px[(size_t)i * nobs + o] : (Word)0;
                    ks[g] = (o < nobs) ? d->pk[(size_t)i * nobs + o] : 0;
                }
                const Word* ga = (const Word*)((const unsigned char*)d->atab + (size_t)i * d->ktab_stride + tab_bytes);
                for (int e = lane; e < ngrp * 16; e += 32) tbA[e] = ga[e];
                __syncwarp();
            }
            constexpr int NA = (NG == 1) ? 4 : 2;
            ChunkAcc<NG, NA> acc;
            acc.reset();
            int ex_bin[EXACT ? NG : 1], ex_cnt[EXACT ? NG : 1];
            if constexpr (EXACT) {
#pragma unroll
                for (int g = 0; g < NG; g++) ex_bin[g] = ex_cnt[g] = 0;
            }

            // first ket of the chunk
            if (lane == 0) {
                fence_proxy_async();
                tma_load(buf ? tb1 : tb0, ktab + (size_t)j0 * d->ktab_stride, tab_bytes, buf ? &bars[1] : &bars[0],
                         p.dbg_extra_tx);
            }
            for (int64_t j = j0; j < j1; j++) {
                // prefetch the next ket's tables into the other buffer
                if (j + 1 < j1 && lane == 0) {
                    fence_proxy_async();
                    tma_load(buf ? tb0 : tb1, ktab + (size_t)(j + 1) * d->ktab_stride, tab_bytes,
                             buf ? &bars[0] : &bars[1]);
                }
                bool ok_wait;
                if (buf) {
                    ok_wait = mbar_wait(&bars[1], par1, polls);
                    par1 ^= 1;
                } else {
                    ok_wait = mbar_wait(&bars[0], par0, polls);
                    par0 ^= 1;
                }
                if (!ok_wait) {
                    // Record the timeout, then give the prefetch into the other
                    // buffer (if one was issued) a bounded wait before leaving.
                    if (lane == 0) atomicOr(d->status, DS_TIMEOUT);
                    if (j + 1 < j1) {
                        if (buf) mbar_wait(&bars[0], par0, 1u << 22);
                        else mbar_wait(&bars[1], par1, 1u << 22);
                    }
                    timed_out = true;
                    break;
                }
                const Word* T = buf ? tb1 : tb0;
                const KetTrailer& kt = *(const KetTrailer*)(T + 3 * ngrp * 16);  // the ket's scalars
                const Word glB = (Word)kt.gl, ghB = (Word)kt.gh, vB = (Word)kt.v, sB = (Word)kt.s;
                const int phB = kt.phase, kcB = kt.coef_k, rcB = kt.coef_r;

                // ---- D = V·U_B (Four Russians): F_D = F_V·F_B, y = F_V·P_B,
                //      K = M_D·F_Dᵀ = (F_V·K_B ⊕ M_V)·G_A  (G_B·F_Bᵀ = I, F_Vᵀ = G_A)
                Word fD[RPL], yP[RPL], Y[RPL], Kr[RPL];
#pragma unroll
                for (int k = 0; k < RPL; k++) {
                    fD[k] = yP[k] = Kr[k] = 0;
                    Y[k] = MV[k];
                }
#pragma unroll (UNROLL_COMP / 2 > 0 ? UNROLL_COMP / 2 : 1)
                for (int g = 0; g < GMAX; g += 2) {
                    if (g < ngrp) {
#pragma unroll
                        for (int k = 0; k < RPL; k++) {
                            const Word* e0 = T + (g * 16 + nib<Word, RPL>(FV[k], g)) * 3;
                            const Word* e1 = T + ((g + 1) * 16 + nib<Word, RPL>(FV[k], g + 1)) * 3;
                            fD[k] ^= e0[0] ^ e1[0];
                            yP[k] ^= e0[1] ^ e1[1];
                            Y[k] ^= e0[2] ^ e1[2];
                        }
                    }
                }
#pragma unroll (UNROLL_BRA / 2 > 0 ? UNROLL_BRA / 2 : 1)
                for (int g = 0; g < GMAX; g += 2) {
                    if (g < ngrp) {
#pragma unroll
                        for (int k = 0; k < RPL; k++) {
                            const int j0 = g * 16 + nib<Word, RPL>(Y[k], g);
                            const int j1 = (g + 1) * 16 + nib<Word, RPL>(Y[k], g + 1);
                            Kr[k] ^= tbA[j0] ^ tbA[j1];
                        }
                    }
                }
                // γ_D (eq. of the composed tableau) and the uniform bit planes
                Word g0 = 0, g1 = 0, diag = 0, fvs = 0, Lw[RPL];
                const Word w = vB & sB;
#pragma unroll
                for (int k = 0; k < RPL; k++) {
                    const int gsum = popc<Word>(FV[k] & glB) + 2 * popc<Word>(FV[k] & ghB);
                    const int gm = (int)((gamV >> (2 * k)) & 3) + gsum + 2 * parity<Word>(yP[k] & FV[k]);
                    g0 |= (Word)__ballot_sync(FULL, gm & 1) << (32 * k);
                    g1 |= (Word)__ballot_sync(FULL, gm & 2) << (32 * k);
                    diag |= (Word)__ballot_sync(FULL, own_bit<Word>(Kr[k], k, (uint32_t)own[0])) << (32 * k);
                    fvs |= (Word)__ballot_sync(FULL, parity<Word>(fD[k] & w)) << (32 * k);
                    Lw[k] = Kr[k] & (own[k] - 1);
                }
                // J: the symmetric coupling matrix, J[a][b] = K[max][min]
                Word J[RPL], LwT[RPL];
                transpose_lower(Lw, LwT, lane);
#pragma unroll
                for (int k = 0; k < RPL; k++) {
                    J[k] = Lw[k] | LwT[k];
                    sF[32 * k + lane] = fD[k];
                    sJ[32 * k + lane] = (J[k] & vA) | (Lw[k] & ~vA);
                }
                __syncwarp();

                const Word full = (n >= 8 * (int)sizeof(Word)) ? ~(Word)0 : (((Word)1 << n) - 1);
                const Word cons = ~vB & full;
                // ---- per-observable start: the fixed coordinates x' = x ∧ ¬v_A
                Word h[NG], rhs[NG];
                int ph[NG];
                bool zero[NG];
#pragma unroll
                for (int g = 0; g < NG; g++) {
                    const Word x = xs[g], xf = x & ~vA & full;
                    const int gx = popc<Word>(xf & g0) + 2 * popc<Word>(xf & g1);
                    Word xF = 0, Mx = 0, t = xf;
                    while (t) {
                        const int q = ffs0<Word>(t);
                        t &= t - 1;
                        xF ^= sF[q];
                        Mx ^= sJ[q];
                    }
                    ph[g] = phB + 2 * gx + 4 * parity<Word>(((Mx ^ diag) & xf) ^ (xF & w));
                    h[g] = (x ^ Mx) & vA;
                    rhs[g] = (sB ^ xF) & cons;
                    zero[g] = 32 * g + lane >= nobs;  // unused lanes count as zero
                }
                __syncwarp();  // sF/sJ are rewritten by the next ket

                // ---- the exponential sum over z ∈ span(v_A)
                Word hs = (g1 ^ diag ^ fvs) & vA, L0 = g0 & vA, alive = vA;
                int r = popc<Word>(vA) + popc<Word>(vB);
                Word Fc[RPL];
#pragma unroll
                for (int k = 0; k < RPL; k++) Fc[k] = fD[k] & cons;
                // constraints (z·F)_b = rhs_b for b ∉ v_B, by substitution
                Word crem = cons;
                while (crem) {
                    const Word bb = crem & (~crem + 1);  // the lowest remaining constraint column
                    crem ^= bb;
                    Word l = 0;
#pragma unroll
                    for (int k = 0; k < RPL; k++) l |= (Word)__ballot_sync(FULL, (Fc[k] & bb) != 0) << (32 * k);
                    l &= alive;
                    bool c[NG];
#pragma unroll
                    for (int g = 0; g < NG; g++) c[g] = (rhs[g] & bb) != 0;
                    if (l == 0) {  // a consistency condition
#pragma unroll
                        for (int g = 0; g < NG; g++) zero[g] |= c[g];
                        continue;
                    }
                    on_bit<Word, sizeof(Word) == 8>(l, [&](auto slot, int q) {
                        constexpr int H = decltype(slot)::value;
                        const Word lp = l ^ ((Word)(1u << q) << (32 * H));
                        const Word Fk = shfl<Word>(Fc[H], q);
#pragma unroll
                        for (int k = 0; k < RPL; k++)
                            if (own_bit<Word>(lp, k, (uint32_t)own[0])) Fc[k] ^= Fk;
#pragma unroll
                        for (int g = 0; g < NG; g++)
                            if (c[g]) rhs[g] ^= Fk;
                        g_subst<Word, RPL, NG, H>(q, lp, c, J, hs, L0, alive, h, ph, own);
                    });
                }
                // summation (sum_out); dead: every observable's term became zero
                // on the way (sum_out stops there).
                Word IE = 0, IO = 0;
                bool dead;
                if constexpr (sizeof(Word) == 8) {
                    // The variables of rows 32..63 first (highest first), then the
                    // rest on 32-bit words in one row slot: every update is masked by
                    // `alive`, so once no variable is left in the high half nothing
                    // above bit 31 changes again.
                    dead = sum_out<Word, RPL, NG, true>(J, hs, L0, alive, IE, IO, r, h, ph, zero, own,
                                                        ~(Word)0xffffffffu);
                    if (!dead) {
                        uint32_t J32[1] = {(uint32_t)J[0]};
                        const uint32_t own32[1] = {(uint32_t)own[0]};
                        uint32_t hs32 = (uint32_t)hs, L032 = (uint32_t)L0, alive32 = (uint32_t)alive, IE32 = 0,
                                 IO32 = 0;
                        uint32_t h32[NG];
#pragma unroll
                        for (int g = 0; g < NG; g++) h32[g] = (uint32_t)h[g];
                        dead = sum_out<uint32_t, 1, NG, false>(J32, hs32, L032, alive32, IE32, IO32, r, h32, ph, zero,
                                                               own32, ~0u);
                        const Word hi = ~(Word)0xffffffffu;
                        hs = (hs & hi) | hs32;
#pragma unroll
                        for (int g = 0; g < NG; g++) h[g] = (h[g] & hi) | h32[g];
                        IE |= IE32;
                        IO |= IO32;
                    }
                } else {
                    dead = sum_out<Word, RPL, NG, false>(J, hs, L0, alive, IE, IO, r, h, ph, zero, own, ~(Word)0);
                }
                if (!dead) {
                    r -= 2 * popc<Word>(IE) + popc<Word>(IO);
#pragma unroll
                    for (int g = 0; g < NG; g++) {
                        const Word hbits = hs ^ h[g];
                        zero[g] |= (hbits & IE) != 0;
                        ph[g] += popc<Word>(IO) - 2 * popc<Word>(hbits & IO);
                    }
                }

                const int kpair = (kcB - kcA) & 7;
                const int rpair = rcA + rcB + r;
                const int wgt = (tri && j != i) ? 2 : 1;
#pragma unroll
                for (int g = 0; g < NG; g++) {
                    const int o = 32 * g + lane;
                    if (p.dbg_k && o == 0) {
                        const size_t di = (size_t)i * chiB + j;
                        p.dbg_k[di] = zero[g] ? (uint8_t)255 : (uint8_t)((ks[g] + ph[g]) & 7);
                        p.dbg_r[di] = r;
                    }
                    if (!zero[g] && o < nobs) {
                        const int k = (kpair + ks[g] + ph[g]) & 7;
                        int sgn, m;
                        re_part(k, rpair, sgn, m);
                        if constexpr (EXACT) {
                            unsigned long long* bins = d->counts + (size_t)o * 2 * kExactBins;
                            if (sgn) exact_add(bins, ex_bin[g], ex_cnt[g], m, sgn * wgt, d->status);
                            if (cplx) {
                                im_part(k, rpair, sgn, m);
                                const int b = m + kExactMOffset;
                                if (sgn && b >= 0 && b < kExactBins)
                                    atomicAdd(bins + kExactBins + b, (unsigned long long)(long long)(sgn * wgt));
                                else if (sgn)
                                    atomicOr(d->status, DS_RANGE);
                            }
                        } else {
                            double* pp = rec + (size_t)o * 8;
                            if (sgn) acc.add(g, m & 1, sgn * wgt, (m & 1) ? ((m - 1) >> 1) : (m >> 1), p.mixed, pp);
                            if (NA == 4 && cplx) {
                                im_part(k, rpair, sgn, m);
                                if (sgn)
                                    acc.add(g, (NA == 4 ? 2 : 0) + (m & 1), sgn * wgt,
                                            (m & 1) ? ((m - 1) >> 1) : (m >> 1), p.mixed, pp);
                            }
                        }
                    }
                }
                __syncwarp();  // all lanes done with buffer `buf`
                buf ^= 1;
            }
            // ---- fold the chunk into the task's double-double record
#pragma unroll
            for (int g = 0; g < NG; g++) {
                const int o = 32 * g + lane;
                if constexpr (EXACT) {
                    if (o < nobs) exact_flush(d->counts + (size_t)o * 2 * kExactBins, ex_bin[g], ex_cnt[g]);
                } else {
                    if (o < nobs) acc.flush_group(g, rec + (size_t)o * 8, p.mixed);
                }
            }
        }
        unsigned long long next = 0;
        if (lane == 0) next = atomicAdd(p.counter, 1ULL);
        task = (int64_t)shfl<unsigned long long>(next, 0) + p.nwarps;
    }
}

// Reduction of the per-task records in two fixed-order passes (deterministic):
// block (observable, split) folds its slice of the unit's task records into a
// double-double partial, then one block per observable folds the partials in
// split order and applies the unit's scale.
__device__ __forceinline__ int unit_of(const int64_t* __restrict__ begin, int num, int64_t x) {
    int lo = 0, hi = num;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (begin[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Double-double tree over the block's 256 threads (8 lanes: 4 classes × (hi, lo)).
__device__ __forceinline__ void block_fold(double (&acc)[8], double (&sh)[8][256]) {
#pragma unroll
    for (int t = 0; t < 8; t++) sh[t][threadIdx.x] = acc[t];
    __syncthreads();
    for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride) {
#pragma unroll
            for (int t = 0; t < 4; t++) {
                double s, e;
                two_sum_d(sh[2 * t][threadIdx.x], sh[2 * t][threadIdx.x + stride], s, e);
                sh[2 * t][threadIdx.x] = s;
                sh[2 * t + 1][threadIdx.x] += e + sh[2 * t + 1][threadIdx.x + stride];
            }
        }
        __syncthreads();
    }
}

__device__ __forceinline__ void dd_add8(double (&acc)[8], const double* __restrict__ pp) {
#pragma unroll
    for (int t = 0; t < 4; t++) {
        double s, e;
        two_sum_d(acc[2 * t], pp[2 * t], s, e);
        acc[2 * t] = s;
        acc[2 * t + 1] += e + pp[2 * t + 1];
    }
}

__global__ void __launch_bounds__(256) reduce_tasks_kernel(MultiLaunch p, const int64_t* __restrict__ obs_begin,
                                                           int nsplit, double* __restrict__ part) {
    __shared__ double sh[8][256];
    const int64_t ob = blockIdx.x;
    const int split = blockIdx.y;
    const int ds = unit_of(obs_begin, p.num_descs, ob);
    const PairDesc* d = p.descs + ds;
    const int o = (int)(ob - obs_begin[ds]);
    const int64_t ntasks = p.task_begin[ds + 1] - p.task_begin[ds];
    const int64_t per = (ntasks + nsplit - 1) / nsplit;
    const int64_t t0 = (int64_t)split * per, t1 = min(t0 + per, ntasks);
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t tl = t0 + threadIdx.x; tl < t1; tl += blockDim.x)
        dd_add8(acc, p.records + d->rec0 + (tl * d->nobs + o) * 8);
    block_fold(acc, sh);
    if (threadIdx.x < 8) part[((size_t)ob * nsplit + split) * 8 + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(32) reduce_final_kernel(MultiLaunch p, const int64_t* __restrict__ obs_begin,
                                                          int nsplit, const double* __restrict__ part,
                                                          double* __restrict__ out) {
    const int64_t ob = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (ob >= obs_begin[p.num_descs]) return;
    const PairDesc* d = p.descs + unit_of(obs_begin, p.num_descs, ob);
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int sp = 0; sp < nsplit; sp++) dd_add8(acc, part + ((size_t)ob * nsplit + sp) * 8);
    const double r2 = 0.70710678118654752440;
    const double re = (acc[0] + acc[1]) + (acc[2] + acc[3]) * r2;
    const double im = (acc[4] + acc[5]) + (acc[6] + acc[7]) * r2;
    out[2 * ob] = re * d->scale_re - im * d->scale_im;
    out[2 * ob + 1] = re * d->scale_im + im * d->scale_re;
}

// Row-staged variant of the pair kernel (no term tables): B's rows are
// staged in shared memory and composed bit by bit.  It needs no per-term
// table storage, which is what nsg_exp_value_noalloc's fixed scratch
// affords; one observable per lane group.
template <typename Word, int RPL, int NG>
__global__ void __launch_bounds__(PWARPS * 32) pair_kernel_rows(PairLaunch p) {
    using Eng = dev::WarpCH<Word, 1, RPL>;
    __shared__ Word sGs[PWARPS][64], sFs[PWARPS][64], sMs[PWARPS][64];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gwarp = blockIdx.x * PWARPS + wid;
    Word* sG = sGs[wid];
    Word* sF = sFs[wid];
    Word* sM = sMs[wid];
    const TermsView& A = p.A;
    const TermsView& Bt = p.B;
    const int n = A.n;
    const int64_t chiA = A.chi, chiB = Bt.chi;
    const int nobs = p.nobs;

    // per-row (A) state
    int64_t cur_i = -1;
    Word GV[RPL], FV[RPL], MV[RPL];
    uint32_t gamV = 0;
    Word vA = 0, sA = 0;
    int kcA = 0, rcA = 0;
    Word xs[NG];
    int ks[NG];

    const int64_t cpr = p.triangular ? 0 : (chiB + p.chunk - 1) / p.chunk;

    for (int64_t c = gwarp; c < p.total_chunks; c += p.nwarps) {
        int64_t i, j0, j1;
        if (p.triangular) {
            int64_t lo = 0, hi = chiA;  // find i: off[i] <= c < off[i+1]
            while (hi - lo > 1) {
                int64_t mid = (lo + hi) >> 1;
                if (p.row_chunk_off[mid] <= c) lo = mid;
                else hi = mid;
            }
            i = lo;
            j0 = i + (c - p.row_chunk_off[i]) * p.chunk;
            j1 = min(j0 + (int64_t)p.chunk, chiB);
        } else {
            i = c / cpr;
            j0 = (c % cpr) * p.chunk;
            j1 = min(j0 + (int64_t)p.chunk, chiB);
        }
        if (i != cur_i) {
            cur_i = i;
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                size_t o = (size_t)i * 64 + 32 * k + lane;
                GV[k] = lowbits<Word>(p.fr.GV[o]);
                FV[k] = lowbits<Word>(p.fr.FV[o]);
                MV[k] = lowbits<Word>(p.fr.MV[o]);
            }
            uint64_t gvl = p.fr.GVL[i], gvh = p.fr.GVH[i];
            gamV = 0;
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                int r = 32 * k + lane;
                int g = (int)((gvl >> r) & 1) | ((int)((gvh >> r) & 1) << 1);
                gamV |= (uint32_t)g << (2 * k);
            }
            vA = lowbits<Word>(A.V[i * A.W]);
            sA = lowbits<Word>(A.S[i * A.W]);
            kcA = A.coef_k[i];
            rcA = A.coef_r[i];
#pragma unroll
            for (int g = 0; g < NG; g++) {
                int o = 32 * g + lane;
                xs[g] = (o < nobs) ? lowbits<Word>(p.px[(size_t)i * nobs + o]) : 0;
                ks[g] = (o < nobs) ? p.pk[(size_t)i * nobs + o] : 0;
            }
        }
        constexpr int NA = (NG == 1) ? 4 : 2;
        ChunkAcc<NG, NA> acc;
        acc.reset();

        for (int64_t j = j0; j < j1; j++) {
            // ---- stage B's rows
            __syncwarp();
            for (int r = lane; r < 64; r += 32) {
                size_t idx = ((size_t)j * Bt.R + r) * Bt.W;  // word 0 (n ≤ 64)
                sG[r] = lowbits<Word>(Bt.G[idx]);
                sF[r] = lowbits<Word>(Bt.F[idx]);
                sM[r] = lowbits<Word>(Bt.M[idx]);
            }
            const Word glB = lowbits<Word>(Bt.GL[j * Bt.W]), ghB = lowbits<Word>(Bt.GH[j * Bt.W]);
            __syncwarp();

            // ---- D = V·U_B: G_D = G_V G_B, F_D = F_V F_B, M_D = F_V M_B ⊕ M_V G_B,
            //      γ_D = γ_V + Σ_{q∈F_V} γ_B,q + 2·Σ_{q<r∈F_V} M_B,q·F_B,r.
            Word gD[RPL], fD[RPL], mf[RPL], mg[RPL];
            int cnt[RPL];
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                gD[k] = fD[k] = mf[k] = mg[k] = 0;
                cnt[k] = 0;
            }
            for (int q = 0; q < n; q++) {
                const Word gb = sG[q], fb = sF[q], mb = sM[q];
#pragma unroll
                for (int k = 0; k < RPL; k++) {
                    const Word sg = (Word)0 - ((GV[k] >> q) & 1);
                    const Word sf = (Word)0 - ((FV[k] >> q) & 1);
                    const Word sm = (Word)0 - ((MV[k] >> q) & 1);
                    gD[k] ^= gb & sg;
                    cnt[k] += popc<Word>(mf[k] & fb & sf);
                    fD[k] ^= fb & sf;
                    mf[k] ^= mb & sf;
                    mg[k] ^= gb & sm;
                }
            }
            Eng e;
            e.lane = lane;
            e.n = n;
            e.err = 0;
            e.gam = 0;
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                e.G[k].w[0] = gD[k];
                e.F[k].w[0] = fD[k];
                e.M[k].w[0] = mf[k] ^ mg[k];
                int gsum = popc<Word>(FV[k] & glB) + 2 * popc<Word>(FV[k] & ghB);
                int g = (int)((gamV >> (2 * k)) & 3) + gsum + 2 * (cnt[k] & 1);
                e.gam |= (uint32_t)(g & 3) << (2 * k);
            }
            e.v.w[0] = lowbits<Word>(Bt.V[j * Bt.W]);
            e.s.w[0] = lowbits<Word>(Bt.S[j * Bt.W]);
            e.phase = Bt.phase[j];

            // ---- U_{H,A}: H on every qubit of v_A (form/left_multiplication/h.rs)
            Word hv = vA;
            while (hv) {
                int q = dev::ffs0<Word>(hv);
                hv &= hv - 1;
                e.left_h(q);
            }
            if (e.err && lane == 0) atomicOr(p.status, DS_INVARIANT);

            // ---- stage the transformed ket's F, M rows; γ planes by ballot
            __syncwarp();
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                int r = 32 * k + lane;
                if (r < 64) {
                    sF[r] = e.F[k].w[0];
                    sM[r] = e.M[k].w[0];
                }
            }
            Word gl2 = 0, gh2 = 0;
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                int g = e.gam_of(k);
                uint32_t b0 = __ballot_sync(FULL, g & 1), b1 = __ballot_sync(FULL, (g >> 1) & 1);
                gl2 |= (Word)b0 << (32 * k);
                gh2 |= (Word)b1 << (32 * k);
            }
            __syncwarp();
            const Word vv = e.v.w[0], ss = e.s.w[0];
            const int rv = popc<Word>(vv);

            // ---- amplitudes ⟨x|ket⟩ for this lane's observables
            Word u[NG], mac[NG];
            int c2[NG];
#pragma unroll
            for (int g = 0; g < NG; g++) {
                u[g] = mac[g] = 0;
                c2[g] = 0;
            }
            for (int q = 0; q < n; q++) {
                const Word f = sF[q], m = sM[q];
#pragma unroll
                for (int g = 0; g < NG; g++) {
                    const Word sel = (Word)0 - ((xs[g] >> q) & 1);
                    c2[g] += popc<Word>(mac[g] & f & sel);
                    mac[g] ^= m & sel;
                    u[g] ^= f & sel;
                }
            }
            const int kpair = (Bt.coef_k[j] - kcA) & 7;
            const int rpair = rcA + Bt.coef_r[j] + rv;
            const int wgt = (p.triangular && j != i) ? 2 : 1;
#pragma unroll
            for (int g = 0; g < NG; g++) {
                const int o = 32 * g + lane;
                const bool ok = (((u[g] ^ ss) & ~vv) == 0);
                const int gsum = popc<Word>(xs[g] & gl2) + 2 * popc<Word>(xs[g] & gh2);
                const int sg = c2[g] + popc<Word>(u[g] & mac[g]) + popc<Word>(u[g] & vv & ss);
                const int kamp = (e.phase + 2 * gsum + 4 * (sg & 1)) & 7;
                if (p.dbg_k && o == 0) {
                    size_t di = (size_t)i * chiB + j;
                    p.dbg_k[di] = ok ? (uint8_t)((ks[g] + kamp) & 7) : (uint8_t)255;
                    p.dbg_r[di] = rv;
                }
                if (ok && o < nobs) {
                    double* pp = p.partials + ((size_t)gwarp * nobs + o) * 8;
                    const int k = (kpair + ks[g] + kamp) & 7;
                    int sgn, m;
                    re_part(k, rpair, sgn, m);
                    if (sgn) acc.add(g, m & 1, sgn * wgt, (m & 1) ? ((m - 1) >> 1) : (m >> 1), p.mixed, pp);
                    if (NA == 4 && p.complex_out) {
                        im_part(k, rpair, sgn, m);
                        if (sgn)
                            acc.add(g, (NA == 4 ? 2 : 0) + (m & 1), sgn * wgt, (m & 1) ? ((m - 1) >> 1) : (m >> 1),
                                    p.mixed, pp);
                    }
                }
            }
        }
        // ---- flush the chunk into this warp's double-double partials
#pragma unroll
        for (int g = 0; g < NG; g++) {
            const int o = 32 * g + lane;
            if (o < nobs) acc.flush_group(g, p.partials + ((size_t)gwarp * nobs + o) * 8, p.mixed);
        }
    }
}

// One block per observable; fixed-order double-double tree.
__global__ void reduce_kernel(const double* __restrict__ partials, int nwarps, int nobs, int complex_out,
                              double sre, double sim, double* __restrict__ out) {
    __shared__ double sh[8][256];
    const int o = blockIdx.x;
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int w = threadIdx.x; w < nwarps; w += blockDim.x) {
        const double* pp = partials + ((size_t)w * nobs + o) * 8;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            double s, e;
            two_sum_d(acc[2 * t], pp[2 * t], s, e);
            acc[2 * t] = s;
            acc[2 * t + 1] += e + pp[2 * t + 1];
        }
    }
#pragma unroll
    for (int t = 0; t < 8; t++) sh[t][threadIdx.x] = acc[t];
    __syncthreads();
    for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
        if (threadIdx.x < stride) {
#pragma unroll
            for (int t = 0; t < 4; t++) {
                double s, e;
                two_sum_d(sh[2 * t][threadIdx.x], sh[2 * t][threadIdx.x + stride], s, e);
                sh[2 * t][threadIdx.x] = s;
                sh[2 * t + 1][threadIdx.x] += e + sh[2 * t + 1][threadIdx.x + stride];
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double r2 = 0.70710678118654752440;
        double X = sh[0][0] + sh[1][0], Y = sh[2][0] + sh[3][0];
        double Xi = sh[4][0] + sh[5][0], Yi = sh[6][0] + sh[7][0];
        double re = X + Y * r2, im = Xi + Yi * r2;
        if (complex_out) {
            out[2 * o] = re * sre - im * sim;
            out[2 * o + 1] = re * sim + im * sre;
        } else {
            out[o] = re * sre;
        }
    }
}

// Dynamic shared memory above 48 KB needs an opt-in per kernel (and device);
// it is set outside stream capture (the first launch of a shape is never a
// captured one: plans run once before they capture).
template <typename Word, int RPL, int NG, int MINB, bool EXACT = false>
cudaError_t allow_smem(size_t smem, cudaStream_t st) {
    if (smem <= 48 * 1024) return cudaSuccess;
    if (st) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) return cudaSuccess;
    }
    return cudaFuncSetAttribute(pair_kernel<Word, RPL, NG, MINB, EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem);
}

template <typename Word, int RPL, int NG, int MINB, bool EXACT = false>
cudaError_t launch_pairs_ng(const MultiLaunch& p, cudaStream_t st) {
    const size_t smem = (size_t)p.warp_smem * PWARPS;
    cudaError_t e = allow_smem<Word, RPL, NG, MINB, EXACT>(smem, st);
    if (e != cudaSuccess) return e;
    pair_kernel<Word, RPL, NG, MINB, EXACT><<<p.blocks, PWARPS * 32, smem, st>>>(p);
    return cudaGetLastError();
}

// The exact-count mode has one variant per row width and observable groups
// (the largest register budget, two blocks per SM).
template <typename Word, int RPL, int NG>
cudaError_t launch_pairs_minb(const MultiLaunch& p, cudaStream_t st) {
    if (p.exact) return launch_pairs_ng<Word, RPL, NG, 2, true>(p, st);
    switch (p.minb) {
        case 2: return launch_pairs_ng<Word, RPL, NG, 2>(p, st);
        case 3: return launch_pairs_ng<Word, RPL, NG, 3>(p, st);
        case 5: return launch_pairs_ng<Word, RPL, NG, 5>(p, st);
        case 6:  // 32-bit rows only (the host caps 64-bit rows at five)
            if constexpr (sizeof(Word) == 4) return launch_pairs_ng<Word, RPL, NG, 6>(p, st);
            else return launch_pairs_ng<Word, RPL, NG, 5>(p, st);
        default: return launch_pairs_ng<Word, RPL, NG, 4>(p, st);
    }
}

template <typename Word, int RPL, int NG, int MINB, bool EXACT = false>
int resident_blocks_ng(size_t warp_smem) {
    int nb = 0;
    if (allow_smem<Word, RPL, NG, MINB, EXACT>(warp_smem * PWARPS, nullptr) != cudaSuccess) return 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, pair_kernel<Word, RPL, NG, MINB, EXACT>, PWARPS * 32,
                                                      warp_smem * PWARPS) != cudaSuccess)
        return 1;
    return nb > 0 ? nb : 1;
}

template <typename Word, int RPL, int NG>
int resident_blocks_minb(size_t warp_smem, int minb) {
    if (minb == 0) return resident_blocks_ng<Word, RPL, NG, 2, true>(warp_smem);  // exact mode
    switch (minb) {
        case 2: return resident_blocks_ng<Word, RPL, NG, 2>(warp_smem);
        case 3: return resident_blocks_ng<Word, RPL, NG, 3>(warp_smem);
        case 5: return resident_blocks_ng<Word, RPL, NG, 5>(warp_smem);
        case 6:
            if constexpr (sizeof(Word) == 4) return resident_blocks_ng<Word, RPL, NG, 6>(warp_smem);
            else return resident_blocks_ng<Word, RPL, NG, 5>(warp_smem);
        default: return resident_blocks_ng<Word, RPL, NG, 4>(warp_smem);
    }
}

template <typename Word, int RPL>
int resident_blocks_w(int nobs_max, size_t warp_smem, int minb) {
    const int ng = (nobs_max + 31) / 32;
    if (ng <= 1) return resident_blocks_minb<Word, RPL, 1>(warp_smem, minb);
    if (ng <= 2) return resident_blocks_minb<Word, RPL, 2>(warp_smem, minb);
    if (ng <= 4) return resident_blocks_minb<Word, RPL, 4>(warp_smem, minb);
    return resident_blocks_minb<Word, RPL, 8>(warp_smem, minb);
}

template <typename Word, int RPL>
cudaError_t launch_pairs_w(const MultiLaunch& p, cudaStream_t st) {
    const int ng = (p.nobs_max + 31) / 32;
    if (ng <= 1) return launch_pairs_minb<Word, RPL, 1>(p, st);
    if (ng <= 2) return launch_pairs_minb<Word, RPL, 2>(p, st);
    if (ng <= 4) return launch_pairs_minb<Word, RPL, 4>(p, st);
    if (ng <= 8) return launch_pairs_minb<Word, RPL, 8>(p, st);
    return cudaErrorInvalidValue;
}

// Eight independent 32-bit logic chains per thread; every step is one
// three-input logic op (lop3.b32, truth table 0x78 = a ^ (b & c)) per chain,
// issued as volatile inline PTX so no step is folded away; the loop index
// enters once per 128 ops so iterations cannot be collapsed, and every
// thread stores its result.
__device__ __forceinline__ uint32_t lop3_78(uint32_t a, uint32_t b, uint32_t c) {
    uint32_t d;
    asm volatile("lop3.b32 %0, %1, %2, %3, 0x78;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
    return d;
}

__global__ void int_probe_kernel(uint64_t iters, uint32_t* sink) {
    uint32_t a0 = threadIdx.x, a1 = a0 * 3u + 1u, a2 = a0 * 5u + 7u, a3 = a0 * 7u + 3u;
    uint32_t a4 = a0 ^ 0x9e3779b9u, a5 = a1 ^ 0x7f4a7c15u, a6 = a2 ^ 0x85ebca6bu, a7 = a3 ^ 0xc2b2ae35u;
    const uint32_t k = blockIdx.x | 0x1234u;
    for (uint64_t i = 0; i < iters; i++) {
        a0 ^= (uint32_t)i;
#pragma unroll
        for (int u = 0; u < 16; u++) {  // 8 independent ops per round, rounds chained
            uint32_t b0 = lop3_78(a0, a1, a2), b1 = lop3_78(a1, a2, a3), b2 = lop3_78(a2, a3, a4);
            uint32_t b3 = lop3_78(a3, a4, a5), b4 = lop3_78(a4, a5, a6), b5 = lop3_78(a5, a6, a7);
            uint32_t b6 = lop3_78(a6, a7, a0), b7 = lop3_78(a7, a0, k);
            a0 = b0; a1 = b1; a2 = b2; a3 = b3; a4 = b4; a5 = b5; a6 = b6; a7 = b7;
        }
    }
    sink[blockIdx.x * blockDim.x + threadIdx.x] = a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7;
}

}  // namespace

cudaError_t launch_int_probe(uint64_t iters, int blocks, int threads, uint32_t* sink, cudaStream_t st) {
    int_probe_kernel<<<blocks, threads, 0, st>>>(iters, sink);
    return cudaGetLastError();
}

cudaError_t launch_frames(const TermsView& t, FrameView fr, cudaStream_t st) {
    if (t.chi == 0) return cudaSuccess;
    frames_kernel<<<(unsigned)((t.chi + FWARPS - 1) / FWARPS), FWARPS * 32, 0, st>>>(t, fr);
    return cudaGetLastError();
}

cudaError_t launch_pauli_frames(const TermsView& t, const DevPauli* d_paulis, int nobs, uint64_t* x_out,
                                uint8_t* k_out, cudaStream_t st) {
    if (t.chi == 0 || nobs == 0) return cudaSuccess;
    pauli_frames_kernel<<<(unsigned)((t.chi + FWARPS - 1) / FWARPS), FWARPS * 32, 0, st>>>(t, d_paulis, nobs, x_out,
                                                                                          k_out);
    return cudaGetLastError();
}

static int pair_word_bytes(int n) { return n <= 32 ? 4 : 8; }

size_t ket_table_stride(int n) {  // bytes per term: [ngrp][16][F, P, K] words, trailer, [G][ngrp][16] words
    return (size_t)4 * ket_table_groups(n) * 16 * pair_word_bytes(n) + sizeof(KetTrailer);
}

size_t ket_table_ket_bytes(int n) { return (size_t)3 * ket_table_groups(n) * 16 * pair_word_bytes(n) + sizeof(KetTrailer); }

size_t ket_table_bra_bytes(int n) { return (size_t)ket_table_groups(n) * 16 * pair_word_bytes(n); }

int ket_table_groups(int n) { return n <= 0 ? 2 : ((n + 3) / 4 + 1) & ~1; }

cudaError_t launch_ket_tables(const TermsView& t, void* out, cudaStream_t st) {
    if (t.chi == 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((t.chi + FWARPS - 1) / FWARPS);
    if (t.n <= 32)
        ket_tables_kernel<uint32_t><<<blocks, FWARPS * 32, 0, st>>>(t, ket_table_groups(t.n), ket_table_stride(t.n),
                                                                    (unsigned char*)out);
    else
        ket_tables_kernel<uint64_t><<<blocks, FWARPS * 32, 0, st>>>(t, ket_table_groups(t.n), ket_table_stride(t.n),
                                                                    (unsigned char*)out);
    return cudaGetLastError();
}

cudaError_t launch_pairs_rows(const PairLaunch& p, cudaStream_t st) {
    if (p.total_chunks == 0) return cudaSuccess;
    if (p.nobs > 32) return cudaErrorInvalidValue;
    if (p.A.n <= 32) pair_kernel_rows<uint32_t, 1, 1><<<p.blocks, PWARPS * 32, 0, st>>>(p);
    else pair_kernel_rows<uint64_t, 2, 1><<<p.blocks, PWARPS * 32, 0, st>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_pairs_multi(const MultiLaunch& m, int word_bytes, cudaStream_t st) {
    if (m.total_tasks == 0) return cudaSuccess;
    if (word_bytes == 4) return launch_pairs_w<uint32_t, 1>(m, st);
    return launch_pairs_w<uint64_t, 2>(m, st);
}

int pair_resident_warps(int word_bytes, int nobs_max, size_t warp_smem, int minb) {
    // The occupancy query per launch shape, remembered (it costs a driver round trip).
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, size_t, int>, int> cache;
    int dev = 0;
    cudaGetDevice(&dev);
    const auto key = std::make_tuple(dev, word_bytes, (nobs_max + 31) / 32, warp_smem, minb);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    const int nb = word_bytes == 4 ? resident_blocks_w<uint32_t, 1>(nobs_max, warp_smem, minb)
                                   : resident_blocks_w<uint64_t, 2>(nobs_max, warp_smem, minb);
    const int w = nb * PWARPS * device_sm_count();
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = w;
    return w;
}

int reduce_splits(int64_t total_obs) {
    const int64_t want = 2 * (int64_t)device_sm_count();  // blocks to keep every SM busy
    const int64_t s = (want + total_obs - 1) / std::max<int64_t>(total_obs, 1);
    return (int)std::min<int64_t>(std::max<int64_t>(s, 1), 32);
}

cudaError_t launch_reduce_multi(const MultiLaunch& m, const int64_t* obs_begin, int64_t total_obs, double* out,
                                double* scratch, cudaStream_t st) {
    if (total_obs == 0) return cudaSuccess;
    const int nsplit = reduce_splits(total_obs);
    reduce_tasks_kernel<<<dim3((unsigned)total_obs, (unsigned)nsplit), 256, 0, st>>>(m, obs_begin, nsplit, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce_final_kernel<<<(unsigned)((total_obs + 31) / 32), 32, 0, st>>>(m, obs_begin, nsplit, scratch, out);
    return cudaGetLastError();
}

size_t pair_warp_smem_bytes(size_t ket_bytes_max, size_t bra_bytes_max, int word_bytes) {
    size_t b = 2 * ket_bytes_max + bra_bytes_max + 2 * 64 * (size_t)word_bytes + 2 * sizeof(uint64_t);
    return (b + 127) & ~(size_t)127;
}

cudaError_t launch_reduce(const double* partials, int nwarps, int nobs, bool complex_out, double scale_re,
                          double scale_im, double* out, cudaStream_t st) {
    if (nobs == 0) return cudaSuccess;
    reduce_kernel<<<nobs, 256, 0, st>>>(partials, nwarps, nobs, complex_out ? 1 : 0, scale_re, scale_im, out);
    return cudaGetLastError();
}

}  // namespace nsg
