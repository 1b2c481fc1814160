// kernels_pairs.cu — the χ² pair sums behind exp_value, norm and
// inner_product (crates/necstar/src/state/stabilizer_decomposed_state/
// {exp_value,norm,inner_product}.rs).
//
// Every pair value ⟨A|P|B⟩ between two CH-form terms is an exact
// e^{iπk/4}·2^{-r/2} (or 0) — a canonical number, so any exact method gives
// the reference's (k, r).  The reference computes it by Gauss-eliminating A
// to |0^n⟩ (a recorded list of O(n²) gates, form/inner_product.rs:52-123)
// and replaying that list on a clone of B.  Here the same quantity is
// evaluated in A's frame with per-term precomputation:
//
//   |A⟩ = φ_A U_A U_{H,A}|s_A⟩,  V = U_A^{-1} (tableau precomputed per A)
//   ⟨A|P|B⟩ = conj(φ_A)·μ_{A,P}·⟨x_{A,P}| U_{H,A}·(V·U_B)·U_{H,B}|s_B⟩·φ_B
//
// with (x_{A,P}, μ_{A,P}) the Pauli seen from A's frame (precomputed per
// (A, P)), V·U_B a product of two control-type Cliffords (one GF(2) matrix
// pass), U_{H,A} applied with the reference's left_multiply_h rule, and the
// final computational-basis amplitude in closed form (arXiv:1808.00128
// eqs. 48-55).  One warp evaluates one pair with the tableau rows spread
// over its lanes; the 32 lanes then evaluate up to 32 observables each
// against the same transformed ket, so a batch of observables shares all of
// the per-pair GF(2) work.
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "device_state.hpp"
#include "warp_chform.cuh"

namespace nsg {
namespace {

using dev::FULL;
using dev::popc;
using dev::WarpCH;

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

template <typename Word, int RPL, int NG>
__global__ void __launch_bounds__(PWARPS * 32) pair_kernel(PairLaunch p) {
    using Eng = WarpCH<Word, 1, RPL>;
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

template <typename Word, int RPL>
cudaError_t launch_pairs_w(const PairLaunch& p, cudaStream_t st) {
    int ng = (p.nobs + 31) / 32;
    dim3 grid(p.blocks), block(PWARPS * 32);
    if (ng <= 1) pair_kernel<Word, RPL, 1><<<grid, block, 0, st>>>(p);
    else if (ng <= 2) pair_kernel<Word, RPL, 2><<<grid, block, 0, st>>>(p);
    else if (ng <= 4) pair_kernel<Word, RPL, 4><<<grid, block, 0, st>>>(p);
    else if (ng <= 8) pair_kernel<Word, RPL, 8><<<grid, block, 0, st>>>(p);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
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

cudaError_t launch_pairs(const PairLaunch& p, cudaStream_t st) {
    if (p.total_chunks == 0) return cudaSuccess;
    if (p.A.n <= 32) return launch_pairs_w<uint32_t, 1>(p, st);
    return launch_pairs_w<uint64_t, 2>(p, st);
}

cudaError_t launch_reduce(const double* partials, int nwarps, int nobs, bool complex_out, double scale_re,
                          double scale_im, double* out, cudaStream_t st) {
    if (nobs == 0) return cudaSuccess;
    reduce_kernel<<<nobs, 256, 0, st>>>(partials, nwarps, nobs, complex_out ? 1 : 0, scale_re, scale_im, out);
    return cudaGetLastError();
}

}  // namespace nsg
