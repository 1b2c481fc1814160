// kernels_terms.cu — per-term kernels: compile (kron + Clifford run +
// post-selection + discard), stable compaction, gate application, projection,
// discard, pack/unpack and the dense statevector.
//
// One warp owns one term (warp_chform.cuh); a block of 4 warps stages the
// shared primitive-op list through shared memory so all warps of the block
// read each op from one broadcast load.
#include <cuda_runtime.h>

#include "device_state.hpp"
#include "warp_chform.cuh"

namespace nsg {
namespace {

using dev::BV;
using dev::WarpCH;

constexpr int WARPS = 4;
constexpr int OPS_CHUNK = 2048;
constexpr int kCompileWarps = 4;  // warps per block of the compile kernel

// A warp-held term with W 64-bit words per row in RPL row slots of 32 rows
// (RPL = 2W holds every row of the storage; the compile kernel uses RPL = 3
// for widths 65-96).
template <int W, int RPL = 2 * W, typename Word = uint64_t>
using Eng = WarpCH<Word, W, RPL>;

// ---- load / store a term between HBM (any storage W) and a warp engine -----
template <int W, int RPL = 2 * W>
__device__ __forceinline__ void load_term(Eng<W, RPL>& e, const TermsView& tv, int64_t term) {
    e.n = tv.n;
    e.err = 0;
    e.phase = tv.phase[term];
    e.gam = 0;
#pragma unroll
    for (int k = 0; k < RPL; k++) {
        int r = 32 * k + e.lane;
#pragma unroll
        for (int w = 0; w < W; w++) {
            uint64_t g = 0, f = 0, m = 0;
            if (r < tv.R && w < tv.W) {
                size_t idx = ((size_t)term * tv.R + r) * tv.W + w;
                g = tv.G[idx];
                f = tv.F[idx];
                m = tv.M[idx];
            }
            e.G[k].w[w] = g;
            e.F[k].w[w] = f;
            e.M[k].w[w] = m;
        }
        int gw = r >> 6;
        uint64_t gl = (gw < tv.W) ? tv.GL[(size_t)term * tv.W + gw] : 0;
        uint64_t gh = (gw < tv.W) ? tv.GH[(size_t)term * tv.W + gw] : 0;
        int g = (int)((gl >> (r & 63)) & 1) | ((int)((gh >> (r & 63)) & 1) << 1);
        e.gam_set(k, g);
    }
#pragma unroll
    for (int w = 0; w < W; w++) {
        e.v.w[w] = (w < tv.W) ? tv.V[(size_t)term * tv.W + w] : 0;
        e.s.w[w] = (w < tv.W) ? tv.S[(size_t)term * tv.W + w] : 0;
    }
}

// A term held as 32-bit words (two per storage word).
template <int W, int RPL>
__device__ __forceinline__ void load_term(Eng<W, RPL, uint32_t>& e, const TermsView& tv, int64_t term) {
    e.n = tv.n;
    e.err = 0;
    e.phase = tv.phase[term];
    e.gam = 0;
#pragma unroll
    for (int k = 0; k < RPL; k++) {
        int r = 32 * k + e.lane;
#pragma unroll
        for (int sw = 0; 2 * sw < W; sw++) {
            uint64_t g = 0, f = 0, m = 0;
            if (r < tv.R && sw < tv.W) {
                size_t idx = ((size_t)term * tv.R + r) * tv.W + sw;
                g = tv.G[idx];
                f = tv.F[idx];
                m = tv.M[idx];
            }
            e.G[k].w[2 * sw] = (uint32_t)g;
            e.F[k].w[2 * sw] = (uint32_t)f;
            e.M[k].w[2 * sw] = (uint32_t)m;
            if (2 * sw + 1 < W) {
                e.G[k].w[2 * sw + 1] = (uint32_t)(g >> 32);
                e.F[k].w[2 * sw + 1] = (uint32_t)(f >> 32);
                e.M[k].w[2 * sw + 1] = (uint32_t)(m >> 32);
            }
        }
        int gw = r >> 6;
        uint64_t gl = (gw < tv.W) ? tv.GL[(size_t)term * tv.W + gw] : 0;
        uint64_t gh = (gw < tv.W) ? tv.GH[(size_t)term * tv.W + gw] : 0;
        int g = (int)((gl >> (r & 63)) & 1) | ((int)((gh >> (r & 63)) & 1) << 1);
        e.gam_set(k, g);
    }
#pragma unroll
    for (int sw = 0; 2 * sw < W; sw++) {
        const uint64_t vv = (sw < tv.W) ? tv.V[(size_t)term * tv.W + sw] : 0;
        const uint64_t ss = (sw < tv.W) ? tv.S[(size_t)term * tv.W + sw] : 0;
        e.v.w[2 * sw] = (uint32_t)vv;
        e.s.w[2 * sw] = (uint32_t)ss;
        if (2 * sw + 1 < W) {
            e.v.w[2 * sw + 1] = (uint32_t)(vv >> 32);
            e.s.w[2 * sw + 1] = (uint32_t)(ss >> 32);
        }
    }
}

// The storage word w of a row held as 32-bit words (two of them per word).
template <int W>
__device__ __forceinline__ uint64_t storage_word(const BV<uint32_t, W>& x, int w) {
    const uint32_t lo = (2 * w < W) ? x.w[(2 * w < W) ? 2 * w : 0] : 0u;
    const uint32_t hi = (2 * w + 1 < W) ? x.w[(2 * w + 1 < W) ? 2 * w + 1 : 0] : 0u;
    return (uint64_t)lo | ((uint64_t)hi << 32);
}

template <int W, int RPL>
__device__ __forceinline__ void store_term(const Eng<W, RPL, uint32_t>& e, const TermsView& tv, int64_t term) {
#pragma unroll
    for (int k = 0; k < 4; k++) {  // every row slot of the storage; slots the engine does not hold are zero
        int r = 32 * k + e.lane;
        if (r < tv.R) {
#pragma unroll
            for (int w = 0; w < 2; w++) {
                if (w < tv.W) {
                    const bool held = k < RPL;
                    const int kk = k < RPL ? k : 0;
                    size_t idx = ((size_t)term * tv.R + r) * tv.W + w;
                    tv.G[idx] = held ? storage_word<W>(e.G[kk], w) : 0;
                    tv.F[idx] = held ? storage_word<W>(e.F[kk], w) : 0;
                    tv.M[idx] = held ? storage_word<W>(e.M[kk], w) : 0;
                }
            }
        }
    }
    uint64_t gl[2] = {0, 0}, gh[2] = {0, 0};
#pragma unroll
    for (int k = 0; k < RPL; k++) {
        int g = e.gam_of(k);
        uint32_t b0 = __ballot_sync(dev::FULL, g & 1);
        uint32_t b1 = __ballot_sync(dev::FULL, (g >> 1) & 1);
        gl[k >> 1] |= (uint64_t)b0 << (32 * (k & 1));
        gh[k >> 1] |= (uint64_t)b1 << (32 * (k & 1));
    }
    if (e.lane == 0) {
#pragma unroll
        for (int w = 0; w < 2; w++) {
            if (w < tv.W) {
                tv.GL[(size_t)term * tv.W + w] = gl[w];
                tv.GH[(size_t)term * tv.W + w] = gh[w];
                tv.V[(size_t)term * tv.W + w] = storage_word<W>(e.v, w);
                tv.S[(size_t)term * tv.W + w] = storage_word<W>(e.s, w);
            }
        }
        tv.phase[term] = (uint8_t)e.phase;
    }
}

template <int W, int RPL = 2 * W>
__device__ __forceinline__ void store_term(const Eng<W, RPL>& e, const TermsView& tv, int64_t term) {
#pragma unroll
    for (int k = 0; k < 4; k++) {  // every row slot of the storage; slots the engine does not hold are zero
        int r = 32 * k + e.lane;
        if (r < tv.R) {
#pragma unroll
            for (int w = 0; w < 2; w++) {
                if (w < tv.W) {
                    const bool held = k < RPL && w < W;
                    const int kk = k < RPL ? k : 0, ww = w < W ? w : 0;
                    size_t idx = ((size_t)term * tv.R + r) * tv.W + w;
                    tv.G[idx] = held ? e.G[kk].w[ww] : 0;
                    tv.F[idx] = held ? e.F[kk].w[ww] : 0;
                    tv.M[idx] = held ? e.M[kk].w[ww] : 0;
                }
            }
        }
    }
    // γ planes by ballot: slot k covers rows 32k..32k+31 = word k/2, half k%2.
    uint64_t gl[2] = {0, 0}, gh[2] = {0, 0};
#pragma unroll
    for (int k = 0; k < RPL; k++) {
        int g = e.gam_of(k);
        uint32_t b0 = __ballot_sync(dev::FULL, g & 1);
        uint32_t b1 = __ballot_sync(dev::FULL, (g >> 1) & 1);
        gl[k >> 1] |= (uint64_t)b0 << (32 * (k & 1));
        gh[k >> 1] |= (uint64_t)b1 << (32 * (k & 1));
    }
    if (e.lane == 0) {
#pragma unroll
        for (int w = 0; w < 2; w++) {
            if (w < tv.W) {
                tv.GL[(size_t)term * tv.W + w] = gl[w];
                tv.GH[(size_t)term * tv.W + w] = gh[w];
                tv.V[(size_t)term * tv.W + w] = (w < W) ? e.v.w[(w < W) ? w : 0] : 0;
                tv.S[(size_t)term * tv.W + w] = (w < W) ? e.s.w[(w < W) ? w : 0] : 0;
            }
        }
        tv.phase[term] = (uint8_t)e.phase;
    }
}

template <int W, int RPL = 2 * W, typename Word = uint64_t>
__device__ __forceinline__ void apply_prim(Eng<W, RPL, Word>& e, uint32_t code) {
    uint32_t op = code & 0xff, a = (code >> 8) & 0xff, b = (code >> 16) & 0xff;
    switch (op) {
        case P_H: e.left_h(a); break;
        case P_X:
        case P_Y:  // one copy of the X rule: Y = i·X·Z
            if (op == P_Y) e.left_z(a);
            e.left_x(a);
            if (op == P_Y) e.phase = (e.phase + 2) & 7;
            break;
        case P_Z: e.left_z(a); break;
        case P_S:
        case P_SDG: e.left_s_like(a, op == P_S ? 3 : 1); break;  // one copy of the S rule
        case P_CX: e.left_cx(a, b); break;
        case P_CZ: e.left_cz(a, b); break;
        default: e.err = 9; break;
    }
}

// ---- compile ------------------------------------------------------------------
// CW warps per block: a compile launch has one warp per T-term, often only a few
// per SM, so small blocks spread them evenly over the SMs.
template <int W, int RPL, int CW, typename Word = uint64_t>
__global__ void __launch_bounds__(CW * 32) compile_kernel(
    const uint32_t* __restrict__ ops, int nops, int n, int t, int64_t chi_t,
    const uint64_t* __restrict__ tG, const uint64_t* __restrict__ tF, const uint64_t* __restrict__ tM,
    const uint8_t* __restrict__ tGam, const uint64_t* __restrict__ tV, const uint64_t* __restrict__ tS,
    const uint8_t* __restrict__ tPhase, const uint8_t* __restrict__ tCk, const int32_t* __restrict__ tCr,
    TermsView out, int32_t* __restrict__ keep, int* __restrict__ status) {
    __shared__ uint32_t sops[OPS_CHUNK];
    const int lane = threadIdx.x & 31;
    const int64_t term = (int64_t)blockIdx.x * CW + (threadIdx.x >> 5);
    const bool active = term < chi_t;
    const int width = n + t;

    Eng<W, RPL, Word> e;
    constexpr int WB = 8 * (int)sizeof(Word);
    e.lane = lane;
    e.init_zero(width);
    if (active) {
        // kron(|0^n⟩, T-term) (form/kron.rs:12-59): T rows shifted by n rows and n columns.
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            int r = 32 * k + lane;
            if (r >= n && r < width) {
                int tr = r - n;
                size_t idx = (size_t)term * t + tr;
                BV<Word, W> g = BV<Word, W>::zero(), f = g, m = g;
                uint64_t gw = tG[idx], fw = tF[idx], mw = tM[idx];
#pragma unroll
                for (int w = 0; w < W; w++) {
                    int lo = WB * w;
                    // bit c of the shifted row = bit (c - n) of the T row
                    auto sh = [&](uint64_t x) -> Word {
                        int off = lo - n;  // T bit index of this word's bit 0
                        if (off >= 64 || off <= -WB) return 0;
                        return (Word)(off >= 0 ? (x >> off) : (x << (-off)));
                    };
                    g.w[w] = sh(gw);
                    f.w[w] = sh(fw);
                    m.w[w] = sh(mw);
                }
                e.G[k] = g;
                e.F[k] = f;
                e.M[k] = m;
                e.gam_set(k, tGam[idx]);
            }
        }
        uint64_t vv = tV[term], ss = tS[term];
#pragma unroll
        for (int w = 0; w < W; w++) {
            int off = WB * w - n;
            e.v.w[w] = (off >= 64 || off <= -WB) ? (Word)0 : (Word)(off >= 0 ? (vv >> off) : (vv << (-off)));
            e.s.w[w] = (off >= 64 || off <= -WB) ? (Word)0 : (Word)(off >= 0 ? (ss >> off) : (ss << (-off)));
        }
        e.phase = tPhase[term];
    }

    for (int base = 0; base < nops; base += OPS_CHUNK) {
        int cnt = min(OPS_CHUNK, nops - base);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) sops[i] = ops[base + i];
        __syncthreads();
        if (active && !e.err) {
            for (int i = 0; i < cnt; i++) apply_prim<W, RPL, Word>(e, sops[i]);
        }
    }
    if (!active) return;

    // Post-select the ancillas onto |0⟩ in reverse order (compiler/mod.rs:104-120).
    int ndet = 0;
    bool ok = true;
    for (int q = width - 1; q >= n && !e.err; q--) {
        int r = e.project(q, false);
        if (r < 0) {
            ok = false;
            break;
        }
        ndet += r;
    }
    if (ok && !e.err) {
        for (int q = width - 1; q >= n && !e.err; q--) e.discard(q);  // :124-127
    }
    if (e.err) {
        if (lane == 0) atomicOr(status, e.err == 2 ? DS_CANNOT_DISCARD : DS_INVARIANT);
        ok = false;
    }
    if (lane == 0) {
        keep[term] = ok ? 1 : 0;
        out.coef_k[term] = tCk[term];
        out.coef_r[term] = tCr[term] - ndet;  // coeff.amplify(ndet) (scalar.rs:108-119)
    }
    if (ok) store_term<W, RPL>(e, out, term);
}

// ---- |T⟩^{⊗t} expansion --------------------------------------------------------
// cat_state.rs:162-188 builds cat(m) for m > 6 from cat(m−4) and cat(6): every
// pair of terms is joined (kron), then Sdg(q0), CX(q0, q1), H(q0) on the two
// boundary qubits q0 = m−5, q1 = m−4, both projected onto |0⟩ and discarded.
// Unrolled, term ci of cat(t) is base term i0 of cat(m0) joined with cat(6)
// terms j_1..j_L, ci = ((i0·3 + j_1)·3 + …)·3 + j_L (the product is i-major,
// stabilizer_decomposed_state/kron.rs:11-16), and its coefficient is the
// product of theirs.  t_state.rs:29-71 appends an X·S copy of every term
// (coefficient × e^{-iπ/4}) and scales all by 2^{-1/2}.  One warp builds one
// term with the same rules in the same order as the host construction.
template <int W>
__device__ __forceinline__ BV<uint64_t, W> small_row(uint64_t x, int off) {
    BV<uint64_t, W> r = BV<uint64_t, W>::zero();
    for (int c = 0; c < 6; c++)
        if ((x >> c) & 1) r.set(off + c, true);
    return r;
}

template <int W>
__device__ __forceinline__ void join_small(Eng<W>& e, const TSmallTerm& b, int off) {
#pragma unroll
    for (int k = 0; k < 2 * W; k++) {
        const int r = 32 * k + e.lane;
        if (r >= off && r < off + 6) {
            e.G[k] = small_row<W>(b.G[r - off], off);
            e.F[k] = small_row<W>(b.F[r - off], off);
            e.M[k] = small_row<W>(b.M[r - off], off);
            e.gam_set(k, b.gam[r - off]);
        }
    }
    e.v = e.v | small_row<W>(b.v, off);
    e.s = e.s | small_row<W>(b.s, off);
    e.phase = (e.phase + b.phase) & 7;
}

template <int W>
__global__ void __launch_bounds__(WARPS * 32) t_tensor_kernel(TPrelude pre, int64_t chi_cat, TTensorOut out,
                                                              int* __restrict__ status) {
    const int lane = threadIdx.x & 31;
    const int64_t term = (int64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    if (term >= 2 * chi_cat) return;  // warp-uniform
    const bool xs_copy = term >= chi_cat;
    const int64_t ci = xs_copy ? term - chi_cat : term;
    int64_t p3 = 1;  // 3^L: the digits j_1..j_L are ci mod 3^L, most significant first
    for (int l = 0; l < pre.L; l++) p3 *= 3;
    int64_t rem = ci % p3;
    const TSmallTerm& b0 = pre.base[ci / p3];
    Eng<W> e;
    e.lane = lane;
    e.init_zero(0);
    e.n = 0;
    join_small<W>(e, b0, 0);
    e.n = pre.m0;
    int ck = b0.k, cr = b0.r;
    bool ok = true;
    for (int l = 1; l <= pre.L && ok; l++) {
        const int w = pre.m0 + 4 * (l - 1);
        p3 /= 3;
        const TSmallTerm& b = pre.cat6[rem / p3];
        rem %= p3;
        join_small<W>(e, b, w);
        e.n = w + 6;
        ck += b.k;
        cr += b.r;
        const int q0 = w - 1, q1 = w;
        e.left_sdg(q0);
        e.left_cx(q0, q1);
        e.left_h(q0);
        if (e.project(q0, false) < 0 || e.project(q1, false) < 0) ok = false;
        if (ok) {
            e.discard(q1);
            e.discard(q0);
        }
        if (e.err) ok = false;
    }
    if (ok && xs_copy) {
        e.left_x(0);
        e.left_s(0);
        ck += 7;
    }
    if (!ok || e.err) {
        if (lane == 0) atomicOr(status, DS_INVARIANT);
        return;
    }
    const int t = pre.t;
#pragma unroll
    for (int k = 0; k < 2 * W; k++) {
        const int r = 32 * k + lane;
        if (r < t) {
            const size_t idx = (size_t)term * t + r;
            out.G[idx] = e.G[k].w[0];
            out.F[idx] = e.F[k].w[0];
            out.M[idx] = e.M[k].w[0];
            out.gam[idx] = (uint8_t)e.gam_of(k);
        }
    }
    if (lane == 0) {
        out.V[term] = e.v.w[0];
        out.S[term] = e.s.w[0];
        out.phase[term] = (uint8_t)e.phase;
        out.ck[term] = (uint8_t)(ck & 7);
        out.cr[term] = cr + 1;  // × ONE_OVER_SQRT_2 (t_state.rs:59-64)
    }
}

// ---- compaction -------------------------------------------------------------
__global__ void scan_keep_kernel(const int32_t* __restrict__ keep, int64_t n, int32_t* __restrict__ pos,
                                 int64_t* __restrict__ count) {
    // Single block exclusive scan (χ ≤ a few 10^6).
    __shared__ int32_t warp_tot[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t base = 0; base < n; base += blockDim.x) {
        int64_t i = base + threadIdx.x;
        int32_t x = (i < n) ? keep[i] : 0;
        int32_t incl = x;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            int32_t y = __shfl_up_sync(dev::FULL, incl, d);
            if (lane >= d) incl += y;
        }
        if (lane == 31) warp_tot[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int32_t w = (lane < (int)(blockDim.x >> 5)) ? warp_tot[lane] : 0;
            int32_t wi = w;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                int32_t y = __shfl_up_sync(dev::FULL, wi, d);
                if (lane >= d) wi += y;
            }
            warp_tot[lane] = wi - w;  // exclusive
        }
        __syncthreads();
        int64_t excl = carry + warp_tot[wid] + incl - x;
        if (i < n) pos[i] = (int32_t)excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = carry;
}

__global__ void gather_kernel(TermsView in, const int32_t* __restrict__ keep, const int32_t* __restrict__ pos,
                              TermsView out) {
    const int64_t term = (int64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (term >= in.chi || !keep[term]) return;
    const int64_t dst = pos[term];
    const size_t rowwords = (size_t)in.R * in.W;
    for (size_t i = lane; i < rowwords; i += 32) {
        out.G[dst * rowwords + i] = in.G[term * rowwords + i];
        out.F[dst * rowwords + i] = in.F[term * rowwords + i];
        out.M[dst * rowwords + i] = in.M[term * rowwords + i];
    }
    for (int w = lane; w < in.W; w += 32) {
        out.V[dst * in.W + w] = in.V[term * in.W + w];
        out.S[dst * in.W + w] = in.S[term * in.W + w];
        out.GL[dst * in.W + w] = in.GL[term * in.W + w];
        out.GH[dst * in.W + w] = in.GH[term * in.W + w];
    }
    if (lane == 0) {
        out.phase[dst] = in.phase[term];
        out.coef_k[dst] = in.coef_k[term];
        out.coef_r[dst] = in.coef_r[term];
    }
}

// ---- gate application / projection / discard on a compiled state ----------
template <int W>
__global__ void __launch_bounds__(WARPS * 32) apply_ops_kernel(const uint32_t* __restrict__ ops, int nops,
                                                              TermsView tv, int* __restrict__ status) {
    __shared__ uint32_t sops[OPS_CHUNK];
    const int64_t term = (int64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    const bool active = term < tv.chi;
    Eng<2 * W, 2 * W, uint32_t> e;  // 32-bit words
    e.lane = threadIdx.x & 31;
    if (active) load_term(e, tv, term);
    for (int base = 0; base < nops; base += OPS_CHUNK) {
        int cnt = min(OPS_CHUNK, nops - base);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) sops[i] = ops[base + i];
        __syncthreads();
        if (active && !e.err)
            for (int i = 0; i < cnt; i++) apply_prim<2 * W, 2 * W, uint32_t>(e, sops[i]);
    }
    if (!active) return;
    if (e.err && e.lane == 0) atomicOr(status, DS_INVARIANT);
    store_term(e, tv, term);
}

// ---- short runs of gates without H, one thread per term ----------------------
// S, Sdg, Z, X, Y, CZ and CX each change a few rows of a term (the left
// multiplication rules of form/left_multiplication/{s,z,x,y,cz,cx}.rs, the same
// updates as WarpCH's left_*), so a call with a few of them reads and writes
// only those rows in place instead of moving every term through a warp: an S
// gate touches 3·8W + 2 bytes of a term, not the whole tableau.
template <int W>
__global__ void __launch_bounds__(256) row_ops_kernel(TermsView tv, RowOps ops) {
    const int64_t term = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (term >= tv.chi) return;
    const size_t rb = (size_t)term * tv.R;
    auto at = [&](uint32_t r, int w) -> size_t { return (rb + r) * W + w; };
    auto gam = [&](uint32_t q) -> int {
        const size_t o = (size_t)term * W + (q >> 6);
        return (int)((tv.GL[o] >> (q & 63)) & 1) | ((int)((tv.GH[o] >> (q & 63)) & 1) << 1);
    };
    auto set_gam = [&](uint32_t q, int g) {
        const size_t o = (size_t)term * W + (q >> 6);
        const uint64_t bit = 1ull << (q & 63);
        tv.GL[o] = (g & 1) ? (tv.GL[o] | bit) : (tv.GL[o] & ~bit);
        tv.GH[o] = (g & 2) ? (tv.GH[o] | bit) : (tv.GH[o] & ~bit);
    };
    int phase = tv.phase[term];
    for (int i = 0; i < ops.n; i++) {
        const uint32_t code = ops.code[i], op = code & 0xff, a = (code >> 8) & 0xff, b = (code >> 16) & 0xff;
        switch (op) {
            case P_S:
            case P_SDG:  // M[a] ^= G[a]; γ_a -= 1 (S) or += 1 (Sdg)
#pragma unroll
                for (int w = 0; w < W; w++) tv.M[at(a, w)] ^= tv.G[at(a, w)];
                set_gam(a, gam(a) + (op == P_S ? 3 : 1));
                break;
            case P_Z: set_gam(a, gam(a) + 2); break;
            case P_CZ:  // M[a] ^= G[b]; M[b] ^= G[a]
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const uint64_t ga = tv.G[at(a, w)], gb = tv.G[at(b, w)];
                    tv.M[at(a, w)] ^= gb;
                    tv.M[at(b, w)] ^= ga;
                }
                break;
            case P_CX: {  // c = a, t = b: γ_c += γ_t + 2·(M_c·F_t); F_c ^= F_t; M_c ^= M_t; G_t ^= G_c
                int dot = 0;
#pragma unroll
                for (int w = 0; w < W; w++) dot += __popcll(tv.M[at(a, w)] & tv.F[at(b, w)]);
                set_gam(a, gam(a) + gam(b) + 2 * (dot & 1));
#pragma unroll
                for (int w = 0; w < W; w++) {
                    tv.F[at(a, w)] ^= tv.F[at(b, w)];
                    tv.M[at(a, w)] ^= tv.M[at(b, w)];
                    tv.G[at(b, w)] ^= tv.G[at(a, w)];
                }
                break;
            }
            case P_X:
            case P_Y: {  // Y = i·X·Z: γ_a += 2 first, then the X rule, then the phase i
                if (op == P_Y) set_gam(a, gam(a) + 2);
                int beta = 0;
#pragma unroll
                for (int w = 0; w < W; w++) {
                    const size_t o = (size_t)term * W + w;
                    const uint64_t v = tv.V[o], s = tv.S[o], f = tv.F[at(a, w)], m = tv.M[at(a, w)];
                    beta += __popcll((m & ~v & s) ^ (f & v & (m ^ s)));
                    tv.S[o] = s ^ (f & ~v) ^ (m & v);
                }
                phase += 4 * (beta & 1) + 2 * gam(a) + (op == P_Y ? 2 : 0);
                break;
            }
            default: break;  // the host sends no other op here
        }
    }
    tv.phase[term] = (uint8_t)(phase & 7);
}

template <int W>
__global__ void __launch_bounds__(WARPS * 32) project_kernel(TermsView tv, int q, int outcome,
                                                            int32_t* __restrict__ keep, int* __restrict__ status) {
    const int64_t term = (int64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    if (term >= tv.chi) return;
    Eng<2 * W, 2 * W, uint32_t> e;  // 32-bit words
    e.lane = threadIdx.x & 31;
    load_term(e, tv, term);
    int r = e.project(q, outcome != 0);
    if (e.err) {
        if (e.lane == 0) atomicOr(status, DS_INVARIANT);
        r = -1;
    }
    if (e.lane == 0) {
        keep[term] = (r >= 0) ? 1 : 0;
        if (r == 0) tv.coef_r[term] += 1;  // amplify(-1): r -= -1 (projection.rs:44)
    }
    if (r == 0) store_term(e, tv, term);
}

template <int W>
__global__ void __launch_bounds__(WARPS * 32) discard_kernel(TermsView tv, int q, int* __restrict__ status) {
    const int64_t term = (int64_t)blockIdx.x * WARPS + (threadIdx.x >> 5);
    if (term >= tv.chi) return;
    Eng<2 * W, 2 * W, uint32_t> e;  // 32-bit words
    e.lane = threadIdx.x & 31;
    load_term(e, tv, term);
    e.discard(q);
    if (e.err && e.lane == 0) atomicOr(status, e.err == 2 ? DS_CANNOT_DISCARD : DS_INVARIANT);
    store_term(e, tv, term);  // width n-1 in the same storage
}

// ---- pack / unpack bool bytes -------------------------------------------------
__global__ void unpack_kernel(TermsView tv, uint8_t* G, uint8_t* F, uint8_t* M, uint8_t* gam, uint8_t* v,
                              uint8_t* s) {
    const int n = tv.n;
    const int64_t total = tv.chi * n * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t term = i / ((int64_t)n * n);
        int rc = (int)(i % ((int64_t)n * n));
        int r = rc / n, c = rc % n;
        size_t idx = ((size_t)term * tv.R + r) * tv.W + (c >> 6);
        G[i] = (tv.G[idx] >> (c & 63)) & 1;
        F[i] = (tv.F[idx] >> (c & 63)) & 1;
        M[i] = (tv.M[idx] >> (c & 63)) & 1;
        if (c == 0) {
            size_t w = (size_t)term * tv.W + (r >> 6);
            int g = (int)((tv.GL[w] >> (r & 63)) & 1) | ((int)((tv.GH[w] >> (r & 63)) & 1) << 1);
            gam[term * n + r] = (uint8_t)(2 * g);  // Z8 exponent of the reference's PhaseFactor
            v[term * n + r] = (tv.V[w] >> (r & 63)) & 1;
            s[term * n + r] = (tv.S[w] >> (r & 63)) & 1;
        }
    }
}

__global__ void pack_kernel(TermsView tv, const uint8_t* G, const uint8_t* F, const uint8_t* M, const uint8_t* gam,
                            const uint8_t* v, const uint8_t* s) {
    // one thread per (term, row word): builds the words of row r
    const int n = tv.n;
    const int64_t total = tv.chi * tv.R;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t term = i / tv.R;
        int r = (int)(i % tv.R);
        for (int w = 0; w < tv.W; w++) {
            uint64_t g = 0, f = 0, m = 0;
            if (r < n) {
                for (int b = 0; b < 64; b++) {
                    int c = 64 * w + b;
                    if (c >= n) break;
                    size_t bi = ((size_t)term * n + r) * n + c;
                    g |= (uint64_t)(G[bi] & 1) << b;
                    f |= (uint64_t)(F[bi] & 1) << b;
                    m |= (uint64_t)(M[bi] & 1) << b;
                }
            }
            size_t idx = ((size_t)term * tv.R + r) * tv.W + w;
            tv.G[idx] = g;
            tv.F[idx] = f;
            tv.M[idx] = m;
        }
        if (r < tv.W) {  // vectors: thread r of the term builds word r
            int w = r;
            uint64_t gl = 0, gh = 0, vv = 0, ss = 0;
            for (int b = 0; b < 64; b++) {
                int q = 64 * w + b;
                if (q >= n) break;
                int g = (gam[term * n + q] >> 1) & 3;
                gl |= (uint64_t)(g & 1) << b;
                gh |= (uint64_t)((g >> 1) & 1) << b;
                vv |= (uint64_t)(v[term * n + q] & 1) << b;
                ss |= (uint64_t)(s[term * n + q] & 1) << b;
            }
            tv.GL[term * tv.W + w] = gl;
            tv.GH[term * tv.W + w] = gh;
            tv.V[term * tv.W + w] = vv;
            tv.S[term * tv.W + w] = ss;
        }
    }
}

// ---- dense statevector (n ≤ 28; tests and to_statevector) -------------------
// ⟨x|U_C U_H|s⟩ = i^{Σ_{p∈x}γ_p}·(-1)^{Σ_{p<q∈x} M_p·F_q + u·m + Σ_{j∈v} u_j s_j}·2^{-|v|/2}
// with u = xF, m = xM, nonzero iff u_j = s_j for all j ∉ v.  Same value as
// amplitude_at_computational_basis (form/amplitude.rs:28-44).
__global__ void statevector_kernel(TermsView tv, double gf_re, double gf_im, double* __restrict__ out) {
    const int n = tv.n;
    const int64_t dim = (int64_t)1 << n;
    const double r2 = 0.70710678118654752440;
    const double cr[8] = {1, r2, 0, -r2, -1, -r2, 0, r2};
    const double ci[8] = {0, r2, 1, r2, 0, -r2, -1, -r2};
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < dim; x += (int64_t)gridDim.x * blockDim.x) {
        double ar = 0.0, ai = 0.0;
        for (int64_t term = 0; term < tv.chi; term++) {
            const uint64_t* F = tv.F + (size_t)term * tv.R * tv.W;
            const uint64_t* M = tv.M + (size_t)term * tv.R * tv.W;
            uint64_t u = 0, m = 0;
            int cnt = 0, gsum = 0;
            uint64_t gl = tv.GL[term * tv.W], gh = tv.GH[term * tv.W];
            for (int p = 0; p < n; p++) {
                if ((x >> p) & 1) {
                    uint64_t fp = F[(size_t)p * tv.W], mp = M[(size_t)p * tv.W];
                    cnt += __popcll(m & fp);
                    u ^= fp;
                    m ^= mp;
                    gsum += (int)((gl >> p) & 1) + 2 * (int)((gh >> p) & 1);
                }
            }
            uint64_t v = tv.V[term * tv.W], s = tv.S[term * tv.W];
            if (((u ^ s) & ~v) != 0) continue;
            cnt += __popcll(u & m) + __popcll(u & v & s);
            int k = (tv.phase[term] + 2 * gsum + 4 * (cnt & 1) + tv.coef_k[term]) & 7;
            int rr = __popcll(v) + tv.coef_r[term];
            double mag = exp2(-0.5 * (double)rr);
            ar += mag * cr[k];
            ai += mag * ci[k];
        }
        out[2 * x] = ar * gf_re - ai * gf_im;
        out[2 * x + 1] = ar * gf_im + ai * gf_re;
    }
}

inline int blocks_for(int64_t chi) { return (int)((chi + WARPS - 1) / WARPS); }

}  // namespace

cudaError_t launch_compile(const uint32_t* d_ops, int nops, int n, int t, int64_t chi_t, const uint64_t* tG,
                           const uint64_t* tF, const uint64_t* tM, const uint8_t* tGam, const uint64_t* tV,
                           const uint64_t* tS, const uint8_t* tPhase, const uint8_t* tCk, const int32_t* tCr,
                           TermsView out, int32_t* keep, int* status, cudaStream_t st) {
    if (chi_t == 0) return cudaSuccess;
    int width = n + t;
    constexpr int CW = kCompileWarps;
    dim3 grid((unsigned)((chi_t + CW - 1) / CW)), block(CW * 32);
    if (width <= 64)
        compile_kernel<2, 2, CW, uint32_t><<<grid, block, 0, st>>>(d_ops, nops, n, t, chi_t, tG, tF, tM, tGam, tV, tS, tPhase,
                                                         tCk, tCr, out, keep, status);
    else if (width <= 96)  // three row slots of three 32-bit words: 96 rows of 96 columns
        compile_kernel<3, 3, CW, uint32_t><<<grid, block, 0, st>>>(d_ops, nops, n, t, chi_t, tG, tF, tM, tGam, tV, tS, tPhase,
                                                         tCk, tCr, out, keep, status);
    else
        compile_kernel<4, 4, CW, uint32_t><<<grid, block, 0, st>>>(d_ops, nops, n, t, chi_t, tG, tF, tM, tGam, tV, tS, tPhase,
                                                         tCk, tCr, out, keep, status);
    return cudaGetLastError();
}

cudaError_t launch_t_tensor(const TPrelude& pre, int64_t chi_cat, TTensorOut out, int* status, cudaStream_t st) {
    if (chi_cat == 0) return cudaSuccess;
    dim3 grid(blocks_for(2 * chi_cat)), block(WARPS * 32);
    if (pre.t + 2 <= 64)  // the widest intermediate term has t + 2 qubits
        t_tensor_kernel<1><<<grid, block, 0, st>>>(pre, chi_cat, out, status);
    else
        t_tensor_kernel<2><<<grid, block, 0, st>>>(pre, chi_cat, out, status);
    return cudaGetLastError();
}

cudaError_t launch_compact(const TermsView& in, const int32_t* keep, int32_t* scan_tmp, TermsView out,
                           int64_t* d_count, cudaStream_t st) {
    if (in.chi == 0) return cudaMemsetAsync(d_count, 0, sizeof(int64_t), st);
    scan_keep_kernel<<<1, 1024, 0, st>>>(keep, in.chi, scan_tmp, d_count);
    gather_kernel<<<blocks_for(in.chi), WARPS * 32, 0, st>>>(in, keep, scan_tmp, out);
    return cudaGetLastError();
}

cudaError_t launch_apply_ops(const uint32_t* d_ops, int nops, TermsView terms, int* status, cudaStream_t st) {
    if (terms.chi == 0 || nops == 0) return cudaSuccess;
    if (terms.W == 1)
        apply_ops_kernel<1><<<blocks_for(terms.chi), WARPS * 32, 0, st>>>(d_ops, nops, terms, status);
    else
        apply_ops_kernel<2><<<blocks_for(terms.chi), WARPS * 32, 0, st>>>(d_ops, nops, terms, status);
    return cudaGetLastError();
}

cudaError_t launch_row_ops(const RowOps& ops, TermsView terms, cudaStream_t st) {
    if (terms.chi == 0 || ops.n == 0) return cudaSuccess;
    const unsigned blocks = (unsigned)((terms.chi + 255) / 256);
    if (terms.W == 1)
        row_ops_kernel<1><<<blocks, 256, 0, st>>>(terms, ops);
    else
        row_ops_kernel<2><<<blocks, 256, 0, st>>>(terms, ops);
    return cudaGetLastError();
}

cudaError_t launch_project(TermsView terms, int qubit, int outcome, int32_t* keep, int* status, cudaStream_t st) {
    if (terms.chi == 0) return cudaSuccess;
    if (terms.W == 1)
        project_kernel<1><<<blocks_for(terms.chi), WARPS * 32, 0, st>>>(terms, qubit, outcome, keep, status);
    else
        project_kernel<2><<<blocks_for(terms.chi), WARPS * 32, 0, st>>>(terms, qubit, outcome, keep, status);
    return cudaGetLastError();
}

cudaError_t launch_discard(TermsView terms, int qubit, int* status, cudaStream_t st) {
    if (terms.chi == 0) return cudaSuccess;
    if (terms.W == 1)
        discard_kernel<1><<<blocks_for(terms.chi), WARPS * 32, 0, st>>>(terms, qubit, status);
    else
        discard_kernel<2><<<blocks_for(terms.chi), WARPS * 32, 0, st>>>(terms, qubit, status);
    return cudaGetLastError();
}

cudaError_t launch_unpack(const TermsView& t, uint8_t* G, uint8_t* F, uint8_t* M, uint8_t* gam, uint8_t* v,
                          uint8_t* s, cudaStream_t st) {
    if (t.chi == 0) return cudaSuccess;
    int64_t total = t.chi * t.n * t.n;
    int blocks = (int)std::min<int64_t>((total + 255) / 256, 65535);
    unpack_kernel<<<blocks, 256, 0, st>>>(t, G, F, M, gam, v, s);
    return cudaGetLastError();
}

cudaError_t launch_pack(TermsView t, const uint8_t* G, const uint8_t* F, const uint8_t* M, const uint8_t* gam,
                        const uint8_t* v, const uint8_t* s, cudaStream_t st) {
    if (t.chi == 0) return cudaSuccess;
    int64_t total = t.chi * t.R;
    int blocks = (int)std::min<int64_t>((total + 255) / 256, 65535);
    pack_kernel<<<blocks, 256, 0, st>>>(t, G, F, M, gam, v, s);
    return cudaGetLastError();
}

// Word k of a width-n bit row with the bits at and above n cleared.
__device__ __forceinline__ uint64_t row_word(const uint64_t* src, int n, int k) {
    const int lo = 64 * k;
    if (n <= lo) return 0;
    return n >= lo + 64 ? src[k] : src[k] & ((1ULL << (n - lo)) - 1);
}

// Word w of (row << sh) for a width-n row held in words.
__device__ __forceinline__ uint64_t shifted_word(const uint64_t* src, int n, int sh, int w) {
    const int ws = sh >> 6, bs = sh & 63;
    const int hi = w - ws, lo = hi - 1;
    uint64_t x = hi >= 0 ? row_word(src, n, hi) << bs : 0;
    if (bs && lo >= 0) x |= row_word(src, n, lo) >> (64 - bs);
    return x;
}

// Term (i, j) ↦ i·χ_B + j of A ⊗ B (stabilizer_decomposed_state/kron.rs:7-22
// with form/kron.rs:12-59): G, F, M block-diagonal, γ, v, s concatenated (B's
// qubits after A's), phase factors multiplied, coefficients multiplied.  One
// thread per (output term, row slot), as pack_kernel.
__global__ void kron_kernel(TermsView A, TermsView B, TermsView O) {
    const int64_t total = O.chi * O.R;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t term = t / O.R;
        const int r = (int)(t % O.R);
        const int64_t i = term / B.chi, j = term % B.chi;
        const uint64_t *g = nullptr, *f = nullptr, *m = nullptr;
        int width = 0, sh = 0;
        if (r < A.n) {
            const size_t o = ((size_t)i * A.R + r) * A.W;
            g = A.G + o; f = A.F + o; m = A.M + o; width = A.n;
        } else if (r < O.n) {
            const size_t o = ((size_t)j * B.R + (r - A.n)) * B.W;
            g = B.G + o; f = B.F + o; m = B.M + o; width = B.n; sh = A.n;
        }
        for (int w = 0; w < O.W; w++) {
            const size_t idx = ((size_t)term * O.R + r) * O.W + w;
            O.G[idx] = g ? shifted_word(g, width, sh, w) : 0;
            O.F[idx] = f ? shifted_word(f, width, sh, w) : 0;
            O.M[idx] = m ? shifted_word(m, width, sh, w) : 0;
        }
        if (r < O.W) {  // vectors: word r of the term
            const size_t oa = (size_t)i * A.W, ob = (size_t)j * B.W, oo = (size_t)term * O.W + r;
            O.V[oo] = shifted_word(A.V + oa, A.n, 0, r) | shifted_word(B.V + ob, B.n, A.n, r);
            O.S[oo] = shifted_word(A.S + oa, A.n, 0, r) | shifted_word(B.S + ob, B.n, A.n, r);
            O.GL[oo] = shifted_word(A.GL + oa, A.n, 0, r) | shifted_word(B.GL + ob, B.n, A.n, r);
            O.GH[oo] = shifted_word(A.GH + oa, A.n, 0, r) | shifted_word(B.GH + ob, B.n, A.n, r);
        }
        if (r == 0) {
            O.phase[term] = (uint8_t)((A.phase[i] + B.phase[j]) & 7);
            O.coef_k[term] = (uint8_t)((A.coef_k[i] + B.coef_k[j]) & 7);
            O.coef_r[term] = A.coef_r[i] + B.coef_r[j];
        }
    }
}

cudaError_t launch_kron(TermsView A, TermsView B, TermsView O, cudaStream_t st) {
    if (O.chi == 0) return cudaSuccess;
    const int64_t total = O.chi * O.R;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 65535);
    kron_kernel<<<blocks, 256, 0, st>>>(A, B, O);
    return cudaGetLastError();
}

cudaError_t launch_statevector(const TermsView& t, double gf_re, double gf_im, double* out, cudaStream_t st) {
    int64_t dim = (int64_t)1 << t.n;
    int blocks = (int)std::min<int64_t>((dim + 255) / 256, 65535);
    statevector_kernel<<<blocks, 256, 0, st>>>(t, gf_re, gf_im, out);
    return cudaGetLastError();
}

int device_sm_count() {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

}  // namespace nsg
