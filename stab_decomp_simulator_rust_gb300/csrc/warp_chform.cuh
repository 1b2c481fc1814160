// warp_chform.cuh — one CH-form term held by one warp.
//
// Layout: row r of G, F, M lives in lane (r & 31), slot (r >> 5); a row is W
// words of `Word` (u32 or u64), bit c of the row is column c.  γ_r (an
// exponent of i, mod 4) is kept by the row's lane as 2 bits per slot.  The
// vectors v, s and the Z8 phase are warp-uniform.  Row operations move a row
// between lanes with one shuffle per word; column operations (the right
// multiplications inside _resolve_superposition) are lane-local, so an H gate
// costs O(W) instructions per lane instead of the reference's O(w²) byte loop.
//
// Every rule reproduces the reference's update exactly (same pivots, same
// order), so the tableau bits match crates/stabilizer-ch-form-rust/src/form/.
// Where the reference applies a sequence of column operations that commute
// (resolve_superposition.rs:155-176, discard.rs:152-158, :174-178) they are
// applied as one masked update; each such batch is annotated with why the
// result is identical.
//
// Invariant violations that the reference turns into panics
// (resolve_superposition.rs:121, discard.rs:140,155) set `err` instead.
#pragma once

#include <cstdint>

namespace nsg {
namespace dev {

constexpr unsigned FULL = 0xffffffffu;

template <typename Word>
__device__ __forceinline__ Word shfl(Word x, int src) {
    return __shfl_sync(FULL, x, src);
}

template <typename Word>
__device__ __forceinline__ int popc(Word x);
template <>
__device__ __forceinline__ int popc<uint32_t>(uint32_t x) { return __popc(x); }
template <>
__device__ __forceinline__ int popc<uint64_t>(uint64_t x) { return __popcll(x); }

template <typename Word>
__device__ __forceinline__ int ffs0(Word x);  // index of lowest set bit, -1 if none
template <>
__device__ __forceinline__ int ffs0<uint32_t>(uint32_t x) { return __ffs(x) - 1; }
template <>
__device__ __forceinline__ int ffs0<uint64_t>(uint64_t x) { return __ffsll((long long)x) - 1; }

// ---- W-word bit vectors (uniform or per lane) -----------------------------
template <typename Word, int W>
struct BV {
    static constexpr int B = 8 * sizeof(Word);
    Word w[W];

    __device__ __forceinline__ static BV zero() {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) r.w[k] = 0;
        return r;
    }
    // Word selection by a run-time bit index is written with masks over every
    // word (never a guarded or indexed access), so the vector stays in registers.
    __device__ __forceinline__ bool bit(int q) const {
        Word x = 0;
#pragma unroll
        for (int k = 0; k < W; k++) x |= w[k] & ((q / B) == k ? ~(Word)0 : (Word)0);
        return (x >> (q & (B - 1))) & 1;
    }
    __device__ __forceinline__ void flip(int q) {
        const Word m = (Word)1 << (q & (B - 1));
#pragma unroll
        for (int k = 0; k < W; k++) w[k] ^= ((q / B) == k) ? m : (Word)0;
    }
    __device__ __forceinline__ void set(int q, bool b) {
#pragma unroll
        for (int k = 0; k < W; k++) {
            const Word m = ((q / B) == k) ? ((Word)1 << (q & (B - 1))) : (Word)0;
            w[k] = b ? (w[k] | m) : (w[k] & ~m);
        }
    }
    __device__ __forceinline__ bool any() const {
        Word a = 0;
#pragma unroll
        for (int k = 0; k < W; k++) a |= w[k];
        return a != 0;
    }
    __device__ __forceinline__ int parity() const {
        int p = 0;
#pragma unroll
        for (int k = 0; k < W; k++) p += popc<Word>(w[k]);
        return p & 1;
    }
    __device__ __forceinline__ int count() const {
        int p = 0;
#pragma unroll
        for (int k = 0; k < W; k++) p += popc<Word>(w[k]);
        return p;
    }
    __device__ __forceinline__ int first() const {  // lowest set bit or -1
        int r = -1;
#pragma unroll
        for (int k = W - 1; k >= 0; k--) {
            int f = ffs0<Word>(w[k]);
            if (f >= 0) r = f + k * B;
        }
        return r;
    }
    __device__ __forceinline__ bool operator==(const BV& o) const {
        bool e = true;
#pragma unroll
        for (int k = 0; k < W; k++) e &= (w[k] == o.w[k]);
        return e;
    }
    __device__ __forceinline__ BV operator^(const BV& o) const {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) r.w[k] = w[k] ^ o.w[k];
        return r;
    }
    __device__ __forceinline__ BV operator&(const BV& o) const {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) r.w[k] = w[k] & o.w[k];
        return r;
    }
    __device__ __forceinline__ BV operator|(const BV& o) const {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) r.w[k] = w[k] | o.w[k];
        return r;
    }
    __device__ __forceinline__ BV operator~() const {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) r.w[k] = ~w[k];
        return r;
    }
    __device__ __forceinline__ BV& operator^=(const BV& o) {
#pragma unroll
        for (int k = 0; k < W; k++) w[k] ^= o.w[k];
        return *this;
    }
    // r = cond ? mask : 0
    __device__ __forceinline__ static BV select(bool cond, const BV& m) {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) r.w[k] = cond ? m.w[k] : (Word)0;
        return r;
    }
    // Mask of the first n bits.
    __device__ __forceinline__ static BV low(int n) {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) {
            int lo = k * B;
            if (n >= lo + B) r.w[k] = ~(Word)0;
            else if (n <= lo) r.w[k] = 0;
            else r.w[k] = ((Word)1 << (n - lo)) - 1;
        }
        return r;
    }
    __device__ __forceinline__ BV shfl_from(int src) const {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) r.w[k] = shfl<Word>(w[k], src);
        return r;
    }
    // Remove bit q: bits above q move down by one.
    __device__ __forceinline__ BV drop_bit(int q) const {
        BV r;
#pragma unroll
        for (int k = 0; k < W; k++) {
            Word x = w[k];
            Word carry_in = (k + 1 < W) ? (w[(k + 1 < W) ? k + 1 : k] & 1) : 0;
            int lo = k * B;
            Word res;
            if (q >= lo + B) {
                res = x;  // q above this word: unchanged
            } else if (q < lo) {
                res = (x >> 1);  // whole word shifts down
            } else {
                int b = q - lo;
                Word below = (b == 0) ? (Word)0 : (x & (((Word)1 << b) - 1));
                Word above = (b == B - 1) ? (Word)0 : ((x >> (b + 1)) << b);
                res = below | above;
            }
            if (q < lo + B) res |= carry_in << (B - 1);
            r.w[k] = res;
        }
        return r;
    }
};

// ---- the warp-held term ----------------------------------------------------
template <typename Word, int W, int RPL>
struct WarpCH {
    using V = BV<Word, W>;
    static constexpr int B = 8 * sizeof(Word);
    static constexpr int MAXW = (32 * RPL < W * B) ? 32 * RPL : W * B;

    V G[RPL], F[RPL], M[RPL];  // this lane's rows
    uint32_t gam;              // 2 bits per slot
    V v, s;                    // uniform
    int phase;                 // uniform Z8
    int n;                     // uniform width
    int lane;
    int err;                   // uniform: 0 ok, else invariant id

    // ---- per-lane row access (slot index must be warp-uniform)
    __device__ __forceinline__ int gam_of(int sl) const { return (gam >> (2 * sl)) & 3; }
    __device__ __forceinline__ void gam_set(int sl, int g) {
        gam = (gam & ~(3u << (2 * sl))) | ((uint32_t)(g & 3) << (2 * sl));
    }
    __device__ __forceinline__ V pick(const V (&X)[RPL], int sl) const {
        V r = V::zero();
#pragma unroll
        for (int k = 0; k < RPL; k++) r = r | V::select(sl == k, X[k]);
        return r;
    }
    __device__ __forceinline__ V row(const V (&X)[RPL], int q) const {
        return pick(X, q >> 5).shfl_from(q & 31);
    }
    __device__ __forceinline__ int gam_row(int q) const {
        return shfl<uint32_t>((uint32_t)gam_of(q >> 5), q & 31);
    }
    __device__ __forceinline__ bool owns(int q) const { return lane == (q & 31); }
    // Row updates by a warp-uniform row index are written as masked updates of
    // every slot (not as a guarded write to slot q >> 5): a guarded write is
    // turned into an indexed one, which moves the term to local memory.
    __device__ __forceinline__ bool on_row(int q, int k) const { return owns(q) && (q >> 5) == k; }
    __device__ __forceinline__ void xor_row(V (&X)[RPL], int q, const V& val) {
#pragma unroll
        for (int k = 0; k < RPL; k++) X[k] ^= V::select(on_row(q, k), val);
    }

    __device__ __forceinline__ void init_zero(int width) {  // StabilizerCHForm::new
        n = width;
        err = 0;
        phase = 0;
        gam = 0;
        v = V::zero();
        s = V::zero();
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            int r = k * 32 + lane;
            G[k] = V::zero();
            F[k] = V::zero();
            M[k] = V::zero();
            if (r < width) {
                G[k].set(r, true);
                F[k].set(r, true);
            }
        }
    }

    // ---- left multiplications (form/left_multiplication/*.rs) --------------
    __device__ __forceinline__ void left_cx(int c, int t) {  // cx.rs:13-51
        V Gc = row(G, c), Ft = row(F, t), Mt = row(M, t);
        int gt = gam_row(t);
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            const bool on = on_row(c, k);
            const int dot = (M[k] & Ft).parity();
            gam_set(k, gam_of(k) + (on ? gt + 2 * dot : 0));
            F[k] ^= V::select(on, Ft);
            M[k] ^= V::select(on, Mt);
        }
        xor_row(G, t, Gc);
    }
    __device__ __forceinline__ void left_cz(int a, int b) {  // cz.rs:12-35
        V Ga = row(G, a), Gb = row(G, b);
        xor_row(M, a, Gb);
        xor_row(M, b, Ga);
    }
    __device__ __forceinline__ void left_s_like(int q, int dg) {  // s.rs:13-33 (dg = -1 S, +1 Sdg)
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            const bool on = on_row(q, k);
            M[k] ^= V::select(on, G[k]);
            gam_set(k, gam_of(k) + (on ? dg : 0));
        }
    }
    __device__ __forceinline__ void left_s(int q) { left_s_like(q, 3); }
    __device__ __forceinline__ void left_sdg(int q) { left_s_like(q, 1); }
    __device__ __forceinline__ void left_z(int q) {  // z.rs:7-14
#pragma unroll
        for (int k = 0; k < RPL; k++) gam_set(k, gam_of(k) + (on_row(q, k) ? 2 : 0));
    }
    __device__ __forceinline__ int beta_of(const V& Fq, const V& Mq) const {  // x.rs:20-29
        V b = (Mq & ~v & s) ^ (Fq & v & (Mq ^ s));
        return b.parity();
    }
    __device__ __forceinline__ void left_x(int q) {  // x.rs:12-48
        V Fq = row(F, q), Mq = row(M, q);
        int gq = gam_row(q);
        if (beta_of(Fq, Mq)) phase = (phase + 4) & 7;
        s ^= (Fq & ~v) ^ (Mq & v);
        phase = (phase + 2 * gq) & 7;
    }
    __device__ __forceinline__ void left_y(int q) {  // y.rs:4-11
        left_z(q);
        left_x(q);
        phase = (phase + 2) & 7;
    }

    // ---- right multiplications, lane-local (form/right_multiplication/*.rs)
    // right_cx(c, t): G[:,c] ^= G[:,t]; F[:,t] ^= F[:,c]; M[:,c] ^= M[:,t]
    __device__ __forceinline__ void right_cx(int c, int t) {
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            if (G[k].bit(t)) G[k].flip(c);
            if (F[k].bit(c)) F[k].flip(t);
            if (M[k].bit(t)) M[k].flip(c);
        }
    }
    // right_s (s.rs:8-24): M[:,q] ^= F[:,q]; γ_p -= 1 where F[p,q].
    __device__ __forceinline__ void right_s(int q) {
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            if (F[k].bit(q)) {
                M[k].flip(q);
                gam_set(k, gam_of(k) + 3);
            }
        }
    }

    // _resolve_superposition (resolve_superposition.rs:6-176); delta is Z8.
    __device__ __forceinline__ void resolve(const V& t, const V& u, int delta) {
        if (t == u) {  // handle_same_vecs_case :115-133
            if (delta == 4) {
                err = 1;
                return;
            }
            s = t;
            if (delta == 2) phase = (phase + 1) & 7;
            if (delta == 6) phase = (phase + 7) & 7;
            return;
        }
        V diff = t ^ u;
        V d0 = diff & ~v, d1 = diff & v;
        int pivot;
        if (!d0.any()) {
            // pivot = D1[0]; right_cx(i, pivot) for i in D1[1:].  Each step
            // changes only column i of G/M (from column pivot, never changed)
            // and column pivot of F (from column i, never changed), so the
            // sequence equals one masked update.
            pivot = d1.first();
            V rest = d1;
            rest.flip(pivot);
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                G[k] ^= V::select(G[k].bit(pivot), rest);
                if ((F[k] & rest).parity()) F[k].flip(pivot);
                M[k] ^= V::select(M[k].bit(pivot), rest);
            }
        } else {
            // pivot = D0[0]; right_cx(pivot, i) for i in D0[1:]: column pivot
            // of G/M accumulates columns i (unchanged), columns i of F take
            // column pivot (unchanged).  Then right_cz(pivot, i) for i in D1:
            // F is not modified by CZ, columns i ∉ {pivot} ∪ D0.
            pivot = d0.first();
            V rest = d0;
            rest.flip(pivot);
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                if ((G[k] & rest).parity()) G[k].flip(pivot);
                F[k] ^= V::select(F[k].bit(pivot), rest);
                if ((M[k] & rest).parity()) M[k].flip(pivot);
                // right_cz(pivot, i), i ∈ D1 (cz.rs:8-35)
                bool fp = F[k].bit(pivot);
                int par = (F[k] & d1).parity();
                if (par) M[k].flip(pivot);
                M[k] ^= V::select(fp, d1);
                if (fp && par) gam_set(k, gam_of(k) + 2);
            }
        }
        bool vp = v.bit(pivot);
        bool sp, vnew = vp;
        bool do_rs = false;
        int dph = 0;
        if (t.bit(pivot)) {
            s = u;
            switch (delta) {
                case 0: sp = false; vnew = !vp; break;
                case 4: sp = true; vnew = !vp; dph = 4; break;
                case 2:
                    if (vp) { dph = 1; sp = false; do_rs = true; }
                    else { sp = true; vnew = true; do_rs = true; dph = 2; }
                    break;
                default:
                    if (vp) { dph = 7; sp = true; do_rs = true; }
                    else { sp = false; vnew = true; do_rs = true; dph = 6; }
                    break;
            }
        } else {
            s = t;
            switch (delta) {
                case 0: sp = false; vnew = !vp; break;
                case 4: sp = true; vnew = !vp; break;
                case 2:
                    if (vp) { dph = 1; sp = true; do_rs = true; }
                    else { sp = false; vnew = true; do_rs = true; }
                    break;
                default:
                    if (vp) { dph = 7; sp = false; do_rs = true; }
                    else { sp = true; vnew = true; do_rs = true; }
                    break;
            }
        }
        s.set(pivot, sp);
        v.set(pivot, vnew);
        phase = (phase + dph) & 7;
        if (do_rs) right_s(pivot);
    }

    __device__ __forceinline__ void left_h(int q) {  // h.rs:13-65
        V Gq = row(G, q), Fq = row(F, q), Mq = row(M, q);
        int gq = gam_row(q);
        V t = s ^ (Gq & v);
        V u = s ^ (Fq & ~v) ^ (Mq & v);
        int alpha = (Gq & ~v & s).parity();
        int beta = beta_of(Fq, Mq);
        int delta = (2 * gq + ((alpha ^ beta) ? 4 : 0)) & 7;
        if (alpha) phase = (phase + 4) & 7;
        resolve(t, u, delta);
    }

    // project (project.rs:33-76): returns 1 deterministic, 0 random, -1 impossible.
    __device__ __forceinline__ int project(int q, bool outcome) {
        V Gq = row(G, q);
        V gv = Gq & v;
        if (!gv.any()) {
            int val = (Gq & s).parity();
            return (val == (int)outcome) ? 1 : -1;
        }
        V t = gv ^ s;
        int alpha = (Gq & ~v & s).parity();
        int delta = (alpha ^ (int)outcome) ? 4 : 0;
        V scopy = s;
        resolve(scopy, t, delta);
        return 0;
    }

    // Column c of a matrix as a warp-uniform bit vector (bit r = X[r][c]).
    __device__ __forceinline__ V column(const V (&X)[RPL], int c) const {
        V r = V::zero();
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            uint32_t b = __ballot_sync(FULL, X[k].bit(c));
            int lo = k * 32;
#pragma unroll
            for (int w = 0; w < W; w++) {
                if (lo >= w * B && lo < (w + 1) * B) r.w[w] |= (Word)b << (lo - w * B);
            }
        }
        return r & V::low(n);
    }

    // discard (discard.rs:21-181): q must already be projected onto |0⟩.
    __device__ void discard(int q) {
        V valid = V::low(n);
        if (v.bit(q) || s.bit(q)) {  // set_s_v_to_false :98-132
            V cleanm = ~v & ~s & valid;
            cleanm.set(q, false);
            int clean = cleanm.first();
            if (clean < 0) {
                V cand = ~v & s & valid;
                int f = cand.first();
                if (f >= 0) {
                    cand.flip(f);
                    int sc = cand.first();
                    if (sc >= 0) {
                        right_cx(f, sc);
                        s.set(sc, false);
                        clean = sc;
                    }
                }
            }
            if (clean < 0) {
                err = 2;  // CannotDiscardQubit
                return;
            }
            if (clean != q) {
                right_cx(clean, q);
                right_cx(q, clean);
                right_cx(clean, q);
                bool vq = v.bit(q), vc = v.bit(clean), sq = s.bit(q), sc2 = s.bit(clean);
                v.set(q, vc);
                v.set(clean, vq);
                s.set(q, sc2);
                s.set(clean, sq);
            }
        }
        // transform_g :135-161
        {
            V Gq = row(G, q);
            if (!Gq.bit(q)) {
                V m = Gq & valid;
                m.set(q, false);
                int pivot = m.first();
                if (pivot < 0) {
                    err = 3;
                    return;
                }
                right_cx(q, pivot);
            }
            // left_cx(q, i) for i ≠ q with G[i][q]: each step only changes row i
            // of G (and row q of F, M), so the set of rows is column q now.
            V colq = column(G, q);
            colq.set(q, false);
            while (colq.any()) {
                int i = colq.first();
                colq.flip(i);
                left_cx(q, i);
            }
            // right_cx(i, q) for i ≠ q with G[q][i]: column i of G/M takes column
            // q (unchanged), column q of F accumulates columns i (unchanged).
            Gq = row(G, q);
            V mask = Gq & valid;
            mask.set(q, false);
            if ((mask & v).any()) {
                err = 4;
                return;
            }
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                G[k] ^= V::select(G[k].bit(q), mask);
                if ((F[k] & mask).parity()) F[k].flip(q);
                M[k] ^= V::select(M[k].bit(q), mask);
            }
        }
        // transform_m :164-181
        {
            V colq = column(M, q);
            colq.set(q, false);
            while (colq.any()) {
                int i = colq.first();
                colq.flip(i);
                left_cx(q, i);
            }
            V Mq = row(M, q);
            if (Mq.bit(q)) left_sdg(q);
            Mq = row(M, q);
            V mask = Mq & valid;
            mask.set(q, false);
            // right_cz(q, i) for i in mask: F unchanged; column q of M
            // accumulates columns i of F, columns i of M take column q of F.
#pragma unroll
            for (int k = 0; k < RPL; k++) {
                bool fq = F[k].bit(q);
                int par = (F[k] & mask).parity();
                if (par) M[k].flip(q);
                M[k] ^= V::select(fq, mask);
                if (fq && par) gam_set(k, gam_of(k) + 2);
            }
        }
        remove_qubit(q);
    }

    // Removes row and column q (n -> n-1).
    __device__ __forceinline__ void remove_qubit(int q) {
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            G[k] = G[k].drop_bit(q);
            F[k] = F[k].drop_bit(q);
            M[k] = M[k].drop_bit(q);
        }
        v = v.drop_bit(q);
        s = s.drop_bit(q);
        // rows r >= q take row r+1
        V nG[RPL], nF[RPL], nM[RPL];
        uint32_t ngam = gam;
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            int src = (lane + 1) & 31;
            int ks = (lane == 31) ? k + 1 : k;  // slot of row r+1
            V g1 = G[k].shfl_from(src), f1 = F[k].shfl_from(src), m1 = M[k].shfl_from(src);
            uint32_t gm1 = shfl<uint32_t>((uint32_t)gam_of(k), src);
            V g2 = V::zero(), f2 = V::zero(), m2 = V::zero();
            uint32_t gm2 = 0;
            if (k + 1 < RPL) {
                g2 = G[(k + 1 < RPL) ? k + 1 : k].shfl_from(0);
                f2 = F[(k + 1 < RPL) ? k + 1 : k].shfl_from(0);
                m2 = M[(k + 1 < RPL) ? k + 1 : k].shfl_from(0);
                gm2 = shfl<uint32_t>((uint32_t)gam_of((k + 1 < RPL) ? k + 1 : k), 0);
            }
            int r = k * 32 + lane;
            bool moved = r >= q;
            bool from_next_slot = (ks != k);
            V gn = from_next_slot ? g2 : g1, fn = from_next_slot ? f2 : f1, mn = from_next_slot ? m2 : m1;
            uint32_t gmn = from_next_slot ? gm2 : gm1;
            if (r >= n - 1) {
                gn = V::zero();
                fn = V::zero();
                mn = V::zero();
                gmn = 0;
            }
            nG[k] = moved ? gn : G[k];
            nF[k] = moved ? fn : F[k];
            nM[k] = moved ? mn : M[k];
            if (moved) ngam = (ngam & ~(3u << (2 * k))) | ((gmn & 3) << (2 * k));
        }
#pragma unroll
        for (int k = 0; k < RPL; k++) {
            G[k] = nG[k];
            F[k] = nF[k];
            M[k] = nM[k];
        }
        gam = ngam;
        n -= 1;
    }
};

}  // namespace dev
}  // namespace nsg
