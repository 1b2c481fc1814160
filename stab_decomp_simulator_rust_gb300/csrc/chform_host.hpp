// chform_host.hpp — bit-packed host CH-form used for the |T⟩^{⊗t} expansion
// and for small host-side steps of the product library.
//
// A CH-form term ω·U_C·U_H|s⟩ (arXiv:1808.00128) of width w ≤ 128 with rows
// packed into two 64-bit words.  The update rules and their order are those of
// crates/stabilizer-ch-form-rust/src/form/{left_multiplication,
// right_multiplication,resolve_superposition,project,discard,kron}.rs, so the
// bits produced are the reference's bits.  γ is stored as an exponent of i
// (the reference's Z8 PhaseFactor divided by 2); `phase` is a Z8 exponent.
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

namespace nsg {

constexpr int HW = 2;      // words per row on the host
constexpr int HMAX = 128;  // maximum width

struct HostError {
    int code;
    int64_t a, b;
};

struct HRow {
    uint64_t w[HW];
};

static inline bool hbit(const uint64_t* v, int q) { return (v[q >> 6] >> (q & 63)) & 1ULL; }
static inline void hset(uint64_t* v, int q, bool b) {
    uint64_t m = 1ULL << (q & 63);
    if (b) v[q >> 6] |= m;
    else v[q >> 6] &= ~m;
}
static inline void hflip(uint64_t* v, int q) { v[q >> 6] ^= 1ULL << (q & 63); }
static inline int hparity(const uint64_t* a) {
    int p = 0;
    for (int k = 0; k < HW; k++) p ^= __builtin_popcountll(a[k]) & 1;
    return p;
}

struct HostCH {
    int n = 0;
    std::vector<HRow> G, F, M;
    std::vector<uint8_t> gam;  // exponent of i, mod 4
    uint64_t v[HW] = {0, 0}, s[HW] = {0, 0};
    int phase = 0;  // Z8

    static HostCH zero_state(int n) {  // form/mod.rs:44-65
        if (n <= 0) throw HostError{1 /*InvalidNumQubits*/, n, -1};
        if (n > HMAX) throw HostError{2 /*TooWide*/, n, HMAX};
        HostCH c;
        c.n = n;
        c.G.assign(n, HRow{{0, 0}});
        c.F.assign(n, HRow{{0, 0}});
        c.M.assign(n, HRow{{0, 0}});
        c.gam.assign(n, 0);
        for (int i = 0; i < n; i++) {
            hset(c.G[i].w, i, true);
            hset(c.F[i].w, i, true);
        }
        return c;
    }

    // ---- left multiplications (form/left_multiplication/*.rs)
    void left_cx(int c, int t) {  // cx.rs:13-51
        uint64_t d[HW];
        for (int k = 0; k < HW; k++) d[k] = M[c].w[k] & F[t].w[k];
        int dot = hparity(d);
        gam[c] = (uint8_t)((gam[c] + gam[t] + 2 * dot) & 3);
        for (int k = 0; k < HW; k++) {
            G[t].w[k] ^= G[c].w[k];
            F[c].w[k] ^= F[t].w[k];
            M[c].w[k] ^= M[t].w[k];
        }
    }
    void left_cz(int a, int b) {  // cz.rs:12-35
        for (int k = 0; k < HW; k++) M[a].w[k] ^= G[b].w[k];
        for (int k = 0; k < HW; k++) M[b].w[k] ^= G[a].w[k];
    }
    void left_s(int q) {  // s.rs:13-22
        for (int k = 0; k < HW; k++) M[q].w[k] ^= G[q].w[k];
        gam[q] = (uint8_t)((gam[q] + 3) & 3);
    }
    void left_sdg(int q) {  // s.rs:24-33
        for (int k = 0; k < HW; k++) M[q].w[k] ^= G[q].w[k];
        gam[q] = (uint8_t)((gam[q] + 1) & 3);
    }
    void left_z(int q) { gam[q] = (uint8_t)((gam[q] + 2) & 3); }  // z.rs:7-14
    int beta_of(int q) const {  // x.rs:20-29, h.rs:53-62
        uint64_t b[HW];
        for (int k = 0; k < HW; k++) {
            uint64_t mm = M[q].w[k], ff = F[q].w[k], vv = v[k], ss = s[k];
            b[k] = (mm & ~vv & ss) ^ (ff & vv & (mm ^ ss));
        }
        return hparity(b);
    }
    void left_x(int q) {  // x.rs:12-48
        if (beta_of(q)) phase = (phase + 4) & 7;
        for (int k = 0; k < HW; k++) s[k] ^= (F[q].w[k] & ~v[k]) ^ (M[q].w[k] & v[k]);
        phase = (phase + 2 * gam[q]) & 7;
    }
    void left_y(int q) {  // y.rs:4-11
        left_z(q);
        left_x(q);
        phase = (phase + 2) & 7;
    }

    // ---- right multiplications (form/right_multiplication/*.rs)
    void right_cx(int c, int t) {  // cx.rs:7-26 (G[:,c]^=G[:,t]; F[:,t]^=F[:,c]; M[:,c]^=M[:,t])
        for (int r = 0; r < n; r++) {
            if (hbit(G[r].w, t)) hflip(G[r].w, c);
            if (hbit(F[r].w, c)) hflip(F[r].w, t);
            if (hbit(M[r].w, t)) hflip(M[r].w, c);
        }
    }
    void right_cz(int a, int b) {  // cz.rs:8-35
        for (int r = 0; r < n; r++) {
            bool fa = hbit(F[r].w, a), fb = hbit(F[r].w, b);
            if (fb) hflip(M[r].w, a);
            if (fa) hflip(M[r].w, b);
            if (fa && fb) gam[r] = (uint8_t)((gam[r] + 2) & 3);
        }
    }
    void right_s(int q) {  // s.rs:8-24
        for (int r = 0; r < n; r++) {
            if (hbit(F[r].w, q)) {
                hflip(M[r].w, q);
                gam[r] = (uint8_t)((gam[r] + 3) & 3);
            }
        }
    }

    // _resolve_superposition (resolve_superposition.rs:6-176); delta is Z8.
    void resolve(const uint64_t* t, const uint64_t* u, int delta) {
        bool same = true;
        for (int k = 0; k < HW; k++) same &= (t[k] == u[k]);
        if (same) {
            if (delta == 4) throw HostError{3 /*invariant*/, 1, -1};
            std::memcpy(s, t, sizeof(s));
            if (delta == 2) phase = (phase + 1) & 7;
            if (delta == 6) phase = (phase + 7) & 7;
            return;
        }
        std::vector<int> d0, d1;
        for (int i = 0; i < n; i++) {
            if (hbit(t, i) != hbit(u, i)) (hbit(v, i) ? d1 : d0).push_back(i);
        }
        int pivot;
        if (d0.empty()) {
            pivot = d1[0];
            for (size_t k = 1; k < d1.size(); k++) right_cx(d1[k], pivot);
        } else {
            pivot = d0[0];
            for (size_t k = 1; k < d0.size(); k++) right_cx(pivot, d0[k]);
            for (int i : d1) right_cz(pivot, i);
        }
        bool vp = hbit(v, pivot);
        if (hbit(t, pivot)) {
            std::memcpy(s, u, sizeof(s));
            switch (delta) {
                case 0: hset(s, pivot, false); hset(v, pivot, !vp); break;
                case 4: hset(s, pivot, true); hset(v, pivot, !vp); phase = (phase + 4) & 7; break;
                case 2:
                    if (vp) { phase = (phase + 1) & 7; hset(s, pivot, false); right_s(pivot); }
                    else { hset(s, pivot, true); hset(v, pivot, true); right_s(pivot); phase = (phase + 2) & 7; }
                    break;
                default:  // 6
                    if (vp) { phase = (phase + 7) & 7; hset(s, pivot, true); right_s(pivot); }
                    else { hset(s, pivot, false); hset(v, pivot, true); right_s(pivot); phase = (phase + 6) & 7; }
                    break;
            }
        } else {
            std::memcpy(s, t, sizeof(s));
            switch (delta) {
                case 0: hset(s, pivot, false); hset(v, pivot, !vp); break;
                case 4: hset(s, pivot, true); hset(v, pivot, !vp); break;
                case 2:
                    if (vp) { phase = (phase + 1) & 7; hset(s, pivot, true); right_s(pivot); }
                    else { hset(s, pivot, false); hset(v, pivot, true); right_s(pivot); }
                    break;
                default:  // 6
                    if (vp) { phase = (phase + 7) & 7; hset(s, pivot, false); right_s(pivot); }
                    else { hset(s, pivot, true); hset(v, pivot, true); right_s(pivot); }
                    break;
            }
        }
    }

    void left_h(int q) {  // h.rs:13-65
        uint64_t t[HW], u[HW], a[HW];
        for (int k = 0; k < HW; k++) {
            uint64_t gg = G[q].w[k], ff = F[q].w[k], mm = M[q].w[k], vv = v[k], ss = s[k];
            t[k] = ss ^ (gg & vv);
            u[k] = ss ^ (ff & ~vv) ^ (mm & vv);
            a[k] = gg & ~vv & ss;
        }
        int alpha = hparity(a), beta = beta_of(q);
        int delta = (2 * gam[q] + ((alpha ^ beta) ? 4 : 0)) & 7;
        if (alpha) phase = (phase + 4) & 7;
        resolve(t, u, delta);
    }

    // project (project.rs:33-76): 1 deterministic, 0 random, -1 impossible.
    int project(int q, bool outcome) {
        uint64_t gv[HW], a[HW], gs[HW];
        bool det = true;
        for (int k = 0; k < HW; k++) {
            gv[k] = G[q].w[k] & v[k];
            if (gv[k]) det = false;
            gs[k] = G[q].w[k] & s[k];
            a[k] = G[q].w[k] & ~v[k] & s[k];
        }
        if (det) return (hparity(gs) == (int)outcome) ? 1 : -1;
        uint64_t t[HW], scopy[HW];
        for (int k = 0; k < HW; k++) {
            t[k] = gv[k] ^ s[k];
            scopy[k] = s[k];
        }
        int delta = (hparity(a) ^ (int)outcome) ? 4 : 0;
        resolve(scopy, t, delta);
        return 0;
    }

    // discard (discard.rs:21-181)
    void discard(int q) {
        if (hbit(v, q) || hbit(s, q)) {  // set_s_v_to_false :98-132
            int clean = -1;
            for (int i = 0; i < n; i++)
                if (i != q && !hbit(v, i) && !hbit(s, i)) { clean = i; break; }
            if (clean < 0) {
                int f = -1, sc = -1;
                for (int i = 0; i < n; i++)
                    if (!hbit(v, i) && hbit(s, i)) {
                        if (f < 0) f = i;
                        else { sc = i; break; }
                    }
                if (f >= 0 && sc >= 0) {
                    right_cx(f, sc);
                    hset(s, sc, false);
                    clean = sc;
                }
            }
            if (clean < 0) throw HostError{4 /*CannotDiscard*/, q, -1};
            if (clean != q) {
                right_cx(clean, q);
                right_cx(q, clean);
                right_cx(clean, q);
                bool vq = hbit(v, q), vc = hbit(v, clean), sq = hbit(s, q), sc2 = hbit(s, clean);
                hset(v, q, vc); hset(v, clean, vq);
                hset(s, q, sc2); hset(s, clean, sq);
            }
        }
        // transform_g :135-161
        if (!hbit(G[q].w, q)) {
            int pivot = -1;
            for (int i = 0; i < n; i++)
                if (i != q && hbit(G[q].w, i)) { pivot = i; break; }
            if (pivot < 0) throw HostError{3, 3, -1};
            right_cx(q, pivot);
        }
        for (int i = 0; i < n; i++)
            if (i != q && hbit(G[i].w, q)) left_cx(q, i);
        for (int i = 0; i < n; i++) {
            if (i != q && hbit(G[q].w, i)) {
                if (hbit(v, i)) throw HostError{3, 4, -1};
                right_cx(i, q);
            }
        }
        // transform_m :164-181
        for (int i = 0; i < n; i++)
            if (i != q && hbit(M[i].w, q)) left_cx(q, i);
        if (hbit(M[q].w, q)) left_sdg(q);
        for (int i = 0; i < n; i++)
            if (i != q && hbit(M[q].w, i)) right_cz(q, i);
        // remove row/column q
        auto drop_bit = [q](uint64_t* w) {
            uint64_t out[HW] = {0, 0};
            int o = 0;
            for (int i = 0; i < HMAX; i++) {
                if (i == q) continue;
                if (hbit(w, i)) hset(out, o, true);
                o++;
            }
            std::memcpy(w, out, sizeof(out));
        };
        G.erase(G.begin() + q);
        F.erase(F.begin() + q);
        M.erase(M.begin() + q);
        gam.erase(gam.begin() + q);
        n -= 1;
        for (int r = 0; r < n; r++) {
            drop_bit(G[r].w);
            drop_bit(F[r].w);
            drop_bit(M[r].w);
        }
        drop_bit(v);
        drop_bit(s);
    }

    // kron (kron.rs:12-59)
    static HostCH kron(const HostCH& a, const HostCH& b) {
        HostCH r = zero_state(a.n + b.n);
        auto shifted = [](const uint64_t* w, int sh, uint64_t* out) {
            for (int i = 0; i < HMAX - sh; i++)
                if (hbit(w, i)) hset(out, i + sh, true);
        };
        for (int i = 0; i < a.n; i++) {
            r.G[i] = a.G[i];
            r.F[i] = a.F[i];
            r.M[i] = a.M[i];
            r.gam[i] = a.gam[i];
        }
        for (int i = 0; i < b.n; i++) {
            HRow g{{0, 0}}, f{{0, 0}}, m{{0, 0}};
            shifted(b.G[i].w, a.n, g.w);
            shifted(b.F[i].w, a.n, f.w);
            shifted(b.M[i].w, a.n, m.w);
            r.G[a.n + i] = g;
            r.F[a.n + i] = f;
            r.M[a.n + i] = m;
            r.gam[a.n + i] = b.gam[i];
        }
        uint64_t vv[HW] = {0, 0}, ss[HW] = {0, 0};
        std::memcpy(vv, a.v, sizeof(vv));
        std::memcpy(ss, a.s, sizeof(ss));
        shifted(b.v, a.n, vv);
        shifted(b.s, a.n, ss);
        std::memcpy(r.v, vv, sizeof(vv));
        std::memcpy(r.s, ss, sizeof(ss));
        r.phase = (a.phase + b.phase) & 7;
        return r;
    }
};

// Exact coefficient phase·2^(-r/2) (crates/necstar/src/state/types/scalar.rs:12-15).
struct HScalar {
    int k;      // Z8
    int32_t r;  // exponent numerator
};

struct HostDecomp {
    int n = 0;
    std::vector<HostCH> terms;
    std::vector<HScalar> coef;
};

// ---- cat and T-tensor states (crates/necstar/src/state/magic_states/cat_state.rs:16-188,
// t_state.rs:29-71).
static HostCH zero_minus_i_one(int m) {
    HostCH c = HostCH::zero_state(m);
    c.left_h(0);
    for (int i = 1; i < m; i++) c.left_cx(0, i);
    c.left_sdg(0);
    return c;
}
static HostCH even_parity(int m) {
    HostCH c = HostCH::zero_state(m);
    for (int i = 0; i < m - 1; i++) c.left_h(i);
    for (int i = 0; i < m - 1; i++) c.left_cx(i, m - 1);
    return c;
}
static HostCH even_parity_flipped(int m) {
    HostCH c = even_parity(m);
    for (int i = 0; i < m; i++)
        for (int j = i + 1; j < m; j++) c.left_cz(i, j);
    return c;
}

static HostDecomp cat_state(int m) {
    HostDecomp d;
    switch (m) {
        case 1:
            d.n = 1;
            d.terms = {HostCH::zero_state(1)};
            d.coef = {{0, 0}};
            return d;
        case 2: {
            HostCH c = HostCH::zero_state(2);
            c.left_h(0);
            c.left_cx(0, 1);
            c.left_s(1);
            d.n = 2;
            d.terms = {c};
            d.coef = {{0, 0}};
            return d;
        }
        case 4:
            d.n = 4;
            d.terms = {zero_minus_i_one(4), even_parity(4)};
            d.coef = {{7, 1}, {2, 0}};
            return d;
        case 6:
            d.n = 6;
            d.terms = {zero_minus_i_one(6), even_parity(6), even_parity_flipped(6)};
            d.coef = {{0, 2}, {3, 1}, {5, 1}};
            return d;
        case 3:
        case 5: {
            d = cat_state(m + 1);
            for (auto& c : d.terms) {
                c.project(m, false);  // deterministic or random; never impossible here
                c.discard(m);
            }
            d.n = m;
            return d;
        }
        default: {
            if (m <= 0) throw HostError{1, m, -1};
            HostDecomp a = cat_state(m - 4), b = cat_state(6);
            d.n = m;
            int q0 = m - 5, q1 = m - 4;
            for (size_t i = 0; i < a.terms.size(); i++)
                for (size_t j = 0; j < b.terms.size(); j++) {
                    HostCH c = HostCH::kron(a.terms[i], b.terms[j]);
                    c.left_sdg(q0);
                    c.left_cx(q0, q1);
                    c.left_h(q0);
                    c.project(q0, false);
                    c.project(q1, false);
                    c.discard(q1);
                    c.discard(q0);
                    d.terms.push_back(std::move(c));
                    d.coef.push_back({(a.coef[i].k + b.coef[j].k) & 7, a.coef[i].r + b.coef[j].r});
                }
            return d;
        }
    }
}

static HostDecomp t_tensor_state(int t) {
    HostDecomp cat = cat_state(t);
    HostDecomp d;
    d.n = cat.n;
    size_t chi = cat.terms.size();
    d.terms.reserve(2 * chi);
    d.coef.reserve(2 * chi);
    for (size_t i = 0; i < chi; i++) {
        d.terms.push_back(cat.terms[i]);
        d.coef.push_back({cat.coef[i].k, cat.coef[i].r + 1});  // × ONE_OVER_SQRT_2
    }
    for (size_t i = 0; i < chi; i++) {
        HostCH c = cat.terms[i];
        c.left_x(0);
        c.left_s(0);
        d.terms.push_back(std::move(c));
        d.coef.push_back({(cat.coef[i].k + 7) & 7, cat.coef[i].r + 1});  // × e^{-iπ/4}
    }
    return d;
}

}  // namespace nsg
