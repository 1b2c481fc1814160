// necstar_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of the reference's stabilizer-decomposition path
// (mutekichi/stab-decomp-simulator-rust), one `bool` byte per tableau bit
// exactly as the reference stores it (ndarray::Array2<bool>,
// crates/stabilizer-ch-form-rust/src/form/mod.rs:12-22), with the same rule
// order, pivot choices and term order.  The CUDA path is checked against it:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// it.  The product library never links or calls it.
//
// The reference is Rust and no Rust toolchain was available to build it
// (no cargo/rustc), so this is a port.  Its outputs are pinned against the
// reference's own known-answer tests (T-tensor statevectors t=1..11, the
// Toffoli-state expectation values, the χ=2 statevector, the doctest
// amplitudes, the gate-API error variants) and against an independent dense
// statevector simulator restated from
// crates/stabilizer-ch-form-rust/tests/common/mod.rs:108-200.
//
// Floating point follows the reference's f64 arithmetic: PhaseFactor::to_complex
// uses cos/sin of k·π/4 and Scalar::to_complex uses powf(2, -r/2)
// (crates/necstar/src/state/types/scalar.rs:30-38).  Build with
// -ffp-contract=off so no FMA contraction changes the rounding.
//
// Seeded RNG streams of the reference come from third-party crates pinned in
// Cargo.lock and not part of the reference tree: rand 0.8.5 StdRng
// (= rand_chacha 0.3.1 ChaCha12Rng) and rand_distr 0.4.3 Binomial.  The
// StdRng stream is restated here from the published ChaCha algorithm
// (Bernstein 2008) in StdRng::from_seed's layout, together with rand's
// conversions to f64 and to a u8 drawn from 0..=1; it is pinned to the
// ChaCha known-answer vectors (RFC 7539 §2.3.2 and A.1, the eSTREAM 12-round
// zero-key block).  With it, measure() and random_clifford() draw what the
// reference draws for a given seed.  Binomial is not restated; sampling is
// compared by distribution against the exact marginal.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <random>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../include/necstar_gpu.h"

namespace orc {

using cplx = std::complex<double>;

// ---------------------------------------------------------------------------
// Errors (crates/stabilizer-ch-form-rust/src/error/mod.rs:7-67,
// crates/necstar/src/error/mod.rs:10-91)
struct Error {
    int code;
    int64_t a, b, c;
    std::string msg;
};

[[noreturn]] static void fail(int code, int64_t a = -1, int64_t b = -1, const std::string& msg = "") {
    throw Error{code, a, b, -1, msg};
}

// ---------------------------------------------------------------------------
// Complex arithmetic written out so the rounding is the textbook formula used
// by num_complex (no Annex G special-casing, no contraction).
static inline cplx cmul(cplx a, cplx b) {
    return cplx(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}

// PhaseFactor::to_complex (form/types/phase_factor.rs:18-21 and
// necstar state/types/phase_factor.rs:21-24): angle = k·FRAC_PI_4.
static inline cplx phase_to_complex(int k) {
    const double FRAC_PI_4 = 0.78539816339744830961566084581987572;
    double ang = (double)k * FRAC_PI_4;
    return cplx(std::cos(ang), std::sin(ang));
}

// Exact scalar phase·2^(-r/2) or zero (state/types/scalar.rs:12-15).
struct Scalar {
    bool zero;
    int k;      // Z8
    int64_t r;  // isize in the reference
};

static inline Scalar scalar_mul(Scalar a, Scalar b) {
    if (a.zero || b.zero) return Scalar{true, 0, 0};
    return Scalar{false, (a.k + b.k) % 8, a.r + b.r};
}
static inline Scalar scalar_conj(Scalar a) {
    if (a.zero) return a;
    return Scalar{false, (8 - a.k) % 8, a.r};
}
// Scalar::to_complex (state/types/scalar.rs:30-38)
static inline cplx scalar_to_complex(Scalar a) {
    if (a.zero) return cplx(0.0, 0.0);
    double norm = std::pow(2.0, -((double)a.r) / 2.0);
    cplx p = phase_to_complex(a.k);
    return cplx(p.real() * norm, p.imag() * norm);
}
// Amplify::amplify (state/types/scalar.rs:108-119): r -= factor.
static inline Scalar scalar_amplify(Scalar a, int64_t f) {
    if (a.zero) return a;
    return Scalar{false, a.k, a.r - f};
}

// ---------------------------------------------------------------------------
// CH-form state (crates/stabilizer-ch-form-rust/src/form/mod.rs:12-22).
struct ChForm {
    int n = 0;
    std::vector<uint8_t> G, F, M;  // n×n row-major bools
    std::vector<uint8_t> gamma;    // Z8 exponents, always in {0,2,4,6}
    std::vector<uint8_t> v, s;
    cplx omega{1.0, 0.0};
    int phase = 0;  // Z8

    uint8_t& g(int i, int j) { return G[(size_t)i * n + j]; }
    uint8_t& f(int i, int j) { return F[(size_t)i * n + j]; }
    uint8_t& m(int i, int j) { return M[(size_t)i * n + j]; }
    uint8_t g(int i, int j) const { return G[(size_t)i * n + j]; }
    uint8_t f(int i, int j) const { return F[(size_t)i * n + j]; }
    uint8_t m(int i, int j) const { return M[(size_t)i * n + j]; }
};

// StabilizerCHForm::new (form/mod.rs:44-65)
static ChForm ch_new(int n) {
    if (n == 0) fail(NSG_ERR_INVALID_NUM_QUBITS, 0);
    ChForm c;
    c.n = n;
    c.G.assign((size_t)n * n, 0);
    c.F.assign((size_t)n * n, 0);
    c.M.assign((size_t)n * n, 0);
    for (int i = 0; i < n; i++) {
        c.g(i, i) = 1;
        c.f(i, i) = 1;
    }
    c.gamma.assign(n, 0);
    c.v.assign(n, 0);
    c.s.assign(n, 0);
    c.omega = cplx(1.0, 0.0);
    c.phase = 0;
    return c;
}

// xor_rows / xor_columns (form/matrix_operations.rs:7-29)
static void xor_rows(std::vector<uint8_t>& mat, int n, int target, int source) {
    for (int j = 0; j < n; j++) mat[(size_t)target * n + j] ^= mat[(size_t)source * n + j];
}
static void xor_cols(std::vector<uint8_t>& mat, int n, int target, int source) {
    for (int i = 0; i < n; i++) mat[(size_t)i * n + target] ^= mat[(size_t)i * n + source];
}

static inline void check_q(const ChForm& c, int q) {
    if (q < 0 || q >= c.n) fail(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, q, c.n);
}
static inline void check_qq(const ChForm& c, int a, int b) {
    check_q(c, a);
    check_q(c, b);
    if (a == b) fail(NSG_ERR_DUPLICATE_QUBIT_INDICES, a);
}

// left_multiply_cx (form/left_multiplication/cx.rs:13-51)
static void left_cx(ChForm& c, int control, int target) {
    check_qq(c, control, target);
    int n = c.n;
    uint8_t dot = 0;
    for (int j = 0; j < n; j++) dot ^= (c.m(control, j) & c.f(target, j));
    int gc = c.gamma[control], gt = c.gamma[target];
    c.gamma[control] = (uint8_t)((gc + gt + (dot ? 4 : 0)) % 8);
    xor_rows(c.G, n, target, control);
    xor_rows(c.F, n, control, target);
    xor_rows(c.M, n, control, target);
}

// left_multiply_cz (form/left_multiplication/cz.rs:12-35)
static void left_cz(ChForm& c, int q1, int q2) {
    check_qq(c, q1, q2);
    int n = c.n;
    for (int j = 0; j < n; j++) c.m(q1, j) ^= c.g(q2, j);
    for (int j = 0; j < n; j++) c.m(q2, j) ^= c.g(q1, j);
}

// left_multiply_s / left_multiply_sdg (form/left_multiplication/s.rs:13-33)
static void left_s(ChForm& c, int q) {
    check_q(c, q);
    for (int j = 0; j < c.n; j++) c.m(q, j) ^= c.g(q, j);
    c.gamma[q] = (uint8_t)((c.gamma[q] + 6) % 8);  // × MINUS_I
}
static void left_sdg(ChForm& c, int q) {
    check_q(c, q);
    for (int j = 0; j < c.n; j++) c.m(q, j) ^= c.g(q, j);
    c.gamma[q] = (uint8_t)((c.gamma[q] + 2) % 8);  // × PLUS_I
}

// left_multiply_x (form/left_multiplication/x.rs:12-48)
static void left_x(ChForm& c, int q) {
    check_q(c, q);
    int n = c.n;
    uint8_t beta = 0;
    for (int j = 0; j < n; j++) {
        uint8_t mm = c.m(q, j), ff = c.f(q, j), vv = c.v[j], ss = c.s[j];
        uint8_t t1 = mm & (uint8_t)!vv & ss;
        uint8_t t23 = ff & vv & (mm ^ ss);
        beta ^= t1 ^ t23;
    }
    if (beta) c.phase = (c.phase + 4) % 8;
    for (int j = 0; j < n; j++) {
        uint8_t vv = c.v[j];
        c.s[j] ^= (c.f(q, j) & (uint8_t)!vv) ^ (c.m(q, j) & vv);
    }
    c.phase = (c.phase + c.gamma[q]) % 8;
}

// left_multiply_z (form/left_multiplication/z.rs:7-14)
static void left_z(ChForm& c, int q) {
    check_q(c, q);
    c.gamma[q] = (uint8_t)((c.gamma[q] + 4) % 8);
}

// left_multiply_y (form/left_multiplication/y.rs:4-11)
static void left_y(ChForm& c, int q) {
    left_z(c, q);
    left_x(c, q);
    c.phase = (c.phase + 2) % 8;
}

// right_multiply_cx (form/right_multiplication/cx.rs:7-26) — follows the code:
// G[:,control] ^= G[:,target]; F[:,target] ^= F[:,control]; M[:,control] ^= M[:,target].
static void right_cx(ChForm& c, int control, int target) {
    check_qq(c, control, target);
    xor_cols(c.G, c.n, control, target);
    xor_cols(c.F, c.n, target, control);
    xor_cols(c.M, c.n, control, target);
}

// right_multiply_cz (form/right_multiplication/cz.rs:8-35)
static void right_cz(ChForm& c, int q1, int q2) {
    check_qq(c, q1, q2);
    int n = c.n;
    std::vector<uint8_t> f1(n), f2(n);
    for (int p = 0; p < n; p++) {
        f1[p] = c.f(p, q1);
        f2[p] = c.f(p, q2);
    }
    for (int p = 0; p < n; p++) c.m(p, q1) ^= f2[p];
    for (int p = 0; p < n; p++) c.m(p, q2) ^= f1[p];
    for (int p = 0; p < n; p++)
        if (f1[p] && f2[p]) c.gamma[p] = (uint8_t)((c.gamma[p] + 4) % 8);
}

// right_multiply_s (form/right_multiplication/s.rs:8-24)
static void right_s(ChForm& c, int q) {
    check_q(c, q);
    int n = c.n;
    for (int p = 0; p < n; p++) c.m(p, q) ^= c.f(p, q);
    for (int p = 0; p < n; p++)
        if (c.f(p, q)) c.gamma[p] = (uint8_t)((c.gamma[p] + 6) % 8);
}

// _resolve_superposition (form/resolve_superposition.rs:6-176)
static void resolve(ChForm& c, const std::vector<uint8_t>& t, const std::vector<uint8_t>& u, int delta) {
    int n = c.n;
    if (t == u) {  // handle_same_vecs_case :115-133
        switch (delta) {
            case 0: c.s = t; break;
            case 4: fail(NSG_ERR_DEVICE_INVARIANT, 1, -1, "Inconsistent state: superposition with -1 coefficient.");
            case 2: c.s = t; c.phase = (c.phase + 1) % 8; break;
            case 6: c.s = t; c.phase = (c.phase + 7) % 8; break;
            default: fail(NSG_ERR_DEVICE_INVARIANT, 2);
        }
        return;
    }
    // get_differing_indices :135-153
    std::vector<int> d0, d1;
    for (int i = 0; i < n; i++) {
        if (t[i] != u[i]) {
            if (c.v[i]) d1.push_back(i);
            else d0.push_back(i);
        }
    }
    // apply_basis_transform_circuit :155-176
    int pivot;
    if (d0.empty()) {
        pivot = d1[0];
        for (size_t k = 1; k < d1.size(); k++) right_cx(c, d1[k], pivot);
    } else {
        pivot = d0[0];
        for (size_t k = 1; k < d0.size(); k++) right_cx(c, pivot, d0[k]);
        for (int i : d1) right_cz(c, pivot, i);
    }
    if (t[pivot]) {
        c.s = u;
        switch (delta) {
            case 0: c.s[pivot] = 0; c.v[pivot] = !c.v[pivot]; break;
            case 4: c.s[pivot] = 1; c.v[pivot] = !c.v[pivot]; c.phase = (c.phase + 4) % 8; break;
            case 2:
                if (c.v[pivot]) {
                    c.phase = (c.phase + 1) % 8;
                    c.s[pivot] = 0;
                    right_s(c, pivot);
                } else {
                    c.s[pivot] = 1;
                    c.v[pivot] = 1;
                    right_s(c, pivot);
                    c.phase = (c.phase + 2) % 8;
                }
                break;
            case 6:
                if (c.v[pivot]) {
                    c.phase = (c.phase + 7) % 8;
                    c.s[pivot] = 1;
                    right_s(c, pivot);
                } else {
                    c.s[pivot] = 0;
                    c.v[pivot] = 1;
                    right_s(c, pivot);
                    c.phase = (c.phase + 6) % 8;
                }
                break;
            default: fail(NSG_ERR_DEVICE_INVARIANT, 2);
        }
    } else {
        c.s = t;
        switch (delta) {
            case 0: c.s[pivot] = 0; c.v[pivot] = !c.v[pivot]; break;
            case 4: c.s[pivot] = 1; c.v[pivot] = !c.v[pivot]; break;
            case 2:
                if (c.v[pivot]) {
                    c.phase = (c.phase + 1) % 8;
                    c.s[pivot] = 1;
                    right_s(c, pivot);
                } else {
                    c.s[pivot] = 0;
                    c.v[pivot] = 1;
                    right_s(c, pivot);
                }
                break;
            case 6:
                if (c.v[pivot]) {
                    c.phase = (c.phase + 7) % 8;
                    c.s[pivot] = 0;
                    right_s(c, pivot);
                } else {
                    c.s[pivot] = 1;
                    c.v[pivot] = 1;
                    right_s(c, pivot);
                }
                break;
            default: fail(NSG_ERR_DEVICE_INVARIANT, 2);
        }
    }
}

// left_multiply_h + prepare_h_superposition_args (form/left_multiplication/h.rs:13-65)
static void left_h(ChForm& c, int q) {
    check_q(c, q);
    int n = c.n;
    std::vector<uint8_t> t(n), u(n);
    uint8_t alpha = 0, beta = 0;
    for (int j = 0; j < n; j++) {
        uint8_t gg = c.g(q, j), ff = c.f(q, j), mm = c.m(q, j), vv = c.v[j], ss = c.s[j];
        t[j] = ss ^ (gg & vv);
        u[j] = ss ^ (ff & (uint8_t)!vv) ^ (mm & vv);
        alpha ^= (gg & (uint8_t)!vv & ss);
        uint8_t t1 = mm & (uint8_t)!vv & ss;
        uint8_t t23 = ff & vv & (mm ^ ss);
        beta ^= t1 ^ t23;
    }
    int delta = (alpha ^ beta) ? (c.gamma[q] + 4) % 8 : c.gamma[q];
    if (alpha) c.phase = (c.phase + 4) % 8;
    resolve(c, t, u, delta);
}

static void left_sqrt_x(ChForm& c, int q) {  // sqrt_x.rs:6-10
    left_h(c, q);
    left_s(c, q);
    left_h(c, q);
}
static void left_sqrt_xdg(ChForm& c, int q) {  // sqrt_x.rs:12-16
    left_h(c, q);
    left_sdg(c, q);
    left_h(c, q);
}
static void left_swap(ChForm& c, int a, int b) {  // swap.rs:7-24
    check_qq(c, a, b);
    left_cx(c, a, b);
    left_cx(c, b, a);
    left_cx(c, a, b);
}

// apply_gate (form/gate_application.rs:162-177), Clifford opcodes only.
static void apply_clifford(ChForm& c, const nsg_gate& g) {
    int a = (int)g.q0, b = (int)g.q1;
    switch (g.op) {
        case NSG_GATE_H: left_h(c, a); break;
        case NSG_GATE_X: left_x(c, a); break;
        case NSG_GATE_Y: left_y(c, a); break;
        case NSG_GATE_Z: left_z(c, a); break;
        case NSG_GATE_S: left_s(c, a); break;
        case NSG_GATE_SDG: left_sdg(c, a); break;
        case NSG_GATE_SQRT_X: left_sqrt_x(c, a); break;
        case NSG_GATE_SQRT_XDG: left_sqrt_xdg(c, a); break;
        case NSG_GATE_CX: left_cx(c, a, b); break;
        case NSG_GATE_CZ: left_cz(c, a, b); break;
        case NSG_GATE_SWAP: left_swap(c, a, b); break;
        default: fail(NSG_ERR_GATE_NOT_CLIFFORD, g.op);
    }
}

// get_qubit_state (form/get_qubit_state.rs:6-31): returns -1 superposition, else value.
static int qubit_state(const ChForm& c, int q) {
    check_q(c, q);
    bool determined = true;
    for (int j = 0; j < c.n; j++)
        if (c.g(q, j) && c.v[j]) determined = false;
    if (!determined) return -1;
    int acc = 0;
    for (int j = 0; j < c.n; j++)
        if (c.g(q, j) && c.s[j]) acc++;
    return acc % 2;
}

// project (form/project.rs:33-76): true = deterministic.
static bool project(ChForm& c, int q, bool outcome) {
    check_q(c, q);
    int st = qubit_state(c, q);
    if (st >= 0) {
        if ((st == 1) != outcome) fail(NSG_ERR_IMPOSSIBLE_PROJECTION, q, outcome ? 1 : 0);
        return true;
    }
    int n = c.n;
    std::vector<uint8_t> t(n);
    int cnt = 0;
    for (int j = 0; j < n; j++) {
        t[j] = (c.g(q, j) & c.v[j]) ^ c.s[j];
        if (c.g(q, j) && !c.v[j] && c.s[j]) cnt++;
    }
    bool alpha = (cnt % 2) != 0;
    int delta = (alpha ^ outcome) ? 4 : 0;
    std::vector<uint8_t> s_copy = c.s;
    resolve(c, s_copy, t, delta);
    return false;
}

// discard helpers (form/discard.rs:98-181)
static void set_s_v_to_false(ChForm& c, int q) {
    if (!c.v[q] && !c.s[q]) return;
    int n = c.n;
    int clean = -1;
    for (int i = 0; i < n; i++)
        if (i != q && !c.v[i] && !c.s[i]) { clean = i; break; }
    if (clean < 0) {
        int first = -1, second = -1;
        for (int i = 0; i < n; i++) {
            if (!c.v[i] && c.s[i]) {
                if (first < 0) first = i;
                else { second = i; break; }
            }
        }
        if (first >= 0 && second >= 0) {
            right_cx(c, first, second);
            c.s[second] = 0;
            clean = second;
        }
    }
    if (clean < 0) fail(NSG_ERR_CANNOT_DISCARD_QUBIT, q);
    if (clean == q) return;
    right_cx(c, clean, q);
    right_cx(c, q, clean);
    right_cx(c, clean, q);
    std::swap(c.v[q], c.v[clean]);
    std::swap(c.s[q], c.s[clean]);
}

static void transform_g(ChForm& c, int q) {
    int n = c.n;
    if (!c.g(q, q)) {
        int pivot = -1;
        for (int i = 0; i < n; i++)
            if (i != q && c.g(q, i)) { pivot = i; break; }
        if (pivot < 0) fail(NSG_ERR_DEVICE_INVARIANT, 3, -1, "Cannot zero G row due to G matrix state.");
        right_cx(c, q, pivot);
    }
    for (int i = 0; i < n; i++)
        if (i != q && c.g(i, q)) left_cx(c, q, i);
    for (int i = 0; i < n; i++) {
        if (i != q && c.g(q, i)) {
            if (c.v[i]) fail(NSG_ERR_DEVICE_INVARIANT, 4, -1, "Cannot zero G column due to v vector state.");
            right_cx(c, i, q);
        }
    }
}

static void transform_m(ChForm& c, int q) {
    int n = c.n;
    for (int i = 0; i < n; i++)
        if (i != q && c.m(i, q)) left_cx(c, q, i);
    if (c.m(q, q)) left_sdg(c, q);
    for (int i = 0; i < n; i++)
        if (i != q && c.m(q, i)) right_cz(c, q, i);
}

// discard (form/discard.rs:21-44)
static void discard(ChForm& c, int q) {
    check_q(c, q);
    set_s_v_to_false(c, q);
    transform_g(c, q);
    transform_m(c, q);
    int n = c.n, nn = n - 1;
    auto shrink = [&](const std::vector<uint8_t>& mat) {
        std::vector<uint8_t> out((size_t)nn * nn);
        int ni = 0;
        for (int i = 0; i < n; i++) {
            if (i == q) continue;
            int nj = 0;
            for (int j = 0; j < n; j++) {
                if (j == q) continue;
                out[(size_t)ni * nn + nj] = mat[(size_t)i * n + j];
                nj++;
            }
            ni++;
        }
        return out;
    };
    auto shrinkv = [&](const std::vector<uint8_t>& vec) {
        std::vector<uint8_t> out;
        out.reserve(nn);
        for (int i = 0; i < n; i++)
            if (i != q) out.push_back(vec[i]);
        return out;
    };
    c.G = shrink(c.G);
    c.F = shrink(c.F);
    c.M = shrink(c.M);
    c.gamma = shrinkv(c.gamma);
    c.v = shrinkv(c.v);
    c.s = shrinkv(c.s);
    c.n = nn;
}

// kron (form/kron.rs:12-59)
static ChForm kron(const ChForm& a, const ChForm& b) {
    int nt = a.n + b.n;
    ChForm r = ch_new(nt);
    for (int i = 0; i < a.n; i++)
        for (int j = 0; j < a.n; j++) {
            r.g(i, j) = a.g(i, j);
            r.f(i, j) = a.f(i, j);
            r.m(i, j) = a.m(i, j);
        }
    for (int i = 0; i < b.n; i++)
        for (int j = 0; j < b.n; j++) {
            r.g(a.n + i, a.n + j) = b.g(i, j);
            r.f(a.n + i, a.n + j) = b.f(i, j);
            r.m(a.n + i, a.n + j) = b.m(i, j);
        }
    for (int i = 0; i < a.n; i++) {
        r.gamma[i] = a.gamma[i];
        r.v[i] = a.v[i];
        r.s[i] = a.s[i];
    }
    for (int i = 0; i < b.n; i++) {
        r.gamma[a.n + i] = b.gamma[i];
        r.v[a.n + i] = b.v[i];
        r.s[a.n + i] = b.s[i];
    }
    r.omega = cmul(a.omega, b.omega);
    r.phase = (a.phase + b.phase) % 8;
    return r;
}

// amplitude_at_zero (form/amplitude.rs:10-22): CH-form Scalar (r = |v|).
static Scalar amplitude_at_zero(const ChForm& c) {
    for (int j = 0; j < c.n; j++)
        if (!c.v[j] && c.s[j]) return Scalar{true, 0, 0};
    int64_t w = 0;
    for (int j = 0; j < c.n; j++) w += c.v[j];
    return Scalar{false, c.phase, w};
}

// amplitude_at_computational_basis (form/amplitude.rs:28-44)
static Scalar amplitude_at_basis(const ChForm& c, const std::vector<uint8_t>& bits) {
    ChForm cl = c;
    for (int i = 0; i < c.n; i++)
        if (bits[i]) left_x(cl, i);
    return amplitude_at_zero(cl);
}

// Internal gate list of the normalisation (form/types/internal_gate.rs:2-9).
struct IGate {
    uint8_t op;  // 0 H, 1 Sdg, 2 X, 3 CX, 4 CZ
    int a, b;
};

// get_normalize_to_zero_ops (form/inner_product.rs:52-123)
static std::vector<IGate> normalize_to_zero_ops(const ChForm& self, int* phase_out) {
    std::vector<IGate> ops;
    ChForm cl = self;
    int n = cl.n;
    for (int j = 0; j < n; j++) {
        int pivot_row = j;
        if (!cl.g(j, j)) {
            int k = -1;
            for (int kk = j + 1; kk < n; kk++)
                if (cl.g(kk, j)) { k = kk; break; }
            if (k < 0) fail(NSG_ERR_DEVICE_INVARIANT, 5, -1, "G matrix is not full rank, invalid stabilizer state.");
            pivot_row = k;
        }
        if (pivot_row != j) {
            ops.push_back({3, pivot_row, j});
            left_cx(cl, pivot_row, j);
            ops.push_back({3, j, pivot_row});
            left_cx(cl, j, pivot_row);
            ops.push_back({3, pivot_row, j});
            left_cx(cl, pivot_row, j);
        }
        for (int i = 0; i < n; i++) {
            if (i != j && cl.g(i, j)) {
                ops.push_back({3, j, i});
                left_cx(cl, j, i);
            }
        }
    }
    for (int r = 0; r < n; r++)
        for (int c = r + 1; c < n; c++)
            if (cl.m(r, c)) {
                ops.push_back({4, r, c});
                left_cz(cl, r, c);
            }
    for (int q = 0; q < n; q++)
        if (cl.m(q, q)) {
            ops.push_back({1, q, -1});
            left_sdg(cl, q);
        }
    for (int i = 0; i < n; i++)
        if (cl.v[i]) {
            ops.push_back({0, i, -1});
            left_h(cl, i);
        }
    for (int i = 0; i < n; i++)
        if (cl.s[i]) {
            ops.push_back({2, i, -1});
            left_x(cl, i);
        }
    *phase_out = cl.phase;
    return ops;
}

// get_ops_applied_state (form/inner_product.rs:125-138)
static ChForm ops_applied(const ChForm& other, const std::vector<IGate>& ops) {
    ChForm st = other;
    for (const IGate& o : ops) {
        switch (o.op) {
            case 0: left_h(st, o.a); break;
            case 1: left_sdg(st, o.a); break;
            case 2: left_x(st, o.a); break;
            case 3: left_cx(st, o.a, o.b); break;
            case 4: left_cz(st, o.a, o.b); break;
        }
    }
    return st;
}

// StabilizerCHForm::inner_product (form/inner_product.rs:14-48), returned as the
// exact CH-form Scalar `res * phase.conjugated()`; ω is 1 on every path.
static Scalar ch_inner_product_scalar(const ChForm& self, const ChForm& other) {
    if (self.n != other.n) fail(NSG_ERR_QUBIT_COUNT_MISMATCH, self.n, other.n);
    int ph = 0;
    std::vector<IGate> ops = normalize_to_zero_ops(self, &ph);
    ChForm tr = ops_applied(other, ops);
    Scalar res = amplitude_at_zero(tr);
    if (res.zero) return res;
    return Scalar{false, (res.k + (8 - ph) % 8) % 8, res.r};
}

// to_statevector (form/statevector.rs:12-27)
static std::vector<cplx> ch_statevector(const ChForm& c) {
    size_t dim = (size_t)1 << c.n;
    std::vector<cplx> sv(dim);
    std::vector<uint8_t> bits(c.n);
    for (size_t i = 0; i < dim; i++) {
        for (int j = 0; j < c.n; j++) bits[j] = (i >> j) & 1;
        sv[i] = cmul(scalar_to_complex(amplitude_at_basis(c, bits)), c.omega);
    }
    return sv;
}

// ---------------------------------------------------------------------------
// Pauli strings (crates/stabilizer-ch-form-rust/src/types/pauli/mod.rs:43-143)
struct PauliTerm {
    int op;  // 1 X, 2 Y, 3 Z (0 I allowed, ignored)
    int qubit;
};
struct Pauli {
    bool sparse;
    std::vector<int> dense;  // little-endian ops
    std::vector<PauliTerm> terms;
};

static Pauli pauli_from_abi(const nsg_pauli* p) {
    Pauli r;
    if (!p) fail(NSG_ERR_INVALID_ARGUMENT);
    if (p->kind == NSG_PAULI_DENSE) {
        r.sparse = false;
        for (uint32_t i = 0; i < p->len; i++) r.dense.push_back(p->ops[i]);
    } else if (p->kind == NSG_PAULI_SPARSE) {
        r.sparse = true;
        for (uint32_t i = 0; i < p->len; i++) r.terms.push_back({(int)p->ops[i], (int)p->qubits[i]});
    } else {
        fail(NSG_ERR_INVALID_ARGUMENT);
    }
    return r;
}

// apply_pauli (form/gate_application.rs:186-210)
static void apply_pauli(ChForm& c, const Pauli& p) {
    auto one = [&](int op, int q) {
        switch (op) {
            case 0: break;
            case 1: left_x(c, q); break;
            case 2: left_y(c, q); break;
            case 3: left_z(c, q); break;
        }
    };
    if (!p.sparse) {
        for (size_t q = 0; q < p.dense.size(); q++) one(p.dense[q], (int)q);
    } else {
        for (const auto& t : p.terms) one(t.op, t.qubit);
    }
}

// ---------------------------------------------------------------------------
// Stabilizer-decomposed state (crates/necstar/src/state/stabilizer_decomposed_state/mod.rs:19-24)
struct SDState {
    int num_qubits = 0;
    std::vector<ChForm> stabs;
    std::vector<Scalar> coeffs;
    cplx global_factor{1.0, 0.0};
};

// validate_qargs (stabilizer_decomposed_state/mod.rs:44-67)
static void validate_qargs(const SDState& st, const std::vector<int>& qargs) {
    if (qargs.empty()) fail(NSG_ERR_EMPTY_QUBIT_INDICES);
    for (int q : qargs)
        if (q < 0 || q >= st.num_qubits) fail(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, q, st.num_qubits);
    if (qargs.size() > 1) {
        std::vector<int> sorted = qargs;
        std::sort(sorted.begin(), sorted.end());
        for (size_t i = 1; i < sorted.size(); i++)
            if (sorted[i - 1] == sorted[i]) fail(NSG_ERR_DUPLICATE_QUBIT_INDEX, sorted[i]);
    }
}

// StabilizerDecomposedState::kron (stabilizer_decomposed_state/kron.rs:7-22)
static SDState sd_kron(const SDState& a, const SDState& b) {
    SDState r;
    r.num_qubits = a.num_qubits + b.num_qubits;
    for (size_t i = 0; i < a.stabs.size(); i++)
        for (size_t j = 0; j < b.stabs.size(); j++) {
            r.stabs.push_back(kron(a.stabs[i], b.stabs[j]));
            r.coeffs.push_back(scalar_mul(a.coeffs[i], b.coeffs[j]));
        }
    return r;
}

// ---------------------------------------------------------------------------
// Magic states (crates/necstar/src/state/magic_states/cat_state.rs, t_state.rs)
static const Scalar S_ONE{false, 0, 0};
static const Scalar S_ONE_OVER_SQRT2{false, 0, 1};

static ChForm zero_minus_i_one_state(int nq) {  // cat_state.rs:16-29
    if (nq == 0) fail(NSG_ERR_INVALID_NUM_QUBITS, 0);
    ChForm st = ch_new(nq);
    left_h(st, 0);
    for (int i = 1; i < nq; i++) left_cx(st, 0, i);
    left_sdg(st, 0);
    return st;
}
static ChForm even_parity_state(int nq) {  // :32-42
    ChForm st = ch_new(nq);
    for (int i = 0; i < nq - 1; i++) left_h(st, i);
    for (int i = 0; i < nq - 1; i++) left_cx(st, i, nq - 1);
    return st;
}
static ChForm even_parity_phase_flipped_state(int nq) {  // :45-53
    ChForm st = even_parity_state(nq);
    for (int i = 0; i < nq; i++)
        for (int j = i + 1; j < nq; j++) left_cz(st, i, j);
    return st;
}
static SDState mk_sd(int nq, std::vector<ChForm> stabs, std::vector<Scalar> coeffs) {
    SDState r;
    r.num_qubits = nq;
    r.stabs = std::move(stabs);
    r.coeffs = std::move(coeffs);
    return r;
}
static SDState cat1() { return mk_sd(1, {ch_new(1)}, {S_ONE}); }  // :56-61
static SDState cat2() {                                              // :64-72
    ChForm st = ch_new(2);
    left_h(st, 0);
    left_cx(st, 0, 1);
    left_s(st, 1);
    return mk_sd(2, {st}, {S_ONE});
}
static SDState cat4() {  // :75-94
    return mk_sd(4, {zero_minus_i_one_state(4), even_parity_state(4)},
                 {Scalar{false, 7, 1}, Scalar{false, 2, 0}});
}
static SDState cat6() {  // :97-121
    return mk_sd(6, {zero_minus_i_one_state(6), even_parity_state(6), even_parity_phase_flipped_state(6)},
                 {Scalar{false, 0, 2}, Scalar{false, 3, 1}, Scalar{false, 5, 1}});
}
static void project_onto_cat(ChForm& st, int q0, int q1) {  // :123-135
    left_sdg(st, q0);
    left_cx(st, q0, q1);
    left_h(st, q0);
    project(st, q0, false);
    project(st, q1, false);
    discard(st, q1);
    discard(st, q0);
}
static void reduce_cat(SDState& st) {  // :150-159
    int nq = st.num_qubits;
    for (auto& c : st.stabs) {
        project(c, nq - 1, false);
        discard(c, nq - 1);
    }
    st.num_qubits -= 1;
}
static SDState construct_cat(int nq) {  // :162-188
    switch (nq) {
        case 0: fail(NSG_ERR_INVALID_NUM_QUBITS, 0);
        case 1: return cat1();
        case 2: return cat2();
        case 3: { SDState s = cat4(); reduce_cat(s); return s; }
        case 4: return cat4();
        case 5: { SDState s = cat6(); reduce_cat(s); return s; }
        case 6: return cat6();
        default: {
            SDState pair = sd_kron(construct_cat(nq - 4), construct_cat(6));
            for (auto& c : pair.stabs) project_onto_cat(c, nq - 5, nq - 4);
            pair.num_qubits -= 2;
            return pair;
        }
    }
}
// construct_t_tensor_state (magic_states/t_state.rs:29-71)
static SDState construct_t_tensor(int nq) {
    SDState cat = construct_cat(nq);
    SDState r;
    r.num_qubits = cat.num_qubits;
    std::vector<Scalar> orig;
    for (auto c : cat.coeffs) orig.push_back(scalar_mul(c, S_ONE_OVER_SQRT2));
    r.stabs = cat.stabs;
    r.coeffs = orig;
    for (size_t i = 0; i < cat.stabs.size(); i++) {
        ChForm st = cat.stabs[i];
        left_x(st, 0);
        left_s(st, 0);
        r.stabs.push_back(st);
        r.coeffs.push_back(scalar_mul(orig[i], Scalar{false, 7, 0}));
    }
    return r;
}

// One term of construct_cat(nq) (cat_state.rs:162-188) without building the
// others.  The recursion's term order is i-major over kron(cat(nq-4), cat(6))
// (stabilizer_decomposed_state/kron.rs:11-16) and every later step
// (project_onto_cat, reduce_cat) acts on each term alone, so term ci is
// term ci/3 of cat(nq-4) joined with term ci%3 of cat(6).
static int64_t cat_rank(int nq) {
    static const int64_t small[7] = {0, 1, 1, 2, 2, 3, 3};
    if (nq <= 0) fail(NSG_ERR_INVALID_NUM_QUBITS, 0);
    return nq <= 6 ? small[nq] : cat_rank(nq - 4) * 3;
}
static std::pair<ChForm, Scalar> cat_term(int nq, int64_t ci) {
    if (ci < 0 || ci >= cat_rank(nq)) fail(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, ci, cat_rank(nq));
    if (nq <= 6) {
        SDState s = construct_cat(nq);
        return {s.stabs[(size_t)ci], s.coeffs[(size_t)ci]};
    }
    auto a = cat_term(nq - 4, ci / 3);
    SDState c6 = cat6();
    ChForm st = kron(a.first, c6.stabs[(size_t)(ci % 3)]);
    project_onto_cat(st, nq - 5, nq - 4);
    return {st, scalar_mul(a.second, c6.coeffs[(size_t)(ci % 3)])};
}
// Term k of construct_t_tensor(nq) (t_state.rs:29-71): cat terms first
// (coefficient·2^(-1/2)), then their copies with X·S on qubit 0 (·e^(-iπ/4)).
static int64_t t_tensor_rank(int nq) { return 2 * cat_rank(nq); }
static std::pair<ChForm, Scalar> t_tensor_term(int nq, int64_t k) {
    const int64_t cr = cat_rank(nq);
    if (k < 0 || k >= 2 * cr) fail(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, k, 2 * cr);
    auto c = cat_term(nq, k % cr);
    Scalar coef = scalar_mul(c.second, S_ONE_OVER_SQRT2);
    if (k >= cr) {
        left_x(c.first, 0);
        left_s(c.first, 0);
        coef = scalar_mul(coef, Scalar{false, 7, 0});
    }
    return {c.first, coef};
}

// construct_toffoli_state / construct_toffoli_tensor_state
// (crates/necstar/src/state/magic_states/toffoli_state.rs:12-40).
static SDState construct_toffoli() {
    ChForm a = ch_new(3);  // |0+0⟩
    left_h(a, 1);
    ChForm b = ch_new(3);  // |1⟩⊗Bell
    left_x(b, 0);
    left_h(b, 1);
    left_cx(b, 1, 2);
    return mk_sd(3, {a, b}, {S_ONE_OVER_SQRT2, S_ONE_OVER_SQRT2});
}
static SDState construct_toffoli_tensor(int k) {
    if (k == 0) fail(NSG_ERR_INVALID_NUM_QUBITS, 0);
    if (k == 1) return construct_toffoli();
    return sd_kron(construct_toffoli_tensor(k - 1), construct_toffoli());
}

// ---------------------------------------------------------------------------
// Compiler (crates/necstar/src/state/compiler/mod.rs:44-140)
static bool is_clifford_op(uint32_t op) { return op <= NSG_GATE_SWAP; }

// Lowering (compiler/mod.rs:49-63): T/Tdg -> CX(target, n+k) [+ Sdg(target)].
static std::vector<nsg_gate> lower_circuit(int n, const std::vector<nsg_gate>& gates, int* t_out) {
    int t = 0;
    std::vector<nsg_gate> cl;
    for (const auto& g : gates) {
        if (is_clifford_op(g.op)) {
            cl.push_back(g);
        } else if (g.op == NSG_GATE_T || g.op == NSG_GATE_TDG) {
            int anc = n + t;
            cl.push_back(nsg_gate{NSG_GATE_CX, g.q0, (uint32_t)anc, 0});
            if (g.op == NSG_GATE_TDG) cl.push_back(nsg_gate{NSG_GATE_SDG, g.q0, 0, 0});
            t++;
        } else {
            fail(NSG_ERR_GATE_NOT_SUPPORTED, g.op, -1, "Gate CCX is not supported.");
        }
    }
    *t_out = t;
    return cl;
}

// The per-term body of the compile loop (compiler/mod.rs:92-131): kron with
// |0^n⟩, every Clifford, post-selection of the ancillas in reverse order;
// false when a projection is impossible (the term is dropped).
static bool compile_one(int n, int t, const std::vector<nsg_gate>& cl, const ChForm& tterm, Scalar tcoef,
                        ChForm& out, Scalar& coef) {
    ChForm full = kron(ch_new(n), tterm);
    for (const auto& g : cl) apply_clifford(full, g);
    int ndet = 0;
    for (int q = n + t - 1; q >= n; q--) {
        try {
            if (project(full, q, false)) ndet++;
        } catch (const Error& e) {
            if (e.code == NSG_ERR_IMPOSSIBLE_PROJECTION) return false;
            throw;
        }
    }
    for (int q = n + t - 1; q >= n; q--) discard(full, q);
    out = std::move(full);
    coef = scalar_amplify(tcoef, ndet);
    return true;
}

static SDState compile(int n, const std::vector<nsg_gate>& gates) {
    int t = 0;
    std::vector<nsg_gate> cl = lower_circuit(n, gates, &t);
    if (t == 0) {  // :66-80
        ChForm c = ch_new(n);
        for (const auto& g : cl) apply_clifford(c, g);
        return mk_sd(n, {c}, {S_ONE});
    }
    SDState tt = construct_t_tensor(t);
    SDState out;
    out.num_qubits = n;
    for (size_t k = 0; k < tt.stabs.size(); k++) {
        ChForm full;
        Scalar coef;
        if (compile_one(n, t, cl, tt.stabs[k], tt.coeffs[k], full, coef)) {
            out.stabs.push_back(std::move(full));
            out.coeffs.push_back(coef);
        }
    }
    return out;
}

// The compile loop restricted to the T-tensor terms `tidx` (each built on its
// own by t_tensor_term): the kept terms in the order given, kept[i] = 1 when
// term tidx[i] survives post-selection.  Terms are independent in the loop
// and the drop rule depends on the term alone, so these are exactly the
// terms the whole compile keeps for those indices.
static SDState compile_terms(int n, const std::vector<nsg_gate>& gates, const std::vector<int64_t>& tidx,
                             uint8_t* kept, int threads) {
    int t = 0;
    std::vector<nsg_gate> cl = lower_circuit(n, gates, &t);
    SDState out;
    out.num_qubits = n;
    if (t == 0) {
        for (size_t i = 0; i < tidx.size(); i++) {
            if (tidx[i] != 0) fail(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, tidx[i], 1);
            ChForm c = ch_new(n);
            for (const auto& g : cl) apply_clifford(c, g);
            out.stabs.push_back(c);
            out.coeffs.push_back(S_ONE);
            kept[i] = 1;
        }
        return out;
    }
    const size_t m = tidx.size();
    std::vector<ChForm> terms(m);
    std::vector<Scalar> coefs(m);
    std::vector<uint8_t> ok(m, 0);
    std::vector<Error> errs;
    std::mutex emu;
    std::atomic<size_t> next{0};
    std::vector<std::thread> pool;
    for (int th = 0; th < std::max(1, threads); th++)
        pool.emplace_back([&]() {
            try {
                for (size_t i; (i = next.fetch_add(1)) < m;) {
                    auto tt = t_tensor_term(t, tidx[i]);
                    ok[i] = compile_one(n, t, cl, tt.first, tt.second, terms[i], coefs[i]) ? 1 : 0;
                }
            } catch (const Error& e) {
                std::lock_guard<std::mutex> lk(emu);
                errs.push_back(e);
            }
        });
    for (auto& th : pool) th.join();
    if (!errs.empty()) throw errs[0];
    for (size_t i = 0; i < m; i++) {
        kept[i] = ok[i];
        if (ok[i]) {
            out.stabs.push_back(std::move(terms[i]));
            out.coeffs.push_back(coefs[i]);
        }
    }
    return out;
}

// ---------------------------------------------------------------------------
// Exact accumulation of Σ phase·2^(-r/2) terms.  Every real (imaginary) part
// is ±2^(-m/2) for an integer m; even m goes to X, odd m to Y, both as signed
// counts per power of two, so the sum is X + Y/√2 exactly.
struct BigBin {
    // Non-negative binary number Σ bit_p 2^(p - OFF) stored in 64-bit limbs.
    static constexpr int OFF = 4096;  // position of 2^0
    std::vector<uint64_t> limb = std::vector<uint64_t>(8192 / 64 + 2, 0);
    void add(uint64_t count, int64_t pos) {  // += count · 2^(pos)
        int64_t p = pos + OFF;
        if (p < 0 || p + 64 >= (int64_t)limb.size() * 64) throw std::runtime_error("exact sum range");
        size_t w = (size_t)(p / 64);
        int b = (int)(p % 64);
        unsigned __int128 v = (unsigned __int128)count << b;
        uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
        unsigned __int128 acc = (unsigned __int128)limb[w] + lo;
        limb[w] = (uint64_t)acc;
        uint64_t carry = (uint64_t)(acc >> 64);
        acc = (unsigned __int128)limb[w + 1] + hi + carry;
        limb[w + 1] = (uint64_t)acc;
        carry = (uint64_t)(acc >> 64);
        for (size_t k = w + 2; carry && k < limb.size(); k++) {
            acc = (unsigned __int128)limb[k] + carry;
            limb[k] = (uint64_t)acc;
            carry = (uint64_t)(acc >> 64);
        }
    }
    int cmp(const BigBin& o) const {
        for (size_t k = limb.size(); k-- > 0;) {
            if (limb[k] != o.limb[k]) return limb[k] < o.limb[k] ? -1 : 1;
        }
        return 0;
    }
    void sub(const BigBin& o) {  // requires *this >= o
        uint64_t borrow = 0;
        for (size_t k = 0; k < limb.size(); k++) {
            unsigned __int128 a = limb[k], b = (unsigned __int128)o.limb[k] + borrow;
            if (a >= b) { limb[k] = (uint64_t)(a - b); borrow = 0; }
            else { limb[k] = (uint64_t)(((unsigned __int128)1 << 64) + a - b); borrow = 1; }
        }
    }
    double to_double() const {
        // Top 64 significant bits, then scale.
        for (size_t k = limb.size(); k-- > 0;) {
            if (limb[k] == 0) continue;
            int top = 63 - __builtin_clzll(limb[k]);
            int64_t msb = (int64_t)k * 64 + top;  // absolute bit position
            // gather 64 bits ending at msb
            unsigned __int128 window = ((unsigned __int128)limb[k] << 64) | (k > 0 ? limb[k - 1] : 0);
            int shift = top + 64 - 63;  // keep bits msb..msb-63
            uint64_t mant = (uint64_t)(window >> shift);
            return std::ldexp((double)mant, (int)(msb - 63 - OFF));
        }
        return 0.0;
    }
};

struct ExactSum {
    // Every real (imaginary) part of a pair term is ±2^(-m/2) for an integer m;
    // even m goes to X, odd m to Y (as 2^(-(m-1)/2)/√2), so the sum is X + Y/√2
    // with X, Y exact dyadic rationals held as positive/negative big binaries.
    BigBin xp, xn, yp, yn;
    void add_real_part(int k, int64_t r, int sign_mul = 1) {
        int sgn;
        int64_t m;
        switch (k & 7) {
            case 0: sgn = 1; m = r; break;
            case 4: sgn = -1; m = r; break;
            case 1: case 7: sgn = 1; m = r + 1; break;
            case 3: case 5: sgn = -1; m = r + 1; break;
            default: return;
        }
        add_m(sgn * sign_mul, m);
    }
    void add_imag_part(int k, int64_t r, int sign_mul = 1) {
        int sgn;
        int64_t m;
        switch (k & 7) {
            case 2: sgn = 1; m = r; break;
            case 6: sgn = -1; m = r; break;
            case 1: case 3: sgn = 1; m = r + 1; break;
            case 5: case 7: sgn = -1; m = r + 1; break;
            default: return;
        }
        add_m(sgn * sign_mul, m);
    }
    void add_m(int sgn, int64_t m) {
        uint64_t cnt = (uint64_t)(sgn < 0 ? -sgn : sgn);
        if (((m % 2) + 2) % 2 == 0) {
            (sgn > 0 ? xp : xn).add(cnt, -(m / 2));
        } else {
            (sgn > 0 ? yp : yn).add(cnt, -((m - 1) / 2));
        }
    }
    static double diff(BigBin p, const BigBin& n) {
        int c = p.cmp(n);
        if (c == 0) return 0.0;
        if (c > 0) { p.sub(n); return p.to_double(); }
        BigBin q = n;
        q.sub(p);
        return -q.to_double();
    }
    double value() const {
        double x = diff(xp, xn), y = diff(yp, yn);
        return x + y * 0.70710678118654752440084436210484903928;
    }
};

// exp_value (stabilizer_decomposed_state/exp_value.rs:7-61) in the reference's
// summation order; also returns the exact value.
static void validate_pauli(const SDState& st, const Pauli& p) {
    if (!p.sparse) {
        if ((int)p.dense.size() != st.num_qubits)
            fail(NSG_ERR_INVALID_PAULI_STRING_LENGTH, st.num_qubits, (int64_t)p.dense.size());
    } else {
        int maxq = 0;
        for (auto& t : p.terms) maxq = std::max(maxq, t.qubit);
        if (maxq >= st.num_qubits) fail(NSG_ERR_INVALID_PAULI_STRING_LENGTH, st.num_qubits, maxq + 1);
    }
}

static double exp_value(const SDState& st, const Pauli& p, double* exact_out) {
    validate_pauli(st, p);
    cplx acc(0.0, 0.0);
    ExactSum ex;
    size_t chi = st.stabs.size();
    for (size_t i = 0; i < chi; i++) {
        ChForm ev = st.stabs[i];
        apply_pauli(ev, p);
        Scalar ipd = ch_inner_product_scalar(st.stabs[i], ev);
        cplx ipdc = cmul(cmul(st.stabs[i].omega, ev.omega), scalar_to_complex(ipd));
        Scalar cd = scalar_mul(scalar_conj(st.coeffs[i]), st.coeffs[i]);
        acc += cmul(scalar_to_complex(cd), ipdc);
        Scalar td = scalar_mul(cd, ipd);
        if (!td.zero) ex.add_real_part(td.k, td.r);
        for (size_t j = i + 1; j < chi; j++) {
            Scalar ip = ch_inner_product_scalar(st.stabs[j], ev);
            cplx ipc = cmul(cmul(st.stabs[j].omega, ev.omega), scalar_to_complex(ip));
            Scalar cc = scalar_mul(scalar_conj(st.coeffs[j]), st.coeffs[i]);
            cplx term = cmul(scalar_to_complex(cc), ipc);
            acc += term + std::conj(term);
            Scalar tt = scalar_mul(cc, ip);
            if (!tt.zero) ex.add_real_part(tt.k, tt.r, 2);
        }
    }
    double gf2 = std::norm(st.global_factor);
    if (exact_out) *exact_out = ex.value() * gf2;
    return acc.real() * gf2;
}

// The exact accumulator of exp_value as integer counts: every term of the
// χ² sum (exp_value.rs:38-58, with the factor 2 of the j > i terms) has a
// real part sign·2^(-m/2); counts[o][m + m_off] is the signed number of
// them for observable o, so ⟨P_o⟩ = |g|²·Σ_m counts[o][m+m_off]·2^(-m/2)
// exactly.  Rows i are spread over `threads` host threads, each with its
// own counts (integer sums: the result does not depend on the split).
static void exp_value_counts(const SDState& st, const std::vector<Pauli>& ps, int threads, int64_t m_off,
                             int64_t bins, int64_t* counts) {
    for (const Pauli& p : ps) validate_pauli(st, p);
    const size_t chi = st.stabs.size(), nobs = ps.size();
    threads = std::max(1, threads);
    std::vector<std::vector<int64_t>> part(threads, std::vector<int64_t>((size_t)(nobs * bins), 0));
    std::atomic<size_t> next{0};
    std::vector<Error> errs;
    std::mutex emu;
    std::vector<std::thread> pool;
    for (int th = 0; th < threads; th++)
        pool.emplace_back([&, th]() {
            try {
                int64_t* c = part[th].data();
                auto add = [&](size_t o, Scalar tt, int64_t w) {
                    if (tt.zero) return;
                    int sgn;
                    int64_t m;
                    switch (tt.k & 7) {
                        case 0: sgn = 1; m = tt.r; break;
                        case 4: sgn = -1; m = tt.r; break;
                        case 1: case 7: sgn = 1; m = tt.r + 1; break;
                        case 3: case 5: sgn = -1; m = tt.r + 1; break;
                        default: return;
                    }
                    if (m + m_off < 0 || m + m_off >= bins) fail(NSG_ERR_DEVICE_INVARIANT, m, bins, "exact count range");
                    c[o * bins + (m + m_off)] += sgn * w;
                };
                for (size_t i; (i = next.fetch_add(1)) < chi;) {
                    for (size_t o = 0; o < nobs; o++) {
                        ChForm ev = st.stabs[i];
                        apply_pauli(ev, ps[o]);
                        add(o, scalar_mul(scalar_mul(scalar_conj(st.coeffs[i]), st.coeffs[i]),
                                          ch_inner_product_scalar(st.stabs[i], ev)), 1);
                        for (size_t j = i + 1; j < chi; j++)
                            add(o, scalar_mul(scalar_mul(scalar_conj(st.coeffs[j]), st.coeffs[i]),
                                              ch_inner_product_scalar(st.stabs[j], ev)), 2);
                    }
                }
            } catch (const Error& e) {
                std::lock_guard<std::mutex> lk(emu);
                errs.push_back(e);
            }
        });
    for (auto& th : pool) th.join();
    if (!errs.empty()) throw errs[0];
    std::fill(counts, counts + nobs * bins, 0);
    for (int th = 0; th < threads; th++)
        for (size_t x = 0; x < (size_t)(nobs * bins); x++) counts[x] += part[th][x];
}

// Σ_m counts[m + m_off]·2^(-m/2), evaluated exactly and rounded once.
static double counts_value(const int64_t* counts, int64_t m_off, int64_t bins) {
    ExactSum ex;
    for (int64_t b = 0; b < bins; b++) {
        const int64_t c = counts[b];
        if (c == 0) continue;
        const int64_t m = b - m_off;
        const uint64_t mag = (uint64_t)(c < 0 ? -c : c);
        if (((m % 2) + 2) % 2 == 0) (c > 0 ? ex.xp : ex.xn).add(mag, -(m / 2));
        else (c > 0 ? ex.yp : ex.yn).add(mag, -((m - 1) / 2));
    }
    return ex.value();
}

// norm_squared (stabilizer_decomposed_state/norm.rs:8-30)
static double norm_squared(const SDState& st, double* exact_out = nullptr) {
    cplx sum(0.0, 0.0);
    ExactSum ex;
    size_t chi = st.stabs.size();
    for (size_t i = 0; i < chi; i++) {
        Scalar ipd = ch_inner_product_scalar(st.stabs[i], st.stabs[i]);
        Scalar cd = scalar_mul(scalar_conj(st.coeffs[i]), st.coeffs[i]);
        sum += cmul(scalar_to_complex(cd), scalar_to_complex(ipd));
        Scalar td = scalar_mul(cd, ipd);
        if (!td.zero) ex.add_real_part(td.k, td.r);
        for (size_t j = i + 1; j < chi; j++) {
            Scalar ip = ch_inner_product_scalar(st.stabs[i], st.stabs[j]);
            Scalar cc = scalar_mul(scalar_conj(st.coeffs[i]), st.coeffs[j]);
            cplx term = cmul(scalar_to_complex(cc), scalar_to_complex(ip));
            sum += term + std::conj(term);
            Scalar tt = scalar_mul(cc, ip);
            if (!tt.zero) ex.add_real_part(tt.k, tt.r, 2);
        }
    }
    double gf2 = std::norm(st.global_factor);
    if (exact_out) *exact_out = ex.value() * gf2;
    return sum.real() * gf2;
}

// inner_product (stabilizer_decomposed_state/inner_product.rs:9-19)
static cplx sd_inner_product(const SDState& a, const SDState& b, cplx* exact_out) {
    if (a.num_qubits != b.num_qubits) fail(NSG_ERR_QUBIT_COUNT_MISMATCH, a.num_qubits, b.num_qubits);
    cplx res(0.0, 0.0);
    ExactSum exr, exi;
    for (size_t i = 0; i < a.stabs.size(); i++)
        for (size_t j = 0; j < b.stabs.size(); j++) {
            Scalar ip = ch_inner_product_scalar(a.stabs[i], b.stabs[j]);
            cplx ipc = cmul(cmul(a.stabs[i].omega, b.stabs[j].omega), scalar_to_complex(ip));
            Scalar cc = scalar_mul(scalar_conj(a.coeffs[i]), b.coeffs[j]);
            res += cmul(scalar_to_complex(cc), ipc);
            Scalar tt = scalar_mul(cc, ip);
            if (!tt.zero) {
                exr.add_real_part(tt.k, tt.r);
                exi.add_imag_part(tt.k, tt.r);
            }
        }
    cplx gfac = cmul(std::conj(a.global_factor), b.global_factor);
    if (exact_out) *exact_out = cmul(cplx(exr.value(), exi.value()), gfac);
    return cmul(cmul(res, std::conj(a.global_factor)), b.global_factor);
}

// project_unnormalized (stabilizer_decomposed_state/projection.rs:27-57)
static void project_unnormalized(SDState& st, int q, bool outcome) {
    if (q < 0 || q >= st.num_qubits) fail(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, q, st.num_qubits);
    std::vector<ChForm> ns;
    std::vector<Scalar> nc;
    for (size_t i = 0; i < st.stabs.size(); i++) {
        ChForm c = st.stabs[i];
        try {
            bool det = project(c, q, outcome);
            ns.push_back(std::move(c));
            nc.push_back(det ? st.coeffs[i] : scalar_amplify(st.coeffs[i], -1));
        } catch (const Error& e) {
            if (e.code != NSG_ERR_IMPOSSIBLE_PROJECTION) throw;
        }
    }
    st.stabs = std::move(ns);
    st.coeffs = std::move(nc);
}

// project_normalized (projection.rs:10-21)
static void project_normalized(SDState& st, int q, bool outcome) {
    project_unnormalized(st, q, outcome);
    double nrm = std::sqrt(norm_squared(st));
    if (std::fabs(nrm) < 1e-12 || std::isnan(nrm)) fail(NSG_ERR_IMPOSSIBLE_PROJECTION, q, outcome ? 1 : 0);
    st.global_factor = st.global_factor / nrm;
}

// discard (stabilizer_decomposed_state/discard.rs:5-12)
static void sd_discard(SDState& st, int q) {
    for (auto& c : st.stabs) discard(c, q);
    st.num_qubits -= 1;
}

// apply_gate (stabilizer_decomposed_state/gates.rs:7-30)
static void sd_apply_gate(SDState& st, const nsg_gate& g) {
    if (!is_clifford_op(g.op)) fail(NSG_ERR_NON_CLIFFORD_GATE_APPLICATION, g.op);
    for (auto& c : st.stabs) apply_clifford(c, g);
}

// to_statevector (stabilizer_decomposed_state/statevector.rs:12-24)
static std::vector<cplx> sd_statevector(const SDState& st) {
    if (st.num_qubits > 28) fail(NSG_ERR_STATEVECTOR_TOO_LARGE, st.num_qubits);
    size_t dim = (size_t)1 << st.num_qubits;
    std::vector<cplx> sv(dim, cplx(0, 0));
    for (size_t i = 0; i < st.stabs.size(); i++) {
        std::vector<cplx> s = ch_statevector(st.stabs[i]);
        cplx c = scalar_to_complex(st.coeffs[i]);
        for (size_t k = 0; k < dim; k++) sv[k] = sv[k] + cmul(s[k], c);
    }
    for (size_t k = 0; k < dim; k++) sv[k] = cmul(sv[k], st.global_factor);
    return sv;
}

// ---------------------------------------------------------------------------
// rand 0.8.5 StdRng::from_seed(seed) = rand_chacha 0.3.1 ChaCha12Rng: the
// ChaCha keystream (12 rounds) with key = seed, a 64-bit block counter from 0
// and a zero 64-bit stream id, consumed as little-endian 32-bit words.
static uint32_t chacha_rotl(uint32_t v, int c) { return (v << c) | (v >> (32 - c)); }

static void chacha_block_words(const uint32_t input[16], int rounds, uint32_t out[16]) {
    uint32_t w[16];
    for (int i = 0; i < 16; i++) w[i] = input[i];
    auto qr = [&w](int a, int b, int c, int d) {
        w[a] += w[b]; w[d] ^= w[a]; w[d] = chacha_rotl(w[d], 16);
        w[c] += w[d]; w[b] ^= w[c]; w[b] = chacha_rotl(w[b], 12);
        w[a] += w[b]; w[d] ^= w[a]; w[d] = chacha_rotl(w[d], 8);
        w[c] += w[d]; w[b] ^= w[c]; w[b] = chacha_rotl(w[b], 7);
    };
    for (int dr = 0; dr < rounds / 2; dr++) {
        for (int col = 0; col < 4; col++) qr(col, col + 4, col + 8, col + 12);       // column round
        for (int col = 0; col < 4; col++)                                            // diagonal round
            qr(col, 4 + (col + 1) % 4, 8 + (col + 2) % 4, 12 + (col + 3) % 4);
    }
    for (int i = 0; i < 16; i++) out[i] = w[i] + input[i];
}

struct Rng {
    uint8_t key[32];
    uint64_t block = 0;
    uint8_t ks[64];  // current keystream block as bytes
    int used = 64;

    explicit Rng(const uint8_t* seed32) {
        if (seed32) {
            std::memcpy(key, seed32, 32);
        } else {
            std::random_device rd;
            for (int i = 0; i < 32; i++) key[i] = (uint8_t)rd();
        }
    }
    void refill() {
        uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
        for (int i = 0; i < 8; i++)
            in[4 + i] = (uint32_t)key[4 * i] | (uint32_t)key[4 * i + 1] << 8 | (uint32_t)key[4 * i + 2] << 16 |
                        (uint32_t)key[4 * i + 3] << 24;
        in[12] = (uint32_t)block;
        in[13] = (uint32_t)(block >> 32);
        in[14] = in[15] = 0;
        uint32_t out[16];
        chacha_block_words(in, 12, out);
        for (int i = 0; i < 16; i++)
            for (int b = 0; b < 4; b++) ks[4 * i + b] = (uint8_t)(out[i] >> (8 * b));
        block++;
        used = 0;
    }
    uint32_t next_u32() {
        if (used == 64) refill();
        uint32_t v = (uint32_t)ks[used] | (uint32_t)ks[used + 1] << 8 | (uint32_t)ks[used + 2] << 16 |
                     (uint32_t)ks[used + 3] << 24;
        used += 4;
        return v;
    }
    uint64_t next_u64() {  // rand_core BlockRng: low word first
        uint64_t lo = next_u32();
        uint64_t hi = next_u32();
        return (hi << 32) | lo;
    }
    // rng.gen::<f64>(): 53 random bits scaled by 2^-53.
    double uniform() { return std::ldexp((double)(next_u64() >> 11), -53); }
    // rng.gen_range(0..=1) for u8: Lemire's widening multiply of a u32 draw by
    // the range (2); the rejection zone is the whole u32 range here.
    uint8_t range01() {
        const uint64_t range = 2;
        for (;;) {
            const uint64_t prod = (uint64_t)next_u32() * range;
            const uint32_t lo = (uint32_t)prod;
            const uint32_t zone = UINT32_MAX - (uint32_t)(((uint64_t)UINT32_MAX - range + 1) % range);
            if (lo <= zone) return (uint8_t)(prod >> 32);
        }
    }
};

static uint64_t splitmix(uint64_t& x) {  // SplitMix64 (pair sampling of the CPU timing)
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// CliffordCircuit::random_clifford
// (crates/stabilizer-ch-form-rust/src/circuit/random_clifford.rs:177-212).
// sample_quantum_mallows :7-45
static void rc_mallows(int n, Rng& rng, std::vector<uint8_t>& h, std::vector<size_t>& s) {
    h.assign(n, 0);
    s.assign(n, 0);
    std::vector<size_t> avail;
    for (int i = 0; i < n; i++) avail.push_back(i);
    for (int i = 0; i < n; i++) {
        const int m = n - i;
        const double r = rng.uniform();
        const double val = r * (std::pow(4.0, m) - 1.0) + 1.0;
        const double cl = std::ceil(std::log2(val));
        // `ceil_log as isize` saturates (NaN → 0)
        long long ci = std::isnan(cl) ? 0 : (cl >= 9.2e18 ? LLONG_MAX : (long long)cl);
        long long a = (ci > 2LL * m) ? 0 : (2LL * m + 1 - ci);
        if (a <= 0) a = 1;
        long long k1;
        if (a <= m) {
            h[i] = 1;
            k1 = a;
        } else {
            h[i] = 0;
            k1 = 2LL * m - a + 1;
        }
        // k1 - 1 wraps to usize::MAX when k1 = 0, which takes the pop branch
        if (k1 >= 1 && (size_t)(k1 - 1) < avail.size()) {
            s[i] = avail[(size_t)(k1 - 1)];
            avail.erase(avail.begin() + (k1 - 1));
        } else {
            s[i] = avail.back();
            avail.pop_back();
        }
    }
}

static std::vector<nsg_gate> rc_random_clifford(int n, const uint8_t* seed32) {
    std::vector<nsg_gate> qc;
    if (n == 0) return qc;
    Rng rng(seed32);
    // generate_clifford_params :62-122
    std::vector<uint8_t> h;
    std::vector<size_t> s;
    rc_mallows(n, rng, h, s);
    typedef std::vector<std::vector<uint8_t>> Mat;
    Mat gamma1(n, std::vector<uint8_t>(n, 0)), gamma2 = gamma1, delta1 = gamma1, delta2 = gamma1;
    for (int i = 0; i < n; i++) delta1[i][i] = delta2[i][i] = 1;
    std::vector<uint8_t> pz(n), px(n);
    for (int i = 0; i < n; i++) pz[i] = rng.range01();
    for (int i = 0; i < n; i++) px[i] = rng.range01();
    for (int i = 0; i < n; i++) {
        gamma2[i][i] = rng.range01();
        if (h[i] == 1) gamma1[i][i] = rng.range01();
    }
    for (int i = 1; i < n; i++)
        for (int j = 0; j < i; j++) {
            uint8_t b2 = rng.range01();
            gamma2[i][j] = b2;
            gamma2[j][i] = b2;
            delta2[i][j] = rng.range01();
            const bool hi = h[i] == 1, hj = h[j] == 1;
            const size_t si = s[i], sj = s[j];
            if (((si < sj || hj) && hi) || (hj && sj < si)) {
                uint8_t b = rng.range01();
                gamma1[i][j] = b;
                gamma1[j][i] = b;
            }
            if ((si < sj || hj) && (si > sj || !hi) && (hj || !hi)) delta1[i][j] = rng.range01();
        }
    // apply_hadamard_free_layer :125-165, apply_permutation_layer :168-180
    auto layer = [&](const Mat& gamma, const Mat& delta, bool paulis) {
        for (int j = 0; j < n; j++)
            for (int i = j + 1; i < n; i++)
                if (delta[i][j] == 1) qc.push_back({NSG_GATE_CX, (uint32_t)j, (uint32_t)i, 0});
        for (int i = 0; i < n; i++) {
            if (gamma[i][i] == 1) qc.push_back({NSG_GATE_S, (uint32_t)i, 0, 0});
            for (int j = 0; j < i; j++)
                if (gamma[i][j] == 1) qc.push_back({NSG_GATE_CZ, (uint32_t)i, (uint32_t)j, 0});
        }
        if (paulis)
            for (int i = 0; i < n; i++) {
                if (pz[i] == 1 && px[i] == 1) qc.push_back({NSG_GATE_Y, (uint32_t)i, 0, 0});
                else if (pz[i] == 1) qc.push_back({NSG_GATE_Z, (uint32_t)i, 0, 0});
                else if (px[i] == 1) qc.push_back({NSG_GATE_X, (uint32_t)i, 0, 0});
            }
    };
    layer(gamma2, delta2, true);
    std::vector<size_t> p;
    for (int i = 0; i < n; i++) p.push_back(i);
    for (int i = 0; i < n; i++)
        if (p[i] != s[i]) {
            size_t j = std::find(p.begin(), p.end(), s[i]) - p.begin();
            qc.push_back({NSG_GATE_SWAP, (uint32_t)i, (uint32_t)j, 0});
            std::swap(p[i], p[j]);
        }
    for (int i = 0; i < n; i++)
        if (h[i] == 1) qc.push_back({NSG_GATE_H, (uint32_t)i, 0, 0});
    layer(gamma1, delta1, false);
    return qc;
}

// measure (stabilizer_decomposed_state/measurement.rs:10-103)
static std::vector<uint8_t> sd_measure(SDState& st, const std::vector<int>& qargs, const uint8_t* seed) {
    validate_qargs(st, qargs);
    Rng rng(seed);
    std::vector<uint8_t> out;
    for (int q : qargs) {
        SDState z = st, o = st;
        project_unnormalized(z, q, false);
        project_unnormalized(o, q, true);
        double p0 = norm_squared(z), p1 = norm_squared(o);
        double tot = p0 + p1;
        if (std::fabs(tot) < 1e-12) fail(NSG_ERR_NOT_IMPLEMENTED, -1, -1, "Measurement on a zero-norm state is not possible.");
        double u = rng.uniform();
        bool res = !(u < p0 / tot);
        double nsq = res ? p1 : p0;
        st = res ? o : z;
        double nrm = std::sqrt(nsq);
        if (std::fabs(nrm) < 1e-12) fail(NSG_ERR_NOT_IMPLEMENTED, -1, -1, "Measurement resulted in a zero-norm state, which is not physical.");
        st.global_factor = st.global_factor * cplx(1.0 / nrm, 0.0);
        out.push_back(res ? 1 : 0);
    }
    return out;
}

// Exact marginal distribution of `qargs` (bit i of the outcome ↔ qargs[i]),
// by the same project/discard recursion as sampling.rs:80-189 with every branch
// taken; used as the reference distribution for sampling tests.
static void marginal_rec(const SDState& st, const std::vector<std::pair<int, int>>& qs, size_t idx,
                         uint64_t outcome, double prob, std::map<uint64_t, double>& out) {
    if (prob <= 0.0) return;
    if (idx == qs.size()) {
        out[outcome] += prob;
        return;
    }
    int q = qs[idx].first, bit = qs[idx].second;
    SDState z = st, o = st;
    project_unnormalized(z, q, false);
    project_unnormalized(o, q, true);
    double n0 = norm_squared(z), n1 = norm_squared(o);
    double p0 = std::min(1.0, std::max(0.0, n0 / (n0 + n1)));
    if (p0 > 0.0) {
        sd_discard(z, q);
        marginal_rec(z, qs, idx + 1, outcome, prob * p0, out);
    }
    if (p0 < 1.0) {
        for (auto& c : o.stabs) left_x(c, q);
        sd_discard(o, q);
        marginal_rec(o, qs, idx + 1, outcome | (1ULL << bit), prob * (1.0 - p0), out);
    }
}

// ---------------------------------------------------------------------------
// Dense statevector simulator (restated from
// crates/stabilizer-ch-form-rust/tests/common/mod.rs:108-200), extended with
// T/Tdg, used as an independent check.
static void dense_apply(std::vector<cplx>& sv, int n, const nsg_gate& g) {
    size_t dim = (size_t)1 << n;
    const double r2 = 0.70710678118654752440;
    auto one = [&](int q, cplx m00, cplx m01, cplx m10, cplx m11) {
        for (size_t i = 0; i < dim; i++) {
            if (((i >> q) & 1) == 0) {
                size_t j = i | ((size_t)1 << q);
                cplx a = sv[i], b = sv[j];
                sv[i] = m00 * a + m01 * b;
                sv[j] = m10 * a + m11 * b;
            }
        }
    };
    int a = (int)g.q0, b = (int)g.q1;
    cplx I(0, 1);
    switch (g.op) {
        case NSG_GATE_H: one(a, r2, r2, r2, -r2); break;
        case NSG_GATE_X: one(a, 0, 1, 1, 0); break;
        case NSG_GATE_Y: one(a, 0, -I, I, 0); break;
        case NSG_GATE_Z: one(a, 1, 0, 0, -1); break;
        case NSG_GATE_S: one(a, 1, 0, 0, I); break;
        case NSG_GATE_SDG: one(a, 1, 0, 0, -I); break;
        case NSG_GATE_SQRT_X: one(a, cplx(0.5, 0.5), cplx(0.5, -0.5), cplx(0.5, -0.5), cplx(0.5, 0.5)); break;
        case NSG_GATE_SQRT_XDG: one(a, cplx(0.5, -0.5), cplx(0.5, 0.5), cplx(0.5, 0.5), cplx(0.5, -0.5)); break;
        case NSG_GATE_T: one(a, 1, 0, 0, cplx(r2, r2)); break;
        case NSG_GATE_TDG: one(a, 1, 0, 0, cplx(r2, -r2)); break;
        case NSG_GATE_CX:
            for (size_t i = 0; i < dim; i++)
                if (((i >> a) & 1) && !((i >> b) & 1)) std::swap(sv[i], sv[i | ((size_t)1 << b)]);
            break;
        case NSG_GATE_CZ:
            for (size_t i = 0; i < dim; i++)
                if (((i >> a) & 1) && ((i >> b) & 1)) sv[i] = -sv[i];
            break;
        case NSG_GATE_SWAP:
            for (size_t i = 0; i < dim; i++) {
                size_t b1 = (i >> a) & 1, b2 = (i >> b) & 1;
                if (b1 != b2) {
                    size_t j = i ^ ((size_t)1 << a) ^ ((size_t)1 << b);
                    if (i < j) std::swap(sv[i], sv[j]);
                }
            }
            break;
        default: fail(NSG_ERR_GATE_NOT_SUPPORTED, g.op);
    }
}

}  // namespace orc

// ===========================================================================
// C API used by the tests (ctypes) and by bench.py's CPU-baseline leg.
using namespace orc;

static thread_local std::string g_err_msg;
static thread_local int64_t g_err_args[3] = {-1, -1, -1};

static int set_err(const Error& e) {
    g_err_msg = e.msg;
    g_err_args[0] = e.a;
    g_err_args[1] = e.b;
    g_err_args[2] = e.c;
    return e.code;
}

#define ORC_TRY try {
#define ORC_CATCH                                      \
    }                                                  \
    catch (const Error& e) { return set_err(e); }      \
    catch (const std::exception& e) {                  \
        g_err_msg = e.what();                          \
        return NSG_ERR_INVALID_ARGUMENT;               \
    }                                                  \
    return NSG_OK;

extern "C" {

const char* orc_last_error_message(void) { return g_err_msg.c_str(); }
void orc_last_error_args(int64_t out[3]) {
    for (int i = 0; i < 3; i++) out[i] = g_err_args[i];
}

int orc_state_from_circuit(uint32_t n, const nsg_gate* gates, size_t ng, void** out) {
    ORC_TRY
    std::vector<nsg_gate> gv(gates, gates + ng);
    *out = new SDState(compile((int)n, gv));
    ORC_CATCH
}

int orc_t_tensor_state(uint32_t t, void** out) {
    ORC_TRY
    *out = new SDState(construct_t_tensor((int)t));
    ORC_CATCH
}

int orc_cat_state(uint32_t t, void** out) {
    ORC_TRY
    *out = new SDState(construct_cat((int)t));
    ORC_CATCH
}

// Terms tidx[0..count) of the T-tensor state |T⟩^{⊗t}, each built on its own.
int orc_t_tensor_terms(uint32_t t, const int64_t* tidx, size_t count, void** out) {
    ORC_TRY
    SDState* st = new SDState();
    st->num_qubits = (int)t;
    for (size_t i = 0; i < count; i++) {
        auto tt = t_tensor_term((int)t, tidx[i]);
        st->stabs.push_back(tt.first);
        st->coeffs.push_back(tt.second);
    }
    *out = st;
    ORC_CATCH
}

int orc_toffoli_tensor_state(uint32_t k, void** out) {
    ORC_TRY
    *out = new SDState(construct_toffoli_tensor((int)k));
    ORC_CATCH
}

int orc_t_tensor_rank(uint32_t t, uint64_t* out) {
    ORC_TRY
    *out = t == 0 ? 1 : (uint64_t)t_tensor_rank((int)t);
    ORC_CATCH
}

// The compile loop over the chosen T-tensor terms only (kept[i] per term).
int orc_compile_terms(uint32_t n, const nsg_gate* gates, size_t ng, const int64_t* tidx, size_t count,
                      int32_t threads, uint8_t* kept, void** out) {
    ORC_TRY
    std::vector<nsg_gate> gv(gates, gates + ng);
    std::vector<int64_t> ti(tidx, tidx + count);
    *out = new SDState(compile_terms((int)n, gv, ti, kept, threads));
    ORC_CATCH
}

// Signed counts of the real parts of exp_value's pair terms per power of
// √2 (counts[o·bins + m + m_off]), and each observable's exact value.
int orc_exp_value_counts(void* stv, const nsg_pauli* ps, size_t nobs, int32_t threads, int64_t m_off, int64_t bins,
                         int64_t* counts, double* exact) {
    ORC_TRY
    SDState* st = (SDState*)stv;
    std::vector<Pauli> pv;
    for (size_t o = 0; o < nobs; o++) pv.push_back(pauli_from_abi(&ps[o]));
    exp_value_counts(*st, pv, threads, m_off, bins, counts);
    const double gf2 = std::norm(st->global_factor);
    for (size_t o = 0; o < nobs; o++) exact[o] = counts_value(counts + o * bins, m_off, bins) * gf2;
    ORC_CATCH
}

// Σ_m counts[m + m_off]·2^(-m/2), exactly, rounded once (for counts from any source).
int orc_counts_value(const int64_t* counts, int64_t m_off, int64_t bins, double* out) {
    ORC_TRY
    *out = counts_value(counts, m_off, bins);
    ORC_CATCH
}

int orc_state_from_terms(uint32_t n, uint64_t chi, const uint8_t* G, const uint8_t* F, const uint8_t* M,
                         const uint8_t* gamma, const uint8_t* v, const uint8_t* s, const uint8_t* phase,
                         const uint8_t* coef_phase, const int32_t* coef_r, const uint8_t* coef_zero,
                         const double gf[2], void** out) {
    ORC_TRY
    SDState* st = new SDState();
    st->num_qubits = (int)n;
    size_t nn = (size_t)n * n;
    for (uint64_t t = 0; t < chi; t++) {
        ChForm c = ch_new((int)n);
        std::memcpy(c.G.data(), G + t * nn, nn);
        std::memcpy(c.F.data(), F + t * nn, nn);
        std::memcpy(c.M.data(), M + t * nn, nn);
        std::memcpy(c.gamma.data(), gamma + t * n, n);
        std::memcpy(c.v.data(), v + t * n, n);
        std::memcpy(c.s.data(), s + t * n, n);
        c.phase = phase[t];
        st->stabs.push_back(std::move(c));
        st->coeffs.push_back(Scalar{coef_zero[t] != 0, coef_phase[t], coef_r[t]});
    }
    st->global_factor = cplx(gf[0], gf[1]);
    *out = st;
    ORC_CATCH
}

void orc_state_free(void* st) { delete (SDState*)st; }

int orc_state_kron(void* a, void* b, void** out) {
    ORC_TRY
    *out = new SDState(sd_kron(*(SDState*)a, *(SDState*)b));
    ORC_CATCH
}

int orc_state_clone(void* st, void** out) {
    ORC_TRY
    *out = new SDState(*(SDState*)st);
    ORC_CATCH
}

int orc_num_qubits(void* st, uint32_t* out) {
    *out = (uint32_t)((SDState*)st)->num_qubits;
    return 0;
}
int orc_stabilizer_rank(void* st, uint64_t* out) {
    *out = ((SDState*)st)->stabs.size();
    return 0;
}

int orc_export_terms(void* stv, uint8_t* G, uint8_t* F, uint8_t* M, uint8_t* gamma, uint8_t* v, uint8_t* s,
                     uint8_t* phase, uint8_t* coef_phase, int32_t* coef_r, uint8_t* coef_zero, double gf[2]) {
    ORC_TRY
    SDState* st = (SDState*)stv;
    size_t n = (size_t)st->num_qubits, nn = n * n;
    for (size_t t = 0; t < st->stabs.size(); t++) {
        const ChForm& c = st->stabs[t];
        if ((size_t)c.n != n) fail(NSG_ERR_DEVICE_INVARIANT, 6);
        std::memcpy(G + t * nn, c.G.data(), nn);
        std::memcpy(F + t * nn, c.F.data(), nn);
        std::memcpy(M + t * nn, c.M.data(), nn);
        std::memcpy(gamma + t * n, c.gamma.data(), n);
        std::memcpy(v + t * n, c.v.data(), n);
        std::memcpy(s + t * n, c.s.data(), n);
        phase[t] = (uint8_t)c.phase;
        coef_phase[t] = (uint8_t)st->coeffs[t].k;
        coef_r[t] = (int32_t)st->coeffs[t].r;
        coef_zero[t] = st->coeffs[t].zero ? 1 : 0;
    }
    gf[0] = st->global_factor.real();
    gf[1] = st->global_factor.imag();
    ORC_CATCH
}

int orc_apply_gates(void* st, const nsg_gate* gates, size_t ng) {
    ORC_TRY
    for (size_t i = 0; i < ng; i++) sd_apply_gate(*(SDState*)st, gates[i]);
    ORC_CATCH
}

int orc_exp_value(void* st, const nsg_pauli* p, double* out, double* exact) {
    ORC_TRY
    *out = exp_value(*(SDState*)st, pauli_from_abi(p), exact);
    ORC_CATCH
}

int orc_norm(void* st, double* out, double* exact_sq) {
    ORC_TRY
    *out = std::sqrt(norm_squared(*(SDState*)st, exact_sq));
    ORC_CATCH
}

int orc_inner_product(void* a, void* b, double out[2], double exact[2]) {
    ORC_TRY
    cplx ex;
    cplx r = sd_inner_product(*(SDState*)a, *(SDState*)b, &ex);
    out[0] = r.real();
    out[1] = r.imag();
    if (exact) {
        exact[0] = ex.real();
        exact[1] = ex.imag();
    }
    ORC_CATCH
}

// Exact value of one pair term ⟨S_i| P |S_j⟩ as the CH-form Scalar (without
// coefficients).  P may be NULL (identity).  The reference evaluates
// S_i.inner_product(P·S_j) (exp_value.rs:38-57).
int orc_pair_scalar(void* stv, uint64_t i, uint64_t j, const nsg_pauli* p, int32_t* zero, int32_t* k, int64_t* r) {
    ORC_TRY
    SDState* st = (SDState*)stv;
    ChForm ev = st->stabs[j];
    if (p) apply_pauli(ev, pauli_from_abi(p));
    Scalar sc = ch_inner_product_scalar(st->stabs[i], ev);
    *zero = sc.zero;
    *k = sc.k;
    *r = sc.r;
    ORC_CATCH
}

int orc_project_unnormalized(void* st, uint32_t q, int32_t outcome) {
    ORC_TRY
    project_unnormalized(*(SDState*)st, (int)q, outcome != 0);
    ORC_CATCH
}
int orc_project_normalized(void* st, uint32_t q, int32_t outcome) {
    ORC_TRY
    project_normalized(*(SDState*)st, (int)q, outcome != 0);
    ORC_CATCH
}
int orc_discard(void* st, uint32_t q) {
    ORC_TRY
    SDState* s = (SDState*)st;
    if ((int)q >= s->num_qubits) fail(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, q, s->num_qubits);
    sd_discard(*s, (int)q);
    ORC_CATCH
}

int orc_measure(void* st, const uint32_t* qargs, size_t k, const uint8_t* seed32, uint8_t* out) {
    ORC_TRY
    std::vector<int> q(qargs, qargs + k);
    std::vector<uint8_t> r = sd_measure(*(SDState*)st, q, seed32);
    std::memcpy(out, r.data(), r.size());
    ORC_CATCH
}

int orc_random_clifford(uint32_t n, const uint8_t* seed32, nsg_gate* out, size_t cap, size_t* nout) {
    ORC_TRY
    std::vector<nsg_gate> g = rc_random_clifford((int)n, seed32);
    *nout = g.size();
    if (g.size() > cap) fail(NSG_ERR_BUFFER_TOO_SMALL, (int64_t)g.size(), (int64_t)cap);
    std::copy(g.begin(), g.end(), out);
    ORC_CATCH
}

int orc_random_words(const uint8_t* seed32, uint32_t* out, size_t count) {
    ORC_TRY
    Rng rng(seed32);
    for (size_t i = 0; i < count; i++) out[i] = rng.next_u32();
    ORC_CATCH
}

int orc_random_doubles(const uint8_t* seed32, double* out, size_t count) {
    ORC_TRY
    Rng rng(seed32);
    for (size_t i = 0; i < count; i++) out[i] = rng.uniform();
    ORC_CATCH
}

int orc_chacha_block(const uint32_t* input, int32_t rounds, uint32_t* out) {
    ORC_TRY
    chacha_block_words(input, rounds, out);
    ORC_CATCH
}

// Exact marginal of qargs: writes up to `cap` (outcome, probability) pairs.
int orc_marginal(void* stv, const uint32_t* qargs, size_t k, uint64_t* outcomes, double* probs, size_t cap,
                 size_t* nout) {
    ORC_TRY
    SDState* st = (SDState*)stv;
    std::vector<int> q(qargs, qargs + k);
    validate_qargs(*st, q);
    if (k > 64) fail(NSG_ERR_SAMPLING_TOO_MANY_QUBITS);
    std::vector<std::pair<int, int>> sorted;
    for (size_t i = 0; i < k; i++) sorted.push_back({(int)qargs[i], (int)i});
    std::sort(sorted.begin(), sorted.end(), [](auto& a, auto& b) { return a.first > b.first; });
    std::map<uint64_t, double> mp;
    marginal_rec(*st, sorted, 0, 0, 1.0, mp);
    *nout = mp.size();
    size_t i = 0;
    for (auto& kv : mp) {
        if (i >= cap) break;
        outcomes[i] = kv.first;
        probs[i] = kv.second;
        i++;
    }
    ORC_CATCH
}

int orc_to_statevector(void* st, double* out, size_t cap) {
    ORC_TRY
    std::vector<cplx> sv = sd_statevector(*(SDState*)st);
    if (sv.size() > cap) fail(NSG_ERR_BUFFER_TOO_SMALL, (int64_t)sv.size(), (int64_t)cap);
    for (size_t i = 0; i < sv.size(); i++) {
        out[2 * i] = sv[i].real();
        out[2 * i + 1] = sv[i].imag();
    }
    ORC_CATCH
}

// Dense statevector of a Clifford+T circuit from |0^n⟩ (independent check).
int orc_dense_simulate(uint32_t n, const nsg_gate* gates, size_t ng, double* out) {
    ORC_TRY
    if (n > 24) fail(NSG_ERR_STATEVECTOR_TOO_LARGE, n);
    std::vector<cplx> sv((size_t)1 << n, cplx(0, 0));
    sv[0] = 1.0;
    for (size_t i = 0; i < ng; i++) dense_apply(sv, (int)n, gates[i]);
    for (size_t i = 0; i < sv.size(); i++) {
        out[2 * i] = sv[i].real();
        out[2 * i + 1] = sv[i].imag();
    }
    ORC_CATCH
}

// Single CH-form checks: apply a Clifford list to |0^n⟩ and dump its bits and
// statevector (gate-API known-answer tests, tests/gate_api.rs:6-61).
int orc_chform_run(uint32_t n, const nsg_gate* gates, size_t ng, uint8_t* G, uint8_t* F, uint8_t* M,
                   uint8_t* gamma, uint8_t* v, uint8_t* s, uint8_t* phase, double* sv_out) {
    ORC_TRY
    ChForm c = ch_new((int)n);
    for (size_t i = 0; i < ng; i++) apply_clifford(c, gates[i]);
    size_t nn = (size_t)n * n;
    if (G) {
        std::memcpy(G, c.G.data(), nn);
        std::memcpy(F, c.F.data(), nn);
        std::memcpy(M, c.M.data(), nn);
        std::memcpy(gamma, c.gamma.data(), n);
        std::memcpy(v, c.v.data(), n);
        std::memcpy(s, c.s.data(), n);
        *phase = (uint8_t)c.phase;
    }
    if (sv_out) {
        std::vector<cplx> sv = ch_statevector(c);
        for (size_t i = 0; i < sv.size(); i++) {
            sv_out[2 * i] = sv[i].real();
            sv_out[2 * i + 1] = sv[i].imag();
        }
    }
    ORC_CATCH
}

// CPU baseline timing: evaluates `num_pairs` pair terms of exp_value(P) with the
// reference algorithm (clone S_i, apply P, S_j.inner_product), drawn uniformly
// from the upper triangle (j ≥ i), over `threads` host threads.  Returns the
// wall time in seconds; the per-pair cost is the reference's.
int orc_time_pairs(void* stv, const nsg_pauli* p, uint64_t num_pairs, uint64_t seed, int32_t threads,
                   double* seconds, double* checksum) {
    ORC_TRY
    SDState* st = (SDState*)stv;
    Pauli pl = pauli_from_abi(p);
    validate_pauli(*st, pl);
    size_t chi = st->stabs.size();
    if (threads < 1) threads = 1;
    std::vector<double> sums(threads, 0.0);
    std::atomic<uint64_t> next{0};
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    std::vector<Error> errs;
    std::mutex emu;
    for (int th = 0; th < threads; th++) {
        pool.emplace_back([&, th]() {
            try {
                uint64_t x = seed * 0x9E3779B97F4A7C15ULL + (uint64_t)th + 1;
                double acc = 0.0;
                while (true) {
                    uint64_t idx = next.fetch_add(1);
                    if (idx >= num_pairs) break;
                    uint64_t h1 = splitmix(x), h2 = splitmix(x);
                    size_t i = (size_t)(h1 % chi), j = (size_t)(h2 % chi);
                    if (j < i) std::swap(i, j);
                    ChForm ev = st->stabs[i];
                    apply_pauli(ev, pl);
                    Scalar ip = ch_inner_product_scalar(st->stabs[j], ev);
                    Scalar cc = scalar_mul(scalar_conj(st->coeffs[j]), st->coeffs[i]);
                    cplx term = cmul(scalar_to_complex(cc), scalar_to_complex(ip));
                    acc += term.real();
                }
                sums[th] = acc;
            } catch (const Error& e) {
                std::lock_guard<std::mutex> lk(emu);
                errs.push_back(e);
            }
        });
    }
    for (auto& t : pool) t.join();
    auto t1 = std::chrono::steady_clock::now();
    if (!errs.empty()) throw errs[0];
    *seconds = std::chrono::duration<double>(t1 - t0).count();
    double cs = 0.0;
    for (double v : sums) cs += v;
    *checksum = cs;
    ORC_CATCH
}

}  // extern "C"
