// api.cu — the C ABI (include/necstar_gpu.h): state handles, validation in
// the reference's error order, gate lowering, and the host drivers of
// projection, measurement and sampling.  All heavy work runs in the kernels
// of kernels_terms.cu and kernels_pairs.cu; nothing here falls back to a CPU
// implementation of the pair sums or of the CH-form updates of compiled
// terms (the |T⟩^{⊗t} expansion, a per-t constant input, is built on the
// host once per process and cached).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/necstar_gpu.h"
#include "chform_host.hpp"
#include "device_state.hpp"
#include "host_rng.hpp"
#include "random_clifford.hpp"

using namespace nsg;

// ---------------------------------------------------------------------------
// Errors
namespace {

thread_local std::string g_msg;
thread_local int64_t g_args[3] = {-1, -1, -1};

struct ApiError {
    nsg_status code;
};

[[noreturn]] void raise(nsg_status code, int64_t a, int64_t b, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_msg = buf;
    g_args[0] = a;
    g_args[1] = b;
    g_args[2] = -1;
    throw ApiError{code};
}

const char* gate_name(uint32_t op) {  // QuantumGate::name (crates/necstar/src/circuit/gates.rs:209-226)
    static const char* names[] = {"H", "X", "Y", "Z", "S", "Sdg", "SqrtX", "SqrtXdg",
                                  "CX", "CZ", "Swap", "T", "Tdg", "CCX"};
    return op < 14 ? names[op] : "?";
}

// Messages follow the thiserror texts of crates/necstar/src/error/mod.rs:10-91
// and crates/stabilizer-ch-form-rust/src/error/mod.rs:7-67.
[[noreturn]] void err_oob(int64_t q, int64_t n) {
    raise(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, q, n, "Qubit index %lld is out of bounds for %lld qubits.",
          (long long)q, (long long)n);
}
[[noreturn]] void err_dup_gate(int64_t q) {
    raise(NSG_ERR_DUPLICATE_QUBIT_INDICES, q, -1,
          "Two-qubit gate requires two different qubit indices, but got the same: %lld.", (long long)q);
}
[[noreturn]] void err_impossible(int64_t q, bool desired) {
    raise(NSG_ERR_IMPOSSIBLE_PROJECTION, q, desired ? 1 : 0,
          "Impossible projection on qubit %lld: cannot project determined state |%d> onto |%d>.", (long long)q,
          desired ? 0 : 1, desired ? 1 : 0);
}

void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        raise(NSG_ERR_CUDA, (int64_t)e, -1, "CUDA error in %s: %s", what, cudaGetErrorString(e));
    }
}
#define CK(x) cuda_check((x), #x)

// ---------------------------------------------------------------------------
// Device buffers
template <typename T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    cudaStream_t st = nullptr;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    DBuf(DBuf&& o) noexcept { *this = std::move(o); }
    DBuf& operator=(DBuf&& o) noexcept {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            st = o.st;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    void alloc(size_t count, cudaStream_t s) {
        release();
        st = s;
        n = count;
        if (count) {
            cudaError_t e = cudaMallocAsync((void**)&p, count * sizeof(T), s);
            if (e == cudaErrorMemoryAllocation)
                raise(NSG_ERR_OUT_OF_MEMORY, (int64_t)(count * sizeof(T)), -1, "device allocation of %zu bytes failed",
                      count * sizeof(T));
            cuda_check(e, "cudaMallocAsync");
        }
    }
    void rehome(cudaStream_t s) { st = s; }
    // Freed with cudaFree (it waits for the device), not stream-ordered: after
    // states made of hundreds of per-stream buffers were freed with
    // cudaFreeAsync, later stream-ordered allocations and launches slowed down
    // 10-30x on GB300 (a second batch of 512 compiles: 11-33 s instead of
    // 1.2 s); with cudaFree every repeat took 1.2 s.  cudaFree waits for the
    // work on the device, so a launch still reading the buffer is never cut
    // short; no buffer is freed inside a stream capture.
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    ~DBuf() { release(); }
};

struct TermStore {
    int n = 0, W = 1, R = 64;
    int64_t chi = 0, cap = 0;
    DBuf<uint64_t> G, F, M, V, S, GL, GH;
    DBuf<uint8_t> phase, ck;
    DBuf<int32_t> cr;

    void alloc(int n_, int64_t cap_, cudaStream_t st) {
        n = n_;
        W = n <= 64 ? 1 : 2;
        R = 64 * W;
        cap = std::max<int64_t>(cap_, 1);
        size_t rows = (size_t)cap * R * W, vec = (size_t)cap * W;
        G.alloc(rows, st);
        F.alloc(rows, st);
        M.alloc(rows, st);
        V.alloc(vec, st);
        S.alloc(vec, st);
        GL.alloc(vec, st);
        GH.alloc(vec, st);
        phase.alloc(cap, st);
        ck.alloc(cap, st);
        cr.alloc(cap, st);
    }
    void rehome(cudaStream_t st) {
        G.rehome(st); F.rehome(st); M.rehome(st); V.rehome(st); S.rehome(st);
        GL.rehome(st); GH.rehome(st); phase.rehome(st); ck.rehome(st); cr.rehome(st);
    }
    TermsView view() const {
        TermsView t;
        t.n = n;
        t.W = W;
        t.R = R;
        t.chi = chi;
        t.G = G.p;
        t.F = F.p;
        t.M = M.p;
        t.V = V.p;
        t.S = S.p;
        t.GL = GL.p;
        t.GH = GH.p;
        t.phase = phase.p;
        t.coef_k = ck.p;
        t.coef_r = cr.p;
        return t;
    }
    void copy_from(const TermStore& o, cudaStream_t st) {
        alloc(o.n, std::max<int64_t>(o.chi, 1), st);
        W = o.W;
        R = o.R;
        chi = o.chi;
        size_t rows = (size_t)chi * R * W, vec = (size_t)chi * W;
        CK(cudaMemcpyAsync(G.p, o.G.p, rows * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(F.p, o.F.p, rows * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(M.p, o.M.p, rows * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(V.p, o.V.p, vec * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(S.p, o.S.p, vec * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(GL.p, o.GL.p, vec * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(GH.p, o.GH.p, vec * 8, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(phase.p, o.phase.p, chi, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(ck.p, o.ck.p, chi, cudaMemcpyDeviceToDevice, st));
        CK(cudaMemcpyAsync(cr.p, o.cr.p, chi * 4, cudaMemcpyDeviceToDevice, st));
    }
};

// ---------------------------------------------------------------------------
// |T⟩^{⊗t} expansion, cached per t (host) and per (device, t) (device).
// Device copy of the expansion; allocated once per (device, t) with plain
// cudaMalloc and kept for the life of the process (never freed, so no CUDA
// call runs from a static destructor).
struct TTensorDev {
    int64_t chi = 0;
    uint64_t *G = nullptr, *F = nullptr, *M = nullptr, *V = nullptr, *S = nullptr;
    uint8_t *gam = nullptr, *phase = nullptr, *ck = nullptr;
    int32_t* cr = nullptr;
};

template <typename T>
T* dev_alloc_forever(size_t count, cudaStream_t st) {  // zeroed in stream order
    T* p = nullptr;
    size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
    cudaError_t e = cudaMalloc((void**)&p, bytes);
    if (e == cudaErrorMemoryAllocation) raise(NSG_ERR_OUT_OF_MEMORY, (int64_t)bytes, -1, "device allocation failed");
    cuda_check(e, "cudaMalloc");
    cuda_check(cudaMemsetAsync(p, 0, bytes, st), "cudaMemsetAsync");
    return p;
}

std::mutex g_cache_mu;
std::map<std::pair<int, int>, std::shared_ptr<TTensorDev>> g_tt_dev;

TSmallTerm small_term(const HostCH& c, HScalar coef) {
    TSmallTerm r;
    std::memset(&r, 0, sizeof(r));
    for (int i = 0; i < c.n && i < 6; i++) {
        r.G[i] = c.G[i].w[0];
        r.F[i] = c.F[i].w[0];
        r.M[i] = c.M[i].w[0];
        r.gam[i] = c.gam[i];
    }
    r.v = c.v[0];
    r.s = c.s[0];
    r.phase = (uint8_t)c.phase;
    r.k = coef.k;
    r.r = coef.r;
    return r;
}

// The cat-state pieces the device expansion of |T⟩^{⊗t} joins (t ≤ 64): the
// terms of cat(m0) and of cat(6), built on the host (≤ 6 qubits each).
TPrelude t_prelude(int t) {
    TPrelude pre;
    pre.t = t;
    pre.L = t > 6 ? (t - 3) / 4 : 0;
    pre.m0 = t - 4 * pre.L;
    try {
        HostDecomp base = cat_state(pre.m0), six = cat_state(6);
        pre.nbase = (int)base.terms.size();
        for (int i = 0; i < pre.nbase; i++) pre.base[i] = small_term(base.terms[i], base.coef[i]);
        for (int j = 0; j < 3; j++) pre.cat6[j] = small_term(six.terms[j], six.coef[j]);
    } catch (const HostError& e) {
        raise(NSG_ERR_DEVICE_INVARIANT, e.code, e.a, "cat-state construction failed (%d)", e.code);
    }
    return pre;
}

// The expansion of |T⟩^{⊗t} on the device, built once per (device, t).
std::shared_ptr<TTensorDev> t_tensor_dev(int t, cudaStream_t st, int* status) {
    int dev = 0;
    CK(cudaGetDevice(&dev));
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        auto it = g_tt_dev.find({dev, t});
        if (it != g_tt_dev.end()) return it->second;
    }
    auto d = std::make_shared<TTensorDev>();
    CK(cudaStreamSynchronize(st));
    if (t == 0) {  // the Clifford-only circuit: one empty term, coefficient 1
        d->chi = 1;
        d->G = dev_alloc_forever<uint64_t>(1, st);
        d->F = dev_alloc_forever<uint64_t>(1, st);
        d->M = dev_alloc_forever<uint64_t>(1, st);
        d->gam = dev_alloc_forever<uint8_t>(1, st);
        d->V = dev_alloc_forever<uint64_t>(1, st);
        d->S = dev_alloc_forever<uint64_t>(1, st);
        d->phase = dev_alloc_forever<uint8_t>(1, st);
        d->ck = dev_alloc_forever<uint8_t>(1, st);
        d->cr = dev_alloc_forever<int32_t>(1, st);
        CK(cudaStreamSynchronize(st));  // the cache is shared by every stream
    } else {
        const TPrelude pre = t_prelude(t);
        int64_t chi_cat = pre.nbase;
        for (int l = 0; l < pre.L; l++) chi_cat *= 3;
        d->chi = 2 * chi_cat;
        const size_t rows = (size_t)d->chi * t;
        d->G = dev_alloc_forever<uint64_t>(rows, st);
        d->F = dev_alloc_forever<uint64_t>(rows, st);
        d->M = dev_alloc_forever<uint64_t>(rows, st);
        d->gam = dev_alloc_forever<uint8_t>(rows, st);
        d->V = dev_alloc_forever<uint64_t>(d->chi, st);
        d->S = dev_alloc_forever<uint64_t>(d->chi, st);
        d->phase = dev_alloc_forever<uint8_t>(d->chi, st);
        d->ck = dev_alloc_forever<uint8_t>(d->chi, st);
        d->cr = dev_alloc_forever<int32_t>(d->chi, st);
        TTensorOut o;
        o.G = d->G;
        o.F = d->F;
        o.M = d->M;
        o.V = d->V;
        o.S = d->S;
        o.gam = d->gam;
        o.phase = d->phase;
        o.ck = d->ck;
        o.cr = d->cr;
        CK(launch_t_tensor(pre, chi_cat, o, status, st));
        int h = 0;
        CK(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (h) {
            CK(cudaMemsetAsync(status, 0, sizeof(int), st));
            CK(cudaStreamSynchronize(st));
            raise(NSG_ERR_DEVICE_INVARIANT, h, t, "T-state expansion failed on the device (status %d, t = %d)", h, t);
        }
    }
    std::lock_guard<std::mutex> lk(g_cache_mu);
    auto it = g_tt_dev.find({dev, t});
    if (it != g_tt_dev.end()) return it->second;  // another thread finished first (its copy is kept)
    g_tt_dev[{dev, t}] = d;
    return d;
}

// ---------------------------------------------------------------------------
// Gate lowering with the reference's index checks.
//
// The reference checks indices when a gate is applied to a term
// (form/left_multiplication/*.rs): one-qubit gates check q < n; CX/CZ check
// control, then target, then equality; SWAP the same before its three CX;
// SqrtX/SqrtXdg check through their first H.  For a circuit with T gates
// the terms have width n+t during compilation (compiler/mod.rs:97-102).
void lower_clifford(const nsg_gate& g, int width, std::vector<uint32_t>& out) {
    auto chk1 = [&](uint32_t q) {
        if ((int64_t)q >= width) err_oob(q, width);
    };
    auto chk2 = [&](uint32_t a, uint32_t b) {
        chk1(a);
        chk1(b);
        if (a == b) err_dup_gate(a);
    };
    switch (g.op) {
        case NSG_GATE_H: chk1(g.q0); out.push_back(enc_op(P_H, g.q0)); break;
        case NSG_GATE_X: chk1(g.q0); out.push_back(enc_op(P_X, g.q0)); break;
        case NSG_GATE_Y: chk1(g.q0); out.push_back(enc_op(P_Y, g.q0)); break;
        case NSG_GATE_Z: chk1(g.q0); out.push_back(enc_op(P_Z, g.q0)); break;
        case NSG_GATE_S: chk1(g.q0); out.push_back(enc_op(P_S, g.q0)); break;
        case NSG_GATE_SDG: chk1(g.q0); out.push_back(enc_op(P_SDG, g.q0)); break;
        case NSG_GATE_SQRT_X:  // sqrt_x.rs:6-10
            chk1(g.q0);
            out.push_back(enc_op(P_H, g.q0));
            out.push_back(enc_op(P_S, g.q0));
            out.push_back(enc_op(P_H, g.q0));
            break;
        case NSG_GATE_SQRT_XDG:  // sqrt_x.rs:12-16
            chk1(g.q0);
            out.push_back(enc_op(P_H, g.q0));
            out.push_back(enc_op(P_SDG, g.q0));
            out.push_back(enc_op(P_H, g.q0));
            break;
        case NSG_GATE_CX: chk2(g.q0, g.q1); out.push_back(enc_op(P_CX, g.q0, g.q1)); break;
        case NSG_GATE_CZ: chk2(g.q0, g.q1); out.push_back(enc_op(P_CZ, g.q0, g.q1)); break;
        case NSG_GATE_SWAP:  // swap.rs:7-24
            chk2(g.q0, g.q1);
            out.push_back(enc_op(P_CX, g.q0, g.q1));
            out.push_back(enc_op(P_CX, g.q1, g.q0));
            out.push_back(enc_op(P_CX, g.q0, g.q1));
            break;
        default:
            raise(NSG_ERR_GATE_NOT_CLIFFORD, g.op, -1, "Attempted to convert a non-Clifford gate to a Clifford gate: %s",
                  gate_name(g.op));
    }
}

// ---------------------------------------------------------------------------
// Pauli strings -> bit form.  apply_pauli (form/gate_application.rs:186-210)
// multiplies the ops on from the left in list order; composing them here
// keeps repeated qubits exact.
DevPauli to_dev_pauli(const nsg_pauli& p, int n) {
    if (p.kind == NSG_PAULI_DENSE) {  // exp_value.rs:9-17
        if ((int)p.len != n)
            raise(NSG_ERR_INVALID_PAULI_STRING_LENGTH, n, p.len, "Invalid Pauli string length: expected %d, found %u.", n,
                  p.len);
    } else if (p.kind == NSG_PAULI_SPARSE) {  // :18-26
        uint32_t maxq = 0;
        for (uint32_t i = 0; i < p.len; i++) maxq = std::max(maxq, p.qubits ? p.qubits[i] : 0u);
        if ((int64_t)maxq >= n)
            raise(NSG_ERR_INVALID_PAULI_STRING_LENGTH, n, (int64_t)maxq + 1,
                  "Invalid Pauli string length: expected %d, found %u.", n, maxq + 1);
    } else {
        raise(NSG_ERR_INVALID_ARGUMENT, p.kind, -1, "invalid Pauli kind %u", p.kind);
    }
    if (p.len && !p.ops) raise(NSG_ERR_INVALID_ARGUMENT, -1, -1, "null Pauli ops");
    if (p.kind == NSG_PAULI_SPARSE && p.len && !p.qubits) raise(NSG_ERR_INVALID_ARGUMENT, -1, -1, "null Pauli qubits");
    DevPauli d{0, 0, 0, 0};
    int e = 0;  // P = i^e X(px) Z(pz)
    for (uint32_t i = 0; i < p.len; i++) {
        uint32_t q = (p.kind == NSG_PAULI_DENSE) ? i : p.qubits[i];
        uint8_t op = p.ops[i];
        uint64_t bit = 1ULL << q;
        int xq = (d.px >> q) & 1;
        switch (op) {
            case NSG_PAULI_I: break;
            case NSG_PAULI_X: d.px ^= bit; break;                           // X_q·X(px)Z(pz)
            case NSG_PAULI_Z: e += 2 * xq; d.pz ^= bit; break;              // Z_q X(px) = (-1)^{px_q} X(px) Z_q
            case NSG_PAULI_Y: e += 1 + 2 * xq; d.px ^= bit; d.pz ^= bit; break;  // Y = iXZ
            default: raise(NSG_ERR_INVALID_ARGUMENT, op, -1, "invalid Pauli op %u", op);
        }
    }
    d.ny = e & 3;
    return d;
}

}  // namespace

// ---------------------------------------------------------------------------
// Live states by identity, so a plan can tell a freed (or replaced) state.
static std::mutex g_states_mu;
static std::map<const nsg_state*, uint64_t> g_states;
static uint64_t g_next_uid = 1;

static uint64_t register_state(const nsg_state* s) {
    std::lock_guard<std::mutex> lk(g_states_mu);
    const uint64_t id = g_next_uid++;
    g_states[s] = id;
    return id;
}
static void unregister_state(const nsg_state* s) {
    std::lock_guard<std::mutex> lk(g_states_mu);
    g_states.erase(s);
}
static bool state_alive(const nsg_state* s, uint64_t uid) {
    std::lock_guard<std::mutex> lk(g_states_mu);
    auto it = g_states.find(s);
    return it != g_states.end() && it->second == uid;
}

// Stabilizers common to every term of a compiled state (the zero test of
// nsg_zero_screen).  The state is (1 ⊗ ⟨0|^t) U' (|0^n⟩ ⊗ |T⟩^{⊗t}) with U'
// the lowered circuit (T, Tdg = CX onto an ancilla [+ Sdg]); for a data
// Z string Z^a, R = U' (Z^a ⊗ 1) U'† satisfies R·U'(|0^n⟩ ⊗ φ) = U'(|0^n⟩ ⊗ φ)
// for every ancilla state φ, and when R has no X component on the ancillas
// (1 ⊗ ⟨0|^t) R = ±R_d (1 ⊗ ⟨0|^t), so ±R_d stabilizes every term.  A Pauli P
// that anticommutes with such an R_d has ⟨s_a|P|s_b⟩ = 0 for every pair, so
// ⟨P⟩ = 0 exactly.  Bit-sliced images (signs are not needed): bit j of
// sx[q] / sz[q] is the x / z bit at qubit q of the image of Z_j; the ancilla
// X parts span `anc` (an XOR basis, one vector per leading bit).  P = X(px)
// Z(pz) anticommutes with the image of Z^a iff a·v_P = 1, v_P = ⊕_{q ∈ px} sz[q]
// ⊕ ⊕_{q ∈ pz} sx[q]; such an a with no ancilla X part exists iff v_P is
// outside the span of the ancilla rows.
struct ZeroScreen {
    int n = 0;
    uint64_t sx[64] = {}, sz[64] = {};
    uint64_t anc[64] = {};  // anc[b]: the basis vector whose highest bit is b (0 = none)

    // Conjugation of every image by one primitive op (gates act on qubits < w).
    static void conj(uint64_t* X, uint64_t* Z, uint32_t code) {
        const uint32_t op = code & 0xff, a = (code >> 8) & 0xff, b = (code >> 16) & 0xff;
        switch (op) {
            case P_H: std::swap(X[a], Z[a]); break;
            case P_S:
            case P_SDG: Z[a] ^= X[a]; break;
            case P_CX: X[b] ^= X[a]; Z[a] ^= Z[b]; break;  // control a, target b
            case P_CZ: Z[a] ^= X[b]; Z[b] ^= X[a]; break;
            default: break;  // X, Y, Z change signs only
        }
    }
    void insert_anc(uint64_t v) {
        for (int bit = 63; bit >= 0 && v; bit--) {
            if (!((v >> bit) & 1)) continue;
            if (!anc[bit]) {
                anc[bit] = v;
                return;
            }
            v ^= anc[bit];
        }
    }
    bool zero(uint64_t px, uint64_t pz) const {
        uint64_t v = 0;
        for (int q = 0; q < n; q++) {
            if ((px >> q) & 1) v ^= sz[q];
            if ((pz >> q) & 1) v ^= sx[q];
        }
        for (int bit = 63; bit >= 0 && v; bit--)
            if (((v >> bit) & 1) && anc[bit]) v ^= anc[bit];
        return v != 0;
    }
    void apply(const std::vector<uint32_t>& ops) {  // Clifford gates on the n data qubits
        for (uint32_t c : ops) conj(sx, sz, c);
    }
};

// The zero test of a lowered circuit (n ≤ 64; null beyond).
std::shared_ptr<const ZeroScreen> screen_of(int n, int t, const std::vector<uint32_t>& ops) {
    if (n > 64) return nullptr;
    const int w = n + t;
    std::vector<uint64_t> X((size_t)w, 0), Z((size_t)w, 0);
    for (int j = 0; j < n; j++) Z[j] = 1ull << j;
    for (uint32_t c : ops) ZeroScreen::conj(X.data(), Z.data(), c);
    auto s = std::make_shared<ZeroScreen>();
    s->n = n;
    for (int q = 0; q < n; q++) {
        s->sx[q] = X[q];
        s->sz[q] = Z[q];
    }
    for (int q = n; q < w; q++) s->insert_anc(X[q]);
    return s;
}

struct nsg_state {
    int device = 0;
    cudaStream_t own = nullptr;
    cudaStream_t st = nullptr;
    TermStore t;
    double gf_re = 1.0, gf_im = 0.0;
    uint64_t uid = 0;         // process-unique identity (plans check it)
    uint64_t layout_gen = 0;  // bumped whenever the term storage is replaced or reshaped
    // Common stabilizers of the terms (compiled states, through Clifford
    // gates); null when unknown.  Shared between clones, replaced on change.
    std::shared_ptr<const ZeroScreen> screen;
    // cached bra frames
    bool frames_ok = false;
    DBuf<uint64_t> fGV, fFV, fMV, fGVL, fGVH;
    DBuf<int> status;
    // cached term tables (Four-Russians tables of every term, n ≤ 64)
    bool ket_ok = false;
    DBuf<unsigned char> ktab;

    const void* ket_tables() {
        if (!ket_ok) {
            ktab.alloc(std::max<size_t>((size_t)t.chi, 1) * ket_table_stride(t.n), st);
            CK(launch_ket_tables(t.view(), ktab.p, st));
            ket_ok = true;
        }
        return ktab.p;
    }

    void init_stream() {
        uid = register_state(this);
        CK(cudaGetDevice(&device));
        CK(cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking));
        st = own;
        // [0] status bits, [1] detail claimed, [2..4] where the first
        // invariant was seen (kernel-specific: pair i, j and qubit).
        status.alloc(8, st);
        CK(cudaMemsetAsync(status.p, 0, 8 * sizeof(int), st));
    }
    ~nsg_state() {
        unregister_state(this);
        // Finish work on the current stream, then free everything on our own.
        if (st) cudaStreamSynchronize(st);
        t.rehome(own);
        fGV.rehome(own);
        fFV.rehome(own);
        fMV.rehome(own);
        fGVL.rehome(own);
        fGVH.rehome(own);
        status.rehome(own);
        ktab.rehome(own);
        ktab.release();
        t = TermStore();
        fGV.release();
        fFV.release();
        fMV.release();
        fGVL.release();
        fGVH.release();
        status.release();
        if (own) {
            cudaStreamSynchronize(own);
            cudaStreamDestroy(own);
        }
    }
    void invalidate() {
        frames_ok = false;
        ket_ok = false;
    }
    FrameView frames() {
        if (!frames_ok) {
            size_t cap = (size_t)std::max<int64_t>(t.chi, 1);
            fGV.alloc(cap * 64, st);
            fFV.alloc(cap * 64, st);
            fMV.alloc(cap * 64, st);
            fGVL.alloc(cap, st);
            fGVH.alloc(cap, st);
            FrameView fr{fGV.p, fFV.p, fMV.p, fGVL.p, fGVH.p};
            CK(launch_frames(t.view(), fr, st));
            frames_ok = true;
        }
        return FrameView{fGV.p, fFV.p, fMV.p, fGVL.p, fGVH.p};
    }
    // Reads and clears the device status word; maps it to an API error.
    void check_status(int64_t qubit = -1) {
        int h[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        CK(cudaMemcpyAsync(h, status.p, sizeof(h), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (h[0]) {
            CK(cudaMemsetAsync(status.p, 0, sizeof(h), st));
            CK(cudaStreamSynchronize(st));
            if (h[0] & DS_CANNOT_DISCARD)
                raise(NSG_ERR_CANNOT_DISCARD_QUBIT, qubit, -1, "Cannot discard qubit %lld because it is not in a proper state",
                      (long long)qubit);
            if (h[0] & DS_TIMEOUT) raise(NSG_ERR_TIMEOUT, h[0], -1, "a bounded device wait ran out (status %d)", h[0]);
            if (h[0] == DS_RANGE)
                raise(NSG_ERR_INVALID_ARGUMENT, h[0], -1,
                      "a pair term's exponent fell outside the exact count bins (status %d)", h[0]);
            raise(NSG_ERR_DEVICE_INVARIANT, h[0], -1, "device invariant violated (status %d; at %d %d %d)", h[0], h[2],
                  h[3], h[4]);
        }
    }
};

namespace {

#define API_BEGIN try {
#define API_END                               \
    }                                         \
    catch (const ApiError& e) { return e.code; } \
    catch (const std::exception& e) {         \
        g_msg = e.what();                     \
        return NSG_ERR_INVALID_ARGUMENT;      \
    }                                         \
    return NSG_OK;

// Makes a state's device current for the length of a call (and restores the
// caller's): a state's memory and stream belong to the device that was current
// when it was created.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        int cur = 0;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != dev) {
            prev = cur;
            cudaSetDevice(dev);
        }
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

void need(const void* p, const char* what) {
    if (!p) raise(NSG_ERR_INVALID_ARGUMENT, -1, -1, "null %s", what);
}

void require_pairs_width(const nsg_state* s) {
    if (s->t.n > 64) raise(NSG_ERR_TOO_WIDE, s->t.n, 64, "pair sums support at most 64 qubits, got %d", s->t.n);
}

// Replaces the terms of `s` by the kept ones (stable order).
void compact_into(nsg_state* s, DBuf<int32_t>& keep) {
    TermStore out;
    out.alloc(s->t.n, std::max<int64_t>(s->t.chi, 1), s->st);
    out.W = s->t.W;
    out.R = s->t.R;
    DBuf<int32_t> pos;
    pos.alloc(std::max<int64_t>(s->t.chi, 1), s->st);
    DBuf<int64_t> cnt;
    cnt.alloc(1, s->st);
    TermsView ov = out.view();
    CK(launch_compact(s->t.view(), keep.p, pos.p, ov, cnt.p, s->st));
    int64_t h = 0;
    CK(cudaMemcpyAsync(&h, cnt.p, sizeof(int64_t), cudaMemcpyDeviceToHost, s->st));
    CK(cudaStreamSynchronize(s->st));
    out.chi = h;
    s->t = std::move(out);
    s->layout_gen++;
    s->invalidate();
    s->screen.reset();  // a projection: the common stabilizers are no longer known
}

// Process-wide pair-kernel timing (nsg_profile_*).
std::mutex g_prof_mu;
bool g_prof_on = false;
double g_prof_ms = 0.0;
uint64_t g_prof_launches = 0, g_prof_pairs = 0;

// One pair sum of the batched driver: the χ_A×χ_B pair space of (a, b)
// (triangular i ≤ j when a == b) for up to 256 observables.
struct PairUnit {
    nsg_state* a = nullptr;
    nsg_state* b = nullptr;
    const DevPauli* paulis = nullptr;  // host
    int nobs = 0;
    bool triangular = true;
    bool complex_out = false;
    double* out = nullptr;  // host: nobs values, or nobs (re, im) pairs when complex_out
    int64_t* counts = nullptr;  // exact mode (host): [nobs][2][kExactBins] signed counts (re, im)
};

constexpr int kMaxObsPerUnit = 256;  // 8 observable groups of 32 lanes

// Orders `st` after all work queued so far on `other`.
void join_stream(cudaStream_t st, cudaStream_t other) {
    if (other == st) return;
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, other));
    CK(cudaStreamWaitEvent(st, ev, 0));
    cudaEventDestroy(ev);
}

// Device sources of one unit: the bra state's frames and term tables and the
// ket state's term tables (a state's own caches, or a plan's copies).
struct UnitSources {
    FrameView fr;
    const void* atab = nullptr;
    const void* ktab = nullptr;
};

// ---- tuning of captured batches ----------------------------------------------
// The tiling of one row width that ran fastest on a sample, per device and
// workload class: kernel variant (blocks per SM its registers allow), tasks
// per resident warp and kets per chunk.  Also appended to the file named by
// NSG_TUNE_CACHE, one JSON object per line:
// {"key": "...", "minb": k, "tasks_per_warp": t, "chunk": c}.
struct TuneChoice {
    int minb = 0, tasks_per_warp = 64, chunk = 32;
};
std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune;
bool g_tune_loaded = false;
constexpr int kMinbCandidates[5] = {2, 3, 4, 5, 6};
// The most blocks per SM a variant of that row width has: six only for 32-bit
// rows (64-bit rows would spill at the 85 registers six blocks leave).
int max_minb(int wb) { return wb == 4 ? 6 : 5; }
constexpr int kTpwCandidates[3] = {16, 64, 256};
// Task records of one launch stay below this (tasks × observables × 64 B); a
// launch with many observables gets fewer, longer tasks.
constexpr int64_t kMaxRecordBytes = 512ll << 20;
constexpr int kChunkCandidates[3] = {16, 32, 64};

// Device names by ordinal (cudaGetDeviceProperties is slow; asked once per device).
std::string device_name(int device) {
    static std::mutex mu;
    static std::map<int, std::string> names;
    std::lock_guard<std::mutex> lk(mu);
    auto it = names.find(device);
    if (it != names.end()) return it->second;
    cudaDeviceProp prop;
    std::string name = "gpu";
    if (cudaGetDeviceProperties(&prop, device) == cudaSuccess) name = prop.name;
    for (char& c : name)
        if (c == '"' || c == '\\' || c == ' ') c = '_';
    names[device] = name;
    return name;
}

std::string tune_key(int device, int wb, int nobs_max, int n_mean, uint64_t pairs) {
    const std::string name = device_name(device);
    int lg = 0;
    while ((pairs >> lg) > 1) lg++;
    char buf[256];
    std::snprintf(buf, sizeof(buf), "%s|w%d|g%d|n%d|p%d", name.c_str(), wb * 8, (nobs_max + 31) / 32,
                  (n_mean + 7) / 8 * 8, lg / 2 * 2);
    return buf;
}

void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char* path = std::getenv("NSG_TUNE_CACHE");
    if (!path || !*path) return;
    FILE* f = std::fopen(path, "r");
    if (!f) return;
    char line[512];
    while (std::fgets(line, sizeof(line), f)) {
        char key[256];
        TuneChoice c;
        const int got = std::sscanf(line, " {\"key\": \"%255[^\"]\", \"minb\": %d, \"tasks_per_warp\": %d, \"chunk\": %d}",
                                    key, &c.minb, &c.tasks_per_warp, &c.chunk);
        if (got >= 2 && c.minb >= 2 && c.minb <= 6 && c.tasks_per_warp >= 1 && c.tasks_per_warp <= 1024 &&
            c.chunk >= 1 && c.chunk <= 1024)
            g_tune[key] = c;  // a line without the last two fields keeps their defaults
    }
    std::fclose(f);
}

bool tune_lookup(const std::string& key, TuneChoice& c) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load_locked();
    auto it = g_tune.find(key);
    if (it == g_tune.end()) return false;
    c = it->second;
    return true;
}

void tune_store(const std::string& key, const TuneChoice& c) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    tune_load_locked();
    g_tune[key] = c;
    const char* path = std::getenv("NSG_TUNE_CACHE");
    if (!path || !*path) return;
    if (FILE* f = std::fopen(path, "a")) {
        std::fprintf(f, "{\"key\": \"%s\", \"minb\": %d, \"tasks_per_warp\": %d, \"chunk\": %d}\n", key.c_str(),
                     c.minb, c.tasks_per_warp, c.chunk);
        std::fclose(f);
    }
}

// The pair-kernel variant when nothing was tuned for a workload class, from
// full-launch timings on GB300 (χ = 972 at n = 28 and 40, χ = 2916 at n = 60;
// 1, 64 and 256 observables; six blocks for 32-bit rows from the 512-circuit
// workload): six blocks per SM for 32-bit rows; for 64-bit rows four up to
// n = 48, beyond that three, or two with more than 128 observables (their
// per-lane state needs the registers).
int default_minb(int wb, int nobs_max, int n_mean) {
    if (wb == 4) return 6;
    if (n_mean <= 48) return 4;
    return nobs_max > 128 ? 2 : 3;
}

// Tiling of a pair launch, per row width ([0] 32-bit, [1] 64-bit rows): kets
// per chunk, tasks per resident warp and the kernel variant (blocks per SM its
// registers allow).  0 = the tuning cache's choice for the workload class,
// else the defaults: 32 kets, 64 tasks per warp, default_minb.  Many small
// tasks keep the warps that run at one time on neighbouring tasks — with the
// ket-major chunk order, on the same few ket blocks — so the ket tables they
// read stay in L2: on the 512-circuit workload's 64-bit launch 8 tasks per
// warp read 2.1 TB from DRAM, 128 read 3.4 GB (≈ the tables once) and ran
// 7.5 % faster.
struct PairTiling {
    int chunk[2] = {0, 0};
    int tasks_per_warp[2] = {0, 0};
    int minb[2] = {0, 0};
};

// The tiling of direct (uncaptured) pair sums: the defaults, or the values set
// by nsg_set_pair_tiling (0 keeps a default).
std::mutex g_tiling_mu;
PairTiling g_tiling_override;
PairTiling pair_tiling_override() {
    std::lock_guard<std::mutex> lk(g_tiling_mu);
    return g_tiling_override;
}
// Barrier-wait settings of the pair launches (nsg_debug_set_wait).
uint32_t g_poll_limit = 0, g_extra_tx = 0;

// Everything one batched evaluation needs on the device, built once
// (descriptors uploaded) and enqueued any number of times.
struct PairBatch {
    struct Launch {
        int wb = 8;
        MultiLaunch m;
        DBuf<unsigned char> blob;  // descriptors | task_begin | obs_begin | row-chunk prefixes
        DBuf<double> rec;          // task records, then the task counter
        const int64_t* d_obegin = nullptr;
        std::vector<int64_t> obegin;
        std::vector<size_t> units;  // indices into `live`
        size_t out_off = 0;         // first observable of this launch in `dout`
        std::vector<int64_t> task_pairs;  // pairs covered by tasks [0, k) (prefix, for sampled timing)
        int64_t pairs_total = 0;          // pairs of the whole launch
        size_t rec_used = 0;              // doubles of `rec` to clear before a launch (records, counter)
        double* red_scratch = nullptr;    // partials of the two-pass reduction
        int chunk = 32, tpw = 8, minb = 4;  // the tiling the launch was built with
    };
    std::vector<PairUnit*> live;
    std::vector<UnitSources> src;
    std::vector<size_t> unit_obs, unit_px, unit_out;  // per live unit
    DBuf<DevPauli> dp;
    DBuf<uint64_t> px;
    DBuf<uint8_t> pk;
    std::vector<Launch> launches;
    DBuf<double> dout;  // (re, im) per observable, launches concatenated
    DBuf<unsigned long long> dcounts;  // exact mode: [tot_obs][2][kExactBins]
    bool exact = false;
    size_t tot_obs = 0;
    uint64_t pairs = 0;
};

// with_samples: also the pair counts of the first tasks (for timing samples).
void build_batch(PairBatch& b, const PairTiling& tl, bool mixed, cudaStream_t st, bool with_samples = false,
                 uint8_t* dbg_k = nullptr, int32_t* dbg_r = nullptr, bool exact = false) {
    const size_t L = b.live.size();
    b.exact = exact;
    b.tot_obs = 0;
    size_t tot_px = 0;
    b.unit_obs.assign(L, 0);
    b.unit_px.assign(L, 0);
    b.unit_out.assign(L, 0);
    for (size_t k = 0; k < L; k++) {
        b.unit_obs[k] = b.tot_obs;
        b.unit_px[k] = tot_px;
        b.tot_obs += (size_t)b.live[k]->nobs;
        tot_px += (size_t)b.live[k]->a->t.chi * b.live[k]->nobs;
    }
    std::vector<DevPauli> hp;
    hp.reserve(b.tot_obs);
    for (PairUnit* u : b.live) hp.insert(hp.end(), u->paulis, u->paulis + u->nobs);
    b.dp.alloc(std::max<size_t>(b.tot_obs, 1), st);
    CK(cudaMemcpyAsync(b.dp.p, hp.data(), b.tot_obs * sizeof(DevPauli), cudaMemcpyHostToDevice, st));
    b.px.alloc(std::max<size_t>(tot_px, 1), st);
    b.pk.alloc(std::max<size_t>(tot_px, 1), st);
    b.dout.alloc(2 * std::max<size_t>(b.tot_obs, 1), st);
    if (exact) b.dcounts.alloc(std::max<size_t>(b.tot_obs, 1) * 2 * kExactBins, st);
    b.launches.clear();
    b.pairs = 0;
    size_t out_base = 0;
    for (int wb : {4, 8}) {
        std::vector<size_t> sel;
        for (size_t k = 0; k < L; k++)
            if ((b.live[k]->b->t.n <= 32 ? 4 : 8) == wb) sel.push_back(k);
        if (sel.empty()) continue;
        b.launches.emplace_back();
        PairBatch::Launch& ln = b.launches.back();
        ln.wb = wb;
        ln.units = sel;
        ln.out_off = out_base;
        // Host descriptors; row-chunk prefixes of the triangular units in one buffer.
        std::vector<PairDesc> descs(sel.size());
        std::vector<int64_t> tbegin(sel.size() + 1, 0), offs;
        ln.obegin.assign(sel.size() + 1, 0);
        std::vector<size_t> off_at(sel.size(), 0);
        size_t tab_max = 0, bra_max = 0;
        int nobs_max = 1;
        for (size_t q = 0; q < sel.size(); q++) nobs_max = std::max(nobs_max, b.live[sel[q]]->nobs);
        // The tiling of this row width: as given, else the tuning cache's choice
        // for the workload class, else the defaults.
        const int widx = wb == 4 ? 0 : 1;
        int chunk = tl.chunk[widx], tpw = tl.tasks_per_warp[widx];
        int minb = exact ? -1 : tl.minb[widx];
        if (minb == 0 || chunk == 0 || tpw == 0) {
            uint64_t pairs = 0, nsum = 0;
            for (size_t q = 0; q < sel.size(); q++) {
                const int64_t chi = b.live[sel[q]]->a->t.chi;
                pairs += (uint64_t)(chi * (chi + 1) / 2);
                nsum += (uint64_t)b.live[sel[q]]->a->t.n * (uint64_t)(chi * (chi + 1) / 2);
            }
            int dev = 0;
            CK(cudaGetDevice(&dev));
            const int n_mean = pairs ? (int)(nsum / pairs) : 0;
            TuneChoice c;
            const bool hit = tune_lookup(tune_key(dev, wb, nobs_max, n_mean, pairs), c);
            if (minb == 0) minb = hit ? std::min(c.minb, max_minb(wb)) : default_minb(wb, nobs_max, n_mean);
            if (tpw == 0) tpw = hit ? c.tasks_per_warp : TuneChoice().tasks_per_warp;
            if (chunk == 0) chunk = hit ? c.chunk : TuneChoice().chunk;
        }
        ln.chunk = chunk;
        ln.tpw = tpw;
        ln.minb = minb;
        for (size_t q = 0; q < sel.size(); q++) {
            PairUnit* u = b.live[sel[q]];
            const UnitSources& s = b.src[sel[q]];
            const int64_t chiA = u->a->t.chi, chiB = u->b->t.chi;
            PairDesc& d = descs[q];
            d.A = u->a->t.view();
            d.B = u->b->t.view();
            d.fr = s.fr;
            d.ktab = s.ktab;
            d.atab = s.atab;
            d.ktab_stride = ket_table_stride(u->b->t.n);
            d.ket_bytes = (uint32_t)ket_table_ket_bytes(u->b->t.n);
            d.ngrp = ket_table_groups(u->b->t.n);
            d.nobs = u->nobs;
            d.px = b.px.p + b.unit_px[sel[q]];
            d.pk = b.pk.p + b.unit_px[sel[q]];
            d.triangular = u->triangular ? 1 : 0;
            d.complex_out = u->complex_out ? 1 : 0;
            d.status = u->a->status.p;
            if (exact) d.counts = b.dcounts.p + b.unit_obs[sel[q]] * 2 * kExactBins;
            if (u->complex_out) {  // conj(g_a)·g_b (stabilizer_decomposed_state/inner_product.rs:18)
                d.scale_re = u->a->gf_re * u->b->gf_re + u->a->gf_im * u->b->gf_im;
                d.scale_im = u->a->gf_re * u->b->gf_im - u->a->gf_im * u->b->gf_re;
            } else {  // |g|² (exp_value.rs:60, norm.rs:29)
                d.scale_re = u->a->gf_re * u->a->gf_re + u->a->gf_im * u->a->gf_im;
                d.scale_im = 0.0;
            }
            // Ket-major chunks: ket block kb (kets kb·chunk ..) against every bra that
            // pairs with it (triangular: the bras up to the block's last ket).
            int64_t nch;
            d.nblk = (chiB + chunk - 1) / chunk;
            if (u->triangular) {
                off_at[q] = offs.size();
                int64_t acc = 0;
                for (int64_t kb = 0; kb < d.nblk; kb++) {
                    offs.push_back(acc);
                    acc += std::min<int64_t>((kb + 1) * chunk, chiA);
                }
                offs.push_back(acc);
                nch = acc;
                b.pairs += (uint64_t)(chiA * (chiA + 1) / 2);
            } else {
                nch = chiA * d.nblk;
                b.pairs += (uint64_t)(chiA * chiB);
            }
            d.nchunks = nch;
            ln.obegin[q + 1] = ln.obegin[q] + u->nobs;
            b.unit_out[sel[q]] = out_base + (size_t)ln.obegin[q];
            tab_max = std::max(tab_max, (size_t)d.ket_bytes);
            bra_max = std::max(bra_max, ket_table_bra_bytes(u->b->t.n));
        }
        out_base += (size_t)ln.obegin.back();
        for (const PairDesc& d : descs)  // imaginary parts are accumulated with one observable group only
            if (d.complex_out && nobs_max > 32)
                raise(NSG_ERR_INVALID_ARGUMENT, nobs_max, 32, "complex pair sums take at most 32 observables per launch");
        // Tasks: about tasks_per_warp per resident warp, never spanning two units.
        const size_t warp_smem = pair_warp_smem_bytes(tab_max, bra_max, wb);
        const int64_t resident = pair_resident_warps(wb, nobs_max, warp_smem, exact ? 0 : minb);
        int64_t total_chunks = 0;
        for (const PairDesc& d : descs) total_chunks += d.nchunks;
        const int64_t want = std::min<int64_t>((int64_t)tpw * resident,
                                               std::max<int64_t>(resident, kMaxRecordBytes / (64 * (int64_t)nobs_max)));
        const int64_t task_chunks = std::max<int64_t>(1, (total_chunks + want - 1) / want);
        int64_t rec_doubles = 0;
        for (size_t q = 0; q < sel.size(); q++) {
            const int64_t nt = (descs[q].nchunks + task_chunks - 1) / task_chunks;
            tbegin[q + 1] = tbegin[q] + nt;
            descs[q].rec0 = rec_doubles;
            rec_doubles += nt * descs[q].nobs * 8;
        }
        const int64_t total_tasks = tbegin.back();
        // Pairs covered by tasks [0, k) for the first tasks (two rounds of the
        // grid), for timing samples: pairs before chunk c of unit q in closed form.
        {
            auto pairs_before = [&](size_t q, int64_t c) -> int64_t {
                const PairUnit* u = b.live[sel[q]];
                const int64_t chiA = u->a->t.chi, chiB = u->b->t.chi;
                if (!u->triangular) {  // full blocks of χ_A bras, then r bras of block kb
                    const int64_t kb = c / chiA, r = c - kb * chiA;
                    const int64_t a = std::min<int64_t>(kb * chunk, chiB), e = std::min<int64_t>(a + chunk, chiB);
                    return a * chiA + r * (e - a);
                }
                const int64_t nblk = descs[q].nblk;
                const int64_t* off = offs.data() + off_at[q];
                const int64_t kb = (int64_t)(std::upper_bound(off, off + nblk + 1, c) - off) - 1;
                if (kb >= nblk) return chiA * (chiA + 1) / 2;
                // every pair with j below the block, then bras 0 .. r-1 against it
                const int64_t a = kb * chunk, e = std::min<int64_t>(a + chunk, chiA), r = c - off[kb];
                int64_t before = a * (a + 1) / 2;
                if (r <= a) return before + r * (e - a);
                return before + a * (e - a) + (r - a) * e - (r - a) * (a + r - 1) / 2;
            };
            ln.pairs_total = 0;
            for (size_t q = 0; q < sel.size(); q++) ln.pairs_total += pairs_before(q, descs[q].nchunks);
            const int64_t lim =
                with_samples ? std::min<int64_t>(total_tasks, 2 * (int64_t)tpw * resident) : 0;
            ln.task_pairs.assign((size_t)lim + 1, 0);
            int64_t before = 0;  // pairs of the units before q
            size_t q = 0;
            for (int64_t k = 1; k <= lim; k++) {
                while (k > tbegin[q + 1]) {
                    before += pairs_before(q, descs[q].nchunks);
                    q++;
                }
                ln.task_pairs[(size_t)k] =
                    before + pairs_before(q, std::min<int64_t>((k - tbegin[q]) * task_chunks, descs[q].nchunks));
            }
        }
        // One buffer: descriptors | task_begin | obs_begin | row-chunk prefixes.
        const size_t b_desc = sel.size() * sizeof(PairDesc);
        const size_t b_db = tbegin.size() * 8, b_ob = ln.obegin.size() * 8, b_off = offs.size() * 8;
        ln.blob.alloc(b_desc + b_db + b_ob + b_off, st);
        int64_t* d_db = (int64_t*)(ln.blob.p + b_desc);
        int64_t* d_ob = (int64_t*)(ln.blob.p + b_desc + b_db);
        int64_t* d_off = (int64_t*)(ln.blob.p + b_desc + b_db + b_ob);
        for (size_t q = 0; q < sel.size(); q++)
            if (descs[q].triangular) descs[q].blk_chunk_off = d_off + off_at[q];
        std::vector<unsigned char> hb(b_desc + b_db + b_ob + b_off);
        std::memcpy(hb.data(), descs.data(), b_desc);
        std::memcpy(hb.data() + b_desc, tbegin.data(), b_db);
        std::memcpy(hb.data() + b_desc + b_db, ln.obegin.data(), b_ob);
        if (b_off) std::memcpy(hb.data() + b_desc + b_db + b_ob, offs.data(), b_off);
        // (a pageable source is staged before the call returns, so hb may go out of scope)
        CK(cudaMemcpyAsync(ln.blob.p, hb.data(), hb.size(), cudaMemcpyHostToDevice, st));
        ln.d_obegin = d_ob;

        MultiLaunch& m = ln.m;
        m.descs = (const PairDesc*)ln.blob.p;
        m.num_descs = (int)sel.size();
        m.task_begin = d_db;
        m.total_tasks = total_tasks;
        m.task_chunks = (int)task_chunks;
        m.chunk = chunk;
        m.nobs_max = nobs_max;
        m.mixed = mixed;
        m.exact = exact;
        {
            std::lock_guard<std::mutex> lk(g_tiling_mu);
            m.poll_limit = g_poll_limit;
            m.dbg_extra_tx = g_extra_tx;
        }
        const int wpb = 4;  // warps per block of the pair kernel
        const int64_t warps = std::min<int64_t>(total_tasks, resident);
        m.blocks = (int)std::max<int64_t>(1, (warps + wpb - 1) / wpb);
        m.nwarps = m.blocks * wpb;
        m.minb = exact ? 2 : minb;
        m.tab_bytes_max = tab_max;
        m.bra_bytes_max = bra_max;
        m.warp_smem = warp_smem;
        if (sel.size() == 1) {
            m.dbg_k = dbg_k;
            m.dbg_r = dbg_r;
        }
        // records, then the task counter, then the reduction's partials
        const size_t red = (size_t)reduce_splits(ln.obegin.back()) * (size_t)ln.obegin.back() * 8;
        ln.rec.alloc((size_t)rec_doubles + 1 + red, st);
        ln.rec_used = (size_t)rec_doubles + 1;
        m.records = ln.rec.p;
        m.counter = (unsigned long long*)(ln.rec.p + rec_doubles);
        ln.red_scratch = ln.rec.p + rec_doubles + 1;
    }
}

// Enqueues the Pauli frames, the pair launches and the reductions of a built
// batch on `st` (no host synchronisation).  With `max_tasks` > 0 only the first
// tasks of each launch run (a timing sample; results are not meaningful).
void enqueue_batch(PairBatch& b, cudaStream_t st, float* pair_ms = nullptr, int64_t max_tasks = 0) {
    for (size_t k = 0; k < b.live.size(); k++)
        CK(launch_pauli_frames(b.live[k]->a->t.view(), b.dp.p + b.unit_obs[k], b.live[k]->nobs,
                               b.px.p + b.unit_px[k], b.pk.p + b.unit_px[k], st));
    if (b.exact) CK(cudaMemsetAsync(b.dcounts.p, 0, b.dcounts.n * sizeof(unsigned long long), st));
    for (PairBatch::Launch& ln : b.launches) {
        CK(cudaMemsetAsync(ln.rec.p, 0, ln.rec_used * sizeof(double), st));
        MultiLaunch m = ln.m;
        if (max_tasks > 0 && max_tasks < m.total_tasks) {
            m.total_tasks = max_tasks;
            const int64_t warps = std::min<int64_t>(max_tasks, (int64_t)m.nwarps);
            m.blocks = (int)std::max<int64_t>(1, (warps + 3) / 4);
            m.nwarps = m.blocks * 4;
        }
        cudaEvent_t ev0 = nullptr, ev1 = nullptr;
        if (pair_ms) {
            CK(cudaEventCreate(&ev0));
            CK(cudaEventCreate(&ev1));
            CK(cudaEventRecord(ev0, st));
        }
        CK(launch_pairs_multi(m, ln.wb, st));
        if (pair_ms) {
            CK(cudaEventRecord(ev1, st));
            CK(cudaEventSynchronize(ev1));
            float ms = 0.f;
            CK(cudaEventElapsedTime(&ms, ev0, ev1));
            cudaEventDestroy(ev0);
            cudaEventDestroy(ev1);
            *pair_ms += ms;
        }
        if (!b.exact)
            CK(launch_reduce_multi(m, ln.d_obegin, ln.obegin.back(), b.dout.p + 2 * ln.out_off, ln.red_scratch, st));
    }
}

// Copies the (re, im) results (2 per observable, launch order) into the units.
void scatter_batch(const PairBatch& b, const double* host) {
    for (size_t k = 0; k < b.live.size(); k++) {
        PairUnit* u = b.live[k];
        const double* r = host + 2 * b.unit_out[k];
        if (u->complex_out) {
            std::memcpy(u->out, r, 2 * (size_t)u->nobs * sizeof(double));
        } else {
            for (int o = 0; o < u->nobs; o++) u->out[o] = r[2 * o];
        }
    }
}

std::vector<PairUnit*> live_units(std::vector<PairUnit>& units) {
    std::vector<PairUnit*> live;
    for (auto& u : units) {
        const size_t nout = (u.complex_out ? 2 : 1) * (size_t)u.nobs;
        std::fill(u.out, u.out + nout, 0.0);
        if (u.nobs > 0 && u.a->t.chi > 0 && u.b->t.chi > 0) live.push_back(&u);
    }
    return live;
}

std::vector<nsg_state*> distinct_states(const std::vector<PairUnit*>& live) {
    std::vector<nsg_state*> s;
    for (PairUnit* u : live) {
        s.push_back(u->a);
        s.push_back(u->b);
    }
    std::sort(s.begin(), s.end());
    s.erase(std::unique(s.begin(), s.end()), s.end());
    return s;
}

// The batched Σ-pairs driver.  Every unit becomes one descriptor of a
// persistent pair launch (one launch per word width: states of ≤ 32 qubits
// run on 32-bit rows, wider ones on 64-bit rows), followed by one reduction
// launch; all of it on `st`.  Bra frames and term tables are built (once per
// state, cached) on each state's own stream and joined into `st`.
void run_pair_units(std::vector<PairUnit>& units, bool mixed, cudaStream_t st, uint8_t* dbg_k = nullptr,
                    int32_t* dbg_r = nullptr, bool exact = false) {
    PairBatch b;
    b.live = live_units(units);
    if (b.live.empty()) return;
    for (PairUnit* u : b.live) {
        UnitSources s;
        s.fr = u->a->frames();
        s.atab = u->a->ket_tables();
        s.ktab = u->b->ket_tables();
        b.src.push_back(s);
    }
    const std::vector<nsg_state*> touched = distinct_states(b.live);
    for (nsg_state* s : touched) join_stream(st, s->st);
    build_batch(b, pair_tiling_override(), mixed, st, false, dbg_k, dbg_r, exact);
    bool prof;
    {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        prof = g_prof_on;
    }
    float prof_ms = 0.f;
    enqueue_batch(b, st, prof ? &prof_ms : nullptr);
    std::vector<double> hout(2 * b.tot_obs);
    std::vector<int64_t> hcounts(exact ? b.tot_obs * 2 * kExactBins : 0);
    if (exact)
        CK(cudaMemcpyAsync(hcounts.data(), b.dcounts.p, hcounts.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    else
        CK(cudaMemcpyAsync(hout.data(), b.dout.p, hout.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (prof) {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        g_prof_ms += prof_ms;
        g_prof_launches += b.launches.size();
        g_prof_pairs += b.pairs;
    }
    if (exact) {
        for (size_t k = 0; k < b.live.size(); k++)
            if (b.live[k]->counts)
                std::memcpy(b.live[k]->counts, hcounts.data() + b.unit_obs[k] * 2 * kExactBins,
                            (size_t)b.live[k]->nobs * 2 * kExactBins * sizeof(int64_t));
    } else {
        scatter_batch(b, hout.data());
    }
    // The launches ran on `st`; each bra state's status words report its units.
    for (nsg_state* s : touched) s->check_status();
}

// Σ-pairs of one (a, b) for any number of observables (split into units of
// at most 256), in one launch on a's stream.
void run_pairs(nsg_state* a, nsg_state* b, const std::vector<DevPauli>& paulis, bool triangular, bool complex_out,
               bool mixed, std::vector<double>& out, uint8_t* dbg_k = nullptr, int32_t* dbg_r = nullptr) {
    const size_t nobs = paulis.size();
    out.assign(complex_out ? 2 * nobs : nobs, 0.0);
    std::vector<PairUnit> units;
    for (size_t base = 0; base < nobs; base += kMaxObsPerUnit) {
        PairUnit u;
        u.a = a;
        u.b = b;
        u.paulis = paulis.data() + base;
        u.nobs = (int)std::min<size_t>(kMaxObsPerUnit, nobs - base);
        u.triangular = triangular;
        u.complex_out = complex_out;
        u.out = out.data() + (complex_out ? 2 * base : base);
        units.push_back(u);
    }
    run_pair_units(units, mixed, a->st, units.size() == 1 ? dbg_k : nullptr, units.size() == 1 ? dbg_r : nullptr);
}

double norm_squared(nsg_state* s) {
    require_pairs_width(s);
    std::vector<DevPauli> id(1, DevPauli{0, 0, 0, 0});
    std::vector<double> out;
    run_pairs(s, s, id, true, false, false, out);
    return out[0];
}

void validate_qargs(const nsg_state* s, const uint32_t* q, size_t k) {  // stabilizer_decomposed_state/mod.rs:44-67
    if (k == 0) raise(NSG_ERR_EMPTY_QUBIT_INDICES, -1, -1, "Qubit index list is empty.");
    for (size_t i = 0; i < k; i++)
        if ((int)q[i] >= s->t.n) err_oob(q[i], s->t.n);
    std::vector<uint32_t> sorted(q, q + k);
    std::sort(sorted.begin(), sorted.end());
    for (size_t i = 1; i < k; i++)
        if (sorted[i] == sorted[i - 1])
            raise(NSG_ERR_DUPLICATE_QUBIT_INDEX, sorted[i], -1, "Duplicate qubit index found: %u.", sorted[i]);
}

void project_unnorm(nsg_state* s, uint32_t q, bool outcome) {  // projection.rs:27-57
    if ((int)q >= s->t.n) err_oob(q, s->t.n);
    DBuf<int32_t> keep;
    keep.alloc(std::max<int64_t>(s->t.chi, 1), s->st);
    CK(launch_project(s->t.view(), (int)q, outcome ? 1 : 0, keep.p, s->status.p, s->st));
    s->check_status();
    compact_into(s, keep);
}

void discard_q(nsg_state* s, uint32_t q) {  // discard.rs:5-12
    if ((int)q >= s->t.n) err_oob(q, s->t.n);
    CK(launch_discard(s->t.view(), (int)q, s->status.p, s->st));
    s->check_status(q);
    s->t.n -= 1;
    s->layout_gen++;
    s->invalidate();
    s->screen.reset();
}

// Clifford gates applied to a state move its common stabilizers with them.
void conj_screen(nsg_state* s, const std::vector<uint32_t>& ops) {
    if (!s->screen) return;
    auto ns = std::make_shared<ZeroScreen>(*s->screen);
    ns->apply(ops);
    s->screen = std::move(ns);
}

void apply_ops(nsg_state* s, const std::vector<uint32_t>& ops) {
    if (ops.empty() || s->t.chi == 0) return;
    // A few gates without H (one gate of a gate-by-gate caller, mostly): one
    // thread per term updates the rows they touch; nothing to allocate or
    // check, so the call does not wait for the device.
    bool row_only = ops.size() <= (size_t)kRowOpsMax;
    for (uint32_t c : ops) row_only = row_only && (c & 0xff) != P_H;
    if (row_only) {
        RowOps r{};
        r.n = (int)ops.size();
        for (size_t i = 0; i < ops.size(); i++) r.code[i] = ops[i];
        CK(launch_row_ops(r, s->t.view(), s->st));
        s->invalidate();
        conj_screen(s, ops);
        return;
    }
    DBuf<uint32_t> d;
    d.alloc(ops.size(), s->st);
    CK(cudaMemcpyAsync(d.p, ops.data(), ops.size() * 4, cudaMemcpyHostToDevice, s->st));
    CK(launch_apply_ops(d.p, (int)ops.size(), s->t.view(), s->status.p, s->st));
    s->check_status();
    s->invalidate();
    conj_screen(s, ops);
}

nsg_state* clone_state(const nsg_state* s) {
    auto* c = new nsg_state();
    c->init_stream();
    CK(cudaStreamSynchronize(s->st));
    c->t.copy_from(s->t, c->st);
    c->gf_re = s->gf_re;
    c->gf_im = s->gf_im;
    c->screen = s->screen;
    CK(cudaStreamSynchronize(c->st));
    return c;
}

// Probabilities of outcome 0/1 of qubit q (unnormalised): ⟨ψ|(I±Z_q)/2|ψ⟩,
// identical to norm_squared of the two projected states
// (measurement.rs:35-65, sampling.rs:103-153) from one pass over the pairs.
void outcome_weights(nsg_state* s, uint32_t q, double& w0, double& w1) {
    require_pairs_width(s);
    std::vector<DevPauli> ps(2, DevPauli{0, 0, 0, 0});
    ps[1].pz = 1ULL << q;
    std::vector<double> out;
    run_pairs(s, s, ps, true, false, false, out);
    w0 = 0.5 * (out[0] + out[1]);
    w1 = 0.5 * (out[0] - out[1]);
    if (w0 < 0.0) w0 = 0.0;
    if (w1 < 0.0) w1 = 0.0;
}

struct ShotOut {
    uint64_t lo, hi, count;
};

// recursive_sample (sampling.rs:80-189) with the binomial split of the
// reference and the same descending qubit order.
void sample_rec(nsg_state* s, const std::vector<std::pair<uint32_t, uint32_t>>& qs, size_t idx, uint64_t shots,
                uint64_t lo, uint64_t hi, HostRng& rng, std::vector<ShotOut>& out) {
    if (shots == 0) return;
    if (idx == qs.size()) {
        out.push_back({lo, hi, shots});
        return;
    }
    uint32_t q = qs[idx].first, bit = qs[idx].second;
    double w0, w1;
    outcome_weights(s, q, w0, w1);
    double tot = w0 + w1;
    double p0 = tot > 0 ? std::min(1.0, std::max(0.0, w0 / tot)) : 0.0;
    uint64_t n0 = rng.binomial(shots, p0), n1 = shots - n0;
    if (n0 > 0) {
        std::unique_ptr<nsg_state> z(n1 > 0 ? clone_state(s) : nullptr);
        nsg_state* zz = z ? z.get() : s;
        project_unnorm(zz, q, false);
        discard_q(zz, q);
        sample_rec(zz, qs, idx + 1, n0, lo, hi, rng, out);
    }
    if (n1 > 0) {
        nsg_state* oo = s;  // the 0-branch worked on a clone when both are taken
        project_unnorm(oo, q, true);
        std::vector<uint32_t> xo{enc_op(P_X, q)};
        apply_ops(oo, xo);  // |1⟩ -> |0⟩ before discarding (sampling.rs:175-176)
        discard_q(oo, q);
        uint64_t nlo = lo, nhi = hi;
        if (bit < 64) nlo |= 1ULL << bit;
        else nhi |= 1ULL << (bit - 64);
        sample_rec(oo, qs, idx + 1, n1, nlo, nhi, rng, out);
    }
}

// The marginal distribution of the qubits qs (processing order: bit i of x ↔
// qs[i]) from one batched pass over every Z-string on them:
// p(x) = 2^{-k}·Σ_S (-1)^{|x∧S|}·⟨Z_S⟩/⟨I⟩, a Walsh–Hadamard transform.
std::vector<double> walsh_marginal(nsg_state* s, const std::vector<std::pair<uint32_t, uint32_t>>& qs) {
    require_pairs_width(s);
    const size_t k = qs.size(), N = (size_t)1 << k;
    std::vector<DevPauli> ps(N, DevPauli{0, 0, 0, 0});
    for (size_t S = 0; S < N; S++)
        for (size_t i = 0; i < k; i++)
            if ((S >> i) & 1) ps[S].pz |= 1ULL << qs[i].first;
    std::vector<double> e;
    run_pairs(s, s, ps, true, false, false, e);
    const double norm2 = e[0];
    for (size_t len = 1; len < N; len <<= 1)
        for (size_t i = 0; i < N; i += 2 * len)
            for (size_t j = i; j < i + len; j++) {
                const double a = e[j], b = e[j + len];
                e[j] = a + b;
                e[j + len] = a - b;
            }
    for (size_t x = 0; x < N; x++) e[x] = (norm2 > 0.0) ? std::max(0.0, e[x] / ((double)N * norm2)) : 0.0;
    return e;
}

// recursive_sample's binomial splitting (sampling.rs:80-189), same node order
// and draws as sample_rec, with the branch weights read off the marginal.
void sample_marginal(const std::vector<double>& p, const std::vector<std::pair<uint32_t, uint32_t>>& qs, size_t idx,
                     uint32_t prefix, uint64_t shots, uint64_t lo, uint64_t hi, HostRng& rng, std::vector<ShotOut>& out) {
    if (shots == 0) return;
    if (idx == qs.size()) {
        out.push_back({lo, hi, shots});
        return;
    }
    const uint32_t low = (1u << idx) - 1;
    double w0 = 0.0, w1 = 0.0;
    for (size_t x = 0; x < p.size(); x++)
        if ((x & low) == prefix) ((x >> idx) & 1 ? w1 : w0) += p[x];
    const double tot = w0 + w1;
    const double p0 = tot > 0 ? std::min(1.0, std::max(0.0, w0 / tot)) : 0.0;
    const uint64_t n0 = rng.binomial(shots, p0), n1 = shots - n0;
    sample_marginal(p, qs, idx + 1, prefix, n0, lo, hi, rng, out);
    if (n1 > 0) {
        const uint32_t bit = qs[idx].second;
        uint64_t nlo = lo, nhi = hi;
        if (bit < 64) nlo |= 1ULL << bit;
        else nhi |= 1ULL << (bit - 64);
        sample_marginal(p, qs, idx + 1, prefix | (1u << idx), n1, nlo, nhi, rng, out);
    }
}

constexpr size_t kMarginalMaxQubits = 8;  // 2^8 Z-strings: one pair pass

// Device time per pair of one launch of a built batch, on its first tasks
// (`rounds` per resident warp, or all of them for rounds = 0; records and
// counter cleared first).  *ms_out receives the launch's time.
double sample_ns_per_pair(PairBatch& b, size_t li, cudaStream_t st, int rounds, float* ms_out = nullptr) {
    PairBatch::Launch& ln = b.launches[li];
    MultiLaunch m = ln.m;
    const int64_t k = rounds > 0 ? std::min<int64_t>(m.total_tasks, (int64_t)rounds * m.nwarps) : m.total_tasks;
    m.total_tasks = k;
    CK(cudaMemsetAsync(ln.rec.p, 0, ln.rec_used * sizeof(double), st));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, st));
    CK(launch_pairs_multi(m, ln.wb, st));
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms_out) *ms_out = ms;
    const int64_t pairs = k == ln.m.total_tasks ? ln.pairs_total
                                                 : (ln.task_pairs.size() > (size_t)k ? ln.task_pairs[(size_t)k] : 0);
    return pairs > 0 ? 1e6 * ms / (double)pairs : 1e300;
}

}  // namespace

// ---------------------------------------------------------------------------
// A plan's copy of one state's derived data and the identity it was built on.
struct PlanState {
    nsg_state* s = nullptr;
    uint64_t uid = 0, gen = 0;
    int n = 0;
    int64_t chi = 0;
    double gf_re = 1.0, gf_im = 0.0;
    DBuf<uint64_t> gv, fv, mv, gvl, gvh;
    DBuf<unsigned char> tab;
    FrameView frames() const { return FrameView{gv.p, fv.p, mv.p, gvl.p, gvh.p}; }
};

struct nsg_plan {
    int device = 0;
    cudaStream_t st = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<std::unique_ptr<PlanState>> states;
    std::vector<DevPauli> paulis;
    std::vector<PairUnit> units;
    std::vector<double> results;  // one per observable, in the caller's order
    PairBatch batch;
    double* pinned = nullptr;
    PairTiling tiling;
    bool timed = false;

    ~nsg_plan() {
        if (st) cudaStreamSynchronize(st);
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (pinned) cudaFreeHost(pinned);
        batch = PairBatch();  // device buffers are freed on the plan's stream
        states.clear();
        if (st) {
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    }
    // Frames and term tables of every state, from their current terms.
    void enqueue_derived() {
        for (auto& ps : states) {
            if (ps->chi == 0) continue;
            CK(launch_frames(ps->s->t.view(), ps->frames(), st));
            CK(launch_ket_tables(ps->s->t.view(), ps->tab.p, st));
        }
    }
    PlanState* find(const nsg_state* s) {
        for (auto& ps : states)
            if (ps->s == s) return ps.get();
        return nullptr;
    }
    void build(PairBatch& b, const PairTiling& tl, bool mixed, bool with_samples = false) {
        b.live = live_units(units);
        b.src.clear();
        for (PairUnit* u : b.live) {
            UnitSources src;
            src.fr = find(u->a)->frames();
            src.atab = find(u->a)->tab.p;
            src.ktab = find(u->b)->tab.p;
            b.src.push_back(src);
        }
        build_batch(b, tl, mixed, st, with_samples);
    }
};


// ===========================================================================
extern "C" {

const char* nsg_version(void) { return "necstar-gb300 0.1"; }

const char* nsg_last_error_message(void) { return g_msg.c_str(); }

nsg_status nsg_last_error_args(int64_t out[3]) {
    if (!out) return NSG_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < 3; i++) out[i] = g_args[i];
    return NSG_OK;
}

namespace {
// StabDecompCompiler::compile (compiler/mod.rs:44-140) on the device, in two
// phases so that many circuits can be enqueued before any host wait:
// compile_enqueue lowers the circuit (with the reference's checks, in its
// order), creates the state and queues the compile kernel and the stable
// compaction of the kept terms; compile_finish waits for that work and
// installs the compacted terms.  A batch lowers every circuit first, stages
// all op lists in one pinned buffer (so no copy waits for queued work) and
// queues the compiles on four work streams; the buffers move to each state's
// own stream when it is finished.
struct PendingCompile {
    std::unique_ptr<nsg_state> s;
    cudaStream_t ws = nullptr;   // the stream the work is queued on (the state's own when null)
    TermStore out;               // the compaction's target
    DBuf<int32_t> keep, pos;
    DBuf<int64_t> cnt;
    DBuf<uint32_t> dops;
    int64_t chi_t = 0;
    int64_t* h_count = nullptr;  // pinned slot the kept count is copied to
};

// A circuit lowered to the primitive op list of the compile kernel.
struct Lowered {
    int n = 0, t = 0;
    std::vector<uint32_t> ops;
};

Lowered lower_circuit(uint32_t num_qubits, const nsg_gate* gates, size_t num_gates) {
    if (num_gates) need(gates, "gates");
    const int n = (int)num_qubits;
    // Lowering (compiler/mod.rs:49-63): T/Tdg -> CX(target, n+k) [+ Sdg(target)].
    int t = 0;
    for (size_t i = 0; i < num_gates; i++) {
        uint32_t op = gates[i].op;
        if (op == NSG_GATE_T || op == NSG_GATE_TDG) t++;
        else if (op > NSG_GATE_SWAP)
            raise(NSG_ERR_GATE_NOT_SUPPORTED, op, -1, "Gate %s is not supported.", gate_name(op));
    }
    if (n == 0) raise(NSG_ERR_INVALID_NUM_QUBITS, 0, -1, "Number of qubits must be greater than zero, got 0.");
    const int width = n + t;
    if (width > 128 || t > 64)
        raise(NSG_ERR_TOO_WIDE, width, 128, "compilation width %d (n=%d, t=%d) exceeds the supported 128 (t <= 64)",
              width, n, t);
    std::vector<uint32_t> ops;
    ops.reserve(num_gates + t);
    int k = 0;
    for (size_t i = 0; i < num_gates; i++) {
        const nsg_gate& g = gates[i];
        if (g.op == NSG_GATE_T || g.op == NSG_GATE_TDG) {
            nsg_gate cx{NSG_GATE_CX, g.q0, (uint32_t)(n + k), 0};
            lower_clifford(cx, width, ops);
            if (g.op == NSG_GATE_TDG) {
                nsg_gate sdg{NSG_GATE_SDG, g.q0, 0, 0};
                lower_clifford(sdg, width, ops);
            }
            k++;
        } else {
            lower_clifford(g, width, ops);
        }
    }
    Lowered lw;
    lw.n = n;
    lw.t = t;
    lw.ops = std::move(ops);
    return lw;
}

// src_ops: the op list to copy to the device (lw.ops, or a pinned copy of it:
// a copy from pageable memory first waits for the work queued on the stream).
void compile_enqueue(const Lowered& lw, const uint32_t* src_ops, PendingCompile& pc, cudaStream_t work = nullptr) {
    const int n = lw.n, t = lw.t;
    const std::vector<uint32_t>& ops = lw.ops;
    pc.s = std::make_unique<nsg_state>();
    nsg_state* s = pc.s.get();
    s->init_stream();
    cudaStream_t st = s->st;
    if (work) {
        join_stream(work, s->st);  // the status words are cleared on the state's stream
        st = work;
    }
    pc.ws = st;
    auto tt = t_tensor_dev(t, st, s->status.p);
    pc.chi_t = tt->chi;
    pc.dops.alloc(std::max<size_t>(ops.size(), 1), st);
    if (!ops.empty()) CK(cudaMemcpyAsync(pc.dops.p, src_ops, ops.size() * 4, cudaMemcpyHostToDevice, st));
    TermStore raw;
    raw.alloc(n, tt->chi, st);
    raw.chi = tt->chi;
    pc.keep.alloc(tt->chi, st);
    TermsView rv = raw.view();
    CK(launch_compile(pc.dops.p, (int)ops.size(), n, t, tt->chi, tt->G, tt->F, tt->M, tt->gam, tt->V, tt->S,
                      tt->phase, tt->ck, tt->cr, rv, pc.keep.p, s->status.p, st));
    s->t = std::move(raw);
    pc.out.alloc(s->t.n, std::max<int64_t>(s->t.chi, 1), st);
    pc.out.W = s->t.W;
    pc.out.R = s->t.R;
    pc.pos.alloc(std::max<int64_t>(s->t.chi, 1), st);
    pc.cnt.alloc(1, st);
    CK(launch_compact(s->t.view(), pc.keep.p, pc.pos.p, pc.out.view(), pc.cnt.p, st));
    CK(cudaMemcpyAsync(pc.h_count, pc.cnt.p, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
}

void compile_finish(PendingCompile& pc, std::vector<uint8_t>* keep_out) {
    nsg_state* s = pc.s.get();
    CK(cudaStreamSynchronize(pc.ws));
    s->check_status();
    if (keep_out) {
        std::vector<int32_t> hk((size_t)pc.chi_t);
        CK(cudaMemcpyAsync(hk.data(), pc.keep.p, hk.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, pc.ws));
        CK(cudaStreamSynchronize(pc.ws));
        keep_out->assign(hk.size(), 0);
        for (size_t i = 0; i < hk.size(); i++) (*keep_out)[i] = hk[i] ? 1 : 0;
    }
    pc.out.chi = *pc.h_count;
    s->t = std::move(pc.out);  // the uncompacted terms are freed on the work stream
    s->t.rehome(s->st);        // from now on the state's own stream uses (and frees) its terms
    s->layout_gen++;
    s->invalidate();
    pc.keep.release();
    pc.pos.release();
    pc.cnt.release();
    pc.dops.release();
}

// Pinned host slots for the kept counts of a compile batch.
struct PinnedCounts {
    int64_t* p = nullptr;
    explicit PinnedCounts(size_t n) { CK(cudaMallocHost((void**)&p, std::max<size_t>(n, 1) * sizeof(int64_t))); }
    ~PinnedCounts() {
        if (p) cudaFreeHost(p);
    }
};

std::unique_ptr<nsg_state> compile_state(uint32_t num_qubits, const nsg_gate* gates, size_t num_gates,
                                         std::vector<uint8_t>* keep_out) {
    int64_t count = 0;
    PendingCompile pc;
    pc.h_count = &count;  // pageable: the copy completes before the stream wait returns
    const Lowered lw = lower_circuit(num_qubits, gates, num_gates);
    compile_enqueue(lw, lw.ops.data(), pc);
    compile_finish(pc, keep_out);
    pc.s->screen = screen_of(lw.n, lw.t, lw.ops);
    return std::move(pc.s);
}
}  // namespace

nsg_status nsg_state_from_circuit(uint32_t num_qubits, const nsg_gate* gates, size_t num_gates, nsg_state** out) {
    API_BEGIN
    need(out, "out");
    *out = nullptr;
    *out = compile_state(num_qubits, gates, num_gates, nullptr).release();
    API_END
}

nsg_status nsg_states_from_circuits(size_t num_circuits, const uint32_t* num_qubits, const nsg_gate* const* gates,
                                    const size_t* num_gates, nsg_state** out) {
    API_BEGIN
    if (num_circuits) {
        need(num_qubits, "num_qubits");
        need(gates, "gates");
        need(num_gates, "num_gates");
        need(out, "out");
    }
    for (size_t c = 0; c < num_circuits; c++) out[c] = nullptr;
    // Lower every circuit first (the reference's checks; the failing circuit's
    // index in args[2]), then stage all op lists in one pinned buffer.
    std::vector<Lowered> lw(num_circuits);
    std::vector<size_t> op_off(num_circuits + 1, 0);
    for (size_t c = 0; c < num_circuits; c++) {
        try {
            lw[c] = lower_circuit(num_qubits[c], gates[c], num_gates[c]);
        } catch (const ApiError&) {
            g_args[2] = (int64_t)c;
            throw;
        }
        op_off[c + 1] = op_off[c] + lw[c].ops.size();
    }
    struct Pinned {
        uint32_t* p = nullptr;
        ~Pinned() {
            if (p) cudaFreeHost(p);
        }
    } staged;
    CK(cudaMallocHost((void**)&staged.p, std::max<size_t>(op_off.back(), 1) * sizeof(uint32_t)));
    for (size_t c = 0; c < num_circuits; c++)
        if (!lw[c].ops.empty()) std::memcpy(staged.p + op_off[c], lw[c].ops.data(), lw[c].ops.size() * sizeof(uint32_t));
    PinnedCounts counts(num_circuits);
    // A few work streams (small compile launches overlap); circuit c on stream c mod 4.
    struct WorkStreams {
        cudaStream_t st[4] = {nullptr, nullptr, nullptr, nullptr};
        ~WorkStreams() {
            for (cudaStream_t s : st)
                if (s) cudaStreamDestroy(s);  // destroyed once its queued work (frees included) is done
        }
    } work;
    for (cudaStream_t& ws : work.st) CK(cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking));
    auto sync_all = [&]() {
        for (cudaStream_t ws : work.st) CK(cudaStreamSynchronize(ws));
    };
    std::vector<PendingCompile> pend(num_circuits);
    for (size_t c = 0; c < num_circuits; c++) {
        pend[c].h_count = counts.p + c;
        try {
            compile_enqueue(lw[c], staged.p + op_off[c], pend[c], work.st[c % 4]);
        } catch (const ApiError& e) {
            g_args[2] = (int64_t)c;  // the failing circuit
            sync_all();
            throw;
        }
    }
    for (size_t c = 0; c < num_circuits; c++) {
        try {
            compile_finish(pend[c], nullptr);
            pend[c].s->screen = screen_of(lw[c].n, lw[c].t, lw[c].ops);
        } catch (const ApiError& e) {
            g_args[2] = (int64_t)c;
            sync_all();
            throw;
        }
    }
    for (size_t c = 0; c < num_circuits; c++) out[c] = pend[c].s.release();
    API_END
}

nsg_status nsg_debug_compile_keep(uint32_t num_qubits, const nsg_gate* gates, size_t num_gates, uint8_t* keep,
                                  size_t capacity, uint64_t* num_t_terms) {
    API_BEGIN
    need(num_t_terms, "num_t_terms");
    std::vector<uint8_t> k;
    std::unique_ptr<nsg_state> s = compile_state(num_qubits, gates, num_gates, &k);
    *num_t_terms = k.size();
    if (k.size() > capacity) raise(NSG_ERR_BUFFER_TOO_SMALL, (int64_t)k.size(), (int64_t)capacity, "keep buffer too small");
    if (!k.empty()) {
        need(keep, "keep");
        std::memcpy(keep, k.data(), k.size());
    }
    API_END
}

nsg_status nsg_state_select(const nsg_state* cstate, const uint64_t* indices, size_t count, nsg_state** out) {
    API_BEGIN
    need(cstate, "state");
    need(out, "out");
    *out = nullptr;
    if (count) need(indices, "indices");
    DeviceScope ds_(cstate->device);
    for (size_t i = 0; i < count; i++) {
        if ((int64_t)indices[i] >= cstate->t.chi)
            raise(NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS, (int64_t)indices[i], cstate->t.chi, "term index %llu out of range",
                  (unsigned long long)indices[i]);
        if (i && indices[i] <= indices[i - 1])
            raise(NSG_ERR_INVALID_ARGUMENT, (int64_t)i, -1, "term indices must be strictly ascending");
    }
    nsg_state* src = const_cast<nsg_state*>(cstate);
    auto s = std::unique_ptr<nsg_state>(clone_state(src));
    std::vector<int32_t> hk((size_t)std::max<int64_t>(s->t.chi, 1), 0);
    for (size_t i = 0; i < count; i++) hk[indices[i]] = 1;
    DBuf<int32_t> keep;
    keep.alloc(hk.size(), s->st);
    CK(cudaMemcpyAsync(keep.p, hk.data(), hk.size() * sizeof(int32_t), cudaMemcpyHostToDevice, s->st));
    compact_into(s.get(), keep);
    s->screen = cstate->screen;  // every kept term keeps the common stabilizers
    *out = s.release();
    API_END
}

nsg_status nsg_state_from_terms(uint32_t num_qubits, uint64_t num_terms, const uint8_t* G, const uint8_t* F,
                                const uint8_t* M, const uint8_t* gamma, const uint8_t* v, const uint8_t* s_,
                                const uint8_t* phase, const uint8_t* coef_phase, const int32_t* coef_r,
                                const uint8_t* coef_zero, const double global_factor[2], nsg_state** out) {
    API_BEGIN
    need(out, "out");
    *out = nullptr;
    const int n = (int)num_qubits;
    if (n > 128) raise(NSG_ERR_TOO_WIDE, n, 128, "width %d exceeds 128", n);
    if (num_terms) {
        need(G, "G"); need(F, "F"); need(M, "M"); need(gamma, "gamma"); need(v, "v"); need(s_, "s");
        need(phase, "phase"); need(coef_phase, "coef_phase"); need(coef_r, "coef_r");
    }
    if (coef_zero)
        for (uint64_t i = 0; i < num_terms; i++)
            if (coef_zero[i]) raise(NSG_ERR_NOT_IMPLEMENTED, (int64_t)i, -1, "Not implemented: zero coefficients");
    auto st_ = std::make_unique<nsg_state>();
    st_->init_stream();
    cudaStream_t st = st_->st;
    st_->t.alloc(n, (int64_t)num_terms, st);
    st_->t.chi = (int64_t)num_terms;
    const size_t nn = (size_t)n * n * num_terms, nv = (size_t)n * num_terms;
    DBuf<uint8_t> dG, dF, dM, dg, dv, ds;
    if (num_terms && n) {
        dG.alloc(nn, st); dF.alloc(nn, st); dM.alloc(nn, st);
        dg.alloc(nv, st); dv.alloc(nv, st); ds.alloc(nv, st);
        CK(cudaMemcpyAsync(dG.p, G, nn, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dF.p, F, nn, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dM.p, M, nn, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dg.p, gamma, nv, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dv.p, v, nv, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(ds.p, s_, nv, cudaMemcpyHostToDevice, st));
        CK(launch_pack(st_->t.view(), dG.p, dF.p, dM.p, dg.p, dv.p, ds.p, st));
    }
    if (num_terms) {
        CK(cudaMemcpyAsync(st_->t.phase.p, phase, num_terms, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(st_->t.ck.p, coef_phase, num_terms, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(st_->t.cr.p, coef_r, num_terms * 4, cudaMemcpyHostToDevice, st));
    }
    if (global_factor) {
        st_->gf_re = global_factor[0];
        st_->gf_im = global_factor[1];
    }
    CK(cudaStreamSynchronize(st));
    *out = st_.release();
    API_END
}

void nsg_state_free(nsg_state* state) {
    if (!state) return;
    DeviceScope ds_(state->device);
    delete state;
}

nsg_status nsg_state_clone(const nsg_state* state, nsg_state** out) {
    API_BEGIN
    need(state, "state");
    need(out, "out");
    DeviceScope ds_(state->device);
    *out = clone_state(state);
    API_END
}

nsg_status nsg_num_qubits(const nsg_state* state, uint32_t* out) {
    API_BEGIN
    need(state, "state");
    need(out, "out");
    *out = (uint32_t)state->t.n;
    API_END
}

nsg_status nsg_stabilizer_rank(const nsg_state* state, uint64_t* out) {
    API_BEGIN
    need(state, "state");
    need(out, "out");
    *out = (uint64_t)state->t.chi;
    API_END
}

nsg_status nsg_state_set_stream(nsg_state* state, void* cuda_stream) {
    API_BEGIN
    need(state, "state");
    CK(cudaStreamSynchronize(state->st));
    state->st = cuda_stream ? (cudaStream_t)cuda_stream : state->own;
    // Buffers are freed on the stream that last uses them.
    state->t.rehome(state->st);
    state->fGV.rehome(state->st);
    state->fFV.rehome(state->st);
    state->fMV.rehome(state->st);
    state->fGVL.rehome(state->st);
    state->fGVH.rehome(state->st);
    state->status.rehome(state->st);
    state->ktab.rehome(state->st);
    API_END
}

nsg_status nsg_apply_gates(nsg_state* state, const nsg_gate* gates, size_t num_gates) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    if (num_gates) need(gates, "gates");
    // apply_gates (stabilizer_decomposed_state/gates.rs:7-37): gates apply in
    // order; the first failing gate stops after its predecessors took effect.
    // Index checks happen inside the per-term loop, so with no terms only
    // non-Clifford gates fail.
    std::vector<uint32_t> ops;
    ApiError pending{NSG_OK};
    std::string pmsg;
    int64_t pargs[3] = {-1, -1, -1};
    for (size_t i = 0; i < num_gates; i++) {
        const nsg_gate& g = gates[i];
        if (g.op > NSG_GATE_SWAP) {
            if (g.op > NSG_GATE_CCX) {
                pending = ApiError{NSG_ERR_INVALID_ARGUMENT};
                pmsg = "invalid gate opcode";
            } else {
                pending = ApiError{NSG_ERR_NON_CLIFFORD_GATE_APPLICATION};
                pmsg = std::string("Direct application of non-Clifford gate ") + gate_name(g.op) + " is not supported.";
                pargs[0] = g.op;
            }
            break;
        }
        if (state->t.chi == 0) continue;
        try {
            lower_clifford(g, state->t.n, ops);
        } catch (const ApiError& e) {
            pending = e;
            pmsg = g_msg;
            for (int j = 0; j < 3; j++) pargs[j] = g_args[j];
            break;
        }
    }
    apply_ops(state, ops);
    if (pending.code != NSG_OK) {
        g_msg = pmsg;
        for (int j = 0; j < 3; j++) g_args[j] = pargs[j];
        return pending.code;
    }
    API_END
}

nsg_status nsg_exp_value(const nsg_state* state, const nsg_pauli* pauli, double* out) {
    return nsg_exp_value_batch(state, pauli, 1, NSG_PRECISION_FP64, out);
}

nsg_status nsg_zero_screen(const nsg_state* cstate, const nsg_pauli* paulis, size_t num_paulis, uint8_t* zero) {
    API_BEGIN
    need(cstate, "state");
    if (num_paulis) {
        need(paulis, "paulis");
        need(zero, "zero");
    }
    nsg_state* state = const_cast<nsg_state*>(cstate);
    require_pairs_width(state);
    const std::shared_ptr<const ZeroScreen> sc = state->screen;
    for (size_t i = 0; i < num_paulis; i++) {
        const DevPauli d = to_dev_pauli(paulis[i], state->t.n);
        zero[i] = (sc && sc->zero(d.px, d.pz)) ? 1 : 0;
    }
    API_END
}

nsg_status nsg_zero_screen_circuit(uint32_t num_qubits, const nsg_gate* gates, size_t num_gates,
                                   const nsg_pauli* paulis, size_t num_paulis, uint8_t* zero) {
    API_BEGIN
    if (num_paulis) {
        need(paulis, "paulis");
        need(zero, "zero");
    }
    const Lowered lw = lower_circuit(num_qubits, gates, num_gates);
    if (lw.n > 64) raise(NSG_ERR_TOO_WIDE, lw.n, 64, "state width %d exceeds the supported 64 qubits", lw.n);
    const std::shared_ptr<const ZeroScreen> sc = screen_of(lw.n, lw.t, lw.ops);
    for (size_t i = 0; i < num_paulis; i++) {
        const DevPauli d = to_dev_pauli(paulis[i], lw.n);
        zero[i] = sc->zero(d.px, d.pz) ? 1 : 0;
    }
    API_END
}

nsg_status nsg_exp_value_batch(const nsg_state* cstate, const nsg_pauli* paulis, size_t num_paulis,
                               uint32_t precision, double* out) {
    API_BEGIN
    need(cstate, "state");
    DeviceScope ds_(cstate->device);
    if (num_paulis) {
        need(paulis, "paulis");
        need(out, "out");
    }
    if (precision > NSG_PRECISION_MIXED) raise(NSG_ERR_INVALID_ARGUMENT, precision, -1, "invalid precision");
    nsg_state* state = const_cast<nsg_state*>(cstate);
    require_pairs_width(state);
    std::vector<DevPauli> dp(num_paulis);
    for (size_t i = 0; i < num_paulis; i++) dp[i] = to_dev_pauli(paulis[i], state->t.n);
    std::vector<double> r;
    run_pairs(state, state, dp, true, false, precision == NSG_PRECISION_MIXED, r);
    if (num_paulis) std::memcpy(out, r.data(), num_paulis * sizeof(double));
    API_END
}

nsg_status nsg_exp_value_multi(const nsg_state* const* states, size_t num_states, const nsg_pauli* paulis,
                               const uint64_t* pauli_offsets, uint32_t precision, double* out) {
    API_BEGIN
    need(pauli_offsets, "pauli_offsets");
    if (num_states) need(states, "states");
    if (precision > NSG_PRECISION_MIXED) raise(NSG_ERR_INVALID_ARGUMENT, precision, -1, "invalid precision");
    if (pauli_offsets[0] != 0) raise(NSG_ERR_INVALID_ARGUMENT, (int64_t)pauli_offsets[0], -1, "pauli_offsets[0] must be 0");
    for (size_t c = 0; c < num_states; c++) {
        need(states[c], "state");
        if (pauli_offsets[c + 1] < pauli_offsets[c])
            raise(NSG_ERR_INVALID_ARGUMENT, (int64_t)c, -1, "pauli_offsets not ascending at %zu", c);
        require_pairs_width(states[c]);
        if (states[c]->device != states[0]->device)
            raise(NSG_ERR_INVALID_ARGUMENT, states[c]->device, states[0]->device, "all states must live on one device");
    }
    const uint64_t total = num_states ? pauli_offsets[num_states] : 0;
    if (total) {
        need(paulis, "paulis");
        need(out, "out");
    }
    // Observables in device form, with the per-state length checks of exp_value.rs:9-27.
    std::vector<DevPauli> dp(total);
    for (size_t c = 0; c < num_states; c++)
        for (uint64_t k = pauli_offsets[c]; k < pauli_offsets[c + 1]; k++)
            dp[k] = to_dev_pauli(paulis[k], states[c]->t.n);
    std::vector<PairUnit> units;
    for (size_t c = 0; c < num_states; c++) {
        nsg_state* s = const_cast<nsg_state*>(states[c]);
        for (uint64_t base = pauli_offsets[c]; base < pauli_offsets[c + 1]; base += kMaxObsPerUnit) {
            PairUnit u;
            u.a = s;
            u.b = s;
            u.paulis = dp.data() + base;
            u.nobs = (int)std::min<uint64_t>(kMaxObsPerUnit, pauli_offsets[c + 1] - base);
            u.triangular = true;
            u.complex_out = false;
            u.out = out + base;
            units.push_back(u);
        }
    }
    if (!units.empty()) {
        DeviceScope ds_(states[0]->device);
        run_pair_units(units, precision == NSG_PRECISION_MIXED, const_cast<nsg_state*>(states[0])->st);
    }
    API_END
}

nsg_status nsg_exp_value_counts(const nsg_state* cstate, const nsg_pauli* paulis, size_t num_paulis, int64_t* counts,
                                double* scale) {
    API_BEGIN
    need(cstate, "state");
    DeviceScope ds_(cstate->device);
    if (num_paulis) {
        need(paulis, "paulis");
        need(counts, "counts");
    }
    nsg_state* state = const_cast<nsg_state*>(cstate);
    require_pairs_width(state);
    std::vector<DevPauli> dp(num_paulis);
    for (size_t i = 0; i < num_paulis; i++) dp[i] = to_dev_pauli(paulis[i], state->t.n);
    if (num_paulis) std::memset(counts, 0, num_paulis * kExactBins * sizeof(int64_t));
    std::vector<int64_t> both(2 * kExactBins * std::min<size_t>(num_paulis, kMaxObsPerUnit));
    std::vector<double> unused(std::max<size_t>(num_paulis, 1));
    for (size_t base = 0; base < num_paulis; base += kMaxObsPerUnit) {
        std::vector<PairUnit> units(1);
        PairUnit& u = units[0];
        u.a = state;
        u.b = state;
        u.paulis = dp.data() + base;
        u.nobs = (int)std::min<size_t>(kMaxObsPerUnit, num_paulis - base);
        u.triangular = true;
        u.out = unused.data() + base;
        std::fill(both.begin(), both.end(), 0);
        u.counts = both.data();
        run_pair_units(units, false, state->st, nullptr, nullptr, true);
        for (int o = 0; o < u.nobs; o++)  // the real-part bins of each observable
            std::memcpy(counts + (base + o) * kExactBins, both.data() + (size_t)o * 2 * kExactBins,
                        kExactBins * sizeof(int64_t));
    }
    if (scale) *scale = state->gf_re * state->gf_re + state->gf_im * state->gf_im;
    API_END
}

nsg_status nsg_set_pair_tiling(int32_t chunk, int32_t tasks_per_warp) {
    API_BEGIN
    if (chunk < 0 || chunk > 1024 || tasks_per_warp < 0 || tasks_per_warp > 1024)
        raise(NSG_ERR_INVALID_ARGUMENT, chunk, tasks_per_warp, "tiling out of range");
    std::lock_guard<std::mutex> lk(g_tiling_mu);
    for (int w = 0; w < 2; w++) {
        g_tiling_override.chunk[w] = chunk;  // 0: the tuning cache's choice, else the default
        g_tiling_override.tasks_per_warp[w] = tasks_per_warp;
    }
    API_END
}

nsg_status nsg_debug_set_wait(uint32_t poll_limit, uint32_t extra_tx_bytes) {
    API_BEGIN
    if (extra_tx_bytes > 1024) raise(NSG_ERR_INVALID_ARGUMENT, extra_tx_bytes, 1024, "extra bytes out of range");
    std::lock_guard<std::mutex> lk(g_tiling_mu);
    g_poll_limit = poll_limit;
    g_extra_tx = extra_tx_bytes;
    API_END
}

nsg_status nsg_plan_create(const nsg_state* const* states, size_t num_states, const nsg_pauli* paulis,
                           const uint64_t* pauli_offsets, uint32_t precision, nsg_plan** out) {
    API_BEGIN
    need(out, "out");
    *out = nullptr;
    need(pauli_offsets, "pauli_offsets");
    if (num_states) need(states, "states");
    if (precision > NSG_PRECISION_MIXED) raise(NSG_ERR_INVALID_ARGUMENT, precision, -1, "invalid precision");
    if (pauli_offsets[0] != 0) raise(NSG_ERR_INVALID_ARGUMENT, (int64_t)pauli_offsets[0], -1, "pauli_offsets[0] must be 0");
    for (size_t c = 0; c < num_states; c++) {
        need(states[c], "state");
        if (pauli_offsets[c + 1] < pauli_offsets[c])
            raise(NSG_ERR_INVALID_ARGUMENT, (int64_t)c, -1, "pauli_offsets not ascending at %zu", c);
        require_pairs_width(states[c]);
        if (states[c]->device != states[0]->device)
            raise(NSG_ERR_INVALID_ARGUMENT, states[c]->device, states[0]->device, "all states must live on one device");
    }
    const uint64_t total = num_states ? pauli_offsets[num_states] : 0;
    if (total) need(paulis, "paulis");
    const bool mixed = precision == NSG_PRECISION_MIXED;
    auto plan = std::make_unique<nsg_plan>();
    plan->device = num_states ? states[0]->device : 0;
    DeviceScope ds_(plan->device);
    CK(cudaStreamCreateWithFlags(&plan->st, cudaStreamNonBlocking));
    cudaStream_t st = plan->st;
    plan->paulis.resize(total);
    for (size_t c = 0; c < num_states; c++)
        for (uint64_t k = pauli_offsets[c]; k < pauli_offsets[c + 1]; k++)
            plan->paulis[k] = to_dev_pauli(paulis[k], states[c]->t.n);
    plan->results.assign(total, 0.0);
    // Each distinct state: its identity and the plan's own frames and term tables.
    for (size_t c = 0; c < num_states; c++) {
        nsg_state* s = const_cast<nsg_state*>(states[c]);
        if (plan->find(s)) continue;
        auto ps = std::make_unique<PlanState>();
        ps->s = s;
        ps->uid = s->uid;
        ps->gen = s->layout_gen;
        ps->n = s->t.n;
        ps->chi = s->t.chi;
        ps->gf_re = s->gf_re;
        ps->gf_im = s->gf_im;
        const size_t cap = (size_t)std::max<int64_t>(s->t.chi, 1);
        ps->gv.alloc(cap * 64, st);
        ps->fv.alloc(cap * 64, st);
        ps->mv.alloc(cap * 64, st);
        ps->gvl.alloc(cap, st);
        ps->gvh.alloc(cap, st);
        ps->tab.alloc(cap * ket_table_stride(s->t.n), st);
        join_stream(st, s->st);
        plan->states.push_back(std::move(ps));
    }
    for (size_t c = 0; c < num_states; c++) {
        nsg_state* s = const_cast<nsg_state*>(states[c]);
        for (uint64_t base = pauli_offsets[c]; base < pauli_offsets[c + 1]; base += kMaxObsPerUnit) {
            PairUnit u;
            u.a = s;
            u.b = s;
            u.paulis = plan->paulis.data() + base;
            u.nobs = (int)std::min<uint64_t>(kMaxObsPerUnit, pauli_offsets[c + 1] - base);
            u.out = plan->results.data() + base;
            plan->units.push_back(u);
        }
    }
    plan->enqueue_derived();

    // Tiling per row width — kernel variant, tasks per resident warp, kets per
    // chunk — from the cache, or timed on the plan's own work: the variants
    // first (default tasks and chunk), then tasks per warp with the fastest
    // variant, then the chunk length with both.
    PairTiling tl;
    {
        PairBatch probe;
        PairTiling none;
        for (int w = 0; w < 2; w++) {
            none.chunk[w] = TuneChoice().chunk;
            none.tasks_per_warp[w] = TuneChoice().tasks_per_warp;
            none.minb[w] = 4;
        }
        plan->build(probe, none, mixed, true);
        std::vector<std::string> keys(2);
        bool need_time[2] = {false, false};
        for (const PairBatch::Launch& ln : probe.launches) {
            const int idx = ln.wb == 4 ? 0 : 1;
            uint64_t pairs = 0, nsum = 0;
            for (size_t q : ln.units) {
                const int64_t chi = probe.live[q]->a->t.chi;
                pairs += (uint64_t)(chi * (chi + 1) / 2);
                nsum += (uint64_t)probe.live[q]->a->t.n * (uint64_t)(chi * (chi + 1) / 2);
            }
            keys[idx] = tune_key(plan->device, ln.wb, ln.m.nobs_max, pairs ? (int)(nsum / pairs) : 0, pairs);
            TuneChoice c;
            if (tune_lookup(keys[idx], c)) {
                tl.minb[idx] = c.minb;
                tl.tasks_per_warp[idx] = c.tasks_per_warp;
                tl.chunk[idx] = c.chunk;
            } else {
                need_time[idx] = true;
            }
        }
        if (need_time[0] || need_time[1]) {
            plan->timed = true;
            // Whole launches when the default variant's estimate is short, else
            // two rounds of tasks per resident warp.
            int rounds[2] = {2, 2};
            for (size_t k = 0; k < probe.live.size(); k++)
                CK(launch_pauli_frames(probe.live[k]->a->t.view(), probe.dp.p + probe.unit_obs[k], probe.live[k]->nobs,
                                       probe.px.p + probe.unit_px[k], probe.pk.p + probe.unit_px[k], st));
            for (size_t li = 0; li < probe.launches.size(); li++) {
                const int idx = probe.launches[li].wb == 4 ? 0 : 1;
                if (!need_time[idx]) continue;
                float ms = 0.f;
                sample_ns_per_pair(probe, li, st, 1);
                sample_ns_per_pair(probe, li, st, 2, &ms);
                const MultiLaunch& m = probe.launches[li].m;
                const double frac = (double)std::min<int64_t>(m.total_tasks, 2 * (int64_t)m.nwarps) / (double)m.total_tasks;
                if (ms / frac < 40.0) rounds[idx] = 0;
            }
            TuneChoice best[2];
            double best_ns[2] = {1e300, 1e300};
            for (int w = 0; w < 2; w++) best[w] = TuneChoice();
            // one stage: time the candidates `vals` of one field (the others at their best so far)
            auto stage = [&](int field, const int* vals, int nvals) {
                for (int v = 0; v < nvals; v++) {
                    PairTiling tc = tl;
                    bool any = false, on[2] = {false, false};
                    for (int idx = 0; idx < 2; idx++) {
                        if (!need_time[idx]) continue;
                        if (field == 0 && vals[v] > max_minb(idx == 0 ? 4 : 8)) continue;
                        on[idx] = true;
                        TuneChoice c = best[idx];
                        if (c.minb == 0) c.minb = 4;
                        if (field == 0) c.minb = vals[v];
                        if (field == 1) c.tasks_per_warp = vals[v];
                        if (field == 2) c.chunk = vals[v];
                        tc.minb[idx] = c.minb;
                        tc.tasks_per_warp[idx] = c.tasks_per_warp;
                        tc.chunk[idx] = c.chunk;
                        any = true;
                    }
                    if (!any) continue;
                    PairBatch b;
                    plan->build(b, tc, mixed, true);
                    for (size_t k = 0; k < b.live.size(); k++)
                        CK(launch_pauli_frames(b.live[k]->a->t.view(), b.dp.p + b.unit_obs[k], b.live[k]->nobs,
                                               b.px.p + b.unit_px[k], b.pk.p + b.unit_px[k], st));
                    for (size_t li = 0; li < b.launches.size(); li++) {
                        const int idx = b.launches[li].wb == 4 ? 0 : 1;
                        if (!need_time[idx] || !on[idx]) continue;
                        sample_ns_per_pair(b, li, st, 1);  // first launch of the candidate: warm-up
                        const double ns = sample_ns_per_pair(b, li, st, rounds[idx]);
                        if (ns < best_ns[idx]) {
                            best_ns[idx] = ns;
                            best[idx].minb = tc.minb[idx];
                            best[idx].tasks_per_warp = tc.tasks_per_warp[idx];
                            best[idx].chunk = tc.chunk[idx];
                        }
                    }
                    CK(cudaStreamSynchronize(st));
                }
                for (int idx = 0; idx < 2; idx++)
                    if (need_time[idx]) {
                        tl.minb[idx] = best[idx].minb;
                        tl.tasks_per_warp[idx] = best[idx].tasks_per_warp;
                        tl.chunk[idx] = best[idx].chunk;
                    }
            };
            for (int idx = 0; idx < 2; idx++)
                if (need_time[idx]) {
                    tl.tasks_per_warp[idx] = TuneChoice().tasks_per_warp;
                    tl.chunk[idx] = TuneChoice().chunk;
                }
            stage(0, kMinbCandidates, 5);
            stage(1, kTpwCandidates, 3);
            stage(2, kChunkCandidates, 3);
            for (int idx = 0; idx < 2; idx++)
                if (need_time[idx]) tune_store(keys[idx], best[idx]);
        }
    }
    plan->build(plan->batch, tl, mixed);
    for (const PairBatch::Launch& ln : plan->batch.launches) {  // the tiling each launch was built with
        const int idx = ln.wb == 4 ? 0 : 1;
        plan->tiling.chunk[idx] = ln.chunk;
        plan->tiling.tasks_per_warp[idx] = ln.tpw;
        plan->tiling.minb[idx] = ln.minb;
    }
    const size_t nres = 2 * std::max<size_t>(plan->batch.tot_obs, 1);
    CK(cudaMallocHost(&plan->pinned, nres * sizeof(double)));
    if (!plan->batch.live.empty()) {
        // One uncaptured run (checks the launches), then the capture.
        enqueue_batch(plan->batch, st);
        CK(cudaStreamSynchronize(st));
        CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        plan->enqueue_derived();
        enqueue_batch(plan->batch, st);
        CK(cudaMemcpyAsync(plan->pinned, plan->batch.dout.p, 2 * plan->batch.tot_obs * sizeof(double),
                           cudaMemcpyDeviceToHost, st));
        CK(cudaStreamEndCapture(st, &plan->graph));
        CK(cudaGraphInstantiate(&plan->exec, plan->graph, 0));
    }
    for (auto& ps : plan->states) ps->s->check_status();
    *out = plan.release();
    API_END
}

nsg_status nsg_plan_run(nsg_plan* plan, double* out) {
    API_BEGIN
    need(plan, "plan");
    for (auto& ps : plan->states) {
        const nsg_state* s = ps->s;
        if (!state_alive(s, ps->uid) || s->layout_gen != ps->gen || s->t.n != ps->n || s->t.chi != ps->chi ||
            s->gf_re != ps->gf_re || s->gf_im != ps->gf_im)
            raise(NSG_ERR_INVALID_ARGUMENT, -1, -1,
                  "a state of the plan was freed or changed its rank, width or global factor; create a new plan");
    }
    if (!plan->results.empty()) need(out, "out");
    if (plan->exec) {
        DeviceScope ds_(plan->device);
        for (auto& ps : plan->states) join_stream(plan->st, ps->s->st);
        CK(cudaGraphLaunch(plan->exec, plan->st));
        CK(cudaStreamSynchronize(plan->st));
        scatter_batch(plan->batch, plan->pinned);
        for (auto& ps : plan->states) ps->s->check_status();
    }
    if (!plan->results.empty()) std::memcpy(out, plan->results.data(), plan->results.size() * sizeof(double));
    API_END
}

nsg_status nsg_plan_info(const nsg_plan* plan, int32_t chunk[2], int32_t tasks_per_warp[2], int32_t minb[2],
                         int32_t* timed) {
    API_BEGIN
    need(plan, "plan");
    for (int w = 0; w < 2; w++) {
        if (chunk) chunk[w] = plan->tiling.chunk[w];
        if (tasks_per_warp) tasks_per_warp[w] = plan->tiling.tasks_per_warp[w];
    }
    if (minb) {
        minb[0] = plan->tiling.minb[0];
        minb[1] = plan->tiling.minb[1];
    }
    if (timed) *timed = plan->timed ? 1 : 0;
    API_END
}

void nsg_plan_free(nsg_plan* plan) { delete plan; }

nsg_status nsg_inner_product(const nsg_state* a, const nsg_state* b, double out[2]) {
    API_BEGIN
    need(a, "a");
    need(b, "b");
    need(out, "out");
    if (a->device != b->device)
        raise(NSG_ERR_INVALID_ARGUMENT, a->device, b->device, "the two states live on different devices");
    DeviceScope ds_(a->device);
    if (a->t.n != b->t.n)
        raise(NSG_ERR_QUBIT_COUNT_MISMATCH, a->t.n, b->t.n,
              "The qubit counts of the two states must match for calculating inner product, got %d and %d.", a->t.n,
              b->t.n);
    nsg_state* aa = const_cast<nsg_state*>(a);
    nsg_state* bb = const_cast<nsg_state*>(b);
    require_pairs_width(aa);
    if (aa != bb) CK(cudaStreamSynchronize(bb->st));
    std::vector<DevPauli> id(1, DevPauli{0, 0, 0, 0});
    std::vector<double> r;
    run_pairs(aa, bb, id, false, true, false, r);
    out[0] = r[0];
    out[1] = r[1];
    API_END
}

nsg_status nsg_norm(const nsg_state* state, double* out) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    need(out, "out");
    *out = std::sqrt(norm_squared(const_cast<nsg_state*>(state)));
    API_END
}

nsg_status nsg_project_unnormalized(nsg_state* state, uint32_t qubit, int32_t outcome) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    project_unnorm(state, qubit, outcome != 0);
    API_END
}

nsg_status nsg_project_normalized(nsg_state* state, uint32_t qubit, int32_t outcome) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    project_unnorm(state, qubit, outcome != 0);  // projection.rs:10-21
    double nrm = std::sqrt(norm_squared(state));
    if (std::fabs(nrm) < 1e-12 || std::isnan(nrm)) err_impossible(qubit, outcome != 0);
    state->gf_re /= nrm;
    state->gf_im /= nrm;
    API_END
}

nsg_status nsg_discard(nsg_state* state, uint32_t qubit) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    discard_q(state, qubit);
    API_END
}

nsg_status nsg_measure(nsg_state* state, const uint32_t* qargs, size_t num_qargs, const uint8_t* seed32,
                       uint8_t* out) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    if (num_qargs) {
        need(qargs, "qargs");
        need(out, "out");
    }
    validate_qargs(state, qargs, num_qargs);
    HostRng rng(seed32);
    for (size_t i = 0; i < num_qargs; i++) {  // measurement.rs:34-103
        uint32_t q = qargs[i];
        double p0, p1;
        outcome_weights(state, q, p0, p1);
        double tot = p0 + p1;
        if (std::fabs(tot) < 1e-12)
            raise(NSG_ERR_NOT_IMPLEMENTED, -1, -1, "Not implemented: Measurement on a zero-norm state is not possible.");
        double u = rng.uniform();
        bool one = !(u < p0 / tot);
        double nsq = one ? p1 : p0;
        double nrm = std::sqrt(nsq);
        if (std::fabs(nrm) < 1e-12)
            raise(NSG_ERR_NOT_IMPLEMENTED, -1, -1,
                  "Not implemented: Measurement resulted in a zero-norm state, which is not physical.");
        project_unnorm(state, q, one);
        state->gf_re /= nrm;
        state->gf_im /= nrm;
        out[i] = one ? 1 : 0;
    }
    API_END
}

nsg_status nsg_measure_all(nsg_state* state, const uint8_t* seed32, uint8_t* out) {
    API_BEGIN
    need(state, "state");
    std::vector<uint32_t> q(state->t.n);
    for (int i = 0; i < state->t.n; i++) q[i] = i;
    nsg_status rc = nsg_measure(state, q.data(), q.size(), seed32, out);
    if (rc != NSG_OK) return rc;
    API_END
}

nsg_status nsg_sample(const nsg_state* cstate, const uint32_t* qargs, size_t num_qargs, uint64_t shots,
                      const uint8_t* seed32, uint64_t* outcomes, uint64_t* counts, size_t capacity,
                      size_t* num_out) {
    API_BEGIN
    need(cstate, "state");
    DeviceScope ds_(cstate->device);
    need(num_out, "num_out");
    nsg_state* state = const_cast<nsg_state*>(cstate);
    if (num_qargs) need(qargs, "qargs");
    validate_qargs(state, qargs, num_qargs);
    if (num_qargs > 128) raise(NSG_ERR_SAMPLING_TOO_MANY_QUBITS, -1, -1, "Sampling more than 128 qubits is not supported.");
    HostRng rng(seed32);
    std::vector<std::pair<uint32_t, uint32_t>> qs;  // (qarg, bit), descending qarg (sampling.rs:31-37)
    for (size_t i = 0; i < num_qargs; i++) qs.push_back({qargs[i], (uint32_t)i});
    std::stable_sort(qs.begin(), qs.end(), [](auto& a, auto& b) { return a.first > b.first; });
    std::vector<ShotOut> res;
    if (num_qargs <= kMarginalMaxQubits && state->t.n <= 64) {
        // The node weights of the split tree all come from one marginal.
        std::vector<double> p = walsh_marginal(state, qs);
        sample_marginal(p, qs, 0, 0, shots, 0, 0, rng, res);
    } else {
        std::unique_ptr<nsg_state> work(clone_state(state));
        sample_rec(work.get(), qs, 0, shots, 0, 0, rng, res);
    }
    *num_out = res.size();
    if (res.size() > capacity)
        raise(NSG_ERR_BUFFER_TOO_SMALL, (int64_t)res.size(), (int64_t)capacity,
              "sample needs room for %zu outcomes, got %zu", res.size(), capacity);
    for (size_t i = 0; i < res.size(); i++) {
        outcomes[2 * i] = res[i].lo;
        outcomes[2 * i + 1] = res[i].hi;
        counts[i] = res[i].count;
    }
    API_END
}

nsg_status nsg_to_statevector(const nsg_state* state, double* out, size_t capacity_complex) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    const int n = state->t.n;
    if (n > 28)
        raise(NSG_ERR_STATEVECTOR_TOO_LARGE, n, -1,
              "Calculating the statevector for a state with %d qubits is not feasible.", n);
    if (n > 64) raise(NSG_ERR_TOO_WIDE, n, 64, "too wide");
    size_t dim = (size_t)1 << n;
    need(out, "out");
    if (capacity_complex < dim)
        raise(NSG_ERR_BUFFER_TOO_SMALL, (int64_t)dim, (int64_t)capacity_complex, "statevector needs %zu entries", dim);
    cudaStream_t st = state->st;
    DBuf<double> d;
    d.alloc(2 * dim, st);
    CK(launch_statevector(state->t.view(), state->gf_re, state->gf_im, d.p, st));
    CK(cudaMemcpyAsync(out, d.p, 2 * dim * sizeof(double), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    API_END
}

nsg_status nsg_export_terms(const nsg_state* state, uint8_t* G, uint8_t* F, uint8_t* M, uint8_t* gamma, uint8_t* v,
                            uint8_t* s, uint8_t* phase, uint8_t* coef_phase, int32_t* coef_r, uint8_t* coef_zero,
                            double global_factor[2]) {
    API_BEGIN
    need(state, "state");
    DeviceScope ds_(state->device);
    cudaStream_t st = state->st;
    const int64_t chi = state->t.chi;
    const int n = state->t.n;
    const size_t nn = (size_t)n * n * chi, nv = (size_t)n * chi;
    if (chi && n) {
        need(G, "G"); need(F, "F"); need(M, "M"); need(gamma, "gamma"); need(v, "v"); need(s, "s");
        DBuf<uint8_t> dG, dF, dM, dg, dv, ds;
        dG.alloc(nn, st); dF.alloc(nn, st); dM.alloc(nn, st);
        dg.alloc(nv, st); dv.alloc(nv, st); ds.alloc(nv, st);
        CK(launch_unpack(state->t.view(), dG.p, dF.p, dM.p, dg.p, dv.p, ds.p, st));
        CK(cudaMemcpyAsync(G, dG.p, nn, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(F, dF.p, nn, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(M, dM.p, nn, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(gamma, dg.p, nv, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(v, dv.p, nv, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(s, ds.p, nv, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
    }
    if (chi) {
        if (phase) CK(cudaMemcpyAsync(phase, state->t.phase.p, chi, cudaMemcpyDeviceToHost, st));
        if (coef_phase) CK(cudaMemcpyAsync(coef_phase, state->t.ck.p, chi, cudaMemcpyDeviceToHost, st));
        if (coef_r) CK(cudaMemcpyAsync(coef_r, state->t.cr.p, chi * 4, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (coef_zero) std::memset(coef_zero, 0, chi);
    }
    if (global_factor) {
        global_factor[0] = state->gf_re;
        global_factor[1] = state->gf_im;
    }
    API_END
}

nsg_status nsg_profile_enable(int32_t enabled) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_on = enabled != 0;
    return NSG_OK;
}

nsg_status nsg_profile_read(double* pair_kernel_ms, uint64_t* launches, uint64_t* pairs) {
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (pair_kernel_ms) *pair_kernel_ms = g_prof_ms;
    if (launches) *launches = g_prof_launches;
    if (pairs) *pairs = g_prof_pairs;
    g_prof_ms = 0.0;
    g_prof_launches = 0;
    g_prof_pairs = 0;
    return NSG_OK;
}

nsg_status nsg_probe_int_ops(uint64_t iters, double* seconds, uint64_t* ops) {
    API_BEGIN
    need(seconds, "seconds");
    need(ops, "ops");
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    const int sms = device_sm_count(), threads = 256, blocks = sms * 8;
    uint32_t* sink = nullptr;
    CK(cudaMalloc((void**)&sink, (size_t)blocks * threads * sizeof(uint32_t)));
    CK(launch_int_probe(2, blocks, threads, sink, st));  // warm-up
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, st));
    CK(launch_int_probe(iters, blocks, threads, sink, st));
    CK(cudaEventRecord(e1, st));
    CK(cudaEventSynchronize(e1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    cudaStreamDestroy(st);
    *seconds = ms * 1e-3;
    *ops = (uint64_t)blocks * threads * iters * 16 * 8;
    API_END
}

nsg_status nsg_state_kron(const nsg_state* a, const nsg_state* b, nsg_state** out) {
    API_BEGIN
    need(a, "a");
    need(b, "b");
    need(out, "out");
    *out = nullptr;
    if (a->device != b->device)
        raise(NSG_ERR_INVALID_ARGUMENT, a->device, b->device, "the two states live on different devices");
    DeviceScope ds_(a->device);
    const int n = a->t.n + b->t.n;
    if (n > 128) raise(NSG_ERR_TOO_WIDE, n, 128, "width %d exceeds 128", n);
    const int64_t ca = a->t.chi, cb = b->t.chi;
    if (ca && cb > (int64_t)(INT64_MAX / 256) / ca)
        raise(NSG_ERR_OUT_OF_MEMORY, ca, cb, "%lld x %lld terms do not fit", (long long)ca, (long long)cb);
    auto o = std::make_unique<nsg_state>();
    o->init_stream();
    CK(cudaStreamSynchronize(a->st));  // the inputs' pending work, then ours
    if (b != a) CK(cudaStreamSynchronize(b->st));
    o->t.alloc(n, ca * cb, o->st);
    o->t.chi = ca * cb;
    CK(launch_kron(a->t.view(), b->t.view(), o->t.view(), o->st));
    // global factors multiply (kron.rs builds its result with factor 1; both are 1 wherever the reference calls it)
    o->gf_re = a->gf_re * b->gf_re - a->gf_im * b->gf_im;
    o->gf_im = a->gf_re * b->gf_im + a->gf_im * b->gf_re;
    CK(cudaStreamSynchronize(o->st));
    *out = o.release();
    API_END
}

nsg_status nsg_random_clifford(uint32_t n, const uint8_t* seed32, nsg_gate* out, size_t capacity, size_t* num_out) {
    API_BEGIN
    need(num_out, "num_out");
    *num_out = 0;
    if (n > (1u << 24))  // 2n² + 3n gates and n² bytes per layer matrix must stay addressable
        raise(NSG_ERR_INVALID_ARGUMENT, n, 1 << 24, "random Clifford circuits are limited to 2^24 qubits, got %u", n);
    const uint64_t bound = random_clifford_max_gates(n);
    if (bound) need(out, "out");
    if (capacity < bound)
        raise(NSG_ERR_BUFFER_TOO_SMALL, (int64_t)bound, (int64_t)capacity,
              "capacity %zu is below the %llu gates a random Clifford on %u qubits may need", capacity,
              (unsigned long long)bound, n);
    HostRng rng(seed32);
    const std::vector<nsg_gate> g = random_clifford_gates(n, rng);
    std::copy(g.begin(), g.end(), out);
    *num_out = g.size();
    API_END
}

nsg_status nsg_random_words(const uint8_t* seed32, uint32_t* out, size_t count) {
    API_BEGIN
    need(seed32, "seed32");
    if (count) need(out, "out");
    HostRng rng(seed32);
    for (size_t i = 0; i < count; i++) out[i] = rng.next_u32();
    API_END
}

nsg_status nsg_debug_chacha_block(const uint32_t input[16], int32_t rounds, uint32_t output[16]) {
    API_BEGIN
    need(input, "input");
    need(output, "output");
    if (rounds <= 0 || rounds % 2 != 0 || rounds > 64)
        raise(NSG_ERR_INVALID_ARGUMENT, rounds, -1, "rounds must be a positive even number up to 64, got %d", rounds);
    ChaChaCore::block(input, rounds, output);
    API_END
}

nsg_status nsg_debug_t_tensor(uint32_t t, nsg_state** out) {
    API_BEGIN
    need(out, "out");
    *out = nullptr;
    if (t == 0 || t > 64) raise(NSG_ERR_INVALID_ARGUMENT, t, 64, "t must be in 1..64, got %u", t);
    auto probe = std::make_unique<nsg_state>();
    probe->init_stream();
    auto tt = t_tensor_dev((int)t, probe->st, probe->status.p);
    const size_t chi = (size_t)tt->chi, rows = chi * t;
    std::vector<uint64_t> G(rows), F(rows), M(rows), V(chi), S(chi);
    std::vector<uint8_t> gam(rows), ph(chi), ck(chi);
    std::vector<int32_t> cr(chi);
    cudaStream_t st = probe->st;
    CK(cudaMemcpyAsync(G.data(), tt->G, rows * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(F.data(), tt->F, rows * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(M.data(), tt->M, rows * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(gam.data(), tt->gam, rows, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(V.data(), tt->V, chi * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(S.data(), tt->S, chi * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ph.data(), tt->phase, chi, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(ck.data(), tt->ck, chi, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(cr.data(), tt->cr, chi * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    // The term-dump layout of nsg_state_from_terms: bits as bytes, γ as Z8 (2·exponent of i).
    std::vector<uint8_t> bG(rows * t), bF(rows * t), bM(rows * t), bgam(rows), bv(rows), bs(rows);
    for (size_t i = 0; i < chi; i++)
        for (uint32_t r = 0; r < t; r++) {
            const size_t row = i * t + r;
            for (uint32_t c = 0; c < t; c++) {
                bG[row * t + c] = (G[row] >> c) & 1;
                bF[row * t + c] = (F[row] >> c) & 1;
                bM[row * t + c] = (M[row] >> c) & 1;
            }
            bgam[row] = (uint8_t)(2 * gam[row]);
            bv[row] = (V[i] >> r) & 1;
            bs[row] = (S[i] >> r) & 1;
        }
    const double gf[2] = {1.0, 0.0};
    nsg_status rc = nsg_state_from_terms(t, chi, bG.data(), bF.data(), bM.data(), bgam.data(), bv.data(), bs.data(),
                                         ph.data(), ck.data(), cr.data(), nullptr, gf, out);
    if (rc != NSG_OK) return rc;
    API_END
}

nsg_status nsg_toffoli_tensor_state(uint32_t num_tensors, nsg_state** out) {
    API_BEGIN
    need(out, "out");
    *out = nullptr;
    // construct_toffoli_tensor_state (magic_states/toffoli_state.rs:33-40).
    if (num_tensors == 0)
        raise(NSG_ERR_INVALID_NUM_QUBITS, 0, -1, "Number of qubits must be greater than zero, got 0.");
    if (num_tensors > 21)
        raise(NSG_ERR_TOO_WIDE, 3 * (int64_t)num_tensors, 63, "%u Toffoli states need %u qubits; at most 21 (63 qubits)",
              num_tensors, 3 * num_tensors);
    // construct_toffoli_state (toffoli_state.rs:12-31): |0+0⟩ and |1⟩⊗Bell, each with 2^{-1/2}.
    HostCH a = HostCH::zero_state(3), b = HostCH::zero_state(3);
    a.left_h(1);
    b.left_x(0);
    b.left_h(1);
    b.left_cx(1, 2);
    const HostCH* terms[2] = {&a, &b};
    std::vector<uint8_t> bG(18), bF(18), bM(18), bgam(6), bv(6), bs(6), ph(2), ck(2, 0);
    std::vector<int32_t> cr(2, 1);
    for (int i = 0; i < 2; i++) {
        const HostCH& c = *terms[i];
        for (int r = 0; r < 3; r++) {
            for (int q = 0; q < 3; q++) {
                bG[i * 9 + r * 3 + q] = hbit(c.G[r].w, q);
                bF[i * 9 + r * 3 + q] = hbit(c.F[r].w, q);
                bM[i * 9 + r * 3 + q] = hbit(c.M[r].w, q);
            }
            bgam[i * 3 + r] = (uint8_t)(2 * c.gam[r]);  // the dump's γ is the Z8 exponent, 2·(power of i)
            bv[i * 3 + r] = hbit(c.v, r);
            bs[i * 3 + r] = hbit(c.s, r);
        }
        ph[i] = (uint8_t)c.phase;
    }
    const double gf[2] = {1.0, 0.0};
    nsg_state* base = nullptr;
    nsg_status rc = nsg_state_from_terms(3, 2, bG.data(), bF.data(), bM.data(), bgam.data(), bv.data(), bs.data(),
                                         ph.data(), ck.data(), cr.data(), nullptr, gf, &base);
    if (rc != NSG_OK) return rc;
    std::unique_ptr<nsg_state> base_owner(base), acc;  // acc empty: the result is the base itself
    for (uint32_t k = 1; k < num_tensors; k++) {  // construct(k) = construct(k-1).kron(construct(1))
        nsg_state* next = nullptr;
        rc = nsg_state_kron(acc ? acc.get() : base, base, &next);
        if (rc != NSG_OK) return rc;
        acc.reset(next);
    }
    *out = acc ? acc.release() : base_owner.release();
    API_END
}

nsg_status nsg_debug_pair_values(const nsg_state* cstate, const nsg_pauli* pauli, uint8_t* k, int32_t* r) {
    API_BEGIN
    need(cstate, "state");
    DeviceScope ds_(cstate->device);
    need(k, "k");
    need(r, "r");
    nsg_state* state = const_cast<nsg_state*>(cstate);
    require_pairs_width(state);
    std::vector<DevPauli> dp(1, DevPauli{0, 0, 0, 0});
    if (pauli) dp[0] = to_dev_pauli(*pauli, state->t.n);
    const int64_t chi = state->t.chi;
    if (chi == 0) return NSG_OK;
    DBuf<uint8_t> dk;
    DBuf<int32_t> dr;
    dk.alloc((size_t)chi * chi, state->st);
    dr.alloc((size_t)chi * chi, state->st);
    std::vector<double> out;
    run_pairs(state, state, dp, false, true, false, out, dk.p, dr.p);
    CK(cudaMemcpyAsync(k, dk.p, (size_t)chi * chi, cudaMemcpyDeviceToHost, state->st));
    CK(cudaMemcpyAsync(r, dr.p, (size_t)chi * chi * 4, cudaMemcpyDeviceToHost, state->st));
    CK(cudaStreamSynchronize(state->st));
    API_END
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Read-only access to a state and to the error slot for other translation
// units of this library (noalloc.cu).
namespace nsg {

bool state_internals(const nsg_state* s, TermsView* tv, cudaStream_t* st, int** status, int* device, double* gf2) {
    if (!s) return false;
    *tv = s->t.view();
    *st = s->st;
    *status = s->status.p;
    *device = s->device;
    *gf2 = s->gf_re * s->gf_re + s->gf_im * s->gf_im;
    return true;
}

void set_last_error(const char* msg, int64_t a, int64_t b) {
    g_msg = msg;
    g_args[0] = a;
    g_args[1] = b;
    g_args[2] = -1;
}

}  // namespace nsg
