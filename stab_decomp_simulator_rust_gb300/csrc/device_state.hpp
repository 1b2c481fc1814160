// device_state.hpp — the HBM layout of a stabilizer-decomposed state and the
// launchers of the kernels that operate on it.
//
// Terms are stored structure-of-arrays.  A term of width n uses W = ⌈n/64⌉
// 64-bit words per row and R = 64·W row slots, so lane l of a warp reads rows
// l, l+32, ... of one term as contiguous 8·W-byte chunks (coalesced):
//   G, F, M   [cap][R][W]   tableau rows (row r, column c = bit c)
//   V, S      [cap][W]      the bit vectors v, s
//   GL, GH    [cap][W]      γ as two bit planes: γ_r = GL_r + 2·GH_r (power of i)
//   phase     [cap]         Z8 exponent of the CH-form phase factor
//   coef_k    [cap]         Z8 phase of the exact coefficient
//   coef_r    [cap]         its exponent: coefficient = e^{iπk/4}·2^{-r/2}
// The reference's ω is 1 on every path (form/kron.rs:55 and
// form/mod.rs:76-81 are its only writers) and is not stored.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace nsg {

struct TermsView {
    int n = 0;        // width
    int W = 1;        // words per row
    int R = 64;       // row slots per term
    int64_t chi = 0;  // number of terms
    uint64_t* G = nullptr;
    uint64_t* F = nullptr;
    uint64_t* M = nullptr;
    uint64_t* V = nullptr;
    uint64_t* S = nullptr;
    uint64_t* GL = nullptr;
    uint64_t* GH = nullptr;
    uint8_t* phase = nullptr;
    uint8_t* coef_k = nullptr;
    int32_t* coef_r = nullptr;
};

// Per-term "bra frame": the tableau of U_C^{-1} (rows G_V, F_V, M_V, γ_V)
// used by the pair kernel; W = 1 only (n ≤ 64).
struct FrameView {
    uint64_t* GV = nullptr;  // [chi][64]
    uint64_t* FV = nullptr;
    uint64_t* MV = nullptr;
    uint64_t* GVL = nullptr;  // [chi] γ_V planes
    uint64_t* GVH = nullptr;
};

// Pauli observable in bit form (n ≤ 64): P = i^{ny}·X(px)·Z(pz).
struct DevPauli {
    uint64_t px, pz;
    int32_t ny;
    int32_t pad;
};

// Encoded primitive gate: op | q0 << 8 | q1 << 16.
enum PrimOp : uint32_t {
    P_H = 0, P_X = 1, P_Y = 2, P_Z = 3, P_S = 4, P_SDG = 5, P_CX = 8, P_CZ = 9
};
inline uint32_t enc_op(uint32_t op, uint32_t a, uint32_t b = 0) { return op | (a << 8) | (b << 16); }

// Device status word bits set by kernels (never a trap).
enum DevStatus : int {
    DS_OK = 0,
    DS_INVARIANT = 1,  // reference panic paths
    DS_CANNOT_DISCARD = 2,
    DS_TIMEOUT = 4,  // a bounded wait on a shared-memory barrier ran out
    DS_RANGE = 8,    // an exact count fell outside the count bins
};

// Exact accumulation: signed counts of pair-term real (and imaginary) parts
// sign·2^{-m/2} per m, at index m + kExactMOffset of kExactBins bins.
constexpr int kExactBins = 512;
constexpr int kExactMOffset = 192;

// ---- launchers (kernels_*.cu) ------------------------------------------------

// |T⟩^{⊗t} expansion on the device.  A small term (width ≤ 6) of the cat
// states the expansion is assembled from: rows of G, F, M, γ per row, v, s,
// phase, and its coefficient e^{iπk/4}·2^{-r/2}.
struct TSmallTerm {
    uint64_t G[6], F[6], M[6];
    uint8_t gam[6];
    uint8_t phase;
    uint8_t pad;
    uint64_t v, s;
    int32_t k, r;
};
// cat(t) for t > 6 is cat(m0) joined L times with cat(6) (m0 = t − 4L ∈ [3, 6];
// for t ≤ 6, m0 = t and L = 0): the host supplies the terms of both.
struct TPrelude {
    int t = 0, m0 = 0, L = 0, nbase = 0;
    TSmallTerm base[3];
    TSmallTerm cat6[3];
};
// The expansion in the layout the compile kernel reads: per term t rows.
struct TTensorOut {
    uint64_t *G = nullptr, *F = nullptr, *M = nullptr, *V = nullptr, *S = nullptr;
    uint8_t *gam = nullptr, *phase = nullptr, *ck = nullptr;
    int32_t* cr = nullptr;
};
// Builds all 2·χ_cat terms of |T⟩^{⊗t} (t ≤ 64); status bit DS_INVARIANT if a
// projection the construction relies on turns out impossible.
cudaError_t launch_t_tensor(const TPrelude& pre, int64_t chi_cat, TTensorOut out, int* status, cudaStream_t st);

// Compile: build |0^n⟩⊗T-term, apply the primitive op list, post-select the t
// ancillas (reverse order) and discard them.  T-terms have width t ≤ 64 in
// one word per row.  Writes unpacked results to `out` at the term's index and
// keep[i] (1 kept, 0 dropped) and ndet[i].
cudaError_t launch_compile(const uint32_t* d_ops, int nops, int n, int t, int64_t chi_t,
                           const uint64_t* tG, const uint64_t* tF, const uint64_t* tM,
                           const uint8_t* tGam, const uint64_t* tV, const uint64_t* tS,
                           const uint8_t* tPhase, const uint8_t* tCk, const int32_t* tCr,
                           TermsView out, int32_t* keep, int* status, cudaStream_t st);

// Stable compaction of kept terms from `in` into `out` (same n/W); returns the
// number kept through *d_count (device).  keep[] is consumed as 0/1 flags.
cudaError_t launch_compact(const TermsView& in, const int32_t* keep, int32_t* scan_tmp,
                           TermsView out, int64_t* d_count, cudaStream_t st);

// Apply a primitive op list to every term (QuantumState::apply_* loops).
cudaError_t launch_apply_ops(const uint32_t* d_ops, int nops, TermsView terms, int* status,
                             cudaStream_t st);

// A short list of primitive ops without H (S, Sdg, Z, X, Y, CZ, CX), passed by
// value: one thread per term updates only the rows the ops touch.  These
// updates cannot fail, so there is no status word.
constexpr int kRowOpsMax = 8;
struct RowOps {
    int n;
    uint32_t code[kRowOpsMax];
};
cudaError_t launch_row_ops(const RowOps& ops, TermsView terms, cudaStream_t st);

// Project every term on (qubit, outcome): keep[i] = 0 if impossible; the
// coefficient is amplified by -1 for random outcomes (projection.rs:27-57).
cudaError_t launch_project(TermsView terms, int qubit, int outcome, int32_t* keep, int* status,
                           cudaStream_t st);

// Discard qubit from every term (n -> n-1, same W storage).
cudaError_t launch_discard(TermsView terms, int qubit, int* status, cudaStream_t st);

// Unpack to bool bytes (the nsg_export_terms layout) / pack from them.
cudaError_t launch_unpack(const TermsView& t, uint8_t* G, uint8_t* F, uint8_t* M, uint8_t* gam,
                          uint8_t* v, uint8_t* s, cudaStream_t st);
cudaError_t launch_pack(TermsView t, const uint8_t* G, const uint8_t* F, const uint8_t* M,
                        const uint8_t* gam, const uint8_t* v, const uint8_t* s, cudaStream_t st);

// A ⊗ B term by term (output term i·χ_B + j), into O (width n_A + n_B, χ_A·χ_B
// terms allocated by the caller).
cudaError_t launch_kron(TermsView A, TermsView B, TermsView O, cudaStream_t st);

// Bra frames (U_C^{-1} tableau) of every term; n ≤ 64.
cudaError_t launch_frames(const TermsView& t, FrameView fr, cudaStream_t st);

// Pauli frames: x_{A,P} and Z8 phase k_{A,P} for every (term A, observable P).
cudaError_t launch_pauli_frames(const TermsView& t, const DevPauli* d_paulis, int nobs,
                                uint64_t* x_out, uint8_t* k_out, cudaStream_t st);

// One launch of the row-staged pair kernel (launch_pairs_rows).
struct PairLaunch {
    TermsView A;   // bra terms (frames computed from these)
    FrameView fr;  // frames of A
    TermsView B;   // ket terms
    const uint64_t* px = nullptr;  // [chiA][nobs] x_{A,P}
    const uint8_t* pk = nullptr;   // [chiA][nobs] k_{A,P}
    int nobs = 1;
    bool triangular = true;  // exp_value/norm (A == B, i ≤ j) vs inner product (all pairs)
    bool complex_out = false;
    bool mixed = false;
    int chunk = 32;
    int64_t total_chunks = 0;
    const int64_t* row_chunk_off = nullptr;  // triangular: [chiA+1] prefix of chunks per row
    double* partials = nullptr;              // [nwarps][nobs][8]
    int nwarps = 0;
    int blocks = 0;
    int warps_per_block = 4;
    int* status = nullptr;
    uint8_t* dbg_k = nullptr;  // optional per-pair dump [chiA][chiB]
    int32_t* dbg_r = nullptr;
};

// One unit of a batched pair-sum launch: bra terms A (with their frames and
// Pauli frames) against ket terms B (with their term tables).
struct PairDesc {
    TermsView A;
    TermsView B;
    FrameView fr;                  // frames of A
    const void* ktab = nullptr;    // term tables of B (ket side)
    const void* atab = nullptr;    // term tables of A (its G table is the bra side)
    size_t ktab_stride = 0;        // bytes per term of both (A and B have the same width)
    uint32_t ket_bytes = 0;        // the part of a term's tables the kernel copies per ket
    int ngrp = 0;
    int nobs = 0;
    const uint64_t* px = nullptr;  // [chiA][nobs] x_{A,P}
    const uint8_t* pk = nullptr;   // [chiA][nobs] Z8 phase
    int triangular = 1;            // exp_value/norm (A == B, i ≤ j) vs inner product (all pairs)
    int complex_out = 0;
    const int64_t* blk_chunk_off = nullptr;  // triangular: [nblk+1] chunk prefix of the ket blocks
    int64_t nblk = 0;                        // ket blocks of `chunk` kets
    int64_t nchunks = 0;                     // chunks of the unit
    int64_t rec0 = 0;                        // first double of the unit's task records
    double scale_re = 1.0, scale_im = 0.0;   // |g|² or conj(g_a)·g_b
    int* status = nullptr;                   // the owning state's status words
    unsigned long long* counts = nullptr;    // exact mode: [nobs][2][kExactBins] signed counts (re, im)
};

// A persistent launch over the task lists of many units.  Each unit's chunks
// are cut into tasks of task_chunks chunks; warp w starts with task w and
// takes further tasks from *counter.  Every task accumulates into its own
// record ([nobs of its unit][8] doubles at rec0 + task·nobs·8), so the sums do
// not depend on the schedule.
struct MultiLaunch {
    const PairDesc* descs = nullptr;      // device [num_descs]
    int num_descs = 0;
    const int64_t* task_begin = nullptr;  // device [num_descs+1] first global task of each unit
    int64_t total_tasks = 0;
    int task_chunks = 1;
    int chunk = 32;
    int nobs_max = 1;
    bool mixed = false;
    bool exact = false;                   // integer counts per power of √2 instead of FP sums (descs[].counts)
    double* records = nullptr;
    unsigned long long* counter = nullptr;  // zero before the launch
    int nwarps = 0;
    int blocks = 0;
    int minb = 4;                         // kernel variant: blocks per SM its registers allow (2..5)
    size_t tab_bytes_max = 0;             // largest ket_bytes among the units
    size_t bra_bytes_max = 0;             // largest bra (G) table among the units
    size_t warp_smem = 0;
    uint8_t* dbg_k = nullptr;             // single-unit per-pair dump [chiA][chiB]
    int32_t* dbg_r = nullptr;
    uint32_t poll_limit = 0;              // polls of a bounded barrier wait (0: 2^22)
    uint32_t dbg_extra_tx = 0;            // test hook: bytes a chunk's first ket barrier expects beyond its copy
};

// word_bytes: 4 when every unit of the launch has n ≤ 32, 8 when every unit
// has 32 < n ≤ 64 (units are split by word width; term tables are built with
// the word width of their state, ket_table_stride).
cudaError_t launch_pairs_multi(const MultiLaunch& m, int word_bytes, cudaStream_t st);
// out: 2 doubles (re, im) per observable, observables of unit u starting at obs_begin[u].
// scratch: reduce_splits(total_obs) · total_obs · 8 doubles.
cudaError_t launch_reduce_multi(const MultiLaunch& m, const int64_t* obs_begin, int64_t total_obs, double* out,
                                double* scratch, cudaStream_t st);
int reduce_splits(int64_t total_obs);
size_t pair_warp_smem_bytes(size_t ket_bytes_max, size_t bra_bytes_max, int word_bytes);
// Warps of the pair kernel resident on the whole device at once.
int pair_resident_warps(int word_bytes, int nobs_max, size_t warp_smem, int minb);

// The same sums with B's rows staged per pair instead of term tables (no
// per-term table storage; at most 32 observables).
cudaError_t launch_pairs_rows(const PairLaunch& p, cudaStream_t st);

// Term tables: per term, Four-Russians tables of F, the ordered-sign matrix
// P, K = M·Fᵀ and G, plus the term's scalars (n ≤ 64); sizes below.
int ket_table_groups(int n);
size_t ket_table_stride(int n);      // bytes per term
size_t ket_table_ket_bytes(int n);   // the leading part read per ket (F, P, K tables and scalars)
size_t ket_table_bra_bytes(int n);   // the trailing G table, read per bra
cudaError_t launch_ket_tables(const TermsView& t, void* out, cudaStream_t st);

// Reduce per-warp partials to one value (re, im) per observable, scaled by
// `scale` (|global factor|² or the complex conj(g_a)·g_b).
cudaError_t launch_reduce(const double* partials, int nwarps, int nobs, bool complex_out,
                          double scale_re, double scale_im, double* out, cudaStream_t st);

// Dense statevector of the decomposed state (n ≤ 28): out[2^n] complex.
cudaError_t launch_statevector(const TermsView& t, double gf_re, double gf_im, double* out,
                               cudaStream_t st);

int device_sm_count();

// Integer-pipe probe kernel (measurement helper).
cudaError_t launch_int_probe(uint64_t iters, int blocks, int threads, uint32_t* sink, cudaStream_t st);

}  // namespace nsg
