/*
 * necstar_gpu.h — C ABI of the GB300-native stabilizer-decomposition engine.
 *
 * The exported functions are the drop-in boundary for the reference's public
 * `QuantumState` API (crates/necstar/src/state/mod.rs:67-706).  Every call
 * returns an `nsg_status`; results go into caller-provided buffers; a state is
 * an opaque handle that owns its χ CH-form terms in device memory.  A Rust
 * crate binds these with `extern "C"` declarations of the same signatures;
 * Python binds them with ctypes (stab_decomp_simulator_rust_gb300/_ffi.py).
 *
 * Threading: each state owns one CUDA stream.  Calls on different states may
 * run concurrently from different host threads; calls on the same state must be
 * serialised by the caller (the reference takes `&mut self` for the mutating
 * calls and holds the GIL in its Python layer, python/src/state.rs:13-222).
 */
#ifndef NECSTAR_GPU_H
#define NECSTAR_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes.  One per variant of necstar::Error
 * (crates/necstar/src/error/mod.rs:10-91) and of the CH-form crate's Error
 * (crates/stabilizer-ch-form-rust/src/error/mod.rs:7-67).  The reference's
 * `panic!`/`unreachable!` invariant checks (form/inner_product.rs:66,
 * form/resolve_superposition.rs:121, form/discard.rs:140,155) become
 * NSG_ERR_DEVICE_INVARIANT: the kernels record them in a status word and
 * never trap.  The numeric payload of the last error (qubit index, qubit
 * count, ...) is available from nsg_last_error_args().                     */
typedef int32_t nsg_status;

#define NSG_OK                                 0
#define NSG_ERR_QUBIT_INDEX_OUT_OF_BOUNDS      1  /* args: index, num_qubits      */
#define NSG_ERR_INVALID_NUM_QUBITS             2  /* args: num_qubits             */
#define NSG_ERR_GATE_NOT_CLIFFORD              3  /* args: gate op                */
#define NSG_ERR_STATEVECTOR_TOO_LARGE          4  /* args: num_qubits             */
#define NSG_ERR_NON_CLIFFORD_GATE_APPLICATION  5  /* args: gate op                */
#define NSG_ERR_QUBIT_COUNT_MISMATCH           6  /* args: left, right            */
#define NSG_ERR_MEASUREMENT_TOO_MANY_QUBITS    7
#define NSG_ERR_SAMPLING_TOO_MANY_QUBITS       8
#define NSG_ERR_IMPOSSIBLE_PROJECTION          9  /* args: qubit, desired outcome */
#define NSG_ERR_DUPLICATE_QUBIT_INDEX         10  /* args: index (qarg lists)     */
#define NSG_ERR_INVALID_PAULI_STRING_LENGTH   11  /* args: expected, found        */
#define NSG_ERR_EMPTY_QUBIT_INDICES           12
#define NSG_ERR_GATE_NOT_SUPPORTED            13  /* args: gate op (compiler)     */
#define NSG_ERR_DUPLICATE_QUBIT_INDICES       14  /* args: index (two-qubit gate) */
#define NSG_ERR_CANNOT_DISCARD_QUBIT          15  /* args: qubit                  */
#define NSG_ERR_NOT_IMPLEMENTED               16
#define NSG_ERR_PAULI_STRING_PARSING          17
#define NSG_ERR_INVALID_ARGUMENT              18  /* null pointer, bad enum value */
#define NSG_ERR_QASM_PARSING                  19  /* QasmParsingError (host-side circuit parser) */
#define NSG_ERR_IO                            20  /* Io (host-side QASM file writer)             */
#define NSG_ERR_CUDA                         100  /* args: cudaError_t            */
#define NSG_ERR_DEVICE_INVARIANT             101  /* args: invariant id, term     */
#define NSG_ERR_TIMEOUT                      102
#define NSG_ERR_OUT_OF_MEMORY                103
#define NSG_ERR_BUFFER_TOO_SMALL             104  /* args: required, given        */
#define NSG_ERR_TOO_WIDE                     105  /* args: width, supported max   */

/* ------------------------------------------------------------------------ */
/* Gates.  Opcodes follow the order of the QuantumGate enum
 * (crates/necstar/src/circuit/gates.rs:7-42).  One-qubit gates use q0;
 * CX uses (q0 = control, q1 = target); CZ and SWAP use (q0, q1);
 * CCX uses (q0, q1 = controls, q2 = target).                               */
enum nsg_gate_op {
    NSG_GATE_H = 0,
    NSG_GATE_X = 1,
    NSG_GATE_Y = 2,
    NSG_GATE_Z = 3,
    NSG_GATE_S = 4,
    NSG_GATE_SDG = 5,
    NSG_GATE_SQRT_X = 6,
    NSG_GATE_SQRT_XDG = 7,
    NSG_GATE_CX = 8,
    NSG_GATE_CZ = 9,
    NSG_GATE_SWAP = 10,
    NSG_GATE_T = 11,
    NSG_GATE_TDG = 12,
    NSG_GATE_CCX = 13
};

typedef struct nsg_gate {
    uint32_t op;
    uint32_t q0;
    uint32_t q1;
    uint32_t q2;
} nsg_gate;

/* ------------------------------------------------------------------------ */
/* Pauli strings.  Mirrors PauliString::{Dense, Sparse}
 * (crates/stabilizer-ch-form-rust/src/types/pauli/mod.rs:43-46).  A dense
 * string lists one op per qubit in little-endian order (ops[q] acts on qubit
 * q; the reference reverses the text form into this order, :70).  A sparse
 * string lists (qubits[k], ops[k]) pairs.                                   */
enum nsg_pauli_op { NSG_PAULI_I = 0, NSG_PAULI_X = 1, NSG_PAULI_Y = 2, NSG_PAULI_Z = 3 };
enum nsg_pauli_kind { NSG_PAULI_DENSE = 0, NSG_PAULI_SPARSE = 1 };

typedef struct nsg_pauli {
    uint32_t kind;           /* nsg_pauli_kind                               */
    uint32_t len;            /* dense: number of ops; sparse: number of terms */
    const uint8_t* ops;      /* nsg_pauli_op per entry                       */
    const uint32_t* qubits;  /* sparse only: qubit of each term              */
} nsg_pauli;

/* Accumulation modes of the χ² pair sums (exact per-pair phase/exponent in
 * both; only the coefficient-weighted accumulation differs).                */
enum nsg_precision {
    NSG_PRECISION_FP64 = 0,  /* compensated FP64 per lane, FP64 reduction    */
    NSG_PRECISION_MIXED = 1  /* compensated FP32 per lane with per-tile
                                power-of-two scaling, FP64 final reduction  */
};

/* Exact accumulation (nsg_exp_value_counts): every pair term of the χ² sum
 * has a real part sign·2^(-m/2) for an integer m; the count for m is at
 * index m + NSG_EXACT_M_OFFSET of NSG_EXACT_BINS bins.                       */
#define NSG_EXACT_BINS                       512
#define NSG_EXACT_M_OFFSET                   192

typedef struct nsg_state nsg_state;

/* ------------------------------------------------------------------------ */
/* Library                                                                   */

/* Version string of the library. */
const char* nsg_version(void);

/* Text of the last error raised on the calling thread, in the wording of the
 * reference's thiserror messages (crates/necstar/src/error/mod.rs:10-91). */
const char* nsg_last_error_message(void);

/* Numeric payload of the last error on the calling thread (see the status
 * list above); unused slots are -1. */
nsg_status nsg_last_error_args(int64_t out[3]);

/* ------------------------------------------------------------------------ */
/* Construction.                                                             */

/* Compiles a Clifford+T circuit into its stabilizer decomposition on the
 * current CUDA device.  Replaces QuantumState::from_circuit
 * (crates/necstar/src/state/mod.rs:98-102 → state/compiler/mod.rs:44-140). */
nsg_status nsg_state_from_circuit(uint32_t num_qubits, const nsg_gate* gates,
                                  size_t num_gates, nsg_state** out);

/* Batched form of nsg_state_from_circuit (no reference counterpart): circuit
 * c (num_qubits[c], gates[c][0..num_gates[c])) becomes out[c], the same
 * state nsg_state_from_circuit gives.  Every circuit is validated and its
 * compile queued on its own stream before the call waits for any of them.
 * On an error no state is returned and the failing circuit's index is in
 * nsg_last_error_args()[2]. */
nsg_status nsg_states_from_circuits(size_t num_circuits, const uint32_t* num_qubits,
                                    const nsg_gate* const* gates, const size_t* num_gates,
                                    nsg_state** out);

/* Builds a state from explicit CH-form terms given as bool bytes (the layout
 * of nsg_export_terms).  Replaces StabilizerDecomposedState::new
 * (crates/necstar/src/state/stabilizer_decomposed_state/mod.rs:28-41); also
 * the resume half of the checkpoint format. */
nsg_status nsg_state_from_terms(uint32_t num_qubits, uint64_t num_terms,
                                const uint8_t* G, const uint8_t* F, const uint8_t* M,
                                const uint8_t* gamma, const uint8_t* v, const uint8_t* s,
                                const uint8_t* phase, const uint8_t* coef_phase,
                                const int32_t* coef_r, const uint8_t* coef_zero,
                                const double global_factor[2], nsg_state** out);

/* Releases a state (Drop). */
void nsg_state_free(nsg_state* state);

/* Deep copy (Clone). */
nsg_status nsg_state_clone(const nsg_state* state, nsg_state** out);

/* QuantumState::num_qubits (crates/necstar/src/state/mod.rs:681-685). */
nsg_status nsg_num_qubits(const nsg_state* state, uint32_t* out);

/* QuantumState::stabilizer_rank (crates/necstar/src/state/mod.rs:692-696). */
nsg_status nsg_stabilizer_rank(const nsg_state* state, uint64_t* out);

/* Routes the state's work onto a caller-owned cudaStream_t (NULL restores
 * the state's own stream). */
nsg_status nsg_state_set_stream(nsg_state* state, void* cuda_stream);

/* ------------------------------------------------------------------------ */
/* Gates on a compiled state.                                                */

/* QuantumState::apply_gates (crates/necstar/src/state/mod.rs:522-526 →
 * stabilizer_decomposed_state/gates.rs:7-37); T/Tdg/CCX give
 * NSG_ERR_NON_CLIFFORD_GATE_APPLICATION.  A list that lowers to at most eight
 * primitive gates without H (one S, Sdg, X, Y, Z, CX, CZ or SWAP gate, for
 * instance) is applied by one thread per term to the rows it touches and the
 * call returns without waiting for the device; other lists run one warp per
 * term over the whole gate list and wait for its status. */
nsg_status nsg_apply_gates(nsg_state* state, const nsg_gate* gates, size_t num_gates);

/* ------------------------------------------------------------------------ */
/* χ² pair sums.                                                             */

/* QuantumState::exp_value (crates/necstar/src/state/mod.rs:309-313 →
 * stabilizer_decomposed_state/exp_value.rs:7-61).  Plain single-observable
 * FP64 path. */
nsg_status nsg_exp_value(const nsg_state* state, const nsg_pauli* pauli, double* out);

/* Batched form: many observables on one state in one pass over the χ² pair
 * space (no reference counterpart; same result per observable as
 * nsg_exp_value). */
nsg_status nsg_exp_value_batch(const nsg_state* state, const nsg_pauli* paulis,
                               size_t num_paulis, uint32_t precision, double* out);

/* Batched form across states: observables paulis[pauli_offsets[c] ..
 * pauli_offsets[c+1]) on states[c], all in one persistent launch.  out has
 * pauli_offsets[num_states] entries.  No reference counterpart. */
nsg_status nsg_exp_value_multi(const nsg_state* const* states, size_t num_states,
                               const nsg_pauli* paulis, const uint64_t* pauli_offsets,
                               uint32_t precision, double* out);

/* The exact accumulator of exp_value (no reference counterpart; the exact sum
 * the FP64 and mixed results are measured against): for observable o,
 * counts[o·NSG_EXACT_BINS + m + NSG_EXACT_M_OFFSET] is the signed number of
 * pair terms of the reference's χ² sum (stabilizer_decomposed_state/
 * exp_value.rs:38-58, the j > i terms counted twice) whose real part is
 * 2^(-m/2), so ⟨P_o⟩ = scale·Σ_m counts[..m..]·2^(-m/2) exactly, with
 * *scale = |global factor|² (may be NULL).  Integer counts: the result does
 * not depend on the schedule.  An exponent outside the bins gives
 * NSG_ERR_INVALID_ARGUMENT. */
nsg_status nsg_exp_value_counts(const nsg_state* state, const nsg_pauli* paulis, size_t num_paulis,
                                int64_t* counts, double* scale);

/* Observables whose ⟨P⟩ is exactly 0 without any pair work (no reference
 * counterpart; exp_value itself always sums the pairs).  A compiled state is
 * (1 ⊗ ⟨0|^t) U' (|0^n⟩ ⊗ |T⟩^{⊗t}) with U' the lowered circuit (T and Tdg as a
 * CX onto an ancilla); the images under U' of data-qubit Z strings with no X
 * component on the ancillas are, restricted to the data qubits, stabilizers
 * common to every term, and a Pauli that anticommutes with one of them has a
 * zero term for every pair.  zero[i] = 1: ⟨P_i⟩ = 0 exactly; 0: not decided by
 * this test.  The generators follow Clifford gates (nsg_apply_gates), clones
 * and term selections; projection, discard and measurement drop them (every
 * entry 0 afterwards), as do states not made by compiling a circuit.  Host
 * work only, O(n) words per observable. */
nsg_status nsg_zero_screen(const nsg_state* state, const nsg_pauli* paulis, size_t num_paulis, uint8_t* zero);
/* The same test for a circuit, without compiling it (host only; no GPU
 * needed); the circuit's checks and errors are nsg_state_from_circuit's. */
nsg_status nsg_zero_screen_circuit(uint32_t num_qubits, const nsg_gate* gates, size_t num_gates,
                                   const nsg_pauli* paulis, size_t num_paulis, uint8_t* zero);

/* Tiling of the direct (uncaptured) pair sums of this process: kets per
 * chunk and tasks per resident warp of the persistent pair launch; 0 takes
 * the tuned choice of the workload class if a plan tuned one, else the
 * default (32 and 64).  Results do not depend on it beyond FP rounding of the
 * partial sums (no reference counterpart). */
nsg_status nsg_set_pair_tiling(int32_t chunk, int32_t tasks_per_warp);

/* ⟨P⟩ for callers that cannot allocate device memory at call time — a
 * process whose GPU memory is already fully reserved by another allocator,
 * or a latency-critical loop where cudaMalloc/cudaFree would synchronise the
 * device.  Same value as nsg_exp_value; no counterpart in the reference.
 * All scratch comes from one 16 MiB static device array (held by every GPU
 * that loads the library until exit): n ≤ 64 (NSG_ERR_TOO_WIDE above) and
 * χ ≤ 8192 (NSG_ERR_BUFFER_TOO_SMALL above).  The first call on a device
 * looks up the array's address (make it before any stream capture); CUDA
 * loads device code lazily, so the array's memory is taken when that first
 * call runs: make one call on each device before another allocator reserves
 * its memory (or set CUDA_MODULE_LOADING=EAGER).  Like every entry point the
 * call runs on the state's device and restores the caller's.  All calls
 * share the array, so calls that overlap on the GPU race.  Synchronous: *out
 * is a host double. */
nsg_status nsg_exp_value_noalloc(const nsg_state* state, const nsg_pauli* pauli, double* out);

/* A captured batched evaluation (no reference counterpart): the work of
 * nsg_exp_value_multi — frames and term tables of every state, Pauli frames,
 * the persistent pair launches, the reductions and the copy of the results
 * to pinned host memory — captured once in a CUDA graph on the plan's own
 * stream.  nsg_plan_run replays it and writes pauli_offsets[num_states]
 * doubles to out.  Every run re-reads the states' current terms, so Clifford
 * gates applied in place (nsg_apply_gates) are seen by the next run; an
 * operation that changes a state's rank, width or global factor (projection,
 * discard, measurement) or frees it makes nsg_plan_run fail with
 * NSG_ERR_INVALID_ARGUMENT.  Creation picks, for each row width, the
 * pair-kernel variant (2-6 blocks per SM for 32-bit rows, 2-5 for 64-bit
 * rows), the tasks per resident warp (16,
 * 64, 256) and the kets per chunk (16, 32, 64), in that order, by timing the
 * candidates on the plan's own work (whole launches when short, else the
 * first two tasks per resident warp); the choice is remembered per device
 * and workload class for the process (direct calls of the same class use it
 * too) and, when the environment variable NSG_TUNE_CACHE names a file, read
 * from and appended to it (one JSON object per line). */
typedef struct nsg_plan nsg_plan;
nsg_status nsg_plan_create(const nsg_state* const* states, size_t num_states, const nsg_pauli* paulis,
                           const uint64_t* pauli_offsets, uint32_t precision, nsg_plan** out);
nsg_status nsg_plan_run(nsg_plan* plan, double* out);
/* The tiling in use for 32-bit ([0]) and 64-bit ([1]) rows: kets per chunk,
 * tasks per resident warp, the kernel variant (blocks per SM its registers
 * allow); 0 where the plan has no launch of that width.  *timed = 1 when
 * creation timed candidates, 0 when it took them from the cache. */
nsg_status nsg_plan_info(const nsg_plan* plan, int32_t chunk[2], int32_t tasks_per_warp[2], int32_t minb[2],
                         int32_t* timed);
void nsg_plan_free(nsg_plan* plan);

/* QuantumState::inner_product ⟨a|b⟩ (crates/necstar/src/state/mod.rs:165-172 →
 * stabilizer_decomposed_state/inner_product.rs:9-19).  out = {re, im}. */
nsg_status nsg_inner_product(const nsg_state* a, const nsg_state* b, double out[2]);

/* QuantumState::norm (crates/necstar/src/state/mod.rs:702-706 →
 * stabilizer_decomposed_state/norm.rs:8-35). */
nsg_status nsg_norm(const nsg_state* state, double* out);

/* ------------------------------------------------------------------------ */
/* Projection, discard, measurement, sampling.                              */

/* QuantumState::project_normalized (crates/necstar/src/state/mod.rs:348-354 →
 * stabilizer_decomposed_state/projection.rs:10-21). */
nsg_status nsg_project_normalized(nsg_state* state, uint32_t qubit, int32_t outcome);

/* QuantumState::project_unnormalized (crates/necstar/src/state/mod.rs:406-412 →
 * stabilizer_decomposed_state/projection.rs:27-57). */
nsg_status nsg_project_unnormalized(nsg_state* state, uint32_t qubit, int32_t outcome);

/* QuantumState::discard (crates/necstar/src/state/mod.rs:452-456 →
 * stabilizer_decomposed_state/discard.rs:5-12). */
nsg_status nsg_discard(nsg_state* state, uint32_t qubit);

/* QuantumState::measure (crates/necstar/src/state/mod.rs:201-205 →
 * stabilizer_decomposed_state/measurement.rs:10-24).  seed32 may be NULL
 * (entropy).  out[k] = outcome of qargs[k] (0/1). */
nsg_status nsg_measure(nsg_state* state, const uint32_t* qargs, size_t num_qargs,
                       const uint8_t* seed32, uint8_t* out);

/* QuantumState::measure_all (crates/necstar/src/state/mod.rs:233-237).
 * out has num_qubits entries. */
nsg_status nsg_measure_all(nsg_state* state, const uint8_t* seed32, uint8_t* out);

/* QuantumState::sample (crates/necstar/src/state/mod.rs:273-284 →
 * stabilizer_decomposed_state/sampling.rs:13-189).  Outcome k is returned as
 * a 128-bit integer in outcomes[2k] (low word) and outcomes[2k+1] (high
 * word); bit i ↔ qargs[i] (ShotCount packing,
 * crates/necstar/src/types/shot_count/mod.rs:11-68).  counts[k] is its
 * frequency.  At most `capacity` outcomes are written; *num_out receives the
 * number of distinct outcomes (NSG_ERR_BUFFER_TOO_SMALL if above capacity). */
nsg_status nsg_sample(const nsg_state* state, const uint32_t* qargs, size_t num_qargs,
                      uint64_t shots, const uint8_t* seed32, uint64_t* outcomes,
                      uint64_t* counts, size_t capacity, size_t* num_out);

/* QuantumState::to_statevector (crates/necstar/src/state/mod.rs:134-138 →
 * stabilizer_decomposed_state/statevector.rs:12-24); out holds 2^n complex
 * values as interleaved (re, im); n ≤ 28. */
nsg_status nsg_to_statevector(const nsg_state* state, double* out, size_t capacity_complex);

/* |a⟩ ⊗ |b⟩ as a new state of n_a + n_b ≤ 128 qubits (b's qubits follow a's):
 * term i·χ_b + j is the CH-form kron of a's term i and b's term j with the
 * product coefficient, in the order of StabilizerDecomposedState::kron
 * (crates/necstar/src/state/stabilizer_decomposed_state/kron.rs:7-22, with
 * StabilizerCHForm::kron, crates/stabilizer-ch-form-rust/src/form/kron.rs:12-59;
 * crate-internal in the reference, where it builds the magic states).  The
 * global factors multiply (the reference's result has factor 1, which is the
 * product wherever it calls it).  Both states must be on one device. */
nsg_status nsg_state_kron(const nsg_state* a, const nsg_state* b, nsg_state** out);

/* |Toffoli⟩^{⊗k} = ((|000⟩ + |100⟩ + |010⟩ + |111⟩)/2)^{⊗k} as a state of
 * 3k qubits and 2^k terms, in the order of construct_toffoli_tensor_state
 * (crates/necstar/src/state/magic_states/toffoli_state.rs:12-40: the
 * two-term |0+0⟩, |1⟩⊗Bell decomposition, each term 2^{-1/2}, joined by
 * kron): the base state is built on the host and the joins run on the
 * device (nsg_state_kron).  1 ≤ k ≤ 21 (n ≤ 63): k = 0 gives
 * NSG_ERR_INVALID_NUM_QUBITS, larger k NSG_ERR_TOO_WIDE.  The reference
 * marks the construction crate-internal and unused (Toffoli-state injection
 * is not implemented there either). */
nsg_status nsg_toffoli_tensor_state(uint32_t num_tensors, nsg_state** out);

/* QuantumCircuit::random_clifford (crates/necstar/src/circuit/mod.rs:289-291
 * → crates/stabilizer-ch-form-rust/src/circuit/random_clifford.rs:177-212):
 * a uniformly random n-qubit Clifford as a gate list (Bravyi–Maslov canonical
 * form U = F1·H·S·F2, drawn and emitted in the reference's order from the
 * seeded stream below).  out must hold 2n² + 3n gates (the bound; fewer are
 * written, *num_out of them); seed32 may be NULL (entropy); n = 0 gives no
 * gates; n ≤ 2^24. */
nsg_status nsg_random_clifford(uint32_t n, const uint8_t* seed32, nsg_gate* out, size_t capacity,
                               size_t* num_out);

/* The seeded stream that measure, sample and random_clifford draw from: the
 * first `count` 32-bit words of ChaCha with 12 rounds keyed by the 32 seed
 * bytes (64-bit block counter from 0, stream id 0), the generator behind the
 * reference's StdRng::from_seed (rand 0.8.5 / rand_chacha 0.3.1). */
nsg_status nsg_random_words(const uint8_t* seed32, uint32_t* out, size_t count);

/* Diagnostic: one ChaCha block (input words 0-15 → output words 0-15 after
 * `rounds` rounds and the feed-forward addition), for known-answer tests of
 * the stream above. */
nsg_status nsg_debug_chacha_block(const uint32_t input[16], int32_t rounds, uint32_t output[16]);

/* ------------------------------------------------------------------------ */
/* Parity dump / checkpoint.  Writes every term as bool bytes:
 *   G, F, M: [term][row][col]   (num_terms · n · n bytes each)
 *   gamma:   [term][row]        Z8 exponent k of the reference's γ (0,2,4,6)
 *   v, s:    [term][qubit]
 *   phase:   [term]             Z8 exponent of the CH-form phase factor
 *   coef_phase, coef_r, coef_zero: [term]  Scalar coefficient
 *                               (crates/necstar/src/state/types/scalar.rs:12-15)
 * and the global factor {re, im}.  Matches the field list of
 * StabilizerCHForm (crates/stabilizer-ch-form-rust/src/form/mod.rs:12-22);
 * ω is always 1 on every path of the reference and is not stored.          */
nsg_status nsg_export_terms(const nsg_state* state, uint8_t* G, uint8_t* F, uint8_t* M,
                            uint8_t* gamma, uint8_t* v, uint8_t* s, uint8_t* phase,
                            uint8_t* coef_phase, int32_t* coef_r, uint8_t* coef_zero,
                            double global_factor[2]);

/* Measurement helpers (no counterpart in the reference).  When enabled,
 * every pair-kernel launch is bracketed by CUDA events on its stream and
 * the elapsed time, launch count and pair count accumulate process-wide;
 * nsg_profile_read returns and resets the totals. */
nsg_status nsg_profile_enable(int32_t enabled);
nsg_status nsg_profile_read(double* pair_kernel_ms, uint64_t* launches, uint64_t* pairs);

/* Integer-pipe probe: runs a kernel of dependent-free 32-bit LOP3/XOR chains
 * on every SM for `iters` iterations and returns its duration and the number
 * of 32-bit logic operations executed (the measured peak used as the
 * roofline denominator of the integer-bound pair kernel). */
nsg_status nsg_probe_int_ops(uint64_t iters, double* seconds, uint64_t* ops);

/* Diagnostic: the exact value of every pair term ⟨S_i| P |S_j⟩ (no
 * coefficients) as k[i·χ+j] = Z8 phase (255 for a zero amplitude) and
 * r[i·χ+j] with value e^{iπk/4}·2^{-r/2}; the per-pair quantity the
 * reference computes in StabilizerCHForm::inner_product
 * (crates/stabilizer-ch-form-rust/src/form/inner_product.rs:14-48) when
 * exp_value evaluates S_i against P·S_j (exp_value.rs:38-57).  Evaluates the
 * full χ×χ square with the production pair kernel; for parity tests. */
nsg_status nsg_debug_pair_values(const nsg_state* state, const nsg_pauli* pauli,
                                 uint8_t* k, int32_t* r);

/* Diagnostic: compiles the circuit like nsg_state_from_circuit and writes,
 * per term of |T⟩^{⊗t} (in the expansion's order), keep = 1 when the term
 * survives the post-selection of the ancillas (compiler/mod.rs:108-131);
 * the compiled state's term i is the i-th kept term.  *num_t_terms is the
 * expansion's size (NSG_ERR_BUFFER_TOO_SMALL above capacity). */
nsg_status nsg_debug_compile_keep(uint32_t num_qubits, const nsg_gate* gates, size_t num_gates,
                                  uint8_t* keep, size_t capacity, uint64_t* num_t_terms);

/* A new state holding the terms indices[0..count) (strictly ascending) of
 * `state`, with their coefficients and the same global factor; for sampled
 * parity checks of large states (no reference counterpart). */
nsg_status nsg_state_select(const nsg_state* state, const uint64_t* indices, size_t count, nsg_state** out);

/* Test hook for the bounded barrier waits of the pair kernel (the waits that
 * replace a hang by NSG_ERR_TIMEOUT): poll_limit polls per wait (0 restores
 * 2^22) and, when extra_tx_bytes > 0 (≤ 1024), the barrier of the first ket
 * of every chunk expects that many bytes more than its bulk copy delivers,
 * so that wait runs out after the copy has landed and the call returns
 * NSG_ERR_TIMEOUT with no copy in flight.  Applies to launches built after
 * the call; 0, 0 restores normal operation. */
nsg_status nsg_debug_set_wait(uint32_t poll_limit, uint32_t extra_tx_bytes);

/* The device expansion of |T⟩^{⊗t} (construct_t_tensor_state,
 * crates/necstar/src/state/magic_states/t_state.rs:29-71; 1 ≤ t ≤ 64) as a
 * state of t qubits whose terms and coefficients are the expansion's, in its
 * order — for parity tests against the oracle. */
nsg_status nsg_debug_t_tensor(uint32_t t, nsg_state** out);

#ifdef __cplusplus
}
#endif

#endif /* NECSTAR_GPU_H */
