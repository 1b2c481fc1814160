// noalloc.cu — nsg_exp_value_noalloc: ⟨P⟩ without any device allocation.
//
// Some callers cannot call cudaMalloc at the moment they need an expectation
// value: a host process whose device memory is already fully reserved by
// another allocator (a framework's caching allocator holding the whole GPU
// fails every further cudaMalloc), or a latency-critical loop where
// cudaMalloc/cudaFree would synchronise the device.  This entry point runs
// the kernels of nsg_exp_value (bra frames, Pauli frames, the pair sum, the
// FP64 reduction; the pair sum in its row-staged form, which needs no
// per-term tables) but takes all of their scratch from one file-scope
// device array, g_noalloc_scratch, of 16 MiB.  Every GPU that loads the
// library holds that array until the process exits.
//
// Limits: n ≤ 64 qubits (NSG_ERR_TOO_WIDE above) and χ ≤ 8192 terms (the
// frames of 8192 terms plus the pair-kernel partials fit the 16 MiB;
// NSG_ERR_BUFFER_TOO_SMALL above), checked before anything runs.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (host code cannot use the symbol itself) and
// caches it per device; make that first call before any stream capture.
// CUDA loads a library's device code lazily by default, so the 16 MiB are
// taken from the device when that first call runs (or when the module is
// loaded for another reason): a caller whose memory another allocator will
// reserve makes one call on each device before that allocator takes the
// memory (or sets CUDA_MODULE_LOADING=EAGER).  The call runs on the state's
// device and restores the caller's current device, like every other entry
// point.  All calls share the array and it keeps the previous call's
// contents: the call clears the partial sums it accumulates into, and calls
// that overlap on the GPU (two streams, two threads) race on the array.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/necstar_gpu.h"
#include "device_state.hpp"

namespace nsg {
bool state_internals(const nsg_state* s, TermsView* tv, cudaStream_t* st, int** status, int* device, double* gf2);
void set_last_error(const char* msg, int64_t a, int64_t b);
}  // namespace nsg

using namespace nsg;

namespace {

constexpr size_t kScratchBytes = 16u << 20;  // 16 MiB
constexpr int64_t kMaxTerms = 8192;
constexpr int kMaxWarps = 4096;
constexpr int kWarpsPerBlock = 4;
constexpr int kChunk = 32;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_setup_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Row-chunk offsets of the triangular pair space (one thread; χ ≤ 8192).
__global__ void noalloc_offsets_kernel(int64_t chi, int chunk, int64_t* off) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        int64_t acc = 0;
        for (int64_t i = 0; i < chi; i++) {
            off[i] = acc;
            acc += (chi - i + chunk - 1) / chunk;
        }
        off[chi] = acc;
    }
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

nsg_status fail(nsg_status code, const char* msg, int64_t a = -1, int64_t b = -1) {
    set_last_error(msg, a, b);
    return code;
}

nsg_status cuda_fail(cudaError_t e) {
    set_last_error(cudaGetErrorString(e), (int64_t)e, -1);
    return NSG_ERR_CUDA;
}

// The state's device is current for the length of the call; the caller's is restored.
struct DeviceSwitch {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceSwitch(int dev) {
        int cur = 0;
        err = cudaGetDevice(&cur);
        if (err == cudaSuccess && cur != dev) {
            err = cudaSetDevice(dev);
            if (err == cudaSuccess) prev = cur;
        }
    }
    ~DeviceSwitch() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

}  // namespace

extern "C" nsg_status nsg_exp_value_noalloc(const nsg_state* state, const nsg_pauli* pauli, double* out) {
    if (!state || !pauli || !out) return fail(NSG_ERR_INVALID_ARGUMENT, "null argument");
    TermsView tv;
    cudaStream_t st;
    int* status = nullptr;
    int sdev = 0;
    double gf2 = 1.0;
    if (!state_internals(state, &tv, &st, &status, &sdev, &gf2)) return fail(NSG_ERR_INVALID_ARGUMENT, "null state");
    const int n = tv.n;
    if (n > 64) return fail(NSG_ERR_TOO_WIDE, "nsg_exp_value_noalloc supports at most 64 qubits", n, 64);
    if (tv.chi > kMaxTerms)
        return fail(NSG_ERR_BUFFER_TOO_SMALL, "nsg_exp_value_noalloc supports at most 8192 terms", tv.chi, kMaxTerms);

    // Pauli string -> bit form, with the length checks of exp_value.rs:9-27
    // and the argument checks of nsg_exp_value.
    DevPauli dp{0, 0, 0, 0};
    if (pauli->len && !pauli->ops) return fail(NSG_ERR_INVALID_ARGUMENT, "null Pauli ops");
    if (pauli->kind == NSG_PAULI_SPARSE && pauli->len && !pauli->qubits)
        return fail(NSG_ERR_INVALID_ARGUMENT, "null Pauli qubits");
    if (pauli->kind == NSG_PAULI_DENSE) {
        if ((int)pauli->len != n) return fail(NSG_ERR_INVALID_PAULI_STRING_LENGTH, "Invalid Pauli string length.", n, pauli->len);
    } else if (pauli->kind == NSG_PAULI_SPARSE) {
        uint32_t maxq = 0;
        for (uint32_t i = 0; i < pauli->len; i++) maxq = maxq > pauli->qubits[i] ? maxq : pauli->qubits[i];
        if ((int64_t)maxq >= n) return fail(NSG_ERR_INVALID_PAULI_STRING_LENGTH, "Invalid Pauli string length.", n, maxq + 1);
    } else {
        return fail(NSG_ERR_INVALID_ARGUMENT, "invalid Pauli kind", pauli->kind);
    }
    int e = 0;
    for (uint32_t i = 0; i < pauli->len; i++) {
        uint32_t q = pauli->kind == NSG_PAULI_DENSE ? i : pauli->qubits[i];
        uint64_t bit = 1ULL << q;
        int xq = (int)((dp.px >> q) & 1);
        switch (pauli->ops[i]) {
            case NSG_PAULI_I: break;
            case NSG_PAULI_X: dp.px ^= bit; break;
            case NSG_PAULI_Z: e += 2 * xq; dp.pz ^= bit; break;
            case NSG_PAULI_Y: e += 1 + 2 * xq; dp.px ^= bit; dp.pz ^= bit; break;
            default: return fail(NSG_ERR_INVALID_ARGUMENT, "invalid Pauli op", pauli->ops[i]);
        }
    }
    dp.ny = e & 3;

    const int dev = sdev;
    if (dev < 0 || dev >= kMaxDevices) return fail(NSG_ERR_INVALID_ARGUMENT, "device index too large", dev);
    DeviceSwitch on_dev(dev);
    cudaError_t ce = on_dev.err;
    if (ce != cudaSuccess) return cuda_fail(ce);
    unsigned char* base;
    {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (ce != cudaSuccess) return cuda_fail(ce);
            g_scratch_ptr[dev] = (unsigned char*)p;
        }
        base = g_scratch_ptr[dev];
    }
    if (tv.chi == 0) {
        *out = 0.0;
        return NSG_OK;
    }

    // Carve the scratch.
    const size_t chi = (size_t)tv.chi;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        unsigned char* p = base + off;
        off += align256(bytes);
        return p;
    };
    FrameView fr;
    fr.GV = (uint64_t*)take(chi * 64 * 8);
    fr.FV = (uint64_t*)take(chi * 64 * 8);
    fr.MV = (uint64_t*)take(chi * 64 * 8);
    fr.GVL = (uint64_t*)take(chi * 8);
    fr.GVH = (uint64_t*)take(chi * 8);
    uint64_t* px = (uint64_t*)take(chi * 8);
    uint8_t* pk = (uint8_t*)take(chi);
    DevPauli* dpp = (DevPauli*)take(sizeof(DevPauli));
    int64_t* offs = (int64_t*)take((chi + 1) * 8);
    double* partials = (double*)take((size_t)kMaxWarps * 8 * sizeof(double));
    double* dout = (double*)take(2 * sizeof(double));
    if (off > kScratchBytes) return fail(NSG_ERR_BUFFER_TOO_SMALL, "scratch layout exceeds 16 MiB", (int64_t)off);

    int64_t total_chunks = 0;
    for (size_t i = 0; i < chi; i++) total_chunks += (int64_t)((chi - i + kChunk - 1) / kChunk);
    int sms = device_sm_count();
    int64_t want = (total_chunks + kWarpsPerBlock - 1) / kWarpsPerBlock;
    int64_t cap = (int64_t)sms * 16 < kMaxWarps / kWarpsPerBlock ? (int64_t)sms * 16 : kMaxWarps / kWarpsPerBlock;
    int blocks = (int)(want < cap ? (want > 0 ? want : 1) : cap);

    PairLaunch pl;
    pl.A = tv;
    pl.fr = fr;
    pl.B = tv;
    pl.px = px;
    pl.pk = pk;
    pl.nobs = 1;
    pl.triangular = true;
    pl.complex_out = false;
    pl.mixed = false;
    pl.chunk = kChunk;
    pl.total_chunks = total_chunks;
    pl.row_chunk_off = offs;
    pl.blocks = blocks;
    pl.warps_per_block = kWarpsPerBlock;
    pl.nwarps = blocks * kWarpsPerBlock;
    pl.partials = partials;
    pl.status = status;

    if ((ce = cudaMemcpyAsync(dpp, &dp, sizeof(dp), cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_fail(ce);
    if ((ce = cudaMemsetAsync(partials, 0, (size_t)pl.nwarps * 8 * sizeof(double), st)) != cudaSuccess)
        return cuda_fail(ce);
    noalloc_offsets_kernel<<<1, 32, 0, st>>>((int64_t)chi, kChunk, offs);
    if ((ce = cudaGetLastError()) != cudaSuccess) return cuda_fail(ce);
    if ((ce = launch_frames(tv, fr, st)) != cudaSuccess) return cuda_fail(ce);
    if ((ce = launch_pauli_frames(tv, dpp, 1, px, pk, st)) != cudaSuccess) return cuda_fail(ce);
    if ((ce = launch_pairs_rows(pl, st)) != cudaSuccess) return cuda_fail(ce);
    if ((ce = launch_reduce(partials, pl.nwarps, 1, false, gf2, 0.0, dout, st)) != cudaSuccess) return cuda_fail(ce);
    double h = 0.0;
    int hs[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // the state's status words (bits, detail claimed, detail)
    if ((ce = cudaMemcpyAsync(&h, dout, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_fail(ce);
    if ((ce = cudaMemcpyAsync(hs, status, sizeof(hs), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_fail(ce);
    if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(ce);
    if (hs[0]) {
        if ((ce = cudaMemsetAsync(status, 0, sizeof(hs), st)) != cudaSuccess) return cuda_fail(ce);
        if ((ce = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(ce);
        if (hs[0] & DS_TIMEOUT) return fail(NSG_ERR_TIMEOUT, "a bounded device wait ran out", hs[0]);
        if (hs[0] & DS_CANNOT_DISCARD) return fail(NSG_ERR_CANNOT_DISCARD_QUBIT, "cannot discard qubit", hs[0]);
        return fail(NSG_ERR_DEVICE_INVARIANT, "device invariant violated", hs[0], hs[2]);
    }
    *out = h;
    return NSG_OK;
}
