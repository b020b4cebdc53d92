// cf_noalloc.cu -- cf_mea_scratch: MEA folding that allocates no device memory.
//
// Who needs it.  cf_mea grows its engine's device buffers (inputs, outputs,
// descriptors, the fold arena) with cudaMalloc whenever a batch is larger
// than any before it, and frees the old ones with cudaFree.  Two kinds of
// caller cannot accept that: a process whose framework allocator has already
// reserved nearly all device memory, where a fresh cudaMalloc fails although
// the fold itself needs little; and a latency-bound serving loop, where
// cudaFree waits for the whole device and stalls every other stream.  This
// entry point instead works inside one fixed array in device global memory,
// reserved by the CUDA driver when this module is loaded.
//
// What it runs.  The MEA mode of the persistent warp-per-sequence kernel
// (cf_warp.cu), the same code cf_mea's batched path launches for short
// sequences, so the dot-brackets are identical to cf_mea's.  The number of
// warp slots (one fold arena each) is whatever fits in the scratch after the
// inputs and outputs, so throughput is lower than cf_mea's on large batches.
//
// Limits.  A batch is rejected with CF_EINVAL when its inputs, outputs and
// one CTA's worth of fold slots (8 slots sized for the longest sequence) do
// not fit in CF_SCRATCH_BYTES, or when its longest sequence is above the warp
// kernel's limit (1024 nt).  With the 64 MiB scratch one CTA of slots fits
// for longest sequences up to about 740 nt; the inputs and outputs take 2
// bytes per nucleotide (3 with a mask) plus 32 bytes per sequence.
//
// What starts at zero.  The kernel's status word and its work-queue head (the
// first two ints of the scratch) must be zero at launch; the call clears them
// with cudaMemsetAsync on its stream before every launch.  Nothing else needs
// clearing: every table cell, descriptor and output byte is written before it
// is read.
//
// Concurrency.  There is one scratch per device per process, so two calls
// that overlapped in time on one device would race on it.  Calls are
// therefore serialised by a process-wide lock, held until the call's stream
// has drained; a call never returns with work still running in the scratch.
//
// Set-up.  The first call on each device (with that device current) resolves
// the scratch's device address with cudaGetSymbolAddress, which also makes the
// CUDA driver load this module if it is loaded lazily.  Make that first call before
// any stream capture begins.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/contrafold_gb300.h"
#include "cf_host.h"
#include "cf_warp.h"

static_assert(CF_SCRATCH_BYTES % 256 == 0, "scratch size must keep 256-byte alignment");

// The scratch: inputs, descriptors, outputs and fold arenas of one call.
static __device__ __align__(256) unsigned char g_cf_scratch[CF_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
constexpr int kSlotsPerCta = cf::kWarpThreads / 32;

std::mutex g_lock;
unsigned char* g_addr[kMaxDevices] = {};   // scratch address per device, resolved once

size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte offsets of one call's regions inside the scratch.
struct Layout {
    size_t status = 0;    // int[2]: status word, work-queue head
    size_t offs = 0;      // int64[n + 1]
    size_t descs = 0;     // SeqDesc[n]
    size_t seqs = 0;      // nbytes
    size_t mask = 0;      // nbytes (only when a mask is given)
    size_t structs = 0;   // nbytes
    size_t arena = 0;     // fold slots, slot_bytes each
    size_t slot_bytes = 0;
    int64_t slots = 0;    // how many fit
};

Layout layout_for(int n, size_t nbytes, bool has_mask, int Lmax) {
    Layout Y;
    Y.status = 0;
    Y.offs = 256;
    Y.descs = Y.offs + up256(sizeof(int64_t) * ((size_t)n + 1));
    Y.seqs = Y.descs + up256(sizeof(cf::SeqDesc) * (size_t)n);
    Y.mask = Y.seqs + up256(nbytes);
    Y.structs = Y.mask + (has_mask ? up256(nbytes) : 0);
    Y.arena = Y.structs + up256(nbytes);
    Y.slot_bytes = sizeof(float) * (size_t)cf::warp_slot_words(Lmax);
    Y.slots = Y.arena < CF_SCRATCH_BYTES ? (int64_t)((CF_SCRATCH_BYTES - Y.arena) / Y.slot_bytes) : 0;
    return Y;
}

__global__ void k_scratch_descs(const int64_t* __restrict__ offs, int n, cf::SeqDesc* __restrict__ descs) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    cf::SeqDesc D;
    D.seq_off = offs[b];
    D.ws_off = 0;
    D.L = (int32_t)(offs[b + 1] - offs[b]);
    D.idx = b;
    descs[b] = D;
}

#define CF_CUDA_S(call)                                                                   \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            char m_[256];                                                                 \
            std::snprintf(m_, sizeof m_, "%s: %s", #call, cudaGetErrorString(e_));        \
            return cf::engine_fail(CF_ECUDA, m_);                                         \
        }                                                                                 \
    } while (0)

// The same for calls made once work is queued on `st`: the stream is drained
// (its own error ignored) before the failure is returned, so the lock is
// released only when nothing of this call can still write the scratch.
#define CF_CUDA_Q(call)                                                                   \
    do {                                                                                  \
        cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) {                                                          \
            char m_[256];                                                                 \
            std::snprintf(m_, sizeof m_, "%s: %s", #call, cudaGetErrorString(e_));        \
            (void)cudaStreamSynchronize(st);                                              \
            return cf::engine_fail(CF_ECUDA, m_);                                         \
        }                                                                                 \
    } while (0)

}  // namespace

extern "C" int cf_mea_scratch(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask,
                              int32_t n, float gamma, char* struct_out) {
    // ---- the same argument checks as cf_mea, all on the host ----
    if (!e) return cf::engine_fail(CF_EINVAL, "engine is NULL");
    if (n < 0) return cf::engine_fail(CF_EINVAL, "negative batch size");
    if (n > 0 && !struct_out) return cf::engine_fail(CF_EINVAL, "struct_out is NULL");
    if (!(gamma > 0.0f)) return cf::engine_fail(CF_EINVAL, "gamma must be > 0");
    if (n > 0 && !offsets) return cf::engine_fail(CF_EINVAL, "offsets is NULL");
    if (n > 0 && offsets[0] != 0) return cf::engine_fail(CF_EINVAL, "offsets[0] must be 0");
    int Lmax = 0;
    for (int b = 0; b < n; ++b) {
        const int64_t L = offsets[b + 1] - offsets[b];
        if (L < 0) return cf::engine_fail(CF_EINVAL, "offsets must be non-decreasing");
        if (L > CF_MAX_LEN) return cf::engine_fail(CF_EINVAL, "sequence longer than CF_MAX_LEN");
        if (L > Lmax) Lmax = (int)L;
    }
    if (n > 0 && offsets[n] > 0 && !seqs) return cf::engine_fail(CF_EINVAL, "seqs is NULL");
    if (n == 0) return CF_OK;
    if (Lmax > cf::kWarpMaxLen) {
        char m[160];
        std::snprintf(m, sizeof m, "cf_mea_scratch: longest sequence is %d nt, the limit is %d nt", Lmax,
                      cf::kWarpMaxLen);
        return cf::engine_fail(CF_EINVAL, m);
    }
    const size_t nbytes = (size_t)offsets[n];
    const Layout Y = layout_for(n, nbytes, mask != nullptr, Lmax);
    if (Y.slots < kSlotsPerCta) {
        char m[256];
        std::snprintf(m, sizeof m,
                      "cf_mea_scratch: batch needs %zu bytes of scratch (inputs, outputs and %d fold slots of "
                      "%zu bytes for its %d-nt longest sequence); the static scratch holds %zu bytes",
                      Y.arena + kSlotsPerCta * Y.slot_bytes, kSlotsPerCta, Y.slot_bytes, Lmax,
                      (size_t)CF_SCRATCH_BYTES);
        return cf::engine_fail(CF_EINVAL, m);
    }

    std::lock_guard<std::mutex> guard(g_lock);
    const int dev = cf::engine_device(e);
    if (dev < 0 || dev >= kMaxDevices) return cf::engine_fail(CF_EINVAL, "cf_mea_scratch: device index out of range");
    CF_CUDA_S(cudaSetDevice(dev));
    if (g_addr[dev] == nullptr) {   // set-up, once per device
        void* p = nullptr;
        CF_CUDA_S(cudaGetSymbolAddress(&p, g_cf_scratch));
        g_addr[dev] = static_cast<unsigned char*>(p);
    }
    unsigned char* S = g_addr[dev];
    const cudaStream_t st = cf::engine_stream(e);

    const int mode = cf::kWarpMea;
    const size_t smem = cf::warp_smem_bytes(Lmax);
    int rc = cf::engine_ensure_smem(e, smem);
    if (rc) return rc;
    int per_sm = 0, sms = 0;
    CF_CUDA_S(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cf::warp_kernel(mode), cf::kWarpThreads, smem));
    CF_CUDA_S(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int64_t grid = (int64_t)(per_sm > 0 ? per_sm : 1) * sms;
    if (grid > Y.slots / kSlotsPerCta) grid = Y.slots / kSlotsPerCta;
    if (grid > (n + kSlotsPerCta - 1) / kSlotsPerCta) grid = (n + kSlotsPerCta - 1) / kSlotsPerCta;

    int* status = reinterpret_cast<int*>(S + Y.status);
    int64_t* d_offs = reinterpret_cast<int64_t*>(S + Y.offs);
    cf::SeqDesc* d_descs = reinterpret_cast<cf::SeqDesc*>(S + Y.descs);
    uint8_t* d_seqs = S + Y.seqs;
    uint8_t* d_mask = mask ? S + Y.mask : nullptr;
    char* d_structs = reinterpret_cast<char*>(S + Y.structs);

    CF_CUDA_Q(cudaMemsetAsync(status, 0, 2 * sizeof(int), st));
    CF_CUDA_Q(cudaMemcpyAsync(d_offs, offsets, sizeof(int64_t) * ((size_t)n + 1), cudaMemcpyHostToDevice, st));
    if (nbytes) CF_CUDA_Q(cudaMemcpyAsync(d_seqs, seqs, nbytes, cudaMemcpyHostToDevice, st));
    if (mask && nbytes) CF_CUDA_Q(cudaMemcpyAsync(d_mask, mask, nbytes, cudaMemcpyHostToDevice, st));
    k_scratch_descs<<<(n + 255) / 256, 256, 0, st>>>(d_offs, n, d_descs);
    CF_CUDA_Q(cudaGetLastError());

    cf::WarpArgs W;
    W.descs = d_descs;
    W.n = n;
    W.Lmax = Lmax;
    W.seqs = d_seqs;
    W.mask = d_mask;
    W.blob32 = cf::engine_blob32(e);
    W.ws = reinterpret_cast<float*>(S + Y.arena);
    W.slot_words = (int64_t)(Y.slot_bytes / sizeof(float));
    W.counter = status + 1;
    W.gamma = gamma;
    W.logz = nullptr;
    W.structs = d_structs;
    W.post_out = nullptr;
    W.post_offs = nullptr;
    W.n_samples = 0;
    W.seed = 0;
    W.seeds = nullptr;
    W.stream_idx = nullptr;
    W.out = nullptr;
    W.status = status;
    void* args[] = {&W};
    {
        const cudaError_t le = cudaLaunchKernel(cf::warp_kernel(mode), dim3((unsigned)grid), dim3(cf::kWarpThreads),
                                                args, smem, st);
        if (le != cudaSuccess) {   // report the launch shape with the error
            cudaFuncAttributes fa{};
            cudaFuncGetAttributes(&fa, cf::warp_kernel(mode));
            char m[320];
            std::snprintf(m, sizeof m,
                          "cf_mea_scratch: launch of %lld CTAs with %zu bytes of dynamic shared memory failed: %s "
                          "(kernel: %zu bytes static, %d allowed dynamic, %d registers)",
                          (long long)grid, smem, cudaGetErrorString(le), fa.sharedSizeBytes,
                          fa.maxDynamicSharedSizeBytes, fa.numRegs);
            (void)cudaStreamSynchronize(st);
            return cf::engine_fail(CF_ECUDA, m);
        }
    }

    int h = 0;
    if (nbytes) CF_CUDA_Q(cudaMemcpyAsync(struct_out, d_structs, nbytes, cudaMemcpyDeviceToHost, st));
    CF_CUDA_Q(cudaMemcpyAsync(&h, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CF_CUDA_Q(cudaStreamSynchronize(st));
    if (h != CF_OK) return cf::engine_fail(h, "a kernel reported an internal limit (traceback stack/queue)");
    return CF_OK;
}
