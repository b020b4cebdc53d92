// cf_warp.cu -- the batched path: one persistent kernel in which every WARP
// folds whole sequences, pulled from a device work queue.
//
// A warp runs the complete pipeline of one sequence -- inside (pipelined
// two-phase diagonals), F5, then for MEA / BPP the outside, the posterior and
// the gamma-weighted decode with traceback, or for sampling the stochastic
// tracebacks -- synchronising only with __syncwarp.  Sequences do not wait on
// each other, so a CTA has no block-wide barriers after set-up: the 8 warps
// of a CTA (and the 32+ warps of an SM) are independent instruction streams
// that hide each other's log-sum-exp latency.  The host sorts the batch by
// length (longest first) so the queue hands out the expensive folds early.
//
// Per-cell arithmetic is shared with the per-sequence CTA kernels
// (cf_inside.cuh, cf_outside.cuh, cf_mea.cuh, cf_sample.cuh): results are
// identical, bit for bit.
// This module runs one sequence per warp: 32+ independent warps per SM hide
// memory latency, so the chains use plain loops (no register pipelines) and a
// small register budget keeps the SM full.
#ifndef CF_CHAIN_PF
#define CF_CHAIN_PF 0
#endif
// bifurcation-chain operands arrive through a CF_CHAIN_ASYNC-deep cp.async
// ring in shared memory (hides DRAM latency without prefetch registers).
// Depth 4 measured best on GB300 (4: 25.3k, 6: 25.2k, 8: 23.7k 200-nt MEA
// folds/s): a shallower ring leaves more of the SM's L1 / shared carve-out to L1.
#ifndef CF_CHAIN_ASYNC
#define CF_CHAIN_ASYNC 4
#endif
#define CF_CHAIN_THREADS 256
#ifndef CF_WARP_MIN_BLOCKS
#define CF_WARP_MIN_BLOCKS 4
#endif
#include "cf_mea.cuh"
#include "cf_outside.cuh"
#include "cf_sample.cuh"
#include "cf_warp.h"

namespace cf {

struct WarpSmemHead {
    SmemTabs<float> tabs;
    PolyTables poly;
};

// Per-warp region: s, pc (code stride each), PB (4 x W words), stack (Lmax + 8 words).
__host__ __device__ __forceinline__ int warp_region_bytes(int Lmax) {
    const int cs = (Lmax + 2 + 15) & ~15;
    return 2 * cs + 4 * 4 * pb_words(Lmax) + 4 * (Lmax + 8);
}

__device__ __forceinline__ void build_seq_warp(const uint8_t* __restrict__ seqs, const uint8_t* __restrict__ mask,
                                               int64_t off, int L, int W, int8_t* s, int8_t* pc, uint32_t* PB,
                                               int lane) {
    for (int t = lane; t < L + 2; t += 32) {
        int8_t code = 4, p = 4;
        if (t >= 1 && t <= L) {
            code = base_code(seqs[off + t - 1]);
            p = (mask != nullptr && mask[off + t - 1] != 0) ? (int8_t)5 : code;
        }
        s[t] = code;
        pc[t] = p;
    }
    __syncwarp();
    for (int w = 0; w < W; ++w) {
        const int b = w * 32 + lane;
        const int x = (b <= L + 1) ? pc[b] : 5;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const unsigned bits = __ballot_sync(0xffffffffu, partner_code(c, x));
            if (lane == 0) PB[c * W + w] = bits;
        }
    }
    __syncwarp();
}

// Pairable FC cells grouped by diagonal (see cf_seq.cuh), built by one warp.
__device__ __forceinline__ void build_plist_warp(const SeqV& Q, PairList P, int lane) {
    const int L = Q.L;
    const unsigned below = (1u << lane) - 1u;
    int o = 0;
    for (int d = 0; d <= L; ++d) {
        if (lane == 0) P.poff[d] = o;
        for (int i0 = 1; i0 + d <= L - 1; i0 += 32) {
            const int i = i0 + lane;
            const bool ok = (i + d <= L - 1) && Q.pairable(i, i + d + 1);
            const unsigned mk = __ballot_sync(0xffffffffu, ok);
            if (ok) P.pl[o + __popc(mk & below)] = (int16_t)i;
            o += __popc(mk);
        }
    }
    if (lane == 0) P.poff[L + 1] = o;
    __syncwarp();
}

template <int MODE>
__device__ __forceinline__ void fold_one(const WarpArgs& A, const WarpSmemHead* sm, const SeqDesc& D, const SeqV& Q,
                                         float* base, uint32_t* stack, int lane) {
    const int L = Q.L, m = L + 1;
    const Arena32 ar = arena32(L);
    InTabs<float> T;
    T.FC = base + ar.FC; T.FM = base + ar.FM; T.FM1 = base + ar.FM1; T.F5 = base + ar.F5; T.m = m;
    T.sized(L);
    float* FB = base + ar.FB;
    const int fbs = (int)pad32(L + 2);
    const PairList PLs = plist_at(base + ar.PL, L);
    build_plist_warp(Q, PLs, lane);

    // ---------------- inside: A(t) and B(t-1) per step ----------------
    auto inside = [&](auto sr) {
        using S = decltype(sr);
        for (int t = 0; t <= L + 1; ++t) {
            const int dB = t - 1;
            if (dB >= 0 && dB <= L - 2) {
                const int o = PLs.poff[dB], cnt = PLs.poff[dB + 1] - o;
                for (int k0 = 0; k0 < cnt; k0 += 32) {
                    const int k = k0 + lane;
                    const unsigned lanes = __ballot_sync(0xffffffffu, k < cnt);
                    if (k >= cnt) continue;
                    const int i = PLs.pl[o + k];
                    inside_B<S>(sr, &sm->tabs, Q, T, i, i + dB, FB[(dB & 1) * fbs + i], lanes);
                }
            }
            if (t <= L)
                for (int i = lane; i <= L - t; i += 32) FB[(t & 1) * fbs + i] = inside_A<S>(sr, &sm->tabs, Q, T, i, i + t);
            __syncwarp();
        }
        exterior_warp<S>(sr, &sm->tabs, Q, T);
    };
    if constexpr (MODE == kWarpLogZ || MODE == kWarpSample) inside(LseAcc32{});
    else inside(Lse32{&sm->poly});

    if constexpr (MODE == kWarpLogZ) {
        if (lane == 0) A.logz[D.idx] = T.F5[L];
        return;
    }
    if constexpr (MODE == kWarpSample) {
        SampleCtx<SeqV> X;
        X.tb = &sm->tabs;
        X.Q = Q;
        X.T = T;
        const uint64_t sd = A.seeds != nullptr ? A.seeds[D.idx] : A.seed;
        const uint2 key = make_uint2((uint32_t)sd, (uint32_t)(sd >> 32));
        const int sidx = A.stream_idx != nullptr ? A.stream_idx[D.idx] : (A.seeds != nullptr ? 0 : D.idx);
        for (int smp = 0; smp < A.n_samples; ++smp) {
            char* out = A.out + D.seq_off * (int64_t)A.n_samples + (int64_t)smp * L;
            for (int t = lane; t < L; t += 32) out[t] = '.';
            __syncwarp();
            sample_one(X, smp, sidx, key, out, stack, A.status, lane);
            __syncwarp();
        }
        if (A.logz != nullptr && lane == 0) A.logz[D.idx] = T.F5[L];
        return;
    }

    // ---------------- outside: A(t) and B(t-1) per step, t descending ----------------
    const Lse32 sr{&sm->poly};
    OutTabs O;
    O.FC = T.FC; O.FM = T.FM; O.FM1 = T.FM1; O.F5 = T.F5;
    O.FCo = base + ar.FCo; O.FMo = base + ar.FMo; O.FM1o = base + ar.FM1o; O.FM2o = base + ar.FM2o;
    O.F5o = base + ar.F5o; O.m = m;
    O.sized(L);
    exterior_outside_warp(sr, &sm->tabs, Q, O);
    for (int t = L; t >= 0; --t) {
        const int dB = t - 1;
        if (dB >= 0 && dB <= L - 2) {
            const int o = PLs.poff[dB], cnt = PLs.poff[dB + 1] - o;
            for (int k0 = 0; k0 < cnt; k0 += 32) {
                const int k = k0 + lane;
                const unsigned lanes = __ballot_sync(0xffffffffu, k < cnt);
                if (k >= cnt) continue;
                const int a = PLs.pl[o + k];
                outside_B(sr, &sm->tabs, Q, O, a, a + dB, lanes);
            }
        }
        for (int a = lane; a <= L - t; a += 32) outside_A_merged(sr, &sm->tabs, Q, O, a, a + t);
        __syncwarp();
    }

    // ---------------- posterior into the FMo slot ----------------
    float* POST = O.FMo;
    const float Z = T.F5[L];
    const int64_t tot = tri_size(L);
    for (int64_t c = lane; c < tot; c += 32) POST[c] = 0.0f;
    float* dense = (MODE == kWarpBpp) ? A.post_out + A.post_offs[D.idx] : nullptr;
    if (dense != nullptr)
        for (int64_t c = lane; c < (int64_t)L * L; c += 32) dense[c] = 0.0f;
    __syncwarp();
    const int total = PLs.poff[L + 1];
    for (int c0 = 0; c0 < total; c0 += 32) {
        const int c = c0 + lane;
        const unsigned lanes = __ballot_sync(0xffffffffu, c < total);
        if (c >= total) continue;
        const int d = plist_diag(PLs, L, c);
        const int a = PLs.pl[c], b = a + d + 1;
        const float v = posterior_pair(&sm->tabs, &sm->poly, Q, O, Z, a, b, lanes);
        POST[tri_off(d + 1, m) + a] = v;
        if (dense != nullptr) dense[(int64_t)(a - 1) * L + (b - 1)] = v;
    }
    __syncwarp();
    if constexpr (MODE == kWarpBpp) {
        if (A.logz != nullptr && lane == 0) A.logz[D.idx] = Z;
        return;
    }

    // ---------------- MEA decode ----------------
    float* up = base + ar.up;
    float* score = O.FM2o;
    int* tbk = reinterpret_cast<int*>(base + ar.FM);
    const float two_g = __fmul_rn(2.0f, A.gamma);
    for (int i = 1 + lane; i <= L; i += 32) up[i] = mea_unpaired(POST, L, two_g, i);
    __syncwarp();
    for (int d = 0; d <= L; ++d) {
        for (int i = lane; i <= L - d; i += 32) mea_cell(Q, POST, up, score, tbk, L, i, i + d);
        __syncwarp();
    }
    char* out = A.structs + D.seq_off;
    for (int t = lane; t < L; t += 32) out[t] = '.';
    __syncwarp();
    if (lane == 0) {
        int* qi = reinterpret_cast<int*>(base + ar.queue);
        mea_traceback(tbk, L, qi, qi + 2 * L + 4, out, A.status);
    }
    __syncwarp();
}

template <int MODE>
__global__ void __launch_bounds__(kWarpThreads, CF_WARP_MIN_BLOCKS) k_fold_warp(WarpArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<WarpSmemHead*>(smem_raw);
    load_tabs(&sm->tabs, A.blob32);
    load_poly_tables(&sm->poly);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int W = pb_words(A.Lmax);
    const int cs = (A.Lmax + 2 + 15) & ~15;
    unsigned char* mine = smem_raw + sizeof(WarpSmemHead) + (size_t)wib * warp_region_bytes(A.Lmax);
    int8_t* s = reinterpret_cast<int8_t*>(mine);
    int8_t* pc = s + cs;
    uint32_t* PB = reinterpret_cast<uint32_t*>(mine + 2 * cs);
    uint32_t* stack = PB + 4 * W;
    const int64_t slot = (int64_t)blockIdx.x * (kWarpThreads / 32) + wib;
    float* base = A.ws + slot * A.slot_words;
    for (;;) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= A.n) break;
        const SeqDesc D = A.descs[item];
        build_seq_warp(A.seqs, A.mask, D.seq_off, D.L, W, s, pc, PB, lane);
        const SeqV Q{s, pc, PB, W, D.L};
        fold_one<MODE>(A, sm, D, Q, base, stack, lane);
        __syncwarp();
    }
}

template __global__ void k_fold_warp<kWarpLogZ>(WarpArgs);
template __global__ void k_fold_warp<kWarpMea>(WarpArgs);
template __global__ void k_fold_warp<kWarpBpp>(WarpArgs);
template __global__ void k_fold_warp<kWarpSample>(WarpArgs);

size_t warp_smem_bytes(int Lmax) {
    return sizeof(WarpSmemHead) + (size_t)(kWarpThreads / 32) * warp_region_bytes(Lmax);
}

int64_t warp_slot_words(int Lmax) { return arena32(Lmax).total; }

const void* warp_kernel(int mode) {
    switch (mode) {
        case kWarpLogZ: return (const void*)k_fold_warp<kWarpLogZ>;
        case kWarpMea: return (const void*)k_fold_warp<kWarpMea>;
        case kWarpBpp: return (const void*)k_fold_warp<kWarpBpp>;
        default: return (const void*)k_fold_warp<kWarpSample>;
    }
}

}  // namespace cf
