// cf_sample.cu -- standalone sampler kernel over inside tables already in the
// arena (one warp per (sequence, sample) work item).  The traceback itself is
// in cf_sample.cuh.
#include "cf_sample.cuh"
#include "cf_sample.h"

namespace cf {

constexpr int kSampleWarps = 8;   // warps per CTA

struct SampleSmem {
    SmemTabs<float> tabs;
};

// Per-warp scratch: codes s[L+2], pc[L+2], packed stack[L+8].
__host__ __device__ __forceinline__ int sample_region_bytes(int Lmax) {
    const int codes = ((Lmax + 2 + 15) & ~15) * 2;
    return codes + 4 * (Lmax + 8);
}

__global__ void __launch_bounds__(kSampleWarps * 32) k_sample32(SampleArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SampleSmem*>(smem_raw);
    load_tabs(&sm->tabs, A.blob32);
    __syncthreads();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int region = sample_region_bytes(A.Lmax);
    unsigned char* mine = smem_raw + sizeof(SampleSmem) + (size_t)wib * region;
    const int cstride = (A.Lmax + 2 + 15) & ~15;
    int8_t* s = reinterpret_cast<int8_t*>(mine);
    int8_t* pc = s + cstride;
    uint32_t* stack = reinterpret_cast<uint32_t*>(mine + 2 * cstride);
    const int64_t n_items = (int64_t)A.n * A.n_samples;
    const int64_t gw = (int64_t)blockIdx.x * kSampleWarps + wib;
    const int64_t nw = (int64_t)gridDim.x * kSampleWarps;
    const uint2 key = make_uint2((uint32_t)A.seed, (uint32_t)(A.seed >> 32));

    for (int64_t item = gw; item < n_items; item += nw) {
        const int b = (int)(item / A.n_samples), smp = (int)(item % A.n_samples);
        const SeqDesc D = A.descs[b];
        const int L = D.L;
        for (int t = lane; t < L + 2; t += 32) {
            int8_t code = 4, p = 4;
            if (t >= 1 && t <= L) {
                code = base_code(A.seqs[D.seq_off + t - 1]);
                p = (A.mask != nullptr && A.mask[D.seq_off + t - 1] != 0) ? (int8_t)5 : code;
            }
            s[t] = code;
            pc[t] = p;
        }
        char* out = A.out + D.seq_off * (int64_t)A.n_samples + (int64_t)smp * L;
        for (int t = lane; t < L; t += 32) out[t] = '.';
        __syncwarp();
        SampleCtx<SeqView> X;
        X.tb = &sm->tabs;
        X.Q = SeqView{s, pc, L};
        const Arena32 ar = arena32(L);
        float* base = A.ws + D.ws_off;
        X.T.FC = base + ar.FC; X.T.FM = base + ar.FM; X.T.FM1 = base + ar.FM1; X.T.F5 = base + ar.F5;
        X.T.m = L + 1;
        X.T.sized(L);
        const int sidx = A.stream_idx != nullptr ? A.stream_idx[D.idx] : (A.seeds != nullptr ? 0 : D.idx);
        if (A.seeds != nullptr) {
            const uint64_t sd = A.seeds[D.idx];
            sample_one(X, smp, sidx, make_uint2((uint32_t)sd, (uint32_t)(sd >> 32)), out, stack, A.status, lane);
        } else {
            sample_one(X, smp, sidx, key, out, stack, A.status, lane);
        }
        __syncwarp();
    }
}

size_t sample_smem_bytes(int Lmax) { return sizeof(SampleSmem) + (size_t)kSampleWarps * sample_region_bytes(Lmax); }
int sample_threads() { return kSampleWarps * 32; }

}  // namespace cf
