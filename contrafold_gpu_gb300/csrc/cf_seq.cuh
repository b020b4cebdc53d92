// cf_seq.cuh -- per-sequence shared-memory views, partner bit sets and the
// pairable-cell lists shared by the fold kernels.
#pragma once

#include "cf_device.cuh"

namespace cf {

// Words of one partner bit set for sequences up to Lmax (bits 0 .. Lmax+1
// plus one spare word so a funnel shift may read word w+1).
__host__ __device__ __forceinline__ int pb_words(int Lmax) { return ((Lmax + 2) >> 5) + 2; }

// Sequence view: base codes s[0..L+1] (N sentinels), pairing codes pc[0..L+1]
// (5 = forced unpaired), and for each base c in A C G U the bit set PB[c] of
// positions b whose pairing code is a canonical partner of c.  pairable(a, b)
// (canonical and neither forced, cpu.py:186,206) is bit b of PB[pc[a]].
struct SeqV {
    const int8_t* s;
    const int8_t* pc;
    const uint32_t* PB;   // [4][W]
    int W;
    int L;
    __device__ __forceinline__ bool pairable(int a, int b) const {
        const int c = pc[a];
        return c < 4 && ((PB[c * W + (b >> 5)] >> (b & 31)) & 1u);
    }
    // Bits [lo, lo + cnt) of PB[pc[a]] (cnt <= 32), bit k <-> position lo + k.
    __device__ __forceinline__ uint32_t window(int a, int lo, int cnt) const {
        const int c = pc[a];
        if (c >= 4 || cnt <= 0) return 0u;
        const uint32_t* r = PB + c * W + (lo >> 5);
        const uint32_t x = __funnelshift_r(r[0], r[1], lo & 31);
        return cnt >= 32 ? x : (x & ((1u << cnt) - 1u));
    }
};

__device__ __forceinline__ bool partner_code(int c, int x) { return (CANON6 >> (c * 6 + x)) & 1ull; }

// Build s, pc, PB for one sequence (whole CTA).  Position b of PB covers
// 0 .. L+1; higher bits are zero.
__device__ __forceinline__ void build_seq(const uint8_t* __restrict__ seqs, const uint8_t* __restrict__ mask,
                                          int64_t off, int L, int W, int8_t* s, int8_t* pc, uint32_t* PB) {
    for (int t = threadIdx.x; t < L + 2; t += blockDim.x) {
        int8_t code = 4, p = 4;
        if (t >= 1 && t <= L) {
            code = base_code(seqs[off + t - 1]);
            p = (mask != nullptr && mask[off + t - 1] != 0) ? (int8_t)5 : code;
        }
        s[t] = code;
        pc[t] = p;
    }
    __syncthreads();
    // one warp per 32-position word, four ballots (one per base)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int w = warp; w < W; w += nw) {
        const int b = w * 32 + lane;
        const int x = (b <= L + 1) ? pc[b] : 5;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const unsigned bits = __ballot_sync(0xffffffffu, partner_code(c, x));
            if (lane == 0) PB[c * W + w] = bits;
        }
    }
}

// Pairable FC cells of one sequence: (i, j) with 1 <= i <= j <= L-1 and
// pairable(i, j+1), grouped by diagonal d = j - i.  poff[d] .. poff[d+1] index
// pl[] (int16 i, ascending).  Built once by the inside kernel in the arena and
// read by the outside and posterior kernels.
struct PairList {
    int32_t* poff;   // [L + 2]
    int16_t* pl;     // [tri_size(L)]
};

// Diagonal d of list entry c (poff[d] <= c < poff[d+1]), 0 <= c < poff[L+1].
__device__ __forceinline__ int plist_diag(const PairList& P, int L, int c) {
    int lo = 0, hi = L;   // the largest d with poff[d] <= c
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (P.poff[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ PairList plist_at(float* base, int L) {
    PairList P;
    P.poff = reinterpret_cast<int32_t*>(base);
    P.pl = reinterpret_cast<int16_t*>(base + pad32(L + 3));
    return P;
}

// Whole-CTA build of the pair list (requires the sequence view).
__device__ __forceinline__ void build_plist(const SeqV& Q, PairList P) {
    const int L = Q.L;
    // count per diagonal (cells with 1 <= i, i + d <= L - 1)
    for (int d = threadIdx.x; d <= L; d += blockDim.x) {
        int cnt = 0;
        for (int i = 1; i + d <= L - 1; ++i) cnt += Q.pairable(i, i + d + 1);
        P.poff[d + 1] = cnt;
    }
    __syncthreads();
    // exclusive scan by warp 0 (chunks of 32 diagonals)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        int carry = 0;
        if (lane == 0) P.poff[0] = 0;
        for (int d0 = 1; d0 <= L + 1; d0 += 32) {
            const int d = d0 + lane;
            int v = d <= L + 1 ? P.poff[d] : 0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= o) v += y;
            }
            if (d <= L + 1) P.poff[d] = v + carry;
            carry += __shfl_sync(0xffffffffu, v, 31);
        }
    }
    __syncthreads();
    for (int d = threadIdx.x; d <= L; d += blockDim.x) {
        int o = P.poff[d];
        for (int i = 1; i + d <= L - 1; ++i)
            if (Q.pairable(i, i + d + 1)) P.pl[o++] = (int16_t)i;
    }
    __syncthreads();
}

}  // namespace cf
