// cf_device.cuh -- device-side building blocks shared by the fold kernels.
//
// Arithmetic contract: the FP32 paths must reproduce, bit for bit, the
// reference's float32 CPU engine (gpu_contrafold/cpu.py:527-820), so every
// add and multiply below is an explicitly rounded __fadd_rn / __fmul_rn (no
// contraction into FMA, whatever the compiler flags), and every accumulation
// runs in the reference's order.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#ifdef CF_CHECK
#include <cstdio>
#endif

#include "../../include/contrafold_gb300.h"

namespace cf {

// Sentinels of the reference (cpu.py:21-22, 523-524): float32(-1e30), float32(-5e29).
#define CF_NEG32 ((float)-1e30)
#define CF_HALF32 ((float)-5e29)
#define CF_NEG64 (-1e30)
#define CF_HALF64 (-5e29)
constexpr int CMAX = 30;   // C_MAX_SINGLE (cpu.py:31)
constexpr int DHP = 30;    // D_HAIRPIN (cpu.py:32)

// ---------------------------------------------------------------------------
// Per-sequence descriptor and work-arena layout.
// Triangular, diagonal-major tables: cell (i, j), 0 <= i <= j <= L, lives at
// tri_off(j - i) + i with m = L + 1.  Consecutive i on one diagonal are
// contiguous, so a warp working on one diagonal reads rows (FM1[i, i+s]) and
// columns (FM[j-s, j]) of the DP with unit stride across lanes.
// ---------------------------------------------------------------------------
struct SeqDesc {
    int64_t seq_off;   // offset of the sequence in the ASCII / mask buffers
    int64_t ws_off;    // offset (in 4-byte words) of the sequence's arena slice
    int32_t L;         // length
    int32_t idx;       // position in the caller's batch
};

__host__ __device__ __forceinline__ int64_t tri_size(int L) {
    const int64_t m = L + 1;
    return m * (m + 1) / 2;
}
// d * (d - 1) is never negative (d and d - 1 share a sign or one is 0) and
// below 2^31 for d <= 32,768, so the halving is a shift (no signed-division
// rounding fix-up).
__host__ __device__ __forceinline__ int tri_off(int d, int m) { return d * m - ((d * (d - 1)) >> 1); }

// ---------------------------------------------------------------------------
// Checked table access (debug builds: -DCF_CHECK, build.py --check).  The DP
// table pointers of the views (InTabs, OutTabs) become TabPtr, whose
// subscript and offset check the cell index against the table's size (set by
// the views' sized(L)); an index outside it is reported with printf (the first
// 16 per module) and replaced by 0, so the access stays inside the table and
// the kernel goes on -- no trap, no fault.  In normal builds CF_TAB(R) is R*
// and sized() is empty: the generated code is unchanged.
// ---------------------------------------------------------------------------
#ifdef CF_CHECK
static __device__ unsigned cf_check_hits;   // violations seen by this module's kernels

__device__ __forceinline__ int64_t cf_checked_index(int64_t i, int64_t n) {
    if (i >= 0 && i < n) return i;
    if (atomicAdd(&cf_check_hits, 1u) < 16u)
        printf("cf_check: block %d thread %d: cell %lld outside a table of %lld cells\n", (int)blockIdx.x,
               (int)threadIdx.x, (long long)i, (long long)n);
    return 0;
}

template <typename R>
struct TabPtr {
    R* p = nullptr;
    int64_t n = INT64_MAX;   // cells; unchecked until sized
    TabPtr() = default;
    __host__ __device__ TabPtr(R* q) : p(q) {}
    template <typename Q>
    __host__ __device__ TabPtr(const TabPtr<Q>& o) : p(o.p), n(o.n) {}
    __device__ R& operator[](int i) const { return p[cf_checked_index(i, n)]; }
    __device__ R& operator[](int64_t i) const { return p[cf_checked_index(i, n)]; }
    __device__ R* operator+(int o) const { return p + cf_checked_index(o, n); }
    __device__ operator R*() const { return p; }
};
#define CF_TAB(R) ::cf::TabPtr<R>
#define CF_SIZE_TAB(t, cells) ((t).n = (int64_t)(cells))
#else
#define CF_TAB(R) R*
#define CF_SIZE_TAB(t, cells) ((void)0)
#endif

// Round a word count up to 32 words (128 bytes).
__host__ __device__ __forceinline__ int64_t pad32(int64_t w) { return (w + 31) & ~int64_t(31); }

// Pairable-cell list of one sequence (see cf_seq.cuh): poff[L+2] int32 and
// pl[tri_size(L)] int16, in 4-byte words.
__host__ __device__ __forceinline__ int64_t plist_words(int L) {
    return pad32(L + 3) + pad32(tri_size(L) / 2 + 1);
}

// FP32 fold arena of one sequence (words).  The inside tables and the pair
// list come first so an inside-only arena (logZ, sampling) is a prefix of the
// full one.  Aliases: POST reuses FMo after the outside pass; the MEA score
// table reuses FM2o and its argmax table FM.
struct Arena32 {
    int64_t FC, FM, FM1, F5, FB, PL, FCo, FMo, FM1o, FM2o, F5o, up, queue, total;
};
__host__ __device__ __forceinline__ Arena32 arena32(int L) {
    Arena32 a;
    const int64_t t = pad32(tri_size(L));
    const int64_t v = pad32(L + 2);
    a.FC = 0; a.FM = t; a.FM1 = 2 * t; a.F5 = 3 * t; a.FB = 3 * t + v; a.PL = a.FB + 2 * v;
    const int64_t o = a.PL + plist_words(L);
    a.FCo = o; a.FMo = o + t; a.FM1o = o + 2 * t; a.FM2o = o + 3 * t;
    a.F5o = o + 4 * t; a.up = a.F5o + v; a.queue = a.up + v;
    a.total = a.queue + pad32(4 * (int64_t)L + 16);
    return a;
}
// Inside-only arena (logZ, sampling): FC FM FM1 F5, the FM2 step buffers and
// the pair list -- the prefix of Arena32.
__host__ __device__ __forceinline__ int64_t arena32_inside_words(int L) {
    return 3 * pad32(tri_size(L)) + 3 * pad32(L + 2) + plist_words(L);
}
// FP64 arena (Viterbi / exact logZ): FC FM FM1 F5 in doubles, then (in 4-byte
// words) the pair list and the traceback stack.
struct Arena64 {
    int64_t FC, FM, FM1, F5, FB;   // offsets in doubles (FB: two FM2 step buffers)
    int64_t PL, stack, total;      // offsets in 4-byte words
};
__host__ __device__ __forceinline__ Arena64 arena64(int L) {
    Arena64 a;
    const int64_t t = pad32(tri_size(L));
    const int64_t v = pad32(L + 2);
    a.FC = 0; a.FM = t; a.FM1 = 2 * t; a.F5 = 3 * t; a.FB = 3 * t + v;
    a.PL = 2 * (3 * t + 3 * v);
    a.stack = a.PL + plist_words(L);
    a.total = a.stack + pad32(3 * (4 * (int64_t)L + 16));
    return a;
}

// ---------------------------------------------------------------------------
// Fast_LogPlusEquals / Fast_Exp in float32 (cpu.py:527-580), branch-free.
// The reference picks one of eight (six) cubic segments with nested
// comparisons; here the segment index is the number of segment boundaries
// that are <= d, which selects the same cubic.  Coefficients come from shared
// memory (one float4 per segment) because lanes of a warp fall into different
// segments.  The evaluation order ((c0*d + c1)*d + c2)*d + c3 is the
// reference's.
//
// Segment lookup: bin = floor(d) in 0..11 holds at most one boundary (the
// boundaries 0.66, 1.63, 2.49, 3.38, 4.43, 5.79, 7.82 fall in distinct unit
// intervals), so seg = (boundaries below the bin) + (d >= the boundary inside
// the bin), read from a 12-entry table -- the same count as comparing d with
// all seven.  Fast_Exp uses the same scheme on u = -x over its five
// boundaries (0.67, 1.48, 2.49, 3.84, 5.86: distinct unit intervals too).
// ---------------------------------------------------------------------------
#define LSE_T0 ((float)0.6615367791)
#define LSE_T1 ((float)1.6320158198)
#define LSE_T2 ((float)2.4912588184)
#define LSE_T3 ((float)3.3792499610)
#define LSE_T4 ((float)4.4261691294)
#define LSE_T5 ((float)5.7890710412)
#define LSE_T6 ((float)7.8162726752)
#define LSE_TMAX ((float)11.8624794162)

#define FEXP_T0 ((float)-9.91152)
#define FEXP_T1 ((float)-5.8622823336)
#define FEXP_T2 ((float)-3.8396630909)
#define FEXP_T3 ((float)-2.4915033807)
#define FEXP_T4 ((float)-1.4805375919)
#define FEXP_T5 ((float)-0.6725053211)

constexpr int kLseBins = 12;    // unit bins of d over [0, 12)
constexpr int kFexpBins = 10;   // unit bins of -x over [0, 10)

struct PolyTables {
    float4 lse[8];
    float4 fexp[6];
    float2 lse_bin[kLseBins];     // {boundary inside the bin or +FLT_MAX, int bits: boundaries below}
    float2 fexp_bin[kFexpBins];   // {-boundary inside the bin or -FLT_MAX, int bits: boundaries above}
};

__device__ __forceinline__ void load_poly_tables(PolyTables* t) {
    for (int k = threadIdx.x; k < 16 + kLseBins + kFexpBins; k += blockDim.x) {
        if (k < 8) {
            const float c[8][4] = {
                {(float)-0.0065591595, (float)0.1276442762, (float)0.4996554598, (float)0.6931542306},
                {(float)-0.0155157557, (float)0.1446775699, (float)0.4882939746, (float)0.6958092989},
                {(float)-0.0128909247, (float)0.1301028251, (float)0.5150398748, (float)0.6795585882},
                {(float)-0.0072142647, (float)0.0877540853, (float)0.6208708362, (float)0.5909675829},
                {(float)-0.0031455354, (float)0.0467229449, (float)0.7592532310, (float)0.4348794399},
                {(float)-0.0010110698, (float)0.0185943421, (float)0.8831730747, (float)0.2523695427},
                {(float)-0.0001962780, (float)0.0046084408, (float)0.9634431978, (float)0.0983148903},
                {(float)-0.0000113994, (float)0.0003734731, (float)0.9959107193, (float)0.0149855051}};
            t->lse[k] = make_float4(c[k][0], c[k][1], c[k][2], c[k][3]);
        } else if (k < 14) {
            const float c[6][4] = {
                {(float)0.0000803850, (float)0.0021627428, (float)0.0194708555, (float)0.0588080014},
                {(float)0.0013889414, (float)0.0244676474, (float)0.1471290604, (float)0.3042757740},
                {(float)0.0072335607, (float)0.0906002677, (float)0.3983111356, (float)0.6245959221},
                {(float)0.0232410351, (float)0.2085645908, (float)0.6906367911, (float)0.8682322329},
                {(float)0.0573782771, (float)0.3580258429, (float)0.9121133217, (float)0.9793091728},
                {(float)0.1199175927, (float)0.4815668234, (float)0.9975991939, (float)0.9999505077}};
            const int s = k - 8;
            t->fexp[s] = make_float4(c[s][0], c[s][1], c[s][2], c[s][3]);
        } else if (k < 16 + kLseBins) {
            if (k >= 16) {
                const int b = k - 16;
                const float lo = (float)b, hi = (float)(b + 1);
                const float T[7] = {LSE_T0, LSE_T1, LSE_T2, LSE_T3, LSE_T4, LSE_T5, LSE_T6};
                int base = 0;
                float inner = 3.402823466e38f;
                for (int i = 0; i < 7; ++i) {
                    if (T[i] <= lo) ++base;
                    else if (T[i] < hi) inner = T[i];
                }
                t->lse_bin[b] = make_float2(inner, __int_as_float(base));
            }
        } else if (k < 16 + kLseBins + kFexpBins) {
            const int b = k - 16 - kLseBins;
            const float lo = (float)b, hi = (float)(b + 1);
            const float U[5] = {-FEXP_T1, -FEXP_T2, -FEXP_T3, -FEXP_T4, -FEXP_T5};
            int base = 0;   // boundaries U_k >= hi: u <= U_k for every u of the bin
            float inner = -3.402823466e38f;
            for (int i = 0; i < 5; ++i) {
                if (U[i] >= hi) ++base;
                else if (U[i] >= lo) inner = U[i];
            }
            t->fexp_bin[b] = make_float2(inner, __int_as_float(base));
        }
    }
}

__device__ __forceinline__ float cubic(const float4 c, float x) {
    float r = __fmul_rn(c.x, x);
    r = __fadd_rn(r, c.y);
    r = __fmul_rn(r, x);
    r = __fadd_rn(r, c.z);
    r = __fmul_rn(r, x);
    return __fadd_rn(r, c.w);
}

// CF_LSE_SELECT = 1 picks the segment's coefficients with a chain of
// compare-and-select on constants held in the instruction stream (no shared
// memory on the dependency path: 110 against 160 cycles per dependent term
// measured on GB300, at more instructions per term); 0 reads them from the
// bin tables.  Both give the segment the reference's comparisons give.
#ifndef CF_LSE_SELECT
#define CF_LSE_SELECT 0
#endif

// Fast_LogPlusEquals by compare-and-select: segment k's coefficients replace
// the running ones when d >= T_(k-1), so the last boundary below d wins --
// the segment of the reference's nested comparisons.
__device__ __forceinline__ float lse32_select(float a, float b) {
    const float hi = fmaxf(a, b);
    const float lo = fminf(a, b);
    const float d = __fsub_rn(hi, lo);
    float c0 = (float)-0.0065591595, c1 = (float)0.1276442762, c2 = (float)0.4996554598, c3 = (float)0.6931542306;
#define CF_LSE_SEG(T, x0, x1, x2, x3) \
    if (d >= (T)) { c0 = (float)(x0); c1 = (float)(x1); c2 = (float)(x2); c3 = (float)(x3); }
    CF_LSE_SEG(LSE_T0, -0.0155157557, 0.1446775699, 0.4882939746, 0.6958092989)
    CF_LSE_SEG(LSE_T1, -0.0128909247, 0.1301028251, 0.5150398748, 0.6795585882)
    CF_LSE_SEG(LSE_T2, -0.0072142647, 0.0877540853, 0.6208708362, 0.5909675829)
    CF_LSE_SEG(LSE_T3, -0.0031455354, 0.0467229449, 0.7592532310, 0.4348794399)
    CF_LSE_SEG(LSE_T4, -0.0010110698, 0.0185943421, 0.8831730747, 0.2523695427)
    CF_LSE_SEG(LSE_T5, -0.0001962780, 0.0046084408, 0.9634431978, 0.0983148903)
    CF_LSE_SEG(LSE_T6, -0.0000113994, 0.0003734731, 0.9959107193, 0.0149855051)
#undef CF_LSE_SEG
    float r = __fmul_rn(c0, d);
    r = __fadd_rn(r, c1);
    r = __fmul_rn(r, d);
    r = __fadd_rn(r, c2);
    r = __fmul_rn(r, d);
    r = __fadd_rn(r, c3);
    const float res = __fadd_rn(lo, r);
    return d >= LSE_TMAX ? hi : res;
}

// log(exp(a) + exp(b)), CONTRAfold Fast_LogPlusEquals (RealT = float).
__device__ __forceinline__ float lse32(const PolyTables* __restrict__ pt, float a, float b) {
#if CF_LSE_SELECT
    (void)pt;
    return lse32_select(a, b);
#else
    // the larger and the smaller argument (the reference swaps on a < b; for
    // the finite inputs here fmaxf / fminf give the same pair)
    const float hi = fmaxf(a, b);
    const float lo = fminf(a, b);
    const float d = __fsub_rn(hi, lo);
    const float2 e = pt->lse_bin[min(__float2int_rz(d), kLseBins - 1)];
    const int seg = __float_as_int(e.y) + (d >= e.x);
    const float r = cubic(pt->lse[seg], d);
    const float res = __fadd_rn(lo, r);
    // The reference also returns hi when lo is below the zero threshold; for
    // finite inputs that case is covered: lo < -5e29 < hi makes d at least
    // one float spacing there (~4e22) >= LSE_TMAX, and lo == hi gives
    // res = lo + cubic(0) == lo (0.69 is far below half a spacing of lo).
    return d >= LSE_TMAX ? hi : res;
#endif
}

// exp(x), CONTRAfold Fast_Exp (RealT = float).  For x >= 0 the reference
// evaluates exp in double precision and rounds (cpu.py:578-580).
__device__ __forceinline__ float fexp32(const PolyTables* __restrict__ pt, float x) {
    if (x >= 0.0f) {
        if (x > (float)46.052) return (float)1e20;
        return (float)exp((double)x);
    }
    const float u = -x;   // x < 0: x >= T_k  <=>  u <= -T_k
    const float2 e = pt->fexp_bin[min(__float2int_rz(u), kFexpBins - 1)];
    const int seg = __float_as_int(e.y) + (u <= e.x);
    const float r = cubic(pt->fexp[seg], x);
    return x < FEXP_T0 ? 0.0f : r;
}

// FP64 log-sum-exp with exact log1p/exp (cpu.py:154-162).
__device__ __forceinline__ double lse64(double a, double b) {
    if (a < CF_HALF64) return b;
    if (b < CF_HALF64) return a;
    if (a > b) return a + log1p(exp(b - a));
    return b + log1p(exp(a - b));
}

// ---------------------------------------------------------------------------
// Scoring tables in shared memory.
// ---------------------------------------------------------------------------
template <typename Real>
struct ParamView {
    const Real* b;   // blob (layout CF_OFF_*)
    __device__ __forceinline__ Real bp(int x, int y) const { return b[CF_OFF_BP + x * 5 + y]; }
    __device__ __forceinline__ Real stack(int a, int c, int e, int f) const {
        return b[CF_OFF_STACK + ((a * 5 + c) * 5 + e) * 5 + f];
    }
    __device__ __forceinline__ Real tm(int a, int c, int e, int f) const {
        return b[CF_OFF_TM + ((a * 5 + c) * 5 + e) * 5 + f];
    }
    __device__ __forceinline__ Real hc(int x, int y) const { return b[CF_OFF_HC + x * 5 + y]; }
    __device__ __forceinline__ Real dl(int x, int y, int z) const { return b[CF_OFF_DL + (x * 5 + y) * 5 + z]; }
    __device__ __forceinline__ Real dr(int x, int y, int z) const { return b[CF_OFF_DR + (x * 5 + y) * 5 + z]; }
    __device__ __forceinline__ Real hp(int k) const { return b[CF_OFF_HPCUM + k]; }
    __device__ __forceinline__ Real cs(int l1, int l2) const { return b[CF_OFF_CS + l1 * 31 + l2]; }
    __device__ __forceinline__ Real i11(int x, int y) const { return b[CF_OFF_I11 + x * 5 + y]; }
    __device__ __forceinline__ Real b01(int x) const { return b[CF_OFF_B01 + x]; }
    __device__ __forceinline__ Real mb() const { return b[CF_OFF_MB]; }
    __device__ __forceinline__ Real mu() const { return b[CF_OFF_MU]; }
    __device__ __forceinline__ Real mp() const { return b[CF_OFF_MP]; }
    __device__ __forceinline__ Real eu() const { return b[CF_OFF_EU]; }
    __device__ __forceinline__ Real ep() const { return b[CF_OFF_EP]; }
};

// Canonical pairs AU UA CG GC GU UG (cpu.py:25) over "pairing codes" 0..5:
// 0..3 = ACGU, 4 = N, 5 = forced unpaired.  Bit (x*6 + y).
constexpr uint64_t CANON6 = (1ull << (0 * 6 + 3)) | (1ull << (3 * 6 + 0)) | (1ull << (1 * 6 + 2)) |
                            (1ull << (2 * 6 + 1)) | (1ull << (2 * 6 + 3)) | (1ull << (3 * 6 + 2));
__device__ __forceinline__ bool pairable_codes(int x, int y) { return (CANON6 >> (x * 6 + y)) & 1ull; }

// ASCII -> base code (cpu.py:23-29, 138-144): A C G U/T -> 0..3, anything else 4.
__device__ __forceinline__ int8_t base_code(uint8_t c) {
    if (c >= 'a' && c <= 'z') c = (uint8_t)(c - 32);
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'U':
        case 'T': return 3;
        default: return 4;
    }
}

// Sequence view in shared memory: s[0..L+1] base codes with N sentinels,
// pc[0..L+1] pairing codes (5 where forced unpaired).
struct SeqView {
    const int8_t* s;
    const int8_t* pc;
    int L;
    __device__ __forceinline__ bool pairable(int a, int b) const { return pairable_codes(pc[a], pc[b]); }
};

// Encode sequence `D` into shared memory arrays s/pc (cooperative over the CTA).
__device__ __forceinline__ void encode_seq(const uint8_t* __restrict__ seqs, const uint8_t* __restrict__ mask,
                                           int64_t off, int L, int8_t* s, int8_t* pc) {
    for (int t = threadIdx.x; t < L + 2; t += blockDim.x) {
        int8_t code = 4, p = 4;
        if (t >= 1 && t <= L) {
            code = base_code(seqs[off + t - 1]);
            p = (mask != nullptr && mask[off + t - 1] != 0) ? (int8_t)5 : code;
        }
        s[t] = code;
        pc[t] = p;
    }
}

// Shared-memory header common to the FP32 kernels.
struct SmemHead32 {
    PolyTables poly;
    float blob[CF_BLOB_LEN + 3];   // +3 pads to 16 bytes
    float jB[625];                 // hc[a][b] + tm[a][b][c][d] (cpu.py:191,211-212)
};

// Load the FP32 blob and derived tables.  jB = hc + tm is the same float add
// the reference does inline, so precomputing it keeps the bits.
__device__ __forceinline__ void load_head32(SmemHead32* h, const float* __restrict__ gblob) {
    load_poly_tables(&h->poly);
    for (int t = threadIdx.x; t < CF_BLOB_LEN; t += blockDim.x) h->blob[t] = gblob[t];
    for (int t = threadIdx.x; t < 625; t += blockDim.x) {
        const int a = t / 125, c = (t / 25) % 5;
        h->jB[t] = __fadd_rn(gblob[CF_OFF_HC + a * 5 + c], gblob[CF_OFF_TM + t]);
    }
}

__device__ __forceinline__ int idx4(int a, int b, int c, int d) { return ((a * 5 + b) * 5 + c) * 5 + d; }

}  // namespace cf
