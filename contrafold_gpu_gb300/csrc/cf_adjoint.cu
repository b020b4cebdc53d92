// cf_adjoint.cu -- differentiation of logZ: expected feature counts and
// per-position unpaired probabilities (new capability; the reference has no
// gradient).
//
// logZ = log sum_s exp(score(s)) is linear-in-parameters inside the exp, so
//   d logZ / d(table entry e)  = E[#uses of e]         (expected counts)
//   d logZ / d u_k             = P(position k unpaired)
// where u is a soft per-position unpaired bonus added for every unpaired
// position (hairpin and single-branch loop interiors, multiloop and exterior
// unpaired positions) -- a soft DMS/SHAPE constraint.  Counts come from the
// inside/outside tables: every transition t of the recursion has probability
// exp(outside(parent) + inside(children) + score(t) - logZ); the kernel below
// enumerates all transitions and adds that probability to each
// parameter-table entry the transition's score uses.  P(k unpaired) is
// 1 - sum over the pairs (k, x) of P(pair), and P(pair (i, j+1)) =
// exp(FCo[i][j] + FC[i][j] - logZ).  Inside and outside are
// evaluated with the accurate float32 log-sum-exp so the counts are the
// derivative of the logZ that cf_logz reports (within float32 rounding).
//
// Kernels: one CTA per sequence, one warp per DP cell: the lanes split the
// cell's candidate terms (the 496 single-branch window slots, the O(L)
// bifurcation and outside chains) and combine their partial sums with a
// fixed butterfly, so every cell costs a few warp iterations instead of one
// thread's serial loop, and lanes never idle on a short diagonal.
// k_adj_inside fills the inside tables; k_adj_outside then walks the
// diagonals downwards, computing the outside values of diagonal t and, in the
// same step, the transition probabilities of diagonal t + 1 (whose outside
// values are final by then).  No result has a bitwise target (the reference
// has no gradient), but every sum is taken in a fixed order, so results are
// the same on every run.
//
// Memory.  The bifurcation and exterior terms read FC, FM, FM1 and the
// outside FM2o at every span, so those four tables are kept whole.  FCo,
// FMo and FM1o are read only within 32 diagonals of the one being computed
// (the single-branch window) and by the counts of their own diagonal, so they
// live in ring buffers of 33, 2 and 3 diagonals.  The inside FM2 is needed
// by the counts of its own diagonal only: it is checkpointed on every k-th
// diagonal and recomputed on the others from FM1 and FM (the same chain in
// the same order, so bitwise the stored value).  k = 1 keeps every diagonal.
//
// Counts are accumulated in 128-bit fixed point (value x 2^62, integer
// atomics): integer addition is exact and order-independent, so the counts
// and unpaired probabilities are deterministic -- bitwise the same for every
// run, thread schedule and checkpoint spacing.
#include "cf_kernels.h"
#include "cf_outside.cuh"

namespace cf {
namespace {

constexpr int kWin = (CMAX + 1) * (CMAX + 2) / 2;   // single-branch window slots, l1 + l2 <= CMAX
constexpr int kAdjWarps = kFoldThreads / 32;

struct AdjSmem {
    SmemTabs<float> tabs;
    unsigned long long cnt_lo[CF_BLOB_LEN];   // fixed-point counts (x 2^62), low 64 bits
    unsigned cnt_hi[CF_BLOB_LEN];             // carries out of cnt_lo (units of 4)
    unsigned char win_l1[kWin], win_l2[kWin]; // window slot -> (l1, l2), rows l1 ascending
};

__device__ __forceinline__ void load_window(AdjSmem* sm) {
    for (int c = threadIdx.x; c < kWin; c += blockDim.x) {
        // row l1 holds CMAX + 1 - l1 slots and starts at l1 (CMAX + 1) - l1 (l1 - 1) / 2
        int l1 = 0, start = 0;
        while (start + (CMAX + 1 - l1) <= c) start += CMAX + 1 - l1++;
        sm->win_l1[c] = (unsigned char)l1;
        sm->win_l2[c] = (unsigned char)(c - start);
    }
}

// Cells of the FM2 checkpoints (diagonals 0, k, 2k, ... <= L) and the offset
// of checkpoint c (diagonal c k, m - c k cells).
__host__ __device__ __forceinline__ int64_t ckpt_off(int c, int m, int k) {
    return (int64_t)c * m - (int64_t)k * c * (c - 1) / 2;
}
__host__ __device__ __forceinline__ int64_t ckpt_cells(int L, int k) { return ckpt_off(L / k + 1, L + 1, k); }

constexpr int kRingFCo = 33;   // FCo: spans t .. t + 32
constexpr int kRingFMo = 2;    // FMo: spans t, t + 1
constexpr int kRingFM1o = 3;   // FM1o: spans t .. t + 2

// Adjoint arena (4-byte words): FC FM FM1 (triangles), F5, F5o, FM2o
// (triangle), the FCo / FMo / FM1o ring buffers, the FM2 checkpoints, the
// FP64 bonus prefix U, and the fixed-point pairing probability of every
// position (128 bits each: a low and a high uint64 array).
struct ArenaAdj {
    int64_t FC, FM, FM1, F5, F5o, FM2o, RC, RM, R1, FM2, U, PD, total;
};
__host__ __device__ __forceinline__ ArenaAdj arena_adj(int L, int k) {
    ArenaAdj r;
    const int64_t t = pad32(tri_size(L)), v = pad32(L + 2), rw = pad32(L + 1);
    r.FC = 0; r.FM = t; r.FM1 = 2 * t; r.F5 = 3 * t; r.F5o = r.F5 + v; r.FM2o = r.F5o + v;
    r.RC = r.FM2o + t;
    r.RM = r.RC + kRingFCo * rw;
    r.R1 = r.RM + kRingFMo * rw;
    r.FM2 = r.R1 + kRingFM1o * rw;
    r.U = r.FM2 + pad32(ckpt_cells(L, k));
    r.PD = r.U + 2 * v;                 // doubles
    r.total = r.PD + 4 * v;             // 2 x uint64[L + 2]
    return r;
}

// Outside values of one diagonal live in a ring slot: cell (a, a + t) of
// table X at X[(t mod R) * rw + a].
struct AdjView {
    InTabs<float> I;
    float* F5o;
    float* FM2o;      // triangle
    float* RC;        // FCo ring
    float* RM;        // FMo ring
    float* R1;        // FM1o ring
    float* FM2;       // checkpoints
    const double* U;  // U[k] = sum_{t<=k} u_t
    unsigned long long* PD;   // [2][L + 2]: P(position paired), low and high words
    int m, rw, k, L;
    __device__ __forceinline__ float& fco(int a, int t) const { return RC[(t % kRingFCo) * rw + a]; }
    __device__ __forceinline__ float& fmo(int a, int t) const { return RM[(t % kRingFMo) * rw + a]; }
    __device__ __forceinline__ float& fm1o(int a, int t) const { return R1[(t % kRingFM1o) * rw + a]; }
    __device__ __forceinline__ float& fm2o(int a, int b) const { return FM2o[tri_off(b - a, m) + a]; }
};

__device__ __forceinline__ AdjView adj_view(const FoldArgs& A, const SeqDesc& D, int k) {
    const ArenaAdj r = arena_adj(D.L, k);
    float* base = A.ws + D.ws_off;
    AdjView V;
    V.I.FC = base + r.FC; V.I.FM = base + r.FM; V.I.FM1 = base + r.FM1; V.I.F5 = base + r.F5;
    V.I.m = D.L + 1;
    V.I.sized(D.L);
    V.F5o = base + r.F5o;
    V.FM2o = base + r.FM2o;
    V.RC = base + r.RC; V.RM = base + r.RM; V.R1 = base + r.R1;
    V.FM2 = base + r.FM2;
    V.U = reinterpret_cast<const double*>(base + r.U);
    V.PD = reinterpret_cast<unsigned long long*>(base + r.PD);
    V.m = D.L + 1;
    V.rw = (int)pad32(D.L + 1);
    V.k = k;
    V.L = D.L;
    return V;
}

// bonus of the unpaired stretch (lo, hi]: U[hi] - U[lo]
__device__ __forceinline__ float bon(const double* U, int lo, int hi) { return (float)(U[hi] - U[lo]); }
__device__ __forceinline__ float ubon(const double* U, int k) { return (float)(U[k] - U[k - 1]); }

__device__ __forceinline__ SeqView adj_setup(AdjSmem* sm, const FoldArgs& A, SeqDesc& D) {
    D = A.descs[blockIdx.x];
    load_tabs(&sm->tabs, A.blob32);
    load_window(sm);
    int8_t* s = reinterpret_cast<int8_t*>(sm + 1);
    const int stride = (D.L + 2 + 15) & ~15;
    int8_t* pc = s + stride;
    encode_seq(A.seqs, A.mask, D.seq_off, D.L, s, pc);
    __syncthreads();
    return SeqView{s, pc, D.L};
}

// e of the single-branch candidate (outer (i, j+1), inner (p+1, q)), the
// reference's operation order (cpu.py:207-220).
__device__ __forceinline__ float single_e(const ParamView<float>& P, const SmemTabs<float>* tb, const SeqView& Q,
                                          int i, int j, int p, int q) {
    const int l1 = p - i, l2 = j - q;
    const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
    if (l1 == 0 && l2 == 0) return __fadd_rn(P.bp(si1, sj), P.stack(si, sj1, si1, sj));
    const float jB1 = tb->jB[idx4(si, sj1, si1, sj)];
    const float jB2 = tb->jB[idx4(Q.s[q], Q.s[p + 1], Q.s[q + 1], Q.s[p])];
    float snuc = 0.0f;
    if (l1 == 0 && l2 == 1) snuc = P.b01(sj);
    else if (l1 == 1 && l2 == 0) snuc = P.b01(si1);
    else if (l1 == 1 && l2 == 1) snuc = P.i11(si1, sj);
    return __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(P.cs(l1, l2), P.bp(Q.s[p + 1], Q.s[q])), jB1), jB2), snuc);
}


// Log-sum-exp of the 32 lanes' partial sums by a fixed butterfly; every lane
// gets the same value (LseAcc32's plus is symmetric in its arguments).
__device__ __forceinline__ float warp_lse(float x) {
    const LseAcc32 sr{};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x = sr.plus(x, __shfl_xor_sync(0xffffffffu, x, o));
    return x;
}
__device__ __forceinline__ unsigned long long warp_sum(unsigned long long x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    return x;
}

// FM2[i][j] = (+)_{i<k<j} FM1[i][k] * FM[k][j], live terms only; lane l takes
// k = i + 1 + l, i + 33 + l, ...  Called by a whole warp; the inside and the
// recomputation in the outside use this one function, so a recomputed FM2 is
// bitwise the stored one.
__device__ __forceinline__ float fm2_warp(const InTabs<float>& T, int i, int j, int lane) {
    const LseAcc32 sr{};
    float fm2 = CF_NEG32;
    for (int k = i + 1 + lane; k < j; k += 32) {
        const float a = T.FM1[T.at(i, k)], b = T.FM[T.at(k, j)];
        if (a > CF_HALF32 && b > CF_HALF32) fm2 = sr.plus(fm2, __fadd_rn(a, b));
    }
    return warp_lse(fm2);
}


}  // namespace

// ---------------------------------------------------------------------------
// Inside with bonus (accurate float32 log-sum-exp); FM2 kept on every ckpt-th
// diagonal.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kFoldThreads) k_adj_inside(FoldArgs A, const float* bonus, int ckpt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<AdjSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = adj_setup(sm, A, D);
    const ParamView<float> P{sm->tabs.blob};
    const AdjView V = adj_view(A, D, ckpt);
    const LseAcc32 sr{};
    const int L = D.L, m = L + 1;
    double* U = const_cast<double*>(V.U);
    if (threadIdx.x == 0) {
        double acc = 0.0;
        U[0] = 0.0;
        for (int k = 1; k <= L; ++k) {
            acc += bonus ? (double)bonus[D.seq_off + k - 1] : 0.0;
            U[k] = acc;
        }
        U[L + 1] = acc;
    }
    __syncthreads();
    const InTabs<float>& T = V.I;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = 0; d <= L; ++d) {
        const bool keep = d % ckpt == 0;
        float* fm2_ck = V.FM2 + (keep ? ckpt_off(d / ckpt, m, ckpt) : 0);
        for (int i = warp; i + d <= L; i += kAdjWarps) {   // one warp per cell
            const int j = i + d, at = tri_off(d, m) + i;
            const bool fm_region = (0 < i) && (i + 2 <= j) && (j < L);
            const bool fc_cell = (0 < i) && (j < L) && Q.pairable(i, j + 1);
            const float fm2 = fm_region ? fm2_warp(T, i, j, lane) : CF_NEG32;
            float fc = CF_NEG32;
            if (fc_cell) {
                const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
                // single-branch candidates: window slot c = (l1, l2), inner pair (p+1, q)
                float part = CF_NEG32;
                for (int c = lane; c < kWin; c += 32) {
                    const int l1 = sm->win_l1[c], l2 = sm->win_l2[c];
                    if (l1 + l2 > d - 2) continue;   // q >= p + 2
                    const int p = i + l1, q = j - l2;
                    if (!Q.pairable(p + 1, q)) continue;
                    const float inner = T.FC[T.at(p + 1, q - 1)];
                    if (!(inner > CF_HALF32)) continue;
                    const float e = single_e(P, &sm->tabs, Q, i, j, p, q);
                    const float b = __fadd_rn(bon(V.U, i, p), bon(V.U, q, j));
                    part = sr.plus(part, __fadd_rn(__fadd_rn(e, inner), b));
                }
                const float jB = sm->tabs.jB[idx4(si, sj1, si1, sj)];
                float acc = __fadd_rn(__fadd_rn(jB, P.hp(d <= DHP ? d : DHP)), bon(V.U, i, j));
                acc = sr.plus(acc, warp_lse(part));
                if (fm2 > CF_HALF32) {
                    const float jA = junctionA<LseAcc32>(P, L, Q, i, j);
                    acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(fm2, jA), P.mp()), P.mb()));
                }
                fc = acc;
            }
            float fm1 = CF_NEG32, fm = CF_NEG32;
            if (fm_region) {
                float acc = CF_NEG32;
                const float fin = T.FC[T.at(i + 1, j - 1)];
                if (Q.pairable(i + 1, j) && fin > CF_HALF32) {
                    const float jAji = junctionA_rev<LseAcc32>(P, L, Q, i, j);
                    acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(fin, jAji), P.mp()), P.bp(Q.s[i + 1], Q.s[j])));
                }
                const float ext = T.FM1[T.at(i + 1, j)];
                if (ext > CF_HALF32) acc = sr.plus(acc, __fadd_rn(__fadd_rn(ext, P.mu()), ubon(V.U, i + 1)));
                fm1 = acc;
                acc = CF_NEG32;
                if (fm2 > CF_HALF32) acc = sr.plus(acc, fm2);
                const float prev = T.FM[T.at(i, j - 1)];
                if (prev > CF_HALF32) acc = sr.plus(acc, __fadd_rn(__fadd_rn(prev, P.mu()), ubon(V.U, j)));
                if (fm1 > CF_HALF32) acc = sr.plus(acc, fm1);
                fm = acc;
            }
            if (lane == 0) {
                if (keep) fm2_ck[i] = fm2;
                T.FC[at] = fc;
                T.FM1[at] = fm1;
                T.FM[at] = fm;
            }
        }
        __syncthreads();
    }
    // exterior (one warp; sequential chain, terms in parallel)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        float prev = 0.0f;
        if (lane == 0) T.F5[0] = 0.0f;
        for (int j = 1; j <= L; ++j) {
            float acc = __fadd_rn(__fadd_rn(prev, P.eu()), ubon(V.U, j));
            for (int k0 = 0; k0 < j; k0 += 32) {
                const int k = k0 + lane;
                bool ok = false;
                float term = 0.0f;
                if (k < j && Q.pairable(k + 1, j)) {
                    const float fcin = T.FC[T.at(k + 1, j - 1)], f5k = T.F5[k];
                    if (fcin > CF_HALF32 && f5k > CF_HALF32) {
                        const float jA = junctionA_rev<LseAcc32>(P, L, Q, k, j);
                        term = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(f5k, fcin), P.ep()), P.bp(Q.s[k + 1], Q.s[j])), jA);
                        ok = true;
                    }
                }
                unsigned msk = __ballot_sync(0xffffffffu, ok);
                while (msk) {
                    const int t = __ffs(msk) - 1;
                    msk &= msk - 1;
                    acc = sr.plus(acc, __shfl_sync(0xffffffffu, term, t));
                }
            }
            if (lane == 0) T.F5[j] = acc;
            prev = acc;
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------------------
// Outside with bonus (gathers; any order -- no bitwise target) and, one
// diagonal behind, the transition probabilities -> fixed-point expected counts
// ---------------------------------------------------------------------------
namespace {

// Fixed point: a probability v (float, < 4) as the integer v x 2^62 (exact:
// a float has 24 significant bits).  A 128-bit sum of such integers is exact
// in any order.
__device__ __forceinline__ unsigned long long fixp(float v) { return __float2ull_rn(ldexpf(v, 62)); }

__device__ __forceinline__ void add128(unsigned long long* lo, unsigned* hi, unsigned long long x) {
    const unsigned long long old = atomicAdd(lo, x);
    if (old + x < old) atomicAdd(hi, 1u);
}
__device__ __forceinline__ void add128g(unsigned long long* lo, unsigned long long* hi, unsigned long long x) {
    const unsigned long long old = atomicAdd(lo, x);
    if (old + x < old) atomicAdd(hi, 1ull);
}

struct Counter {
    AdjSmem* sm;
    unsigned long long* pd;   // global [2][L + 2]: P(position paired), low and high words
    int n;                    // L + 2
    __device__ __forceinline__ void add(int e, unsigned long long v) const { add128(&sm->cnt_lo[e], &sm->cnt_hi[e], v); }
    // positions a and b paired with each other with probability v
    __device__ __forceinline__ void pair(int a, int b, unsigned long long v) const {
        add128g(pd + a, pd + n + a, v);
        add128g(pd + b, pd + n + b, v);
    }
};

// jA(i, j) of the pair (i, j+1): entries hc[s_i][s_j+1], dl (i < L), dr (j > 0)
__device__ __forceinline__ void count_jA(const Counter& C, const SeqView& Q, int L, int i, int j, unsigned long long v) {
    C.add(CF_OFF_HC + Q.s[i] * 5 + Q.s[j + 1], v);
    if (i < L) C.add(CF_OFF_DL + (Q.s[i] * 5 + Q.s[j + 1]) * 5 + Q.s[i + 1], v);
    if (j > 0) C.add(CF_OFF_DR + (Q.s[i] * 5 + Q.s[j + 1]) * 5 + Q.s[j], v);
}
// jA(j, i) of the pair (i+1, j)
__device__ __forceinline__ void count_jA_rev(const Counter& C, const SeqView& Q, int L, int i, int j,
                                             unsigned long long v) {
    C.add(CF_OFF_HC + Q.s[j] * 5 + Q.s[i + 1], v);
    if (j < L) C.add(CF_OFF_DL + (Q.s[j] * 5 + Q.s[i + 1]) * 5 + Q.s[j + 1], v);
    if (i > 0) C.add(CF_OFF_DR + (Q.s[j] * 5 + Q.s[i + 1]) * 5 + Q.s[i], v);
}
// jB = hc + tm of the pair (a, b+1) with inner neighbours (a+1, b)
__device__ __forceinline__ void count_jB(const Counter& C, int sa, int sb1, int sa1, int sb, unsigned long long v) {
    C.add(CF_OFF_HC + sa * 5 + sb1, v);
    C.add(CF_OFF_TM + idx4(sa, sb1, sa1, sb), v);
}

// Outside values of cell (a, b), span t, into the ring slots of diagonal t.
// Called by a whole warp; lane 0 writes.
__device__ __forceinline__ void outside_cell(const AdjSmem* sm, const ParamView<float>& P, const SeqView& Q,
                                             const AdjView& V, int a, int b, int lane) {
    const LseAcc32 sr{};
    const int L = V.L, t = b - a;
    const InTabs<float>& I = V.I;
    const bool fm_region = (0 < a) && (a + 2 <= b) && (b < L);
    float fmo = CF_NEG32, fm1o = CF_NEG32;
    if (fm_region) {
        // FMo[a][b]: multiloop FM2o[i][b] * FM1[i][a] over i < a, and the extension
        float part = CF_NEG32;
        for (int i = 1 + lane; i < a; i += 32) {
            const float src = V.fm2o(i, b), f1 = I.FM1[I.at(i, a)];
            if (src > CF_HALF32 && f1 > CF_HALF32) part = sr.plus(part, __fadd_rn(src, f1));
        }
        float acc = warp_lse(part);
        if (b + 1 < L) acc = sr.plus(acc, __fadd_rn(__fadd_rn(V.fmo(a, t + 1), P.mu()), ubon(V.U, b + 1)));
        fmo = acc;
        // FM1o[a][b]: FM2o[a][j] * FM[b][j] over j > b, the extension, and FMo
        part = CF_NEG32;
        for (int j = b + 1 + lane; j < L; j += 32) {
            const float src = V.fm2o(a, j), fmk = I.FM[I.at(b, j)];
            if (src > CF_HALF32 && fmk > CF_HALF32) part = sr.plus(part, __fadd_rn(src, fmk));
        }
        acc = warp_lse(part);
        if (a >= 2) acc = sr.plus(acc, __fadd_rn(__fadd_rn(V.fm1o(a - 1, t + 1), P.mu()), ubon(V.U, a)));
        fm1o = sr.plus(acc, fmo);
    }
    float fco = CF_NEG32;
    if (0 < a && b < L && Q.pairable(a, b + 1)) {
        const int sa = Q.s[a], sb1 = Q.s[b + 1];
        // the pair (a, b+1) as the inner pair of a single-branch loop closed by
        // (i, j+1) = (a-1-l1, b+2+l2)
        float part = CF_NEG32;
        for (int c = lane; c < kWin; c += 32) {
            const int i = a - 1 - sm->win_l1[c], j = b + 1 + sm->win_l2[c];
            if (i < 1 || j >= L || !Q.pairable(i, j + 1)) continue;
            const float src = V.fco(i, j - i);
            if (!(src > CF_HALF32)) continue;
            const float e = single_e(P, &sm->tabs, Q, i, j, a - 1, b + 1);
            const float bb = __fadd_rn(bon(V.U, i, a - 1), bon(V.U, b + 1, j));
            part = sr.plus(part, __fadd_rn(__fadd_rn(src, e), bb));
        }
        float acc = warp_lse(part);
        const float f5k = I.F5[a - 1];
        if (f5k > CF_HALF32) {
            const float jA = junctionA_rev<LseAcc32>(P, L, Q, a - 1, b + 1);
            acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V.F5o[b + 1], P.ep()), P.bp(sa, sb1)), jA), f5k));
        }
        if (a >= 2 && b + 1 < L) {
            const float jAji = junctionA_rev<LseAcc32>(P, L, Q, a - 1, b + 1);
            acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(V.fm1o(a - 1, t + 2), jAji), P.mp()), P.bp(sa, sb1)));
        }
        fco = acc;
    }
    float fm2o = CF_NEG32;
    if (fm_region) fm2o = sr.plus(fm2o, fmo);
    if (fco > CF_HALF32) {
        const float jA = junctionA<LseAcc32>(P, L, Q, a, b);
        fm2o = sr.plus(fm2o, __fadd_rn(__fadd_rn(__fadd_rn(fco, jA), P.mp()), P.mb()));
    }
    if (lane == 0) {
        V.fmo(a, t) = fmo;
        V.fm1o(a, t) = fm1o;
        V.fco(a, t) = fco;
        V.fm2o(a, b) = fm2o;
    }
}

// Transitions out of the states of cell (i, j) (its outside values final).
// Called by a whole warp: the lanes split the single-branch window; lane 0
// counts the cell's other transitions.
__device__ __forceinline__ void count_cell(const AdjSmem* sm, const ParamView<float>& P, const SeqView& Q,
                                           const AdjView& V, const Counter& C, float Z, int i, int j, int lane) {
    const int L = V.L, d = j - i, m = V.m;
    const InTabs<float>& I = V.I;
    auto prob = [&](float x) { return fixp(expf(__fsub_rn(x, Z))); };
    const bool fm_region = (0 < i) && (i + 2 <= j) && (j < L);
    if (0 < i && j < L && Q.pairable(i, j + 1)) {
        const float fco = V.fco(i, d);
        if (fco > CF_HALF32) {
            const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
            const float jB = sm->tabs.jB[idx4(si, sj1, si1, sj)];
            // single-branch loops: window slot c = (l1, l2), inner pair (p+1, q)
            unsigned long long outer_jB = 0;
            for (int c = lane; c < kWin; c += 32) {
                const int l1 = sm->win_l1[c], l2 = sm->win_l2[c];
                if (l1 + l2 > d - 2) continue;
                const int p = i + l1, q = j - l2;
                if (!Q.pairable(p + 1, q)) continue;
                const float inner = I.FC[I.at(p + 1, q - 1)];
                if (!(inner > CF_HALF32)) continue;
                const float e = single_e(P, &sm->tabs, Q, i, j, p, q);
                const float bb = __fadd_rn(bon(V.U, i, p), bon(V.U, q, j));
                const unsigned long long v = prob(__fadd_rn(fco, __fadd_rn(__fadd_rn(e, inner), bb)));
                if (l1 == 0 && l2 == 0) {
                    C.add(CF_OFF_BP + si1 * 5 + sj, v);
                    C.add(CF_OFF_STACK + idx4(si, sj1, si1, sj), v);
                } else {
                    const int sa = Q.s[p + 1], sq = Q.s[q];
                    C.add(CF_OFF_CS + l1 * 31 + l2, v);
                    C.add(CF_OFF_BP + sa * 5 + sq, v);
                    outer_jB += v;
                    count_jB(C, sq, sa, Q.s[q + 1], Q.s[p], v);
                    if (l1 == 0 && l2 == 1) C.add(CF_OFF_B01 + sj, v);
                    else if (l1 == 1 && l2 == 0) C.add(CF_OFF_B01 + si1, v);
                    else if (l1 == 1 && l2 == 1) C.add(CF_OFF_I11 + si1 * 5 + sj, v);
                }
            }
            // the probabilities of the loops closed by one pair sum to at most
            // P(pair) <= 1, so the warp's total fits 64 bits
            outer_jB = warp_sum(outer_jB);
            // multiloop closed by (i, j+1): FM2 from its checkpoint, or recomputed (whole warp)
            float fm2 = CF_NEG32;
            if (fm_region) fm2 = d % V.k == 0 ? V.FM2[ckpt_off(d / V.k, m, V.k) + i] : fm2_warp(I, i, j, lane);
            if (lane == 0) {
                if (outer_jB != 0) count_jB(C, si, sj1, si1, sj, outer_jB);
                // the pair (i, j+1) itself
                const float fc = I.FC[I.at(i, j)];
                if (fc > CF_HALF32) C.pair(i, j + 1, prob(__fadd_rn(fco, fc)));
                // hairpin
                const int hl = d <= DHP ? d : DHP;
                const unsigned long long v = prob(__fadd_rn(fco, __fadd_rn(__fadd_rn(jB, P.hp(hl)), bon(V.U, i, j))));
                count_jB(C, si, sj1, si1, sj, v);
                C.add(CF_OFF_HPCUM + hl, v);
                if (fm2 > CF_HALF32) {
                    const float jA = junctionA<LseAcc32>(P, L, Q, i, j);
                    const unsigned long long w =
                        prob(__fadd_rn(fco, __fadd_rn(__fadd_rn(__fadd_rn(fm2, jA), P.mp()), P.mb())));
                    count_jA(C, Q, L, i, j, w);
                    C.add(CF_OFF_MP, w);
                    C.add(CF_OFF_MB, w);
                }
            }
        }
    }
    if (fm_region && lane == 0) {
        const float fm1o = V.fm1o(i, d);
        if (fm1o > CF_HALF32) {
            const float fin = I.FC[I.at(i + 1, j - 1)];
            if (Q.pairable(i + 1, j) && fin > CF_HALF32) {
                const float jAji = junctionA_rev<LseAcc32>(P, L, Q, i, j);
                const unsigned long long v = prob(__fadd_rn(fm1o, __fadd_rn(__fadd_rn(__fadd_rn(fin, jAji), P.mp()),
                                                                             P.bp(Q.s[i + 1], Q.s[j]))));
                count_jA_rev(C, Q, L, i, j, v);
                C.add(CF_OFF_MP, v);
                C.add(CF_OFF_BP + Q.s[i + 1] * 5 + Q.s[j], v);
            }
            const float ext = I.FM1[I.at(i + 1, j)];
            if (ext > CF_HALF32) {
                const unsigned long long v = prob(__fadd_rn(fm1o, __fadd_rn(__fadd_rn(ext, P.mu()), ubon(V.U, i + 1))));
                C.add(CF_OFF_MU, v);
            }
        }
        const float fmo = V.fmo(i, d);
        const float prev = I.FM[I.at(i, j - 1)];
        if (fmo > CF_HALF32 && prev > CF_HALF32) {
            const unsigned long long v = prob(__fadd_rn(fmo, __fadd_rn(__fadd_rn(prev, P.mu()), ubon(V.U, j))));
            C.add(CF_OFF_MU, v);
        }
    }
}

// 128-bit fixed point (hi: units of 2^64, lo) -> double
__device__ __forceinline__ double fixp_value(double hi, unsigned long long lo) {
    return hi * 4.0 + (double)(lo >> 10) * 0x1p-52 + (double)(lo & 1023ull) * 0x1p-62;
}

}  // namespace

__global__ void __launch_bounds__(kFoldThreads) k_adj_outside(FoldArgs A, const float* bonus, int ckpt,
                                                               double* counts_out, double* unpaired_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<AdjSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = adj_setup(sm, A, D);
    const ParamView<float> P{sm->tabs.blob};
    const AdjView V = adj_view(A, D, ckpt);
    const LseAcc32 sr{};
    const int L = D.L;
    const InTabs<float>& I = V.I;
    for (int e = threadIdx.x; e < CF_BLOB_LEN; e += blockDim.x) {
        sm->cnt_lo[e] = 0ull;
        sm->cnt_hi[e] = 0u;
    }
    for (int k = threadIdx.x; k < 2 * (L + 2); k += blockDim.x) V.PD[k] = 0ull;
    // exterior outside F5o (one warp)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        if (lane == 0) V.F5o[L] = 0.0f;
        __syncwarp();
        for (int k = L - 1; k >= 0; --k) {
            float acc = CF_NEG32;
            for (int j0 = L; j0 >= k + 2; j0 -= 32) {
                const int j = j0 - lane;
                bool ok = false;
                float term = 0.0f;
                if (j >= k + 2 && Q.pairable(k + 1, j)) {
                    const float fcin = I.FC[I.at(k + 1, j - 1)];
                    if (fcin > CF_HALF32) {
                        const float jA = junctionA_rev<LseAcc32>(P, L, Q, k, j);
                        term = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(V.F5o[j], P.ep()), P.bp(Q.s[k + 1], Q.s[j])), jA), fcin);
                        ok = true;
                    }
                }
                unsigned msk = __ballot_sync(0xffffffffu, ok);
                while (msk) {
                    const int t = __ffs(msk) - 1;
                    msk &= msk - 1;
                    acc = sr.plus(acc, __shfl_sync(0xffffffffu, term, t));
                }
            }
            acc = sr.plus(acc, __fadd_rn(__fadd_rn(V.F5o[k + 1], P.eu()), ubon(V.U, k + 1)));
            if (lane == 0) V.F5o[k] = acc;
            __syncwarp();
        }
    }
    __syncthreads();
    const Counter C{sm, V.PD, L + 2};
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float Z = I.F5[L];
    // step t: outside values of diagonal t, counts of diagonal t + 1 (final since the last step)
    for (int t = L; t >= -1; --t) {
        const int no = t >= 0 ? L + 1 - t : 0;
        const int nc = t + 1 <= L ? L - t : 0;
        for (int c = warp; c < no + nc; c += kAdjWarps) {   // one warp per cell
            if (c < no) outside_cell(sm, P, Q, V, c, c + t, lane);
            else count_cell(sm, P, Q, V, C, Z, c - no, c - no + t + 1, lane);
        }
        __syncthreads();
    }
    // exterior transitions: threads over j
    for (int j = 1 + threadIdx.x; j <= L; j += blockDim.x) {
        const float f5o = V.F5o[j];
        if (!(f5o > CF_HALF32)) continue;
        {
            const unsigned long long v =
                fixp(expf(__fsub_rn(__fadd_rn(f5o, __fadd_rn(__fadd_rn(I.F5[j - 1], P.eu()), ubon(V.U, j))), Z)));
            C.add(CF_OFF_EU, v);
        }
        for (int k = 0; k < j; ++k) {
            if (!Q.pairable(k + 1, j)) continue;
            const float fcin = I.FC[I.at(k + 1, j - 1)], f5k = I.F5[k];
            if (!(fcin > CF_HALF32) || !(f5k > CF_HALF32)) continue;
            const float jA = junctionA_rev<LseAcc32>(P, L, Q, k, j);
            const unsigned long long v = fixp(expf(__fsub_rn(
                __fadd_rn(f5o, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(f5k, fcin), P.ep()), P.bp(Q.s[k + 1], Q.s[j])), jA)),
                Z)));
            count_jA_rev(C, Q, L, k, j, v);
            C.add(CF_OFF_EP, v);
            C.add(CF_OFF_BP + Q.s[k + 1] * 5 + Q.s[j], v);
        }
    }
    __syncthreads();
    double* out = counts_out + (int64_t)D.idx * CF_BLOB_LEN;
    for (int e = threadIdx.x; e < CF_BLOB_LEN; e += blockDim.x) out[e] = fixp_value((double)sm->cnt_hi[e], sm->cnt_lo[e]);
    // P(k unpaired) = 1 - P(k paired): 2^62 minus the 128-bit sum, exact, then rounded once
    const int n = L + 2;
    for (int k = 1 + threadIdx.x; k <= L; k += blockDim.x) {
        const unsigned long long pl = V.PD[k], one = 1ull << 62;
        const long long ph = (long long)V.PD[n + k];
        const unsigned long long lo = one - pl;
        const long long hi = -ph - (pl > one ? 1 : 0);
        unpaired_out[D.seq_off + k - 1] = fixp_value((double)hi, lo);
    }
    if (threadIdx.x == 0 && A.logz) A.logz[D.idx] = Z;
}

size_t adj_smem_bytes(int Lmax) { return sizeof(AdjSmem) + 2 * (size_t)((Lmax + 2 + 15) & ~15); }
int64_t adj_arena_words(int L, int ckpt) { return arena_adj(L, ckpt).total; }
int adj_auto_checkpoint(int L) { return L < 512 ? 1 : 8; }

}  // namespace cf
