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
// enumerates all transitions and adds that probability, in FP64, to each
// parameter-table entry the transition's score uses.  Inside and outside are
// evaluated with the accurate float32 log-sum-exp so the counts are the
// derivative of the logZ that cf_logz reports (within float32 rounding).
//
// Kernels: one CTA per sequence, threads over the cells of a span (the shape
// of the plain path); the transition pass runs over all cells at once and
// accumulates into shared-memory FP64 counters with atomics.
#include "cf_kernels.h"
#include "cf_outside.cuh"

namespace cf {
namespace {

struct AdjSmem {
    SmemTabs<float> tabs;
};

// Adjoint arena: the FP32 arena plus the inside FM2 table, the FP64 prefix of
// the bonus and the FP64 difference array of the unpaired probabilities.
struct ArenaAdj {
    Arena32 a;
    int64_t FM2, U, UD, total;
};
__host__ __device__ __forceinline__ ArenaAdj arena_adj(int L) {
    ArenaAdj r;
    r.a = arena32(L);
    r.FM2 = r.a.total;
    r.U = r.FM2 + pad32(tri_size(L));               // words; doubles: 2 words each
    r.UD = r.U + 2 * pad32(L + 2);
    r.total = r.UD + 2 * pad32(L + 2);
    return r;
}

struct AdjView {
    InTabs<float> I;
    OutTabs O;
    float* FM2;
    const double* U;   // U[k] = sum_{t<=k} u_t
    double* UD;        // unpaired-probability difference array
    int m;
};

__device__ __forceinline__ AdjView adj_view(const FoldArgs& A, const SeqDesc& D) {
    const ArenaAdj r = arena_adj(D.L);
    float* base = A.ws + D.ws_off;
    AdjView V;
    V.I.FC = base + r.a.FC; V.I.FM = base + r.a.FM; V.I.FM1 = base + r.a.FM1; V.I.F5 = base + r.a.F5;
    V.I.m = D.L + 1;
    V.I.sized(D.L);
    V.O.FC = V.I.FC; V.O.FM = V.I.FM; V.O.FM1 = V.I.FM1; V.O.F5 = V.I.F5;
    V.O.FCo = base + r.a.FCo; V.O.FMo = base + r.a.FMo; V.O.FM1o = base + r.a.FM1o; V.O.FM2o = base + r.a.FM2o;
    V.O.F5o = base + r.a.F5o; V.O.m = D.L + 1;
    V.O.sized(D.L);
    V.FM2 = base + r.FM2;
    V.U = reinterpret_cast<const double*>(base + r.U);
    V.UD = reinterpret_cast<double*>(base + r.UD);
    V.m = D.L + 1;
    return V;
}

// bonus of the unpaired stretch (lo, hi]: U[hi] - U[lo]
__device__ __forceinline__ float bon(const double* U, int lo, int hi) { return (float)(U[hi] - U[lo]); }
__device__ __forceinline__ float ubon(const double* U, int k) { return (float)(U[k] - U[k - 1]); }

__device__ __forceinline__ SeqView adj_setup(AdjSmem* sm, const FoldArgs& A, SeqDesc& D) {
    D = A.descs[blockIdx.x];
    load_tabs(&sm->tabs, A.blob32);
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

}  // namespace

// ---------------------------------------------------------------------------
// Inside with bonus (accurate float32 log-sum-exp)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kFoldThreads) k_adj_inside(FoldArgs A, const float* bonus) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<AdjSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = adj_setup(sm, A, D);
    const ParamView<float> P{sm->tabs.blob};
    const AdjView V = adj_view(A, D);
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
    for (int d = 0; d <= L; ++d) {
        for (int i = threadIdx.x; i + d <= L; i += blockDim.x) {
            const int j = i + d, at = tri_off(d, m) + i;
            const bool fm_region = (0 < i) && (i + 2 <= j) && (j < L);
            const bool fc_cell = (0 < i) && (j < L) && Q.pairable(i, j + 1);
            float fm2 = CF_NEG32;
            if (fm_region)
                for (int k = i + 1; k < j; ++k) {
                    const float a = T.FM1[T.at(i, k)], b = T.FM[T.at(k, j)];
                    if (a > CF_HALF32 && b > CF_HALF32) fm2 = sr.plus(fm2, __fadd_rn(a, b));
                }
            V.FM2[at] = fm2;
            float fc = CF_NEG32;
            if (fc_cell) {
                const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
                const float jB = sm->tabs.jB[idx4(si, sj1, si1, sj)];
                float acc = __fadd_rn(__fadd_rn(jB, P.hp(d <= DHP ? d : DHP)), bon(V.U, i, j));
                const int pmax = (i + CMAX < j) ? i + CMAX : j;
                for (int p = i; p <= pmax; ++p) {
                    int qmin = p + 2;
                    if (p - i + j - CMAX > qmin) qmin = p - i + j - CMAX;
                    for (int q = j; q >= qmin; --q) {
                        if (!Q.pairable(p + 1, q)) continue;
                        const float inner = T.FC[T.at(p + 1, q - 1)];
                        if (!(inner > CF_HALF32)) continue;
                        const float e = single_e(P, &sm->tabs, Q, i, j, p, q);
                        const float b = __fadd_rn(bon(V.U, i, p), bon(V.U, q, j));
                        acc = sr.plus(acc, __fadd_rn(__fadd_rn(e, inner), b));
                    }
                }
                if (fm2 > CF_HALF32) {
                    const float jA = junctionA<LseAcc32>(P, L, Q, i, j);
                    acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(fm2, jA), P.mp()), P.mb()));
                }
                fc = acc;
            }
            T.FC[at] = fc;
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
            T.FM1[at] = fm1;
            T.FM[at] = fm;
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
// Outside with bonus (gathers; any order -- no bitwise target)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kFoldThreads) k_adj_outside(FoldArgs A, const float* bonus) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<AdjSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = adj_setup(sm, A, D);
    const ParamView<float> P{sm->tabs.blob};
    const AdjView V = adj_view(A, D);
    const LseAcc32 sr{};
    const int L = D.L, m = L + 1;
    const OutTabs& T = V.O;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        if (lane == 0) T.F5o[L] = 0.0f;
        __syncwarp();
        for (int k = L - 1; k >= 0; --k) {
            float acc = CF_NEG32;
            for (int j0 = L; j0 >= k + 2; j0 -= 32) {
                const int j = j0 - lane;
                bool ok = false;
                float term = 0.0f;
                if (j >= k + 2 && Q.pairable(k + 1, j)) {
                    const float fcin = T.FC[T.at(k + 1, j - 1)];
                    if (fcin > CF_HALF32) {
                        const float jA = junctionA_rev<LseAcc32>(P, L, Q, k, j);
                        term = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(T.F5o[j], P.ep()), P.bp(Q.s[k + 1], Q.s[j])), jA), fcin);
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
            acc = sr.plus(acc, __fadd_rn(__fadd_rn(T.F5o[k + 1], P.eu()), ubon(V.U, k + 1)));
            if (lane == 0) T.F5o[k] = acc;
            __syncwarp();
        }
    }
    __syncthreads();
    for (int d = L; d >= 0; --d) {
        for (int a = threadIdx.x; a + d <= L; a += blockDim.x) {
            const int b = a + d, at = tri_off(d, m) + a;
            const bool fm_region = (0 < a) && (a + 2 <= b) && (b < L);
            float fmo = CF_NEG32, fm1o = CF_NEG32;
            if (fm_region) {
                float acc = CF_NEG32;
                for (int i = 1; i < a; ++i) {
                    const float src = T.FM2o[T.at(i, b)], f1 = T.FM1[T.at(i, a)];
                    if (src > CF_HALF32 && f1 > CF_HALF32) acc = sr.plus(acc, __fadd_rn(src, f1));
                }
                if (b + 1 < L) acc = sr.plus(acc, __fadd_rn(__fadd_rn(T.FMo[T.at(a, b + 1)], P.mu()), ubon(V.U, b + 1)));
                fmo = acc;
                acc = CF_NEG32;
                if (a >= 2) acc = sr.plus(acc, __fadd_rn(__fadd_rn(T.FM1o[T.at(a - 1, b)], P.mu()), ubon(V.U, a)));
                for (int j = b + 1; j < L; ++j) {
                    const float src = T.FM2o[T.at(a, j)], fmk = T.FM[T.at(b, j)];
                    if (src > CF_HALF32 && fmk > CF_HALF32) acc = sr.plus(acc, __fadd_rn(src, fmk));
                }
                fm1o = sr.plus(acc, fmo);
            }
            T.FMo[at] = fmo;
            T.FM1o[at] = fm1o;
            float fco = CF_NEG32;
            if (0 < a && b < L && Q.pairable(a, b + 1)) {
                const int sa = Q.s[a], sb1 = Q.s[b + 1];
                float acc = CF_NEG32;
                const float f5k = T.F5[a - 1];
                if (f5k > CF_HALF32) {
                    const float jA = junctionA_rev<LseAcc32>(P, L, Q, a - 1, b + 1);
                    acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(T.F5o[b + 1], P.ep()), P.bp(sa, sb1)), jA), f5k));
                }
                if (a >= 2 && b + 1 < L) {
                    const float jAji = junctionA_rev<LseAcc32>(P, L, Q, a - 1, b + 1);
                    acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(T.FM1o[T.at(a - 1, b + 1)], jAji), P.mp()), P.bp(sa, sb1)));
                }
                for (int l1 = 0; l1 <= CMAX; ++l1) {
                    const int i = a - 1 - l1;
                    if (i < 1) break;
                    for (int l2 = 0; l1 + l2 <= CMAX; ++l2) {
                        const int j = b + 1 + l2;
                        if (j >= L) break;
                        if (!Q.pairable(i, j + 1)) continue;
                        const float src = T.FCo[T.at(i, j)];
                        if (!(src > CF_HALF32)) continue;
                        const float e = single_e(P, &sm->tabs, Q, i, j, a - 1, b + 1);
                        const float bb = __fadd_rn(bon(V.U, i, a - 1), bon(V.U, b + 1, j));
                        acc = sr.plus(acc, __fadd_rn(__fadd_rn(src, e), bb));
                    }
                }
                fco = acc;
            }
            T.FCo[at] = fco;
            float fm2o = CF_NEG32;
            if (fm_region) fm2o = sr.plus(fm2o, fmo);
            if (fco > CF_HALF32) {
                const float jA = junctionA<LseAcc32>(P, L, Q, a, b);
                fm2o = sr.plus(fm2o, __fadd_rn(__fadd_rn(__fadd_rn(fco, jA), P.mp()), P.mb()));
            }
            T.FM2o[at] = fm2o;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Transition probabilities -> FP64 expected counts
// ---------------------------------------------------------------------------
namespace {

struct Counter {
    double* c;    // shared [CF_BLOB_LEN]
    double* ud;   // global unpaired difference array [L + 2]
    __device__ __forceinline__ void add(int e, double v) const { atomicAdd(c + e, v); }
    // positions (lo, hi] unpaired with probability v
    __device__ __forceinline__ void unp(int lo, int hi, double v) const {
        if (hi <= lo) return;
        atomicAdd(ud + lo + 1, v);
        atomicAdd(ud + hi + 1, -v);
    }
};

// jA(i, j) of the pair (i, j+1): entries hc[s_i][s_j+1], dl (i < L), dr (j > 0)
__device__ __forceinline__ void count_jA(const Counter& C, const SeqView& Q, int L, int i, int j, double v) {
    C.add(CF_OFF_HC + Q.s[i] * 5 + Q.s[j + 1], v);
    if (i < L) C.add(CF_OFF_DL + (Q.s[i] * 5 + Q.s[j + 1]) * 5 + Q.s[i + 1], v);
    if (j > 0) C.add(CF_OFF_DR + (Q.s[i] * 5 + Q.s[j + 1]) * 5 + Q.s[j], v);
}
// jA(j, i) of the pair (i+1, j)
__device__ __forceinline__ void count_jA_rev(const Counter& C, const SeqView& Q, int L, int i, int j, double v) {
    C.add(CF_OFF_HC + Q.s[j] * 5 + Q.s[i + 1], v);
    if (j < L) C.add(CF_OFF_DL + (Q.s[j] * 5 + Q.s[i + 1]) * 5 + Q.s[j + 1], v);
    if (i > 0) C.add(CF_OFF_DR + (Q.s[j] * 5 + Q.s[i + 1]) * 5 + Q.s[i], v);
}
// jB = hc + tm of the pair (a, b+1) with inner neighbours (a+1, b)
__device__ __forceinline__ void count_jB(const Counter& C, int sa, int sb1, int sa1, int sb, double v) {
    C.add(CF_OFF_HC + sa * 5 + sb1, v);
    C.add(CF_OFF_TM + idx4(sa, sb1, sa1, sb), v);
}

}  // namespace

__global__ void __launch_bounds__(kFoldThreads) k_adj_counts(FoldArgs A, const float* bonus, double* counts_out,
                                                              double* unpaired_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<AdjSmem*>(smem_raw);
    __shared__ double cnt[CF_BLOB_LEN];
    SeqDesc D;
    const SeqView Q = adj_setup(sm, A, D);
    const ParamView<float> P{sm->tabs.blob};
    const AdjView V = adj_view(A, D);
    const int L = D.L, m = L + 1;
    for (int e = threadIdx.x; e < CF_BLOB_LEN; e += blockDim.x) cnt[e] = 0.0;
    for (int k = threadIdx.x; k < L + 2; k += blockDim.x) V.UD[k] = 0.0;
    __syncthreads();
    const Counter C{cnt, V.UD};
    const InTabs<float>& I = V.I;
    const OutTabs& O = V.O;
    const float Z = I.F5[L];
    auto prob = [&](float x) -> double { return (double)expf(__fsub_rn(x, Z)); };
    const int ncell = (int)tri_size(L);
    // cells (i, j) in diagonal-major order, all independent
    int i = threadIdx.x;
    for (int d = 0; d <= L; ++d) {
        const int cntd = m - d;
        for (; i < cntd; i += blockDim.x) {
            const int j = i + d;
            const bool fm_region = (0 < i) && (i + 2 <= j) && (j < L);
            if (0 < i && j < L && Q.pairable(i, j + 1)) {
                const float fco = O.FCo[tri_off(d, m) + i];
                if (fco > CF_HALF32) {
                    const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
                    const float jB = sm->tabs.jB[idx4(si, sj1, si1, sj)];
                    // hairpin
                    {
                        const int hl = d <= DHP ? d : DHP;
                        const double v = prob(__fadd_rn(fco, __fadd_rn(__fadd_rn(jB, P.hp(hl)), bon(V.U, i, j))));
                        count_jB(C, si, sj1, si1, sj, v);
                        C.add(CF_OFF_HPCUM + hl, v);
                        C.unp(i, j, v);
                    }
                    // single-branch loops
                    double outer_jB = 0.0;
                    const int pmax = (i + CMAX < j) ? i + CMAX : j;
                    for (int p = i; p <= pmax; ++p) {
                        int qmin = p + 2;
                        if (p - i + j - CMAX > qmin) qmin = p - i + j - CMAX;
                        for (int q = j; q >= qmin; --q) {
                            if (!Q.pairable(p + 1, q)) continue;
                            const float inner = I.FC[I.at(p + 1, q - 1)];
                            if (!(inner > CF_HALF32)) continue;
                            const float e = single_e(P, &sm->tabs, Q, i, j, p, q);
                            const float bb = __fadd_rn(bon(V.U, i, p), bon(V.U, q, j));
                            const double v = prob(__fadd_rn(fco, __fadd_rn(__fadd_rn(e, inner), bb)));
                            const int l1 = p - i, l2 = j - q;
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
                            C.unp(i, p, v);
                            C.unp(q, j, v);
                        }
                    }
                    if (outer_jB != 0.0) count_jB(C, si, sj1, si1, sj, outer_jB);
                    // multiloop closed by (i, j+1)
                    const float fm2 = V.FM2[tri_off(d, m) + i];
                    if (fm2 > CF_HALF32) {
                        const float jA = junctionA<LseAcc32>(P, L, Q, i, j);
                        const double v = prob(__fadd_rn(fco, __fadd_rn(__fadd_rn(__fadd_rn(fm2, jA), P.mp()), P.mb())));
                        count_jA(C, Q, L, i, j, v);
                        C.add(CF_OFF_MP, v);
                        C.add(CF_OFF_MB, v);
                    }
                }
            }
            if (fm_region) {
                const float fm1o = O.FM1o[tri_off(d, m) + i];
                if (fm1o > CF_HALF32) {
                    const float fin = I.FC[I.at(i + 1, j - 1)];
                    if (Q.pairable(i + 1, j) && fin > CF_HALF32) {
                        const float jAji = junctionA_rev<LseAcc32>(P, L, Q, i, j);
                        const double v = prob(__fadd_rn(fm1o, __fadd_rn(__fadd_rn(__fadd_rn(fin, jAji), P.mp()),
                                                                           P.bp(Q.s[i + 1], Q.s[j]))));
                        count_jA_rev(C, Q, L, i, j, v);
                        C.add(CF_OFF_MP, v);
                        C.add(CF_OFF_BP + Q.s[i + 1] * 5 + Q.s[j], v);
                    }
                    const float ext = I.FM1[I.at(i + 1, j)];
                    if (ext > CF_HALF32) {
                        const double v = prob(__fadd_rn(fm1o, __fadd_rn(__fadd_rn(ext, P.mu()), ubon(V.U, i + 1))));
                        C.add(CF_OFF_MU, v);
                        C.unp(i, i + 1, v);
                    }
                }
                const float fmo = O.FMo[tri_off(d, m) + i];
                const float prev = I.FM[I.at(i, j - 1)];
                if (fmo > CF_HALF32 && prev > CF_HALF32) {
                    const double v = prob(__fadd_rn(fmo, __fadd_rn(__fadd_rn(prev, P.mu()), ubon(V.U, j))));
                    C.add(CF_OFF_MU, v);
                    C.unp(j - 1, j, v);
                }
            }
        }
        i -= cntd;
    }
    (void)ncell;
    // exterior transitions: threads over j
    for (int j = 1 + threadIdx.x; j <= L; j += blockDim.x) {
        const float f5o = O.F5o[j];
        if (!(f5o > CF_HALF32)) continue;
        {
            const double v = prob(__fadd_rn(f5o, __fadd_rn(__fadd_rn(I.F5[j - 1], P.eu()), ubon(V.U, j))));
            C.add(CF_OFF_EU, v);
            C.unp(j - 1, j, v);
        }
        for (int k = 0; k < j; ++k) {
            if (!Q.pairable(k + 1, j)) continue;
            const float fcin = I.FC[I.at(k + 1, j - 1)], f5k = I.F5[k];
            if (!(fcin > CF_HALF32) || !(f5k > CF_HALF32)) continue;
            const float jA = junctionA_rev<LseAcc32>(P, L, Q, k, j);
            const double v = prob(__fadd_rn(f5o, __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(f5k, fcin), P.ep()),
                                                                      P.bp(Q.s[k + 1], Q.s[j])), jA)));
            count_jA_rev(C, Q, L, k, j, v);
            C.add(CF_OFF_EP, v);
            C.add(CF_OFF_BP + Q.s[k + 1] * 5 + Q.s[j], v);
        }
    }
    __syncthreads();
    double* out = counts_out + (int64_t)D.idx * CF_BLOB_LEN;
    for (int e = threadIdx.x; e < CF_BLOB_LEN; e += blockDim.x) out[e] = cnt[e];
    if (threadIdx.x == 0) {
        double acc = 0.0;
        for (int k = 1; k <= L; ++k) {
            acc += V.UD[k];
            unpaired_out[D.seq_off + k - 1] = acc;
        }
        if (A.logz) A.logz[D.idx] = Z;
    }
}

size_t adj_smem_bytes(int Lmax) { return sizeof(AdjSmem) + 2 * (size_t)((Lmax + 2 + 15) & ~15); }
int64_t adj_arena_words(int L) { return arena_adj(L).total; }

}  // namespace cf
