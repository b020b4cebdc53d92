// cf_plain.cu -- the plain path: the reference's launch shape for every phase.
//
// One CTA per sequence; on each span (diagonal) the threads stride over the
// cells i (gpu.py:79-82), one __syncthreads between spans; a cell walks its
// whole single-branch window (31 x 31 / 2 positions) and tests pairability
// position by position, as gpu.py:92-116 does, and evaluates FM2 in the cell.
// The outside pass and the posterior (which the reference only has on the
// CPU, cpu.py:680-819) follow the same shape.  This is the baseline the
// batched kernels (cf_warp.cu, cf_fold.cu) are measured against; all paths
// produce bitwise the same tables.
#include "cf_kernels.h"
#include "cf_mea.cuh"
#include "cf_outside.cuh"

namespace cf {
namespace {

// One inside cell (i, j).  Writes FC, FM1, FM at (i, j) (the semiring zero
// where the reference leaves the cell at NEG).
template <class S>
__device__ __forceinline__ void plain_inside_cell(const S& sr, const SmemTabs<typename S::Real>* __restrict__ tb,
                                            const SeqView& Q, const InTabs<typename S::Real>& T, int i,
                                            int j) {
    using R = typename S::Real;
    const ParamView<R> P{tb->blob};
    const int L = Q.L, m = T.m, d = j - i;
    const R NEG = S::neg(), HALF = S::half();
    const bool fm_region = (0 < i) && (i + 2 <= j) && (j < L);
    const bool fc_cell = (0 < i) && (j < L) && Q.pairable(i, j + 1);

    // FM2[i][j] = (+)_{i<k<j} FM1[i][k] * FM[k][j]   (cpu.py:179-183)
    R fm2 = NEG;
    if (fm_region || fc_cell) {
        int o1 = tri_off(1, m) + i;          // FM1[i][i+1]
        int o2 = tri_off(d - 1, m) + i + 1;  // FM[i+1][j]
        for (int k = i + 1; k < j; ++k) {
            const R a = T.FM1[o1];
            const R b = T.FM[o2];
            if (a > HALF && b > HALF) fm2 = sr.plus(fm2, S::add(a, b));
            const int s1 = k - i;            // span of FM1[i][k]
            o1 += m - s1;                    // -> span s1 + 1
            o2 += 1 - (m - (j - k - 1));     // FM[k+1][j]: span j-k-1, one position right
        }
    }

    // FC[i][j], pair (i, j+1)   (cpu.py:185-230)
    R fc = NEG;
    if (fc_cell) {
        const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
        const R jB = tb->jB[idx4(si, sj1, si1, sj)];
        R acc = sr.plus(NEG, S::add(jB, P.hp(d <= DHP ? d : DHP)));
        const int pmax = (i + CMAX < j) ? i + CMAX : j;
        for (int p = i; p <= pmax; ++p) {
            const int l1 = p - i;
            int qmin = p + 2;
            const int alt = l1 + j - CMAX;
            if (alt > qmin) qmin = alt;
            const int a = p + 1;
            const int pca = Q.pc[a], sa = Q.s[a], sp = Q.s[p];
            for (int q = j; q >= qmin; --q) {
                if (!pairable_codes(pca, Q.pc[q])) continue;
                const R inner = T.FC[tri_off(q - 1 - a, m) + a];
                if (!(inner > HALF)) continue;
                const int l2 = j - q;
                R e;
                if (l1 == 0 && l2 == 0) {
                    e = S::add(P.bp(si1, sj), P.stack(si, sj1, si1, sj));
                } else {
                    const int sq = Q.s[q];
                    const R jB2 = tb->jB[idx4(sq, sa, Q.s[q + 1], sp)];
                    R snuc = R(0);
                    if (l1 == 0 && l2 == 1) snuc = P.b01(sj);
                    else if (l1 == 1 && l2 == 0) snuc = P.b01(si1);
                    else if (l1 == 1 && l2 == 1) snuc = P.i11(si1, sj);
                    e = S::add(S::add(S::add(S::add(P.cs(l1, l2), P.bp(sa, sq)), jB), jB2), snuc);
                }
                acc = sr.plus(acc, S::add(e, inner));
            }
        }
        if (fm2 > HALF) {
            const R jA = junctionA<S>(P, L, Q, i, j);
            acc = sr.plus(acc, S::add(S::add(S::add(fm2, jA), P.mp()), P.mb()));
        }
        fc = acc;
    }
    T.FC[T.at(i, j)] = fc;

    // FM1[i][j]   (cpu.py:232-246)
    R fm1 = NEG;
    if (fm_region) {
        R acc = NEG;
        const R fin = T.FC[T.at(i + 1, j - 1)];
        if (Q.pairable(i + 1, j) && fin > HALF) {
            const R jAji = junctionA_rev<S>(P, L, Q, i, j);
            acc = sr.plus(acc, S::add(S::add(S::add(fin, jAji), P.mp()), P.bp(Q.s[i + 1], Q.s[j])));
        }
        const R ext = T.FM1[T.at(i + 1, j)];
        if (ext > HALF) acc = sr.plus(acc, S::add(ext, P.mu()));
        fm1 = acc;
    }
    T.FM1[T.at(i, j)] = fm1;

    // FM[i][j]   (cpu.py:248-257)
    R fm = NEG;
    if (fm_region) {
        R acc = NEG;
        if (fm2 > HALF) acc = sr.plus(acc, fm2);
        const R prev = T.FM[T.at(i, j - 1)];
        if (prev > HALF) acc = sr.plus(acc, S::add(prev, P.mu()));
        if (fm1 > HALF) acc = sr.plus(acc, fm1);
        fm = acc;
    }
    T.FM[T.at(i, j)] = fm;
}


// One outside cell (a, b): FMo, FM1o, FCo, FM2o.  Needs every cell of larger
// span finished.
__device__ __forceinline__ void plain_outside_cell(const Lse32& sr, const SmemTabs<float>* __restrict__ tb,
                                             const SeqView& Q, const OutTabs& T, int a, int b) {
    const ParamView<float> P{tb->blob};
    const int L = Q.L, m = T.m;
    const bool fm_region = (0 < a) && (a + 2 <= b) && (b < L);

    // FMo[a][b]: FM2o distribution of sources (i, b), i = 1 .. a-1 ascending,
    // k = a (cpu.py:753-758); then block 1 of source (a, b+1):
    // FMo[a][b] (+)= FMo[a][b+1] + mu (cpu.py:705).
    float fmo = CF_NEG32;
    if (fm_region) {
        float acc = CF_NEG32;
        for (int i = 1; i < a; ++i) {
            const float src = T.FM2o[T.at(i, b)];
            const float f1 = T.FM1[T.at(i, a)];
            if (src > CF_HALF32 && f1 > CF_HALF32) acc = sr.plus(acc, __fadd_rn(src, f1));
        }
        if (b + 1 < L) acc = sr.plus(acc, __fadd_rn(T.FMo[T.at(a, b + 1)], P.mu()));
        fmo = acc;
    }
    T.FMo[T.at(a, b)] = fmo;

    // FM1o[a][b]: block 2 of source (a-1, b): FM1o[a-1][b] + mu (cpu.py:715);
    // FM2o distribution of sources (a, j), j = L-1 .. b+1, k = b (cpu.py:756);
    // block 1 of source (a, b): (+)= FMo[a][b] (cpu.py:706).
    float fm1o = CF_NEG32;
    if (fm_region) {
        float acc = CF_NEG32;
        if (a >= 2) acc = sr.plus(acc, __fadd_rn(T.FM1o[T.at(a - 1, b)], P.mu()));
        for (int j = L - 1; j > b; --j) {
            const float src = T.FM2o[T.at(a, j)];
            const float fmk = T.FM[T.at(b, j)];
            if (src > CF_HALF32 && fmk > CF_HALF32) acc = sr.plus(acc, __fadd_rn(src, fmk));
        }
        acc = sr.plus(acc, fmo);
        fm1o = acc;
    }
    T.FM1o[T.at(a, b)] = fm1o;

    // FCo[a][b], pair (a, b+1):
    //  1. exterior term of the F5o phase, k = a-1, j = b+1 (cpu.py:695-699);
    //  2. sources (i, j) = (a-1-l1, b+1+l2) of the main loop, i ascending
    //     (l1 = 30 .. 0), j descending (l2 = 30-l1 .. 0); the source (a-1, b+1)
    //     first contributes through FM1o (block 2, cpu.py:708-714) and then
    //     through its single-branch loop (block 3, cpu.py:717-745).
    float fco = CF_NEG32;
    if (0 < a && b < L && Q.pairable(a, b + 1)) {
        const int sa = Q.s[a], sb1 = Q.s[b + 1];
        float acc = CF_NEG32;
        {
            const float f5k = T.F5[a - 1];
            if (f5k > CF_HALF32) {
                const float jA = junctionA_rev<Lse32>(P, L, Q, a - 1, b + 1);
                const float temp = __fadd_rn(__fadd_rn(__fadd_rn(T.F5o[b + 1], P.ep()), P.bp(sa, sb1)), jA);
                acc = sr.plus(acc, __fadd_rn(temp, f5k));
            }
        }
        const float bp_ab = P.bp(sa, sb1);
        // jB of the inner pair (p+1, q) = (a, b+1): hc[s[q]][s[p+1]] + tm[s[q]][s[p+1]][s[q+1]][s[p]]
        const float jB2 = tb->jB[idx4(sb1, sa, Q.s[b + 2 <= L + 1 ? b + 2 : L + 1], Q.s[a - 1])];
        for (int l1 = CMAX; l1 >= 0; --l1) {
            const int i = a - 1 - l1;
            if (i < 1) continue;
            const int si = Q.s[i], si1 = Q.s[i + 1], pci = Q.pc[i];
            for (int l2 = CMAX - l1; l2 >= 0; --l2) {
                const int j = b + 1 + l2;
                if (j >= L) continue;
                if (l1 == 0 && l2 == 0) {
                    const float jAji = junctionA_rev<Lse32>(P, L, Q, a - 1, b + 1);
                    acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(T.FM1o[T.at(a - 1, b + 1)], jAji), P.mp()), bp_ab));
                }
                if (!pairable_codes(pci, Q.pc[j + 1])) continue;
                const float src = T.FCo[T.at(i, j)];
                if (!(src > CF_HALF32)) continue;
                const int sj = Q.s[j];
                float e;
                if (l1 == 0 && l2 == 0) {
                    e = __fadd_rn(P.bp(si1, sj), P.stack(si, Q.s[j + 1], si1, sj));
                } else {
                    const float jBij = tb->jB[idx4(si, Q.s[j + 1], si1, sj)];
                    float snuc = 0.0f;
                    if (l1 == 0 && l2 == 1) snuc = P.b01(sj);
                    else if (l1 == 1 && l2 == 0) snuc = P.b01(si1);
                    else if (l1 == 1 && l2 == 1) snuc = P.i11(si1, sj);
                    e = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(P.cs(l1, l2), bp_ab), jBij), jB2), snuc);
                }
                acc = sr.plus(acc, __fadd_rn(src, e));
            }
        }
        fco = acc;
    }
    T.FCo[T.at(a, b)] = fco;

    // FM2o[a][b] (cpu.py:702-704, 746-751)
    float fm2o = CF_NEG32;
    if (fm_region) fm2o = sr.plus(fm2o, fmo);
    if (fco > CF_HALF32) {   // implies 0 < a, b < L, pairable(a, b+1)
        const float jA = junctionA<Lse32>(P, L, Q, a, b);
        fm2o = sr.plus(fm2o, __fadd_rn(__fadd_rn(__fadd_rn(fco, jA), P.mp()), P.mb()));
    }
    T.FM2o[T.at(a, b)] = fm2o;
}


// Posterior of the pair (a, b), 1 <= a < b <= L (cpu.py:760-819).  The
// reference adds fexp32 terms into POST[a][b] from sources (i, j) =
// (a-1-l1, b+l2) visited i descending (l1 = 0 ..), j ascending (l2 = 0 ..);
// source (a-1, b) adds its multiloop (FM1o) term right after its stacking
// term; the exterior term comes last.  Returns the clipped value.
__device__ __forceinline__ float plain_posterior_cell(const SmemTabs<float>* __restrict__ tb, const PolyTables* pt,
                                                const SeqView& Q, const OutTabs& T, float Z, int a, int b) {
    const ParamView<float> P{tb->blob};
    const int L = Q.L;
    if (!Q.pairable(a, b)) return 0.0f;
    const float fcin = T.FC[T.at(a, b - 1)];
    if (!(fcin > CF_HALF32)) return 0.0f;
    const int sa = Q.s[a], sb = Q.s[b];
    const float bp_ab = P.bp(sa, sb);
    // jB of the inner pair (p+1, q) = (a, b)
    const float jB2 = tb->jB[idx4(sb, sa, Q.s[b + 1], Q.s[a - 1])];
    float post = 0.0f;
    for (int l1 = 0; l1 <= CMAX; ++l1) {
        const int i = a - 1 - l1;
        if (i < 1) break;
        const int si = Q.s[i], si1 = Q.s[i + 1], pci = Q.pc[i];
        for (int l2 = 0; l1 + l2 <= CMAX; ++l2) {
            const int j = b + l2;
            if (j >= L) break;
            if (pairable_codes(pci, Q.pc[j + 1])) {
                const float outside = __fsub_rn(T.FCo[T.at(i, j)], Z);
                if (outside > CF_HALF32) {
                    const int sj = Q.s[j];
                    float e;
                    if (l1 == 0 && l2 == 0) {
                        e = __fadd_rn(__fadd_rn(__fadd_rn(outside, P.bp(si1, sj)), P.stack(si, Q.s[j + 1], si1, sj)), fcin);
                    } else {
                        const float jBij = tb->jB[idx4(si, Q.s[j + 1], si1, sj)];
                        float snuc = 0.0f;
                        if (l1 == 0 && l2 == 1) snuc = P.b01(sj);
                        else if (l1 == 1 && l2 == 0) snuc = P.b01(si1);
                        else if (l1 == 1 && l2 == 1) snuc = P.i11(si1, sj);
                        e = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(outside, jBij), P.cs(l1, l2)), fcin), bp_ab), jB2), snuc);
                    }
                    post = __fadd_rn(post, fexp32(pt, e));
                }
            }
            if (l1 == 0 && l2 == 0) {
                const float fo = T.FM1o[T.at(a - 1, b)];
                if (fo > CF_HALF32) {
                    const float jAji = junctionA_rev<Lse32>(P, L, Q, a - 1, b);
                    const float x = __fsub_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(fo, fcin), jAji), P.mp()), bp_ab), Z);
                    post = __fadd_rn(post, fexp32(pt, x));
                }
            }
        }
    }
    const float outside = __fsub_rn(T.F5o[b], Z);
    const float f5k = T.F5[a - 1];
    if (outside > CF_HALF32 && f5k > CF_HALF32) {
        const float jA = junctionA_rev<Lse32>(P, L, Q, a - 1, b);
        const float x = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(outside, f5k), fcin), P.ep()), bp_ab), jA);
        post = __fadd_rn(post, fexp32(pt, x));
    }
    if (post < 0.0f) post = 0.0f;
    else if (post > 1.0f) post = 1.0f;
    return post;
}


struct PlainSmem {
    SmemTabs<float> tabs;
    PolyTables poly;
};

// Shared set-up: tables and the sequence codes of descs[blockIdx.x].
__device__ __forceinline__ SeqView plain_setup(PlainSmem* sm, const FoldArgs& A, SeqDesc& D) {
    D = A.descs[blockIdx.x];
    load_tabs(&sm->tabs, A.blob32);
    load_poly_tables(&sm->poly);
    int8_t* s = reinterpret_cast<int8_t*>(sm + 1);
    const int stride = (D.L + 2 + 15) & ~15;
    int8_t* pc = s + stride;
    encode_seq(A.seqs, A.mask, D.seq_off, D.L, s, pc);
    __syncthreads();
    return SeqView{s, pc, D.L};
}

__device__ __forceinline__ OutTabs plain_out(const FoldArgs& A, const SeqDesc& D) {
    const Arena32 a = arena32(D.L);
    float* base = A.ws + D.ws_off;
    OutTabs T;
    T.FC = base + a.FC; T.FM = base + a.FM; T.FM1 = base + a.FM1; T.F5 = base + a.F5;
    T.FCo = base + a.FCo; T.FMo = base + a.FMo; T.FM1o = base + a.FM1o; T.FM2o = base + a.FM2o;
    T.F5o = base + a.F5o;
    T.m = D.L + 1;
    T.sized(D.L);
    return T;
}

}  // namespace

__global__ void __launch_bounds__(kFoldThreads) k_plain_inside32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<PlainSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = plain_setup(sm, A, D);
    const Lse32 sr{&sm->poly};
    const Arena32 ar = arena32(D.L);
    float* base = A.ws + D.ws_off;
    InTabs<float> T;
    T.FC = base + ar.FC; T.FM = base + ar.FM; T.FM1 = base + ar.FM1; T.F5 = base + ar.F5; T.m = D.L + 1;
    T.sized(D.L);
    for (int d = 0; d <= D.L; ++d) {
        for (int i = threadIdx.x; i + d <= D.L; i += blockDim.x) plain_inside_cell<Lse32>(sr, &sm->tabs, Q, T, i, i + d);
        __syncthreads();
    }
    if (threadIdx.x < 32) exterior_warp<Lse32>(sr, &sm->tabs, Q, T);
}

__global__ void __launch_bounds__(kFoldThreads) k_plain_outside32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<PlainSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = plain_setup(sm, A, D);
    const Lse32 sr{&sm->poly};
    const OutTabs T = plain_out(A, D);
    if (threadIdx.x < 32) exterior_outside_warp(sr, &sm->tabs, Q, T);
    __syncthreads();
    for (int d = D.L; d >= 0; --d) {
        for (int a = threadIdx.x; a + d <= D.L; a += blockDim.x) plain_outside_cell(sr, &sm->tabs, Q, T, a, a + d);
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kFoldThreads) k_plain_posterior32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<PlainSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = plain_setup(sm, A, D);
    const OutTabs T = plain_out(A, D);
    const int L = D.L, m = L + 1;
    const float Z = T.F5[L];
    float* POST = T.FMo;
    float* dense = A.post_out ? A.post_out + A.post_offs[D.idx] : nullptr;
    int a = threadIdx.x;
    for (int d = 0; d <= L; ++d) {
        const int cnt = m - d;
        for (; a < cnt; a += blockDim.x) {
            const int b = a + d;
            float v = 0.0f;
            if (a >= 1 && d >= 1) v = plain_posterior_cell(&sm->tabs, &sm->poly, Q, T, Z, a, b);
            POST[tri_off(d, m) + a] = v;
            if (dense != nullptr && a >= 1) {
                dense[(int64_t)(a - 1) * L + (b - 1)] = v;
                if (d >= 1) dense[(int64_t)(b - 1) * L + (a - 1)] = 0.0f;
            }
        }
        a -= cnt;
    }
    if (A.logz != nullptr && threadIdx.x == 0) A.logz[D.idx] = Z;
}

__global__ void __launch_bounds__(kFoldThreads) k_plain_mea32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<PlainSmem*>(smem_raw);
    SeqDesc D;
    const SeqView Q = plain_setup(sm, A, D);
    const int L = D.L;
    const Arena32 ar = arena32(L);
    float* base = A.ws + D.ws_off;
    const float two_g = __fmul_rn(2.0f, A.gamma);
    for (int i = 1 + threadIdx.x; i <= L; i += blockDim.x) base[ar.up + i] = mea_unpaired(base + ar.FMo, L, two_g, i);
    __syncthreads();
    for (int d = 0; d <= L; ++d) {
        for (int i = threadIdx.x; i + d <= L; i += blockDim.x)
            mea_cell(Q, base + ar.FMo, base + ar.up, base + ar.FM2o, reinterpret_cast<int*>(base + ar.FM), L, i, i + d);
        __syncthreads();
    }
    char* out = A.structs + D.seq_off;
    for (int t = threadIdx.x; t < L; t += blockDim.x) out[t] = '.';
    __syncthreads();
    if (threadIdx.x == 0) {
        int* qi = reinterpret_cast<int*>(base + ar.queue);
        mea_traceback(reinterpret_cast<const int*>(base + ar.FM), L, qi, qi + 2 * L + 4, out, A.status);
    }
}

size_t plain_smem_bytes(int Lmax) { return sizeof(PlainSmem) + 2 * (size_t)((Lmax + 2 + 15) & ~15); }

}  // namespace cf
