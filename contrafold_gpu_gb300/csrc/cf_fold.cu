// cf_fold.cu -- fold kernels: inside (FP32 / FP64 / Viterbi), outside,
// posterior, MEA decode, Viterbi traceback.
//
// Scheduling: a CTA owns a GROUP of sequences (group size 1 is the plain
// one-sequence-per-block path of gpu.py:508; larger groups are the batched
// path).  The CTA walks the DP diagonals of all its sequences in lock step;
// on each diagonal the threads take the cells of every sequence of the group
// (flattened), so short diagonals of several sequences fill the warps that one
// sequence alone would leave idle.  One __syncthreads separates diagonals.
#include "cf_kernels.h"
#include "cf_outside.cuh"

namespace cf {

// ---------------------------------------------------------------------------
// Shared-memory carve-up
// ---------------------------------------------------------------------------
template <typename R>
struct SmemFold {
    SmemTabs<R> tabs;
    PolyTables poly;
    int L[kMaxGroup];
    int64_t ws[kMaxGroup];
    int64_t soff[kMaxGroup];
    int idx[kMaxGroup];
    int n;        // sequences in this group
    int Lmax;
};

template <typename R>
__device__ __forceinline__ int8_t* seq_smem(SmemFold<R>* sm) {
    return reinterpret_cast<int8_t*>(sm + 1);
}

// Load tables + group descriptors + encoded sequences.  Returns stride of
// the per-sequence code arrays.
template <typename R>
__device__ __forceinline__ int setup_group(SmemFold<R>* sm, const FoldArgs& A, const R* __restrict__ gblob) {
    const int g0 = blockIdx.x * A.group;
    const int ng = min(A.group, A.n - g0);
    if (threadIdx.x == 0) {
        int lmax = 0;
        for (int g = 0; g < ng; ++g) {
            const SeqDesc D = A.descs[g0 + g];
            sm->L[g] = D.L;
            sm->ws[g] = D.ws_off;
            sm->soff[g] = D.seq_off;
            sm->idx[g] = D.idx;
            lmax = max(lmax, D.L);
        }
        sm->n = ng;
        sm->Lmax = lmax;
    }
    load_tabs(&sm->tabs, gblob);
    load_poly_tables(&sm->poly);
    __syncthreads();
    const int stride = (sm->Lmax + 2 + 15) & ~15;
    int8_t* base = seq_smem(sm);
    for (int g = 0; g < sm->n; ++g)
        encode_seq(A.seqs, A.mask, sm->soff[g], sm->L[g], base + (2 * g) * stride, base + (2 * g + 1) * stride);
    __syncthreads();
    return stride;
}

template <typename R>
__device__ __forceinline__ SeqView seq_view(SmemFold<R>* sm, int stride, int g) {
    int8_t* base = seq_smem(sm);
    return SeqView{base + (2 * g) * stride, base + (2 * g + 1) * stride, sm->L[g]};
}

// Walk diagonals d = d_begin .. d_end (step +1 or -1) over all sequences of
// the group; call f(g, i, i + d) for every cell.
template <typename R, typename F>
__device__ __forceinline__ void wavefront(SmemFold<R>* sm, int d_begin, int d_end, int step, F f) {
    const int ng = sm->n;
    for (int d = d_begin; step > 0 ? d <= d_end : d >= d_end; d += step) {
        // cells of sequence g on diagonal d: L_g + 1 - d (if positive)
        int total = 0;
        for (int g = 0; g < ng; ++g) total += max(0, sm->L[g] + 1 - d);
        for (int c = threadIdx.x; c < total; c += blockDim.x) {
            int g = 0, r = c;
            while (true) {
                const int cnt = max(0, sm->L[g] + 1 - d);
                if (r < cnt) break;
                r -= cnt;
                ++g;
            }
            f(g, r, r + d);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Inside (any semiring): fills FC/FM/FM1/F5 of each sequence; writes logZ.
// ---------------------------------------------------------------------------
template <class S>
__device__ __forceinline__ InTabs<typename S::Real> in_tabs(const FoldArgs& A, int64_t ws_off, int L) {
    using R = typename S::Real;
    InTabs<R> T;
    if (sizeof(R) == 4) {
        const Arena32 a = arena32(L);
        float* base = A.ws + ws_off;
        T.FC = reinterpret_cast<R*>(base + a.FC);
        T.FM = reinterpret_cast<R*>(base + a.FM);
        T.FM1 = reinterpret_cast<R*>(base + a.FM1);
        T.F5 = reinterpret_cast<R*>(base + a.F5);
    } else {
        const Arena64 a = arena64(L);
        double* base = reinterpret_cast<double*>(A.ws + ws_off);
        T.FC = reinterpret_cast<R*>(base + a.FC);
        T.FM = reinterpret_cast<R*>(base + a.FM);
        T.FM1 = reinterpret_cast<R*>(base + a.FM1);
        T.F5 = reinterpret_cast<R*>(base + a.F5);
    }
    T.m = L + 1;
    return T;
}

template <class S>
__device__ __forceinline__ S make_sr(const PolyTables* pt);
template <>
__device__ __forceinline__ Lse32 make_sr<Lse32>(const PolyTables* pt) { return Lse32{pt}; }
template <>
__device__ __forceinline__ LseAcc32 make_sr<LseAcc32>(const PolyTables*) { return LseAcc32{}; }
template <>
__device__ __forceinline__ Lse64 make_sr<Lse64>(const PolyTables*) { return Lse64{}; }
template <>
__device__ __forceinline__ Max64 make_sr<Max64>(const PolyTables*) { return Max64{}; }

template <class S>
__device__ __forceinline__ void inside_group(SmemFold<typename S::Real>* sm, const FoldArgs& A, int stride) {
    using R = typename S::Real;
    const S sr = make_sr<S>(&sm->poly);
    wavefront(sm, 0, sm->Lmax, +1, [&](int g, int i, int j) {
        const SeqView Q = seq_view(sm, stride, g);
        const InTabs<R> T = in_tabs<S>(A, sm->ws[g], Q.L);
        inside_cell<S>(sr, &sm->tabs, Q, T, i, j);
    });
    // exterior recurrence: one warp per sequence
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int g = warp; g < sm->n; g += nwarps) {
        const SeqView Q = seq_view(sm, stride, g);
        const InTabs<R> T = in_tabs<S>(A, sm->ws[g], Q.L);
        exterior_warp<S>(sr, &sm->tabs, Q, T);
    }
    __syncthreads();
}

__global__ void __launch_bounds__(kFoldThreads) k_inside32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    const int stride = setup_group(sm, A, A.blob32);
    inside_group<Lse32>(sm, A, stride);
    if (A.logz != nullptr)
        for (int g = threadIdx.x; g < sm->n; g += blockDim.x) {
            const InTabs<float> T = in_tabs<Lse32>(A, sm->ws[g], sm->L[g]);
            A.logz[sm->idx[g]] = T.F5[sm->L[g]];
        }
}

// Same recurrence with accurate float32 log-sum-exp: logZ_batch and the sampler.
__global__ void __launch_bounds__(kFoldThreads) k_inside32acc(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    const int stride = setup_group(sm, A, A.blob32);
    inside_group<LseAcc32>(sm, A, stride);
    if (A.logz != nullptr)
        for (int g = threadIdx.x; g < sm->n; g += blockDim.x) {
            const InTabs<float> T = in_tabs<LseAcc32>(A, sm->ws[g], sm->L[g]);
            A.logz[sm->idx[g]] = T.F5[sm->L[g]];
        }
}

__global__ void __launch_bounds__(kFoldThreads) k_inside64(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<double>*>(smem_raw);
    const int stride = setup_group(sm, A, A.blob64);
    inside_group<Lse64>(sm, A, stride);
    for (int g = threadIdx.x; g < sm->n; g += blockDim.x) {
        const InTabs<double> T = in_tabs<Lse64>(A, sm->ws[g], sm->L[g]);
        A.logz64[sm->idx[g]] = T.F5[sm->L[g]];
    }
}

// ---------------------------------------------------------------------------
// Outside + posterior + MEA (FP32)
// ---------------------------------------------------------------------------
__device__ __forceinline__ OutTabs out_tabs(const FoldArgs& A, int64_t ws_off, int L) {
    const Arena32 a = arena32(L);
    float* base = A.ws + ws_off;
    OutTabs T;
    T.FC = base + a.FC; T.FM = base + a.FM; T.FM1 = base + a.FM1; T.F5 = base + a.F5;
    T.FCo = base + a.FCo; T.FMo = base + a.FMo; T.FM1o = base + a.FM1o; T.FM2o = base + a.FM2o;
    T.F5o = base + a.F5o;
    T.m = L + 1;
    return T;
}

__global__ void __launch_bounds__(kFoldThreads) k_outside32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    const int stride = setup_group(sm, A, A.blob32);
    const Lse32 sr{&sm->poly};
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int g = warp; g < sm->n; g += nwarps) {
        const SeqView Q = seq_view(sm, stride, g);
        exterior_outside_warp(sr, &sm->tabs, Q, out_tabs(A, sm->ws[g], Q.L));
    }
    __syncthreads();
    wavefront(sm, sm->Lmax, 0, -1, [&](int g, int a, int b) {
        const SeqView Q = seq_view(sm, stride, g);
        outside_cell(sr, &sm->tabs, Q, out_tabs(A, sm->ws[g], Q.L), a, b);
    });
}

// Posterior of every pair; POST goes to the FMo slot (triangular) and, for
// cf_bpp, densely into the caller's L x L matrix.
__global__ void __launch_bounds__(kFoldThreads) k_posterior32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    const int stride = setup_group(sm, A, A.blob32);
    for (int g = 0; g < sm->n; ++g) {
        const SeqView Q = seq_view(sm, stride, g);
        const int L = Q.L, m = L + 1;
        const OutTabs T = out_tabs(A, sm->ws[g], L);
        const float Z = T.F5[L];
        float* POST = T.FMo;
        float* dense = A.post_out ? A.post_out + A.post_offs[sm->idx[g]] : nullptr;
        // all cells (a, b) with 0 <= a <= b <= L, walked in triangular order
        // (thread t takes flattened cells t, t + blockDim, ...); pairs need 1 <= a < b
        int a = threadIdx.x;
        for (int d = 0; d <= L; ++d) {
            const int cnt = m - d;
            for (; a < cnt; a += blockDim.x) {
                const int b = a + d;
                float v = 0.0f;
                if (a >= 1 && d >= 1) v = posterior_cell(&sm->tabs, &sm->poly, Q, T, Z, a, b);
                POST[tri_off(d, m) + a] = v;
                if (dense != nullptr && a >= 1) {
                    dense[(int64_t)(a - 1) * L + (b - 1)] = v;
                    if (d >= 1) dense[(int64_t)(b - 1) * L + (a - 1)] = 0.0f;
                }
            }
            a -= cnt;
        }
    }
    if (A.logz != nullptr)
        for (int g = threadIdx.x; g < sm->n; g += blockDim.x) {
            const OutTabs T = out_tabs(A, sm->ws[g], sm->L[g]);
            A.logz[sm->idx[g]] = T.F5[sm->L[g]];
        }
}

// MEA decode (cpu.py:823-895): unpaired weights, gamma-weighted max-plus DP
// with the reference's strict-'>' candidate order, BFS traceback.
__global__ void __launch_bounds__(kFoldThreads) k_mea32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    const int stride = setup_group(sm, A, A.blob32);
    const float two_g = __fmul_rn(2.0f, A.gamma);
    // unpaired scores up[i] = (1 - sum_j POST) / (2 gamma), j ascending
    for (int g = 0; g < sm->n; ++g) {
        const int L = sm->L[g], m = L + 1;
        const Arena32 ar = arena32(L);
        float* base = A.ws + sm->ws[g];
        const float* POST = base + ar.FMo;
        float* up = base + ar.up;
        for (int i = 1 + threadIdx.x; i <= L; i += blockDim.x) {
            float u = 1.0f;
            for (int jj = 1; jj < i; ++jj) u = __fsub_rn(u, POST[tri_off(i - jj, m) + jj]);
            for (int jj = i + 1; jj <= L; ++jj) u = __fsub_rn(u, POST[tri_off(jj - i, m) + i]);
            up[i] = __fdiv_rn(u, two_g);
        }
    }
    __syncthreads();
    wavefront(sm, 0, sm->Lmax, +1, [&](int g, int i, int j) {
        const SeqView Q = seq_view(sm, stride, g);
        const int m = Q.L + 1;
        const Arena32 ar = arena32(Q.L);
        float* base = A.ws + sm->ws[g];
        const float* POST = base + ar.FMo;
        const float* up = base + ar.up;
        float* score = base + ar.FM2o;
        int* tb = reinterpret_cast<int*>(base + ar.FM);
        const int c = tri_off(j - i, m) + i;
        if (i == j) { score[c] = 0.0f; tb[c] = 0; return; }
        float best = -1.0f;
        int arg = -1;
        float v = __fadd_rn(up[i + 1], score[tri_off(j - i - 1, m) + i + 1]);
        if (v > best) { best = v; arg = 1; }
        v = __fadd_rn(up[j], score[tri_off(j - 1 - i, m) + i]);
        if (v > best) { best = v; arg = 2; }
        if (i + 2 <= j) {
            if (Q.pairable(i + 1, j)) {
                v = __fadd_rn(POST[tri_off(j - i - 1, m) + i + 1], score[tri_off(j - i - 2, m) + i + 1]);
                if (v > best) { best = v; arg = 3; }
            }
            int o1 = tri_off(1, m) + i;               // score[i][i+1]
            int o2 = tri_off(j - i - 1, m) + i + 1;   // score[i+1][j]
            for (int k = i + 1; k < j; ++k) {
                v = __fadd_rn(score[o1], score[o2]);
                if (v > best) { best = v; arg = k + 4; }
                o1 += m - (k - i);
                o2 += 1 - (m - (j - k - 1));
            }
        }
        score[c] = best;
        tb[c] = arg;
    });
    // traceback: one thread per sequence
    for (int g = 0; g < sm->n; ++g) {
        const int L = sm->L[g];
        char* out = A.structs + sm->soff[g];
        for (int t = threadIdx.x; t < L; t += blockDim.x) out[t] = '.';
    }
    __syncthreads();
    for (int g = threadIdx.x; g < sm->n; g += blockDim.x) {
        const int L = sm->L[g], m = L + 1;
        const Arena32 ar = arena32(L);
        float* base = A.ws + sm->ws[g];
        const int* tb = reinterpret_cast<const int*>(base + ar.FM);
        int* qi = reinterpret_cast<int*>(base + ar.queue);
        int* qj = qi + 2 * L + 4;
        char* out = A.structs + sm->soff[g];
        int head = 0, tail = 1;
        qi[0] = 0; qj[0] = L;
        while (head < tail) {
            const int i = qi[head], j = qj[head];
            ++head;
            const int t = tb[tri_off(j - i, m) + i];
            if (t <= 0) continue;
            if (tail + 2 > 2 * L + 4) { atomicExch(A.status, CF_EDEVICE); break; }
            if (t == 1) { qi[tail] = i + 1; qj[tail] = j; ++tail; }
            else if (t == 2) { qi[tail] = i; qj[tail] = j - 1; ++tail; }
            else if (t == 3) {
                out[i] = '(';        // pair (i+1, j), 1-based
                out[j - 1] = ')';
                qi[tail] = i + 1; qj[tail] = j - 1; ++tail;
            } else {
                const int k = t - 4;
                qi[tail] = i; qj[tail] = k; ++tail;
                qi[tail] = k; qj[tail] = j; ++tail;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Viterbi: max-plus inside in FP64, then the reference's EPS first-match
// traceback (cpu.py:396-501), one thread per sequence.
// ---------------------------------------------------------------------------
__device__ void viterbi_traceback(const SmemTabs<double>* tb, const SeqView& Q, const InTabs<double>& T,
                                  int* st, char* out, int* status) {
    const ParamView<double> P{tb->blob};
    const int L = Q.L;
    const double EPS = 1e-6, HALF = CF_HALF64;
    const int cap = 4 * L + 16;
    int *st_t = st, *st_i = st + cap, *st_j = st + 2 * cap;
    int sp = 0;
#define VPUSH(tt, ii, jj)                                   \
    do {                                                    \
        if (sp >= cap) { atomicExch(status, CF_EDEVICE); return; } \
        st_t[sp] = (tt); st_i[sp] = (ii); st_j[sp] = (jj); ++sp; \
    } while (0)
    VPUSH(0, 0, L);
    while (sp > 0) {
        --sp;
        const int typ = st_t[sp], i = st_i[sp], j = st_j[sp];
        if (typ == 0) {
            if (j == 0) continue;
            const double val = T.F5[j];
            bool done = false;
            if (T.F5[j - 1] > HALF && fabs(__dadd_rn(__dadd_rn(T.F5[j - 1], P.eu()), -val)) <= EPS) {
                VPUSH(0, 0, j - 1);
                done = true;
            }
            if (!done) {
                for (int k = 0; k < j; ++k) {
                    if (!Q.pairable(k + 1, j)) continue;
                    const double fcin = T.FC[T.at(k + 1, j - 1)];
                    if (!(fcin > HALF) || !(T.F5[k] > HALF)) continue;
                    const double jA = junctionA_rev<Max64>(P, L, Q, k, j);
                    const double v = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(T.F5[k], fcin), P.ep()), P.bp(Q.s[k + 1], Q.s[j])), jA);
                    if (fabs(__dadd_rn(v, -val)) <= EPS) {
                        out[k] = '(';
                        out[j - 1] = ')';
                        VPUSH(1, k + 1, j - 1);
                        VPUSH(0, 0, k);
                        break;
                    }
                }
            }
        } else if (typ == 1) {
            const double val = T.FC[T.at(i, j)];
            const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
            const double jB = tb->jB[idx4(si, sj1, si1, sj)];
            const int d = j - i;
            bool done = fabs(__dadd_rn(__dadd_rn(jB, P.hp(d <= DHP ? d : DHP)), -val)) <= EPS;
            if (!done) {
                const int pmax = (i + CMAX < j) ? i + CMAX : j;
                for (int p = i; p <= pmax && !done; ++p) {
                    const int l1 = p - i;
                    int qmin = p + 2;
                    const int alt = l1 + j - CMAX;
                    if (alt > qmin) qmin = alt;
                    for (int q = j; q >= qmin; --q) {
                        const int l2 = j - q;
                        if (!Q.pairable(p + 1, q)) continue;
                        const double inner = T.FC[T.at(p + 1, q - 1)];
                        if (!(inner > HALF)) continue;
                        double e;
                        if (p == i && q == j) {
                            e = __dadd_rn(P.bp(si1, sj), P.stack(si, sj1, si1, sj));
                        } else {
                            const double jB2 = tb->jB[idx4(Q.s[q], Q.s[p + 1], Q.s[q + 1], Q.s[p])];
                            double snuc = 0.0;
                            if (l1 == 0 && l2 == 1) snuc = P.b01(sj);
                            else if (l1 == 1 && l2 == 0) snuc = P.b01(si1);
                            else if (l1 == 1 && l2 == 1) snuc = P.i11(si1, sj);
                            e = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(P.cs(l1, l2), P.bp(Q.s[p + 1], Q.s[q])), jB), jB2), snuc);
                        }
                        if (fabs(__dadd_rn(__dadd_rn(e, inner), -val)) <= EPS) {
                            out[p] = '(';
                            out[q - 1] = ')';
                            VPUSH(1, p + 1, q - 1);
                            done = true;
                            break;
                        }
                    }
                }
            }
            if (!done) {
                const double jA = junctionA<Max64>(P, L, Q, i, j);
                for (int k = i + 1; k < j; ++k) {
                    const double f1 = T.FM1[T.at(i, k)], fm = T.FM[T.at(k, j)];
                    if (f1 > HALF && fm > HALF &&
                        fabs(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(f1, fm), jA), P.mp()), P.mb()), -val)) <= EPS) {
                        VPUSH(3, i, k);
                        VPUSH(2, k, j);
                        break;
                    }
                }
            }
        } else if (typ == 2) {
            const double val = T.FM[T.at(i, j)];
            bool done = false;
            for (int k = i + 1; k < j; ++k) {
                const double f1 = T.FM1[T.at(i, k)], fm = T.FM[T.at(k, j)];
                if (f1 > HALF && fm > HALF && fabs(__dadd_rn(__dadd_rn(f1, fm), -val)) <= EPS) {
                    VPUSH(3, i, k);
                    VPUSH(2, k, j);
                    done = true;
                    break;
                }
            }
            const double prev = T.FM[T.at(i, j - 1)];
            if (!done && prev > HALF && fabs(__dadd_rn(__dadd_rn(prev, P.mu()), -val)) <= EPS) {
                VPUSH(2, i, j - 1);
                done = true;
            }
            const double f1 = T.FM1[T.at(i, j)];
            if (!done && f1 > HALF && fabs(__dadd_rn(f1, -val)) <= EPS) VPUSH(3, i, j);
        } else {
            const double val = T.FM1[T.at(i, j)];
            bool done = false;
            if (Q.pairable(i + 1, j)) {
                const double fin = T.FC[T.at(i + 1, j - 1)];
                if (fin > HALF) {
                    const double jAji = junctionA_rev<Max64>(P, L, Q, i, j);
                    const double v = __dadd_rn(__dadd_rn(__dadd_rn(fin, jAji), P.mp()), P.bp(Q.s[i + 1], Q.s[j]));
                    if (fabs(__dadd_rn(v, -val)) <= EPS) {
                        out[i] = '(';
                        out[j - 1] = ')';
                        VPUSH(1, i + 1, j - 1);
                        done = true;
                    }
                }
            }
            const double ext = T.FM1[T.at(i + 1, j)];
            if (!done && ext > HALF && fabs(__dadd_rn(__dadd_rn(ext, P.mu()), -val)) <= EPS) VPUSH(3, i + 1, j);
        }
    }
#undef VPUSH
}

__global__ void __launch_bounds__(kFoldThreads) k_viterbi64(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<double>*>(smem_raw);
    const int stride = setup_group(sm, A, A.blob64);
    inside_group<Max64>(sm, A, stride);
    for (int g = 0; g < sm->n; ++g) {
        const int L = sm->L[g];
        char* out = A.structs + sm->soff[g];
        for (int t = threadIdx.x; t < L; t += blockDim.x) out[t] = '.';
    }
    __syncthreads();
    for (int g = threadIdx.x; g < sm->n; g += blockDim.x) {
        const SeqView Q = seq_view(sm, stride, g);
        const InTabs<double> T = in_tabs<Max64>(A, sm->ws[g], Q.L);
        const Arena64 ar = arena64(Q.L);
        int* st = reinterpret_cast<int*>(reinterpret_cast<double*>(A.ws + sm->ws[g]) + ar.stack);
        viterbi_traceback(&sm->tabs, Q, T, st, A.structs + sm->soff[g], A.status);
    }
}

// ---------------------------------------------------------------------------
size_t fold_smem_bytes(int Lmax, int group, bool fp64) {
    const size_t head = fp64 ? sizeof(SmemFold<double>) : sizeof(SmemFold<float>);
    const size_t stride = (size_t)((Lmax + 2 + 15) & ~15);
    return head + 2 * stride * group;
}

}  // namespace cf
