// cf_fold.cu -- fold kernels: inside (FP32 / FP64 / Viterbi), outside,
// posterior, MEA decode, Viterbi traceback.
//
// Scheduling: a CTA owns a GROUP of sequences (group size 1 is the plain
// one-sequence-per-block path of gpu.py:508; larger groups are the batched
// path).  The CTA walks the DP diagonals of all its sequences in lock step;
// on each diagonal the threads take the cells of every sequence of the group
// (flattened), so short diagonals of several sequences fill the warps that one
// sequence alone would leave idle.  One barrier separates diagonals.  The
// cluster kernels give a group to the CTAs of a thread-block cluster instead
// of one CTA (a "team", below), with a cluster barrier between diagonals.
#include "cf_kernels.h"
#include "cf_mea.cuh"
#include "cf_outside.cuh"

namespace cf {

// ---------------------------------------------------------------------------
// Shared memory: parameter tables + group descriptors, then per sequence the
// codes (s, pc) and the four partner bit sets.
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
    int gcap;     // sequences per CTA of the launch (sizes the dynamic region)
    int Lmax;
    int step_ctr[2];   // per-step work counters of step_items (by step parity)
};

__host__ __device__ __forceinline__ int code_stride(int Lmax) { return (Lmax + 2 + 15) & ~15; }

// Item index of this thread when one serial item per thread is dealt over the
// warps first: thread (w, lane) takes item w + lane * warps.  A bijection of
// [0, blockDim.x).
__device__ __forceinline__ int tb_index() {
    return (threadIdx.x >> 5) + (threadIdx.x & 31) * (int)(blockDim.x >> 5);
}

template <typename R>
__device__ __forceinline__ unsigned char* dyn_smem(SmemFold<R>* sm) {
    return reinterpret_cast<unsigned char*>(sm + 1);
}

template <typename R>
__device__ __forceinline__ SeqV seq_v(SmemFold<R>* sm, int g) {
    const int cs = code_stride(sm->Lmax), W = pb_words(sm->Lmax);
    unsigned char* base = dyn_smem(sm);
    const int8_t* s = reinterpret_cast<const int8_t*>(base + (2 * g) * cs);
    const int8_t* pc = reinterpret_cast<const int8_t*>(base + (2 * g + 1) * cs);
    const uint32_t* PB = reinterpret_cast<const uint32_t*>(base + 2 * sm->gcap * cs) + (size_t)g * 4 * W;
    return SeqV{s, pc, PB, W, sm->L[g]};
}

// Build codes and partner bit sets of the group's sequences (descriptors
// already in shared memory).
template <typename R>
__device__ __forceinline__ void build_group_seqs(SmemFold<R>* sm, const FoldArgs& A) {
    const int cs = code_stride(sm->Lmax), W = pb_words(sm->Lmax);
    unsigned char* base = dyn_smem(sm);
    for (int g = 0; g < sm->n; ++g) {
        int8_t* s = reinterpret_cast<int8_t*>(base + (2 * g) * cs);
        int8_t* pc = reinterpret_cast<int8_t*>(base + (2 * g + 1) * cs);
        uint32_t* PB = reinterpret_cast<uint32_t*>(base + 2 * sm->gcap * cs) + (size_t)g * 4 * W;
        build_seq(A.seqs, A.mask, sm->soff[g], sm->L[g], W, s, pc, PB);
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Teams: the threads that fold one group together.  CtaTeam is one CTA (the
// batched kernels); ClusterTeam is the C CTAs of a thread-block cluster, on C
// SMs, folding the same group (the latency kernels).  Work of a diagonal step
// is split over tid() / nthreads(); sync() separates steps (a cluster barrier
// with release / acquire semantics for ClusterTeam, so table cells written in
// global memory by one CTA are read by the others after it).  Every sync() is
// reached by all threads of the team: the loops around them run the same trip
// counts in every CTA (each CTA loads the same group descriptors), and
// rank-0-only work sits between two syncs, not around one.
// ---------------------------------------------------------------------------
struct CtaTeam {
    static constexpr int kChainPF = cf::kChainPF;   // bifurcation-chain register pipeline depth
    __device__ __forceinline__ int rank() const { return 0; }
    __device__ __forceinline__ int size() const { return 1; }
    __device__ __forceinline__ int tid() const { return threadIdx.x; }
    __device__ __forceinline__ int nthreads() const { return blockDim.x; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
};

// The fused MEA kernels' team: the chain pipeline one term shallower (fused MEA
// at 4 CTAs per SM, 64 registers: depth 2 / 3 / 4 / 6 measured 33.1k / 33.9k /
// 33.2k / 31.5k folds/s on 10,000 x 200 nt; the per-phase, BPP and sampling
// kernels keep kChainPF).
#ifndef CF_FUSED_MEA_CHAIN_PF
#define CF_FUSED_MEA_CHAIN_PF 3
#endif
struct CtaTeamMea : CtaTeam {
    static constexpr int kChainPF = CF_FUSED_MEA_CHAIN_PF;
};

struct ClusterTeam {
    static constexpr int kChainPF = CF_CLUSTER_CHAIN_PF;
    int r, c;   // rank of this CTA in the cluster, cluster size
    __device__ __forceinline__ int rank() const { return r; }
    __device__ __forceinline__ int size() const { return c; }
    __device__ __forceinline__ int tid() const { return r * blockDim.x + threadIdx.x; }
    __device__ __forceinline__ int nthreads() const { return c * blockDim.x; }
    __device__ __forceinline__ void sync() const {
        asm volatile("barrier.cluster.arrive.release;\n" ::: "memory");
        asm volatile("barrier.cluster.wait.acquire;\n" ::: "memory");
    }
};

__device__ __forceinline__ int cluster_ctarank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
    return (int)r;
}

// Load tables, group descriptors, sequence codes and partner bit sets of
// group `gi` (default: this CTA's index).
template <typename R>
__device__ __forceinline__ void setup_group(SmemFold<R>* sm, const FoldArgs& A, const R* __restrict__ gblob,
                                            int gi = -1) {
    const int g0 = (gi < 0 ? (int)blockIdx.x : gi) * A.group;
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
        sm->gcap = A.group;
        sm->Lmax = lmax;
    }
    load_tabs(&sm->tabs, gblob);
    load_poly_tables(&sm->poly);
    __syncthreads();
    build_group_seqs(sm, A);
}

// ---------------------------------------------------------------------------
// Arena views
// ---------------------------------------------------------------------------
template <typename R>
struct InView {
    InTabs<R> T;
    R* FB;        // two FM2 step buffers of stride fbs
    int fbs;
    PairList PLs;
};

template <typename R>
__device__ __forceinline__ InView<R> in_view(const FoldArgs& A, int64_t ws_off, int L) {
    InView<R> V;
    if (sizeof(R) == 4) {
        const Arena32 a = arena32(L);
        float* base = A.ws + ws_off;
        V.T.FC = reinterpret_cast<R*>(base + a.FC);
        V.T.FM = reinterpret_cast<R*>(base + a.FM);
        V.T.FM1 = reinterpret_cast<R*>(base + a.FM1);
        V.T.F5 = reinterpret_cast<R*>(base + a.F5);
        V.FB = reinterpret_cast<R*>(base + a.FB);
        V.PLs = plist_at(base + a.PL, L);
    } else {
        const Arena64 a = arena64(L);
        double* base = reinterpret_cast<double*>(A.ws + ws_off);
        V.T.FC = reinterpret_cast<R*>(base + a.FC);
        V.T.FM = reinterpret_cast<R*>(base + a.FM);
        V.T.FM1 = reinterpret_cast<R*>(base + a.FM1);
        V.T.F5 = reinterpret_cast<R*>(base + a.F5);
        V.FB = reinterpret_cast<R*>(base + a.FB);
        V.PLs = plist_at(A.ws + ws_off + a.PL, L);
    }
    V.T.m = L + 1;
    V.T.sized(L);
    V.fbs = (int)pad32(L + 2);
    return V;
}

__device__ __forceinline__ OutTabs out_tabs(const FoldArgs& A, int64_t ws_off, int L) {
    const Arena32 a = arena32(L);
    float* base = A.ws + ws_off;
    OutTabs T;
    T.FC = base + a.FC; T.FM = base + a.FM; T.FM1 = base + a.FM1; T.F5 = base + a.F5;
    T.FCo = base + a.FCo; T.FMo = base + a.FMo; T.FM1o = base + a.FM1o; T.FM2o = base + a.FM2o;
    T.F5o = base + a.F5o;
    T.m = L + 1;
    T.sized(L);
    return T;
}

__device__ __forceinline__ PairList plist_of(const FoldArgs& A, int64_t ws_off, int L) {
    return plist_at(A.ws + ws_off + arena32(L).PL, L);
}

// ---------------------------------------------------------------------------
// One pipelined step over the group: phase-B items (pairable cells of
// diagonal dB, from the pair lists) then phase-A items (every cell of
// diagonal dA).  The B block is padded to a multiple of 32 so that each warp
// holds one kind of item.  fB(g, i), fA(g, i) process one cell.
//
// Warps claim 32-item chunks from a shared counter (B chunks, the costlier
// window walks, come first), so a warp that drew cheap cells takes more and
// the step's barrier waits less for the slowest warp.  Step `t` uses counter
// t & 1 and clears the other one for step t + 1 (nobody uses it after the
// previous step's barrier); both start at zero (step_ctr_init).  In a cluster
// team the step's chunks are dealt round-robin to the CTAs (chunk k to rank
// k mod size) and each CTA's warps claim its chunks from its own counter.
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ void step_ctr_init(SmemFold<R>* sm) {
    if (threadIdx.x == 0) sm->step_ctr[0] = sm->step_ctr[1] = 0;
    __syncthreads();
}

template <typename R, class Team, typename GetPL, typename FB, typename FA>
__device__ __forceinline__ void step_items(SmemFold<R>* sm, const Team& tm, int t, int dB, int dA, GetPL getpl, FB fB, FA fA) {
    const int ng = sm->n;
    int NB = 0, NA = 0;
    for (int g = 0; g < ng; ++g) {
        const int L = sm->L[g];
        if (dB >= 0 && dB <= L - 2) {
            const PairList PLs = getpl(g);
            NB += PLs.poff[dB + 1] - PLs.poff[dB];
        }
        if (dA >= 0) NA += max(0, L + 1 - dA);
    }
    const int NB32 = (NB + 31) & ~31;
    const int total = NB32 + NA;
    int* ctr = &sm->step_ctr[t & 1];
    if (threadIdx.x == 0) sm->step_ctr[(t & 1) ^ 1] = 0;
    const int lane = threadIdx.x & 31;
    for (;;) {
        // the CTA's q-th chunk is chunk q * size + rank of the team's step
        int q = 0;
        if (lane == 0) q = atomicAdd(ctr, 1);
        q = __shfl_sync(0xffffffffu, q, 0);
        const int base = (q * tm.size() + tm.rank()) * 32;
        if (base >= total) break;
        const int c = base + lane;
        if (c >= total) continue;   // only in the last A chunk (the B block is whole warps)
        if (c < NB32) {
            // B items fill whole warps (NB32 is a multiple of 32): the lanes
            // holding a cell walk it together (see inside_B)
            const unsigned lanes = __ballot_sync(0xffffffffu, c < NB);
            if (c >= NB) continue;
            int r = c, g = 0;
            for (;; ++g) {
                const int L = sm->L[g];
                if (dB <= L - 2) {
                    const PairList PLs = getpl(g);
                    const int o = PLs.poff[dB], cnt = PLs.poff[dB + 1] - o;
                    if (r < cnt) { fB(g, (int)PLs.pl[o + r], lanes); break; }
                    r -= cnt;
                }
            }
        } else {
            int r = c - NB32, g = 0;
            for (;; ++g) {
                const int cnt = max(0, sm->L[g] + 1 - dA);
                if (r < cnt) { fA(g, r); break; }
                r -= cnt;
            }
        }
    }
    tm.sync();
}

// ---------------------------------------------------------------------------
// Inside (any semiring): pair lists, FC/FM/FM1 wavefront, F5.
// ---------------------------------------------------------------------------
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

template <class S, class Team = CtaTeam>
__device__ __forceinline__ void inside_group(SmemFold<typename S::Real>* sm, const FoldArgs& A, const Team tm = Team{}) {
    using R = typename S::Real;
    const S sr = make_sr<S>(&sm->poly);
    if (tm.rank() == 0)
        for (int g = 0; g < sm->n; ++g) build_plist(seq_v(sm, g), in_view<R>(A, sm->ws[g], sm->L[g]).PLs);
    if (tm.size() > 1) tm.sync();   // the pair lists, for every CTA of the team
    auto getpl = [&](int g) { return in_view<R>(A, sm->ws[g], sm->L[g]).PLs; };
    step_ctr_init(sm);
    for (int t = 0; t <= sm->Lmax + 1; ++t) {
        step_items(
            sm, tm, t, t - 1, t <= sm->Lmax ? t : -1, getpl,
            [&](int g, int i, unsigned lanes) {   // phase B(t-1): FC of a pairable cell
                const SeqV Q = seq_v(sm, g);
                const InView<R> V = in_view<R>(A, sm->ws[g], Q.L);
                const R fm2 = V.FB[((t - 1) & 1) * V.fbs + i];
                inside_B<S>(sr, &sm->tabs, Q, V.T, i, i + t - 1, fm2, lanes);
            },
            [&](int g, int i) {   // phase A(t): FM2, FM1, FM
                const SeqV Q = seq_v(sm, g);
                const InView<R> V = in_view<R>(A, sm->ws[g], Q.L);
                V.FB[(t & 1) * V.fbs + i] = inside_A<S, Team::kChainPF>(sr, &sm->tabs, Q, V.T, i, i + t);
            });
    }
    // exterior recurrence: one warp per sequence
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (tm.rank() == 0)
        for (int g = warp; g < sm->n; g += nwarps)
            exterior_warp<S>(sr, &sm->tabs, seq_v(sm, g), in_view<R>(A, sm->ws[g], sm->L[g]).T);
    tm.sync();
}

template <int NT>
__global__ void __launch_bounds__(NT, NT == kFoldThreads ? kFoldMinBlocks : 1) k_inside32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    setup_group(sm, A, A.blob32);
    inside_group<Lse32>(sm, A);
    if (A.logz != nullptr)
        for (int g = threadIdx.x; g < sm->n; g += blockDim.x)
            A.logz[sm->idx[g]] = in_view<float>(A, sm->ws[g], sm->L[g]).T.F5[sm->L[g]];
}

// Same recurrence with accurate float32 log-sum-exp: logZ_batch and the sampler.
template <int NT>
__global__ void __launch_bounds__(NT, NT == kFoldThreads ? kFoldMinBlocks : 1) k_inside32acc(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    setup_group(sm, A, A.blob32);
    inside_group<LseAcc32>(sm, A);
    if (A.logz != nullptr)
        for (int g = threadIdx.x; g < sm->n; g += blockDim.x)
            A.logz[sm->idx[g]] = in_view<float>(A, sm->ws[g], sm->L[g]).T.F5[sm->L[g]];
}

__global__ void __launch_bounds__(kFoldThreads, kFoldMinBlocks) k_inside64(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<double>*>(smem_raw);
    setup_group(sm, A, A.blob64);
    inside_group<Lse64>(sm, A);
    for (int g = threadIdx.x; g < sm->n; g += blockDim.x)
        A.logz64[sm->idx[g]] = in_view<double>(A, sm->ws[g], sm->L[g]).T.F5[sm->L[g]];
}

// ---------------------------------------------------------------------------
// Outside + posterior + MEA (FP32)
// ---------------------------------------------------------------------------
template <class Team = CtaTeam>
__device__ __forceinline__ void outside_group(SmemFold<float>* sm, const FoldArgs& A, const Team tm = Team{}) {
    const Lse32 sr{&sm->poly};
    const int warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (tm.rank() == 0)
        for (int g = warp; g < sm->n; g += nwarps)
            exterior_outside_warp(sr, &sm->tabs, seq_v(sm, g), out_tabs(A, sm->ws[g], sm->L[g]));
    tm.sync();
    auto getpl = [&](int g) { return plist_of(A, sm->ws[g], sm->L[g]); };
    step_ctr_init(sm);
    for (int t = sm->Lmax; t >= 0; --t) {
        step_items(
            sm, tm, t, t - 1, t, getpl,
            [&](int g, int a, unsigned lanes) {   // phase B(t-1): FCo of a pairable cell
                const SeqV Q = seq_v(sm, g);
                outside_B(sr, &sm->tabs, Q, out_tabs(A, sm->ws[g], Q.L), a, a + t - 1, lanes);
            },
            [&](int g, int a) {   // phase A(t): FMo, FM1o, FM2o
                const SeqV Q = seq_v(sm, g);
                outside_A_merged<Team::kChainPF>(sr, &sm->tabs, Q, out_tabs(A, sm->ws[g], Q.L), a, a + t);
            });
    }
}

// Posterior of every pairable pair; POST goes to the FMo slot (triangular,
// zero elsewhere) and, for cf_bpp, densely into the caller's L x L matrix.
template <class Team = CtaTeam>
__device__ __forceinline__ void posterior_group(SmemFold<float>* sm, const FoldArgs& A, const Team tm = Team{}) {
    for (int g = 0; g < sm->n; ++g) {
        const int L = sm->L[g];
        float* POST = out_tabs(A, sm->ws[g], L).FMo;
        const int64_t tot = tri_size(L);
        for (int64_t c = tm.tid(); c < tot; c += tm.nthreads()) POST[c] = 0.0f;
        if (A.post_out) {
            float* dense = A.post_out + A.post_offs[sm->idx[g]];
            for (int64_t c = tm.tid(); c < (int64_t)L * L; c += tm.nthreads()) dense[c] = 0.0f;
        }
    }
    tm.sync();
    for (int g = 0; g < sm->n; ++g) {
        const SeqV Q = seq_v(sm, g);
        const int L = Q.L, m = L + 1;
        const OutTabs T = out_tabs(A, sm->ws[g], L);
        const PairList PLs = plist_of(A, sm->ws[g], L);
        const float Z = T.F5[L];
        float* POST = T.FMo;
        float* dense = A.post_out ? A.post_out + A.post_offs[sm->idx[g]] : nullptr;
        // pairable FC cells (i, i+d) <-> pairs (a, b) = (i, i+d+1), in list
        // order, whole warps at a time (team thread k takes entries k, k + nthreads, ...)
        const int total = PLs.poff[L + 1];
        const int lane = threadIdx.x & 31;
        for (int c0 = tm.tid() - lane; c0 < total; c0 += tm.nthreads()) {
            const int c = c0 + lane;
            const unsigned lanes = __ballot_sync(0xffffffffu, c < total);
            if (c >= total) continue;
            const int d = plist_diag(PLs, L, c);
            const int a = PLs.pl[c], b = a + d + 1;
            const float v = posterior_pair(&sm->tabs, &sm->poly, Q, T, Z, a, b, lanes);
            POST[tri_off(d + 1, m) + a] = v;
            if (dense != nullptr) dense[(int64_t)(a - 1) * L + (b - 1)] = v;
        }
    }
    tm.sync();
    if (A.logz != nullptr && tm.rank() == 0)
        for (int g = threadIdx.x; g < sm->n; g += blockDim.x) {
            const OutTabs T = out_tabs(A, sm->ws[g], sm->L[g]);
            A.logz[sm->idx[g]] = T.F5[sm->L[g]];
        }
}

template <int NT>
__global__ void __launch_bounds__(NT, NT == kFoldThreads ? kFoldMinBlocks : 1) k_outside32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    setup_group(sm, A, A.blob32);
    outside_group(sm, A);
}

template <int NT>
__global__ void __launch_bounds__(NT, NT == kFoldThreads ? kFoldMinBlocks : 1) k_posterior32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    setup_group(sm, A, A.blob32);
    posterior_group(sm, A);
}

// Walk diagonals d = d_begin .. d_end (step +1) over all sequences of the
// group; call f(g, i, i + d) for every cell.  One barrier per diagonal.
template <typename R, class Team, typename F>
__device__ __forceinline__ void wavefront(SmemFold<R>* sm, const Team& tm, int d_begin, int d_end, int step, F f) {
    const int ng = sm->n;
    for (int d = d_begin; step > 0 ? d <= d_end : d >= d_end; d += step) {
        int total = 0;
        for (int g = 0; g < ng; ++g) total += max(0, sm->L[g] + 1 - d);
        for (int c = tm.tid(); c < total; c += tm.nthreads()) {
            int g = 0, r = c;
            while (true) {
                const int cnt = max(0, sm->L[g] + 1 - d);
                if (r < cnt) break;
                r -= cnt;
                ++g;
            }
            f(g, r, r + d);
        }
        tm.sync();
    }
}

// MEA decode (cpu.py:823-895): unpaired weights, gamma-weighted max-plus DP
// with the reference's strict-'>' candidate order, BFS traceback.
template <class Team = CtaTeam>
__device__ __forceinline__ void mea_group(SmemFold<float>* sm, const FoldArgs& A, const Team tm = Team{}) {
    const float two_g = __fmul_rn(2.0f, A.gamma);
    for (int g = 0; g < sm->n; ++g) {
        const int L = sm->L[g];
        const Arena32 ar = arena32(L);
        float* base = A.ws + sm->ws[g];
        for (int i = 1 + tm.tid(); i <= L; i += tm.nthreads()) base[ar.up + i] = mea_unpaired(base + ar.FMo, L, two_g, i);
    }
    tm.sync();
    wavefront(sm, tm, 0, sm->Lmax, +1, [&](int g, int i, int j) {
        const SeqV Q = seq_v(sm, g);
        const Arena32 ar = arena32(Q.L);
        float* base = A.ws + sm->ws[g];
        mea_cell<Team::kChainPF>(Q, base + ar.FMo, base + ar.up, base + ar.FM2o, reinterpret_cast<int*>(base + ar.FM), Q.L, i, j);
    });
    for (int g = 0; g < sm->n; ++g) {
        const int L = sm->L[g];
        char* out = A.structs + sm->soff[g];
        for (int t = tm.tid(); t < L; t += tm.nthreads()) out[t] = '.';
    }
    tm.sync();
    // one traceback per thread, dealt over the warps first (lane 0 of every
    // warp, then lane 1, ...): lanes of one warp with different tracebacks
    // would run them one after another
    if (tm.rank() == 0)
        for (int g = tb_index(); g < sm->n; g += blockDim.x) {
            const int L = sm->L[g];
            const Arena32 ar = arena32(L);
            float* base = A.ws + sm->ws[g];
            int* qi = reinterpret_cast<int*>(base + ar.queue);
            mea_traceback(reinterpret_cast<const int*>(base + ar.FM), L, qi, qi + 2 * L + 4, A.structs + sm->soff[g],
                          A.status);
        }
    tm.sync();
}

// MEA decode (cpu.py:823-895): unpaired weights, gamma-weighted max-plus DP
// with the reference's strict-'>' candidate order, BFS traceback.
template <int NT>
__global__ void __launch_bounds__(NT, NT == kFoldThreads ? kFoldMinBlocks : 1) k_mea32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    setup_group(sm, A, A.blob32);
    mea_group(sm, A);
}

// ---------------------------------------------------------------------------
// Fused grouped fold: one launch runs inside -> outside -> posterior -> MEA
// decode (MODE 0) or posterior into the caller's matrices (MODE 1) for the
// CTA's group.  MODE 2 is MODE 0 built for the register budget of the other
// fold kernels (kFoldMinBlocks per SM instead of kFoldMinBlocksMea): on a
// device shared with them, a CTA of any of them fits the slot another frees
// (an 80-register CTA never fits where a 64-register one left).  Each CTA goes on to its next phase as soon as its own group
// is done, instead of every phase waiting for the slowest CTA of the grid.
// ---------------------------------------------------------------------------
template <int NT, int MODE>
__global__ void __launch_bounds__(NT, NT == kFoldThreads ? (MODE == 0 ? kFoldMinBlocksMea : kFoldMinBlocks) : 1)
    k_fold_group32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    setup_group(sm, A, A.blob32);
    if constexpr (MODE == 0 || MODE == 2) {
        inside_group<Lse32>(sm, A, CtaTeamMea{});
        outside_group(sm, A, CtaTeamMea{});
        __syncthreads();
        FoldArgs Ap = A;
        Ap.post_out = nullptr;
        Ap.logz = nullptr;
        posterior_group(sm, Ap, CtaTeamMea{});
        mea_group(sm, A, CtaTeamMea{});
    } else {
        inside_group<Lse32>(sm, A);
        outside_group(sm, A);
        __syncthreads();
        posterior_group(sm, A);
    }
}

// ---------------------------------------------------------------------------
// Cluster fold (latency of long sequences): the kClusterCtas CTAs of a
// thread-block cluster, on as many SMs, fold one group together -- each
// diagonal step's cells are dealt over all of them, with a cluster barrier
// between steps; the serial exterior recurrences and the traceback run on
// rank 0.  MODE 0: MEA, 1: BPP (as k_fold_group32); 2: the inside with the
// accurate log-sum-exp alone (logZ, and the tables the sampler draws from).
// No CTA touches another's shared memory, so CTAs may leave independently.
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __cluster_dims__(kClusterCtas, 1, 1) __launch_bounds__(kFoldThreads, kClusterMinBlocks)
    k_fold_cluster32(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    const ClusterTeam tm{cluster_ctarank(), kClusterCtas};
    setup_group(sm, A, A.blob32, (int)blockIdx.x / kClusterCtas);
    if constexpr (MODE == 2) {
        inside_group<LseAcc32>(sm, A, tm);
        if (A.logz != nullptr && tm.rank() == 0)
            for (int g = threadIdx.x; g < sm->n; g += blockDim.x)
                A.logz[sm->idx[g]] = in_view<float>(A, sm->ws[g], sm->L[g]).T.F5[sm->L[g]];
    } else {
        inside_group<Lse32>(sm, A, tm);
        outside_group(sm, A, tm);
        if constexpr (MODE == 0) {
            FoldArgs Ap = A;
            Ap.post_out = nullptr;
            Ap.logz = nullptr;
            posterior_group(sm, Ap, tm);
            mea_group(sm, A, tm);
        } else {
            posterior_group(sm, A, tm);
        }
    }
}

// ---------------------------------------------------------------------------
// Persistent fused fold: each CTA takes one sequence at a time from a device
// work queue and runs inside -> outside -> posterior -> MEA decode (or the
// inside alone for logZ) before taking the next.  Only one or two sequences
// per SM are in flight, so the DP tables that every diagonal step re-reads
// stay resident in L2; the CTA's arena slot is reused across sequences.
// ---------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(kFoldThreads, kFoldMinBlocks) k_fold_cta(FoldArgs A, int* counter, int64_t slot_words) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<float>*>(smem_raw);
    __shared__ int item_s;
    load_tabs(&sm->tabs, A.blob32);
    load_poly_tables(&sm->poly);
    const int64_t slot = (int64_t)blockIdx.x * slot_words;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) {
            const int item = atomicAdd(counter, 1);
            item_s = item;
            if (item < A.n) {
                const SeqDesc D = A.descs[item];
                sm->L[0] = D.L;
                sm->ws[0] = slot;
                sm->soff[0] = D.seq_off;
                sm->idx[0] = D.idx;
                sm->n = 1;
                sm->gcap = 1;
                sm->Lmax = D.L;
            }
        }
        __syncthreads();
        if (item_s >= A.n) break;
        build_group_seqs(sm, A);
        if constexpr (MODE == kCtaLogZ) {
            inside_group<LseAcc32>(sm, A);
            if (threadIdx.x == 0) A.logz[sm->idx[0]] = in_view<float>(A, sm->ws[0], sm->L[0]).T.F5[sm->L[0]];
            continue;
        }
        inside_group<Lse32>(sm, A);
        outside_group(sm, A);
        __syncthreads();
        posterior_group(sm, A);
        if constexpr (MODE == kCtaMea) mea_group(sm, A);
    }
}

template __global__ void k_fold_cta<kCtaLogZ>(FoldArgs, int*, int64_t);
template __global__ void k_fold_cta<kCtaMea>(FoldArgs, int*, int64_t);
template __global__ void k_fold_cta<kCtaBpp>(FoldArgs, int*, int64_t);

const void* cta_kernel(int mode) {
    switch (mode) {
        case kCtaLogZ: return (const void*)k_fold_cta<kCtaLogZ>;
        case kCtaMea: return (const void*)k_fold_cta<kCtaMea>;
        default: return (const void*)k_fold_cta<kCtaBpp>;
    }
}

// ---------------------------------------------------------------------------
// Viterbi: max-plus inside in FP64, then the reference's EPS first-match
// traceback (cpu.py:396-501), one thread per sequence.
// ---------------------------------------------------------------------------
__device__ void viterbi_traceback(const SmemTabs<double>* tb, const SeqV& Q, const InTabs<double>& T,
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

__global__ void __launch_bounds__(kFoldThreads, kFoldMinBlocks) k_viterbi64(FoldArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<SmemFold<double>*>(smem_raw);
    setup_group(sm, A, A.blob64);
    inside_group<Max64>(sm, A);
    for (int g = 0; g < sm->n; ++g) {
        const int L = sm->L[g];
        char* out = A.structs + sm->soff[g];
        for (int t = threadIdx.x; t < L; t += blockDim.x) out[t] = '.';
    }
    __syncthreads();
    for (int g = tb_index(); g < sm->n; g += blockDim.x) {   // tracebacks dealt over the warps first
        const SeqV Q = seq_v(sm, g);
        const InTabs<double> T = in_view<double>(A, sm->ws[g], Q.L).T;
        const Arena64 ar = arena64(Q.L);
        int* st = reinterpret_cast<int*>(A.ws + sm->ws[g] + ar.stack);   // stack offset is in 4-byte words
        viterbi_traceback(&sm->tabs, Q, T, st, A.structs + sm->soff[g], A.status);
    }
}

// ---------------------------------------------------------------------------
template __global__ void k_inside32<kFoldThreads>(FoldArgs);
template __global__ void k_inside32<kFoldThreadsWide>(FoldArgs);
template __global__ void k_inside32acc<kFoldThreads>(FoldArgs);
template __global__ void k_inside32acc<kFoldThreadsWide>(FoldArgs);
template __global__ void k_outside32<kFoldThreads>(FoldArgs);
template __global__ void k_outside32<kFoldThreadsWide>(FoldArgs);
template __global__ void k_posterior32<kFoldThreads>(FoldArgs);
template __global__ void k_posterior32<kFoldThreadsWide>(FoldArgs);
template __global__ void k_mea32<kFoldThreads>(FoldArgs);
template __global__ void k_mea32<kFoldThreadsWide>(FoldArgs);

template __global__ void k_fold_group32<kFoldThreads, 0>(FoldArgs);
template __global__ void k_fold_group32<kFoldThreads, 1>(FoldArgs);
template __global__ void k_fold_group32<kFoldThreads, 2>(FoldArgs);
template __global__ void k_fold_group32<kFoldThreadsWide, 0>(FoldArgs);
template __global__ void k_fold_group32<kFoldThreadsWide, 1>(FoldArgs);

FoldKernels fold_kernels(bool wide) {
    if (wide)
        return {k_inside32<kFoldThreadsWide>, k_inside32acc<kFoldThreadsWide>, k_outside32<kFoldThreadsWide>,
                k_posterior32<kFoldThreadsWide>, k_mea32<kFoldThreadsWide>,
                k_fold_group32<kFoldThreadsWide, 0>, k_fold_group32<kFoldThreadsWide, 1>,
                k_fold_group32<kFoldThreads, 2>};
    return {k_inside32<kFoldThreads>, k_inside32acc<kFoldThreads>, k_outside32<kFoldThreads>,
            k_posterior32<kFoldThreads>, k_mea32<kFoldThreads>,
            k_fold_group32<kFoldThreads, 0>, k_fold_group32<kFoldThreads, 1>, k_fold_group32<kFoldThreads, 2>};
}

ClusterKernels cluster_kernels() {
    return {k_fold_cluster32<0>, k_fold_cluster32<1>, k_fold_cluster32<2>};
}

size_t fold_smem_bytes(int Lmax, int group, bool fp64) {
    const size_t head = fp64 ? sizeof(SmemFold<double>) : sizeof(SmemFold<float>);
    return head + 2 * (size_t)code_stride(Lmax) * group + (size_t)group * 4 * pb_words(Lmax) * 4;
}

}  // namespace cf
