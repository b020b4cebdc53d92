// cf_inside.cuh -- the inside recurrence (FC / FM1 / FM / F5) over one of
// three semirings, evaluated one DP cell per thread on a diagonal wavefront.
//
//   Lse32  float32, CONTRAfold Fast_LogPlusEquals   (cpu.py:595-678, gpu.py:79-183)
//   Lse64  float64, exact log1p/exp                 (cpu.py:165-275)
//   Max64  float64, max-plus (Viterbi forward)      (cpu.py:302-394)
//
// Every cell accumulates its candidates in the reference's order -- FM2 over
// k ascending; FC: hairpin, single-branch loops p ascending / q descending,
// multibranch; FM1: pair, then extension; FM: FM2, extension, FM1 -- with the
// same left-to-right additions, so the FP32 tables are bitwise equal to the
// reference's float32 tables.
#pragma once

#include <type_traits>

#include "cf_device.cuh"

namespace cf {

struct Lse32 {
    using Real = float;
    const PolyTables* pt;
    static __device__ __forceinline__ Real neg() { return CF_NEG32; }
    static __device__ __forceinline__ Real half() { return CF_HALF32; }
    static __device__ __forceinline__ Real add(Real a, Real b) { return __fadd_rn(a, b); }
    __device__ __forceinline__ Real plus(Real acc, Real x) const { return lse32(pt, acc, x); }
};

// float32 log-sum-exp with accurate log1pf/expf.  Used where the result is
// compared with the FP64 engine (logZ within 5e-4) rather than bitwise
// against the reference's Fast_LogPlusEquals arithmetic.
struct LseAcc32 {
    using Real = float;
    static __device__ __forceinline__ Real neg() { return CF_NEG32; }
    static __device__ __forceinline__ Real half() { return CF_HALF32; }
    static __device__ __forceinline__ Real add(Real a, Real b) { return __fadd_rn(a, b); }
    __device__ __forceinline__ Real plus(Real acc, Real x) const {
        if (acc < CF_HALF32) return x;
        if (x < CF_HALF32) return acc;
        const float hi = fmaxf(acc, x), lo = fminf(acc, x);
        return __fadd_rn(hi, log1pf(expf(__fsub_rn(lo, hi))));
    }
};

struct Lse64 {
    using Real = double;
    static __device__ __forceinline__ Real neg() { return CF_NEG64; }
    static __device__ __forceinline__ Real half() { return CF_HALF64; }
    static __device__ __forceinline__ Real add(Real a, Real b) { return __dadd_rn(a, b); }
    __device__ __forceinline__ Real plus(Real acc, Real x) const { return lse64(acc, x); }
};

struct Max64 {
    using Real = double;
    static __device__ __forceinline__ Real neg() { return CF_NEG64; }
    static __device__ __forceinline__ Real half() { return CF_HALF64; }
    static __device__ __forceinline__ Real add(Real a, Real b) { return __dadd_rn(a, b); }
    // strict '>' keeps the earlier value on ties, as `if v > best` does
    __device__ __forceinline__ Real plus(Real acc, Real x) const { return x > acc ? x : acc; }
};

// Shared-memory scoring tables for semiring real type R.
template <typename R>
struct SmemTabs {
    R blob[CF_BLOB_LEN + 3];
    R jB[625];   // hc[a][b] + tm[a][b][c][d]: the reference's ScoreJunctionB sum
};

template <typename R>
__device__ __forceinline__ void load_tabs(SmemTabs<R>* t, const R* __restrict__ g) {
    for (int k = threadIdx.x; k < CF_BLOB_LEN; k += blockDim.x) t->blob[k] = g[k];
    for (int k = threadIdx.x; k < 625; k += blockDim.x) {
        const int a = k / 125, c = (k / 25) % 5;
        const R hc = g[CF_OFF_HC + a * 5 + c];
        const R tm = g[CF_OFF_TM + k];
        t->jB[k] = hc + tm;   // single rounded add (fp contraction cannot apply)
    }
}

// Inside tables of one sequence, triangular diagonal-major (see cf_device.cuh).
template <typename R>
struct InTabs {
    CF_TAB(R) FC;
    CF_TAB(R) FM;
    CF_TAB(R) FM1;
    CF_TAB(R) F5;
    int m;   // L + 1
    __device__ __forceinline__ int at(int i, int j) const { return tri_off(j - i, m) + i; }
    // table sizes for checked builds (nothing otherwise)
    __device__ __forceinline__ void sized(int L) {
        CF_SIZE_TAB(FC, tri_size(L));
        CF_SIZE_TAB(FM, tri_size(L));
        CF_SIZE_TAB(FM1, tri_size(L));
        CF_SIZE_TAB(F5, L + 2);
        (void)L;
    }
};

// ScoreJunctionA(i, j) for the pair (i, j+1) (cpu.py:224-228).
template <class S, class QV>
__device__ __forceinline__ typename S::Real junctionA(const ParamView<typename S::Real>& P, int L,
                                                      const QV& Q, int i, int j) {
    using R = typename S::Real;
    R jA = P.hc(Q.s[i], Q.s[j + 1]);
    if (i < L) jA = S::add(jA, P.dl(Q.s[i], Q.s[j + 1], Q.s[i + 1]));
    if (j > 0) jA = S::add(jA, P.dr(Q.s[i], Q.s[j + 1], Q.s[j]));
    return jA;
}

// ScoreJunctionA(j, i) for the pair (i+1, j) as used by FM1 / F5 (cpu.py:237-241, 268-272).
template <class S, class QV>
__device__ __forceinline__ typename S::Real junctionA_rev(const ParamView<typename S::Real>& P, int L,
                                                          const QV& Q, int i, int j) {
    using R = typename S::Real;
    R jA = P.hc(Q.s[j], Q.s[i + 1]);
    if (j < L) jA = S::add(jA, P.dl(Q.s[j], Q.s[i + 1], Q.s[j + 1]));
    if (i > 0) jA = S::add(jA, P.dr(Q.s[j], Q.s[i + 1], Q.s[i]));
    return jA;
}

// ---------------------------------------------------------------------------
// Prefetched sequential chains.  A bifurcation chain folds n terms x_k * y_k
// (k ascending) into an accumulator; each step depends on the previous one,
// but the operand loads do not.  `ld(px, py)` yields the addresses of the next
// term's two operands in k order (it carries its own incremental addressing);
// `step(k, x, y)` folds term k.  Three ways to run a chain, chosen per
// translation unit (each .cu file is its own device module, compiled without
// relocatable device code):
//   CF_CHAIN_ASYNC = D > 0: a D-deep asynchronous-copy pipeline.  Each thread
//     copies the operands of term k + D (cp.async, global -> shared) into its
//     own slots of a ring of D + 1 shared-memory slots while it folds term k,
//     so global-memory latency overlaps D dependent log-sum-exp steps without
//     holding the prefetched values in registers.  The copy for term k + D
//     goes to the slot read at term k - 1, whose value the fold of term k - 1
//     has already consumed.  The module defines CF_CHAIN_THREADS (its block
//     size); float chains only.
//   CF_CHAIN_PF = PF > 0: a rolling register pipeline of 2*PF terms (the
//     default of the PFD template parameter; latency kernels pass a deeper one).
//   both 0: load, then fold.
// ---------------------------------------------------------------------------
#ifndef CF_CHAIN_PF
#define CF_CHAIN_PF 4
#endif
#ifndef CF_CHAIN_ASYNC
#define CF_CHAIN_ASYNC 0
#endif
constexpr int kChainPF = CF_CHAIN_PF;
constexpr int kChainAsync = CF_CHAIN_ASYNC;
// CF_FLAT_WALK = 1 walks the single-branch windows (inside_B, outside_B,
// posterior_pair) in flattened lockstep (each lane on its own row sequence),
// 0 in row lockstep.  Results are identical.
#ifndef CF_FLAT_WALK
#define CF_FLAT_WALK 0
#endif
// CF_CHAIN_UNROLL = 1 unrolls the asynchronous pipeline over its ring slots
// (constant slot addresses, more code)
#ifndef CF_CHAIN_UNROLL
#define CF_CHAIN_UNROLL 0
#endif
constexpr bool kChainUnroll = CF_CHAIN_UNROLL != 0;

__device__ __forceinline__ void cp_async_f32(float* smem, const float* gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

#if CF_CHAIN_ASYNC > 0
// ring[slot][operand][thread]: consecutive threads use consecutive words
__shared__ float cf_chain_ring[CF_CHAIN_ASYNC + 1][2][CF_CHAIN_THREADS];
#endif

template <typename R, int PFD = kChainPF, class Ld, class Step>
__device__ __forceinline__ void prefetched_chain(int n, Ld ld, Step step) {
#if CF_CHAIN_ASYNC > 0
    if constexpr (sizeof(R) == 4) {
        constexpr int D = kChainAsync, NS = kChainAsync + 1;
        const int tid = threadIdx.x;
        auto issue = [&](int slot) {
            const R *px, *py;
            ld(px, py);
            cp_async_f32(&cf_chain_ring[slot][0][tid], px);
            cp_async_f32(&cf_chain_ring[slot][1][tid], py);
        };
#pragma unroll
        for (int u = 0; u < D; ++u) {
            if (u < n) issue(u);
            cp_async_commit();
        }
        if constexpr (kChainUnroll) {
            // unrolled over the ring: term k sits in slot k mod NS, term k + D
            // goes to slot (k + D) mod NS = (k - 1) mod NS -- compile-time slots
            for (int k0 = 0; k0 < n; k0 += NS) {
#pragma unroll
                for (int u = 0; u < NS; ++u) {
                    const int k = k0 + u;
                    if (k < n) {
                        cp_async_wait<D - 1>();   // term k has landed
                        const R x = cf_chain_ring[u][0][tid], y = cf_chain_ring[u][1][tid];
                        if (k + D < n) issue((u + D) % NS);
                        cp_async_commit();
                        step(k, x, y);
                    }
                }
            }
        } else {
            int rd = 0, wr = D;   // slots of term k and of term k + D
            for (int k = 0; k < n; ++k) {
                cp_async_wait<D - 1>();   // term k has landed
                const R x = cf_chain_ring[rd][0][tid], y = cf_chain_ring[rd][1][tid];
                if (k + D < n) issue(wr);
                cp_async_commit();
                step(k, x, y);
                rd = rd + 1 == NS ? 0 : rd + 1;
                wr = wr + 1 == NS ? 0 : wr + 1;
            }
        }
        cp_async_wait<0>();
        return;
    }
#endif
    if constexpr (PFD == 0) {
        for (int k = 0; k < n; ++k) {
            const R *px, *py;
            ld(px, py);
            step(k, *px, *py);
        }
    } else {
        R xa[PFD], ya[PFD], xb[PFD], yb[PFD];
        auto load = [&](R& x, R& y) {
            const R *px, *py;
            ld(px, py);
            x = *px;
            y = *py;
        };
#pragma unroll
        for (int u = 0; u < PFD; ++u)
            if (u < n) load(xa[u], ya[u]);
        int k0 = 0;
        // whole blocks: the next block's loads and this block's steps are all
        // in range, so no per-term checks
        for (; k0 + 2 * PFD <= n; k0 += PFD) {
#pragma unroll
            for (int u = 0; u < PFD; ++u) load(xb[u], yb[u]);
#pragma unroll
            for (int u = 0; u < PFD; ++u) step(k0 + u, xa[u], ya[u]);
#pragma unroll
            for (int u = 0; u < PFD; ++u) {
                xa[u] = xb[u];
                ya[u] = yb[u];
            }
        }
        for (; k0 < n; k0 += PFD) {
#pragma unroll
            for (int u = 0; u < PFD; ++u)
                if (k0 + PFD + u < n) load(xb[u], yb[u]);
#pragma unroll
            for (int u = 0; u < PFD; ++u)
                if (k0 + u < n) step(k0 + u, xa[u], ya[u]);
#pragma unroll
            for (int u = 0; u < PFD; ++u) {
                xa[u] = xb[u];
                ya[u] = yb[u];
            }
        }
    }
}

// One row of a lockstep window walk (see inside_B): every lane of the group
// runs `slots` iterations (the largest candidate count among them) and takes
// the set bits of its own mask, highest first (HI) or lowest first; the
// table value of the next candidate, `ld(bit)`, is loaded before the current
// one is used, `use(bit, v)`.  (Two to eight loads ahead measured slower, in
// the batched and in the cluster kernels alike.)
template <bool HI, typename R, class Ld, class Use>
__device__ __forceinline__ void lockstep_row(uint32_t msk, int slots, Ld ld, Use use) {
    auto take = [&](int& bit) -> bool {
        if (msk == 0u) return false;
        if constexpr (HI) {
            bit = 31 - __clz(msk);
            msk ^= 1u << bit;
        } else {
            bit = __ffs(msk) - 1;
            msk &= msk - 1u;
        }
        return true;
    };
    int bit = 0;
    R v = R(0);
    bool h = take(bit);
    if (h) v = ld(bit);
    for (int k = 0; k < slots; ++k) {
        int bn = 0;
        R vn = R(0);
        const bool hn = take(bn);
        if (hn) vn = ld(bn);
        if (h) use(bit, v);
        h = hn;
        bit = bn;
        v = vn;
    }
}

// ---------------------------------------------------------------------------
// Two-phase cell evaluation.  On diagonal t:
//   phase A (every cell): FM2 (kept for phase B), FM1, FM -- they read FC only
//           up to diagonal t-2;
//   phase B (pairable cells only): FC, which reads FC up to diagonal t-2 and the
//           cell's own FM2.
// The fold kernels run A(t) and B(t-1) in the same step, one barrier per step.
// ---------------------------------------------------------------------------

// Phase A of inside cell (i, j), 0 <= i <= j <= L.  Returns FM2[i][j] (the
// semiring zero where the cell needs none).  Writes FM1, FM, and FC = zero
// for cells that cannot close a pair (pairable cells get FC in phase B).
template <class S, int CPF = kChainPF, class QV>
__device__ __forceinline__ typename S::Real inside_A(const S& sr, const SmemTabs<typename S::Real>* __restrict__ tb,
                                                     const QV& Q, const InTabs<typename S::Real>& T, int i, int j) {
    using R = typename S::Real;
    const ParamView<R> P{tb->blob};
    const int L = Q.L, m = T.m, d = j - i;
    const R NEG = S::neg(), HALF = S::half();
    const int at = tri_off(d, m) + i;
    if (i == 0 || j == L) {
        T.FC[at] = NEG;
        T.FM1[at] = NEG;
        T.FM[at] = NEG;
        return NEG;
    }
    const bool fm_region = i + 2 <= j;
    const bool fc_cell = Q.pairable(i, j + 1);
    if (!fc_cell) T.FC[at] = NEG;
    // FM2[i][j] = (+)_{i<k<j} FM1[i][k] * FM[k][j]   (cpu.py:179-183)
    R fm2 = NEG;
    if (fm_region) {
        // term k = i+1 .. j-1: FM1[i][k] (span s1 = k-i), FM[k][j] (span s2 = j-k)
        int o1 = tri_off(1, m) + i;          // FM1[i][i+1]
        int o2 = tri_off(d - 1, m) + i + 1;  // FM[i+1][j]
        int s1 = 1, s2 = d - 1;
        prefetched_chain<R, CPF>(
            d - 1,
            [&](const R*& x, const R*& y) {
                x = T.FM1 + o1;
                y = T.FM + o2;
                o1 += m - s1;
                o2 += s2 - m;           // FM[k+1][j]: span s2-1, one position right
                ++s1;
                --s2;
            },
            [&](int, R x, R y) {
                // Terms with an operand at the zero sentinel are skipped by the
                // reference; here they are folded unconditionally (no divergent
                // branch): such a term is <= NEG and every semiring's plus keeps
                // the accumulator -- or, from the NEG start, yields another
                // sub-HALF value, which all readers of FM2 treat as zero.
                fm2 = sr.plus(fm2, S::add(x, y));
            });
    }
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
    T.FM1[at] = fm1;
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
    T.FM[at] = fm;
    return fm2;
}

// Phase B of a pairable inside cell (i, j) (1 <= i <= j <= L-1, pair (i, j+1)):
// FC[i][j] (cpu.py:185-230).  The single-branch candidates are the pairable
// inner pairs (p+1, q) of the window, walked p ascending and, within a row,
// q descending (highest set bit of the partner mask first) -- the reference's
// order -- so only valid candidates cost work.
//
// `lanes` names the lanes of the warp that evaluate cells together (all of
// them call inside_B with the same mask).  They walk the window in lockstep:
// row by row (the rows and each row's q range depend only on d = j - i), and
// within a row for as many slots as the lane with the most candidates has.  A
// lane with fewer candidates idles in the remaining slots, so the warp never
// splits into per-lane paths; each lane still folds exactly its own
// candidates in the reference's order.
template <class S, class QV>
__device__ __forceinline__ void inside_B(const S& sr, const SmemTabs<typename S::Real>* __restrict__ tb,
                                         const QV& Q, const InTabs<typename S::Real>& T, int i, int j,
                                         typename S::Real fm2, unsigned lanes) {
    using R = typename S::Real;
    const ParamView<R> P{tb->blob};
    const int L = Q.L, m = T.m, d = j - i;
    const R NEG = S::neg(), HALF = S::half();
    const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
    const R jB = tb->jB[idx4(si, sj1, si1, sj)];
    R acc = sr.plus(NEG, S::add(jB, P.hp(d <= DHP ? d : DHP)));
    const int nrows = (d < CMAX ? d : CMAX) + 1;
    // one single-branch candidate: inner pair (p+1, q) of row l1, table value v
    auto fold = [&](int l1, int q, R sn0, R sn1, R v) {
        // no zero-threshold test on v: a visited candidate is a pairable
        // cell, whose FC always holds its hairpin term, and acc (likewise) is
        // finite, so a sub-threshold v would leave acc unchanged in any case
        const int p = i + l1;
        const int l2 = j - q, a = p + 1;
        R e;
        if (l1 == 0 && l2 == 0) {
            e = S::add(P.bp(si1, sj), P.stack(si, sj1, si1, sj));
        } else {
            const int sq = Q.s[q], sa = Q.s[a];
            const R jB2 = tb->jB[idx4(sq, sa, Q.s[q + 1], Q.s[p])];
            const R snuc = l2 == 0 ? sn0 : (l2 == 1 ? sn1 : R(0));
            e = S::add(S::add(S::add(P.cs(l1, l2), P.bp(sa, sq)), jB), jB2);
            // the reference adds snuc = 0 too; that add is skipped where snuc is 0
            // for the whole row (l1 >= 2): x + 0 is x except that -0 becomes +0,
            // which no comparison, log-sum-exp or max can see and later sums keep
            // only in the sign of a zero (the Viterbi is bound by the FP64 pipe:
            // one add of six per candidate)
            if (l1 < 2) e = S::add(e, snuc);
        }
        acc = sr.plus(acc, S::add(e, v));
    };
#if CF_FLAT_WALK
    // Flattened lockstep: each lane walks its own candidate sequence (rows
    // l1 ascending, q descending within a row) and moves to its next row as
    // soon as its row is exhausted, so a lane idles only once it has no
    // candidates left -- not at the end of every row, as the row-lockstep
    // walk does.  The next candidate's table value is loaded before the
    // current one is folded.
    int l1 = -1, qlo = 0;
    uint32_t msk = 0u;
    R sn0 = R(0), sn1 = R(0);
    auto next = [&](int& ql1, int& qq, R& q0, R& q1) -> bool {
        while (msk == 0u) {
            if (++l1 >= nrows) return false;
            const int p = i + l1;
            qlo = (p + 2 > l1 + j - CMAX) ? p + 2 : l1 + j - CMAX;
            msk = Q.window(p + 1, qlo, j - qlo + 1);
            sn0 = l1 == 1 ? P.b01(si1) : R(0);
            sn1 = l1 == 0 ? P.b01(sj) : (l1 == 1 ? P.i11(si1, sj) : R(0));
        }
        const int bit = 31 - __clz(msk);
        msk ^= 1u << bit;
        ql1 = l1;
        qq = qlo + bit;
        q0 = sn0;
        q1 = sn1;
        return true;
    };
    int cl1 = 0, cq = 0;
    R c0 = R(0), c1 = R(0), cv = R(0);
    bool have = next(cl1, cq, c0, c1);
    if (have) cv = T.FC[tri_off(cq - 2 - (i + cl1), m) + i + cl1 + 1];
    while (__any_sync(lanes, have)) {
        int nl1 = 0, nq = 0;
        R n0 = R(0), n1 = R(0), nv = R(0);
        const bool hn = have && next(nl1, nq, n0, n1);
        if (hn) nv = T.FC[tri_off(nq - 2 - (i + nl1), m) + i + nl1 + 1];
        if (have) fold(cl1, cq, c0, c1, cv);
        have = hn;
        cl1 = nl1; cq = nq; c0 = n0; c1 = n1; cv = nv;
    }
#else
    // rows p = i + l1, l1 = 0 .. min(30, d); row q range [qlo, j],
    // qlo = max(p + 2, l1 + j - 30)
    const int nr = __reduce_max_sync(lanes, nrows);
    for (int l1 = 0; l1 < nr; ++l1) {
        const int p = i + l1;
        const int qlo = (p + 2 > l1 + j - CMAX) ? p + 2 : l1 + j - CMAX;
        // the 1-nt bulge and 1x1 terms of this row by l2 = 0, 1 (zero beyond)
        const R sn0 = l1 == 1 ? P.b01(si1) : R(0);
        const R sn1 = l1 == 0 ? P.b01(sj) : (l1 == 1 ? P.i11(si1, sj) : R(0));
        uint32_t msk = l1 < nrows ? Q.window(p + 1, qlo, j - qlo + 1) : 0u;
        const int slots = __reduce_max_sync(lanes, __popc(msk));
        lockstep_row<true, R>(
            msk, slots, [&](int bit) -> R { return T.FC[tri_off(qlo + bit - 2 - p, m) + p + 1]; },
            [&](int bit, R v) { fold(l1, qlo + bit, sn0, sn1, v); });
    }
#endif
    if (fm2 > HALF) {
        const R jA = junctionA<S>(P, L, Q, i, j);
        acc = sr.plus(acc, S::add(S::add(S::add(fm2, jA), P.mp()), P.mb()));
    }
    T.FC[tri_off(d, m) + i] = acc;
}

// Exterior recurrence F5 (cpu.py:259-274) by one warp.  F5[j] is a sequential
// chain over k; the lanes evaluate 32 candidate terms at a time and every lane
// then folds them in k order (warp-uniform), so the chain is the reference's.
template <class S, class QV>
__device__ __forceinline__ void exterior_warp(const S& sr, const SmemTabs<typename S::Real>* __restrict__ tb,
                                              const QV& Q, const InTabs<typename S::Real>& T) {
    using R = typename S::Real;
    const ParamView<R> P{tb->blob};
    const int L = Q.L, lane = threadIdx.x & 31;
    const R HALF = S::half();
    R f5prev = R(0);
    if (lane == 0) T.F5[0] = R(0);
    for (int j = 1; j <= L; ++j) {
        R acc = S::add(f5prev, P.eu());
        for (int k0 = 0; k0 < j; k0 += 32) {
            const int k = k0 + lane;
            bool ok = false;
            R term = R(0);
            if (k < j && Q.pairable(k + 1, j)) {
                const R fcin = T.FC[T.at(k + 1, j - 1)];
                const R f5k = T.F5[k];
                if (fcin > HALF && f5k > HALF) {
                    const R jA = junctionA_rev<S>(P, L, Q, k, j);
                    term = S::add(S::add(S::add(S::add(f5k, fcin), P.ep()), P.bp(Q.s[k + 1], Q.s[j])), jA);
                    ok = true;
                }
            }
            unsigned mask = __ballot_sync(0xffffffffu, ok);
            while (mask) {
                const int t = __ffs(mask) - 1;
                mask &= mask - 1;
                const R v = __shfl_sync(0xffffffffu, term, t);
                acc = sr.plus(acc, v);
            }
        }
        if (lane == 0) T.F5[j] = acc;
        f5prev = acc;
        __syncwarp();
    }
}

}  // namespace cf
