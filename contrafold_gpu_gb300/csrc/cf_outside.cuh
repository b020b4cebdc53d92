// cf_outside.cuh -- outside pass and posterior in float32.
//
// The reference (gpu_contrafold/cpu.py:680-819) computes the outside tables
// and the posterior by SCATTERING from each source cell into its children,
// sources visited i ascending / j descending (outside) and i descending / j
// ascending (posterior).  Float log-sum-exp and float += are not associative,
// so the value of a target depends on the order its contributions arrive.
// Here each target GATHERS its contributions, enumerating its sources in
// exactly the order the reference's scatter reaches it, with each
// contribution computed by the same operations -- a parallel formulation
// with bitwise the reference's results.  The derivation of each order is next
// to the code.
//
// Outside cells run in two phases per diagonal t (descending):
//   phase A (every cell): FMo, FM1o (read FM2o of larger spans, FMo / FM1o of
//           span t+1) and FM2o (reads the cell's own FMo and FCo);
//   phase B (pairable cells): FCo (reads FCo of spans >= t+2, FM1o of span t+2).
// A step runs A(t) and B(t-1); FCo(t) was produced one step earlier.
#pragma once

#include "cf_inside.cuh"
#include "cf_seq.cuh"

namespace cf {

struct OutTabs {
    CF_TAB(const float) FC;
    CF_TAB(const float) FM;
    CF_TAB(const float) FM1;
    CF_TAB(const float) F5;
    CF_TAB(float) FCo;
    CF_TAB(float) FMo;
    CF_TAB(float) FM1o;
    CF_TAB(float) FM2o;
    CF_TAB(float) F5o;
    int m;
    __device__ __forceinline__ int at(int i, int j) const { return tri_off(j - i, m) + i; }
    // table sizes for checked builds (nothing otherwise)
    __device__ __forceinline__ void sized(int L) {
        CF_SIZE_TAB(FC, tri_size(L));
        CF_SIZE_TAB(FM, tri_size(L));
        CF_SIZE_TAB(FM1, tri_size(L));
        CF_SIZE_TAB(F5, L + 2);
        CF_SIZE_TAB(FCo, tri_size(L));
        CF_SIZE_TAB(FMo, tri_size(L));
        CF_SIZE_TAB(FM1o, tri_size(L));
        CF_SIZE_TAB(FM2o, tri_size(L));
        CF_SIZE_TAB(F5o, L + 2);
        (void)L;
    }
};

// F5o (cpu.py:684-699) by one warp, k = L-1 .. 0.  Target k receives, in the
// reference's order, the pair terms of iterations j = L .. k+2 and then the
// unpaired term F5o[k+1] + eu of iteration j = k+1.
template <class QV>
__device__ __forceinline__ void exterior_outside_warp(const Lse32& sr, const SmemTabs<float>* __restrict__ tb,
                                                      const QV& Q, const OutTabs& T) {
    const ParamView<float> P{tb->blob};
    const int L = Q.L, lane = threadIdx.x & 31;
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
                    const float jA = junctionA_rev<Lse32>(P, L, Q, k, j);
                    const float temp = __fadd_rn(__fadd_rn(__fadd_rn(T.F5o[j], P.ep()), P.bp(Q.s[k + 1], Q.s[j])), jA);
                    term = __fadd_rn(temp, fcin);
                    ok = true;
                }
            }
            unsigned mask = __ballot_sync(0xffffffffu, ok);
            while (mask) {
                const int t = __ffs(mask) - 1;
                mask &= mask - 1;
                acc = sr.plus(acc, __shfl_sync(0xffffffffu, term, t));
            }
        }
        acc = sr.plus(acc, __fadd_rn(T.F5o[k + 1], P.eu()));
        if (lane == 0) T.F5o[k] = acc;
        __syncwarp();
    }
}

// Phase A of outside cell (a, b), 0 <= a <= b <= L: FMo, FM1o, FM2o.
__device__ __forceinline__ void outside_A(const Lse32& sr, const SmemTabs<float>* __restrict__ tb,
                                          const SeqV& Q, const OutTabs& T, int a, int b) {
    const ParamView<float> P{tb->blob};
    const int L = Q.L, m = T.m, t = b - a;
    const int at = tri_off(t, m) + a;
    const bool fm_region = (0 < a) && (a + 2 <= b) && (b < L);

    // FMo[a][b]: FM2o distribution of sources (i, b), i = 1 .. a-1 ascending,
    // k = a (cpu.py:753-758); then block 1 of source (a, b+1):
    // FMo[a][b] (+)= FMo[a][b+1] + mu (cpu.py:705).
    float fmo = CF_NEG32, fm1o = CF_NEG32;
    if (fm_region) {
        float acc = CF_NEG32;
        // i = a - u, u = a-1 .. 1: FM2o[i][b] at span t+u, FM1[i][a] at span u
        for (int u = a - 1; u >= 1; --u) {
            const float src = T.FM2o[tri_off(t + u, m) + a - u];
            const float f1 = T.FM1[tri_off(u, m) + a - u];
            if (src > CF_HALF32 && f1 > CF_HALF32) acc = sr.plus(acc, __fadd_rn(src, f1));
        }
        if (b + 1 < L) acc = sr.plus(acc, __fadd_rn(T.FMo[tri_off(t + 1, m) + a], P.mu()));
        fmo = acc;

        // FM1o[a][b]: block 2 of source (a-1, b): FM1o[a-1][b] + mu (cpu.py:715);
        // FM2o distribution of sources (a, j), j = L-1 .. b+1, k = b (cpu.py:756);
        // block 1 of source (a, b): (+)= FMo[a][b] (cpu.py:706).
        acc = CF_NEG32;
        if (a >= 2) acc = sr.plus(acc, __fadd_rn(T.FM1o[tri_off(t + 1, m) + a - 1], P.mu()));
        // j = b + v, v = L-1-b .. 1: FM2o[a][j] at span t+v, FM[b][j] at span v
        for (int v = L - 1 - b; v >= 1; --v) {
            const float src = T.FM2o[tri_off(t + v, m) + a];
            const float fmk = T.FM[tri_off(v, m) + b];
            if (src > CF_HALF32 && fmk > CF_HALF32) acc = sr.plus(acc, __fadd_rn(src, fmk));
        }
        fm1o = sr.plus(acc, fmo);
    }
    T.FMo[at] = fmo;
    T.FM1o[at] = fm1o;

    // FM2o[a][b] (cpu.py:702-704, 746-751); FCo[a][b] came from phase B.
    float fm2o = CF_NEG32;
    if (fm_region) fm2o = sr.plus(fm2o, fmo);
    if (0 < a && b < L && Q.pairable(a, b + 1)) {
        const float fco = T.FCo[at];
        if (fco > CF_HALF32) {
            const float jA = junctionA<Lse32>(P, L, Q, a, b);
            fm2o = sr.plus(fm2o, __fadd_rn(__fadd_rn(__fadd_rn(fco, jA), P.mp()), P.mb()));
        }
    }
    T.FM2o[at] = fm2o;
}

// Phase A as one loop: the FMo chain (a-1 terms) and the FM1o chain (L-1-b
// terms) run back to back in a single loop of (a-1) + (L-1-b) = L-2-t
// iterations, which is the same for every cell of diagonal t -- lanes of a
// warp working on one diagonal stay converged.  Each chain keeps the
// reference's order (see outside_A).
template <int CPF = kChainPF>
__device__ __forceinline__ void outside_A_merged(const Lse32& sr, const SmemTabs<float>* __restrict__ tb,
                                                 const SeqV& Q, const OutTabs& T, int a, int b) {
    const ParamView<float> P{tb->blob};
    const int L = Q.L, m = T.m, t = b - a;
    const int at = tri_off(t, m) + a;
    const bool fm_region = (0 < a) && (a + 2 <= b) && (b < L);
    float fmo = CF_NEG32, fm1o = CF_NEG32;
    if (fm_region) {
        const int n1 = a - 1, n2 = L - 1 - b, K = n1 + n2;
        float acc = CF_NEG32;
        auto switch_chain = [&]() {
            if (b + 1 < L) acc = sr.plus(acc, __fadd_rn(T.FMo[tri_off(t + 1, m) + a], P.mu()));
            fmo = acc;
            acc = CF_NEG32;
            if (a >= 2) acc = sr.plus(acc, __fadd_rn(T.FM1o[tri_off(t + 1, m) + a - 1], P.mu()));
        };
        // loader: phase 1 (k < n1) reads FM2o[a-w][b], FM1[a-w][a] with w = n1-k;
        // phase 2 reads FM2o[a][b+w], FM[b][b+w] with w = n2-(k-n1)
        int kl = 0, w = n1;
        int addr1 = tri_off(t + n1, m) + a - n1, addr2 = tri_off(n1, m) + a - n1;
        const float* tab2 = T.FM1;
        int first = 1;
        prefetched_chain<float, CPF>(
            K,
            [&](const float*& x, const float*& y) {
                if (kl == n1) {
                    w = n2;
                    addr1 = tri_off(t + n2, m) + a;
                    addr2 = tri_off(n2, m) + b;
                    tab2 = T.FM;
                    first = 0;
                }
                x = T.FM2o + addr1;
                y = tab2 + addr2;
                addr1 -= (m - t - w + 1) - first;
                addr2 -= (m - w + 1) - first;
                --w;
                ++kl;
            },
            [&](int k, float x, float y) {
                if (k == n1) switch_chain();
                // unguarded fold: a sentinel operand makes the term <= NEG, which
                // Fast_LogPlusEquals discards (it returns the larger argument)
                acc = sr.plus(acc, __fadd_rn(x, y));
            });
        if (K == n1) switch_chain();
        fm1o = sr.plus(acc, fmo);
    }
    T.FMo[at] = fmo;
    T.FM1o[at] = fm1o;
    float fm2o = CF_NEG32;
    if (fm_region) fm2o = sr.plus(fm2o, fmo);
    if (0 < a && b < L && Q.pairable(a, b + 1)) {
        const float fco = T.FCo[at];
        if (fco > CF_HALF32) {
            const float jA = junctionA<Lse32>(P, L, Q, a, b);
            fm2o = sr.plus(fm2o, __fadd_rn(__fadd_rn(__fadd_rn(fco, jA), P.mp()), P.mb()));
        }
    }
    T.FM2o[at] = fm2o;
}

// Phase B of a pairable outside cell (a, b) (pair (a, b+1)): FCo[a][b].
//  1. exterior term of the F5o phase, k = a-1, j = b+1 (cpu.py:695-699);
//  2. sources (i, j) = (a-1-l1, b+1+l2) of the main loop, i ascending
//     (l1 = 30 .. 0) and j descending; a source contributes through its
//     single-branch loop (block 3, cpu.py:717-745) iff pairable(i, j+1), so
//     each row walks the partner mask of position i over j+1 = b+2 ..
//     b+2+(30-l1), highest bit first.  Source (a-1, b+1) first contributes
//     through FM1o (block 2, cpu.py:708-714), then through block 3.
// `lanes`: the lanes evaluating cells together, walked in lockstep as in
// inside_B (rows from the largest l1max among them, per row as many slots as
// the lane with the most candidates).
__device__ __forceinline__ void outside_B(const Lse32& sr, const SmemTabs<float>* __restrict__ tb,
                                          const SeqV& Q, const OutTabs& T, int a, int b, unsigned lanes) {
    const ParamView<float> P{tb->blob};
    const int L = Q.L, m = T.m, t = b - a;
    const int sa = Q.s[a], sb1 = Q.s[b + 1];
    const float bp_ab = P.bp(sa, sb1);
    float acc = CF_NEG32;
    {
        const float f5k = T.F5[a - 1];
        if (f5k > CF_HALF32) {
            const float jA = junctionA_rev<Lse32>(P, L, Q, a - 1, b + 1);
            const float temp = __fadd_rn(__fadd_rn(__fadd_rn(T.F5o[b + 1], P.ep()), bp_ab), jA);
            acc = sr.plus(acc, __fadd_rn(temp, f5k));
        }
    }
    // jB of the inner pair (p+1, q) = (a, b+1): hc[s[q]][s[p+1]] + tm[s[q]][s[p+1]][s[q+1]][s[p]]
    const float jB2 = tb->jB[idx4(sb1, sa, Q.s[b + 2], Q.s[a - 1])];
    const int l1max = (a - 2 < CMAX) ? a - 2 : CMAX;   // i = a-1-l1 >= 1
    auto rowmask = [&](int l1) -> uint32_t {
        const int jmax = (b + 1 + CMAX - l1 < L - 1) ? b + 1 + CMAX - l1 : L - 1;
        return Q.window(a - 1 - l1, b + 2, jmax - b);
    };
    // single-branch source (i, j) = (a-1-l1, j) with l2 = j - (b+1)
    auto src_val = [&](int l1, int j) -> float {
        const int i = a - 1 - l1;
        return T.FCo[tri_off(j - i, m) + i];
    };
    // the 1-nt bulge and 1x1 terms of row l1 by l2 = 0, 1 (l2 = 1 is j = b+2)
    const int sb2 = Q.s[b + 2];
    auto snuc_row = [&](int l1, float& sn0, float& sn1) {
        const int si1 = l1 <= l1max ? Q.s[a - l1] : 4;   // rows past this lane's last are empty
        sn0 = l1 == 1 ? P.b01(si1) : 0.0f;
        sn1 = l1 == 0 ? P.b01(sb2) : (l1 == 1 ? P.i11(si1, sb2) : 0.0f);
    };
    auto source = [&](int l1, int j, float v, float sn0, float sn1) {
        const int i = a - 1 - l1;
        if (!(v > CF_HALF32)) return;
        const int l2 = j - (b + 1);
        const int si = Q.s[i], si1 = Q.s[i + 1], sj = Q.s[j];
        float e;
        if (l1 == 0 && l2 == 0) {
            e = __fadd_rn(P.bp(si1, sj), P.stack(si, Q.s[j + 1], si1, sj));
        } else {
            const float jBij = tb->jB[idx4(si, Q.s[j + 1], si1, sj)];
            e = __fadd_rn(__fadd_rn(__fadd_rn(P.cs(l1, l2), bp_ab), jBij), jB2);
            if (l1 < 2) e = __fadd_rn(e, l2 == 0 ? sn0 : (l2 == 1 ? sn1 : 0.0f));   // + 0 skipped (see inside_B)
        }
        acc = sr.plus(acc, __fadd_rn(v, e));
    };
    uint32_t m0 = 0u;
#if CF_FLAT_WALK
    // flattened lockstep (see inside_B): rows l1max .. 0 of this lane, within a
    // row highest j first; row 0 without its stacking source
    {
        int l1 = l1max + 1;
        uint32_t msk = 0u;
        float sn0 = 0.0f, sn1 = 0.0f;
        auto next = [&](int& ql1, int& qj, float& q0, float& q1) -> bool {
            while (msk == 0u) {
                if (--l1 < 0) return false;
                msk = rowmask(l1);
                if (l1 == 0) {
                    m0 = msk;
                    msk &= ~1u;   // the stacking source comes after the FM1o term
                }
                snuc_row(l1, sn0, sn1);
            }
            const int bit = 31 - __clz(msk);
            msk ^= 1u << bit;
            ql1 = l1;
            qj = b + 1 + bit;
            q0 = sn0;
            q1 = sn1;
            return true;
        };
        int cl1 = 0, cj = 0;
        float c0 = 0.0f, c1 = 0.0f, cv = 0.0f;
        bool have = next(cl1, cj, c0, c1);
        if (have) cv = src_val(cl1, cj);
        while (__any_sync(lanes, have)) {
            int nl1 = 0, nj = 0;
            float n0 = 0.0f, n1 = 0.0f, nv = 0.0f;
            const bool hn = have && next(nl1, nj, n0, n1);
            if (hn) nv = src_val(nl1, nj);
            if (have) source(cl1, cj, cv, c0, c1);
            have = hn;
            cl1 = nl1; cj = nj; c0 = n0; c1 = n1; cv = nv;
        }
    }
#else
    const int lm = __reduce_max_sync(lanes, l1max + 1) - 1;
    for (int l1 = lm; l1 >= 0; --l1) {
        uint32_t msk = l1 <= l1max ? rowmask(l1) : 0u;
        if (l1 == 0) {
            m0 = msk;
            msk &= ~1u;   // the stacking source comes after the FM1o term
        }
        const int slots = __reduce_max_sync(lanes, __popc(msk));
        float sn0, sn1;
        snuc_row(l1, sn0, sn1);
        lockstep_row<true, float>(
            msk, slots, [&](int bit) { return src_val(l1, b + 1 + bit); },
            [&](int bit, float v) { source(l1, b + 1 + bit, v, sn0, sn1); });
    }
#endif
    if (l1max >= 0) {
        if (b + 1 < L) {
            const float v = T.FM1o[tri_off(t + 2, m) + a - 1];
            const float jAji = junctionA_rev<Lse32>(P, L, Q, a - 1, b + 1);
            acc = sr.plus(acc, __fadd_rn(__fadd_rn(__fadd_rn(v, jAji), P.mp()), bp_ab));
        }
        if (m0 & 1u) source(0, b + 1, src_val(0, b + 1), 0.0f, 0.0f);   // stacking: no snuc
    }
    T.FCo[tri_off(t, m) + a] = acc;
}

// Posterior of the pair (a, b), 1 <= a < b <= L, pairable (cpu.py:760-819).
// The reference adds fexp32 terms into POST[a][b] from sources (i, j) =
// (a-1-l1, b+l2) visited i descending (l1 = 0 ..), j ascending (l2 = 0 ..),
// each iff pairable(i, j+1) and its outside value is live; source (a-1, b)
// adds its multiloop (FM1o) term right after its stacking term; the exterior
// term comes last.  Returns the clipped value.
// `lanes`: the lanes evaluating pairs together, walked in lockstep as in
// inside_B.
__device__ __forceinline__ float posterior_pair(const SmemTabs<float>* __restrict__ tb, const PolyTables* pt,
                                                const SeqV& Q, const OutTabs& T, float Z, int a, int b,
                                                unsigned lanes) {
    const ParamView<float> P{tb->blob};
    const int L = Q.L, m = T.m;
    const float fcin = T.FC[tri_off(b - 1 - a, m) + a];
    const bool live = fcin > CF_HALF32;
    const int sa = Q.s[a], sb = Q.s[b];
    const float bp_ab = P.bp(sa, sb);
    // jB of the inner pair (p+1, q) = (a, b)
    const float jB2 = tb->jB[idx4(sb, sa, Q.s[b + 1], Q.s[a - 1])];
    float post = 0.0f;
    const int l1max = live ? ((a - 2 < CMAX) ? a - 2 : CMAX) : -1;   // i = a-1-l1 >= 1
    auto rowmask = [&](int l1) -> uint32_t {
        const int jmax = (b + CMAX - l1 < L - 1) ? b + CMAX - l1 : L - 1;
        return Q.window(a - 1 - l1, b + 1, jmax - b + 1);
    };
    // single-branch source (i, j) = (a-1-l1, j), l2 = j - b
    auto src_val = [&](int l1, int j) -> float {
        const int i = a - 1 - l1;
        return T.FCo[tri_off(j - i, m) + i];
    };
    // the 1-nt bulge and 1x1 terms of row l1 by l2 = 0, 1 (l2 = 1 is j = b+1)
    const int sb1 = Q.s[b + 1];
    auto snuc_row = [&](int l1, float& sn0, float& sn1) {
        const int si1 = l1 <= l1max ? Q.s[a - l1] : 4;   // rows past this lane's last are empty
        sn0 = l1 == 1 ? P.b01(si1) : 0.0f;
        sn1 = l1 == 0 ? P.b01(sb1) : (l1 == 1 ? P.i11(si1, sb1) : 0.0f);
    };
    auto source = [&](int l1, int j, float fco, float sn0, float sn1) {
        const int i = a - 1 - l1;
        const float outside = __fsub_rn(fco, Z);
        if (!(outside > CF_HALF32)) return;
        const int l2 = j - b;
        const int si = Q.s[i], si1 = Q.s[i + 1], sj = Q.s[j];
        float e;
        if (l1 == 0 && l2 == 0) {
            e = __fadd_rn(__fadd_rn(__fadd_rn(outside, P.bp(si1, sj)), P.stack(si, Q.s[j + 1], si1, sj)), fcin);
        } else {
            const float jBij = tb->jB[idx4(si, Q.s[j + 1], si1, sj)];
            e = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(outside, jBij), P.cs(l1, l2)), fcin), bp_ab), jB2);
            if (l1 < 2) e = __fadd_rn(e, l2 == 0 ? sn0 : (l2 == 1 ? sn1 : 0.0f));   // + 0 skipped (see inside_B)
        }
        post = __fadd_rn(post, fexp32(pt, e));
    };
    // row 0: the stacking source (a-1, b), its multiloop term, then j ascending
    uint32_t m0 = 0u;
    if (l1max >= 0) {
        m0 = rowmask(0);
        if (m0 & 1u) source(0, b, src_val(0, b), 0.0f, 0.0f);   // stacking: no snuc
        if (b < L) {
            const float v = T.FM1o[tri_off(b - a + 1, m) + a - 1];
            if (v > CF_HALF32) {
                const float jAji = junctionA_rev<Lse32>(P, L, Q, a - 1, b);
                const float x = __fsub_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(v, fcin), jAji), P.mp()), bp_ab), Z);
                post = __fadd_rn(post, fexp32(pt, x));
            }
        }
        m0 &= ~1u;
    }
#if CF_FLAT_WALK
    // flattened lockstep (see inside_B): rows 0 .. l1max of this lane, within
    // a row lowest j first
    {
        int l1 = 0;
        uint32_t msk = m0;
        float sn0 = 0.0f, sn1 = 0.0f;
        snuc_row(0, sn0, sn1);
        auto next = [&](int& ql1, int& qj, float& q0, float& q1) -> bool {
            while (msk == 0u) {
                if (++l1 > l1max) return false;
                msk = rowmask(l1);
                snuc_row(l1, sn0, sn1);
            }
            const int bit = __ffs(msk) - 1;
            msk &= msk - 1u;
            ql1 = l1;
            qj = b + bit;
            q0 = sn0;
            q1 = sn1;
            return true;
        };
        int cl1 = 0, cj = 0;
        float c0 = 0.0f, c1 = 0.0f, cv = 0.0f;
        bool have = next(cl1, cj, c0, c1);
        if (have) cv = src_val(cl1, cj);
        while (__any_sync(lanes, have)) {
            int nl1 = 0, nj = 0;
            float n0 = 0.0f, n1 = 0.0f, nv = 0.0f;
            const bool hn = have && next(nl1, nj, n0, n1);
            if (hn) nv = src_val(nl1, nj);
            if (have) source(cl1, cj, cv, c0, c1);
            have = hn;
            cl1 = nl1; cj = nj; c0 = n0; c1 = n1; cv = nv;
        }
    }
#else
    const int lm = __reduce_max_sync(lanes, l1max + 1) - 1;
    for (int l1 = 0; l1 <= lm; ++l1) {
        uint32_t msk = l1 == 0 ? m0 : (l1 <= l1max ? rowmask(l1) : 0u);
        const int slots = __reduce_max_sync(lanes, __popc(msk));
        float sn0, sn1;
        snuc_row(l1, sn0, sn1);
        lockstep_row<false, float>(
            msk, slots, [&](int bit) { return src_val(l1, b + bit); },
            [&](int bit, float v) { source(l1, b + bit, v, sn0, sn1); });
    }
#endif
    if (!live) return 0.0f;
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

}  // namespace cf
