// cf_outside.cuh -- outside pass, posterior and MEA decode in float32.
//
// The reference (gpu_contrafold/cpu.py:680-819) computes the outside tables
// and the posterior by SCATTERING from each source cell into its children,
// sources visited i ascending / j descending (outside) and i descending / j
// ascending (posterior).  Float log-sum-exp and float += are not associative,
// so the value of a target depends on the order its contributions arrive.
// Here each target GATHERS its contributions, enumerating its sources in
// exactly the order the reference's scatter reaches it, with each
// contribution computed by the same operations -- a parallel formulation
// with bitwise the reference's results.  Derivations are next to each cell.
#pragma once

#include "cf_inside.cuh"

namespace cf {

struct OutTabs {
    const float* FC;
    const float* FM;
    const float* FM1;
    const float* F5;
    float* FCo;
    float* FMo;
    float* FM1o;
    float* FM2o;
    float* F5o;
    int m;
    __device__ __forceinline__ int at(int i, int j) const { return tri_off(j - i, m) + i; }
};

// F5o (cpu.py:684-699) by one warp, k = L-1 .. 0.  Target k receives, in the
// reference's order, the pair terms of iterations j = L .. k+2 and then the
// unpaired term F5o[k+1] + eu of iteration j = k+1.
__device__ __forceinline__ void exterior_outside_warp(const Lse32& sr, const SmemTabs<float>* __restrict__ tb,
                                                      const SeqView& Q, const OutTabs& T) {
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

// One outside cell (a, b): FMo, FM1o, FCo, FM2o.  Needs every cell of larger
// span finished.
__device__ __forceinline__ void outside_cell(const Lse32& sr, const SmemTabs<float>* __restrict__ tb,
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
__device__ __forceinline__ float posterior_cell(const SmemTabs<float>* __restrict__ tb, const PolyTables* pt,
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

}  // namespace cf
