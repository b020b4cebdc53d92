// cf_sample.cuh -- Boltzmann stochastic traceback (gpu.py:196-477) on the FP32
// inside tables, one WARP per (sequence, sample).
//
// The reference gives each sample one thread that enumerates the candidate
// set of a state three times (max, sum of exp, cumulative pick).  Here the
// 32 lanes evaluate 32 candidates at once: pass 1 sums exp(w - m) chunk by
// chunk with an inclusive warp scan; pass 2 repeats the identical scans and
// stops at the first valid candidate whose running sum reaches r = U * S.
// Because both passes add in the same order, the running sum of pass 2 ends
// at exactly S >= r, so a pick always lands.  m is the state's own inside
// value (FC[i][j], FM[i][j], ...), which keeps the exponents near zero.
// Candidate order and weights follow the reference: F5 (unpaired, then
// k ascending), FC (hairpin, single-branch p ascending / q descending,
// multibranch k ascending), FM (splits k ascending, unpaired, FM1), FM1
// (pair, unpaired).
//
// Random numbers: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11), key = seed, counter =
// (sample, draw, sequence, 0): independent, reproducible streams per
// (seed, sequence, sample).
#pragma once

#include "cf_inside.cuh"

namespace cf {

__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += W0;
        k.y += W1;
    }
    return c;
}

__device__ __forceinline__ float uniform01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// Inclusive warp scan of x (Hillis-Steele, fixed association).
__device__ __forceinline__ float warp_scan(float x, int lane) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const float y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    return x;
}

// Two-pass chunked pick.  `enumerate(chunk)` calls chunk(valid, w, payload)
// warp-uniformly for each group of <= 32 candidates (returns false to stop).
struct Picker {
    int lane;
    float m;          // normaliser (the state's inside value)
    float run;        // running sum of exp(w - m)
    float r;          // target (pass 2)
    bool pass2;
    int picked;       // payload of the pick, or INT32_MIN
    __device__ __forceinline__ bool chunk(bool valid, float w, int payload) {
        const float x = valid ? expf(w - m) : 0.0f;
        const float inc = warp_scan(x, lane);
        const float tot = __shfl_sync(0xffffffffu, inc, 31);
        if (pass2) {
            const bool hit = valid && (run + inc >= r);
            const unsigned hm = __ballot_sync(0xffffffffu, hit);
            if (hm) {
                const int t = __ffs(hm) - 1;
                picked = __shfl_sync(0xffffffffu, payload, t);
                return false;
            }
        }
        run += tot;
        return true;
    }
};

template <class QV>
struct SampleCtx {
    const SmemTabs<float>* tb;
    QV Q;
    InTabs<float> T;
};

// enumerate candidates of F5(j): payload -1 = unpaired, k >= 0 = pair (k+1, j)
template <class C, class QV>
__device__ __forceinline__ void enum_f5(const SampleCtx<QV>& X, int j, int lane, C& ch) {
    const ParamView<float> P{X.tb->blob};
    const int L = X.Q.L;
    {
        const float f = X.T.F5[j - 1];
        const bool v = lane == 0 && f > CF_HALF32;
        if (!ch.chunk(v, __fadd_rn(f, P.eu()), -1)) return;
    }
    for (int k0 = 0; k0 < j; k0 += 32) {
        const int k = k0 + lane;
        bool v = false;
        float w = 0.0f;
        if (k < j && X.Q.pairable(k + 1, j)) {
            const float fcin = X.T.FC[X.T.at(k + 1, j - 1)], f5k = X.T.F5[k];
            if (fcin > CF_HALF32 && f5k > CF_HALF32) {
                const float jA = junctionA_rev<Lse32>(P, L, X.Q, k, j);
                w = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(f5k, fcin), P.ep()), P.bp(X.Q.s[k + 1], X.Q.s[j])), jA);
                v = true;
            }
        }
        if (!ch.chunk(v, w, k)) return;
    }
}

// FC(i, j): payload 0 = hairpin, 1 + (l1 * 32 + l2) = inner pair, 2048 + k = multiloop split
template <class C, class QV>
__device__ __forceinline__ void enum_fc(const SampleCtx<QV>& X, int i, int j, int lane, C& ch) {
    const ParamView<float> P{X.tb->blob};
    const QV& Q = X.Q;
    const int L = Q.L, d = j - i;
    const int si = Q.s[i], sj1 = Q.s[j + 1], si1 = Q.s[i + 1], sj = Q.s[j];
    const float jB = X.tb->jB[idx4(si, sj1, si1, sj)];
    if (!ch.chunk(lane == 0, __fadd_rn(jB, P.hp(d <= DHP ? d : DHP)), 0)) return;
    const int pmax = (i + CMAX < j) ? i + CMAX : j;
    for (int p = i; p <= pmax; ++p) {
        const int l1 = p - i;
        int qmin = p + 2;
        if (l1 + j - CMAX > qmin) qmin = l1 + j - CMAX;
        const int cnt = j - qmin + 1;
        if (cnt <= 0) continue;
        const int q = j - lane;
        bool v = false;
        float w = 0.0f;
        if (lane < cnt && Q.pairable(p + 1, q)) {
            const float inner = X.T.FC[X.T.at(p + 1, q - 1)];
            if (inner > CF_HALF32) {
                const int l2 = j - q;
                float e;
                if (l1 == 0 && l2 == 0) {
                    e = __fadd_rn(P.bp(si1, sj), P.stack(si, sj1, si1, sj));
                } else {
                    const float jB2 = X.tb->jB[idx4(Q.s[q], Q.s[p + 1], Q.s[q + 1], Q.s[p])];
                    float sn = 0.0f;
                    if (l1 == 0 && l2 == 1) sn = P.b01(sj);
                    else if (l1 == 1 && l2 == 0) sn = P.b01(si1);
                    else if (l1 == 1 && l2 == 1) sn = P.i11(si1, sj);
                    e = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(P.cs(l1, l2), P.bp(Q.s[p + 1], Q.s[q])), jB), jB2), sn);
                }
                w = __fadd_rn(e, inner);
                v = true;
            }
        }
        if (!ch.chunk(v, w, 1 + (l1 * 32 + (j - q)))) return;
    }
    const float jA = junctionA<Lse32>(P, L, Q, i, j);
    for (int k0 = i + 1; k0 < j; k0 += 32) {
        const int k = k0 + lane;
        bool v = false;
        float w = 0.0f;
        if (k < j) {
            const float f1 = X.T.FM1[X.T.at(i, k)], fm = X.T.FM[X.T.at(k, j)];
            if (f1 > CF_HALF32 && fm > CF_HALF32) {
                w = __fadd_rn(__fadd_rn(__fadd_rn(__fadd_rn(f1, fm), jA), P.mp()), P.mb());
                v = true;
            }
        }
        if (!ch.chunk(v, w, 2048 + k)) return;
    }
}

// FM(i, j): payload k = split, -1 = unpaired j, -2 = FM1(i, j)
template <class C, class QV>
__device__ __forceinline__ void enum_fm(const SampleCtx<QV>& X, int i, int j, int lane, C& ch) {
    const ParamView<float> P{X.tb->blob};
    for (int k0 = i + 1; k0 < j; k0 += 32) {
        const int k = k0 + lane;
        bool v = false;
        float w = 0.0f;
        if (k < j) {
            const float f1 = X.T.FM1[X.T.at(i, k)], fm = X.T.FM[X.T.at(k, j)];
            if (f1 > CF_HALF32 && fm > CF_HALF32) { w = __fadd_rn(f1, fm); v = true; }
        }
        if (!ch.chunk(v, w, k)) return;
    }
    const float prev = X.T.FM[X.T.at(i, j - 1)];
    if (!ch.chunk(lane == 0 && prev > CF_HALF32, __fadd_rn(prev, P.mu()), -1)) return;
    const float f1 = X.T.FM1[X.T.at(i, j)];
    ch.chunk(lane == 0 && f1 > CF_HALF32, f1, -2);
}

// FM1(i, j): payload 0 = pair (i+1, j), 1 = unpaired i+1
template <class C, class QV>
__device__ __forceinline__ void enum_fm1(const SampleCtx<QV>& X, int i, int j, int lane, C& ch) {
    const ParamView<float> P{X.tb->blob};
    const QV& Q = X.Q;
    bool v = false;
    float w = 0.0f;
    if (Q.pairable(i + 1, j)) {
        const float fin = X.T.FC[X.T.at(i + 1, j - 1)];
        if (fin > CF_HALF32) {
            const float jAji = junctionA_rev<Lse32>(P, Q.L, Q, i, j);
            w = __fadd_rn(__fadd_rn(__fadd_rn(fin, jAji), P.mp()), P.bp(Q.s[i + 1], Q.s[j]));
            v = true;
        }
    }
    if (!ch.chunk(lane == 0 && v, w, 0)) return;
    const float ext = X.T.FM1[X.T.at(i + 1, j)];
    ch.chunk(lane == 0 && ext > CF_HALF32, __fadd_rn(ext, P.mu()), 1);
}

template <class E>
__device__ __forceinline__ int pick(E enumerate, float m, float u, int lane, int* status) {
    Picker pk{lane, m, 0.0f, 0.0f, false, INT32_MIN};
    enumerate(pk);
    const float S = pk.run;
    Picker p2{lane, m, 0.0f, u * S, true, INT32_MIN};
    enumerate(p2);
    if (p2.picked == INT32_MIN && lane == 0) atomicExch(status, CF_EDEVICE);
    return p2.picked;
}


// Draw one structure for sample `smp` of the sequence with batch index
// `seq_idx` into out[0..L) (pre-filled with '.'), by the calling warp.  The
// traceback stack (`stack`, L+8 packed (type, i, j) entries in shared memory)
// is bounded: a traceback holds at most one pending state per disjoint
// interval of the sequence.
template <class QV>
__device__ __forceinline__ void sample_one(const SampleCtx<QV>& X, int smp, int seq_idx, uint2 key, char* out,
                                           uint32_t* stack, int* status, int lane) {
    const int L = X.Q.L;
    uint32_t draw = 0;
    int sp = 0;
    const int cap = L + 8;
    bool ok = true;
    auto push = [&](uint32_t typ, int i, int j) {
        if (sp >= cap) { ok = false; return; }
        if (lane == 0) stack[sp] = (typ << 30) | ((uint32_t)i << 15) | (uint32_t)j;
        ++sp;
    };
    push(0, 0, L);
    __syncwarp();
    while (sp > 0 && ok) {
        --sp;
        const uint32_t e = stack[sp];
        __syncwarp();
        const int typ = (int)(e >> 30), i = (int)((e >> 15) & 0x7FFF), j = (int)(e & 0x7FFF);
        if (typ == 0 && j == 0) continue;
        const uint4 rnd = philox4x32_10(make_uint4((uint32_t)smp, draw++, (uint32_t)seq_idx, 0u), key);
        const float u = uniform01(rnd.x);
        if (typ == 0) {
            const int pk = pick([&](auto& c) { enum_f5(X, j, lane, c); }, X.T.F5[j], u, lane, status);
            if (pk == INT32_MIN) break;
            if (pk == -1) {
                push(0, 0, j - 1);
            } else {
                if (lane == 0) { out[pk] = '('; out[j - 1] = ')'; }
                push(1, pk + 1, j - 1);
                push(0, 0, pk);
            }
        } else if (typ == 1) {
            const int pk = pick([&](auto& c) { enum_fc(X, i, j, lane, c); }, X.T.FC[X.T.at(i, j)], u, lane, status);
            if (pk == INT32_MIN) break;
            if (pk >= 2048) {
                const int k = pk - 2048;
                push(3, i, k);
                push(2, k, j);
            } else if (pk >= 1) {
                const int l1 = (pk - 1) >> 5, l2 = (pk - 1) & 31;
                const int p = i + l1, q = j - l2;
                if (lane == 0) { out[p] = '('; out[q - 1] = ')'; }
                push(1, p + 1, q - 1);
            }
        } else if (typ == 2) {
            const int pk = pick([&](auto& c) { enum_fm(X, i, j, lane, c); }, X.T.FM[X.T.at(i, j)], u, lane, status);
            if (pk == INT32_MIN) break;
            if (pk >= 0) {
                push(3, i, pk);
                push(2, pk, j);
            } else if (pk == -1) {
                push(2, i, j - 1);
            } else {
                push(3, i, j);
            }
        } else {
            const int pk = pick([&](auto& c) { enum_fm1(X, i, j, lane, c); }, X.T.FM1[X.T.at(i, j)], u, lane, status);
            if (pk == INT32_MIN) break;
            if (pk == 0) {
                if (lane == 0) { out[i] = '('; out[j - 1] = ')'; }
                push(1, i + 1, j - 1);
            } else {
                push(3, i + 1, j);
            }
        }
        __syncwarp();
    }
    if (!ok && lane == 0) atomicExch(status, CF_EDEVICE);
}

}  // namespace cf
