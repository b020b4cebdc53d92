// cf_mea.cuh -- maximum-expected-accuracy decode (gpu_contrafold/cpu.py:823-895).
//
// The reference fills score[i][j] with strict '>' comparisons over the
// candidate order (init -1, i+1 unpaired, j unpaired, pair (i+1, j),
// bifurcations k ascending), so each cell keeps the FIRST candidate that
// reaches the maximum.  Each cell here evaluates the same candidates in the
// same order with the same float adds, so score and argmax are bitwise the
// reference's; traceback order does not affect the result.
#pragma once

#include "cf_inside.cuh"

namespace cf {

// up[i] = (1 - sum_{j<i} POST[j][i] - sum_{j>i} POST[i][j]) / (2 gamma), the
// subtractions in the reference's order (j ascending).  POST triangular.
__device__ __forceinline__ float mea_unpaired(const float* __restrict__ POST, int L, float two_g, int i) {
    const int m = L + 1;
    float u = 1.0f;
    for (int jj = 1; jj < i; ++jj) u = __fsub_rn(u, POST[tri_off(i - jj, m) + jj]);
    for (int jj = i + 1; jj <= L; ++jj) u = __fsub_rn(u, POST[tri_off(jj - i, m) + i]);
    return __fdiv_rn(u, two_g);
}

// One DP cell (i, j) of the decode.  QV provides pairable(a, b).
template <int CPF = kChainPF, class QV>
__device__ __forceinline__ void mea_cell(const QV& Q, const float* __restrict__ POST, const float* __restrict__ up,
                                         float* __restrict__ score, int* __restrict__ tb, int L, int i, int j) {
    const int m = L + 1;
    const int c = tri_off(j - i, m) + i;
    if (i == j) {
        score[c] = 0.0f;
        tb[c] = 0;
        return;
    }
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
        // bifurcations k = i+1 .. j-1: score[i][k] (span s1 = k-i), score[k][j] (span s2 = j-k)
        int o1 = tri_off(1, m) + i;               // score[i][i+1]
        int o2 = tri_off(j - i - 1, m) + i + 1;   // score[i+1][j]
        int s1 = 1, s2 = j - i - 1;
        prefetched_chain<float, CPF>(
            j - i - 1,
            [&](const float*& x, const float*& y) {
                x = score + o1;
                y = score + o2;
                o1 += m - s1;
                o2 += s2 - m;
                ++s1;
                --s2;
            },
            [&](int k, float x, float y) {
                const float vv = __fadd_rn(x, y);
                if (vv > best) { best = vv; arg = i + 1 + k + 4; }
            });
    }
    score[c] = best;
    tb[c] = arg;
}

// Breadth-first traceback from (0, L) (cpu.py:873-894) by one thread; writes
// '(' / ')' over a buffer the caller pre-filled with '.'.  The queue holds
// 2L+4 entries per coordinate.
__device__ __forceinline__ void mea_traceback(const int* __restrict__ tb, int L, int* qi, int* qj, char* out,
                                              int* status) {
    const int m = L + 1, cap = 2 * L + 4;
    int head = 0, tail = 1;
    qi[0] = 0;
    qj[0] = L;
    while (head < tail) {
        const int i = qi[head], j = qj[head];
        ++head;
        const int t = tb[tri_off(j - i, m) + i];
        if (t <= 0) continue;
        if (tail + 2 > cap) {
            atomicExch(status, CF_EDEVICE);
            return;
        }
        if (t == 1) {
            qi[tail] = i + 1; qj[tail] = j; ++tail;
        } else if (t == 2) {
            qi[tail] = i; qj[tail] = j - 1; ++tail;
        } else if (t == 3) {
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

}  // namespace cf
