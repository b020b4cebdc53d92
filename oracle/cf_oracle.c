/*
 * cf_oracle.c -- TEST INFRASTRUCTURE ONLY.  CPU restatement of the reference
 * CONTRAfold engine (gpu_contrafold/cpu.py) used as the parity checker and as
 * the timed CPU baseline.  Nothing in the product links or calls this file.
 *
 * Every routine follows the reference's loop order and operation order
 * exactly, because the FP32 posterior and the MEA decode are compared bitwise:
 *   lse64          cpu.py:154-162
 *   inside64       cpu.py:165-275   (FP64, exact log1p/exp)
 *   viterbi64      cpu.py:290-502   (FP64 max-plus + EPS=1e-6 first-match traceback)
 *   lse32          cpu.py:527-557   (Fast_LogPlusEquals, 8-segment cubic)
 *   fexp32         cpu.py:560-580   (Fast_Exp, 6-segment cubic; exp in double above 0)
 *   posterior32    cpu.py:583-820   (FP32 inside, outside, posterior, clip)
 *   mea_decode32   cpu.py:823-895
 * Build with -O2 -ffp-contract=off (no fused multiply-add, no fast-math) so
 * each + and * rounds separately, as numpy float32 / float64 scalars do.
 *
 * Parameter blobs use the layout of include/contrafold_gb300.h (CF_OFF_*).
 * Sequences are passed as codes s[0..L+1] (0..3 = ACGU, 4 = N, sentinels
 * s[0] = s[L+1] = 4) and forced[0..L+1] (1 = forced unpaired), 1-based.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/contrafold_gb300.h"

#define CMAX 30
#define DHP 30

static const double NEG64 = -1e30, HALF64 = -5e29;
#define NEG32 ((float)-1e30)
#define HALF32 ((float)-5e29)
#define F(x) ((float)(x))

/* canonical pairs AU UA CG GC GU UG (cpu.py:25); N (4) never pairs */
static int canon(int a, int b) {
    static const unsigned char C[5][5] = {
        {0, 0, 0, 1, 0}, {0, 0, 1, 0, 0}, {0, 1, 0, 1, 0}, {1, 0, 1, 0, 0}, {0, 0, 0, 0, 0}};
    return C[a][b];
}

#define I2(a, b) ((a) * 5 + (b))
#define I3(a, b, c) (((a) * 5 + (b)) * 5 + (c))
#define I4(a, b, c, d) ((((a) * 5 + (b)) * 5 + (c)) * 5 + (d))

/* =========================== FP64 =========================== */

static inline double lse64(double a, double b) {
    if (a < HALF64) return b;
    if (b < HALF64) return a;
    if (a > b) return a + log1p(exp(b - a));
    return b + log1p(exp(a - b));
}

typedef struct {
    const double *bp, *stack, *tm, *hc, *dl, *dr, *hp, *cs, *i11, *b01;
    double mb, mu, mp, eu, ep;
} P64;

static P64 unpack64(const double* blob) {
    P64 p;
    p.bp = blob + CF_OFF_BP; p.stack = blob + CF_OFF_STACK; p.tm = blob + CF_OFF_TM;
    p.hc = blob + CF_OFF_HC; p.dl = blob + CF_OFF_DL; p.dr = blob + CF_OFF_DR;
    p.hp = blob + CF_OFF_HPCUM; p.cs = blob + CF_OFF_CS; p.i11 = blob + CF_OFF_I11;
    p.b01 = blob + CF_OFF_B01;
    p.mb = blob[CF_OFF_MB]; p.mu = blob[CF_OFF_MU]; p.mp = blob[CF_OFF_MP];
    p.eu = blob[CF_OFF_EU]; p.ep = blob[CF_OFF_EP];
    return p;
}

#define OK_PAIR(a, b) (canon(s[a], s[b]) && forced[a] == 0 && forced[b] == 0)

/* inside (cpu.py:165-275).  Tables are (L+2)x(L+2) row-major.  If tabs != NULL
 * the caller receives FC|FM|FM1|F5 (3*(L+2)^2 + (L+2) doubles). */
double oracle_inside64(const int8_t* s, int L, const int8_t* forced, const double* blob,
                       double* tabs) {
    P64 P = unpack64(blob);
    const int n = L + 2;
    double* FC = (double*)malloc(sizeof(double) * (3 * (size_t)n * n + n));
    double* FM = FC + (size_t)n * n;
    double* FM1 = FM + (size_t)n * n;
    double* F5 = FM1 + (size_t)n * n;
    for (size_t t = 0; t < 3 * (size_t)n * n + n; ++t) FC[t] = NEG64;
#define T(A, i, j) A[(size_t)(i) * n + (j)]
    for (int i = L; i >= 0; --i) {
        for (int j = i; j <= L; ++j) {
            double FM2 = NEG64;
            for (int k = i + 1; k < j; ++k)
                if (T(FM1, i, k) > HALF64 && T(FM, k, j) > HALF64)
                    FM2 = lse64(FM2, T(FM1, i, k) + T(FM, k, j));
            if (0 < i && j < L && OK_PAIR(i, j + 1)) {
                double sum = NEG64;
                double jB = P.hc[I2(s[i], s[j + 1])] + P.tm[I4(s[i], s[j + 1], s[i + 1], s[j])];
                sum = lse64(sum, jB + P.hp[j - i <= DHP ? j - i : DHP]);
                int pmax = i + CMAX < j ? i + CMAX : j;
                for (int p = i; p <= pmax; ++p) {
                    int l1 = p - i;
                    int qmin = p + 2, alt = p - i + j - CMAX;
                    if (alt > qmin) qmin = alt;
                    for (int q = j; q >= qmin; --q) {
                        int l2 = j - q;
                        if (OK_PAIR(p + 1, q) && T(FC, p + 1, q - 1) > HALF64) {
                            double e;
                            if (p == i && q == j) {
                                e = P.bp[I2(s[i + 1], s[j])] + P.stack[I4(s[i], s[j + 1], s[i + 1], s[j])];
                            } else {
                                double jB1 = P.hc[I2(s[i], s[j + 1])] + P.tm[I4(s[i], s[j + 1], s[i + 1], s[j])];
                                double jB2 = P.hc[I2(s[q], s[p + 1])] + P.tm[I4(s[q], s[p + 1], s[q + 1], s[p])];
                                double snuc = 0.0;
                                if (l1 == 0 && l2 == 1) snuc = P.b01[s[j]];
                                else if (l1 == 1 && l2 == 0) snuc = P.b01[s[i + 1]];
                                else if (l1 == 1 && l2 == 1) snuc = P.i11[I2(s[i + 1], s[j])];
                                e = P.cs[l1 * 31 + l2] + P.bp[I2(s[p + 1], s[q])] + jB1 + jB2 + snuc;
                            }
                            sum = lse64(sum, e + T(FC, p + 1, q - 1));
                        }
                    }
                }
                if (FM2 > HALF64) {
                    double jA = P.hc[I2(s[i], s[j + 1])];
                    if (i < L) jA += P.dl[I3(s[i], s[j + 1], s[i + 1])];
                    if (j > 0) jA += P.dr[I3(s[i], s[j + 1], s[j])];
                    sum = lse64(sum, FM2 + jA + P.mp + P.mb);
                }
                T(FC, i, j) = sum;
            }
            if (0 < i && i + 2 <= j && j < L) {
                double sum = NEG64;
                if (OK_PAIR(i + 1, j) && T(FC, i + 1, j - 1) > HALF64) {
                    double jAji = P.hc[I2(s[j], s[i + 1])];
                    if (j < L) jAji += P.dl[I3(s[j], s[i + 1], s[j + 1])];
                    if (i > 0) jAji += P.dr[I3(s[j], s[i + 1], s[i])];
                    sum = lse64(sum, T(FC, i + 1, j - 1) + jAji + P.mp + P.bp[I2(s[i + 1], s[j])]);
                }
                if (T(FM1, i + 1, j) > HALF64) sum = lse64(sum, T(FM1, i + 1, j) + P.mu);
                T(FM1, i, j) = sum;
            }
            if (0 < i && i + 2 <= j && j < L) {
                double sum = NEG64;
                if (FM2 > HALF64) sum = lse64(sum, FM2);
                if (T(FM, i, j - 1) > HALF64) sum = lse64(sum, T(FM, i, j - 1) + P.mu);
                if (T(FM1, i, j) > HALF64) sum = lse64(sum, T(FM1, i, j));
                T(FM, i, j) = sum;
            }
        }
    }
    F5[0] = 0.0;
    for (int j = 1; j <= L; ++j) {
        double sum = F5[j - 1] + P.eu;
        for (int k = 0; k < j; ++k) {
            if (OK_PAIR(k + 1, j) && T(FC, k + 1, j - 1) > HALF64 && F5[k] > HALF64) {
                double jA = P.hc[I2(s[j], s[k + 1])];
                if (j < L) jA += P.dl[I3(s[j], s[k + 1], s[j + 1])];
                if (k > 0) jA += P.dr[I3(s[j], s[k + 1], s[k])];
                sum = lse64(sum, F5[k] + T(FC, k + 1, j - 1) + P.ep + P.bp[I2(s[k + 1], s[j])] + jA);
            }
        }
        F5[j] = sum;
    }
    double z = F5[L];
    if (tabs) memcpy(tabs, FC, sizeof(double) * (3 * (size_t)n * n + n));
    free(FC);
    return z;
}

/* Extension of inside64 (not in the reference): a soft per-position unpaired
 * bonus u[1..L] added for every unpaired position -- hairpin interiors,
 * single-branch loop interiors, multiloop (FM1 / FM extensions) and exterior
 * unpaired positions.  With u == NULL this is inside64.  Used as the FP64
 * finite-difference oracle of the adjoint. */
double oracle_inside64_bonus(const int8_t* s, int L, const int8_t* forced, const double* blob,
                             const double* u) {
    if (!u) return oracle_inside64(s, L, forced, blob, NULL);
    P64 P = unpack64(blob);
    const int n = L + 2;
    double* U = (double*)calloc((size_t)n, sizeof(double));
    for (int k = 1; k <= L; ++k) U[k] = U[k - 1] + u[k];
    double* FC = (double*)malloc(sizeof(double) * (3 * (size_t)n * n + n));
    double* FM = FC + (size_t)n * n;
    double* FM1 = FM + (size_t)n * n;
    double* F5 = FM1 + (size_t)n * n;
    for (size_t t = 0; t < 3 * (size_t)n * n + n; ++t) FC[t] = NEG64;
    for (int i = L; i >= 0; --i) {
        for (int j = i; j <= L; ++j) {
            double FM2 = NEG64;
            for (int k = i + 1; k < j; ++k)
                if (T(FM1, i, k) > HALF64 && T(FM, k, j) > HALF64)
                    FM2 = lse64(FM2, T(FM1, i, k) + T(FM, k, j));
            if (0 < i && j < L && OK_PAIR(i, j + 1)) {
                double sum = NEG64;
                double jB = P.hc[I2(s[i], s[j + 1])] + P.tm[I4(s[i], s[j + 1], s[i + 1], s[j])];
                sum = lse64(sum, jB + P.hp[j - i <= DHP ? j - i : DHP] + (U[j] - U[i]));
                int pmax = i + CMAX < j ? i + CMAX : j;
                for (int p = i; p <= pmax; ++p) {
                    int l1 = p - i;
                    int qmin = p + 2, alt = p - i + j - CMAX;
                    if (alt > qmin) qmin = alt;
                    for (int q = j; q >= qmin; --q) {
                        int l2 = j - q;
                        if (OK_PAIR(p + 1, q) && T(FC, p + 1, q - 1) > HALF64) {
                            double e;
                            if (p == i && q == j) {
                                e = P.bp[I2(s[i + 1], s[j])] + P.stack[I4(s[i], s[j + 1], s[i + 1], s[j])];
                            } else {
                                double jB1 = P.hc[I2(s[i], s[j + 1])] + P.tm[I4(s[i], s[j + 1], s[i + 1], s[j])];
                                double jB2 = P.hc[I2(s[q], s[p + 1])] + P.tm[I4(s[q], s[p + 1], s[q + 1], s[p])];
                                double snuc = 0.0;
                                if (l1 == 0 && l2 == 1) snuc = P.b01[s[j]];
                                else if (l1 == 1 && l2 == 0) snuc = P.b01[s[i + 1]];
                                else if (l1 == 1 && l2 == 1) snuc = P.i11[I2(s[i + 1], s[j])];
                                e = P.cs[l1 * 31 + l2] + P.bp[I2(s[p + 1], s[q])] + jB1 + jB2 + snuc;
                            }
                            double bon = (U[p] - U[i]) + (U[j] - U[q]);
                            sum = lse64(sum, e + T(FC, p + 1, q - 1) + bon);
                        }
                    }
                }
                if (FM2 > HALF64) {
                    double jA = P.hc[I2(s[i], s[j + 1])];
                    if (i < L) jA += P.dl[I3(s[i], s[j + 1], s[i + 1])];
                    if (j > 0) jA += P.dr[I3(s[i], s[j + 1], s[j])];
                    sum = lse64(sum, FM2 + jA + P.mp + P.mb);
                }
                T(FC, i, j) = sum;
            }
            if (0 < i && i + 2 <= j && j < L) {
                double sum = NEG64;
                if (OK_PAIR(i + 1, j) && T(FC, i + 1, j - 1) > HALF64) {
                    double jAji = P.hc[I2(s[j], s[i + 1])];
                    if (j < L) jAji += P.dl[I3(s[j], s[i + 1], s[j + 1])];
                    if (i > 0) jAji += P.dr[I3(s[j], s[i + 1], s[i])];
                    sum = lse64(sum, T(FC, i + 1, j - 1) + jAji + P.mp + P.bp[I2(s[i + 1], s[j])]);
                }
                if (T(FM1, i + 1, j) > HALF64) sum = lse64(sum, T(FM1, i + 1, j) + P.mu + u[i + 1]);
                T(FM1, i, j) = sum;
            }
            if (0 < i && i + 2 <= j && j < L) {
                double sum = NEG64;
                if (FM2 > HALF64) sum = lse64(sum, FM2);
                if (T(FM, i, j - 1) > HALF64) sum = lse64(sum, T(FM, i, j - 1) + P.mu + u[j]);
                if (T(FM1, i, j) > HALF64) sum = lse64(sum, T(FM1, i, j));
                T(FM, i, j) = sum;
            }
        }
    }
    F5[0] = 0.0;
    for (int j = 1; j <= L; ++j) {
        double sum = F5[j - 1] + P.eu + u[j];
        for (int k = 0; k < j; ++k) {
            if (OK_PAIR(k + 1, j) && T(FC, k + 1, j - 1) > HALF64 && F5[k] > HALF64) {
                double jA = P.hc[I2(s[j], s[k + 1])];
                if (j < L) jA += P.dl[I3(s[j], s[k + 1], s[j + 1])];
                if (k > 0) jA += P.dr[I3(s[j], s[k + 1], s[k])];
                sum = lse64(sum, F5[k] + T(FC, k + 1, j - 1) + P.ep + P.bp[I2(s[k + 1], s[j])] + jA);
            }
        }
        F5[j] = sum;
    }
    double z = F5[L];
    free(FC);
    free(U);
    return z;
}

/* Viterbi + EPS first-match traceback (cpu.py:290-502).  pair[0..L+1]
 * receives the 1-based partner of each position or -1. */
void oracle_viterbi64(const int8_t* s, int L, const int8_t* forced, const double* blob,
                      int64_t* pair) {
    P64 P = unpack64(blob);
    const int n = L + 2;
    double* FC = (double*)malloc(sizeof(double) * (3 * (size_t)n * n + n));
    double* FM = FC + (size_t)n * n;
    double* FM1 = FM + (size_t)n * n;
    double* F5 = FM1 + (size_t)n * n;
    for (size_t t = 0; t < 3 * (size_t)n * n + n; ++t) FC[t] = NEG64;
    for (int i = L; i >= 0; --i) {
        for (int j = i; j <= L; ++j) {
            double FM2 = NEG64;
            for (int k = i + 1; k < j; ++k)
                if (T(FM1, i, k) > HALF64 && T(FM, k, j) > HALF64) {
                    double v = T(FM1, i, k) + T(FM, k, j);
                    if (v > FM2) FM2 = v;
                }
            if (0 < i && j < L && OK_PAIR(i, j + 1)) {
                double best = NEG64;
                double jB = P.hc[I2(s[i], s[j + 1])] + P.tm[I4(s[i], s[j + 1], s[i + 1], s[j])];
                double v = jB + P.hp[j - i <= DHP ? j - i : DHP];
                if (v > best) best = v;
                int pmax = i + CMAX < j ? i + CMAX : j;
                for (int p = i; p <= pmax; ++p) {
                    int l1 = p - i;
                    int qmin = p + 2, alt = p - i + j - CMAX;
                    if (alt > qmin) qmin = alt;
                    for (int q = j; q >= qmin; --q) {
                        int l2 = j - q;
                        if (OK_PAIR(p + 1, q) && T(FC, p + 1, q - 1) > HALF64) {
                            double e;
                            if (p == i && q == j) {
                                e = P.bp[I2(s[i + 1], s[j])] + P.stack[I4(s[i], s[j + 1], s[i + 1], s[j])];
                            } else {
                                double jB2 = P.hc[I2(s[q], s[p + 1])] + P.tm[I4(s[q], s[p + 1], s[q + 1], s[p])];
                                double snuc = 0.0;
                                if (l1 == 0 && l2 == 1) snuc = P.b01[s[j]];
                                else if (l1 == 1 && l2 == 0) snuc = P.b01[s[i + 1]];
                                else if (l1 == 1 && l2 == 1) snuc = P.i11[I2(s[i + 1], s[j])];
                                e = P.cs[l1 * 31 + l2] + P.bp[I2(s[p + 1], s[q])] + jB + jB2 + snuc;
                            }
                            v = e + T(FC, p + 1, q - 1);
                            if (v > best) best = v;
                        }
                    }
                }
                if (FM2 > HALF64) {
                    double jA = P.hc[I2(s[i], s[j + 1])];
                    if (i < L) jA += P.dl[I3(s[i], s[j + 1], s[i + 1])];
                    if (j > 0) jA += P.dr[I3(s[i], s[j + 1], s[j])];
                    v = FM2 + jA + P.mp + P.mb;
                    if (v > best) best = v;
                }
                T(FC, i, j) = best;
            }
            if (0 < i && i + 2 <= j && j < L) {
                double best = NEG64;
                if (OK_PAIR(i + 1, j) && T(FC, i + 1, j - 1) > HALF64) {
                    double jAji = P.hc[I2(s[j], s[i + 1])];
                    if (j < L) jAji += P.dl[I3(s[j], s[i + 1], s[j + 1])];
                    if (i > 0) jAji += P.dr[I3(s[j], s[i + 1], s[i])];
                    double v = T(FC, i + 1, j - 1) + jAji + P.mp + P.bp[I2(s[i + 1], s[j])];
                    if (v > best) best = v;
                }
                if (T(FM1, i + 1, j) > HALF64) {
                    double v = T(FM1, i + 1, j) + P.mu;
                    if (v > best) best = v;
                }
                T(FM1, i, j) = best;
            }
            if (0 < i && i + 2 <= j && j < L) {
                double best = NEG64;
                if (FM2 > HALF64 && FM2 > best) best = FM2;
                if (T(FM, i, j - 1) > HALF64) {
                    double v = T(FM, i, j - 1) + P.mu;
                    if (v > best) best = v;
                }
                if (T(FM1, i, j) > HALF64 && T(FM1, i, j) > best) best = T(FM1, i, j);
                T(FM, i, j) = best;
            }
        }
    }
    F5[0] = 0.0;
    for (int j = 1; j <= L; ++j) {
        double best = F5[j - 1] + P.eu;
        for (int k = 0; k < j; ++k) {
            if (OK_PAIR(k + 1, j) && T(FC, k + 1, j - 1) > HALF64 && F5[k] > HALF64) {
                double jA = P.hc[I2(s[j], s[k + 1])];
                if (j < L) jA += P.dl[I3(s[j], s[k + 1], s[j + 1])];
                if (k > 0) jA += P.dr[I3(s[j], s[k + 1], s[k])];
                double v = F5[k] + T(FC, k + 1, j - 1) + P.ep + P.bp[I2(s[k + 1], s[j])] + jA;
                if (v > best) best = v;
            }
        }
        F5[j] = best;
    }

    /* ---- traceback (cpu.py:396-501) ---- */
    const double EPS = 1e-6;
    for (int t = 0; t < n; ++t) pair[t] = -1;
    int cap = 4 * L + 16;
    int* st = (int*)malloc(sizeof(int) * 3 * cap);
    int *st_t = st, *st_i = st + cap, *st_j = st + 2 * cap;
    int sp = 0;
#define PUSH(tt, ii, jj) do { st_t[sp] = (tt); st_i[sp] = (ii); st_j[sp] = (jj); ++sp; } while (0)
    PUSH(0, 0, L);
    while (sp > 0) {
        --sp;
        int typ = st_t[sp], i = st_i[sp], j = st_j[sp];
        if (typ == 0) {
            if (j == 0) continue;
            double val = F5[j];
            int done = 0;
            if (F5[j - 1] > HALF64 && fabs(F5[j - 1] + P.eu - val) <= EPS) {
                PUSH(0, 0, j - 1);
                done = 1;
            }
            if (!done) {
                for (int k = 0; k < j; ++k) {
                    if (OK_PAIR(k + 1, j) && T(FC, k + 1, j - 1) > HALF64 && F5[k] > HALF64) {
                        double jA = P.hc[I2(s[j], s[k + 1])];
                        if (j < L) jA += P.dl[I3(s[j], s[k + 1], s[j + 1])];
                        if (k > 0) jA += P.dr[I3(s[j], s[k + 1], s[k])];
                        double v = F5[k] + T(FC, k + 1, j - 1) + P.ep + P.bp[I2(s[k + 1], s[j])] + jA;
                        if (fabs(v - val) <= EPS) {
                            pair[k + 1] = j; pair[j] = k + 1;
                            PUSH(1, k + 1, j - 1);
                            PUSH(0, 0, k);
                            break;
                        }
                    }
                }
            }
        } else if (typ == 1) {
            double val = T(FC, i, j);
            double jB = P.hc[I2(s[i], s[j + 1])] + P.tm[I4(s[i], s[j + 1], s[i + 1], s[j])];
            int d = j - i;
            int done = fabs(jB + P.hp[d <= DHP ? d : DHP] - val) <= EPS;
            if (!done) {
                int pmax = i + CMAX < j ? i + CMAX : j;
                for (int p = i; p <= pmax && !done; ++p) {
                    int l1 = p - i;
                    int qmin = p + 2, alt = p - i + j - CMAX;
                    if (alt > qmin) qmin = alt;
                    for (int q = j; q >= qmin; --q) {
                        int l2 = j - q;
                        if (OK_PAIR(p + 1, q) && T(FC, p + 1, q - 1) > HALF64) {
                            double e;
                            if (p == i && q == j) {
                                e = P.bp[I2(s[i + 1], s[j])] + P.stack[I4(s[i], s[j + 1], s[i + 1], s[j])];
                            } else {
                                double jB2 = P.hc[I2(s[q], s[p + 1])] + P.tm[I4(s[q], s[p + 1], s[q + 1], s[p])];
                                double snuc = 0.0;
                                if (l1 == 0 && l2 == 1) snuc = P.b01[s[j]];
                                else if (l1 == 1 && l2 == 0) snuc = P.b01[s[i + 1]];
                                else if (l1 == 1 && l2 == 1) snuc = P.i11[I2(s[i + 1], s[j])];
                                e = P.cs[l1 * 31 + l2] + P.bp[I2(s[p + 1], s[q])] + jB + jB2 + snuc;
                            }
                            if (fabs(e + T(FC, p + 1, q - 1) - val) <= EPS) {
                                pair[p + 1] = q; pair[q] = p + 1;
                                PUSH(1, p + 1, q - 1);
                                done = 1;
                                break;
                            }
                        }
                    }
                }
            }
            if (!done) {
                double jA = P.hc[I2(s[i], s[j + 1])];
                if (i < L) jA += P.dl[I3(s[i], s[j + 1], s[i + 1])];
                if (j > 0) jA += P.dr[I3(s[i], s[j + 1], s[j])];
                for (int k = i + 1; k < j; ++k) {
                    if (T(FM1, i, k) > HALF64 && T(FM, k, j) > HALF64 &&
                        fabs(T(FM1, i, k) + T(FM, k, j) + jA + P.mp + P.mb - val) <= EPS) {
                        PUSH(3, i, k);
                        PUSH(2, k, j);
                        break;
                    }
                }
            }
        } else if (typ == 2) {
            double val = T(FM, i, j);
            int done = 0;
            for (int k = i + 1; k < j; ++k) {
                if (T(FM1, i, k) > HALF64 && T(FM, k, j) > HALF64 &&
                    fabs(T(FM1, i, k) + T(FM, k, j) - val) <= EPS) {
                    PUSH(3, i, k);
                    PUSH(2, k, j);
                    done = 1;
                    break;
                }
            }
            if (!done && T(FM, i, j - 1) > HALF64 && fabs(T(FM, i, j - 1) + P.mu - val) <= EPS) {
                PUSH(2, i, j - 1);
                done = 1;
            }
            if (!done && T(FM1, i, j) > HALF64 && fabs(T(FM1, i, j) - val) <= EPS) PUSH(3, i, j);
        } else {
            double val = T(FM1, i, j);
            int done = 0;
            if (OK_PAIR(i + 1, j) && T(FC, i + 1, j - 1) > HALF64) {
                double jAji = P.hc[I2(s[j], s[i + 1])];
                if (j < L) jAji += P.dl[I3(s[j], s[i + 1], s[j + 1])];
                if (i > 0) jAji += P.dr[I3(s[j], s[i + 1], s[i])];
                if (fabs(T(FC, i + 1, j - 1) + jAji + P.mp + P.bp[I2(s[i + 1], s[j])] - val) <= EPS) {
                    pair[i + 1] = j; pair[j] = i + 1;
                    PUSH(1, i + 1, j - 1);
                    done = 1;
                }
            }
            if (!done && T(FM1, i + 1, j) > HALF64 && fabs(T(FM1, i + 1, j) + P.mu - val) <= EPS)
                PUSH(3, i + 1, j);
        }
    }
#undef PUSH
    free(st);
    free(FC);
}

/* =========================== FP32 =========================== */

/* Optional per-thread counters of guarded semiring updates (the roofline's
 * algorithmic unit), by category:
 *   0 inside single-branch LSE   1 inside bifurcation LSE   2 inside other terms
 *   3 outside single-branch LSE  4 outside bifurcation LSE  5 outside other terms
 *   6 posterior fexp terms       7 MEA max-plus candidates                     */
#define CF_NCOUNT 8
static __thread int64_t* g_cnt = NULL;
#define CNT(k) do { if (g_cnt) g_cnt[k]++; } while (0)

static inline float lse32(float a, float b) {
    if (a < b) { float t = a; a = b; b = t; }
    if (b < HALF32) return a;
    float d = a - b;
    if (d >= F(11.8624794162)) return a;
    float r;
    if (d < F(3.3792499610)) {
        if (d < F(1.6320158198)) {
            if (d < F(0.6615367791))
                r = ((F(-0.0065591595) * d + F(0.1276442762)) * d + F(0.4996554598)) * d + F(0.6931542306);
            else
                r = ((F(-0.0155157557) * d + F(0.1446775699)) * d + F(0.4882939746)) * d + F(0.6958092989);
        } else if (d < F(2.4912588184)) {
            r = ((F(-0.0128909247) * d + F(0.1301028251)) * d + F(0.5150398748)) * d + F(0.6795585882);
        } else {
            r = ((F(-0.0072142647) * d + F(0.0877540853)) * d + F(0.6208708362)) * d + F(0.5909675829);
        }
    } else if (d < F(5.7890710412)) {
        if (d < F(4.4261691294))
            r = ((F(-0.0031455354) * d + F(0.0467229449)) * d + F(0.7592532310)) * d + F(0.4348794399);
        else
            r = ((F(-0.0010110698) * d + F(0.0185943421)) * d + F(0.8831730747)) * d + F(0.2523695427);
    } else if (d < F(7.8162726752)) {
        r = ((F(-0.0001962780) * d + F(0.0046084408)) * d + F(0.9634431978)) * d + F(0.0983148903);
    } else {
        r = ((F(-0.0000113994) * d + F(0.0003734731)) * d + F(0.9959107193)) * d + F(0.0149855051);
    }
    return b + r;
}

static inline float fexp32(float x) {
    if (x < F(-2.4915033807)) {
        if (x < F(-5.8622823336)) {
            if (x < F(-9.91152)) return F(0.0);
            return ((F(0.0000803850) * x + F(0.0021627428)) * x + F(0.0194708555)) * x + F(0.0588080014);
        }
        if (x < F(-3.8396630909))
            return ((F(0.0013889414) * x + F(0.0244676474)) * x + F(0.1471290604)) * x + F(0.3042757740);
        return ((F(0.0072335607) * x + F(0.0906002677)) * x + F(0.3983111356)) * x + F(0.6245959221);
    }
    if (x < F(-0.6725053211)) {
        if (x < F(-1.4805375919))
            return ((F(0.0232410351) * x + F(0.2085645908)) * x + F(0.6906367911)) * x + F(0.8682322329);
        return ((F(0.0573782771) * x + F(0.3580258429)) * x + F(0.9121133217)) * x + F(0.9793091728);
    }
    if (x < F(0.0))
        return ((F(0.1199175927) * x + F(0.4815668234)) * x + F(0.9975991939)) * x + F(0.9999505077);
    if (x > F(46.052)) return F(1e20);
    return (float)exp((double)x);
}

float oracle_lse32(float a, float b) { return lse32(a, b); }
float oracle_fexp32(float x) { return fexp32(x); }

typedef struct {
    const float *bp, *stack, *tm, *hc, *dl, *dr, *hp, *cs, *i11, *b01;
    float mb, mu, mp, eu, ep;
} P32;

static P32 unpack32(const float* blob) {
    P32 p;
    p.bp = blob + CF_OFF_BP; p.stack = blob + CF_OFF_STACK; p.tm = blob + CF_OFF_TM;
    p.hc = blob + CF_OFF_HC; p.dl = blob + CF_OFF_DL; p.dr = blob + CF_OFF_DR;
    p.hp = blob + CF_OFF_HPCUM; p.cs = blob + CF_OFF_CS; p.i11 = blob + CF_OFF_I11;
    p.b01 = blob + CF_OFF_B01;
    p.mb = blob[CF_OFF_MB]; p.mu = blob[CF_OFF_MU]; p.mp = blob[CF_OFF_MP];
    p.eu = blob[CF_OFF_EU]; p.ep = blob[CF_OFF_EP];
    return p;
}

/* Number of floats oracle_posterior32 writes into `tabs` when non-NULL:
 * FC FM FM1 FCo FMo FM1o POST as (L+2)^2 each, then F5, F5o (L+2 each). */
size_t oracle_posterior32_tabs_len(int L) {
    size_t n = (size_t)L + 2;
    return 7 * n * n + 2 * n;
}

/* posterior (cpu.py:583-820), float32: the body is cf_oracle_post.inc */
#define PR float
#define PF_NAME oracle_posterior32
#define PF_PARAMS P32
#define PF_UNPACK unpack32
#define PF_NEG NEG32
#define PF_HALF HALF32
#define PF_LSE lse32
#define PF_EXP fexp32
#include "cf_oracle_post.inc"
#undef PR
#undef PF_NAME
#undef PF_PARAMS
#undef PF_UNPACK
#undef PF_NEG
#undef PF_HALF
#undef PF_LSE
#undef PF_EXP

/* The same recurrences in float64 with exact log-sum-exp and exp: the exact
 * pair probabilities (ours; test oracle of the sampler's frequencies). */
#define PR double
#define PF_NAME oracle_posterior64x
#define PF_PARAMS P64
#define PF_UNPACK unpack64
#define PF_NEG NEG64
#define PF_HALF HALF64
#define PF_LSE lse64
#define PF_EXP exp
#include "cf_oracle_post.inc"
#undef PR
#undef PF_NAME
#undef PF_PARAMS
#undef PF_UNPACK
#undef PF_NEG
#undef PF_HALF
#undef PF_LSE
#undef PF_EXP

/* MEA decode (cpu.py:823-895).  POST is (L+2)x(L+2) as from oracle_posterior32. */
void oracle_mea_decode32(const float* POST, int L, const int8_t* forced, const int8_t* s,
                         float gamma, int64_t* pair) {
    const int n = L + 2;
    const int m = L + 1;
    float g = gamma;
    float two_g = F(2.0) * g;
    float* up = (float*)calloc((size_t)m, sizeof(float));
    for (int i = 1; i <= L; ++i) {
        float u = F(1.0);
        for (int j = 1; j < i; ++j) u -= T(POST, j, i);
        for (int j = i + 1; j <= L; ++j) u -= T(POST, i, j);
        up[i] = u / two_g;
    }
    float* score = (float*)malloc(sizeof(float) * (size_t)m * m);
    int32_t* tb = (int32_t*)malloc(sizeof(int32_t) * (size_t)m * m);
    for (size_t t = 0; t < (size_t)m * m; ++t) { score[t] = F(-1.0); tb[t] = -1; }
#define S(i, j) score[(size_t)(i) * m + (j)]
#define TB(i, j) tb[(size_t)(i) * m + (j)]
    for (int i = L; i >= 0; --i) {
        for (int j = i; j <= L; ++j) {
            if (i == j) {
                if (F(0.0) > S(i, j)) { S(i, j) = F(0.0); TB(i, j) = 0; }
            } else {
                CNT(7); CNT(7); float v = up[i + 1] + S(i + 1, j);
                if (v > S(i, j)) { S(i, j) = v; TB(i, j) = 1; }
                v = up[j] + S(i, j - 1);
                if (v > S(i, j)) { S(i, j) = v; TB(i, j) = 2; }
                if (i + 2 <= j) {
                    if (OK_PAIR(i + 1, j)) {
                        CNT(7); v = T(POST, i + 1, j) + S(i + 1, j - 1);
                        if (v > S(i, j)) { S(i, j) = v; TB(i, j) = 3; }
                    }
                    for (int k = i + 1; k < j; ++k) {
                        CNT(7); v = S(i, k) + S(k, j);
                        if (v > S(i, j)) { S(i, j) = v; TB(i, j) = k + 4; }
                    }
                }
            }
        }
    }
    for (int t = 0; t < n; ++t) pair[t] = -1;
    int cap = 2 * L + 4;
    int* qi = (int*)malloc(sizeof(int) * 2 * cap);
    int* qj = qi + cap;
    int head = 0, tail = 1;
    qi[0] = 0; qj[0] = L;
    while (head < tail) {
        int i = qi[head], j = qj[head];
        ++head;
        int t = TB(i, j);
        if (t <= 0) continue;
        if (t == 1) { qi[tail] = i + 1; qj[tail] = j; ++tail; }
        else if (t == 2) { qi[tail] = i; qj[tail] = j - 1; ++tail; }
        else if (t == 3) {
            pair[i + 1] = j; pair[j] = i + 1;
            qi[tail] = i + 1; qj[tail] = j - 1; ++tail;
        } else {
            int k = t - 4;
            qi[tail] = i; qj[tail] = k; ++tail;
            qi[tail] = k; qj[tail] = j; ++tail;
        }
    }
#undef S
#undef TB
    free(qi); free(tb); free(score); free(up);
}

/* ====================== batch drivers (CPU baseline) ====================== */

/* Encode ASCII -> codes 1-based with sentinels (cpu.py:138-144). */
static void encode_one(const uint8_t* seq, const uint8_t* mask, int L, int8_t* s, int8_t* fo) {
    s[0] = 4; s[L + 1] = 4; fo[0] = 0; fo[L + 1] = 0;
    for (int t = 0; t < L; ++t) {
        uint8_t c = seq[t];
        if (c >= 'a' && c <= 'z') c = (uint8_t)(c - 32);
        int8_t v = 4;
        if (c == 'A') v = 0; else if (c == 'C') v = 1; else if (c == 'G') v = 2;
        else if (c == 'U' || c == 'T') v = 3;
        s[t + 1] = v;
        fo[t + 1] = (mask && mask[t]) ? 1 : 0;
    }
}

static void pairs_to_db(const int64_t* pair, int L, char* out) {
    for (int t = 0; t < L; ++t) out[t] = '.';
    for (int t = 1; t <= L; ++t)
        if (pair[t] > t) { out[t - 1] = '('; out[pair[t] - 1] = ')'; }
}

enum { JOB_MEA = 0, JOB_MFE = 1, JOB_LOGZ64 = 2, JOB_LOGZ32 = 3 };

typedef struct {
    int job;
    const uint8_t* seqs; const int64_t* offs; const uint8_t* mask;
    int n; const float* p32; const double* p64; float gamma;
    char* out_struct; double* out_z;
    int next; pthread_mutex_t mu;
} batch_t;

static void run_one(batch_t* B, int b) {
    int L = (int)(B->offs[b + 1] - B->offs[b]);
    int n = L + 2;
    int8_t* s = (int8_t*)malloc((size_t)2 * n);
    int8_t* fo = s + n;
    encode_one(B->seqs + B->offs[b], B->mask ? B->mask + B->offs[b] : NULL, L, s, fo);
    if (B->job == JOB_MEA) {
        float* POST = (float*)malloc(sizeof(float) * (size_t)n * n);
        int64_t* pair = (int64_t*)malloc(sizeof(int64_t) * n);
        oracle_posterior32(s, L, fo, B->p32, POST, NULL);
        oracle_mea_decode32(POST, L, fo, s, B->gamma, pair);
        pairs_to_db(pair, L, B->out_struct + B->offs[b]);
        free(pair); free(POST);
    } else if (B->job == JOB_MFE) {
        int64_t* pair = (int64_t*)malloc(sizeof(int64_t) * n);
        oracle_viterbi64(s, L, fo, B->p64, pair);
        pairs_to_db(pair, L, B->out_struct + B->offs[b]);
        free(pair);
    } else if (B->job == JOB_LOGZ64) {
        B->out_z[b] = oracle_inside64(s, L, fo, B->p64, NULL);
    } else {
        float* POST = (float*)malloc(sizeof(float) * (size_t)n * n);
        B->out_z[b] = oracle_posterior32(s, L, fo, B->p32, POST, NULL);
        free(POST);
    }
    free(s);
}

static void* worker(void* arg) {
    batch_t* B = (batch_t*)arg;
    for (;;) {
        pthread_mutex_lock(&B->mu);
        int b = B->next++;
        pthread_mutex_unlock(&B->mu);
        if (b >= B->n) break;
        run_one(B, b);
    }
    return NULL;
}

/* Run a batch on `threads` host threads (dynamic work distribution). */
int oracle_batch(int job, const uint8_t* seqs, const int64_t* offs, const uint8_t* mask, int n,
                 const float* p32, const double* p64, float gamma, char* out_struct,
                 double* out_z, int threads) {
    batch_t B;
    B.job = job; B.seqs = seqs; B.offs = offs; B.mask = mask; B.n = n; B.p32 = p32; B.p64 = p64;
    B.gamma = gamma; B.out_struct = out_struct; B.out_z = out_z; B.next = 0;
    pthread_mutex_init(&B.mu, NULL);
    if (threads < 1) threads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * threads);
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, worker, &B);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
    pthread_mutex_destroy(&B.mu);
    return 0;
}

/* Count the guarded updates of one MEA fold (posterior + decode) into cnt[8]. */
void oracle_count_mea_ops(const int8_t* s, int L, const int8_t* forced, const float* blob, float gamma,
                          int64_t* cnt) {
    const int n = L + 2;
    float* POST = (float*)malloc(sizeof(float) * (size_t)n * n);
    int64_t* pair = (int64_t*)malloc(sizeof(int64_t) * n);
    for (int k = 0; k < CF_NCOUNT; ++k) cnt[k] = 0;
    g_cnt = cnt;
    oracle_posterior32(s, L, forced, blob, POST, NULL);
    oracle_mea_decode32(POST, L, forced, s, gamma, pair);
    g_cnt = NULL;
    free(pair);
    free(POST);
}
