// cf_queue.cu -- the dataflow schedule: one persistent launch for batches of
// any length mix, in which warps pull (sequence, step, chunk) work items.
//
// DISABLED: cf_engine_set_schedule refuses this schedule and the schedule
// table does not accept it, so nothing launches this kernel.  In two GPU test
// runs (the 1/3/64-seat MEA/BPP/logZ test and the sampling test) a launch did
// not finish, although every wait below is bounded in time; the cause has not
// been found.  It was also slower than the grouped kernels on every measured
// batch (10,000 x 200 nt MEA 15.8k vs 33.4k folds/s; 4,096 x U{40..400} 12.4k
// vs 16.3k).
//
// Every CTA keeps `seats` sequences in progress at once.  A sequence's fold
// is a chain of steps -- inside diagonals (pipelined two-phase steps
// A(t) + B(t-1)), the exterior recurrence, outside diagonals, the posterior,
// the MEA wavefront, the traceback, or the stochastic tracebacks -- and each
// step is cut into chunks of 32 work items (DP cells, pairs, samples).  A
// warp takes the next chunk of any seat whose current step has chunks left
// (claimed with one shared-memory atomic), folds it, and counts it done; the
// warp that finishes a step's last chunk opens the seat's next step (and runs
// the small serial steps -- the exterior recurrences, the pair list of the
// next diagonal, the traceback -- itself).  When a sequence is finished, the
// same warp takes the next sequence from the launch's global queue (longest
// first) into the seat, so sequences of every length share one launch and the
// SMs stay busy until the queue is empty.  No block-wide barrier is used after
// set-up: a seat waiting for its slowest chunk does not hold up the others.
//
// Ordering: chunk results go to global memory and are published with a CTA
// fence before the done count; a step's parameters are written before its
// claim word is published (fence, then an atomic exchange), and a claimer
// fences after its claim before it reads them.  Waits for work are polls of
// shared memory bounded in time: a warp that finds no work for kIdleLimitNs
// sets CF_ETIMEOUT and leaves (the rest of the CTA then runs out of work too),
// and no warp schedules work for longer than kLaunchLimitNs.
//
// Per-cell arithmetic is the one of the other schedules (cf_inside.cuh,
// cf_outside.cuh, cf_mea.cuh, cf_sample.cuh): results are identical, bit for
// bit, and the reference's per-cell order is kept.
#include "cf_mea.cuh"
#include "cf_outside.cuh"
#include "cf_queue.h"
#include "cf_sample.cuh"

namespace cf {

namespace {

enum Stage : int { kIn = 0, kOut, kPostZero, kPost, kUp, kMea, kSample, kFinished };

// Claim word of a seat: generation (16 bits) | chunks of the step (24) | chunks claimed (24).
__device__ __forceinline__ unsigned long long claim_word(unsigned gen, unsigned total) {
    return ((unsigned long long)(gen & 0xFFFFu) << 48) | ((unsigned long long)(total & 0xFFFFFFu) << 24);
}
__device__ __forceinline__ unsigned cw_total(unsigned long long w) { return (unsigned)(w >> 24) & 0xFFFFFFu; }
__device__ __forceinline__ unsigned cw_claimed(unsigned long long w) { return (unsigned)w & 0xFFFFFFu; }
__device__ __forceinline__ unsigned cw_gen(unsigned long long w) { return (unsigned)(w >> 48); }

// One seat: the sequence in progress and its open step.
struct Seat {
    unsigned long long claim;   // see claim_word
    int done;                   // chunks of the open step finished
    int stage, t;               // open step
    int nb, nb_chunks;          // B items of an inside / outside step and their chunks
    int na;                     // A items (cells of diagonal t), pairs, cells, samples ...
    int pl_o;                   // pair-list offset of the step's B items
    int pl_next;                // pair-list entries written so far (inside)
    SeqDesc D;
};

struct QueueSmemHead {
    SmemTabs<float> tabs;
    PolyTables poly;
    int alive;                  // seats still holding or taking sequences
};

constexpr int kQueueWarps = kQueueThreads / 32;
#ifndef CF_QUEUE_MAX_BACKOFF_NS
#define CF_QUEUE_MAX_BACKOFF_NS 2048
#endif
constexpr unsigned long long kIdleLimitNs = 20ull * 1000 * 1000 * 1000;   // 20 s without any work: give up
// a launch that is still scheduling after this long has lost its way: every
// warp gives up at its next poll, with CF_ETIMEOUT
constexpr unsigned long long kLaunchLimitNs = 120ull * 1000 * 1000 * 1000;

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Shared-memory layout after the head: seats, then per seat the sequence codes
// (s, pc: code stride each; PB: 4 x W words), then per warp a traceback stack
// (sampling only).
struct QueueLayout {
    int cs, W, seat_bytes, stack_words;
    size_t seats_off, codes_off, stacks_off, total;
};

__host__ __device__ __forceinline__ QueueLayout queue_layout(int Lmax, int seats, bool sampling) {
    QueueLayout Y;
    Y.cs = (Lmax + 2 + 15) & ~15;
    Y.W = pb_words(Lmax);
    Y.seat_bytes = 2 * Y.cs + 16 * Y.W;
    Y.stack_words = sampling ? Lmax + 8 : 0;
    Y.seats_off = (sizeof(QueueSmemHead) + 15) & ~size_t(15);
    Y.codes_off = Y.seats_off + (((size_t)seats * sizeof(Seat) + 15) & ~size_t(15));
    Y.stacks_off = Y.codes_off + (size_t)seats * Y.seat_bytes;
    Y.total = Y.stacks_off + (size_t)kQueueWarps * Y.stack_words * 4;
    return Y;
}

template <int MODE>
struct QueueCtx {
    const QueueArgs& A;
    QueueSmemHead* sm;
    Seat* seats;
    unsigned char* codes;
    uint32_t* stack;   // this warp's traceback stack (sampling)
    QueueLayout Y;
    int lane;

    __device__ __forceinline__ SeqV seq(int s) const {
        unsigned char* b = codes + (size_t)s * Y.seat_bytes;
        return SeqV{reinterpret_cast<const int8_t*>(b), reinterpret_cast<const int8_t*>(b + Y.cs),
                    reinterpret_cast<const uint32_t*>(b + 2 * Y.cs), Y.W, seats[s].D.L};
    }
    __device__ __forceinline__ float* base(int s) const {
        return A.ws + ((int64_t)blockIdx.x * A.seats + s) * A.slot_words;
    }
    __device__ __forceinline__ InTabs<float> in_tabs(int s, int L) const {
        const Arena32 ar = arena32(L);
        float* b = base(s);
        InTabs<float> T;
        T.FC = b + ar.FC; T.FM = b + ar.FM; T.FM1 = b + ar.FM1; T.F5 = b + ar.F5; T.m = L + 1;
        T.sized(L);
        return T;
    }
    __device__ __forceinline__ OutTabs out_tabs(int s, int L) const {
        const Arena32 ar = arena32(L);
        float* b = base(s);
        OutTabs O;
        O.FC = b + ar.FC; O.FM = b + ar.FM; O.FM1 = b + ar.FM1; O.F5 = b + ar.F5;
        O.FCo = b + ar.FCo; O.FMo = b + ar.FMo; O.FM1o = b + ar.FM1o; O.FM2o = b + ar.FM2o; O.F5o = b + ar.F5o;
        O.m = L + 1;
        O.sized(L);
        return O;
    }
    __device__ __forceinline__ PairList plist(int s, int L) const { return plist_at(base(s) + arena32(L).PL, L); }

    // ---- serial pieces, run by the warp that opens a step ----

    // Pair-list entries of diagonal dB (pairable cells (i, i + dB), i ascending).
    __device__ void plist_diagonal(int s, int dB) {
        Seat& St = seats[s];
        const SeqV Q = seq(s);
        const PairList PL = plist(s, Q.L);
        const unsigned below = (1u << lane) - 1u;
        int o = St.pl_next;
        if (lane == 0) PL.poff[dB] = o;
        for (int i0 = 1; i0 + dB <= Q.L - 1; i0 += 32) {
            const int i = i0 + lane;
            const bool ok = (i + dB <= Q.L - 1) && Q.pairable(i, i + dB + 1);
            const unsigned mk = __ballot_sync(0xffffffffu, ok);
            if (ok) PL.pl[o + __popc(mk & below)] = (int16_t)i;
            o += __popc(mk);
        }
        if (lane == 0) PL.poff[dB + 1] = o;
        St.pl_next = o;   // every lane writes the same value
        __syncwarp();
    }

    // Takes the next sequence of the launch into seat s; false when the queue is empty.
    __device__ bool admit(int s) {
        int item = 0;
        if (lane == 0) item = atomicAdd(A.counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (item >= A.n) return false;
        const SeqDesc D = A.descs[item];
        unsigned char* b = codes + (size_t)s * Y.seat_bytes;
        build_seq_warp_q(D, reinterpret_cast<int8_t*>(b), reinterpret_cast<int8_t*>(b + Y.cs),
                         reinterpret_cast<uint32_t*>(b + 2 * Y.cs));
        if (lane == 0) {
            seats[s].D = D;
            seats[s].pl_next = 0;
        }
        __syncwarp();
        return true;
    }

    __device__ __forceinline__ void build_seq_warp_q(const SeqDesc& D, int8_t* s, int8_t* pc, uint32_t* PB) {
        const int L = D.L;
        for (int t = lane; t < L + 2; t += 32) {
            int8_t code = 4, p = 4;
            if (t >= 1 && t <= L) {
                code = base_code(A.seqs[D.seq_off + t - 1]);
                p = (A.mask != nullptr && A.mask[D.seq_off + t - 1] != 0) ? (int8_t)5 : code;
            }
            s[t] = code;
            pc[t] = p;
        }
        __syncwarp();
        for (int w = 0; w < Y.W; ++w) {
            const int b = w * 32 + lane;
            const int x = (b <= L + 1) ? pc[b] : 5;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const unsigned bits = __ballot_sync(0xffffffffu, partner_code(c, x));
                if (lane == 0) PB[c * Y.W + w] = bits;
            }
        }
        __syncwarp();
    }

    // Publishes step (stage, t) of seat s with `chunks` chunks; the step's
    // other parameters are already in the seat.
    __device__ __forceinline__ void publish(int s, int stage, int t, int chunks, unsigned gen) {
        if (lane == 0) {
            seats[s].stage = stage;
            seats[s].t = t;
            seats[s].done = 0;
            __threadfence_block();
            atomicExch(&seats[s].claim, claim_word(gen, (unsigned)chunks));
        }
        __syncwarp();
    }

    // Opens the step after (stage, t) of seat s -- running serial steps inline
    // and skipping empty ones -- and publishes it; when the sequence is done,
    // admits the next one (or retires the seat).
    __device__ void advance(int s, int stage, int t, unsigned gen) {
        for (;;) {
            Seat& St = seats[s];
            const int L = St.D.L;
            // next step
            if (stage == kIn) {
                ++t;
                if (t > L + 1) {
                    finish_inside(s);
                    if constexpr (MODE == kQueueLogZ) {
                        stage = kFinished;
                    } else if constexpr (MODE == kQueueSample) {
                        stage = kSample;
                        t = 0;
                        if (A.n_samples <= 0) stage = kFinished;
                    } else {
                        exterior_outside_warp(Lse32{&sm->poly}, &sm->tabs, seq(s), out_tabs(s, L));
                        stage = kOut;
                        t = L;
                    }
                }
            } else if (stage == kOut) {
                --t;
                if (t < 0) { stage = kPostZero; t = 0; }
            } else if (stage == kPostZero) {
                stage = kPost;
            } else if (stage == kPost) {
                if constexpr (MODE == kQueueBpp) {
                    if (A.logz != nullptr && lane == 0) A.logz[St.D.idx] = in_tabs(s, L).F5[L];
                    stage = kFinished;
                } else {
                    stage = kUp;
                }
            } else if (stage == kUp) {
                stage = kMea;
                t = 0;
            } else if (stage == kMea) {
                ++t;
                if (t > L) {
                    traceback(s);
                    stage = kFinished;
                }
            } else if (stage == kSample) {
                stage = kFinished;
            }
            if (stage == kFinished) {
                if (!admit(s)) {
                    if (lane == 0) {
                        atomicExch(&seats[s].claim, claim_word(gen + 1, 0));
                        atomicSub(&sm->alive, 1);
                    }
                    __syncwarp();
                    return;
                }
                stage = kIn;
                t = 0;
                if (lane == 0) PairListPoff0(s);
                __syncwarp();
            }
            // size the step (and build what it needs)
            const int L2 = seats[s].D.L;
            int chunks = 0;
            if (stage == kIn) {
                const int dB = t - 1;
                int nb = 0, o = 0;
                if (dB >= 0 && dB <= L2 - 2) {
                    o = seats[s].pl_next;
                    plist_diagonal(s, dB);
                    nb = seats[s].pl_next - o;
                }
                const int na = t <= L2 ? L2 + 1 - t : 0;
                if (lane == 0) {
                    seats[s].nb = nb; seats[s].nb_chunks = (nb + 31) >> 5; seats[s].pl_o = o; seats[s].na = na;
                }
                chunks = ((nb + 31) >> 5) + ((na + 31) >> 5);
            } else if (stage == kOut) {
                const int dB = t - 1;
                int nb = 0, o = 0;
                if (dB >= 0 && dB <= L2 - 2) {
                    const PairList PL = plist(s, L2);
                    o = PL.poff[dB];
                    nb = PL.poff[dB + 1] - o;
                }
                const int na = L2 + 1 - t;
                if (lane == 0) {
                    seats[s].nb = nb; seats[s].nb_chunks = (nb + 31) >> 5; seats[s].pl_o = o; seats[s].na = na;
                }
                chunks = ((nb + 31) >> 5) + ((na + 31) >> 5);
            } else if (stage == kPostZero) {
                // POST (triangular, the FMo slot) and, for BPP, the caller's dense matrix
                const int tri = (int)tri_size(L2);
                const int dense = (MODE == kQueueBpp) ? L2 * L2 : 0;
                if (lane == 0) { seats[s].nb = tri; seats[s].na = dense; seats[s].nb_chunks = (tri + 1023) >> 10; }
                chunks = ((tri + 1023) >> 10) + ((dense + 1023) >> 10);
            } else if (stage == kPost) {
                const int total = plist(s, L2).poff[L2 + 1];
                if (lane == 0) seats[s].na = total;
                chunks = (total + 31) >> 5;
            } else if (stage == kUp) {
                if (lane == 0) seats[s].na = L2;
                chunks = (L2 + 31) >> 5;
            } else if (stage == kMea) {
                if (lane == 0) seats[s].na = L2 + 1 - t;
                chunks = (L2 + 1 - t + 31) >> 5;
            } else if (stage == kSample) {
                if (lane == 0) seats[s].na = A.n_samples;
                chunks = A.n_samples;
            }
            __syncwarp();
            ++gen;
            if (chunks > 0) {
                publish(s, stage, t, chunks, gen);
                return;
            }
            // an empty step: go straight on to the next one
        }
    }

    __device__ __forceinline__ void PairListPoff0(int s) { plist(s, seats[s].D.L).poff[0] = 0; }

    // After the last inside step: the rest of the pair-list offsets, F5.
    __device__ void finish_inside(int s) {
        const int L = seats[s].D.L;
        const PairList PL = plist(s, L);
        const int total = seats[s].pl_next;
        for (int d = max(1, L - 1) + lane; d <= L + 1; d += 32) PL.poff[d] = total;
        __syncwarp();
        const SeqV Q = seq(s);
        const InTabs<float> T = in_tabs(s, L);
        if constexpr (MODE == kQueueLogZ || MODE == kQueueSample) {
            exterior_warp<LseAcc32>(LseAcc32{}, &sm->tabs, Q, T);
            if (A.logz != nullptr && lane == 0) A.logz[seats[s].D.idx] = T.F5[L];
        } else {
            exterior_warp<Lse32>(Lse32{&sm->poly}, &sm->tabs, Q, T);
        }
        __syncwarp();
    }

    __device__ void traceback(int s) {
        const SeqDesc D = seats[s].D;
        const int L = D.L;
        const Arena32 ar = arena32(L);
        float* b = base(s);
        char* out = A.structs + D.seq_off;
        for (int t = lane; t < L; t += 32) out[t] = '.';
        __syncwarp();
        if (lane == 0) {
            int* qi = reinterpret_cast<int*>(b + ar.queue);
            mea_traceback(reinterpret_cast<const int*>(b + ar.FM), L, qi, qi + 2 * L + 4, out, A.status);
        }
        __syncwarp();
    }

    // ---- one chunk of seat s's open step (parameters read at the claim) ----
    __device__ void run_chunk(int s, int chunk, const Seat& St) {
        const int stage = St.stage, t = St.t;
        const SeqV Q = seq(s);
        const int L = Q.L, m = L + 1;
        if (stage == kIn || stage == kOut) {
            const int nbc = St.nb_chunks;
            if (chunk < nbc) {   // B items: pairable cells of diagonal t - 1, walked in lockstep
                const int k = chunk * 32 + lane;
                const int nb = St.nb;
                const unsigned lanes = __ballot_sync(0xffffffffu, k < nb);
                if (k >= nb) return;
                const PairList PL = plist(s, L);
                const int i = PL.pl[St.pl_o + k];
                if (stage == kIn) {
                    const Arena32 ar = arena32(L);
                    const float fm2 = base(s)[ar.FB + ((t - 1) & 1) * pad32(L + 2) + i];
                    if constexpr (MODE == kQueueLogZ || MODE == kQueueSample)
                        inside_B<LseAcc32>(LseAcc32{}, &sm->tabs, Q, in_tabs(s, L), i, i + t - 1, fm2, lanes);
                    else
                        inside_B<Lse32>(Lse32{&sm->poly}, &sm->tabs, Q, in_tabs(s, L), i, i + t - 1, fm2, lanes);
                } else {
                    outside_B(Lse32{&sm->poly}, &sm->tabs, Q, out_tabs(s, L), i, i + t - 1, lanes);
                }
            } else {             // A items: every cell of diagonal t
                const int i = (chunk - nbc) * 32 + lane;
                if (i > L - t) return;
                if (stage == kIn) {
                    const Arena32 ar = arena32(L);
                    float* fb = base(s) + ar.FB + (t & 1) * pad32(L + 2);
                    if constexpr (MODE == kQueueLogZ || MODE == kQueueSample)
                        fb[i] = inside_A<LseAcc32>(LseAcc32{}, &sm->tabs, Q, in_tabs(s, L), i, i + t);
                    else
                        fb[i] = inside_A<Lse32>(Lse32{&sm->poly}, &sm->tabs, Q, in_tabs(s, L), i, i + t);
                } else {
                    outside_A_merged(Lse32{&sm->poly}, &sm->tabs, Q, out_tabs(s, L), i, i + t);
                }
            }
            return;
        }
        if constexpr (MODE == kQueueMea || MODE == kQueueBpp) {
            if (stage == kPostZero) {
                const int tri = St.nb, tri_chunks = St.nb_chunks;
                if (chunk < tri_chunks) {
                    float* POST = out_tabs(s, L).FMo;
                    const int c1 = min(tri, (chunk + 1) << 10);
                    for (int c = (chunk << 10) + lane; c < c1; c += 32) POST[c] = 0.0f;
                } else {
                    float* dense = A.post_out + A.post_offs[St.D.idx];
                    const int dn = St.na, c1 = min(dn, (chunk - tri_chunks + 1) << 10);
                    for (int c = ((chunk - tri_chunks) << 10) + lane; c < c1; c += 32) dense[c] = 0.0f;
                }
                return;
            }
            if (stage == kPost) {
                const int total = St.na;
                const int c = chunk * 32 + lane;
                const unsigned lanes = __ballot_sync(0xffffffffu, c < total);
                if (c >= total) return;
                const PairList PL = plist(s, L);
                const OutTabs O = out_tabs(s, L);
                const int d = plist_diag(PL, L, c);
                const int a = PL.pl[c], b = a + d + 1;
                const float v = posterior_pair(&sm->tabs, &sm->poly, Q, O, O.F5[L], a, b, lanes);
                O.FMo[tri_off(d + 1, m) + a] = v;
                if constexpr (MODE == kQueueBpp) A.post_out[A.post_offs[St.D.idx] + (int64_t)(a - 1) * L + (b - 1)] = v;
                return;
            }
        }
        if constexpr (MODE == kQueueMea) {
            const Arena32 ar = arena32(L);
            float* b = base(s);
            if (stage == kUp) {
                const int i = 1 + chunk * 32 + lane;
                if (i <= L) b[ar.up + i] = mea_unpaired(b + ar.FMo, L, __fmul_rn(2.0f, A.gamma), i);
                return;
            }
            if (stage == kMea) {
                const int i = chunk * 32 + lane;
                if (i <= L - t)
                    mea_cell(Q, b + ar.FMo, b + ar.up, b + ar.FM2o, reinterpret_cast<int*>(b + ar.FM), L, i, i + t);
                return;
            }
        }
        if constexpr (MODE == kQueueSample) {
            if (stage == kSample) {
                const SeqDesc D = St.D;
                SampleCtx<SeqV> X;
                X.tb = &sm->tabs;
                X.Q = Q;
                X.T = in_tabs(s, L);
                const uint64_t sd = A.seeds != nullptr ? A.seeds[D.idx] : A.seed;
                const uint2 key = make_uint2((uint32_t)sd, (uint32_t)(sd >> 32));
                const int sidx = A.stream_idx != nullptr ? A.stream_idx[D.idx] : (A.seeds != nullptr ? 0 : D.idx);
                char* out = A.out + D.seq_off * (int64_t)A.n_samples + (int64_t)chunk * L;
                for (int u = lane; u < L; u += 32) out[u] = '.';
                __syncwarp();
                sample_one(X, chunk, sidx, key, out, stack, A.status, lane);
                __syncwarp();
            }
        }
    }
};

}  // namespace

template <int MODE>
__global__ void __launch_bounds__(kQueueThreads, kQueueMinBlocks) k_fold_queue(QueueArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    auto* sm = reinterpret_cast<QueueSmemHead*>(smem_raw);
    const QueueLayout Y = queue_layout(A.Lmax, A.seats, MODE == kQueueSample);
    Seat* seats = reinterpret_cast<Seat*>(smem_raw + Y.seats_off);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    load_tabs(&sm->tabs, A.blob32);
    load_poly_tables(&sm->poly);
    for (int s = threadIdx.x; s < A.seats; s += blockDim.x) {
        seats[s].claim = claim_word(0, 0);
        seats[s].done = 0;
    }
    if (threadIdx.x == 0) sm->alive = A.seats;
    __syncthreads();
    QueueCtx<MODE> C{A, sm, seats, smem_raw + Y.codes_off,
                     reinterpret_cast<uint32_t*>(smem_raw + Y.stacks_off) + (size_t)warp * Y.stack_words, Y, lane};
    // each warp opens the first step of the seats it owns at start
    for (int s = warp; s < A.seats; s += kQueueWarps) C.advance(s, kFinished, 0, 0);

    int rot = warp;
    unsigned long long idle_since = 0;
    unsigned backoff = 64;   // ns of sleep between polls, doubled while no work is found
    const unsigned long long t_start = globaltimer();
    for (;;) {
        if (globaltimer() - t_start > kLaunchLimitNs) {
            if (lane == 0) atomicExch(A.status, CF_ETIMEOUT);
            break;
        }
        // find a claimable chunk, starting at a per-warp rotating seat
        int got_seat = -1, got_chunk = 0;
        unsigned got_gen = 0;
        if (lane == 0) {
            for (int k = 0; k < A.seats; ++k) {
                const int s = (rot + k) % A.seats;
                const unsigned long long w = *reinterpret_cast<volatile unsigned long long*>(&seats[s].claim);
                if (cw_claimed(w) >= cw_total(w)) continue;
                const unsigned long long old = atomicAdd(&seats[s].claim, 1ull);
                if (cw_claimed(old) < cw_total(old)) {
                    got_seat = s;
                    got_chunk = (int)cw_claimed(old);
                    got_gen = cw_gen(old);
                    break;
                }
            }
        }
        got_seat = __shfl_sync(0xffffffffu, got_seat, 0);
        if (got_seat < 0) {
            const int alive = *reinterpret_cast<volatile int*>(&sm->alive);
            if (alive <= 0) break;
            const unsigned long long now = globaltimer();
            if (idle_since == 0) idle_since = now;
            else if (now - idle_since > kIdleLimitNs) {
                if (lane == 0) atomicExch(A.status, CF_ETIMEOUT);
                break;
            }
            // back off while idle (a polling warp takes issue slots from working ones)
            __nanosleep(backoff);
            backoff = backoff < CF_QUEUE_MAX_BACKOFF_NS ? 2 * backoff : backoff;
            continue;
        }
        idle_since = 0;
        backoff = 64;
        got_chunk = __shfl_sync(0xffffffffu, got_chunk, 0);
        got_gen = __shfl_sync(0xffffffffu, got_gen, 0);
        rot = got_seat;
        __threadfence_block();   // acquire: the step's parameters and the tables of earlier steps
        asm volatile("" ::: "memory");
        Seat St;
        {
            const volatile Seat* v = &seats[got_seat];
            St.stage = v->stage; St.t = v->t; St.nb = v->nb; St.nb_chunks = v->nb_chunks; St.na = v->na;
            St.pl_o = v->pl_o;
            St.D.seq_off = v->D.seq_off; St.D.ws_off = v->D.ws_off; St.D.L = v->D.L; St.D.idx = v->D.idx;
        }
        const int stage = St.stage, t = St.t;
        C.run_chunk(got_seat, got_chunk, St);
        __syncwarp();
        __threadfence_block();   // release this chunk's results before counting it done
        int last = 0;
        if (lane == 0) {
            const unsigned long long w = *reinterpret_cast<volatile unsigned long long*>(&seats[got_seat].claim);
            last = atomicAdd(&seats[got_seat].done, 1) + 1 == (int)cw_total(w);
        }
        last = __shfl_sync(0xffffffffu, last, 0);
        if (last) {
            __threadfence_block();   // acquire the other chunks' results
            C.advance(got_seat, stage, t, got_gen);
        }
    }
}

template __global__ void k_fold_queue<kQueueLogZ>(QueueArgs);
template __global__ void k_fold_queue<kQueueMea>(QueueArgs);
template __global__ void k_fold_queue<kQueueBpp>(QueueArgs);
template __global__ void k_fold_queue<kQueueSample>(QueueArgs);

size_t queue_smem_bytes(int Lmax, int seats, int mode) { return queue_layout(Lmax, seats, mode == kQueueSample).total; }

int64_t queue_slot_words(int Lmax) { return arena32(Lmax).total; }

const void* queue_kernel(int mode) {
    switch (mode) {
        case kQueueLogZ: return (const void*)k_fold_queue<kQueueLogZ>;
        case kQueueMea: return (const void*)k_fold_queue<kQueueMea>;
        case kQueueBpp: return (const void*)k_fold_queue<kQueueBpp>;
        default: return (const void*)k_fold_queue<kQueueSample>;
    }
}

}  // namespace cf
