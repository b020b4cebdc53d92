// cf_engine.cu -- host side of the C-ABI (include/contrafold_gb300.h).
//
// An engine owns the device parameter blobs, a stream and a growable work
// arena.  Every batch call: validate -> plan (order sequences, assign groups
// and arena slices within the memory budget) -> upload inputs once -> launch
// the phase kernels per slice -> download outputs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/contrafold_gb300.h"
#include "cf_host.h"
#include "cf_kernels.h"
#include "cf_queue.h"
#include "cf_sample.h"
#include "cf_warp.h"


using cf::SeqDesc;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
    g_err = msg;
    return code;
}

#define CF_CUDA(call)                                                                      \
    do {                                                                                   \
        cudaError_t e_ = (call);                                                           \
        if (e_ != cudaSuccess)                                                             \
            return fail(e_ == cudaErrorMemoryAllocation ? CF_ENOMEM : CF_ECUDA,            \
                        std::string(#call) + ": " + cudaGetErrorString(e_));               \
    } while (0)

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;                     // elements
    const cudaStream_t* sp = nullptr;   // set: stream-ordered (re)allocation on *sp
    // Grows geometrically (at least doubling).  An engine's buffers are
    // (re)allocated in stream order on the engine's stream (cudaMallocAsync /
    // cudaFreeAsync from the device's memory pool): cudaFree waits for the
    // whole device, and in the serving loop one worker's growing buffer held
    // the others' batches back for seconds while the rest of the device kept
    // working.  Buffers without a stream (plans) use cudaMalloc / cudaFree.
    int ensure(size_t n) {
        if (n <= cap) return CF_OK;
        release();
        size_t want = std::max<size_t>(std::max<size_t>(n, 1), 2 * cap);
        cudaError_t e = alloc(want);
        if (e == cudaErrorMemoryAllocation && want > std::max<size_t>(n, 1)) {   // no room to double
            cudaGetLastError();
            want = std::max<size_t>(n, 1);
            e = alloc(want);
        }
        if (e != cudaSuccess) {
            p = nullptr;
            return fail(CF_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
        }
        cap = want;
        return CF_OK;
    }
    cudaError_t alloc(size_t elems) {
        void* q = nullptr;
        const cudaError_t e = sp ? cudaMallocAsync(&q, elems * sizeof(T), *sp) : cudaMalloc(&q, elems * sizeof(T));
        p = static_cast<T*>(q);
        return e;
    }
    void release() {
        if (p) {
            if (sp) cudaFreeAsync(p, *sp);
            else cudaFree(p);
        }
        p = nullptr;
        cap = 0;
    }
};

// The dynamic shared-memory limit is an attribute of a kernel function, shared
// by every engine of the process, so it is raised here, process-wide and per
// device, and never lowered: an engine asking for less must not take away what
// another engine's launches rely on.
std::mutex g_smem_mu;
std::map<std::pair<const void*, int>, size_t> g_smem_set;

int raise_smem_limit(const void* fn, int device, size_t bytes) {
    std::lock_guard<std::mutex> lk(g_smem_mu);
    size_t& cur = g_smem_set[{fn, device}];
    if (bytes <= cur) return CF_OK;
    CF_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
    return CF_OK;
}

enum Job { JOB_LOGZ = 0, JOB_LOGZ64, JOB_BPP, JOB_MEA, JOB_MFE, JOB_SAMPLE, JOB_GRAD };

int64_t arena_words(Job job, int L, int grad_ckpt = 1) {
    switch (job) {
        case JOB_LOGZ:
        case JOB_SAMPLE: return cf::pad32(cf::arena32_inside_words(L));
        case JOB_LOGZ64:
        case JOB_MFE: return cf::arena64(L).total;
        case JOB_GRAD: return cf::pad32(cf::adj_arena_words(L, grad_ckpt));
        default: return cf::arena32(L).total;
    }
}

// One row of the schedule table (cf_engine_load_tuning): a batch matches
// when all its conditions hold; the first matching row decides the schedule
// of the automatic batched path.
struct TuneRow {
    int min_len = 0, max_len = CF_MAX_LEN;   // shortest >= min_len, longest <= max_len
    int min_batch = 0, max_batch = 0;        // n >= min_batch, n <= max_batch (0 = no limit)
    int uniform = -1;                        // 1: lengths within 25 %, 0: mixed, -1: either
    unsigned jobs = 0;                       // bit per Job (0 = every job)
    int sched = 3;                           // 1 warp, 2 cta, 3 group, 4 cluster (5, queue: disabled)
    int group = 0;                           // sequences per CTA: grouped kernels / queue seats (0 = automatic)
    int ctas = 0;                            // resident CTAs per SM of the CTA kernel (0 = automatic)
};

// The built-in table (GB300, contrafold_gpu_gb300/autotune.py sweeps):
//  * small batches of long sequences fold on a thread-block cluster each (one
//    600-nt MEA fold 172 -> 144 ms, 1,000 nt 450 -> 297 ms; 64 x 300 nt stays
//    grouped: 69 vs 125 ms): every sequence >= 512 nt and at most two
//    clusters' CTAs per SM (38 sequences on 152 SMs);
//  * large batches of mixed short lengths take the warp-per-sequence kernel
//    (200 nt: n=1024 warp 8.7k vs grouped 10.2k MEA folds/s, n=2048 15.1k vs
//    13.3k; 60 nt: n=2048 172k vs 186k, n=4096 238k vs 191k);
//  * sampling of large mixed batches up to 400 nt folds 4 sequences per CTA
//    (4,096 x U{40..400} x 100 samples: 1.30M samples/s against 1.20M with
//    the MEA-tuned length table's 2);
//  * everything else folds grouped (lengths within 25 %: one wave of full
//    CTAs; mixed: several waves).
std::vector<TuneRow> default_tuning() {
    const unsigned lbms = (1u << JOB_LOGZ) | (1u << JOB_BPP) | (1u << JOB_MEA) | (1u << JOB_SAMPLE);
    const unsigned lbm = (1u << JOB_LOGZ) | (1u << JOB_BPP) | (1u << JOB_MEA);
    std::vector<TuneRow> t(5);
    t[0].min_len = 512; t[0].min_batch = 1; t[0].max_batch = 38; t[0].jobs = lbms; t[0].sched = 4;
    t[1].max_len = 80; t[1].min_batch = 4096; t[1].uniform = 0; t[1].jobs = lbm; t[1].sched = 1;
    t[2].max_len = 80; t[2].uniform = 0; t[2].jobs = lbm; t[2].sched = 3;
    t[3].max_len = 256; t[3].min_batch = 2048; t[3].uniform = 0; t[3].jobs = lbm; t[3].sched = 1;
    t[4].max_len = 400; t[4].min_batch = 1024; t[4].uniform = 0; t[4].jobs = 1u << JOB_SAMPLE; t[4].sched = 3;
    t[4].group = 4;
    return t;
}

// Parses a schedule table: one row per line, '#' starts a comment,
//   min_len max_len min_batch max_batch uniform jobs schedule group ctas_per_sm
// uniform: any | uniform | mixed; jobs: all or a comma list of logz, logz64,
// bpp, mea, mfe, sample; schedule: warp | cta | group | cluster (the disabled
// queue schedule is rejected).
int parse_tuning(std::istream& in, std::vector<TuneRow>& rows, std::string& err) {
    std::string line;
    int ln = 0;
    rows.clear();
    while (std::getline(in, line)) {
        ++ln;
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line.resize(hash);
        std::istringstream ls(line);
        std::string f[9];
        int nf = 0;
        while (nf < 9 && (ls >> f[nf])) ++nf;
        if (nf == 0) continue;
        std::string extra;
        if (nf < 9 || (ls >> extra)) {
            err = "line " + std::to_string(ln) + ": expected 9 fields";
            return CF_EINVAL;
        }
        TuneRow r;
        auto num = [&](const std::string& x, int lo, int hi, int& out) {
            char* end = nullptr;
            const long v = std::strtol(x.c_str(), &end, 10);
            if (end == x.c_str() || *end != 0 || v < lo || v > hi) return false;
            out = (int)v;
            return true;
        };
        if (!num(f[0], 0, CF_MAX_LEN, r.min_len) || !num(f[1], 0, CF_MAX_LEN, r.max_len) ||
            !num(f[2], 0, 1 << 30, r.min_batch) || !num(f[3], 0, 1 << 30, r.max_batch) ||
            !num(f[7], 0, cf::kQueueMaxSeats, r.group) || !num(f[8], 0, 64, r.ctas)) {
            err = "line " + std::to_string(ln) + ": bad number";
            return CF_EINVAL;
        }
        if (f[4] == "any") r.uniform = -1;
        else if (f[4] == "uniform") r.uniform = 1;
        else if (f[4] == "mixed") r.uniform = 0;
        else { err = "line " + std::to_string(ln) + ": uniform must be any, uniform or mixed"; return CF_EINVAL; }
        if (f[5] != "all") {
            std::istringstream js(f[5]);
            std::string j;
            while (std::getline(js, j, ',')) {
                static const char* names[] = {"logz", "logz64", "bpp", "mea", "mfe", "sample"};
                int k = 0;
                while (k < 6 && j != names[k]) ++k;
                if (k == 6) { err = "line " + std::to_string(ln) + ": unknown job '" + j + "'"; return CF_EINVAL; }
                r.jobs |= 1u << k;   // the Job enum's order
            }
        }
        static const char* scheds[] = {"warp", "cta", "group", "cluster"};
        int k = 0;
        while (k < 4 && f[6] != scheds[k]) ++k;
        if (k == 4) { err = "line " + std::to_string(ln) + ": unknown schedule '" + f[6] + "'"; return CF_EINVAL; }
        r.sched = k + 1;
        rows.push_back(r);
    }
    return CF_OK;
}

const TuneRow* match_tuning(const std::vector<TuneRow>& rows, Job job, int n, int Lmin, int Lmax, bool uniform) {
    for (const TuneRow& r : rows) {
        if (Lmin < r.min_len || Lmax > r.max_len || n < r.min_batch) continue;
        if (r.max_batch > 0 && n > r.max_batch) continue;
        if (r.uniform >= 0 && (r.uniform == 1) != uniform) continue;
        if (r.jobs != 0 && !(r.jobs & (1u << job))) continue;
        return &r;
    }
    return nullptr;
}

}  // namespace

struct cf_engine {
    int device = 0;
    cudaStream_t stream = nullptr;       // the stream of the engine's calls: one of the two below
    cudaStream_t stream_lo = nullptr;    // the device's default (lowest) priority
    cudaStream_t stream_hi = nullptr;    // its highest priority (created on first use)
    DevBuf<float> blob32;
    DevBuf<double> blob64;
    DevBuf<float> arena;
    DevBuf<uint8_t> seqs, mask;
    DevBuf<SeqDesc> descs;
    DevBuf<float> logz;
    DevBuf<double> logz64;
    DevBuf<char> structs;
    DevBuf<float> post;
    DevBuf<int64_t> post_offs;
    DevBuf<int> status;
    DevBuf<char> samples;
    DevBuf<uint64_t> seeds;
    DevBuf<int32_t> stream_idx;
    DevBuf<float> bonus;
    DevBuf<double> counts, unpaired;
    // stream-ordered allocation of every buffer above on the engine's stream
    void bind_buffers() {
        const cudaStream_t* s = &stream;
        blob32.sp = s; blob64.sp = s; arena.sp = s; seqs.sp = s; mask.sp = s; descs.sp = s; logz.sp = s;
        logz64.sp = s; structs.sp = s; post.sp = s; post_offs.sp = s; status.sp = s; samples.sp = s; seeds.sp = s;
        stream_idx.sp = s; bonus.sp = s; counts.sp = s; unpaired.sp = s;
    }
    size_t budget = 0;   // bytes; 0 = automatic (half of free memory at first use)
    int mode = 1;        // 0 plain, 1 batched
    int sched = 0;       // batched schedule: 0 auto, 1 warp-persistent, 2 CTA-persistent, 3 grouped, 4 cluster
    int ctas_per_sm = 0; // CTA-persistent occupancy cap (0 = auto)
    int group = 0;       // sequences per CTA of the grouped kernels (0 = auto)
    size_t smem_optin = 0;
    std::vector<TuneRow> tuning = default_tuning();   // schedule table of the automatic path
    int grad_ckpt = 0;   // FM2 checkpoint spacing of cf_grad (0 = automatic by the longest sequence)
    bool shared = false; // the device is shared with other engines' launches: no wide CTAs, no clusters
};

namespace {

// Sequences per CTA of the grouped kernels for mixed lengths, by the median
// length (autotune.py --groups on GB300).
int group_for_length(int L) {
    if (L <= 64) return 8;
    if (L <= 160) return 4;
    if (L <= 320) return 2;
    return 1;
}

int ensure_smem(cf_engine* eng, size_t bytes);

struct Plan {
    bool plain = false;           // reference launch shape (mode 0): cf_plain.cu kernels for BPP/MEA
    bool cta = false;             // persistent CTA-per-sequence fused kernel (batched path)
    bool warp = false;            // persistent warp-per-sequence kernel (batched path)
    bool cluster = false;         // a thread-block cluster per group (latency of long sequences)
    bool queue = false;           // dataflow schedule (disabled: never set, see cf_queue.cu)
    int seats = 0;                // its sequences in progress per CTA
    int wgrid = 0;                // its grid
    int64_t slot_words = 0;       // its arena slot per warp
    std::vector<SeqDesc> descs;   // grouped order
    int grad_ckpt = 1;            // cf_grad: FM2 kept on every grad_ckpt-th diagonal
    std::vector<int> slice_begin; // descs index where each arena slice starts (group aligned)
    std::vector<int64_t> slice_words;
    int group = 1;
    int Lmax = 0;
};

int make_plan(cf_engine* eng, Job job, const int64_t* offsets, int n, Plan& P) {
    P.descs.resize(n);
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    P.group = 1;
    P.Lmax = 0;
    int Lmin = n ? CF_MAX_LEN : 0;
    for (int b = 0; b < n; ++b) {
        P.Lmax = std::max<int>(P.Lmax, (int)(offsets[b + 1] - offsets[b]));
        Lmin = std::min<int>(Lmin, (int)(offsets[b + 1] - offsets[b]));
    }
    // lengths within 25 % of each other: the grouped kernels with whole waves
    // of full CTAs beat the warp kernel (10,000 x 200 nt MEA: 27.7k vs 25.2k
    // folds/s; 10,000 x 100 nt: 121k vs 109k); mixed lengths keep the warp
    // kernel's per-sequence work queue (150-250 nt: 20.8k vs 15.1k)
    const bool uniform = P.Lmax <= Lmin + Lmin / 4;
    const bool batched = eng->mode == 1 && job != JOB_GRAD;
    P.plain = !batched;
    if (batched) {
        std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
            return offsets[x + 1] - offsets[x] > offsets[y + 1] - offsets[y];
        });
        // one group size for the launch (GB300, autotune.py --groups and batch
        // policies): lengths within 25 % of each other fold best as ONE wave of
        // CTAs (kFoldMinBlocks per SM) each holding n / slots sequences (200 nt:
        // n=1000 9.9k -> 14.4k, n=3125 15.0k -> 23.9k MEA folds/s against two
        // per CTA); mixed lengths keep several waves so the long sequences' CTAs
        // do not set the end alone (40-400 nt: 11.8k with 2 per CTA, 6.5k with 9)
        const int Lmed = n ? (int)(offsets[order[n / 2] + 1] - offsets[order[n / 2]]) : 0;
        int sms = 0;
        CF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, eng->device));
        // resident CTAs per SM of the kernel that will run: the fused MEA kernel
        // is built for more than the other grouped kernels
        const int slots =
            std::max(1, (job == JOB_MEA && !eng->shared ? cf::kFoldMinBlocksMea : cf::kFoldMinBlocks) * sms);
        // whole waves: the fewest waves whose groups fit kMaxGroup sequences
        const int waves = std::max(1, (n + cf::kMaxGroup * slots - 1) / (cf::kMaxGroup * slots));
        const int wave_group = std::min(cf::kMaxGroup, std::max(1, (n + waves * slots - 1) / (waves * slots)));
        const int wave2 = std::min(cf::kMaxGroup, std::max(1, (n + 2 * slots - 1) / (2 * slots)));
        P.group = eng->group > 0 ? std::min(cf::kMaxGroup, eng->group)
                                 : uniform ? wave_group : std::min(group_for_length(Lmed), wave2);
    }
    for (int k = 0; k < n; ++k) {
        const int b = order[k];
        P.descs[k].seq_off = offsets[b];
        P.descs[k].L = (int)(offsets[b + 1] - offsets[b]);
        P.descs[k].idx = b;
        P.descs[k].ws_off = 0;
    }
    // arena slices within the budget
    size_t budget = eng->budget;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = fr / 2;
    }
    const int64_t budget_words = (int64_t)(budget / 4);
    // batched schedule: the fused per-sequence CTA kernel keeps only a few
    // sequences per SM in flight (their tables stay in L2); the warp kernel
    // runs one sequence per warp (short sequences, sampling).
    int sched = eng->sched;
    // sampling never takes the warp kernel on its own: it draws a sequence's
    // samples one after another on one warp, the grouped path gives every
    // (sequence, sample) its own warp (1.28M vs 0.72M samples/s on 40-400 nt).
    // Mixed lengths stay one plan, longest first: splitting a 40-400 nt batch
    // at 256 nt into a warp-kernel part and a grouped part on two streams was
    // slower for every job (MEA 8.5k vs 10.7k folds/s).
    int row_ctas = 0, row_group = 0;
    if (sched == 0) {   // the schedule table decides (cf_engine_load_tuning)
        sched = 3;
        if (batched) {
            if (const TuneRow* r = match_tuning(eng->tuning, job, n, Lmin, P.Lmax, uniform)) {
                sched = r->sched;
                row_ctas = r->ctas;
                row_group = r->group;
                if (r->group > 0 && eng->group == 0 && sched == 3) P.group = r->group;
            }
        }
    }
    // on a shared device a cluster waits for 8 SMs of one GPC to be free at
    // once; between other engines' steady launches that took seconds
    if (eng->shared && sched == 4) sched = 3;
    P.cluster = batched && sched == 4 && (job == JOB_LOGZ || job == JOB_BPP || job == JOB_MEA || job == JOB_SAMPLE);
    if (P.cluster) P.group = eng->group > 0 ? std::min(cf::kMaxGroup, eng->group) : 1;
    P.queue = batched && sched == 5 && (job == JOB_LOGZ || job == JOB_BPP || job == JOB_MEA || job == JOB_SAMPLE);
    if (P.queue) {
        // sequences in progress per CTA: enough open chunks for the 8 warps on
        // short sequences, fewer (less L2 working set) on long ones
        int seats = eng->group > 0 ? eng->group : row_group > 0 ? row_group
                  : P.Lmax <= 320 ? 8 : P.Lmax <= 640 ? 4 : 2;
        seats = std::max(1, std::min(seats, cf::kQueueMaxSeats));
        const int mode = job == JOB_LOGZ ? cf::kQueueLogZ : job == JOB_MEA ? cf::kQueueMea
                       : job == JOB_BPP ? cf::kQueueBpp : cf::kQueueSample;
        const size_t smem = cf::queue_smem_bytes(P.Lmax, seats, mode);
        int rc = ensure_smem(eng, smem);
        if (rc) return rc;
        int per_sm = 0, sms = 0;
        CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cf::queue_kernel(mode), cf::kQueueThreads, smem));
        CF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, eng->device));
        if (eng->ctas_per_sm > 0) per_sm = std::min(per_sm, eng->ctas_per_sm);
        else if (row_ctas > 0) per_sm = std::min(per_sm, row_ctas);
        int64_t grid = std::min<int64_t>((int64_t)std::max(per_sm, 1) * sms, (n + seats - 1) / seats);
        P.slot_words = cf::queue_slot_words(P.Lmax);
        while (grid > 1 && grid * seats * P.slot_words > budget_words) --grid;
        if (grid * seats * P.slot_words <= budget_words) {
            P.wgrid = (int)std::max<int64_t>(grid, 1);
            P.seats = seats;
            P.group = 1;
            P.slice_begin = {0, n};
            P.slice_words = {grid * seats * P.slot_words};
            return CF_OK;
        }
        P.queue = false;   // not even one CTA of seats fits: per-sequence kernels, sliced
    }
    P.cta = batched && sched == 2 && (job == JOB_LOGZ || job == JOB_BPP || job == JOB_MEA);
    if (P.cta) {
        const int mode = job == JOB_LOGZ ? cf::kCtaLogZ : job == JOB_MEA ? cf::kCtaMea : cf::kCtaBpp;
        const size_t smem = cf::fold_smem_bytes(P.Lmax, 1, false);
        int rc = ensure_smem(eng, smem);
        if (rc) return rc;
        int per_sm = 0, sms = 0;
        CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cf::cta_kernel(mode), cf::kFoldThreads, smem));
        CF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, eng->device));
        per_sm = std::max(per_sm, 1);
        if (eng->ctas_per_sm > 0) per_sm = std::min(per_sm, eng->ctas_per_sm);
        else if (row_ctas > 0) per_sm = std::min(per_sm, row_ctas);
        else per_sm = std::min(per_sm, P.Lmax <= 160 ? 4 : 3);   // GB300: 4 up to 160 nt
        int64_t grid = std::min<int64_t>((int64_t)per_sm * sms, n);
        P.slot_words = cf::arena32(P.Lmax).total;
        while (grid > 1 && grid * P.slot_words > budget_words) --grid;
        if (grid * P.slot_words <= budget_words) {
            P.wgrid = (int)std::max<int64_t>(grid, 1);
            P.group = 1;
            P.slice_begin = {0, n};
            P.slice_words = {grid * P.slot_words};
            return CF_OK;
        }
        P.cta = false;
    }
    P.warp = batched && sched == 1 && P.Lmax <= cf::kWarpMaxLen &&
             (job == JOB_LOGZ || job == JOB_BPP || job == JOB_MEA || job == JOB_SAMPLE);
    if (P.warp) {
        // persistent grid: resident CTAs per SM x SMs, no more warps than sequences
        const int mode = job == JOB_LOGZ ? cf::kWarpLogZ : job == JOB_MEA ? cf::kWarpMea
                       : job == JOB_BPP ? cf::kWarpBpp : cf::kWarpSample;
        const size_t smem = cf::warp_smem_bytes(P.Lmax);
        int rc = ensure_smem(eng, smem);
        if (rc) return rc;
        int per_sm = 0, sms = 0;
        CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cf::warp_kernel(mode), cf::kWarpThreads, smem));
        CF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, eng->device));
        const int wpb = cf::kWarpThreads / 32;
        int64_t grid = (int64_t)std::max(per_sm, 1) * sms;
        grid = std::min<int64_t>(grid, (n + wpb - 1) / wpb);
        P.slot_words = cf::warp_slot_words(P.Lmax);
        while (grid > 1 && grid * wpb * P.slot_words > budget_words) --grid;
        if (grid * wpb * P.slot_words <= budget_words) {
            P.wgrid = (int)std::max<int64_t>(grid, 1);
            P.group = 1;
            P.slice_begin = {0, n};
            P.slice_words = {grid * wpb * P.slot_words};
            return CF_OK;
        }
        P.warp = false;   // not even one CTA of warp slots fits: per-sequence kernels, sliced
    }
    P.grad_ckpt = eng->grad_ckpt > 0 ? eng->grad_ckpt : cf::adj_auto_checkpoint(P.Lmax);
    P.slice_begin.clear();
    P.slice_words.clear();
    int64_t cur = 0;
    int start = 0;
    for (int k = 0; k < n; k += P.group) {
        int64_t gw = 0;
        const int kend = std::min(n, k + P.group);
        for (int t = k; t < kend; ++t) gw += arena_words(job, P.descs[t].L, P.grad_ckpt);
        if (gw > budget_words) return fail(CF_ENOMEM, "sequence group does not fit the arena budget");
        if (cur + gw > budget_words && k > start) {
            P.slice_begin.push_back(start);
            P.slice_words.push_back(cur);
            start = k;
            cur = 0;
        }
        for (int t = k; t < kend; ++t) {
            P.descs[t].ws_off = cur;
            cur += arena_words(job, P.descs[t].L, P.grad_ckpt);
        }
    }
    P.slice_begin.push_back(start);
    P.slice_words.push_back(cur);
    P.slice_begin.push_back(n);
    return CF_OK;
}

int check_batch(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets, int32_t n) {
    if (!eng) return fail(CF_EINVAL, "engine is NULL");
    if (n < 0) return fail(CF_EINVAL, "negative batch size");
    if (n > 0 && !offsets) return fail(CF_EINVAL, "offsets is NULL");
    if (n > 0 && offsets[0] != 0) return fail(CF_EINVAL, "offsets[0] must be 0");
    for (int b = 0; b < n; ++b) {
        const int64_t L = offsets[b + 1] - offsets[b];
        if (L < 0) return fail(CF_EINVAL, "offsets must be non-decreasing");
        if (L > CF_MAX_LEN) return fail(CF_EINVAL, "sequence longer than CF_MAX_LEN");
    }
    if (n > 0 && offsets[n] > 0 && !seqs) return fail(CF_EINVAL, "seqs is NULL");
    return CF_OK;
}

int ensure_smem(cf_engine* eng, size_t bytes) {
    // set even below 48 KB: static shared memory (the cp.async chain ring)
    // counts against the same 48 KB default limit
    if (eng->smem_optin != 0 && bytes <= eng->smem_optin) return CF_OK;
    bytes = std::max<size_t>(bytes, 48 * 1024);
    int dev_max = 0;
    CF_CUDA(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, eng->device));
    if ((size_t)dev_max < bytes) return fail(CF_EINVAL, "sequence too long for shared-memory staging");
    std::vector<const void*> ks = {(const void*)cf::k_plain_inside32, (const void*)cf::k_plain_outside32,
                                   (const void*)cf::k_plain_posterior32, (const void*)cf::k_plain_mea32,
                                   (const void*)cf::k_inside64, (const void*)cf::k_viterbi64};
    for (bool wide : {false, true}) {
        const cf::FoldKernels fk = cf::fold_kernels(wide);
        for (cf::FoldKernel k : {fk.inside, fk.inside_acc, fk.outside, fk.posterior, fk.mea, fk.fused_mea, fk.fused_bpp,
                                 fk.fused_mea_shared})
            ks.push_back((const void*)k);
    }
    for (int mode = 0; mode < 4; ++mode) ks.push_back(cf::warp_kernel(mode));
    for (int mode = 0; mode < 3; ++mode) ks.push_back(cf::cta_kernel(mode));
    const cf::ClusterKernels ck = cf::cluster_kernels();
    for (cf::FoldKernel k : {ck.mea, ck.bpp, ck.inside_acc}) ks.push_back((const void*)k);
    for (const void* k : ks) {
        const int rc = raise_smem_limit(k, eng->device, bytes);
        if (rc) return rc;
    }
    eng->smem_optin = bytes;
    return CF_OK;
}

// Per-phase device timing with CUDA events (phases: 0 inside, 1 outside,
// 2 posterior, 3 decode / traceback / sampling).
constexpr int kPhases = 4;
struct PhaseTimer {
    bool on = false;
    std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
    size_t used = 0;
    void reset() { used = 0; }
    int begin(int phase, cudaStream_t st, cudaEvent_t* stop) {
        if (!on) return CF_OK;
        if (used == marks.size()) {
            cudaEvent_t a, b;
            CF_CUDA(cudaEventCreate(&a));
            CF_CUDA(cudaEventCreate(&b));
            marks.push_back({phase, {a, b}});
        }
        auto& m = marks[used++];
        m.first = phase;
        CF_CUDA(cudaEventRecord(m.second.first, st));
        *stop = m.second.second;
        return CF_OK;
    }
    int end(cudaEvent_t stop, cudaStream_t st) {
        if (!on) return CF_OK;
        CF_CUDA(cudaEventRecord(stop, st));
        return CF_OK;
    }
    int read(float* ms, int nph) {
        for (int k = 0; k < nph; ++k) ms[k] = 0.f;
        for (size_t u = 0; u < used; ++u) {
            float t = 0.f;
            CF_CUDA(cudaEventSynchronize(marks[u].second.second));
            CF_CUDA(cudaEventElapsedTime(&t, marks[u].second.first, marks[u].second.second));
            if (marks[u].first < nph) ms[marks[u].first] += t;
        }
        return CF_OK;
    }
    ~PhaseTimer() {
        for (auto& m : marks) {
            cudaEventDestroy(m.second.first);
            cudaEventDestroy(m.second.second);
        }
    }
};

struct SampleJob {
    int n_samples = 0;
    uint64_t seed = 0;
    const uint64_t* d_seeds = nullptr;   // per-sequence seeds (cf_sample_seeded) or null
    const int32_t* d_stream = nullptr;   // per-sequence Philox sequence index (cf_sample_tasks) or null
    char* d_out = nullptr;
};

// Device resources one execution uses: descriptors (already uploaded), arena,
// status word, optional phase timer.
struct Exec {
    const SeqDesc* d_descs = nullptr;
    float* arena = nullptr;
    int* status = nullptr;
    PhaseTimer* timer = nullptr;
    int launches = 0;   // kernels launched by the last run
};

#define CF_PHASE(ph, launch)                                                \
    do {                                                                   \
        cudaEvent_t stop_ = nullptr;                                       \
        if (X.timer && (rc = X.timer->begin((ph), st, &stop_))) return rc; \
        launch;                                                            \
        ++X.launches;                                                      \
        CF_CUDA(cudaGetLastError());                                       \
        if (X.timer && (rc = X.timer->end(stop_, st))) return rc;          \
    } while (0)

// Launches `job` over a planned batch whose inputs are already on the device.
int run_device(cf_engine* eng, Job job, const Plan& P, Exec& X, const uint8_t* d_seqs, const uint8_t* d_mask,
               float gamma, float* d_logz, double* d_logz64, char* d_structs, float* d_post,
               const int64_t* d_post_offs, cudaStream_t st, const SampleJob* sj = nullptr) {
    const int n = (int)P.descs.size();
    X.launches = 0;
    if (X.timer) X.timer->reset();
    if (n == 0) return CF_OK;
    int rc;
    if (P.cta) {
        cf::FoldArgs A;
        A.descs = X.d_descs;
        A.n = n;
        A.group = 1;
        A.seqs = d_seqs;
        A.mask = d_mask;
        A.blob32 = eng->blob32.p;
        A.blob64 = eng->blob64.p;
        A.ws = X.arena;
        A.logz = d_logz;
        A.logz64 = nullptr;
        A.structs = d_structs;
        A.post_out = d_post;
        A.post_offs = d_post_offs;
        A.gamma = gamma;
        A.status = X.status;
        const int mode = job == JOB_LOGZ ? cf::kCtaLogZ : job == JOB_MEA ? cf::kCtaMea : cf::kCtaBpp;
        const size_t smem = cf::fold_smem_bytes(P.Lmax, 1, false);
        if ((rc = ensure_smem(eng, smem))) return rc;
        CF_CUDA(cudaMemsetAsync(X.status + 1, 0, sizeof(int), st));
        int* counter = X.status + 1;
        int64_t slot_words = P.slot_words;
        void* args[] = {&A, &counter, &slot_words};
        CF_PHASE(0, (cudaLaunchKernel(cf::cta_kernel(mode), dim3(P.wgrid), dim3(cf::kFoldThreads), args, smem, st)));
        return CF_OK;
    }
    if (P.queue) {
        cf::QueueArgs Q;
        Q.descs = X.d_descs;
        Q.n = n;
        Q.Lmax = P.Lmax;
        Q.seats = P.seats;
        Q.seqs = d_seqs;
        Q.mask = d_mask;
        Q.blob32 = eng->blob32.p;
        Q.ws = X.arena;
        Q.slot_words = P.slot_words;
        Q.counter = X.status + 1;
        Q.gamma = gamma;
        Q.logz = d_logz;
        Q.structs = d_structs;
        Q.post_out = d_post;
        Q.post_offs = d_post_offs;
        Q.n_samples = sj ? sj->n_samples : 0;
        Q.seed = sj ? sj->seed : 0;
        Q.seeds = sj ? sj->d_seeds : nullptr;
        Q.stream_idx = sj ? sj->d_stream : nullptr;
        Q.out = sj ? sj->d_out : nullptr;
        Q.status = X.status;
        const int mode = job == JOB_LOGZ ? cf::kQueueLogZ : job == JOB_MEA ? cf::kQueueMea
                       : job == JOB_BPP ? cf::kQueueBpp : cf::kQueueSample;
        const size_t smem = cf::queue_smem_bytes(P.Lmax, P.seats, mode);
        if ((rc = ensure_smem(eng, smem))) return rc;
        CF_CUDA(cudaMemsetAsync(X.status + 1, 0, sizeof(int), st));
        void* args[] = {&Q};
        CF_PHASE(0, (cudaLaunchKernel(cf::queue_kernel(mode), dim3(P.wgrid), dim3(cf::kQueueThreads), args, smem, st)));
        return CF_OK;
    }
    if (P.warp) {
        cf::WarpArgs W;
        W.descs = X.d_descs;
        W.n = n;
        W.Lmax = P.Lmax;
        W.seqs = d_seqs;
        W.mask = d_mask;
        W.blob32 = eng->blob32.p;
        W.ws = X.arena;
        W.slot_words = P.slot_words;
        W.counter = X.status + 1;
        W.gamma = gamma;
        W.logz = d_logz;
        W.structs = d_structs;
        W.post_out = d_post;
        W.post_offs = d_post_offs;
        W.n_samples = sj ? sj->n_samples : 0;
        W.seed = sj ? sj->seed : 0;
        W.seeds = sj ? sj->d_seeds : nullptr;
        W.stream_idx = sj ? sj->d_stream : nullptr;
        W.out = sj ? sj->d_out : nullptr;
        W.status = X.status;
        const int mode = job == JOB_LOGZ ? cf::kWarpLogZ : job == JOB_MEA ? cf::kWarpMea
                       : job == JOB_BPP ? cf::kWarpBpp : cf::kWarpSample;
        const size_t smem = cf::warp_smem_bytes(P.Lmax);
        if ((rc = ensure_smem(eng, smem))) return rc;
        CF_CUDA(cudaMemsetAsync(X.status + 1, 0, sizeof(int), st));
        void* args[] = {&W};
        CF_PHASE(0, (cudaLaunchKernel(cf::warp_kernel(mode), dim3(P.wgrid), dim3(cf::kWarpThreads), args, smem, st)));
        return CF_OK;
    }
    const bool fp64 = job == JOB_LOGZ64 || job == JOB_MFE;
    const size_t smem = cf::fold_smem_bytes(P.Lmax, P.group, fp64);
    if ((rc = ensure_smem(eng, std::max(smem, cf::plain_smem_bytes(P.Lmax))))) return rc;

    for (size_t s = 0; s + 1 < P.slice_begin.size(); ++s) {
        const int k0 = P.slice_begin[s], k1 = P.slice_begin[s + 1];
        cf::FoldArgs A;
        A.descs = X.d_descs + k0;
        A.n = k1 - k0;
        A.group = P.group;
        A.seqs = d_seqs;
        A.mask = d_mask;
        A.blob32 = eng->blob32.p;
        A.blob64 = eng->blob64.p;
        A.ws = X.arena;
        A.logz = d_logz;
        A.logz64 = d_logz64;
        A.structs = d_structs;
        A.post_out = d_post;
        A.post_offs = d_post_offs;
        A.gamma = gamma;
        A.status = X.status;
        const int grid = (A.n + P.group - 1) / P.group;
        const dim3 blk(cf::kFoldThreads);
        // at most one CTA per SM: the wide per-phase kernels (twice the threads on
        // each diagonal, the latency of small batches of long sequences)
        int sms = 0;
        CF_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, eng->device));
        // (not on a shared device: a 512-thread CTA waits for an SM with room
        // for all of it, which other engines' smaller CTAs kept taking first)
        const bool wide = grid <= sms && !eng->shared;
        const dim3 blkw(wide ? cf::kFoldThreadsWide : cf::kFoldThreads);
        const cf::FoldKernels fk = cf::fold_kernels(wide);
        const cf::FoldKernel k_in = fk.inside, k_inacc = fk.inside_acc, k_out = fk.outside, k_post = fk.posterior,
                             k_dec = fk.mea;
        // cluster schedule: every group on kClusterCtas CTAs of one cluster
        const cf::ClusterKernels ck = cf::cluster_kernels();
        const dim3 cgrid(grid * cf::kClusterCtas);
        switch (job) {
            case JOB_LOGZ:
                if (P.cluster) CF_PHASE(0, (ck.inside_acc<<<cgrid, blk, smem, st>>>(A)));
                else CF_PHASE(0, (k_inacc<<<grid, blkw, smem, st>>>(A)));
                break;
            case JOB_LOGZ64:
                CF_PHASE(0, (cf::k_inside64<<<grid, blk, smem, st>>>(A)));
                break;
            case JOB_BPP:
            case JOB_MEA: {
                cf::FoldArgs Ai = A;
                Ai.logz = nullptr;
                if (P.plain) {
                    const size_t psm = cf::plain_smem_bytes(P.Lmax);
                    CF_PHASE(0, (cf::k_plain_inside32<<<grid, blk, psm, st>>>(Ai)));
                    CF_PHASE(1, (cf::k_plain_outside32<<<grid, blk, psm, st>>>(A)));
                    if (job == JOB_BPP) {
                        CF_PHASE(2, (cf::k_plain_posterior32<<<grid, blk, psm, st>>>(A)));
                    } else {
                        cf::FoldArgs Ap = A;
                        Ap.post_out = nullptr;
                        Ap.logz = nullptr;
                        CF_PHASE(2, (cf::k_plain_posterior32<<<grid, blk, psm, st>>>(Ap)));
                        CF_PHASE(3, (cf::k_plain_mea32<<<grid, blk, psm, st>>>(A)));
                    }
                    break;
                }
                if (P.cluster) {   // fused only: the phases are timed as one
                    CF_PHASE(0, ((job == JOB_BPP ? ck.bpp : ck.mea)<<<cgrid, blk, smem, st>>>(A)));
                    break;
                }
                if (X.timer == nullptr) {   // one launch for all phases; per-phase kernels when timing
                    const cf::FoldKernel fused = job == JOB_BPP ? fk.fused_bpp
                                               : eng->shared ? fk.fused_mea_shared : fk.fused_mea;
                    CF_PHASE(0, (fused<<<grid, blkw, smem, st>>>(A)));
                    break;
                }
                CF_PHASE(0, (k_in<<<grid, blkw, smem, st>>>(Ai)));
                CF_PHASE(1, (k_out<<<grid, blkw, smem, st>>>(A)));
                if (job == JOB_BPP) {
                    CF_PHASE(2, (k_post<<<grid, blkw, smem, st>>>(A)));
                } else {
                    cf::FoldArgs Ap = A;
                    Ap.post_out = nullptr;
                    Ap.logz = nullptr;
                    CF_PHASE(2, (k_post<<<grid, blkw, smem, st>>>(Ap)));
                    CF_PHASE(3, (k_dec<<<grid, blkw, smem, st>>>(A)));
                }
                break;
            }
            case JOB_MFE:
                CF_PHASE(0, (cf::k_viterbi64<<<grid, blk, smem, st>>>(A)));
                break;
            case JOB_SAMPLE: {
                if (P.cluster) CF_PHASE(0, (ck.inside_acc<<<cgrid, blk, smem, st>>>(A)));
                else CF_PHASE(0, (k_inacc<<<grid, blkw, smem, st>>>(A)));
                if (!sj || sj->n_samples <= 0) break;
                cf::SampleArgs S;
                S.descs = A.descs;
                S.n = A.n;
                S.n_samples = sj->n_samples;
                S.Lmax = P.Lmax;
                S.seed = sj->seed;
                S.seeds = sj->d_seeds;
                S.stream_idx = sj->d_stream;
                S.seqs = d_seqs;
                S.mask = d_mask;
                S.blob32 = eng->blob32.p;
                S.ws = X.arena;
                S.out = sj->d_out;
                S.status = X.status;
                const size_t ssm = cf::sample_smem_bytes(P.Lmax);
                if (ssm > 48 * 1024 && (rc = raise_smem_limit((const void*)cf::k_sample32, eng->device, ssm))) return rc;
                const int64_t items = (int64_t)A.n * sj->n_samples;
                const int warps = cf::sample_threads() / 32;
                const int sgrid = (int)std::min<int64_t>((items + warps - 1) / warps, 152 * 16);
                CF_PHASE(3, (cf::k_sample32<<<sgrid, cf::sample_threads(), ssm, st>>>(S)));
                break;
            }
            default:
                return fail(CF_EINVAL, "bad job");
        }
    }
    return CF_OK;
}

int read_status(cf_engine* eng, cudaStream_t st) {
    int h = 0;
    CF_CUDA(cudaMemcpyAsync(&h, eng->status.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaStreamSynchronize(st));
    if (h != CF_OK) return fail(h, "a kernel reported an internal limit (traceback stack/queue)");
    return CF_OK;
}

// Host-buffer front end shared by the synchronous entry points.
int run_host(cf_engine* eng, Job job, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask,
             int32_t n, float gamma, float* logz_out, double* logz64_out, char* struct_out,
             const int64_t* post_offsets, float* post_out, int n_samples = 0, uint64_t seed = 0,
             char* sample_out = nullptr, const uint64_t* seeds = nullptr, const int32_t* stream_idx = nullptr) {
    int rc = check_batch(eng, seqs, offsets, n);
    if (rc) return rc;
    if (n == 0) return CF_OK;
    CF_CUDA(cudaSetDevice(eng->device));
    cudaStream_t st = eng->stream;
    Plan P;
    if ((rc = make_plan(eng, job, offsets, n, P))) return rc;
    const size_t nbytes = (size_t)offsets[n];
    if ((rc = eng->seqs.ensure(nbytes))) return rc;
    if (nbytes) CF_CUDA(cudaMemcpyAsync(eng->seqs.p, seqs, nbytes, cudaMemcpyHostToDevice, st));
    const uint8_t* d_mask = nullptr;
    if (mask) {
        if ((rc = eng->mask.ensure(nbytes))) return rc;
        if (nbytes) CF_CUDA(cudaMemcpyAsync(eng->mask.p, mask, nbytes, cudaMemcpyHostToDevice, st));
        d_mask = eng->mask.p;
    }
    float* d_logz = nullptr;
    double* d_logz64 = nullptr;
    char* d_structs = nullptr;
    float* d_post = nullptr;
    int64_t* d_post_offs = nullptr;
    size_t post_total = 0;
    if (logz_out) {
        if ((rc = eng->logz.ensure(n))) return rc;
        d_logz = eng->logz.p;
    }
    if (logz64_out) {
        if ((rc = eng->logz64.ensure(n))) return rc;
        d_logz64 = eng->logz64.p;
    }
    if (struct_out) {
        if ((rc = eng->structs.ensure(nbytes))) return rc;
        d_structs = eng->structs.p;
    }
    if (post_out) {
        std::vector<int64_t> po(post_offsets, post_offsets + n);
        for (int b = 0; b < n; ++b) {
            const int64_t L = offsets[b + 1] - offsets[b];
            post_total = std::max<size_t>(post_total, (size_t)(po[b] + L * L));
        }
        if ((rc = eng->post.ensure(post_total))) return rc;
        if ((rc = eng->post_offs.ensure(n))) return rc;
        CF_CUDA(cudaMemcpyAsync(eng->post_offs.p, po.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, st));
        d_post = eng->post.p;
        d_post_offs = eng->post_offs.p;
    }
    SampleJob sj;
    const size_t sample_bytes = nbytes * (size_t)std::max(n_samples, 0);
    if (job == JOB_SAMPLE && sample_bytes) {
        if ((rc = eng->samples.ensure(sample_bytes))) return rc;
        sj.n_samples = n_samples;
        sj.seed = seed;
        sj.d_out = eng->samples.p;
        if (seeds) {
            if ((rc = eng->seeds.ensure(n))) return rc;
            CF_CUDA(cudaMemcpyAsync(eng->seeds.p, seeds, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, st));
            sj.d_seeds = eng->seeds.p;
        }
        if (stream_idx) {
            if ((rc = eng->stream_idx.ensure(n))) return rc;
            CF_CUDA(cudaMemcpyAsync(eng->stream_idx.p, stream_idx, sizeof(int32_t) * n, cudaMemcpyHostToDevice, st));
            sj.d_stream = eng->stream_idx.p;
        }
    }
    if ((rc = eng->descs.ensure(n))) return rc;
    CF_CUDA(cudaMemcpyAsync(eng->descs.p, P.descs.data(), sizeof(SeqDesc) * n, cudaMemcpyHostToDevice, st));
    int64_t maxw = 1;
    for (int64_t w : P.slice_words) maxw = std::max(maxw, w);
    if ((rc = eng->arena.ensure((size_t)maxw))) return rc;
    if ((rc = eng->status.ensure(2))) return rc;
    CF_CUDA(cudaMemsetAsync(eng->status.p, 0, sizeof(int), st));
    Exec X;
    X.d_descs = eng->descs.p;
    X.arena = eng->arena.p;
    X.status = eng->status.p;
    if ((rc = run_device(eng, job, P, X, eng->seqs.p, d_mask, gamma, d_logz, d_logz64, d_structs, d_post, d_post_offs,
                         st, &sj)))
        return rc;
    if (sample_out && sample_bytes)
        CF_CUDA(cudaMemcpyAsync(sample_out, sj.d_out, sample_bytes, cudaMemcpyDeviceToHost, st));
    if (logz_out) CF_CUDA(cudaMemcpyAsync(logz_out, d_logz, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    if (logz64_out) CF_CUDA(cudaMemcpyAsync(logz64_out, d_logz64, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    if (struct_out && nbytes) CF_CUDA(cudaMemcpyAsync(struct_out, d_structs, nbytes, cudaMemcpyDeviceToHost, st));
    if (post_out && post_total) CF_CUDA(cudaMemcpyAsync(post_out, d_post, sizeof(float) * post_total, cudaMemcpyDeviceToHost, st));
    return read_status(eng, st);
}

}  // namespace

// ============================ C-ABI ============================
extern "C" {

const char* cf_last_error(void) { return g_err.c_str(); }
const char* cf_version(void) { return "contrafold-gb300 0.1.0 (sm_103a)"; }

int cf_engine_create(const float* params32, const double* params64, int device, cf_engine** out) {
    if (!out || !params32 || !params64) return fail(CF_EINVAL, "NULL argument to cf_engine_create");
    *out = nullptr;
    int ndev = 0;
    CF_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(CF_EINVAL, "no such CUDA device");
    CF_CUDA(cudaSetDevice(device));
    cf_engine* e = new cf_engine();
    e->device = device;
    if (cudaStreamCreateWithFlags(&e->stream_lo, cudaStreamNonBlocking) != cudaSuccess) {
        delete e;
        return fail(CF_ECUDA, "cudaStreamCreate failed");
    }
    e->stream = e->stream_lo;
    e->bind_buffers();
    {
        // freed blocks stay in the device's pool (no unmapping at each
        // synchronisation), so a buffer's regrowth maps no new memory
        static std::mutex pool_mu;
        static std::vector<int> pool_set;
        std::lock_guard<std::mutex> lk(pool_mu);
        if (std::find(pool_set.begin(), pool_set.end(), device) == pool_set.end()) {
            cudaMemPool_t pool;
            if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
                uint64_t keep = UINT64_MAX;
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            }
            cudaGetLastError();
            pool_set.push_back(device);
        }
    }
    int rc = cf_engine_set_params(e, params32, params64);
    if (!rc) {
        // a schedule table written by the tuner, when the environment names one
        const char* tf = std::getenv("CONTRAFOLD_GB300_TUNING");
        if (tf && *tf) rc = cf_engine_load_tuning(e, tf);
    }
    if (rc) {
        cf_engine_destroy(e);
        return rc;
    }
    *out = e;
    return CF_OK;
}

int cf_engine_destroy(cf_engine* e) {
    if (!e) return CF_OK;
    cudaSetDevice(e->device);
    if (e->stream_lo) cudaStreamSynchronize(e->stream_lo);
    if (e->stream_hi) cudaStreamSynchronize(e->stream_hi);
    e->blob32.release(); e->blob64.release(); e->arena.release(); e->seqs.release(); e->mask.release();
    e->descs.release(); e->logz.release(); e->logz64.release(); e->structs.release(); e->post.release();
    e->post_offs.release(); e->status.release(); e->samples.release(); e->seeds.release(); e->stream_idx.release();
    e->bonus.release(); e->counts.release(); e->unpaired.release();
    if (e->stream) cudaStreamSynchronize(e->stream);   // the stream-ordered frees

    if (e->stream_lo) cudaStreamDestroy(e->stream_lo);
    if (e->stream_hi) cudaStreamDestroy(e->stream_hi);
    delete e;
    return CF_OK;
}

int cf_engine_set_shared(cf_engine* e, int on) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    e->shared = on != 0;
    return CF_OK;
}

int cf_engine_set_priority(cf_engine* e, int high) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    CF_CUDA(cudaSetDevice(e->device));
    if (high && !e->stream_hi) {
        int least = 0, greatest = 0;
        CF_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        CF_CUDA(cudaStreamCreateWithPriority(&e->stream_hi, cudaStreamNonBlocking, greatest));
    }
    cudaStream_t next = high ? e->stream_hi : e->stream_lo;
    if (next != e->stream) {
        // the engine's calls are stream-ordered: finish the old stream's work first
        CF_CUDA(cudaStreamSynchronize(e->stream));
        e->stream = next;
    }
    return CF_OK;
}

int cf_engine_set_params(cf_engine* e, const float* params32, const double* params64) {
    if (!e || !params32 || !params64) return fail(CF_EINVAL, "NULL argument to cf_engine_set_params");
    CF_CUDA(cudaSetDevice(e->device));
    int rc;
    if ((rc = e->blob32.ensure(CF_BLOB_LEN))) return rc;
    if ((rc = e->blob64.ensure(CF_BLOB_LEN))) return rc;
    CF_CUDA(cudaMemcpyAsync(e->blob32.p, params32, sizeof(float) * CF_BLOB_LEN, cudaMemcpyHostToDevice, e->stream));
    CF_CUDA(cudaMemcpyAsync(e->blob64.p, params64, sizeof(double) * CF_BLOB_LEN, cudaMemcpyHostToDevice, e->stream));
    CF_CUDA(cudaStreamSynchronize(e->stream));
    return CF_OK;
}

int cf_engine_set_budget(cf_engine* e, size_t bytes) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    e->budget = bytes;
    return CF_OK;
}

int cf_engine_set_mode(cf_engine* e, int mode) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    if (mode != 0 && mode != 1) return fail(CF_EINVAL, "mode must be 0 (plain) or 1 (batched)");
    e->mode = mode;
    return CF_OK;
}

int cf_engine_set_schedule(cf_engine* e, int kind, int ctas_per_sm) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    if (kind == 5)
        return fail(CF_EINVAL, "the queue schedule (kind 5) is disabled: its kernel did not finish in two GPU test "
                               "runs and stays off the GPU until the cause is found");
    if (kind < 0 || kind > 4 || ctas_per_sm < 0) return fail(CF_EINVAL, "bad schedule");
    e->sched = kind;
    e->ctas_per_sm = ctas_per_sm;
    return CF_OK;
}

int cf_engine_set_group(cf_engine* e, int group) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    if (group < 0 || group > cf::kQueueMaxSeats) return fail(CF_EINVAL, "group must be in [0, 64]");
    e->group = group;
    return CF_OK;
}

int cf_engine_load_tuning(cf_engine* e, const char* path) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    if (!path) {
        e->tuning = default_tuning();
        return CF_OK;
    }
    std::ifstream in(path);
    if (!in) return fail(CF_EINVAL, std::string("cannot read tuning table ") + path);
    std::vector<TuneRow> rows;
    std::string err;
    if (parse_tuning(in, rows, err)) return fail(CF_EINVAL, std::string(path) + ": " + err);
    e->tuning = rows;
    return CF_OK;
}

int cf_engine_tuning_rows(const cf_engine* e) { return e ? (int)e->tuning.size() : 0; }

int cf_engine_set_grad_checkpoint(cf_engine* e, int32_t every) {
    if (!e) return fail(CF_EINVAL, "engine is NULL");
    if (every < 0) return fail(CF_EINVAL, "checkpoint spacing must be >= 0");
    e->grad_ckpt = every;
    return CF_OK;
}

size_t cf_grad_arena_bytes(int32_t L, int32_t every) {
    if (L < 0 || L > CF_MAX_LEN) return 0;
    if (every <= 0) every = cf::adj_auto_checkpoint(L);
    return sizeof(float) * (size_t)arena_words(JOB_GRAD, L, every);
}

int cf_logz(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
            float* logz_out) {
    if (n > 0 && !logz_out) return fail(CF_EINVAL, "logz_out is NULL");
    return run_host(e, JOB_LOGZ, seqs, offsets, mask, n, 0.f, logz_out, nullptr, nullptr, nullptr, nullptr);
}

int cf_logz64(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
              double* logz_out) {
    if (n > 0 && !logz_out) return fail(CF_EINVAL, "logz_out is NULL");
    return run_host(e, JOB_LOGZ64, seqs, offsets, mask, n, 0.f, nullptr, logz_out, nullptr, nullptr, nullptr);
}

int cf_bpp(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
           const int64_t* post_offsets, float* post_out, float* logz_out) {
    if (n > 0 && (!post_out || !post_offsets)) return fail(CF_EINVAL, "post_out / post_offsets is NULL");
    return run_host(e, JOB_BPP, seqs, offsets, mask, n, 0.f, logz_out, nullptr, nullptr, post_offsets, post_out);
}

int cf_mea(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n, float gamma,
           char* struct_out) {
    if (n > 0 && !struct_out) return fail(CF_EINVAL, "struct_out is NULL");
    if (!(gamma > 0.0f)) return fail(CF_EINVAL, "gamma must be > 0");
    return run_host(e, JOB_MEA, seqs, offsets, mask, n, gamma, nullptr, nullptr, struct_out, nullptr, nullptr);
}

int cf_mfe(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
           char* struct_out) {
    if (n > 0 && !struct_out) return fail(CF_EINVAL, "struct_out is NULL");
    return run_host(e, JOB_MFE, seqs, offsets, mask, n, 0.f, nullptr, nullptr, struct_out, nullptr, nullptr);
}

int cf_sample(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
              int32_t n_samples, uint64_t seed, char* out) {
    if (n_samples < 0) return fail(CF_EINVAL, "n_samples must be >= 0");
    if (n > 0 && n_samples > 0 && !out) return fail(CF_EINVAL, "out is NULL");
    return run_host(e, JOB_SAMPLE, seqs, offsets, mask, n, 0.f, nullptr, nullptr, nullptr, nullptr, nullptr, n_samples,
                    seed, out);
}

int cf_sample_seeded(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
                     int32_t n_samples, const uint64_t* seeds, char* out) {
    if (n_samples < 0) return fail(CF_EINVAL, "n_samples must be >= 0");
    if (n > 0 && n_samples > 0 && (!out || !seeds)) return fail(CF_EINVAL, "out / seeds is NULL");
    return run_host(e, JOB_SAMPLE, seqs, offsets, mask, n, 0.f, nullptr, nullptr, nullptr, nullptr, nullptr, n_samples,
                    0, out, seeds);
}

int cf_sample_tasks(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
                    int32_t chunk, uint64_t seed, char* out) {
    if (chunk <= 0) return fail(CF_EINVAL, "chunk must be > 0");
    if (n > 0 && !out) return fail(CF_EINVAL, "out is NULL");
    int rc = check_batch(e, seqs, offsets, n);
    if (rc) return rc;
    // the reference's order: tasks sorted by length (stable), cut into chunks;
    // chunk c0 samples with seed + c0, its k-th task with sequence index k
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        return offsets[x + 1] - offsets[x] < offsets[y + 1] - offsets[y];
    });
    std::vector<uint64_t> seeds(n);
    std::vector<int32_t> sidx(n);
    for (int r = 0; r < n; ++r) {
        const int c0 = r - r % chunk;
        seeds[order[r]] = seed + (uint64_t)c0;
        sidx[order[r]] = r - c0;
    }
    return run_host(e, JOB_SAMPLE, seqs, offsets, mask, n, 0.f, nullptr, nullptr, nullptr, nullptr, nullptr, 1, 0, out,
                    seeds.data(), sidx.data());
}

}  // extern "C"

// ============================ adjoint ============================
extern "C" int cf_grad(cf_engine* e, const uint8_t* seqs, const int64_t* offsets, const uint8_t* mask, int32_t n,
                       const float* bonus, float* logz_out, double* counts_out, double* unpaired_out) {
    int rc = check_batch(e, seqs, offsets, n);
    if (rc) return rc;
    if (n > 0 && (!counts_out || !unpaired_out)) return fail(CF_EINVAL, "counts_out / unpaired_out is NULL");
    if (n == 0) return CF_OK;
    CF_CUDA(cudaSetDevice(e->device));
    cudaStream_t st = e->stream;
    Plan P;
    if ((rc = make_plan(e, JOB_GRAD, offsets, n, P))) return rc;
    const size_t nbytes = (size_t)offsets[n];
    if ((rc = e->seqs.ensure(std::max<size_t>(nbytes, 1)))) return rc;
    if (nbytes) CF_CUDA(cudaMemcpyAsync(e->seqs.p, seqs, nbytes, cudaMemcpyHostToDevice, st));
    const uint8_t* d_mask = nullptr;
    if (mask) {
        if ((rc = e->mask.ensure(std::max<size_t>(nbytes, 1)))) return rc;
        if (nbytes) CF_CUDA(cudaMemcpyAsync(e->mask.p, mask, nbytes, cudaMemcpyHostToDevice, st));
        d_mask = e->mask.p;
    }
    const float* d_bonus = nullptr;
    if (bonus) {
        if ((rc = e->bonus.ensure(std::max<size_t>(nbytes, 1)))) return rc;
        if (nbytes) CF_CUDA(cudaMemcpyAsync(e->bonus.p, bonus, nbytes * sizeof(float), cudaMemcpyHostToDevice, st));
        d_bonus = e->bonus.p;
    }
    if ((rc = e->counts.ensure((size_t)n * CF_BLOB_LEN)) || (rc = e->unpaired.ensure(std::max<size_t>(nbytes, 1))) ||
        (rc = e->logz.ensure(n)) || (rc = e->descs.ensure(n)) || (rc = e->status.ensure(2)))
        return rc;
    CF_CUDA(cudaMemcpyAsync(e->descs.p, P.descs.data(), sizeof(SeqDesc) * n, cudaMemcpyHostToDevice, st));
    CF_CUDA(cudaMemsetAsync(e->status.p, 0, sizeof(int), st));
    int64_t maxw = 1;
    for (int64_t w : P.slice_words) maxw = std::max(maxw, w);
    if ((rc = e->arena.ensure((size_t)maxw))) return rc;
    const size_t smem = cf::adj_smem_bytes(P.Lmax);
    {
        int dev_max = 0;
        CF_CUDA(cudaDeviceGetAttribute(&dev_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, e->device));
        if (smem > (size_t)dev_max) return fail(CF_EINVAL, "sequence too long for the adjoint kernels");
        for (const void* k : {(const void*)cf::k_adj_inside, (const void*)cf::k_adj_outside}) {
            const int rs = raise_smem_limit(k, e->device, std::max<size_t>(smem, 48 * 1024));
            if (rs) return rs;
        }
    }
    for (size_t sl = 0; sl + 1 < P.slice_begin.size(); ++sl) {
        const int k0 = P.slice_begin[sl], k1 = P.slice_begin[sl + 1];
        cf::FoldArgs A;
        A.descs = e->descs.p + k0;
        A.n = k1 - k0;
        A.group = 1;
        A.seqs = e->seqs.p;
        A.mask = d_mask;
        A.blob32 = e->blob32.p;
        A.blob64 = e->blob64.p;
        A.ws = e->arena.p;
        A.logz = e->logz.p;
        A.logz64 = nullptr;
        A.structs = nullptr;
        A.post_out = nullptr;
        A.post_offs = nullptr;
        A.gamma = 0.f;
        A.status = e->status.p;
        cf::k_adj_inside<<<A.n, cf::kFoldThreads, smem, st>>>(A, d_bonus, P.grad_ckpt);
        cf::k_adj_outside<<<A.n, cf::kFoldThreads, smem, st>>>(A, d_bonus, P.grad_ckpt, e->counts.p, e->unpaired.p);
        CF_CUDA(cudaGetLastError());
    }
    CF_CUDA(cudaMemcpyAsync(counts_out, e->counts.p, sizeof(double) * n * CF_BLOB_LEN, cudaMemcpyDeviceToHost, st));
    if (nbytes) CF_CUDA(cudaMemcpyAsync(unpaired_out, e->unpaired.p, sizeof(double) * nbytes, cudaMemcpyDeviceToHost, st));
    if (logz_out) CF_CUDA(cudaMemcpyAsync(logz_out, e->logz.p, sizeof(float) * n, cudaMemcpyDeviceToHost, st));
    return read_status(e, st);
}

// ============================ plans (device-resident batches) ============================
struct cf_plan {
    cf_engine* eng = nullptr;
    Job job = JOB_MEA;
    Plan P;
    int n = 0;
    DevBuf<SeqDesc> descs;
    DevBuf<float> arena;
    DevBuf<int> status;
    DevBuf<int64_t> post_offs;   // CF_JOB_BPP: sequence b's matrix at sum_{c<b} L_c^2 floats
    PhaseTimer timer;
    int launches = 0;
    // CUDA graph of the plan's launches, replayed while the run arguments stay
    // the same (cf_plan_set_graph)
    bool graph_on = false;
    cudaGraphExec_t gexec = nullptr;
    const void* g_seqs = nullptr;
    const void* g_mask = nullptr;
    void* g_out = nullptr;
    float g_gamma = 0.f;
    int g_launches = 0;
};

namespace {

// Shared memory run_device will ask for: set before a stream capture, which
// then records kernel launches only.
int plan_prepare_smem(cf_engine* e, Job job, const Plan& P) {
    size_t bytes;
    if (P.cta) {
        bytes = cf::fold_smem_bytes(P.Lmax, 1, false);
    } else if (P.warp) {
        bytes = cf::warp_smem_bytes(P.Lmax);
    } else if (P.queue) {
        const int mode = job == JOB_LOGZ ? cf::kQueueLogZ : job == JOB_MEA ? cf::kQueueMea
                       : job == JOB_BPP ? cf::kQueueBpp : cf::kQueueSample;
        bytes = cf::queue_smem_bytes(P.Lmax, P.seats, mode);
    } else {
        const bool fp64 = job == JOB_LOGZ64 || job == JOB_MFE;
        bytes = std::max(cf::fold_smem_bytes(P.Lmax, P.group, fp64), cf::plain_smem_bytes(P.Lmax));
    }
    return ensure_smem(e, bytes);
}

}  // namespace

extern "C" {

int cf_plan_create(cf_engine* e, int32_t job, const int64_t* offsets, int32_t n, cf_plan** out) {
    if (!out) return fail(CF_EINVAL, "out is NULL");
    *out = nullptr;
    int rc = check_batch(e, reinterpret_cast<const uint8_t*>(1), offsets, n);
    if (rc) return rc;
    if (job != CF_JOB_LOGZ && job != CF_JOB_LOGZ64 && job != CF_JOB_BPP && job != CF_JOB_MEA && job != CF_JOB_MFE)
        return fail(CF_EINVAL, "plans support CF_JOB_LOGZ, CF_JOB_LOGZ64, CF_JOB_BPP, CF_JOB_MEA, CF_JOB_MFE");
    CF_CUDA(cudaSetDevice(e->device));
    cf_plan* p = new cf_plan();
    p->eng = e;
    p->job = job == CF_JOB_LOGZ ? JOB_LOGZ : job == CF_JOB_LOGZ64 ? JOB_LOGZ64 : job == CF_JOB_BPP ? JOB_BPP
           : job == CF_JOB_MEA ? JOB_MEA : JOB_MFE;
    p->n = n;
    if ((rc = make_plan(e, p->job, offsets, n, p->P)) || (rc = p->descs.ensure(std::max(n, 1))) ||
        (rc = p->status.ensure(2))) {
        delete p;
        return rc;
    }
    int64_t maxw = 1;
    for (int64_t w : p->P.slice_words) maxw = std::max(maxw, w);
    if ((rc = p->arena.ensure((size_t)maxw))) {
        p->descs.release(); p->status.release();
        delete p;
        return rc;
    }
    if (n) CF_CUDA(cudaMemcpy(p->descs.p, p->P.descs.data(), sizeof(SeqDesc) * n, cudaMemcpyHostToDevice));
    if (p->job == JOB_BPP) {
        std::vector<int64_t> po(std::max(n, 1), 0);
        int64_t acc = 0;
        for (int b = 0; b < n; ++b) {
            po[b] = acc;
            acc += (offsets[b + 1] - offsets[b]) * (offsets[b + 1] - offsets[b]);
        }
        if ((rc = p->post_offs.ensure(po.size()))) {
            cf_plan_destroy(p);
            return rc;
        }
        CF_CUDA(cudaMemcpy(p->post_offs.p, po.data(), sizeof(int64_t) * po.size(), cudaMemcpyHostToDevice));
    }
    CF_CUDA(cudaMemset(p->status.p, 0, sizeof(int)));
    *out = p;
    return CF_OK;
}

int cf_plan_destroy(cf_plan* p) {
    if (!p) return CF_OK;
    cudaSetDevice(p->eng->device);
    cudaDeviceSynchronize();
    if (p->gexec) cudaGraphExecDestroy(p->gexec);
    p->descs.release(); p->arena.release(); p->status.release(); p->post_offs.release();
    delete p;
    return CF_OK;
}

size_t cf_plan_arena_bytes(const cf_plan* p) { return p ? p->arena.cap * sizeof(float) : 0; }

int cf_plan_run(cf_plan* p, const uint8_t* d_seqs, const uint8_t* d_mask, float gamma, void* d_out, void* stream) {
    if (!p) return fail(CF_EINVAL, "plan is NULL");
    if (p->n > 0 && (!d_out || (!d_seqs && p->P.Lmax > 0))) return fail(CF_EINVAL, "NULL device buffer");
    if (p->job == JOB_MEA && !(gamma > 0.0f)) return fail(CF_EINVAL, "gamma must be > 0");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : p->eng->stream;
    Exec X;
    X.d_descs = p->descs.p;
    X.arena = p->arena.p;
    X.status = p->status.p;
    X.timer = p->timer.on ? &p->timer : nullptr;
    float* lz = p->job == JOB_LOGZ ? static_cast<float*>(d_out) : nullptr;
    double* lz64 = p->job == JOB_LOGZ64 ? static_cast<double*>(d_out) : nullptr;
    char* st_out = (p->job == JOB_MEA || p->job == JOB_MFE) ? static_cast<char*>(d_out) : nullptr;
    float* post = p->job == JOB_BPP ? static_cast<float*>(d_out) : nullptr;
    const int64_t* post_offs = p->job == JOB_BPP ? p->post_offs.p : nullptr;
    if (p->graph_on && !p->timer.on && p->n > 0) {
        const bool hit = p->gexec != nullptr && p->g_seqs == d_seqs && p->g_mask == d_mask && p->g_out == d_out &&
                         p->g_gamma == gamma;
        if (!hit) {   // (re)capture the launches of one run
            int rc = plan_prepare_smem(p->eng, p->job, p->P);
            if (rc) return rc;
            if (p->gexec) {
                CF_CUDA(cudaGraphExecDestroy(p->gexec));
                p->gexec = nullptr;
            }
            CF_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            X.timer = nullptr;
            rc = run_device(p->eng, p->job, p->P, X, d_seqs, d_mask, gamma, lz, lz64, st_out, post, post_offs, st);
            cudaGraph_t g = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(st, &g);
            if (rc || ec != cudaSuccess) {
                if (g) cudaGraphDestroy(g);
                return rc ? rc : fail(CF_ECUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(ec));
            }
            const cudaError_t ei = cudaGraphInstantiate(&p->gexec, g, 0);
            cudaGraphDestroy(g);
            if (ei != cudaSuccess) {
                p->gexec = nullptr;
                return fail(CF_ECUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(ei));
            }
            p->g_seqs = d_seqs;
            p->g_mask = d_mask;
            p->g_out = d_out;
            p->g_gamma = gamma;
            p->g_launches = X.launches;
        }
        CF_CUDA(cudaGraphLaunch(p->gexec, st));
        p->launches = p->g_launches;
        return CF_OK;
    }
    int rc = run_device(p->eng, p->job, p->P, X, d_seqs, d_mask, gamma, lz, lz64, st_out, post, post_offs, st);
    p->launches = X.launches;
    return rc;
}

const char* cf_plan_schedule(const cf_plan* p) {
    if (!p) return "";
    if (p->P.plain) return "plain";
    if (p->P.warp) return "warp";
    if (p->P.cta) return "cta";
    if (p->P.cluster) return "cluster";
    if (p->P.queue) return "queue";
    return "group";
}

int cf_plan_set_graph(cf_plan* p, int on) {
    if (!p) return fail(CF_EINVAL, "plan is NULL");
    p->graph_on = on != 0;
    return CF_OK;
}

int cf_plan_status(cf_plan* p) {
    if (!p) return fail(CF_EINVAL, "plan is NULL");
    int h = 0;
    CF_CUDA(cudaSetDevice(p->eng->device));
    // the runs may be on any stream, non-blocking ones included: wait for the device
    CF_CUDA(cudaDeviceSynchronize());
    CF_CUDA(cudaMemcpy(&h, p->status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h != CF_OK) return fail(h, "a kernel reported an internal limit (traceback stack/queue)");
    return CF_OK;
}

int cf_plan_set_timing(cf_plan* p, int on) {
    if (!p) return fail(CF_EINVAL, "plan is NULL");
    p->timer.on = on != 0;
    return CF_OK;
}

int cf_plan_phase_ms(cf_plan* p, float* ms, int32_t nphases) {
    if (!p || !ms) return fail(CF_EINVAL, "NULL argument");
    if (!p->timer.on) return fail(CF_EINVAL, "timing is off for this plan");
    return p->timer.read(ms, std::min<int32_t>(nphases, kPhases));
}

int cf_plan_launches(const cf_plan* p) { return p ? p->launches : 0; }

int cf_plan_group(const cf_plan* p) { return p ? p->P.group : 0; }

}  // extern "C"

// ============================ accessors for other host units (cf_host.h) ============================
namespace cf {

int engine_device(const cf_engine* e) { return e->device; }
cudaStream_t engine_stream(const cf_engine* e) { return e->stream; }
const float* engine_blob32(const cf_engine* e) { return e->blob32.p; }
int engine_ensure_smem(cf_engine* e, size_t bytes) { return ensure_smem(e, bytes); }
int engine_fail(int code, const char* msg) { return fail(code, msg); }

}  // namespace cf
