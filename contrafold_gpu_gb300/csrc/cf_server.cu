// cf_server.cu -- the serving loop: continuous batching of single-sequence
// requests over several engines.
//
// Requests (logZ, MEA, Boltzmann samples) arrive one sequence at a time.  Each
// worker thread owns one engine (parameters, stream, arena) and loops: take the
// queue whose oldest request is the oldest of all, drain up to max_batch
// requests / max_batch_nt nucleotides from it, fold them as one batch, publish
// the results.  A queue holds requests that can share one batched call: same
// op, same gamma or sample count, and the same length bucket, so a 40-nt
// request never waits behind a 900-nt one.  Requests that arrive while a batch
// runs are picked up by the next free worker; with several workers the batches
// of different streams overlap on the device.
//
// Long requests are kept from blocking short ones: buckets whose upper edge is
// above long_len are "long", and only the first long_workers workers take long
// batches (they take short ones when no long request waits); the others serve
// short buckets only.  The engine picks the kernels per batch (small batches
// fold one sequence per CTA, or per 8-SM thread-block cluster when every
// sequence has 512 nt or more -- the latency-optimal shapes).
//
// Every result is what the same request gives alone: logZ and MEA do not
// depend on batch composition, and samples use a per-request seed
// (cf_sample_seeded).
//
// Tracing: with CONTRAFOLD_GB300_SERVER_TRACE=<file> set when the server is
// created, every batch appends one line to <file>: worker, op, bucket,
// requests, nucleotides, longest sequence, start and end (seconds since the
// server was created), status.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/contrafold_gb300.h"
#include "cf_device.cuh"
#include "cf_host.h"

namespace {

using Clock = std::chrono::steady_clock;

enum State { kQueued = 0, kRunning = 1, kDone = 2 };

struct Req {
    int64_t ticket = 0;
    cf_request r{};
    std::string seq;
    std::string mask;          // empty: no constraint
    int bucket = 0;
    State state = kQueued;
    int status = CF_OK;
    std::string err;
    float logz = 0.f;
    std::string out;           // dot-bracket (MEA) or n_samples * L bytes (sampling)
    Clock::time_point t_submit, t_start, t_done;
};

struct Key {
    int op, bucket, n_samples;
    uint32_t gamma_bits;
    bool operator<(const Key& o) const {
        if (op != o.op) return op < o.op;
        if (bucket != o.bucket) return bucket < o.bucket;
        if (n_samples != o.n_samples) return n_samples < o.n_samples;
        return gamma_bits < o.gamma_bits;
    }
};

int fail(int code, const std::string& msg) { return cf::engine_fail(code, msg.c_str()); }

}  // namespace

struct cf_server {
    int device = 0;
    std::vector<cf_engine*> engines;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::map<Key, std::deque<Req*>> queues;
    std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
    int64_t next_ticket = 1;
    int64_t queued = 0;        // requests in all queues
    int64_t queued_long = 0;   // of which in long buckets
    bool stop = false;
    bool paused = false;
    int32_t max_batch = 4096;
    int64_t max_batch_nt = int64_t(1) << 20;
    double max_batch_cost = 0;          // predicted work of a batch, sum of L^3 (0 = no limit)
    int64_t max_batch_arena = 0;        // device arena bytes of a batch (0 = no limit)
    int32_t long_len = 256;              // buckets whose upper edge is above this are long
    int32_t long_workers = 1;            // workers [0, long_workers) may take long batches
    std::vector<int32_t> edges{96, 192, 256, 384, 640};
    // statistics
    int64_t n_batches = 0, n_done = 0, nt_done = 0, n_cancelled = 0;
    double busy_s = 0;                   // summed batch wall time over workers
    double wait_s = 0, max_wait_s = 0;   // queue wait (submit -> batch start) over requests
    double serve_s = 0, max_serve_s = 0; // batch run time seen by each request
    // batch trace (CONTRAFOLD_GB300_SERVER_TRACE)
    FILE* trace = nullptr;
    std::mutex trace_mu;
    Clock::time_point t_created = Clock::now();

    int bucket_of(int32_t L) const {
        int b = 0;
        while (b < (int)edges.size() && L > edges[b]) ++b;
        return b;
    }
    int32_t bucket_max_len(int b) const { return b < (int)edges.size() ? edges[b] : CF_MAX_LEN; }
    bool is_long(int b) const { return bucket_max_len(b) > long_len; }
};

namespace {

// Device arena bytes one request of L nt takes in a batched call: the full
// FP32 fold arena for MEA, its inside-only prefix for logZ and sampling.
int64_t request_arena_bytes(int op, int L) {
    const int64_t w = op == CF_OP_MEA ? cf::arena32(L).total : cf::arena32_inside_words(L);
    return 4 * w;
}

// Folds one batch on `eng`; fills each request's outputs and status.
void run_batch(cf_server* S, cf_engine* eng, const Key& key, std::vector<Req*>& batch, std::vector<uint8_t>& buf,
               std::vector<int64_t>& offs, std::vector<uint8_t>& mask, std::vector<uint64_t>& seeds,
               std::vector<float>& lz, std::vector<char>& out) {
    const int n = (int)batch.size();
    offs.assign(n + 1, 0);
    bool any_mask = false;
    for (int b = 0; b < n; ++b) {
        offs[b + 1] = offs[b] + (int64_t)batch[b]->seq.size();
        any_mask |= !batch[b]->mask.empty();
    }
    const int64_t nt = offs[n];
    buf.resize(std::max<int64_t>(nt, 1));
    for (int b = 0; b < n; ++b) std::memcpy(buf.data() + offs[b], batch[b]->seq.data(), batch[b]->seq.size());
    if (any_mask) {
        mask.assign(std::max<int64_t>(nt, 1), 0);
        for (int b = 0; b < n; ++b)
            if (!batch[b]->mask.empty()) std::memcpy(mask.data() + offs[b], batch[b]->mask.data(), batch[b]->mask.size());
    }
    const uint8_t* mp = any_mask ? mask.data() : nullptr;
    int rc = CF_OK;
    if (key.op == CF_OP_LOGZ) {
        lz.assign(n, 0.f);
        rc = cf_logz(eng, buf.data(), offs.data(), mp, n, lz.data());
    } else if (key.op == CF_OP_MEA) {
        out.assign(std::max<int64_t>(nt, 1), '.');
        float g;
        std::memcpy(&g, &key.gamma_bits, sizeof g);
        rc = cf_mea(eng, buf.data(), offs.data(), mp, n, g, out.data());
    } else {
        const int64_t tot = nt * key.n_samples;
        out.assign(std::max<int64_t>(tot, 1), '.');
        seeds.resize(n);
        for (int b = 0; b < n; ++b) seeds[b] = batch[b]->r.seed;
        rc = cf_sample_seeded(eng, buf.data(), offs.data(), mp, n, key.n_samples, seeds.data(), out.data());
    }
    const std::string err = rc ? std::string(cf_last_error()) : std::string();
    for (int b = 0; b < n; ++b) {
        Req* q = batch[b];
        q->status = rc;
        q->err = err;
        if (rc) continue;
        if (key.op == CF_OP_LOGZ) q->logz = lz[b];
        else if (key.op == CF_OP_MEA) q->out.assign(out.data() + offs[b], q->seq.size());
        else q->out.assign(out.data() + offs[b] * key.n_samples, q->seq.size() * (size_t)key.n_samples);
    }
}

void worker_loop(cf_server* S, int w) {
    cf_engine* eng = S->engines[w];
    cudaSetDevice(S->device);
    std::vector<Req*> batch;
    std::vector<uint8_t> buf, mask;
    std::vector<int64_t> offs;
    std::vector<uint64_t> seeds;
    std::vector<float> lz;
    std::vector<char> out;
    for (;;) {
        Key key{};
        {
            std::unique_lock<std::mutex> lk(S->mu);
            const bool may_long = w < S->long_workers;   // read under the lock: configure may change it
            auto has_work = [&] {
                return S->queued - S->queued_long > 0 || (may_long && S->queued_long > 0);
            };
            S->cv_work.wait(lk, [&] { return S->stop || (!S->paused && has_work()); });
            if (S->stop) return;
            // oldest long request first (long-capable workers), else the oldest short one
            auto best = S->queues.end();
            for (int pass = may_long ? 0 : 1; pass < 2 && best == S->queues.end(); ++pass)
                for (auto it = S->queues.begin(); it != S->queues.end(); ++it) {
                    if (it->second.empty() || S->is_long(it->first.bucket) != (pass == 0)) continue;
                    if (best == S->queues.end() || it->second.front()->t_submit < best->second.front()->t_submit)
                        best = it;
                }
            if (best == S->queues.end()) continue;
            const bool long_batch = S->is_long(best->first.bucket);
            key = best->first;
            auto& q = best->second;
            batch.clear();
            int64_t nt = 0, arena = 0;
            double cost = 0;
            // oldest first, while the batch stays within its count, nucleotide,
            // predicted-work (sum of L^3: the fold is cubic in the length) and
            // arena-byte limits; the first request is always taken
            while (!q.empty() && (int)batch.size() < S->max_batch) {
                Req* r = q.front();
                const int64_t L = (int64_t)r->seq.size();
                const double c = (double)L * (double)L * (double)L;
                const int64_t a = request_arena_bytes(key.op, (int)L);
                if (!batch.empty() && (nt + L > S->max_batch_nt ||
                                       (S->max_batch_cost > 0 && cost + c > S->max_batch_cost) ||
                                       (S->max_batch_arena > 0 && arena + a > S->max_batch_arena)))
                    break;
                q.pop_front();
                --S->queued;
                if (long_batch) --S->queued_long;
                r->state = kRunning;
                nt += L;
                cost += c;
                arena += a;
                batch.push_back(r);
            }
            if (q.empty()) S->queues.erase(best);
            if (S->queued > 0) S->cv_work.notify_all();
        }
        const auto t0 = Clock::now();
        for (Req* r : batch) r->t_start = t0;
        run_batch(S, eng, key, batch, buf, offs, mask, seeds, lz, out);
        const auto t1 = Clock::now();
        if (S->trace) {
            int64_t nt = 0;
            size_t lmax = 0;
            for (Req* r : batch) {
                nt += (int64_t)r->seq.size();
                lmax = std::max(lmax, r->seq.size());
            }
            std::lock_guard<std::mutex> lk(S->trace_mu);
            std::fprintf(S->trace, "%d %d %d %zu %lld %zu %.6f %.6f %d\n", w, key.op, key.bucket, batch.size(),
                         (long long)nt, lmax, std::chrono::duration<double>(t0 - S->t_created).count(),
                         std::chrono::duration<double>(t1 - S->t_created).count(), batch.empty() ? 0 : batch[0]->status);
        }
        {
            std::lock_guard<std::mutex> lk(S->mu);
            const double serve = std::chrono::duration<double>(t1 - t0).count();
            for (Req* r : batch) {
                r->state = kDone;
                r->t_done = t1;
                S->nt_done += (int64_t)r->seq.size();
                const double wait = std::chrono::duration<double>(t0 - r->t_submit).count();
                S->wait_s += wait;
                S->max_wait_s = std::max(S->max_wait_s, wait);
                S->serve_s += serve;
                S->max_serve_s = std::max(S->max_serve_s, serve);
            }
            S->n_done += (int64_t)batch.size();
            S->n_batches += 1;
            S->busy_s += std::chrono::duration<double>(t1 - t0).count();
        }
        S->cv_done.notify_all();
    }
}

int validate(const cf_request* r, const uint8_t* seq, int32_t len) {
    if (!r) return fail(CF_EINVAL, "request is NULL");
    if (r->op != CF_OP_LOGZ && r->op != CF_OP_MEA && r->op != CF_OP_SAMPLE) return fail(CF_EINVAL, "bad request op");
    if (len < 0 || len > CF_MAX_LEN) return fail(CF_EINVAL, "bad sequence length");
    if (len > 0 && !seq) return fail(CF_EINVAL, "seq is NULL");
    if (r->op == CF_OP_MEA && !(r->gamma > 0.0f)) return fail(CF_EINVAL, "gamma must be > 0");
    if (r->op == CF_OP_SAMPLE && (r->n_samples < 0 || r->n_samples > 1 << 20))
        return fail(CF_EINVAL, "n_samples must be in [0, 2^20]");
    return CF_OK;
}

// Enqueues one request; the caller holds no lock.
int submit_one(cf_server* S, const cf_request* r, const uint8_t* seq, int32_t len, const uint8_t* mask,
               Clock::time_point t_submit, int64_t* ticket) {
    auto q = std::make_unique<Req>();
    q->r = *r;
    if (r->op != CF_OP_MEA) q->r.gamma = 0.f;
    if (r->op != CF_OP_SAMPLE) q->r.n_samples = 0;
    q->seq.assign(reinterpret_cast<const char*>(seq ? seq : reinterpret_cast<const uint8_t*>("")), (size_t)len);
    if (mask) {
        q->mask.resize((size_t)len);
        for (int32_t t = 0; t < len; ++t) q->mask[t] = mask[t] != 0 ? 1 : 0;
    }
    q->t_submit = t_submit;
    Key key;
    key.op = q->r.op;
    key.n_samples = q->r.n_samples;
    std::memcpy(&key.gamma_bits, &q->r.gamma, sizeof(float));
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) return fail(CF_ECANCELLED, "server is shutting down");
        q->bucket = S->bucket_of(len);
        key.bucket = q->bucket;
        q->ticket = S->next_ticket++;
        *ticket = q->ticket;
        S->queues[key].push_back(q.get());
        S->queued += 1;
        if (S->is_long(key.bucket)) S->queued_long += 1;
        S->reqs.emplace(q->ticket, std::move(q));
    }
    S->cv_work.notify_all();
    return CF_OK;
}

// Copies a finished request's outputs; erases it.  Caller holds S->mu.
int collect(cf_server* S, std::unordered_map<int64_t, std::unique_ptr<Req>>::iterator it, float* logz_out, char* out,
            int64_t out_cap, double* latency_ms, Clock::time_point t_ref) {
    Req* q = it->second.get();
    int rc = q->status;
    std::string err = q->err;
    if (rc == CF_OK) {
        if (q->r.op == CF_OP_LOGZ) {
            if (logz_out) *logz_out = q->logz;
        } else if (out) {
            if ((int64_t)q->out.size() > out_cap) {
                rc = CF_EINVAL;
                err = "output buffer too small";
            } else {
                std::memcpy(out, q->out.data(), q->out.size());
            }
        }
    }
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(q->t_done - t_ref).count();
    S->reqs.erase(it);
    if (rc) return fail(rc, err);
    return CF_OK;
}

}  // namespace

extern "C" {

int cf_server_create(const float* params32, const double* params64, int device, int32_t n_workers,
                     cf_server** out) {
    if (!out) return fail(CF_EINVAL, "out is NULL");
    *out = nullptr;
    if (n_workers < 1 || n_workers > 64) return fail(CF_EINVAL, "n_workers must be in [1, 64]");
    auto* S = new cf_server();
    S->device = device;
    for (int w = 0; w < n_workers; ++w) {
        cf_engine* e = nullptr;
        int rc = cf_engine_create(params32, params64, device, &e);
        if (rc) {
            std::string msg = cf_last_error();
            for (cf_engine* x : S->engines) cf_engine_destroy(x);
            delete S;
            return fail(rc, msg);
        }
        cf_engine_set_shared(e, 1);   // the workers' launches share the device
        S->engines.push_back(e);
    }
    if (const char* tp = std::getenv("CONTRAFOLD_GB300_SERVER_TRACE"))
        if (*tp) S->trace = std::fopen(tp, "a");
    for (int w = 0; w < n_workers; ++w) S->workers.emplace_back(worker_loop, S, w);
    *out = S;
    return CF_OK;
}

int cf_server_configure(cf_server* S, int32_t max_batch, int64_t max_batch_nt, int32_t long_len,
                        int32_t long_workers, const int32_t* edges, int32_t n_edges) {
    if (!S) return fail(CF_EINVAL, "server is NULL");
    if (max_batch < 1 || max_batch_nt < 1 || long_len < 0 || n_edges < 0 || (n_edges > 0 && !edges) ||
        long_workers < 1 || long_workers > (int32_t)S->engines.size())
        return fail(CF_EINVAL, "bad server configuration");
    for (int k = 1; k < n_edges; ++k)
        if (edges[k] <= edges[k - 1]) return fail(CF_EINVAL, "bucket edges must increase");
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->queued > 0) return fail(CF_EINVAL, "reconfigure only while no request is queued");
    S->max_batch = max_batch;
    S->max_batch_nt = max_batch_nt;
    S->long_len = long_len;
    S->long_workers = long_workers;
    S->edges.assign(edges, edges + n_edges);
    return CF_OK;
}

int cf_server_set_limits(cf_server* S, double max_batch_cost, int64_t max_batch_arena_bytes) {
    if (!S) return fail(CF_EINVAL, "server is NULL");
    if (!(max_batch_cost >= 0) || max_batch_arena_bytes < 0) return fail(CF_EINVAL, "limits must be >= 0");
    std::lock_guard<std::mutex> lk(S->mu);
    S->max_batch_cost = max_batch_cost;
    S->max_batch_arena = max_batch_arena_bytes;
    return CF_OK;
}

int cf_server_destroy(cf_server* S) {
    if (!S) return CF_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto& t : S->workers) t.join();
    for (cf_engine* e : S->engines) cf_engine_destroy(e);
    if (S->trace) std::fclose(S->trace);
    delete S;
    return CF_OK;
}

int cf_server_pause(cf_server* S, int32_t on) {
    if (!S) return fail(CF_EINVAL, "server is NULL");
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->paused = on != 0;
    }
    S->cv_work.notify_all();
    return CF_OK;
}

int cf_server_submit(cf_server* S, const cf_request* r, const uint8_t* seq, int32_t len, const uint8_t* mask,
                     int64_t* ticket) {
    if (!S || !ticket) return fail(CF_EINVAL, "server / ticket is NULL");
    int rc = validate(r, seq, len);
    if (rc) return rc;
    return submit_one(S, r, seq, len, mask, Clock::now(), ticket);
}

int cf_server_wait(cf_server* S, int64_t ticket, int32_t timeout_ms, float* logz_out, char* out, int64_t out_cap) {
    if (!S) return fail(CF_EINVAL, "server is NULL");
    std::unique_lock<std::mutex> lk(S->mu);
    if (S->reqs.find(ticket) == S->reqs.end()) return fail(CF_EINVAL, "unknown ticket");
    // the request is looked up on every wake-up: another wait on the same
    // ticket may have collected (and freed) it meanwhile
    auto ready = [&] {
        auto f = S->reqs.find(ticket);
        return f == S->reqs.end() || f->second->state == kDone;
    };
    if (timeout_ms < 0) {
        S->cv_done.wait(lk, ready);
    } else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) {
        return fail(CF_ETIMEOUT, "request not finished within the timeout");
    }
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return fail(CF_EINVAL, "ticket collected by another wait");
    return collect(S, it, logz_out, out, out_cap, nullptr, it->second->t_submit);
}

int cf_server_cancel(cf_server* S, int64_t ticket) {
    if (!S) return fail(CF_EINVAL, "server is NULL");
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return fail(CF_EINVAL, "unknown ticket");
    Req* q = it->second.get();
    if (q->state != kQueued) return fail(CF_EINVAL, "request is already running or finished");
    for (auto qi = S->queues.begin(); qi != S->queues.end(); ++qi) {
        auto& d = qi->second;
        auto pos = std::find(d.begin(), d.end(), q);
        if (pos == d.end()) continue;
        d.erase(pos);
        if (d.empty()) S->queues.erase(qi);
        break;
    }
    S->queued -= 1;
    if (S->is_long(q->bucket)) S->queued_long -= 1;
    q->state = kDone;
    q->status = CF_ECANCELLED;
    q->err = "request cancelled";
    q->t_done = Clock::now();
    S->n_cancelled += 1;
    S->cv_done.notify_all();
    return CF_OK;
}

int cf_server_replay(cf_server* S, int32_t n, const double* t_arrive, const cf_request* reqs, const uint8_t* seqs,
                     const int64_t* offsets, const uint8_t* mask, const int64_t* out_offsets, float* logz_out,
                     char* out, double* latency_ms, int32_t* status_out) {
    if (!S) return fail(CF_EINVAL, "server is NULL");
    if (n < 0) return fail(CF_EINVAL, "negative request count");
    if (n == 0) return CF_OK;
    if (!t_arrive || !reqs || !offsets || !latency_ms || !status_out) return fail(CF_EINVAL, "NULL argument");
    for (int k = 0; k < n; ++k) {
        const int64_t L = offsets[k + 1] - offsets[k];
        int rc = validate(&reqs[k], seqs + offsets[k], (int32_t)std::min<int64_t>(L, CF_MAX_LEN + 1));
        if (rc) return rc;
        if (k > 0 && t_arrive[k] < t_arrive[k - 1]) return fail(CF_EINVAL, "arrival times must not decrease");
        if (reqs[k].op != CF_OP_LOGZ && (!out || !out_offsets)) return fail(CF_EINVAL, "out / out_offsets is NULL");
        if (reqs[k].op == CF_OP_LOGZ && !logz_out) return fail(CF_EINVAL, "logz_out is NULL");
    }
    std::vector<int64_t> tickets(n);
    std::vector<Clock::time_point> due(n);
    const auto t0 = Clock::now();
    // submit open-loop; a failed submission (e.g. the server is stopping) ends
    // the submissions, and the requests already in are still collected below
    int nsub = 0, submit_rc = CF_OK;
    std::string submit_err;
    for (int k = 0; k < n; ++k) {
        due[k] = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(t_arrive[k]));
        std::this_thread::sleep_until(due[k]);
        const int32_t L = (int32_t)(offsets[k + 1] - offsets[k]);
        submit_rc = submit_one(S, &reqs[k], seqs + offsets[k], L, mask ? mask + offsets[k] : nullptr, due[k], &tickets[k]);
        if (submit_rc) {
            submit_err = cf_last_error();
            break;
        }
        ++nsub;
    }
    for (int k = 0; k < nsub; ++k) {
        std::unique_lock<std::mutex> lk(S->mu);
        const int64_t tk = tickets[k];
        S->cv_done.wait(lk, [&] {
            auto f = S->reqs.find(tk);
            return f == S->reqs.end() || f->second->state == kDone;
        });
        auto it = S->reqs.find(tk);
        if (it == S->reqs.end()) {   // collected by a wait on the same ticket
            status_out[k] = CF_EINVAL;
            latency_ms[k] = 0.0;
            continue;
        }
        const int64_t L = offsets[k + 1] - offsets[k];
        const int64_t cap = reqs[k].op == CF_OP_SAMPLE ? L * reqs[k].n_samples : L;
        status_out[k] = collect(S, it, reqs[k].op == CF_OP_LOGZ ? logz_out + k : nullptr,
                                reqs[k].op == CF_OP_LOGZ ? nullptr : out + out_offsets[k], cap, latency_ms + k, due[k]);
    }
    for (int k = nsub; k < n; ++k) {   // never submitted
        status_out[k] = CF_ECANCELLED;
        latency_ms[k] = 0.0;
    }
    if (submit_rc) return fail(submit_rc, "cf_server_replay: submission " + std::to_string(nsub) + " failed: " + submit_err);
    return CF_OK;
}

int cf_server_stats(cf_server* S, double* stats, int32_t n_stats) {
    if (!S || !stats) return fail(CF_EINVAL, "NULL argument");
    std::lock_guard<std::mutex> lk(S->mu);
    const double v[] = {(double)S->n_batches, (double)S->n_done, (double)S->nt_done, (double)S->n_cancelled,
                        S->busy_s, (double)S->queued, S->wait_s, S->max_wait_s, S->serve_s, S->max_serve_s};
    for (int k = 0; k < n_stats && k < (int)(sizeof v / sizeof v[0]); ++k) stats[k] = v[k];
    return CF_OK;
}

}  // extern "C"
