/*
 * contrafold_gb300.h -- C-ABI of the GB300 (sm_103a) CONTRAfold folding engine.
 *
 * The engine replaces, behind a plain C interface, the compute entry points of
 * the reference package `gpu_contrafold`:
 *
 *   cf_logz      <- gpu_contrafold/gpu.py:480-517   logZ_batch   (FP32 inside)
 *   cf_logz64    <- gpu_contrafold/cpu.py:165-287   inside/logZ  (FP64 exact log1p/exp)
 *   cf_bpp       <- gpu_contrafold/cpu.py:583-820,926-929  posterior/bpp
 *   cf_mea       <- gpu_contrafold/cpu.py:823-895,932-941  mea_decode/mea
 *   cf_mfe       <- gpu_contrafold/cpu.py:290-519   viterbi/mfe
 *   cf_sample    <- gpu_contrafold/gpu.py:196-477,520-583  sample_kernel/sample_batch
 *
 * Conventions shared by every entry point
 * ---------------------------------------
 * - A batch of n sequences is one byte buffer `seqs` (ASCII, any case; A C G U,
 *   T == U, any other byte is the unknown base N which never pairs and scores 0)
 *   plus `offsets[n+1]` (int64, offsets[0] == 0, sequence b is
 *   seqs[offsets[b] .. offsets[b+1])).
 * - `mask` is NULL (no constraint) or a byte buffer laid out like `seqs`:
 *   mask[offsets[b] + t] != 0 forces position t (0-based) of sequence b unpaired.
 * - Per-sequence string outputs (dot-brackets) use the same offsets: sequence b
 *   writes exactly L_b bytes '(' ')' '.' at out[offsets[b]]; no terminator.
 * - Every call returns a status (CF_OK == 0).  On failure cf_last_error()
 *   returns a thread-local, human-readable message.
 * - Host-buffer calls are synchronous.  One engine must not be used from two
 *   threads at once (one engine per host thread / stream).
 */
#ifndef CONTRAFOLD_GB300_H
#define CONTRAFOLD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define CF_OK        0
#define CF_EINVAL    1   /* bad argument (NULL pointer, bad length, bad gamma ...) */
#define CF_ENOMEM    2   /* device allocation failed or over the engine's memory budget */
#define CF_ETIMEOUT  3   /* a bounded device-side wait expired; the context stays usable */
#define CF_ECUDA     4   /* CUDA runtime error */
#define CF_EDEVICE   5   /* a kernel reported an internal limit (e.g. traceback stack) */

/* Longest sequence accepted (partner indices are stored as int16 in the
 * reference's sampler, gpu.py:559; the same bound is kept). */
#define CF_MAX_LEN 32767

/* ---- parameter blob layout (entries, float32 or float64) ----
 * The blob is the concatenation of the tied tables produced by the loader
 * (gpu_contrafold/cpu.py:40-135), each flattened in C order:
 *   bp[5][5] stack[5][5][5][5] tm[5][5][5][5] hc[5][5] dl[5][5][5] dr[5][5][5]
 *   hp_cum[31] cs[31][31] i11[5][5] b01[5] mb mu mp eu ep                        */
#define CF_OFF_BP      0
#define CF_OFF_STACK   25
#define CF_OFF_TM      650
#define CF_OFF_HC      1275
#define CF_OFF_DL      1300
#define CF_OFF_DR      1425
#define CF_OFF_HPCUM   1550
#define CF_OFF_CS      1581
#define CF_OFF_I11     2542
#define CF_OFF_B01     2567
#define CF_OFF_MB      2572
#define CF_OFF_MU      2573
#define CF_OFF_MP      2574
#define CF_OFF_EU      2575
#define CF_OFF_EP      2576
#define CF_BLOB_LEN    2577

typedef struct cf_engine cf_engine;

/* Create an engine on CUDA device `device` from the float32 and float64 blobs
 * (both CF_BLOB_LEN entries).  The float32 blob drives every FP32 path; the
 * float64 blob drives cf_logz64 and cf_mfe (the reference computes those in
 * float64).  Replaces the per-call parameter upload of gpu.py:500-514. */
int cf_engine_create(const float* params32, const double* params64, int device,
                     cf_engine** out);
int cf_engine_destroy(cf_engine* eng);
/* Replace the parameter tables of an existing engine (e.g. after a gradient step). */
int cf_engine_set_params(cf_engine* eng, const float* params32, const double* params64);
/* Upper bound, in bytes, on the device work arena (0 = unlimited).  Batches
 * larger than the budget are processed in slices; a single sequence that does
 * not fit returns CF_ENOMEM. */
int cf_engine_set_budget(cf_engine* eng, size_t bytes);
/* Select the scheduling of the fold kernels: 0 = plain (one CTA per
 * sequence, threads over the cells of each span, whole-window scans: the
 * reference's gpu.py:55-184 launch shape), 1 = batched (persistent kernels
 * and length-grouped kernels chosen per length range, see
 * cf_engine_set_schedule).  Results are identical. */
int cf_engine_set_mode(cf_engine* eng, int mode);
/* Batched-path schedule (the tuner's knob): kind 0 = automatic by length,
 * 1 = persistent warp-per-sequence kernel, 2 = persistent CTA-per-sequence
 * fused kernel, 3 = length-grouped per-phase kernels, 4 = cluster: each
 * sequence (or group, cf_engine_set_group) folded by the 8 CTAs of a
 * thread-block cluster on 8 SMs -- the latency of long sequences, for logZ,
 * BPP, MEA and sampling (kind 0 follows the schedule table,
 * cf_engine_load_tuning); ctas_per_sm caps the residency of the persistent
 * CTA kernels (0 = automatic).  Results are identical for every choice.
 * Kind 5 (the queue schedule, cf_queue.cu) is disabled and returns
 * CF_EINVAL: its kernel did not finish in two GPU test runs. */
int cf_engine_set_schedule(cf_engine* eng, int kind, int ctas_per_sm);
/* Scheduling priority of the engine's calls: 0 = the device's default
 * (lowest) stream priority, nonzero = its highest.  As SMs free up, pending
 * blocks of higher-priority streams are placed first (running blocks are not
 * preempted).  The serving loop folds short requests at high priority so that
 * batches of long sequences on other engines cannot hold them back.  Waits
 * for the engine's earlier work when the priority changes.  No reference
 * counterpart. */
int cf_engine_set_priority(cf_engine* eng, int high);
/* on != 0: the device runs other engines' launches at the same time (the
 * serving loop's workers).  The engine then launches no 512-thread CTAs and
 * no thread-block clusters (the cluster schedule folds grouped instead):
 * such a launch waits until a whole SM, or 8 SMs of one GPC, have room at
 * once, and between other engines' steady launches of smaller CTAs that took
 * seconds.  Results are identical.  No reference counterpart. */
int cf_engine_set_shared(cf_engine* eng, int on);
/* Sequences per CTA of the length-grouped kernels (schedule kind 3): 1..32
 * (larger values are accepted and capped); 0 = automatic.  The tuner's knob;
 * results are identical for every value. */
int cf_engine_set_group(cf_engine* eng, int group);
/* Schedule table of the automatic batched path (schedule kind 0), written by
 * the tuner (python -m contrafold_gpu_gb300.autotune --write-table FILE).
 * One row per line, '#' starts a comment:
 *   min_len max_len min_batch max_batch uniform jobs schedule group ctas_per_sm
 * A batch matches a row when its shortest sequence has >= min_len nt, its
 * longest <= max_len, its size is in [min_batch, max_batch] (max_batch 0 = no
 * limit), its lengths are all within 25 % of each other (uniform = "uniform"),
 * or not ("mixed"), or either ("any"), and its job is in `jobs` ("all" or a
 * comma list of logz, logz64, bpp, mea, mfe, sample).  The first matching row
 * gives the schedule (warp, cta, group or cluster), the sequences per CTA of
 * the grouped kernels, and the CTAs per SM of the CTA kernels (0 =
 * automatic);
 * a batch no row matches folds grouped.  path NULL restores the built-in
 * table; cf_engine_create loads the file named by the environment variable
 * CONTRAFOLD_GB300_TUNING when it is set.  A malformed file is CF_EINVAL and
 * leaves the table unchanged.  No reference counterpart (the reference has
 * one launch shape).  Results are identical for every table. */
int cf_engine_load_tuning(cf_engine* eng, const char* path);
/* Rows of the engine's schedule table. */
int cf_engine_tuning_rows(const cf_engine* eng);

const char* cf_last_error(void);
const char* cf_version(void);

/* log partition function in FP32 (the recurrence of gpu.py:55-184) with an
 * accurate float32 log-sum-exp (log1pf/expf), within 5e-4 of the FP64 engine.
 * The reference's Fast_LogPlusEquals value (bitwise that of cpu.py:595-678)
 * is what cf_bpp returns in logz_out.  logz_out[n]. */
int cf_logz(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
            const uint8_t* mask, int32_t n, float* logz_out);

/* log partition function, FP64 with exact log1p/exp (cpu.py:154-275). */
int cf_logz64(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
              const uint8_t* mask, int32_t n, double* logz_out);

/* Base-pair posterior matrices (cpu.py:583-820), bitwise the reference's
 * float32 posterior.  Sequence b writes L_b*L_b float32 values (row-major,
 * 0-based, upper triangle; diagonal and lower triangle are 0) at
 * post_out[post_offsets[b]].  logz_out (may be NULL) receives the
 * Fast_LogPlusEquals logZ the posterior is normalised by. */
int cf_bpp(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
           const uint8_t* mask, int32_t n, const int64_t* post_offsets,
           float* post_out, float* logz_out);

/* Maximum-expected-accuracy structures (cpu.py:823-895): inside, outside,
 * posterior and the gamma-weighted decode, all on the device. */
int cf_mea(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
           const uint8_t* mask, int32_t n, float gamma, char* struct_out);

/* Viterbi (maximum-probability) structures with the reference's first-match
 * EPS=1e-6 traceback (cpu.py:290-519), in float64. */
int cf_mfe(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
           const uint8_t* mask, int32_t n, char* struct_out);

/* Boltzmann samples (stochastic traceback, gpu.py:196-477) with Philox4x32-10
 * streams keyed by (seed, sequence index, sample index).  Sequence b writes
 * n_samples * L_b bytes at out[offsets[b] * n_samples] (sample-major). */
int cf_sample(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
              const uint8_t* mask, int32_t n, int32_t n_samples, uint64_t seed,
              char* out);

/* cf_sample with one seed per sequence (no reference counterpart; the serving
 * loop uses it): sequence b draws exactly the samples that cf_sample gives for
 * it alone (n = 1) with seed seeds[b], whatever batch it is folded in. */
int cf_sample_seeded(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
                     const uint8_t* mask, int32_t n, int32_t n_samples,
                     const uint64_t* seeds, char* out);

/* One Boltzmann sample per task, drawn exactly as the reference's pipeline
 * primitive fold_tasks_gpu(seqs, masks, P, chunk, seed) draws them
 * (gpu_contrafold/gpu.py:586-601): the tasks ordered by length (a stable
 * sort), cut into chunks of `chunk`, chunk c0 sampled with seed + c0 and its
 * k-th task with sequence index k -- the samples that cf_sample gives for
 * each chunk -- but every task folded in one submission (the batched fold
 * and sampler kernels over all tasks, each task's Philox key and sequence
 * index given per task).  Task b writes L_b bytes at out[offsets[b]]. */
int cf_sample_tasks(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
                    const uint8_t* mask, int32_t n, int32_t chunk, uint64_t seed,
                    char* out);

/* Differentiation of logZ (no reference counterpart: the reference has no
 * gradient).  With an optional soft per-position unpaired bonus `bonus`
 * (float32, laid out like `seqs`; NULL = 0) added to the score of every
 * unpaired position, returns per sequence b:
 *   logz_out[b]                          logZ (accurate float32 log-sum-exp)
 *   counts_out[b*CF_BLOB_LEN + e]        d logZ / d(parameter-blob entry e) =
 *                                        expected uses of entry e (exact sums)
 *   unpaired_out[offsets[b] + t]         d logZ / d bonus_t = P(t unpaired)
 * The raw-feature gradient is counts_out times the tying Jacobian of the
 * loader (linear, gpu_contrafold/cpu.py:40-135). */
int cf_grad(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
            const uint8_t* mask, int32_t n, const float* bonus, float* logz_out,
            double* counts_out, double* unpaired_out);
/* Memory of cf_grad (no reference counterpart).  The inside tables FC, FM,
 * FM1 and the outside FM2o stay whole; FCo, FMo, FM1o live in ring buffers of
 * a few diagonals (the expected counts are taken one diagonal behind the
 * outside pass); the inside FM2 is kept on every `every`-th diagonal and
 * recomputed on the others (every = 1: all kept; 0: automatic -- 1 below
 * 512 nt, else 8).  The counts are summed in exact 128-bit fixed point, so
 * the results are bitwise the same for every spacing and every run. */
int cf_engine_set_grad_checkpoint(cf_engine* eng, int32_t every);
/* Device bytes cf_grad uses per sequence of L nt at checkpoint spacing
 * `every` (0: automatic); 0 for a bad length. */
size_t cf_grad_arena_bytes(int32_t L, int32_t every);

/* ---- plans: device-resident batches ----
 * A plan fixes a batch's shape (lengths from host `offsets`), orders and
 * groups its sequences, and owns the device descriptors and a work arena sized
 * for it.  cf_plan_run then only launches kernels: `d_seqs`, `d_mask` (NULL =
 * no constraint) and `d_out` are device pointers laid out like the host
 * buffers of the calls above, and the launches are asynchronous on `stream`
 * (a cudaStream_t; NULL selects the engine's stream).  `d_out` is float[n]
 * for CF_JOB_LOGZ, double[n] for CF_JOB_LOGZ64, the dot-bracket buffer
 * for CF_JOB_MEA / CF_JOB_MFE, and for CF_JOB_BPP the posterior matrices
 * packed back to back: sequence b's L_b x L_b float32 matrix (as cf_bpp) at
 * float offset sum_{c<b} L_c^2.  No reference counterpart: the reference
 * re-uploads everything per call (gpu.py:500-514). */
#define CF_JOB_LOGZ   0
#define CF_JOB_LOGZ64 1
#define CF_JOB_BPP    2
#define CF_JOB_MEA    3
#define CF_JOB_MFE    4
typedef struct cf_plan cf_plan;
int cf_plan_create(cf_engine* eng, int32_t job, const int64_t* offsets, int32_t n,
                   cf_plan** out);
int cf_plan_destroy(cf_plan* plan);
size_t cf_plan_arena_bytes(const cf_plan* plan);
int cf_plan_run(cf_plan* plan, const uint8_t* d_seqs, const uint8_t* d_mask, float gamma,
                void* d_out, void* stream);
/* Synchronises the device and returns the device-side status of past runs. */
int cf_plan_status(cf_plan* plan);
/* Per-phase CUDA-event timing of each run (0 inside, 1 outside, 2 posterior,
 * 3 decode); cf_plan_phase_ms waits for the last run and returns milliseconds. */
int cf_plan_set_timing(cf_plan* plan, int on);
int cf_plan_phase_ms(cf_plan* plan, float* ms, int32_t nphases);
/* Kernels launched by the last cf_plan_run; sequences per CTA of the plan. */
int cf_plan_launches(const cf_plan* plan);
/* CUDA graph replay (no reference counterpart): with on != 0, cf_plan_run
 * records the plan's launches into a CUDA graph by stream capture the first
 * time it sees a (d_seqs, d_mask, gamma, d_out) combination, and afterwards
 * launches that graph -- one launch call for all the plan's kernels and
 * memsets.  New arguments re-capture.  Ignored while phase timing is on. */
int cf_plan_set_graph(cf_plan* plan, int on);
/* The plan's schedule: "plain", "warp", "cta", "group" or "cluster" (static
 * string).  A
 * grouped MEA / BPP plan runs all phases in one launch (k_fold_group32) unless
 * phase timing is on, which runs the per-phase kernels. */
const char* cf_plan_schedule(const cf_plan* plan);
int cf_plan_group(const cf_plan* plan);

/* ---- serving loop: continuous batching of single-sequence requests ----
 * No reference counterpart (the reference folds caller-made batches only).
 * A server owns n_workers engines (each with its own stream and arena) and as
 * many worker threads.  Requests queue by (op, gamma / n_samples, length
 * bucket); a free worker takes the queue with the oldest request, folds up to
 * max_batch requests / max_batch_nt nucleotides of it as one batch and
 * publishes the results.  A request's result equals the same request folded
 * alone: logZ (cf_logz), MEA (cf_mea) and samples (cf_sample_seeded with the
 * request's seed). */
#define CF_ECANCELLED 6   /* serving: the request was cancelled or the server stopped */
#define CF_OP_LOGZ   0
#define CF_OP_MEA    1
#define CF_OP_SAMPLE 2
typedef struct cf_request {
    int32_t op;          /* CF_OP_* */
    int32_t n_samples;   /* CF_OP_SAMPLE: samples to draw */
    float gamma;         /* CF_OP_MEA: gamma > 0 */
    int32_t reserved;
    uint64_t seed;       /* CF_OP_SAMPLE: Philox key of this request */
} cf_request;
typedef struct cf_server cf_server;
int cf_server_create(const float* params32, const double* params64, int device,
                     int32_t n_workers, cf_server** out);
/* Joins the workers (running batches finish) and frees everything; no call on
 * the server may be in progress or follow. */
int cf_server_destroy(cf_server* server);
/* Batch limits and length-bucket upper edges (nt, increasing).  Buckets whose
 * upper edge is above long_len are long: only workers [0, long_workers) take
 * them (and take short batches when no long request waits), so the other
 * workers always serve short requests.  Only while no request is queued. */
int cf_server_configure(cf_server* server, int32_t max_batch, int64_t max_batch_nt,
                        int32_t long_len, int32_t long_workers, const int32_t* edges,
                        int32_t n_edges);
/* Batch limits by cost: a worker stops adding requests (oldest first) to a
 * batch when the sum of L^3 over its requests -- the predicted work, the fold
 * being cubic in the length -- would pass max_batch_cost, or the device arena
 * the batch needs (the FP32 fold arena per MEA request, its inside part per
 * logZ / sampling request) would pass max_batch_arena_bytes; 0 = no limit.
 * The first request of a batch is always taken.  Any time. */
int cf_server_set_limits(cf_server* server, double max_batch_cost, int64_t max_batch_arena_bytes);
/* While paused, workers start no new batch (requests keep queueing). */
int cf_server_pause(cf_server* server, int32_t on);
/* Copies the sequence (and mask: NULL or len bytes, != 0 forces unpaired). */
int cf_server_submit(cf_server* server, const cf_request* req, const uint8_t* seq,
                     int32_t len, const uint8_t* mask, int64_t* ticket);
/* Blocks until the request is done (timeout_ms < 0: no limit; on expiry
 * CF_ETIMEOUT and the request stays), then returns its status and outputs and
 * forgets the ticket: logZ in *logz_out, or the dot-bracket (L bytes) or the
 * samples (n_samples * L bytes, sample-major) in out[0 .. out_cap).  Of
 * several threads waiting on one ticket, one gets the outputs, the others
 * CF_EINVAL. */
int cf_server_wait(cf_server* server, int64_t ticket, int32_t timeout_ms,
                   float* logz_out, char* out, int64_t out_cap);
/* A request still queued is dropped; its wait returns CF_ECANCELLED. */
int cf_server_cancel(cf_server* server, int64_t ticket);
/* Open-loop replay: request k is submitted t_arrive[k] seconds after the call
 * starts (non-decreasing), whatever the server's progress; the call returns
 * when all are done.  Sequences and masks are laid out as in cf_logz; outputs
 * go to logz_out[k] (logZ) or out[out_offsets[k] ..] (MEA: L bytes, samples:
 * n_samples * L bytes); latency_ms[k] = completion - scheduled arrival;
 * status_out[k] = the request's status.  If a submission fails (e.g. the
 * server is stopping), the requests already submitted are still collected,
 * the rest get status CF_ECANCELLED, and the call returns the submission's
 * error. */
int cf_server_replay(cf_server* server, int32_t n, const double* t_arrive,
                     const cf_request* reqs, const uint8_t* seqs, const int64_t* offsets,
                     const uint8_t* mask, const int64_t* out_offsets, float* logz_out,
                     char* out, double* latency_ms, int32_t* status_out);
/* stats[0..9] = batches, requests done, nucleotides done, cancelled,
 * summed batch seconds over workers, requests queued now, summed and maximum
 * queue wait (submit to batch start, seconds) over done requests, summed and
 * maximum batch run time seen by a request (seconds). */
int cf_server_stats(cf_server* server, double* stats, int32_t n_stats);

/* ---- MEA without device allocation ----
 * No reference counterpart: the reference allocates its device buffers with
 * Numba on every call.  Same arguments, results and argument errors as cf_mea,
 * but the call allocates no device memory: inputs, descriptors, outputs and the
 * fold arenas live in one static device array of CF_SCRATCH_BYTES, reserved by
 * the CUDA driver when the library's module is loaded.  For callers that cannot let
 * a library allocate while they run (a framework allocator has reserved the
 * device; cudaFree would stall a serving loop's other streams).
 * - Batches whose inputs, outputs and 8 fold slots for the longest sequence do
 *   not fit (longest sequence above ~740 nt, or too many nucleotides) are
 *   rejected with CF_EINVAL and a message giving the bytes needed.
 * - The first call on a device does set-up (resolves the array's address);
 *   make it before any stream capture begins.
 * - The status word and work-queue head must be zero at launch: the call
 *   clears them itself.  Calls share the array, so overlapping calls would
 *   race; the library serialises them with a process-wide lock and each call
 *   returns only after its work has finished.  Synchronous, engine's stream. */
#define CF_SCRATCH_BYTES (64u * 1024u * 1024u)
int cf_mea_scratch(cf_engine* eng, const uint8_t* seqs, const int64_t* offsets,
                   const uint8_t* mask, int32_t n, float gamma, char* struct_out);

#ifdef __cplusplus
}
#endif
#endif /* CONTRAFOLD_GB300_H */
