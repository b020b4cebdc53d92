// cf_queue.h -- launch interface of the dataflow schedule (cf_queue.cu): one
// persistent launch, warps pulling (sequence, step, chunk) work items.
#pragma once

#include <cstddef>
#include <cstdint>

#include "cf_device.cuh"

namespace cf {

constexpr int kQueueThreads = 256;   // 8 warps per CTA
#ifndef CF_QUEUE_MIN_BLOCKS
#define CF_QUEUE_MIN_BLOCKS 3
#endif
constexpr int kQueueMinBlocks = CF_QUEUE_MIN_BLOCKS;
constexpr int kQueueMaxSeats = 64;

enum { kQueueLogZ = 0, kQueueMea = 1, kQueueBpp = 2, kQueueSample = 3 };

struct QueueArgs {
    const SeqDesc* descs;      // [n], longest first (the queue's order); ws_off unused
    int n;
    int Lmax;                  // longest sequence: sizes the seats' codes and arena slots
    int seats;                 // sequences in progress per CTA (1 .. kQueueMaxSeats)
    const uint8_t* seqs;
    const uint8_t* mask;       // nullable
    const float* blob32;
    float* ws;                 // arena: slot_words per seat, grid x seats slots
    int64_t slot_words;
    int* counter;              // global sequence-queue head, zero before the launch
    float gamma;
    float* logz;               // [batch] or null
    char* structs;             // MEA dot-brackets at seq_off
    float* post_out;           // BPP dense matrices
    const int64_t* post_offs;
    int n_samples;
    uint64_t seed;
    const uint64_t* seeds;       // null, or per batch index (the sequence's own Philox key)
    const int32_t* stream_idx;   // null, or per batch index: the Philox sequence index of its draws
    char* out;                   // samples at seq_off * n_samples
    int* status;
};

size_t queue_smem_bytes(int Lmax, int seats, int mode);
int64_t queue_slot_words(int Lmax);
const void* queue_kernel(int mode);

}  // namespace cf
