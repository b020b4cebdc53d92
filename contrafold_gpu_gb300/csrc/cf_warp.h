// cf_warp.h -- launch interface of the persistent warp-per-sequence kernel.
#pragma once

#include <cstddef>
#include <cstdint>

#include "cf_device.cuh"

namespace cf {

constexpr int kWarpThreads = 256;     // 8 warps per CTA
constexpr int kWarpMaxLen = 1024;     // longer sequences take the per-sequence CTA kernels

enum { kWarpLogZ = 0, kWarpMea = 1, kWarpBpp = 2, kWarpSample = 3 };

struct WarpArgs {
    const SeqDesc* descs;      // [n], longest first; ws_off unused (arena slots are per warp)
    int n;
    int Lmax;
    const uint8_t* seqs;
    const uint8_t* mask;       // nullable
    const float* blob32;
    float* ws;                 // arena: one slot of slot_words per warp of the grid
    int64_t slot_words;
    int* counter;              // work-queue head, zero before the launch
    float gamma;
    float* logz;               // [batch] or null
    char* structs;             // MEA dot-brackets at seq_off
    float* post_out;           // BPP dense matrices
    const int64_t* post_offs;
    int n_samples;
    uint64_t seed;
    const uint64_t* seeds;     // null, or per batch index (see SampleArgs::seeds)
    const int32_t* stream_idx; // null, or per batch index (see SampleArgs::stream_idx)
    char* out;                 // samples at seq_off * n_samples
    int* status;
};

size_t warp_smem_bytes(int Lmax);
int64_t warp_slot_words(int Lmax);
const void* warp_kernel(int mode);

}  // namespace cf
