// cf_sample.h -- stochastic-traceback sampler launch interface.
#pragma once

#include <cstddef>
#include <cstdint>

#include "cf_device.cuh"

namespace cf {

struct SampleArgs {
    const SeqDesc* descs;   // [n], ws_off points at each sequence's inside tables
    int n;
    int n_samples;
    int Lmax;
    uint64_t seed;
    const uint64_t* seeds;  // null, or one seed per batch index: sequence b then samples with key
                            // seeds[b] and sequence index 0, exactly as if it were folded alone
    const int32_t* stream_idx;   // null, or per batch index: the sequence index of its Philox draws
    const uint8_t* seqs;
    const uint8_t* mask;
    const float* blob32;
    float* ws;
    char* out;              // sequence b, sample s at out[seq_off * n_samples + s * L]
    int* status;
};

__global__ void k_sample32(SampleArgs A);
size_t sample_smem_bytes(int Lmax);
int sample_threads();

}  // namespace cf
