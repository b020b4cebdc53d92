// cf_kernels.h -- kernel entry points and launch arguments (host + device).
#pragma once

#include <cstddef>
#include <cstdint>

#include "cf_device.cuh"

namespace cf {

constexpr int kFoldThreads = 256;       // threads per fold CTA
#ifndef CF_FOLD_MIN_BLOCKS
#define CF_FOLD_MIN_BLOCKS 3
#endif
constexpr int kFoldMinBlocks = CF_FOLD_MIN_BLOCKS;   // resident CTAs per SM the register budget targets
// ... and for the fused grouped MEA kernel alone (GB300, 10,000 x 200 nt MEA:
// 3 -> 31.9k, 4 -> 33.2k folds/s, 40-400 nt 14.4k -> 16.3k; 4 slowed the
// per-phase kernels, the fused BPP kernel and the sampler's inside 1.5-2.5x)
#ifndef CF_FOLD_MIN_BLOCKS_MEA
#define CF_FOLD_MIN_BLOCKS_MEA 4
#endif
constexpr int kFoldMinBlocksMea = CF_FOLD_MIN_BLOCKS_MEA;
constexpr int kFoldThreadsWide = 512;   // per-phase fold CTA when the grid has at most one CTA per SM:
                                        // a long sequence's diagonal spreads over twice the threads
constexpr int kMaxGroup = 32;       // sequences per CTA on the batched path

struct FoldArgs {
    const SeqDesc* descs;      // [n], grouped: CTA b owns descs[b*group .. b*group+group)
    int n;
    int group;
    const uint8_t* seqs;       // ASCII
    const uint8_t* mask;       // nullable
    const float* blob32;
    const double* blob64;
    float* ws;                 // arena base
    float* logz;               // [batch] or null
    double* logz64;            // [batch] or null
    char* structs;             // dot-brackets at seq_off
    float* post_out;           // dense L*L per sequence or null
    const int64_t* post_offs;  // indexed by SeqDesc::idx
    float gamma;
    int* status;               // device status word (CF_OK or an error code)
};

// FP32 per-phase kernels (k_inside32, k_inside32acc, k_outside32,
// k_posterior32, k_mea32), instantiated for kFoldThreads and kFoldThreadsWide
// threads per CTA in cf_fold.cu and reached through fold_kernels().
using FoldKernel = void (*)(FoldArgs);
struct FoldKernels {
    FoldKernel inside, inside_acc, outside, posterior, mea;
    FoldKernel fused_mea, fused_bpp;   // k_fold_group32: all phases of MEA / BPP in one launch
    FoldKernel fused_mea_shared;       // fused MEA at the other kernels' register budget (shared device)
};
FoldKernels fold_kernels(bool wide);
// k_fold_cluster32: one group folded by the kClusterCtas CTAs of a cluster
// (grid = groups x kClusterCtas, kFoldThreads per CTA)
constexpr int kClusterCtas = 8;
#ifndef CF_CLUSTER_CHAIN_PF
#define CF_CLUSTER_CHAIN_PF 8   // bifurcation-chain pipeline depth in the cluster kernels
#endif
#ifndef CF_CLUSTER_MIN_BLOCKS
#define CF_CLUSTER_MIN_BLOCKS 2   // resident CTAs per SM the cluster kernels' registers target
#endif
constexpr int kClusterMinBlocks = CF_CLUSTER_MIN_BLOCKS;
struct ClusterKernels {
    FoldKernel mea, bpp, inside_acc;
};
ClusterKernels cluster_kernels();
__global__ void k_inside64(FoldArgs A);
__global__ void k_viterbi64(FoldArgs A);

size_t fold_smem_bytes(int Lmax, int group, bool fp64);

// Plain path: the reference's launch shape (cf_plain.cu), one sequence per CTA.
__global__ void k_plain_inside32(FoldArgs A);
__global__ void k_plain_outside32(FoldArgs A);
__global__ void k_plain_posterior32(FoldArgs A);
__global__ void k_plain_mea32(FoldArgs A);
size_t plain_smem_bytes(int Lmax);

// Adjoint (cf_adjoint.cu): inside with a soft unpaired bonus (FM2 kept on
// every ckpt-th diagonal), then the outside with the expected counts folded in.
__global__ void k_adj_inside(FoldArgs A, const float* bonus, int ckpt);
__global__ void k_adj_outside(FoldArgs A, const float* bonus, int ckpt, double* counts_out, double* unpaired_out);
size_t adj_smem_bytes(int Lmax);
int64_t adj_arena_words(int L, int ckpt);
int adj_auto_checkpoint(int L);

// Persistent fused per-sequence kernel (one CTA per sequence at a time).
enum { kCtaLogZ = 0, kCtaMea = 1, kCtaBpp = 2 };
template <int MODE>
__global__ void k_fold_cta(FoldArgs A, int* counter, int64_t slot_words);
const void* cta_kernel(int mode);

}  // namespace cf
