// ranker.h -- the learned candidate ranker: a 12 -> 64 -> 64 -> 1 MLP over
// per-candidate seed features that prunes hopeless candidates before the
// seeded DP. No counterpart in the reference; it is trained on labels the
// plain path produces (see ranker.cu).
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

constexpr int RK_F = RANK_FEATURES;  // features per candidate
constexpr int RK_H = 64;  // hidden width
// fp32 master parameters: W1[64][12], b1[64], W2[64][64] (row n, column k), b2[64], w3[64], b3
constexpr int RK_W1 = 0, RK_B1 = RK_W1 + RK_H * RK_F, RK_W2 = RK_B1 + RK_H, RK_B2 = RK_W2 + RK_H * RK_H,
              RK_W3 = RK_B2 + RK_H, RK_B3 = RK_W3 + RK_H, RK_P = RK_B3 + 1;
// bf16 copies for the tensor-core layers, as 32-bit pairs along k:
// W1b[64][16] (k padded with zeros) then W2b[64][64]
constexpr int RK_WB_WORDS = (RK_H * 16 + RK_H * RK_H) / 2;
// label of a candidate slot that was not aligned (excluded from training)
constexpr uint8_t RK_IGNORE = 255;


// Mate-consistency features of read set A against read set B (same pairs).
struct RankMateArgs {
  const Cand* cand_a;
  const uint32_t* n_cand_a;
  const uint64_t* offs_a;
  const Cand* cand_b;
  const uint32_t* n_cand_b;
  const uint64_t* offs_b;
  uint32_t r0, nr;
  double mean, sd;                 // insert-size model at the start of the chunk
  float* feat_a;
};

struct RankModelDev {
  const float* norm;               // mean[12], 1/std[12]
  const uint32_t* wb;              // RK_WB_WORDS bf16 pairs
  const float* w;                  // RK_P fp32 parameters (biases and w3 used as fp32)
};

// Keep flags into Cand::pad[0] from the logits of a chunk's slots.
struct RankDecideArgs {
  const float* logit;
  const float* feat;
  Cand* cand;
  const uint32_t* n_cand;
  uint32_t nr;
  float tau;                       // keep a candidate whose logit >= tau
  unsigned long long* counters;    // kept, pruned, reads kept whole
};

// Training labels from the plain path's seeded alignments (thread per read).
struct RankLabelArgs {
  const AlnOut* aln;               // nr * MAX_CAND
  const uint32_t* n_cand;
  uint32_t nr;
  uint8_t* label;                  // nr * MAX_CAND
  double cut;                      // positive when lk - lk_max >= cut (log units)
};

void launch_rank_mate(const RankMateArgs& a, cudaStream_t st);
void launch_rank_infer(const float* feat, uint64_t n_slots, const RankModelDev& m, float* logit, int grid,
                       cudaStream_t st);
void launch_rank_decide(const RankDecideArgs& a, cudaStream_t st);
void launch_rank_label(const RankLabelArgs& a, cudaStream_t st);

// Training over n samples (dense features and 0/1 labels).
void launch_rank_stats(const float* feat, uint64_t n, double* acc, cudaStream_t st);  // acc: sum[12], sumsq[12]
void launch_rank_train_step(const float* feat, const uint8_t* label, uint64_t n, uint64_t first, uint32_t count,
                            uint64_t stride_mul, const float* norm, const float* w, float* grad, double w_pos,
                            double w_neg, float* loss_acc, cudaStream_t st);
void launch_rank_adam(float* w, float* grad, float* m, float* v, uint32_t* wb, int step, float lr,
                      cudaStream_t st);
void launch_rank_pack(const float* w, uint32_t* wb, cudaStream_t st);
size_t rank_train_smem();

}  // namespace pbw
