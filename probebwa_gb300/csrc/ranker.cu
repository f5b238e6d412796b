// ranker.cu -- the learned candidate ranker (no counterpart in the
// reference): per-candidate seed features, a 12 -> 64 -> 64 -> 1 MLP with
// BF16 weights and FP32 accumulation on the tensor cores (mma.sync
// m16n8k16), and the kernels that train it on labels the plain path
// produces.
//
// Features of candidate i of a read (the first 20 clusters of
// candidates.rs:30-78, the ones map_candidates aligns, single.rs:114):
//   0 log2(1 + exact seed hits)          1 log2(1 + one-mismatch hits)
//   2 log2(1 + distinct diagonals)        3 log2(1 + diagonal spread)
//   4 log2(1 + read span of the hits)     5 read length
//   6 mean base quality of the read       7 mate distance z-score (pairs)
//   8 opposite-strand mate candidate on the same contig (pairs)
//   9 rank i in the candidate list       10 candidate list size
//  11 mean log2 exact bucket size of the hits' windows (repeat multiplicity)
// The clustering kernel (cluster.cu, binned form) computes features 0-6 and
// 9-11 from its per-bin sums; 7-8 come from the other mate's candidates
// (k_rank_mate). A read whose hits went to the overflow pool has no
// hit-level features (feature 0 = -1): its candidates are all kept.
//
// Label (plain path): the candidate was aligned and either is the read's
// select_best winner (the last maximum, bayesian.rs:193-201) or has
// lk - lk_max >= cut. With the default cut, -60 ln 2 (exp >= 2^-60), terms
// below it cannot change the FP64 sum_exp (at most 19 of them add less than
// half an ulp of the winner's 1.0), so pruning only such candidates leaves
// select_best, sum_exp and finalize_mapq unchanged; a looser cut (e.g.
// ln 1e-12) labels fewer candidates positive, and pruned terms can then move
// the posterior's last bits and, rarely, a MAPQ.
//
// Inference: one warp per tile of 16 candidate slots. Layer 1 is one
// m16n8k16 per 8 hidden units (features padded to k = 16), layer 2 four
// k-steps per 8 hidden units with the layer-1 accumulators repacked in
// registers as the A operand, layer 3 a dot product over the accumulator
// fragments reduced across the quad. Training runs the same arithmetic
// (inputs, weights and layer-1 activations rounded to BF16, FP32 sums) on
// the CUDA cores, one sample per thread, gradients per block in shared
// memory, then Adam on FP32 master weights and a repack of the BF16 copies.
#include <cuda_bf16.h>

#include "ranker.h"

namespace pbw {

namespace {

__device__ __forceinline__ float bf16r(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Thread per candidate slot of read set A.
__global__ void k_rank_mate(RankMateArgs a) {
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (uint64_t)a.nr * MAX_CAND) return;
  const uint32_t r = (uint32_t)(t / MAX_CAND), i = (uint32_t)(t % MAX_CAND);
  if (i >= a.n_cand_a[r]) return;
  float* f = a.feat_a + t * RK_F;
  if (f[0] < 0.f) return;
  const Cand ca = a.cand_a[t];
  const uint64_t rg = (uint64_t)a.r0 + r;
  const long long la = (long long)(a.offs_a[rg + 1] - a.offs_a[rg]);
  const long long lb = (long long)(a.offs_b[rg + 1] - a.offs_b[rg]);
  const uint32_t nb = a.n_cand_b[r];
  double best = 10.0;
  float agree = 0.f;
  for (uint32_t j = 0; j < nb; j++) {
    const Cand cb = a.cand_b[(size_t)r * MAX_CAND + j];
    if (cb.contig != ca.contig || cb.strand == ca.strand) continue;
    agree = 1.f;
    // forward anchor: the mate ends downstream; reverse anchor: upstream
    const long long ins = ca.strand == 0 ? (long long)cb.pos + lb - (long long)ca.pos
                                         : (long long)ca.pos + la - (long long)cb.pos;
    const double z = fabs((double)ins - a.mean) / a.sd;
    best = z < best ? z : best;
  }
  f[7] = (float)best;
  f[8] = agree;
}

__global__ void __launch_bounds__(128) k_rank_infer(const float* feat, uint64_t n_slots, RankModelDev m,
                                                    float* logit) {
  __shared__ uint32_t s_wb[RK_WB_WORDS];
  __shared__ float s_b1[RK_H], s_b2[RK_H], s_w3[RK_H], s_norm[2 * RK_F];
  __shared__ float s_b3;
  for (int k = threadIdx.x; k < RK_WB_WORDS; k += blockDim.x) s_wb[k] = m.wb[k];
  for (int k = threadIdx.x; k < RK_H; k += blockDim.x) {
    s_b1[k] = m.w[RK_B1 + k];
    s_b2[k] = m.w[RK_B2 + k];
    s_w3[k] = m.w[RK_W3 + k];
  }
  if (threadIdx.x < 2 * RK_F) s_norm[threadIdx.x] = m.norm[threadIdx.x];
  if (threadIdx.x == 0) s_b3 = m.w[RK_B3];
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
  const uint64_t tiles = (n_slots + 15) / 16;
  const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
  auto x = [&](uint64_t row, int k) -> float {
    if (row >= n_slots || k >= RK_F) return 0.f;
    return (feat[row * RK_F + k] - s_norm[k]) * s_norm[RK_F + k];
  };
  for (uint64_t tile = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; tile < tiles; tile += nw) {
    const uint64_t row0 = tile * 16 + g, row1 = row0 + 8;
    uint32_t a1[4];
    a1[0] = pack_bf16(x(row0, 2 * q), x(row0, 2 * q + 1));
    a1[1] = pack_bf16(x(row1, 2 * q), x(row1, 2 * q + 1));
    a1[2] = pack_bf16(x(row0, 2 * q + 8), x(row0, 2 * q + 9));
    a1[3] = pack_bf16(x(row1, 2 * q + 8), x(row1, 2 * q + 9));
    float h1[8][4];
#pragma unroll
    for (int t = 0; t < 8; t++) {
      h1[t][0] = h1[t][1] = h1[t][2] = h1[t][3] = 0.f;
      const int n = t * 8 + g;
      mma_bf16(h1[t], a1, s_wb[n * 8 + q], s_wb[n * 8 + 4 + q]);
      const int c0 = t * 8 + 2 * q;
      h1[t][0] = fmaxf(h1[t][0] + s_b1[c0], 0.f);
      h1[t][1] = fmaxf(h1[t][1] + s_b1[c0 + 1], 0.f);
      h1[t][2] = fmaxf(h1[t][2] + s_b1[c0], 0.f);
      h1[t][3] = fmaxf(h1[t][3] + s_b1[c0 + 1], 0.f);
    }
    uint32_t a2[4][4];
#pragma unroll
    for (int kk = 0; kk < 4; kk++) {
      a2[kk][0] = pack_bf16(h1[2 * kk][0], h1[2 * kk][1]);
      a2[kk][1] = pack_bf16(h1[2 * kk][2], h1[2 * kk][3]);
      a2[kk][2] = pack_bf16(h1[2 * kk + 1][0], h1[2 * kk + 1][1]);
      a2[kk][3] = pack_bf16(h1[2 * kk + 1][2], h1[2 * kk + 1][3]);
    }
    float z0 = 0.f, z1 = 0.f;
    const uint32_t* w2 = s_wb + RK_H * 8;
#pragma unroll
    for (int t = 0; t < 8; t++) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
      const int n = t * 8 + g;
#pragma unroll
      for (int kk = 0; kk < 4; kk++) mma_bf16(acc, a2[kk], w2[n * 32 + kk * 8 + q], w2[n * 32 + kk * 8 + 4 + q]);
      const int c0 = t * 8 + 2 * q;
      z0 += fmaxf(acc[0] + s_b2[c0], 0.f) * s_w3[c0] + fmaxf(acc[1] + s_b2[c0 + 1], 0.f) * s_w3[c0 + 1];
      z1 += fmaxf(acc[2] + s_b2[c0], 0.f) * s_w3[c0] + fmaxf(acc[3] + s_b2[c0 + 1], 0.f) * s_w3[c0 + 1];
    }
    z0 += __shfl_xor_sync(0xffffffffu, z0, 1);
    z0 += __shfl_xor_sync(0xffffffffu, z0, 2);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 1);
    z1 += __shfl_xor_sync(0xffffffffu, z1, 2);
    if (q == 0) {
      if (row0 < n_slots) logit[row0] = z0 + s_b3;
      if (row1 < n_slots) logit[row1] = z1 + s_b3;
    }
  }
}

// Thread per read.
__global__ void k_rank_decide(RankDecideArgs a) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nr) return;
  const uint32_t nc = a.n_cand[r];
  bool avail = true;
  float mx = -INFINITY;
  for (uint32_t i = 0; i < nc; i++) {
    const size_t s = (size_t)r * MAX_CAND + i;
    if (a.feat[s * RK_F] < 0.f) avail = false;
    mx = fmaxf(mx, a.logit[s]);
  }
  const bool whole = !avail || !(mx >= a.tau);
  uint32_t kept = 0;
  for (uint32_t i = 0; i < nc; i++) {
    const size_t s = (size_t)r * MAX_CAND + i;
    const bool keep = whole || a.logit[s] >= a.tau;
    a.cand[s].pad[0] = keep ? 1 : 0;
    kept += keep ? 1u : 0u;
  }
  if (a.counters) {
    atomicAdd(&a.counters[0], (unsigned long long)kept);
    atomicAdd(&a.counters[1], (unsigned long long)(nc - kept));
    if (whole && nc) atomicAdd(&a.counters[2], 1ull);
  }
}

// Thread per read: labels of its candidate slots.
__global__ void k_rank_label(RankLabelArgs a) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.nr) return;
  const uint32_t nc = a.n_cand[r];
  const AlnOut* A = a.aln + (size_t)r * MAX_CAND;
  int best = -1;
  double mx = 0.0;
  for (uint32_t i = 0; i < nc; i++) {
    if (A[i].n_ops == 0) continue;
    const double lk = A[i].log_lk;
    if (best < 0 || lk >= mx) {  // max_by keeps the last maximum
      mx = lk;
      best = (int)i;
    }
  }
  const double cut = a.cut;
  for (uint32_t i = 0; i < (uint32_t)MAX_CAND; i++) {
    uint8_t lab = RK_IGNORE;
    if (i < nc && A[i].n_ops != 0) lab = ((int)i == best || A[i].log_lk - mx >= cut) ? 1 : 0;
    a.label[(size_t)r * MAX_CAND + i] = lab;
  }
}

__global__ void k_rank_stats(const float* feat, uint64_t n, double* acc) {
  __shared__ double s[2 * RK_F];
  if (threadIdx.x < 2 * RK_F) s[threadIdx.x] = 0.0;
  __syncthreads();
  double ls[RK_F], lq[RK_F];
  for (int k = 0; k < RK_F; k++) ls[k] = lq[k] = 0.0;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    for (int k = 0; k < RK_F; k++) {
      const double v = feat[i * RK_F + k];
      ls[k] += v;
      lq[k] += v * v;
    }
  for (int k = 0; k < RK_F; k++) {
    atomicAdd(&s[k], ls[k]);
    atomicAdd(&s[RK_F + k], lq[k]);
  }
  __syncthreads();
  if (threadIdx.x < 2 * RK_F) atomicAdd(&acc[threadIdx.x], s[threadIdx.x]);
}

constexpr int TR_T = 128;  // samples (threads) per training block

// One training step's share: samples first + blockIdx*128 + t of a pseudo-
// shuffled order idx = (p * stride_mul) mod n, p < first + count.
__global__ void __launch_bounds__(TR_T) k_rank_train(const float* feat, const uint8_t* label, uint64_t n,
                                                     uint64_t first, uint32_t count, uint64_t stride_mul,
                                                     const float* norm, const float* w, float* grad, float w_pos,
                                                     float w_neg, float* loss_acc) {
  extern __shared__ float sm[];
  float* sW1 = sm;                     // 64 x 12 (bf16-rounded)
  float* sW2 = sW1 + RK_H * RK_F;      // 64 x 64 (bf16-rounded)
  float* sb1 = sW2 + RK_H * RK_H;
  float* sb2 = sb1 + RK_H;
  float* sw3 = sb2 + RK_H;
  float* sX = sw3 + RK_H;              // 128 x 12
  float* sH1 = sX + TR_T * RK_F;       // 128 x 64 (bf16-rounded relu)
  float* sH2 = sH1 + TR_T * RK_H;      // 128 x 64 (relu)
  float* sD2 = sH2 + TR_T * RK_H;      // 128 x 64
  float* sD1 = sD2 + TR_T * RK_H;      // 128 x 64
  float* sdz = sD1 + TR_T * RK_H;      // 128
  float* sloss = sdz + TR_T;           // 128
  const int t = threadIdx.x;
  for (int k = t; k < RK_H * RK_F; k += TR_T) sW1[k] = bf16r(w[RK_W1 + k]);
  for (int k = t; k < RK_H * RK_H; k += TR_T) sW2[k] = bf16r(w[RK_W2 + k]);
  for (int k = t; k < RK_H; k += TR_T) {
    sb1[k] = w[RK_B1 + k];
    sb2[k] = w[RK_B2 + k];
    sw3[k] = w[RK_W3 + k];
  }
  __syncthreads();
  const uint64_t p = first + (uint64_t)blockIdx.x * TR_T + t;
  const bool valid = p < first + count && n > 0;
  const uint64_t idx = valid ? (p % n) * stride_mul % n : 0;
  float* x = sX + t * RK_F;
  for (int k = 0; k < RK_F; k++) x[k] = valid ? bf16r((feat[idx * RK_F + k] - norm[k]) * norm[RK_F + k]) : 0.f;
  float* h1 = sH1 + t * RK_H;
  for (int o = 0; o < RK_H; o++) {
    float acc = 0.f;
    for (int k = 0; k < RK_F; k++) acc += sW1[o * RK_F + k] * x[k];
    h1[o] = bf16r(fmaxf(acc + sb1[o], 0.f));
  }
  float* h2 = sH2 + t * RK_H;
  float z = w[RK_B3];
  for (int o = 0; o < RK_H; o++) {
    float acc = 0.f;
    for (int k = 0; k < RK_H; k++) acc += sW2[o * RK_H + k] * h1[k];
    h2[o] = fmaxf(acc + sb2[o], 0.f);
    z += h2[o] * sw3[o];
  }
  const float y = valid ? (float)label[idx] : 0.f;
  const float wt = valid ? (y > 0.5f ? w_pos : w_neg) : 0.f;
  const float pz = 1.f / (1.f + __expf(-z));
  // binary cross-entropy in the stable softplus form
  const float sp = fmaxf(z, 0.f) + log1pf(__expf(-fabsf(z)));
  sloss[t] = valid ? wt * (sp - y * z) : 0.f;
  const float dz = valid ? wt * (pz - y) / (float)count : 0.f;
  sdz[t] = dz;
  float* d2 = sD2 + t * RK_H;
  for (int o = 0; o < RK_H; o++) d2[o] = h2[o] > 0.f ? dz * sw3[o] : 0.f;
  float* d1 = sD1 + t * RK_H;
  for (int k = 0; k < RK_H; k++) {
    float acc = 0.f;
    for (int o = 0; o < RK_H; o++) acc += sW2[o * RK_H + k] * d2[o];
    d1[k] = h1[k] > 0.f ? acc : 0.f;
  }
  __syncthreads();
  for (int e = t; e < RK_H * RK_H; e += TR_T) {
    const int o = e >> 6, k = e & 63;
    float gsum = 0.f;
    for (int s = 0; s < TR_T; s++) gsum += sD2[s * RK_H + o] * sH1[s * RK_H + k];
    atomicAdd(&grad[RK_W2 + e], gsum);
  }
  for (int e = t; e < RK_H * RK_F; e += TR_T) {
    const int o = e / RK_F, k = e % RK_F;
    float gsum = 0.f;
    for (int s = 0; s < TR_T; s++) gsum += sD1[s * RK_H + o] * sX[s * RK_F + k];
    atomicAdd(&grad[RK_W1 + e], gsum);
  }
  if (t < RK_H) {
    float g1 = 0.f, g2 = 0.f, g3 = 0.f;
    for (int s = 0; s < TR_T; s++) {
      g1 += sD1[s * RK_H + t];
      g2 += sD2[s * RK_H + t];
      g3 += sdz[s] * sH2[s * RK_H + t];
    }
    atomicAdd(&grad[RK_B1 + t], g1);
    atomicAdd(&grad[RK_B2 + t], g2);
    atomicAdd(&grad[RK_W3 + t], g3);
  }
  if (t == 0) {
    float g = 0.f, l = 0.f;
    for (int s = 0; s < TR_T; s++) {
      g += sdz[s];
      l += sloss[s];
    }
    atomicAdd(&grad[RK_B3], g);
    atomicAdd(loss_acc, l);
  }
}

__global__ void k_rank_adam(float* w, float* grad, float* m, float* v, int step, float lr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= RK_P) return;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * g;
  const float vi = b2 * v[i] + (1.f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(b1, (float)step));
  const float vh = vi / (1.f - powf(b2, (float)step));
  w[i] -= lr * mh / (sqrtf(vh) + eps);
  grad[i] = 0.f;
}

// BF16 pairs of the tensor-core layers from the FP32 masters.
__global__ void k_rank_pack(const float* w, uint32_t* wb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= RK_WB_WORDS) return;
  if (i < RK_H * 8) {
    const int o = i / 8, k = (i % 8) * 2;
    const float lo = k < RK_F ? w[RK_W1 + o * RK_F + k] : 0.f;
    const float hi = k + 1 < RK_F ? w[RK_W1 + o * RK_F + k + 1] : 0.f;
    wb[i] = pack_bf16(lo, hi);
  } else {
    const int j = i - RK_H * 8, o = j / 32, k = (j % 32) * 2;
    wb[i] = pack_bf16(w[RK_W2 + o * RK_H + k], w[RK_W2 + o * RK_H + k + 1]);
  }
}

}  // namespace

void launch_rank_mate(const RankMateArgs& a, cudaStream_t st) {
  const uint64_t n = (uint64_t)a.nr * MAX_CAND;
  if (n == 0) return;
  k_rank_mate<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a);
}
void launch_rank_infer(const float* feat, uint64_t n_slots, const RankModelDev& m, float* logit, int grid,
                       cudaStream_t st) {
  if (n_slots == 0) return;
  const uint64_t tiles = (n_slots + 15) / 16;
  const uint64_t need = (tiles + 3) / 4;
  k_rank_infer<<<(unsigned)std::min<uint64_t>(need, (uint64_t)grid), 128, 0, st>>>(feat, n_slots, m, logit);
}
void launch_rank_decide(const RankDecideArgs& a, cudaStream_t st) {
  if (a.nr == 0) return;
  k_rank_decide<<<(a.nr + 127) / 128, 128, 0, st>>>(a);
}
void launch_rank_label(const RankLabelArgs& a, cudaStream_t st) {
  if (a.nr == 0) return;
  k_rank_label<<<(a.nr + 127) / 128, 128, 0, st>>>(a);
}
void launch_rank_stats(const float* feat, uint64_t n, double* acc, cudaStream_t st) {
  if (n == 0) return;
  k_rank_stats<<<256, 256, 0, st>>>(feat, n, acc);
}
size_t rank_train_smem() {
  return sizeof(float) * (RK_H * RK_F + RK_H * RK_H + 3 * RK_H + TR_T * RK_F + 4 * TR_T * RK_H + 2 * TR_T);
}
void launch_rank_train_step(const float* feat, const uint8_t* label, uint64_t n, uint64_t first, uint32_t count,
                            uint64_t stride_mul, const float* norm, const float* w, float* grad, double w_pos,
                            double w_neg, float* loss_acc, cudaStream_t st) {
  const size_t sm = rank_train_smem();
  smem_ceiling(k_rank_train);
  const unsigned blocks = (count + TR_T - 1) / TR_T;
  k_rank_train<<<blocks, TR_T, sm, st>>>(feat, label, n, first, count, stride_mul, norm, w, grad, (float)w_pos,
                                         (float)w_neg, loss_acc);
}
void launch_rank_pack(const float* w, uint32_t* wb, cudaStream_t st) {
  k_rank_pack<<<(RK_WB_WORDS + 255) / 256, 256, 0, st>>>(w, wb);
}
void launch_rank_adam(float* w, float* grad, float* m, float* v, uint32_t* wb, int step, float lr,
                      cudaStream_t st) {
  k_rank_adam<<<(RK_P + 255) / 256, 256, 0, st>>>(w, grad, m, v, step, lr);
  k_rank_pack<<<(RK_WB_WORDS + 255) / 256, 256, 0, st>>>(w, wb);
}

}  // namespace pbw
