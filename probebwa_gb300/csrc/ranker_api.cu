// ranker_api.cu -- training and switching the learned candidate ranker
// (ranker.cu) behind the C ABI. No counterpart in the reference.
//
// pbw_ranker_train maps the caller's reads once with the plain path while
// the pipeline records every candidate slot's features and label; the
// labelled slots are compacted on the device, normalised (per-feature mean
// and standard deviation), and the MLP is trained with Adam on weighted
// binary cross-entropy (positives weighted up, since a wrongly pruned
// positive can change a record and a kept negative only costs one DP). The
// keep threshold is then set on the training candidates so that the
// requested fraction of positives is kept.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_host.h"
#include "pbw_pipeline.h"
#include "ranker.h"

namespace pbw {
namespace {

#define RK_CK(call)                                                \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
      return PBW_ERR_CUDA;                                         \
    }                                                              \
  } while (0)
#define RK_TRY(x)                  \
  do {                             \
    int rc_ = (x);                 \
    if (rc_ != PBW_OK) return rc_; \
  } while (0)

template <class T>
int rk_grow(pbw_handle* h, DevBuf<T>& b, size_t n) {
  if (n <= b.cap) return PBW_OK;
  b.release();
  if (cudaMalloc((void**)&b.p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) {
    b.p = nullptr;
    h->err = "cudaMalloc failed for the ranker (" + std::to_string(n * sizeof(T)) + " bytes)";
    return PBW_ERR_NOMEM;
  }
  b.cap = n;
  return PBW_OK;
}

__global__ void k_flag_labelled(const uint8_t* label, uint64_t n, unsigned int* flag) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = label[i] != RK_IGNORE ? 1u : 0u;
}
__global__ void k_compact_samples(const float* feat, const uint8_t* label, const unsigned int* dst, uint64_t n,
                                  float* feat_out, uint8_t* label_out) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || label[i] == RK_IGNORE) return;
  const uint64_t d = dst[i];
  for (int k = 0; k < RK_F; k++) feat_out[d * RK_F + k] = feat[i * RK_F + k];
  label_out[d] = label[i];
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double uniform(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

int map_for_collection(pbw_handle* h, const pbw_reads* r1, const pbw_reads* r2) {
  auto alloc = [&](std::vector<std::vector<uint8_t>>& keep, const pbw_reads* r, pbw_records& o) {
    uint64_t nn = 0, cc = 0;
    pbw_records_reserve(r, &nn, &cc);
    auto buf = [&](size_t bytes) {
      keep.emplace_back(std::max<size_t>(bytes, 8));
      return (void*)keep.back().data();
    };
    o.n = nn;
    o.contig = (int32_t*)buf(nn * 4);
    o.pos = (uint64_t*)buf(nn * 8);
    o.mapq = (uint8_t*)buf(nn);
    o.flag = (uint16_t*)buf(nn * 2);
    o.mate_contig = (int32_t*)buf(nn * 4);
    o.mate_pos = (uint64_t*)buf(nn * 8);
    o.tlen = (int64_t*)buf(nn * 8);
    o.log_lk = (double*)buf(nn * 8);
    o.posterior = (double*)buf(nn * 8);
    o.as_score = (int32_t*)buf(nn * 4);
    o.nm = (int32_t*)buf(nn * 4);
    o.cigar_off = (uint32_t*)buf((nn + 1) * 4);
    o.cigar = (uint32_t*)buf(cc * 4);
    o.cigar_cap = cc;
  };
  std::vector<std::vector<uint8_t>> keep;
  pbw_records o1{}, o2{};
  alloc(keep, r1, o1);
  if (r2) {
    alloc(keep, r2, o2);
    pbw_insert_model m{h->opt.insert_size_mean, h->opt.insert_size_sd, 0};
    return pbw_map_paired(h, &m, r1, r2, &o1, &o2);
  }
  return pbw_map_single(h, r1, &o1);
}

}  // namespace
}  // namespace pbw

extern "C" {

void pbw_ranker_default_options(pbw_ranker_train_options* o) {
  o->epochs = 3;
  o->batch = 8192;
  o->lr = 2e-3;
  o->recall = 0.9995;
  o->positive_weight = 4.0;
  o->seed = 0x5EED;
  o->label_cut = -60.0 * 0.69314718055994530942;
}

int pbw_ranker_train(pbw_handle* h, const pbw_reads* r1, const pbw_reads* r2, const pbw_ranker_train_options* opt,
                     pbw_ranker_report* rep) {
  using namespace pbw;
  if (!h || !r1) return PBW_ERR_ARG;
  pbw_ranker_train_options o;
  pbw_ranker_default_options(&o);
  if (opt) o = *opt;
  if (o.epochs == 0 || o.batch == 0 || !(o.recall > 0.0 && o.recall <= 1.0)) {
    h->err = "pbw_ranker_train: epochs, batch and recall in (0, 1] required";
    return PBW_ERR_ARG;
  }
  if (r2 && r2->n != r1->n) {
    h->err = "pbw_ranker_train: mates differ in count";
    return PBW_ERR_ARG;
  }
  cudaStream_t st = h->st;
  const auto t0 = std::chrono::steady_clock::now();
  const int sets = r2 ? 2 : 1;
  const uint64_t slots = r1->n * MAX_CAND;
  if ((uint64_t)sets * slots >= (1ull << 32)) {
    h->err = "pbw_ranker_train: more than 2^32 candidate slots";
    return PBW_ERR_LIMIT;
  }
  auto& R = h->rk;
  RK_TRY(rk_grow(h, R.c_feat, (size_t)sets * slots * RK_F));
  RK_TRY(rk_grow(h, R.c_label, (size_t)sets * slots));
  RK_CK(cudaMemsetAsync(R.c_label.p, RK_IGNORE, (size_t)sets * slots, st));
  R.c_slots = slots;
  const bool was_enabled = R.enabled;
  R.label_cut = o.label_cut;
  R.collect = true;
  R.enabled = false;
  int rc = map_for_collection(h, r1, r2);
  R.collect = false;
  R.enabled = was_enabled;
  if (rc != PBW_OK) return rc;
  const auto t1 = std::chrono::steady_clock::now();
  // dense labelled samples
  const uint64_t M = (uint64_t)sets * slots;
  DevBuf<unsigned int> flag, dst, sums;
  RK_TRY(rk_grow(h, flag, M));
  RK_TRY(rk_grow(h, dst, M));
  RK_TRY(rk_grow(h, sums, scan_blocks(M) + 2));
  DevBuf<unsigned int> tot;
  RK_TRY(rk_grow(h, tot, 2));
  k_flag_labelled<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(R.c_label.p, M, flag.p);
  launch_scan_excl(flag.p, M, dst.p, sums.p, tot.p, nullptr, st);
  unsigned int N32 = 0;
  RK_CK(cudaMemcpyAsync(&N32, tot.p, 4, cudaMemcpyDeviceToHost, st));
  RK_CK(cudaStreamSynchronize(st));
  const uint64_t N = N32;
  if (N == 0) {
    h->err = "pbw_ranker_train: no aligned candidates in the training reads";
    return PBW_ERR_ARG;
  }
  DevBuf<float> feat;
  DevBuf<uint8_t> label;
  RK_TRY(rk_grow(h, feat, N * RK_F));
  RK_TRY(rk_grow(h, label, N));
  k_compact_samples<<<(unsigned)((M + 255) / 256), 256, 0, st>>>(R.c_feat.p, R.c_label.p, dst.p, M, feat.p, label.p);
  flag.release();
  dst.release();
  // normalisation
  DevBuf<double> acc;
  RK_TRY(rk_grow(h, acc, 2 * RK_F));
  RK_CK(cudaMemsetAsync(acc.p, 0, 2 * RK_F * sizeof(double), st));
  launch_rank_stats(feat.p, N, acc.p, st);
  double ha[2 * RK_F];
  RK_CK(cudaMemcpyAsync(ha, acc.p, sizeof(ha), cudaMemcpyDeviceToHost, st));
  std::vector<uint8_t> hl(N);
  RK_CK(cudaMemcpyAsync(hl.data(), label.p, N, cudaMemcpyDeviceToHost, st));
  RK_CK(cudaStreamSynchronize(st));
  float norm[2 * RK_F];
  for (int k = 0; k < RK_F; k++) {
    const double mean = ha[k] / (double)N;
    const double var = std::max(ha[RK_F + k] / (double)N - mean * mean, 0.0);
    norm[k] = (float)mean;
    norm[RK_F + k] = (float)(1.0 / std::max(std::sqrt(var), 1e-3));
  }
  const uint64_t pos = (uint64_t)std::count(hl.begin(), hl.end(), (uint8_t)1);
  const uint64_t neg = N - pos;
  // parameters: He-uniform weights, zero biases, the output bias at the prior log-odds
  std::vector<float> w(RK_P, 0.f);
  uint64_t s = o.seed;
  for (int k = 0; k < RK_H * RK_F; k++) w[RK_W1 + k] = (float)((2 * uniform(s) - 1) * std::sqrt(6.0 / RK_F));
  for (int k = 0; k < RK_H * RK_H; k++) w[RK_W2 + k] = (float)((2 * uniform(s) - 1) * std::sqrt(6.0 / RK_H));
  for (int k = 0; k < RK_H; k++) w[RK_W3 + k] = (float)((2 * uniform(s) - 1) * std::sqrt(6.0 / RK_H));
  w[RK_B3] = (pos && neg) ? (float)std::log((double)pos / (double)neg) : 0.f;
  RK_TRY(rk_grow(h, R.d_norm, 2 * RK_F));
  RK_TRY(rk_grow(h, R.d_w, RK_P));
  RK_TRY(rk_grow(h, R.d_m, RK_P));
  RK_TRY(rk_grow(h, R.d_v, RK_P));
  RK_TRY(rk_grow(h, R.d_g, RK_P));
  RK_TRY(rk_grow(h, R.d_loss, 2));
  RK_TRY(rk_grow(h, R.d_wb, RK_WB_WORDS));
  RK_TRY(rk_grow(h, R.d_counters, 4));
  RK_CK(cudaMemcpyAsync(R.d_norm.p, norm, sizeof(norm), cudaMemcpyHostToDevice, st));
  RK_CK(cudaMemcpyAsync(R.d_w.p, w.data(), RK_P * 4, cudaMemcpyHostToDevice, st));
  RK_CK(cudaMemsetAsync(R.d_m.p, 0, RK_P * 4, st));
  RK_CK(cudaMemsetAsync(R.d_v.p, 0, RK_P * 4, st));
  RK_CK(cudaMemsetAsync(R.d_g.p, 0, RK_P * 4, st));
  launch_rank_pack(R.d_w.p, R.d_wb.p, st);
  const double w_neg = neg ? 0.5 * (double)N / (double)neg : 1.0;
  const double w_pos = pos ? 0.5 * (double)N / (double)pos * o.positive_weight : 1.0;
  int step = 0;
  double loss_first = 0, loss_last = 0;
  for (uint32_t e = 0; e < o.epochs; e++) {
    // a multiplier coprime with N gives a fresh visiting order each epoch
    uint64_t mul = 1;
    if (N > 1) {
      do {
        mul = (splitmix(s) % (N - 1)) + 1;
      } while (std::gcd(mul, N) != 1);
    }
    RK_CK(cudaMemsetAsync(R.d_loss.p, 0, 4, st));
    for (uint64_t first = 0; first < N; first += o.batch) {
      const uint32_t cnt = (uint32_t)std::min<uint64_t>(o.batch, N - first);
      launch_rank_train_step(feat.p, label.p, N, first, cnt, mul, R.d_norm.p, R.d_w.p, R.d_g.p, w_pos, w_neg,
                             R.d_loss.p, st);
      launch_rank_adam(R.d_w.p, R.d_g.p, R.d_m.p, R.d_v.p, R.d_wb.p, ++step, (float)o.lr, st);
    }
    float l = 0;
    RK_CK(cudaMemcpyAsync(&l, R.d_loss.p, 4, cudaMemcpyDeviceToHost, st));
    RK_CK(cudaStreamSynchronize(st));
    RK_CK(cudaGetLastError());
    if (e == 0) loss_first = l / (double)N;
    loss_last = l / (double)N;
  }
  // keep threshold: the requested fraction of the positives at or above it
  DevBuf<float> logit;
  RK_TRY(rk_grow(h, logit, N));
  RankModelDev md{R.d_norm.p, R.d_wb.p, R.d_w.p};
  launch_rank_infer(feat.p, N, md, logit.p, h->num_sms * 8, st);
  std::vector<float> lg(N);
  RK_CK(cudaMemcpyAsync(lg.data(), logit.p, N * 4, cudaMemcpyDeviceToHost, st));
  RK_CK(cudaStreamSynchronize(st));
  std::vector<float> pl;
  pl.reserve(pos);
  for (uint64_t i = 0; i < N; i++)
    if (hl[i]) pl.push_back(lg[i]);
  float tau = -INFINITY;
  if (!pl.empty()) {
    std::sort(pl.begin(), pl.end());
    const uint64_t drop = (uint64_t)std::floor((1.0 - o.recall) * (double)pl.size());
    tau = pl[std::min<uint64_t>(drop, pl.size() - 1)];
  }
  uint64_t kept_pos = 0, pruned_neg = 0;
  for (uint64_t i = 0; i < N; i++) {
    if (hl[i]) kept_pos += lg[i] >= tau ? 1 : 0;
    else pruned_neg += lg[i] < tau ? 1 : 0;
  }
  R.tau = tau;
  R.trained = true;
  const auto t2 = std::chrono::steady_clock::now();
  if (rep) {
    rep->samples = N;
    rep->positives = pos;
    rep->loss_first = loss_first;
    rep->loss_last = loss_last;
    rep->tau = tau;
    rep->train_recall = pos ? (double)kept_pos / (double)pos : 1.0;
    rep->train_prune = neg ? (double)pruned_neg / (double)neg : 0.0;
    rep->ms_collect = std::chrono::duration<double, std::milli>(t1 - t0).count();
    rep->ms_train = std::chrono::duration<double, std::milli>(t2 - t1).count();
  }
  return PBW_OK;
}

int pbw_ranker_score(pbw_handle* h, const float* feat, uint64_t n, float* logit) {
  using namespace pbw;
  if (!h || (n && (!feat || !logit))) return PBW_ERR_ARG;
  if (!h->rk.trained) {
    h->err = "pbw_ranker_score: no trained ranker";
    return PBW_ERR_ARG;
  }
  if (n == 0) return PBW_OK;
  DevBuf<float> f, l;
  RK_TRY(rk_grow(h, f, n * RK_F));
  RK_TRY(rk_grow(h, l, n));
  RK_CK(cudaMemcpyAsync(f.p, feat, n * RK_F * 4, cudaMemcpyHostToDevice, h->st));
  RankModelDev md{h->rk.d_norm.p, h->rk.d_wb.p, h->rk.d_w.p};
  launch_rank_infer(f.p, n, md, l.p, h->num_sms * 8, h->st);
  RK_CK(cudaGetLastError());
  RK_CK(cudaMemcpyAsync(logit, l.p, n * 4, cudaMemcpyDeviceToHost, h->st));
  RK_CK(cudaStreamSynchronize(h->st));
  return PBW_OK;
}

int pbw_ranker_enable(pbw_handle* h, int32_t on) {
  if (!h) return PBW_ERR_ARG;
  if (on && !h->rk.trained) {
    h->err = "pbw_ranker_enable: no trained ranker (pbw_ranker_train or pbw_ranker_import first)";
    return PBW_ERR_ARG;
  }
  h->rk.enabled = on != 0;
  if (h->rk.d_counters.p) cudaMemsetAsync(h->rk.d_counters.p, 0, 4 * sizeof(unsigned long long), h->st);
  return PBW_OK;
}

int pbw_ranker_counters(pbw_handle* h, uint64_t* kept, uint64_t* pruned, uint64_t* reads_whole) {
  if (!h) return PBW_ERR_ARG;
  unsigned long long c[4] = {0, 0, 0, 0};
  if (h->rk.d_counters.p) {
    if (cudaMemcpyAsync(c, h->rk.d_counters.p, sizeof(c), cudaMemcpyDeviceToHost, h->st) != cudaSuccess ||
        cudaStreamSynchronize(h->st) != cudaSuccess) {
      h->err = "pbw_ranker_counters: copy failed";
      return PBW_ERR_CUDA;
    }
  }
  if (kept) *kept = c[0];
  if (pruned) *pruned = c[1];
  if (reads_whole) *reads_whole = c[2];
  return PBW_OK;
}

int pbw_ranker_export(const pbw_handle* h, float* out, uint64_t cap, uint64_t* n) {
  using namespace pbw;
  if (!h || !n) return PBW_ERR_ARG;
  *n = 2 * RK_F + RK_P + 1;
  if (!h->rk.trained || !out) return h->rk.trained ? PBW_OK : PBW_ERR_ARG;
  if (cap < *n) return PBW_ERR_CAPACITY;
  if (cudaMemcpy(out, h->rk.d_norm.p, 2 * RK_F * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
      cudaMemcpy(out + 2 * RK_F, h->rk.d_w.p, RK_P * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
    return PBW_ERR_CUDA;
  out[2 * RK_F + RK_P] = h->rk.tau;
  return PBW_OK;
}

int pbw_ranker_import(pbw_handle* h, const float* in, uint64_t n) {
  using namespace pbw;
  if (!h || !in || n != (uint64_t)(2 * RK_F + RK_P + 1)) {
    if (h) h->err = "pbw_ranker_import: expected " + std::to_string(2 * RK_F + RK_P + 1) + " floats";
    return PBW_ERR_ARG;
  }
  auto& R = h->rk;
  RK_TRY(rk_grow(h, R.d_norm, 2 * RK_F));
  RK_TRY(rk_grow(h, R.d_w, RK_P));
  RK_TRY(rk_grow(h, R.d_wb, RK_WB_WORDS));
  RK_TRY(rk_grow(h, R.d_counters, 4));
  RK_CK(cudaMemcpy(R.d_norm.p, in, 2 * RK_F * 4, cudaMemcpyHostToDevice));
  RK_CK(cudaMemcpy(R.d_w.p, in + 2 * RK_F, RK_P * 4, cudaMemcpyHostToDevice));
  launch_rank_pack(R.d_w.p, R.d_wb.p, h->st);
  RK_CK(cudaStreamSynchronize(h->st));
  R.tau = in[2 * RK_F + RK_P];
  R.trained = true;
  return PBW_OK;
}

}  // extern "C"
