// pipeline.cu -- the device pipeline behind pbw_map_single and the stage
// entry points (include/probebwa_gpu.h).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_common.cuh"
#include "pbw_host.h"
#include "pbw_kernels.h"
#include "pbw_pipeline.h"
#include "paired.h"
#include "ranker.h"

namespace pbw {

#define CK(call)                                                   \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
      return PBW_ERR_CUDA;                                         \
    }                                                              \
  } while (0)
#define TRY(x)                     \
  do {                             \
    int rc_ = (x);                 \
    if (rc_ != PBW_OK) return rc_; \
  } while (0)

template <class T>
static int grow(pbw_handle* h, DevBuf<T>& b, size_t n) {
  if (n <= b.cap) return PBW_OK;
  b.release();
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)&b.p, bytes);
  if (e != cudaSuccess) {
    h->err = "cudaMalloc(" + std::to_string(bytes) + "): " + cudaGetErrorString(e);
    b.p = nullptr;
    return PBW_ERR_NOMEM;
  }
  b.cap = n;
  return PBW_OK;
}

int pipeline_init(pbw_handle* h) {
  TRY(grow(h, h->d_cnt32, 16));
  TRY(grow(h, h->d_cnt64, 16));
  for (int i = 0; i < 64; i++) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    h->events.push_back(e);
  }
  return PBW_OK;
}

// Seed hits of reads that overflow the per-read capacity go to a pool, one
// slice of OVF_SLICE_HITS at a time: the reads whose exclusive offset falls
// in slice s are seeded again and clustered in the s-th list-mode pass. A
// read reaches at most one slice past its start, so the pool holds two
// slices; their clustering scratch takes cluster_list_bytes_per_hit bytes
// per pooled hit. A chunk's
// over-capacity reads may hold up to OVF_MAX_SLICES slices of hits.
constexpr size_t OVF_SLICE_HITS = 16ull << 20;
constexpr uint32_t OVF_MAX_SLICES = 16;
// Tiers of the binned K2: reads up to hmax hits (0: the per-read buffer's
// capacity) and threads per block; a tier whose tables do not fit shared
// memory keeps them in the global slab.
struct BinTier {
  uint32_t hmax;
  int threads;
};
constexpr BinTier BIN_TIERS[5] = {{512, 128}, {1024, 256}, {2048, 512}, {4096, 1024}, {0, 1024}};
static uint32_t group_keys(const pbw_handle* h) { return 2u * std::max(h->G.ncontig, 1u); }
// The tiers whose block size the autotuner picks (the 4096-hit tier and the
// slab tier), and the sizes it tries.
static int k2_tuned_tier(const BinTier& t) { return t.hmax == 4096 ? 0 : (t.hmax == 0 ? 1 : -1); }
constexpr int K2_TRIAL_THREADS[3] = {1024, 512, 256};
static size_t cluster_scratch_bytes(const pbw_handle* h, uint32_t hcap) {
  size_t need = 0;
  uint32_t lo = 0;
  const uint32_t gm = group_keys(h);
  for (const BinTier& t : BIN_TIERS) {
    const uint32_t hm = t.hmax ? std::min(t.hmax, hcap) : hcap;
    if (hm <= lo) continue;
    const uint32_t hx = t.hmax ? t.hmax : hcap;
    for (const bool feat : {false, true}) {
      const bool gt = cluster_bins_in_slab(hx, gm, feat);
      for (int i = 0; i < 3; i++) {
        const int thr = k2_tuned_tier(t) >= 0 ? K2_TRIAL_THREADS[i] : t.threads;
        need = std::max(need, cluster_bins_slab_bytes(hx, gm, gt) *
                                  (size_t)cluster_bins_grid(hx, gm, thr, feat, h->num_sms));
      }
    }
    lo = hm;
  }
  return need;
}
// The slice in use: OVF_SLICE_HITS unless pbw_set_tuning lowered it (the
// total the chunk may hold stays OVF_MAX_SLICES * OVF_SLICE_HITS).
static uint64_t ovf_slice_hits(const pbw_handle* h) {
  const uint64_t s = h->tune.ovf_slice_hits;
  return s && s < OVF_SLICE_HITS ? s : OVF_SLICE_HITS;
}
// The pool: two slices.
static uint64_t ovf_pool_hits(const pbw_handle* h) { return 2 * ovf_slice_hits(h); }
static uint32_t ovf_max_slices(const pbw_handle* h) {
  return (uint32_t)((OVF_MAX_SLICES * OVF_SLICE_HITS) / ovf_slice_hits(h));
}

// Scratch sizing for one chunk.
struct ChunkCfg {
  uint32_t ch;      // reads per chunk
  int lmax;
  int lmin;         // shortest read of the call (length bins when below lmax)
  uint32_t hcap;
  uint32_t wcap;
  int nmax;         // longest reference window
};

static ChunkCfg chunk_cfg(pbw_handle* h, uint64_t n, int lmax) {
  ChunkCfg c;
  c.ch = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(n, 1), h->opt.chunk_reads);
  c.lmax = std::max(lmax, 1);
  c.lmin = std::min(std::max(h->call_lmin, 0), c.lmax);
  // per-read hit buffer: 4096 hits cluster with shared-memory tables; long
  // reads on a repeat-rich genome have more (a 3.1 Gbp genome with 45%
  // interspersed repeats gives 250-base reads ~4,100 hits on average, 11,600
  // at the 99th percentile), clustered with global-slab tables up to 16384,
  // the rest through the pool
  c.hcap = c.lmax > 160 ? 16384 : 4096;
  c.wcap = (uint32_t)std::max(c.lmax - KMER + 1, 1);
  const uint64_t rp = std::max<uint64_t>(h->opt.max_indel_len, 10);
  c.nmax = (int)(c.lmax + 10 + rp);
  return c;
}

// Blocks of the window kernel (K3w) and its global slab for windows that do
// not fit a block's shared memory.
static int window_grid(pbw_handle* h) { return h->num_sms * 2; }
static int ensure_window_slab(pbw_handle* h, int lmax, int nmax, int grid) {
  return grow(h, h->d_tb_global, window_slab_bytes(lmax, nmax) * (size_t)grid);
}

static int ensure_chunk(pbw_handle* h, const ChunkCfg& c) {
  TRY(grow(h, h->d_hits, (size_t)c.ch * c.hcap));
  TRY(grow(h, h->d_hit_cnt, c.ch));
  TRY(grow(h, h->d_overflow, c.ch));
  TRY(grow(h, h->d_rep, (size_t)c.ch * c.wcap));
  TRY(grow(h, h->d_cand, (size_t)c.ch * MAX_CAND));
  TRY(grow(h, h->d_n_cand, c.ch));
  TRY(grow(h, h->d_total_cand, c.ch));
  TRY(grow(h, h->d_jobs, (size_t)c.ch * MAX_CAND));
  if (h->tune.length_bins && c.lmin < c.lmax) {
    TRY(grow(h, h->d_jobs_b, (size_t)c.ch * MAX_CAND));
    TRY(grow(h, h->d_bins, job_bin_words()));
  }
  TRY(grow(h, h->d_aln, (size_t)c.ch * MAX_CAND));
  TRY(grow(h, h->d_cig_pool, (size_t)c.ch * MAX_CAND * 24 + 4096));
  TRY(grow(h, h->d_scan_sums, scan_blocks(c.ch) + 4));
  TRY(grow(h, h->d_need, c.ch));
  TRY(grow(h, h->d_ovf_list, c.ch));
  TRY(grow(h, h->d_list_hoff, c.ch));
  TRY(grow(h, h->d_hits_pool, ovf_pool_hits(h)));
  TRY(grow(h, h->d_cl_scratch, ovf_pool_hits(h) * cluster_list_bytes_per_hit(c.hcap, group_keys(h))));
  TRY(grow(h, h->d_cl_big, cluster_scratch_bytes(h, c.hcap)));
  if (h->opt.max_indel_len > 31) TRY(ensure_window_slab(h, c.lmax, c.nmax, window_grid(h)));
  else TRY(grow(h, h->d_tb_global, band_tb_slab_bytes(c.lmax, c.nmax, h->num_sms, (int)h->opt.max_indel_len)));
  return PBW_OK;
}

static int ensure_outputs(pbw_handle* h, uint64_t n, uint64_t cig_cap) {
  TRY(grow(h, h->o_contig, n));
  TRY(grow(h, h->o_mate_contig, n));
  TRY(grow(h, h->o_as, n));
  TRY(grow(h, h->o_nm, n));
  TRY(grow(h, h->o_best, n));
  TRY(grow(h, h->o_pos, n));
  TRY(grow(h, h->o_mate_pos, n));
  TRY(grow(h, h->o_tlen, n));
  TRY(grow(h, h->o_mapq, n));
  TRY(grow(h, h->o_flag, n));
  TRY(grow(h, h->o_log_lk, n));
  TRY(grow(h, h->o_post, n));
  TRY(grow(h, h->o_nops, n));
  TRY(grow(h, h->o_cig_off, n + 1));
  TRY(grow(h, h->o_cigar, cig_cap));
  return PBW_OK;
}

// Resident blocks of the anti-diagonal band kernel (4 warps per block).
struct Timer {
  pbw_handle* h;
  int next = 0;
  cudaEvent_t mark() {
    cudaEvent_t e = h->events[next++ % h->events.size()];
    cudaEventRecord(e, h->st);
    return e;
  }
};

static double ms_between(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

// The process's origin on each device's clock: an event recorded and
// completed when the first handle on the device opens. Calls report their
// compute span against it, so the spans of calls running at once on several
// handles can be merged.
cudaEvent_t device_epoch(int dev) {
  static std::mutex mu;
  static cudaEvent_t ev[64] = {};
  if (dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> g(mu);
  if (!ev[dev]) {
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    if (cudaEventRecord(e, 0) != cudaSuccess || cudaEventSynchronize(e) != cudaSuccess) {
      cudaEventDestroy(e);
      return nullptr;
    }
    ev[dev] = e;
  }
  return ev[dev];
}
static void set_compute_span(pbw_handle* h, cudaEvent_t a, cudaEvent_t b) {
  h->stats.ms_compute = ms_between(a, b);
  cudaEvent_t o = device_epoch(h->device);
  h->stats.t_compute_begin_ms = o ? ms_between(o, a) : 0.0;
  h->stats.t_compute_end_ms = o ? ms_between(o, b) : 0.0;
}

// Buffers receiving one read set's candidates and seeded alignments.
struct MateBufs {
  Cand* cand;
  uint32_t* n_cand;
  AlnOut* aln;
  uint8_t* rep;
  uint8_t mate;
  // CIGAR overflow pool and its cursor (none: the handle's pool and cnt32[2])
  uint32_t* pool = nullptr;
  unsigned int* pool_used = nullptr;
  uint32_t pool_cap = 0;
};

// Ranker buffers of one chunk (ranked or collecting map calls).
static int ensure_ranker_chunk(pbw_handle* h, const ChunkCfg& c) {
  TRY(grow(h, h->rk.d_hit_info, (size_t)c.ch * c.hcap));
  TRY(grow(h, h->rk.d_feat, 2 * (size_t)c.ch * MAX_CAND * RK_F));
  TRY(grow(h, h->rk.d_logit, 2 * (size_t)c.ch * MAX_CAND));
  TRY(grow(h, h->rk.d_counters, 4));
  return PBW_OK;
}

// Where read set `mate` of a chunk keeps its candidate features: the chunk
// scratch when ranking, the slot-indexed collection when collecting, none
// otherwise.
static float* rank_feat(pbw_handle* h, uint32_t ch, int mate, uint32_t r0) {
  if (h->rk.collect) return h->rk.c_feat.p + ((size_t)mate * h->rk.c_slots + (size_t)r0 * MAX_CAND) * RK_F;
  if (h->rk.enabled) return h->rk.d_feat.p + (size_t)mate * ch * MAX_CAND * RK_F;
  return nullptr;
}
static uint8_t* rank_label(pbw_handle* h, int mate, uint32_t r0) {
  return h->rk.collect ? h->rk.c_label.p + (size_t)mate * h->rk.c_slots + (size_t)r0 * MAX_CAND : nullptr;
}

// K1 for reads [r0, r0+nr): the per-read pass, then the pool offsets of the
// reads over the per-read capacity (their list-mode passes run slice by
// slice with the clustering, ovf_slice).
static int seed_phase(pbw_handle* h, const ChunkCfg& cfg, const uint8_t* bases, const uint64_t* offs, uint32_t r0,
                      uint32_t nr, uint8_t* rep, bool ranker_info, uint16_t* hit_rpos) {
  cudaStream_t st = h->st;
  unsigned int* c32 = h->d_cnt32.p;
  SeedArgs sa{};
  sa.G = h->G;
  sa.idx = h->I;
  sa.bases = bases;
  sa.offs = offs;
  sa.r0 = r0;
  sa.nr = nr;
  sa.lmax = cfg.lmax;
  sa.hits = h->d_hits.p;
  sa.hcap = cfg.hcap;
  sa.hit_cnt = h->d_hit_cnt.p;
  sa.overflow = h->d_overflow.p;
  sa.n_overflow = c32 + 3;
  sa.rep = rep;
  sa.wcap = cfg.wcap;
  sa.hit_rpos = hit_rpos;  // optional: each hit's read position (stage entry point)
  sa.hit_info = ranker_info ? h->rk.d_hit_info.p : nullptr;
  sa.counters = h->d_cnt64.p;
  sa.need = h->d_need.p;
  sa.ovf_list = h->d_ovf_list.p;
  sa.n_ovf = c32 + 6;
  CK(cudaMemsetAsync(c32 + 6, 0, 2 * sizeof(unsigned int), st));
  {
    size_t sm = seed_smem_per_warp(cfg.lmax) * 8;
    int bps = (int)std::max<size_t>(1, std::min<size_t>(8, (228 * 1024) / std::max<size_t>(sm, 1)));
    launch_seed(sa, h->num_sms * bps, st);
  }
  // reads over capacity: exact-size pool offsets
  launch_ovf_offsets(h->d_ovf_list.p, c32 + 6, h->d_need.p, h->d_list_hoff.p, h->d_cnt64.p + 8, ovf_slice_hits(h),
                     ovf_max_slices(h), h->d_err.p, c32 + 7, st);
  h->stats.kernel_launches += 2;
  CK(cudaGetLastError());
  return PBW_OK;
}

// Slice s of the over-capacity reads: seeded again in list mode into the
// pool (with their read positions when rpos_pool is set) and, when ca is
// given, clustered from it. Slices past the listed hits exit at once.
static int ovf_slice(pbw_handle* h, const ChunkCfg& cfg, const uint8_t* bases, const uint64_t* offs, uint32_t r0,
                     uint32_t nr, uint8_t* rep, uint32_t s, uint16_t* rpos_pool, const ClusterArgs* ca) {
  cudaStream_t st = h->st;
  unsigned int* c32 = h->d_cnt32.p;
  SeedArgs sl{};
  sl.G = h->G;
  sl.idx = h->I;
  sl.bases = bases;
  sl.offs = offs;
  sl.r0 = r0;
  sl.nr = nr;
  sl.lmax = cfg.lmax;
  sl.hcap = cfg.hcap;
  sl.rep = rep;
  sl.wcap = cfg.wcap;
  sl.hit_rpos_pool = rpos_pool;
  sl.need = h->d_need.p;
  sl.list = h->d_ovf_list.p;
  sl.list_n = c32 + 7;
  sl.list_hoff = h->d_list_hoff.p;
  sl.hits_pool = h->d_hits_pool.p;
  sl.pool_slice = ovf_slice_hits(h);
  sl.slice = s;
  sl.list_total = h->d_cnt64.p + 8;
  launch_seed_list(sl, h->num_sms * 2, st);
  h->stats.kernel_launches += 1;
  if (ca) {
    ClusterArgs cl = *ca;
    cl.list = h->d_ovf_list.p;
    cl.list_n = c32 + 7;
    cl.list_hoff = h->d_list_hoff.p;
    cl.hits_pool = h->d_hits_pool.p;
    cl.need = h->d_need.p;
    cl.scratch = h->d_cl_scratch.p;
    cl.pool_slice = ovf_slice_hits(h);
    cl.slice = s;
    cl.list_total = h->d_cnt64.p + 8;
    launch_cluster_list(cl, cluster_list_bytes_per_hit(cfg.hcap, ca->gmax), h->num_sms, st);
    h->stats.kernel_launches += 1;
  }
  CK(cudaGetLastError());
  return PBW_OK;
}

// K2 after seed_phase: the first max_out candidates of each read into
// cand (nr * max_out), the full count into total_cand, and with feat the
// candidate ranker's features of each kept candidate; the over-capacity
// reads are seeded into the pool and clustered slice by slice.
static int cluster_phase(pbw_handle* h, const ChunkCfg& cfg, const uint8_t* bases, const uint8_t* quals,
                         const uint64_t* offs, uint32_t r0, uint32_t nr, uint8_t* rep, Cand* cand, uint32_t* n_cand,
                         uint32_t* total_cand, uint32_t max_out, float* feat) {
  cudaStream_t st = h->st;
  ClusterArgs ca{};
  ca.hits = h->d_hits.p;
  ca.hit_cnt = h->d_hit_cnt.p;
  ca.overflow = h->d_overflow.p;
  ca.hcap = cfg.hcap;
  ca.offs = offs;
  ca.r0 = r0;
  ca.nr = nr;
  ca.group_width = h->opt.group_width;
  ca.gmax = group_keys(h);
  ca.max_out = max_out;
  ca.cand = cand;
  ca.n_cand = n_cand;
  ca.total_cand = total_cand;
  ca.err = h->d_err.p;
  if (feat) {
    ca.feat = feat;
    ca.hit_info = h->rk.d_hit_info.p;
    ca.quals = quals;
  }
  // reads within the per-read buffer, by hit-count tier
  uint32_t lo = 0;
  auto& T = h->tune;
  for (const BinTier& t : BIN_TIERS) {
    const uint32_t hm = t.hmax ? std::min(t.hmax, cfg.hcap) : cfg.hcap;
    if (hm <= lo) continue;
    ClusterArgs cb = ca;
    cb.h_lo = lo;
    cb.h_hi = hm;
    cb.scratch = h->d_cl_big.p;
    const uint32_t hx = t.hmax ? t.hmax : cfg.hcap;
    const int ti = k2_tuned_tier(t);
    auto launch = [&](int thr) {
      launch_cluster_bins(cb, hx, thr, cluster_bins_grid(hx, ca.gmax, thr, feat != nullptr, h->num_sms), st);
      h->stats.kernel_launches += 1;
    };
    if (ti < 0) {
      launch(t.threads);
    } else if (T.k2_threads[ti] || T.k2_chosen[ti] || !T.autotune) {
      launch(T.k2_threads[ti] ? T.k2_threads[ti] : (T.k2_chosen[ti] ? T.k2_chosen[ti] : t.threads));
    } else {
      // the tier's first chunk: each block size in turn on the same reads
      // (the outputs are the same), the fastest kept
      cudaEvent_t* e = &h->events[28];
      for (int i = 0; i < 3; i++) {
        CK(cudaEventRecord(e[0], st));
        launch(K2_TRIAL_THREADS[i]);
        CK(cudaEventRecord(e[1], st));
        CK(cudaEventSynchronize(e[1]));
        T.k2_ms[ti][i] = (float)ms_between(e[0], e[1]);
      }
      int best = 0;
      for (int i = 1; i < 3; i++)
        if (T.k2_ms[ti][i] < T.k2_ms[ti][best]) best = i;
      T.k2_chosen[ti] = K2_TRIAL_THREADS[best];
    }
    lo = hm;
  }
  const uint32_t ns = ovf_max_slices(h);
  for (uint32_t s = 0; s < ns; s++) TRY(ovf_slice(h, cfg, bases, offs, r0, nr, rep, s, nullptr, &ca));
  CK(cudaGetLastError());
  return PBW_OK;
}

// K1 -> K2 for reads [r0, r0+nr) of one read set; with feat, also the
// ranker's hit-level candidate features. Events ev[0..2] mark the start and
// the seed / cluster boundaries.
static int seed_cluster(pbw_handle* h, const ChunkCfg& cfg, const uint8_t* bases, const uint8_t* quals,
                        const uint64_t* offs, uint32_t r0, uint32_t nr, const MateBufs& mb, cudaEvent_t* ev,
                        float* feat) {
  cudaStream_t st = h->st;
  CK(cudaMemsetAsync(mb.n_cand, 0, nr * sizeof(uint32_t), st));
  CK(cudaEventRecord(ev[0], st));
  TRY(seed_phase(h, cfg, bases, offs, r0, nr, mb.rep, feat != nullptr, nullptr));
  CK(cudaEventRecord(ev[1], st));
  TRY(cluster_phase(h, cfg, bases, quals, offs, r0, nr, mb.rep, mb.cand, mb.n_cand, h->d_total_cand.p, MAX_CAND,
                    feat));
  CK(cudaGetLastError());
  CK(cudaEventRecord(ev[2], st));
  return PBW_OK;
}

// Keep flags of one read set's candidates from the trained model.
static void rank_decide(pbw_handle* h, const float* feat, float* logit, const MateBufs& mb, uint32_t nr) {
  RankModelDev md{h->rk.d_norm.p, h->rk.d_wb.p, h->rk.d_w.p};
  launch_rank_infer(feat, (uint64_t)nr * MAX_CAND, md, logit, h->num_sms * 8, h->st);
  RankDecideArgs da{};
  da.logit = logit;
  da.feat = feat;
  da.cand = mb.cand;
  da.n_cand = mb.n_cand;
  da.nr = nr;
  da.tau = h->rk.tau;
  da.counters = h->rk.d_counters.p;
  launch_rank_decide(da, h->st);
  h->stats.kernel_launches += 2;
}

// Mate-consistency features of both read sets of a chunk of pairs.
static void rank_mate_features(pbw_handle* h, const MateBufs& m1, const MateBufs& m2, const uint64_t* of1,
                               const uint64_t* of2, uint32_t r0, uint32_t nr, float* f1, float* f2, double mean,
                               double sd) {
  RankMateArgs ma{m1.cand, m1.n_cand, of1, m2.cand, m2.n_cand, of2, r0, nr, mean, sd, f1};
  launch_rank_mate(ma, h->st);
  RankMateArgs mb{m2.cand, m2.n_cand, of2, m1.cand, m1.n_cand, of1, r0, nr, mean, sd, f2};
  launch_rank_mate(mb, h->st);
  h->stats.kernel_launches += 2;
}

// Read-length class of a chunk for the tuned band-DP form.
static int length_class(int lmax) { return lmax <= 128 ? 0 : (lmax <= 256 ? 1 : 2); }

// The seeded band DP in the form chosen for this read-length class: forced
// by pbw_set_tuning, or timed once per class on the class's first chunk --
// the 8-lane form runs, the queue and the counters it moved are put back,
// the 16-lane form (and, for bands of 16 to 31, the 4-lane one) runs on the
// same jobs (same results: the DP is exact), and the fastest is kept for the
// class's later chunks.
static int band_dp(pbw_handle* h, const AlignArgs& aa, const ChunkCfg& cfg) {
  cudaStream_t st = h->st;
  const int band = (int)h->opt.max_indel_len;
  const int cls = length_class(cfg.lmax);
  auto& T = h->tune;
  if (!band_has_lanes16(band)) {
    launch_align_band_lanes(aa, h->num_sms, band, 8, st);
    return PBW_OK;
  }
  if (T.band_lanes == 4 || T.band_lanes == 8 || T.band_lanes == 16) {
    launch_align_band_lanes(aa, h->num_sms, band, T.band_lanes, st);
    return PBW_OK;
  }
  if (T.chosen[cls] || !T.autotune) {
    launch_align_band_lanes(aa, h->num_sms, band, T.chosen[cls] ? T.chosen[cls] : 8, st);
    return PBW_OK;
  }
  unsigned int* c32 = h->d_cnt32.p;
  unsigned long long* c64 = h->d_cnt64.p;
  cudaEvent_t* e = &h->events[24];
  // snapshot: CIGAR pool cursor, DP job and cell counters
  CK(cudaMemcpyAsync(c32 + 12, aa.cig_pool_used, sizeof(unsigned int), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c64 + 12, c64 + 3, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
  CK(cudaEventRecord(e[0], st));
  launch_align_band_lanes(aa, h->num_sms, band, 8, st);
  CK(cudaEventRecord(e[1], st));
  CK(cudaMemsetAsync(aa.next_job, 0, sizeof(unsigned int), st));
  CK(cudaMemcpyAsync(aa.cig_pool_used, c32 + 12, sizeof(unsigned int), cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(c64 + 3, c64 + 12, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
  CK(cudaEventRecord(e[2], st));
  launch_align_band_lanes(aa, h->num_sms, band, 16, st);
  CK(cudaEventRecord(e[3], st));
  CK(cudaGetLastError());
  CK(cudaEventSynchronize(e[3]));
  T.ms[cls][0] = (float)ms_between(e[0], e[1]);
  T.ms[cls][1] = (float)ms_between(e[2], e[3]);
  T.ms[cls][2] = 0.f;
  T.chosen[cls] = T.ms[cls][1] < T.ms[cls][0] ? 16 : 8;
  h->stats.kernel_launches += 1;
  if (band_has_lanes4(band)) {
    CK(cudaMemsetAsync(aa.next_job, 0, sizeof(unsigned int), st));
    CK(cudaMemcpyAsync(aa.cig_pool_used, c32 + 12, sizeof(unsigned int), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(c64 + 3, c64 + 12, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
    CK(cudaEventRecord(e[0], st));
    launch_align_band_lanes(aa, h->num_sms, band, 4, st);
    CK(cudaEventRecord(e[1], st));
    CK(cudaGetLastError());
    CK(cudaEventSynchronize(e[1]));
    T.ms[cls][2] = (float)ms_between(e[0], e[1]);
    if (T.ms[cls][2] < std::min(T.ms[cls][0], T.ms[cls][1])) T.chosen[cls] = 4;
    h->stats.kernel_launches += 1;
  }
  return PBW_OK;
}

// Candidates -> jobs -> K3 -> alignment statistics for one read set (with
// the keep flags when prune), and the training labels when labels is set.
// ev[3] marks the end. reset_pool clears the CIGAR pool (the first read set
// of a chunk).
static int align_candidates(pbw_handle* h, const ChunkCfg& cfg, const uint8_t* bases, const uint8_t* quals,
                            const uint64_t* offs, uint32_t r0, uint32_t nr, const MateBufs& mb, cudaEvent_t* ev,
                            bool reset_pool, bool prune, uint8_t* labels) {
  cudaStream_t st = h->st;
  unsigned int* c32 = h->d_cnt32.p;
  uint32_t* pool = mb.pool ? mb.pool : h->d_cig_pool.p;
  unsigned int* pool_used = mb.pool ? mb.pool_used : c32 + 2;
  const uint32_t pool_cap = mb.pool ? mb.pool_cap : (uint32_t)h->d_cig_pool.cap;
  CK(cudaMemsetAsync(c32, 0, 2 * sizeof(unsigned int), st));  // n_jobs, next_job
  if (reset_pool) CK(cudaMemsetAsync(pool_used, 0, sizeof(unsigned int), st));
  MakeJobsArgs ma{};
  ma.G = h->G;
  ma.offs = offs;
  ma.r0 = r0;
  ma.nr = nr;
  ma.cand = mb.cand;
  ma.n_cand = mb.n_cand;
  ma.right_pad = std::max<uint64_t>(h->opt.max_indel_len, 10);
  ma.band = (uint32_t)h->opt.max_indel_len;
  ma.gap_open = h->tab_host.gap_open;
  ma.gap_extend = h->tab_host.gap_extend;
  ma.jobs = h->d_jobs.p;
  ma.n_jobs = c32 + 0;
  ma.out = mb.aln;
  ma.mate = 0;
  ma.prune = prune ? 1 : 0;
  launch_make_jobs_single(ma, st);
  AlignArgs aa{};
  aa.G = h->G;
  aa.tab = h->d_tab.p;
  aa.gc_lnb = h->d_gc_lnb.p;
  aa.gc_lnbm1 = h->d_gc_lnbm1.p;
  aa.bases = bases;
  aa.quals = quals;
  aa.offs = offs;
  aa.bases2 = bases;
  aa.quals2 = quals;
  aa.offs2 = offs;
  aa.jobs = h->d_jobs.p;
  aa.n_jobs = c32 + 0;
  aa.next_job = c32 + 1;
  aa.out = mb.aln;
  aa.cig_pool = pool;
  aa.cig_pool_used = pool_used;
  aa.cig_pool_cap = pool_cap;
  aa.ref_bytes = nullptr;
  aa.lmax = cfg.lmax;
  aa.nmax = cfg.nmax;
  aa.tb_smem = 0;
  aa.tb_global = h->d_tb_global.p;
  aa.tb_global_per_warp = 0;
  aa.counters = h->d_cnt64.p + 3;
  aa.err = h->d_err.p;
  aa.wait_polls = h->tune.wait_polls;
  if (h->tune.length_bins && cfg.lmin < cfg.lmax) {
    // mixed read lengths: the work queue in length bins, longest first
    launch_job_bins(h->d_jobs.p, c32 + 0, offs, h->d_bins.p, h->d_jobs_b.p, h->num_sms * 4, st);
    aa.jobs = h->d_jobs_b.p;
    h->stats.kernel_launches += 3;
  }
  if (h->opt.max_indel_len <= 31) {
    TRY(band_dp(h, aa, cfg));
  } else {
    aa.tb_global = h->d_tb_global.p;
    aa.tb_global_per_warp = window_slab_bytes(cfg.lmax, cfg.nmax);
    launch_align_window(aa, window_grid(h), st);
  }
  launch_aln_stats(aa, (uint64_t)nr * MAX_CAND, st);
  if (labels) {
    RankLabelArgs la{mb.aln, mb.n_cand, nr, labels, h->rk.label_cut};
    launch_rank_label(la, st);
    h->stats.kernel_launches += 1;
  }
  CK(cudaGetLastError());
  CK(cudaEventRecord(ev[3], st));
  h->stats.kernel_launches += 4;
  return PBW_OK;
}

// K1 -> K2 -> [ranker] -> jobs -> K3 for reads [r0, r0+nr) of one read set
// (the single-end chunk; pairs run the halves separately when ranking).
static int run_seed_align(pbw_handle* h, const ChunkCfg& cfg, const uint8_t* bases, const uint8_t* quals,
                          const uint64_t* offs, uint32_t r0, uint32_t nr, const MateBufs& mb,
                          cudaEvent_t* ev, bool reset_pool) {
  float* feat = rank_feat(h, cfg.ch, 0, r0);
  TRY(seed_cluster(h, cfg, bases, quals, offs, r0, nr, mb, ev, feat));
  const bool prune = h->rk.enabled && !h->rk.collect;
  if (prune) rank_decide(h, feat, h->rk.d_logit.p, mb, nr);
  return align_candidates(h, cfg, bases, quals, offs, r0, nr, mb, ev, reset_pool, prune, rank_label(h, 0, r0));
}

// One chunk of single-end reads: seeding through finalize and CIGAR gather.
// Per-phase event pairs are recorded into ev (5 phases).
static int run_chunk_single(pbw_handle* h, const ChunkCfg& cfg, const uint8_t* bases, const uint8_t* quals,
                            const uint64_t* offs, uint32_t r0, uint32_t nr, cudaEvent_t* ev) {
  cudaStream_t st = h->st;
  unsigned int* c32 = h->d_cnt32.p;
  MateBufs mb{h->d_cand.p, h->d_n_cand.p, h->d_aln.p, h->d_rep.p, 0};
  TRY(run_seed_align(h, cfg, bases, quals, offs, r0, nr, mb, ev, true));
  FinalizeArgs fa{};
  fa.G = h->G;
  fa.tab = h->d_tab.p;
  fa.ln_n = h->d_ln_n.p;
  fa.quals = quals;
  fa.offs = offs;
  fa.r0 = r0;
  fa.nr = nr;
  fa.aln = h->d_aln.p;
  fa.n_cand = h->d_n_cand.p;
  fa.cand = h->d_cand.p;
  fa.rep = h->d_rep.p;
  fa.wcap = cfg.wcap;
  fa.gc_lnb = h->d_gc_lnb.p;
  fa.gc_lnbm1 = h->d_gc_lnbm1.p;
  fa.seed_k = h->seed_k;
  fa.contig = h->o_contig.p + r0;
  fa.pos = h->o_pos.p + r0;
  fa.mapq = h->o_mapq.p + r0;
  fa.flag = h->o_flag.p + r0;
  fa.log_lk = h->o_log_lk.p + r0;
  fa.posterior = h->o_post.p + r0;
  fa.as_score = h->o_as.p + r0;
  fa.nm = h->o_nm.p + r0;
  fa.n_ops = h->o_nops.p + r0;
  fa.best = h->o_best.p + r0;
  launch_finalize(fa, 0, st);
  launch_scan_excl(h->o_nops.p + r0, nr, h->o_cig_off.p + r0, h->d_scan_sums.p, c32 + 4, c32 + 4, st);
  CigarGatherArgs ga{};
  ga.offs = offs;
  ga.r0 = r0;
  ga.nr = nr;
  ga.best = h->o_best.p + r0;
  ga.aln = h->d_aln.p;
  ga.cig_pool = h->d_cig_pool.p;
  ga.cig_off = h->o_cig_off.p + r0;
  ga.cigar = h->o_cigar.p;
  launch_cigar_gather(ga, st);
  CK(cudaGetLastError());
  CK(cudaEventRecord(ev[4], st));
  h->stats.kernel_launches += 4;
  return PBW_OK;
}

static int check_device_errors(pbw_handle* h) {
  int err = 0;
  unsigned int c32[8];
  CK(cudaMemcpy(&err, h->d_err.p, 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(c32, h->d_cnt32.p, sizeof(c32), cudaMemcpyDeviceToHost));
  if (c32[3]) {
    h->err = std::to_string(c32[3]) + " read(s) produced more seed hits than the per-read capacity";
    CK(cudaMemset(h->d_cnt32.p + 3, 0, 4));
    return PBW_ERR_LIMIT;
  }
  if (err == 5) {
    h->err = "seed hits of a chunk's over-capacity reads exceed the overflow pool (16 slices of 16 M hits; "
             "one read at most 16 M hits)";
    CK(cudaMemset(h->d_err.p, 0, 4));
    return PBW_ERR_LIMIT;
  }
  if (err == 3) {
    h->err = "the CIGAR overflow pool of a chunk is full (alignments with very many CIGAR operations)";
    CK(cudaMemset(h->d_err.p, 0, 4));
    return PBW_ERR_CAPACITY;
  }
  if (err == 9) {
    h->err = "a window-DP wavefront wait ran out of polls before its producer published (results discarded)";
    CK(cudaMemset(h->d_err.p, 0, 4));
    return PBW_ERR_DEVICE;
  }
  if (err) {
    h->err = "device kernel reported internal error " + std::to_string(err);
    CK(cudaMemset(h->d_err.p, 0, 4));
    return PBW_ERR_DEVICE;
  }
  return PBW_OK;
}

static int copy_records_out(pbw_handle* h, uint64_t n, pbw_records* out, bool paired_fields) {
  unsigned int total = 0;
  CK(cudaMemcpy(&total, h->d_cnt32.p + 4, 4, cudaMemcpyDeviceToHost));
  if (out->cigar_cap < total) {
    h->err = "cigar_cap " + std::to_string(out->cigar_cap) + " < " + std::to_string(total);
    return PBW_ERR_CAPACITY;
  }
  cudaStream_t st = h->st;
  CK(cudaMemcpyAsync(h->o_cig_off.p + n, h->d_cnt32.p + 4, 4, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(out->contig, h->o_contig.p, n * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->pos, h->o_pos.p, n * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->mapq, h->o_mapq.p, n, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->flag, h->o_flag.p, n * 2, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->log_lk, h->o_log_lk.p, n * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->posterior, h->o_post.p, n * 8, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->as_score, h->o_as.p, n * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->nm, h->o_nm.p, n * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->cigar_off, h->o_cig_off.p, (n + 1) * 4, cudaMemcpyDeviceToHost, st));
  CK(cudaMemcpyAsync(out->cigar, h->o_cigar.p, (size_t)total * 4, cudaMemcpyDeviceToHost, st));
  if (paired_fields) {
    CK(cudaMemcpyAsync(out->mate_contig, h->o_mate_contig.p, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(out->mate_pos, h->o_mate_pos.p, n * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(out->tlen, h->o_tlen.p, n * 8, cudaMemcpyDeviceToHost, st));
  }
  CK(cudaStreamSynchronize(st));
  if (!paired_fields) {
    for (uint64_t i = 0; i < n; i++) {
      out->mate_contig[i] = -1;
      out->mate_pos[i] = 0;
      out->tlen[i] = 0;
    }
  }
  return PBW_OK;
}

static int validate_reads(pbw_handle* h, const pbw_reads* r, uint64_t& total, int& lmax, int* lmin = nullptr) {
  if (!r || (r->n && (!r->offsets))) { h->err = "null reads"; return PBW_ERR_ARG; }
  lmax = 0;
  int lo = PBW_MAX_READ_LEN;
  total = r->n ? r->offsets[r->n] - r->offsets[0] : 0;
  if (r->n && r->offsets[0] != 0) { h->err = "offsets[0] must be 0"; return PBW_ERR_ARG; }
  for (uint64_t i = 0; i < r->n; i++) {
    if (r->offsets[i + 1] < r->offsets[i]) { h->err = "offsets must be non-decreasing"; return PBW_ERR_ARG; }
    uint64_t L = r->offsets[i + 1] - r->offsets[i];
    if (L > PBW_MAX_READ_LEN) {
      h->err = "read " + std::to_string(i) + " longer than PBW_MAX_READ_LEN";
      return PBW_ERR_LIMIT;
    }
    lmax = std::max(lmax, (int)L);
    lo = std::min(lo, (int)L);
  }
  if (lmin) *lmin = r->n ? lo : 0;
  if (r->n >= (1ull << 31)) { h->err = "too many reads in one call"; return PBW_ERR_LIMIT; }
  return PBW_OK;
}

// Map reads whose bases/quals/offsets are already on the device.
static int map_single_dev(pbw_handle* h, const uint8_t* d_bases, const uint8_t* d_quals, const uint64_t* d_offs,
                          uint64_t n, uint64_t total_bases, int lmax, pbw_records* out) {
  ChunkCfg cfg = chunk_cfg(h, n, lmax);
  TRY(ensure_chunk(h, cfg));
  if (h->rk.enabled || h->rk.collect) TRY(ensure_ranker_chunk(h, cfg));
  TRY(ensure_outputs(h, std::max<uint64_t>(n, 1), 2 * total_bases + 2 * n + 16));
  CK(cudaMemsetAsync(h->d_cnt32.p, 0, 16 * sizeof(unsigned int), h->st));
  CK(cudaMemsetAsync(h->d_cnt64.p, 0, 16 * sizeof(unsigned long long), h->st));
  std::vector<std::vector<cudaEvent_t>> evs;
  double t_seed = 0, t_cl = 0, t_al = 0, t_fin = 0;
  cudaEvent_t e0 = h->events[0], e1 = h->events[1];
  CK(cudaEventRecord(e0, h->st));
  int ev_next = 2;
  for (uint64_t r0 = 0; r0 < n; r0 += cfg.ch) {
    uint32_t nr = (uint32_t)std::min<uint64_t>(cfg.ch, n - r0);
    cudaEvent_t* ev = &h->events[ev_next];
    TRY(run_chunk_single(h, cfg, d_bases, d_quals, d_offs, (uint32_t)r0, nr, ev));
    // accumulate phase times once the chunk's events complete (next sync)
    CK(cudaEventSynchronize(ev[4]));
    t_seed += ms_between(ev[0], ev[1]);
    t_cl += ms_between(ev[1], ev[2]);
    t_al += ms_between(ev[2], ev[3]);
    t_fin += ms_between(ev[3], ev[4]);
  }
  CK(cudaEventRecord(e1, h->st));
  CK(cudaStreamSynchronize(h->st));
  TRY(check_device_errors(h));
  h->stats.ms_seed = t_seed;
  h->stats.ms_cluster = t_cl;
  h->stats.ms_align = t_al;
  h->stats.ms_finalize = t_fin;
  unsigned long long c64[8];
  CK(cudaMemcpy(c64, h->d_cnt64.p, sizeof(c64), cudaMemcpyDeviceToHost));
  h->stats.seed_probes = c64[0];
  h->stats.seed_entries = c64[1];
  h->stats.seed_hits = c64[2];
  h->stats.dp_jobs = c64[3];
  h->stats.dp_cells = c64[4];
  cudaEvent_t e2 = h->events[ev_next + 5];
  TRY(copy_records_out(h, n, out, false));
  CK(cudaEventRecord(e2, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->stats.ms_d2h = ms_between(e1, e2);
  set_compute_span(h, e0, e1);
  return PBW_OK;
}

static int upload_reads(pbw_handle* h, const pbw_reads* r, uint64_t total, DevBuf<uint8_t>& db, DevBuf<uint8_t>& dq,
                        DevBuf<uint64_t>& doff) {
  TRY(grow(h, db, total + 16));
  TRY(grow(h, dq, total + 16));
  TRY(grow(h, doff, r->n + 1));
  if (total) {
    CK(cudaMemcpyAsync(db.p, r->bases, total, cudaMemcpyHostToDevice, h->st));
    CK(cudaMemcpyAsync(dq.p, r->quals, total, cudaMemcpyHostToDevice, h->st));
  }
  CK(cudaMemcpyAsync(doff.p, r->offsets, (r->n + 1) * 8, cudaMemcpyHostToDevice, h->st));
  return PBW_OK;
}


// ---------------------------------------------------------------------------
// paired end
// ---------------------------------------------------------------------------
// The schedule of map_paired (src/lib.rs:145-185): pairs 0..499 one at a
// time with the model updated after each, then batches of 2000 against a
// frozen snapshot, observations folded in pair order after each batch.
static std::vector<std::pair<uint64_t, uint64_t>> pair_batches(uint64_t n) {
  std::vector<std::pair<uint64_t, uint64_t>> b;
  const uint64_t warm = std::min<uint64_t>(n, 500);
  for (uint64_t i = 0; i < warm; i++) b.push_back({i, 1});
  for (uint64_t s = warm; s < n; s += 2000) b.push_back({s, std::min<uint64_t>(2000, n - s)});
  return b;
}

// Super-chunks of a paired call: whole batches, at most S pairs; pairs
// [a, b) and batches [bi, be).
struct SuperChunk {
  uint64_t a, b;
  size_t bi, be;
};
static std::vector<SuperChunk> pair_super_chunks(const std::vector<std::pair<uint64_t, uint64_t>>& batches,
                                                 uint64_t S) {
  std::vector<SuperChunk> out;
  size_t bi = 0;
  while (bi < batches.size()) {
    const uint64_t a = batches[bi].first;
    size_t be = bi;
    uint64_t b = a;
    while (be < batches.size() && batches[be].first + batches[be].second - a <= S) {
      b = batches[be].first + batches[be].second;
      be++;
    }
    out.push_back({a, b, bi, be});
    bi = be;
  }
  return out;
}
static uint64_t pair_super_chunk_pairs(const pbw_handle* h) { return std::max<uint64_t>(h->opt.chunk_reads, 2000); }

// up_ev: when the reads are still being copied up, event k marks the reads
// of super-chunk k on the device (the compute stream waits for it).
static int map_paired_dev(pbw_handle* h, pbw_insert_model* model, const uint8_t* b1, const uint8_t* q1,
                          const uint64_t* of1, const uint8_t* b2, const uint8_t* q2, const uint64_t* of2, uint64_t n,
                          uint64_t tot1, uint64_t tot2, int lmax, pbw_records* o1, pbw_records* o2,
                          const std::vector<cudaEvent_t>* up_ev) {
  cudaStream_t st = h->st;
  if (!h->st_pair) CK(cudaStreamCreateWithFlags(&h->st_pair, cudaStreamNonBlocking));
  cudaStream_t sp = h->st_pair;
  const auto batches = pair_batches(n);
  // super-chunks: whole batches, at most chunk_reads pairs
  const uint64_t S = pair_super_chunk_pairs(h);
  const std::vector<SuperChunk> chunks = pair_super_chunks(batches, S);
  if (up_ev && up_ev->size() < chunks.size()) {
    h->err = "internal: fewer upload events than super-chunks";
    return PBW_ERR_ARG;
  }
  ChunkCfg cfg = chunk_cfg(h, std::min<uint64_t>(n, S), lmax);
  cfg.ch = (uint32_t)std::min<uint64_t>(n, S);
  TRY(ensure_chunk(h, cfg));
  if (h->rk.enabled || h->rk.collect) TRY(ensure_ranker_chunk(h, cfg));
  const uint32_t ch = cfg.ch;
  // Two buffer sets: super-chunk k's candidates, alignments, repeat marks,
  // read summaries and CIGAR pool live in set k % 2, so that k + 1 can be
  // seeded and aligned (stream st) while k's pair batches run (stream sp).
  const size_t pool_ops = (size_t)ch * (2 * MAX_CAND + MAX_CROSS) * 16 + 4096;
  TRY(grow(h, h->d_cand, 2 * (size_t)ch * MAX_CAND));
  TRY(grow(h, h->d_n_cand, 2 * (size_t)ch));
  TRY(grow(h, h->d_aln, 2 * (size_t)ch * MAX_CAND));
  TRY(grow(h, h->d_rep, 2 * (size_t)ch * cfg.wcap));
  TRY(grow(h, h->d_cand2, 2 * (size_t)ch * MAX_CAND));
  TRY(grow(h, h->d_n_cand2, 2 * (size_t)ch));
  TRY(grow(h, h->d_aln2, 2 * (size_t)ch * MAX_CAND));
  TRY(grow(h, h->d_rep2, 2 * (size_t)ch * cfg.wcap));
  TRY(grow(h, h->d_sum, 4 * (size_t)ch));
  TRY(grow(h, h->d_cig_pool, 2 * pool_ops));
  TRY(grow(h, h->d_work, ch));
  TRY(grow(h, h->d_xout, (size_t)ch * MAX_CROSS));
  TRY(grow(h, h->d_xmeta, (size_t)ch * MAX_CROSS));
  TRY(grow(h, h->d_xjobs, (size_t)2000 * MAX_CROSS));
  TRY(grow(h, h->d_obs, ch));
  TRY(grow(h, h->d_model, 1));
  const uint64_t n2 = 2 * n;
  TRY(ensure_outputs(h, std::max<uint64_t>(n2, 1), 2 * tot1 + 2 * n + 16));
  TRY(grow(h, h->o_cig_off2, n + 1));
  TRY(grow(h, h->o_cigar2, 2 * tot2 + 2 * n + 16));
  TRY(grow(h, h->o_cigsrc, std::max<uint64_t>(n2, 1)));
  TRY(grow(h, h->o_len, std::max<uint64_t>(n2, 1)));
  // wide DP: window = L + 2 * (ceil(5 sd) + L); slabs sized for 8192 columns
  const int wide_n = 8192;
  const int grid_w = window_grid(h);
  // the pair batches' window DP has a traceback slab of its own (the next
  // super-chunk's seeded DP uses d_tb_global meanwhile)
  TRY(grow(h, h->d_tb_pair, window_slab_bytes(cfg.lmax, wide_n) * (size_t)grid_w));
  PairModel pm;
  pm.mean = model->mean;
  pm.sd = model->sd;
  pm.n = model->n_observed;
  pm.ln_2pi_sd2 = std::log(2.0 * 3.141592653589793 * pm.sd * pm.sd);
  if (!h->h_fold.ensure(sizeof(PairModel) + 2000 * sizeof(double) + 16)) {
    h->err = "cudaMallocHost failed";
    return PBW_ERR_NOMEM;
  }
  PairModel* h_pm = (PairModel*)h->h_fold.p;
  double* h_obs = (double*)((char*)h->h_fold.p + sizeof(PairModel));
  uint32_t* h_batch = (uint32_t*)((char*)h->h_fold.p + sizeof(PairModel) + 2000 * sizeof(double));
  *h_pm = pm;
  unsigned int* c32 = h->d_cnt32.p;
  CK(cudaMemcpyAsync(h->d_model.p, h_pm, sizeof(pm), cudaMemcpyHostToDevice, st));
  CK(cudaMemsetAsync(c32, 0, 16 * sizeof(unsigned int), st));
  CK(cudaMemsetAsync(h->d_cnt64.p, 0, 16 * sizeof(unsigned long long), st));
  // events: [0] start; per set s at 1 + 12 s: phase A of mate 1 (4), mate 2
  // (4), pair batches start / end, gather end, phase A end
  cudaEvent_t* E = &h->events[32];
  auto evA1 = [&](int s) { return E + 1 + 12 * s; };
  auto evA2 = [&](int s) { return E + 5 + 12 * s; };
  auto evB = [&](int s) { return E + 9 + 12 * s; };  // 0 batches start, 1 batches end, 2 gather end
  auto evAdone = [&](int s) { return E[12 + 12 * s]; };
  CK(cudaEventRecord(E[0], st));
  double t_seed = 0, t_cl = 0, t_al = 0, t_pair = 0, t_fin = 0;
  const bool ranked = h->rk.enabled || h->rk.collect;
  auto mates = [&](int s, MateBufs& m1, MateBufs& m2) {
    const size_t cs = (size_t)s * ch * MAX_CAND, rs = (size_t)s * ch, ws = (size_t)s * ch * cfg.wcap;
    m1 = MateBufs{h->d_cand.p + cs, h->d_n_cand.p + rs, h->d_aln.p + cs, h->d_rep.p + ws, 0};
    m2 = MateBufs{h->d_cand2.p + cs, h->d_n_cand2.p + rs, h->d_aln2.p + cs, h->d_rep2.p + ws, 0};
    m1.pool = m2.pool = h->d_cig_pool.p + (size_t)s * pool_ops;
    m1.pool_used = m2.pool_used = c32 + (s ? 10 : 2);
    m1.pool_cap = m2.pool_cap = (uint32_t)pool_ops;
  };
  auto collect_times_A = [&](int s) {
    cudaEvent_t* e1 = evA1(s);
    cudaEvent_t* e2 = evA2(s);
    t_seed += ms_between(e1[0], e1[1]) + ms_between(e2[0], e2[1]);
    t_cl += ms_between(e1[1], e1[2]) + ms_between(e2[1], e2[2]);
    t_al += ranked ? ms_between(e2[2], e2[3]) : ms_between(e1[2], e1[3]) + ms_between(e2[2], e2[3]);
  };
  // phase A of super-chunk k on st: both mates through K1-K3 and the read
  // summaries. The ranker's mate feature uses the insert model the host holds
  // when k is enqueued (after the batches of super-chunk k - 2).
  auto phase_A = [&](size_t k) -> int {
    const int s = (int)(k & 1);
    const uint64_t a = chunks[k].a;
    const uint32_t nr = (uint32_t)(chunks[k].b - a);
    if (up_ev) CK(cudaStreamWaitEvent(st, (*up_ev)[k], 0));
    if (k >= 2) CK(cudaStreamWaitEvent(st, evB(s)[2], 0));  // k - 2 is done with set s
    MateBufs m1, m2;
    mates(s, m1, m2);
    if (!ranked) {
      TRY(run_seed_align(h, cfg, b1, q1, of1, (uint32_t)a, nr, m1, evA1(s), true));
      TRY(run_seed_align(h, cfg, b2, q2, of2, (uint32_t)a, nr, m2, evA2(s), false));
    } else {
      // ranker: both read sets' candidates first (the mate features need
      // both), then pruning and the seeded DP of each read set
      float* f1 = rank_feat(h, ch, 0, (uint32_t)a);
      float* f2 = rank_feat(h, ch, 1, (uint32_t)a);
      TRY(seed_cluster(h, cfg, b1, q1, of1, (uint32_t)a, nr, m1, evA1(s), f1));
      TRY(seed_cluster(h, cfg, b2, q2, of2, (uint32_t)a, nr, m2, evA2(s), f2));
      rank_mate_features(h, m1, m2, of1, of2, (uint32_t)a, nr, f1, f2, h_pm->mean, h_pm->sd);
      const bool prune = h->rk.enabled && !h->rk.collect;
      if (prune) {
        rank_decide(h, f1, h->rk.d_logit.p, m1, nr);
        rank_decide(h, f2, h->rk.d_logit.p + (size_t)ch * MAX_CAND, m2, nr);
      }
      TRY(align_candidates(h, cfg, b1, q1, of1, (uint32_t)a, nr, m1, evA1(s), true, prune,
                           rank_label(h, 0, (uint32_t)a)));
      TRY(align_candidates(h, cfg, b2, q2, of2, (uint32_t)a, nr, m2, evA2(s), false, prune,
                           rank_label(h, 1, (uint32_t)a)));
    }
    for (int mate = 0; mate < 2; mate++) {
      ReadSummaryArgs ra{};
      ra.tab = h->d_tab.p;
      ra.ln_n = h->d_ln_n.p;
      ra.gc_lnb = h->d_gc_lnb.p;
      ra.gc_lnbm1 = h->d_gc_lnbm1.p;
      ra.quals = mate ? q2 : q1;
      ra.offs = mate ? of2 : of1;
      ra.r0 = (uint32_t)a;
      ra.nr = nr;
      ra.aln = mate ? m2.aln : m1.aln;
      ra.n_cand = mate ? m2.n_cand : m1.n_cand;
      ra.rep = mate ? m2.rep : m1.rep;
      ra.wcap = cfg.wcap;
      ra.sum = h->d_sum.p + (size_t)(2 * s + mate) * ch;
      launch_read_summary(ra, st);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(evAdone(s), st));
    return PBW_OK;
  };
  // phase B of super-chunk k on sp: the pair batches in order (each batch's
  // observations folded into the model on the host before the next), then
  // the super-chunk's packed CIGARs.
  auto phase_B = [&](size_t k) -> int {
    const int s = (int)(k & 1);
    const uint64_t a = chunks[k].a, b = chunks[k].b;
    const size_t bi = chunks[k].bi, be = chunks[k].be;
    const uint32_t nr = (uint32_t)(b - a);
    MateBufs m1, m2;
    mates(s, m1, m2);
    CK(cudaStreamWaitEvent(sp, evAdone(s), 0));
    CK(cudaEventRecord(evB(s)[0], sp));
    PairArgs pa{};
    pa.G = h->G;
    pa.tab = h->d_tab.p;
    pa.ln_n = h->d_ln_n.p;
    pa.gc_lnb = h->d_gc_lnb.p;
    pa.gc_lnbm1 = h->d_gc_lnbm1.p;
    pa.offs1 = of1;
    pa.offs2 = of2;
    pa.read0 = (uint32_t)a;
    pa.sum[0] = h->d_sum.p + (size_t)(2 * s) * ch;
    pa.sum[1] = h->d_sum.p + (size_t)(2 * s + 1) * ch;
    pa.aln[0] = m1.aln;
    pa.aln[1] = m2.aln;
    pa.cand[0] = m1.cand;
    pa.cand[1] = m2.cand;
    pa.work = h->d_work.p;
    pa.model = h->d_model.p;
    pa.sv_prior_log_prob = h->tab_host.sv_prior_log_prob;
    pa.gap_open = h->tab_host.gap_open;
    pa.gap_extend = h->tab_host.gap_extend;
    pa.jobs = h->d_xjobs.p;
    pa.n_jobs = c32 + 8;
    pa.xout = h->d_xout.p;
    pa.xmeta = h->d_xmeta.p;
    pa.obs = h->d_obs.p;
    pa.out_base = a;
    pa.n_total = n;
    pa.o_contig = h->o_contig.p;
    pa.o_pos = h->o_pos.p;
    pa.o_mapq = h->o_mapq.p;
    pa.o_flag = h->o_flag.p;
    pa.o_mate_contig = h->o_mate_contig.p;
    pa.o_mate_pos = h->o_mate_pos.p;
    pa.o_tlen = h->o_tlen.p;
    pa.o_log_lk = h->o_log_lk.p;
    pa.o_post = h->o_post.p;
    pa.o_as = h->o_as.p;
    pa.o_nm = h->o_nm.p;
    pa.o_nops = h->o_nops.p;
    pa.o_cigsrc = h->o_cigsrc.p;
    pa.o_len = h->o_len.p;
    AlignArgs aa{};
    aa.G = h->G;
    aa.tab = h->d_tab.p;
    aa.gc_lnb = h->d_gc_lnb.p;
    aa.gc_lnbm1 = h->d_gc_lnbm1.p;
    aa.bases = b1;
    aa.quals = q1;
    aa.offs = of1;
    aa.bases2 = b2;
    aa.quals2 = q2;
    aa.offs2 = of2;
    aa.jobs = h->d_xjobs.p;
    aa.n_jobs = c32 + 8;
    aa.next_job = c32 + 9;
    aa.out = h->d_xout.p;
    aa.cig_pool = m1.pool;
    aa.cig_pool_used = m1.pool_used;
    aa.cig_pool_cap = m1.pool_cap;
    aa.ref_bytes = nullptr;
    aa.lmax = cfg.lmax;
    aa.nmax = wide_n;
    aa.tb_smem = 0;
    aa.tb_global = h->d_tb_pair.p;
    aa.tb_global_per_warp = window_slab_bytes(cfg.lmax, wide_n);
    aa.counters = h->d_cnt64.p + 5;  // cross-alignment jobs and cells, apart from the seeded DP's
    aa.err = h->d_err.p;
    aa.wait_polls = h->tune.wait_polls;
    // One batch: decide -> cross-alignment DP -> statistics -> resolve, its
    // observations to the host, the fold there (the model of the next batch).
    // With pair_graphs the device side is captured once per super-chunk as a
    // CUDA graph that reads the batch from device memory ({p0, np}, copied
    // from pinned memory by the graph's first nodes with the model) and is
    // replayed per batch; a capture the runtime refuses falls back to the
    // launches below.
    cudaGraphExec_t gexec = nullptr;
    if (h->tune.pair_graphs) {
      TRY(grow(h, h->d_batch, 2));
      TRY(grow(h, h->d_obs_batch, 2000));
      PairArgs pg = pa;
      pg.batch = h->d_batch.p;
      pg.obs_batch = h->d_obs_batch.p;
      pg.np = 2000;
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(sp, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        cudaMemcpyAsync(h->d_model.p, h_pm, sizeof(PairModel), cudaMemcpyHostToDevice, sp);
        cudaMemcpyAsync(h->d_batch.p, h_batch, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, sp);
        cudaMemsetAsync(c32 + 8, 0, 2 * sizeof(unsigned int), sp);
        launch_pair_decide(pg, sp);
        launch_align_window(aa, grid_w, sp, true);
        launch_aln_stats(aa, (uint64_t)2000 * MAX_CROSS, sp);
        launch_pair_resolve(pg, sp);
        cudaMemcpyAsync(h_obs, h->d_obs_batch.p, 2000 * sizeof(double), cudaMemcpyDeviceToHost, sp);
        const cudaError_t ec = cudaStreamEndCapture(sp, &graph);
        if (ec != cudaSuccess || !graph || cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) gexec = nullptr;
        if (graph) cudaGraphDestroy(graph);
      }
      cudaGetLastError();  // a refused capture leaves no sticky error
    }
    for (size_t q = bi; q < be; q++) {
      pa.p0 = (uint32_t)(batches[q].first - a);
      pa.np = (uint32_t)batches[q].second;
      if (gexec) {
        h_batch[0] = pa.p0;
        h_batch[1] = pa.np;
        CK(cudaGraphLaunch(gexec, sp));
        CK(cudaStreamSynchronize(sp));
        fold_insert_model(pm, h_obs, pa.np);
        *h_pm = pm;
        h->stats.kernel_launches += 4;
        continue;
      }
      CK(cudaMemsetAsync(c32 + 8, 0, 2 * sizeof(unsigned int), sp));
      launch_pair_decide(pa, sp);
      const int gw = (int)std::min<uint64_t>((uint64_t)grid_w, (uint64_t)pa.np * MAX_CROSS);
      launch_align_window(aa, std::max(gw, 1), sp, true);
      launch_aln_stats(aa, (uint64_t)pa.np * MAX_CROSS, sp);
      launch_pair_resolve(pa, sp);
      // the next batch sees the model updated by this batch's observations
      CK(cudaMemcpyAsync(h_obs, h->d_obs.p + pa.p0, (size_t)pa.np * sizeof(double), cudaMemcpyDeviceToHost, sp));
      CK(cudaStreamSynchronize(sp));
      fold_insert_model(pm, h_obs, pa.np);
      *h_pm = pm;
      CK(cudaMemcpyAsync(h->d_model.p, h_pm, sizeof(PairModel), cudaMemcpyHostToDevice, sp));
      h->stats.kernel_launches += 4;
    }
    if (gexec) {
      // the model the graph path left on the host goes to the device for the
      // next super-chunk's direct launches, if any
      CK(cudaMemcpyAsync(h->d_model.p, h_pm, sizeof(PairModel), cudaMemcpyHostToDevice, sp));
      cudaGraphExecDestroy(gexec);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(evB(s)[1], sp));
    // packed CIGARs of this super-chunk's records, mate 1 then mate 2
    launch_scan_excl(h->o_nops.p + a, nr, h->o_cig_off.p + a, h->d_scan_sums.p, c32 + 4, c32 + 4, sp);
    launch_pair_cigar_gather(pa, h->o_cig_off.p, m1.pool, h->o_cigar.p, a, nr, sp);
    // mate 2 records live at n + pair; their offsets go to o_cig_off2
    {
      PairArgs pb = pa;
      pb.o_cigsrc = h->o_cigsrc.p + n;
      pb.o_len = h->o_len.p + n;
      launch_scan_excl(h->o_nops.p + n + a, nr, h->o_cig_off2.p + a, h->d_scan_sums.p, c32 + 5, c32 + 5, sp);
      launch_pair_cigar_gather(pb, h->o_cig_off2.p, m1.pool, h->o_cigar2.p, a, nr, sp);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(evB(s)[2], sp));
    return PBW_OK;
  };
  for (size_t k = 0; k < chunks.size(); k++) {
    if (k >= 2) {
      // the set's previous super-chunk is through both phases: its times
      CK(cudaEventSynchronize(evB((int)(k & 1))[2]));
      collect_times_A((int)(k & 1));
      t_pair += ms_between(evB((int)(k & 1))[0], evB((int)(k & 1))[1]);
      t_fin += ms_between(evB((int)(k & 1))[1], evB((int)(k & 1))[2]);
    }
    TRY(phase_A(k));
    if (k >= 1) TRY(phase_B(k - 1));
  }
  TRY(phase_B(chunks.size() - 1));
  CK(cudaStreamSynchronize(sp));
  CK(cudaStreamSynchronize(st));
  for (size_t k = chunks.size() >= 2 ? chunks.size() - 2 : 0; k < chunks.size(); k++) {
    const int s = (int)(k & 1);
    collect_times_A(s);
    t_pair += ms_between(evB(s)[0], evB(s)[1]);
    t_fin += ms_between(evB(s)[1], evB(s)[2]);
  }
  set_compute_span(h, E[0], evB((int)((chunks.size() - 1) & 1))[2]);
  TRY(check_device_errors(h));
  h->stats.ms_seed = t_seed;
  h->stats.ms_cluster = t_cl;
  h->stats.ms_align = t_al;
  h->stats.ms_pair = t_pair;
  h->stats.ms_finalize = t_fin;
  unsigned long long c64[8];
  CK(cudaMemcpy(c64, h->d_cnt64.p, sizeof(c64), cudaMemcpyDeviceToHost));
  h->stats.seed_probes = c64[0];
  h->stats.seed_entries = c64[1];
  h->stats.seed_hits = c64[2];
  h->stats.dp_jobs = c64[3] + c64[5];
  h->stats.dp_cells = c64[4] + c64[6];
  h->stats.window_jobs = c64[5];
  h->stats.window_cells = c64[6];
  // outputs
  unsigned int tot[2];
  CK(cudaMemcpy(tot, c32 + 4, 8, cudaMemcpyDeviceToHost));
  if (o1->cigar_cap < tot[0] || o2->cigar_cap < tot[1]) {
    h->err = "cigar_cap too small";
    return PBW_ERR_CAPACITY;
  }
  cudaEvent_t e1 = h->events[20], e2 = h->events[21];
  CK(cudaEventRecord(e1, st));
  CK(cudaMemcpyAsync(h->o_cig_off.p + n, c32 + 4, 4, cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(h->o_cig_off2.p + n, c32 + 5, 4, cudaMemcpyDeviceToDevice, st));
  pbw_records* outs[2] = {o1, o2};
  for (int k = 0; k < 2; k++) {
    pbw_records* o = outs[k];
    const uint64_t g = (uint64_t)k * n;
    CK(cudaMemcpyAsync(o->contig, h->o_contig.p + g, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->pos, h->o_pos.p + g, n * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->mapq, h->o_mapq.p + g, n, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->flag, h->o_flag.p + g, n * 2, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->mate_contig, h->o_mate_contig.p + g, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->mate_pos, h->o_mate_pos.p + g, n * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->tlen, h->o_tlen.p + g, n * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->log_lk, h->o_log_lk.p + g, n * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->posterior, h->o_post.p + g, n * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->as_score, h->o_as.p + g, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->nm, h->o_nm.p + g, n * 4, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(o->cigar_off, (k ? h->o_cig_off2.p : h->o_cig_off.p), (n + 1) * 4, cudaMemcpyDeviceToHost,
                       st));
    CK(cudaMemcpyAsync(o->cigar, (k ? h->o_cigar2.p : h->o_cigar.p), (size_t)tot[k] * 4, cudaMemcpyDeviceToHost,
                       st));
  }
  CK(cudaEventRecord(e2, st));
  CK(cudaStreamSynchronize(st));
  h->stats.ms_d2h = ms_between(e1, e2);
  model->mean = pm.mean;
  model->sd = pm.sd;
  model->n_observed = pm.n;
  return PBW_OK;
}
}  // namespace pbw

using namespace pbw;

extern "C" {

int pbw_map_single(pbw_handle* h, const pbw_reads* reads, pbw_records* out) {
  if (!h || !reads || !out) return PBW_ERR_ARG;
  if (out->n < reads->n) { h->err = "records array smaller than reads"; return PBW_ERR_CAPACITY; }
  cudaSetDevice(h->device);
  h->stats = pbw_stats{};
  uint64_t total;
  int lmax, lmin;
  TRY(validate_reads(h, reads, total, lmax, &lmin));
  h->call_lmin = lmin;
  if (reads->n == 0) {
    if (out->cigar_off) out->cigar_off[0] = 0;
    return PBW_OK;
  }
  cudaEvent_t a = h->events[30], b = h->events[31];
  CK(cudaEventRecord(a, h->st));
  TRY(upload_reads(h, reads, total, h->d_bases, h->d_quals, h->d_offs));
  CK(cudaEventRecord(b, h->st));
  TRY(map_single_dev(h, h->d_bases.p, h->d_quals.p, h->d_offs.p, reads->n, total, lmax, out));
  h->stats.ms_h2d = ms_between(a, b);
  h->stats.ms_total = h->stats.ms_h2d + h->stats.ms_seed + h->stats.ms_cluster + h->stats.ms_align +
                      h->stats.ms_finalize + h->stats.ms_d2h;
  return PBW_OK;
}


int pbw_map_paired(pbw_handle* h, pbw_insert_model* model, const pbw_reads* r1, const pbw_reads* r2,
                   pbw_records* o1, pbw_records* o2) {
  if (!h || !model || !r1 || !r2 || !o1 || !o2) return PBW_ERR_ARG;
  cudaSetDevice(h->device);
  h->stats = pbw_stats{};
  if (r1->n != r2->n) {
    h->err = "paired-end inputs have different read counts (" + std::to_string(r1->n) + " vs " +
             std::to_string(r2->n) + ")";
    return PBW_ERR_ARG;
  }
  if (o1->n < r1->n || o2->n < r2->n) { h->err = "records array smaller than reads"; return PBW_ERR_CAPACITY; }
  uint64_t t1, t2;
  int l1, l2, m1, m2;
  TRY(validate_reads(h, r1, t1, l1, &m1));
  TRY(validate_reads(h, r2, t2, l2, &m2));
  h->call_lmin = std::min(m1, m2);
  const uint64_t n = r1->n;
  if (n == 0) {
    if (o1->cigar_off) o1->cigar_off[0] = 0;
    if (o2->cigar_off) o2->cigar_off[0] = 0;
    return PBW_OK;
  }
  // The reads go up on a copy stream one super-chunk at a time (the offsets
  // with the first), so that super-chunk k + 1 is copied while k is mapped;
  // each super-chunk's seeding waits for its event.
  TRY(grow(h, h->d_bases, t1 + 16));
  TRY(grow(h, h->d_quals, t1 + 16));
  TRY(grow(h, h->d_offs, n + 1));
  TRY(grow(h, h->d_bases2, t2 + 16));
  TRY(grow(h, h->d_quals2, t2 + 16));
  TRY(grow(h, h->d_offs2, n + 1));
  if (!h->st_up) CK(cudaStreamCreateWithFlags(&h->st_up, cudaStreamNonBlocking));
  const std::vector<SuperChunk> chunks = pair_super_chunks(pair_batches(n), pair_super_chunk_pairs(h));
  while (h->up_ev.size() < chunks.size()) {
    cudaEvent_t e;
    CK(cudaEventCreate(&e));
    h->up_ev.push_back(e);
  }
  cudaEvent_t a = h->events[30];
  CK(cudaEventRecord(a, h->st));
  CK(cudaStreamWaitEvent(h->st_up, a, 0));
  cudaStream_t su = h->st_up;
  CK(cudaMemcpyAsync(h->d_offs.p, r1->offsets, (n + 1) * 8, cudaMemcpyHostToDevice, su));
  CK(cudaMemcpyAsync(h->d_offs2.p, r2->offsets, (n + 1) * 8, cudaMemcpyHostToDevice, su));
  for (size_t k = 0; k < chunks.size(); k++) {
    const pbw_reads* rr[2] = {r1, r2};
    uint8_t* db[2] = {h->d_bases.p, h->d_bases2.p};
    uint8_t* dq[2] = {h->d_quals.p, h->d_quals2.p};
    for (int m = 0; m < 2; m++) {
      const uint64_t x0 = rr[m]->offsets[chunks[k].a], x1 = rr[m]->offsets[chunks[k].b];
      if (x1 > x0) {
        CK(cudaMemcpyAsync(db[m] + x0, rr[m]->bases + x0, x1 - x0, cudaMemcpyHostToDevice, su));
        CK(cudaMemcpyAsync(dq[m] + x0, rr[m]->quals + x0, x1 - x0, cudaMemcpyHostToDevice, su));
      }
    }
    CK(cudaEventRecord(h->up_ev[k], su));
  }
  const int rc = map_paired_dev(h, model, h->d_bases.p, h->d_quals.p, h->d_offs.p, h->d_bases2.p, h->d_quals2.p,
                                h->d_offs2.p, n, t1, t2, std::max(l1, l2), o1, o2, &h->up_ev);
  // no copy of the caller's reads is in flight when the call returns (after
  // a success they have all landed already: every super-chunk waited for them)
  cudaStreamSynchronize(su);
  if (rc != PBW_OK) return rc;
  // copy time the mapping could not hide (until the first super-chunk was
  // up), and the whole call from the first copy to the last record read back
  h->stats.ms_h2d = ms_between(a, h->up_ev[0]);
  h->stats.ms_total = ms_between(a, h->events[21]);
  return PBW_OK;
}

int pbw_map_single_device(pbw_handle* h, const pbw_reads* dev_reads, pbw_records* out) {
  if (!h || !dev_reads || !out) return PBW_ERR_ARG;
  cudaSetDevice(h->device);
  h->stats = pbw_stats{};
  const uint64_t n = dev_reads->n;
  if (out->n < n) { h->err = "records array smaller than reads"; return PBW_ERR_CAPACITY; }
  if (n == 0) return PBW_OK;
  // read lengths are needed for sizing: one small copy of the offsets
  std::vector<uint64_t> offs(n + 1);
  CK(cudaMemcpy(offs.data(), dev_reads->offsets, (n + 1) * 8, cudaMemcpyDeviceToHost));
  pbw_reads hr{n, nullptr, nullptr, offs.data()};
  uint64_t total;
  int lmax, lmin;
  TRY(validate_reads(h, &hr, total, lmax, &lmin));
  h->call_lmin = lmin;
  TRY(map_single_dev(h, dev_reads->bases, dev_reads->quals, dev_reads->offsets, n, total, lmax, out));
  h->stats.ms_total = h->stats.ms_seed + h->stats.ms_cluster + h->stats.ms_align + h->stats.ms_finalize +
                      h->stats.ms_d2h;
  return PBW_OK;
}

int pbw_align_batch(pbw_handle* h, uint64_t n, const uint8_t* reads, const uint8_t* quals, const uint64_t* read_off,
                    const uint8_t* refs, const uint64_t* ref_off, const int64_t* hint, const uint64_t* band,
                    int32_t* score, uint64_t* offset, uint32_t* cigar_off, uint32_t* cigar, uint64_t cigar_cap) {
  if (!h) return PBW_ERR_ARG;
  cudaSetDevice(h->device);
  if (n == 0) {
    if (cigar_off) cigar_off[0] = 0;
    return PBW_OK;
  }
  const uint64_t qtot = read_off[n], rtot = ref_off[n];
  int lmax = 0, nmax = 0;
  for (uint64_t i = 0; i < n; i++) {
    lmax = std::max<int>(lmax, (int)(read_off[i + 1] - read_off[i]));
    nmax = std::max<int>(nmax, (int)(ref_off[i + 1] - ref_off[i]));
  }
  if (lmax > PBW_MAX_READ_LEN || nmax > 16384) { h->err = "problem larger than the device limits"; return PBW_ERR_LIMIT; }
  TRY(grow(h, h->d_bases, qtot + 16));
  TRY(grow(h, h->d_quals, qtot + 16));
  TRY(grow(h, h->d_offs, n + 1));
  TRY(grow(h, h->d_bases2, rtot + 16));
  TRY(grow(h, h->d_jobs, n));
  TRY(grow(h, h->d_aln, n));
  TRY(grow(h, h->d_cig_pool, (size_t)(qtot + rtot) * 2 + 64));
  CK(cudaMemcpy(h->d_bases.p, reads, qtot, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_quals.p, quals, qtot, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_offs.p, read_off, (n + 1) * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_bases2.p, refs, rtot, cudaMemcpyHostToDevice));
  // band <= 31: anti-diagonal band kernel; wider: window kernel (column tiles)
  std::vector<AlnJob> js, jw;
  int lmax_s = 1, nmax_s = 1, lmax_w = 1, nmax_w = 1, bmax_s = 0;
  for (uint64_t i = 0; i < n; i++) {
    AlnJob J;
    memset(&J, 0, sizeof(J));
    J.ref_start = ref_off[i];
    J.ref_end = ref_off[i + 1];
    J.hint = hint[i];
    J.read = (uint32_t)i;
    J.slot = (uint32_t)i;
    J.band = (uint32_t)std::min<uint64_t>(band[i], 1ull << 30);
    J.valid = 1;
    J.gap_open = h->tab_host.gap_open;
    J.gap_extend = h->tab_host.gap_extend;
    const int m = (int)(read_off[i + 1] - read_off[i]);
    const int nn = (int)(ref_off[i + 1] - ref_off[i]);
    // K3b holds the read and window of four alignments per warp in shared
    // memory: bands <= 31 over windows of at most 1280 columns
    if (band[i] <= 31 && nn <= 1280) {
      js.push_back(J);
      lmax_s = std::max(lmax_s, m);
      nmax_s = std::max(nmax_s, nn);
      bmax_s = std::max(bmax_s, (int)band[i]);
    } else {
      jw.push_back(J);
      lmax_w = std::max(lmax_w, m);
      nmax_w = std::max(nmax_w, nn);
    }
  }
  CK(cudaMemset(h->d_err.p, 0, 4));
  AlignArgs aa{};
  aa.G = h->G;
  aa.tab = h->d_tab.p;
  aa.gc_lnb = h->d_gc_lnb.p;
  aa.gc_lnbm1 = h->d_gc_lnbm1.p;
  aa.bases = h->d_bases.p;
  aa.quals = h->d_quals.p;
  aa.offs = h->d_offs.p;
  aa.bases2 = h->d_bases.p;
  aa.quals2 = h->d_quals.p;
  aa.offs2 = h->d_offs.p;
  aa.out = h->d_aln.p;
  aa.cig_pool = h->d_cig_pool.p;
  aa.cig_pool_used = h->d_cnt32.p + 2;
  aa.cig_pool_cap = (uint32_t)h->d_cig_pool.cap;
  aa.ref_bytes = h->d_bases2.p;
  aa.counters = h->d_cnt64.p + 3;
  aa.err = h->d_err.p;
  aa.wait_polls = h->tune.wait_polls;
  CK(cudaMemset(h->d_cnt32.p, 0, 16 * 4));
  if (!js.empty()) {
    CK(cudaMemcpy(h->d_jobs.p, js.data(), js.size() * sizeof(AlnJob), cudaMemcpyHostToDevice));
    unsigned int cnt = (unsigned int)js.size();
    CK(cudaMemcpy(h->d_cnt32.p + 0, &cnt, 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(h->d_cnt32.p + 1, 0, 4));
    aa.jobs = h->d_jobs.p;
    aa.n_jobs = h->d_cnt32.p + 0;
    aa.next_job = h->d_cnt32.p + 1;
    aa.lmax = lmax_s;
    aa.nmax = nmax_s;
    aa.tb_smem = 0;
    TRY(grow(h, h->d_tb_global, band_tb_slab_bytes(lmax_s, nmax_s, h->num_sms, bmax_s)));
    aa.tb_global = h->d_tb_global.p;
    aa.tb_global_per_warp = 0;
    launch_align_band(aa, h->num_sms, bmax_s, h->st);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
  }
  if (!jw.empty()) {
    CK(cudaMemcpy(h->d_jobs.p, jw.data(), jw.size() * sizeof(AlnJob), cudaMemcpyHostToDevice));
    unsigned int cnt = (unsigned int)jw.size();
    CK(cudaMemcpy(h->d_cnt32.p + 0, &cnt, 4, cudaMemcpyHostToDevice));
    CK(cudaMemset(h->d_cnt32.p + 1, 0, 4));
    const int grid = window_grid(h);
    TRY(ensure_window_slab(h, lmax_w, nmax_w, grid));
    aa.jobs = h->d_jobs.p;
    aa.n_jobs = h->d_cnt32.p + 0;
    aa.next_job = h->d_cnt32.p + 1;
    aa.lmax = lmax_w;
    aa.nmax = nmax_w;
    aa.tb_smem = 0;
    aa.tb_global = h->d_tb_global.p;
    aa.tb_global_per_warp = window_slab_bytes(lmax_w, nmax_w);
    launch_align_window(aa, grid, h->st);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->st));
  }
  int err = 0;
  CK(cudaMemcpy(&err, h->d_err.p, 4, cudaMemcpyDeviceToHost));
  if (err) {
    CK(cudaMemset(h->d_err.p, 0, 4));
    if (err == 3) {
      h->err = "the CIGAR overflow pool is full (alignments with very many CIGAR operations)";
      return PBW_ERR_CAPACITY;
    }
    if (err == 9) {
      h->err = "a window-DP wavefront wait ran out of polls before its producer published (results discarded)";
      return PBW_ERR_DEVICE;
    }
    h->err = "align kernel error " + std::to_string(err);
    return PBW_ERR_DEVICE;
  }
  std::vector<AlnOut> outs(n);
  CK(cudaMemcpy(outs.data(), h->d_aln.p, n * sizeof(AlnOut), cudaMemcpyDeviceToHost));
  unsigned int pool_used = 0;
  CK(cudaMemcpy(&pool_used, h->d_cnt32.p + 2, 4, cudaMemcpyDeviceToHost));
  std::vector<uint32_t> pool(pool_used);
  if (pool_used) CK(cudaMemcpy(pool.data(), h->d_cig_pool.p, pool_used * 4, cudaMemcpyDeviceToHost));
  uint64_t co = 0;
  for (uint64_t i = 0; i < n; i++) {
    score[i] = outs[i].score;
    offset[i] = outs[i].pos - ref_off[i];
    cigar_off[i] = (uint32_t)co;
    const uint32_t* src = outs[i].n_ops > CIG_INLINE ? pool.data() + outs[i].cig_pool : outs[i].cig;
    for (uint32_t k = 0; k < outs[i].n_ops; k++) {
      if (co >= cigar_cap) { h->err = "cigar capacity"; return PBW_ERR_CAPACITY; }
      cigar[co++] = src[k];
    }
  }
  cigar_off[n] = (uint32_t)co;
  return PBW_OK;
}

int pbw_records_reserve(const pbw_reads* reads, uint64_t* n_records, uint64_t* cigar_cap) {
  if (!reads || !n_records || !cigar_cap) return PBW_ERR_ARG;
  const uint64_t total = reads->n ? reads->offsets[reads->n] - reads->offsets[0] : 0;
  *n_records = reads->n;
  *cigar_cap = 2 * total + 2 * reads->n + 1;
  return PBW_OK;
}

int pbw_mapq_batch(pbw_handle* h, const pbw_reads* reads, const uint64_t* lk_off, const double* lks,
                   const uint64_t* win_off, const double* repeat, const uint8_t* rev, const uint64_t* ref_off,
                   const uint8_t* refs, const uint32_t* cigar_off, const uint32_t* cigar, uint8_t* mapq,
                   double* posterior, uint32_t* best, double* sum_exp) {
  if (!h || !reads || !lk_off || !lks || !win_off || !rev || !ref_off || !cigar_off || !mapq || !posterior ||
      !best || !sum_exp)
    return PBW_ERR_ARG;
  cudaSetDevice(h->device);
  const uint64_t n = reads->n;
  if (n == 0) return PBW_OK;
  for (uint64_t i = 0; i < n; i++) {
    if (lk_off[i + 1] <= lk_off[i]) { h->err = "pbw_mapq_batch: read without candidates"; return PBW_ERR_ARG; }
    if (reads->offsets[i + 1] - reads->offsets[i] > PBW_MAX_READ_LEN) {
      h->err = "pbw_mapq_batch: read longer than PBW_MAX_READ_LEN";
      return PBW_ERR_LIMIT;
    }
  }
  const uint64_t qt = reads->offsets[n], nl = lk_off[n], nw = win_off[n], nr = ref_off[n], nc = cigar_off[n];
  DevBuf<uint8_t> d_b, d_q, d_rev, d_refs, d_mapq;
  DevBuf<uint64_t> d_o, d_lo, d_wo, d_ro, d_co;
  DevBuf<double> d_lk, d_rep, d_post, d_se;
  DevBuf<uint32_t> d_cig, d_best;
  TRY(grow(h, d_b, qt + 1));
  TRY(grow(h, d_q, qt + 1));
  TRY(grow(h, d_o, n + 1));
  TRY(grow(h, d_lo, n + 1));
  TRY(grow(h, d_lk, nl));
  TRY(grow(h, d_wo, n + 1));
  TRY(grow(h, d_rep, nw + 1));
  TRY(grow(h, d_rev, n));
  TRY(grow(h, d_ro, n + 1));
  TRY(grow(h, d_refs, nr + 1));
  TRY(grow(h, d_co, n + 1));
  TRY(grow(h, d_cig, nc + 1));
  TRY(grow(h, d_mapq, n));
  TRY(grow(h, d_post, n));
  TRY(grow(h, d_best, n));
  TRY(grow(h, d_se, n));
  std::vector<uint64_t> o(n + 1), co(n + 1);
  for (uint64_t i = 0; i <= n; i++) {
    o[i] = reads->offsets[i] - reads->offsets[0];
    co[i] = cigar_off[i];
  }
  CK(cudaMemcpy(d_b.p, reads->bases + reads->offsets[0], qt - reads->offsets[0], cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_q.p, reads->quals + reads->offsets[0], qt - reads->offsets[0], cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_o.p, o.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_lo.p, lk_off, (n + 1) * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_lk.p, lks, nl * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_wo.p, win_off, (n + 1) * 8, cudaMemcpyHostToDevice));
  if (nw) CK(cudaMemcpy(d_rep.p, repeat, nw * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_rev.p, rev, n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_ro.p, ref_off, (n + 1) * 8, cudaMemcpyHostToDevice));
  if (nr) CK(cudaMemcpy(d_refs.p, refs, nr, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(d_co.p, co.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
  if (nc) CK(cudaMemcpy(d_cig.p, cigar, nc * 4, cudaMemcpyHostToDevice));
  MapqBatchArgs a{};
  a.tab = h->d_tab.p;
  a.ln_n = h->d_ln_n.p;
  a.gc_lnb = h->d_gc_lnb.p;
  a.gc_lnbm1 = h->d_gc_lnbm1.p;
  a.n = n;
  a.bases = d_b.p;
  a.quals = d_q.p;
  a.offs = d_o.p;
  a.lk_off = d_lo.p;
  a.lks = d_lk.p;
  a.win_off = d_wo.p;
  a.repeat = d_rep.p;
  a.rev = d_rev.p;
  a.ref_off = d_ro.p;
  a.refs = d_refs.p;
  a.cig_off = d_co.p;
  a.cigar = d_cig.p;
  a.mapq = d_mapq.p;
  a.post = d_post.p;
  a.best = d_best.p;
  a.sum_exp = d_se.p;
  launch_mapq_batch(a, h->st);
  CK(cudaGetLastError());
  CK(cudaStreamSynchronize(h->st));
  CK(cudaMemcpy(mapq, d_mapq.p, n, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(posterior, d_post.p, n * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(best, d_best.p, n * 4, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(sum_exp, d_se.p, n * 8, cudaMemcpyDeviceToHost));
  return PBW_OK;
}

int pbw_seed_batch(pbw_handle* h, const pbw_reads* reads, uint64_t* hit_off, uint64_t* hits, uint32_t* hit_read_pos,
                   uint64_t hit_cap, uint64_t* win_off, double* repeat_prob, uint64_t win_cap) {
  if (!h || !reads || !hit_off || !win_off) return PBW_ERR_ARG;
  cudaSetDevice(h->device);
  uint64_t total;
  int lmax;
  TRY(validate_reads(h, reads, total, lmax));
  const uint64_t n = reads->n;
  hit_off[0] = 0;
  win_off[0] = 0;
  if (n == 0) return PBW_OK;
  TRY(upload_reads(h, reads, total, h->d_bases, h->d_quals, h->d_offs));
  ChunkCfg cfg = chunk_cfg(h, n, lmax);
  TRY(ensure_chunk(h, cfg));
  TRY(grow(h, h->d_hit_rpos, (size_t)cfg.ch * cfg.hcap));
  DevBuf<uint16_t> rpos_pool;
  TRY(grow(h, rpos_pool, ovf_pool_hits(h)));
  CK(cudaMemsetAsync(h->d_cnt32.p, 0, 16 * 4, h->st));
  std::vector<uint32_t> cnt, need, ovf;
  std::vector<uint8_t> over, rep;
  std::vector<unsigned long long> hw, hoff, pool;
  std::vector<uint16_t> rp, prp;
  uint64_t ho = 0, wo = 0;
  for (uint64_t r0 = 0; r0 < n; r0 += cfg.ch) {
    const uint32_t nr = (uint32_t)std::min<uint64_t>(cfg.ch, n - r0);
    TRY(seed_phase(h, cfg, h->d_bases.p, h->d_offs.p, (uint32_t)r0, nr, h->d_rep.p, false,
                   h->d_hit_rpos.p));
    CK(cudaStreamSynchronize(h->st));
    TRY(check_device_errors(h));
    cnt.resize(nr);
    over.resize(nr);
    need.resize(nr);
    hw.resize((size_t)nr * cfg.hcap);
    rp.resize((size_t)nr * cfg.hcap);
    rep.resize((size_t)nr * cfg.wcap);
    unsigned int c32[8];
    CK(cudaMemcpy(c32, h->d_cnt32.p, sizeof(c32), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(cnt.data(), h->d_hit_cnt.p, nr * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(over.data(), h->d_overflow.p, nr, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(need.data(), h->d_need.p, nr * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(hw.data(), h->d_hits.p, hw.size() * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(rp.data(), h->d_hit_rpos.p, rp.size() * 2, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(rep.data(), h->d_rep.p, rep.size(), cudaMemcpyDeviceToHost));
    // over-capacity reads: their hits sit in the pool at list_hoff[item]
    const uint32_t n_list = c32[7];
    ovf.resize(n_list);
    hoff.resize(n_list);
    uint64_t pool_n = 0;
    if (n_list) {
      CK(cudaMemcpy(ovf.data(), h->d_ovf_list.p, n_list * 4, cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(hoff.data(), h->d_list_hoff.p, n_list * 8, cudaMemcpyDeviceToHost));
      for (uint32_t i = 0; i < n_list; i++) pool_n = std::max<uint64_t>(pool_n, hoff[i] + need[ovf[i]]);
      pool.resize(pool_n);
      prp.resize(pool_n);
      // the pool holds one slice at a time: each slice's hits come back
      // before the next list-mode pass reuses it
      const uint64_t S = ovf_slice_hits(h);
      for (uint32_t s = 0; (uint64_t)s * S < pool_n; s++) {
        TRY(ovf_slice(h, cfg, h->d_bases.p, h->d_offs.p, (uint32_t)r0, nr, h->d_rep.p, s, rpos_pool.p, nullptr));
        CK(cudaStreamSynchronize(h->st));
        TRY(check_device_errors(h));
        uint64_t lo = ~0ull, hi = 0;
        for (uint32_t i = 0; i < n_list; i++) {
          if (hoff[i] / S != s) continue;
          lo = std::min<uint64_t>(lo, hoff[i]);
          hi = std::max<uint64_t>(hi, hoff[i] + need[ovf[i]]);
        }
        if (hi <= lo) continue;
        const uint64_t base = (uint64_t)s * S;
        CK(cudaMemcpy(pool.data() + lo, h->d_hits_pool.p + (lo - base), (hi - lo) * 8, cudaMemcpyDeviceToHost));
        CK(cudaMemcpy(prp.data() + lo, rpos_pool.p + (lo - base), (hi - lo) * 2, cudaMemcpyDeviceToHost));
      }
    }
    std::vector<int64_t> item_of(nr, -1);
    for (uint32_t i = 0; i < n_list; i++) item_of[ovf[i]] = i;
    for (uint32_t r = 0; r < nr; r++) {
      const uint64_t rg = r0 + r;
      hit_off[rg] = ho;
      win_off[rg] = wo;
      const uint64_t L = reads->offsets[rg + 1] - reads->offsets[rg];
      const unsigned long long* src = hw.data() + (size_t)r * cfg.hcap;
      const uint16_t* src_rp = rp.data() + (size_t)r * cfg.hcap;
      uint32_t nh = cnt[r];
      if (over[r]) {
        if (item_of[r] < 0) {
          h->err = "over-capacity read missing from the overflow list";
          return PBW_ERR_DEVICE;
        }
        src = pool.data() + hoff[item_of[r]];
        src_rp = prp.data() + hoff[item_of[r]];
        nh = need[r];
      }
      for (uint32_t k = 0; k < nh; k++) {
        if (ho >= hit_cap) { h->err = "hit capacity"; return PBW_ERR_CAPACITY; }
        const unsigned long long w = src[k];
        const uint32_t gk = (uint32_t)(w >> 40);
        const long long diag = (long long)(w & ((1ull << 40) - 1)) - (long long)DIAG_BIAS;
        const uint32_t rpos = src_rp[k];
        const bool rev = gk & 1u;
        const unsigned long long pos = rev ? (unsigned long long)(diag - rpos) : (unsigned long long)(diag + rpos);
        hits[ho] = ((unsigned long long)(rev ? 1 : 0) << 63) | ((unsigned long long)(gk >> 1) << 40) | pos;
        hit_read_pos[ho] = rpos;
        ho++;
      }
      const uint64_t nw = L >= 15 ? L - 14 : 0;
      for (uint64_t w = 0; w < nw; w++) {
        if (wo >= win_cap) { h->err = "window capacity"; return PBW_ERR_CAPACITY; }
        const uint8_t c = rep[(size_t)r * cfg.wcap + w];
        const uint8_t q = reads->quals[reads->offsets[rg] + w];
        repeat_prob[wo++] = c == 2 ? 1.0 : (c == 1 ? h->tab_host.nrp[q] : 0.0);
      }
    }
  }
  hit_off[n] = ho;
  win_off[n] = wo;
  return PBW_OK;
}

int pbw_cluster_batch(pbw_handle* h, const pbw_reads* reads, uint32_t max_per_read, uint32_t* n_cand,
                      uint32_t* total_cand, uint32_t* cand_contig, uint64_t* cand_pos, uint8_t* cand_strand,
                      double* cand_score) {
  if (!h || !reads || max_per_read == 0) return PBW_ERR_ARG;
  if (max_per_read > 256) {
    h->err = "pbw_cluster_batch: max_per_read is at most 256";
    return PBW_ERR_LIMIT;
  }
  cudaSetDevice(h->device);
  uint64_t total;
  int lmax;
  TRY(validate_reads(h, reads, total, lmax));
  const uint64_t n = reads->n;
  if (n == 0) return PBW_OK;
  TRY(upload_reads(h, reads, total, h->d_bases, h->d_quals, h->d_offs));
  ChunkCfg cfg = chunk_cfg(h, n, lmax);
  TRY(ensure_chunk(h, cfg));
  DevBuf<Cand> dc;
  DevBuf<uint32_t> dn, dt;
  TRY(grow(h, dc, (size_t)cfg.ch * max_per_read));
  TRY(grow(h, dn, cfg.ch));
  TRY(grow(h, dt, cfg.ch));
  CK(cudaMemsetAsync(h->d_cnt32.p, 0, 16 * 4, h->st));
  std::vector<Cand> c;
  for (uint64_t r0 = 0; r0 < n; r0 += cfg.ch) {
    const uint32_t nr = (uint32_t)std::min<uint64_t>(cfg.ch, n - r0);
    CK(cudaMemsetAsync(dn.p, 0, nr * 4, h->st));
    CK(cudaMemsetAsync(dt.p, 0, nr * 4, h->st));
    TRY(seed_phase(h, cfg, h->d_bases.p, h->d_offs.p, (uint32_t)r0, nr, h->d_rep.p, false, nullptr));
    TRY(cluster_phase(h, cfg, h->d_bases.p, h->d_quals.p, h->d_offs.p, (uint32_t)r0, nr, h->d_rep.p, dc.p, dn.p,
                      dt.p, max_per_read, nullptr));
    CK(cudaStreamSynchronize(h->st));
    TRY(check_device_errors(h));
    c.resize((size_t)nr * max_per_read);
    CK(cudaMemcpy(c.data(), dc.p, c.size() * sizeof(Cand), cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(n_cand + r0, dn.p, nr * 4, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(total_cand + r0, dt.p, nr * 4, cudaMemcpyDeviceToHost));
    const size_t base = (size_t)r0 * max_per_read;
    for (size_t i = 0; i < c.size(); i++) {
      cand_contig[base + i] = c[i].contig;
      cand_pos[base + i] = c[i].pos;
      cand_strand[base + i] = c[i].strand;
      cand_score[base + i] = (double)c[i].score;
    }
  }
  return PBW_OK;
}

}  // extern "C"
