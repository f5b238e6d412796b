// pbw_pipeline.h -- the handle and its device buffers.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/probebwa_gpu.h"
#include "pbw_common.cuh"
#include "pbw_kernels.h"
#include "paired.h"

namespace pbw {

// Owned device allocation that only grows.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t cap = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  ~DevBuf() { release(); }
};

// Pinned host staging that only grows.
struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
  HostBuf() = default;
  HostBuf(const HostBuf&) = delete;
  HostBuf& operator=(const HostBuf&) = delete;
  bool ensure(size_t n) {
    if (n <= cap) return true;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    if (cudaMallocHost(&p, n) != cudaSuccess) return false;
    cap = n;
    return true;
  }
  ~HostBuf() {
    if (p) cudaFreeHost(p);
  }
};

// The process's origin event on a device (recorded when the first handle
// on it opens); nullptr if it cannot be created.
cudaEvent_t device_epoch(int dev);

}  // namespace pbw

struct pbw_handle {
  std::string err;
  pbw_options opt;
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
  cudaStream_t st = nullptr;
  std::string species, assembly;
  std::vector<std::string> names;
  std::vector<uint64_t> lens;
  uint64_t total_length = 0;
  uint64_t seed_k = 15;
  uint64_t n_ent = 0;
  // index
  pbw::DevBuf<unsigned long long> d_bits;
  pbw::DevBuf<unsigned int> d_nmask;
  pbw::DevBuf<unsigned int> d_nblk;  // 1 bit per 1024-base block: holds an N
  pbw::DevBuf<unsigned long long> d_cbase, d_clen;
  pbw::DevBuf<int> d_name_class;
  pbw::DevBuf<unsigned int> d_csr;
  pbw::DevBuf<unsigned long long> d_ent;
  pbw::DevGenome G{};
  pbw::DevIndex I{};
  // parameter tables
  pbw::DevTables tab_host{};
  pbw::DevBuf<pbw::DevTables> d_tab;
  pbw::DevBuf<double> d_ln_n, d_gc_lnb, d_gc_lnbm1;
  pbw::DevBuf<int> d_err;
  // inputs of a call
  pbw::DevBuf<uint8_t> d_bases, d_quals, d_bases2, d_quals2;
  pbw::DevBuf<uint64_t> d_offs, d_offs2;
  // per-chunk work
  pbw::DevBuf<unsigned long long> d_hits;
  pbw::DevBuf<uint32_t> d_hit_cnt;
  pbw::DevBuf<uint16_t> d_hit_rpos;
  pbw::DevBuf<uint8_t> d_overflow, d_rep;
  pbw::DevBuf<pbw::Cand> d_cand;
  pbw::DevBuf<uint32_t> d_n_cand, d_total_cand;
  pbw::DevBuf<pbw::AlnJob> d_jobs;
  pbw::DevBuf<pbw::AlnOut> d_aln;
  pbw::DevBuf<uint32_t> d_cig_pool;
  pbw::DevBuf<unsigned int> d_cnt32;        // 0 n_jobs, 1 next_job, 2 cig_pool_used, 3 n_overflow, 4 cig_total
  pbw::DevBuf<unsigned long long> d_cnt64;  // 0 probes, 1 entries, 2 hits, 3 dp jobs, 4 dp cells
  pbw::DevBuf<unsigned int> d_scan_sums;
  pbw::DevBuf<unsigned char> d_tb_global;
  pbw::DevBuf<unsigned char> d_tb_pair;  // the pair batches' window-DP traceback slab
  // reads with more seed hits than the per-read capacity
  pbw::DevBuf<uint32_t> d_need, d_ovf_list;
  pbw::DevBuf<unsigned long long> d_list_hoff, d_hits_pool;
  pbw::DevBuf<unsigned char> d_cl_scratch;
  pbw::DevBuf<unsigned char> d_cl_big;  // K2 global slabs for reads of 4096-16384 hits
  // outputs of a call
  pbw::DevBuf<int32_t> o_contig, o_mate_contig, o_as, o_nm, o_best;
  pbw::DevBuf<unsigned long long> o_pos, o_mate_pos;
  pbw::DevBuf<long long> o_tlen;
  pbw::DevBuf<uint8_t> o_mapq;
  pbw::DevBuf<uint16_t> o_flag;
  pbw::DevBuf<double> o_log_lk, o_post;
  pbw::DevBuf<uint32_t> o_nops, o_cig_off, o_cigar;
  // paired-end buffers
  pbw::DevBuf<uint32_t> o_cig_off2, o_cigar2, o_len;
  pbw::DevBuf<const pbw::AlnOut*> o_cigsrc;
  pbw::DevBuf<pbw::Cand> d_cand2;
  pbw::DevBuf<uint32_t> d_n_cand2;
  pbw::DevBuf<pbw::AlnOut> d_aln2, d_xout;
  pbw::DevBuf<uint8_t> d_rep2;
  pbw::DevBuf<pbw::ReadSum> d_sum;
  pbw::DevBuf<pbw::PairWork> d_work;
  pbw::DevBuf<pbw::XMeta> d_xmeta;
  pbw::DevBuf<pbw::PairModel> d_model;
  pbw::DevBuf<double> d_obs;
  pbw::DevBuf<pbw::AlnJob> d_xjobs;
  // learned candidate ranker (ranker.cu): model, per-chunk scratch and the
  // training-data collection of pbw_ranker_train
  struct Ranker {
    bool trained = false;
    bool enabled = false;     // prune candidates in map calls
    bool collect = false;     // write features and labels of every slot (plain path)
    float tau = 0.f;          // keep a candidate whose logit >= tau
    double label_cut = 0.0;   // training label: lk - lk_max >= label_cut
    pbw::DevBuf<float> d_norm, d_w, d_m, d_v, d_g, d_loss;
    pbw::DevBuf<uint32_t> d_wb;
    pbw::DevBuf<uint16_t> d_hit_info;
    pbw::DevBuf<float> d_feat, d_logit;               // 2 read sets x chunk slots
    pbw::DevBuf<unsigned long long> d_counters;       // kept, pruned, reads kept whole
    pbw::DevBuf<float> c_feat;                        // collection: slot-indexed
    pbw::DevBuf<uint8_t> c_label;
    uint64_t c_slots = 0;                             // slots per read set in the collection
  } rk;
  // batching: seeded-DP form per read-length class, length bins, graphs
  struct Tuning {
    int autotune = 1;       // time the 8-, 16- and 4-lane band DP on a class's first chunk, keep the fastest
    int band_lanes = 0;     // 0: the tuned (or 8) form; 4, 8 or 16: forced
    int length_bins = 1;    // order the seeded DP queue by read length in mixed-length chunks
    int pair_graphs = 1;    // one CUDA graph launch per batch of pairs
    int chosen[3] = {0, 0, 0};  // lanes per read-length class (<= 128, <= 256, longer); 0: not tuned
    float ms[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // the trial: 8, 16, 4 lanes
    uint32_t wait_polls = 0;  // window-DP wavefront waits: polls before giving up (0 = the kernel's default)
    uint32_t ovf_slice_hits = 0;  // over-capacity reads: hits per pool slice (0 = the default, 16 M)
    int k2_threads[2] = {0, 0};   // K2 block size of the 4096-hit and the slab tier: 0 tuned, else forced
    int k2_chosen[2] = {0, 0};    // tuned block sizes (0: not tuned)
    float k2_ms[2][3] = {{0, 0, 0}, {0, 0, 0}};  // the trial: 1024, 512, 256 threads
  } tune;
  int call_lmin = 0;        // shortest read of the current call
  pbw::DevBuf<pbw::AlnJob> d_jobs_b;
  pbw::DevBuf<unsigned int> d_bins;
  pbw::DevBuf<uint32_t> d_batch;
  pbw::DevBuf<double> d_obs_batch;
  pbw::HostBuf h_stage;
  pbw::HostBuf h_fold;  // one batch's insert-size observations + the model
  std::vector<cudaEvent_t> events;
  // paired calls: reads go up on a copy stream, one event per super-chunk
  cudaStream_t st_up = nullptr;
  cudaStream_t st_pair = nullptr;  // paired calls: the pair batches, beside the next super-chunk's seeding
  std::vector<cudaEvent_t> up_ev;
  pbw_stats stats{};
  ~pbw_handle() {
    for (auto e : events) cudaEventDestroy(e);
    for (auto e : up_ev) cudaEventDestroy(e);
    if (st_up) cudaStreamDestroy(st_up);
    if (st_pair) cudaStreamDestroy(st_pair);
    if (st) cudaStreamDestroy(st);
  }
};

namespace pbw {
int pipeline_init(pbw_handle* h);
}

// GenomeIndex::load (src/index/genome.rs:80-86) of prefix.stidx into the
// handle's device genome (2-bit words, N mask, contig bases and lengths) and
// its contig names and lengths.
int load_genome(pbw_handle* h, const std::string& prefix);
