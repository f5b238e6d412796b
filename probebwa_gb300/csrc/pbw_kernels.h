// pbw_kernels.h -- kernel argument blocks and launchers (host <-> device).
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

#include "pbw_common.cuh"
#include "../../include/probebwa_gpu.h"

namespace pbw {

// ---- K1 seeding ----
struct SeedArgs {
  DevGenome G;
  DevIndex idx;
  const uint8_t* bases;
  const uint64_t* offs;
  uint32_t r0, nr;          // reads [r0, r0+nr) of the offsets array
  int lmax;                 // longest read in the chunk
  unsigned long long* hits; // nr * hcap
  uint32_t hcap;
  uint32_t* hit_cnt;        // nr
  uint8_t* overflow;        // nr
  unsigned int* n_overflow; // 1
  uint8_t* rep;             // nr * wcap: 0 none, 1 neighbour repetitive, 2 exact repetitive
  uint32_t wcap;
  uint16_t* hit_rpos;       // optional nr * hcap read positions (stage entry point)
  uint16_t* hit_rpos_pool;  // optional, list mode: read positions beside hits_pool
  uint16_t* hit_info;       // optional nr * hcap: read position | log2 exact bucket << 10 | neighbour << 15
  unsigned long long* counters;  // probes, entries, hits
  // overflow handling: reads with more than hcap hits are queued with their
  // exact hit count and seeded again in list mode into a pool
  uint32_t* need;           // nr: exact hit count of an overflowed read
  uint32_t* ovf_list;       // overflowed chunk-relative read indices
  unsigned int* n_ovf;      // queue length
  const uint32_t* list;     // list mode: work item w is read list[w]
  const unsigned int* list_n;
  const unsigned long long* list_hoff;  // exclusive prefix of the listed reads' hit counts
  unsigned long long* hits_pool;
  // the pool holds one slice at a time: item w belongs to slice
  // list_hoff[w] / pool_slice and sits at list_hoff[w] - slice * pool_slice
  unsigned long long pool_slice;
  uint32_t slice;
  const unsigned long long* list_total;  // all listed hits (slices past it exit at once)
};
__host__ __device__ inline size_t seed_smem_per_warp(int lmax) {
  int W = lmax - KMER + 1 > 0 ? lmax - KMER + 1 : 1;
  // prefix counts (lmax + 1 words of 8 bytes), then the window arrays and the codes
  size_t s = (size_t)(lmax + 1) * 8 + (size_t)(4 * W + 1) * 4 + (size_t)lmax;
  return (s + 15) & ~(size_t)15;
}
void launch_seed(const SeedArgs& a, int grid, cudaStream_t st);

// ---- K2 clustering ----
struct Cand {
  unsigned long long pos;   // 0-based candidate position (candidates.rs:62-71)
  uint32_t contig;
  uint32_t score;           // cluster size
  uint8_t strand;
  uint8_t pad[7];
};
struct ClusterArgs {
  const unsigned long long* hits;
  const uint32_t* hit_cnt;
  const uint8_t* overflow;
  uint32_t hcap;
  const uint64_t* offs;
  uint32_t r0, nr;
  int group_width;
  uint32_t max_out;         // candidates kept per read (20 for mapping)
  Cand* cand;               // nr * max_out
  uint32_t* n_cand;         // nr: kept
  uint32_t* total_cand;     // nr: all clusters (optional)
  uint32_t h_lo, h_hi;      // process reads with h_lo < H <= h_hi
  uint32_t gmax;            // distinct (contig, strand) keys: 2 * contigs
  int* err;                 // device error word
  // list mode (overflowed reads): hits in the pool, tables in global scratch
  const uint32_t* list;
  const unsigned int* list_n;
  const unsigned long long* list_hoff;
  const unsigned long long* hits_pool;
  const uint32_t* need;
  unsigned char* scratch;   // list mode: cluster_list_bytes_per_hit per pooled hit; tiers: the slabs
  unsigned long long pool_slice;  // as SeedArgs: the slice of the pool in use
  uint32_t slice;
  const unsigned long long* list_total;
  // with the candidate ranker: per kept candidate RANK_FEATURES seed features
  // (list-mode reads, whose hits are in the pool, get feature 0 = -1: no
  // hit-level features)
  float* feat;                      // nr * MAX_CAND * RANK_FEATURES
  const uint16_t* hit_info;         // nr * hcap: read position | log2 bucket << 10 | neighbour << 15
  const uint8_t* quals;             // the reads' Phred scores (at offs)
};
// K2 of the over-capacity reads of one pool slice (list mode), tables in
// a.scratch at bytes_per_hit (cluster_list_bytes_per_hit(hcap, gmax)) per
// pooled hit.
size_t cluster_list_bytes_per_hit(uint32_t hcap, uint32_t gmax);
void launch_cluster_list(const ClusterArgs& a, size_t bytes_per_hit, int grid, cudaStream_t st);
// K2 by diagonal bins (no sort of the hits; cluster.cu) for reads of
// h_lo < H <= h_hi <= hmax hits, one block per read: the tables in shared
// memory, or, when they do not fit (cluster_bins_in_slab), in a.scratch.
// a.scratch holds grid slabs of cluster_bins_slab_bytes(hmax, gmax, in_slab);
// the grid is cluster_bins_grid (the blocks that are resident at once).
size_t cluster_bins_slab_bytes(uint32_t hmax, uint32_t gmax, bool table_in_slab);
size_t cluster_bins_smem_bytes(uint32_t hmax, uint32_t gmax, bool feat);
bool cluster_bins_in_slab(uint32_t hmax, uint32_t gmax, bool feat);
int cluster_bins_grid(uint32_t hmax, uint32_t gmax, int threads, bool feat, int num_sms);
void launch_cluster_bins(const ClusterArgs& a, uint32_t hmax, int threads, int grid, cudaStream_t st);
void launch_seed_list(const SeedArgs& a, int grid, cudaStream_t st);
// Exclusive offsets of the listed (over-capacity) reads' hit counts, their
// total, and the list length for the list-mode passes; a read needing more
// than one slice (pool_slice hits), or a total beyond max_slices slices, is
// error 5 and empties the list.
void launch_ovf_offsets(const uint32_t* list, const unsigned int* list_n, const uint32_t* need,
                        unsigned long long* hoff, unsigned long long* total, unsigned long long pool_slice,
                        uint32_t max_slices, int* err, unsigned int* list_n_out, cudaStream_t st);

// ---- K3 alignment ----
// One alignment problem: query = read (forward) or its reverse complement,
// against ref window [ref_start, ref_end) of contig, banded around
// j = i + hint (smith_waterman.rs:190-194).
struct AlnJob {
  unsigned long long ref_start, ref_end;
  long long hint;
  uint32_t read;            // index into the offsets array
  uint32_t slot;            // output slot
  uint32_t contig;
  uint32_t band;            // band half-width (max_indel_len, or the window length)
  uint8_t rev;              // query is the reverse complement
  uint8_t valid;
  uint8_t mate;             // 0: reads in bases/quals/offs, 1: in bases2/quals2/offs2
  uint8_t pad;
  uint32_t pad2;
  int32_t gap_open, gap_extend;
};
struct AlnOut {
  double log_lk;
  unsigned long long pos;   // true_start, 0-based (single.rs:135)
  int32_t score;
  uint32_t span;            // cigar_reference_span
  uint32_t n_ops;
  uint32_t cig_pool;        // offset into the CIGAR pool when n_ops > CIG_INLINE
  uint32_t cig[CIG_INLINE];
  // log_entropy inputs (bayesian.rs:306-357) and edit distance
  int32_t n_hq, m_hq, readlen, ins_runs, del_runs, gc, total, nm;
};
struct AlignArgs {
  DevGenome G;
  const DevTables* tab;
  const double* gc_lnb;     // gc tables, triangular by total
  const double* gc_lnbm1;
  const uint8_t* bases;     // reads (also used for explicit problems)
  const uint8_t* quals;
  const uint64_t* offs;
  const uint8_t* bases2;    // second read set (mate 2) for paired jobs
  const uint8_t* quals2;
  const uint64_t* offs2;
  const AlnJob* jobs;
  const unsigned int* n_jobs;  // device count (work queue size)
  unsigned int* next_job;      // work queue head
  AlnOut* out;
  uint32_t* cig_pool;
  unsigned int* cig_pool_used;
  uint32_t cig_pool_cap;
  // explicit reference windows (pbw_align_batch): if non-null, job.ref_* index these bytes
  const uint8_t* ref_bytes;
  int lmax;                 // longest query
  int nmax;                 // longest reference window
  size_t tb_smem;           // unused (0)
  unsigned char* tb_global; // K3w: per-block slabs for windows too wide for shared memory
  size_t tb_global_per_warp;  // K3w: bytes of one block's slab
  unsigned long long* counters;  // jobs, cells
  int* err;
  uint32_t wait_polls;      // K3w: polls before a wavefront wait gives up (error 9); 0 = WIN_SPIN_LIMIT
};
// K3b, band <= band_max <= 31; grid sized from the shared memory per warp.
// AlignArgs::tb_global must hold band_tb_slab_bytes(lmax, nmax, num_sms,
// band_max) bytes (the per-alignment traceback rows).
void launch_align_band(const AlignArgs& a, int num_sms, int band_max, cudaStream_t st);
// The same with 4, 8 or 16 lanes per alignment (16: bands with
// band_has_lanes16; 4: bands with band_has_lanes4).
void launch_align_band_lanes(const AlignArgs& a, int num_sms, int band_max, int lanes, cudaStream_t st);
bool band_has_lanes16(int band_max);
bool band_has_lanes4(int band_max);
size_t band_tb_slab_bytes(int lmax, int nmax, int num_sms, int band_max);
// K3w, one job per block of 8 warps; tb_global_per_warp is the global slab of
// one block (window_slab_bytes), used by windows that do not fit the block's
// shared memory. wide: 8 window columns per lane and one block per SM, for
// batches of fewer ~1,000-column windows than SMs (the paired path's
// cross-alignments); else 4 columns per lane and two blocks per SM.
void launch_align_window(const AlignArgs& a, int grid, cudaStream_t st, bool wide = false);
size_t window_smem_bytes(int lmax, int nmax);
// Likelihood, log_entropy counts and edit distance of every aligned job from
// its CIGAR (after K3b / K3w); max_jobs bounds the device job count.
void launch_aln_stats(const AlignArgs& a, uint64_t max_jobs, cudaStream_t st);
// per job: window symbols, gap opens, traceback ops, (lmax + 7) / 8 traceback
// words per column; 16-byte aligned pieces
constexpr size_t window_slab_bytes(int lmax, int nmax) {
  return (((size_t)nmax + 15) & ~(size_t)15) + ((4 * (size_t)nmax + 15) & ~(size_t)15) +
         (((size_t)lmax + nmax + 2 + 15) & ~(size_t)15) +
         ((4 * ((size_t)nmax + 1) * (((size_t)lmax + 7) / 8) + 15) & ~(size_t)15);
}

// ---- K4 finalize (single-end) ----
struct FinalizeArgs {
  DevGenome G;
  const DevTables* tab;
  const double* ln_n;
  const uint8_t* quals;
  const uint64_t* offs;
  uint32_t r0, nr;
  const AlnOut* aln;        // nr * MAX_CAND
  const uint32_t* n_cand;
  const Cand* cand;
  const uint8_t* rep;
  uint32_t wcap;
  const double* gc_lnb;
  const double* gc_lnbm1;
  uint64_t seed_k;
  // outputs (device, chunk-relative)
  int32_t* contig;
  unsigned long long* pos;
  uint8_t* mapq;
  uint16_t* flag;
  double* log_lk;
  double* posterior;
  int32_t* as_score;
  int32_t* nm;
  uint32_t* n_ops;          // per read CIGAR op count
  int32_t* best;            // per read winning slot (-1 unmapped)
};
void launch_finalize(const FinalizeArgs& a, int grid, cudaStream_t st);

// ---- MapqCalculator batch (pbw_mapq_batch) ----
struct MapqBatchArgs {
  const DevTables* tab;
  const double* ln_n;
  const double* gc_lnb;
  const double* gc_lnbm1;
  uint64_t n;
  const uint8_t* bases;
  const uint8_t* quals;
  const uint64_t* offs;
  const uint64_t* lk_off;
  const double* lks;
  const uint64_t* win_off;
  const double* repeat;
  const uint8_t* rev;
  const uint64_t* ref_off;
  const uint8_t* refs;
  const uint64_t* cig_off;
  const uint32_t* cigar;
  uint8_t* mapq;
  double* post;
  uint32_t* best;
  double* sum_exp;
};
void launch_mapq_batch(const MapqBatchArgs& a, cudaStream_t st);

// ---- host parameter tables (api.cu) ----
void fill_tables(const pbw_options& opt, uint64_t total_length, DevTables& T);
void gap_costs(uint32_t gop, uint32_t gep, int32_t& go, int32_t& ge);
void set_handleless_error(const std::string& s);

// ---- index build ----
void launch_build_csr_counts(const uint32_t* tab, uint64_t n, uint64_t npos, unsigned int* counts, int* err,
                             cudaStream_t st);
uint32_t host_unmix32(uint32_t h);
void launch_build_csr_fill(const uint32_t* tab, uint64_t n, const unsigned long long* pos_in, uint64_t npos,
                           const unsigned int* csr, unsigned long long* ent, const unsigned long long* clen,
                           uint32_t ncontig, int* err, cudaStream_t st);

}  // namespace pbw
