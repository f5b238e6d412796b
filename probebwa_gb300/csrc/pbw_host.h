// pbw_host.h -- glue-kernel argument blocks and launchers used by the host pipeline.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

struct MakeJobsArgs {
  DevGenome G;
  const uint64_t* offs;
  uint32_t r0, nr;
  const Cand* cand;
  const uint32_t* n_cand;
  uint64_t right_pad;       // max(max_indel_len, 10)
  uint32_t band;            // max_indel_len
  int32_t gap_open, gap_extend;
  AlnJob* jobs;
  unsigned int* n_jobs;
  AlnOut* out;
  uint8_t mate;             // read set of the jobs (AlnJob::mate)
  uint8_t prune;            // skip candidates whose Cand::pad[0] (ranker keep flag) is 0
};

struct CigarGatherArgs {
  const uint64_t* offs;
  uint32_t r0, nr;
  const int32_t* best;
  const AlnOut* aln;
  const uint32_t* cig_pool;
  const uint32_t* cig_off;  // chunk-relative exclusive offsets (including the chunk base)
  uint32_t* cigar;          // packed output for the whole call
};

void launch_make_jobs_single(const MakeJobsArgs& a, cudaStream_t st);
void launch_cigar_gather(const CigarGatherArgs& a, cudaStream_t st);
uint64_t scan_blocks(uint64_t n);
void launch_scan_excl(unsigned int* a, uint64_t n, unsigned int* out, unsigned int* block_sums, unsigned int* total,
                      const unsigned int* base_in, cudaStream_t st);

// Reorders the n_jobs (device count) alignment jobs into out by read-length
// bins, longest first (batching.cu); bins holds job_bin_words() entries.
size_t job_bin_words();
void launch_job_bins(const AlnJob* jobs, const unsigned int* n_jobs, const uint64_t* offs, unsigned int* bins,
                     AlnJob* out, int grid, cudaStream_t st);

// Stable LSD radix sort of n (key, value) pairs by key bits
// [8 * first_digit, 8 * (first_digit + passes)). Input in k[0] / v[0]; the
// passes ping-pong with k[1] / v[1]; returns the index of the buffers that
// hold the result. hist holds radix_hist_entries(n) entries, sums
// scan_blocks(radix_hist_entries(n)) + 2.
uint64_t radix_hist_entries(uint64_t n);
int radix_sort_pairs(unsigned long long* k[2], unsigned long long* v[2], uint64_t n, int first_digit, int passes,
                     unsigned int* hist, unsigned int* sums, cudaStream_t st);

}  // namespace pbw
