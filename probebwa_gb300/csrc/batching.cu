// batching.cu -- ordering of the seeded DP's work queue by read length (no
// counterpart in the reference).
//
// The band DP (align_band.cu) is a persistent kernel that takes alignments
// from a device work queue, several per warp, so a warp runs as long as its
// longest alignment. When a chunk mixes read lengths (trimmed reads of
// 60-250 bases), the queue is reordered into 16-base length bins, longest
// first: the alignments a warp takes together have similar lengths, and the
// long ones start early instead of trailing at the end of the launch. A
// counting sort on the device: bin counts, a 64-entry scan, a scatter with
// per-bin cursors (order inside a bin is free: every job writes its own
// output slot).
#include "pbw_host.h"

namespace pbw {

namespace {

constexpr int NBIN = 64;  // 16-base bins up to PBW_MAX_READ_LEN

__device__ __forceinline__ int job_bin(const AlnJob& J, const uint64_t* offs) {
  const uint64_t L = offs[J.read + 1] - offs[J.read];
  const int b = (int)(L >> 4);
  return NBIN - 1 - (b < NBIN ? b : NBIN - 1);  // longest first
}

__global__ void k_job_count(const AlnJob* jobs, const unsigned int* n_jobs, const uint64_t* offs,
                            unsigned int* bins) {
  __shared__ unsigned int c[NBIN];
  for (int k = threadIdx.x; k < NBIN; k += blockDim.x) c[k] = 0;
  __syncthreads();
  const unsigned int n = *n_jobs;
  for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
    atomicAdd(&c[job_bin(jobs[q], offs)], 1u);
  __syncthreads();
  for (int k = threadIdx.x; k < NBIN; k += blockDim.x)
    if (c[k]) atomicAdd(&bins[k], c[k]);
}

// bins: counts in, exclusive starts out (the cursors of the scatter).
__global__ void k_job_starts(unsigned int* bins) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned int run = 0;
  for (int k = 0; k < NBIN; k++) {
    const unsigned int c = bins[k];
    bins[k] = run;
    run += c;
  }
}

__global__ void k_job_scatter(const AlnJob* jobs, const unsigned int* n_jobs, const uint64_t* offs,
                              unsigned int* cursor, AlnJob* out) {
  const unsigned int n = *n_jobs;
  for (unsigned int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const AlnJob J = jobs[q];
    out[atomicAdd(&cursor[job_bin(J, offs)], 1u)] = J;
  }
}

}  // namespace

size_t job_bin_words() { return NBIN; }

void launch_job_bins(const AlnJob* jobs, const unsigned int* n_jobs, const uint64_t* offs, unsigned int* bins,
                     AlnJob* out, int grid, cudaStream_t st) {
  cudaMemsetAsync(bins, 0, NBIN * sizeof(unsigned int), st);
  k_job_count<<<grid, 256, 0, st>>>(jobs, n_jobs, offs, bins);
  k_job_starts<<<1, 32, 0, st>>>(bins);
  k_job_scatter<<<grid, 256, 0, st>>>(jobs, n_jobs, offs, bins, out);
}

}  // namespace pbw
