// radix_sort.cu -- stable least-significant-digit radix sort of (u64 key,
// u64 value) pairs on the device, 8 key bits per pass; used by the
// coordinate sort (coord_sort.cu) and the hash-table build (index_build.cu).
//
// Each pass: per-tile digit histograms (tiles of 4096 keys) written
// digit-major, one exclusive scan of that table (every tile's start for every
// digit), and a scatter in which each tile ranks its keys in input order (a
// warp match on the digit, then per-digit prefixes over the warps of the
// block), so equal digits keep their order and the sort is stable.
#include "pbw_host.h"

namespace pbw {

namespace {

constexpr int RS_T = 256, RS_ROUNDS = 16, RS_TILE = RS_T * RS_ROUNDS, RS_WARPS = RS_T / 32;

__global__ void __launch_bounds__(RS_T) k_radix_hist(const unsigned long long* key, uint64_t n, int shift,
                                                     unsigned int* hist, uint32_t nb) {
  __shared__ unsigned int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
  for (int j = 0; j < RS_ROUNDS; j++) {
    const uint64_t i = base + (uint64_t)j * RS_T + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(unsigned)(key[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_T) k_radix_scatter(const unsigned long long* key, const unsigned long long* val,
                                                        uint64_t n, int shift, const unsigned int* start, uint32_t nb,
                                                        unsigned long long* key_out, unsigned long long* val_out) {
  __shared__ unsigned int base[256];
  __shared__ unsigned int wcnt[RS_WARPS][257];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  base[threadIdx.x] = start[(uint64_t)threadIdx.x * nb + blockIdx.x];
  const uint64_t tile = (uint64_t)blockIdx.x * RS_TILE;
  const unsigned int lt = (1u << lane) - 1u;
  for (int j = 0; j < RS_ROUNDS; j++) {
    for (int k = threadIdx.x; k < RS_WARPS * 257; k += RS_T) (&wcnt[0][0])[k] = 0;
    __syncthreads();
    const uint64_t i = tile + (uint64_t)j * RS_T + threadIdx.x;
    const bool ok = i < n;
    const unsigned long long kk = ok ? key[i] : 0ull;
    const unsigned int d = ok ? (unsigned)(kk >> shift) & 255u : 256u;
    const unsigned int peers = __match_any_sync(0xffffffffu, d);
    const unsigned int rank = __popc(peers & lt);
    if (rank == 0) wcnt[w][d] = __popc(peers);
    __syncthreads();
    {
      // per digit: exclusive prefix over the warps, on top of the running base
      const unsigned int dd = threadIdx.x;
      unsigned int run = base[dd];
      for (int q = 0; q < RS_WARPS; q++) {
        const unsigned int t = wcnt[q][dd];
        wcnt[q][dd] = run;
        run += t;
      }
      base[dd] = run;
    }
    __syncthreads();
    if (ok) {
      const unsigned int p = wcnt[w][d] + rank;
      key_out[p] = kk;
      val_out[p] = val[i];
    }
    __syncthreads();
  }
}

}  // namespace

uint64_t radix_hist_entries(uint64_t n) { return ((n + RS_TILE - 1) / RS_TILE) * 256; }

int radix_sort_pairs(unsigned long long* k[2], unsigned long long* v[2], uint64_t n, int first_digit, int passes,
                     unsigned int* hist, unsigned int* sums, cudaStream_t st) {
  int cur = 0;
  if (n == 0) return cur;
  const uint32_t nb = (uint32_t)((n + RS_TILE - 1) / RS_TILE);
  const uint64_t nh = (uint64_t)nb * 256;
  for (int p = 0; p < passes; p++) {
    const int shift = 8 * (first_digit + p);
    k_radix_hist<<<nb, RS_T, 0, st>>>(k[cur], n, shift, hist, nb);
    launch_scan_excl(hist, nh, nullptr, sums, nullptr, nullptr, st);
    k_radix_scatter<<<nb, RS_T, 0, st>>>(k[cur], v[cur], n, shift, hist, nb, k[cur ^ 1], v[cur ^ 1]);
    cur ^= 1;
  }
  return cur;
}

}  // namespace pbw
