// index.cu -- device construction of the dense 15-mer CSR from a .sthash
// table (src/index/hashtable.rs:60-70) and validation of every occurrence.
//
// The file maps mix(raw) -> (offset, count) into a flat positions array
// (hashtable.rs:297-313). mix (hashtable.rs:117-124) is a bijection on u32,
// so each key is inverted back to its raw 30-bit 15-mer code; the buckets are
// then laid out in raw-code order behind a 4^15+1 prefix array, one random
// 8-byte read per lookup. Bucket contents keep the file's order (scan order,
// capped at max_count), which fixes the seed-hit emission order.
#include "pbw_common.cuh"
#include "pbw_kernels.h"
#include "pbw_host.h"

namespace pbw {

// Multiplicative inverse of an odd 32-bit constant (Newton iteration).
__host__ __device__ constexpr uint32_t inv32(uint32_t a) {
  uint32_t x = a;
  for (int i = 0; i < 5; i++) x *= 2u - a * x;
  return x;
}

// Inverse of mix (hashtable.rs:117-124).
__host__ __device__ inline uint32_t unmix32(uint32_t h) {
  h ^= h >> 16;
  h *= inv32(0x846ca68bu);
  h ^= (h >> 15) ^ (h >> 30);
  h *= inv32(0x7feb352du);
  h ^= h >> 16;
  return h;
}

__global__ void k_csr_counts(const uint32_t* tab, uint64_t n, uint64_t npos, unsigned int* counts, int* err) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t key = tab[3 * i], off = tab[3 * i + 1], cnt = tab[3 * i + 2];
  uint32_t raw = unmix32(key);
  if (raw >= NKMER || (uint64_t)off + cnt > npos) {
    atomicExch(err, 10);
    return;
  }
  if (atomicExch(&counts[raw], cnt) != 0u) atomicExch(err, 11);  // duplicate key
}

__global__ void k_csr_fill(const uint32_t* tab, uint64_t n, const unsigned long long* pos_in,
                           const unsigned int* csr, unsigned long long* ent, const unsigned long long* clen,
                           uint32_t ncontig, int* err) {
  // one warp per table entry
  uint64_t w = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= n) return;
  uint32_t key = tab[3 * w], off = tab[3 * w + 1], cnt = tab[3 * w + 2];
  uint32_t raw = unmix32(key);
  if (raw >= NKMER) return;
  uint32_t dst = csr[raw];
  for (uint32_t t = lane; t < cnt; t += 32) {
    unsigned long long p = pos_in[(uint64_t)off + t];
    uint32_t cid = (uint32_t)((p >> 40) & ((1ull << 23) - 1));
    unsigned long long pos = p & ((1ull << 40) - 1);
    if (cid >= ncontig || pos >= clen[cid]) atomicExch(err, 12);
    ent[(uint64_t)dst + t] = p;
  }
}

void launch_build_csr_counts(const uint32_t* tab, uint64_t n, uint64_t npos, unsigned int* counts, int* err,
                             cudaStream_t st) {
  if (n == 0) return;
  k_csr_counts<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(tab, n, npos, counts, err);
}

void launch_build_csr_fill(const uint32_t* tab, uint64_t n, const unsigned long long* pos_in, uint64_t,
                           const unsigned int* csr, unsigned long long* ent, const unsigned long long* clen,
                           uint32_t ncontig, int* err, cudaStream_t st) {
  if (n == 0) return;
  uint64_t threads = n * 32;
  k_csr_fill<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(tab, n, pos_in, csr, ent, clen, ncontig, err);
}

uint32_t host_unmix32(uint32_t h) { return unmix32(h); }

}  // namespace pbw
