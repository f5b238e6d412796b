// cluster.cu -- K2: candidate clustering (src/mapper/candidates.rs:30-78),
// one thread block per read.
//
// The reference groups hits by (contig, strand) in an FxHashMap, visits the
// groups in that map's iteration order, sorts each group's diagonals, splits
// at gaps > 50, emits one candidate per cluster (truncating mean diagonal),
// then stable-sorts candidates by hit count, descending. Here:
//   1. the read's hit words ((contig, strand) << 40 | diagonal) are sorted in
//      shared memory (bitonic, key + emission index), which makes every group
//      contiguous with ascending diagonals;
//   2. block scans mark group and cluster boundaries and give cluster sums;
//   3. each group's first emission index gives the FxHashMap insertion
//      order, and one thread replays std's SwissTable insertion for those
//      keys (FxHasher of rustc-hash 2.1.3, probing by the group width) to get
//      the iteration rank of every group;
//   4. clusters are sorted by (count desc, group rank, diagonal order) --
//      exactly the stable sort of the reference -- and the first max_out
//      are written.
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

// FxHasher (rustc-hash 2.1.3, 64-bit) over the key (usize contig, Strand):
// h = (0 + contig) * K; h = (h + discriminant) * K; finish = rotl(h, 26).
__device__ __forceinline__ unsigned long long fx_hash_group(uint32_t cid, uint32_t strand) {
  const unsigned long long K = 0xf1357aea2e62a9c5ull;
  unsigned long long h = (unsigned long long)cid * K;
  h = (h + strand) * K;
  return (h << 26) | (h >> 38);
}

__device__ __forceinline__ uint32_t next_pow2(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}

// Block bitonic sort of (key, val) pairs, n a power of two.
__device__ void bitonic_kv(unsigned long long* k, uint32_t* v, uint32_t n) {
  for (uint32_t size = 2; size <= n; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t t = threadIdx.x; t < n / 2; t += blockDim.x) {
        uint32_t i = 2 * t - (t & (stride - 1));
        uint32_t j = i + stride;
        bool asc = (i & size) == 0;
        unsigned long long a = k[i], b = k[j];
        if ((a > b) == asc) {
          k[i] = b;
          k[j] = a;
          uint32_t x = v[i];
          v[i] = v[j];
          v[j] = x;
        }
      }
      __syncthreads();
    }
  }
}

// In-place inclusive block scan (sum) of n elements.
template <class T>
__device__ void block_scan_incl(T* a, uint32_t n, T* warp_tmp) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T carry = 0;
  for (uint32_t base = 0; base < n; base += blockDim.x) {
    uint32_t i = base + threadIdx.x;
    T x = i < n ? a[i] : (T)0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      T y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) warp_tmp[wid] = x;
    __syncthreads();
    if (wid == 0) {
      T s = lane < nw ? warp_tmp[lane] : (T)0;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, s, d);
        if (lane >= d) s += y;
      }
      if (lane < nw) warp_tmp[lane] = s;
    }
    __syncthreads();
    T add = carry + (wid > 0 ? warp_tmp[wid - 1] : (T)0);
    if (i < n) a[i] = x + add;
    T tot = warp_tmp[nw - 1];
    __syncthreads();
    carry += tot;
  }
}

// Capacity of a SwissTable with the given bucket count (bucket_mask_to_capacity).
__device__ __forceinline__ uint32_t swiss_cap(uint32_t buckets) {
  if (buckets == 0) return 0;
  return buckets < 8 ? buckets - 1 : buckets / 8 * 7;
}
// capacity_to_buckets for a capacity request.
__device__ __forceinline__ uint32_t swiss_buckets(uint32_t cap) {
  if (cap < 8) return cap < 4 ? 4 : 8;
  uint32_t adj = (uint32_t)(((unsigned long long)cap * 8) / 7);
  return next_pow2(adj);
}
// find_insert_slot over an empty-marked (0xFFFFFFFF) table.
__device__ __forceinline__ uint32_t swiss_find(const uint32_t* t, uint32_t nb, unsigned long long h, int W) {
  uint32_t mask = nb - 1;
  uint32_t pos = (uint32_t)(h & mask);
  if (nb <= (uint32_t)W) {
    for (uint32_t i = 0; i < nb; i++) {
      uint32_t s = (pos + i) & mask;
      if (t[s] == 0xFFFFFFFFu) return s;
    }
    return 0;
  }
  uint32_t stride = 0;
  for (uint32_t guard = 0; guard <= nb; guard++) {
    for (uint32_t b = 0; b < (uint32_t)W; b++) {
      uint32_t s = (pos + b) & mask;
      if (t[s] == 0xFFFFFFFFu) return s;
    }
    stride += W;
    pos = (pos + stride) & mask;
  }
  return 0xFFFFFFFFu;
}

size_t cluster_smem(uint32_t hmax, int threads) {
  uint32_t np = 1;
  while (np < hmax) np <<= 1;
  // keys 8, vals 4, a 4, b 4, pre 8, gmin 4, gfirst 4, ggk 4, rank 4, clstart 4, clgrp 4 per element
  size_t s = (size_t)np * 52 + 64;
  (void)threads;
  return (s + 15) & ~(size_t)15;
}

// Clusters one read's H hits. Work arrays are carved from base (shared
// memory, or a global scratch slab for reads with very many hits) for
// NP = next_pow2(H) or more elements.
__device__ void cluster_read(const ClusterArgs& p, uint32_t r, uint32_t H, const unsigned long long* hits,
                             unsigned char* base, uint32_t NP, uint32_t* wtmp32, unsigned long long* wtmp64,
                             uint32_t& sh_G, uint32_t& sh_C, bool list_mode) {
  unsigned long long* keys = (unsigned long long*)base;
  unsigned long long* pre = keys + NP;           // NP + 1
  uint32_t* vals = (uint32_t*)(pre + NP + 1);
  uint32_t* a = vals + NP;                       // a and b contiguous: reused as 2*NP slots
  uint32_t* b = a + NP;
  uint32_t* gmin = b + NP;
  uint32_t* gfirst = gmin + NP;
  uint32_t* ggk = gfirst + NP;
  uint32_t* rank = ggk + NP;
  uint32_t* clstart = rank + NP;                 // NP + 1
  uint32_t* clgrp = clstart + NP + 1;
  const uint64_t rg = (uint64_t)p.r0 + r;
  const long long L = (long long)(p.offs[rg + 1] - p.offs[rg]);
  const uint32_t n = next_pow2(H);
  for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
    keys[i] = i < H ? hits[i] : ~0ull;
    vals[i] = i;
  }
  __syncthreads();
  bitonic_kv(keys, vals, n);
  if (p.sorted_hits && !list_mode) {
    for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
      p.sorted_hits[(size_t)r * p.hcap + i] = keys[i];
      p.hit_src[(size_t)r * p.hcap + i] = (uint16_t)vals[i];
    }
  }
  // boundaries
  for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
    unsigned long long k = keys[i];
    uint32_t gk = (uint32_t)(k >> 40);
    long long d = (long long)(k & ((1ull << 40) - 1));
    bool gs = i == 0, cs = i == 0;
    if (i > 0) {
      unsigned long long kp = keys[i - 1];
      gs = (uint32_t)(kp >> 40) != gk;
      long long dp = (long long)(kp & ((1ull << 40) - 1));
      cs = gs || (d - dp > 50);  // MERGE_DISTANCE (candidates.rs:27)
    }
    a[i] = cs ? 1u : 0u;
    b[i] = gs ? 1u : 0u;
    pre[i] = (unsigned long long)d;
  }
  __syncthreads();
  block_scan_incl<uint32_t>(a, H, wtmp32);
  block_scan_incl<uint32_t>(b, H, wtmp32);
  block_scan_incl<unsigned long long>(pre, H, wtmp64);
  if (threadIdx.x == 0) {
    sh_C = a[H - 1];
    sh_G = b[H - 1];
  }
  __syncthreads();
  const uint32_t C = sh_C, G = sh_G;
  for (uint32_t g = threadIdx.x; g < G; g += blockDim.x) gmin[g] = 0xFFFFFFFFu;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
    uint32_t cl = a[i] - 1, g = b[i] - 1;
    bool cs = i == 0 || a[i] != a[i - 1];
    bool gs = i == 0 || b[i] != b[i - 1];
    if (gs) {
      ggk[g] = (uint32_t)(keys[i] >> 40);
      gfirst[g] = cl;
    }
    if (cs) {
      clstart[cl] = i;
      clgrp[cl] = g;
    }
    atomicMin(&gmin[g], vals[i]);
  }
  if (threadIdx.x == 0) clstart[C] = H;
  __syncthreads();
  // group insertion order = ascending first emission index
  const uint32_t ng = next_pow2(G);
  for (uint32_t g = threadIdx.x; g < ng; g += blockDim.x) {
    keys[g] = g < G ? (((unsigned long long)gmin[g] << 32) | g) : ~0ull;
    vals[g] = g;
  }
  __syncthreads();
  bitonic_kv(keys, vals, ng);
  // replay SwissTable insertion (single thread); slots live in a|b
  if (threadIdx.x == 0) {
    uint32_t* slots = a;  // 2*NP entries
    uint32_t nb = 0, items = 0;
    int bad = 0;
    for (uint32_t t = 0; t < G && !bad; t++) {
      uint32_t g = (uint32_t)(keys[t] & 0xFFFFFFFFu);
      uint32_t gk = ggk[g];
      unsigned long long h = fx_hash_group(gk >> 1, gk & 1u);
      if (items + 1 > swiss_cap(nb)) {
        uint32_t need = max(items + 1, swiss_cap(nb) + 1);
        uint32_t nnb = swiss_buckets(need);
        if (nnb > 2 * NP) { bad = 1; break; }
        // rehash: old entries in bucket order into a fresh table at the
        // upper half, then move back (nnb <= 2*NP, old table nb <= NP)
        uint32_t* fresh = slots + (2 * NP - nnb);
        // old table occupies slots[0..nb); fresh region must not overlap it
        if (nb > 2 * NP - nnb) {
          // copy old table out of the way into rank[] scratch (G <= NP)
          for (uint32_t s = 0; s < nb; s++) rank[s] = slots[s];
          for (uint32_t s = 0; s < nnb; s++) fresh[s] = 0xFFFFFFFFu;
          for (uint32_t s = 0; s < nb; s++)
            if (rank[s] != 0xFFFFFFFFu) {
              uint32_t og = rank[s];
              uint32_t ogk = ggk[og];
              uint32_t q = swiss_find(fresh, nnb, fx_hash_group(ogk >> 1, ogk & 1u), p.group_width);
              fresh[q] = og;
            }
        } else {
          for (uint32_t s = 0; s < nnb; s++) fresh[s] = 0xFFFFFFFFu;
          for (uint32_t s = 0; s < nb; s++)
            if (slots[s] != 0xFFFFFFFFu) {
              uint32_t og = slots[s];
              uint32_t ogk = ggk[og];
              uint32_t q = swiss_find(fresh, nnb, fx_hash_group(ogk >> 1, ogk & 1u), p.group_width);
              fresh[q] = og;
            }
        }
        for (uint32_t s = 0; s < nnb; s++) slots[s] = fresh[s];
        nb = nnb;
      }
      uint32_t q = swiss_find(slots, nb, h, p.group_width);
      if (q == 0xFFFFFFFFu) { bad = 1; break; }
      slots[q] = g;
      items++;
    }
    if (bad) {
      atomicExch(p.err, 1);
    } else {
      uint32_t rk = 0;
      for (uint32_t s = 0; s < nb; s++)
        if (slots[s] != 0xFFFFFFFFu) rank[slots[s]] = rk++;
    }
  }
  __syncthreads();
  // cluster order keys: count desc, group rank asc, diagonal order asc
  const uint32_t nc = next_pow2(C);
  for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x) {
    unsigned long long key = ~0ull;
    if (c < C) {
      uint32_t g = clgrp[c];
      uint32_t cnt = clstart[c + 1] - clstart[c];
      key = ((unsigned long long)(0xFFFFFu - cnt) << 44) | ((unsigned long long)rank[g] << 24) |
            (unsigned long long)(c - gfirst[g]);
    }
    keys[c] = key;
    vals[c] = c;
  }
  __syncthreads();
  bitonic_kv(keys, vals, nc);
  const uint32_t nout = min(C, p.max_out);
  for (uint32_t i = threadIdx.x; i < nout; i += blockDim.x) {
    uint32_t c = vals[i];
    uint32_t s = clstart[c], e = clstart[c + 1];
    uint32_t cnt = e - s;
    unsigned long long sumb = pre[e - 1] - (s > 0 ? pre[s - 1] : 0ull);
    long long sum = (long long)sumb - (long long)cnt * (long long)DIAG_BIAS;
    long long avg = sum / (long long)cnt;  // truncation toward zero, as Rust's i64 '/'
    uint32_t gk = ggk[clgrp[c]];
    long long posi = (gk & 1u) ? avg - L + KMER : avg;
    Cand cd;
    cd.pos = posi > 0 ? (unsigned long long)posi : 0ull;
    cd.contig = gk >> 1;
    cd.strand = (uint8_t)(gk & 1u);
    cd.score = cnt;
    cd.pad[0] = 1;
    p.cand[(size_t)r * p.max_out + i] = cd;
    if (p.cand_span) p.cand_span[(size_t)r * p.max_out + i] = list_mode ? 0xFFFFFFFFu : (s | (e << 16));
  }
  if (threadIdx.x == 0) {
    p.n_cand[r] = nout;
    if (p.total_cand) p.total_cand[r] = C;
  }
  __syncthreads();
}

__global__ void k_cluster(ClusterArgs p, uint32_t np_max) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long wtmp64[32];
  __shared__ uint32_t wtmp32[32];
  __shared__ uint32_t sh_G, sh_C;
  for (uint32_t r = blockIdx.x; r < p.nr; r += gridDim.x) {
    const uint32_t H = p.hit_cnt[r];
    if (p.overflow[r]) continue;
    if (!(H > p.h_lo && H <= p.h_hi)) continue;
    if (H == 0) {
      if (threadIdx.x == 0) {
        p.n_cand[r] = 0;
        if (p.total_cand) p.total_cand[r] = 0;
      }
      continue;
    }
    cluster_read(p, r, H, p.hits + (size_t)r * p.hcap, smem_raw, np_max, wtmp32, wtmp64, sh_G, sh_C, false);
  }
}

// Reads with more hits than shared memory sorts (p.h_lo < H <= p.h_hi, both
// above the shared-memory tier): hits in the per-read buffer, work arrays in
// one global slab per block (p.scratch, slab_bytes each).
__global__ void k_cluster_big(ClusterArgs p, uint32_t np_max, size_t slab_bytes) {
  __shared__ unsigned long long wtmp64[32];
  __shared__ uint32_t wtmp32[32];
  __shared__ uint32_t sh_G, sh_C;
  unsigned char* slab = p.scratch + (size_t)blockIdx.x * slab_bytes;
  for (uint32_t r = blockIdx.x; r < p.nr; r += gridDim.x) {
    const uint32_t H = p.hit_cnt[r];
    if (p.overflow[r]) continue;
    if (!(H > p.h_lo && H <= p.h_hi)) continue;
    cluster_read(p, r, H, p.hits + (size_t)r * p.hcap, slab, np_max, wtmp32, wtmp64, sh_G, sh_C, false);
  }
}

// Overflowed reads (list mode): hits in the pool, arrays in global scratch.
__global__ void k_cluster_list(ClusterArgs p) {
  __shared__ unsigned long long wtmp64[32];
  __shared__ uint32_t wtmp32[32];
  __shared__ uint32_t sh_G, sh_C;
  const unsigned int n = *p.list_n;
  const unsigned long long s_lo = (unsigned long long)p.slice * p.pool_slice;
  if (s_lo >= *p.list_total) return;
  for (uint32_t w = blockIdx.x; w < n; w += gridDim.x) {
    if (p.list_hoff[w] / p.pool_slice != p.slice) continue;
    const uint32_t r = p.list[w];
    const uint32_t H = p.need[r];
    const unsigned long long off = p.list_hoff[w] - s_lo;
    uint32_t NP = next_pow2(H);
    cluster_read(p, r, H, p.hits_pool + off, p.scratch + 2 * off * 56, NP, wtmp32, wtmp64, sh_G, sh_C, true);
  }
}

void launch_cluster(const ClusterArgs& a, uint32_t hmax, int threads, cudaStream_t st) {
  uint32_t np = 1;
  while (np < hmax) np <<= 1;
  size_t sm = cluster_smem(hmax, threads);
  int grid = (int)(a.nr < 65535u * 4 ? a.nr : 65535u * 4);
  if (grid < 1) grid = 1;
  cudaFuncSetAttribute(k_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_cluster<<<grid, threads, sm, st>>>(a, np);
}

size_t cluster_big_slab_bytes(uint32_t hmax) {
  uint32_t np = 1;
  while (np < hmax) np <<= 1;
  return ((size_t)np * 56 + 64 + 255) & ~(size_t)255;
}

void launch_cluster_big(const ClusterArgs& a, uint32_t hmax, int grid, cudaStream_t st) {
  uint32_t np = 1;
  while (np < hmax) np <<= 1;
  k_cluster_big<<<grid, 1024, 0, st>>>(a, np, cluster_big_slab_bytes(hmax));
}

void launch_cluster_list(const ClusterArgs& a, int grid, cudaStream_t st) {
  k_cluster_list<<<grid, 256, 0, st>>>(a);
}

}  // namespace pbw
