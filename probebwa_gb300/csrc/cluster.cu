// cluster.cu -- K2: candidate clustering (src/mapper/candidates.rs:30-78),
// one thread block per read.
//
// The reference groups hits by (contig, strand) in an FxHashMap, visits the
// groups in that map's iteration order, sorts each group's diagonals, splits
// at gaps > 50, emits one candidate per cluster (truncating mean diagonal),
// then stable-sorts candidates by hit count, descending.
//
// Reads whose hits fit the per-read buffer take the binned form
// (cluster_read_bins, below the shared helpers): no sort of the hits, a hash
// table of 51-wide diagonal bins. Reads seeded into the overflow pool take
// the sorted form (cluster_read), in global scratch:
//   1. the read's hit words ((contig, strand) << 40 | diagonal) are sorted
//      (bitonic, key + emission index), which makes every group contiguous
//      with ascending diagonals;
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

// std's SwissTable insertion replayed over the G groups in insertion order
// (order[t] & 0xFFFFFFFF is the t-th group; ggk[g] its (contig << 1 | strand)
// key), with FxHasher and probe groups of W buckets; rank[g] receives the
// group's iteration position. slots holds cap2 >= 2 * next_pow2(G) buckets
// (the largest table of G items with room for a rehash copy); rank doubles
// as rehash scratch. Returns false if the table would outgrow slots.
__device__ bool swiss_replay(const unsigned long long* order, uint32_t G, const uint32_t* ggk, uint32_t* slots,
                             uint32_t cap2, uint32_t* rank, int W) {
  uint32_t nb = 0, items = 0;
  for (uint32_t t = 0; t < G; t++) {
    const uint32_t g = (uint32_t)(order[t] & 0xFFFFFFFFu);
    const uint32_t gk = ggk[g];
    const unsigned long long h = fx_hash_group(gk >> 1, gk & 1u);
    if (items + 1 > swiss_cap(nb)) {
      const uint32_t need = max(items + 1, swiss_cap(nb) + 1);
      const uint32_t nnb = swiss_buckets(need);
      if (nnb > cap2) return false;
      // rehash: old entries in bucket order into a fresh table at the upper
      // end, then move back; when the regions overlap the old table is first
      // copied out to rank[] (nb <= G entries of scratch)
      uint32_t* fresh = slots + (cap2 - nnb);
      const uint32_t* old = slots;
      if (nb > cap2 - nnb) {
        for (uint32_t s = 0; s < nb; s++) rank[s] = slots[s];
        old = rank;
      }
      for (uint32_t s = 0; s < nnb; s++) fresh[s] = 0xFFFFFFFFu;
      for (uint32_t s = 0; s < nb; s++) {
        if (old[s] == 0xFFFFFFFFu) continue;
        const uint32_t og = old[s];
        const uint32_t ogk = ggk[og];
        const uint32_t q = swiss_find(fresh, nnb, fx_hash_group(ogk >> 1, ogk & 1u), W);
        fresh[q] = og;
      }
      for (uint32_t s = 0; s < nnb; s++) slots[s] = fresh[s];
      nb = nnb;
    }
    const uint32_t q = swiss_find(slots, nb, h, W);
    if (q == 0xFFFFFFFFu) return false;
    slots[q] = g;
    items++;
  }
  uint32_t rk = 0;
  for (uint32_t s = 0; s < nb; s++)
    if (slots[s] != 0xFFFFFFFFu) rank[slots[s]] = rk++;
  return true;
}

uint32_t next_pow2_host(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}


// Clusters one read's H hits. Work arrays are carved from base (shared
// memory, or a global scratch slab for reads with very many hits) for
// NP = next_pow2(H) or more elements.
__device__ void cluster_read(const ClusterArgs& p, uint32_t r, uint32_t H, const unsigned long long* hits,
                             unsigned char* base, uint32_t NP, uint32_t* wtmp32, unsigned long long* wtmp64,
                             uint32_t& sh_G, uint32_t& sh_C) {
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
  if (threadIdx.x == 0 && !swiss_replay(keys, G, ggk, a, 2 * NP, rank, p.group_width)) atomicExch(p.err, 1);
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
  }
  if (p.feat) {
    // no hit-level features for reads clustered from the pool: feature 0 = -1
    // makes the ranker keep all their candidates
    for (uint32_t i = threadIdx.x; i < (uint32_t)MAX_CAND * RANK_FEATURES; i += blockDim.x)
      p.feat[(size_t)r * MAX_CAND * RANK_FEATURES + i] =
          (i % RANK_FEATURES == 0 && i / RANK_FEATURES < nout) ? -1.f : 0.f;
  }
  if (threadIdx.x == 0) {
    p.n_cand[r] = nout;
    if (p.total_cand) p.total_cand[r] = C;
  }
  __syncthreads();
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
    cluster_read(p, r, H, p.hits_pool + off, p.scratch + 2 * off * 56, NP, wtmp32, wtmp64, sh_G, sh_C);
  }
}

// ---------------------------------------------------------------------------
// K2 by diagonal bins. The clusters of cluster_hits are the maximal runs of a
// group's sorted diagonals whose neighbours differ by at most MERGE_DISTANCE
// (50). Cut the diagonal axis into bins of 51: two hits of one bin are at
// most 50 apart, so a bin never splits; bins two or more apart are more than
// 50 apart, so they never join; two adjacent bins join exactly when the lower
// one's largest diagonal and the upper one's smallest are at most 50 apart.
// So the hits need no sort: a hash table keyed by (group, bin) collects each
// bin's hit count, diagonal sum, diagonal set (a 51-bit mask: smallest,
// largest and distinct diagonals) and first emission index with shared-memory
// atomics, and only the non-empty bins are sorted. From the sorted bins come
// the group boundaries, the clusters (runs of joined bins), each group's
// first emission index -- the FxHashMap insertion order whose SwissTable
// replay gives the iteration order -- and the cluster order of the
// reference's stable sort (count desc, group rank, diagonal order).
// ---------------------------------------------------------------------------
constexpr int BIN_W = 51;  // MERGE_DISTANCE + 1 (candidates.rs:27)
constexpr unsigned long long BIN_EMPTY = ~0ull;
constexpr unsigned long long M40 = (1ull << 40) - 1;

__device__ __forceinline__ uint32_t bin_slot(unsigned long long key, uint32_t T) {
  unsigned long long k = key ^ (key >> 33);
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return (uint32_t)k & (T - 1);
}

// Per-block scratch of the bin path (global slab): arrays of NPB entries.
struct BinScratch {
  unsigned long long *ckey, *cacc, *cmask, *ps, *cinf;
  uint32_t *cemin, *a, *bb, *pc, *gmin, *ggk, *gfirst, *rank, *clstart, *clgrp, *slots, *crmn, *crmx, *perm;
  __device__ void carve(unsigned char* base, uint32_t NPB) {
    unsigned long long* q = (unsigned long long*)base;
    ckey = q; cacc = q + NPB; cmask = q + 2 * NPB; ps = q + 3 * NPB; cinf = q + 4 * NPB;
    uint32_t* u = (uint32_t*)(q + 5 * NPB);
    cemin = u; a = u + NPB; bb = u + 2 * NPB; pc = u + 3 * NPB; gmin = u + 4 * NPB; ggk = u + 5 * NPB;
    gfirst = u + 6 * NPB; rank = u + 7 * NPB; clstart = u + 8 * NPB; clgrp = u + 9 * NPB + 1;
    slots = u + 10 * NPB + 2;  // 2 * NPB
    crmn = u + 12 * NPB + 2; crmx = u + 13 * NPB + 2; perm = u + 14 * NPB + 2;
  }
};
__host__ __device__ inline size_t bin_scratch_bytes(uint32_t NPB) {
  return (((size_t)NPB * (5 * 8 + 15 * 4) + 64) + 255) & ~(size_t)255;
}
// table entry: key, count | diagonal-offset sum, diagonal mask, first emission
// (28 bytes); with the ranker's features also exact hits | bucket-size sum
// and the smallest and largest read position (16 bytes)
__host__ __device__ inline size_t bin_table_bytes(uint32_t T, bool feat = false) {
  return (size_t)T * (feat ? 44 : 28);
}

// Clusters one read's H hits with a table of T = next_pow2(H) entries at tab
// (room for TMAX), scratch S of TMAX entries and sort space of 12 * TMAX
// bytes at sortbuf.
template <bool FEAT>
__device__ void cluster_read_bins(const ClusterArgs& p, uint32_t r, uint32_t H, const unsigned long long* hits,
                                  unsigned char* tab, const BinScratch& S, unsigned char* sortbuf,
                                  uint32_t* wtmp32, unsigned long long* wtmp64, uint32_t& sh_n) {
  const uint32_t T = next_pow2(H);  // >= H >= the bins of the read
  unsigned long long* tkey = (unsigned long long*)tab;
  unsigned long long* tacc = tkey + T;
  unsigned long long* tmask = tacc + T;
  unsigned long long* tinf = tmask + T;                        // FEAT
  uint32_t* temin = (uint32_t*)(tmask + (FEAT ? 2 : 1) * T);
  uint32_t* trmn = temin + T;                                  // FEAT
  uint32_t* trmx = trmn + T;                                   // FEAT
  for (uint32_t s = threadIdx.x; s < T; s += blockDim.x) {
    tkey[s] = BIN_EMPTY;
    tacc[s] = 0;
    tmask[s] = 0;
    temin[s] = 0xFFFFFFFFu;
    if (FEAT) {
      tinf[s] = 0;
      trmn[s] = 0xFFFFFFFFu;
      trmx[s] = 0;
    }
  }
  if (threadIdx.x == 0) sh_n = 0;
  __syncthreads();
  // aggregate: one table entry per (group, bin)
  for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
    const unsigned long long w = hits[i];
    const unsigned long long d = w & M40;
    const unsigned long long b = d / BIN_W;
    const uint32_t off = (uint32_t)(d - b * BIN_W);
    const unsigned long long key = ((w >> 40) << 35) | b;
    uint32_t s = bin_slot(key, T);
    for (uint32_t guard = 0; guard < T; guard++) {
      const unsigned long long prev = atomicCAS(&tkey[s], BIN_EMPTY, key);
      if (prev == BIN_EMPTY || prev == key) break;
      s = (s + 1) & (T - 1);
    }
    atomicAdd(&tacc[s], (1ull << 40) | off);
    atomicOr(&tmask[s], 1ull << off);
    atomicMin(&temin[s], i);
    if (FEAT) {
      // hit info: read position | log2 exact bucket size << 10 | neighbour << 15
      const uint32_t info = p.hit_info[(size_t)r * p.hcap + i];
      atomicAdd(&tinf[s], ((info >> 15) ? 0ull : (1ull << 32)) | ((info >> 10) & 31u));
      atomicMin(&trmn[s], info & 0x3FFu);
      atomicMax(&trmx[s], info & 0x3FFu);
    }
  }
  __syncthreads();
  // compact the non-empty bins (any order: they are sorted next)
  for (uint32_t s = threadIdx.x; s < T; s += blockDim.x) {
    if (tkey[s] == BIN_EMPTY) continue;
    const uint32_t k = atomicAdd(&sh_n, 1u);
    S.ckey[k] = tkey[s];
    S.cacc[k] = tacc[s];
    S.cmask[k] = tmask[s];
    S.cemin[k] = temin[s];
    if (FEAT) {
      S.cinf[k] = tinf[s];
      S.crmn[k] = trmn[s];
      S.crmx[k] = trmx[s];
    }
  }
  __syncthreads();
  const uint32_t nb = sh_n;
  // sort the bins by (group, bin)
  const uint32_t nbp = next_pow2(nb);
  unsigned long long* skey = (unsigned long long*)sortbuf;
  uint32_t* sval = (uint32_t*)(skey + nbp);
  for (uint32_t i = threadIdx.x; i < nbp; i += blockDim.x) {
    skey[i] = i < nb ? S.ckey[i] : ~0ull;
    sval[i] = i;
  }
  __syncthreads();
  bitonic_kv(skey, sval, nbp);
  // bin i of the sorted order: group and cluster starts, count and diagonal sum
  for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) {
    const unsigned long long key = skey[i];
    const uint32_t e = sval[i];
    const unsigned long long b = key & ((1ull << 35) - 1);
    const unsigned long long acc = S.cacc[e];
    const uint32_t cnt = (uint32_t)(acc >> 40);
    bool gs = i == 0, cs = i == 0;
    if (i > 0) {
      const unsigned long long kp = skey[i - 1];
      gs = (kp >> 35) != (key >> 35);
      const unsigned long long bp = kp & ((1ull << 35) - 1);
      const unsigned long long lo = b * BIN_W + (unsigned long long)(__ffsll((long long)S.cmask[e]) - 1);
      const unsigned long long hi = bp * BIN_W + (unsigned long long)(63 - __clzll((long long)S.cmask[sval[i - 1]]));
      cs = gs || bp + 1 != b || lo - hi > (unsigned long long)(BIN_W - 1);
    }
    S.a[i] = cs ? 1u : 0u;
    S.bb[i] = gs ? 1u : 0u;
    S.pc[i] = cnt;
    S.ps[i] = b * BIN_W * cnt + (acc & M40);
    if (FEAT) S.perm[i] = e;
  }
  __syncthreads();
  block_scan_incl<uint32_t>(S.a, nb, wtmp32);
  block_scan_incl<uint32_t>(S.bb, nb, wtmp32);
  block_scan_incl<uint32_t>(S.pc, nb, wtmp32);
  block_scan_incl<unsigned long long>(S.ps, nb, wtmp64);
  const uint32_t C = S.a[nb - 1], G = S.bb[nb - 1];
  for (uint32_t g = threadIdx.x; g < G; g += blockDim.x) S.gmin[g] = 0xFFFFFFFFu;
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) {
    const uint32_t cl = S.a[i] - 1, g = S.bb[i] - 1;
    const bool cs = i == 0 || S.a[i] != S.a[i - 1];
    const bool gs = i == 0 || S.bb[i] != S.bb[i - 1];
    if (gs) {
      S.ggk[g] = (uint32_t)(skey[i] >> 35);
      S.gfirst[g] = cl;
    }
    if (cs) {
      S.clstart[cl] = i;
      S.clgrp[cl] = g;
    }
    atomicMin(&S.gmin[g], S.cemin[sval[i]]);
  }
  if (threadIdx.x == 0) S.clstart[C] = nb;
  __syncthreads();
  // group insertion order = ascending first emission index; SwissTable replay
  const uint32_t ng = next_pow2(G);
  for (uint32_t g = threadIdx.x; g < ng; g += blockDim.x) {
    skey[g] = g < G ? (((unsigned long long)S.gmin[g] << 32) | g) : ~0ull;
    sval[g] = g;
  }
  __syncthreads();
  bitonic_kv(skey, sval, ng);
  // (a table of G items never needs more than 2 * next_pow2(G) buckets, and
  // a small one starts at 4 or 8)
  if (threadIdx.x == 0 && !swiss_replay(skey, G, S.ggk, S.slots, max(16u, 2 * ng), S.rank, p.group_width))
    atomicExch(p.err, 1);
  __syncthreads();
  // clusters by (count desc, group rank, diagonal order)
  const uint32_t nc = next_pow2(C);
  for (uint32_t c = threadIdx.x; c < nc; c += blockDim.x) {
    unsigned long long key = ~0ull;
    if (c < C) {
      const uint32_t g = S.clgrp[c];
      const uint32_t s = S.clstart[c], e = S.clstart[c + 1];
      const uint32_t cnt = S.pc[e - 1] - (s > 0 ? S.pc[s - 1] : 0u);
      key = ((unsigned long long)(0xFFFFFu - cnt) << 44) | ((unsigned long long)S.rank[g] << 24) |
            (unsigned long long)(c - S.gfirst[g]);
    }
    skey[c] = key;
    sval[c] = c;
  }
  __syncthreads();
  bitonic_kv(skey, sval, nc);
  const uint64_t rg = (uint64_t)p.r0 + r;
  const long long L = (long long)(p.offs[rg + 1] - p.offs[rg]);
  const uint32_t nout = min(C, p.max_out);
  for (uint32_t i = threadIdx.x; i < nout; i += blockDim.x) {
    const uint32_t c = sval[i];
    const uint32_t s = S.clstart[c], e = S.clstart[c + 1];
    const uint32_t cnt = S.pc[e - 1] - (s > 0 ? S.pc[s - 1] : 0u);
    const unsigned long long sumb = S.ps[e - 1] - (s > 0 ? S.ps[s - 1] : 0ull);
    const long long sum = (long long)sumb - (long long)cnt * (long long)DIAG_BIAS;
    const long long avg = sum / (long long)cnt;  // truncation toward zero, as Rust's i64 '/'
    const uint32_t gk = S.ggk[S.clgrp[c]];
    const long long posi = (gk & 1u) ? avg - L + KMER : avg;
    Cand cd;
    cd.pos = posi > 0 ? (unsigned long long)posi : 0ull;
    cd.contig = gk >> 1;
    cd.strand = (uint8_t)(gk & 1u);
    cd.score = cnt;
    cd.pad[0] = 1;
    p.cand[(size_t)r * p.max_out + i] = cd;
  }
  if (FEAT) {
    // the candidate ranker's seed features of each kept candidate (a warp per
    // candidate): exact and one-mismatch hits, distinct diagonals, diagonal
    // spread, read span of the hits, read length, mean base quality, rank and
    // list size, mean log2 exact-bucket size (slots 7 and 8 are the mate
    // features, filled for pairs later)
    uint32_t qs = 0;
    const uint64_t q0 = p.offs[rg];
    for (uint32_t k = threadIdx.x; k < (uint32_t)L; k += blockDim.x) qs += p.quals[q0 + k];
    for (int d = 16; d; d >>= 1) qs += __shfl_xor_sync(0xffffffffu, qs, d);
    if ((threadIdx.x & 31) == 0) wtmp32[threadIdx.x >> 5] = qs;
    __syncthreads();
    if (threadIdx.x == 0) {
      uint32_t t = 0;
      for (uint32_t w = 0; w < blockDim.x / 32; w++) t += wtmp32[w];
      sh_n = t;
    }
    __syncthreads();
    const float meanq = L ? (float)sh_n / (float)L : 0.f;
    for (uint32_t i = threadIdx.x; i < (uint32_t)MAX_CAND; i += blockDim.x) {
      float* f = p.feat + ((size_t)r * MAX_CAND + i) * RANK_FEATURES;
      if (i >= nout) {
        for (int k = 0; k < RANK_FEATURES; k++) f[k] = 0.f;
        continue;
      }
      const uint32_t c = sval[i];
      const uint32_t s = S.clstart[c], e = S.clstart[c + 1];
      uint32_t ne = 0, nd = 0, l2s = 0, rmin = 0xFFFFFFFFu, rmax = 0;
      for (uint32_t k = s; k < e; k++) {
        const uint32_t ce = S.perm[k];
        ne += (uint32_t)(S.cinf[ce] >> 32);
        l2s += (uint32_t)(S.cinf[ce] & 0xFFFFFFFFu);
        nd += (uint32_t)__popcll(S.cmask[ce]);
        rmin = min(rmin, S.crmn[ce]);
        rmax = max(rmax, S.crmx[ce]);
      }
      const uint32_t cf = S.perm[s], cl = S.perm[e - 1];
      const unsigned long long lo = (S.ckey[cf] & ((1ull << 35) - 1)) * BIN_W +
                                    (unsigned long long)(__ffsll((long long)S.cmask[cf]) - 1);
      const unsigned long long hi = (S.ckey[cl] & ((1ull << 35) - 1)) * BIN_W +
                                    (unsigned long long)(63 - __clzll((long long)S.cmask[cl]));
      const uint32_t nh = S.pc[e - 1] - (s > 0 ? S.pc[s - 1] : 0u);
      f[0] = log2f(1.f + (float)ne);
      f[1] = log2f(1.f + (float)(nh - ne));
      f[2] = log2f(1.f + (float)nd);
      f[3] = log2f(1.f + (float)(hi - lo));
      f[4] = log2f(1.f + (nh ? (float)(rmax - rmin + KMER) : 0.f));
      f[5] = (float)L;
      f[6] = meanq;
      f[7] = 10.f;
      f[8] = 0.f;
      f[9] = (float)i;
      f[10] = (float)nout;
      f[11] = nh ? (float)l2s / (float)nh : 0.f;
    }
  }
  if (threadIdx.x == 0) {
    p.n_cand[r] = nout;
    if (p.total_cand) p.total_cand[r] = C;
  }
  __syncthreads();
}

// Reads of h_lo < H <= h_hi hits (h_hi <= T) from the per-read buffer. The
// table sits in shared memory, or with GT in the block's slab; FEAT adds the
// candidate ranker's features.
template <bool GT, bool FEAT>
__global__ void k_cluster_bins(ClusterArgs p, uint32_t T, size_t slab_bytes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long wtmp64[32];
  __shared__ uint32_t wtmp32[32];
  __shared__ uint32_t sh_n;
  unsigned char* slab = p.scratch + (size_t)blockIdx.x * slab_bytes;
  BinScratch S;
  S.carve(slab, T);
  unsigned char* tab = GT ? slab + bin_scratch_bytes(T) : smem_raw;
  unsigned char* sortbuf = GT ? tab + bin_table_bytes(T, FEAT) : smem_raw;
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
    cluster_read_bins<FEAT>(p, r, H, p.hits + (size_t)r * p.hcap, tab, S, sortbuf, wtmp32, wtmp64, sh_n);
  }
}

size_t cluster_bins_slab_bytes(uint32_t hmax, bool table_in_slab) {
  const uint32_t T = next_pow2_host(hmax);
  return bin_scratch_bytes(T) + (table_in_slab ? bin_table_bytes(T, true) + (size_t)T * 12 : 0);
}

size_t cluster_bins_smem_bytes(uint32_t hmax, bool feat) {
  // the table, later reused as sort space (12 bytes per entry)
  const uint32_t T = next_pow2_host(hmax);
  return std::max(bin_table_bytes(T, feat), (size_t)T * 12);
}

template <bool GT, bool FEAT>
static void launch_bins(const ClusterArgs& a, uint32_t T, int threads, int grid, size_t slab, cudaStream_t st) {
  const size_t sm = GT ? 0 : cluster_bins_smem_bytes(T, FEAT);
  if (!GT) cudaFuncSetAttribute(k_cluster_bins<GT, FEAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_cluster_bins<GT, FEAT><<<grid, threads, sm, st>>>(a, T, slab);
}

void launch_cluster_bins(const ClusterArgs& a, uint32_t hmax, int threads, int grid, bool table_in_slab,
                         cudaStream_t st) {
  const uint32_t T = next_pow2_host(hmax);
  const size_t slab = cluster_bins_slab_bytes(hmax, table_in_slab);
  const bool feat = a.feat != nullptr;
  if (table_in_slab) {
    if (feat) launch_bins<true, true>(a, T, threads, grid, slab, st);
    else launch_bins<true, false>(a, T, threads, grid, slab, st);
  } else {
    if (feat) launch_bins<false, true>(a, T, threads, grid, slab, st);
    else launch_bins<false, false>(a, T, threads, grid, slab, st);
  }
}

void launch_cluster_list(const ClusterArgs& a, int grid, cudaStream_t st) {
  k_cluster_list<<<grid, 256, 0, st>>>(a);
}

}  // namespace pbw
