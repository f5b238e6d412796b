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
// K2 by diagonal bins, without sorting. The clusters of cluster_hits are the
// maximal runs of a group's sorted diagonals whose neighbours differ by at
// most MERGE_DISTANCE (50). Cut the diagonal axis into bins of 51: two hits
// of one bin are at most 50 apart, so a bin never splits; bins two or more
// apart are more than 50 apart, so they never join; two adjacent bins join
// exactly when the lower one's largest diagonal and the upper one's smallest
// are at most 50 apart. Per read (one block):
//   A. every hit goes into a hash table keyed by (group, bin) -- hit count,
//      diagonal sum, the bin's diagonal set as a 51-bit mask -- and its group
//      into a second table holding the group's first emission index (the
//      FxHashMap insertion order);
//   B. a bin whose lower neighbour does not join it starts a cluster; its
//      thread walks the upper neighbours by lookups and records the
//      cluster's count, diagonal sum, group and first bin;
//   C. the groups, sorted by first emission, are replayed through std's
//      SwissTable insertion (FxHasher of rustc-hash 2.1.3, probing by the
//      group width), which gives each group's iteration rank;
//   D. the reference's final stable sort orders clusters by (count desc,
//      group rank, diagonal order); the key (0x7FFF - count) << 49 | rank
//      << 35 | first bin is unique per cluster, and only the first max_out
//      are needed: a radix select finds the max_out-th key and the keys up
//      to it are sorted.
// With the candidate ranker, bins and clusters also carry each candidate's
// seed features (exact hits, bucket sizes, read positions).
// ---------------------------------------------------------------------------
constexpr int BIN_W = 51;  // MERGE_DISTANCE + 1 (candidates.rs:27)
constexpr unsigned long long BIN_EMPTY = ~0ull;
constexpr uint32_t GRP_EMPTY = 0xFFFFFFFFu;  // group keys (contig << 1 | strand) are below 2^24
constexpr uint32_t NO_SLOT = 0xFFFFFFFFu;
constexpr unsigned long long M40 = (1ull << 40) - 1;
constexpr unsigned long long M35 = (1ull << 35) - 1;
// smallest bin table: room, after the cluster keys, for the selection
// (Tb + 384 of the bin region's 3Tb words)
constexpr uint32_t BIN_TMIN = 256;
constexpr uint32_t BIN_MAX_OUT = 256;  // candidates one read may return

// Table sizes of a read of H hits: bins at load <= 0.625 (a read's hits are
// mostly in bins of their own, and probe runs of a fuller open-addressed
// table grow fast), groups in a power of two at least as large.
__host__ __device__ inline uint32_t np2(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}
__host__ __device__ inline uint32_t bin_tsize(uint32_t H) {
  const uint32_t t = ((uint32_t)(((uint64_t)H * 8 + 4) / 5) + 31) & ~31u;
  return t < BIN_TMIN ? BIN_TMIN : t;
}
__host__ __device__ inline uint32_t grp_tsize(uint32_t H) { return np2(bin_tsize(H)); }

__device__ __forceinline__ uint32_t hash_slot(unsigned long long key, uint32_t T) {
  unsigned long long k = key ^ (key >> 33);
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return (uint32_t)(((k & 0xFFFFFFFFull) * T) >> 32);  // any T
}

// Slot of key in an open-addressed table of T (a power of two) 64-bit keys,
// inserting it if absent (a table never holds more than T keys).
__device__ __forceinline__ uint32_t insert64(unsigned long long* keys, unsigned long long key, uint32_t T) {
  uint32_t s = hash_slot(key, T);
  for (uint32_t guard = 0; guard < T; guard++) {
    const unsigned long long cur = keys[s];
    if (cur == key) return s;
    if (cur == BIN_EMPTY) {
      const unsigned long long prev = atomicCAS(&keys[s], BIN_EMPTY, key);
      if (prev == BIN_EMPTY || prev == key) return s;
    }
    s = s + 1 < T ? s + 1 : 0;
  }
  return NO_SLOT;
}
__device__ __forceinline__ uint32_t find64(const unsigned long long* keys, unsigned long long key, uint32_t T) {
  uint32_t s = hash_slot(key, T);
  for (uint32_t guard = 0; guard < T; guard++) {
    const unsigned long long cur = keys[s];
    if (cur == key) return s;
    if (cur == BIN_EMPTY) return NO_SLOT;
    s = s + 1 < T ? s + 1 : 0;
  }
  return NO_SLOT;
}
__device__ __forceinline__ uint32_t insert32(uint32_t* keys, uint32_t key, uint32_t T) {
  uint32_t s = hash_slot(key, T);
  for (uint32_t guard = 0; guard < T; guard++) {
    const uint32_t cur = keys[s];
    if (cur == key) return s;
    if (cur == GRP_EMPTY) {
      const uint32_t prev = atomicCAS(&keys[s], GRP_EMPTY, key);
      if (prev == GRP_EMPTY || prev == key) return s;
    }
    s = s + 1 < T ? s + 1 : 0;
  }
  return NO_SLOT;
}
__device__ __forceinline__ uint32_t find32(const uint32_t* keys, uint32_t key, uint32_t T) {
  uint32_t s = hash_slot(key, T);
  for (uint32_t guard = 0; guard < T; guard++) {
    const uint32_t cur = keys[s];
    if (cur == key) return s;
    if (cur == GRP_EMPTY) return NO_SLOT;
    s = s + 1 < T ? s + 1 : 0;
  }
  return NO_SLOT;
}

// Tables of one read of up to hmax hits: bins (key, count << 40 | offset
// sum, diagonal mask; with the ranker also exact hits << 32 | bucket-size
// sum and the read-position range) and groups (key, first emission then
// rank).
__host__ __device__ inline size_t bin_table_bytes(uint32_t hmax, bool feat) {
  return (size_t)bin_tsize(hmax) * (feat ? 40 : 24) + (size_t)grp_tsize(hmax) * 8;
}
// Per-block cluster records in the global slab (TM entries each): diagonal
// sum, first bin, count, group slot, group key; with the ranker exact hits,
// bucket-size sum, distinct diagonals, read-position range and diagonal
// spread; and the SwissTable replay's buckets.
struct ClusterRecs {
  unsigned long long *sum, *b0;
  uint32_t *cnt, *gslot, *gk, *ne, *l2s, *nd, *rmn, *rmx, *spread, *slots;
  __device__ void carve(unsigned char* base, uint32_t hmax) {
    const uint32_t TM = bin_tsize(hmax);
    unsigned long long* q = (unsigned long long*)base;
    sum = q;
    b0 = q + TM;
    uint32_t* u = (uint32_t*)(q + 2 * TM);
    cnt = u; gslot = u + TM; gk = u + 2 * TM; ne = u + 3 * TM; l2s = u + 4 * TM; nd = u + 5 * TM;
    rmn = u + 6 * TM; rmx = u + 7 * TM; spread = u + 8 * TM;
    slots = u + 9 * TM;  // 2 * grp_tsize(hmax)
  }
};
__host__ __device__ inline size_t cluster_recs_bytes(uint32_t hmax) {
  return ((size_t)bin_tsize(hmax) * (2 * 8 + 9 * 4) + (size_t)grp_tsize(hmax) * 8 + 255) & ~(size_t)255;
}

template <bool FEAT>
__device__ void cluster_read_bins(const ClusterArgs& p, uint32_t r, uint32_t H, const unsigned long long* hits,
                                  unsigned char* tab, const ClusterRecs& S, uint32_t* wtmp32,
                                  unsigned long long* wtmp64, uint32_t& sh_n, uint32_t* sh_sel, uint32_t* sh_hist) {
  const uint32_t T = bin_tsize(H);   // bin slots (the bins and clusters of the read <= H)
  const uint32_t TG = grp_tsize(H);  // group slots
  unsigned long long* bkey = (unsigned long long*)tab;
  unsigned long long* bacc = bkey + T;
  unsigned long long* bmask = bacc + T;
  unsigned long long* binf = bmask + T;                         // FEAT
  uint32_t* brmn = (uint32_t*)(bmask + (FEAT ? 2 : 1) * T);     // FEAT
  uint32_t* brmx = brmn + T;                                    // FEAT
  uint32_t* gkey = (uint32_t*)tab + (FEAT ? 10 : 6) * T;
  uint32_t* gval = gkey + TG;
  for (uint32_t s = threadIdx.x; s < TG; s += blockDim.x) {
    gkey[s] = GRP_EMPTY;
    gval[s] = 0xFFFFFFFFu;
  }
  for (uint32_t s = threadIdx.x; s < T; s += blockDim.x) {
    bkey[s] = BIN_EMPTY;
    bacc[s] = 0;
    bmask[s] = 0;
    if (FEAT) {
      binf[s] = 0;
      brmn[s] = 0xFFFFFFFFu;
      brmx[s] = 0;
    }
  }
  if (threadIdx.x == 0) sh_n = 0;
  __syncthreads();
  // A. bins and groups
  for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
    const unsigned long long w = hits[i];
    const unsigned long long d = w & M40;
    const unsigned long long b = d / BIN_W;
    const uint32_t off = (uint32_t)(d - b * BIN_W);
    const uint32_t gk = (uint32_t)(w >> 40);
    const uint32_t s = insert64(bkey, ((unsigned long long)gk << 35) | b, T);
    const uint32_t g = insert32(gkey, gk, TG);
    if (s == NO_SLOT || g == NO_SLOT) {
      atomicExch(p.err, 1);
      continue;
    }
    atomicAdd(&bacc[s], (1ull << 40) | off);
    atomicOr(&bmask[s], 1ull << off);
    if (gval[g] > i) atomicMin(&gval[g], i);
    if (FEAT) {
      // hit info: read position | log2 exact bucket size << 10 | neighbour << 15
      const uint32_t info = p.hit_info[(size_t)r * p.hcap + i];
      atomicAdd(&binf[s], ((info >> 15) ? 0ull : (1ull << 32)) | ((info >> 10) & 31u));
      atomicMin(&brmn[s], info & 0x3FFu);
      atomicMax(&brmx[s], info & 0x3FFu);
    }
  }
  __syncthreads();
  // B. clusters: runs of joined bins, walked from each run's first bin
  for (uint32_t s = threadIdx.x; s < T; s += blockDim.x) {
    const unsigned long long key = bkey[s];
    if (key == BIN_EMPTY) continue;
    const unsigned long long b = key & M35;
    unsigned long long m = bmask[s];
    const unsigned long long lo = b * BIN_W + (unsigned long long)(__ffsll((long long)m) - 1);
    if (b > 0) {
      const uint32_t q = find64(bkey, key - 1, T);
      if (q != NO_SLOT &&
          lo - ((b - 1) * BIN_W + (unsigned long long)(63 - __clzll((long long)bmask[q]))) <= (unsigned)(BIN_W - 1))
        continue;  // joined to the bin below
    }
    uint32_t cnt = 0, ne = 0, l2s = 0, nd = 0, rmn = 0xFFFFFFFFu, rmx = 0;
    unsigned long long sum = 0, cb = b;
    uint32_t cur = s;
    while (true) {
      const unsigned long long acc = bacc[cur];
      const uint32_t c = (uint32_t)(acc >> 40);
      cnt += c;
      sum += cb * BIN_W * c + (acc & M40);
      if (FEAT) {
        ne += (uint32_t)(binf[cur] >> 32);
        l2s += (uint32_t)(binf[cur] & 0xFFFFFFFFu);
        nd += (uint32_t)__popcll(m);
        rmn = min(rmn, brmn[cur]);
        rmx = max(rmx, brmx[cur]);
      }
      const uint32_t q = find64(bkey, key - b + cb + 1, T);
      if (q == NO_SLOT) break;
      const unsigned long long mq = bmask[q];
      const unsigned long long hi = cb * BIN_W + (unsigned long long)(63 - __clzll((long long)m));
      if ((cb + 1) * BIN_W + (unsigned long long)(__ffsll((long long)mq) - 1) - hi > (unsigned)(BIN_W - 1)) break;
      cur = q;
      m = mq;
      cb++;
    }
    const uint32_t k = atomicAdd(&sh_n, 1u);
    const uint32_t gk = (uint32_t)(key >> 35);
    S.cnt[k] = cnt;
    S.sum[k] = sum;
    S.b0[k] = b;
    S.gk[k] = gk;
    S.gslot[k] = find32(gkey, gk, TG);
    if (FEAT) {
      S.ne[k] = ne;
      S.l2s[k] = l2s;
      S.nd[k] = nd;
      S.rmn[k] = rmn;
      S.rmx[k] = rmx;
      S.spread[k] = (uint32_t)(cb * BIN_W + (unsigned long long)(63 - __clzll((long long)m)) - lo);
    }
  }
  __syncthreads();
  const uint32_t C = sh_n;
  // C. groups in first-emission order, SwissTable replay (the bin table's
  // space holds the sort); gval becomes the group's iteration rank
  unsigned long long* okey = bkey;               // ng <= TG <= 2T words
  uint32_t* oval = (uint32_t*)(bkey + 2 * T);    // ng <= 2T half-words
  __syncthreads();
  if (threadIdx.x == 0) sh_n = 0;
  __syncthreads();
  for (uint32_t g = threadIdx.x; g < TG; g += blockDim.x) {
    if (gkey[g] == GRP_EMPTY) continue;
    const uint32_t k = atomicAdd(&sh_n, 1u);
    okey[k] = ((unsigned long long)gval[g] << 32) | g;
  }
  __syncthreads();
  const uint32_t G = sh_n;
  const uint32_t ng = next_pow2(G);
  for (uint32_t k = threadIdx.x; k < ng; k += blockDim.x) {
    if (k >= G) okey[k] = ~0ull;
    oval[k] = k;
  }
  __syncthreads();
  bitonic_kv(okey, oval, ng);
  if (threadIdx.x == 0 && !swiss_replay(okey, G, gkey, S.slots, max(16u, 2 * ng), gval, p.group_width))
    atomicExch(p.err, 1);
  __syncthreads();
  // D. cluster order keys (count desc, group rank, diagonal order); the first
  // max_out by repeated block-wide minima
  unsigned long long* ck = bkey;
  for (uint32_t c = threadIdx.x; c < C; c += blockDim.x)
    ck[c] = ((unsigned long long)(0x7FFFu - S.cnt[c]) << 49) | ((unsigned long long)gval[S.gslot[c]] << 35) | S.b0[c];
  __syncthreads();
  const uint32_t nout = min(min(C, p.max_out), BIN_MAX_OUT);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // the nout-th smallest key by an MSB-first radix select (8 bits a pass);
  // the keys are unique, so exactly nout keys are <= it
  unsigned long long prefix = 0, pmask = 0;
  if (nout < C) {
    uint32_t need = nout;
    for (int shift = 56; shift >= 0; shift -= 8) {
      for (uint32_t q = threadIdx.x; q < 256; q += blockDim.x) sh_hist[q] = 0;
      __syncthreads();
      for (uint32_t c = threadIdx.x; c < C; c += blockDim.x) {
        const unsigned long long v = ck[c];
        if ((v & pmask) == prefix) atomicAdd(&sh_hist[(v >> shift) & 255u], 1u);
      }
      __syncthreads();
      if (wid == 0) {
        // warp scan over 256 bins, 8 per lane
        uint32_t loc[8], tot = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
          loc[q] = sh_hist[lane * 8 + q];
          tot += loc[q];
        }
        uint32_t incl = tot;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
          if (lane >= d) incl += y;
        }
        uint32_t before = incl - tot;
        if (before < need && need <= incl) {
#pragma unroll
          for (int q = 0; q < 8; q++) {
            if (before < need && need <= before + loc[q]) {
              wtmp32[0] = (uint32_t)(lane * 8 + q);
              wtmp32[1] = need - before;
            }
            before += loc[q];
          }
        }
      }
      __syncthreads();
      prefix |= (unsigned long long)wtmp32[0] << shift;
      pmask |= 255ull << shift;
      need = wtmp32[1];
      __syncthreads();
    }
  } else {
    prefix = ~0ull;
  }
  // the selected keys, sorted (at most BIN_MAX_OUT of them)
  if (threadIdx.x == 0) sh_n = 0;
  __syncthreads();
  unsigned long long* selk = ck + T;
  uint32_t* selv = (uint32_t*)(selk + BIN_MAX_OUT);
  for (uint32_t c = threadIdx.x; c < C; c += blockDim.x) {
    const unsigned long long v = ck[c];
    if (v <= prefix) {
      const uint32_t q = atomicAdd(&sh_n, 1u);
      if (q < BIN_MAX_OUT) {
        selk[q] = v;
        selv[q] = c;
      }
    }
  }
  __syncthreads();
  const uint32_t ns = next_pow2(nout);
  for (uint32_t q = threadIdx.x; q < ns; q += blockDim.x)
    if (q >= nout) selk[q] = ~0ull;
  __syncthreads();
  bitonic_kv(selk, selv, ns);
  for (uint32_t q = threadIdx.x; q < nout; q += blockDim.x) sh_sel[q] = selv[q];
  __syncthreads();
  const uint64_t rg = (uint64_t)p.r0 + r;
  const long long L = (long long)(p.offs[rg + 1] - p.offs[rg]);
  for (uint32_t i = threadIdx.x; i < nout; i += blockDim.x) {
    const uint32_t c = sh_sel[i];
    const uint32_t cnt = S.cnt[c];
    const long long sum = (long long)S.sum[c] - (long long)cnt * (long long)DIAG_BIAS;
    const long long avg = sum / (long long)cnt;  // truncation toward zero, as Rust's i64 '/'
    const uint32_t gk = S.gk[c];
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
    // the candidate ranker's seed features of each kept candidate: exact and
    // one-mismatch hits, distinct diagonals, diagonal spread, read span of
    // the hits, read length, mean base quality, rank and list size, mean
    // log2 exact-bucket size (7 and 8, the mate features, come later)
    uint32_t qs = 0;
    const uint64_t q0 = p.offs[rg];
    for (uint32_t k = threadIdx.x; k < (uint32_t)L; k += blockDim.x) qs += p.quals[q0 + k];
    for (int d = 16; d; d >>= 1) qs += __shfl_xor_sync(0xffffffffu, qs, d);
    if (lane == 0) wtmp32[wid] = qs;
    __syncthreads();
    uint32_t qt = 0;
    for (int w2 = 0; w2 < nw; w2++) qt += wtmp32[w2];
    const float meanq = L ? (float)qt / (float)L : 0.f;
    for (uint32_t i = threadIdx.x; i < (uint32_t)MAX_CAND; i += blockDim.x) {
      float* f = p.feat + ((size_t)r * MAX_CAND + i) * RANK_FEATURES;
      if (i >= nout) {
        for (int k = 0; k < RANK_FEATURES; k++) f[k] = 0.f;
        continue;
      }
      const uint32_t c = sh_sel[i];
      const uint32_t nh = S.cnt[c], ne = S.ne[c];
      f[0] = log2f(1.f + (float)ne);
      f[1] = log2f(1.f + (float)(nh - ne));
      f[2] = log2f(1.f + (float)S.nd[c]);
      f[3] = log2f(1.f + (float)S.spread[c]);
      f[4] = log2f(1.f + (nh ? (float)(S.rmx[c] - S.rmn[c] + KMER) : 0.f));
      f[5] = (float)L;
      f[6] = meanq;
      f[7] = 10.f;
      f[8] = 0.f;
      f[9] = (float)i;
      f[10] = (float)nout;
      f[11] = nh ? (float)S.l2s[c] / (float)nh : 0.f;
    }
  }
  if (threadIdx.x == 0) {
    p.n_cand[r] = nout;
    if (p.total_cand) p.total_cand[r] = C;
  }
  __syncthreads();
}

// Reads of h_lo < H <= h_hi hits (h_hi <= TM) from the per-read buffer. The
// tables sit in shared memory, or with GT in the block's slab after the
// cluster records; FEAT adds the candidate ranker's features.
template <bool GT, bool FEAT>
__global__ void k_cluster_bins(ClusterArgs p, uint32_t hmax, size_t slab_bytes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long wtmp64[32];
  __shared__ uint32_t wtmp32[32];
  __shared__ uint32_t sh_n;
  __shared__ uint32_t sh_sel[BIN_MAX_OUT];
  __shared__ uint32_t sh_hist[256];
  unsigned char* slab = p.scratch + (size_t)blockIdx.x * slab_bytes;
  ClusterRecs S;
  S.carve(slab, hmax);
  unsigned char* tab = GT ? slab + cluster_recs_bytes(hmax) : smem_raw;
  for (uint32_t r = blockIdx.x; r < p.nr; r += gridDim.x) {
    const uint32_t H = p.hit_cnt[r];
    if (p.overflow[r]) continue;
    if (!(H > p.h_lo && H <= p.h_hi)) continue;
    if (H == 0) {
      if (threadIdx.x == 0) {
        p.n_cand[r] = 0;
        if (p.total_cand) p.total_cand[r] = 0;
      }
      if (FEAT)
        for (uint32_t i = threadIdx.x; i < (uint32_t)MAX_CAND * RANK_FEATURES; i += blockDim.x)
          p.feat[(size_t)r * MAX_CAND * RANK_FEATURES + i] = 0.f;
      continue;
    }
    cluster_read_bins<FEAT>(p, r, H, p.hits + (size_t)r * p.hcap, tab, S, wtmp32, wtmp64, sh_n, sh_sel, sh_hist);
  }
}

size_t cluster_bins_slab_bytes(uint32_t hmax, bool table_in_slab) {
  return cluster_recs_bytes(hmax) + (table_in_slab ? bin_table_bytes(hmax, true) : 0);
}

size_t cluster_bins_smem_bytes(uint32_t hmax, bool feat) { return bin_table_bytes(hmax, feat); }

// Whether a tier's tables go to the global slab: more than one block's
// shared memory.
bool cluster_bins_in_slab(uint32_t hmax, bool feat) { return bin_table_bytes(hmax, feat) > 220 * 1024; }

template <bool GT, bool FEAT>
static int bins_blocks_per_sm(uint32_t hmax, int threads) {
  const size_t sm = GT ? 0 : bin_table_bytes(hmax, FEAT);
  if (!GT) cudaFuncSetAttribute(k_cluster_bins<GT, FEAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cluster_bins<GT, FEAT>, threads, sm) != cudaSuccess) n = 1;
  return std::max(n, 1);
}

// Resident blocks of the binned K2 on num_sms SMs (the kernel loops over
// reads, so its grid is what fits at once); the table-in-slab tier runs one
// block per SM.
int cluster_bins_grid(uint32_t hmax, int threads, bool feat, int num_sms) {
  if (cluster_bins_in_slab(hmax, feat)) return num_sms;
  return num_sms * (feat ? bins_blocks_per_sm<false, true>(hmax, threads)
                         : bins_blocks_per_sm<false, false>(hmax, threads));
}

template <bool GT, bool FEAT>
static void launch_bins(const ClusterArgs& a, uint32_t hmax, int threads, int grid, size_t slab, cudaStream_t st) {
  const size_t sm = GT ? 0 : bin_table_bytes(hmax, FEAT);
  if (!GT) cudaFuncSetAttribute(k_cluster_bins<GT, FEAT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_cluster_bins<GT, FEAT><<<grid, threads, sm, st>>>(a, hmax, slab);
}

void launch_cluster_bins(const ClusterArgs& a, uint32_t hmax, int threads, int grid, cudaStream_t st) {
  const bool feat = a.feat != nullptr;
  const bool gt = cluster_bins_in_slab(hmax, feat);
  const size_t slab = cluster_bins_slab_bytes(hmax, gt);
  if (gt) {
    if (feat) launch_bins<true, true>(a, hmax, threads, grid, slab, st);
    else launch_bins<true, false>(a, hmax, threads, grid, slab, st);
  } else {
    if (feat) launch_bins<false, true>(a, hmax, threads, grid, slab, st);
    else launch_bins<false, false>(a, hmax, threads, grid, slab, st);
  }
}

void launch_cluster_list(const ClusterArgs& a, int grid, cudaStream_t st) {
  k_cluster_list<<<grid, 256, 0, st>>>(a);
}

}  // namespace pbw
