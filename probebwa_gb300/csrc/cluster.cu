// cluster.cu -- K2: candidate clustering (src/mapper/candidates.rs:30-78),
// one thread block per read.
//
// The reference groups hits by (contig, strand) in an FxHashMap, visits the
// groups in that map's iteration order, sorts each group's diagonals, splits
// at gaps > 50, emits one candidate per cluster (truncating mean diagonal),
// then stable-sorts candidates by hit count, descending.
//
// Every read takes the binned form (cluster_read_bins, below the shared
// helpers): no sort of the hits, a hash table of 51-wide diagonal bins. Reads
// within the per-read hit buffer run by hit-count tier with their tables in
// shared memory or, for the largest tier, a per-block global slab; reads
// seeded into the overflow pool (list mode) keep their tables in global
// scratch beside their pooled hits.
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

// swiss_find by one warp: the lanes test the W buckets of a probe group (or
// the nb buckets of a small table from pos on) at once, and the lowest empty
// one in probe order wins.
__device__ __forceinline__ uint32_t swiss_find_warp(const uint32_t* t, uint32_t nb, unsigned long long h, int W,
                                                    int lane) {
  const uint32_t mask = nb - 1;
  uint32_t pos = (uint32_t)(h & mask);
  if (nb <= (uint32_t)W) {
    const bool e = (uint32_t)lane < nb && t[(pos + lane) & mask] == 0xFFFFFFFFu;
    const unsigned b = __ballot_sync(0xffffffffu, e);
    return b ? (pos + (uint32_t)__ffs((int)b) - 1) & mask : 0u;
  }
  uint32_t stride = 0;
  for (uint32_t guard = 0; guard <= nb; guard++) {
    const bool e = lane < W && t[(pos + lane) & mask] == 0xFFFFFFFFu;
    const unsigned b = __ballot_sync(0xffffffffu, e);
    if (b) return (pos + (uint32_t)__ffs((int)b) - 1) & mask;
    stride += W;
    pos = (pos + stride) & mask;
  }
  return 0xFFFFFFFFu;
}

constexpr uint32_t SWISS_WARP_SLOTS = 512;  // buckets of the shared-memory replay (groups <= 256)

// swiss_find over a table of nb <= 64 buckets (nb a power of two) held as
// a free-bucket mask in two 32-bit halves, replicated with period nb (bit i
// is bucket i mod nb), so that every probe window, wrapping or not, is the
// low bits of one 64-bit rotation: the first free bucket of the circular
// scan from h (nb <= W; wl = nb) or of the first probe group of W buckets
// with one (triangular probing; wl = W).
__device__ __forceinline__ uint32_t swiss_find_free(uint32_t lo, uint32_t hi, uint32_t nb, uint32_t h, uint32_t wl) {
  const uint32_t mask = nb - 1, gm = (1u << wl) - 1u;
  uint32_t pos = h & mask, stride = 0;
  for (uint32_t guard = 0; guard <= nb; guard++) {
    const bool low = pos < 32;
    const uint32_t win = __funnelshift_r(low ? lo : hi, low ? hi : lo, pos) & gm;
    if (win) return (pos + (uint32_t)__ffs((int)win) - 1) & mask;
    stride += wl;
    pos = (pos + stride) & mask;
  }
  return 0xFFFFFFFFu;
}

constexpr uint32_t SWISS_MASK_GROUPS = 56;  // the largest table of 56 items has 64 buckets

// swiss_replay of at most 56 groups by one warp in registers (all 32 lanes
// call it): the table's free buckets as a replicated mask every lane holds
// (swiss_find_free), bucket s's insertion index and hash in lane s / 2, and
// insertion t's hash in lane t % 32, moved between lanes by shuffles; the
// same insertions and rehashes (old buckets in bucket order) as
// swiss_replay. The next item's shuffles are issued before the current
// item's probe, so only the free mask is carried from item to item. The
// ranks come out in parallel: a bucket's rank is the number of occupied
// buckets before it.
__device__ bool swiss_replay_regs(uint32_t G, const uint32_t* ord, const uint32_t* ggk, uint32_t* rank,
                                  uint32_t* gk_by_rank, int W, int lane) {
  constexpr uint32_t EMPTY = 0xFFFFFFFFu;
  constexpr unsigned FULL = 0xffffffffu;
  uint32_t h0 = 0, h1 = 0;  // hashes of insertions lane and lane + 32
  if ((uint32_t)lane < G) {
    const uint32_t gk = ggk[ord[lane]];
    h0 = (uint32_t)fx_hash_group(gk >> 1, gk & 1u);
  }
  if ((uint32_t)lane + 32 < G) {
    const uint32_t gk = ggk[ord[lane + 32]];
    h1 = (uint32_t)fx_hash_group(gk >> 1, gk & 1u);
  }
  uint32_t b0 = EMPTY, b1 = EMPTY, hb0 = 0, hb1 = 0;  // buckets 2 lane and 2 lane + 1: item, hash
  uint32_t lo = 0, hi = 0;                            // free mask (no table yet)
  uint32_t nb = 0, wl = 0, unit = 0, cap = 0;         // unit: bits at multiples of nb in a half
  auto put = [&](uint32_t q, uint32_t t, uint32_t h) {
    const bool mine = (uint32_t)lane == (q >> 1), odd = (q & 1) != 0;
    b0 = mine && !odd ? t : b0;
    hb0 = mine && !odd ? h : hb0;
    b1 = mine && odd ? t : b1;
    hb1 = mine && odd ? h : hb1;
  };
  auto take = [&](uint32_t q) {  // mark bucket q (every copy of it) occupied
    const uint32_t c = nb == 64 ? 1u << (q & 31) : unit << q;
    lo &= (nb < 64 || q < 32) ? ~c : ~0u;
    hi &= (nb < 64 || q >= 32) ? ~c : ~0u;
  };
  uint32_t hn = __shfl_sync(FULL, h0, 0);
  for (uint32_t t = 0; t < G; t++) {
    const uint32_t ht = hn;
    const uint32_t tn = min(t + 1, G - 1);
    hn = __shfl_sync(FULL, tn < 32 ? h0 : h1, (int)(tn & 31));
    if (t + 1 > cap) {  // t items are in the table
      const uint32_t nnb = swiss_buckets(max(t + 1, cap + 1));
      if (nnb > 64) return false;
      unsigned long long m =
          nb == 0 ? 0ull : ~(((unsigned long long)hi << 32) | lo) & (nb == 64 ? ~0ull : (1ull << nb) - 1ull);
      const uint32_t o0 = b0, o1 = b1, g0 = hb0, g1 = hb1;
      b0 = b1 = EMPTY;
      nb = nnb;
      cap = swiss_cap(nb);
      wl = min(nb, (uint32_t)W);
      unit = nb >= 32 ? 1u : 0xFFFFFFFFu / ((1u << nb) - 1u);
      lo = hi = 0xFFFFFFFFu;
      uint32_t sb = m ? (uint32_t)__ffsll((long long)m) - 1 : 0;
      uint32_t ot = __shfl_sync(FULL, (sb & 1) ? o1 : o0, (int)(sb >> 1));
      uint32_t oh = __shfl_sync(FULL, (sb & 1) ? g1 : g0, (int)(sb >> 1));
      while (m) {
        const uint32_t ct = ot, chh = oh;
        m &= m - 1;
        sb = m ? (uint32_t)__ffsll((long long)m) - 1 : 0;
        ot = __shfl_sync(FULL, (sb & 1) ? o1 : o0, (int)(sb >> 1));
        oh = __shfl_sync(FULL, (sb & 1) ? g1 : g0, (int)(sb >> 1));
        const uint32_t q = swiss_find_free(lo, hi, nb, chh, wl);
        take(q);
        put(q, ct, chh);
      }
    }
    const uint32_t q = swiss_find_free(lo, hi, nb, ht, wl);
    if (q == EMPTY) return false;
    take(q);
    put(q, t, ht);
  }
  const unsigned long long occ =
      G == 0 ? 0ull : ~(((unsigned long long)hi << 32) | lo) & (nb == 64 ? ~0ull : (1ull << nb) - 1ull);
  for (uint32_t hb = 0; hb < 2; hb++) {
    const uint32_t sb = 2 * (uint32_t)lane + hb;
    if ((occ >> sb) & 1ull) {
      const uint32_t g = ord[hb ? b1 : b0];
      const uint32_t rr = (uint32_t)__popcll(occ & ((1ull << sb) - 1ull));
      rank[g] = rr;
      gk_by_rank[rr] = ggk[g];
    }
  }
  __syncwarp();
  return true;
}

// swiss_replay by one warp over shared memory (all 32 lanes call it): the
// same insertions and rehashes (old buckets in bucket order), with each
// probe group tested by the lanes together. aux holds 1280 words: ord, the
// group slots in insertion order (<= 256, the input), the low 32 bits of
// their hashes (<= 256; tables of <= 512 buckets use no more), the buckets
// (cap2 <= 512, each holding an insertion index) and the rehash copy of the
// old buckets (<= 256). rank[g] receives each group's iteration position and
// gk_by_rank[rank] its key.
__device__ bool swiss_replay_warp(uint32_t G, const uint32_t* ggk, uint32_t* aux, uint32_t cap2, uint32_t* rank,
                                  uint32_t* gk_by_rank, int W, int lane) {
  constexpr uint32_t EMPTY = 0xFFFFFFFFu;
  const uint32_t* ord = aux;
  uint32_t* hs = aux + 256;
  uint32_t* slots = aux + 512;
  uint32_t* olds = aux + 512 + SWISS_WARP_SLOTS;
  if (G <= SWISS_MASK_GROUPS) return swiss_replay_regs(G, ord, ggk, rank, gk_by_rank, W, lane);
  for (uint32_t t = lane; t < G; t += 32) {
    const uint32_t gk = ggk[ord[t]];
    hs[t] = (uint32_t)fx_hash_group(gk >> 1, gk & 1u);
  }
  __syncwarp();
  uint32_t nb = 0, items = 0;
  for (uint32_t t = 0; t < G; t++) {
    if (items + 1 > swiss_cap(nb)) {
      const uint32_t need = max(items + 1, swiss_cap(nb) + 1);
      const uint32_t nnb = swiss_buckets(need);
      if (nnb > cap2) return false;
      for (uint32_t s = lane; s < nb; s += 32) olds[s] = slots[s];
      __syncwarp();
      for (uint32_t s = lane; s < nnb; s += 32) slots[s] = EMPTY;
      __syncwarp();
      for (uint32_t s = 0; s < nb; s++) {
        const uint32_t ot = olds[s];
        if (ot == EMPTY) continue;
        const uint32_t q = swiss_find_warp(slots, nnb, hs[ot], W, lane);
        if (lane == 0) slots[q] = ot;
        __syncwarp();
      }
      nb = nnb;
    }
    const uint32_t q = swiss_find_warp(slots, nb, hs[t], W, lane);
    if (q == EMPTY) return false;
    if (lane == 0) slots[q] = t;
    __syncwarp();
    items++;
  }
  // iteration rank = position among the occupied buckets
  uint32_t rk = 0;
  for (uint32_t s0 = 0; s0 < nb; s0 += 32) {
    const uint32_t s = s0 + lane;
    const bool occ = s < nb && slots[s] != EMPTY;
    const unsigned b = __ballot_sync(0xffffffffu, occ);
    if (occ) {
      const uint32_t g = ord[slots[s]];
      const uint32_t rr = rk + (uint32_t)__popc(b & ((1u << lane) - 1u));
      rank[g] = rr;
      gk_by_rank[rr] = ggk[g];
    }
    rk += (uint32_t)__popc(b);
  }
  __syncwarp();
  return true;
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
// table grow fast); groups at load <= 0.5 of the distinct (contig, strand)
// keys the read can have, min(H, gmax) with gmax = 2 * contigs.
__host__ __device__ inline uint32_t np2(uint32_t x) {
  uint32_t p = 1;
  while (p < x) p <<= 1;
  return p;
}
__host__ __device__ inline uint32_t bin_tsize(uint32_t H) {
  const uint32_t t = ((uint32_t)(((uint64_t)H * 8 + 4) / 5) + 31) & ~31u;
  return t < BIN_TMIN ? BIN_TMIN : t;
}
__host__ __device__ inline uint32_t grp_tsize(uint32_t H, uint32_t gmax) {
  const uint32_t g = H < gmax ? H : gmax;
  return np2(g < 8 ? 16 : 2 * g);
}

// Slot of a key in a table of T slots (any T): two 32-bit multiplicative
// mixes (the low word carries the bin, the high word the group and the
// bin's top bits), the high bits of the product scaled to T.
__device__ __forceinline__ uint32_t hash_slot(unsigned long long key, uint32_t T) {
  uint32_t h = (uint32_t)key * 0x9E3779B1u ^ (uint32_t)(key >> 32) * 0x85EBCA77u;
  h ^= h >> 15;
  h *= 0x2C1B3C6Du;
  return __umulhi(h, T);
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

// Tables of one read of up to hmax hits: bins (64-bit key; 32-bit count,
// offset sum and two diagonal-mask halves; with the ranker also 32-bit exact
// hits, bucket-size sum and read-position range), the clusters' 64-bit
// order keys, and groups (key, first emission then rank, key by rank).
__host__ __device__ inline size_t bin_table_bytes(uint32_t hmax, uint32_t gmax, bool feat) {
  return (size_t)bin_tsize(hmax) * (feat ? 48 : 32) + (size_t)grp_tsize(hmax, gmax) * 12;
}
// Global scratch of the rare paths (per block, or per read in list mode):
// the block-wide group order when a read has more than 256 groups, and the
// exact cluster order when a count or a rank does not fit the 64-bit key.
struct BinScratch {
  unsigned long long *okey, *khi, *klo;
  uint32_t *oval, *slots;
  __device__ void carve(unsigned char* base, uint32_t hmax, uint32_t gmax) {
    const uint32_t TG = grp_tsize(hmax, gmax), NP = np2(bin_tsize(hmax));
    okey = (unsigned long long*)base;
    khi = okey + TG;
    klo = khi + NP;
    oval = (uint32_t*)(klo + NP);
    slots = oval + TG;
  }
};
__host__ __device__ inline size_t bin_scratch_bytes(uint32_t hmax, uint32_t gmax) {
  const size_t TG = grp_tsize(hmax, gmax), NP = np2(bin_tsize(hmax));
  return (TG * 16 + NP * 16 + 255) & ~(size_t)255;
}

// The bin table of one read.
struct BinTab {
  unsigned long long* key;
  uint32_t *cnt, *sum, *mlo, *mhi, *ne, *l2s, *rmn, *rmx;
  uint32_t T;
  __device__ unsigned long long mask(uint32_t s) const { return ((unsigned long long)mhi[s] << 32) | mlo[s]; }
  // Whether occupied slot s starts a cluster: its lower neighbour bin is
  // absent or more than MERGE_DISTANCE below its smallest diagonal.
  __device__ bool starts(uint32_t s, unsigned long long k) const {
    const unsigned long long b = k & M35;
    if (b == 0) return true;
    const uint32_t q = find64(key, k - 1, T);
    if (q == NO_SLOT) return true;
    const unsigned long long lo = b * BIN_W + (unsigned long long)(__ffsll((long long)mask(s)) - 1);
    const unsigned long long hi = (b - 1) * BIN_W + (unsigned long long)(63 - __clzll((long long)mask(q)));
    return lo - hi > (unsigned)(BIN_W - 1);
  }
  // Next slot of the cluster after slot cur (bin cb, mask m), or NO_SLOT.
  __device__ uint32_t next(unsigned long long k, unsigned long long b0, unsigned long long cb,
                           unsigned long long m) const {
    const uint32_t q = find64(key, k - b0 + cb + 1, T);
    if (q == NO_SLOT) return NO_SLOT;
    const unsigned long long hi = cb * BIN_W + (unsigned long long)(63 - __clzll((long long)m));
    if ((cb + 1) * BIN_W + (unsigned long long)(__ffsll((long long)mask(q)) - 1) - hi > (unsigned)(BIN_W - 1))
      return NO_SLOT;
    return q;
  }
  // Hit count of the cluster starting at slot s.
  __device__ uint32_t count(uint32_t s, unsigned long long k) const {
    const unsigned long long b0 = k & M35;
    uint32_t c = 0, cur = s;
    unsigned long long cb = b0;
    while (true) {
      c += cnt[cur];
      const uint32_t q = next(k, b0, cb, mask(cur));
      if (q == NO_SLOT) return c;
      cur = q;
      cb++;
    }
  }
};

// Cluster order key: count descending (16 bits), group rank (13 bits), first
// bin (35 bits); unique per cluster. Counts above 0xFFFF or ranks above
// 0x1FFF take the exact path instead.
constexpr uint32_t KEY_CNT_MAX = 0xFFFFu, KEY_RANK_MAX = 0x1FFFu;
// Bin links: 16-bit slot indices, so tables of up to 32767 slots
// (LINK_NONE ends a cluster).
constexpr uint32_t LINK_MAX_SLOTS = 32767u;
constexpr uint16_t LINK_NONE = 0xFFFFu;
__device__ __forceinline__ unsigned long long cluster_key(uint32_t cnt, uint32_t rank, unsigned long long b0) {
  return ((unsigned long long)(KEY_CNT_MAX - min(cnt, KEY_CNT_MAX)) << 48) |
         ((unsigned long long)min(rank, KEY_RANK_MAX) << 35) | b0;
}

// Keys-only block bitonic sort of 64-bit keys, n a power of two.
__device__ void bitonic_k(unsigned long long* k, uint32_t n) {
  for (uint32_t size = 2; size <= n; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t t = threadIdx.x; t < n / 2; t += blockDim.x) {
        const uint32_t i = 2 * t - (t & (stride - 1)), j = i + stride;
        const unsigned long long a = k[i], b = k[j];
        if ((a > b) == ((i & size) == 0)) {
          k[i] = b;
          k[j] = a;
        }
      }
      __syncthreads();
    }
  }
}
// Block bitonic sort of 128-bit keys (hi, lo), n a power of two.
__device__ void bitonic_k2(unsigned long long* hi, unsigned long long* lo, uint32_t n) {
  for (uint32_t size = 2; size <= n; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t t = threadIdx.x; t < n / 2; t += blockDim.x) {
        const uint32_t i = 2 * t - (t & (stride - 1)), j = i + stride;
        const unsigned long long ah = hi[i], al = lo[i], bh = hi[j], bl = lo[j];
        const bool gt = ah > bh || (ah == bh && al > bl);
        if (gt == ((i & size) == 0)) {
          hi[i] = bh;
          lo[i] = bl;
          hi[j] = ah;
          lo[j] = al;
        }
      }
      __syncthreads();
    }
  }
}

// Group ranks for reads of more than 256 groups: first-emission sort and the
// serial replay, in global scratch.
__device__ void group_ranks_block(const ClusterArgs& p, uint32_t TG, const uint32_t* gkey, uint32_t* gval,
                                  uint32_t* grk, const BinScratch& X, uint32_t& sh_n) {
  if (threadIdx.x == 0) sh_n = 0;
  __syncthreads();
  for (uint32_t g = threadIdx.x; g < TG; g += blockDim.x) {
    if (gkey[g] == GRP_EMPTY) continue;
    const uint32_t k = atomicAdd(&sh_n, 1u);
    X.okey[k] = ((unsigned long long)gval[g] << 32) | g;
  }
  __syncthreads();
  const uint32_t G = sh_n, ng = np2(G);
  for (uint32_t k = threadIdx.x; k < ng; k += blockDim.x) {
    if (k >= G) X.okey[k] = ~0ull;
    X.oval[k] = k;
  }
  __syncthreads();
  bitonic_kv(X.okey, X.oval, ng);
  if (threadIdx.x == 0 && !swiss_replay(X.okey, G, gkey, X.slots, max(16u, 2 * ng), gval, p.group_width))
    atomicExch(p.err, 1);
  __syncthreads();
  for (uint32_t g = threadIdx.x; g < TG; g += blockDim.x)
    if (gkey[g] != GRP_EMPTY && gval[g] < TG) grk[gval[g]] = gkey[g];
  __syncthreads();
}

// Barrier among the threads of warps 1.. of the block (named barrier 1;
// __syncthreads is barrier 0).
__device__ __forceinline__ void sync_upper_warps() {
  asm volatile("bar.sync 1, %0;" ::"r"(blockDim.x - 32) : "memory");
}

// early_groups: the groups are collected in a pass of their own before the
// bins, so that warp 0 ranks them (B) while the other warps bin the hits (A)
// and link the bins (C1); otherwise A collects both and B runs beside C1
// only.
// grp_sh: when not null, a shared-memory home for the group table (gkey,
// gval, grk: 3 * GRP_SH_SLOTS words), used when the read's group table fits
// (tables in global memory: each hit's group probe then stays on the SM).
constexpr uint32_t GRP_SH_SLOTS = 1024;
template <bool FEAT>
__device__ void cluster_read_bins(const ClusterArgs& p, uint32_t r, uint32_t H, const unsigned long long* hits,
                                  unsigned char* tab, const BinScratch& X, uint32_t* wtmp32, uint32_t& sh_n,
                                  uint32_t* sh_aux, bool early_groups, uint32_t* grp_sh) {
  const uint32_t T = bin_tsize(H);            // bin slots (the bins and clusters of the read <= H)
  const uint32_t TG = grp_tsize(H, p.gmax);   // group slots
  const int lane = threadIdx.x & 31;
  BinTab B;
  B.T = T;
  B.key = (unsigned long long*)tab;
  B.cnt = (uint32_t*)(B.key + T);
  B.sum = B.cnt + T;
  B.mlo = B.cnt + 2 * T;
  B.mhi = B.cnt + 3 * T;
  B.ne = B.cnt + 4 * T;   // FEAT
  B.l2s = B.cnt + 5 * T;  // FEAT
  B.rmn = B.cnt + 6 * T;  // FEAT
  B.rmx = B.cnt + 7 * T;  // FEAT
  unsigned long long* ck = (unsigned long long*)(B.cnt + (FEAT ? 8 : 4) * T);  // cluster keys
  uint32_t* gkey = grp_sh && TG <= GRP_SH_SLOTS ? grp_sh : (uint32_t*)(ck + T);
  uint32_t* gval = gkey + TG;  // first emission index, then iteration rank
  uint32_t* grk = gval + TG;   // group key by rank
  for (uint32_t s = threadIdx.x; s < TG; s += blockDim.x) {
    gkey[s] = GRP_EMPTY;
    gval[s] = 0xFFFFFFFFu;
  }
  for (uint32_t s = threadIdx.x; s < T; s += blockDim.x) {
    B.key[s] = BIN_EMPTY;
    B.cnt[s] = 0;
    B.sum[s] = 0;
    B.mlo[s] = 0;
    B.mhi[s] = 0;
    if (FEAT) {
      B.ne[s] = 0;
      B.l2s[s] = 0;
      B.rmn[s] = 0xFFFFFFFFu;
      B.rmx[s] = 0;
    }
  }
  if (T <= LINK_MAX_SLOTS) {
    uint32_t* jw = (uint32_t*)((unsigned char*)ck + 5 * (size_t)T);  // the joined bytes, T/4 words
    for (uint32_t s = threadIdx.x; s < T / 4; s += blockDim.x) jw[s] = 0;
  }
  if (threadIdx.x == 0) {
    sh_n = 0;
    wtmp32[30] = 0;  // exact-path flag
  }
  __syncthreads();
  if (early_groups) {
    // A0. the groups and their first-emission indices
    for (uint32_t i = threadIdx.x; i < H; i += blockDim.x) {
      const uint32_t g = insert32(gkey, (uint32_t)(hits[i] >> 40), TG);
      if (g == NO_SLOT) {
        atomicExch(p.err, 1);
        continue;
      }
      if (gval[g] > i) atomicMin(&gval[g], i);
    }
    __syncthreads();
  }
  // A. bins (and groups unless collected in A0) by warps 1.. with
  // early_groups, else by the whole block (32-bit counters: same-address
  // 32-bit adds from one warp combine in the shared-memory unit, 64-bit ones
  // serialise)
  // (each thread loads its next hit, and its info, before binning the
  // current one, so that the load's latency overlaps the insert's)
  const uint32_t a0 = early_groups ? 32 : 0, astep = blockDim.x - a0;
  const bool abin = threadIdx.x >= a0;
  uint32_t i = threadIdx.x - a0;
  unsigned long long w_next = abin && i < H ? hits[i] : 0ull;
  uint32_t info_next = FEAT && abin && i < H ? p.hit_info[(size_t)r * p.hcap + i] : 0u;
  for (; abin && i < H; i += astep) {
    const unsigned long long w = w_next;
    const uint32_t info = info_next;
    if (i + astep < H) {
      w_next = hits[i + astep];
      if (FEAT) info_next = p.hit_info[(size_t)r * p.hcap + i + astep];
    }
    const unsigned long long d = w & M40;
    // diagonal / 51 in 32 bits while the diagonal fits (every contig under
    // 4 Gbp), in 64 bits otherwise
    unsigned long long b;
    uint32_t off;
    if (d < (1ull << 32)) {
      const uint32_t b32 = (uint32_t)d / (uint32_t)BIN_W;
      b = b32;
      off = (uint32_t)d - b32 * (uint32_t)BIN_W;
    } else {
      b = d / BIN_W;
      off = (uint32_t)(d - b * BIN_W);
    }
    const uint32_t gk = (uint32_t)(w >> 40);
    const uint32_t s = insert64(B.key, ((unsigned long long)gk << 35) | b, T);
    if (!early_groups) {
      const uint32_t g = insert32(gkey, gk, TG);
      if (g == NO_SLOT) {
        atomicExch(p.err, 1);
        continue;
      }
      if (gval[g] > i) atomicMin(&gval[g], i);
    }
    if (s == NO_SLOT) {
      atomicExch(p.err, 1);
      continue;
    }
    atomicAdd(&B.cnt[s], 1u);
    atomicAdd(&B.sum[s], off);
    atomicOr(off < 32 ? &B.mlo[s] : &B.mhi[s], 1u << (off & 31u));
    if (FEAT) {
      // hit info: read position | log2 exact bucket size << 10 | neighbour << 15
      atomicAdd(&B.ne[s], (info >> 15) ? 0u : 1u);
      atomicAdd(&B.l2s[s], (info >> 10) & 31u);
      atomicMin(&B.rmn[s], info & 0x3FFu);
      atomicMax(&B.rmx[s], info & 0x3FFu);
    }
  }
  if (!early_groups) __syncthreads();
  else if (threadIdx.x >= 32) sync_upper_warps();
  // B + C1. Warp 0 computes the group iteration ranks (B) while the other
  // warps link the bins (C1): each occupied bin looks up its upper
  // neighbour once, and when the two join, records the link (a 16-bit slot
  // index in the cluster-key area's upper quarter) and marks the upper bin
  // as joined from below (a byte per slot before it). Tables of more than
  // 32767 slots (list mode only) keep no links: their walks look the
  // neighbours up. The cluster keys written later take at most 5T of the
  // area's 8T bytes (a read has at most H <= T / 1.6 clusters).
  const bool linked = T <= LINK_MAX_SLOTS;
  uint16_t* nxt = (uint16_t*)((unsigned char*)ck + 6 * (size_t)T);
  uint8_t* joined = (unsigned char*)ck + 5 * (size_t)T;
  if (threadIdx.x < 32) {
    // B: the groups in first-emission order (counting rank; first-emission
    // indices are distinct) replayed through std's SwissTable insertion in
    // shared memory; more than 256 groups take the block-wide form in global
    // scratch after this phase
    unsigned long long* pairs = (unsigned long long*)(sh_aux + 512);  // 256 (first emission << 32 | slot)
    uint32_t G = 0;
    for (uint32_t g0 = 0; g0 < TG; g0 += 32) {
      const uint32_t g = g0 + lane;
      const bool occ = g < TG && gkey[g] != GRP_EMPTY;
      const unsigned bal = __ballot_sync(0xffffffffu, occ);
      if (occ) {
        const uint32_t e = G + (uint32_t)__popc(bal & ((1u << lane) - 1u));
        if (e < 256) pairs[e] = ((unsigned long long)gval[g] << 32) | g;
      }
      G += (uint32_t)__popc(bal);
    }
    if (lane == 0) wtmp32[31] = G;
    if (G <= 256) {
      __syncwarp();
      for (uint32_t e = lane; e < G; e += 32) {
        const unsigned long long v = pairs[e];
        uint32_t rk = 0;
        for (uint32_t f = 0; f < G; f++) rk += pairs[f] < v ? 1u : 0u;
        sh_aux[rk] = (uint32_t)v;
      }
      __syncwarp();
      if (!swiss_replay_warp(G, gkey, sh_aux, max(16u, 2 * np2(G)), gval, grk, p.group_width, lane) && lane == 0)
        atomicExch(p.err, 1);
    }
  } else if (linked) {
    for (uint32_t s = threadIdx.x - 32; s < T; s += blockDim.x - 32) {
      const unsigned long long k = B.key[s];
      if (k == BIN_EMPTY) continue;
      const unsigned long long b = k & M35;
      const uint32_t q = B.next(k, b, b, B.mask(s));
      nxt[s] = q == NO_SLOT ? LINK_NONE : (uint16_t)q;
      if (q != NO_SLOT) joined[q] = 1;
    }
  }
  __syncthreads();
  if (wtmp32[31] > 256) {
    group_ranks_block(p, TG, gkey, gval, grk, X, sh_n);
    if (threadIdx.x == 0) sh_n = 0;
    __syncthreads();
  }
  // C2: each cluster counted along its links from its first bin, its order
  // key into ck (T and the block are multiples of 32, so each warp claims
  // its round's key slots with one atomic)
  for (uint32_t s = threadIdx.x; s < T; s += blockDim.x) {
    const unsigned long long k = B.key[s];
    const bool start = k != BIN_EMPTY && (linked ? joined[s] == 0 : B.starts(s, k));
    uint32_t cnt = 0, rank = 0;
    if (start) {
      if (linked) {
        for (uint32_t cur = s; cur != LINK_NONE; cur = nxt[cur]) cnt += B.cnt[cur];
      } else {
        cnt = B.count(s, k);
      }
      rank = gval[find32(gkey, (uint32_t)(k >> 35), TG)];
      if (cnt > KEY_CNT_MAX || rank > KEY_RANK_MAX) wtmp32[30] = 1;
    }
    const unsigned em = __ballot_sync(0xffffffffu, start);
    uint32_t kb = 0;
    if (lane == 0 && em) kb = atomicAdd(&sh_n, (uint32_t)__popc(em));
    kb = __shfl_sync(0xffffffffu, kb, 0);
    if (start) ck[kb + (uint32_t)__popc(em & ((1u << lane) - 1u))] = cluster_key(cnt, rank, k & M35);
  }
  __syncthreads();
  const uint32_t C = sh_n;
  __syncthreads();  // every thread holds C before sh_n is counted again
  const bool exact = wtmp32[30] != 0;
  const uint32_t nout = min(min(C, p.max_out), BIN_MAX_OUT);
  // D. the first nout clusters in order. Fast path: the nout-th smallest key
  // by an MSB-first radix select (8 bits a pass; the keys are unique, so
  // exactly nout keys are <= it), then those keys sorted. Exact path: every
  // cluster's (count, rank, first bin) sorted as 128-bit keys in scratch.
  unsigned long long* selk = (unsigned long long*)(sh_aux + 256);  // BIN_MAX_OUT sorted keys
  if (!exact) {
    uint32_t* sh_hist = sh_aux;
    unsigned long long prefix = 0, pmask = 0;
    if (nout < C) {
      uint32_t need = nout;
      const int wid = threadIdx.x >> 5;
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
    if (threadIdx.x == 0) sh_n = 0;
    __syncthreads();
    for (uint32_t c = threadIdx.x; c < C; c += blockDim.x) {
      const unsigned long long v = ck[c];
      if (v <= prefix) {
        const uint32_t q = atomicAdd(&sh_n, 1u);
        if (q < BIN_MAX_OUT) selk[q] = v;
      }
    }
    __syncthreads();
    const uint32_t ns = np2(nout);
    for (uint32_t q = threadIdx.x; q < ns; q += blockDim.x)
      if (q >= nout) selk[q] = ~0ull;
    __syncthreads();
    bitonic_k(selk, ns);
  } else {
    if (threadIdx.x == 0) sh_n = 0;
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < T; s += blockDim.x) {
      const unsigned long long k = B.key[s];
      if (k == BIN_EMPTY || !B.starts(s, k)) continue;
      const uint32_t cnt = B.count(s, k);
      const uint32_t rank = gval[find32(gkey, (uint32_t)(k >> 35), TG)];
      const uint32_t q = atomicAdd(&sh_n, 1u);
      X.khi[q] = ((unsigned long long)(~cnt) << 32) | rank;
      X.klo[q] = k & M35;
    }
    __syncthreads();
    const uint32_t nc = np2(C);
    for (uint32_t q = C + threadIdx.x; q < nc; q += blockDim.x) {
      X.khi[q] = ~0ull;
      X.klo[q] = ~0ull;
    }
    __syncthreads();
    bitonic_k2(X.khi, X.klo, nc);
  }
  // E. the candidates: each selected cluster walked again from its first
  // bin for its diagonal sum (and the ranker's seed features)
  const uint64_t rg = (uint64_t)p.r0 + r;
  const long long L = (long long)(p.offs[rg + 1] - p.offs[rg]);
  float meanq = 0.f;
  if (FEAT) {
    uint32_t qs = 0;
    const uint64_t q0 = p.offs[rg];
    for (uint32_t k = threadIdx.x; k < (uint32_t)L; k += blockDim.x) qs += p.quals[q0 + k];
    for (int d = 16; d; d >>= 1) qs += __shfl_xor_sync(0xffffffffu, qs, d);
    if (lane == 0) wtmp32[threadIdx.x >> 5] = qs;
    __syncthreads();
    uint32_t qt = 0;
    for (int w2 = 0; w2 < (int)(blockDim.x >> 5); w2++) qt += wtmp32[w2];
    meanq = L ? (float)qt / (float)L : 0.f;
  }
  for (uint32_t i = threadIdx.x; i < (FEAT ? max(nout, (uint32_t)MAX_CAND) : nout); i += blockDim.x) {
    if (FEAT && i >= nout) {
      if (i < (uint32_t)MAX_CAND) {
        float* f = p.feat + ((size_t)r * MAX_CAND + i) * RANK_FEATURES;
        for (int q = 0; q < RANK_FEATURES; q++) f[q] = 0.f;
      }
      continue;
    }
    uint32_t rank;
    unsigned long long b0;
    if (!exact) {
      const unsigned long long v = selk[i];
      rank = (uint32_t)(v >> 35) & KEY_RANK_MAX;
      b0 = v & M35;
    } else {
      rank = (uint32_t)X.khi[i];
      b0 = X.klo[i];
    }
    const uint32_t gk = grk[rank];
    const unsigned long long k = ((unsigned long long)gk << 35) | b0;
    const uint32_t s0 = find64(B.key, k, T);
    uint32_t cur = s0;
    uint32_t cnt = 0, ne = 0, l2s = 0, nd = 0, rmn = 0xFFFFFFFFu, rmx = 0;
    unsigned long long sum = 0, cb = b0, m = 0;
    while (cur != NO_SLOT) {
      const uint32_t c = B.cnt[cur];
      m = B.mask(cur);
      cnt += c;
      sum += cb * BIN_W * c + B.sum[cur];
      if (FEAT) {
        ne += B.ne[cur];
        l2s += B.l2s[cur];
        nd += (uint32_t)__popcll(m);
        rmn = min(rmn, B.rmn[cur]);
        rmx = max(rmx, B.rmx[cur]);
      }
      const uint32_t q = linked ? (nxt[cur] == LINK_NONE ? NO_SLOT : (uint32_t)nxt[cur]) : B.next(k, b0, cb, m);
      if (q == NO_SLOT) break;
      cur = q;
      cb++;
    }
    if (cnt == 0) {  // a selected cluster must exist
      atomicExch(p.err, 1);
      continue;
    }
    const long long sm = (long long)sum - (long long)cnt * (long long)DIAG_BIAS;
    const long long avg = sm / (long long)cnt;  // truncation toward zero, as Rust's i64 '/'
    const long long posi = (gk & 1u) ? avg - L + KMER : avg;
    Cand cd;
    cd.pos = posi > 0 ? (unsigned long long)posi : 0ull;
    cd.contig = gk >> 1;
    cd.strand = (uint8_t)(gk & 1u);
    cd.score = cnt;
    cd.pad[0] = 1;
    p.cand[(size_t)r * p.max_out + i] = cd;
    if (FEAT && i < (uint32_t)MAX_CAND) {
      // the candidate ranker's seed features: exact and one-mismatch hits,
      // distinct diagonals, diagonal spread, read span of the hits, read
      // length, mean base quality, rank and list size, mean log2
      // exact-bucket size (7 and 8, the mate features, come later)
      const unsigned long long lo = b0 * BIN_W + (unsigned long long)(__ffsll((long long)B.mask(s0)) - 1);
      const uint32_t spread = (uint32_t)(cb * BIN_W + (unsigned long long)(63 - __clzll((long long)m)) - lo);
      float* f = p.feat + ((size_t)r * MAX_CAND + i) * RANK_FEATURES;
      f[0] = log2f(1.f + (float)ne);
      f[1] = log2f(1.f + (float)(cnt - ne));
      f[2] = log2f(1.f + (float)nd);
      f[3] = log2f(1.f + (float)spread);
      f[4] = log2f(1.f + (cnt ? (float)(rmx - rmn + KMER) : 0.f));
      f[5] = (float)L;
      f[6] = meanq;
      f[7] = 10.f;
      f[8] = 0.f;
      f[9] = (float)i;
      f[10] = (float)nout;
      f[11] = cnt ? (float)l2s / (float)cnt : 0.f;
    }
  }
  if (threadIdx.x == 0) {
    p.n_cand[r] = nout;
    if (p.total_cand) p.total_cand[r] = C;
  }
  __syncthreads();
}

template <bool GT, bool FEAT>
__global__ void __launch_bounds__(1024, 1) k_cluster_bins(ClusterArgs p, uint32_t hmax, size_t slab_bytes) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t wtmp32[32];
  __shared__ uint32_t sh_n;
  __shared__ __align__(8) uint32_t sh_aux[1280];
  __shared__ uint32_t sh_grp[GT ? 3 * GRP_SH_SLOTS : 1];  // the group table of a slab-tier read
  unsigned char* slab = p.scratch + (size_t)blockIdx.x * slab_bytes;
  BinScratch X;
  X.carve(slab, hmax, p.gmax);
  unsigned char* tab = GT ? slab + bin_scratch_bytes(hmax, p.gmax) : smem_raw;
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
    cluster_read_bins<FEAT>(p, r, H, p.hits + (size_t)r * p.hcap, tab, X, wtmp32, sh_n, sh_aux, !GT,
                            GT ? sh_grp : nullptr);
  }
}

// Over-capacity reads (list mode): the hits of the reads whose pool offset
// falls in slice p.slice, clustered in the binned form with the records and
// tables of each read in global scratch at bytes_per_hit times its pool
// offset (cluster_list_bytes_per_hit covers every read of more than hcap
// hits). With the ranker these reads get feature 0 = -1 (no hit-level
// features), which keeps all their candidates.
__global__ void __launch_bounds__(1024, 1) k_cluster_list(ClusterArgs p, size_t bytes_per_hit) {
  __shared__ uint32_t wtmp32[32];
  __shared__ uint32_t sh_n;
  __shared__ __align__(8) uint32_t sh_aux[1280];
  const unsigned int n = *p.list_n;
  const unsigned long long s_lo = (unsigned long long)p.slice * p.pool_slice;
  if (s_lo >= *p.list_total) return;
  for (uint32_t w = blockIdx.x; w < n; w += gridDim.x) {
    if (p.list_hoff[w] / p.pool_slice != p.slice) continue;
    const uint32_t r = p.list[w];
    const uint32_t H = p.need[r];
    const unsigned long long off = p.list_hoff[w] - s_lo;
    unsigned char* base = p.scratch + off * bytes_per_hit;
    BinScratch X;
    X.carve(base, H, p.gmax);
    cluster_read_bins<false>(p, r, H, p.hits_pool + off, base + bin_scratch_bytes(H, p.gmax), X, wtmp32, sh_n,
                             sh_aux, false, nullptr);
    if (p.feat) {
      const uint32_t nout = p.n_cand[r];
      for (uint32_t i = threadIdx.x; i < (uint32_t)MAX_CAND * RANK_FEATURES; i += blockDim.x)
        p.feat[(size_t)r * MAX_CAND * RANK_FEATURES + i] =
            (i % RANK_FEATURES == 0 && i / RANK_FEATURES < nout) ? -1.f : 0.f;
      __syncthreads();
    }
  }
}

// Dynamic shared memory a binned block may take (227 KB less room for the
// kernel's static arrays).
constexpr size_t BIN_SMEM_MAX = 220 * 1024;

size_t cluster_bins_slab_bytes(uint32_t hmax, uint32_t gmax, bool table_in_slab) {
  return bin_scratch_bytes(hmax, gmax) + (table_in_slab ? bin_table_bytes(hmax, gmax, true) : 0);
}

size_t cluster_bins_smem_bytes(uint32_t hmax, uint32_t gmax, bool feat) { return bin_table_bytes(hmax, gmax, feat); }

// Whether a tier's tables go to the global slab: more than one block's
// shared memory.
bool cluster_bins_in_slab(uint32_t hmax, uint32_t gmax, bool feat) {
  return bin_table_bytes(hmax, gmax, feat) > BIN_SMEM_MAX;
}

// Scratch bytes per pooled hit of list mode: scratch plus tables of a read of
// H > hcap hits, at most 32 T + 16 NP + 28 TG + 255 bytes with T =
// bin_tsize(H) <= 1.6 H + 32, NP = np2(T) <= 3.2 H + 64 and TG =
// grp_tsize(H, gmax) <= 4 min(H, gmax) + 16; rounded up to 16 bytes.
size_t cluster_list_bytes_per_hit(uint32_t hcap, uint32_t gmax) {
  const double hmin = (double)hcap + 1.0;
  const double g = (double)gmax < hmin ? (double)gmax / hmin : 1.0;
  const double per = 102.4 + 112.0 * g + 2751.0 / hmin;
  return ((size_t)per + 1 + 15) & ~(size_t)15;
}

template <bool GT, bool FEAT>
static int bins_blocks_per_sm(uint32_t hmax, uint32_t gmax, int threads) {
  const size_t sm = GT ? 0 : bin_table_bytes(hmax, gmax, FEAT);
  if (!GT) smem_ceiling(k_cluster_bins<GT, FEAT>);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cluster_bins<GT, FEAT>, threads, sm) != cudaSuccess) n = 1;
  return std::max(n, 1);
}

// Resident blocks of the binned K2 on num_sms SMs (the kernel loops over
// reads, so its grid is what fits at once): by shared memory for tables in
// shared memory, by registers and threads for tables in the global slab.
int cluster_bins_grid(uint32_t hmax, uint32_t gmax, int threads, bool feat, int num_sms) {
  if (cluster_bins_in_slab(hmax, gmax, feat))
    return num_sms * (feat ? bins_blocks_per_sm<true, true>(hmax, gmax, threads)
                           : bins_blocks_per_sm<true, false>(hmax, gmax, threads));
  return num_sms * (feat ? bins_blocks_per_sm<false, true>(hmax, gmax, threads)
                         : bins_blocks_per_sm<false, false>(hmax, gmax, threads));
}

template <bool GT, bool FEAT>
static void launch_bins(const ClusterArgs& a, uint32_t hmax, int threads, int grid, size_t slab, cudaStream_t st) {
  const size_t sm = GT ? 0 : bin_table_bytes(hmax, a.gmax, FEAT);
  if (!GT) smem_ceiling(k_cluster_bins<GT, FEAT>);
  k_cluster_bins<GT, FEAT><<<grid, threads, sm, st>>>(a, hmax, slab);
}

void launch_cluster_bins(const ClusterArgs& a, uint32_t hmax, int threads, int grid, cudaStream_t st) {
  const bool feat = a.feat != nullptr;
  const bool gt = cluster_bins_in_slab(hmax, a.gmax, feat);
  const size_t slab = cluster_bins_slab_bytes(hmax, a.gmax, gt);
  if (gt) {
    if (feat) launch_bins<true, true>(a, hmax, threads, grid, slab, st);
    else launch_bins<true, false>(a, hmax, threads, grid, slab, st);
  } else {
    if (feat) launch_bins<false, true>(a, hmax, threads, grid, slab, st);
    else launch_bins<false, false>(a, hmax, threads, grid, slab, st);
  }
}

void launch_cluster_list(const ClusterArgs& a, size_t bytes_per_hit, int grid, cudaStream_t st) {
  k_cluster_list<<<grid, 1024, 0, st>>>(a, bytes_per_hit);
}

}  // namespace pbw
