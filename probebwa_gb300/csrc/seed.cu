// seed.cu -- K1: 15-mer seeding with one-mismatch neighbours and the
// similarity filter (src/mapper/seeds.rs:91-309), one warp per read.
//
// Per read the warp
//   1. stages the read's base codes in shared memory,
//   2. looks up the exact 15-mer of every window in parallel (one lane per
//      window), giving each window's bucket and its repeat flag
//      (seeds.rs:116-128),
//   3. enumerates the probe items of the read in the reference's order --
//      window by window, the exact probe then the 45 neighbours in
//      position-major A/C/G/T order (probe_1mm_neighbours, seeds.rs:291-309)
//      for neighbour-probed, non-repetitive windows (seeds.rs:132) -- 32
//      items at a time, one lookup per lane,
//   4. flattens the buckets of those 32 items into bucket entries (warp
//      prefix sum), filters 32 entries at a time (passes_similarity_filter,
//      seeds.rs:162-219), and appends the passing hits in emission order with
//      a ballot/popc compaction.
// The emission order matters downstream: it fixes the first-appearance order
// of (contig, strand) groups that cluster_hits' FxHashMap iteration follows.
//
// A hit is stored as one 64-bit word: ((contig << 1 | strand) << 40) |
// (diagonal + DIAG_BIAS), the diagonal of candidates.rs:35-39. That key
// sorts hits by (contig, strand, diagonal), which is what clustering needs.
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

struct SeedWarpSmem {
  // laid out in dynamic shared memory per warp; sizes depend on max L
  uint8_t* codes;      // L forward read codes
  uint32_t* wcode;     // W raw k-mer codes (0xFFFFFFFF: window not ACGT-only)
  uint32_t* woff;      // W exact bucket offsets
  uint32_t* wcnt;      // W exact bucket counts
  uint32_t* iofs;      // W+1 item prefix (exclusive)
};

// neighbour_probed_position (seeds.rs:276-286).
__device__ __forceinline__ bool nb_probed(int rp, int L) {
  if (L <= 34) return true;
  if (L <= 49) return ((rp / 5) % 2) == 0;
  return (rp % 15) < 5;
}

// Count A/C/G/T over [s, s+n) of a code array.
__device__ __forceinline__ void fp_read(const uint8_t* c, int s, int n, int& a, int& cc, int& g, int& t) {
  for (int i = 0; i < n; i++) {
    uint8_t x = c[s + i];
    a += x == 0;
    cc += x == 1;
    g += x == 2;
    t += x == 3;
  }
}

// passes_similarity_filter (seeds.rs:162-219) for one bucket entry.
__device__ bool similarity_ok(const DevGenome& G, const uint8_t* fwd, int L, int rp, bool rev, uint32_t cid,
                              uint64_t ref_pos, bool neighbour) {
  // read side, oriented like the genome (rc(read) for a reverse hit)
  const int k = KMER;
  int ws = rev ? L - rp - k : rp;
  int ra_s = min(ws + k, L), ra_e = min(ra_s + 8, L);
  int rb_e = min(ws, L), rb_s = rb_e >= 4 ? rb_e - 4 : 0;
  // genome side
  uint64_t clen = __ldg(&G.clen[cid]);
  uint64_t reg_s = ref_pos >= 4 ? ref_pos - 4 : 0;
  uint64_t reg_e = min(ref_pos + (uint64_t)k + 8, clen);
  if (reg_s >= reg_e) return true;
  int glen = (int)(reg_e - reg_s);
  int gws = (int)(ref_pos - reg_s);
  int ga_s = min(gws + k, glen), ga_e = min(ga_s + 8, glen);
  int gb_e = min(gws, glen), gb_s = gb_e >= 4 ? gb_e - 4 : 0;
  int after = min(ra_e - ra_s, ga_e - ga_s);
  int before = min(rb_e - rb_s, gb_e - gb_s);
  if (after + before < 12) return true;
  int a = 0, c = 0, g = 0, t = 0;
  if (!rev) {
    fp_read(fwd, ra_s, after, a, c, g, t);
    fp_read(fwd, rb_e - before, before, a, c, g, t);
  } else {
    // rc index i <-> forward index L-1-i, complemented
    for (int i = ra_s; i < ra_s + after; i++) {
      uint8_t x = comp_code(fwd[L - 1 - i]);
      a += x == 0; c += x == 1; g += x == 2; t += x == 3;
    }
    for (int i = rb_e - before; i < rb_e; i++) {
      uint8_t x = comp_code(fwd[L - 1 - i]);
      a += x == 0; c += x == 1; g += x == 2; t += x == 3;
    }
  }
  uint64_t base = __ldg(&G.cbase[cid]) + reg_s;
  for (int i = ga_s; i < ga_s + after; i++) {
    uint8_t x = gcode(G, base + i);
    a -= x == 0; c -= x == 1; g -= x == 2; t -= x == 3;
  }
  for (int i = gb_e - before; i < gb_e; i++) {
    uint8_t x = gcode(G, base + i);
    a -= x == 0; c -= x == 1; g -= x == 2; t -= x == 3;
  }
  int d = abs(a) + abs(c) + abs(g) + abs(t);
  return d <= (neighbour ? 8 : 10);
}

__global__ void __launch_bounds__(256) k_seed(SeedArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int W = p.lmax - KMER + 1 > 0 ? p.lmax - KMER + 1 : 1;
  const size_t per_warp = seed_smem_per_warp(p.lmax);
  unsigned char* my = smem_raw + per_warp * wib;
  uint32_t* wcode = (uint32_t*)my;
  uint32_t* woff = wcode + W;
  uint32_t* wcnt = woff + W;
  uint32_t* iofs = wcnt + W;
  uint8_t* codes = (uint8_t*)(iofs + W + 1);

  unsigned long long n_probe = 0, n_entry = 0, n_hit = 0;
  const int gw = blockIdx.x * wpb + wib;
  const int nwarps = gridDim.x * wpb;
  const bool list_mode = p.list != nullptr;
  const uint32_t nitems = list_mode ? *p.list_n : p.nr;
  const unsigned long long s_lo = list_mode ? (unsigned long long)p.slice * p.pool_slice : 0ull;
  if (list_mode && s_lo >= *p.list_total) return;
  for (uint32_t item = gw; item < nitems; item += nwarps) {
    if (list_mode && p.list_hoff[item] / p.pool_slice != p.slice) continue;
    const uint32_t r = list_mode ? p.list[item] : item;
    const uint64_t rg = (uint64_t)p.r0 + r;
    const uint64_t o0 = p.offs[rg];
    const int L = (int)(p.offs[rg + 1] - o0);
    uint8_t* rep = p.rep + (size_t)r * p.wcap;
    unsigned long long* hits = list_mode ? p.hits_pool + (p.list_hoff[item] - s_lo) : p.hits + (size_t)r * p.hcap;
    const uint32_t hcap = list_mode ? p.need[r] : p.hcap;
    if (L < KMER) {
      if (lane == 0 && !list_mode) { p.hit_cnt[r] = 0; p.overflow[r] = 0; }
      continue;
    }
    const int nw = L - KMER + 1;
    for (int i = lane; i < L; i += 32) codes[i] = base_code(p.bases[o0 + i]);
    __syncwarp();
    // exact lookups, one lane per window
    for (int w = lane; w < nw; w += 32) {
      uint32_t code = 0;
      bool ok = true;
#pragma unroll
      for (int t = 0; t < KMER; t++) {
        uint8_t c = codes[w + t];
        ok &= c < 4;
        code = (code << 2) | (c & 3);
      }
      uint32_t off = 0, cnt = 0, items = 0;
      uint8_t rp = 0;
      if (ok) {
        off = __ldg(&p.idx.csr[code]);
        cnt = __ldg(&p.idx.csr[code + 1]) - off;
        bool repv = cnt >= REPEAT_SKIP;
        rp = repv ? 2 : 0;
        items = 1 + ((nb_probed(w, L) && !repv) ? 45 : 0);
      }
      wcode[w] = ok ? code : 0xFFFFFFFFu;
      woff[w] = off;
      wcnt[w] = cnt;
      iofs[w] = items;
      rep[w] = rp;
    }
    __syncwarp();
    // exclusive prefix of items over windows
    uint32_t carry = 0;
    for (int w0 = 0; w0 < nw; w0 += 32) {
      int w = w0 + lane;
      uint32_t v = w < nw ? iofs[w] : 0;
      uint32_t s = v;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, s, d);
        if (lane >= d) s += y;
      }
      if (w < nw) iofs[w] = carry + s - v;
      carry += __shfl_sync(0xffffffffu, s, 31);
    }
    if (lane == 0) iofs[nw] = carry;
    __syncwarp();
    const uint32_t T = carry;
    n_probe += 0;  // counted per item below
    uint32_t nh = 0;
    bool over = false;
    for (uint32_t t0 = 0; t0 < T; t0 += 32) {
      uint32_t t = t0 + lane;
      uint32_t off = 0, cnt = 0;
      int w = 0;
      bool nb = false;
      if (t < T) {
        // window of item t: last w with iofs[w] <= t
        int lo = 0, hi = nw - 1;
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (iofs[mid] <= t) lo = mid; else hi = mid - 1;
        }
        w = lo;
        uint32_t v = t - iofs[w];
        if (v == 0) {
          off = woff[w];
          cnt = wcnt[w];
        } else {
          uint32_t vv = v - 1;
          int pos = vv / 3, alt = vv % 3;
          uint32_t code = wcode[w];
          int sh = 2 * (KMER - 1 - pos);
          uint32_t orig = (code >> sh) & 3u;
          uint32_t nbv = (uint32_t)alt < orig ? (uint32_t)alt : (uint32_t)alt + 1;
          uint32_t nc = (code & ~(3u << sh)) | (nbv << sh);
          off = __ldg(&p.idx.csr[nc]);
          cnt = __ldg(&p.idx.csr[nc + 1]) - off;
          nb = true;
          if (cnt >= REPEAT_SKIP) rep[w] = 1;  // seeds.rs:137-139 (exact not repetitive here)
        }
        n_probe++;
      }
      // inclusive scan of bucket sizes
      uint32_t cum = cnt;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, cum, d);
        if (lane >= d) cum += y;
      }
      const uint32_t Ec = __shfl_sync(0xffffffffu, cum, 31);
      for (uint32_t e0 = 0; e0 < Ec; e0 += 32) {
        uint32_t e = e0 + lane;
        // source item (lane) of entry e: first lane s with cum[s] > e
        int lo = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1) {
          uint32_t cv = __shfl_sync(0xffffffffu, cum, lo + step - 1);
          if (cv <= e) lo += step;
        }
        int s = min(lo, 31);
        uint32_t s_cum = __shfl_sync(0xffffffffu, cum, s);
        uint32_t s_cnt = __shfl_sync(0xffffffffu, cnt, s);
        uint32_t s_off = __shfl_sync(0xffffffffu, off, s);
        int s_w = __shfl_sync(0xffffffffu, w, s);
        bool s_nb = __shfl_sync(0xffffffffu, nb, s);
        bool pass = false;
        unsigned long long word = 0;
        if (e < Ec) {
          uint32_t ei = s_off + (e - (s_cum - s_cnt));
          unsigned long long pk = __ldg(&p.idx.ent[ei]);
          bool rev = (pk >> 63) & 1ull;
          uint32_t cid = (uint32_t)((pk >> 40) & ((1ull << 23) - 1));
          uint64_t rpos = pk & ((1ull << 40) - 1);
          if (cid < p.G.ncontig) {
            pass = similarity_ok(p.G, codes, L, s_w, rev, cid, rpos, s_nb);
          } else {
            pass = false;  // cannot happen with a validated index
          }
          long long diag = rev ? (long long)rpos + s_w : (long long)rpos - s_w;
          word = ((unsigned long long)((cid << 1) | (rev ? 1u : 0u)) << 40) |
                 (unsigned long long)(diag + (long long)DIAG_BIAS);
          n_entry++;
        }
        unsigned int bal = __ballot_sync(0xffffffffu, pass);
        unsigned int rank = __popc(bal & ((1u << lane) - 1u));
        if (pass) {
          uint32_t slot = nh + rank;
          if (slot < hcap) {
            hits[slot] = word;
            if (p.hit_rpos && !list_mode) p.hit_rpos[(size_t)r * p.hcap + slot] = (uint16_t)s_w;
            if (p.hit_rpos_pool && list_mode) p.hit_rpos_pool[p.list_hoff[item] - s_lo + slot] = (uint16_t)s_w;
            if (p.hit_info && !list_mode) {
              const uint32_t wc = wcnt[s_w];
              const uint32_t l2 = min(32u - (uint32_t)__clz(wc), 31u);
              p.hit_info[(size_t)r * p.hcap + slot] =
                  (uint16_t)(((uint32_t)s_w & 0x3FFu) | (l2 << 10) | (s_nb ? 0x8000u : 0u));
            }
          }
          n_hit++;
        }
        nh += __popc(bal);
      }
    }
    if (nh > hcap) over = true;
    __syncwarp();
    if (lane == 0 && !list_mode) {
      p.hit_cnt[r] = over ? p.hcap : nh;
      p.overflow[r] = over ? 1 : 0;
      if (over) {
        if (p.ovf_list) {
          p.need[r] = nh;
          p.ovf_list[atomicAdd(p.n_ovf, 1u)] = r;
        } else {
          atomicAdd(p.n_overflow, 1u);
        }
      }
    }
    __syncwarp();
  }
  // counters (the list-mode pass repeats work already counted)
  if (list_mode) return;
  for (int d = 16; d >= 1; d >>= 1) {
    n_probe += __shfl_down_sync(0xffffffffu, n_probe, d);
    n_entry += __shfl_down_sync(0xffffffffu, n_entry, d);
    n_hit += __shfl_down_sync(0xffffffffu, n_hit, d);
  }
  if (lane == 0 && p.counters) {
    atomicAdd(&p.counters[0], n_probe);
    atomicAdd(&p.counters[1], n_entry);
    atomicAdd(&p.counters[2], n_hit);
  }
}

// Exclusive offsets of the overflowed reads' exact hit counts (one block,
// a scan of 1024 at a time), their total, and the checks of the slice
// limits.
__global__ void k_ovf_offsets(const uint32_t* list, const unsigned int* list_n, const uint32_t* need,
                              unsigned long long* hoff, unsigned long long* total, unsigned long long pool_slice,
                              uint32_t max_slices, int* err, unsigned int* list_n_out) {
  __shared__ unsigned long long wsum[32];
  __shared__ unsigned long long carry;
  __shared__ int bad;
  const unsigned int n = *list_n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (threadIdx.x == 0) {
    carry = 0;
    bad = 0;
  }
  __syncthreads();
  for (unsigned int base = 0; base < n; base += blockDim.x) {
    const unsigned int i = base + threadIdx.x;
    const unsigned long long v = i < n ? need[list[i]] : 0ull;
    if (v > pool_slice) bad = 1;
    unsigned long long s = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, s, d);
      if (lane >= d) s += y;
    }
    if (lane == 31) wsum[wid] = s;
    __syncthreads();
    if (wid == 0) {
      unsigned long long t = lane < nw ? wsum[lane] : 0ull;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, t, d);
        if (lane >= d) t += y;
      }
      if (lane < nw) wsum[lane] = t;
    }
    __syncthreads();
    const unsigned long long before = carry + (wid ? wsum[wid - 1] : 0ull) + s - v;
    if (i < n) hoff[i] = before;
    __syncthreads();
    if (threadIdx.x == 0) carry += wsum[nw - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const unsigned long long tot = carry;
    // items start in slices [0, max_slices) and reach at most one slice past their start
    const bool over = bad || (tot > 0 && (tot - 1) / pool_slice >= max_slices);
    if (over) atomicExch(err, 5);
    *total = over ? 0ull : tot;
    *list_n_out = over ? 0u : n;
  }
}

void launch_ovf_offsets(const uint32_t* list, const unsigned int* list_n, const uint32_t* need,
                        unsigned long long* hoff, unsigned long long* total, unsigned long long pool_slice,
                        uint32_t max_slices, int* err, unsigned int* list_n_out, cudaStream_t st) {
  k_ovf_offsets<<<1, 1024, 0, st>>>(list, list_n, need, hoff, total, pool_slice, max_slices, err, list_n_out);
}

void launch_seed_list(const SeedArgs& a, int grid, cudaStream_t st) {
  const int threads = 256;
  size_t sm = seed_smem_per_warp(a.lmax) * (threads / 32);
  cudaFuncSetAttribute(k_seed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_seed<<<grid, threads, sm, st>>>(a);
}

void launch_seed(const SeedArgs& a, int grid, cudaStream_t st) {
  const int threads = 256;
  size_t sm = seed_smem_per_warp(a.lmax) * (threads / 32);
  cudaFuncSetAttribute(k_seed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_seed<<<grid, threads, sm, st>>>(a);
}

}  // namespace pbw
