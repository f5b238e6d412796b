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

// passes_similarity_filter (seeds.rs:162-219) for one bucket entry. The
// flanks are up to 8 bases after and 4 before the 15-mer, clipped to the
// read and to the genome (clip_flanks); a hit whose flanks are not both whole
// has after + before < 12 and passes. Otherwise the filter is the L1 distance
// between the A/C/G/T counts of those 12 read bases (in the hit's
// orientation) and of the 12 genome bases, at most 10 (8 for a neighbour
// hit). Read counts come from the read's prefix counts (pc4: four 16-bit
// fields A C G T per position), genome counts from the 27-base window
// [ref_pos - 4, ref_pos + 23) read as 2-bit words, by mask and popcount, N
// bases (the contig's N runs) counting as none of the four; the N-mask words
// are read only for 1024-base blocks that hold an N.
__device__ __forceinline__ bool similarity_ok(const DevGenome& G, const unsigned long long* pc4, int L, int rp,
                                              bool rev, uint32_t cid, uint64_t ref_pos, bool neighbour) {
  constexpr int k = KMER;
  const uint64_t clen = __ldg(&G.clen[cid]);
  if (ref_pos < 4 || ref_pos + k + 8 > clen) return true;
  unsigned long long rc;  // read counts in genome orientation
  if (!rev) {
    if (rp < 4 || rp + k + 8 > L) return true;
    rc = pc4[rp + k + 8] - pc4[rp + k] + pc4[rp] - pc4[rp - 4];
  } else {
    // the reverse-complemented read's flanks: after = [rp - 8, rp) and
    // before = [rp + 15, rp + 19) of the forward read, complemented
    if (rp < 8 || rp + k + 4 > L) return true;
    const unsigned long long f = pc4[rp] - pc4[rp - 8] + pc4[rp + k + 4] - pc4[rp + k];
    rc = (f << 48) | ((f >> 16 & 0xFFFFull) << 32) | ((f >> 32 & 0xFFFFull) << 16) | (f >> 48);
  }
  const uint64_t gs = __ldg(&G.cbase[cid]) + ref_pos - 4;
  const uint32_t sh = (uint32_t)(gs & 31);
  const uint64_t wi = gs >> 5;
  unsigned long long X = __ldg(&G.bits[wi]);
  // the N-mask words only where the window's 1024-base blocks hold an N
  const uint64_t b0 = wi >> 5, b1 = (wi + 1) >> 5;
  const bool has_n = ((__ldg(&G.nblk[b0 >> 5]) >> (b0 & 31)) & 1u) != 0 ||
                     (sh > 5 && ((__ldg(&G.nblk[b1 >> 5]) >> (b1 & 31)) & 1u) != 0);
  uint32_t NM = has_n ? __ldg(&G.nmask[wi]) : 0u;
  if (sh) {
    X >>= 2 * sh;
    NM >>= sh;
    if (sh > 5) {  // the window reaches into the next word
      X |= __ldg(&G.bits[wi + 1]) << (64 - 2 * sh);
      if (has_n) NM |= __ldg(&G.nmask[wi + 1]) << (32 - sh);
    }
  }
  // bases 0-3 and 19-26 of the window, one bit per base at even positions
  unsigned long long valid = 0x55ull | (0x5555ull << 38);
  if (NM & 0x7FFFFFFu) {
    unsigned long long n = NM;
    n = (n | (n << 16)) & 0x0000FFFF0000FFFFull;
    n = (n | (n << 8)) & 0x00FF00FF00FF00FFull;
    n = (n | (n << 4)) & 0x0F0F0F0F0F0F0F0Full;
    n = (n | (n << 2)) & 0x3333333333333333ull;
    n = (n | (n << 1)) & 0x5555555555555555ull;
    valid &= ~n;
  }
  int d = 0;
#pragma unroll
  for (int c = 0; c < 4; c++) {
    const unsigned long long t = ~(X ^ (0x5555555555555555ull * (unsigned long long)c));
    const int g = __popcll(t & (t >> 1) & valid);
    d += abs((int)((rc >> (16 * c)) & 0xFFFFull) - g);
  }
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
  unsigned long long* pc4 = (unsigned long long*)my;  // lmax + 1 prefix counts
  uint32_t* wcode = (uint32_t*)(pc4 + p.lmax + 1);
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
    // base codes and their prefix counts (A C G T in four 16-bit fields)
    unsigned long long run = 0;
    if (lane == 0) pc4[0] = 0;
    for (int i0 = 0; i0 < L; i0 += 32) {
      const int i = i0 + lane;
      const uint8_t c = i < L ? base_code(p.bases[o0 + i]) : (uint8_t)4;
      if (i < L) codes[i] = c;
      unsigned long long v = c < 4 ? 1ull << (16 * c) : 0ull;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= d) v += y;
      }
      if (i < L) pc4[i + 1] = run + v;
      run += __shfl_sync(0xffffffffu, v, 31);
    }
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
            pass = similarity_ok(p.G, pc4, L, s_w, rev, cid, rpos, s_nb);
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
  smem_ceiling(k_seed);
  k_seed<<<grid, threads, sm, st>>>(a);
}

void launch_seed(const SeedArgs& a, int grid, cudaStream_t st) {
  const int threads = 256;
  size_t sm = seed_smem_per_warp(a.lmax) * (threads / 32);
  smem_ceiling(k_seed);
  k_seed<<<grid, threads, sm, st>>>(a);
}

}  // namespace pbw
