// mapq.cu -- single-end glue kernels around K3 and K4 (FP64 MAPQ).
//
//   k_make_jobs_single  candidates -> alignment windows of
//                       SingleEndMapper::map_candidates (src/mapper/single.rs:105-133)
//   k_finalize_single   select_best + finalize_mapq per read
//                       (src/mapper/single.rs:164-209, src/mapq/bayesian.rs:193-282)
//   k_cigar_gather      per-read CIGAR of the winner into the packed output
//   scan kernels        exclusive u32 prefix sums (three-pass)
#include "mapq_dev.cuh"
#include "pbw_common.cuh"
#include "pbw_kernels.h"
#include "pbw_host.h"

namespace pbw {

__global__ void k_make_jobs_single(MakeJobsArgs p) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= p.nr) return;
  const uint64_t rg = (uint64_t)p.r0 + r;
  const uint64_t L = p.offs[rg + 1] - p.offs[rg];
  const uint32_t nc = p.n_cand[r];
  for (uint32_t i = 0; i < nc; i++) {
    const Cand c = p.cand[(size_t)r * MAX_CAND + i];
    const uint32_t slot = r * MAX_CAND + i;
    p.out[slot].n_ops = 0;  // marks a skipped candidate
    if (p.prune && !c.pad[0]) continue;  // pruned by the candidate ranker
    const unsigned long long clen = p.G.clen[c.contig];
    // left pad 10, right pad max(max_indel_len, 10) (single.rs:109-118)
    const unsigned long long rs = c.pos >= 10 ? c.pos - 10 : 0;
    unsigned long long re = c.pos + L + p.right_pad;
    if (re > clen) re = clen;
    if (rs >= re) continue;
    AlnJob J;
    J.ref_start = rs;
    J.ref_end = re;
    J.hint = 10;  // the left pad, even when pos < 10 (single.rs:132)
    J.read = (uint32_t)rg;
    J.slot = slot;
    J.contig = c.contig;
    J.band = p.band;
    J.rev = c.strand;
    J.valid = 1;
    J.mate = p.mate;
    J.pad = 0;
    J.pad2 = 0;
    J.gap_open = p.gap_open;
    J.gap_extend = p.gap_extend;
    unsigned int q = atomicAdd(p.n_jobs, 1u);
    p.jobs[q] = J;
  }
}

// One thread per read (serial FP64 per read; see k_read_summary).
__global__ void k_finalize_single(FinalizeArgs p) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= p.nr) return;
  const uint64_t rg = (uint64_t)p.r0 + r;
  const uint64_t qo = p.offs[rg];
  const int L = (int)(p.offs[rg + 1] - qo);
  const uint32_t nc = p.n_cand[r];
  const AlnOut* A = p.aln + (size_t)r * MAX_CAND;
  // select_best over the aligned candidates, in candidate order
  int best = -1;
  double mx = 0.0;
  for (uint32_t i = 0; i < nc; i++) {
    if (A[i].n_ops == 0) continue;
    double v = A[i].log_lk;
    if (best < 0 || v >= mx) { mx = v; best = (int)i; }
  }
  if (best < 0) {  // unmapped_record (single.rs:362-383)
    p.contig[r] = -1;
    p.pos[r] = 0;
    p.mapq[r] = 0;
    p.flag[r] = 0x4;
    p.log_lk[r] = 0.0;
    p.posterior[r] = 0.0;
    p.as_score[r] = 0;
    p.nm[r] = 0;
    p.n_ops[r] = 1;
    p.best[r] = -1;
    return;
  }
  double se = -0.0;
  for (uint32_t i = 0; i < nc; i++) {
    if (A[i].n_ops == 0) continue;
    se += exp(A[i].log_lk - mx);
  }
  const AlnOut& W = A[best];
  const uint8_t* q = p.quals + qo;
  const uint8_t* rep = p.rep + (size_t)r * p.wcap;
  const int nwin = L >= KMER ? L - KMER + 1 : 0;
  const double pmiss = missing_locus_thread(q, L, rep, nwin, p.tab);
  EntropyIn e{W.n_hq, W.m_hq, W.readlen, W.ins_runs, W.del_runs, W.gc, W.total};
  const double ent = log_entropy(e, p.tab, p.gc_lnb, p.gc_lnbm1, p.ln_n);
  uint8_t mq;
  double post;
  finalize_mapq(se, ent, pmiss, p.tab, mq, post);
  const Cand c = p.cand[(size_t)r * MAX_CAND + best];
  p.contig[r] = (int32_t)c.contig;
  p.pos[r] = W.pos + 1;
  p.mapq[r] = mq;
  p.flag[r] = c.strand ? 0x10 : 0;
  p.log_lk[r] = W.log_lk;
  p.posterior[r] = post;
  p.as_score[r] = W.score;
  p.nm[r] = W.nm;
  p.n_ops[r] = W.n_ops;
  p.best[r] = (int32_t)(r * MAX_CAND + best);
}

// MapqCalculator::select_best + finalize_mapq (bayesian.rs:193-201,
// 251-282) for explicit inputs, one thread per read: the last maximum of the
// candidates' log-likelihoods and the sequential sum of exp(lk - max); the
// log_entropy counts (bayesian.rs:306-357) walked over the winner's CIGAR,
// query (the read, reverse-complemented when rev) and reference window; the
// missing-locus probability over the read's qualities and repeat mask.
__global__ void k_mapq_batch(MapqBatchArgs p) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.n) return;
  const uint64_t l0 = p.lk_off[i], l1 = p.lk_off[i + 1];
  double mx = p.lks[l0];
  uint32_t b = 0;
  for (uint64_t k = l0; k < l1; k++)
    if (p.lks[k] >= mx) {
      mx = p.lks[k];
      b = (uint32_t)(k - l0);
    }
  double se = -0.0;
  for (uint64_t k = l0; k < l1; k++) se += exp(p.lks[k] - mx);
  const uint64_t qo = p.offs[i];
  const int m = (int)(p.offs[i + 1] - qo);
  const bool rev = p.rev[i] != 0;
  const uint8_t* rw = p.refs + p.ref_off[i];
  const uint64_t nrw = p.ref_off[i + 1] - p.ref_off[i];
  long long n_hq = 0, m_hq = 0, readlen = 0, indel_runs = 0, del_runs = 0;
  uint64_t refpos = 0;
  int cur = 0;
  for (uint64_t k = p.cig_off[i]; k < p.cig_off[i + 1]; k++) {
    const uint32_t op = p.cigar[k] & 15u, len = p.cigar[k] >> 4;
    if (op == 1) {
      indel_runs += (len > 0 && cur != 1) ? 1 : 0;
      cur = len > 0 ? 1 : cur;
      readlen += len;
    } else if (op == 2) {
      if (len > 0 && cur != 2) {
        del_runs++;
        indel_runs++;
      }
      cur = len > 0 ? 2 : cur;
      refpos += len;
    } else if (op == 0) {
      for (uint32_t t = 0; t < len; t++) {
        if (cur != 0) indel_runs++;
        cur = 0;
        if (readlen >= m || refpos >= nrw) break;
        const uint64_t src = rev ? qo + (uint64_t)(m - 1 - readlen) : qo + (uint64_t)readlen;
        const uint8_t q = p.quals[src];
        const uint8_t a = rev ? comp_ascii(up_ascii(p.bases[src])) : up_ascii(p.bases[src]);
        const uint8_t r = rw[refpos];
        const bool hq = q >= 10;
        n_hq += hq ? 1 : 0;
        m_hq += (a != r && a != 'N' && r != 'N' && hq) ? 1 : 0;
        readlen++;
        refpos++;
      }
    }
  }
  int gc = 0, tot = 0;
  for (uint64_t k = 0; k < nrw; k++) {
    const uint8_t r = rw[k];
    gc += (r == 'G' || r == 'C') ? 1 : 0;
    tot += (r == 'G' || r == 'C' || r == 'A' || r == 'T') ? 1 : 0;
  }
  EntropyIn e{(int)n_hq, (int)m_hq, (int)readlen, (int)(indel_runs - del_runs), (int)del_runs, gc, tot};
  const double ent = log_entropy(e, p.tab, p.gc_lnb, p.gc_lnbm1, p.ln_n);
  const double pmiss = missing_locus_mask(p.quals + qo, m, p.repeat + p.win_off[i],
                                          (int)(p.win_off[i + 1] - p.win_off[i]), p.tab);
  uint8_t mq;
  double post;
  finalize_mapq(se, ent, pmiss, p.tab, mq, post);
  p.mapq[i] = mq;
  p.post[i] = post;
  p.best[i] = b;
  p.sum_exp[i] = se;
}

void launch_mapq_batch(const MapqBatchArgs& a, cudaStream_t st) {
  if (a.n == 0) return;
  k_mapq_batch<<<(unsigned)((a.n + 31) / 32), 32, 0, st>>>(a);
}

__global__ void k_cigar_gather(CigarGatherArgs p) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= p.nr) return;
  const uint32_t dst = p.cig_off[r];
  const int32_t b = p.best[r];
  if (b < 0) {
    const uint64_t rg = (uint64_t)p.r0 + r;
    const uint32_t L = (uint32_t)(p.offs[rg + 1] - p.offs[rg]);
    p.cigar[dst] = (L << 4) | 4u;  // {L}S
    return;
  }
  const AlnOut& A = p.aln[b];
  const uint32_t* src = A.n_ops > CIG_INLINE ? p.cig_pool + A.cig_pool : A.cig;
  for (uint32_t k = 0; k < A.n_ops; k++) p.cigar[dst + k] = src[k];
}

// ---- three-pass exclusive scan of u32 ----
constexpr int SCAN_T = 512;
constexpr int SCAN_PER = 8;  // elements per thread
constexpr int SCAN_TILE = SCAN_T * SCAN_PER;

__global__ void k_scan_reduce(const unsigned int* a, uint64_t n, unsigned int* sums) {
  __shared__ unsigned int w[SCAN_T / 32];
  uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
  unsigned int s = 0;
  for (int k = 0; k < SCAN_PER; k++) {
    uint64_t i = base + (uint64_t)k * SCAN_T + threadIdx.x;
    if (i < n) s += a[i];
  }
  for (int d = 16; d >= 1; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
  if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < SCAN_T / 32 ? w[threadIdx.x] : 0;
    for (int d = 16; d >= 1; d >>= 1) s += __shfl_down_sync(0xffffffffu, s, d);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
  }
}

__global__ void k_scan_sums(unsigned int* sums, uint64_t nb, unsigned int* total, const unsigned int* base_in) {
  // single block: exclusive scan of block sums in place
  __shared__ unsigned int w[SCAN_T / 32];
  __shared__ unsigned int carry;
  if (threadIdx.x == 0) carry = base_in ? *base_in : 0u;
  __syncthreads();
  for (uint64_t b0 = 0; b0 < nb; b0 += SCAN_T) {
    uint64_t i = b0 + threadIdx.x;
    unsigned int v = i < nb ? sums[i] : 0;
    unsigned int x = v;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int d = 1; d < 32; d <<= 1) {
      unsigned int y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) w[wid] = x;
    __syncthreads();
    if (wid == 0) {
      unsigned int z = lane < SCAN_T / 32 ? w[lane] : 0;
      for (int d = 1; d < 32; d <<= 1) {
        unsigned int y = __shfl_up_sync(0xffffffffu, z, d);
        if (lane >= d) z += y;
      }
      if (lane < SCAN_T / 32) w[lane] = z;
    }
    __syncthreads();
    unsigned int excl = carry + (wid > 0 ? w[wid - 1] : 0) + x - v;
    if (i < nb) sums[i] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += w[SCAN_T / 32 - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0 && total) *total = carry;
}

__global__ void k_scan_apply(unsigned int* a, uint64_t n, const unsigned int* sums, unsigned int* out) {
  __shared__ unsigned int w[SCAN_T / 32];
  __shared__ unsigned int carry;
  uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
  if (threadIdx.x == 0) carry = sums[blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k < SCAN_PER; k++) {
    uint64_t i = base + (uint64_t)k * SCAN_T + threadIdx.x;
    unsigned int v = i < n ? a[i] : 0;
    unsigned int x = v;
    for (int d = 1; d < 32; d <<= 1) {
      unsigned int y = __shfl_up_sync(0xffffffffu, x, d);
      if (lane >= d) x += y;
    }
    if (lane == 31) w[wid] = x;
    __syncthreads();
    if (wid == 0) {
      unsigned int z = lane < SCAN_T / 32 ? w[lane] : 0;
      for (int d = 1; d < 32; d <<= 1) {
        unsigned int y = __shfl_up_sync(0xffffffffu, z, d);
        if (lane >= d) z += y;
      }
      if (lane < SCAN_T / 32) w[lane] = z;
    }
    __syncthreads();
    unsigned int excl = carry + (wid > 0 ? w[wid - 1] : 0) + x - v;
    if (i < n) (out ? out : a)[i] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += w[SCAN_T / 32 - 1];
    __syncthreads();
  }
}

uint64_t scan_blocks(uint64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

// Exclusive scan of a[0..n) into out (or in place). block_sums must hold
// scan_blocks(n) entries. total (device) receives the sum plus base_in.
void launch_scan_excl(unsigned int* a, uint64_t n, unsigned int* out, unsigned int* block_sums, unsigned int* total,
                      const unsigned int* base_in, cudaStream_t st) {
  uint64_t nb = scan_blocks(n);
  if (nb == 0) nb = 1;
  k_scan_reduce<<<(unsigned)nb, SCAN_T, 0, st>>>(a, n, block_sums);
  k_scan_sums<<<1, SCAN_T, 0, st>>>(block_sums, nb, total, base_in);
  k_scan_apply<<<(unsigned)nb, SCAN_T, 0, st>>>(a, n, block_sums, out);
}

void launch_make_jobs_single(const MakeJobsArgs& a, cudaStream_t st) {
  if (a.nr == 0) return;
  k_make_jobs_single<<<(a.nr + 127) / 128, 128, 0, st>>>(a);
}
void launch_finalize(const FinalizeArgs& a, int, cudaStream_t st) {
  if (a.nr == 0) return;
  const int threads = 128;
  k_finalize_single<<<(unsigned)(((uint64_t)a.nr + threads - 1) / threads), threads, 0, st>>>(a);
}
void launch_cigar_gather(const CigarGatherArgs& a, cudaStream_t st) {
  if (a.nr == 0) return;
  k_cigar_gather<<<(a.nr + 127) / 128, 128, 0, st>>>(a);
}

}  // namespace pbw
