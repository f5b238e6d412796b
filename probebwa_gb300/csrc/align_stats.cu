// align_stats.cu -- per-alignment likelihood and counts from the CIGAR, one
// thread per alignment, after the DP kernels (align_band.cu,
// align_window.cu) wrote each alignment's position, span and CIGAR.
//
// The forward walk over the CIGAR yields the alignment log-likelihood
// (bayesian.rs:142-179: llk_match / llk_mismatch by quality for each aligned
// read base, ln(1/4) for each inserted base, summed sequentially in FP64 in
// operation order), the log_entropy counts (bayesian.rs:306-357: high-quality
// bases and mismatches, read length, indel and deletion runs, GC and ACGT
// counts of the reference span) and the edit distance. The sum is a serial
// FP64 chain per alignment; with one alignment per thread every lane of a
// warp feeds the FP64 pipe. Read symbols are those the DP saw: upper case,
// reverse complemented for the reverse strand, raw for explicit problems.
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {


// Symbols are compared as codes: reference A0 C1 G2 T3 N4 from the 2-bit
// words and N mask; read bytes through base_code (upper case, A C G T N, any
// other byte 5, which equals no reference code) and, on the reverse strand,
// complemented (3 - c for A C G T, N otherwise, as comp_ascii). Equal codes
// are exactly equal ASCII symbols of the byte comparisons (bayesian.rs:156).
// Explicit problems (raw bytes on both sides) compare the bytes themselves.
template <bool EXPLICIT>
__global__ void __launch_bounds__(128) k_aln_stats(AlignArgs p) {
  __shared__ double s_llk[2][256];
  __shared__ uint8_t s_code[256];
  // launched for the largest job count of a batch: blocks past the real
  // count leave before staging the tables (the whole block, so no barrier
  // is left waiting)
  if (blockIdx.x * blockDim.x >= *p.n_jobs) return;
  for (int k = threadIdx.x; k < 256; k += blockDim.x) {
    s_llk[0][k] = p.tab->llk_match[k];
    s_llk[1][k] = p.tab->llk_mismatch[k];
    s_code[k] = base_code((uint8_t)k);
  }
  __syncthreads();
  const unsigned int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= *p.n_jobs) return;
  const AlnJob J = p.jobs[t];
  if (!J.valid) return;
  AlnOut* O = p.out + J.slot;
  const uint32_t nops = O->n_ops;
  if (nops == 0) return;
  const uint32_t* cig = O->cig;
  if (nops > CIG_INLINE) {
    if (O->cig_pool == 0xFFFFFFFFu) return;  // pool overflow, reported by the DP kernel
    cig = p.cig_pool + O->cig_pool;
  }
  if ((cig[0] & 15u) == 4u) return;  // empty problem: its counts are already zero
  const uint8_t* bases = J.mate ? p.bases2 : p.bases;
  const uint8_t* quals = J.mate ? p.quals2 : p.quals;
  const uint64_t* offs = J.mate ? p.offs2 : p.offs;
  const uint64_t qo = offs[J.read];
  const int m = (int)(offs[J.read + 1] - qo);
  const uint64_t rpos = O->pos;
  const int span = (int)O->span;
  const bool rev = !EXPLICIT && J.rev;
  // read cursor: walks the read forwards, or backwards on the reverse strand
  const uint8_t* qb = bases + qo + (rev ? m - 1 : 0);
  const uint8_t* qq = quals + qo + (rev ? m - 1 : 0);
  const long long dir = rev ? -1 : 1;
  // gsafe: the contig's first base, read (and ignored) when the operation has no reference base
  const uint64_t gsafe = EXPLICIT ? 0 : __ldg(&p.G.cbase[J.contig]);
  const uint64_t gb = gsafe + rpos;
  const double ln_quarter = p.tab->ln_quarter;
  double lk = 0.0;
  int qi = 0, ri = 0, cur = 0;
  int n_hq = 0, m_hq = 0, readlen = 0, indel_runs = 0, del_runs = 0, nm = 0, gc = 0, tot = 0;
  // One operation per iteration with plain loads (the reads, qualities and
  // genome words a lane walks stay in L1): no per-lane reload branches, so the
  // lanes of a warp step through their different CIGARs together.
  uint32_t k = 0;
  int op = 0, left = 0;
  while (true) {
    if (left == 0) {
      if (k == nops) break;
      const uint32_t w = cig[k++];
      op = (int)(w & 15u);
      left = (int)(w >> 4);
      indel_runs += cur != op ? 1 : 0;
      del_runs += (op == 2 && cur != 2) ? 1 : 0;
      cur = op;
      if (left == 0) continue;
    }
    left--;
    const bool isM = op == 0, isI = op == 1;
    const bool rv = !isI && ri < span;
    const bool qv = qi < m;
    const bool mcond = isM && qv && rv;
    uint32_t rc, ac;  // reference and read symbols (codes, or raw bytes for explicit problems)
    if (EXPLICIT) {
      rc = rv ? p.ref_bytes[rpos + ri] : 0u;
      ac = mcond ? *qb : 0u;
    } else {
      const uint64_t gp = rv ? gb + (uint64_t)ri : gsafe;
      const unsigned long long gw = __ldg(&p.G.bits[gp >> 5]);
      const unsigned int gm = __ldg(&p.G.nmask[gp >> 5]);
      rc = ((gm >> (gp & 31)) & 1u) ? 4u : (uint32_t)((gw >> ((gp & 31) * 2)) & 3ull);
      const uint32_t c0 = mcond ? s_code[*qb] : 4u;
      ac = rev ? (c0 < 4u ? 3u - c0 : 4u) : c0;
    }
    const uint32_t q = mcond ? (uint32_t)*qq : 0u;
    const uint32_t nsym = EXPLICIT ? (uint32_t)'N' : 4u;
    const bool mism = ac != rc;
    // a D operation adds +0.0, which leaves lk unchanged (lk is never -0.0)
    lk += mcond ? s_llk[mism ? 1 : 0][q] : ((isI && qv) ? ln_quarter : 0.0);
    const bool hq = q >= 10u;
    n_hq += (mcond && hq) ? 1 : 0;
    m_hq += (mcond && mism && ac != nsym && rc != nsym && hq) ? 1 : 0;
    nm += ((mcond && mism) || !isM) ? 1 : 0;
    readlen += (mcond || isI) ? 1 : 0;
    if (EXPLICIT) {
      gc += (rv && (rc == 'G' || rc == 'C')) ? 1 : 0;
      tot += (rv && (rc == 'G' || rc == 'C' || rc == 'A' || rc == 'T')) ? 1 : 0;
    } else {
      gc += (rv && (rc == 1u || rc == 2u)) ? 1 : 0;
      tot += (rv && rc < 4u) ? 1 : 0;
    }
    const bool adv_q = op != 2;
    qi += adv_q ? 1 : 0;
    qb += adv_q ? dir : 0;
    qq += adv_q ? dir : 0;
    ri += isI ? 0 : 1;
  }
  O->log_lk = lk;
  O->n_hq = n_hq;
  O->m_hq = m_hq;
  O->readlen = readlen;
  O->ins_runs = indel_runs - del_runs;
  O->del_runs = del_runs;
  O->gc = gc;
  O->total = tot;
  O->nm = nm;
}

void launch_aln_stats(const AlignArgs& a, uint64_t max_jobs, cudaStream_t st) {
  if (max_jobs == 0) return;
  if (a.ref_bytes) k_aln_stats<true><<<(unsigned)((max_jobs + 127) / 128), 128, 0, st>>>(a);
  else k_aln_stats<false><<<(unsigned)((max_jobs + 127) / 128), 128, 0, st>>>(a);
}

}  // namespace pbw
