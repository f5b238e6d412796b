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

__device__ __forceinline__ uint8_t up_ascii_s(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }
__device__ __forceinline__ uint8_t comp_ascii_s(uint8_t b) {
  switch (b) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'C': return 'G';
    case 'G': return 'C';
    default: return 'N';
  }
}

__global__ void __launch_bounds__(128) k_aln_stats(AlignArgs p) {
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
  const uint64_t gb = p.ref_bytes ? 0 : __ldg(&p.G.cbase[J.contig]) + rpos;
  auto rsym = [&](int ri) -> uint8_t {
    if (p.ref_bytes) return p.ref_bytes[rpos + ri];
    return (uint8_t)"ACGTN"[gcode(p.G, gb + ri)];
  };
  auto qsym = [&](int qi) -> uint8_t {
    if (p.ref_bytes) return bases[qo + qi];
    if (!J.rev) return up_ascii_s(bases[qo + qi]);
    return comp_ascii_s(up_ascii_s(bases[qo + m - 1 - qi]));
  };
  auto qqual = [&](int qi) -> uint8_t { return (p.ref_bytes || !J.rev) ? quals[qo + qi] : quals[qo + m - 1 - qi]; };
  const DevTables* T = p.tab;
  double lk = 0.0;
  int qi = 0, ri = 0, cur = 0;
  int n_hq = 0, m_hq = 0, readlen = 0, indel_runs = 0, del_runs = 0, nm = 0, gc = 0, tot = 0;
  for (uint32_t k = 0; k < nops; k++) {
    const uint32_t w = cig[k];
    const int op = (int)(w & 15u);
    const int len = (int)(w >> 4);
    indel_runs += cur != op ? 1 : 0;
    del_runs += (op == 2 && cur != 2) ? 1 : 0;
    cur = op;
    if (op == 1) {
      for (int u = 0; u < len; u++) {
        if (qi < m) lk += T->ln_quarter;
        qi++;
      }
      readlen += len;
      nm += len;
      continue;
    }
    for (int u = 0; u < len; u++) {
      const uint8_t r = ri < span ? rsym(ri) : (uint8_t)0;
      gc += (r == 'G' || r == 'C') ? 1 : 0;
      tot += (r == 'G' || r == 'C' || r == 'A' || r == 'T') ? 1 : 0;
      if (op == 0) {
        if (qi < m && ri < span) {
          const uint8_t a = qsym(qi);
          const uint8_t q = qqual(qi);
          lk += a == r ? T->llk_match[q] : T->llk_mismatch[q];
          const bool hq = q >= 10;
          n_hq += hq ? 1 : 0;
          m_hq += (a != r && a != 'N' && r != 'N' && hq) ? 1 : 0;
          nm += a != r ? 1 : 0;
          readlen++;
        }
        qi++;
      } else {
        nm++;
      }
      ri++;
    }
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
  k_aln_stats<<<(unsigned)((max_jobs + 127) / 128), 128, 0, st>>>(a);
}

}  // namespace pbw
