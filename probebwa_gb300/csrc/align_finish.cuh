// align_finish.cuh -- traceback and per-alignment bookkeeping shared by the
// two DP kernels (anti-diagonal band: align_band.cu, column tiles:
// align_window.cu).
//
// traceback (src/align/smith_waterman.rs:299-344): from (m, endJ, endS),
// j == 0 emits an insertion; M follows tb_m to the parent state and moves
// diagonally; I / D follow tb_i / tb_d (0 = opened from M). Cells never
// written read as 0. collapse_cigar (:365-381) merges equal neighbours.
// The forward walk then yields cigar_reference_span (cigar.rs:23-28), the
// alignment log-likelihood (bayesian.rs:142-179, sequential FP64 sum over
// host-built per-quality terms), the log_entropy counts (bayesian.rs:306-357)
// and the edit distance.
#pragma once
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

// tbr(i, j) -> traceback nibble (tb_m | tb_i << 2 | tb_d << 3), 0 outside.
// rsym(j)   -> reference symbol (ASCII) at window index j (0-based).
// qs(i), qq(i) -> query symbol and Phred quality at read index i (0-based).
template <class TbRead, class RefSym, class QSym, class QQual>
__device__ void finish_alignment(int m, int endV, int endJ, int endS, QSym qs, QQual qq,
                                 uint8_t* ops, TbRead tbr, RefSym rsym, unsigned long long ref_start,
                                 const DevTables* T, AlnOut* O, uint32_t* cig_pool, unsigned int* cig_pool_used,
                                 uint32_t cig_pool_cap, int* err) {
  // The loops below are written without data-dependent branches so that the
  // lanes of one warp that finish different alignments stay converged.
  // traceback, ops in reverse order: 0 = M, 1 = I, 2 = D
  int i = m, j = endJ, st = endS, nops = 0;
  while (i > 0) {
    const bool j0 = j == 0;
    const uint32_t nib = j0 ? 0u : tbr(i, j);
    const int op = j0 ? 1 : st;
    const int from_m = (int)(nib & 3u), from_i = (int)((nib >> 2) & 1u), from_d = (int)((nib >> 2) & 2u);
    const int nst = j0 ? st : (st == 0 ? from_m : (st == 1 ? from_i : from_d));
    ops[nops++] = (uint8_t)op;
    i -= op != 2 ? 1 : 0;
    j -= op != 1 ? 1 : 0;
    st = nst;
  }
  const int off = j;
  // runs (collapse_cigar) and cigar_reference_span
  uint32_t ncig = 0;
  int span = 0, lastop = -1;
  for (int k = nops - 1; k >= 0; k--) {
    const int op = ops[k];
    ncig += op != lastop ? 1u : 0u;
    lastop = op;
    span += op != 1 ? 1 : 0;
  }
  uint32_t pool_base = 0xFFFFFFFFu;
  if (ncig > CIG_INLINE) {
    pool_base = atomicAdd(cig_pool_used, ncig);
    if (pool_base + ncig > cig_pool_cap) {
      atomicExch(err, 3);
      pool_base = 0xFFFFFFFFu;
    }
  }
  uint32_t* cdst = ncig > CIG_INLINE ? (pool_base != 0xFFFFFFFFu ? cig_pool + pool_base : nullptr) : O->cig;
  // forward walk: CIGAR runs, likelihood (sequential FP64 sum in op order),
  // log_entropy counts, edit distance, GC of the reference span
  uint32_t ci = 0, run = 0;
  lastop = -1;
  double lk = 0.0;
  int qi = 0, ri = 0;
  int n_hq = 0, m_hq = 0, readlen = 0, indel_runs = 0, del_runs = 0, cur = 0, nm = 0, gc = 0, tot = 0;
  for (int k = nops - 1; k >= 0; k--) {
    const int op = ops[k];
    if (op != lastop && lastop >= 0 && cdst) cdst[ci] = (run << 4) | (uint32_t)lastop;
    ci += (op != lastop && lastop >= 0) ? 1u : 0u;
    run = op != lastop ? 1u : run + 1u;
    lastop = op;
    const bool isM = op == 0, isI = op == 1, isD = op == 2;
    indel_runs += cur != op ? 1 : 0;
    del_runs += (isD && cur != 2) ? 1 : 0;
    cur = op;
    const bool qv = qi < m;
    const uint8_t a = qv ? qs(qi) : (uint8_t)0;
    const uint8_t q = qv ? qq(qi) : (uint8_t)0;
    const uint8_t r = isI ? (uint8_t)0 : rsym(off + ri);
    const bool mcond = isM && qv && ri < span;
    const bool mism = a != r;
    const double tm = mism ? T->llk_mismatch[q] : T->llk_match[q];
    // adding +0.0 leaves lk unchanged: lk starts at +0.0 and every term is
    // negative or +0.0, so lk is never -0.0
    lk += mcond ? tm : ((isI && qv) ? T->ln_quarter : 0.0);
    const bool hq = q >= 10;
    n_hq += (mcond && hq) ? 1 : 0;
    m_hq += (mcond && mism && a != 'N' && r != 'N' && hq) ? 1 : 0;
    nm += ((mcond && mism) || !isM) ? 1 : 0;
    readlen += (mcond || isI) ? 1 : 0;
    const bool g_or_c = !isI && (r == 'G' || r == 'C');
    gc += g_or_c ? 1 : 0;
    tot += (g_or_c || (!isI && (r == 'A' || r == 'T'))) ? 1 : 0;
    qi += isD ? 0 : 1;
    ri += isI ? 0 : 1;
  }
  if (lastop >= 0 && cdst) cdst[ci] = (run << 4) | (uint32_t)lastop;
  O->log_lk = lk;
  O->pos = ref_start + (unsigned long long)off;
  O->score = endV;
  O->span = (uint32_t)span;
  O->n_ops = ncig;
  O->cig_pool = pool_base;
  O->n_hq = n_hq;
  O->m_hq = m_hq;
  O->readlen = readlen;
  O->ins_runs = indel_runs - del_runs;
  O->del_runs = del_runs;
  O->gc = gc;
  O->total = tot;
  O->nm = nm;
}

// Output of an empty problem (smith_waterman.rs:166-168).
__device__ inline void finish_empty(int m, unsigned long long ref_start, AlnOut* O) {
  O->score = 0;
  O->pos = ref_start;
  O->n_ops = 1;
  O->cig[0] = ((uint32_t)m << 4) | 4u;
  O->cig_pool = 0xFFFFFFFFu;
  O->span = 0;
  O->log_lk = 0.0;
  O->n_hq = O->m_hq = O->readlen = O->ins_runs = O->del_runs = O->gc = O->total = O->nm = 0;
}

// Last-maximum endpoint (smith_waterman.rs:248-251) given the best in-band
// (value, j, state) of the final row and that row's band [fjs, fje]: the
// out-of-band positions hold NEG_INF and the last of them is (n, I) if the
// band ends before n, else (fjs-1, I).
__device__ inline void resolve_endpoint(int& V, int& J, int& S, int fjs, int fje, int n) {
  const int oobJ = fje < n ? n : fjs - 1;
  if (J < 0 || V < NEG || (V == NEG && (oobJ > J || (oobJ == J && S == 0)))) {
    V = NEG;
    J = oobJ;
    S = 1;
  }
}

}  // namespace pbw
