// align_finish.cuh -- traceback and CIGAR shared by the two DP kernels
// (anti-diagonal band: align_band.cu, column tiles: align_window.cu).
//
// traceback (src/align/smith_waterman.rs:299-344): from (m, endJ, endS),
// j == 0 emits an insertion; M follows tb_m to the parent state and moves
// diagonally; I / D follow tb_i / tb_d (0 = opened from M). Cells never
// written read as 0. collapse_cigar (:365-381) merges equal neighbours, and
// cigar_reference_span (cigar.rs:23-28) is the count of M and D operations.
// The per-alignment likelihood and counts that walk the CIGAR afterwards run
// in their own kernel, one thread per alignment (align_stats.cu).
#pragma once
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

// tbr(i, j) -> traceback nibble (tb_m | tb_i << 2 | tb_d << 3), 0 outside.
// Writes score, pos, span and the CIGAR (inline or in the pool) of O. The
// loops have no data-dependent branches, so the lanes of one warp that trace
// different alignments stay converged.
template <class TbRead>
__device__ void traceback_cigar(int m, int endV, int endJ, int endS, uint8_t* ops, TbRead tbr,
                                unsigned long long ref_start, AlnOut* O, uint32_t* cig_pool,
                                unsigned int* cig_pool_used, uint32_t cig_pool_cap, int* err) {
  // ops in reverse order: 0 = M, 1 = I, 2 = D
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
  uint32_t ci = 0, run = 0;
  lastop = -1;
  for (int k = nops - 1; k >= 0; k--) {
    const int op = ops[k];
    if (op != lastop && lastop >= 0 && cdst) cdst[ci] = (run << 4) | (uint32_t)lastop;
    ci += (op != lastop && lastop >= 0) ? 1u : 0u;
    run = op != lastop ? 1u : run + 1u;
    lastop = op;
  }
  if (lastop >= 0 && cdst) cdst[ci] = (run << 4) | (uint32_t)lastop;
  O->pos = ref_start + (unsigned long long)off;
  O->score = endV;
  O->span = (uint32_t)span;
  O->n_ops = ncig;
  O->cig_pool = pool_base;
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
