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
  int i = m, j = endJ, st = endS, nops = 0;
  while (i > 0) {
    if (j == 0) {
      ops[nops++] = 1;
      i--;
      continue;
    }
    const uint32_t nib = tbr(i, j);
    if (st == 0) {
      ops[nops++] = 0;
      i--;
      j--;
      st = (int)(nib & 3u);
    } else if (st == 1) {
      ops[nops++] = 1;
      i--;
      st = (nib & 4u) ? 1 : 0;
    } else {
      ops[nops++] = 2;
      j--;
      st = (nib & 8u) ? 2 : 0;
    }
  }
  const int off = j;
  uint32_t ncig = 0;
  int lastop = -1;
  for (int k = nops - 1; k >= 0; k--) {
    const int op = ops[k];
    if (op != lastop) {
      ncig++;
      lastop = op;
    }
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
  int span = 0;
  lastop = -1;
  for (int k = nops - 1; k >= 0; k--) {
    const int op = ops[k];
    if (op != lastop) {
      if (lastop >= 0) {
        if (cdst) cdst[ci] = (run << 4) | (uint32_t)lastop;
        ci++;
      }
      lastop = op;
      run = 0;
    }
    run++;
    if (op != 1) span++;
  }
  if (lastop >= 0 && cdst) cdst[ci] = (run << 4) | (uint32_t)lastop;
  double lk = 0.0;
  int qi = 0, ri = 0;
  int n_hq = 0, m_hq = 0, readlen = 0, indel_runs = 0, del_runs = 0, cur = 0, nm = 0;
  for (int k = nops - 1; k >= 0; k--) {
    const int op = ops[k];
    if (op == 0) {
      if (cur != 0) indel_runs++;
      cur = 0;
      if (qi < m && ri < span) {
        const uint8_t a = qs(qi), r = rsym(off + ri);
        const uint8_t q = qq(qi);
        lk += a == r ? T->llk_match[q] : T->llk_mismatch[q];
        const bool hq = q >= 10;
        if (hq) n_hq++;
        if (a != r && a != 'N' && r != 'N' && hq) m_hq++;
        if (a != r) nm++;
        readlen++;
      }
      qi++;
      ri++;
    } else if (op == 1) {
      if (cur != 1) indel_runs++;
      cur = 1;
      readlen++;
      if (qi < m) lk += T->ln_quarter;
      qi++;
      nm++;
    } else {
      if (cur != 2) {
        del_runs++;
        indel_runs++;
      }
      cur = 2;
      ri++;
      nm++;
    }
  }
  int gc = 0, tot = 0;
  for (int r = 0; r < span; r++) {
    const uint8_t b = rsym(off + r);
    if (b == 'G' || b == 'C') {
      gc++;
      tot++;
    } else if (b == 'A' || b == 'T') {
      tot++;
    }
  }
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
