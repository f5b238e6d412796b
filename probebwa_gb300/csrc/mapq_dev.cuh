// mapq_dev.cuh -- FP64 MAPQ arithmetic of src/mapq/bayesian.rs on the device.
//
// Every sum and product runs in the reference's order; the build uses
// -fmad=false so no a*b+c is fused (Rust never fuses either). Quantities with
// integer or quality-indexed inputs come from tables built on the host with
// the oracle's libm (DevTables, gc tables, ln_n); exp/log/log10/pow of
// continuous values use CUDA's double-precision functions.
#pragma once
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

constexpr double LN_10 = 2.302585092994045684017991454684364208;
constexpr double DB = -0.1 * LN_10;  // bayesian.rs:36

// logadd (bayesian.rs:47-58).
__device__ __forceinline__ double logadd(double a, double b) {
  if (a > b) { double t = a; a = b; b = t; }
  if (b >= a + 10.0) return a;
  if (b >= a + 4.0) return fmax(a - 1.0, 0.0);
  if (b >= a + 2.0) return fmax(a - 2.0, 0.0);
  return fmax(a - 3.0, 0.0);
}
// py_int_round (bayesian.rs:63-65).
__device__ __forceinline__ double py_int_round(double x) { return trunc(x + 0.5); }

// phred_n_choose_m (bayesian.rs:72-86) with ln(k) from a host table.
__device__ inline double phred_n_choose_m(long long n, long long m, const double* ln_n, int ln_max) {
  if (m > n / 2) m = n - m;
  if (m <= 0) return 0.0;
  double phred = 0.0;
  while (m > 1) {
    double a = n < ln_max ? ln_n[n] : log((double)n);
    double b = m < ln_max ? ln_n[m] : log((double)m);
    phred += a - b;
    n--;
    m--;
  }
  phred += n < ln_max ? ln_n[n] : log((double)n);
  return py_int_round(10.0 * phred / LN_10);
}

// ln(b) and ln(max(b-1, 1e-6)) of the GC-adjusted alphabet size
// (bayesian.rs:359-364, 445-466) for a window with gc G/C among tot ACGT.
__device__ inline void gc_terms(int gc, int tot, const DevTables* T, const double* lnb_tab, const double* lnbm1_tab,
                                double& lnb, double& lnbm1) {
  if (tot <= T->gc_tmax) {
    size_t idx = (size_t)tot * (tot + 1) / 2 + gc;
    lnb = lnb_tab[idx];
    lnbm1 = lnbm1_tab[idx];
    return;
  }
  double f = tot == 0 ? 0.5 : (double)gc / (double)tot;
  f = fmin(fmax(f, 1e-6), 1.0 - 1e-6);
  double b = exp(-f * log(f / 2.0) - (1.0 - f) * log((1.0 - f) / 2.0));
  lnb = log(b);
  lnbm1 = log(fmax(b - 1.0, 1e-6));
}

struct EntropyIn {
  int n_hq, m_hq, readlen, ins_runs, del_runs, gc, total;
};

// log_entropy (bayesian.rs:306-373) from the walk's counts.
__device__ inline double log_entropy(const EntropyIn& e, const DevTables* T, const double* lnb_tab,
                                     const double* lnbm1_tab, const double* ln_n) {
  double lnb, lnbm1;
  gc_terms(e.gc, e.total, T, lnb_tab, lnbm1_tab, lnb, lnbm1);
  double match_term = py_int_round(10.0 * ((double)e.n_hq * lnb - T->ln_two_g) / LN_10);
  double mismatch_term = py_int_round(10.0 * (double)e.m_hq * lnbm1 / LN_10);
  double pos_choice = phred_n_choose_m(e.readlen, 2LL * e.ins_runs + e.del_runs, ln_n, T->ln_n_max);
  double del_term = e.del_runs > 0 ? py_int_round((double)e.del_runs * 10.0 * T->ln30 / LN_10) : 0.0;
  return match_term - mismatch_term - phred_n_choose_m(e.n_hq, e.m_hq, ln_n, T->ln_n_max) - pos_choice - del_term;
}

// missing_locus_probability (bayesian.rs:405-439) for one phase (0..4):
// returns exp(sum over non-overlapping 15-windows of ln(p_miss)).
// rep: per-window repeat code (0 none, 1 neighbour repetitive, 2 exact
// repetitive) or null when no seeding ran (repeat probability 0).
__device__ inline double missing_phase(int phase, const uint8_t* q, int len, const uint8_t* rep, int nwin,
                                       const DevTables* T) {
  double logp = 0.0;
  for (int st = phase; st + KMER <= len; st += KMER) {
    double rp = 0.0;
    if (rep && st < nwin) {
      uint8_t c = rep[st];
      rp = c == 2 ? 1.0 : (c == 1 ? T->nrp[q[st]] : 0.0);
    }
    double z = 1.0;
    for (int t = 0; t < KMER; t++) z = z * T->ml_one_minus_q[q[st + t]];
    double p1 = -0.0;
    for (int t = 0; t < KMER; t++) p1 = p1 + T->ml_q_over[q[st + t]];
    double p2 = 1.0 - z * (1.0 + p1);
    p2 = p2 < 0.0 ? 0.0 : (p2 > 1.0 ? 1.0 : p2);
    double pm = 1.0 - (1.0 - p2) * (1.0 - rp);
    pm = pm < 1e-300 ? 1e-300 : (pm > 1.0 ? 1.0 : pm);
    logp += log(pm);
  }
  return exp(logp);
}

// missing_phase with the repeat mask given as probabilities per window
// (the f64 repeat_mask of find_seed_hits, seeds.rs:91-151).
__device__ inline double missing_phase_mask(int phase, const uint8_t* q, int len, const double* mask, int nmask,
                                            const DevTables* T) {
  double logp = 0.0;
  for (int st = phase; st + KMER <= len; st += KMER) {
    const double rp = st < nmask ? mask[st] : 0.0;
    double z = 1.0;
    for (int t = 0; t < KMER; t++) z = z * T->ml_one_minus_q[q[st + t]];
    double p1 = -0.0;
    for (int t = 0; t < KMER; t++) p1 = p1 + T->ml_q_over[q[st + t]];
    double p2 = 1.0 - z * (1.0 + p1);
    p2 = p2 < 0.0 ? 0.0 : (p2 > 1.0 ? 1.0 : p2);
    double pm = 1.0 - (1.0 - p2) * (1.0 - rp);
    pm = pm < 1e-300 ? 1e-300 : (pm > 1.0 ? 1.0 : pm);
    logp += log(pm);
  }
  return exp(logp);
}
__device__ inline double missing_locus_mask(const uint8_t* q, int len, const double* mask, int nmask,
                                            const DevTables* T) {
  if (len < KMER) return 0.5;
  double s = 0.0;
  for (int k = 0; k < 5; k++) s += missing_phase_mask(k, q, len, mask, nmask, T);
  return fmin(s / 5.0, 0.99);
}

// Whole missing-locus probability by one thread: offset_means starts at 0.0
// and adds phases 0..4 in order.
__device__ inline double missing_locus_thread(const uint8_t* q, int len, const uint8_t* rep, int nwin,
                                              const DevTables* T) {
  if (len < KMER) return 0.5;
  double s = 0.0;
  for (int k = 0; k < 5; k++) s += missing_phase(k, q, len, rep, nwin, T);
  return fmin(s / 5.0, 0.99);
}

// wrong_mapping_probability (bayesian.rs:227-230).
__device__ __forceinline__ double wrong_prob(double sum_exp, const DevTables* T) {
  double bp = 1.0 / fmax(sum_exp, 1.0);
  return fmax(1.0 - bp, T->floor_wrong);
}

// finalize_mapq (bayesian.rs:251-282) given the missing-locus probability.
__device__ inline void finalize_mapq(double sum_exp, double entropy_raw, double p_missing_raw, const DevTables* T,
                                     uint8_t& mapq, double& post) {
  double pw = wrong_prob(sum_exp, T);
  double lnpw = pw == T->floor_wrong ? T->ln_floor_wrong : log(pw);
  double wrongmapping = py_int_round(lnpw / DB);
  double entropy = entropy_raw - 3.0;
  if (entropy <= 0.0) {
    mapq = 0;
    post = 0.0;
    return;
  }
  double pmiss = fmax(p_missing_raw, 1e-30);
  double l10;
  if (pmiss == 0.99) l10 = T->log10_099;
  else if (pmiss == 1e-30) l10 = T->log10_1e30;
  else l10 = log10(pmiss);
  double notfound = -10.0 * l10;
  double combined = logadd(wrongmapping, notfound);
  double pp = logadd(entropy, combined);
  pp = pp < 0.0 ? 0.0 : (pp > 99.0 ? 99.0 : pp);
  mapq = (uint8_t)round(pp);
  double pprob;
  if (pp == trunc(pp)) pprob = T->pow_neg_tenth[(int)pp];
  else pprob = pow(10.0, -pp / 10.0);
  post = 1.0 - pprob;
}

}  // namespace pbw
