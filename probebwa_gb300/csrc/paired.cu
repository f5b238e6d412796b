// paired.cu -- K5: the paired-end joint posterior (src/mapper/paired.rs).
//
// Per pair, after both mates went through K1-K3 (seeded candidates):
//   k_read_summary   per read: aligned candidates, select_best / sum_exp,
//                    wrong-mapping and missing-locus probabilities, the
//                    posterior shortlist (shortlist_indices, paired.rs:553-566)
//                    and the read's own single-end MAPQ (independent_record)
//   k_pair_decide    per pair against the batch's insert-size snapshot: fast
//                    path (paired.rs:266-291) or the raw candidate pairs with a
//                    cross-alignment job per shortlisted anchor
//                    (align_mate_near, paired.rs:450-468) into a work queue
//   (K3w)            the whole-window DPs of those jobs
//   k_pair_resolve   dedup, joint likelihoods (pair_distance_log_lk,
//                    paired.rs:486-496), select_best, mapq_for_winning_pair
//                    (paired.rs:398-435), flags / TLEN / proper pair and the
//                    insert-size observation (map_pair_readonly, paired.rs:154-234)
//   fold_insert_model (host) the serial InsertSizeDistribution::update over
//                    the batch's observations in pair order (paired.rs:139-143)
#include <algorithm>
#include <cmath>

#include "mapq_dev.cuh"
#include "paired.h"
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

constexpr double PROPER_PAIR_SD = 5.0;       // paired.rs:49
constexpr double FAST_PATH_CLOSE_SD = 4.0;   // paired.rs:57
constexpr double FAST_PATH_MAX_WRONG = 0.01; // paired.rs:64
constexpr double SHORTLIST_MASS = 0.999;     // paired.rs:71
constexpr int SHORTLIST_MIN = 3;             // paired.rs:72
constexpr int SHORTLIST_MAX = 20;            // paired.rs:73

// One thread per read: the work is serial FP64 per read (GB300 runs FP64 at a
// low rate, so every lane of a warp must carry a read for the pipe to be
// used at all).
__global__ void k_read_summary(ReadSummaryArgs p) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= p.nr) return;
  const uint64_t rg = (uint64_t)p.r0 + r;
  const uint64_t qo = p.offs[rg];
  const int L = (int)(p.offs[rg + 1] - qo);
  const AlnOut* A = p.aln + (size_t)r * MAX_CAND;
  const uint32_t nc = p.n_cand[r];
  ReadSum S;
  S.n_aln = 0;
  for (uint32_t i = 0; i < nc; i++)
    if (A[i].n_ops != 0) S.vslot[S.n_aln++] = (uint8_t)i;
  const int nwin = L >= KMER ? L - KMER + 1 : 0;
  const double pmiss = missing_locus_thread(p.quals + qo, L, p.rep + (size_t)r * p.wcap, nwin, p.tab);
  S.missing = pmiss;
  S.best = -1;
  S.sum_exp = 0.0;
  S.wrong = 1.0;
  S.n_short = 0;
  S.own_mapq = 0;
  S.own_post = 0.0;
  if (S.n_aln > 0) {
    double lk[MAX_CAND];
    double mx = 0.0;
    for (int k = 0; k < S.n_aln; k++) {
      lk[k] = A[S.vslot[k]].log_lk;
      if (k == 0 || lk[k] >= mx) { mx = lk[k]; S.best = k; }
    }
    double ex[MAX_CAND];
    double se = -0.0;
    for (int k = 0; k < S.n_aln; k++) {
      ex[k] = exp(lk[k] - mx);
      se += ex[k];
    }
    S.sum_exp = se;
    S.wrong = wrong_prob(se, p.tab);
    // posterior_fractions (bayesian.rs:208-216) then shortlist_indices: stable
    // sort by posterior descending, take while < 20 and not (>= 3 and mass >= 0.999)
    double post[MAX_CAND];
    int order[MAX_CAND];
    for (int k = 0; k < S.n_aln; k++) {
      post[k] = ex[k] / se;
      order[k] = k;
    }
    for (int a = 1; a < S.n_aln; a++) {  // stable insertion sort
      int v = order[a];
      int b = a - 1;
      while (b >= 0 && post[order[b]] < post[v]) {
        order[b + 1] = order[b];
        b--;
      }
      order[b + 1] = v;
    }
    double cum = 0.0;
    int take = 0;
    for (int t = 0; t < S.n_aln; t++) {
      if (take >= SHORTLIST_MAX) break;
      if (take >= SHORTLIST_MIN && cum >= SHORTLIST_MASS) break;
      cum += post[order[t]];
      take++;
    }
    S.n_short = (uint8_t)take;
    for (int t = 0; t < take; t++) S.shortlist[t] = (uint8_t)order[t];
    const AlnOut& W = A[S.vslot[S.best]];
    EntropyIn e{W.n_hq, W.m_hq, W.readlen, W.ins_runs, W.del_runs, W.gc, W.total};
    double ent = log_entropy(e, p.tab, p.gc_lnb, p.gc_lnbm1, p.ln_n);
    finalize_mapq(se, ent, pmiss, p.tab, S.own_mapq, S.own_post);
  }
  p.sum[r] = S;
}

// A candidate alignment seen by the pair kernels: own (seeded) or cross.
struct CandView {
  const AlnOut* a;
  uint32_t contig;
  uint8_t strand;
};

__device__ __forceinline__ CandView own_view(const PairArgs& p, int mate, uint32_t pl, int k) {
  const ReadSum& S = p.sum[mate][pl];
  const uint32_t slot = pl * MAX_CAND + S.vslot[k];
  CandView v;
  v.a = p.aln[mate] + slot;
  const Cand& c = p.cand[mate][slot];
  v.contig = c.contig;
  v.strand = c.strand;
  return v;
}

__device__ __forceinline__ CandView cross_view(const PairArgs& p, uint32_t cslot) {
  CandView v;
  v.a = p.xout + cslot;
  v.contig = p.xmeta[cslot].contig;
  v.strand = p.xmeta[cslot].strand;
  return v;
}

__device__ __forceinline__ bool same_locus(const CandView& a, const CandView& b) {  // paired.rs:517-519
  return a.contig == b.contig && a.a->pos == b.a->pos && a.strand == b.strand;
}
__device__ __forceinline__ long long implied_insert(const CandView& a, const CandView& b) {  // paired.rs:534-538
  const CandView& up = a.a->pos <= b.a->pos ? a : b;
  const CandView& dn = a.a->pos <= b.a->pos ? b : a;
  return (long long)(dn.a->pos + dn.a->span) - (long long)up.a->pos;
}
__device__ __forceinline__ bool is_fr(const CandView& a, const CandView& b) {  // paired.rs:544-547
  const CandView& up = a.a->pos <= b.a->pos ? a : b;
  const CandView& dn = a.a->pos <= b.a->pos ? b : a;
  return up.strand == 0 && dn.strand == 1;
}

// f64 -> usize cast of Rust: saturating, NaN -> 0.
__device__ __forceinline__ unsigned long long sat_u64(double x) {
  if (!(x > 0.0)) return 0ull;
  if (x >= 18446744073709551615.0) return ~0ull;
  return (unsigned long long)x;
}

__global__ void k_pair_decide(PairArgs p) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t np = p.batch ? p.batch[1] : p.np, p0 = p.batch ? p.batch[0] : p.p0;
  if (t >= np) return;
  const uint32_t pl = p0 + t;  // pair index within the super-chunk
  const ReadSum& S1 = p.sum[0][pl];
  const ReadSum& S2 = p.sum[1][pl];
  PairWork& W = p.work[pl];
  W.n_raw = 0;
  W.n_cross = 0;
  if (S1.n_aln == 0 && S2.n_aln == 0) {
    W.state = PAIR_UNMAPPED;
    return;
  }
  const double mean = p.model->mean, sd = p.model->sd;
  if (S1.n_aln > 0 && S2.n_aln > 0) {
    if (S1.wrong < FAST_PATH_MAX_WRONG && S2.wrong < FAST_PATH_MAX_WRONG && S1.missing < FAST_PATH_MAX_WRONG &&
        S2.missing < FAST_PATH_MAX_WRONG) {
      const CandView bx = own_view(p, 0, pl, S1.best), by = own_view(p, 1, pl, S2.best);
      const double gap = (double)implied_insert(bx, by);
      if (bx.contig == by.contig && is_fr(bx, by) && fabs(gap - mean) <= FAST_PATH_CLOSE_SD * sd) {
        W.state = PAIR_FAST;
        return;
      }
    }
  }
  W.state = PAIR_JOINT;
  // align_mate_near (paired.rs:450-468) as a job; returns false if the window is empty
  const unsigned long long meanu = sat_u64(fmax(mean, 0.0));
  const double rr = ceil(PROPER_PAIR_SD * sd);
  auto cross = [&](int mate, const CandView& anchor) -> int {
    const uint64_t* offs = mate == 0 ? p.offs1 : p.offs2;
    const uint64_t rg = (uint64_t)p.read0 + pl;
    const unsigned long long mlen = offs[rg + 1] - offs[rg];
    const unsigned long long radius = sat_u64(rr) + mlen;
    unsigned long long expected;
    uint8_t mstrand;
    if (anchor.strand == 0) {
      expected = anchor.a->pos + (meanu >= mlen ? meanu - mlen : 0ull);
      mstrand = 1;
    } else {
      const unsigned long long ae = anchor.a->pos + anchor.a->span;
      expected = ae >= meanu ? ae - meanu : 0ull;
      mstrand = 0;
    }
    const unsigned long long clen = p.G.clen[anchor.contig];
    const unsigned long long rs = expected >= radius ? expected - radius : 0ull;
    unsigned long long re = expected + mlen + radius;
    if (re > clen) re = clen;
    if (rs >= re) return -1;
    const int k = W.n_cross++;
    const uint32_t cslot = pl * MAX_CROSS + k;
    AlnJob J;
    J.ref_start = rs;
    J.ref_end = re;
    J.hint = (long long)(expected - rs);
    J.read = (uint32_t)rg;
    J.slot = cslot;
    J.contig = anchor.contig;
    J.band = (uint32_t)min(re - rs, (unsigned long long)(1u << 30));
    J.rev = mstrand;
    J.valid = 1;
    J.mate = (uint8_t)mate;
    J.pad = 0;
    J.pad2 = 0;
    J.gap_open = p.gap_open;
    J.gap_extend = p.gap_extend;
    p.xmeta[cslot].contig = anchor.contig;
    p.xmeta[cslot].strand = mstrand;
    p.xout[cslot].n_ops = 0;
    const unsigned int q = atomicAdd(p.n_jobs, 1u);
    p.jobs[q] = J;
    return k;
  };
  if (S1.n_aln > 0 && S2.n_aln > 0) {
    W.raw_x[W.n_raw] = (int16_t)S1.best;
    W.raw_y[W.n_raw] = (int16_t)S2.best;
    W.n_raw++;
    for (int s = 0; s < S1.n_short; s++) {
      const int i = S1.shortlist[s];
      const int k = cross(1, own_view(p, 0, pl, i));
      if (k >= 0) {
        W.raw_x[W.n_raw] = (int16_t)i;
        W.raw_y[W.n_raw] = (int16_t)(-(k + 1));
        W.n_raw++;
      }
    }
    for (int s = 0; s < S2.n_short; s++) {
      const int j = S2.shortlist[s];
      const int k = cross(0, own_view(p, 1, pl, j));
      if (k >= 0) {
        W.raw_x[W.n_raw] = (int16_t)(-(k + 1));
        W.raw_y[W.n_raw] = (int16_t)j;
        W.n_raw++;
      }
    }
  } else if (S1.n_aln == 0) {
    const int k = cross(0, own_view(p, 1, pl, S2.best));
    if (k >= 0) {
      W.raw_x[W.n_raw] = (int16_t)(-(k + 1));
      W.raw_y[W.n_raw] = (int16_t)S2.best;
      W.n_raw++;
    }
  } else {
    const int k = cross(1, own_view(p, 0, pl, S1.best));
    if (k >= 0) {
      W.raw_x[W.n_raw] = (int16_t)S1.best;
      W.raw_y[W.n_raw] = (int16_t)(-(k + 1));
      W.n_raw++;
    }
  }
}

struct RecOut {
  int32_t contig;
  unsigned long long pos;  // 1-based, 0 unmapped
  uint8_t mapq;
  uint8_t strand;
  double log_lk, post;
  int32_t as, nm;
  const AlnOut* a;         // CIGAR source (null: unmapped)
};

__device__ __forceinline__ RecOut make_rec(const CandView& v, uint8_t mapq, double post) {  // single.rs:338-359
  RecOut r;
  r.contig = (int32_t)v.contig;
  r.pos = v.a->pos + 1;
  r.mapq = mapq;
  r.strand = v.strand;
  r.log_lk = v.a->log_lk;
  r.post = post;
  r.as = v.a->score;
  r.nm = v.a->nm;
  r.a = v.a;
  return r;
}
__device__ __forceinline__ RecOut unmapped_rec() {  // single.rs:362-383
  RecOut r;
  r.contig = -1;
  r.pos = 0;
  r.mapq = 0;
  r.strand = 0;
  r.log_lk = 0.0;
  r.post = 0.0;
  r.as = 0;
  r.nm = 0;
  r.a = nullptr;
  return r;
}

__device__ __forceinline__ void fin(const PairArgs& p, double se, const CandView& v, double pmiss, uint8_t& q,
                                    double& post) {
  EntropyIn e{v.a->n_hq, v.a->m_hq, v.a->readlen, v.a->ins_runs, v.a->del_runs, v.a->gc, v.a->total};
  const double ent = log_entropy(e, p.tab, p.gc_lnb, p.gc_lnbm1, p.ln_n);
  finalize_mapq(se, ent, pmiss, p.tab, q, post);
}

// InsertSizeDistribution::log_likelihood (insert_size.rs:23-30) with the
// batch's ln(2*pi*sd^2) precomputed on the host (fold_insert_model).
__device__ __forceinline__ double insert_ll(const PairModel* M, double x) {
  if (M->sd <= 0.0) return -1e300;
  const double diff = x - M->mean;
  return -0.5 * (diff * diff) / (M->sd * M->sd) - 0.5 * M->ln_2pi_sd2;
}

__global__ void k_pair_resolve(PairArgs p) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t np = p.batch ? p.batch[1] : p.np, p0 = p.batch ? p.batch[0] : p.p0;
  if (t >= np) return;
  const uint32_t pl = p0 + t;
  const ReadSum& S1 = p.sum[0][pl];
  const ReadSum& S2 = p.sum[1][pl];
  const PairWork& W = p.work[pl];
  const PairModel* M = p.model;
  RecOut o1, o2;
  bool confident = false;
  if (W.state == PAIR_UNMAPPED) {
    o1 = unmapped_rec();
    o2 = unmapped_rec();
  } else if (W.state == PAIR_FAST) {
    o1 = make_rec(own_view(p, 0, pl, S1.best), S1.own_mapq, S1.own_post);
    o2 = make_rec(own_view(p, 1, pl, S2.best), S2.own_mapq, S2.own_post);
    confident = true;
  } else if (W.n_raw == 0) {
    o1 = S1.n_aln > 0 ? make_rec(own_view(p, 0, pl, S1.best), S1.own_mapq, S1.own_post) : unmapped_rec();
    o2 = S2.n_aln > 0 ? make_rec(own_view(p, 1, pl, S2.best), S2.own_mapq, S2.own_post) : unmapped_rec();
    confident = true;
  } else {
    auto view = [&](int mate, int16_t ref) -> CandView {
      return ref >= 0 ? own_view(p, mate, pl, ref) : cross_view(p, pl * MAX_CROSS + (uint32_t)(-ref - 1));
    };
    int keep[MAX_RAW];
    int nk = 0;
    for (int i = 0; i < W.n_raw; i++) {
      const CandView x = view(0, W.raw_x[i]), y = view(1, W.raw_y[i]);
      if (x.a->n_ops == 0 || y.a->n_ops == 0) continue;  // cannot happen: failed jobs are never listed
      bool dup = false;
      for (int k = 0; k < nk && !dup; k++) {
        const CandView px = view(0, W.raw_x[keep[k]]), py = view(1, W.raw_y[keep[k]]);
        dup = same_locus(px, x) && same_locus(py, y);
      }
      if (!dup) keep[nk++] = i;
    }
    double jl[MAX_RAW];
    int bi = 0;
    double mx = 0.0;
    for (int k = 0; k < nk; k++) {
      const CandView x = view(0, W.raw_x[keep[k]]), y = view(1, W.raw_y[keep[k]]);
      double pd;
      if (x.contig != y.contig || !is_fr(x, y)) {
        pd = p.sv_prior_log_prob;
      } else {
        pd = fmax(insert_ll(M, (double)implied_insert(x, y)), p.sv_prior_log_prob);
      }
      jl[k] = x.a->log_lk + y.a->log_lk + pd;
      if (k == 0 || jl[k] >= mx) {
        mx = jl[k];
        bi = k;
      }
    }
    double se = -0.0;
    for (int k = 0; k < nk; k++) se += exp(jl[k] - mx);
    const CandView bx = view(0, W.raw_x[keep[bi]]), by = view(1, W.raw_y[keep[bi]]);
    const bool bx_own = S1.n_aln > 0 && same_locus(bx, own_view(p, 0, pl, S1.best));
    const bool by_own = S2.n_aln > 0 && same_locus(by, own_view(p, 1, pl, S2.best));
    uint8_t q1, q2;
    double p1, p2;
    if (bx_own && by_own) {
      fin(p, S1.sum_exp, bx, S1.missing, q1, p1);
      fin(p, S2.sum_exp, by, S2.missing, q2, p2);
    } else if (bx_own != by_own) {
      if (bx_own) fin(p, S1.sum_exp, bx, S1.missing, q1, p1);
      else fin(p, S2.sum_exp, by, S2.missing, q1, p1);
      q2 = q1;
      p2 = p1;
    } else {
      fin(p, se, bx, S1.missing, q1, p1);
      fin(p, se, by, S2.missing, q2, p2);
    }
    o1 = make_rec(bx, q1, p1);
    o2 = make_rec(by, q2, p2);
    confident = bx_own && by_own;
  }
  // flags, mate fields, TLEN, proper pair, observation (paired.rs:166-231)
  const bool m1 = o1.pos != 0, m2 = o2.pos != 0;
  uint16_t f1 = 0x1 | 0x40, f2 = 0x1 | 0x80;
  if (!m1) f1 |= 0x4;
  if (!m2) f2 |= 0x4;
  if (!m2) f1 |= 0x8;
  if (!m1) f2 |= 0x8;
  if (m1 && o1.strand) f1 |= 0x10;
  if (m2 && o2.strand) f2 |= 0x10;
  if (m2 && o2.strand) f1 |= 0x20;
  if (m1 && o1.strand) f2 |= 0x20;
  int32_t mc1 = -1, mc2 = -1;
  unsigned long long mp1 = 0, mp2 = 0;
  long long tl1 = 0, tl2 = 0;
  double obs = nan("");
  if (m1 && m2 && p.G.name_class[o1.contig] == p.G.name_class[o2.contig]) {
    const RecOut& up = o1.pos <= o2.pos ? o1 : o2;
    const RecOut& dn = o1.pos <= o2.pos ? o2 : o1;
    const long long de = (long long)(dn.pos + dn.a->span) - 1;
    long long ins = de - (long long)up.pos + 1;
    if (ins < 0) ins = 0;
    const bool within = fabs((double)ins - M->mean) < PROPER_PAIR_SD * M->sd;
    const bool fr = up.strand == 0 && dn.strand == 1;  // is_fr_orientation (paired.rs:572-575)
    const bool proper = within && fr;
    if (proper) {
      f1 |= 0x2;
      f2 |= 0x2;
    }
    mc1 = o2.contig;
    mc2 = o1.contig;
    mp1 = o2.pos;
    mp2 = o1.pos;
    tl1 = o1.pos <= o2.pos ? ins : -ins;
    tl2 = o2.pos <= o1.pos ? ins : -ins;
    if (proper && confident) obs = (double)ins;
  }
  const uint64_t g1 = (uint64_t)p.out_base + pl, g2 = (uint64_t)p.out_base + p.n_total + pl;
  const RecOut* os[2] = {&o1, &o2};
  const uint64_t gi[2] = {g1, g2};
  const uint16_t fl[2] = {f1, f2};
  const int32_t mcs[2] = {mc1, mc2};
  const unsigned long long mps[2] = {mp1, mp2};
  const long long tls[2] = {tl1, tl2};
  const uint64_t* offs[2] = {p.offs1, p.offs2};
  for (int k = 0; k < 2; k++) {
    const RecOut& o = *os[k];
    const uint64_t g = gi[k];
    p.o_contig[g] = o.contig;
    p.o_pos[g] = o.pos;
    p.o_mapq[g] = o.mapq;
    p.o_flag[g] = fl[k];
    p.o_mate_contig[g] = mcs[k];
    p.o_mate_pos[g] = mps[k];
    p.o_tlen[g] = tls[k];
    p.o_log_lk[g] = o.log_lk;
    p.o_post[g] = o.post;
    p.o_as[g] = o.as;
    p.o_nm[g] = o.nm;
    if (o.a) {
      p.o_nops[g] = o.a->n_ops;
      p.o_cigsrc[g] = o.a;
    } else {
      const uint64_t rg = (uint64_t)p.read0 + pl;
      p.o_nops[g] = 1;
      p.o_cigsrc[g] = nullptr;
      p.o_len[g] = (uint32_t)(offs[k][rg + 1] - offs[k][rg]);
    }
  }
  p.obs[pl] = obs;
  if (p.obs_batch) p.obs_batch[t] = obs;
}

// InsertSizeDistribution::update (insert_size.rs:32-44) over one batch's
// observations in pair order (paired.rs:139-143; NaN = the pair gave none),
// then the next batch's ln(2*pi*sd^2) (insert_size.rs:29).
//
// This runs in the host runtime between batches. The recurrence is one
// dependent chain of about twenty FP64 operations per observation (two
// divisions and a square root among them); on GB300 a dependent FP64 chain
// costs ~40 cycles per operation, ~0.4 us per observation, while the host
// cores take ~20 ns. Host code is compiled without FMA contraction, so every
// operation rounds exactly as the reference's f64 arithmetic, and the
// logarithm is the host libm's, as in the reference.
void fold_insert_model(PairModel& M, const double* obs, uint32_t np) {
  double mean = M.mean, sd = M.sd;
  unsigned long long n = M.n;
  for (uint32_t i = 0; i < np; i++) {
    const double x = obs[i];
    if (std::isnan(x)) continue;
    n++;
    const double nn = (double)n;
    const double delta = x - mean;
    mean += delta / nn;
    const double delta2 = x - mean;
    const double var = nn > 1.0 ? ((sd * sd) * (nn - 1.0) + delta * delta2) / nn : sd * sd;
    sd = std::max(std::sqrt(var), 1.0);
  }
  M.mean = mean;
  M.sd = sd;
  M.n = n;
  M.ln_2pi_sd2 = std::log(2.0 * 3.141592653589793115997963468544185161590576171875 * sd * sd);
}

__global__ void k_pair_cigar_gather(const PairArgs p, const uint32_t* cig_off, const uint32_t* cig_pool, uint32_t* cigar,
                                    uint64_t g0, uint32_t n) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint64_t g = g0 + t;
  const uint32_t dst = cig_off[g];
  const AlnOut* a = p.o_cigsrc[g];
  if (!a) {
    cigar[dst] = (p.o_len[g] << 4) | 4u;
    return;
  }
  const uint32_t* src = a->n_ops > CIG_INLINE ? cig_pool + a->cig_pool : a->cig;
  for (uint32_t k = 0; k < a->n_ops; k++) cigar[dst + k] = src[k];
}

void launch_read_summary(const ReadSummaryArgs& a, cudaStream_t st) {
  if (a.nr == 0) return;
  k_read_summary<<<(unsigned)(((uint64_t)a.nr + 127) / 128), 128, 0, st>>>(a);
}
// A batch has at most 2000 pairs of serial FP64 work, and an SM's FP64 pipe
// takes two lanes per clock: one warp per block spreads a batch over ~60 SMs.
void launch_pair_decide(const PairArgs& a, cudaStream_t st) {
  if (a.np == 0) return;
  k_pair_decide<<<(a.np + 31) / 32, 32, 0, st>>>(a);
}
void launch_pair_resolve(const PairArgs& a, cudaStream_t st) {
  if (a.np == 0) return;
  k_pair_resolve<<<(a.np + 31) / 32, 32, 0, st>>>(a);
}
void launch_pair_cigar_gather(const PairArgs& a, const uint32_t* cig_off, const uint32_t* cig_pool, uint32_t* cigar,
                              uint64_t g0, uint32_t n, cudaStream_t st) {
  if (n == 0) return;
  k_pair_cigar_gather<<<(n + 127) / 128, 128, 0, st>>>(a, cig_off, cig_pool, cigar, g0, n);
}

}  // namespace pbw
