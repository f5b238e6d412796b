// paired.h -- argument blocks of the paired-end kernels (paired.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

constexpr int MAX_CROSS = 2 * MAX_CAND;   // shortlist cross-alignments per pair (20 + 20)
constexpr int MAX_RAW = MAX_CROSS + 1;    // + the independent best-best pair

enum : uint8_t { PAIR_UNMAPPED = 0, PAIR_FAST = 1, PAIR_JOINT = 2 };

// Per read: what the joint posterior needs from its own candidates.
struct ReadSum {
  double sum_exp;    // select_best denominator over the aligned candidates
  double wrong;      // wrong_mapping_probability(sum_exp)
  double missing;    // missing_locus_probability(read, repeat_mask)
  double own_post;   // posterior of the read's own single-end record
  int32_t n_aln;     // aligned candidates (the `alignments` vector)
  int32_t best;      // argmax (last maximum) in that vector, -1 if empty
  uint8_t own_mapq;
  uint8_t n_short;
  uint8_t vslot[MAX_CAND];      // candidate slot of the k-th aligned candidate
  uint8_t shortlist[MAX_CAND];  // shortlist_indices, indices into the aligned vector
};

struct PairWork {
  int16_t raw_x[MAX_RAW];  // >= 0: mate-1 aligned index; < 0: -(cross slot + 1)
  int16_t raw_y[MAX_RAW];  // >= 0: mate-2 aligned index; < 0: -(cross slot + 1)
  uint8_t state;
  uint8_t n_raw;
  uint8_t n_cross;
  uint8_t pad;
};

struct XMeta {
  uint32_t contig;
  uint8_t strand;
  uint8_t pad[3];
};

// InsertSizeDistribution (src/types.rs:266-270) on the device, plus the
// batch constant ln(2*pi*sd^2) of log_likelihood.
struct PairModel {
  double mean;
  double sd;
  unsigned long long n;
  double ln_2pi_sd2;
};

struct ReadSummaryArgs {
  const DevTables* tab;
  const double* ln_n;
  const double* gc_lnb;
  const double* gc_lnbm1;
  const uint8_t* quals;
  const uint64_t* offs;
  uint32_t r0, nr;
  const AlnOut* aln;        // nr * MAX_CAND
  const uint32_t* n_cand;
  const uint8_t* rep;
  uint32_t wcap;
  ReadSum* sum;
};

struct PairArgs {
  DevGenome G;
  const DevTables* tab;
  const double* ln_n;
  const double* gc_lnb;
  const double* gc_lnbm1;
  const uint64_t* offs1;
  const uint64_t* offs2;
  uint32_t read0;           // read index of super-chunk pair 0 in the offsets arrays
  uint32_t p0, np;          // the batch: super-chunk pairs [p0, p0 + np)
  const uint32_t* batch;    // optional device {p0, np} in place of p0 / np (one graph replayed per batch;
                            // np above is then only the grid bound)
  double* obs_batch;        // optional: the batch's observations again at batch-relative indices
  const ReadSum* sum[2];
  const AlnOut* aln[2];
  const Cand* cand[2];
  PairWork* work;
  PairModel* model;
  double sv_prior_log_prob;
  int32_t gap_open, gap_extend;
  AlnJob* jobs;
  unsigned int* n_jobs;
  AlnOut* xout;             // cross-alignment outputs, super-chunk pairs * MAX_CROSS
  XMeta* xmeta;
  double* obs;
  // records: mate 1 at out_base + pair, mate 2 at out_base + n_total + pair
  uint64_t out_base;
  uint64_t n_total;
  int32_t* o_contig;
  unsigned long long* o_pos;
  uint8_t* o_mapq;
  uint16_t* o_flag;
  int32_t* o_mate_contig;
  unsigned long long* o_mate_pos;
  long long* o_tlen;
  double* o_log_lk;
  double* o_post;
  int32_t* o_as;
  int32_t* o_nm;
  uint32_t* o_nops;
  const AlnOut** o_cigsrc;
  uint32_t* o_len;
};

void launch_read_summary(const ReadSummaryArgs& a, cudaStream_t st);
void launch_pair_decide(const PairArgs& a, cudaStream_t st);
void launch_pair_resolve(const PairArgs& a, cudaStream_t st);
void fold_insert_model(PairModel& M, const double* obs, uint32_t np);
void launch_pair_cigar_gather(const PairArgs& a, const uint32_t* cig_off, const uint32_t* cig_pool, uint32_t* cigar,
                              uint64_t g0, uint32_t n, cudaStream_t st);

}  // namespace pbw
