// pbw_common.cuh -- device data layout and helpers shared by the kernels.
//
// HBM layout (one handle):
//   genome   2-bit bases, 32 per 64-bit word (base g at bits 2*(g%32) of word
//            g/32; the reference's packed bytes, src/index/genome.rs:17-45,
//            read as little-endian words). Every contig starts on a word
//            boundary (global base offset a multiple of 32).
//   nmask    1 bit per base (same global indexing), set where Contig::slice
//            overlays 'N' (src/index/genome.rs:60-66).
//   csr      dense CSR over the 4^15 raw 15-mer codes: bucket of code c is
//            entries[csr[c] .. csr[c+1]). Raw code = 2 bits per base, first
//            base most significant (src/index/hashtable.rs:107-113); the file
//            stores mix(raw), which is a bijection, so the loader inverts it.
//   entries  packed occurrences in the file's bucket order
//            (src/index/hashtable.rs:157-171: strand<<63 | contig<<40 | pos).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include <mutex>
#include <set>
#include <utility>

namespace pbw {

constexpr int KMER = 15;
constexpr uint64_t NKMER = 1ull << 30;           // 4^15 raw codes
constexpr int MAX_CAND = 20;                     // single.rs:114 take(20)
constexpr int32_t NEG = INT32_MIN / 2;           // smith_waterman.rs:173
constexpr uint64_t DIAG_BIAS = 1ull << 16;       // > PBW_MAX_READ_LEN
constexpr uint32_t REPEAT_SKIP = 64;             // seeds.rs:45
constexpr int RANK_FEATURES = 12;                // candidate ranker: seed features per candidate
constexpr int CIG_INLINE = 12;                   // CIGAR ops kept inline per alignment

// Internal base codes. Reference bases: A0 C1 G2 T3 N4. Reads: the same plus
// 5 for any other byte (never equal to a reference base, as in the byte
// comparisons of smith_waterman.rs:204 and bayesian.rs:156).
__host__ __device__ inline uint8_t base_code(uint8_t b) {
  if (b >= 'a' && b <= 'z') b = (uint8_t)(b - 32);
  switch (b) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    case 'N': return 4;
    default: return 5;
  }
}
// DnaSeq::reverse_complement (src/types.rs:34-48): non-ACGT -> N.
__host__ __device__ inline uint8_t comp_code(uint8_t c) { return c < 4 ? (uint8_t)(3 - c) : (uint8_t)4; }

// ASCII of a reference code 0..4 (A C G T N) from a packed constant: no
// memory access, so lanes with different codes stay in one instruction.
__host__ __device__ __forceinline__ uint8_t code_ascii(uint32_t c) { return (uint8_t)(0x4E54474341ull >> (8 * c)); }
// DnaSeq::from_ascii upper-casing and reverse_complement on ASCII (A<->T,
// C<->G, anything else N), as selects rather than a switch.
__host__ __device__ __forceinline__ uint8_t up_ascii(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }
__host__ __device__ __forceinline__ uint8_t comp_ascii(uint8_t b) {
  return b == 'A' ? (uint8_t)'T' : b == 'T' ? (uint8_t)'A' : b == 'C' ? (uint8_t)'G' : b == 'G' ? (uint8_t)'C' : (uint8_t)'N';
}

struct DevGenome {
  const unsigned long long* bits;
  const unsigned int* nmask;
  const unsigned int* nblk;         // 1 bit per 1024-base block (32 nmask words): the block holds an N
  const unsigned long long* cbase;  // per contig: global base offset
  const unsigned long long* clen;   // per contig: length
  const int* name_class;            // per contig: first contig index with the same name
  unsigned int ncontig;
};

struct DevIndex {
  const unsigned int* csr;          // NKMER + 1
  const unsigned long long* ent;
};

// Reference base code at global position gp (0..3, or 4 for N).
__device__ __forceinline__ uint8_t gcode(const DevGenome& g, uint64_t gp) {
  unsigned long long w = __ldg(&g.bits[gp >> 5]);
  unsigned int nm = __ldg(&g.nmask[gp >> 5]);
  if ((nm >> (gp & 31)) & 1u) return 4;
  return (uint8_t)((w >> ((gp & 31) * 2)) & 3ull);
}

// Quality-indexed and integer-indexed tables computed on the host with the
// same libm as the oracle (parameter setup at open time).
struct DevTables {
  double llk_match[256];    // ln(max(1-e, 1e-300)), e = 10^(-logadd(q,sub)/10)  (bayesian.rs:152-157)
  double llk_mismatch[256]; // ln(max(e/3, 1e-300))
  double ml_one_minus_q[256];  // 1 - q_i            (bayesian.rs:412-427)
  double ml_q_over[256];       // q_i / (1 - q_i)
  double nrp[256];             // 10^(-q/10)         (seeds.rs:134)
  double pow_neg_tenth[100];   // 10^(-p/10) for integral p in [0, 99] (bayesian.rs:280)
  int32_t mmpen[256];          // mismatch_penalty(q) (smith_waterman.rs:272-275)
  double ln_quarter;           // ln(0.25)
  double ln_two_g;             // ln(2 * genome_size)
  double del_term;             // py_int_round(10 * ln(30) / ln(10)) per deletion run is computed from this
  double ln30;
  double subphred;
  double floor_wrong;          // exp(99 * DB)
  double ln_floor_wrong;       // ln(exp(99 * DB))
  double log10_099;            // log10(0.99): missing-locus cap (bayesian.rs:438)
  double log10_1e30;           // log10(1e-30): missing-locus floor (bayesian.rs:273)
  double sv_prior_log_prob;
  int32_t gap_open, gap_extend;  // seeded aligner (SmithWatermanAligner::new)
  int32_t ln_n_max;            // entries in ln_n
  int32_t gc_tmax;             // totals covered by gc tables
};

// Dynamic shared-memory limit of a kernel: once per kernel and device, the
// device's per-block maximum less the kernel's static shared memory. The
// limit is only a ceiling (each launch's occupancy follows its own size), and
// one value for every launch keeps launches from several host threads (one
// handle each) from lowering it under one another.
inline void smem_ceiling_impl(const void* fn) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  std::lock_guard<std::mutex> g(mu);
  if (!done.insert({fn, dev}).second) return;
  int mx = 0;
  cudaFuncAttributes a{};
  if (cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return;
  if (cudaFuncGetAttributes(&a, fn) != cudaSuccess) return;
  cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, mx - (int)a.sharedSizeBytes);
}
template <class K>
inline void smem_ceiling(K* kernel) {
  smem_ceiling_impl((const void*)kernel);
}

}  // namespace pbw
