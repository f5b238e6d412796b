// oracle.h -- CPU restatement of probebwa's read-mapping path.
//
// TEST INFRASTRUCTURE ONLY. This is the correctness oracle and the timed CPU
// baseline for the GB300 mapper in probebwa_gb300/. Only tests/, the smoke
// check in __graft_entry__.py and the CPU-baseline leg of bench.py may load
// it. The product never links, loads or calls anything under oracle/.
//
// The reference (GUIBA-EX/probebwa) is pure Rust and cannot be built in this
// environment (no Rust toolchain), so every function here restates the
// reference's behaviour in C++17, citing the reference file:line it follows.
// Parity of this restatement is pinned against the reference's own
// known-answer tests (tests/mapping.rs, tests/integration.rs,
// src/index/hashtable.rs unit tests), re-run in tests/test_oracle_kat.py.
//
// The one behaviour no reference test pins is the iteration order of the
// FxHashMap that groups seed hits by (contig, strand) in
// src/mapper/candidates.rs:34-46. It decides the order of equal-score
// candidates. It is restated from the published algorithms of rustc-hash
// 2.1.3 (FxHasher) and of std's SwissTable (hashbrown), with the SIMD group
// width as a parameter (16 on x86_64/SSE2, 8 on aarch64/NEON): parity of
// that tie order is unpinned.
#pragma once
#include <cstdint>
#include <cstddef>

#ifdef __cplusplus
extern "C" {
#endif

// Mapper options: MapperOptions (src/types.rs:207-249) plus the SwissTable
// group width used for the candidate tie order.
typedef struct {
  double substitution_rate;  // default 0.001
  double insert_size_mean;   // default 250
  double insert_size_sd;     // default 60
  uint64_t max_indel_len;    // default 30
  uint32_t gap_open_phred;   // default 40
  uint32_t gap_extend_phred; // default 3
  double sv_prior_phred;     // default 55
  int32_t threads;           // worker threads (0 = all cores)
  int32_t group_width;       // 16 or 8
  uint64_t dense_min_buckets;  // .sthash tables with more buckets load as a direct-address map (default 2^24)
} orc_options;

// Reads as structure-of-arrays: concatenated sequence bytes and Phred
// scores (offset already subtracted), n+1 offsets.
typedef struct {
  uint64_t n;
  const uint8_t* bases;
  const uint8_t* quals;
  const uint64_t* offsets;
} orc_reads;

// Output records as structure-of-arrays (same field meaning as pbw_records
// in the product's C ABI). cigar ops are (len << 4) | op with op 0=M 1=I
// 2=D 4=S.
typedef struct {
  uint64_t n;
  int32_t* contig;
  uint64_t* pos;
  uint8_t* mapq;
  uint16_t* flag;
  int32_t* mate_contig;
  uint64_t* mate_pos;
  int64_t* tlen;
  double* log_lk;
  double* posterior;
  int32_t* as_score;
  int32_t* nm;
  uint32_t* cigar_off;
  uint32_t* cigar;
  uint64_t cigar_cap;
} orc_records;

typedef struct {
  double mean;
  double sd;
  uint64_t n_observed;
} orc_insert_model;

void orc_default_options(orc_options* o);
const char* orc_last_error(void);

// ---- index files (src/index/genome.rs, src/index/hashtable.rs) ----
int orc_build_genome(const char* out_prefix, const char* species, const char* assembly,
                     int nfiles, const char** fasta_paths);
int orc_build_genome_from_seqs(const char* out_prefix, const char* species, const char* assembly,
                               int ncontigs, const char** names, const uint8_t** seqs,
                               const uint64_t* lens);
int orc_build_hash(const char* genome_prefix, const char* out_prefix, uint64_t k,
                   uint64_t stride, uint64_t max_count);

// ---- mapper handle ----
void* orc_open(const char* genome_prefix, const char* hash_prefix, const orc_options* opt);
void orc_close(void* h);
uint64_t orc_num_contigs(void* h);
uint64_t orc_genome_total_length(void* h);

// Single-end map_reads path (src/lib.rs:86-104 + src/mapper/single.rs:164-209).
int orc_map_single(void* h, const orc_reads* reads, orc_records* out);
// Paired-end map_paired path (src/lib.rs:145-185) including the 500-pair
// serial warm-up and 2000-pair frozen-model batches; model is in/out.
int orc_map_paired(void* h, orc_insert_model* model, const orc_reads* r1, const orc_reads* r2,
                   orc_records* o1, orc_records* o2);

// ---- stage entry points for stage-level parity tests ----
// find_seed_hits (src/mapper/seeds.rs:91-151) for one read. Hits are written
// as (read_pos, contig, ref_pos, strand) in emission order.
int64_t orc_seed_read(void* h, const uint8_t* bases, const uint8_t* quals, uint64_t len,
                      uint64_t* hit_read_pos, uint32_t* hit_contig, uint64_t* hit_ref_pos,
                      uint8_t* hit_strand, uint64_t hit_cap, double* repeat_prob);
// cluster_hits (src/mapper/candidates.rs:30-78): full candidate list.
int64_t orc_cluster_read(void* h, const uint8_t* bases, const uint8_t* quals, uint64_t len,
                         uint32_t* cand_contig, uint64_t* cand_pos, uint8_t* cand_strand,
                         double* cand_score, uint64_t cand_cap);
// SmithWatermanAligner::new + align (src/align/smith_waterman.rs:113-255).
/* MapqCalculator::select_best + finalize_mapq (src/mapq/bayesian.rs:193-201,
 * 251-282) for a batch; see pbw_mapq_batch for the layout. */
int orc_mapq_batch(void* h, const orc_reads* reads, const uint64_t* lk_off, const double* lks,
                   const uint64_t* win_off, const double* repeat, const uint8_t* rev, const uint64_t* ref_off,
                   const uint8_t* refs, const uint32_t* cigar_off, const uint32_t* cigar, uint8_t* mapq,
                   double* posterior, uint32_t* best, double* sum_exp);
int orc_align(const uint8_t* read, const uint8_t* qual, uint64_t m, const uint8_t* ref, uint64_t n,
              int64_t hint, uint64_t band, uint32_t gop, uint32_t gep, int32_t* score,
              uint64_t* offset, uint32_t* cigar, uint64_t cigar_cap, uint64_t* n_ops);
// SAM text for a record set (src/io/sam.rs:37-143). Writes to path.
int orc_write_sam(void* h, const char* path, const char* command_line, const orc_reads* reads,
                  const char* const* read_ids, const orc_records* recs);
// SAM stream of the records numbered r * n_src + s (record r of source s;
// n_src 2 = mates 1 and 2) listed in sel, with an optional --readgroup spec
// and the SO:coordinate header (format_sam_records_sorted, sam.rs:83-108).
// path "-" = standard output.
int orc_sam_write(void* h, const char* command_line, const char* read_group, int coordinate_sorted, uint32_t n_src,
                  const orc_reads* const* reads, const char* const* const* ids, const orc_records* const* recs,
                  const uint64_t* sel, uint64_t n_sel, const char* path);
// sort_for_coordinate_order (sam.rs:114-124) of the numbered records in sel.
int orc_sort_coordinate(void* h, uint32_t n_src, const orc_records* const* recs, const uint64_t* sel, uint64_t n_sel,
                        uint64_t* out);
// The `probebwa map` command (src/main.rs:51-111, 130-189) restated over this
// oracle: same flags, same SAM stream; argv[1] must be "map". Returns the exit
// status (0; 1 on an error, reported on stderr as "Error: ..."; 2 on a usage
// error).
int orc_cli_main(int argc, char** argv);

// ---- FASTQ / FASTA reads (src/io/fastx.rs) ----
// Parses a file into an internal buffer; returns a handle with n reads.
void* orc_reads_parse(const char* path, int fasta, uint8_t quality_offset, const char* adapter);
uint64_t orc_reads_count(void* rh);
uint64_t orc_reads_total_bases(void* rh);
void orc_reads_export(void* rh, uint8_t* bases, uint8_t* quals, uint64_t* offsets);
const char* orc_reads_id(void* rh, uint64_t i);
void orc_reads_free(void* rh);

// Timing helper for the CPU baseline: maps reads and returns wall seconds.
double orc_time_map_single(void* h, const orc_reads* reads, orc_records* out);
double orc_time_map_paired(void* h, orc_insert_model* model, const orc_reads* r1,
                           const orc_reads* r2, orc_records* o1, orc_records* o2);

#ifdef __cplusplus
}
#endif
