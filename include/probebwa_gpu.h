/* probebwa_gpu.h -- C ABI of the GB300 (sm_103a) probebwa mapping path.
 *
 * Plain C types only: pointers, sizes and status codes. Every call returns
 * PBW_OK (0) or a negative PBW_ERR_* code; pbw_last_error(h) (or
 * pbw_last_error(NULL) for a call without a handle, such as a failed
 * pbw_open, on the calling thread) describes the failure. No C++
 * exception or CUDA error crosses this boundary.
 *
 * Each entry point names the reference interface it replaces
 * (GUIBA-EX/probebwa, file:line).
 *
 * Threading: one handle owns one CUDA stream and its device buffers; calls on
 * one handle must be serialised by the caller. Different handles are
 * independent.
 */
#ifndef PROBEBWA_GPU_H
#define PROBEBWA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBW_ABI_VERSION 1

#define PBW_OK 0
#define PBW_ERR_ARG -1        /* invalid argument */
#define PBW_ERR_IO -2         /* cannot open / read an index file */
#define PBW_ERR_FORMAT -3     /* malformed .stidx / .sthash */
#define PBW_ERR_CUDA -4       /* CUDA runtime error */
#define PBW_ERR_NOMEM -5      /* device or host allocation failed */
#define PBW_ERR_LIMIT -6      /* input beyond a documented device limit */
#define PBW_ERR_CAPACITY -7   /* caller-provided output array too small */
#define PBW_ERR_DEVICE -8     /* a kernel reported an internal error */

/* Longest read the device path maps (bases). Longer reads: PBW_ERR_LIMIT. */
#define PBW_MAX_READ_LEN 1024

typedef struct pbw_handle pbw_handle;

/* MapperOptions (src/types.rs:207-249) plus device settings. */
typedef struct {
  double substitution_rate;   /* --substitution-rate, default 0.001 */
  double insert_size_mean;    /* insert-size prior mean, default 250 */
  double insert_size_sd;      /* insert-size prior sd, default 60 */
  uint64_t max_indel_len;     /* seeded DP band, default 30 */
  uint32_t gap_open_phred;    /* --gapopen, default 40 */
  uint32_t gap_extend_phred;  /* --gapextend, default 3 */
  double sv_prior_phred;      /* --svprior, default 55 */
  /* SwissTable group width whose iteration order the candidate tie order
   * follows: 16 = the reference built for x86_64 (SSE2), 8 = aarch64. */
  int32_t group_width;
  int32_t device;             /* CUDA device ordinal */
  uint64_t chunk_reads;       /* reads per device chunk (0 = default) */
} pbw_options;

/* Reads as structure-of-arrays (Read, src/types.rs:79-84): concatenated
 * sequence bytes (any case; uppercased like DnaSeq::from_ascii), Phred
 * scores with the ASCII offset already removed (QualityScores::scores), and
 * n+1 offsets shared by both arrays (sequence and quality have equal
 * length). */
typedef struct {
  uint64_t n;
  const uint8_t* bases;
  const uint8_t* quals;
  const uint64_t* offsets;
} pbw_reads;

/* Output records as structure-of-arrays (AlignmentRecord, src/types.rs:181-203).
 * contig / mate_contig are indices into the genome's contigs (-1 = '*').
 * pos and mate_pos are 1-based (0 = unmapped / none). flag is the SAM FLAG of
 * src/io/sam.rs:126-143. log_lk = alignment_score, posterior =
 * posterior_prob. as_score (the DP score the reference computes and drops,
 * src/mapper/single.rs:128) and nm (edit distance) are derived fields.
 * cigar holds (len << 4) | op with op 0=M 1=I 2=D 4=S; cigar_off has n+1
 * entries; cigar_cap is the capacity of cigar (2*total_bases + 2*n always
 * suffices). SEQ/QUAL are not copied: they are the input read, reverse-
 * complemented and reversed when (flag & 0x10). */
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
} pbw_records;

/* InsertSizeDistribution (src/types.rs:266-270). */
typedef struct {
  double mean;
  double sd;
  uint64_t n_observed;
} pbw_insert_model;

/* Per-call device timing (milliseconds, CUDA events) and work counters. */
typedef struct {
  double ms_total;
  double ms_h2d;
  double ms_seed;
  double ms_cluster;
  double ms_align;
  double ms_finalize;
  double ms_pair;
  double ms_d2h;
  uint64_t seed_probes;       /* hash lookups */
  uint64_t seed_entries;      /* bucket entries read */
  uint64_t seed_hits;         /* hits that passed the similarity filter */
  uint64_t dp_jobs;           /* alignments */
  uint64_t dp_cells;          /* DP cells (smith_waterman.rs:191-203 bands) */
  uint64_t kernel_launches;   /* kernels launched by the call */
  uint64_t window_jobs;       /* paired path: mate rescue / shortlist cross-alignments (also in dp_jobs) */
  uint64_t window_cells;      /* their DP cells (also in dp_cells) */
  double ms_compute;          /* device span of the mapping work, input copy and record copy excluded; the
                                 phases above overlap in paired calls, so their sum can exceed it */
  double t_compute_begin_ms;  /* that span's ends on the device clock, in ms from an origin event the */
  double t_compute_end_ms;    /* process records on the device when its first handle opens: the spans of
                                 calls running at once on several handles merge as max(end) - min(begin) */
} pbw_stats;

void pbw_default_options(pbw_options* opt);

/* Open an index: replaces GenomeIndex::load (src/index/genome.rs:80-86) +
 * HashTable::load (src/index/hashtable.rs:73-79) + the SingleEndMapper /
 * PairedEndMapper constructors (src/mapper/single.rs:52-70,
 * src/mapper/paired.rs:85-99). Reads <prefix>.stidx and <prefix>.sthash and
 * uploads a 2-bit genome, an N mask and a dense k-mer CSR to the device. */
int pbw_open(const char* genome_prefix, const char* hash_prefix, const pbw_options* opt, pbw_handle** out);
void pbw_close(pbw_handle* h);
const char* pbw_last_error(const pbw_handle* h);

/* Index facts: contig count, total length, contig names / lengths. */
uint64_t pbw_num_contigs(const pbw_handle* h);
uint64_t pbw_total_length(const pbw_handle* h);
const char* pbw_contig_name(const pbw_handle* h, uint64_t i);
uint64_t pbw_contig_length(const pbw_handle* h, uint64_t i);

/* Single-end mapping: replaces SingleEndMapper::map (src/mapper/single.rs:164-209)
 * applied per read by map_reads_with_format (src/lib.rs:86-104). Host buffers
 * in and out. */
int pbw_map_single(pbw_handle* h, const pbw_reads* reads, pbw_records* out);

/* Paired-end mapping: replaces map_paired (src/lib.rs:145-185), i.e.
 * PairedEndMapper::map_pair for the first 500 pairs and
 * PairedEndMapper::map_pairs_batch (src/mapper/paired.rs:127-146) for batches
 * of 2000 after them. model is the insert-size model, read and updated. */
int pbw_map_paired(pbw_handle* h, pbw_insert_model* model, const pbw_reads* r1, const pbw_reads* r2,
                   pbw_records* o1, pbw_records* o2);

/* Stage entry points for parity tests. */

/* SmithWatermanAligner::new(band, gop, gep).align(read, qual, ref, hint)
 * (src/align/smith_waterman.rs:113-255) for a batch of independent problems.
 * reads/quals/refs are concatenated with n+1 offsets; outputs score, offset
 * and CIGAR (packed as in pbw_records, cigar_off n+1). */
int pbw_align_batch(pbw_handle* h, uint64_t n, const uint8_t* reads, const uint8_t* quals,
                    const uint64_t* read_off, const uint8_t* refs, const uint64_t* ref_off,
                    const int64_t* hint, const uint64_t* band, int32_t* score, uint64_t* offset,
                    uint32_t* cigar_off, uint32_t* cigar, uint64_t cigar_cap);

/* find_seed_hits (src/mapper/seeds.rs:91-151) for a batch of reads: per read
 * the hit count and, in emission order, hits packed as
 * (strand << 63) | (contig << 40) | ref_pos with read_pos in hit_read_pos;
 * repeat_prob per 15-mer window (n_windows = len - 14). hit_off (n+1) and
 * win_off (n+1) are computed by the call. Reads with more hits than the
 * per-read buffer (4096) are seeded again into the overflow pool as in a map
 * call, so every read's list is complete; PBW_ERR_CAPACITY when hit_cap or
 * win_cap is too small. */
int pbw_seed_batch(pbw_handle* h, const pbw_reads* reads, uint64_t* hit_off, uint64_t* hits,
                   uint32_t* hit_read_pos, uint64_t hit_cap, uint64_t* win_off, double* repeat_prob,
                   uint64_t win_cap);

/* cluster_hits (src/mapper/candidates.rs:30-78) after seeding: per read the
 * first max_per_read candidates in final order (contig, 0-based position,
 * strand, score) and the full candidate count. Row i of the candidate
 * arrays starts at i * max_per_read (1 <= max_per_read <= 256); its first
 * n_cand[i] entries are set.
 * Over-capacity reads are clustered from the overflow pool as in a map call. */
int pbw_cluster_batch(pbw_handle* h, const pbw_reads* reads, uint32_t max_per_read, uint32_t* n_cand,
                      uint32_t* total_cand, uint32_t* cand_contig, uint64_t* cand_pos, uint8_t* cand_strand,
                      double* cand_score);

/* MapqCalculator::select_best + finalize_mapq (src/mapq/bayesian.rs:193-201,
 * 251-282) for a batch of n = reads->n reads. Per read i: the candidates'
 * log-likelihoods lks[lk_off[i] .. lk_off[i+1]) (at least one); the repeat
 * mask of find_seed_hits, one probability per 15-mer window,
 * repeat[win_off[i] .. win_off[i+1]); and the winning alignment: rev[i]
 * (query = the read's reverse complement), the reference window passed to
 * finalize_mapq refs[ref_off[i] .. ref_off[i+1]) (it starts at the
 * alignment's first reference base) and its CIGAR cigar[cigar_off[i] ..
 * cigar_off[i+1]) packed as in pbw_records. Outputs: mapq, posterior, the
 * winner's index among the read's candidates (the last maximum) and sum_exp
 * (the softmax denominator). Host buffers in and out. Reference windows
 * of more than 1280 ACGT bases take their GC terms from the device libm. */
int pbw_mapq_batch(pbw_handle* h, const pbw_reads* reads, const uint64_t* lk_off, const double* lks,
                   const uint64_t* win_off, const double* repeat, const uint8_t* rev, const uint64_t* ref_off,
                   const uint8_t* refs, const uint32_t* cigar_off, const uint32_t* cigar, uint8_t* mapq,
                   double* posterior, uint32_t* best, double* sum_exp);

/* Output sizes for a map call on these reads: the number of records (one per
 * read) and a CIGAR capacity that always suffices (pbw_records.cigar_cap). */
int pbw_records_reserve(const pbw_reads* reads, uint64_t* n_records, uint64_t* cigar_cap);

/* Timing and counters of the last map call on this handle. */
int pbw_last_stats(const pbw_handle* h, pbw_stats* st);

/* Device-resident variant of pbw_map_single for throughput measurement:
 * bases/quals/offsets are device pointers; records are written to host
 * arrays as in pbw_map_single but no host-to-device input copy happens. */
int pbw_map_single_device(pbw_handle* h, const pbw_reads* dev_reads, pbw_records* out);

/* SAM text (src/io/sam.rs:69-108, format_sam :37-58) for records produced by
 * a map call: header (@HD, @SQ per contig, @PG with command_line) then one
 * line per record. read_ids[i] is the QNAME. Writes to path. Same as
 * pbw_sam_write with one source, no read group, unsorted. */
int pbw_write_sam(pbw_handle* h, const char* path, const char* command_line, const pbw_reads* reads,
                  const char* const* read_ids, const pbw_records* recs);

/* Header settings of a SAM stream (format_sam_records_sorted, sam.rs:83-108). */
typedef struct {
  const char* command_line;  /* @PG CL: (main.rs:154, argv joined by ' ') */
  const char* read_group;    /* --readgroup "ID:id,TAG:value,..." (ReadGroup::parse,
                                sam.rs:17-32) or NULL: adds the @RG line and an
                                RG:Z:<id> tag on every record */
  int32_t coordinate_sorted; /* @HD SO:coordinate instead of SO:unsorted */
} pbw_sam_options;

/* Records of one map call with the reads they came from. */
typedef struct {
  const pbw_reads* reads;       /* SEQ / QUAL: the input reads, one per record */
  const char* const* read_ids;  /* QNAME per record */
  const pbw_records* recs;
} pbw_sam_source;

/* Selected records as SAM text, formatted on the device. n_src is 1 (single-
 * end) or 2 (pairs: source 0 = mate 1, source 1 = mate 2, the output order of
 * map_paired, lib.rs:171-181). Records are numbered r * n_src + s (record r of
 * source s): sel lists the records to write, in output order (the records
 * kept by --labelfilter, main.rs:158-160, or a pbw_sort_coordinate order);
 * sel == NULL writes every record in number order. pbw_sam_write writes the
 * stream to path ("-" = standard output). pbw_sam_format puts it in out
 * (capacity cap bytes) and sets *len to its length; with out == NULL it only
 * sets *len. Errors: PBW_ERR_ARG (bad read-group spec, mismatched sources,
 * a selection entry naming no record), PBW_ERR_CAPACITY (cap < *len),
 * PBW_ERR_IO. */
int pbw_sam_write(pbw_handle* h, const pbw_sam_options* opt, uint32_t n_src, const pbw_sam_source* src,
                  const uint64_t* sel, uint64_t n_sel, const char* path);
int pbw_sam_format(pbw_handle* h, const pbw_sam_options* opt, uint32_t n_src, const pbw_sam_source* src,
                   const uint64_t* sel, uint64_t n_sel, char* out, uint64_t cap, uint64_t* len);

/* The same stream as BAM (write_bam / write_bam_indexed, src/io/bam.rs:19-57):
 * the SAM text formatted on the device is parsed back record by record (QUAL
 * characters read as Phred+33, so raw score bytes outside '!'..'~' are an
 * error, as for a strict SAM parser), encoded as BAM records and written as
 * BGZF blocks compressed on the host threads (zlib, opened at run time as
 * libz.so.1). With write_index (which needs opt->coordinate_sorted and
 * records in coordinate order, see pbw_sort_coordinate) a BAI goes to
 * path + ".bai". Errors as pbw_sam_write, and PBW_ERR_FORMAT for a record
 * that does not parse. */
int pbw_bam_write(pbw_handle* h, const pbw_sam_options* opt, uint32_t n_src, const pbw_sam_source* src,
                  const uint64_t* sel, uint64_t n_sel, const char* path, int32_t write_index);

/* write_bam / write_bam_indexed (src/io/bam.rs:19-57) on SAM text as the
 * reference calls them: the len bytes of sam (a header, then one record per
 * line) are encoded as by pbw_bam_write, with the reference dictionary taken
 * from the header's @SQ lines (SN, LN) as a SAM parser builds it. Host code;
 * no handle or device. write_index needs @HD SO:coordinate and records in
 * that order. Errors (pbw_last_error(NULL)): PBW_ERR_FORMAT (an @SQ line
 * without SN or LN, a record that does not parse, an RNAME not in the
 * dictionary), PBW_ERR_ARG, PBW_ERR_IO. */
int pbw_bam_write_text(const char* sam, uint64_t len, const char* path, int32_t write_index);

/* Coordinate order of the selected records (sort_for_coordinate_order,
 * sam.rs:114-124): stable sort by (index of the contig's name, the last
 * index when names repeat; position), unmapped records (pos 0) last, on the
 * device. sel / n_sel / numbering as pbw_sam_write (sel must not be NULL when
 * n_sel > 0); sorted[n_sel] receives the record numbers in order. Only
 * recs->contig and recs->pos of the sources are read. */
int pbw_sort_coordinate(pbw_handle* h, uint32_t n_src, const pbw_sam_source* src, const uint64_t* sel,
                        uint64_t n_sel, uint64_t* sorted);

/* Reads from a file: replaces read_reads_files_with_preprocessing
 * (src/io/fastx.rs:19-48) for one path -- read_fastq (:133-147) or
 * read_fasta_as_reads (:161-174), then strip_mate_suffix (:77-81) and, when
 * adapter is not NULL, strip_adapter (:97-117). quality_offset is 33 or 64
 * (--phred64). pbw_reads_get gives the reads as pbw_reads (the quality track
 * has the sequence's length: missing scores are 30); pbw_reads_id the i-th
 * read ID (NUL-terminated, valid until pbw_reads_free). The IDs are stored
 * back to back: ID i + 1 starts right after the NUL that ends ID i. A path ending in
 * ".gz" is gunzipped first (open_maybe_gz, :120-129; zlib is opened at run
 * time as libz.so.1). Errors: PBW_ERR_IO (cannot open, corrupt gzip) and
 * PBW_ERR_FORMAT (text that is not UTF-8); pbw_last_error(NULL) names the
 * file. */
typedef struct pbw_read_set pbw_read_set;
int pbw_reads_load(const char* path, int fasta, uint8_t quality_offset, const char* adapter, pbw_read_set** out);
int pbw_reads_get(const pbw_read_set* rs, pbw_reads* view);
const char* pbw_reads_id(const pbw_read_set* rs, uint64_t i);
void pbw_reads_free(pbw_read_set* rs);

/* build-genome (GenomeIndexBuilder, src/index/genome.rs:98-148): the FASTA
 * files (gunzipped when a name ends in ".gz") into out_prefix.stidx, one contig
 * per record, in file order. Host code; no device is used. Errors:
 * PBW_ERR_IO, PBW_ERR_FORMAT (text that is not UTF-8), described by
 * pbw_last_error(NULL). */
int pbw_build_genome(const char* out_prefix, const char* species, const char* assembly, uint32_t n_files,
                     const char* const* fasta_paths);

/* build-hash (HashTableBuilder::build + save, src/index/hashtable.rs:81-87,
 * 248-322) on the given CUDA device: the occurrence table of
 * genome_prefix.stidx written to out_prefix.sthash -- forward and reverse-
 * complement windows every stride bases, windows with a non-ACGT base
 * skipped, the first max_count occurrences of each hash in scan order, groups
 * in ascending hash order. The reference's defaults are k 15, stride 5,
 * max_count 300. Limits: 1 <= k <= 32, fewer than 2^32 windows
 * (PBW_ERR_LIMIT). Errors are described by pbw_last_error(NULL). */
int pbw_build_hash(const char* genome_prefix, const char* out_prefix, uint64_t k, uint64_t stride,
                   uint64_t max_count, int32_t device);

/* Batching settings of a handle (no counterpart in the reference).
 * autotune: the seeded band DP exists with 8 lanes per alignment (8 band
 *   columns each at the default band of 30), 16 lanes (4 each) and, for
 *   bands of 16 to 31, 4 lanes (16 each); with autotune the first chunk of
 *   each read-length class (<= 128, <= 256, longer bases) runs every form on
 *   the same alignments and the fastest is kept for the class (the results
 *   are the same either way). band_lanes 4, 8 or 16 forces a form (4 runs
 *   as 8 for bands without a 4-lane form); 0 leaves it to the tuner (8
 *   without it).
 * length_bins: in a chunk whose reads differ in length, the seeded DP's work
 *   queue is ordered by 16-base length bins, longest first.
 * pair_graphs: each batch of pairs (decide, cross-alignment DP, statistics,
 *   resolve, observation copy) is one CUDA graph launch, captured once per
 *   chunk of pairs.
 * chosen_lanes / tuned_ms are outputs of pbw_get_tuning: the form chosen
 * per read-length class (0 = not tuned yet) and the timings (8 lanes, 16
 * lanes, 4 lanes, ms; 0 = not run) that chose it. All settings are on by
 * default.
 * wait_polls: the whole-window DP's warps wait for the warp to their left
 *   with a bounded spin; after this many polls (0 = the default, 2^22) the
 *   wait gives up, the call discards its results and returns PBW_ERR_DEVICE.
 *   Lowering it only serves to exercise that path.
 * ovf_slice_hits: reads with more seed hits than the per-read buffer holds
 *   (4096, or 16384 when the longest read of the call exceeds 160 bases) are
 *   seeded again into an overflow pool one slice of this many hits at a time
 *   (0 = the default, 16 M; larger values are clamped to it). The pool and its
 *   clustering scratch hold two slices, so a smaller slice also takes less
 *   device memory. A chunk's over-capacity reads may hold 16 default slices in
 *   all, and one read one slice.
 * k2_threads: K2 (clustering) runs each read as one block; for the two
 *   largest hit-count tiers the autotuner times blocks of 1024, 512 and 256
 *   threads on the handle's first chunk (same results; smaller blocks put
 *   more reads in flight per SM) and keeps the fastest per tier.
 * pbw_set_tuning reads the inputs and clears the tuned choices. */
typedef struct {
  int32_t autotune;
  int32_t band_lanes;
  int32_t length_bins;
  int32_t pair_graphs;
  int32_t chosen_lanes[3];
  float tuned_ms[3][3];
  uint32_t wait_polls;
  uint32_t ovf_slice_hits;
  int32_t k2_threads[2];      /* K2 block size for the 2049-4096-hit tier and the 4097-16384-hit tier
                                 (tables in global slabs): 0 = tuned (or 1024), else 256, 512 or 1024 */
  int32_t k2_chosen[2];       /* (read) the tuned block sizes, 0 = not tuned yet */
  float k2_tuned_ms[2][3];    /* (read) the tuning trial's times for 1024, 512 and 256 threads */
} pbw_tuning;
int pbw_get_tuning(const pbw_handle* h, pbw_tuning* t);
int pbw_set_tuning(pbw_handle* h, const pbw_tuning* t);

/* Learned candidate ranker (no counterpart in the reference): a small MLP
 * (12 seed features -> 64 -> 64 -> 1, BF16 weights, FP32 accumulation on the
 * tensor cores) that scores each of a read's candidates before the seeded
 * DP and prunes the ones it expects neither to win nor to enter the MAPQ
 * posterior. Reads whose best score is below the threshold, or whose hits
 * overflowed the per-read buffer, keep every candidate.
 *
 * pbw_ranker_train maps r1 (and r2 as mates, or NULL) once with the plain
 * path, labels every aligned candidate (the read's select_best winner, or
 * lk - lk_max >= label_cut), trains the model on the GPU and sets the keep
 * threshold so that `recall` of the positive training candidates is kept.
 * pbw_ranker_enable switches pruning on or off for later map calls on the
 * handle (and clears the counters); pbw_ranker_counters returns candidates
 * kept and pruned and reads kept whole since then. pbw_ranker_export /
 * pbw_ranker_import move a trained model (2*12 normalisation values, 5057
 * weights, the threshold) between handles. */
typedef struct {
  uint32_t epochs;          /* passes over the training candidates (3) */
  uint32_t batch;           /* candidates per Adam step (8192) */
  double lr;                /* Adam learning rate (2e-3) */
  double recall;            /* fraction of positive training candidates kept (0.9995) */
  double positive_weight;   /* extra loss weight of positives over class balance (4) */
  uint64_t seed;            /* weight initialisation */
  double label_cut;         /* a candidate is positive when lk - lk_max >= label_cut (-60 ln 2: pruning
                               cannot change sum_exp; looser, e.g. ln 1e-12, prunes more) */
} pbw_ranker_train_options;

typedef struct {
  uint64_t samples;         /* aligned training candidates */
  uint64_t positives;
  double loss_first, loss_last;  /* mean weighted loss, first and last epoch */
  double tau;               /* logit threshold */
  double train_recall;      /* positives kept on the training candidates */
  double train_prune;       /* negatives pruned on the training candidates */
  double ms_collect, ms_train;
} pbw_ranker_report;

void pbw_ranker_default_options(pbw_ranker_train_options* o);
int pbw_ranker_train(pbw_handle* h, const pbw_reads* r1, const pbw_reads* r2, const pbw_ranker_train_options* opt,
                     pbw_ranker_report* rep);
int pbw_ranker_enable(pbw_handle* h, int32_t on);
int pbw_ranker_counters(pbw_handle* h, uint64_t* kept, uint64_t* pruned, uint64_t* reads_whole);
int pbw_ranker_export(const pbw_handle* h, float* out, uint64_t cap, uint64_t* n);
/* The trained model's logits for n caller feature rows (12 floats each, the
 * layout above), on the tensor-core inference kernel: the stage entry point
 * of the ranker. */
int pbw_ranker_score(pbw_handle* h, const float* feat, uint64_t n, float* logit);
int pbw_ranker_import(pbw_handle* h, const float* in, uint64_t n);

/* Allocation-free window alignment. No counterpart in the reference: it exists
 * for callers that must not call cudaMalloc -- a host application whose own
 * allocator has reserved the GPU's memory (a framework's caching allocator, a
 * pool sized at start-up) or a loop with a fixed device-memory budget. It
 * performs the same alignment as pbw_align_batch
 * (SmithWatermanAligner::align) on the wide-band DP kernel and needs no
 * handle.
 *
 * Every pointer is DEVICE memory owned by the caller: n problems with reads /
 * quals concatenated at read_off (n+1), reference windows concatenated at
 * ref_off (n+1), hint[n], band[n]; outputs score[n], offset[n] (start of the
 * alignment in its window), n_ops[n] and cigar[n * cigar_stride] ((len << 4) |
 * op, op 0=M 1=I 2=D 4=S), the i-th CIGAR at cigar + i * cigar_stride.
 * stream is a cudaStream_t (NULL = legacy default stream); the call
 * synchronises that stream: it returns after the stream has finished its work.
 *
 * Limits: n <= 4096 problems per call, reads <= 256 bases, windows <= 2048
 * bases; beyond them PBW_ERR_LIMIT (a read or window over its limit is
 * detected on the device, the others are still aligned), and a CIGAR longer
 * than cigar_stride gives PBW_ERR_CAPACITY; pbw_last_error(NULL) describes
 * the failure. CIGARs longer than 12 operations share a static pool sized for
 * the worst case (2 x 256 + 1 operations for each of 4096 problems).
 *
 * Scratch: a file-scope device array of about 14 MB, held on every GPU that
 * loads the library until the process exits. The first call on a device (with
 * that device current) looks up the array's device address and writes its
 * parameter table with a synchronous copy; that first call should come before
 * any stream capture. Every call reuses the same array and clears its
 * counters first, so calls that overlap on the GPU (two streams, two host
 * threads) race and must be serialised by the caller. */
int pbw_align_noalloc(uint64_t n, const uint8_t* reads, const uint8_t* quals, const uint64_t* read_off,
                      const uint8_t* refs, const uint64_t* ref_off, const int64_t* hint, const uint64_t* band,
                      uint32_t gap_open_phred, uint32_t gap_extend_phred, int32_t* score, uint64_t* offset,
                      uint32_t* n_ops, uint32_t* cigar, uint32_t cigar_stride, void* stream);

/* Measured integer throughput of a device (no counterpart in the reference):
 * G operations/s of add.s32 and of max.s32 over independent dependency
 * chains on every SM, timed with CUDA events. The banded DP is a max-plus
 * recurrence on 32-bit integers; these are its roofline denominators. */
int pbw_int32_peak(int32_t device, double* add_gops, double* max_gops);

#ifdef __cplusplus
}
#endif

#endif /* PROBEBWA_GPU_H */
