// api.cu -- the C ABI (include/probebwa_gpu.h): index loading, host-side
// parameter tables, and the device pipeline of one map call.
//
// Pipeline of pbw_map_single (per chunk of reads, all on the handle's stream):
//   K1 k_seed            seed hits + repeat codes            (seed.cu)
//   K2 k_cluster x2      candidates (small / large hit sets)  (cluster.cu)
//      k_make_jobs       candidate windows -> work queue       (mapq.cu)
//   K3 k_align_band      banded DP + traceback + likelihood    (align_band.cu)
//   K4 k_finalize        select_best + MAPQ -> records         (mapq.cu)
//      scan + gather     packed CIGARs                         (mapq.cu)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_common.cuh"
#include "pbw_host.h"
#include "pbw_kernels.h"
#include "pbw_pipeline.h"

using namespace pbw;

static thread_local std::string g_open_err;  // per thread: loaders may run concurrently

namespace pbw {
// Errors of calls without a handle (a failed pbw_open, handle-free entry
// points), read through pbw_last_error(NULL).
void set_handleless_error(const std::string& s) { g_open_err = s; }
}  // namespace pbw

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
#define CK(call)                                                        \
  do {                                                                  \
    cudaError_t e_ = (call);                                            \
    if (e_ != cudaSuccess) {                                            \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);      \
      return PBW_ERR_CUDA;                                              \
    }                                                                   \
  } while (0)

template <class T>
static int dev_alloc(pbw_handle* h, DevBuf<T>& b, size_t n) {
  if (n <= b.cap) return PBW_OK;
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.cap = 0;
  size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)&b.p, bytes);
  if (e != cudaSuccess) {
    h->err = std::string("cudaMalloc(") + std::to_string(bytes) + "): " + cudaGetErrorString(e);
    return PBW_ERR_NOMEM;
  }
  b.cap = n;
  return PBW_OK;
}

#define TRY(x)             \
  do {                     \
    int rc_ = (x);         \
    if (rc_ != PBW_OK) return rc_; \
  } while (0)

// ---------------------------------------------------------------------------
// index files
// ---------------------------------------------------------------------------
struct FileReader {
  FILE* f = nullptr;
  explicit FileReader(const std::string& p) { f = fopen(p.c_str(), "rb"); }
  ~FileReader() { if (f) fclose(f); }
  bool read(void* dst, size_t n) { return n == 0 || fread(dst, 1, n, f) == n; }
  bool u64(uint64_t& v) { return read(&v, 8); }
  bool str(std::string& s) {
    uint64_t n;
    if (!u64(n) || n > (1ull << 32)) return false;
    s.resize(n);
    return read(&s[0], n);
  }
};

static double h_logadd(double a, double b) {
  if (a > b) std::swap(a, b);
  if (b >= a + 10.0) return a;
  if (b >= a + 4.0) return std::max(a - 1.0, 0.0);
  if (b >= a + 2.0) return std::max(a - 2.0, 0.0);
  return std::max(a - 3.0, 0.0);
}
static double h_py_int_round(double x) { return std::trunc(x + 0.5); }
static int32_t h_sat_i32(double x) {
  if (std::isnan(x)) return 0;
  if (x >= 2147483647.0) return INT32_MAX;
  if (x <= -2147483648.0) return INT32_MIN;
  return (int32_t)x;
}

static const double H_LN_10 = 2.302585092994045684017991454684364208;
static const double H_DB = -0.1 * H_LN_10;

// Host parameter tables: quality- and integer-indexed values computed once
// with the host libm (the same one the CPU reference path uses).
namespace pbw {
void fill_tables(const pbw_options& opt, uint64_t total_length, DevTables& T) {
  memset(&T, 0, sizeof(T));
  const double sub = opt.substitution_rate;
  T.subphred = h_py_int_round(std::log(std::max(sub, 1e-30)) / H_DB);  // bayesian.rs:104
  for (int q = 0; q < 256; q++) {
    double eq = h_logadd((double)q, T.subphred);
    double e = std::pow(10.0, -eq / 10.0);
    T.llk_match[q] = std::log(std::max(1.0 - e, 1e-300));
    T.llk_mismatch[q] = std::log(std::max(e / 3.0, 1e-300));
    double qi = std::min(std::pow(10.0, -eq / 10.0), 1.0 - 1e-12);
    T.ml_one_minus_q[q] = 1.0 - qi;
    T.ml_q_over[q] = qi / (1.0 - qi);
    T.nrp[q] = std::pow(10.0, -(double)q / 10.0);
    double scale = std::min(std::max((double)q / 30.0, 0.2), 1.0);
    T.mmpen[q] = h_sat_i32(std::round(-30.0 * scale));
  }
  for (int p = 0; p < 100; p++) T.pow_neg_tenth[p] = std::pow(10.0, -(double)p / 10.0);
  T.ln_quarter = std::log(0.25);
  T.ln_two_g = std::log(2.0 * (double)std::max<uint64_t>(total_length, 1));
  T.ln30 = std::log(30.0);
  T.floor_wrong = std::exp(99.0 * H_DB);
  T.ln_floor_wrong = std::log(T.floor_wrong);
  T.log10_099 = std::log10(0.99);
  T.log10_1e30 = std::log10(1e-30);
  T.sv_prior_log_prob = -opt.sv_prior_phred / 10.0 * H_LN_10;
  gap_costs(opt.gap_open_phred, opt.gap_extend_phred, T.gap_open, T.gap_extend);
  T.ln_n_max = 4096;
  T.gc_tmax = 1280;
}

// SmithWatermanAligner::new (smith_waterman.rs:113-130): gap costs scaled
// from the -90 / -1 baseline at --gapopen 40 / --gapextend 3, at most -1.
void gap_costs(uint32_t gop, uint32_t gep, int32_t& go, int32_t& ge) {
  go = std::min(h_sat_i32(std::round(-90.0 * (double)gop / 40.0)), -1);
  ge = std::min(h_sat_i32(std::round(-1.0 * (double)gep / 3.0)), -1);
}
}  // namespace pbw

static int build_tables(pbw_handle* h) {
  DevTables T;
  fill_tables(h->opt, h->total_length, T);
  const int LNMAX = T.ln_n_max;
  const int TMAX = T.gc_tmax;
  h->tab_host = T;
  TRY(dev_alloc(h, h->d_tab, 1));
  CK(cudaMemcpy(h->d_tab.p, &T, sizeof(T), cudaMemcpyHostToDevice));
  std::vector<double> ln_n(LNMAX);
  for (int k = 0; k < LNMAX; k++) ln_n[k] = std::log((double)k);
  TRY(dev_alloc(h, h->d_ln_n, LNMAX));
  CK(cudaMemcpy(h->d_ln_n.p, ln_n.data(), LNMAX * sizeof(double), cudaMemcpyHostToDevice));
  size_t ng = (size_t)(TMAX + 1) * (TMAX + 2) / 2;
  std::vector<double> lnb(ng), lnbm1(ng);
  for (int tot = 0; tot <= TMAX; tot++) {
    for (int gc = 0; gc <= tot; gc++) {
      // gc_content + effective_alphabet_size (bayesian.rs:445-466)
      double f = tot == 0 ? 0.5 : (double)gc / (double)tot;
      f = std::min(std::max(f, 1e-6), 1.0 - 1e-6);
      double b = std::exp(-f * std::log(f / 2.0) - (1.0 - f) * std::log((1.0 - f) / 2.0));
      size_t idx = (size_t)tot * (tot + 1) / 2 + gc;
      lnb[idx] = std::log(b);
      lnbm1[idx] = std::log(std::max(b - 1.0, 1e-6));
    }
  }
  TRY(dev_alloc(h, h->d_gc_lnb, ng));
  TRY(dev_alloc(h, h->d_gc_lnbm1, ng));
  CK(cudaMemcpy(h->d_gc_lnb.p, lnb.data(), ng * sizeof(double), cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_gc_lnbm1.p, lnbm1.data(), ng * sizeof(double), cudaMemcpyHostToDevice));
  return PBW_OK;
}

// GenomeIndex::load (src/index/genome.rs:80-86) into the device layout.
int load_genome(pbw_handle* h, const std::string& prefix) {
  FileReader fr(prefix + ".stidx");
  if (!fr.f) { h->err = "cannot open " + prefix + ".stidx"; return PBW_ERR_IO; }
  uint64_t nc;
  if (!fr.str(h->species) || !fr.str(h->assembly) || !fr.u64(nc)) { h->err = "stidx: truncated header"; return PBW_ERR_FORMAT; }
  if (nc >= (1ull << 23)) { h->err = "stidx: too many contigs for 23-bit packing"; return PBW_ERR_LIMIT; }
  std::vector<uint64_t> words;
  std::vector<uint32_t> nmask;
  std::vector<unsigned long long> cbase, clen;
  uint64_t gbase = 0;
  for (uint64_t c = 0; c < nc; c++) {
    std::string name;
    uint64_t npk;
    if (!fr.str(name) || !fr.u64(npk)) { h->err = "stidx: truncated contig"; return PBW_ERR_FORMAT; }
    std::vector<uint8_t> packed(npk);
    if (!fr.read(packed.data(), npk)) { h->err = "stidx: truncated packed sequence"; return PBW_ERR_FORMAT; }
    uint64_t nr;
    if (!fr.u64(nr)) { h->err = "stidx: truncated n_runs"; return PBW_ERR_FORMAT; }
    std::vector<uint32_t> runs(2 * nr);
    if (!fr.read(runs.data(), 8 * nr)) { h->err = "stidx: truncated n_runs"; return PBW_ERR_FORMAT; }
    uint64_t len;
    if (!fr.u64(len)) { h->err = "stidx: truncated length"; return PBW_ERR_FORMAT; }
    if (len >= (1ull << 39)) { h->err = "stidx: contig longer than 2^39"; return PBW_ERR_LIMIT; }
    if (npk < (len + 3) / 4) { h->err = "stidx: packed sequence shorter than length"; return PBW_ERR_FORMAT; }
    const uint64_t nw = (len + 31) / 32;
    words.resize(gbase / 32 + nw, 0);
    nmask.resize(gbase / 32 + nw, 0);
    if (nw) memcpy(&words[gbase / 32], packed.data(), std::min<uint64_t>(npk, nw * 8));
    // bytes past the length may carry bits: they are never read
    for (uint64_t k = 0; k < nr; k++) {
      uint64_t s = std::min<uint64_t>(runs[2 * k], len), e = std::min<uint64_t>(runs[2 * k + 1], len);
      for (uint64_t p = s; p < e;) {
        uint64_t g = gbase + p;
        if ((g & 31) == 0 && p + 32 <= e) {
          nmask[g >> 5] = 0xFFFFFFFFu;
          p += 32;
        } else {
          nmask[g >> 5] |= 1u << (g & 31);
          p++;
        }
      }
    }
    h->names.push_back(name);
    h->lens.push_back(len);
    cbase.push_back(gbase);
    clen.push_back(len);
    gbase += nw * 32;
  }
  uint64_t total;
  if (!fr.u64(total)) { h->err = "stidx: truncated total_length"; return PBW_ERR_FORMAT; }
  h->total_length = total;
  std::map<std::string, int> first;
  std::vector<int> name_class;
  for (size_t i = 0; i < h->names.size(); i++) {
    auto it = first.find(h->names[i]);
    if (it == first.end()) { first[h->names[i]] = (int)i; name_class.push_back((int)i); }
    else name_class.push_back(it->second);
  }
  const size_t nwords = std::max<size_t>(words.size(), 1);
  words.resize(nwords, 0);
  nmask.resize(nwords, 0);
  // one bit per 1024-base block (32 mask words): whether the block holds an
  // N; ~380 KB for 3.1 Gbp, so it stays in L2 while the seeding kernel skips
  // the N-mask words of N-free blocks
  const size_t nblocks = (nwords + 31) / 32;
  std::vector<uint32_t> nblk((nblocks + 31) / 32, 0u);
  for (size_t b = 0; b < nblocks; b++) {
    uint32_t any = 0;
    const size_t e = std::min(nwords, (b + 1) * 32);
    for (size_t w = b * 32; w < e; w++) any |= nmask[w];
    if (any) nblk[b >> 5] |= 1u << (b & 31);
  }
  TRY(dev_alloc(h, h->d_bits, nwords));
  TRY(dev_alloc(h, h->d_nmask, nwords));
  TRY(dev_alloc(h, h->d_nblk, nblk.size()));
  CK(cudaMemcpy(h->d_nblk.p, nblk.data(), nblk.size() * 4, cudaMemcpyHostToDevice));
  TRY(dev_alloc(h, h->d_cbase, std::max<size_t>(nc, 1)));
  TRY(dev_alloc(h, h->d_clen, std::max<size_t>(nc, 1)));
  TRY(dev_alloc(h, h->d_name_class, std::max<size_t>(nc, 1)));
  CK(cudaMemcpy(h->d_bits.p, words.data(), nwords * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(h->d_nmask.p, nmask.data(), nwords * 4, cudaMemcpyHostToDevice));
  if (nc) {
    CK(cudaMemcpy(h->d_cbase.p, cbase.data(), nc * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->d_clen.p, clen.data(), nc * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->d_name_class.p, name_class.data(), nc * 4, cudaMemcpyHostToDevice));
  }
  h->G.bits = h->d_bits.p;
  h->G.nmask = h->d_nmask.p;
  h->G.nblk = h->d_nblk.p;
  h->G.cbase = h->d_cbase.p;
  h->G.clen = h->d_clen.p;
  h->G.name_class = h->d_name_class.p;
  h->G.ncontig = (unsigned int)nc;
  return PBW_OK;
}

// HashTable::load (src/index/hashtable.rs:73-79) streamed to the device,
// then the dense CSR is built there (index.cu).
static int load_hash(pbw_handle* h, const std::string& prefix) {
  FileReader fr(prefix + ".sthash");
  if (!fr.f) { h->err = "cannot open " + prefix + ".sthash"; return PBW_ERR_IO; }
  uint64_t n;
  if (!fr.u64(n)) { h->err = "sthash: truncated"; return PBW_ERR_FORMAT; }
  if (n > NKMER) { h->err = "sthash: more keys than 15-mers"; return PBW_ERR_FORMAT; }
  DevBuf<uint32_t> d_tab;
  DevBuf<unsigned long long> d_pos;
  TRY(dev_alloc(h, d_tab, std::max<uint64_t>(3 * n, 1)));
  // (key, offset, count) entries as they stream past: the sum of the counts
  // and the furthest bucket end
  uint64_t sum_cnt = 0, max_end = 0;
  auto tally = [&](const uint8_t* p, size_t c) {
    for (size_t o = 0; o + 12 <= c; o += 12) {
      uint32_t off, cnt;
      memcpy(&off, p + o + 4, 4);
      memcpy(&cnt, p + o + 8, 4);
      sum_cnt += cnt;
      max_end = std::max<uint64_t>(max_end, (uint64_t)off + cnt);
    }
  };
  // chunks hold whole 12-byte table entries and whole 8-byte positions
  const size_t CH = 48ull << 20;
  std::vector<uint8_t> buf(CH);
  auto stream_to = [&](void* dst, uint64_t bytes, bool table) -> bool {
    uint64_t done = 0;
    while (done < bytes) {
      size_t c = (size_t)std::min<uint64_t>(CH, bytes - done);
      if (!fr.read(buf.data(), c)) return false;
      if (table) tally(buf.data(), c);
      if (cudaMemcpy((char*)dst + done, buf.data(), c, cudaMemcpyHostToDevice) != cudaSuccess) return false;
      done += c;
    }
    return true;
  };
  if (!stream_to(d_tab.p, 12 * n, true)) { h->err = "sthash: truncated table"; return PBW_ERR_FORMAT; }
  uint64_t np;
  if (!fr.u64(np)) { h->err = "sthash: truncated positions"; return PBW_ERR_FORMAT; }
  if (np >= (1ull << 32)) { h->err = "sthash: more than 2^32 occurrences"; return PBW_ERR_LIMIT; }
  // every bucket inside the positions and the buckets no larger than them
  // together: the CSR fill below then reads and writes in bounds
  if (max_end > np || sum_cnt > np) { h->err = "sthash: table entries point beyond the positions"; return PBW_ERR_FORMAT; }
  TRY(dev_alloc(h, d_pos, std::max<uint64_t>(np, 1)));
  if (!stream_to(d_pos.p, 8 * np, false)) { h->err = "sthash: truncated positions"; return PBW_ERR_FORMAT; }
  uint64_t k, stride, total;
  if (!fr.u64(k) || !fr.u64(stride) || !fr.u64(total)) { h->err = "sthash: truncated trailer"; return PBW_ERR_FORMAT; }
  if (k != (uint64_t)KMER) { h->err = "sthash: k != 15 is not supported by the device path"; return PBW_ERR_LIMIT; }
  h->seed_k = k;
  h->n_ent = np;
  TRY(dev_alloc(h, h->d_csr, NKMER + 1));
  TRY(dev_alloc(h, h->d_ent, std::max<uint64_t>(np, 1)));
  TRY(dev_alloc(h, h->d_err, 4));
  // the table and positions went up by cudaMemcpy on the legacy stream,
  // which the handle's non-blocking stream does not wait for
  CK(cudaDeviceSynchronize());
  CK(cudaMemsetAsync(h->d_err.p, 0, 16, h->st));
  CK(cudaMemsetAsync(h->d_csr.p, 0, (NKMER + 1) * 4, h->st));
  launch_build_csr_counts(d_tab.p, n, np, h->d_csr.p, h->d_err.p, h->st);
  // keys outside the 15-mers, buckets past the positions and repeated keys
  // stop the load before the fill
  {
    CK(cudaStreamSynchronize(h->st));
    CK(cudaGetLastError());
    int err0 = 0;
    CK(cudaMemcpy(&err0, h->d_err.p, 4, cudaMemcpyDeviceToHost));
    if (err0) {
      h->err = "sthash: invalid table entry (code " + std::to_string(err0) + ")";
      return PBW_ERR_FORMAT;
    }
  }
  DevBuf<unsigned int> sums;
  TRY(dev_alloc(h, sums, scan_blocks(NKMER + 1) + 1));
  launch_scan_excl(h->d_csr.p, NKMER + 1, nullptr, sums.p, nullptr, nullptr, h->st);
  launch_build_csr_fill(d_tab.p, n, d_pos.p, np, h->d_csr.p, h->d_ent.p, h->d_clen.p, h->G.ncontig, h->d_err.p, h->st);
  CK(cudaStreamSynchronize(h->st));
  CK(cudaGetLastError());
  int err = 0;
  CK(cudaMemcpy(&err, h->d_err.p, 4, cudaMemcpyDeviceToHost));
  unsigned int last = 0;
  CK(cudaMemcpy(&last, h->d_csr.p + NKMER, 4, cudaMemcpyDeviceToHost));
  d_tab.release();
  d_pos.release();
  sums.release();
  if (err) {
    h->err = "sthash: invalid table entry (code " + std::to_string(err) + ")";
    return PBW_ERR_FORMAT;
  }
  (void)last;
  h->I.csr = h->d_csr.p;
  h->I.ent = h->d_ent.p;
  return PBW_OK;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void pbw_default_options(pbw_options* o) {
  o->substitution_rate = 0.001;
  o->insert_size_mean = 250.0;
  o->insert_size_sd = 60.0;
  o->max_indel_len = 30;
  o->gap_open_phred = 40;
  o->gap_extend_phred = 3;
  o->sv_prior_phred = 55.0;
  o->group_width = 16;
  o->device = 0;
  o->chunk_reads = 0;
}

int pbw_open(const char* genome_prefix, const char* hash_prefix, const pbw_options* opt, pbw_handle** out) {
  if (!genome_prefix || !out) { g_open_err = "null argument"; return PBW_ERR_ARG; }
  *out = nullptr;
  std::unique_ptr<pbw_handle> h(new pbw_handle());
  if (opt) h->opt = *opt;
  else pbw_default_options(&h->opt);
  if (h->opt.group_width != 8 && h->opt.group_width != 16) { g_open_err = "group_width must be 8 or 16"; return PBW_ERR_ARG; }
  if (h->opt.chunk_reads == 0) h->opt.chunk_reads = 131072;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { g_open_err = "no CUDA device"; return PBW_ERR_CUDA; }
  if (h->opt.device < 0 || h->opt.device >= ndev) { g_open_err = "bad device ordinal"; return PBW_ERR_ARG; }
  h->device = h->opt.device;
  if (cudaSetDevice(h->device) != cudaSuccess) { g_open_err = "cudaSetDevice failed"; return PBW_ERR_CUDA; }
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, h->device);
  h->num_sms = prop.multiProcessorCount;
  h->smem_optin = (size_t)prop.sharedMemPerBlockOptin;
  if (cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking) != cudaSuccess) { g_open_err = "stream"; return PBW_ERR_CUDA; }
  if (!pbw::device_epoch(h->device)) { g_open_err = "epoch event"; return PBW_ERR_CUDA; }
  int rc = load_genome(h.get(), genome_prefix);
  if (rc == PBW_OK) rc = load_hash(h.get(), hash_prefix ? hash_prefix : genome_prefix);
  if (rc == PBW_OK) rc = build_tables(h.get());
  if (rc == PBW_OK) rc = pipeline_init(h.get());
  // every upload above (legacy-stream copies from pageable memory may still
  // be in flight when cudaMemcpy returns) is complete before the handle's
  // stream runs a kernel on it
  if (rc == PBW_OK && cudaDeviceSynchronize() != cudaSuccess) {
    h->err = "cudaDeviceSynchronize failed after loading the index";
    rc = PBW_ERR_CUDA;
  }
  if (rc != PBW_OK) {
    g_open_err = h->err;
    return rc;
  }
  *out = h.release();
  return PBW_OK;
}

void pbw_close(pbw_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->st);
  delete h;
}

const char* pbw_last_error(const pbw_handle* h) { return h ? h->err.c_str() : g_open_err.c_str(); }

uint64_t pbw_num_contigs(const pbw_handle* h) { return h ? h->names.size() : 0; }
uint64_t pbw_total_length(const pbw_handle* h) { return h ? h->total_length : 0; }
const char* pbw_contig_name(const pbw_handle* h, uint64_t i) {
  return (h && i < h->names.size()) ? h->names[i].c_str() : nullptr;
}
uint64_t pbw_contig_length(const pbw_handle* h, uint64_t i) { return (h && i < h->lens.size()) ? h->lens[i] : 0; }

int pbw_get_tuning(const pbw_handle* h, pbw_tuning* t) {
  if (!h || !t) return PBW_ERR_ARG;
  const auto& T = h->tune;
  t->autotune = T.autotune;
  t->band_lanes = T.band_lanes;
  t->length_bins = T.length_bins;
  t->pair_graphs = T.pair_graphs;
  t->wait_polls = T.wait_polls;
  t->ovf_slice_hits = T.ovf_slice_hits;
  for (int c = 0; c < 3; c++) {
    t->chosen_lanes[c] = T.chosen[c];
    for (int j = 0; j < 3; j++) t->tuned_ms[c][j] = T.ms[c][j];
  }
  for (int i = 0; i < 2; i++) {
    t->k2_threads[i] = T.k2_threads[i];
    t->k2_chosen[i] = T.k2_chosen[i];
    for (int j = 0; j < 3; j++) t->k2_tuned_ms[i][j] = T.k2_ms[i][j];
  }
  return PBW_OK;
}

int pbw_set_tuning(pbw_handle* h, const pbw_tuning* t) {
  if (!h || !t) return PBW_ERR_ARG;
  if (t->band_lanes != 0 && t->band_lanes != 4 && t->band_lanes != 8 && t->band_lanes != 16) {
    h->err = "pbw_set_tuning: band_lanes must be 0, 4, 8 or 16";
    return PBW_ERR_ARG;
  }
  for (int i = 0; i < 2; i++) {
    const int k = t->k2_threads[i];
    if (k != 0 && k != 256 && k != 512 && k != 1024) {
      h->err = "pbw_set_tuning: k2_threads must be 0, 256, 512 or 1024";
      return PBW_ERR_ARG;
    }
  }
  auto& T = h->tune;
  T.autotune = t->autotune != 0;
  T.band_lanes = t->band_lanes;
  T.length_bins = t->length_bins != 0;
  T.pair_graphs = t->pair_graphs != 0;
  T.wait_polls = t->wait_polls;
  T.ovf_slice_hits = t->ovf_slice_hits;
  for (int c = 0; c < 3; c++) {
    T.chosen[c] = 0;
    T.ms[c][0] = T.ms[c][1] = T.ms[c][2] = 0.f;
  }
  for (int i = 0; i < 2; i++) {
    T.k2_threads[i] = t->k2_threads[i];
    T.k2_chosen[i] = 0;
    for (int j = 0; j < 3; j++) T.k2_ms[i][j] = 0.f;
  }
  return PBW_OK;
}

int pbw_last_stats(const pbw_handle* h, pbw_stats* st) {
  if (!h || !st) return PBW_ERR_ARG;
  *st = h->stats;
  return PBW_OK;
}

}  // extern "C"
