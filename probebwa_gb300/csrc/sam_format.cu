// sam_format.cu -- SAM text formatted on the device (src/io/sam.rs:37-143).
//
// The reference builds the whole SAM stream in one String on the host
// (main.rs:172-176, format_sam_records). Here the records, reads and IDs of
// a map call go to the device once; a length pass gives every selected
// record's line length (one warp per record), a u64 exclusive scan turns the
// lengths into byte offsets, and a write pass puts each line at its offset
// (one warp per record: lane 0 writes the numeric and name columns, the
// whole warp copies SEQ and QUAL with coalesced stores). Text comes back in
// chunks of records to a file or a caller buffer; the header (a few hundred
// bytes) is built on the host.
//
// Line format (format_sam, sam.rs:37-58): QNAME FLAG RNAME POS MAPQ CIGAR
// RNEXT PNEXT TLEN SEQ QUAL, tab-separated, then "\tRG:Z:<id>" when a read
// group is set, then '\n'. RNAME / RNEXT are contig names ('*' for none),
// CIGAR is '*' when it has no operations. SEQ is the read upper-cased, and
// for a mapped reverse-strand record (pos != 0 and FLAG 0x10) reverse-
// complemented (A<->T, C<->G, anything else N); QUAL is the raw Phred scores
// as bytes, reversed with SEQ. Both go through String::from_utf8_lossy: valid
// UTF-8 is copied, each maximal invalid subsequence becomes U+FFFD (EF BF BD).
// Lines whose bytes are all ASCII (the normal case) take the warp-parallel
// path; others are converted by lane 0.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_pipeline.h"

namespace pbw {

namespace {

struct SamSrcDev {
  const uint8_t* bases;
  const uint8_t* quals;
  const uint64_t* offs;
  const char* ids;
  const uint64_t* id_off;
  const uint16_t* flag;
  const int32_t* contig;
  const unsigned long long* pos;
  const uint8_t* mapq;
  const uint32_t* cig_off;
  const uint32_t* cigar;
  const int32_t* mate_contig;
  const unsigned long long* mate_pos;
  const long long* tlen;
};

struct SamArgs {
  SamSrcDev src[2];
  uint32_t n_src;
  const unsigned long long* sel;  // record r of source s is number r * n_src + s
  uint64_t n_sel;
  const char* names;
  const uint64_t* name_off;
  uint32_t n_names;
  const char* rg;  // read-group ID (rg_len 0: none)
  uint32_t rg_len;
  unsigned long long* len;  // line length per selected record, then its byte offset
};

constexpr int SAM_WARPS = 8;  // warps per block, one record per warp

__device__ __forceinline__ uint32_t ndig(unsigned long long v) {
  uint32_t d = 1;
  while (v >= 10) {
    v /= 10;
    d++;
  }
  return d;
}
__device__ __forceinline__ uint32_t ndig_signed(long long v) {
  return v < 0 ? 1 + ndig((unsigned long long)0 - (unsigned long long)v) : ndig((unsigned long long)v);
}
__device__ __forceinline__ char* put_u64(char* o, unsigned long long v) {
  const uint32_t d = ndig(v);
  for (uint32_t k = d; k-- > 0;) {
    o[k] = (char)('0' + (int)(v % 10));
    v /= 10;
  }
  return o + d;
}
__device__ __forceinline__ char* put_i64(char* o, long long v) {
  if (v < 0) {
    *o++ = '-';
    return put_u64(o, (unsigned long long)0 - (unsigned long long)v);
  }
  return put_u64(o, (unsigned long long)v);
}
__device__ __forceinline__ uint8_t up(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }
__device__ __forceinline__ uint8_t compl_base(uint8_t b) {
  return b == 'A' ? 'T' : b == 'T' ? 'A' : b == 'C' ? 'G' : b == 'G' ? 'C' : 'N';
}

// Byte k of the SEQ or QUAL column before the UTF-8 step.
struct Column {
  const uint8_t* p;
  uint32_t n;
  bool rev;   // reversed (reverse-strand mapped record)
  bool seq;   // SEQ: upper-cased, complemented when reversed
  __device__ __forceinline__ uint8_t at(uint32_t k) const {
    const uint8_t b = p[rev ? n - 1 - k : k];
    if (!seq) return b;
    return rev ? compl_base(up(b)) : up(b);
  }
};

// String::from_utf8_lossy over a column: returns the output length and, with
// out != nullptr, writes the bytes.
__device__ uint32_t lossy(const Column& c, char* out) {
  uint32_t i = 0, o = 0;
  while (i < c.n) {
    const uint8_t b = c.at(i);
    if (b < 0x80) {
      if (out) out[o] = (char)b;
      o++;
      i++;
      continue;
    }
    uint32_t need = 0;
    uint8_t lo = 0x80, hi = 0xBF;
    if (b >= 0xC2 && b <= 0xDF) need = 1;
    else if (b == 0xE0) { need = 2; lo = 0xA0; }
    else if ((b >= 0xE1 && b <= 0xEC) || b == 0xEE || b == 0xEF) need = 2;
    else if (b == 0xED) { need = 2; hi = 0x9F; }
    else if (b == 0xF0) { need = 3; lo = 0x90; }
    else if (b >= 0xF1 && b <= 0xF3) need = 3;
    else if (b == 0xF4) { need = 3; hi = 0x8F; }
    uint32_t j = 1;
    bool ok = need > 0;
    if (ok) {
      for (; j <= need; j++) {
        if (i + j >= c.n) { ok = false; break; }
        const uint8_t cc = c.at(i + j);
        if (cc < (j == 1 ? lo : 0x80) || cc > (j == 1 ? hi : 0xBF)) { ok = false; break; }
      }
    }
    if (ok) {
      if (out)
        for (uint32_t t = 0; t <= need; t++) out[o + t] = (char)c.at(i + t);
      o += need + 1;
      i += need + 1;
    } else {
      if (out) { out[o] = (char)0xEF; out[o + 1] = (char)0xBF; out[o + 2] = (char)0xBD; }
      o += 3;
      i += need > 0 ? j : 1;
    }
  }
  return o;
}

// Whether a column holds any byte >= 0x80 (warp-wide answer).
__device__ __forceinline__ bool warp_non_ascii(const Column& c, int lane) {
  bool any = false;
  for (uint32_t k = lane; k < c.n; k += 32) any |= c.at(k) >= 0x80;
  return __any_sync(0xffffffffu, any);
}

struct RecView {
  const SamSrcDev* s;
  uint64_t r;
  uint64_t q0;
  uint32_t m;
  bool rev;
};

__device__ __forceinline__ RecView rec_view(const SamArgs& a, uint64_t i) {
  const unsigned long long g = a.sel[i];
  RecView v;
  v.s = &a.src[g % a.n_src];
  v.r = g / a.n_src;
  v.q0 = v.s->offs[v.r];
  v.m = (uint32_t)(v.s->offs[v.r + 1] - v.q0);
  v.rev = v.s->pos[v.r] != 0 && (v.s->flag[v.r] & 0x10);
  return v;
}

__device__ __forceinline__ uint32_t name_len(const SamArgs& a, int32_t c) {
  return (c >= 0 && (uint32_t)c < a.n_names) ? (uint32_t)(a.name_off[c + 1] - a.name_off[c]) : 1u;
}
__device__ __forceinline__ char* put_name(const SamArgs& a, char* o, int32_t c) {
  if (c >= 0 && (uint32_t)c < a.n_names) {
    for (uint64_t k = a.name_off[c]; k < a.name_off[c + 1]; k++) *o++ = a.names[k];
  } else {
    *o++ = '*';
  }
  return o;
}

// The line up to and including the tab before SEQ: its length, or (with out)
// its bytes.
__device__ uint32_t head(const SamArgs& a, const RecView& v, char* out) {
  const SamSrcDev& s = *v.s;
  const uint64_t r = v.r;
  const uint64_t i0 = s.id_off[r], i1 = s.id_off[r + 1];
  const uint32_t c0 = s.cig_off[r], c1 = s.cig_off[r + 1];
  if (!out) {
    uint32_t L = (uint32_t)(i1 - i0) + 1;
    L += ndig(s.flag[r]) + 1;
    L += name_len(a, s.contig[r]) + 1;
    L += ndig(s.pos[r]) + 1;
    L += ndig(s.mapq[r]) + 1;
    if (c1 == c0) L += 1;
    for (uint32_t k = c0; k < c1; k++) L += ndig(s.cigar[k] >> 4) + 1;
    L += 1;
    L += name_len(a, s.mate_contig[r]) + 1;
    L += ndig(s.mate_pos[r]) + 1;
    L += ndig_signed(s.tlen[r]) + 1;
    return L;
  }
  char* o = out;
  for (uint64_t k = i0; k < i1; k++) *o++ = s.ids[k];
  *o++ = '\t';
  o = put_u64(o, s.flag[r]);
  *o++ = '\t';
  o = put_name(a, o, s.contig[r]);
  *o++ = '\t';
  o = put_u64(o, s.pos[r]);
  *o++ = '\t';
  o = put_u64(o, s.mapq[r]);
  *o++ = '\t';
  if (c1 == c0) *o++ = '*';
  for (uint32_t k = c0; k < c1; k++) {
    const uint32_t w = s.cigar[k];
    o = put_u64(o, w >> 4);
    const uint32_t op = w & 15u;
    *o++ = op == 0 ? 'M' : op == 1 ? 'I' : op == 2 ? 'D' : op == 4 ? 'S' : op == 5 ? 'H' : 'X';
  }
  *o++ = '\t';
  o = put_name(a, o, s.mate_contig[r]);
  *o++ = '\t';
  o = put_u64(o, s.mate_pos[r]);
  *o++ = '\t';
  o = put_i64(o, s.tlen[r]);
  *o++ = '\t';
  return (uint32_t)(o - out);
}

__global__ void __launch_bounds__(SAM_WARPS * 32) k_sam_len(SamArgs a) {
  const int lane = threadIdx.x & 31;
  const uint64_t i = (uint64_t)blockIdx.x * SAM_WARPS + (threadIdx.x >> 5);
  if (i >= a.n_sel) return;
  const RecView v = rec_view(a, i);
  const Column cs{v.s->bases + v.q0, v.m, v.rev, true};
  const Column cq{v.s->quals + v.q0, v.m, v.rev, false};
  const bool wide_s = warp_non_ascii(cs, lane);
  const bool wide_q = warp_non_ascii(cq, lane);
  if (lane != 0) return;
  unsigned long long L = head(a, v, nullptr);
  L += (wide_s ? lossy(cs, nullptr) : v.m) + 1;
  L += wide_q ? lossy(cq, nullptr) : v.m;
  L += a.rg_len ? 6 + a.rg_len : 0;
  L += 1;
  a.len[i] = L;
}

// Writes the lines of selected records [i0, i1) into text, which starts at
// byte offset base of the stream.
__global__ void __launch_bounds__(SAM_WARPS * 32) k_sam_write(SamArgs a, uint64_t i0, uint64_t i1,
                                                              unsigned long long base, char* text) {
  const int lane = threadIdx.x & 31;
  const uint64_t i = i0 + (uint64_t)blockIdx.x * SAM_WARPS + (threadIdx.x >> 5);
  if (i >= i1) return;
  const RecView v = rec_view(a, i);
  const Column cs{v.s->bases + v.q0, v.m, v.rev, true};
  const Column cq{v.s->quals + v.q0, v.m, v.rev, false};
  const bool wide_s = warp_non_ascii(cs, lane);
  const bool wide_q = warp_non_ascii(cq, lane);
  char* o = text + (a.len[i] - base);
  uint32_t h = 0;
  if (lane == 0) h = head(a, v, o);
  h = __shfl_sync(0xffffffffu, h, 0);
  o += h;
  uint32_t ls = v.m;
  if (wide_s) {
    if (lane == 0) ls = lossy(cs, o);
    ls = __shfl_sync(0xffffffffu, ls, 0);
  } else {
    for (uint32_t k = lane; k < v.m; k += 32) o[k] = (char)cs.at(k);
  }
  o += ls;
  if (lane == 0) *o = '\t';
  o += 1;
  uint32_t lq = v.m;
  if (wide_q) {
    if (lane == 0) lq = lossy(cq, o);
    lq = __shfl_sync(0xffffffffu, lq, 0);
  } else {
    for (uint32_t k = lane; k < v.m; k += 32) o[k] = (char)cq.at(k);
  }
  o += lq;
  if (lane == 0) {
    if (a.rg_len) {
      const char tag[6] = {'\t', 'R', 'G', ':', 'Z', ':'};
      for (int k = 0; k < 6; k++) *o++ = tag[k];
      for (uint32_t k = 0; k < a.rg_len; k++) *o++ = a.rg[k];
    }
    *o = '\n';
  }
}

// u64 exclusive scan in place: tiles of 1024 (256 threads x 4), tile sums,
// one block over the sums, then the tile carries applied.
constexpr int SC_T = 256, SC_PER = 4, SC_TILE = SC_T * SC_PER;

__device__ __forceinline__ unsigned long long block_excl(unsigned long long x, unsigned long long* w,
                                                          unsigned long long* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned long long inc = x;
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned long long y = __shfl_up_sync(0xffffffffu, inc, d);
    if (lane >= d) inc += y;
  }
  if (lane == 31) w[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    unsigned long long z = lane < SC_T / 32 ? w[lane] : 0;
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned long long y = __shfl_up_sync(0xffffffffu, z, d);
      if (lane >= d) z += y;
    }
    if (lane < SC_T / 32) w[lane] = z;
  }
  __syncthreads();
  const unsigned long long ex = (wid > 0 ? w[wid - 1] : 0) + inc - x;
  *total = w[SC_T / 32 - 1];
  __syncthreads();
  return ex;
}

__global__ void __launch_bounds__(SC_T) k_scan64_tiles(unsigned long long* a, uint64_t n, unsigned long long* sums) {
  __shared__ unsigned long long w[SC_T / 32];
  const uint64_t b = (uint64_t)blockIdx.x * SC_TILE + (uint64_t)threadIdx.x * SC_PER;
  unsigned long long v[SC_PER], t = 0;
  for (int k = 0; k < SC_PER; k++) {
    v[k] = b + k < n ? a[b + k] : 0;
    t += v[k];
  }
  unsigned long long tot;
  unsigned long long ex = block_excl(t, w, &tot);
  for (int k = 0; k < SC_PER; k++) {
    if (b + k < n) a[b + k] = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(SC_T) k_scan64_sums(unsigned long long* sums, uint64_t nb, unsigned long long* total) {
  __shared__ unsigned long long w[SC_T / 32];
  unsigned long long carry = 0;
  for (uint64_t b0 = 0; b0 < nb; b0 += SC_T) {
    const uint64_t i = b0 + threadIdx.x;
    const unsigned long long x = i < nb ? sums[i] : 0;
    unsigned long long tot;
    const unsigned long long ex = block_excl(x, w, &tot);
    if (i < nb) sums[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(SC_T) k_scan64_apply(unsigned long long* a, uint64_t n, const unsigned long long* sums) {
  const uint64_t b = (uint64_t)blockIdx.x * SC_TILE + (uint64_t)threadIdx.x * SC_PER;
  const unsigned long long c = sums[blockIdx.x];
  for (int k = 0; k < SC_PER; k++)
    if (b + k < n) a[b + k] += c;
}

#define SCK(call)                                                  \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
      return PBW_ERR_CUDA;                                         \
    }                                                              \
  } while (0)

// Device allocations of one formatting call.
struct Scratch {
  std::vector<void*> ptrs;
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t alloc(T*& p, size_t n) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(q);
    p = (T*)q;
    return e;
  }
};

template <class T>
cudaError_t upload(Scratch& S, const T* host, size_t n, const T*& dev, cudaStream_t st) {
  T* d = nullptr;
  cudaError_t e = S.alloc(d, n);
  if (e != cudaSuccess) return e;
  if (n) e = cudaMemcpyAsync(d, host, n * sizeof(T), cudaMemcpyHostToDevice, st);
  dev = d;
  return e;
}

struct ReadGroupSpec {
  std::string id, header_line;
};

// ReadGroup::parse (sam.rs:17-32).
int parse_read_group(pbw_handle* h, const char* spec, ReadGroupSpec& rg) {
  std::string s(spec);
  std::vector<std::string> fields;
  bool have_id = false;
  size_t a = 0;
  while (true) {
    const size_t e = s.find(',', a);
    const std::string pair = s.substr(a, e == std::string::npos ? std::string::npos : e - a);
    const size_t c = pair.find(':');
    if (c == std::string::npos) {
      h->err = "--readgroup: expected TAG:VALUE, got '" + pair + "'";
      return PBW_ERR_ARG;
    }
    const std::string tag = pair.substr(0, c), value = pair.substr(c + 1);
    if (tag == "ID") {
      rg.id = value;
      have_id = true;
    }
    fields.push_back(tag + ":" + value);
    if (e == std::string::npos) break;
    a = e + 1;
  }
  if (!have_id) {
    h->err = "--readgroup must set at least an ID tag";
    return PBW_ERR_ARG;
  }
  rg.header_line = "@RG";
  for (auto& f : fields) rg.header_line += "\t" + f;
  return PBW_OK;
}

// Output of the formatter: a FILE* or a caller buffer.
struct Sink {
  FILE* f = nullptr;
  char* buf = nullptr;
  uint64_t cap = 0, used = 0;
  bool put(const char* p, size_t n) {
    if (f) return fwrite(p, 1, n, f) == n;
    if (used + n > cap) return false;
    memcpy(buf + used, p, n);
    used += n;
    return true;
  }
};

std::string sam_header(pbw_handle* h, const pbw_sam_options* o, const ReadGroupSpec* rg) {
  std::string out = std::string("@HD\tVN:1.6\tSO:") + (o->coordinate_sorted ? "coordinate" : "unsorted") + "\n";
  for (size_t c = 0; c < h->names.size(); c++)
    out += "@SQ\tSN:" + h->names[c] + "\tLN:" + std::to_string(h->lens[c]) + "\n";
  out += std::string("@PG\tID:probebwa\tPN:probebwa\tVN:0.1.0\tCL:") + (o->command_line ? o->command_line : "") + "\n";
  if (rg) out += rg->header_line + "\n";
  return out;
}

constexpr uint64_t SAM_CHUNK = 1u << 18;  // records per write pass

// Formats the selected records. Sizing mode (sink == nullptr) only sets
// *total_len (header included).
int sam_run(pbw_handle* h, const pbw_sam_options* o, uint32_t n_src, const pbw_sam_source* src,
            const uint64_t* sel, uint64_t n_sel, Sink* sink, uint64_t* total_len) {
  if (!h || !o || !src || n_src < 1 || n_src > 2) {
    if (h) h->err = "pbw_sam: bad arguments";
    return PBW_ERR_ARG;
  }
  for (uint32_t s = 0; s < n_src; s++) {
    if (!src[s].reads || !src[s].recs || !src[s].read_ids || src[s].reads->n != src[s].recs->n) {
      h->err = "pbw_sam: source " + std::to_string(s) + " needs reads, IDs and records of equal count";
      return PBW_ERR_ARG;
    }
  }
  ReadGroupSpec rg;
  const bool have_rg = o->read_group != nullptr;
  if (have_rg) {
    int rc = parse_read_group(h, o->read_group, rg);
    if (rc != PBW_OK) return rc;
  }
  const std::string hdr = sam_header(h, o, have_rg ? &rg : nullptr);
  // the selection: record numbers r * n_src + s
  std::vector<unsigned long long> all;
  const unsigned long long* selp = (const unsigned long long*)sel;
  if (!sel) {
    for (uint32_t s = 1; s < n_src; s++)
      if (src[s].recs->n != src[0].recs->n) {
        h->err = "pbw_sam: paired sources must hold the same number of records";
        return PBW_ERR_ARG;
      }
    n_sel = src[0].recs->n * n_src;
    all.resize(n_sel);
    for (uint64_t i = 0; i < n_sel; i++) all[i] = i;
    selp = all.data();
  } else {
    for (uint64_t i = 0; i < n_sel; i++)
      if (sel[i] / n_src >= src[sel[i] % n_src].recs->n) {
        h->err = "pbw_sam: selection entry " + std::to_string(i) + " names no record";
        return PBW_ERR_ARG;
      }
  }
  cudaStream_t st = h->st;
  Scratch S;
  SamArgs a{};
  a.n_src = n_src;
  a.n_sel = n_sel;
  for (uint32_t s = 0; s < n_src; s++) {
    const pbw_reads* R = src[s].reads;
    const pbw_records* C = src[s].recs;
    const uint64_t n = C->n, nb = R->offsets[n];
    // QNAMEs, concatenated
    std::vector<char> ids;
    std::vector<uint64_t> id_off(n + 1, 0);
    for (uint64_t i = 0; i < n; i++) {
      const char* q = src[s].read_ids[i] ? src[s].read_ids[i] : "";
      ids.insert(ids.end(), q, q + strlen(q));
      id_off[i + 1] = ids.size();
    }
    SamSrcDev& d = a.src[s];
    SCK(upload(S, R->bases, nb, d.bases, st));
    SCK(upload(S, R->quals, nb, d.quals, st));
    SCK(upload(S, R->offsets, n + 1, d.offs, st));
    SCK(upload(S, ids.data(), ids.size(), d.ids, st));
    SCK(upload(S, id_off.data(), n + 1, d.id_off, st));
    SCK(upload(S, C->flag, n, d.flag, st));
    SCK(upload(S, C->contig, n, d.contig, st));
    SCK(upload(S, (const unsigned long long*)C->pos, n, d.pos, st));
    SCK(upload(S, C->mapq, n, d.mapq, st));
    SCK(upload(S, C->cigar_off, n + 1, d.cig_off, st));
    SCK(upload(S, C->cigar, C->cigar_off[n], d.cigar, st));
    SCK(upload(S, C->mate_contig, n, d.mate_contig, st));
    SCK(upload(S, (const unsigned long long*)C->mate_pos, n, d.mate_pos, st));
    SCK(upload(S, (const long long*)C->tlen, n, d.tlen, st));
    // no host vector may be freed before its copy has been read
    SCK(cudaStreamSynchronize(st));
  }
  {
    std::vector<char> names;
    std::vector<uint64_t> off(h->names.size() + 1, 0);
    for (size_t c = 0; c < h->names.size(); c++) {
      names.insert(names.end(), h->names[c].begin(), h->names[c].end());
      off[c + 1] = names.size();
    }
    a.n_names = (uint32_t)h->names.size();
    SCK(upload(S, names.data(), names.size(), a.names, st));
    SCK(upload(S, off.data(), off.size(), a.name_off, st));
    if (have_rg) {
      SCK(upload(S, rg.id.data(), rg.id.size(), a.rg, st));
      a.rg_len = (uint32_t)rg.id.size();
    }
    SCK(upload(S, selp, n_sel, a.sel, st));
    SCK(cudaStreamSynchronize(st));
  }
  // lengths -> offsets
  const uint64_t nb = (n_sel + SC_TILE - 1) / SC_TILE;
  unsigned long long *len = nullptr, *sums = nullptr;
  SCK(S.alloc(len, n_sel + 1));
  SCK(S.alloc(sums, nb + 2));
  a.len = len;
  unsigned long long body = 0;
  if (n_sel) {
    k_sam_len<<<(unsigned)((n_sel + SAM_WARPS - 1) / SAM_WARPS), SAM_WARPS * 32, 0, st>>>(a);
    k_scan64_tiles<<<(unsigned)nb, SC_T, 0, st>>>(len, n_sel, sums);
    k_scan64_sums<<<1, SC_T, 0, st>>>(sums, nb, sums + nb);
    k_scan64_apply<<<(unsigned)nb, SC_T, 0, st>>>(len, n_sel, sums);
    SCK(cudaGetLastError());
    SCK(cudaMemcpyAsync(&body, sums + nb, sizeof(body), cudaMemcpyDeviceToHost, st));
    SCK(cudaStreamSynchronize(st));
    // offsets[n_sel] = body: the end of the last chunk
    SCK(cudaMemcpyAsync(len + n_sel, sums + nb, sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
  }
  *total_len = hdr.size() + body;
  if (!sink) return PBW_OK;
  if (!sink->f && sink->cap < *total_len) {
    h->err = "pbw_sam_format: buffer of " + std::to_string(sink->cap) + " bytes, text needs " +
             std::to_string(*total_len);
    return PBW_ERR_CAPACITY;
  }
  if (!sink->put(hdr.data(), hdr.size())) {
    h->err = "pbw_sam: short write";
    return PBW_ERR_IO;
  }
  if (n_sel == 0) return PBW_OK;
  // chunk boundaries in bytes: offsets at every SAM_CHUNK-th record
  const uint64_t n_ch = (n_sel + SAM_CHUNK - 1) / SAM_CHUNK;
  std::vector<unsigned long long> cut(n_ch + 1, 0);
  for (uint64_t c = 0; c <= n_ch; c++) {
    const uint64_t i = std::min<uint64_t>(c * SAM_CHUNK, n_sel);
    SCK(cudaMemcpyAsync(&cut[c], len + i, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  }
  SCK(cudaStreamSynchronize(st));
  unsigned long long max_chunk = 0;
  for (uint64_t c = 0; c < n_ch; c++) max_chunk = std::max(max_chunk, cut[c + 1] - cut[c]);
  char* text = nullptr;
  SCK(S.alloc(text, max_chunk));
  HostBuf& stage = h->h_stage;
  if (!sink->f) {
    // caller buffer: copy straight into it
    for (uint64_t c = 0; c < n_ch; c++) {
      const uint64_t i0 = c * SAM_CHUNK, i1 = std::min<uint64_t>(i0 + SAM_CHUNK, n_sel);
      k_sam_write<<<(unsigned)((i1 - i0 + SAM_WARPS - 1) / SAM_WARPS), SAM_WARPS * 32, 0, st>>>(a, i0, i1, cut[c], text);
      SCK(cudaGetLastError());
      SCK(cudaMemcpyAsync(sink->buf + sink->used, text, cut[c + 1] - cut[c], cudaMemcpyDeviceToHost, st));
      SCK(cudaStreamSynchronize(st));
      sink->used += cut[c + 1] - cut[c];
    }
    return PBW_OK;
  }
  if (!stage.ensure(max_chunk)) {
    h->err = "cudaMallocHost for SAM staging failed";
    return PBW_ERR_NOMEM;
  }
  for (uint64_t c = 0; c < n_ch; c++) {
    const uint64_t i0 = c * SAM_CHUNK, i1 = std::min<uint64_t>(i0 + SAM_CHUNK, n_sel);
    const uint64_t bytes = cut[c + 1] - cut[c];
    k_sam_write<<<(unsigned)((i1 - i0 + SAM_WARPS - 1) / SAM_WARPS), SAM_WARPS * 32, 0, st>>>(a, i0, i1, cut[c], text);
    SCK(cudaGetLastError());
    SCK(cudaMemcpyAsync(stage.p, text, bytes, cudaMemcpyDeviceToHost, st));
    SCK(cudaStreamSynchronize(st));
    if (!sink->put((const char*)stage.p, bytes)) {
      h->err = "pbw_sam: short write";
      return PBW_ERR_IO;
    }
  }
  return PBW_OK;
}

}  // namespace

}  // namespace pbw

extern "C" {

int pbw_sam_write(pbw_handle* h, const pbw_sam_options* opt, uint32_t n_src, const pbw_sam_source* src,
                  const uint64_t* sel, uint64_t n_sel, const char* path) {
  if (!h || !path) return PBW_ERR_ARG;
  const bool to_stdout = strcmp(path, "-") == 0;
  FILE* f = to_stdout ? stdout : fopen(path, "wb");
  if (!f) {
    h->err = std::string("cannot write ") + path;
    return PBW_ERR_IO;
  }
  pbw::Sink sink;
  sink.f = f;
  uint64_t total = 0;
  int rc = pbw::sam_run(h, opt, n_src, src, sel, n_sel, &sink, &total);
  if (to_stdout) {
    if (fflush(f) != 0 && rc == PBW_OK) {
      h->err = "short write to stdout";
      rc = PBW_ERR_IO;
    }
  } else if (fclose(f) != 0 && rc == PBW_OK) {
    h->err = std::string("short write to ") + path;
    rc = PBW_ERR_IO;
  }
  return rc;
}

int pbw_sam_format(pbw_handle* h, const pbw_sam_options* opt, uint32_t n_src, const pbw_sam_source* src,
                   const uint64_t* sel, uint64_t n_sel, char* out, uint64_t cap, uint64_t* len) {
  if (!h || !len) return PBW_ERR_ARG;
  if (!out) return pbw::sam_run(h, opt, n_src, src, sel, n_sel, nullptr, len);
  pbw::Sink sink;
  sink.buf = out;
  sink.cap = cap;
  return pbw::sam_run(h, opt, n_src, src, sel, n_sel, &sink, len);
}

int pbw_write_sam(pbw_handle* h, const char* path, const char* command_line, const pbw_reads* reads,
                  const char* const* read_ids, const pbw_records* recs) {
  if (!h || !path || !reads || !recs || !read_ids) return PBW_ERR_ARG;
  pbw_sam_options o{};
  o.command_line = command_line;
  pbw_sam_source s{reads, read_ids, recs};
  return pbw_sam_write(h, &o, 1, &s, nullptr, 0, path);
}

}  // extern "C"
