// bam.cpp -- BAM output and its BAI index (src/io/bam.rs:19-57, main.rs:178-186).
//
// The reference formats the SAM stream (format_sam_records) and hands the
// text to noodles, which parses it back into records and writes them as
// BGZF-compressed BAM; with --index it then builds a BAI. The same order
// here: the SAM text comes from the device formatter (pbw_sam_format), each
// line is parsed and encoded as a BAM record the way a SAM parser reads it
// (QUAL characters are Phred+33, so the raw score bytes this mapper writes
// become score - 33 and bytes outside '!'..'~' are an error, as a strict
// parser reports them; SEQ uses the 16 IUPAC codes "=ACMGRSVTWYHKDBN"), the
// stream is cut into 65,280-byte BGZF blocks compressed on all host threads
// (zlib's raw deflate, opened at run time), and the BAI is built from the
// records' virtual offsets: per reference the bins with their merged chunks,
// the metadata pseudo-bin 37450, and the 16 kbp linear index (SAM
// specification section 5).
//
// The bytes are not those of noodles (its deflate and header re-serialisation
// are not available here); what is pinned is the reference's own CLI test
// (tests/cli.rs:46-80, 148-195): BGZF with the BAM magic, records in
// coordinate order with --index, a BAI with its magic.
#include <algorithm>
#include <array>
#include <atomic>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <string_view>
#include <thread>
#include <vector>

#include <dlfcn.h>

#include "../../include/probebwa_gpu.h"
#include "abi_guard.h"
#include "pbw_pipeline.h"

namespace {

// ---- zlib, opened at run time (the z_stream of its public API, LP64) ----
struct ZS {
  const unsigned char* next_in;
  unsigned avail_in;
  unsigned long total_in;
  unsigned char* next_out;
  unsigned avail_out;
  unsigned long total_out;
  const char* msg;
  void* state;
  void* zalloc;
  void* zfree;
  void* opaque;
  int data_type;
  unsigned long adler;
  unsigned long reserved;
};
struct Zlib {
  const char* (*version)() = nullptr;
  int (*init2)(ZS*, int, int, int, int, int, const char*, int) = nullptr;
  int (*deflate)(ZS*, int) = nullptr;
  int (*end)(ZS*) = nullptr;
  unsigned long (*crc32)(unsigned long, const unsigned char*, unsigned) = nullptr;
  bool ok = false;
};
const Zlib& zlib() {
  static Zlib z = [] {
    Zlib r;
    void* lib = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
    if (!lib) return r;
    r.version = (const char* (*)())dlsym(lib, "zlibVersion");
    r.init2 = (int (*)(ZS*, int, int, int, int, int, const char*, int))dlsym(lib, "deflateInit2_");
    r.deflate = (int (*)(ZS*, int))dlsym(lib, "deflate");
    r.end = (int (*)(ZS*))dlsym(lib, "deflateEnd");
    r.crc32 = (unsigned long (*)(unsigned long, const unsigned char*, unsigned))dlsym(lib, "crc32");
    r.ok = r.version && r.init2 && r.deflate && r.end && r.crc32;
    return r;
  }();
  return z;
}

constexpr size_t BGZF_BLOCK = 65280;  // uncompressed bytes per block
const unsigned char BGZF_EOF[28] = {0x1f, 0x8b, 0x08, 0x04, 0, 0, 0, 0, 0, 0xff, 0x06, 0, 0x42, 0x43,
                                    0x02, 0,    0x1b, 0,    0x03, 0, 0, 0, 0, 0, 0, 0,    0,    0};

void put16(std::vector<unsigned char>& o, uint32_t v) {
  o.push_back((unsigned char)v);
  o.push_back((unsigned char)(v >> 8));
}
void put32(std::vector<unsigned char>& o, uint32_t v) {
  for (int i = 0; i < 4; i++) o.push_back((unsigned char)(v >> (8 * i)));
}
void put64(std::vector<unsigned char>& o, uint64_t v) {
  for (int i = 0; i < 8; i++) o.push_back((unsigned char)(v >> (8 * i)));
}

// One BGZF block (gzip member with the BC extra field) of in[0, n).
bool bgzf_block(const unsigned char* in, size_t n, std::vector<unsigned char>& out) {
  const Zlib& z = zlib();
  out.clear();
  for (int level : {6, 0}) {
    std::vector<unsigned char> buf(n + n / 8 + 1024);
    ZS s;
    memset(&s, 0, sizeof(s));
    if (z.init2(&s, level, 8, -15, 8, 0, z.version(), (int)sizeof(ZS)) != 0) return false;
    s.next_in = in;
    s.avail_in = (unsigned)n;
    s.next_out = buf.data();
    s.avail_out = (unsigned)buf.size();
    const int rc = z.deflate(&s, 4 /* Z_FINISH */);
    const size_t clen = buf.size() - s.avail_out;
    z.end(&s);
    if (rc != 1 /* Z_STREAM_END */) return false;
    const size_t total = 18 + clen + 8;
    if (total > 65536) continue;  // incompressible: stored deflate blocks fit
    const unsigned char hdr[16] = {0x1f, 0x8b, 0x08, 0x04, 0, 0, 0, 0, 0, 0xff, 0x06, 0, 0x42, 0x43, 0x02, 0};
    out.insert(out.end(), hdr, hdr + 16);
    put16(out, (uint32_t)(total - 1));
    out.insert(out.end(), buf.data(), buf.data() + clen);
    put32(out, (uint32_t)z.crc32(0, in, (unsigned)n));
    put32(out, (uint32_t)n);
    return true;
  }
  return false;
}

// reg2bin of the SAM specification (section 5.3): [beg, end), 0-based.
int reg2bin(int64_t beg, int64_t end) {
  --end;
  if (beg >> 14 == end >> 14) return (int)(((1 << 15) - 1) / 7 + (beg >> 14));
  if (beg >> 17 == end >> 17) return (int)(((1 << 12) - 1) / 7 + (beg >> 17));
  if (beg >> 20 == end >> 20) return (int)(((1 << 9) - 1) / 7 + (beg >> 20));
  if (beg >> 23 == end >> 23) return (int)(((1 << 6) - 1) / 7 + (beg >> 23));
  if (beg >> 26 == end >> 26) return (int)(((1 << 3) - 1) / 7 + (beg >> 26));
  return 0;
}

}  // namespace

namespace {

// Where a record went, for the index.
struct RecIdx {
  int32_t ref;
  int64_t beg, end;  // 0-based reference span (end > beg)
  int bin;
  bool unmapped;
  uint64_t u0, u1;   // uncompressed stream offsets of the record
};

struct Field {
  const char* p;
  size_t n;
  bool is(const char* s) const { return n == strlen(s) && memcmp(p, s, n) == 0; }
};

// A decimal integer of at most 18 digits (no overflow), optionally signed.
bool parse_i64(const Field& f, int64_t& v) {
  if (f.n == 0) return false;
  size_t i = 0;
  bool neg = false;
  if (f.p[0] == '-' || f.p[0] == '+') {
    neg = f.p[0] == '-';
    i = 1;
  }
  if (i == f.n || f.n - i > 18) return false;
  int64_t x = 0;
  for (; i < f.n; i++) {
    if (f.p[i] < '0' || f.p[i] > '9') return false;
    x = x * 10 + (f.p[i] - '0');
  }
  v = neg ? -x : x;
  return true;
}

const char* SEQ_CODES = "=ACMGRSVTWYHKDBN";

// 4-bit SEQ code of a byte (lower case as upper case), 0xFF for a byte that
// is not one of the 16 IUPAC symbols.
const unsigned char* seq_code_table() {
  static const auto table = [] {
    std::array<unsigned char, 256> t;
    t.fill(0xFF);
    for (int k = 0; k < 16; k++) {
      t[(unsigned char)SEQ_CODES[k]] = (unsigned char)k;
      if (SEQ_CODES[k] >= 'A' && SEQ_CODES[k] <= 'Z') t[(unsigned char)(SEQ_CODES[k] + 32)] = (unsigned char)k;
    }
    return t;
  }();
  return table.data();
}

using RefMap = std::map<std::string, int32_t, std::less<>>;

// One SAM record line as a BAM record (block_size first) appended to out;
// on an error out is left as it was.
bool encode_record(const char* line, size_t len, const RefMap& refs, std::vector<unsigned char>& out, RecIdx& ix,
                   std::string& err) {
  thread_local std::vector<Field> f;
  thread_local std::vector<uint32_t> cig;
  f.clear();
  size_t a = 0;
  for (size_t i = 0; i <= len; i++)
    if (i == len || line[i] == '\t') {
      f.push_back(Field{line + a, i - a});
      a = i + 1;
    }
  if (f.size() < 11) {
    err = "SAM record with fewer than 11 fields";
    return false;
  }
  auto ref_of = [&](const Field& x, int32_t same) -> int32_t {
    if (x.is("*")) return -1;
    if (x.is("=")) return same;
    auto it = refs.find(std::string_view(x.p, x.n));
    return it == refs.end() ? -2 : it->second;
  };
  int64_t flag, pos, mapq, pnext, tlen;
  constexpr int64_t POS_MAX = 0x7FFFFFFF;  // SAM POS / PNEXT / TLEN ranges (int32 in BAM)
  if (!parse_i64(f[1], flag) || !parse_i64(f[3], pos) || !parse_i64(f[4], mapq) || !parse_i64(f[7], pnext) ||
      !parse_i64(f[8], tlen) || flag < 0 || flag > 0xFFFF || mapq < 0 || mapq > 255 || pos < 0 || pos > POS_MAX ||
      pnext < 0 || pnext > POS_MAX || tlen < -POS_MAX || tlen > POS_MAX) {
    err = "SAM record with a malformed or out-of-range number";
    return false;
  }
  const int32_t ref = ref_of(f[2], -1);
  const int32_t nref = ref_of(f[6], ref);
  if (ref == -2 || nref == -2) {
    err = "SAM record names a reference sequence missing from the header";
    return false;
  }
  if (f[0].n == 0 || f[0].n > 254) {
    err = "invalid read name";
    return false;
  }
  // CIGAR
  cig.clear();
  int64_t span = 0;
  if (!f[5].is("*")) {
    int64_t v = 0;
    bool any = false;
    for (size_t i = 0; i < f[5].n; i++) {
      const char c = f[5].p[i];
      if (c >= '0' && c <= '9') {
        v = v * 10 + (c - '0');
        any = true;
        if (v >= (1 << 28)) {  // BAM operation lengths have 28 bits
          err = "CIGAR operation too long";
          return false;
        }
        continue;
      }
      const char* ops = "MIDNSHP=X";
      const char* q = strchr(ops, c);
      if (!q || !any || c == 0) {
        err = "invalid CIGAR";
        return false;
      }
      const int op = (int)(q - ops);
      cig.push_back((uint32_t)(v << 4) | (uint32_t)op);
      if (op == 0 || op == 2 || op == 3 || op == 7 || op == 8) span += v;
      v = 0;
      any = false;
    }
    if (any) {
      err = "invalid CIGAR";
      return false;
    }
    if (cig.size() > 0xFFFF) {  // the 16-bit operation count of a BAM record
      err = "CIGAR with more than 65535 operations";
      return false;
    }
  }
  const Field& sq = f[9];
  const Field& ql = f[10];
  const size_t l_seq = (sq.is("*") || sq.n == 0) ? 0 : sq.n;
  const int32_t p0 = (int32_t)(pos - 1);
  const bool unmapped = (flag & 4) != 0;
  const int64_t beg = p0 < 0 ? -1 : p0;
  const int64_t end = beg < 0 ? 0 : beg + (span > 0 && !unmapped ? span : 1);
  const int bin = reg2bin(beg, end);
  // fixed fields, name and CIGAR, then SEQ, QUAL and the optional fields as
  // they are checked
  const size_t start = out.size();
  auto fail = [&](const char* what) {
    out.resize(start);
    err = what;
    return false;
  };
  put32(out, 0);  // block_size, patched below
  put32(out, (uint32_t)ref);
  put32(out, (uint32_t)p0);
  out.push_back((unsigned char)(f[0].n + 1));
  out.push_back((unsigned char)mapq);
  put16(out, (uint32_t)bin);
  put16(out, (uint32_t)cig.size());
  put16(out, (uint32_t)flag);
  put32(out, (uint32_t)l_seq);
  put32(out, (uint32_t)nref);
  put32(out, (uint32_t)(int32_t)(pnext - 1));
  put32(out, (uint32_t)(int32_t)tlen);
  out.insert(out.end(), f[0].p, f[0].p + f[0].n);
  out.push_back(0);
  for (uint32_t c : cig) put32(out, c);
  // SEQ: two 4-bit codes a byte, the first in the high nibble
  const unsigned char* code = seq_code_table();
  const size_t s0 = out.size();
  out.resize(s0 + (l_seq + 1) / 2, 0);
  for (size_t i = 0; i < l_seq; i++) {
    const unsigned char k = code[(unsigned char)sq.p[i]];
    if (k == 0xFF) return fail("invalid sequence base");
    out[s0 + i / 2] |= (unsigned char)(k << ((i & 1) ? 0 : 4));
  }
  // QUAL: Phred+33 characters, or 0xFF for each base when absent
  const size_t q0 = out.size();
  out.resize(q0 + l_seq, 0xFF);
  if (!(ql.is("*") || ql.n == 0)) {
    if (ql.n != l_seq) return fail("quality scores and sequence differ in length");
    for (size_t i = 0; i < l_seq; i++) {
      const unsigned char c = (unsigned char)ql.p[i];
      if (c < '!' || c > '~') return fail("invalid quality score");
      out[q0 + i] = (unsigned char)(c - 33);
    }
  }
  // optional fields: TAG:TYPE:VALUE, Z and i only (what this mapper writes)
  for (size_t k = 11; k < f.size(); k++) {
    const Field& t = f[k];
    if (t.n < 5 || t.p[2] != ':' || t.p[4] != ':') return fail("invalid optional field");
    if (t.p[3] == 'Z') {
      out.push_back((unsigned char)t.p[0]);
      out.push_back((unsigned char)t.p[1]);
      out.push_back('Z');
      out.insert(out.end(), t.p + 5, t.p + t.n);
      out.push_back(0);
    } else if (t.p[3] == 'i') {
      int64_t v;
      if (!parse_i64(Field{t.p + 5, t.n - 5}, v) || v < INT32_MIN || v > INT32_MAX) return fail("invalid optional field");
      out.push_back((unsigned char)t.p[0]);
      out.push_back((unsigned char)t.p[1]);
      out.push_back('i');
      put32(out, (uint32_t)(int32_t)v);
    } else {
      return fail("unsupported optional field type");
    }
  }
  if (end > POS_MAX + 1) return fail("alignment ends beyond 2^31");
  ix.ref = ref;
  ix.beg = beg;
  ix.end = end;
  ix.bin = bin;
  ix.unmapped = unmapped;
  const uint32_t bs = (uint32_t)(out.size() - start - 4);
  for (int i = 0; i < 4; i++) out[start + i] = (unsigned char)(bs >> (8 * i));
  return true;
}

}  // namespace

namespace {

// BAI of a coordinate-sorted record stream (SAM specification section 5.2).
std::vector<unsigned char> build_bai(const std::vector<RecIdx>& recs, size_t n_ref,
                                     const std::vector<uint64_t>& block_coff) {
  auto voff = [&](uint64_t u) -> uint64_t {
    const uint64_t b = u / BGZF_BLOCK;
    return (block_coff[b] << 16) | (u % BGZF_BLOCK);
  };
  struct Ref {
    std::map<uint32_t, std::vector<std::pair<uint64_t, uint64_t>>> bins;
    std::vector<uint64_t> lin;
    uint64_t beg = ~0ull, end = 0, mapped = 0, unmapped = 0;
  };
  std::vector<Ref> R(n_ref);
  uint64_t no_coor = 0;
  for (const RecIdx& r : recs) {
    if (r.ref < 0 || (size_t)r.ref >= n_ref || r.beg < 0) {
      no_coor++;
      continue;
    }
    Ref& x = R[r.ref];
    const uint64_t v0 = voff(r.u0), v1 = voff(r.u1);
    auto& ch = x.bins[(uint32_t)r.bin];
    if (!ch.empty() && ch.back().second == v0) ch.back().second = v1;
    else ch.push_back({v0, v1});
    const int64_t w0 = r.beg >> 14, w1 = (r.end - 1) >> 14;
    if ((int64_t)x.lin.size() <= w1) x.lin.resize((size_t)w1 + 1, 0);
    for (int64_t w = w0; w <= w1; w++)
      if (x.lin[(size_t)w] == 0 || v0 < x.lin[(size_t)w]) x.lin[(size_t)w] = v0;
    x.beg = std::min(x.beg, v0);
    x.end = std::max(x.end, v1);
    if (r.unmapped) x.unmapped++;
    else x.mapped++;
  }
  std::vector<unsigned char> o = {'B', 'A', 'I', 1};
  put32(o, (uint32_t)n_ref);
  for (Ref& x : R) {
    const bool any = x.end > 0;
    put32(o, (uint32_t)(x.bins.size() + (any ? 1 : 0)));
    for (auto& kv : x.bins) {
      put32(o, kv.first);
      put32(o, (uint32_t)kv.second.size());
      for (auto& c : kv.second) {
        put64(o, c.first);
        put64(o, c.second);
      }
    }
    if (any) {  // metadata pseudo-bin: the reference's span and its record counts
      put32(o, 37450);
      put32(o, 2);
      put64(o, x.beg);
      put64(o, x.end);
      put64(o, x.mapped);
      put64(o, x.unmapped);
    }
    // windows without records take the offset of the next window that has one
    for (size_t w = x.lin.size(); w-- > 0;)
      if (x.lin[w] == 0 && w + 1 < x.lin.size()) x.lin[w] = x.lin[w + 1];
    put32(o, (uint32_t)x.lin.size());
    for (uint64_t v : x.lin) put64(o, v);
  }
  put64(o, no_coor);
  return o;
}

bool write_all(const std::string& path, const std::vector<std::vector<unsigned char>>& parts, std::string& err) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    err = "cannot write " + path;
    return false;
  }
  bool ok = true;
  for (auto& p : parts) ok = ok && fwrite(p.data(), 1, p.size(), f) == p.size();
  ok = (fclose(f) == 0) && ok;
  if (!ok) err = "short write to " + path;
  return ok;
}

}  // namespace

namespace {

// The BAM stream of a SAM text whose reference dictionary is names / lens:
// the header lines verbatim, the references, every record line encoded,
// BGZF blocks deflated on all host threads; with write_index the BAI of the
// (coordinate-sorted) records next to it. Returns a PBW status and sets err.
int bam_from_text(const char* text, size_t len, const std::vector<std::string>& names,
                  const std::vector<uint64_t>& lens, const char* path, bool write_index, std::string& err) {
  // header lines, then records
  size_t hdr_end = 0;
  while (hdr_end < len && text[hdr_end] == '@') {
    const char* nl = (const char*)memchr(text + hdr_end, '\n', len - hdr_end);
    hdr_end = nl ? (size_t)(nl - text) + 1 : len;
  }
  RefMap refs;
  for (size_t c = 0; c < names.size(); c++) refs.emplace(names[c], (int32_t)c);
  std::vector<unsigned char> u;
  u.reserve(len + 4096);  // a BAM stream is about the size of its SAM text or smaller
  u.insert(u.end(), {'B', 'A', 'M', 1});
  put32(u, (uint32_t)hdr_end);
  u.insert(u.end(), text, text + hdr_end);
  put32(u, (uint32_t)names.size());
  for (size_t c = 0; c < names.size(); c++) {
    put32(u, (uint32_t)(names[c].size() + 1));
    u.insert(u.end(), names[c].begin(), names[c].end());
    u.push_back(0);
    put32(u, (uint32_t)lens[c]);
  }
  // records: contiguous slices of whole lines encoded on the host threads,
  // then joined in order (the stream offsets of each slice's records shift
  // by the bytes before it)
  struct Slice {
    size_t b = 0, e = 0;
    std::vector<unsigned char> bytes;
    std::vector<RecIdx> recs;
    bool ok = true;
    std::string err;
  };
  const size_t body = len - hdr_end;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const size_t ns = body < (4u << 20) ? 1 : std::min<size_t>(hw, 16);
  std::vector<Slice> sl(ns);
  for (size_t k = 0; k < ns; k++) {
    size_t b = k == 0 ? hdr_end : sl[k - 1].e;
    size_t e = k + 1 == ns ? len : std::max(b, hdr_end + body / ns * (k + 1));
    if (e < len) {  // to the start of the next line
      const char* nl = (const char*)memchr(text + e, '\n', len - e);
      e = nl ? (size_t)(nl - text) + 1 : len;
    }
    sl[k].b = b;
    sl[k].e = e;
  }
  auto encode_slice = [&](Slice& x) {
    x.bytes.reserve(x.e - x.b + 4096);
    for (size_t p = x.b; p < x.e;) {
      const char* nl = (const char*)memchr(text + p, '\n', x.e - p);
      const size_t e = nl ? (size_t)(nl - text) : x.e;
      RecIdx ix;
      ix.u0 = x.bytes.size();
      if (!encode_record(text + p, e - p, refs, x.bytes, ix, x.err)) {
        x.ok = false;
        return;
      }
      ix.u1 = x.bytes.size();
      x.recs.push_back(ix);
      p = e + 1;
    }
  };
  if (ns == 1) {
    encode_slice(sl[0]);
  } else {
    std::vector<std::thread> th;
    for (size_t k = 0; k < ns; k++) th.emplace_back([&, k] { encode_slice(sl[k]); });
    for (auto& t : th) t.join();
  }
  std::vector<RecIdx> recs;
  for (Slice& x : sl) {
    if (!x.ok) {  // the first record that failed, numbered over the whole stream
      err = "BAM: record " + std::to_string(recs.size() + x.recs.size()) + ": " + x.err;
      return PBW_ERR_FORMAT;
    }
    const uint64_t base = u.size();
    u.insert(u.end(), x.bytes.begin(), x.bytes.end());
    for (RecIdx ix : x.recs) {
      ix.u0 += base;
      ix.u1 += base;
      recs.push_back(ix);
    }
    std::vector<unsigned char>().swap(x.bytes);
  }
  // an index describes records in coordinate order: placed records by
  // (reference, position), then the unplaced ones (bam.rs:38-43)
  if (write_index) {
    int64_t last = INT64_MIN;
    for (size_t k = 0; k < recs.size(); k++) {
      const RecIdx& r = recs[k];
      const int64_t key = (r.ref < 0 || r.beg < 0) ? INT64_MAX : ((int64_t)r.ref << 32) | r.beg;
      if (key < last) {
        err = "BAM: record " + std::to_string(k) + " is out of coordinate order; an index needs sorted records";
        return PBW_ERR_ARG;
      }
      last = key;
    }
  }
  // BGZF blocks on all host threads
  const size_t nb = (u.size() + BGZF_BLOCK - 1) / BGZF_BLOCK;
  std::vector<std::vector<unsigned char>> blocks(nb + 1);
  std::atomic<size_t> next(0);
  std::atomic<bool> bad(false);
  const unsigned nt = std::max(1u, std::min<unsigned>(std::thread::hardware_concurrency(), (unsigned)std::max<size_t>(nb, 1)));
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; t++)
    th.emplace_back([&] {
      for (size_t b; (b = next.fetch_add(1)) < nb;) {
        const size_t a = b * BGZF_BLOCK, n = std::min(BGZF_BLOCK, u.size() - a);
        if (!bgzf_block(u.data() + a, n, blocks[b])) bad = true;
      }
    });
  for (auto& t : th) t.join();
  if (bad) {
    err = "BAM: deflate failed";
    return PBW_ERR_IO;
  }
  blocks[nb].assign(BGZF_EOF, BGZF_EOF + sizeof(BGZF_EOF));
  if (!write_all(path, blocks, err)) return PBW_ERR_IO;
  if (write_index) {
    std::vector<uint64_t> coff(nb + 1, 0);
    for (size_t b = 0; b < nb; b++) coff[b + 1] = coff[b] + blocks[b].size();
    std::vector<std::vector<unsigned char>> bai(1, build_bai(recs, names.size(), coff));
    if (!write_all(std::string(path) + ".bai", bai, err)) return PBW_ERR_IO;
  }
  return PBW_OK;
}

// The @HD line's SO value and the @SQ dictionary (SN, LN) of a SAM header,
// as a SAM parser reads them. False for an @SQ line without SN or a valid LN.
bool parse_sam_header(const char* text, size_t len, std::string& sort_order, std::vector<std::string>& names,
                      std::vector<uint64_t>& lens, std::string& err) {
  size_t p = 0;
  while (p < len && text[p] == '@') {
    const char* nl = (const char*)memchr(text + p, '\n', len - p);
    const size_t e = nl ? (size_t)(nl - text) : len;
    const std::string line(text + p, e - p);
    std::vector<std::string> f;
    for (size_t a = 0;;) {
      const size_t b = line.find('\t', a);
      f.push_back(line.substr(a, b == std::string::npos ? std::string::npos : b - a));
      if (b == std::string::npos) break;
      a = b + 1;
    }
    if (f[0] == "@HD") {
      for (size_t k = 1; k < f.size(); k++)
        if (f[k].compare(0, 3, "SO:") == 0) sort_order = f[k].substr(3);
    } else if (f[0] == "@SQ") {
      std::string sn;
      bool have_ln = false;
      uint64_t ln = 0;
      for (size_t k = 1; k < f.size(); k++) {
        if (f[k].compare(0, 3, "SN:") == 0) sn = f[k].substr(3);
        if (f[k].compare(0, 3, "LN:") == 0) {
          const std::string v = f[k].substr(3);
          have_ln = !v.empty() && v.size() <= 10 && v.find_first_not_of("0123456789") == std::string::npos;
          if (have_ln) ln = std::stoull(v);
          have_ln = have_ln && ln >= 1 && ln <= 0x7FFFFFFFull;
        }
      }
      if (sn.empty() || !have_ln) {
        err = "BAM: @SQ line without SN or a valid LN: " + line;
        return false;
      }
      names.push_back(sn);
      lens.push_back(ln);
    }
    p = e + 1;
  }
  return true;
}

}  // namespace

namespace {

int bam_write(pbw_handle* h, const pbw_sam_options* opt, uint32_t n_src, const pbw_sam_source* src,
              const uint64_t* sel, uint64_t n_sel, const char* path, int32_t write_index) {
  if (!zlib().ok) {
    h->err = "BAM output needs libz.so.1";
    return PBW_ERR_IO;
  }
  if (write_index && !opt->coordinate_sorted) {
    h->err = "pbw_bam_write: an index needs coordinate-sorted records (coordinate_sorted = 1)";
    return PBW_ERR_ARG;
  }
  // the SAM stream, formatted on the device
  uint64_t len = 0;
  int rc = pbw_sam_format(h, opt, n_src, src, sel, n_sel, nullptr, 0, &len);
  if (rc != PBW_OK) return rc;
  std::vector<char> text(len + 1);
  rc = pbw_sam_format(h, opt, n_src, src, sel, n_sel, text.data(), len, &len);
  if (rc != PBW_OK) return rc;
  std::string err;
  rc = bam_from_text(text.data(), len, h->names, h->lens, path, write_index != 0, err);
  if (rc != PBW_OK) h->err = err;
  return rc;
}

int bam_write_text(const char* sam, uint64_t len, const char* path, int32_t write_index) {
  if (!zlib().ok) {
    pbw::set_handleless_error("BAM output needs libz.so.1");
    return PBW_ERR_IO;
  }
  std::string so, err;
  std::vector<std::string> names;
  std::vector<uint64_t> lens;
  if (!parse_sam_header(sam, (size_t)len, so, names, lens, err)) {
    pbw::set_handleless_error(err);
    return PBW_ERR_FORMAT;
  }
  if (write_index && so != "coordinate") {
    pbw::set_handleless_error("pbw_bam_write_text: an index needs a coordinate-sorted stream (@HD SO:coordinate)");
    return PBW_ERR_ARG;
  }
  const int rc = bam_from_text(sam, (size_t)len, names, lens, path, write_index != 0, err);
  if (rc != PBW_OK) pbw::set_handleless_error(err);
  return rc;
}

}  // namespace

extern "C" int pbw_bam_write(pbw_handle* h, const pbw_sam_options* opt, uint32_t n_src, const pbw_sam_source* src,
                             const uint64_t* sel, uint64_t n_sel, const char* path, int32_t write_index) {
  if (!h || !opt || !path) return PBW_ERR_ARG;
  return pbw::guarded("pbw_bam_write", [h](const std::string& m) { h->err = m; },
                      [&] { return bam_write(h, opt, n_src, src, sel, n_sel, path, write_index); });
}

extern "C" int pbw_bam_write_text(const char* sam, uint64_t len, const char* path, int32_t write_index) {
  if (!sam || !path) {
    pbw::set_handleless_error("pbw_bam_write_text: NULL text or path");
    return PBW_ERR_ARG;
  }
  return pbw::guard_handleless("pbw_bam_write_text", [&] { return bam_write_text(sam, len, path, write_index); });
}
