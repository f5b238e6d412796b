// fastx.cpp -- the input side of the mapping path: FASTQ / FASTA reads into
// the structure-of-arrays layout the map calls take (src/io/fastx.rs).
//
// The file is read into memory once (gunzipped when its name ends in ".gz",
// as open_maybe_gz, fastx.rs:120-129, with every gzip member decoded in turn
// like flate2's MultiGzDecoder) and split into lines with memchr; each record
// is decoded straight into the concatenated base, quality and offset arrays.
// Semantics follow the reference's parsers:
//  * the text must be UTF-8 (each line goes through BufRead::read_line into
//    a String); anything else is an error, as there;
//  * FASTQ (FastqParser, fastx.rs:226-305): ID = first whitespace-separated
//    token of the header line after leading '@'s; sequence lines (trimmed)
//    until a trimmed line starting with '+'; then quality lines (trimmed) until
//    they cover the sequence, at least one line. Bases are upper-cased
//    (DnaSeq::from_ascii, types.rs:12-15), qualities are the byte minus the
//    offset, saturating at 0 (QualityScores::from_phred_ascii, types.rs:57-60);
//  * FASTA reads (FastaAsReadsParser, fastx.rs:161-224): records start at a
//    line beginning with '>' (lines before the first are skipped); ID = first
//    token after leading '>'s; sequence = concatenated trimmed lines up to a
//    trimmed line starting with '>'; every quality 40 (fastx.rs:159);
//  * then per read: a trailing "/1" or "/2" is dropped from the ID
//    (strip_mate_suffix, fastx.rs:77-81) and, with an adapter, the longest
//    3' overlap of at least 6 bases with at most one mismatch per 10 bases
//    (case-insensitive) is cut from the bases and qualities (strip_adapter,
//    fastx.rs:97-117).
// Whitespace (str::trim, str::split_whitespace) is Unicode White_Space: the
// ASCII tab, LF, VT, FF, CR and space, and U+0085, U+00A0, U+1680,
// U+2000-U+200A, U+2028, U+2029, U+202F, U+205F, U+3000 in their UTF-8
// forms. The quality track handed to the map calls has the sequence's
// length: missing scores read as 30, extra ones are dropped.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <dlfcn.h>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_kernels.h"

struct pbw_read_set {
  std::vector<uint8_t> bases, quals;
  std::vector<uint64_t> offsets{0};
  std::vector<char> id_chars;  // NUL-terminated IDs, back to back
  std::vector<uint64_t> id_off;
};

namespace {

inline uint8_t upper(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }

struct Span {
  const char* p;
  size_t n;
};

// Byte length of the White_Space character starting at p[0] (0: none).
inline size_t ws_head(const char* p, size_t n) {
  const uint8_t c = (uint8_t)p[0];
  if (c == ' ' || (c >= 9 && c <= 13)) return 1;
  if (n >= 2 && c == 0xC2 && ((uint8_t)p[1] == 0x85 || (uint8_t)p[1] == 0xA0)) return 2;
  if (n >= 3 && c >= 0xE1 && c <= 0xE3) {
    const uint8_t b = (uint8_t)p[1], d = (uint8_t)p[2];
    if (c == 0xE1) return (b == 0x9A && d == 0x80) ? 3 : 0;  // U+1680
    if (c == 0xE3) return (b == 0x80 && d == 0x80) ? 3 : 0;  // U+3000
    if (b == 0x80 && (d <= 0x8A || d == 0xA8 || d == 0xA9 || d == 0xAF) && d >= 0x80) return 3;
    if (b == 0x81 && d == 0x9F) return 3;  // U+205F
  }
  return 0;
}
// Byte length of the White_Space character ending at p[n-1] (0: none). In
// valid UTF-8 a 2- or 3-byte match at the end is a whole character.
inline size_t ws_tail(const char* p, size_t n) {
  if (n == 0) return 0;
  const uint8_t c = (uint8_t)p[n - 1];
  if (c < 0x80) return (c == ' ' || (c >= 9 && c <= 13)) ? 1 : 0;
  if (n >= 2 && ws_head(p + n - 2, 2) == 2) return 2;
  if (n >= 3 && ws_head(p + n - 3, 3) == 3) return 3;
  return 0;
}
Span trim(Span s) {
  size_t k;
  while (s.n && (k = ws_head(s.p, s.n)) > 0) { s.p += k; s.n -= k; }
  while (s.n && (k = ws_tail(s.p, s.n)) > 0) s.n -= k;
  return s;
}
// The first split_whitespace token (empty when the span is all whitespace).
Span first_token(Span s) {
  size_t a = 0, k;
  while (a < s.n && (k = ws_head(s.p + a, s.n - a)) > 0) a += k;
  size_t b = a;
  while (b < s.n && ws_head(s.p + b, s.n - b) == 0) b++;
  return Span{s.p + a, b - a};
}
// std::str::from_utf8 acceptance: well-formed UTF-8 (no overlong forms,
// surrogates or code points above U+10FFFF).
bool valid_utf8(const char* s, size_t n) {
  size_t i = 0;
  while (i < n) {
    const uint8_t c = (uint8_t)s[i];
    if (c < 0x80) { i++; continue; }
    size_t need;
    uint8_t lo = 0x80, hi = 0xBF;
    if (c >= 0xC2 && c <= 0xDF) need = 1;
    else if (c == 0xE0) { need = 2; lo = 0xA0; }
    else if ((c >= 0xE1 && c <= 0xEC) || c == 0xEE || c == 0xEF) need = 2;
    else if (c == 0xED) { need = 2; hi = 0x9F; }
    else if (c == 0xF0) { need = 3; lo = 0x90; }
    else if (c >= 0xF1 && c <= 0xF3) need = 3;
    else if (c == 0xF4) { need = 3; hi = 0x8F; }
    else return false;
    for (size_t j = 1; j <= need; j++) {
      if (i + j >= n) return false;
      const uint8_t cc = (uint8_t)s[i + j];
      if (cc < (j == 1 ? lo : 0x80) || cc > (j == 1 ? hi : 0xBF)) return false;
    }
    i += need + 1;
  }
  return true;
}
Span strip_leading(Span s, char c) {
  while (s.n && s.p[0] == c) { s.p++; s.n--; }
  return s;
}

// Lines of a buffer; a line keeps its '\n' (as BufRead::read_line).
struct Lines {
  const char* p;
  const char* end;
  bool next(Span& line) {
    if (p >= end) return false;
    const char* nl = (const char*)memchr(p, '\n', (size_t)(end - p));
    const char* e = nl ? nl + 1 : end;
    line = Span{p, (size_t)(e - p)};
    p = e;
    return true;
  }
};

struct Builder {
  pbw_read_set* rs;
  void add(Span id) {
    // strip_mate_suffix
    if (id.n >= 2 && id.p[id.n - 2] == '/' && (id.p[id.n - 1] == '1' || id.p[id.n - 1] == '2')) id.n -= 2;
    rs->id_off.push_back(rs->id_chars.size());
    rs->id_chars.insert(rs->id_chars.end(), id.p, id.p + id.n);
    rs->id_chars.push_back('\0');
  }
};

// strip_adapter: returns the number of bases to keep.
size_t adapter_keep(const uint8_t* seq, size_t rl, const std::string& ad) {
  const size_t mo = std::min(rl, ad.size());
  if (mo < 6) return rl;
  for (size_t ov = mo; ov >= 6; ov--) {
    size_t mm = 0;
    for (size_t t = 0; t < ov; t++) mm += upper(seq[rl - ov + t]) != upper((uint8_t)ad[t]) ? 1 : 0;
    if (mm <= ov / 10) return rl - ov;
  }
  return rl;
}

// Appends one read: bases upper-cased, the quality track cut or padded to the
// (possibly adapter-trimmed) sequence length.
void push_read(pbw_read_set* rs, const std::vector<uint8_t>& seq, const std::vector<uint8_t>& qual, const char* adapter) {
  size_t keep = seq.size();
  if (adapter) keep = adapter_keep(seq.data(), seq.size(), adapter);
  for (size_t t = 0; t < keep; t++) {
    rs->bases.push_back(upper(seq[t]));
    rs->quals.push_back(t < qual.size() ? qual[t] : (uint8_t)30);
  }
  rs->offsets.push_back(rs->bases.size());
}

bool read_file(const char* path, std::vector<char>& buf) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  char tmp[1 << 16];
  size_t n;
  while ((n = fread(tmp, 1, sizeof(tmp), f)) > 0) buf.insert(buf.end(), tmp, tmp + n);
  fclose(f);
  return true;
}

// zlib's stream state (the z_stream of its public API, LP64 layout); the
// library is opened at run time so the build needs no zlib headers.
struct ZStream {
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

// Decodes every gzip member of in (MultiGzDecoder); false with a message on
// a missing zlib or corrupt data.
bool gunzip(const std::vector<char>& in, std::vector<char>& out, std::string& err) {
  static void* lib = dlopen("libz.so.1", RTLD_NOW | RTLD_LOCAL);
  if (!lib) {
    err = "gzip input needs libz.so.1";
    return false;
  }
  using VersionFn = const char* (*)();
  using InitFn = int (*)(ZStream*, int, const char*, int);
  using StepFn = int (*)(ZStream*, int);
  using EndFn = int (*)(ZStream*);
  auto version = (VersionFn)dlsym(lib, "zlibVersion");
  auto init = (InitFn)dlsym(lib, "inflateInit2_");
  auto step = (StepFn)dlsym(lib, "inflate");
  auto reset = (EndFn)dlsym(lib, "inflateReset");
  auto end = (EndFn)dlsym(lib, "inflateEnd");
  if (!version || !init || !step || !reset || !end) {
    err = "libz.so.1 lacks the inflate entry points";
    return false;
  }
  if (in.empty()) return true;
  ZStream z;
  memset(&z, 0, sizeof(z));
  if (init(&z, 15 + 16, version(), (int)sizeof(ZStream)) != 0) {
    err = "inflateInit2 failed";
    return false;
  }
  z.next_in = (const unsigned char*)in.data();
  z.avail_in = 0;
  size_t fed = 0;
  std::vector<char> chunk(1 << 20);
  bool ok = true;
  while (true) {
    if (z.avail_in == 0 && fed < in.size()) {
      const size_t give = std::min<size_t>(in.size() - fed, 1u << 30);
      z.next_in = (const unsigned char*)in.data() + fed;
      z.avail_in = (unsigned)give;
      fed += give;
    }
    z.next_out = (unsigned char*)chunk.data();
    z.avail_out = (unsigned)chunk.size();
    const int rc = step(&z, 0);
    out.insert(out.end(), chunk.data(), chunk.data() + (chunk.size() - z.avail_out));
    if (rc == 1) {  // Z_STREAM_END: a member ended; decode the next one if bytes remain
      if (z.avail_in == 0 && fed == in.size()) break;
      reset(&z);
      continue;
    }
    if (rc == -5 && z.avail_in == 0 && fed == in.size()) {  // Z_BUF_ERROR at end: truncated stream
      ok = false;
      err = "corrupt deflate stream";
      break;
    }
    if (rc != 0 && rc != -5) {
      ok = false;
      err = z.msg ? z.msg : "corrupt deflate stream";
      break;
    }
  }
  end(&z);
  return ok;
}

bool ends_with_gz(const char* path) {
  const size_t n = strlen(path);
  // Path::extension() == "gz": the file name ends in ".gz" and is not ".gz" itself
  if (n < 3 || strcmp(path + n - 3, ".gz") != 0) return false;
  const char* base = strrchr(path, '/');
  base = base ? base + 1 : path;
  return strlen(base) > 3;
}

}  // namespace

namespace pbw {
void set_handleless_error(const std::string& s);
}

extern "C" {

int pbw_reads_load(const char* path, int fasta, uint8_t quality_offset, const char* adapter, pbw_read_set** out) {
  if (!path || !out) return PBW_ERR_ARG;
  *out = nullptr;
  std::vector<char> buf;
  if (!read_file(path, buf)) {
    pbw::set_handleless_error(std::string("cannot open ") + path);
    return PBW_ERR_IO;
  }
  if (ends_with_gz(path)) {
    std::vector<char> raw;
    raw.swap(buf);
    std::string err;
    if (!gunzip(raw, buf, err)) {
      pbw::set_handleless_error(std::string(path) + ": " + err);
      return PBW_ERR_IO;
    }
  }
  if (!valid_utf8(buf.data(), buf.size())) {
    pbw::set_handleless_error(std::string(path) + ": stream did not contain valid UTF-8");
    return PBW_ERR_FORMAT;
  }
  pbw_read_set* rs = new pbw_read_set();
  Builder bld{rs};
  Lines L{buf.data(), buf.data() + buf.size()};
  Span line;
  std::vector<uint8_t> seq, qual;
  if (!fasta) {
    while (L.next(line)) {
      bld.add(first_token(strip_leading(line, '@')));
      seq.clear();
      qual.clear();
      while (L.next(line)) {
        const Span t = trim(line);
        if (t.n && t.p[0] == '+') break;
        seq.insert(seq.end(), (const uint8_t*)t.p, (const uint8_t*)t.p + t.n);
      }
      while (L.next(line)) {
        const Span t = trim(line);
        for (size_t k = 0; k < t.n; k++) {
          const uint8_t c = (uint8_t)t.p[k];
          qual.push_back(c > quality_offset ? (uint8_t)(c - quality_offset) : (uint8_t)0);
        }
        if (qual.size() >= seq.size()) break;
      }
      push_read(rs, seq, qual, adapter);
    }
  } else {
    bool have = false;
    Span header{nullptr, 0};
    while (true) {
      if (!have) {
        bool found = false;
        while (L.next(line))
          if (line.n && line.p[0] == '>') { found = true; break; }
        if (!found) break;
        header = line;
      }
      have = false;
      bld.add(first_token(strip_leading(header, '>')));
      seq.clear();
      while (L.next(line)) {
        const Span t = trim(line);
        if (t.n && t.p[0] == '>') {
          header = line;
          have = true;
          break;
        }
        seq.insert(seq.end(), (const uint8_t*)t.p, (const uint8_t*)t.p + t.n);
      }
      qual.assign(seq.size(), 40);
      push_read(rs, seq, qual, adapter);
      if (!have) break;
    }
  }
  *out = rs;
  return PBW_OK;
}

int pbw_reads_get(const pbw_read_set* rs, pbw_reads* view) {
  if (!rs || !view) return PBW_ERR_ARG;
  view->n = rs->offsets.size() - 1;
  view->bases = rs->bases.data();
  view->quals = rs->quals.data();
  view->offsets = rs->offsets.data();
  return PBW_OK;
}

const char* pbw_reads_id(const pbw_read_set* rs, uint64_t i) {
  if (!rs || i >= rs->id_off.size()) return nullptr;
  return rs->id_chars.data() + rs->id_off[i];
}

void pbw_reads_free(pbw_read_set* rs) { delete rs; }

}  // extern "C"
