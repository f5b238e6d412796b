// fastx_text.h -- text input shared by the reads loader (fastx.cpp) and the
// genome builder (genome_build.cpp): whole-file reads, gzip members,
// UTF-8 checks, lines and the whitespace rules of Rust's str::trim /
// split_whitespace (src/io/fastx.rs, src/index/genome.rs).
#pragma once
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <dlfcn.h>
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include "../../include/probebwa_gpu.h"

namespace pbw {
namespace text {

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
inline Span trim(Span s) {
  size_t k;
  while (s.n && (k = ws_head(s.p, s.n)) > 0) { s.p += k; s.n -= k; }
  while (s.n && (k = ws_tail(s.p, s.n)) > 0) s.n -= k;
  return s;
}
// The first split_whitespace token (empty when the span is all whitespace).
inline Span first_token(Span s) {
  size_t a = 0, k;
  while (a < s.n && (k = ws_head(s.p + a, s.n - a)) > 0) a += k;
  size_t b = a;
  while (b < s.n && ws_head(s.p + b, s.n - b) == 0) b++;
  return Span{s.p + a, b - a};
}
// std::str::from_utf8 acceptance: well-formed UTF-8 (no overlong forms,
// surrogates or code points above U+10FFFF).
inline bool valid_utf8(const char* s, size_t n) {
  size_t i = 0;
  while (i < n) {
    // runs of ASCII 8 bytes at a time (whole characters: i stays on a boundary)
    while (i + 8 <= n) {
      uint64_t w;
      memcpy(&w, s + i, 8);
      if (w & 0x8080808080808080ull) break;
      i += 8;
    }
    if (i >= n) break;
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
inline Span strip_leading(Span s, char c) {
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


inline bool read_file(const char* path, std::vector<char>& buf) {
  FILE* f = fopen(path, "rb");
  if (!f) return false;
  // one read of the whole file when its size is known, then whatever follows
  if (fseeko(f, 0, SEEK_END) == 0) {
    const off_t sz = ftello(f);
    if (sz > 0 && fseeko(f, 0, SEEK_SET) == 0) {
      buf.resize((size_t)sz);
      buf.resize(fread(buf.data(), 1, (size_t)sz, f));
    } else {
      fseeko(f, 0, SEEK_SET);
    }
  }
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
inline bool gunzip(const std::vector<char>& in, std::vector<char>& out, std::string& err) {
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

inline bool ends_with_gz(const char* path) {
  const size_t n = strlen(path);
  // Path::extension() == "gz": the file name ends in ".gz" and is not ".gz" itself
  if (n < 3 || strcmp(path + n - 3, ".gz") != 0) return false;
  const char* base = strrchr(path, '/');
  base = base ? base + 1 : path;
  return strlen(base) > 3;
}

// The text of a file: a regular file is mapped read-only (no copy of its
// bytes); anything else (a pipe, an empty file, a map that fails) and gzip
// input is read or decoded into owned memory.
class Text {
 public:
  Text() = default;
  Text(const Text&) = delete;
  Text& operator=(const Text&) = delete;
  ~Text() { unmap(); }
  const char* data() const { return p_; }
  size_t size() const { return n_; }
  bool map(const char* path) {
    const int fd = open(path, O_RDONLY);
    if (fd < 0) return false;
    struct stat st;
    void* m = MAP_FAILED;
    if (fstat(fd, &st) == 0 && S_ISREG(st.st_mode) && st.st_size > 0)
      m = mmap(nullptr, (size_t)st.st_size, PROT_READ, MAP_PRIVATE | MAP_POPULATE, fd, 0);
    close(fd);
    if (m == MAP_FAILED) return false;
    map_ = m;
    map_len_ = (size_t)st.st_size;
    p_ = (const char*)m;
    n_ = map_len_;
    return true;
  }
  std::vector<char>& own() {
    unmap();
    p_ = own_.data();
    n_ = own_.size();
    return own_;
  }
  void adopt() {  // after filling own()
    p_ = own_.data();
    n_ = own_.size();
  }

 private:
  void unmap() {
    if (map_) munmap(map_, map_len_);
    map_ = nullptr;
  }
  const char* p_ = nullptr;
  size_t n_ = 0;
  std::vector<char> own_;
  void* map_ = nullptr;
  size_t map_len_ = 0;
};

// The whole text of path, gunzipped when the name ends in ".gz", checked to
// be UTF-8. PBW_OK, or PBW_ERR_IO / PBW_ERR_FORMAT with a message in err.
inline int load_text(const char* path, Text& text, std::string& err) {
  if (ends_with_gz(path)) {
    std::vector<char> raw;
    if (!read_file(path, raw)) {
      err = std::string("cannot open ") + path;
      return PBW_ERR_IO;
    }
    std::string e;
    if (!gunzip(raw, text.own(), e)) {
      err = std::string(path) + ": " + e;
      return PBW_ERR_IO;
    }
    text.adopt();
  } else if (!text.map(path)) {
    if (!read_file(path, text.own())) {
      err = std::string("cannot open ") + path;
      return PBW_ERR_IO;
    }
    text.adopt();
  }
  if (!valid_utf8(text.data(), text.size())) {
    err = std::string(path) + ": stream did not contain valid UTF-8";
    return PBW_ERR_FORMAT;
  }
  return PBW_OK;
}

}  // namespace text
}  // namespace pbw
