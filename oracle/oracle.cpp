// oracle.cpp -- CPU restatement of probebwa's read-mapping path.
//
// TEST INFRASTRUCTURE ONLY (see oracle.h): the correctness oracle and the
// timed CPU baseline. Every function cites the reference file:line whose
// behaviour it restates. Compile with -ffp-contract=off: the reference is
// Rust, which never contracts a*b+c into an FMA.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <utility>
#include <vector>

#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

namespace orc {

using u8 = uint8_t;
using u16 = uint16_t;
using u32 = uint32_t;
using u64 = uint64_t;
using i32 = int32_t;
using i64 = int64_t;

static thread_local std::string g_err;

// ---------------------------------------------------------------------------
// Core types (src/types.rs)
// ---------------------------------------------------------------------------
enum Strand : u8 { FWD = 0, REV = 1 };

// CigarOp (src/types.rs:169-175). op: 'M','I','D','S','H'.
struct Cig {
  char op;
  u32 n;
};

struct Read {
  std::string id;
  std::vector<u8> bases;  // uppercased (DnaSeq::from_ascii, types.rs:12-15)
  std::vector<u8> quals;  // Phred scores (QualityScores, types.rs:57-60)
};

// DnaSeq::reverse_complement (src/types.rs:34-48): non-ACGT -> 'N'.
static std::vector<u8> revcomp(const std::vector<u8>& s) {
  std::vector<u8> rc;
  rc.reserve(s.size());
  for (size_t i = s.size(); i-- > 0;) {
    u8 b = s[i];
    u8 c;
    switch (b) {
      case 'A': c = 'T'; break;
      case 'T': c = 'A'; break;
      case 'C': c = 'G'; break;
      case 'G': c = 'C'; break;
      default: c = 'N'; break;
    }
    rc.push_back(c);
  }
  return rc;
}

static inline u8 ascii_upper(u8 b) { return (b >= 'a' && b <= 'z') ? (u8)(b - 32) : b; }

// ---------------------------------------------------------------------------
// bincode 1.3.3 legacy encoding (fixint, little-endian, u64 lengths)
// ---------------------------------------------------------------------------
struct BinWriter {
  std::vector<u8> buf;
  void u32v(u32 v) { for (int i = 0; i < 4; i++) buf.push_back((u8)(v >> (8 * i))); }
  void u64v(u64 v) { for (int i = 0; i < 8; i++) buf.push_back((u8)(v >> (8 * i))); }
  void str(const std::string& s) { u64v(s.size()); buf.insert(buf.end(), s.begin(), s.end()); }
  void bytes(const std::vector<u8>& b) { u64v(b.size()); buf.insert(buf.end(), b.begin(), b.end()); }
  bool save(const std::string& path) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) return false;
    bool ok = fwrite(buf.data(), 1, buf.size(), f) == buf.size();
    fclose(f);
    return ok;
  }
};

struct BinReader {
  std::vector<u8> data;
  size_t p = 0;
  bool load(const std::string& path) {
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    data.resize((size_t)sz);
    bool ok = fread(data.data(), 1, data.size(), f) == data.size();
    fclose(f);
    return ok;
  }
  void need(size_t n) {
    if (p + n > data.size()) throw std::runtime_error("bincode: unexpected end of file");
  }
  u32 u32v() { need(4); u32 v; memcpy(&v, &data[p], 4); p += 4; return v; }
  u64 u64v() { need(8); u64 v; memcpy(&v, &data[p], 8); p += 8; return v; }
  std::string str() { u64 n = u64v(); need(n); std::string s((const char*)&data[p], n); p += n; return s; }
  std::vector<u8> bytes() { u64 n = u64v(); need(n); std::vector<u8> b(data.begin() + p, data.begin() + p + n); p += n; return b; }
};

// ---------------------------------------------------------------------------
// Genome index (src/index/genome.rs, Contig in src/types.rs:107-112)
// ---------------------------------------------------------------------------
struct Contig {
  std::string name;
  std::vector<u8> packed;
  std::vector<std::pair<u32, u32>> n_runs;
  u64 length = 0;

  // Contig::from_ascii (src/index/genome.rs:17-45).
  static Contig from_ascii(const std::string& name, const u8* seq, u64 len) {
    Contig c;
    c.name = name;
    c.length = len;
    c.packed.assign((len + 3) / 4, 0);
    bool in_run = false;
    u64 run_start = 0;
    for (u64 pos = 0; pos < len; pos++) {
      u8 b = seq[pos];
      u8 bits = 0;
      bool acgt = true;
      switch (b) {
        case 'A': case 'a': bits = 0; break;
        case 'C': case 'c': bits = 1; break;
        case 'G': case 'g': bits = 2; break;
        case 'T': case 't': bits = 3; break;
        default: acgt = false; break;
      }
      c.packed[pos / 4] |= (u8)(bits << ((pos % 4) * 2));
      if (acgt) {
        if (in_run) { c.n_runs.push_back({(u32)run_start, (u32)pos}); in_run = false; }
      } else if (!in_run) {
        in_run = true;
        run_start = pos;
      }
    }
    if (in_run) c.n_runs.push_back({(u32)run_start, (u32)len});
    return c;
  }

  // Contig::slice (src/index/genome.rs:48-68): 2-bit decode of [start, end)
  // then overlay 'N' on every n_run.
  std::vector<u8> slice(u64 start, u64 end) const {
    static const u8 BITS2BASE[4] = {'A', 'C', 'G', 'T'};
    start = std::min(start, length);
    end = std::min(end, length);
    std::vector<u8> out;
    if (start >= end) return out;
    out.reserve(end - start);
    for (u64 pos = start; pos < end; pos++) {
      u8 byte = packed[pos / 4];
      out.push_back(BITS2BASE[(byte >> ((pos % 4) * 2)) & 3]);
    }
    for (auto& r : n_runs) {
      u64 os = std::max((u64)r.first, start);
      u64 oe = std::min((u64)r.second, end);
      for (u64 p = os; p < oe; p++) out[p - start] = 'N';
    }
    return out;
  }
};

struct Genome {
  std::string species, assembly;
  std::vector<Contig> contigs;
  u64 total_length = 0;

  // GenomeIndex::save (src/index/genome.rs:88-94): bincode of
  // {species, assembly, contigs: Vec<{name, packed, n_runs, length}>, total_length}.
  bool save(const std::string& prefix) const {
    BinWriter w;
    w.str(species);
    w.str(assembly);
    w.u64v(contigs.size());
    for (auto& c : contigs) {
      w.str(c.name);
      w.bytes(c.packed);
      w.u64v(c.n_runs.size());
      for (auto& r : c.n_runs) { w.u32v(r.first); w.u32v(r.second); }
      w.u64v(c.length);
    }
    w.u64v(total_length);
    return w.save(prefix + ".stidx");
  }

  // GenomeIndex::load (src/index/genome.rs:80-86).
  bool load(const std::string& prefix) {
    BinReader r;
    if (!r.load(prefix + ".stidx")) { g_err = "cannot open " + prefix + ".stidx"; return false; }
    try {
      species = r.str();
      assembly = r.str();
      u64 nc = r.u64v();
      contigs.resize(nc);
      for (auto& c : contigs) {
        c.name = r.str();
        c.packed = r.bytes();
        u64 nr = r.u64v();
        c.n_runs.resize(nr);
        for (auto& x : c.n_runs) { x.first = r.u32v(); x.second = r.u32v(); }
        c.length = r.u64v();
      }
      total_length = r.u64v();
    } catch (std::exception& e) {
      g_err = e.what();
      return false;
    }
    return true;
  }
};

// Minimal FASTA reader (src/index/genome.rs:150-213): headers carried over
// between records, id = first whitespace token after the leading '>'s,
// sequence lines trimmed and concatenated.
// Whitespace is Unicode White_Space, as str::trim / split_whitespace: ASCII
// 9-13 and 32, and U+0085 U+00A0 U+1680 U+2000-200A U+2028 U+2029 U+202F
// U+205F U+3000 in UTF-8. ws_head / ws_tail give the byte length of such a
// character starting at s[i] / ending at s[e-1] (0: none).
static size_t ws_head(const std::string& s, size_t i) {
  const u8 c = (u8)s[i];
  if (c == ' ' || (c >= 9 && c <= 13)) return 1;
  const size_t left = s.size() - i;
  if (left >= 2 && c == 0xC2 && ((u8)s[i + 1] == 0x85 || (u8)s[i + 1] == 0xA0)) return 2;
  if (left >= 3) {
    const uint32_t cp = ((uint32_t)c << 16) | ((uint32_t)(u8)s[i + 1] << 8) | (u8)s[i + 2];
    if (cp == 0xE19A80 || cp == 0xE38080 || cp == 0xE2819F) return 3;
    if (cp >= 0xE28080 && cp <= 0xE2808A) return 3;
    if (cp == 0xE280A8 || cp == 0xE280A9 || cp == 0xE280AF) return 3;
  }
  return 0;
}
static size_t ws_tail(const std::string& s, size_t a, size_t e) {
  for (size_t k = 1; k <= 3 && k <= e - a; k++)
    if (ws_head(s, e - k) == k && (k == 1 || (u8)s[e - k] >= 0xC0)) return k;
  return 0;
}
static std::string trim(const std::string& s) {
  size_t a = 0, b = s.size(), k;
  while (a < b && (k = ws_head(s, a)) > 0) a += k;
  while (b > a && (k = ws_tail(s, a, b)) > 0) b -= k;
  return s.substr(a, b - a);
}
static std::string first_token(const std::string& s) {
  size_t a = 0, k;
  while (a < s.size() && (k = ws_head(s, a)) > 0) a += k;
  size_t b = a;
  while (b < s.size() && ws_head(s, b) == 0) b++;
  return s.substr(a, b - a);
}
// str::from_utf8 acceptance (read_line into a String rejects anything else).
static bool utf8_ok(const std::string& s) {
  size_t i = 0;
  const size_t n = s.size();
  while (i < n) {
    const u8 c = (u8)s[i];
    size_t need = 0;
    u8 lo = 0x80, hi = 0xBF;
    if (c < 0x80) { i++; continue; }
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
      const u8 cc = (u8)s[i + j];
      if (cc < (j == 1 ? lo : 0x80) || cc > (j == 1 ? hi : 0xBF)) return false;
    }
    i += need + 1;
  }
  return true;
}
static std::string trim_start_char(const std::string& s, char c) {
  size_t a = 0;
  while (a < s.size() && s[a] == c) a++;
  return s.substr(a);
}

struct LineReader {
  FILE* f = nullptr;
  explicit LineReader(const std::string& path) { f = fopen(path.c_str(), "rb"); }
  ~LineReader() { if (f) fclose(f); }
  // Returns false at EOF (0 bytes read). The line keeps its '\n'. A line
  // that is not UTF-8 throws, as BufRead::read_line into a String fails.
  bool read_line(std::string& line) {
    line.clear();
    int ch;
    bool any = false;
    while ((ch = fgetc(f)) != EOF) {
      any = true;
      line.push_back((char)ch);
      if (ch == '\n') break;
    }
    if (any && !utf8_ok(line)) throw std::runtime_error("stream did not contain valid UTF-8");
    return any;
  }
};

struct FastaRecord { std::string id; std::vector<u8> seq; };

static std::vector<FastaRecord> read_fasta_records(const std::string& path) {
  std::vector<FastaRecord> out;
  LineReader lr(path);
  if (!lr.f) throw std::runtime_error("cannot open " + path);
  std::string line, pending;
  bool have_pending = false;
  while (true) {
    std::string header;
    if (have_pending) {
      header = pending;
      have_pending = false;
    } else {
      bool found = false;
      while (lr.read_line(line)) {
        if (!line.empty() && line[0] == '>') { found = true; break; }
      }
      if (!found) break;
      header = line;
    }
    FastaRecord rec;
    rec.id = first_token(trim_start_char(header, '>'));
    while (lr.read_line(line)) {
      std::string t = trim(line);
      if (!t.empty() && t[0] == '>') { pending = line; have_pending = true; break; }
      rec.seq.insert(rec.seq.end(), t.begin(), t.end());
    }
    out.push_back(std::move(rec));
  }
  return out;
}

// ---------------------------------------------------------------------------
// 15-mer hash table (src/index/hashtable.rs)
// ---------------------------------------------------------------------------
static const u64 POSITION_BITS = 40;
static const u64 POSITION_MASK = (1ull << 40) - 1;
static const u64 CONTIG_MASK = (1ull << 23) - 1;

// base2bits (hashtable.rs:126-134): non-ACGT maps to 0 like 'A'.
static inline u32 base2bits(u8 b) {
  switch (b) {
    case 'A': case 'a': return 0;
    case 'C': case 'c': return 1;
    case 'G': case 'g': return 2;
    case 'T': case 't': return 3;
    default: return 0;
  }
}
// mix (hashtable.rs:117-124): multiply-xor-shift finaliser, a bijection.
static inline u32 mix32(u32 h) {
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return h;
}
// hash_kmer (hashtable.rs:107-113): first 15 bases, first base most significant.
static inline u32 hash_kmer(const u8* kmer, size_t len) {
  u32 raw = 0;
  size_t n = len < 15 ? len : 15;
  for (size_t i = 0; i < n; i++) raw = (raw << 2) | base2bits(kmer[i]);
  return mix32(raw);
}
// is_acgt_only (hashtable.rs:147-149).
static inline bool is_acgt_only(const u8* p, size_t n) {
  for (size_t i = 0; i < n; i++) {
    switch (p[i]) {
      case 'A': case 'a': case 'C': case 'c': case 'G': case 'g': case 'T': case 't': break;
      default: return false;
    }
  }
  return true;
}
// pack_position / unpack_position (hashtable.rs:157-171).
static inline u64 pack_position(u64 contig, u64 pos, Strand s) {
  return ((u64)(s == REV ? 1 : 0) << 63) | ((contig & CONTIG_MASK) << POSITION_BITS) | (pos & POSITION_MASK);
}
static inline void unpack_position(u64 p, u64& contig, u64& pos, Strand& s) {
  s = ((p >> 63) & 1) ? REV : FWD;
  contig = (p >> POSITION_BITS) & CONTIG_MASK;
  pos = p & POSITION_MASK;
}

// Open-addressed u32 -> (offset, count) map standing in for the
// FxHashMap<u32, (u32, u32)> of hashtable.rs:62 (lookup semantics only).
struct FlatTable {
  std::vector<u32> keys;
  std::vector<std::pair<u32, u32>> vals;
  std::vector<u8> used;
  u64 mask = 0;
  void init(u64 n) {
    u64 cap = 16;
    while (cap < n * 2 + 16) cap <<= 1;
    keys.assign(cap, 0);
    vals.assign(cap, {0, 0});
    used.assign(cap, 0);
    mask = cap - 1;
  }
  static inline u64 slot_of(u32 k) { return (u64)k * 0x9E3779B97F4A7C15ull >> 20; }
  void insert(u32 k, std::pair<u32, u32> v) {
    u64 s = slot_of(k) & mask;
    while (used[s] && keys[s] != k) s = (s + 1) & mask;
    used[s] = 1; keys[s] = k; vals[s] = v;
  }
  inline const std::pair<u32, u32>* get(u32 k) const {
    u64 s = slot_of(k) & mask;
    while (used[s]) {
      if (keys[s] == k) return &vals[s];
      s = (s + 1) & mask;
    }
    return nullptr;
  }
};

// A read-only view of a whole file (mmap).
struct MappedFile {
  const u8* p = nullptr;
  size_t n = 0;
  bool open(const std::string& path) {
    int fd = ::open(path.c_str(), O_RDONLY);
    if (fd < 0) return false;
    struct stat st;
    if (fstat(fd, &st) != 0) { ::close(fd); return false; }
    n = (size_t)st.st_size;
    void* m = n ? mmap(nullptr, n, PROT_READ, MAP_PRIVATE, fd, 0) : nullptr;
    ::close(fd);
    if (n && m == MAP_FAILED) { n = 0; return false; }
    p = (const u8*)m;
    return true;
  }
  ~MappedFile() { if (p) munmap((void*)p, n); }
};

// Direct-address table over the 32-bit hash: word = (count << 32) | offset,
// count 0 = no bucket. Used for tables too large for FlatTable's single-thread
// build (a 3.1 Gbp genome has ~7e8 buckets); an anonymous mapping, so only
// the pages of present keys are ever touched.
struct DenseMap {
  static constexpr size_t BYTES = sizeof(u64) << 32;
  u64* w = nullptr;
  bool init() {
    void* m = mmap(nullptr, BYTES, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS | MAP_NORESERVE, -1, 0);
    if (m == MAP_FAILED) return false;
    w = (u64*)m;
    return true;
  }
  DenseMap() = default;
  DenseMap(const DenseMap&) = delete;
  DenseMap& operator=(const DenseMap&) = delete;
  DenseMap(DenseMap&& o) noexcept : w(o.w) { o.w = nullptr; }
  DenseMap& operator=(DenseMap&& o) noexcept { std::swap(w, o.w); return *this; }
  ~DenseMap() { if (w) munmap(w, BYTES); }
};

template <class F>
static void on_threads(size_t n, F f) {
  unsigned t = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if (n < (1u << 20)) t = 1;
  std::vector<std::thread> th;
  for (unsigned k = 0; k < t; k++) th.emplace_back([&, k] { f(n * k / t, n * (k + 1) / t); });
  for (auto& x : th) x.join();
}

struct HashTable {
  FlatTable table;
  DenseMap dense;  // instead of table for large loaded files
  std::vector<u64> positions;
  u64 k = 15, seed_stride = 5, total_entries = 0;
  // In-file entry order, kept for save() (tables built or loaded through
  // FlatTable).
  std::vector<std::pair<u32, std::pair<u32, u32>>> entries;

  // HashTable::lookup / get (hashtable.rs:90-102).
  inline void lookup(const u8* kmer, size_t len, const u64*& ptr, u64& cnt) const {
    const u32 key = hash_kmer(kmer, len);
    if (dense.w) {
      const u64 v = dense.w[key];
      cnt = v >> 32;
      ptr = cnt ? positions.data() + (u32)v : nullptr;
      return;
    }
    const std::pair<u32, u32>* v = table.get(key);
    if (!v) { ptr = nullptr; cnt = 0; return; }
    ptr = positions.data() + v->first;
    cnt = v->second;
  }

  // HashTable::save (hashtable.rs:81-87): bincode of {table, positions, k,
  // seed_stride, total_entries}. The map is written in the builder's
  // ascending-hash order (a map's content, not its order, is the format).
  bool save(const std::string& prefix) const {
    if (dense.w) { g_err = "save of a table loaded as a direct-address map"; return false; }
    BinWriter w;
    w.u64v(entries.size());
    for (auto& e : entries) { w.u32v(e.first); w.u32v(e.second.first); w.u32v(e.second.second); }
    w.u64v(positions.size());
    for (u64 p : positions) w.u64v(p);
    w.u64v(k);
    w.u64v(seed_stride);
    w.u64v(total_entries);
    return w.save(prefix + ".sthash");
  }

  // HashTable::load (hashtable.rs:73-79) over a mapping of the file.
  bool load(const std::string& prefix, u64 dense_min = 1ull << 24) {
    MappedFile f;
    if (!f.open(prefix + ".sthash")) { g_err = "cannot open " + prefix + ".sthash"; return false; }
    size_t p = 0;
    auto need = [&](size_t n) {
      if (p + n > f.n || p + n < p) throw std::runtime_error("bincode: unexpected end of file");
    };
    auto u64v = [&]() { need(8); u64 v; memcpy(&v, f.p + p, 8); p += 8; return v; };
    try {
      const u64 n = u64v();
      if (n > (f.n - p) / 12) throw std::runtime_error("bincode: unexpected end of file");
      const u8* tab = f.p + p;
      p += n * 12;
      const u64 np = u64v();
      if (np > (f.n - p) / 8) throw std::runtime_error("bincode: unexpected end of file");
      const u8* pos = f.p + p;
      p += np * 8;
      k = u64v();
      seed_stride = u64v();
      total_entries = u64v();
      positions.resize(np);
      on_threads(np, [&](size_t a, size_t b) { memcpy(positions.data() + a, pos + a * 8, (b - a) * 8); });
      auto entry = [&](size_t i, u32& key, u32& off, u32& cnt) {
        memcpy(&key, tab + 12 * i, 4);
        memcpy(&off, tab + 12 * i + 4, 4);
        memcpy(&cnt, tab + 12 * i + 8, 4);
      };
      std::atomic<bool> bad{false};
      if (n > dense_min) {
        if (!dense.init()) { g_err = "cannot map the direct-address table"; return false; }
        on_threads(n, [&](size_t a, size_t b) {
          for (size_t i = a; i < b; i++) {
            u32 key, off, cnt;
            entry(i, key, off, cnt);
            if ((u64)off + cnt > np || cnt == 0) bad = true;
            dense.w[key] = ((u64)cnt << 32) | off;
          }
        });
      } else {
        entries.resize(n);
        table.init(n);
        for (size_t i = 0; i < n; i++) {
          u32 key, off, cnt;
          entry(i, key, off, cnt);
          entries[i] = {key, {off, cnt}};
          table.insert(key, {off, cnt});
          if ((u64)off + cnt > np) bad = true;
        }
      }
      if (bad) { g_err = "sthash: bucket out of range"; return false; }
    } catch (std::exception& e) {
      g_err = e.what();
      return false;
    }
    return true;
  }
};

// HashTableBuilder::build (hashtable.rs:248-322): forward windows at
// i % stride == 0, then reverse-complement windows at rc index i % stride == 0
// stored at forward coordinate len-i-k; each hash keeps its first max_count
// occurrences in scan order; stable sort by hash; one contiguous run each.
static HashTable build_hash_table(const Genome& g, u64 k, u64 stride, u64 max_count) {
  std::vector<std::pair<u32, u64>> pairs;
  std::unordered_map<u32, u32> seen;
  for (size_t cid = 0; cid < g.contigs.size(); cid++) {
    const Contig& c = g.contigs[cid];
    std::vector<u8> seq = c.slice(0, c.length);
    if (seq.size() < k) continue;
    for (u64 i = 0; i + k <= seq.size(); i += stride) {
      const u8* km = &seq[i];
      if (!is_acgt_only(km, k)) continue;
      u32 h = hash_kmer(km, k);
      u32& cnt = seen[h];
      if (cnt < max_count) { pairs.push_back({h, pack_position(cid, i, FWD)}); cnt++; }
    }
    std::vector<u8> rc = revcomp(seq);
    for (u64 i = 0; i + k <= rc.size(); i += stride) {
      const u8* km = &rc[i];
      if (!is_acgt_only(km, k)) continue;
      u32 h = hash_kmer(km, k);
      u32& cnt = seen[h];
      if (cnt < max_count) { pairs.push_back({h, pack_position(cid, seq.size() - i - k, REV)}); cnt++; }
    }
  }
  std::stable_sort(pairs.begin(), pairs.end(),
                   [](const std::pair<u32, u64>& a, const std::pair<u32, u64>& b) { return a.first < b.first; });
  HashTable ht;
  ht.k = k;
  ht.seed_stride = stride;
  ht.positions.reserve(pairs.size());
  size_t i = 0;
  while (i < pairs.size()) {
    u32 h = pairs[i].first;
    size_t start = i;
    while (i < pairs.size() && pairs[i].first == h) i++;
    u32 off = (u32)ht.positions.size();
    for (size_t j = start; j < i; j++) ht.positions.push_back(pairs[j].second);
    ht.entries.push_back({h, {off, (u32)(i - start)}});
    ht.total_entries += i - start;
  }
  ht.table.init(ht.entries.size());
  for (auto& e : ht.entries) ht.table.insert(e.first, e.second);
  return ht;
}

// ---------------------------------------------------------------------------
// Seeding (src/mapper/seeds.rs)
// ---------------------------------------------------------------------------
static const size_t MAX_K = 32;                 // seeds.rs:40
static const u64 REPEAT_SKIP_THRESHOLD = 64;    // seeds.rs:45
static const size_t FP_SPAN = 12;               // seeds.rs:51
static const size_t FP_AFTER_WANT = 8;          // seeds.rs:57
static const size_t FP_BEFORE_WANT = 4;         // seeds.rs:58
static const u32 FP_BASE_THRESHOLD = 10;        // seeds.rs:69
static const u32 FP_NEIGHBOUR_DISCOUNT = 2;     // seeds.rs:70

struct SeedHit {
  u64 read_pos, contig, ref_pos, k;
  Strand strand;
};

struct Range { size_t start, end; size_t len() const { return end - start; } };

// clip_flanks (seeds.rs:224-232).
static inline void clip_flanks(size_t seq_len, size_t ws, size_t k, size_t aw, size_t bw, Range& after, Range& before) {
  size_t as = std::min(ws + k, seq_len);
  size_t ae = std::min(as + aw, seq_len);
  size_t be = std::min(ws, seq_len);
  size_t bs = be >= bw ? be - bw : 0;
  after = {as, ae};
  before = {bs, be};
}

struct Fp { u32 a = 0, c = 0, g = 0, t = 0; };
// compute_fingerprint / merge / distance (seeds.rs:241-271).
static inline void fp_add(Fp& fp, const u8* s, size_t n) {
  for (size_t i = 0; i < n; i++) {
    switch (ascii_upper(s[i])) {
      case 'A': fp.a++; break;
      case 'C': fp.c++; break;
      case 'G': fp.g++; break;
      case 'T': fp.t++; break;
      default: break;
    }
  }
}
static inline u32 absdiff(u32 x, u32 y) { return x > y ? x - y : y - x; }
static inline u32 fp_dist(const Fp& x, const Fp& y) {
  return absdiff(x.a, y.a) + absdiff(x.c, y.c) + absdiff(x.g, y.g) + absdiff(x.t, y.t);
}

// passes_similarity_filter (seeds.rs:162-219).
static bool passes_similarity_filter(const std::vector<u8>& read, const std::vector<u8>& rc_read, size_t read_pos,
                                     size_t k, const Genome& g, u64 cid, u64 ref_pos, Strand strand,
                                     bool is_neighbour) {
  const Contig& contig = g.contigs[cid];
  const std::vector<u8>& rl = strand == FWD ? read : rc_read;
  size_t ws = strand == FWD ? read_pos : read.size() - read_pos - k;
  Range ra, rb;
  clip_flanks(rl.size(), ws, k, FP_AFTER_WANT, FP_BEFORE_WANT, ra, rb);
  u64 region_start = ref_pos >= FP_BEFORE_WANT ? ref_pos - FP_BEFORE_WANT : 0;
  u64 region_end = std::min(ref_pos + k + FP_AFTER_WANT, contig.length);
  if (region_start >= region_end) return true;
  std::vector<u8> gl = contig.slice(region_start, region_end);
  size_t gws = (size_t)(ref_pos - region_start);
  Range ga, gb;
  clip_flanks(gl.size(), gws, k, FP_AFTER_WANT, FP_BEFORE_WANT, ga, gb);
  size_t after_len = std::min(ra.len(), ga.len());
  size_t before_len = std::min(rb.len(), gb.len());
  if (after_len + before_len < FP_SPAN) return true;
  Fp rf, gf;
  fp_add(rf, &rl[ra.start], after_len);
  fp_add(rf, &rl[rb.end - before_len], before_len);
  fp_add(gf, &gl[ga.start], after_len);
  fp_add(gf, &gl[gb.end - before_len], before_len);
  u32 d = fp_dist(rf, gf);
  u32 thr = is_neighbour ? FP_BASE_THRESHOLD - FP_NEIGHBOUR_DISCOUNT : FP_BASE_THRESHOLD;
  return d <= thr;
}

// neighbour_probed_position (seeds.rs:276-286).
static inline bool neighbour_probed_position(size_t read_pos, size_t read_len) {
  if (read_len <= 34) return true;
  if (read_len <= 49) return (read_pos / 5) % 2 == 0;
  return (read_pos % 15) < 5;
}

// find_seed_hits (seeds.rs:91-151): exact lookup at every ACGT-only window,
// then (at sampled, non-repetitive windows) the 45 one-mismatch neighbours
// in position-major, A/C/G/T order (probe_1mm_neighbours, seeds.rs:291-309).
static void find_seed_hits(const Read& read, const HashTable& ht, const Genome& g, std::vector<SeedHit>& hits,
                           std::vector<double>& repeat_prob) {
  size_t k = ht.k;
  hits.clear();
  repeat_prob.clear();
  size_t L = read.bases.size();
  if (L < k || k > MAX_K) return;
  repeat_prob.assign(L - k + 1, 0.0);
  std::vector<u8> rc = revcomp(read.bases);
  static const u8 BASES[4] = {'A', 'C', 'G', 'T'};
  for (size_t rp = 0; rp + k <= L; rp++) {
    const u8* w = &read.bases[rp];
    if (!is_acgt_only(w, k)) continue;
    const u64* ex;
    u64 exn;
    ht.lookup(w, k, ex, exn);
    for (u64 e = 0; e < exn; e++) {
      u64 cid, pos;
      Strand s;
      unpack_position(ex[e], cid, pos, s);
      if (passes_similarity_filter(read.bases, rc, rp, k, g, cid, pos, s, false))
        hits.push_back({rp, cid, pos, k, s});
    }
    bool looks_repetitive = exn >= REPEAT_SKIP_THRESHOLD;
    if (looks_repetitive) repeat_prob[rp] = 1.0;
    if (neighbour_probed_position(rp, L) && !looks_repetitive) {
      u8 qual = rp < read.quals.size() ? read.quals[rp] : 30;
      double nrp = std::pow(10.0, -(double)qual / 10.0);
      u8 buf[MAX_K];
      memcpy(buf, w, k);
      for (size_t i = 0; i < k; i++) {
        u8 orig = buf[i];
        for (u8 base : BASES) {
          if (base == orig) continue;
          buf[i] = base;
          const u64* nb;
          u64 nbn;
          ht.lookup(buf, k, nb, nbn);
          if (nbn >= REPEAT_SKIP_THRESHOLD) repeat_prob[rp] = std::max(repeat_prob[rp], nrp);
          for (u64 e = 0; e < nbn; e++) {
            u64 cid, pos;
            Strand s;
            unpack_position(nb[e], cid, pos, s);
            if (passes_similarity_filter(read.bases, rc, rp, k, g, cid, pos, s, true))
              hits.push_back({rp, cid, pos, k, s});
          }
        }
        buf[i] = orig;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Candidate clustering (src/mapper/candidates.rs) and the iteration order of
// its FxHashMap<(usize, Strand), _> (candidates.rs:34-46).
// ---------------------------------------------------------------------------
// FxHasher (rustc-hash 2.1.3, 64-bit): add_to_hash(i) = (h + i) * K, finish =
// rotate_left(h, 26). The key (usize, Strand) hashes the contig id, then the
// enum discriminant (Forward 0, Reverse 1) as a usize.
static inline u64 fx_hash_group(u64 cid, Strand s) {
  const u64 K = 0xf1357aea2e62a9c5ull;
  u64 h = 0;
  h = (h + cid) * K;
  h = (h + (u64)s) * K;
  return (h << 26) | (h >> 38);
}

// std's SwissTable (hashbrown RawTable) insertion of distinct keys with no
// deletions: growth at capacity (4, 8, 16, 32... buckets, capacity mask for
// < 8 buckets else buckets*7/8), resize reinserts old entries in bucket order,
// insertion takes the first empty slot of the first probe group (triangular
// probing in steps of the group width) that has one, tables no larger than a
// group scan circularly from the home bucket. Iteration visits buckets in
// increasing index. Returns key indices in iteration order.
struct SwissOrder {
  int W;
  std::vector<int> slot;  // -1 empty, else key index
  std::vector<u64> hashes;
  u64 items = 0;
  explicit SwissOrder(int w) : W(w) {}
  static u64 cap_of(u64 buckets) { return buckets < 8 ? (buckets ? buckets - 1 : 0) : buckets / 8 * 7; }
  static u64 buckets_for(u64 cap) {
    if (cap < 8) return cap < 4 ? 4 : 8;
    u64 adj = cap * 8 / 7;
    u64 b = 1;
    while (b < adj) b <<= 1;
    return b;
  }
  u64 find_slot(const std::vector<int>& t, u64 h) const {
    u64 nb = t.size();
    u64 mask = nb - 1;
    u64 pos = h & mask;
    if (nb <= (u64)W) {
      for (u64 i = 0; i < nb; i++) {
        u64 s = (pos + i) & mask;
        if (t[s] < 0) return s;
      }
      return 0;
    }
    u64 stride = 0;
    while (true) {
      for (u64 b = 0; b < (u64)W; b++) {
        u64 s = (pos + b) & mask;
        if (t[s] < 0) return s;
      }
      stride += W;
      pos = (pos + stride) & mask;
    }
  }
  void insert(int key, u64 h) {
    hashes.push_back(h);
    u64 cap = cap_of(slot.size());
    if (items + 1 > cap) {
      u64 need = std::max(items + 1, cap + 1);
      std::vector<int> nt(buckets_for(need), -1);
      for (size_t b = 0; b < slot.size(); b++)
        if (slot[b] >= 0) nt[find_slot(nt, hashes[slot[b]])] = slot[b];
      slot.swap(nt);
    }
    slot[find_slot(slot, h)] = key;
    items++;
  }
  std::vector<int> order() const {
    std::vector<int> o;
    for (int s : slot)
      if (s >= 0) o.push_back(s);
    return o;
  }
};

struct Candidate {
  u64 contig;
  u64 position;
  Strand strand;
  double score;
};

static const i64 MERGE_DISTANCE = 50;  // candidates.rs:27

// cluster_hits (candidates.rs:30-78).
static std::vector<Candidate> cluster_hits(const std::vector<SeedHit>& hits, size_t read_len, int group_width) {
  std::vector<std::pair<u64, Strand>> keys;
  std::map<std::pair<u64, int>, int> index;
  std::vector<std::vector<i64>> diags;
  std::vector<u64> first_k;
  SwissOrder so(group_width);
  for (auto& h : hits) {
    i64 d = h.strand == FWD ? (i64)h.ref_pos - (i64)h.read_pos : (i64)h.ref_pos + (i64)h.read_pos;
    auto key = std::make_pair(h.contig, (int)h.strand);
    auto it = index.find(key);
    int gi;
    if (it == index.end()) {
      gi = (int)keys.size();
      index[key] = gi;
      keys.push_back({h.contig, h.strand});
      diags.emplace_back();
      first_k.push_back(h.k);
      so.insert(gi, fx_hash_group(h.contig, h.strand));
    } else {
      gi = it->second;
    }
    diags[gi].push_back(d);
  }
  std::vector<Candidate> cands;
  for (int gi : so.order()) {
    std::vector<i64>& dh = diags[gi];
    std::stable_sort(dh.begin(), dh.end());
    size_t cs = 0;
    for (size_t idx = 1; idx <= dh.size(); idx++) {
      bool boundary = idx == dh.size() || dh[idx] - dh[idx - 1] > MERGE_DISTANCE;
      if (!boundary) continue;
      i64 sum = 0;
      for (size_t j = cs; j < idx; j++) sum += dh[j];
      i64 avg = sum / (i64)(idx - cs);
      i64 position = keys[gi].second == FWD ? avg : avg - (i64)read_len + (i64)first_k[gi];
      cands.push_back({keys[gi].first, (u64)std::max<i64>(position, 0), keys[gi].second, (double)(idx - cs)});
      cs = idx;
    }
  }
  std::stable_sort(cands.begin(), cands.end(), [](const Candidate& a, const Candidate& b) { return a.score > b.score; });
  return cands;
}

// ---------------------------------------------------------------------------
// Banded affine-gap DP (src/align/smith_waterman.rs) and CIGAR helpers
// (src/align/cigar.rs)
// ---------------------------------------------------------------------------
static const i32 MATCH_SCORE = 20;  // smith_waterman.rs:81

static i32 sat_i32(double x) {
  if (std::isnan(x)) return 0;
  if (x >= 2147483647.0) return INT32_MAX;
  if (x <= -2147483648.0) return INT32_MIN;
  return (i32)x;
}

struct Aligner {
  i32 gap_open, gap_extend;
  i64 band;
  double hp_slope = 1.0;   // smith_waterman.rs:97
  double mm_floor = 0.2;   // smith_waterman.rs:98

  // SmithWatermanAligner::new (smith_waterman.rs:113-130).
  Aligner(u64 band_w, u32 gop, u32 gep) {
    i32 go = sat_i32(std::round(-90.0 * (double)gop / 40.0));
    i32 ge = sat_i32(std::round(-1.0 * (double)gep / 3.0));
    gap_open = std::min(go, -1);
    gap_extend = std::min(ge, -1);
    band = (i64)band_w;
  }
  // mismatch_penalty (smith_waterman.rs:272-275).
  i32 mismatch_penalty(u8 q) const {
    double scale = std::min(std::max((double)q / 30.0, mm_floor), 1.0);
    return sat_i32(std::round(-30.0 * scale));
  }
  // homopolymer_gap_open (smith_waterman.rs:288-291).
  i32 hp_gap_open(u16 run) const {
    i32 disc = sat_i32(std::round((double)(run > 0 ? run - 1 : 0) * hp_slope));
    return std::min(gap_open + disc, -1);
  }

  // align (smith_waterman.rs:163-255) + traceback (:299-344).
  i32 align(const u8* read, const u8* qual, size_t qlen, size_t m, const u8* ref, size_t n, i64 hint,
            std::vector<Cig>& cigar, size_t& offset) const {
    cigar.clear();
    if (m == 0 || n == 0) {
      cigar.push_back({'S', (u32)m});
      offset = 0;
      return 0;
    }
    // precompute_homopolymer_runs (smith_waterman.rs:348-363).
    std::vector<u16> run(n, 1);
    {
      size_t st = 0;
      for (size_t idx = 1; idx <= n; idx++) {
        if (idx == n || ref[idx] != ref[st]) {
          u16 len = (u16)std::min<size_t>(idx - st, 65535);
          for (size_t r = st; r < idx; r++) run[r] = len;
          st = idx;
        }
      }
    }
    const size_t width = n + 1;
    const i32 NEG = INT32_MIN / 2;
    std::vector<i32> dm(width, 0), di(width, NEG), dd(width, NEG);
    std::vector<i32> nm(width, NEG), ni(width, NEG), nd(width, NEG);
    std::vector<u8> tbm((m + 1) * width, 0), tbi((m + 1) * width, 0), tbd((m + 1) * width, 0);
    for (size_t i = 1; i <= m; i++) {
      i64 center = (i64)i + hint;
      i64 js = std::max<i64>(center - band, 1);
      i64 je = std::max<i64>(std::min<i64>(center + band, (i64)n), 0);
      if (js > je) continue;
      std::fill(nm.begin(), nm.end(), NEG);
      std::fill(ni.begin(), ni.end(), NEG);
      std::fill(nd.begin(), nd.end(), NEG);
      u8 q = (i - 1) < qlen ? qual[i - 1] : 30;
      i32 mmp = mismatch_penalty(q);
      size_t rb = i * width;
      for (i64 jj = js; jj <= je; jj++) {
        size_t j = (size_t)jj;
        i32 ms = read[i - 1] == ref[j - 1] ? MATCH_SCORE : mmp;
        i32 fm = dm[j - 1] + ms, fi = di[j - 1] + ms, fd = dd[j - 1] + ms;
        i32 msc = std::max(std::max(fm, fi), fd);
        i32 go = hp_gap_open(run[j - 1]);
        i32 io = dm[j] + go, ie = di[j] + gap_extend;
        i32 isc = std::max(io, ie);
        i32 dop = nm[j - 1] + go, dex = nd[j - 1] + gap_extend;
        i32 dsc = std::max(dop, dex);
        nm[j] = msc;
        ni[j] = isc;
        nd[j] = dsc;
        tbm[rb + j] = msc == fm ? 0 : (msc == fi ? 1 : 2);
        tbi[rb + j] = isc == io ? 0 : 1;
        tbd[rb + j] = dsc == dop ? 0 : 1;
      }
      std::swap(dm, nm);
      std::swap(di, ni);
      std::swap(dd, nd);
    }
    // Endpoint: last maximum over (j, M), (j, I) for j = 0..=n (max_by_key).
    size_t bj = 0;
    i32 bs = dm[0];
    u8 bst = 0;
    for (size_t j = 0; j <= n; j++) {
      if (dm[j] >= bs) { bs = dm[j]; bj = j; bst = 0; }
      if (di[j] >= bs) { bs = di[j]; bj = j; bst = 1; }
    }
    // Traceback.
    std::vector<char> ops;
    size_t i = m, j = bj;
    u8 st = bst;
    while (i > 0) {
      if (j == 0) { ops.push_back('I'); i--; continue; }
      if (st == 0) {
        u8 p = tbm[i * width + j];
        ops.push_back('M');
        i--; j--;
        st = p;
      } else if (st == 1) {
        bool opened = tbi[i * width + j] == 0;
        ops.push_back('I');
        i--;
        st = opened ? 0 : 1;
      } else {
        bool opened = tbd[i * width + j] == 0;
        ops.push_back('D');
        j--;
        st = opened ? 0 : 2;
      }
    }
    std::reverse(ops.begin(), ops.end());
    // collapse_cigar (smith_waterman.rs:365-381).
    for (char o : ops) {
      if (!cigar.empty() && cigar.back().op == o) cigar.back().n++;
      else cigar.push_back({o, 1});
    }
    offset = j;
    return bs;
  }
};

// cigar_reference_span (src/align/cigar.rs:23-28).
static inline u64 ref_span(const std::vector<Cig>& c) {
  u64 s = 0;
  for (auto& o : c)
    if (o.op == 'M' || o.op == 'D') s += o.n;
  return s;
}

// ---------------------------------------------------------------------------
// Bayesian MAPQ (src/mapq/bayesian.rs) and insert-size model
// (src/mapq/insert_size.rs)
// ---------------------------------------------------------------------------
static const double LN_10 = 2.302585092994045684017991454684364208;
static const double DB = -0.1 * LN_10;  // bayesian.rs:36

static double posterior_floor() { return std::exp(99.0 * DB); }  // bayesian.rs:39-41

// logadd (bayesian.rs:47-58).
static inline double logadd(double a, double b) {
  if (a > b) std::swap(a, b);
  if (b >= a + 10.0) return a;
  if (b >= a + 4.0) return std::max(a - 1.0, 0.0);
  if (b >= a + 2.0) return std::max(a - 2.0, 0.0);
  return std::max(a - 3.0, 0.0);
}
// py_int_round (bayesian.rs:63-65).
static inline double py_int_round(double x) { return std::trunc(x + 0.5); }
// phred_n_choose_m (bayesian.rs:72-86).
static double phred_n_choose_m(i64 n, i64 m) {
  if (m > n / 2) m = n - m;
  if (m <= 0) return 0.0;
  double phred = 0.0;
  while (m > 1) {
    phred += std::log((double)n) - std::log((double)m);
    n--;
    m--;
  }
  phred += std::log((double)n);
  return py_int_round(10.0 * phred / LN_10);
}
// gc_content (bayesian.rs:445-456).
static double gc_content(const std::vector<u8>& s) {
  u64 gc = 0, tot = 0;
  for (u8 b : s) {
    switch (ascii_upper(b)) {
      case 'G': case 'C': gc++; tot++; break;
      case 'A': case 'T': tot++; break;
      default: break;
    }
  }
  return tot == 0 ? 0.5 : (double)gc / (double)tot;
}
// effective_alphabet_size (bayesian.rs:463-466).
static double effective_alphabet_size(double f) {
  f = std::min(std::max(f, 1e-6), 1.0 - 1e-6);
  return std::exp(-f * std::log(f / 2.0) - (1.0 - f) * std::log((1.0 - f) / 2.0));
}

static double clampd(double x, double lo, double hi) { return x < lo ? lo : (x > hi ? hi : x); }

struct Mapq {
  double subphred;
  u64 seed_k;
  double genome_size;

  // MapqCalculator::new (bayesian.rs:103-110).
  Mapq(double sub_rate, u64 k, u64 gsize) {
    subphred = py_int_round(std::log(std::max(sub_rate, 1e-30)) / DB);
    seed_k = k;
    genome_size = (double)std::max<u64>(gsize, 1);
  }

  // alignment_log_likelihood_bases (bayesian.rs:142-179).
  double log_lk(const std::vector<u8>& bases, const std::vector<u8>& qual, const std::vector<u8>& ref,
                const std::vector<Cig>& cigar) const {
    double lk = 0.0;
    size_t qi = 0, ri = 0;
    for (auto& op : cigar) {
      if (op.op == 'M') {
        for (u32 t = 0; t < op.n; t++) {
          if (qi >= bases.size() || ri >= ref.size()) break;
          double rq = qi < qual.size() ? (double)qual[qi] : 30.0;
          double eq = logadd(rq, subphred);
          double e = std::pow(10.0, -eq / 10.0);
          double pm = 1.0 - e;
          double p = bases[qi] == ref[ri] ? pm : e / 3.0;
          lk += std::log(std::max(p, 1e-300));
          qi++;
          ri++;
        }
      } else if (op.op == 'I') {
        for (u32 t = 0; t < op.n; t++) {
          if (qi >= bases.size()) break;
          lk += std::log(0.25);
          qi++;
        }
      } else if (op.op == 'D') {
        ri += op.n;
      } else if (op.op == 'S') {
        qi += op.n;
      }
    }
    return lk;
  }

  // select_best (bayesian.rs:193-201): last maximum, sequential exp sum.
  void select_best(const std::vector<double>& lks, size_t& best, double& sum_exp) const {
    double mx = lks[0];
    best = 0;
    for (size_t i = 0; i < lks.size(); i++)
      if (lks[i] >= mx) { mx = lks[i]; best = i; }
    double s = -0.0;
    for (double lk : lks) s += std::exp(lk - mx);
    sum_exp = s;
  }
  // posterior_fractions (bayesian.rs:208-216).
  std::vector<double> posterior_fractions(const std::vector<double>& lks) const {
    std::vector<double> out;
    if (lks.empty()) return out;
    double mx = -INFINITY;
    for (double v : lks) mx = std::fmax(mx, v);
    std::vector<double> ex;
    double s = -0.0;
    for (double v : lks) ex.push_back(std::exp(v - mx));
    for (double e : ex) s += e;
    for (double e : ex) out.push_back(e / s);
    return out;
  }
  // wrong_mapping_probability (bayesian.rs:227-230).
  double wrong_mapping_probability(double sum_exp) const {
    double bp = 1.0 / std::max(sum_exp, 1.0);
    return std::max(1.0 - bp, posterior_floor());
  }

  // log_entropy (bayesian.rs:306-373).
  double log_entropy(const std::vector<Cig>& cigar, const std::vector<u8>& qb, const std::vector<u8>& qq,
                     const std::vector<u8>& rw) const {
    const u8 MIN_Q = 10;
    const double MAX_INDEL_LEN = 30.0;
    i64 n = 0, m = 0;
    u64 readlen = 0, refpos = 0;
    i64 indel_runs = 0, del_runs = 0;
    int cur = 0;
    for (auto& op : cigar) {
      if (op.op == 'I') {
        for (u32 t = 0; t < op.n; t++) {
          if (cur != 1) indel_runs++;
          cur = 1;
          readlen++;
        }
      } else if (op.op == 'D') {
        for (u32 t = 0; t < op.n; t++) {
          if (cur != 2) { del_runs++; indel_runs++; }
          cur = 2;
          refpos++;
        }
      } else if (op.op == 'M') {
        for (u32 t = 0; t < op.n; t++) {
          if (cur != 0) indel_runs++;
          cur = 0;
          if (readlen >= qb.size() || refpos >= rw.size()) break;
          u8 q = readlen < qq.size() ? qq[readlen] : 0;
          bool hq = q >= MIN_Q;
          if (hq) n++;
          u8 a = qb[readlen], r = rw[refpos];
          if (a != r && a != 'N' && r != 'N' && hq) m++;
          readlen++;
          refpos++;
        }
      }
    }
    i64 ins_runs = indel_runs - del_runs;
    double b = effective_alphabet_size(gc_content(rw));
    double two_g = 2.0 * genome_size;
    double match_term = py_int_round(10.0 * ((double)n * std::log(b) - std::log(two_g)) / LN_10);
    double mismatch_term = py_int_round(10.0 * (double)m * std::log(std::max(b - 1.0, 1e-6)) / LN_10);
    double pos_choice = phred_n_choose_m((i64)readlen, 2 * ins_runs + del_runs);
    double del_len_term = del_runs > 0 ? py_int_round((double)del_runs * 10.0 * std::log(MAX_INDEL_LEN) / LN_10) : 0.0;
    return match_term - mismatch_term - phred_n_choose_m(n, m) - pos_choice - del_len_term;
  }

  // missing_locus_probability (bayesian.rs:405-439).
  double missing_locus(const Read& read, const std::vector<double>& mask) const {
    u64 k = seed_k;
    size_t len = read.quals.size();
    if (k == 0 || len < k) return 0.5;
    std::vector<double> q(len);
    for (size_t i = 0; i < len; i++) {
      double eq = logadd((double)read.quals[i], subphred);
      q[i] = std::min(std::pow(10.0, -eq / 10.0), 1.0 - 1e-12);
    }
    double means = 0.0;
    u64 phases = std::min<u64>(k, 5);
    for (u64 ph = 0; ph < phases; ph++) {
      double logp = 0.0;
      u64 st = ph;
      while (st + k <= len) {
        double rp = st < mask.size() ? mask[st] : 0.0;
        double z = 1.0;
        for (u64 t = 0; t < k; t++) z = z * (1.0 - q[st + t]);
        double p1 = -0.0;
        for (u64 t = 0; t < k; t++) p1 = p1 + q[st + t] / (1.0 - q[st + t]);
        double p2 = clampd(1.0 - z * (1.0 + p1), 0.0, 1.0);
        double pm = clampd(1.0 - (1.0 - p2) * (1.0 - rp), 1e-300, 1.0);
        logp += std::log(pm);
        st += k;
      }
      means += std::exp(logp);
    }
    return std::min(means / (double)phases, 0.99);
  }

  // finalize_mapq (bayesian.rs:251-282).
  void finalize(double sum_exp, const Read& read, const std::vector<Cig>& cigar, const std::vector<u8>& qb,
                const std::vector<u8>& qq, const std::vector<u8>& rw, const std::vector<double>& mask, u8& mapq,
                double& post) const {
    double pw = wrong_mapping_probability(sum_exp);
    double wrongmapping = py_int_round(std::log(pw) / DB);
    double entropy = log_entropy(cigar, qb, qq, rw) - 3.0;
    if (entropy <= 0.0) { mapq = 0; post = 0.0; return; }
    double pmiss = std::max(missing_locus(read, mask), 1e-30);
    double notfound = -10.0 * std::log10(pmiss);
    double combined = logadd(wrongmapping, notfound);
    double pp = clampd(logadd(entropy, combined), 0.0, 99.0);
    mapq = (u8)std::round(pp);
    double pprob = std::pow(10.0, -pp / 10.0);
    post = 1.0 - pprob;
  }
};

struct InsertModel {
  double mean, sd;
  u64 n = 0;
  // InsertSizeDistribution::log_likelihood (insert_size.rs:23-30).
  double log_likelihood(double x) const {
    if (sd <= 0.0) return -1e300;
    double diff = x - mean;
    return -0.5 * (diff * diff) / (sd * sd) - 0.5 * std::log(2.0 * M_PI * sd * sd);
  }
  // InsertSizeDistribution::update (insert_size.rs:32-44).
  void update(double obs) {
    n++;
    double nn = (double)n;
    double delta = obs - mean;
    mean += delta / nn;
    double delta2 = obs - mean;
    double var = nn > 1.0 ? ((sd * sd) * (nn - 1.0) + delta * delta2) / nn : sd * sd;
    sd = std::max(std::sqrt(var), 1.0);
  }
};

// ---------------------------------------------------------------------------
// Records (AlignmentRecord, src/types.rs:181-203)
// ---------------------------------------------------------------------------
struct Record {
  i64 contig = -1;      // -1 = '*'
  u64 position = 0;     // 1-based, 0 = unmapped
  u8 mapq = 0;
  std::vector<Cig> cigar;
  Strand strand = FWD;
  bool is_paired = false, proper = false;
  i64 mate_contig = -1;
  bool has_mate_pos = false;
  u64 mate_position = 0;
  bool has_tlen = false;
  i64 tlen = 0;
  double score = 0.0;
  double posterior = 0.0;
  int read_number = 0;
  int mate_strand = -1;   // -1 none, else Strand
  bool mate_unmapped = false;
  // derived fields (no reference counterpart): DP score and edit distance
  i32 as_score = 0;
  i32 nm = 0;
};

// sam_flag (src/io/sam.rs:126-143).
static u16 sam_flag(const Record& r) {
  u16 f = 0;
  bool unmapped = r.position == 0;
  if (r.is_paired) f |= 0x1;
  if (r.proper) f |= 0x2;
  if (unmapped) f |= 0x4;
  if (r.mate_unmapped) f |= 0x8;
  if (!unmapped && r.strand == REV) f |= 0x10;
  if (r.mate_strand == REV) f |= 0x20;
  if (r.read_number == 1) f |= 0x40;
  if (r.read_number == 2) f |= 0x80;
  return f;
}

// ---------------------------------------------------------------------------
// Single-end mapper (src/mapper/single.rs)
// ---------------------------------------------------------------------------
struct CandAln {
  u64 contig;
  u64 position;  // 0-based
  Strand strand;
  std::vector<Cig> cigar;
  double log_lk;
  std::vector<u8> ref_window;
  const std::vector<u8>* out_seq;
  const std::vector<u8>* out_qual;
  i32 dp_score;
};

struct Mapper {
  Genome genome;
  HashTable ht;
  orc_options opt;
  std::unique_ptr<Aligner> sw;
  std::unique_ptr<Mapq> mq;
  double sv_prior_log_prob;
  std::vector<i64> name_class;  // first contig index carrying the same name

  bool open(const std::string& gp, const std::string& hp, const orc_options& o) {
    opt = o;
    if (!genome.load(gp)) return false;
    if (!ht.load(hp, opt.dense_min_buckets)) return false;
    sw.reset(new Aligner(opt.max_indel_len, opt.gap_open_phred, opt.gap_extend_phred));
    mq.reset(new Mapq(opt.substitution_rate, ht.k, genome.total_length));
    sv_prior_log_prob = -opt.sv_prior_phred / 10.0 * LN_10;  // paired.rs:97
    std::map<std::string, i64> first;
    for (size_t i = 0; i < genome.contigs.size(); i++) {
      auto it = first.find(genome.contigs[i].name);
      if (it == first.end()) { first[genome.contigs[i].name] = (i64)i; name_class.push_back((i64)i); }
      else name_class.push_back(it->second);
    }
    return true;
  }

  struct ReadCtx {
    const Read* read;
    std::vector<u8> rc_seq, rc_qual;
  };

  // Edit distance of an alignment (derived; no reference counterpart).
  static i32 edit_distance(const std::vector<Cig>& cigar, const std::vector<u8>& qb, const std::vector<u8>& rw) {
    i32 nm = 0;
    size_t qi = 0, ri = 0;
    for (auto& op : cigar) {
      if (op.op == 'M') {
        for (u32 t = 0; t < op.n; t++, qi++, ri++)
          if (qi < qb.size() && ri < rw.size() && qb[qi] != rw[ri]) nm++;
      } else if (op.op == 'I') { nm += op.n; qi += op.n; }
      else if (op.op == 'D') { nm += op.n; ri += op.n; }
      else if (op.op == 'S') qi += op.n;
    }
    return nm;
  }

  // SingleEndMapper::map_candidates (single.rs:86-162).
  void map_candidates(const ReadCtx& rc, std::vector<CandAln>& alns, std::vector<double>& mask) const {
    const Read& read = *rc.read;
    std::vector<SeedHit> hits;
    find_seed_hits(read, ht, genome, hits, mask);
    std::vector<Candidate> cands = cluster_hits(hits, read.bases.size(), opt.group_width);
    u64 left_pad = 10;
    u64 right_pad = std::max<u64>(opt.max_indel_len, 10);
    alns.clear();
    size_t take = std::min<size_t>(cands.size(), 20);
    for (size_t ci = 0; ci < take; ci++) {
      const Candidate& c = cands[ci];
      const Contig& contig = genome.contigs[c.contig];
      u64 rs = c.position >= left_pad ? c.position - left_pad : 0;
      u64 re = std::min(c.position + read.bases.size() + right_pad, contig.length);
      if (rs >= re) continue;
      std::vector<u8> seg = contig.slice(rs, re);
      const std::vector<u8>& qb = c.strand == FWD ? read.bases : rc.rc_seq;
      const std::vector<u8>& qq = c.strand == FWD ? read.quals : rc.rc_qual;
      CandAln a;
      size_t off;
      a.dp_score = sw->align(qb.data(), qq.data(), qq.size(), qb.size(), seg.data(), seg.size(), (i64)left_pad,
                             a.cigar, off);
      u64 ts = rs + off;
      u64 span = ref_span(a.cigar);
      a.ref_window = contig.slice(ts, std::min(ts + span, contig.length));
      a.log_lk = mq->log_lk(qb, qq, a.ref_window, a.cigar);
      a.contig = c.contig;
      a.position = ts;
      a.strand = c.strand;
      a.out_seq = &qb;
      a.out_qual = &qq;
      alns.push_back(std::move(a));
    }
  }

  Record unmapped_record(const Read& r) const {  // single.rs:362-383
    Record rec;
    rec.cigar.push_back({'S', (u32)r.bases.size()});
    return rec;
  }

  Record to_record(const CandAln& a, u8 mapq, double post) const {  // single.rs:338-359
    Record rec;
    rec.contig = (i64)a.contig;
    rec.position = a.position + 1;
    rec.mapq = mapq;
    rec.cigar = a.cigar;
    rec.strand = a.strand;
    rec.score = a.log_lk;
    rec.posterior = post;
    rec.as_score = a.dp_score;
    rec.nm = edit_distance(a.cigar, *a.out_seq, a.ref_window);
    return rec;
  }

  // SingleEndMapper::map (single.rs:164-209).
  Record map(const Read& read) const {
    ReadCtx rc{&read, revcomp(read.bases), read.quals};
    std::reverse(rc.rc_qual.begin(), rc.rc_qual.end());
    std::vector<CandAln> alns;
    std::vector<double> mask;
    map_candidates(rc, alns, mask);
    if (alns.empty()) return unmapped_record(read);
    std::vector<double> lks;
    for (auto& a : alns) lks.push_back(a.log_lk);
    size_t bi;
    double se;
    mq->select_best(lks, bi, se);
    const CandAln& b = alns[bi];
    u8 mapq;
    double post;
    mq->finalize(se, read, b.cigar, *b.out_seq, *b.out_qual, b.ref_window, mask, mapq, post);
    return to_record(b, mapq, post);
  }

  // SingleEndMapper::align_at_window (single.rs:220-275). The caller keeps
  // the oriented read alive (out_seq/out_qual point into ReadCtx).
  bool align_at_window(const ReadCtx& rc, u64 cid, u64 expected, u64 radius, Strand strand, CandAln& a) const {
    const Read& read = *rc.read;
    const Contig& contig = genome.contigs[cid];
    u64 rs = expected >= radius ? expected - radius : 0;
    u64 re = std::min(expected + read.bases.size() + radius, contig.length);
    if (rs >= re) return false;
    std::vector<u8> seg = contig.slice(rs, re);
    const std::vector<u8>& qb = strand == FWD ? read.bases : rc.rc_seq;
    const std::vector<u8>& qq = strand == FWD ? read.quals : rc.rc_qual;
    Aligner wa(seg.size(), opt.gap_open_phred, opt.gap_extend_phred);
    i64 hint = (i64)(expected >= rs ? expected - rs : 0);
    size_t off;
    a.dp_score = wa.align(qb.data(), qq.data(), qq.size(), qb.size(), seg.data(), seg.size(), hint, a.cigar, off);
    u64 ts = rs + off;
    u64 span = ref_span(a.cigar);
    a.ref_window = contig.slice(ts, std::min(ts + span, contig.length));
    a.log_lk = mq->log_lk(qb, qq, a.ref_window, a.cigar);
    a.contig = cid;
    a.position = ts;
    a.strand = strand;
    a.out_seq = &qb;
    a.out_qual = &qq;
    return true;
  }

  // -------------------------------------------------------------------------
  // Paired-end mapper (src/mapper/paired.rs)
  // -------------------------------------------------------------------------
  static bool same_locus(const CandAln& a, const CandAln& b) {  // paired.rs:517-519
    return a.contig == b.contig && a.position == b.position && a.strand == b.strand;
  }
  static i64 implied_insert_size(const CandAln& a, const CandAln& b) {  // paired.rs:534-538
    const CandAln& up = a.position <= b.position ? a : b;
    const CandAln& dn = a.position <= b.position ? b : a;
    u64 de = dn.position + ref_span(dn.cigar);
    return (i64)de - (i64)up.position;
  }
  static bool is_fr_pair(const CandAln& a, const CandAln& b) {  // paired.rs:544-547
    const CandAln& up = a.position <= b.position ? a : b;
    const CandAln& dn = a.position <= b.position ? b : a;
    return up.strand == FWD && dn.strand == REV;
  }
  static std::vector<size_t> shortlist_indices(const std::vector<double>& post) {  // paired.rs:553-566
    std::vector<size_t> order(post.size());
    for (size_t i = 0; i < order.size(); i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return post[a] > post[b]; });
    double cum = 0.0;
    size_t take = 0;
    for (size_t i : order) {
      if (take >= 20) break;
      if (take >= 3 && cum >= 0.999) break;
      cum += post[i];
      take++;
    }
    order.resize(take);
    return order;
  }
  static bool argmax_index(const std::vector<double>& lk, size_t& idx) {  // paired.rs:511-515
    if (lk.empty()) return false;
    idx = 0;
    double mx = lk[0];
    for (size_t i = 0; i < lk.size(); i++)
      if (lk[i] >= mx) { mx = lk[i]; idx = i; }
    return true;
  }

  // align_mate_near (paired.rs:450-468).
  bool align_mate_near(const ReadCtx& mate, const CandAln& anchor, const InsertModel& im, CandAln& out) const {
    double mm = std::max(im.mean, 0.0);
    u64 mean = mm >= 1.8446744073709552e19 ? UINT64_MAX : (u64)mm;
    u64 mlen = mate.read->bases.size();
    double rr = std::ceil(5.0 * im.sd);
    u64 radius = (rr <= 0.0 ? 0 : (rr >= 1.8446744073709552e19 ? UINT64_MAX : (u64)rr)) + mlen;
    u64 expected;
    Strand ms;
    if (anchor.strand == FWD) {
      expected = anchor.position + (mean >= mlen ? mean - mlen : 0);
      ms = REV;
    } else {
      u64 ae = anchor.position + ref_span(anchor.cigar);
      expected = ae >= mean ? ae - mean : 0;
      ms = FWD;
    }
    return align_at_window(mate, anchor.contig, expected, radius, ms, out);
  }

  double pair_distance_log_lk(const CandAln& a, const CandAln& b, const InsertModel& im) const {  // paired.rs:486-496
    if (a.contig != b.contig || !is_fr_pair(a, b)) return sv_prior_log_prob;
    double gap = (double)implied_insert_size(a, b);
    return std::max(im.log_likelihood(gap), sv_prior_log_prob);
  }

  Record independent_record(const ReadCtx& rc, const std::vector<CandAln>& cands,
                            const std::vector<double>& mask) const {  // paired.rs:499-509
    if (cands.empty()) return unmapped_record(*rc.read);
    std::vector<double> lk;
    for (auto& c : cands) lk.push_back(c.log_lk);
    size_t bi;
    double se;
    mq->select_best(lk, bi, se);
    const CandAln& b = cands[bi];
    u8 mapq;
    double post;
    mq->finalize(se, *rc.read, b.cigar, *b.out_seq, *b.out_qual, b.ref_window, mask, mapq, post);
    return to_record(b, mapq, post);
  }

  // mapq_for_winning_pair (paired.rs:398-435).
  void mapq_for_winning_pair(const ReadCtx& r1, const ReadCtx& r2, const CandAln& bx, const CandAln& by,
                             double pair_se, const std::vector<double>& lk1, const std::vector<double>& lk2,
                             const std::vector<double>& m1, const std::vector<double>& m2, bool bx_own, bool by_own,
                             u8& q1, double& p1, u8& q2, double& p2) const {
    size_t dummy;
    double se1 = 0, se2 = 0;
    if (bx_own && by_own) {
      mq->select_best(lk1, dummy, se1);
      mq->select_best(lk2, dummy, se2);
      mq->finalize(se1, *r1.read, bx.cigar, *bx.out_seq, *bx.out_qual, bx.ref_window, m1, q1, p1);
      mq->finalize(se2, *r2.read, by.cigar, *by.out_seq, *by.out_qual, by.ref_window, m2, q2, p2);
    } else if (bx_own != by_own) {
      u8 aq;
      double ap;
      if (bx_own) {
        mq->select_best(lk1, dummy, se1);
        mq->finalize(se1, *r1.read, bx.cigar, *bx.out_seq, *bx.out_qual, bx.ref_window, m1, aq, ap);
      } else {
        mq->select_best(lk2, dummy, se2);
        mq->finalize(se2, *r2.read, by.cigar, *by.out_seq, *by.out_qual, by.ref_window, m2, aq, ap);
      }
      q1 = q2 = aq;
      p1 = p2 = ap;
    } else {
      mq->finalize(pair_se, *r1.read, bx.cigar, *bx.out_seq, *bx.out_qual, bx.ref_window, m1, q1, p1);
      mq->finalize(pair_se, *r2.read, by.cigar, *by.out_seq, *by.out_qual, by.ref_window, m2, q2, p2);
    }
  }

  // joint_map (paired.rs:239-371). Returns independently_confident.
  bool joint_map(const ReadCtx& r1, const ReadCtx& r2, const std::vector<CandAln>& c1, const std::vector<double>& m1,
                 const std::vector<CandAln>& c2, const std::vector<double>& m2, const InsertModel& im, Record& o1,
                 Record& o2) const {
    std::vector<double> lk1, lk2;
    for (auto& c : c1) lk1.push_back(c.log_lk);
    for (auto& c : c2) lk2.push_back(c.log_lk);
    size_t b1 = 0, b2 = 0;
    bool h1 = argmax_index(lk1, b1), h2 = argmax_index(lk2, b2);
    if (h1 && h2) {  // fast path (paired.rs:266-291)
      size_t d;
      double se1, se2;
      mq->select_best(lk1, d, se1);
      mq->select_best(lk2, d, se2);
      double w1 = mq->wrong_mapping_probability(se1), w2 = mq->wrong_mapping_probability(se2);
      if (w1 < 0.01 && w2 < 0.01) {
        double ms1 = mq->missing_locus(*r1.read, m1), ms2 = mq->missing_locus(*r2.read, m2);
        if (ms1 < 0.01 && ms2 < 0.01) {
          const CandAln& bx = c1[b1];
          const CandAln& by = c2[b2];
          double gap = (double)implied_insert_size(bx, by);
          bool close = bx.contig == by.contig && is_fr_pair(bx, by) && std::fabs(gap - im.mean) <= 4.0 * im.sd;
          if (close) {
            u8 q1, q2;
            double p1, p2;
            mapq_for_winning_pair(r1, r2, bx, by, 1.0, lk1, lk2, m1, m2, true, true, q1, p1, q2, p2);
            o1 = to_record(bx, q1, p1);
            o2 = to_record(by, q2, p2);
            return true;
          }
        }
      }
    }
    // Raw pairs: candidates are stored by value (CandAln copies share the
    // oriented read through out_seq/out_qual pointers).
    std::vector<std::pair<CandAln, CandAln>> raw;
    if (!c1.empty() && !c2.empty()) {
      raw.push_back({c1[b1], c2[b2]});
      std::vector<double> post1 = mq->posterior_fractions(lk1);
      for (size_t i : shortlist_indices(post1)) {
        CandAln y;
        if (align_mate_near(r2, c1[i], im, y)) raw.push_back({c1[i], std::move(y)});
      }
      std::vector<double> post2 = mq->posterior_fractions(lk2);
      for (size_t j : shortlist_indices(post2)) {
        CandAln x;
        if (align_mate_near(r1, c2[j], im, x)) raw.push_back({std::move(x), c2[j]});
      }
    } else if (c1.empty()) {
      CandAln x;
      if (align_mate_near(r1, c2[b2], im, x)) raw.push_back({std::move(x), c2[b2]});
    } else {
      CandAln y;
      if (align_mate_near(r2, c1[b1], im, y)) raw.push_back({c1[b1], std::move(y)});
    }
    if (raw.empty()) {
      o1 = independent_record(r1, c1, m1);
      o2 = independent_record(r2, c2, m2);
      return true;
    }
    std::vector<size_t> keep;
    for (size_t i = 0; i < raw.size(); i++) {
      bool dup = false;
      for (size_t k2 : keep)
        if (same_locus(raw[k2].first, raw[i].first) && same_locus(raw[k2].second, raw[i].second)) { dup = true; break; }
      if (!dup) keep.push_back(i);
    }
    std::vector<double> jl;
    for (size_t i : keep) {
      const CandAln& x = raw[i].first;
      const CandAln& y = raw[i].second;
      jl.push_back(x.log_lk + y.log_lk + pair_distance_log_lk(x, y, im));
    }
    size_t bi;
    double se;
    mq->select_best(jl, bi, se);
    const CandAln& bx = raw[keep[bi]].first;
    const CandAln& by = raw[keep[bi]].second;
    bool bx_own = h1 && same_locus(bx, c1[b1]);
    bool by_own = h2 && same_locus(by, c2[b2]);
    u8 q1, q2;
    double p1, p2;
    mapq_for_winning_pair(r1, r2, bx, by, se, lk1, lk2, m1, m2, bx_own, by_own, q1, p1, q2, p2);
    o1 = to_record(bx, q1, p1);
    o2 = to_record(by, q2, p2);
    return bx_own && by_own;
  }

  // map_pair_readonly (paired.rs:154-234). Returns true and sets obs when the
  // pair yields an insert-size observation.
  bool map_pair_readonly(const Read& a, const Read& b, const InsertModel& im, Record& o1, Record& o2,
                         double& obs) const {
    ReadCtx r1{&a, revcomp(a.bases), a.quals};
    std::reverse(r1.rc_qual.begin(), r1.rc_qual.end());
    ReadCtx r2{&b, revcomp(b.bases), b.quals};
    std::reverse(r2.rc_qual.begin(), r2.rc_qual.end());
    std::vector<CandAln> c1, c2;
    std::vector<double> m1, m2;
    map_candidates(r1, c1, m1);
    map_candidates(r2, c2, m2);
    bool confident;
    if (c1.empty() && c2.empty()) {
      o1 = unmapped_record(a);
      o2 = unmapped_record(b);
      confident = false;
    } else {
      confident = joint_map(r1, r2, c1, m1, c2, m2, im, o1, o2);
    }
    o1.is_paired = o2.is_paired = true;
    o1.read_number = 1;
    o2.read_number = 2;
    bool m1ok = o1.position != 0, m2ok = o2.position != 0;
    o1.mate_unmapped = !m2ok;
    o2.mate_unmapped = !m1ok;
    o1.mate_strand = m2ok ? (int)o2.strand : -1;
    o2.mate_strand = m1ok ? (int)o1.strand : -1;
    bool have_obs = false;
    if (m1ok && m2ok && name_class[o1.contig] == name_class[o2.contig]) {
      const Record& up = o1.position <= o2.position ? o1 : o2;
      const Record& dn = o1.position <= o2.position ? o2 : o1;
      u64 de = dn.position + ref_span(dn.cigar) - 1;
      i64 ins = std::max<i64>((i64)de - (i64)up.position + 1, 0);
      bool within = std::fabs((double)ins - im.mean) < 5.0 * im.sd;
      bool fr = up.strand == FWD && dn.strand == REV;  // is_fr_orientation, paired.rs:572-575
      bool proper = within && fr;
      o1.proper = o2.proper = proper;
      o1.mate_contig = o2.contig;
      o2.mate_contig = o1.contig;
      o1.has_mate_pos = o2.has_mate_pos = true;
      o1.mate_position = o2.position;
      o2.mate_position = o1.position;
      o1.has_tlen = o2.has_tlen = true;
      o1.tlen = o1.position <= o2.position ? ins : -ins;
      o2.tlen = o2.position <= o1.position ? ins : -ins;
      if (proper && confident) { obs = (double)ins; have_obs = true; }
    }
    return have_obs;
  }
};

// ---------------------------------------------------------------------------
// SAM text (src/io/sam.rs)
// ---------------------------------------------------------------------------
// String::from_utf8_lossy: valid UTF-8 passes through, each maximal invalid
// subsequence becomes U+FFFD.
static void utf8_lossy_append(std::string& out, const u8* s, size_t n) {
  size_t i = 0;
  while (i < n) {
    u8 c = s[i];
    if (c < 0x80) { out.push_back((char)c); i++; continue; }
    size_t need = 0;
    u8 lo = 0x80, hi = 0xBF;
    if (c >= 0xC2 && c <= 0xDF) need = 1;
    else if (c == 0xE0) { need = 2; lo = 0xA0; }
    else if ((c >= 0xE1 && c <= 0xEC) || c == 0xEE || c == 0xEF) need = 2;
    else if (c == 0xED) { need = 2; hi = 0x9F; }
    else if (c == 0xF0) { need = 3; lo = 0x90; }
    else if (c >= 0xF1 && c <= 0xF3) need = 3;
    else if (c == 0xF4) { need = 3; hi = 0x8F; }
    else { out += "\xEF\xBF\xBD"; i++; continue; }
    size_t j = 1;
    bool ok = true;
    for (; j <= need; j++) {
      if (i + j >= n) { ok = false; break; }
      u8 cc = s[i + j];
      u8 l = j == 1 ? lo : 0x80, h = j == 1 ? hi : 0xBF;
      if (cc < l || cc > h) { ok = false; break; }
    }
    if (ok) { out.append((const char*)s + i, need + 1); i += need + 1; }
    else { out += "\xEF\xBF\xBD"; i += j; }
  }
}

static std::string cigar_str(const std::vector<Cig>& c) {
  std::string s;
  for (auto& o : c) { s += std::to_string(o.n); s.push_back(o.op); }
  return s;
}

// ---------------------------------------------------------------------------
// FASTQ / FASTA reads (src/io/fastx.rs)
// ---------------------------------------------------------------------------
// FastqParser::next (fastx.rs:239-305).
static std::vector<Read> read_fastq(const std::string& path, u8 qoff) {
  std::vector<Read> out;
  LineReader lr(path);
  if (!lr.f) throw std::runtime_error("cannot open " + path);
  std::string buf;
  while (true) {
    if (!lr.read_line(buf)) break;
    Read r;
    r.id = first_token(trim_start_char(buf, '@'));
    std::vector<u8> seq;
    while (lr.read_line(buf)) {
      std::string t = trim(buf);
      if (!t.empty() && t[0] == '+') break;
      seq.insert(seq.end(), t.begin(), t.end());
    }
    std::vector<u8> qual;
    while (lr.read_line(buf)) {
      std::string t = trim(buf);
      qual.insert(qual.end(), t.begin(), t.end());
      if (qual.size() >= seq.size()) break;
    }
    for (u8& b : seq) b = ascii_upper(b);
    r.bases = seq;
    for (u8 q : qual) r.quals.push_back(q > qoff ? (u8)(q - qoff) : 0);
    out.push_back(std::move(r));
  }
  return out;
}
// read_fasta_as_reads (fastx.rs:161-174): flat Q40.
static std::vector<Read> read_fasta_reads(const std::string& path) {
  std::vector<Read> out;
  for (auto& fr : read_fasta_records(path)) {
    Read r;
    r.id = fr.id;
    r.bases = fr.seq;
    for (u8& b : r.bases) b = ascii_upper(b);
    r.quals.assign(r.bases.size(), 40);
    out.push_back(std::move(r));
  }
  return out;
}
// strip_mate_suffix (fastx.rs:77-81) and strip_adapter (fastx.rs:97-117).
static void preprocess(std::vector<Read>& reads, const std::string* adapter) {
  for (auto& r : reads) {
    size_t L = r.id.size();
    if (L >= 2 && r.id[L - 2] == '/' && (r.id[L - 1] == '1' || r.id[L - 1] == '2')) r.id.resize(L - 2);
    if (adapter) {
      size_t rl = r.bases.size();
      size_t mo = std::min(rl, adapter->size());
      if (mo < 6) continue;
      for (size_t ov = mo; ov >= 6; ov--) {
        size_t mm = 0;
        for (size_t t = 0; t < ov; t++)
          if (ascii_upper(r.bases[rl - ov + t]) != ascii_upper((u8)(*adapter)[t])) mm++;
        if (mm <= ov / 10) {
          r.bases.resize(rl - ov);
          if (r.quals.size() > rl - ov) r.quals.resize(rl - ov);
          break;
        }
      }
    }
  }
}

}  // namespace orc

// ===========================================================================
// C API
// ===========================================================================
using namespace orc;

extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

void orc_default_options(orc_options* o) {
  o->substitution_rate = 0.001;
  o->insert_size_mean = 250.0;
  o->insert_size_sd = 60.0;
  o->max_indel_len = 30;
  o->gap_open_phred = 40;
  o->gap_extend_phred = 3;
  o->sv_prior_phred = 55.0;
  o->threads = 1;
  o->group_width = 16;
  o->dense_min_buckets = 1ull << 24;
}

int orc_build_genome(const char* out_prefix, const char* species, const char* assembly, int nfiles,
                     const char** fasta_paths) {
  try {
    Genome g;
    g.species = species;
    g.assembly = assembly;
    for (int i = 0; i < nfiles; i++)
      for (auto& fr : read_fasta_records(fasta_paths[i]))
        g.contigs.push_back(Contig::from_ascii(first_token(fr.id), fr.seq.data(), fr.seq.size()));
    for (auto& c : g.contigs) g.total_length += c.length;
    if (!g.save(out_prefix)) { g_err = "cannot write genome"; return -1; }
    return 0;
  } catch (std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

int orc_build_genome_from_seqs(const char* out_prefix, const char* species, const char* assembly, int ncontigs,
                               const char** names, const uint8_t** seqs, const uint64_t* lens) {
  Genome g;
  g.species = species;
  g.assembly = assembly;
  for (int i = 0; i < ncontigs; i++) g.contigs.push_back(Contig::from_ascii(names[i], seqs[i], lens[i]));
  for (auto& c : g.contigs) g.total_length += c.length;
  if (!g.save(out_prefix)) { g_err = "cannot write genome"; return -1; }
  return 0;
}

int orc_build_hash(const char* genome_prefix, const char* out_prefix, uint64_t k, uint64_t stride,
                   uint64_t max_count) {
  Genome g;
  if (!g.load(genome_prefix)) return -1;
  HashTable ht = build_hash_table(g, k, stride, max_count);
  if (!ht.save(out_prefix)) { g_err = "cannot write hash"; return -1; }
  return 0;
}

void* orc_open(const char* genome_prefix, const char* hash_prefix, const orc_options* opt) {
  Mapper* m = new Mapper();
  if (!m->open(genome_prefix, hash_prefix, *opt)) { delete m; return nullptr; }
  return m;
}
void orc_close(void* h) { delete (Mapper*)h; }
uint64_t orc_num_contigs(void* h) { return ((Mapper*)h)->genome.contigs.size(); }
uint64_t orc_genome_total_length(void* h) { return ((Mapper*)h)->genome.total_length; }

static Read make_read(const orc_reads* r, uint64_t i) {
  Read rd;
  uint64_t a = r->offsets[i], b = r->offsets[i + 1];
  rd.bases.assign(r->bases + a, r->bases + b);
  for (auto& x : rd.bases) x = ascii_upper(x);
  rd.quals.assign(r->quals + a, r->quals + b);
  return rd;
}

static int write_records(const std::vector<Record>& recs, orc_records* out) {
  uint64_t co = 0;
  for (size_t i = 0; i < recs.size(); i++) {
    const Record& r = recs[i];
    out->contig[i] = (int32_t)r.contig;
    out->pos[i] = r.position;
    out->mapq[i] = r.mapq;
    out->flag[i] = sam_flag(r);
    out->mate_contig[i] = (int32_t)r.mate_contig;
    out->mate_pos[i] = r.has_mate_pos ? r.mate_position : 0;
    out->tlen[i] = r.has_tlen ? r.tlen : 0;
    out->log_lk[i] = r.score;
    out->posterior[i] = r.posterior;
    out->as_score[i] = r.as_score;
    out->nm[i] = r.nm;
    out->cigar_off[i] = (uint32_t)co;
    for (auto& c : r.cigar) {
      if (co >= out->cigar_cap) { g_err = "cigar capacity exceeded"; return -1; }
      uint32_t op = c.op == 'M' ? 0 : c.op == 'I' ? 1 : c.op == 'D' ? 2 : c.op == 'S' ? 4 : 5;
      out->cigar[co++] = (c.n << 4) | op;
    }
  }
  out->cigar_off[recs.size()] = (uint32_t)co;
  return 0;
}

}  // extern "C"

static int nthreads(int t) {
  if (t >= 1) return t;
  unsigned hc = std::thread::hardware_concurrency();
  return hc ? (int)hc : 1;
}

template <class F>
static void parallel_for(int threads, size_t n, F f) {
  if (threads <= 1 || n < 2) {
    for (size_t i = 0; i < n; i++) f(i);
    return;
  }
  std::atomic<size_t> next(0);
  std::vector<std::thread> ts;
  for (int t = 0; t < threads; t++)
    ts.emplace_back([&]() {
      while (true) {
        size_t s = next.fetch_add(64);
        if (s >= n) break;
        size_t e = std::min(n, s + 64);
        for (size_t i = s; i < e; i++) f(i);
      }
    });
  for (auto& t : ts) t.join();
}

extern "C" {

int orc_map_single(void* h, const orc_reads* reads, orc_records* out) {
  Mapper* m = (Mapper*)h;
  std::vector<Record> recs(reads->n);
  parallel_for(nthreads(m->opt.threads), reads->n, [&](size_t i) {
    Read rd = make_read(reads, i);
    recs[i] = m->map(rd);
  });
  return write_records(recs, out);
}

int orc_map_paired(void* h, orc_insert_model* model, const orc_reads* r1, const orc_reads* r2, orc_records* o1,
                   orc_records* o2) {
  Mapper* m = (Mapper*)h;
  if (r1->n != r2->n) { g_err = "paired-end inputs have different read counts"; return -1; }
  size_t n = r1->n;
  std::vector<Record> a(n), b(n);
  InsertModel im{model->mean, model->sd, model->n_observed};
  // map_paired (src/lib.rs:145-185): PAIR_WARMUP_SIZE = 500 serial pairs,
  // then PAIR_BATCH_SIZE = 2000 pairs per frozen-model batch.
  size_t warm = std::min<size_t>(n, 500);
  for (size_t i = 0; i < warm; i++) {
    Read x = make_read(r1, i), y = make_read(r2, i);
    double obs;
    InsertModel snap = im;
    if (m->map_pair_readonly(x, y, snap, a[i], b[i], obs)) im.update(obs);
  }
  int th = nthreads(m->opt.threads);
  for (size_t s = warm; s < n; s += 2000) {
    size_t e = std::min(n, s + 2000);
    InsertModel snap = im;
    std::vector<double> obs(e - s);
    std::vector<char> has(e - s, 0);
    parallel_for(th, e - s, [&](size_t t) {
      Read x = make_read(r1, s + t), y = make_read(r2, s + t);
      has[t] = m->map_pair_readonly(x, y, snap, a[s + t], b[s + t], obs[t]) ? 1 : 0;
    });
    for (size_t t = 0; t < e - s; t++)
      if (has[t]) im.update(obs[t]);
  }
  model->mean = im.mean;
  model->sd = im.sd;
  model->n_observed = im.n;
  if (write_records(a, o1) != 0) return -1;
  return write_records(b, o2);
}

double orc_time_map_single(void* h, const orc_reads* reads, orc_records* out) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = orc_map_single(h, reads, out);
  auto t1 = std::chrono::steady_clock::now();
  return rc == 0 ? std::chrono::duration<double>(t1 - t0).count() : -1.0;
}

double orc_time_map_paired(void* h, orc_insert_model* model, const orc_reads* r1, const orc_reads* r2,
                           orc_records* o1, orc_records* o2) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = orc_map_paired(h, model, r1, r2, o1, o2);
  auto t1 = std::chrono::steady_clock::now();
  return rc == 0 ? std::chrono::duration<double>(t1 - t0).count() : -1.0;
}

int64_t orc_seed_read(void* h, const uint8_t* bases, const uint8_t* quals, uint64_t len, uint64_t* hit_read_pos,
                      uint32_t* hit_contig, uint64_t* hit_ref_pos, uint8_t* hit_strand, uint64_t hit_cap,
                      double* repeat_prob) {
  Mapper* m = (Mapper*)h;
  Read rd;
  rd.bases.assign(bases, bases + len);
  for (auto& x : rd.bases) x = ascii_upper(x);
  rd.quals.assign(quals, quals + len);
  std::vector<SeedHit> hits;
  std::vector<double> rp;
  find_seed_hits(rd, m->ht, m->genome, hits, rp);
  for (size_t i = 0; i < rp.size(); i++) repeat_prob[i] = rp[i];
  if (hits.size() > hit_cap) return -(int64_t)hits.size();
  for (size_t i = 0; i < hits.size(); i++) {
    hit_read_pos[i] = hits[i].read_pos;
    hit_contig[i] = (uint32_t)hits[i].contig;
    hit_ref_pos[i] = hits[i].ref_pos;
    hit_strand[i] = hits[i].strand;
  }
  return (int64_t)hits.size();
}

int64_t orc_cluster_read(void* h, const uint8_t* bases, const uint8_t* quals, uint64_t len, uint32_t* cand_contig,
                         uint64_t* cand_pos, uint8_t* cand_strand, double* cand_score, uint64_t cand_cap) {
  Mapper* m = (Mapper*)h;
  Read rd;
  rd.bases.assign(bases, bases + len);
  for (auto& x : rd.bases) x = ascii_upper(x);
  rd.quals.assign(quals, quals + len);
  std::vector<SeedHit> hits;
  std::vector<double> rp;
  find_seed_hits(rd, m->ht, m->genome, hits, rp);
  std::vector<Candidate> c = cluster_hits(hits, len, m->opt.group_width);
  if (c.size() > cand_cap) return -(int64_t)c.size();
  for (size_t i = 0; i < c.size(); i++) {
    cand_contig[i] = (uint32_t)c[i].contig;
    cand_pos[i] = c[i].position;
    cand_strand[i] = c[i].strand;
    cand_score[i] = c[i].score;
  }
  return (int64_t)c.size();
}

int orc_align(const uint8_t* read, const uint8_t* qual, uint64_t m, const uint8_t* ref, uint64_t n, int64_t hint,
              uint64_t band, uint32_t gop, uint32_t gep, int32_t* score, uint64_t* offset, uint32_t* cigar,
              uint64_t cigar_cap, uint64_t* n_ops) {
  Aligner a(band, gop, gep);
  std::vector<Cig> c;
  size_t off;
  *score = a.align(read, qual, m, m, ref, n, hint, c, off);
  *offset = off;
  *n_ops = c.size();
  if (c.size() > cigar_cap) return -1;
  for (size_t i = 0; i < c.size(); i++) {
    uint32_t op = c[i].op == 'M' ? 0 : c[i].op == 'I' ? 1 : c[i].op == 'D' ? 2 : 4;
    cigar[i] = (c[i].n << 4) | op;
  }
  return 0;
}

// format_sam_records (sam.rs:69-108) with format_sam (sam.rs:37-58).
// MapqCalculator::select_best + finalize_mapq (bayesian.rs:193-201, 251-282)
// for a batch of reads, each with its candidates' log-likelihoods, its repeat
// mask and its winner's alignment (strand, reference window as passed to
// finalize_mapq, CIGAR).
int orc_mapq_batch(void* h, const orc_reads* reads, const uint64_t* lk_off, const double* lks,
                   const uint64_t* win_off, const double* repeat, const uint8_t* rev, const uint64_t* ref_off,
                   const uint8_t* refs, const uint32_t* cigar_off, const uint32_t* cigar, uint8_t* mapq,
                   double* posterior, uint32_t* best, double* sum_exp) {
  Mapper* m = (Mapper*)h;
  for (uint64_t i = 0; i < reads->n; i++) {
    if (lk_off[i + 1] <= lk_off[i]) return -1;
    std::vector<double> l(lks + lk_off[i], lks + lk_off[i + 1]);
    size_t b;
    double se;
    m->mq->select_best(l, b, se);
    Read rd = make_read(reads, i);
    std::vector<u8> qb = rev[i] ? revcomp(rd.bases) : rd.bases;
    std::vector<u8> qq = rd.quals;
    if (rev[i]) std::reverse(qq.begin(), qq.end());
    std::vector<u8> rw(refs + ref_off[i], refs + ref_off[i + 1]);
    std::vector<Cig> c;
    for (uint32_t k = cigar_off[i]; k < cigar_off[i + 1]; k++) {
      const uint32_t w = cigar[k];
      const char op = "MID?S"[std::min<uint32_t>(w & 15u, 4u)];
      c.push_back(Cig{op, w >> 4});
    }
    std::vector<double> mask(repeat + win_off[i], repeat + win_off[i + 1]);
    u8 mq;
    double post;
    m->mq->finalize(se, rd, c, qb, qq, rw, mask, mq, post);
    mapq[i] = mq;
    posterior[i] = post;
    best[i] = (uint32_t)b;
    sum_exp[i] = se;
  }
  return 0;
}

}  // extern "C"

// One SAM line without its '\n' (format_sam, sam.rs:37-58). SEQ/QUAL in the
// aligned orientation (reverse-complemented and reversed for a reverse-strand
// mapped record); QUAL is the raw Phred scores as bytes (sam.rs:52).
static void sam_line(std::string& out, const Mapper* m, const orc_reads* reads, const char* const* read_ids,
                     const orc_records* recs, uint64_t i, const std::string* rg_id) {
  out += read_ids[i];
  out += "\t" + std::to_string(recs->flag[i]) + "\t";
  int32_t c = recs->contig[i];
  out += c >= 0 ? m->genome.contigs[c].name : std::string("*");
  out += "\t" + std::to_string(recs->pos[i]) + "\t" + std::to_string((unsigned)recs->mapq[i]) + "\t";
  std::string cs;
  for (uint32_t k = recs->cigar_off[i]; k < recs->cigar_off[i + 1]; k++) {
    uint32_t w = recs->cigar[k];
    static const char OPS[] = "MIDXSH";
    cs += std::to_string(w >> 4);
    cs.push_back(OPS[w & 15]);
  }
  out += cs.empty() ? std::string("*") : cs;
  out += "\t";
  int32_t mc = recs->mate_contig[i];
  out += mc >= 0 ? m->genome.contigs[mc].name : std::string("*");
  out += "\t" + std::to_string(recs->mate_pos[i]) + "\t" + std::to_string(recs->tlen[i]) + "\t";
  uint64_t a = reads->offsets[i], b = reads->offsets[i + 1];
  std::vector<u8> seq(reads->bases + a, reads->bases + b), qual(reads->quals + a, reads->quals + b);
  for (auto& x : seq) x = ascii_upper(x);
  if (recs->pos[i] != 0 && (recs->flag[i] & 0x10)) {
    seq = revcomp(seq);
    std::reverse(qual.begin(), qual.end());
  }
  utf8_lossy_append(out, seq.data(), seq.size());
  out += "\t";
  utf8_lossy_append(out, qual.data(), qual.size());
  if (rg_id) out += "\tRG:Z:" + *rg_id;
}

// ReadGroup::parse (sam.rs:17-32).
static bool parse_read_group(const std::string& spec, std::string& id, std::string& header_line) {
  std::vector<std::string> fields;
  bool have = false;
  size_t a = 0;
  while (true) {
    size_t e = spec.find(',', a);
    std::string pair = spec.substr(a, e == std::string::npos ? std::string::npos : e - a);
    size_t c = pair.find(':');
    if (c == std::string::npos) { g_err = "--readgroup: expected TAG:VALUE, got '" + pair + "'"; return false; }
    std::string tag = pair.substr(0, c), value = pair.substr(c + 1);
    if (tag == "ID") { id = value; have = true; }
    fields.push_back(tag + ":" + value);
    if (e == std::string::npos) break;
    a = e + 1;
  }
  if (!have) { g_err = "--readgroup must set at least an ID tag"; return false; }
  header_line = "@RG";
  for (auto& f : fields) header_line += "\t" + f;
  return true;
}

// format_sam_records_sorted (sam.rs:83-108) over the records numbered
// r * n_src + s (record r of source s) listed in sel.
static bool sam_text(const Mapper* m, const char* command_line, const char* read_group, bool coordinate_sorted,
                     uint32_t n_src, const orc_reads* const* reads, const char* const* const* ids,
                     const orc_records* const* recs, const uint64_t* sel, uint64_t n_sel, std::string& out) {
  std::string rg_id, rg_line;
  if (read_group && !parse_read_group(read_group, rg_id, rg_line)) return false;
  out += std::string("@HD\tVN:1.6\tSO:") + (coordinate_sorted ? "coordinate" : "unsorted") + "\n";
  for (auto& c : m->genome.contigs) out += "@SQ\tSN:" + c.name + "\tLN:" + std::to_string(c.length) + "\n";
  out += std::string("@PG\tID:probebwa\tPN:probebwa\tVN:0.1.0\tCL:") + command_line + "\n";
  if (read_group) out += rg_line + "\n";
  for (uint64_t k = 0; k < n_sel; k++) {
    const uint32_t s = (uint32_t)(sel[k] % n_src);
    const uint64_t r = sel[k] / n_src;
    sam_line(out, m, reads[s], ids[s], recs[s], r, read_group ? &rg_id : nullptr);
    out += "\n";
  }
  return true;
}

// sort_for_coordinate_order (sam.rs:114-124): stable, by (HashMap name ->
// contig index, built in contig order so a repeated name keeps its last
// index; position), unmapped (position 0) last.
static void sort_coordinate(const Mapper* m, uint32_t n_src, const orc_records* const* recs, std::vector<uint64_t>& sel) {
  std::unordered_map<std::string, size_t> index;
  for (size_t i = 0; i < m->genome.contigs.size(); i++) index[m->genome.contigs[i].name] = i;
  auto key = [&](uint64_t g) {
    const orc_records* R = recs[g % n_src];
    const uint64_t r = g / n_src;
    if (R->pos[r] == 0) return std::make_pair(SIZE_MAX, SIZE_MAX);
    size_t ci = SIZE_MAX;
    if (R->contig[r] >= 0) {
      auto it = index.find(m->genome.contigs[R->contig[r]].name);
      if (it != index.end()) ci = it->second;
    }
    return std::make_pair(ci, (size_t)R->pos[r]);
  };
  std::stable_sort(sel.begin(), sel.end(), [&](uint64_t x, uint64_t y) { return key(x) < key(y); });
}

extern "C" {

int orc_write_sam(void* h, const char* path, const char* command_line, const orc_reads* reads,
                  const char* const* read_ids, const orc_records* recs) {
  std::vector<uint64_t> sel(recs->n);
  for (uint64_t i = 0; i < recs->n; i++) sel[i] = i;
  return orc_sam_write(h, command_line, nullptr, 0, 1, &reads, &read_ids, &recs, sel.data(), sel.size(), path);
}

int orc_sam_write(void* h, const char* command_line, const char* read_group, int coordinate_sorted, uint32_t n_src,
                  const orc_reads* const* reads, const char* const* const* ids, const orc_records* const* recs,
                  const uint64_t* sel, uint64_t n_sel, const char* path) {
  std::string out;
  if (!sam_text((Mapper*)h, command_line, read_group, coordinate_sorted != 0, n_src, reads, ids, recs, sel, n_sel,
                out))
    return -1;
  FILE* f = strcmp(path, "-") == 0 ? stdout : fopen(path, "wb");
  if (!f) { g_err = std::string("cannot write ") + path; return -1; }
  bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  if (f == stdout) ok = fflush(f) == 0 && ok;
  else ok = fclose(f) == 0 && ok;
  if (!ok) { g_err = std::string("short write to ") + path; return -1; }
  return 0;
}

int orc_sort_coordinate(void* h, uint32_t n_src, const orc_records* const* recs, const uint64_t* sel, uint64_t n_sel,
                        uint64_t* out) {
  std::vector<uint64_t> v(sel, sel + n_sel);
  sort_coordinate((Mapper*)h, n_src, recs, v);
  std::copy(v.begin(), v.end(), out);
  return 0;
}

struct ReadSet {
  std::vector<Read> reads;
};

void* orc_reads_parse(const char* path, int fasta, uint8_t quality_offset, const char* adapter) {
  try {
    ReadSet* rs = new ReadSet();
    rs->reads = fasta ? read_fasta_reads(path) : read_fastq(path, quality_offset);
    std::string ad = adapter ? adapter : "";
    preprocess(rs->reads, adapter ? &ad : nullptr);
    return rs;
  } catch (std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}
uint64_t orc_reads_count(void* rh) { return ((ReadSet*)rh)->reads.size(); }
uint64_t orc_reads_total_bases(void* rh) {
  uint64_t t = 0;
  for (auto& r : ((ReadSet*)rh)->reads) t += r.bases.size();
  return t;
}
void orc_reads_export(void* rh, uint8_t* bases, uint8_t* quals, uint64_t* offsets) {
  uint64_t o = 0;
  auto& rs = ((ReadSet*)rh)->reads;
  for (size_t i = 0; i < rs.size(); i++) {
    offsets[i] = o;
    memcpy(bases + o, rs[i].bases.data(), rs[i].bases.size());
    // quality track is padded / truncated to the sequence length
    for (size_t t = 0; t < rs[i].bases.size(); t++) quals[o + t] = t < rs[i].quals.size() ? rs[i].quals[t] : 30;
    o += rs[i].bases.size();
  }
  offsets[rs.size()] = o;
}
const char* orc_reads_id(void* rh, uint64_t i) { return ((ReadSet*)rh)->reads[i].id.c_str(); }
void orc_reads_free(void* rh) { delete (ReadSet*)rh; }

}  // extern "C"

// ===========================================================================
// The `probebwa` command line (src/main.rs), restated over this oracle.
// ===========================================================================
namespace {

struct UsageError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// One option of the clap grammar of main.rs:31-111.
struct OptSpec {
  const char* long_name;
  char short_name;
  bool takes_value;
};

// clap-style parse: "--name value", "--name=value", "-x value", "-xvalue",
// "-x=value"; flags take no value; a value may not start with '-' (clap's
// default without allow_hyphen_values) except the lone "-"; a repeated
// single-value option is an error; -M takes one or two values per
// occurrence and occurrences append.
struct Parsed {
  std::map<std::string, std::string> val;
  std::map<std::string, bool> flag;
  std::vector<std::string> multi;
};

Parsed parse_args(int argc, char** argv, int first, const std::vector<OptSpec>& specs, const char* multi_short) {
  Parsed p;
  auto find_long = [&](const std::string& n) -> const OptSpec* {
    for (auto& s : specs)
      if (s.long_name && n == s.long_name) return &s;
    return nullptr;
  };
  auto find_short = [&](char c) -> const OptSpec* {
    for (auto& s : specs)
      if (s.short_name == c) return &s;
    return nullptr;
  };
  auto is_value = [](const char* t) { return t[0] != '-' || t[1] == '\0'; };
  auto set = [&](const OptSpec* s, const std::string& v) {
    std::string key = s->long_name ? s->long_name : std::string(1, s->short_name);
    if (p.val.count(key)) throw UsageError("the argument '--" + key + "' cannot be used multiple times");
    p.val[key] = v;
  };
  for (int i = first; i < argc; i++) {
    std::string t = argv[i];
    if (multi_short && t.size() >= 2 && t[0] == '-' && t[1] == multi_short[0] && (t.size() == 2 || t[1] != '-')) {
      std::vector<std::string> vals;
      if (t.size() > 2) vals.push_back(t.substr(t[2] == '=' ? 3 : 2));
      while (vals.size() < 2 && i + 1 < argc && is_value(argv[i + 1])) vals.push_back(argv[++i]);
      if (vals.empty()) throw UsageError(std::string("a value is required for '-") + multi_short[0] + "'");
      for (auto& v : vals) p.multi.push_back(v);
      continue;
    }
    const OptSpec* s = nullptr;
    std::string inline_val;
    bool has_inline = false;
    if (t.rfind("--", 0) == 0 && t.size() > 2) {
      size_t eq = t.find('=');
      std::string name = t.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
      s = find_long(name);
      if (!s) throw UsageError("unexpected argument '" + t + "' found");
      if (eq != std::string::npos) { inline_val = t.substr(eq + 1); has_inline = true; }
    } else if (t.size() >= 2 && t[0] == '-' && t[1] != '-') {
      s = find_short(t[1]);
      if (!s) throw UsageError("unexpected argument '" + t + "' found");
      if (t.size() > 2) {
        inline_val = t.substr(t[2] == '=' ? 3 : 2);
        has_inline = true;
      }
    } else {
      throw UsageError("unexpected argument '" + t + "' found");
    }
    if (!s->takes_value) {
      if (has_inline) throw UsageError("unexpected value for a flag in '" + t + "'");
      std::string key = s->long_name;
      if (p.flag[key]) throw UsageError("the argument '--" + key + "' cannot be used multiple times");
      p.flag[key] = true;
      continue;
    }
    if (has_inline) {
      set(s, inline_val);
    } else {
      if (i + 1 >= argc || !is_value(argv[i + 1])) throw UsageError("a value is required for '" + t + "'");
      set(s, argv[++i]);
    }
  }
  return p;
}

// Rust's u32/usize from_str: optional '+', decimal digits only.
uint64_t parse_uint(const std::string& s, uint64_t max, const char* what) {
  size_t i = s.size() && s[0] == '+' ? 1 : 0;
  if (i == s.size()) throw UsageError(std::string("invalid value '") + s + "' for '" + what + "'");
  uint64_t v = 0;
  for (; i < s.size(); i++) {
    if (s[i] < '0' || s[i] > '9') throw UsageError(std::string("invalid value '") + s + "' for '" + what + "'");
    v = v * 10 + (uint64_t)(s[i] - '0');
    if (v > max) throw UsageError(std::string("invalid value '") + s + "' for '" + what + "'");
  }
  return v;
}
// f64::from_str: decimal or exponent notation, inf / infinity / nan; no
// surrounding whitespace, no hexadecimal.
double parse_f64(const std::string& s, const char* what) {
  const std::string bad = std::string("invalid value '") + s + "' for '" + what + "'";
  if (s.empty() || isspace((unsigned char)s[0])) throw UsageError(bad);
  std::string low;
  for (char c : s) low.push_back((char)tolower((unsigned char)c));
  size_t k = (low[0] == '+' || low[0] == '-') ? 1 : 0;
  if (low.compare(k, std::string::npos, "0x", 0, 2) == 0) throw UsageError(bad);
  const std::string body = low.substr(k);
  if (body == "inf" || body == "infinity") return low[0] == '-' ? -INFINITY : INFINITY;
  if (body == "nan") return NAN;
  for (char c : body)
    if (!(isdigit((unsigned char)c) || c == '.' || c == 'e' || c == '+' || c == '-')) throw UsageError(bad);
  char* end = nullptr;
  double v = strtod(s.c_str(), &end);
  if (end != s.c_str() + s.size()) throw UsageError(bad);
  return v;
}

struct RecordSet {
  std::vector<int32_t> contig, mate_contig, as_score, nm;
  std::vector<uint64_t> pos, mate_pos;
  std::vector<uint8_t> mapq;
  std::vector<uint16_t> flag;
  std::vector<int64_t> tlen;
  std::vector<double> log_lk, posterior;
  std::vector<uint32_t> cigar_off, cigar;
  orc_records c{};
  void alloc(uint64_t n, uint64_t bases) {
    contig.resize(n); mate_contig.resize(n); as_score.resize(n); nm.resize(n);
    pos.resize(n); mate_pos.resize(n); mapq.resize(n); flag.resize(n); tlen.resize(n);
    log_lk.resize(n); posterior.resize(n); cigar_off.resize(n + 1);
    cigar.resize(2 * bases + 2 * n + 16);
    c = orc_records{n, contig.data(), pos.data(), mapq.data(), flag.data(), mate_contig.data(), mate_pos.data(),
                    tlen.data(), log_lk.data(), posterior.data(), as_score.data(), nm.data(), cigar_off.data(),
                    cigar.data(), cigar.size()};
  }
};

struct ReadSoA {
  std::vector<u8> bases, quals;
  std::vector<uint64_t> offsets{0};
  std::vector<std::string> ids;
  std::vector<const char*> id_ptrs;
  orc_reads c{};
  void from(const std::vector<Read>& rs) {
    for (auto& r : rs) {
      for (size_t t = 0; t < r.bases.size(); t++) {
        bases.push_back(r.bases[t]);
        quals.push_back(t < r.quals.size() ? r.quals[t] : 30);
      }
      offsets.push_back(bases.size());
      ids.push_back(r.id);
    }
    for (auto& s : ids) id_ptrs.push_back(s.c_str());
    c = orc_reads{rs.size(), bases.data(), quals.data(), offsets.data()};
  }
};

std::vector<Read> load_reads(const std::string& path, bool fasta, u8 qoff, const std::string* adapter) {
  std::vector<Read> rs = fasta ? read_fasta_reads(path) : read_fastq(path, qoff);
  preprocess(rs, adapter);
  return rs;
}

int cli_map(int argc, char** argv) {
  static const std::vector<OptSpec> specs = {
      {"genome", 'g', true},       {"hash", 'h', true},        {"substitution-rate", 's', true},
      {"threads", 't', true},      {"gapopen", 0, true},       {"gapextend", 0, true},
      {"svprior", 0, true},        {"phred64", 0, false},      {"inputformat", 0, true},
      {"readgroup", 0, true},      {"outputformat", 'f', true}, {"output", 'o', true},
      {"labelfilter", 0, true},    {"casava8", 0, false},      {"adapter-strip", 0, true},
      {"index", 0, false}};
  Parsed p = parse_args(argc, argv, 2, specs, "M");
  if (!p.val.count("genome")) throw UsageError("the following required arguments were not provided: --genome");
  if (!p.val.count("hash")) throw UsageError("the following required arguments were not provided: --hash");
  orc_options o;
  orc_default_options(&o);
  if (p.val.count("substitution-rate")) o.substitution_rate = parse_f64(p.val["substitution-rate"], "--substitution-rate");
  if (p.val.count("threads")) o.threads = (int32_t)parse_uint(p.val["threads"], 1u << 20, "--threads");
  if (p.val.count("gapopen")) o.gap_open_phred = (uint32_t)parse_uint(p.val["gapopen"], 0xFFFFFFFFu, "--gapopen");
  if (p.val.count("gapextend")) o.gap_extend_phred = (uint32_t)parse_uint(p.val["gapextend"], 0xFFFFFFFFu, "--gapextend");
  if (p.val.count("svprior")) o.sv_prior_phred = parse_f64(p.val["svprior"], "--svprior");
  const u8 qoff = p.flag["phred64"] ? 64 : 33;
  const std::string informat = p.val.count("inputformat") ? p.val["inputformat"] : "fastq";
  if (informat != "fasta" && informat != "fastq")
    throw std::runtime_error("--inputformat must be 'fastq' or 'fasta', got '" + informat + "'");
  const std::string outformat = p.val.count("outputformat") ? p.val["outputformat"] : "sam";
  if (outformat != "sam" && outformat != "bam")
    throw std::runtime_error("--outputformat must be 'sam' or 'bam', got '" + outformat + "'");
  const char* rg = p.val.count("readgroup") ? p.val["readgroup"].c_str() : nullptr;
  if (rg) {
    std::string id, line;
    if (!parse_read_group(rg, id, line)) throw std::runtime_error(g_err);
  }
  std::string cl;
  for (int i = 0; i < argc; i++) cl += (i ? " " : "") + std::string(argv[i]);
  // map_paired runs its batches on rayon's global pool (all cores) whatever
  // --threads says (lib.rs:145-185); single-end honours --threads (lib.rs:97-104)
  if (p.multi.size() == 2) o.threads = 0;
  std::unique_ptr<Mapper> m(new Mapper());
  if (!m->open(p.val["genome"], p.val["hash"], o)) throw std::runtime_error(g_err);
  const bool fasta = informat == "fasta";
  std::string adapter = p.val.count("adapter-strip") ? p.val["adapter-strip"] : "";
  const std::string* ad = p.val.count("adapter-strip") ? &adapter : nullptr;
  // map_reads_with_format (lib.rs:65-104): two files = pairs, else single-end over all files
  const bool paired = p.multi.size() == 2;
  ReadSoA R[2];
  RecordSet S[2];
  uint32_t n_src = paired ? 2 : 1;
  if (paired) {
    R[0].from(load_reads(p.multi[0], fasta, qoff, ad));
    R[1].from(load_reads(p.multi[1], fasta, qoff, ad));
    if (R[0].c.n != R[1].c.n)
      throw std::runtime_error("paired-end input files have different read counts (" + std::to_string(R[0].c.n) +
                               " vs " + std::to_string(R[1].c.n) + ")");
    S[0].alloc(R[0].c.n, R[0].bases.size());
    S[1].alloc(R[1].c.n, R[1].bases.size());
    orc_insert_model im{o.insert_size_mean, o.insert_size_sd, 0};
    if (orc_map_paired(m.get(), &im, &R[0].c, &R[1].c, &S[0].c, &S[1].c) != 0) throw std::runtime_error(g_err);
  } else {
    std::vector<Read> all;
    for (auto& f : p.multi) {
      auto rs = load_reads(f, fasta, qoff, ad);
      all.insert(all.end(), rs.begin(), rs.end());
    }
    R[0].from(all);
    S[0].alloc(R[0].c.n, R[0].bases.size());
    if (orc_map_single(m.get(), &R[0].c, &S[0].c) != 0) throw std::runtime_error(g_err);
  }
  // record order: pairs interleaved (lib.rs:171-181)
  std::vector<uint64_t> sel;
  const uint64_t n = R[0].c.n;
  for (uint64_t i = 0; i < n * n_src; i++) {
    if (p.val.count("labelfilter")) {
      const std::string& id = R[i % n_src].ids[i / n_src];
      if (id.rfind(p.val["labelfilter"], 0) != 0) continue;
    }
    sel.push_back(i);
  }
  const bool index = p.flag["index"];
  if (index) {
    if (outformat != "bam") throw std::runtime_error("--index requires --outputformat=bam");
    if (!p.val.count("output"))
      throw std::runtime_error("--index requires --output FILE (an index needs a real file to index)");
    const orc_records* rp[2] = {&S[0].c, &S[1].c};
    sort_coordinate(m.get(), n_src, rp, sel);
  }
  if (outformat == "bam") throw std::runtime_error("BAM output is not built (SAM only)");
  const orc_reads* rp[2] = {&R[0].c, &R[1].c};
  const char* const* ip[2] = {R[0].id_ptrs.data(), R[1].id_ptrs.data()};
  const orc_records* sp[2] = {&S[0].c, &S[1].c};
  const std::string out = p.val.count("output") ? p.val["output"] : "-";
  if (orc_sam_write(m.get(), cl.c_str(), rg, index ? 1 : 0, n_src, rp, ip, sp, sel.data(), sel.size(), out.c_str()) != 0)
    throw std::runtime_error(g_err);
  return 0;
}

int cli_build_genome(int argc, char** argv) {
  static const std::vector<OptSpec> specs = {{"species", 's', true}, {"assembly", 'a', true}, {nullptr, 'G', true}};
  // positional FASTA files follow the options
  std::vector<char*> opts{argv[0], argv[1]};
  std::vector<std::string> files;
  for (int i = 2; i < argc; i++) {
    if (argv[i][0] == '-' && argv[i][1] != '\0') {
      opts.push_back(argv[i]);
      std::string t = argv[i];
      bool inline_v = (t.rfind("--", 0) == 0) ? t.find('=') != std::string::npos : t.size() > 2;
      if (!inline_v && i + 1 < argc) opts.push_back(argv[++i]);
    } else {
      files.push_back(argv[i]);
    }
  }
  Parsed p = parse_args((int)opts.size(), opts.data(), 2, specs, nullptr);
  for (const char* k : {"species", "assembly", "G"})
    if (!p.val.count(k)) throw UsageError(std::string("the following required arguments were not provided: ") + k);
  printf("Building genome index for %s %s...\n", p.val["species"].c_str(), p.val["assembly"].c_str());
  std::vector<const char*> fp;
  for (auto& f : files) fp.push_back(f.c_str());
  if (orc_build_genome(p.val["G"].c_str(), p.val["species"].c_str(), p.val["assembly"].c_str(), (int)fp.size(),
                       fp.data()) != 0)
    throw std::runtime_error(g_err);
  printf("Done. Index written to %s.stidx\n", p.val["G"].c_str());
  return 0;
}

int cli_build_hash(int argc, char** argv) {
  static const std::vector<OptSpec> specs = {{"genome", 'g', true}, {nullptr, 'H', true}};
  Parsed p = parse_args(argc, argv, 2, specs, nullptr);
  if (!p.val.count("genome") || !p.val.count("H")) throw UsageError("--genome and -H are required");
  printf("Building 15-mer hash table...\n");
  if (orc_build_hash(p.val["genome"].c_str(), p.val["H"].c_str(), 15, 5, 300) != 0) throw std::runtime_error(g_err);
  printf("Done. Hash table written to %s.sthash\n", p.val["H"].c_str());
  return 0;
}

}  // namespace

extern "C" int orc_cli_main(int argc, char** argv) {
  try {
    if (argc < 2) throw UsageError("a subcommand is required: map, build-genome, build-hash");
    const std::string cmd = argv[1];
    if (cmd == "map") return cli_map(argc, argv);
    if (cmd == "build-genome") return cli_build_genome(argc, argv);
    if (cmd == "build-hash") return cli_build_hash(argc, argv);
    throw UsageError("unrecognized subcommand '" + cmd + "'");
  } catch (UsageError& e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 2;
  } catch (std::exception& e) {
    fprintf(stderr, "Error: %s\n", e.what());
    return 1;
  }
}
