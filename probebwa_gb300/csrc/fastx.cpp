// fastx.cpp -- the input side of the mapping path: FASTQ / FASTA reads into
// the structure-of-arrays layout the map calls take (src/io/fastx.rs).
//
// A regular file is mapped read-only (other inputs are read into memory; a
// name ending in ".gz" is gunzipped, as open_maybe_gz, fastx.rs:120-129, with
// every gzip member decoded in turn like flate2's MultiGzDecoder), checked
// to be UTF-8 eight ASCII bytes at a time, and split into lines with memchr;
// each record is decoded straight into the concatenated base, quality and
// offset arrays.
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
#include <memory>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "abi_guard.h"
#include "fastx_text.h"
#include "pbw_kernels.h"

struct pbw_read_set {
  std::vector<uint8_t> bases, quals;
  std::vector<uint64_t> offsets{0};
  std::vector<char> id_chars;  // NUL-terminated IDs, back to back
  std::vector<uint64_t> id_off;
};

namespace {

using namespace pbw::text;

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

// Sequence text appended to the read set's bases, upper-cased.
void append_bases(pbw_read_set* rs, Span t) {
  const size_t o = rs->bases.size();
  rs->bases.resize(o + t.n);
  uint8_t* d = rs->bases.data() + o;
  for (size_t k = 0; k < t.n; k++) d[k] = upper((uint8_t)t.p[k]);
}

// Quality text appended to the read set's quals: the byte minus the offset,
// saturating at 0.
void append_quals(pbw_read_set* rs, Span t, uint8_t offset) {
  const size_t o = rs->quals.size();
  rs->quals.resize(o + t.n);
  uint8_t* d = rs->quals.data() + o;
  for (size_t k = 0; k < t.n; k++) {
    const uint8_t c = (uint8_t)t.p[k];
    d[k] = c > offset ? (uint8_t)(c - offset) : (uint8_t)0;
  }
}

// Ends the read whose bases start at b0 (its qualities, as many as were
// given, start at b0 too): the adapter's 3' overlap is cut, and the quality
// track is cut or padded with 30 to the kept length.
void end_read(pbw_read_set* rs, size_t b0, const std::string* adapter) {
  const size_t n = rs->bases.size() - b0;
  const size_t keep = adapter ? adapter_keep(rs->bases.data() + b0, n, *adapter) : n;
  rs->bases.resize(b0 + keep);
  rs->quals.resize(b0 + keep, 30);
  rs->offsets.push_back(b0 + keep);
}

}  // namespace

namespace {

int reads_load(const char* path, int fasta, uint8_t quality_offset, const char* adapter, pbw_read_set** out) {
  pbw::text::Text buf;
  std::string err;
  const int lrc = pbw::text::load_text(path, buf, err);
  if (lrc != PBW_OK) {
    pbw::set_handleless_error(err);
    return lrc;
  }
  std::unique_ptr<pbw_read_set> owner(new pbw_read_set());
  pbw_read_set* rs = owner.get();
  // sequence bytes are at most half of a FASTQ file, at most all of a FASTA one
  rs->bases.reserve(fasta ? buf.size() : buf.size() / 2 + 64);
  rs->quals.reserve(rs->bases.capacity());
  const std::string ad_s = adapter ? adapter : "";
  const std::string* ad = adapter ? &ad_s : nullptr;
  Builder bld{rs};
  Lines L{buf.data(), buf.data() + buf.size()};
  Span line;
  if (!fasta) {
    while (L.next(line)) {
      bld.add(first_token(strip_leading(line, '@')));
      const size_t b0 = rs->bases.size();  // == rs->quals.size(): every read ends both at its length
      while (L.next(line)) {
        const Span t = trim(line);
        if (t.n && t.p[0] == '+') break;
        append_bases(rs, t);
      }
      const size_t n = rs->bases.size() - b0;
      while (L.next(line)) {
        append_quals(rs, trim(line), quality_offset);
        if (rs->quals.size() - b0 >= n) break;
      }
      end_read(rs, b0, ad);
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
      const size_t b0 = rs->bases.size();
      while (L.next(line)) {
        const Span t = trim(line);
        if (t.n && t.p[0] == '>') {
          header = line;
          have = true;
          break;
        }
        append_bases(rs, t);
      }
      rs->quals.resize(rs->bases.size(), 40);  // FASTA reads: every quality 40
      end_read(rs, b0, ad);
      if (!have) break;
    }
  }
  *out = owner.release();
  return PBW_OK;
}

}  // namespace

extern "C" {

int pbw_reads_load(const char* path, int fasta, uint8_t quality_offset, const char* adapter, pbw_read_set** out) {
  if (!path || !out) return PBW_ERR_ARG;
  *out = nullptr;
  return pbw::guard_handleless("pbw_reads_load",
                               [&] { return reads_load(path, fasta, quality_offset, adapter, out); });
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
