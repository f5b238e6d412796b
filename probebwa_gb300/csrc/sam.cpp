// sam.cpp -- SAM text for mapped records (src/io/sam.rs:37-143).
//
// Header: @HD VN:1.6 SO:unsorted, one @SQ per contig, @PG with the caller's
// command line (sam.rs:92-100). Records: 11 mandatory columns, no optional
// tags; RNEXT is the mate contig name (never '='); SEQ and QUAL are the input
// read in the aligned orientation, QUAL written as the raw Phred score bytes
// (String::from_utf8_lossy of the scores, sam.rs:52); CIGAR '*' only when
// empty.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_pipeline.h"

namespace {

// String::from_utf8_lossy: valid UTF-8 is copied, each maximal invalid
// subsequence becomes U+FFFD.
void utf8_lossy_append(std::string& out, const uint8_t* s, size_t n) {
  size_t i = 0;
  while (i < n) {
    uint8_t c = s[i];
    if (c < 0x80) {
      out.push_back((char)c);
      i++;
      continue;
    }
    size_t need = 0;
    uint8_t lo = 0x80, hi = 0xBF;
    if (c >= 0xC2 && c <= 0xDF) need = 1;
    else if (c == 0xE0) { need = 2; lo = 0xA0; }
    else if ((c >= 0xE1 && c <= 0xEC) || c == 0xEE || c == 0xEF) need = 2;
    else if (c == 0xED) { need = 2; hi = 0x9F; }
    else if (c == 0xF0) { need = 3; lo = 0x90; }
    else if (c >= 0xF1 && c <= 0xF3) need = 3;
    else if (c == 0xF4) { need = 3; hi = 0x8F; }
    else {
      out += "\xEF\xBF\xBD";
      i++;
      continue;
    }
    size_t j = 1;
    bool ok = true;
    for (; j <= need; j++) {
      if (i + j >= n) { ok = false; break; }
      uint8_t cc = s[i + j];
      uint8_t l = j == 1 ? lo : 0x80, h = j == 1 ? hi : 0xBF;
      if (cc < l || cc > h) { ok = false; break; }
    }
    if (ok) {
      out.append((const char*)s + i, need + 1);
      i += need + 1;
    } else {
      out += "\xEF\xBF\xBD";
      i += j;
    }
  }
}

uint8_t upper(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }
uint8_t comp(uint8_t b) {
  switch (b) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'C': return 'G';
    case 'G': return 'C';
    default: return 'N';
  }
}

}  // namespace

extern "C" int pbw_write_sam(pbw_handle* h, const char* path, const char* command_line, const pbw_reads* reads,
                             const char* const* read_ids, const pbw_records* recs) {
  if (!h || !path || !reads || !recs || !read_ids) return PBW_ERR_ARG;
  std::string out;
  out += "@HD\tVN:1.6\tSO:unsorted\n";
  for (size_t c = 0; c < h->names.size(); c++)
    out += "@SQ\tSN:" + h->names[c] + "\tLN:" + std::to_string(h->lens[c]) + "\n";
  out += std::string("@PG\tID:probebwa\tPN:probebwa\tVN:0.1.0\tCL:") + (command_line ? command_line : "") + "\n";
  static const char OPS[] = "MIDXSHXXXXXXXXXX";
  std::vector<uint8_t> seq, qual;
  for (uint64_t i = 0; i < recs->n; i++) {
    out += read_ids[i];
    out += '\t';
    out += std::to_string(recs->flag[i]);
    out += '\t';
    const int32_t c = recs->contig[i];
    out += (c >= 0 && (size_t)c < h->names.size()) ? h->names[c] : std::string("*");
    out += '\t';
    out += std::to_string(recs->pos[i]);
    out += '\t';
    out += std::to_string((unsigned)recs->mapq[i]);
    out += '\t';
    std::string cs;
    for (uint32_t k = recs->cigar_off[i]; k < recs->cigar_off[i + 1]; k++) {
      cs += std::to_string(recs->cigar[k] >> 4);
      cs.push_back(OPS[recs->cigar[k] & 15]);
    }
    out += cs.empty() ? std::string("*") : cs;
    out += '\t';
    const int32_t mc = recs->mate_contig[i];
    out += (mc >= 0 && (size_t)mc < h->names.size()) ? h->names[mc] : std::string("*");
    out += '\t';
    out += std::to_string(recs->mate_pos[i]);
    out += '\t';
    out += std::to_string(recs->tlen[i]);
    out += '\t';
    const uint64_t a = reads->offsets[i], b = reads->offsets[i + 1];
    seq.assign(reads->bases + a, reads->bases + b);
    qual.assign(reads->quals + a, reads->quals + b);
    for (auto& x : seq) x = upper(x);
    if (recs->pos[i] != 0 && (recs->flag[i] & 0x10)) {
      std::reverse(seq.begin(), seq.end());
      for (auto& x : seq) x = comp(x);
      std::reverse(qual.begin(), qual.end());
    }
    utf8_lossy_append(out, seq.data(), seq.size());
    out += '\t';
    utf8_lossy_append(out, qual.data(), qual.size());
    out += '\n';
  }
  FILE* f = fopen(path, "wb");
  if (!f) {
    h->err = std::string("cannot write ") + path;
    return PBW_ERR_IO;
  }
  bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  fclose(f);
  if (!ok) {
    h->err = std::string("short write to ") + path;
    return PBW_ERR_IO;
  }
  return PBW_OK;
}
