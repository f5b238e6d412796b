// genome_build.cpp -- `build-genome`: FASTA files into a .stidx genome index
// (GenomeIndexBuilder, src/index/genome.rs:98-148).
//
// Each file is read whole (gunzipped for a ".gz" name, UTF-8 checked, as the
// reads loader); records follow the genome's FastaReader (genome.rs:150-213):
// a record starts at a line beginning with '>', its name is the first
// whitespace-separated token after the leading '>'s, its sequence the
// concatenated trimmed lines up to the next trimmed line starting with '>'.
// Contig::from_ascii (genome.rs:17-45) packs A C G T (either case) as 0 1 2 3,
// base p at bits (p % 4) * 2 of byte p / 4, any other byte as 0 plus an entry
// in the half-open runs of non-ACGT positions. The file is bincode's legacy
// layout (fixed-width little-endian integers, u64 length prefixes) of
// GenomeIndex { species, assembly, contigs: [Contig { name, packed, n_runs,
// length }], total_length } (genome.rs:72-77, types.rs:107-112).
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "abi_guard.h"
#include "fastx_text.h"

namespace pbw {
void set_handleless_error(const std::string& s);
}

namespace {

using namespace pbw::text;

struct Contig {
  std::string name;
  std::vector<uint8_t> packed;
  std::vector<uint32_t> runs;  // start, end pairs
  uint64_t length = 0;
};

void pack_contig(Contig& c, const std::vector<uint8_t>& seq) {
  c.length = seq.size();
  c.packed.assign((seq.size() + 3) / 4, 0);
  bool in_run = false;
  uint64_t run_start = 0;
  for (uint64_t p = 0; p < seq.size(); p++) {
    const uint8_t b = seq[p];
    uint8_t bits = 0;
    bool acgt = true;
    switch (b) {
      case 'A': case 'a': bits = 0; break;
      case 'C': case 'c': bits = 1; break;
      case 'G': case 'g': bits = 2; break;
      case 'T': case 't': bits = 3; break;
      default: acgt = false;
    }
    c.packed[p >> 2] |= (uint8_t)(bits << ((p & 3) * 2));
    if (acgt) {
      if (in_run) {
        c.runs.push_back((uint32_t)run_start);
        c.runs.push_back((uint32_t)p);
        in_run = false;
      }
    } else if (!in_run) {
      in_run = true;
      run_start = p;
    }
  }
  if (in_run) {
    c.runs.push_back((uint32_t)run_start);
    c.runs.push_back((uint32_t)seq.size());
  }
}

int add_fasta(const char* path, std::vector<Contig>& out) {
  Text buf;
  std::string err;
  const int rc = load_text(path, buf, err);
  if (rc != PBW_OK) {
    pbw::set_handleless_error(err);
    return rc;
  }
  Lines L{buf.data(), buf.data() + buf.size()};
  Span line, header{nullptr, 0};
  bool have = false;
  std::vector<uint8_t> seq;
  while (true) {
    if (!have) {
      bool found = false;
      while (L.next(line))
        if (line.n && line.p[0] == '>') {
          found = true;
          break;
        }
      if (!found) break;
      header = line;
    }
    have = false;
    const Span id = first_token(strip_leading(header, '>'));
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
    out.emplace_back();
    out.back().name.assign(id.p, id.n);
    pack_contig(out.back(), seq);
    if (!have) break;
  }
  return PBW_OK;
}

struct Writer {
  FILE* f;
  bool ok = true;
  void bytes(const void* p, size_t n) {
    if (n && fwrite(p, 1, n, f) != n) ok = false;
  }
  void u64(uint64_t v) {
    uint8_t b[8];
    for (int i = 0; i < 8; i++) b[i] = (uint8_t)(v >> (8 * i));
    bytes(b, 8);
  }
  void u32(uint32_t v) {
    uint8_t b[4];
    for (int i = 0; i < 4; i++) b[i] = (uint8_t)(v >> (8 * i));
    bytes(b, 4);
  }
  void str(const std::string& s) {
    u64(s.size());
    bytes(s.data(), s.size());
  }
};

}  // namespace

namespace {

int build_genome(const char* out_prefix, const char* species, const char* assembly, uint32_t n_files,
                 const char* const* fasta_paths) {
  std::vector<Contig> contigs;
  for (uint32_t i = 0; i < n_files; i++) {
    const int rc = add_fasta(fasta_paths[i], contigs);
    if (rc != PBW_OK) return rc;
  }
  const std::string path = std::string(out_prefix) + ".stidx";
  std::vector<char> vbuf(1 << 22);  // stdio buffer; outlives the stream
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) {
    pbw::set_handleless_error("cannot write " + path);
    return PBW_ERR_IO;
  }
  setvbuf(f, vbuf.data(), _IOFBF, vbuf.size());
  Writer w{f};
  w.str(species);
  w.str(assembly);
  w.u64(contigs.size());
  uint64_t total = 0;
  for (const Contig& c : contigs) {
    w.str(c.name);
    w.u64(c.packed.size());
    w.bytes(c.packed.data(), c.packed.size());
    w.u64(c.runs.size() / 2);
    for (uint32_t v : c.runs) w.u32(v);
    w.u64(c.length);
    total += c.length;
  }
  w.u64(total);
  const bool closed = fclose(f) == 0;
  if (!w.ok || !closed) {
    pbw::set_handleless_error("short write to " + path);
    return PBW_ERR_IO;
  }
  return PBW_OK;
}

}  // namespace

extern "C" int pbw_build_genome(const char* out_prefix, const char* species, const char* assembly, uint32_t n_files,
                                const char* const* fasta_paths) {
  if (!out_prefix || !species || !assembly || (n_files && !fasta_paths)) {
    pbw::set_handleless_error("pbw_build_genome: null argument");
    return PBW_ERR_ARG;
  }
  return pbw::guard_handleless("pbw_build_genome",
                               [&] { return build_genome(out_prefix, species, assembly, n_files, fasta_paths); });
}
