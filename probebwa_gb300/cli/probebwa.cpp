// probebwa.cpp -- the `probebwa` command line over the C ABI
// (include/probebwa_gpu.h): the drop-in for the reference binary's `map`
// subcommand (src/main.rs:51-111, 130-189).
//
// Subcommands map, build-genome and build-hash. For map: same flags, same
// checks in the same order, same SAM stream:
//   probebwa map -g|--genome PREFIX -h|--hash PREFIX [-s|--substitution-rate F]
//     [-t|--threads N] [--gapopen N] [--gapextend N] [--svprior F] [--phred64]
//     [--inputformat fastq|fasta] [--readgroup ID:x,...] [-f|--outputformat sam]
//     [-o|--output FILE] [--labelfilter PREFIX] [--casava8]
//     [--adapter-strip SEQ] [--index] -M READS [READS2]
// Two read files map as pairs (records interleaved mate 1, mate 2, lib.rs:
// 171-181); one (or three and more) as single-end reads. --threads is accepted
// and has no effect (the mapping runs on the GPU); --casava8 changes nothing
// in the reference either (fastx.rs:29-41). -f bam writes BGZF BAM to the
// --output file (required, as in the reference) and --index (which needs it)
// coordinate-sorts the records on the GPU and writes FILE.bai beside it
// (main.rs:162-186, pbw_bam_write). Errors: usage errors exit 2, others
// print "Error: ..." and exit 1. build-genome / build-hash write the same
// index files as the reference's subcommands (the hash table is built on the
// GPU).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <initializer_list>
#include <map>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/probebwa_gpu.h"

namespace {

struct Usage : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct Fail : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---- arguments (clap's grammar for the derive in main.rs:31-111) ----
struct Flag {
  const char* name;  // long name ("" for -M)
  char short_name;
  bool value;        // takes a value
};

const Flag MAP_FLAGS[] = {
    {"genome", 'g', true},      {"hash", 'h', true},         {"substitution-rate", 's', true},
    {"threads", 't', true},     {"gapopen", 0, true},        {"gapextend", 0, true},
    {"svprior", 0, true},       {"phred64", 0, false},       {"inputformat", 0, true},
    {"readgroup", 0, true},     {"outputformat", 'f', true}, {"output", 'o', true},
    {"labelfilter", 0, true},   {"casava8", 0, false},       {"adapter-strip", 0, true},
    {"index", 0, false},
};
const Flag GENOME_FLAGS[] = {{"species", 's', true}, {"assembly", 'a', true}, {"", 'G', true}};
const Flag HASH_FLAGS[] = {{"genome", 'g', true}, {"", 'H', true}};

struct Args {
  std::map<std::string, std::string> opt;
  std::map<std::string, bool> on;
  std::vector<std::string> reads;  // -M values, appended over occurrences
  std::vector<std::string> files;  // positional arguments
  bool has(const char* k) const { return opt.count(k) != 0; }
  std::string get(const char* k, const char* dflt) const {
    auto it = opt.find(k);
    return it == opt.end() ? dflt : it->second;
  }
};

bool looks_like_value(const char* t) { return t[0] != '-' || t[1] == '\0'; }

// flags: the subcommand's options; with_m: -M takes one or two values per
// occurrence; positional: bare arguments are collected in files.
Args parse(int argc, char** argv, const Flag* flags, size_t n_flags, bool with_m, bool positional) {
  Args a;
  for (int i = 2; i < argc; i++) {
    const std::string t = argv[i];
    if (with_m && t.size() >= 2 && t[0] == '-' && t[1] == 'M') {
      int got = 0;
      if (t.size() > 2) {
        a.reads.push_back(t.substr(t[2] == '=' ? 3 : 2));
        got++;
      }
      while (got < 2 && i + 1 < argc && looks_like_value(argv[i + 1])) {
        a.reads.push_back(argv[++i]);
        got++;
      }
      if (!got) throw Usage("a value is required for '-M <READS>...' but none was supplied");
      continue;
    }
    if (positional && looks_like_value(argv[i])) {
      a.files.push_back(t);
      continue;
    }
    const Flag* f = nullptr;
    bool inline_v = false;
    std::string v;
    if (t.size() > 2 && t[0] == '-' && t[1] == '-') {
      const size_t eq = t.find('=');
      const std::string name = t.substr(2, eq == std::string::npos ? std::string::npos : eq - 2);
      for (size_t q = 0; q < n_flags; q++)
        if (flags[q].name[0] && name == flags[q].name) f = &flags[q];
      if (eq != std::string::npos) {
        inline_v = true;
        v = t.substr(eq + 1);
      }
    } else if (t.size() >= 2 && t[0] == '-' && t[1] != '-') {
      for (size_t q = 0; q < n_flags; q++)
        if (flags[q].short_name && flags[q].short_name == t[1]) f = &flags[q];
      if (t.size() > 2) {
        inline_v = true;
        v = t.substr(t[2] == '=' ? 3 : 2);
      }
    }
    if (!f) throw Usage("unexpected argument '" + t + "' found");
    const std::string key = f->name[0] ? f->name : std::string(1, f->short_name);
    if (!f->value) {
      if (inline_v) throw Usage("unexpected value for '--" + key + "'");
      if (a.on[key]) throw Usage("the argument '--" + key + "' cannot be used multiple times");
      a.on[key] = true;
      continue;
    }
    if (!inline_v) {
      if (i + 1 >= argc || !looks_like_value(argv[i + 1]))
        throw Usage("a value is required for '--" + key + "' but none was supplied");
      v = argv[++i];
    }
    if (a.has(key.c_str())) throw Usage("the argument '--" + key + "' cannot be used multiple times");
    a.opt[key] = v;
  }
  return a;
}

void require(const Args& a, std::initializer_list<const char*> keys) {
  for (const char* k : keys)
    if (!a.has(k)) throw Usage(std::string("the following required arguments were not provided: ") + k);
}

// u32 / usize as Rust's from_str: optional '+', then decimal digits.
uint64_t to_uint(const std::string& s, uint64_t max, const char* what) {
  size_t i = (!s.empty() && s[0] == '+') ? 1 : 0;
  if (i == s.size()) throw Usage("invalid value '" + s + "' for '--" + what + "'");
  uint64_t v = 0;
  for (; i < s.size(); i++) {
    if (s[i] < '0' || s[i] > '9') throw Usage("invalid value '" + s + "' for '--" + what + "'");
    v = v * 10 + (uint64_t)(s[i] - '0');
    if (v > max) throw Usage("invalid value '" + s + "' for '--" + what + "'");
  }
  return v;
}

// f64 as Rust's from_str: decimal / exponent forms, inf, infinity, nan (any
// case, optional sign); no whitespace, no hexadecimal.
double to_f64(const std::string& s, const char* what) {
  const std::string bad = "invalid value '" + s + "' for '--" + what + "'";
  if (s.empty()) throw Usage(bad);
  size_t k = (s[0] == '+' || s[0] == '-') ? 1 : 0;
  std::string body;
  for (size_t i = k; i < s.size(); i++) body.push_back((char)((s[i] >= 'A' && s[i] <= 'Z') ? s[i] + 32 : s[i]));
  if (body == "inf" || body == "infinity") return s[0] == '-' ? -HUGE_VAL : HUGE_VAL;
  if (body == "nan") return std::nan("");
  if (body.empty()) throw Usage(bad);
  for (char c : body)
    if (!((c >= '0' && c <= '9') || c == '.' || c == 'e' || c == '+' || c == '-')) throw Usage(bad);
  char* end = nullptr;
  const double v = strtod(s.c_str(), &end);
  if (end != s.c_str() + s.size()) throw Usage(bad);
  return v;
}

// The checks of ReadGroup::parse (sam.rs:17-32); the @RG line itself is
// built by pbw_sam_write.
void check_read_group(const std::string& spec) {
  bool id = false;
  size_t a = 0;
  while (true) {
    const size_t e = spec.find(',', a);
    const std::string pair = spec.substr(a, e == std::string::npos ? std::string::npos : e - a);
    const size_t c = pair.find(':');
    if (c == std::string::npos) throw Fail("--readgroup: expected TAG:VALUE, got '" + pair + "'");
    if (pair.compare(0, c, "ID") == 0 && c == 2) id = true;
    if (e == std::string::npos) break;
    a = e + 1;
  }
  if (!id) throw Fail("--readgroup must set at least an ID tag");
}

// Phase wall times on stderr when PROBEBWA_TIMING is set (no effect on output).
struct Timer {
  const char* what;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  explicit Timer(const char* w) : what(w) {}
  ~Timer() {
    static const bool on = getenv("PROBEBWA_TIMING") != nullptr;
    if (on)
      fprintf(stderr, "[probebwa] %s: %.3f s\n", what,
              std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count());
  }
};

// ---- reads and records ----
struct ReadFile {
  pbw_read_set* rs = nullptr;
  pbw_reads view{};
  ReadFile() = default;
  ReadFile(const ReadFile&) = delete;
  ~ReadFile() { pbw_reads_free(rs); }
};

// The reads of one source: one file's read set as it is, or several files
// concatenated (single-end runs over more than two files).
struct Reads {
  std::vector<ReadFile*> files;
  std::vector<uint8_t> bases, quals;
  std::vector<uint64_t> offsets{0};
  std::vector<const char*> id_ptrs;  // into the read sets
  pbw_reads view{};
  ~Reads() {
    for (ReadFile* f : files) delete f;
  }
  uint64_t n() const { return view.n; }
  void finish() {
    for (ReadFile* f : files)
      for (uint64_t i = 0; i < f->view.n; i++) id_ptrs.push_back(pbw_reads_id(f->rs, i));
    if (files.size() == 1) {
      view = files[0]->view;
      return;
    }
    for (ReadFile* f : files) {
      const pbw_reads& v = f->view;
      const uint64_t base = offsets.back();
      bases.insert(bases.end(), v.bases, v.bases + v.offsets[v.n]);
      quals.insert(quals.end(), v.quals, v.quals + v.offsets[v.n]);
      for (uint64_t i = 0; i < v.n; i++) offsets.push_back(base + v.offsets[i + 1]);
    }
    view = pbw_reads{id_ptrs.size(), bases.data(), quals.data(), offsets.data()};
  }
};

struct Records {
  std::vector<int32_t> contig, mate_contig, as_score, nm;
  std::vector<uint64_t> pos, mate_pos;
  std::vector<uint8_t> mapq;
  std::vector<uint16_t> flag;
  std::vector<int64_t> tlen;
  std::vector<double> log_lk, posterior;
  std::vector<uint32_t> cigar_off, cigar;
  pbw_records view{};
  void alloc(const pbw_reads& r) {
    uint64_t n = 0, cap = 0;
    pbw_records_reserve(&r, &n, &cap);
    contig.resize(n);
    mate_contig.resize(n);
    as_score.resize(n);
    nm.resize(n);
    pos.resize(n);
    mate_pos.resize(n);
    mapq.resize(n);
    flag.resize(n);
    tlen.resize(n);
    log_lk.resize(n);
    posterior.resize(n);
    cigar_off.resize(n + 1);
    cigar.resize(cap ? cap : 1);
    view = pbw_records{n,          contig.data(), pos.data(),      mapq.data(),      flag.data(),
                       mate_contig.data(), mate_pos.data(), tlen.data(), log_lk.data(), posterior.data(),
                       as_score.data(), nm.data(), cigar_off.data(), cigar.data(), cap};
  }
};

struct Handle {
  pbw_handle* h = nullptr;
  ~Handle() { pbw_close(h); }
  void check(int rc) const {
    if (rc != PBW_OK) throw Fail(pbw_last_error(h));
  }
};

int run_map(int argc, char** argv) {
  const Args a = parse(argc, argv, MAP_FLAGS, sizeof(MAP_FLAGS) / sizeof(MAP_FLAGS[0]), true, false);
  require(a, {"genome", "hash"});
  pbw_options o;
  pbw_default_options(&o);
  if (a.has("substitution-rate")) o.substitution_rate = to_f64(a.get("substitution-rate", ""), "substitution-rate");
  if (a.has("threads")) (void)to_uint(a.get("threads", ""), ~0ull, "threads");
  if (a.has("gapopen")) o.gap_open_phred = (uint32_t)to_uint(a.get("gapopen", ""), 0xFFFFFFFFu, "gapopen");
  if (a.has("gapextend")) o.gap_extend_phred = (uint32_t)to_uint(a.get("gapextend", ""), 0xFFFFFFFFu, "gapextend");
  if (a.has("svprior")) o.sv_prior_phred = to_f64(a.get("svprior", ""), "svprior");
  const uint8_t qoff = a.on.count("phred64") ? 64 : 33;
  const std::string informat = a.get("inputformat", "fastq");
  if (informat != "fasta" && informat != "fastq")
    throw Fail("--inputformat must be 'fastq' or 'fasta', got '" + informat + "'");
  const std::string outformat = a.get("outputformat", "sam");
  if (outformat != "sam" && outformat != "bam")
    throw Fail("--outputformat must be 'sam' or 'bam', got '" + outformat + "'");
  const bool have_rg = a.has("readgroup");
  const std::string rg = a.get("readgroup", "");
  if (have_rg) check_read_group(rg);
  std::string cl;
  for (int i = 0; i < argc; i++) cl += (i ? " " : "") + std::string(argv[i]);

  // The index load (pbw_open) and the read files are independent: they run on
  // their own threads, then mapping starts.
  const bool fasta = informat == "fasta";
  const std::string adapter = a.get("adapter-strip", "");
  const char* ad = a.has("adapter-strip") ? adapter.c_str() : nullptr;
  const bool paired = a.reads.size() == 2;
  const uint32_t n_src = paired ? 2 : 1;
  Handle H;
  Reads R[2];
  Records S[2];
  std::vector<ReadFile*> files(a.reads.size(), nullptr);
  for (auto& f : files) f = new ReadFile();
  for (size_t i = 0; i < files.size(); i++) R[paired ? i : 0].files.push_back(files[i]);
  std::vector<int> load_rc(files.size(), PBW_OK);
  std::vector<std::string> load_err(files.size());
  int open_rc = PBW_OK;
  std::string open_err;
  {
    Timer tm("load (index + reads, concurrent)");
    std::vector<std::thread> th;
    th.emplace_back([&] {
      open_rc = pbw_open(a.get("genome", "").c_str(), a.get("hash", "").c_str(), &o, &H.h);
      if (open_rc != PBW_OK) open_err = pbw_last_error(nullptr);
    });
    for (size_t i = 0; i < files.size(); i++)
      th.emplace_back([&, i] {
        load_rc[i] = pbw_reads_load(a.reads[i].c_str(), fasta ? 1 : 0, qoff, ad, &files[i]->rs);
        if (load_rc[i] == PBW_OK) pbw_reads_get(files[i]->rs, &files[i]->view);
        else load_err[i] = pbw_last_error(nullptr);
      });
    for (auto& t : th) t.join();
  }
  if (open_rc != PBW_OK) throw Fail(open_err);
  for (size_t i = 0; i < files.size(); i++)
    if (load_rc[i] != PBW_OK) throw Fail(load_err[i]);
  if (paired) {
    R[0].finish();
    R[1].finish();
    if (R[0].n() != R[1].n())
      throw Fail("paired-end input files have different read counts (" + std::to_string(R[0].n()) + " vs " +
                 std::to_string(R[1].n()) + ")");
    S[0].alloc(R[0].view);
    S[1].alloc(R[1].view);
    pbw_insert_model m{o.insert_size_mean, o.insert_size_sd, 0};
    Timer tm("map (pairs)");
    H.check(pbw_map_paired(H.h, &m, &R[0].view, &R[1].view, &S[0].view, &S[1].view));
  } else {
    R[0].finish();
    S[0].alloc(R[0].view);
    Timer tm("map (single-end)");
    H.check(pbw_map_single(H.h, &R[0].view, &S[0].view));
  }
  // --labelfilter (main.rs:158-160)
  std::vector<uint64_t> sel;
  const uint64_t n = R[0].n() * n_src;
  const bool filter = a.has("labelfilter");
  const std::string prefix = a.get("labelfilter", "");
  for (uint64_t g = 0; g < n; g++)
    if (!filter || strncmp(R[g % n_src].id_ptrs[g / n_src], prefix.c_str(), prefix.size()) == 0) sel.push_back(g);
  pbw_sam_source src[2];
  for (uint32_t s = 0; s < n_src; s++) src[s] = pbw_sam_source{&R[s].view, R[s].id_ptrs.data(), &S[s].view};
  const bool index = a.on.count("index") != 0;
  if (index) {
    if (outformat != "bam") throw Fail("--index requires --outputformat=bam");
    if (!a.has("output")) throw Fail("--index requires --output FILE (an index needs a real file to index)");
    std::vector<uint64_t> sorted(sel.size() + 1);
    H.check(pbw_sort_coordinate(H.h, n_src, src, sel.data(), sel.size(), sorted.data()));
    sorted.resize(sel.size());
    sel.swap(sorted);
  }
  pbw_sam_options so{cl.c_str(), have_rg ? rg.c_str() : nullptr, index ? 1 : 0};
  const uint64_t none = 0;  // an empty selection still passes a list (NULL means every record)
  if (outformat == "bam") {
    if (!a.has("output"))
      throw Fail("--outputformat=bam requires --output FILE (binary output shouldn't go to a terminal)");
    Timer tm("BAM (SAM formatted on the GPU, BGZF on the host threads)");
    H.check(pbw_bam_write(H.h, &so, n_src, src, sel.empty() ? &none : sel.data(), sel.size(),
                          a.get("output", "").c_str(), index ? 1 : 0));
    return 0;
  }
  Timer tm("SAM (format on the GPU + write)");
  H.check(pbw_sam_write(H.h, &so, n_src, src, sel.empty() ? &none : sel.data(), sel.size(),
                        a.get("output", "-").c_str()));
  return 0;
}

// build-genome (main.rs:33-41, 118-123): FASTA files -> PREFIX.stidx.
int run_build_genome(int argc, char** argv) {
  const Args a = parse(argc, argv, GENOME_FLAGS, 3, false, true);
  require(a, {"species", "assembly", "G"});
  printf("Building genome index for %s %s...\n", a.get("species", "").c_str(), a.get("assembly", "").c_str());
  fflush(stdout);
  std::vector<const char*> files;
  for (const std::string& f : a.files) files.push_back(f.c_str());
  if (pbw_build_genome(a.get("G", "").c_str(), a.get("species", "").c_str(), a.get("assembly", "").c_str(),
                       (uint32_t)files.size(), files.data()) != PBW_OK)
    throw Fail(pbw_last_error(nullptr));
  printf("Done. Index written to %s.stidx\n", a.get("G", "").c_str());
  return 0;
}

// build-hash (main.rs:43-49, 124-128): PREFIX.stidx -> OUT.sthash, built on
// the GPU with the reference's k 15, stride 5, 300 occurrences per hash.
int run_build_hash(int argc, char** argv) {
  const Args a = parse(argc, argv, HASH_FLAGS, 2, false, false);
  require(a, {"genome", "H"});
  printf("Building 15-mer hash table...\n");
  fflush(stdout);
  if (pbw_build_hash(a.get("genome", "").c_str(), a.get("H", "").c_str(), 15, 5, 300, 0) != PBW_OK)
    throw Fail(pbw_last_error(nullptr));
  printf("Done. Hash table written to %s.sthash\n", a.get("H", "").c_str());
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    if (argc < 2) throw Usage("a subcommand is required (map, build-genome, build-hash)");
    const std::string cmd = argv[1];
    if (cmd == "map") return run_map(argc, argv);
    if (cmd == "build-genome") return run_build_genome(argc, argv);
    if (cmd == "build-hash") return run_build_hash(argc, argv);
    throw Usage("unrecognized subcommand '" + cmd + "'");
  } catch (const Usage& e) {
    fprintf(stderr, "error: %s\n", e.what());
    return 2;
  } catch (const std::exception& e) {
    fprintf(stderr, "Error: %s\n", e.what());
    return 1;
  }
}
