// index_build.cu -- `build-hash` on the device: the k-mer occurrence table of
// a genome index (HashTableBuilder::build, src/index/hashtable.rs:248-322)
// written as a .sthash file (HashTable::save, hashtable.rs:81-87).
//
// The reference scans each contig's forward windows at multiples of the
// stride, then the windows of its reverse complement at multiples of the
// stride (stored at forward coordinate len - i - k, strand bit set), skips
// windows with a non-ACGT base, hashes each window (the first min(k, 15)
// bases as 2-bit codes, first base most significant, through the
// multiply-xor-shift mix, hashtable.rs:107-124), keeps the first max_count
// occurrences of each hash in that scan order, and stores the occurrences
// grouped by hash in ascending hash order, each group in scan order.
//
// Device steps, all over the genome already in HBM (2-bit words + N mask):
//  1. one thread per window, in scan order: N check, hash, packed position
//     (bit 63 strand, bits 62..40 contig, bits 39..0 position);
//  2. order-preserving compaction of the windows without N (scan of flags);
//  3. stable LSD radix sort by hash (4 passes of 8 bits) -- equal hashes keep
//     scan order, so the first max_count of each run are the ones the
//     reference's running count admits;
//  4. runs of equal hash: starts, counts capped at max_count, their exclusive
//     scan as the offsets of the groups in the positions array; the table
//     (hash, offset, count) and the positions come back to the host and are
//     written in bincode's layout, the map in ascending-hash order.
#include <algorithm>
#include <cstdio>
#include <memory>
#include <string>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_host.h"
#include "pbw_pipeline.h"

namespace pbw {
void set_handleless_error(const std::string& s);

namespace {

__device__ __forceinline__ uint32_t mix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x7feb352du;
  h ^= h >> 15;
  h *= 0x846ca68bu;
  h ^= h >> 16;
  return h;
}

struct WinArgs {
  const unsigned long long* bits;
  const unsigned int* nmask;
  const unsigned long long* cbase;
  const unsigned long long* clen;
  const unsigned long long* wbase;  // first window number of each contig (n_contigs + 1 entries)
  uint32_t n_contigs;
  uint64_t n_win;
  uint32_t k, stride;
  unsigned long long* key;
  unsigned long long* val;
  unsigned int* valid;
};

__global__ void __launch_bounds__(256) k_hash_windows(WinArgs a) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t w = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; w < a.n_win; w += step) {
    uint32_t lo = 0, hi = a.n_contigs;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (a.wbase[mid] <= w) lo = mid;
      else hi = mid;
    }
    const uint32_t c = lo;
    const uint64_t nwc = (a.wbase[c + 1] - a.wbase[c]) >> 1;
    const uint64_t j = w - a.wbase[c];
    const bool rc = j >= nwc;
    const uint64_t jj = rc ? j - nwc : j;
    const uint64_t L = a.clen[c];
    const uint64_t p = rc ? L - jj * a.stride - a.k : jj * a.stride;
    const uint64_t g0 = a.cbase[c] + p;
    const uint32_t s = (uint32_t)(g0 & 31);
    const uint64_t wi = g0 >> 5;
    const bool two = s + a.k > 32;
    // N mask of the window's k bases
    unsigned int m = a.nmask[wi] >> s;
    if (two) m |= a.nmask[wi + 1] << (32 - s);
    const unsigned int kmask = a.k >= 32 ? 0xFFFFFFFFu : ((1u << a.k) - 1u);
    const bool ok = (m & kmask) == 0;
    // 2-bit bases, base t of the window at bits 2t
    unsigned long long b = a.bits[wi] >> (2 * s);
    if (two) b |= a.bits[wi + 1] << (64 - 2 * s);
    const uint32_t nh = a.k < 15 ? a.k : 15;
    uint32_t code = 0;
    for (uint32_t t = 0; t < nh; t++) {
      const uint32_t base = rc ? 3u - (uint32_t)((b >> (2 * (a.k - 1 - t))) & 3ull) : (uint32_t)((b >> (2 * t)) & 3ull);
      code = (code << 2) | base;
    }
    a.key[w] = mix32(code);
    a.val[w] = ((unsigned long long)(rc ? 1u : 0u) << 63) | ((unsigned long long)c << 40) | p;
    a.valid[w] = ok ? 1u : 0u;
  }
}

__global__ void k_compact(const unsigned long long* key, const unsigned long long* val, const unsigned int* valid,
                          const unsigned int* dst, uint64_t n, unsigned long long* key_out,
                          unsigned long long* val_out) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    if (valid[i]) {
      key_out[dst[i]] = key[i];
      val_out[dst[i]] = val[i];
    }
  }
}

__global__ void k_heads(const unsigned long long* key, uint64_t n, unsigned int* head) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step)
    head[i] = (i == 0 || (uint32_t)key[i] != (uint32_t)key[i - 1]) ? 1u : 0u;
}

__global__ void k_run_starts(const unsigned int* head, const unsigned int* rid, uint64_t n, unsigned int* start) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step)
    if (head[i]) start[rid[i]] = (unsigned int)i;
}

__global__ void k_run_counts(const unsigned int* start, uint64_t n_runs, uint64_t n, uint32_t max_count,
                             unsigned int* cnt) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_runs; r += step) {
    const uint64_t e = r + 1 < n_runs ? start[r + 1] : n;
    const uint64_t len = e - start[r];
    cnt[r] = (unsigned int)(len < max_count ? len : max_count);
  }
}

// cnt holds the capped counts; off their exclusive scan.
__global__ void k_emit_table(const unsigned long long* key, const unsigned int* start, const unsigned int* cnt,
                             const unsigned int* off, uint64_t n_runs, unsigned int* tab) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_runs; r += step) {
    tab[3 * r] = (unsigned int)key[start[r]];
    tab[3 * r + 1] = off[r];
    tab[3 * r + 2] = cnt[r];
  }
}

__global__ void k_emit_positions(const unsigned long long* val, const unsigned int* head, const unsigned int* rid,
                                 const unsigned int* start, const unsigned int* off, uint64_t n, uint32_t max_count,
                                 unsigned long long* pos_out) {
  const uint64_t step = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += step) {
    const unsigned int r = rid[i] + head[i] - 1u;
    const uint64_t rank = i - start[r];
    if (rank < max_count) pos_out[off[r] + rank] = val[i];
  }
}

struct Mem {
  std::vector<void*> ptrs;
  ~Mem() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  bool alloc(T*& p, uint64_t n) {
    void* q = nullptr;
    if (cudaMalloc(&q, std::max<uint64_t>(n, 1) * sizeof(T)) != cudaSuccess) return false;
    ptrs.push_back(q);
    p = (T*)q;
    return true;
  }
};

bool write_sthash(const std::string& path, const std::vector<uint32_t>& tab, uint64_t n_runs,
                  const std::vector<unsigned long long>& pos, uint64_t k, uint64_t stride) {
  FILE* f = fopen(path.c_str(), "wb");
  if (!f) return false;
  std::vector<char> vbuf(1 << 22);
  setvbuf(f, vbuf.data(), _IOFBF, vbuf.size());
  bool ok = true;
  auto u64 = [&](uint64_t v) {
    uint8_t b[8];
    for (int i = 0; i < 8; i++) b[i] = (uint8_t)(v >> (8 * i));
    ok = ok && fwrite(b, 1, 8, f) == 8;
  };
  // little-endian hosts: the arrays' memory is their bincode encoding
  u64(n_runs);
  if (n_runs) ok = ok && fwrite(tab.data(), 4, 3 * n_runs, f) == 3 * n_runs;
  u64(pos.size());
  if (!pos.empty()) ok = ok && fwrite(pos.data(), 8, pos.size(), f) == pos.size();
  u64(k);
  u64(stride);
  u64(pos.size());
  ok = (fclose(f) == 0) && ok;
  return ok;
}

#define IB_CK(call)                                                            \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess) {                                                   \
      set_handleless_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
      return PBW_ERR_CUDA;                                                     \
    }                                                                          \
  } while (0)
#define IB_ALLOC(p, n)                                                         \
  do {                                                                         \
    if (!M.alloc(p, n)) {                                                      \
      set_handleless_error("cudaMalloc failed in build-hash");                 \
      return PBW_ERR_NOMEM;                                                    \
    }                                                                          \
  } while (0)

}  // namespace
}  // namespace pbw

extern "C" int pbw_build_hash(const char* genome_prefix, const char* out_prefix, uint64_t k, uint64_t stride,
                              uint64_t max_count, int32_t device) {
  using namespace pbw;
  if (!genome_prefix || !out_prefix) {
    set_handleless_error("pbw_build_hash: null argument");
    return PBW_ERR_ARG;
  }
  if (stride == 0 || k == 0) {
    set_handleless_error("pbw_build_hash: k and stride must be positive");
    return PBW_ERR_ARG;
  }
  if (k > 32) {
    set_handleless_error("pbw_build_hash: k above 32 is beyond the device window");
    return PBW_ERR_LIMIT;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    set_handleless_error("pbw_build_hash: no such CUDA device");
    return PBW_ERR_CUDA;
  }
  IB_CK(cudaSetDevice(device));
  std::unique_ptr<pbw_handle> h(new pbw_handle());
  h->device = device;
  IB_CK(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  int rc = load_genome(h.get(), genome_prefix);
  if (rc != PBW_OK) {
    set_handleless_error(h->err);
    return rc;
  }
  cudaStream_t st = h->st;
  const uint32_t nc = (uint32_t)h->lens.size();
  std::vector<unsigned long long> wbase(nc + 1, 0);
  for (uint32_t c = 0; c < nc; c++) {
    const uint64_t L = h->lens[c];
    const uint64_t nw = L >= k ? (L - k) / stride + 1 : 0;
    wbase[c + 1] = wbase[c] + 2 * nw;
  }
  const uint64_t n_win = wbase[nc];
  if (n_win >= (1ull << 32)) {
    set_handleless_error("pbw_build_hash: more than 2^32 windows");
    return PBW_ERR_LIMIT;
  }
  const std::string path = std::string(out_prefix) + ".sthash";
  std::vector<uint32_t> tab;
  std::vector<unsigned long long> pos;
  uint64_t n_runs = 0;
  if (n_win > 0 && max_count > 0) {
    Mem M;
    unsigned long long *kb[2], *vb[2], *d_wbase;
    unsigned int *flag, *idx, *start, *cnt, *off, *d_tab, *sums, *hist, *d_tot;
    unsigned long long* d_pos;
    IB_ALLOC(kb[0], n_win);
    IB_ALLOC(kb[1], n_win);
    IB_ALLOC(vb[0], n_win);
    IB_ALLOC(vb[1], n_win);
    IB_ALLOC(flag, n_win);
    IB_ALLOC(idx, n_win);
    IB_ALLOC(d_wbase, nc + 1);
    IB_ALLOC(d_tot, 4);
    const uint64_t nh = radix_hist_entries(n_win);
    IB_ALLOC(hist, nh);
    IB_ALLOC(sums, std::max(scan_blocks(nh), scan_blocks(n_win)) + 2);
    IB_CK(cudaMemcpyAsync(d_wbase, wbase.data(), (nc + 1) * 8, cudaMemcpyHostToDevice, st));
    int grid = 0;
    IB_CK(cudaDeviceGetAttribute(&grid, cudaDevAttrMultiProcessorCount, device));
    grid *= 8;
    WinArgs wa{h->G.bits, h->G.nmask, h->G.cbase, h->G.clen, d_wbase, nc, n_win, (uint32_t)k, (uint32_t)stride,
               kb[0], vb[0], flag};
    k_hash_windows<<<grid, 256, 0, st>>>(wa);
    // 2. keep the windows without N, in scan order
    launch_scan_excl(flag, n_win, idx, sums, d_tot, nullptr, st);
    k_compact<<<grid, 256, 0, st>>>(kb[0], vb[0], flag, idx, n_win, kb[1], vb[1]);
    unsigned int n_valid32 = 0;
    IB_CK(cudaMemcpyAsync(&n_valid32, d_tot, 4, cudaMemcpyDeviceToHost, st));
    IB_CK(cudaStreamSynchronize(st));
    const uint64_t n = n_valid32;
    if (n > 0) {
      // 3. stable sort by the 32-bit hash
      unsigned long long* k2[2] = {kb[1], kb[0]};
      unsigned long long* v2[2] = {vb[1], vb[0]};
      const int which = radix_sort_pairs(k2, v2, n, 0, 4, hist, sums, st);
      const unsigned long long* key = k2[which];
      const unsigned long long* val = v2[which];
      // 4. runs of equal hash
      k_heads<<<grid, 256, 0, st>>>(key, n, flag);
      launch_scan_excl(flag, n, idx, sums, d_tot, nullptr, st);
      unsigned int runs32 = 0;
      IB_CK(cudaMemcpyAsync(&runs32, d_tot, 4, cudaMemcpyDeviceToHost, st));
      IB_CK(cudaStreamSynchronize(st));
      n_runs = runs32;
      IB_ALLOC(start, n_runs);
      IB_ALLOC(cnt, n_runs);
      IB_ALLOC(off, n_runs);
      IB_ALLOC(d_tab, 3 * n_runs);
      k_run_starts<<<grid, 256, 0, st>>>(flag, idx, n, start);
      k_run_counts<<<grid, 256, 0, st>>>(start, n_runs, n, (uint32_t)std::min<uint64_t>(max_count, 0xFFFFFFFFu), cnt);
      launch_scan_excl(cnt, n_runs, off, sums, d_tot, nullptr, st);
      unsigned int kept32 = 0;
      IB_CK(cudaMemcpyAsync(&kept32, d_tot, 4, cudaMemcpyDeviceToHost, st));
      IB_CK(cudaStreamSynchronize(st));
      IB_ALLOC(d_pos, kept32);
      k_emit_table<<<grid, 256, 0, st>>>(key, start, cnt, off, n_runs, d_tab);
      k_emit_positions<<<grid, 256, 0, st>>>(val, flag, idx, start, off, n,
                                             (uint32_t)std::min<uint64_t>(max_count, 0xFFFFFFFFu), d_pos);
      IB_CK(cudaGetLastError());
      tab.resize(3 * n_runs);
      pos.resize(kept32);
      IB_CK(cudaMemcpyAsync(tab.data(), d_tab, 12 * n_runs, cudaMemcpyDeviceToHost, st));
      if (kept32) IB_CK(cudaMemcpyAsync(pos.data(), d_pos, 8ull * kept32, cudaMemcpyDeviceToHost, st));
      IB_CK(cudaStreamSynchronize(st));
    }
  }
  if (!write_sthash(path, tab, n_runs, pos, k, stride)) {
    set_handleless_error("cannot write " + path);
    return PBW_ERR_IO;
  }
  return PBW_OK;
}
