// coord_sort.cu -- coordinate order of records for `--index` output
// (sort_for_coordinate_order, src/io/sam.rs:114-124), as a stable device
// radix sort.
//
// The reference sorts records by (index of the contig's name among the
// genome's contigs, position), unmapped records (position 0) last, with a
// stable sort: equal keys keep their input order. Contig indices come from a
// name -> index map built in contig order, so a name that occurs twice maps
// to its last index; a record whose contig has no name in the map sorts after
// every named contig and before the unmapped ones.
//
// Keys are packed into one integer, rank * (max_pos + 1) + pos, with the
// unmapped key above every mapped one, and sorted least-significant digit
// first, 8 bits per pass, as many passes as the largest key needs. Each pass:
// per-tile digit histograms (tiles of 4096 keys), an exclusive scan of the
// digit-major histogram table, and a scatter in which every tile ranks its
// keys in input order (warp match on the digit, then per-digit prefixes over
// the warps of the block), which keeps the sort stable.
#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_host.h"
#include "pbw_pipeline.h"

namespace pbw {

namespace {

constexpr int RS_T = 256, RS_ROUNDS = 16, RS_TILE = RS_T * RS_ROUNDS, RS_WARPS = RS_T / 32;

struct KeyArgs {
  const int32_t* contig[2];
  const unsigned long long* pos[2];
  uint32_t n_src;
  const unsigned long long* sel;
  uint64_t n;
  const uint32_t* rank;  // contig id -> rank among the names
  uint32_t n_contigs;
  unsigned long long span;      // max_pos + 1
  unsigned long long unmapped;  // key of an unmapped record
  unsigned long long* key;
  unsigned long long* val;
};

__global__ void k_coord_keys(KeyArgs a) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const unsigned long long g = a.sel[i];
  const uint32_t s = (uint32_t)(g % a.n_src);
  const uint64_t r = g / a.n_src;
  const unsigned long long p = (s ? a.pos[1] : a.pos[0])[r];
  const int32_t c = (s ? a.contig[1] : a.contig[0])[r];
  const unsigned long long rk = (c >= 0 && (uint32_t)c < a.n_contigs) ? a.rank[c] : a.n_contigs;
  a.key[i] = p == 0 ? a.unmapped : rk * a.span + p;
  a.val[i] = g;
}

__global__ void __launch_bounds__(RS_T) k_radix_hist(const unsigned long long* key, uint64_t n, int shift,
                                                     unsigned int* hist, uint32_t nb) {
  __shared__ unsigned int cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint64_t base = (uint64_t)blockIdx.x * RS_TILE;
  for (int j = 0; j < RS_ROUNDS; j++) {
    const uint64_t i = base + (uint64_t)j * RS_T + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(unsigned)(key[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(uint64_t)threadIdx.x * nb + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_T) k_radix_scatter(const unsigned long long* key, const unsigned long long* val,
                                                        uint64_t n, int shift, const unsigned int* start, uint32_t nb,
                                                        unsigned long long* key_out, unsigned long long* val_out) {
  __shared__ unsigned int base[256];
  __shared__ unsigned int wcnt[RS_WARPS][257];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  base[threadIdx.x] = start[(uint64_t)threadIdx.x * nb + blockIdx.x];
  const uint64_t tile = (uint64_t)blockIdx.x * RS_TILE;
  const unsigned int lt = (1u << lane) - 1u;
  for (int j = 0; j < RS_ROUNDS; j++) {
    for (int k = threadIdx.x; k < RS_WARPS * 257; k += RS_T) (&wcnt[0][0])[k] = 0;
    __syncthreads();
    const uint64_t i = tile + (uint64_t)j * RS_T + threadIdx.x;
    const bool ok = i < n;
    const unsigned long long kk = ok ? key[i] : 0ull;
    const unsigned int d = ok ? (unsigned)(kk >> shift) & 255u : 256u;
    const unsigned int peers = __match_any_sync(0xffffffffu, d);
    const unsigned int rank = __popc(peers & lt);
    if (rank == 0) wcnt[w][d] = __popc(peers);
    __syncthreads();
    {
      // per digit: exclusive prefix over the warps, on top of the running base
      const unsigned int dd = threadIdx.x;
      unsigned int run = base[dd];
      for (int q = 0; q < RS_WARPS; q++) {
        const unsigned int t = wcnt[q][dd];
        wcnt[q][dd] = run;
        run += t;
      }
      base[dd] = run;
    }
    __syncthreads();
    if (ok) {
      const unsigned int p = wcnt[w][d] + rank;
      key_out[p] = kk;
      val_out[p] = val[i];
    }
    __syncthreads();
  }
}

#define RCK(call)                                                  \
  do {                                                             \
    cudaError_t e_ = (call);                                       \
    if (e_ != cudaSuccess) {                                       \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_); \
      rc = PBW_ERR_CUDA;                                           \
      goto done;                                                   \
    }                                                              \
  } while (0)

}  // namespace

}  // namespace pbw

extern "C" int pbw_sort_coordinate(pbw_handle* h, uint32_t n_src, const pbw_sam_source* src, const uint64_t* sel,
                                   uint64_t n_sel, uint64_t* sorted) {
  using namespace pbw;
  if (!h) return PBW_ERR_ARG;
  if (!src || n_src < 1 || n_src > 2 || !sorted || (n_sel && !sel) || n_sel >= (1ull << 32)) {
    h->err = "pbw_sort_coordinate: bad arguments";
    return PBW_ERR_ARG;
  }
  for (uint32_t s = 0; s < n_src; s++)
    if (!src[s].recs) {
      h->err = "pbw_sort_coordinate: source without records";
      return PBW_ERR_ARG;
    }
  // contig id -> rank of its name (the last contig carrying that name)
  const uint32_t nc = (uint32_t)h->names.size();
  std::unordered_map<std::string, uint32_t> last;
  for (uint32_t c = 0; c < nc; c++) last[h->names[c]] = c;
  std::vector<uint32_t> rank(nc);
  for (uint32_t c = 0; c < nc; c++) rank[c] = last[h->names[c]];
  unsigned long long max_pos = 0;
  for (uint64_t i = 0; i < n_sel; i++) {
    const uint32_t s = (uint32_t)(sel[i] % n_src);
    const uint64_t r = sel[i] / n_src;
    if (r >= src[s].recs->n) {
      h->err = "pbw_sort_coordinate: selection entry " + std::to_string(i) + " names no record";
      return PBW_ERR_ARG;
    }
    max_pos = std::max<unsigned long long>(max_pos, src[s].recs->pos[r]);
  }
  if (n_sel == 0) return PBW_OK;
  if (max_pos >= (1ull << 40) || nc >= (1u << 23)) {
    h->err = "pbw_sort_coordinate: position or contig count beyond the packed record layout";
    return PBW_ERR_LIMIT;
  }
  const unsigned long long span = max_pos + 1;
  const unsigned long long unmapped = ((unsigned long long)nc + 1) * span;
  int bits = 0;
  while (bits < 64 && (unmapped >> bits) != 0) bits++;
  const int passes = (bits + 7) / 8;
  const uint32_t nb = (uint32_t)((n_sel + RS_TILE - 1) / RS_TILE);
  const uint64_t nh = (uint64_t)nb * 256;
  cudaStream_t st = h->st;
  int rc = PBW_OK;
  std::vector<void*> mem;
  auto alloc = [&](void** p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 1));
    if (e == cudaSuccess) mem.push_back(*p);
    return e;
  };
  unsigned long long *d_sel = nullptr, *k0 = nullptr, *k1 = nullptr, *v0 = nullptr, *v1 = nullptr;
  unsigned long long *d_pos[2] = {nullptr, nullptr};
  int32_t* d_contig[2] = {nullptr, nullptr};
  uint32_t* d_rank = nullptr;
  unsigned int *hist = nullptr, *sums = nullptr;
  KeyArgs ka{};
  RCK(alloc((void**)&d_sel, n_sel * 8));
  RCK(alloc((void**)&k0, n_sel * 8));
  RCK(alloc((void**)&k1, n_sel * 8));
  RCK(alloc((void**)&v0, n_sel * 8));
  RCK(alloc((void**)&v1, n_sel * 8));
  RCK(alloc((void**)&d_rank, (size_t)nc * 4));
  RCK(alloc((void**)&hist, nh * 4));
  RCK(alloc((void**)&sums, (scan_blocks(nh) + 2) * 4));
  for (uint32_t s = 0; s < n_src; s++) {
    const uint64_t n = src[s].recs->n;
    RCK(alloc((void**)&d_pos[s], n * 8));
    RCK(alloc((void**)&d_contig[s], n * 4));
    RCK(cudaMemcpyAsync(d_pos[s], src[s].recs->pos, n * 8, cudaMemcpyHostToDevice, st));
    RCK(cudaMemcpyAsync(d_contig[s], src[s].recs->contig, n * 4, cudaMemcpyHostToDevice, st));
    ka.pos[s] = d_pos[s];
    ka.contig[s] = d_contig[s];
  }
  RCK(cudaMemcpyAsync(d_sel, sel, n_sel * 8, cudaMemcpyHostToDevice, st));
  if (nc) RCK(cudaMemcpyAsync(d_rank, rank.data(), (size_t)nc * 4, cudaMemcpyHostToDevice, st));
  ka.n_src = n_src;
  ka.sel = d_sel;
  ka.n = n_sel;
  ka.rank = d_rank;
  ka.n_contigs = nc;
  ka.span = span;
  ka.unmapped = unmapped;
  ka.key = k0;
  ka.val = v0;
  k_coord_keys<<<(unsigned)((n_sel + 255) / 256), 256, 0, st>>>(ka);
  for (int p = 0; p < passes; p++) {
    const int shift = 8 * p;
    k_radix_hist<<<nb, RS_T, 0, st>>>(k0, n_sel, shift, hist, nb);
    launch_scan_excl(hist, nh, nullptr, sums, nullptr, nullptr, st);
    k_radix_scatter<<<nb, RS_T, 0, st>>>(k0, v0, n_sel, shift, hist, nb, k1, v1);
    std::swap(k0, k1);
    std::swap(v0, v1);
  }
  RCK(cudaGetLastError());
  RCK(cudaMemcpyAsync(sorted, v0, n_sel * 8, cudaMemcpyDeviceToHost, st));
  RCK(cudaStreamSynchronize(st));
done:
  cudaStreamSynchronize(st);
  for (void* q : mem) cudaFree(q);
  return rc;
}
