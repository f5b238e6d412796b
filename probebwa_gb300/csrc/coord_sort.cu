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
// unmapped key above every mapped one, and sorted by the stable LSD radix
// sort of radix_sort.cu, as many 8-bit passes as the largest key needs.
#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/probebwa_gpu.h"
#include "pbw_host.h"
#include "pbw_pipeline.h"

namespace pbw {

namespace {

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
  const uint64_t nh = radix_hist_entries(n_sel);
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
  {
    unsigned long long* kb[2] = {k0, k1};
    unsigned long long* vb[2] = {v0, v1};
    const int which = radix_sort_pairs(kb, vb, n_sel, 0, passes, hist, sums, st);
    RCK(cudaGetLastError());
    RCK(cudaMemcpyAsync(sorted, vb[which], n_sel * 8, cudaMemcpyDeviceToHost, st));
  }
  RCK(cudaStreamSynchronize(st));
done:
  cudaStreamSynchronize(st);
  for (void* q : mem) cudaFree(q);
  return rc;
}
