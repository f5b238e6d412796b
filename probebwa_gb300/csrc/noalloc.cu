// noalloc.cu -- window alignment for callers that cannot allocate device memory.
//
// pbw_align_noalloc runs the window DP of align_window.cu with every piece of
// scratch -- jobs, per-alignment outputs, queue counters, the CIGAR overflow
// pool, the per-block slabs for windows too large for shared memory and the
// parameter table -- inside one file-scope device array. Inputs and outputs
// are device memory owned by the caller. It is for callers that must not call
// cudaMalloc: a host application whose own allocator has reserved the GPU's
// memory (a framework's caching allocator, a memory pool sized at start-up),
// or a loop with a fixed device-memory budget that may not grow at run time.
// It calls no cudaMalloc, cudaFree or allocating library routine, and it
// synchronises the caller's stream before returning.
#include <algorithm>
#include <cstring>
#include <string>

#include "../../include/probebwa_gpu.h"
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

// Limits of the allocation-free path.
constexpr uint64_t NA_MAX_PROBLEMS = 4096;
constexpr int NA_MAX_READ = 256;
constexpr int NA_MAX_REF = 2048;
constexpr int NA_BLOCKS = 16;                 // window kernel blocks (8 warps each)
// CIGARs longer than CIG_INLINE operations spill into the pool. Runs of M
// and I consume at least one read base each and runs of D sit between them,
// so a read of m bases has at most 2m + 1 operations: the pool holds that
// for every problem of a full call.
constexpr uint64_t NA_POOL_OPS = NA_MAX_PROBLEMS * (2 * NA_MAX_READ + 1);

constexpr size_t na16(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t NA_SLAB = window_slab_bytes(NA_MAX_READ, NA_MAX_REF);
constexpr size_t NA_OFF_TAB = 0;
constexpr size_t NA_OFF_CNT = na16(NA_OFF_TAB + sizeof(DevTables));
constexpr size_t NA_OFF_JOBS = na16(NA_OFF_CNT + 64);
constexpr size_t NA_OFF_OUT = na16(NA_OFF_JOBS + NA_MAX_PROBLEMS * sizeof(AlnJob));
constexpr size_t NA_OFF_POOL = na16(NA_OFF_OUT + NA_MAX_PROBLEMS * sizeof(AlnOut));
constexpr size_t NA_OFF_SLAB = na16(NA_OFF_POOL + NA_POOL_OPS * 4);
constexpr size_t NA_BYTES = na16(NA_OFF_SLAB + NA_SLAB * NA_BLOCKS);  // about 14 MB

// The scratch. Every GPU that loads this library holds it until the process
// exits. In host code the name is only a handle for cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

// counters inside the scratch: 0 n_jobs, 1 next_job, 2 cig_pool_used, 3 error
__global__ void k_noalloc_jobs(uint64_t n, const uint64_t* read_off, const uint64_t* ref_off, const int64_t* hint,
                               const uint64_t* band, int32_t go, int32_t ge, unsigned char* base) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int* cnt = (unsigned int*)(base + NA_OFF_CNT);
  if (i == 0) cnt[0] = (unsigned int)n;
  if (i >= n) return;
  AlnJob* jobs = (AlnJob*)(base + NA_OFF_JOBS);
  AlnOut* outs = (AlnOut*)(base + NA_OFF_OUT);
  const uint64_t m = read_off[i + 1] - read_off[i];
  const uint64_t w = ref_off[i + 1] - ref_off[i];
  AlnJob J;
  J.ref_start = ref_off[i];
  J.ref_end = ref_off[i + 1];
  J.hint = hint[i];
  J.read = (uint32_t)i;
  J.slot = (uint32_t)i;
  J.contig = 0;
  J.band = (uint32_t)min(band[i], (uint64_t)(1u << 30));
  J.rev = 0;
  J.valid = 1;
  J.mate = 0;
  J.pad = 0;
  J.pad2 = 0;
  J.gap_open = go;
  J.gap_extend = ge;
  if (m > (uint64_t)NA_MAX_READ || w > (uint64_t)NA_MAX_REF) {
    J.valid = 0;
    atomicExch((int*)&cnt[3], 6);
  }
  outs[i].n_ops = 0;
  jobs[i] = J;
}

__global__ void k_noalloc_out(uint64_t n, const uint64_t* ref_off, const unsigned char* base, int32_t* score,
                              uint64_t* offset, uint32_t* n_ops, uint32_t* cigar, uint32_t stride) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const AlnOut& A = ((const AlnOut*)(base + NA_OFF_OUT))[i];
  const uint32_t* pool = (const uint32_t*)(base + NA_OFF_POOL);
  unsigned int* cnt = (unsigned int*)(base + NA_OFF_CNT);
  score[i] = A.score;
  offset[i] = A.pos - ref_off[i];
  n_ops[i] = A.n_ops;
  if (A.n_ops > stride) {
    atomicExch((int*)&cnt[3], 7);
    return;
  }
  const uint32_t* src = A.n_ops > CIG_INLINE ? pool + A.cig_pool : A.cig;
  for (uint32_t k = 0; k < A.n_ops; k++) cigar[i * (uint64_t)stride + k] = src[k];
}

}  // namespace pbw

using namespace pbw;

namespace {
// Per-device set-up state: the scratch's device address and whether its
// parameter table has been written.
constexpr int NA_MAX_DEVICES = 64;
unsigned char* g_scratch_ptr[NA_MAX_DEVICES] = {};
// error text, readable through pbw_last_error(NULL)
struct ErrSink {
  void operator=(const std::string& s) { pbw::set_handleless_error(s); }
} g_noalloc_err;
}  // namespace

extern "C" int pbw_align_noalloc(uint64_t n, const uint8_t* reads, const uint8_t* quals, const uint64_t* read_off,
                                 const uint8_t* refs, const uint64_t* ref_off, const int64_t* hint,
                                 const uint64_t* band, uint32_t gap_open_phred, uint32_t gap_extend_phred,
                                 int32_t* score, uint64_t* offset, uint32_t* n_ops, uint32_t* cigar,
                                 uint32_t cigar_stride, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (n > NA_MAX_PROBLEMS) {
    g_noalloc_err = "pbw_align_noalloc: " + std::to_string(n) + " problems, at most " +
                    std::to_string(NA_MAX_PROBLEMS) + " per call";
    return PBW_ERR_LIMIT;
  }
  if (cigar_stride == 0) {
    g_noalloc_err = "pbw_align_noalloc: cigar_stride must be > 0";
    return PBW_ERR_ARG;
  }
  if (n == 0) return PBW_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES) {
    g_noalloc_err = "pbw_align_noalloc: no usable current device";
    return PBW_ERR_CUDA;
  }
  // First call on this device: find the scratch's device address and write
  // its parameter table (mismatch penalties etc.) with a synchronous copy.
  // This first call should come before any stream capture.
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
      g_noalloc_err = std::string("pbw_align_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return PBW_ERR_CUDA;
    }
    pbw_options o;
    pbw_default_options(&o);
    DevTables T;
    fill_tables(o, 1, T);
    e = cudaMemcpy((unsigned char*)ptr + NA_OFF_TAB, &T, sizeof(T), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      g_noalloc_err = std::string("pbw_align_noalloc: table upload: ") + cudaGetErrorString(e);
      return PBW_ERR_CUDA;
    }
    g_scratch_ptr[dev] = (unsigned char*)ptr;
  }
  unsigned char* base = g_scratch_ptr[dev];
  int32_t go, ge;
  gap_costs(gap_open_phred, gap_extend_phred, go, ge);
  // the previous call's counters and error word must not leak into this one
  if (cudaMemsetAsync(base + NA_OFF_CNT, 0, 64, st) != cudaSuccess) {
    g_noalloc_err = "pbw_align_noalloc: counter reset failed";
    return PBW_ERR_CUDA;
  }
  k_noalloc_jobs<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, read_off, ref_off, hint, band, go, ge, base);
  AlignArgs aa{};
  aa.tab = (const DevTables*)(base + NA_OFF_TAB);
  aa.bases = reads;
  aa.quals = quals;
  aa.offs = read_off;
  aa.bases2 = reads;
  aa.quals2 = quals;
  aa.offs2 = read_off;
  aa.jobs = (const AlnJob*)(base + NA_OFF_JOBS);
  unsigned int* cnt = (unsigned int*)(base + NA_OFF_CNT);
  aa.n_jobs = cnt + 0;
  aa.next_job = cnt + 1;
  aa.out = (AlnOut*)(base + NA_OFF_OUT);
  aa.cig_pool = (uint32_t*)(base + NA_OFF_POOL);
  aa.cig_pool_used = cnt + 2;
  aa.cig_pool_cap = (uint32_t)NA_POOL_OPS;
  aa.ref_bytes = refs;
  aa.lmax = NA_MAX_READ;
  aa.nmax = NA_MAX_REF;
  aa.tb_smem = 0;
  aa.tb_global = base + NA_OFF_SLAB;
  aa.tb_global_per_warp = NA_SLAB;
  aa.counters = nullptr;
  aa.err = (int*)(cnt + 3);
  launch_align_window(aa, NA_BLOCKS, st);
  k_noalloc_out<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n, ref_off, base, score, offset, n_ops, cigar,
                                                              cigar_stride);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_noalloc_err = std::string("pbw_align_noalloc: launch: ") + cudaGetErrorString(e);
    return PBW_ERR_CUDA;
  }
  int err = 0;
  e = cudaMemcpyAsync(&err, base + NA_OFF_CNT + 12, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    g_noalloc_err = std::string("pbw_align_noalloc: ") + cudaGetErrorString(e);
    return PBW_ERR_CUDA;
  }
  if (err == 6) {
    g_noalloc_err = "pbw_align_noalloc: a read longer than 256 or a reference window longer than 2048";
    return PBW_ERR_LIMIT;
  }
  if (err == 7) {
    g_noalloc_err = "pbw_align_noalloc: a CIGAR has more operations than cigar_stride";
    return PBW_ERR_CAPACITY;
  }
  if (err == 3) {
    g_noalloc_err = "pbw_align_noalloc: the static CIGAR overflow pool (" + std::to_string(NA_POOL_OPS) +
                    " operations) is full";
    return PBW_ERR_CAPACITY;
  }
  if (err == 9) {
    g_noalloc_err = "pbw_align_noalloc: a wavefront wait of the window DP gave up; results discarded";
    return PBW_ERR_DEVICE;
  }
  if (err) {
    g_noalloc_err = "pbw_align_noalloc: device error " + std::to_string(err);
    return PBW_ERR_DEVICE;
  }
  return PBW_OK;
}
