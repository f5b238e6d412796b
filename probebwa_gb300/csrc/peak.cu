// peak.cu -- measured integer throughput of the GPU, the denominator of the
// banded DP's roofline (the DP is a max-plus recurrence on 32-bit integers:
// adds and maxes on the integer pipes, no memory traffic to speak of).
//
// Every thread runs NCH chains of add.s32 (or max.s32) written as inline
// PTX; chain c takes chain c+1's value as its second operand (x[c] op=
// x[c+1]), which leaves four independent operations per step and no closed
// form for a compiler to fold. Blocks fill every SM several times over, and
// the kernel is timed with CUDA events after a warm-up launch.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/probebwa_gpu.h"

namespace {

constexpr int NCH = 8;       // independent chains per thread
constexpr int UNROLL = 16;   // operations per chain per loop iteration

template <bool MAX>
__global__ void k_int_chains(int iters, int seed, int* out) {
  int x[NCH];
#pragma unroll
  for (int c = 0; c < NCH; c++) x[c] = (int)(blockIdx.x * blockDim.x + threadIdx.x) * (c + 1) + seed;
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int u = 0; u < UNROLL; u++) {
#pragma unroll
      for (int c = 0; c < NCH; c++) {
        if (MAX) {
          asm volatile("max.s32 %0, %0, %1;" : "+r"(x[c]) : "r"(x[(c + 1) % NCH]));
        } else {
          asm volatile("add.s32 %0, %0, %1;" : "+r"(x[c]) : "r"(x[(c + 1) % NCH]));
        }
      }
    }
  }
  int acc = 0;
#pragma unroll
  for (int c = 0; c < NCH; c++) acc ^= x[c];
  if (acc == 0x7fffffff) out[0] = acc;  // keeps the chains alive
}

template <bool MAX>
double run(int device, int* out) {
  cudaDeviceProp pr;
  if (cudaGetDeviceProperties(&pr, device) != cudaSuccess) return -1.0;
  const int threads = 256;
  const int blocks = pr.multiProcessorCount * 8;
  const int iters = 4096;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_int_chains<MAX><<<blocks, threads>>>(64, 1, out);
  cudaEventRecord(a);
  k_int_chains<MAX><<<blocks, threads>>>(iters, 7, out);
  cudaEventRecord(b);
  cudaEventSynchronize(b);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (cudaGetLastError() != cudaSuccess || ms <= 0.f) return -1.0;
  const double ops = (double)blocks * threads * iters * UNROLL * NCH;
  return ops / (ms * 1e-3) / 1e9;
}

}  // namespace

extern "C" int pbw_int32_peak(int32_t device, double* add_gops, double* max_gops) {
  if (!add_gops || !max_gops) return PBW_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return PBW_ERR_CUDA;
  int* out = nullptr;
  if (cudaMalloc((void**)&out, sizeof(int)) != cudaSuccess) return PBW_ERR_NOMEM;
  *add_gops = run<false>(device, out);
  *max_gops = run<true>(device, out);
  cudaFree(out);
  return (*add_gops > 0 && *max_gops > 0) ? PBW_OK : PBW_ERR_CUDA;
}
