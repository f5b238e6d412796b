// align_band.cu -- K3b: the seeded DP (band <= 31, i.e. the max_indel_len
// band of SingleEndMapper, src/mapper/single.rs:59) as an anti-diagonal
// wavefront in band coordinates.
//
// Cell (i, c) of the band (c = j - (i + hint - band), 0 <= c <= 2*band)
// depends on (i-1, c) [diagonal], (i-1, c+1) [up] and (i, c-1) [left], so all
// cells with the same d = 2i + c are independent. Lane k owns columns 2k and
// 2k+1: at step d it computes column 2k + (d & 1) of row (d - (d & 1))/2 - k.
// Even steps take the left value from lane k-1 (its odd column, one step
// earlier) and odd steps take the up value from lane k+1 (its even column,
// one step earlier): two shuffles per step, and every lane computes one cell
// per step -- 2*m + 2*band + 2 steps per alignment. The traceback of a row is
// one byte per lane (both columns' nibbles), 32 bytes per row in shared
// memory. Integer semantics are those of the window kernel (align_window.cu).
#include "align_finish.cuh"
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

static __host__ __device__ inline size_t b16(size_t x) { return (x + 15) & ~(size_t)15; }

// per warp: query symbols, qualities, mismatch penalty per row; reference
// symbols and gap open per column; traceback rows; traceback ops
__host__ __device__ inline size_t band_smem_bytes(int lmax, int nmax) {
  return 2 * b16(lmax) + b16(4 * (size_t)lmax) + b16(nmax) + b16(4 * (size_t)nmax) + b16(32 * ((size_t)lmax + 1)) +
         b16((size_t)lmax + nmax + 2);
}
size_t band_smem_per_warp(int lmax, int nmax) { return band_smem_bytes(lmax, nmax); }

__device__ __forceinline__ uint8_t up_ascii_b(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }
__device__ __forceinline__ uint8_t comp_ascii_b(uint8_t b) {
  switch (b) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'C': return 'G';
    case 'G': return 'C';
    default: return 'N';
  }
}

__global__ void __launch_bounds__(128) k_align_band(AlignArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  unsigned char* my = smem_raw + band_smem_bytes(p.lmax, p.nmax) * wib;
  uint8_t* qs = my;
  uint8_t* qq = qs + b16(p.lmax);
  int32_t* qmm = (int32_t*)(qq + b16(p.lmax));
  uint8_t* rs = (uint8_t*)qmm + b16(4 * (size_t)p.lmax);
  int32_t* go = (int32_t*)(rs + b16(p.nmax));
  uint8_t* tb = (uint8_t*)go + b16(4 * (size_t)p.nmax);
  uint8_t* ops = tb + b16(32 * ((size_t)p.lmax + 1));
  const unsigned int njobs = *p.n_jobs;
  unsigned long long cells_acc = 0, jobs_acc = 0;

  while (true) {
    unsigned int jid = 0;
    if (lane == 0) jid = atomicAdd(p.next_job, 1u);
    jid = __shfl_sync(0xffffffffu, jid, 0);
    if (jid >= njobs) break;
    const AlnJob J = p.jobs[jid];
    AlnOut* O = p.out + J.slot;
    if (!J.valid) continue;
    jobs_acc++;
    const uint8_t* qbases = J.mate ? p.bases2 : p.bases;
    const uint8_t* qquals = J.mate ? p.quals2 : p.quals;
    const uint64_t* qoffs = J.mate ? p.offs2 : p.offs;
    const uint64_t qo = qoffs[J.read];
    const int m = (int)(qoffs[J.read + 1] - qo);
    const int n = (int)(J.ref_end - J.ref_start);
    for (int i = lane; i < m; i += 32) {
      uint8_t s, q;
      if (p.ref_bytes) {
        s = qbases[qo + i];
        q = qquals[qo + i];
      } else if (!J.rev) {
        s = up_ascii_b(qbases[qo + i]);
        q = qquals[qo + i];
      } else {
        s = comp_ascii_b(up_ascii_b(qbases[qo + m - 1 - i]));
        q = qquals[qo + m - 1 - i];
      }
      qs[i] = s;
      qq[i] = q;
      qmm[i] = __ldg(&p.tab->mmpen[q]);
    }
    if (p.ref_bytes) {
      for (int j = lane; j < n; j += 32) rs[j] = p.ref_bytes[J.ref_start + j];
    } else {
      const uint64_t gb = __ldg(&p.G.cbase[J.contig]) + J.ref_start;
      for (int j = lane; j < n; j += 32) rs[j] = (uint8_t)"ACGTN"[gcode(p.G, gb + j)];
    }
    __syncwarp();
    if (m == 0 || n == 0) {
      if (lane == 0) finish_empty(m, J.ref_start, O);
      continue;
    }
    // gap open per column (smith_waterman.rs:288-291, 348-363)
    {
      int carry = 0;
      for (int c0 = 0; c0 < n; c0 += 32) {
        const int j = c0 + lane;
        int v = (j < n && (j == 0 || rs[j] != rs[j - 1])) ? j : -1;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, v, d);
          if (lane >= d) v = max(v, y);
        }
        v = max(v, carry);
        if (j < n) go[j] = v;
        carry = __shfl_sync(0xffffffffu, v, 31);
      }
      __syncwarp();
      int carry_e = n - 1;
      for (int c0 = ((n - 1) >> 5) << 5; c0 >= 0; c0 -= 32) {
        const int j = c0 + lane;
        int v = (j < n && (j == n - 1 || rs[j + 1] != rs[j])) ? j : INT32_MAX;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          int y = __shfl_down_sync(0xffffffffu, v, d);
          if (lane + d < 32) v = min(v, y);
        }
        v = min(v, carry_e);
        if (j < n) {
          int run = v - go[j] + 1;
          if (run > 65535) run = 65535;
          long long g = (long long)J.gap_open + (run - 1);
          go[j] = g > -1 ? -1 : (int32_t)g;
        }
        carry_e = __shfl_sync(0xffffffffu, v, 0);
      }
      __syncwarp();
    }
    const int32_t ge = J.gap_extend;
    const int B = (int)J.band;
    const long long hint = J.hint;
    long long r0l = 1 - hint - (long long)B;
    const int R0 = r0l > 1 ? (int)min(r0l, (long long)m + 1) : 1;
    long long r1l = (long long)n + B - hint;
    const int R1 = r1l < (long long)m ? (int)max(r1l, 0ll) : m;
    const int c_even = 2 * lane, c_odd = 2 * lane + 1;
    const bool ev_ok = c_even <= 2 * B, od_ok = c_odd <= 2 * B;
    // j of column c in row i
    auto jof = [&](int i, int c) -> long long { return (long long)i + hint - B + c; };
    // initial row values (the row before R0): M = 0 where 0 <= j <= n
    auto init_m = [&](int c) -> int32_t {
      const long long j = jof(R0 - 1, c);
      return (j >= 0 && j <= n) ? 0 : NEG;
    };
    // last even / odd column outputs; they start as the initial row, which
    // has M = 0 at every j of the window -- also just beyond the band, where
    // the first processed row's last column looks up
    int32_t EM = init_m(c_even), EI = NEG, ED = NEG;
    int32_t OM = init_m(c_odd), OI = NEG, OD = NEG;
    unsigned long long bestKey = 0;
    unsigned long long cells = 0;
    uint32_t tbyte = 0;
    if (R1 >= R0) {
      // step d covers cells with 2i + c = d; lane k first touches row R0 at d = 2*R0 + 2k
      const int d0 = 2 * R0, d1 = 2 * R1 + 2 * B;
      for (int d = d0; d <= d1 + 1; d++) {
        const int par = d & 1;
        const int c = 2 * lane + par;
        const int i = ((d - par) >> 1) - lane;
        const bool col_ok = par ? od_ok : ev_ok;
        const long long j = jof(i, c);
        const bool on = col_ok && i >= R0 && i <= R1 && j >= 1 && j <= n;
        // neighbour values from the previous step (warp-uniform parity)
        int32_t dM, dI, dD, uM, uI, lM, lD;
        if (!par) {
          const int32_t sM = __shfl_up_sync(0xffffffffu, OM, 1);  // lane k-1 odd column (i, 2k-1)
          const int32_t sD = __shfl_up_sync(0xffffffffu, OD, 1);
          dM = EM; dI = EI; dD = ED;                 // (i-1, 2k)
          uM = OM; uI = OI;                          // (i-1, 2k+1)
          lM = lane ? sM : NEG; lD = lane ? sD : NEG;
        } else {
          const int32_t sM = __shfl_down_sync(0xffffffffu, EM, 1);  // lane k+1 even column (i-1, 2k+2)
          const int32_t sI = __shfl_down_sync(0xffffffffu, EI, 1);
          dM = OM; dI = OI; dD = OD;                 // (i-1, 2k+1)
          uM = lane < 31 ? sM : NEG; uI = lane < 31 ? sI : NEG;
          lM = EM; lD = ED;                          // (i, 2k)
        }
        int32_t oM = NEG, oI = NEG, oD = NEG;
        if (!on && i == R0 - 1) oM = init_m(c);  // the initial row, as the lane passes it
        if (on) {
          const int jj = (int)j;
          const int32_t sc = qs[i - 1] == rs[jj - 1] ? 20 : qmm[i - 1];
          const int32_t g = go[jj - 1];
          const int32_t fm = dM + sc, fi = dI + sc, fd = dD + sc;
          const int32_t Mv = max(max(fm, fi), fd);
          const uint32_t tm = Mv == fm ? 0u : (Mv == fi ? 1u : 2u);
          const int32_t io = uM + g, ie = uI + ge;
          const int32_t Iv = max(io, ie);
          const uint32_t ti = Iv == io ? 0u : 1u;
          const int32_t dop = lM + g, dex = lD + ge;
          const int32_t Dv = max(dop, dex);
          const uint32_t td = Dv == dop ? 0u : 1u;
          oM = Mv;
          oI = Iv;
          oD = Dv;
          tbyte |= (tm | (ti << 2) | (td << 3)) << (par * 4);
          cells++;
          if (i == R1) {
            const unsigned long long kM = ((unsigned long long)((long long)Mv + 2147483648LL) << 32) |
                                          ((unsigned long long)jj << 1);
            const unsigned long long kI = ((unsigned long long)((long long)Iv + 2147483648LL) << 32) |
                                          ((unsigned long long)jj << 1) | 1ull;
            bestKey = max(bestKey, max(kM, kI));
          }
        }
        if (par) {
          if (i >= R0 && i <= R1 && (ev_ok || od_ok)) tb[(size_t)(i - R0) * 32 + lane] = (uint8_t)tbyte;
          tbyte = 0;
          OM = oM;
          OI = oI;
          OD = oD;
        } else {
          EM = oM;
          EI = oI;
          ED = oD;
        }
      }
    }
    cells_acc += cells;
    for (int s = 16; s >= 1; s >>= 1) bestKey = max(bestKey, __shfl_xor_sync(0xffffffffu, bestKey, s));
    __syncwarp();
    int endV, endJ, endS;
    if (R1 < R0) {
      endV = 0;
      endJ = n;
      endS = 0;
    } else {
      if (bestKey == 0) {
        endV = NEG;
        endJ = -1;
        endS = 0;
      } else {
        endV = (int)((long long)(bestKey >> 32) - 2147483648LL);
        endJ = (int)((bestKey >> 1) & 0x7FFFFFFFull);
        endS = (int)(bestKey & 1ull);
      }
      long long fjs = (long long)R1 + hint - B, fje = (long long)R1 + hint + B;
      if (fjs < 1) fjs = 1;
      if (fje > n) fje = n;
      if (fje < 0) fje = 0;
      resolve_endpoint(endV, endJ, endS, (int)fjs, (int)fje, n);
    }
    if (lane == 0) {
      auto tbr = [&](int i, int jj) -> uint32_t {
        if (i < R0 || i > R1 || jj < 1 || jj > n) return 0u;
        const long long c = (long long)jj - ((long long)i + hint - B);
        if (c < 0 || c > 2 * B) return 0u;
        return (uint32_t)(tb[(size_t)(i - R0) * 32 + (c >> 1)] >> ((c & 1) * 4)) & 15u;
      };
      auto rsym = [&](int jj) -> uint8_t { return rs[jj]; };
      finish_alignment(m, endV, endJ, endS, qs, qq, ops, tbr, rsym, J.ref_start, p.tab, O, p.cig_pool,
                       p.cig_pool_used, p.cig_pool_cap, p.err);
    }
    __syncwarp();
  }
  for (int s = 16; s >= 1; s >>= 1) {
    cells_acc += __shfl_down_sync(0xffffffffu, cells_acc, s);
    jobs_acc += __shfl_down_sync(0xffffffffu, jobs_acc, s);
  }
  if (lane == 0 && p.counters) {
    atomicAdd(&p.counters[0], jobs_acc / 32);
    atomicAdd(&p.counters[1], cells_acc);
  }
}

void launch_align_band(const AlignArgs& a, int grid, cudaStream_t st) {
  const int threads = 128;
  size_t sm = band_smem_bytes(a.lmax, a.nmax) * (threads / 32);
  cudaFuncSetAttribute(k_align_band, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_align_band<<<grid, threads, sm, st>>>(a);
}

}  // namespace pbw
