// align_band.cu -- K3b: the seeded DP (band <= 31, i.e. the max_indel_len
// band of SingleEndMapper, src/mapper/single.rs:59) of
// SmithWatermanAligner::align (src/align/smith_waterman.rs:113-255), several
// alignments per warp.
//
// Band coordinates: cell (i, c) is window column j = i + hint - band + c,
// 0 <= c <= 2*band. It depends on (i-1, c) [diagonal], (i-1, c+1) [up] and
// (i, c-1) [left]. An alignment gets G lanes (8 or 16; 32/G alignments per
// warp); lane k owns the C consecutive band columns c = k*C .. k*C + C - 1
// (G*C > 2*band + 1) and lags lane k-1 by
// one row: at step s it computes its C cells of row i = R0 + s - k from left
// to right. The left input of its first column is lane k-1's last column of
// the same row (computed one step earlier, __shfl_up_sync); the up input of
// its last column is lane k+1's first column one row up (computed earlier in
// the same step, __shfl_down_sync). Everything else stays in registers: the
// lane's previous row gives its diagonal and up inputs. An alignment takes
// m + G - 1 steps of C cells per lane.
//
// Shared memory per alignment: the read as packed words (symbol, quality,
// mismatch penalty), the window as (gap open, symbol) pairs, the traceback
// (4 bits per cell, G*C/2 bytes per row) and the traceback ops. The
// alignment's first lane then runs the traceback and bookkeeping
// (align_finish.cuh).
//
// Cells outside the band, outside [1, n] or outside rows [R0, R1] hold
// NEG_INF exactly as in the reference; rows before R0 hold the initial row
// (M = 0 at every window column, smith_waterman.rs:174-176).
#include <algorithm>
#include <cstdlib>

#include "align_finish.cuh"
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

constexpr int B_PADC = 16;   // window padding (columns) on each side, >= C
constexpr int B_PADR = 16;   // read padding (rows) on each side, >= lanes per alignment

static __host__ __device__ inline size_t b16(size_t x) { return (x + 15) & ~(size_t)15; }

struct BandLayout {
  size_t o_col, o_tb, o_ops, bytes;
};
// Offsets inside one alignment's area (traceback rows of row_bytes); the
// areas of one warp start 32 bytes apart modulo 128 so that the alignments of
// a warp use different banks.
__host__ __device__ inline BandLayout band_layout(int lmax, int nmax, int row_bytes) {
  BandLayout L;
  L.o_col = b16(4 * ((size_t)lmax + 2 * B_PADR));
  L.o_tb = L.o_col + b16(8 * ((size_t)nmax + 2 * B_PADC));
  L.o_ops = L.o_tb + b16((size_t)(lmax + 1) * row_bytes);
  const size_t s = L.o_ops + b16((size_t)lmax + nmax + 2);
  L.bytes = ((s + 127) & ~(size_t)127) + 32;
  return L;
}

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

template <int C>
__device__ __forceinline__ void store_tb(unsigned char* row, int k, uint32_t word) {
  if (C == 8) ((uint32_t*)row)[k] = word;
  else if (C == 4) ((uint16_t*)row)[k] = (uint16_t)word;
  else row[k] = (uint8_t)word;
}

template <int C, int G>
__global__ void __launch_bounds__(32) k_align_band(AlignArgs p, BandLayout LY) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int BJ = 32 / G;         // alignments per warp
  constexpr int ROWB = G * C / 2;    // traceback bytes per row
  const int lane = threadIdx.x & 31;
  const int g = lane / G, k = lane % G;
  unsigned char* my = smem_raw + (size_t)g * LY.bytes;
  int32_t* rowi = (int32_t*)my + B_PADR;         // rowi[i - 1] describes read row i
  int2* coli = (int2*)(my + LY.o_col) + B_PADC;  // coli[j - 1] = (gap open, symbol) of window column j
  unsigned char* tb = my + LY.o_tb;
  uint8_t* ops = my + LY.o_ops;
  const unsigned int njobs = *p.n_jobs;
  unsigned long long cells_acc = 0, jobs_acc = 0;

  while (true) {
    unsigned int jid0 = 0;
    if (lane == 0) jid0 = atomicAdd(p.next_job, (unsigned)BJ);
    jid0 = __shfl_sync(FULL, jid0, 0);
    if (jid0 >= njobs) break;
    const unsigned int jid = jid0 + g;
    AlnJob J;
    J.valid = 0;
    if (jid < njobs) J = p.jobs[jid];
    const bool act = J.valid != 0;
    int m = 0, n = 0;
    if (act) {
      const uint8_t* qbases = J.mate ? p.bases2 : p.bases;
      const uint8_t* qquals = J.mate ? p.quals2 : p.quals;
      const uint64_t* qoffs = J.mate ? p.offs2 : p.offs;
      const uint64_t qo = qoffs[J.read];
      m = (int)(qoffs[J.read + 1] - qo);
      n = (int)(J.ref_end - J.ref_start);
      if (k == 0) jobs_acc++;
      // stage the read and the window
      for (int i = k; i < m; i += G) {
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
        rowi[i] = (int32_t)((uint32_t)__ldg(&p.tab->mmpen[q]) << 16) | ((int32_t)q << 8) | (int32_t)s;
      }
      rowi[-1 - k] = 0;
      rowi[m + k] = 0;
      if (p.ref_bytes) {
        for (int j = k; j < n; j += G) coli[j] = make_int2(0, p.ref_bytes[J.ref_start + j]);
      } else {
        const uint64_t gb = __ldg(&p.G.cbase[J.contig]) + J.ref_start;
        for (int j = k; j < n; j += G) coli[j] = make_int2(0, (int)(uint8_t)"ACGTN"[gcode(p.G, gb + j)]);
      }
      for (int j = k; j < B_PADC; j += G) {
        coli[-1 - j] = make_int2(0, 0);
        coli[n + j] = make_int2(0, 0);
      }
    }
    __syncwarp();
    // gap open per window column from its homopolymer run (smith_waterman.rs:288-291, 348-363):
    // run start by a forward max-scan, run end by a backward min-scan, G lanes per alignment
    int nmx = act ? n : 0;
    for (int d = 16; d >= 1; d >>= 1) nmx = max(nmx, __shfl_xor_sync(FULL, nmx, d));
    {
      int carry = 0;
      for (int c0 = 0; c0 < nmx; c0 += G) {
        const int j = c0 + k;
        const bool in = act && j < n;
        int v = (in && (j == 0 || coli[j].y != coli[j - 1].y)) ? j : -1;
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
          const int y = __shfl_up_sync(FULL, v, d, G);
          if (k >= d) v = max(v, y);
        }
        v = max(v, carry);
        if (in) coli[j].x = v;
        carry = __shfl_sync(FULL, v, G - 1, G);
      }
      __syncwarp();
      int carry_e = act ? n - 1 : 0;
      const int top = nmx > 0 ? ((nmx - 1) / G) * G : -G;
      for (int c0 = top; c0 >= 0; c0 -= G) {
        const int j = c0 + k;
        const bool in = act && j < n;
        int v = (in && (j == n - 1 || coli[j + 1].y != coli[j].y)) ? j : INT32_MAX;
#pragma unroll
        for (int d = 1; d < G; d <<= 1) {
          const int y = __shfl_down_sync(FULL, v, d, G);
          if (k + d < G) v = min(v, y);
        }
        v = min(v, carry_e);
        if (in) {
          int run = v - coli[j].x + 1;
          if (run > 65535) run = 65535;
          const long long gg = (long long)J.gap_open + (run - 1);
          coli[j].x = gg > -1 ? -1 : (int32_t)gg;
        }
        carry_e = __shfl_sync(FULL, v, 0, G);
      }
      __syncwarp();
    }
    // band geometry of this lane's alignment
    const bool dp = act && m > 0 && n > 0;
    const int B = dp ? (int)J.band : 0;
    const long long hint = dp ? J.hint : 0;
    int R0 = 1, R1 = 0;
    if (dp) {
      const long long r0l = 1 - hint - (long long)B;
      R0 = r0l > 1 ? (int)min(r0l, (long long)m + 1) : 1;
      const long long r1l = (long long)n + B - hint;
      R1 = r1l < (long long)m ? (int)max(r1l, 0ll) : m;
    }
    const int nrows = R1 >= R0 ? R1 - R0 + 1 : 0;
    // j = i + base + c; clamping base keeps every empty set of valid j empty
    const long long basel = hint - B;
    const int base = (int)max(min(basel, (long long)n + 1), -(long long)(m + 2 * B + 2));
    const int32_t ge = dp ? J.gap_extend : 0;
    int lo[C], sp[C];
    int32_t PM[C], PI[C], PD[C];
#pragma unroll
    for (int t = 0; t < C; t++) {
      const int c = k * C + t;
      const int lo_t = max(R0, 1 - base - c), hi_t = min(R1, n - base - c);
      if (c <= 2 * B && hi_t >= lo_t && nrows > 0) {
        lo[t] = lo_t;
        sp[t] = hi_t - lo_t;
        cells_acc += (unsigned long long)(hi_t - lo_t + 1);
      } else {
        lo[t] = 1 << 30;
        sp[t] = 0;
      }
      const int jr = R0 - 1 + base + c;
      PM[t] = (jr >= 0 && jr <= n) ? 0 : NEG;
      PI[t] = NEG;
      PD[t] = NEG;
    }
    int T = nrows > 0 ? nrows + G - 1 : 0;
    for (int d = 16; d >= 1; d >>= 1) T = max(T, __shfl_xor_sync(FULL, T, d));
    unsigned long long bestKey = 0;  // (value + 2^31) << 32 | j << 1 | state; 0 = none
    for (int s = 0; s < T; s++) {
      const int i = R0 + s - k;
      const int32_t sLM = __shfl_up_sync(FULL, PM[C - 1], 1, G);
      const int32_t sLD = __shfl_up_sync(FULL, PD[C - 1], 1, G);
      int32_t lM = k ? sLM : NEG, lD = k ? sLD : NEG;
      const int ri = min(max(i - 1, -B_PADR), m - 1 + B_PADR);
      const int32_t rw = rowi[ri];
      const int32_t qsym = rw & 0xFF;
      const int32_t pen = rw >> 16;
      const int jb = min(max(i + base + k * C - 1, -B_PADC), n + B_PADC - C);
      const bool pre = i < R0;
      uint32_t word = 0;
      int32_t upM = NEG, upI = NEG;
#pragma unroll
      for (int t = 0; t < C; t++) {
        const int2 cv = coli[jb + t];
        const int32_t go = cv.x;
        const int32_t sc = qsym == cv.y ? 20 : pen;
        const int32_t dM = PM[t], dI = PI[t], dD = PD[t];
        const int32_t uM = t < C - 1 ? PM[t + 1] : upM;
        const int32_t uI = t < C - 1 ? PI[t + 1] : upI;
        const int32_t m2 = max(max(dM, dI), dD);
        const int32_t Mv = m2 + sc;
        const uint32_t tm = dM == m2 ? 0u : (dI == m2 ? 1u : 2u);
        const int32_t io = uM + go, ie = uI + ge;
        const int32_t Iv = max(io, ie);
        const int32_t dop = lM + go, dex = lD + ge;
        const int32_t Dv = max(dop, dex);
        word |= (tm | (io >= ie ? 0u : 4u) | (dop >= dex ? 0u : 8u)) << (4 * t);
        const bool on = (unsigned)(i - lo[t]) <= (unsigned)sp[t];
        const int32_t nM = on ? Mv : (pre ? dM : NEG);
        const int32_t nI = on ? Iv : NEG;
        const int32_t nD = on ? Dv : NEG;
        PM[t] = nM;
        PI[t] = nI;
        PD[t] = nD;
        lM = nM;
        lD = nD;
        if (t == 0) {
          const int32_t a = __shfl_down_sync(FULL, nM, 1, G);
          const int32_t b = __shfl_down_sync(FULL, nI, 1, G);
          upM = k < G - 1 ? a : NEG;
          upI = k < G - 1 ? b : NEG;
        }
      }
      if (i >= R0 && i <= R1) {
        store_tb<C>(tb + (size_t)(i - R0) * ROWB, k, word);
        if (i == R1) {
          // last row: in-band (M, I) endpoint candidates (smith_waterman.rs:248-251)
#pragma unroll
          for (int t = 0; t < C; t++) {
            if ((unsigned)(i - lo[t]) <= (unsigned)sp[t]) {
              const unsigned long long jj = (unsigned long long)(i + base + k * C + t);
              const unsigned long long kM = ((unsigned long long)((long long)PM[t] + 2147483648LL) << 32) | (jj << 1);
              const unsigned long long kI =
                  ((unsigned long long)((long long)PI[t] + 2147483648LL) << 32) | (jj << 1) | 1ull;
              bestKey = max(bestKey, max(kM, kI));
            }
          }
        }
      }
    }
    for (int d = G / 2; d >= 1; d >>= 1) bestKey = max(bestKey, __shfl_xor_sync(FULL, bestKey, d, G));
    __syncwarp();
    if (act && k == 0) {
      AlnOut* O = p.out + J.slot;
      if (m == 0 || n == 0) {
        finish_empty(m, J.ref_start, O);
      } else {
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
        auto tbr = [&](int i, int jj) -> uint32_t {
          if (i < R0 || i > R1 || jj < 1 || jj > n) return 0u;
          const long long c = (long long)jj - ((long long)i + basel);
          if (c < 0 || c > 2 * B) return 0u;
          const int ci = (int)c;
          const unsigned char* row = tb + (size_t)(i - R0) * ROWB;
          return (uint32_t)(row[ci >> 1] >> ((ci & 1) * 4)) & 15u;
        };
        traceback_cigar(m, endV, endJ, endS, ops, tbr, J.ref_start, O, p.cig_pool, p.cig_pool_used, p.cig_pool_cap,
                        p.err);
      }
    }
    __syncwarp();
  }
  for (int d = 16; d >= 1; d >>= 1) {
    cells_acc += __shfl_down_sync(0xffffffffu, cells_acc, d);
    jobs_acc += __shfl_down_sync(0xffffffffu, jobs_acc, d);
  }
  if (lane == 0 && p.counters) {
    atomicAdd(&p.counters[0], jobs_acc);
    atomicAdd(&p.counters[1], cells_acc);
  }
}

template <int C, int G>
static void launch_band_c(const AlignArgs& a, int num_sms, cudaStream_t st) {
  const BandLayout LY = band_layout(a.lmax, a.nmax, G * C / 2);
  const size_t sm = LY.bytes * (32 / G);
  cudaFuncSetAttribute(k_align_band<C, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  const int per_sm = (int)std::max<size_t>(1, std::min<size_t>(32, (226 * 1024) / (sm + 1024)));
  k_align_band<C, G><<<num_sms * per_sm, 32, sm, st>>>(a, LY);
}

size_t band_smem_bytes(int lmax, int nmax) { return band_layout(lmax, nmax, 32).bytes * 4; }

// Columns covered per alignment G*C > 2*band_max + 1.
void launch_align_band(const AlignArgs& a, int num_sms, int band_max, cudaStream_t st) {
  static const int lanes = getenv("PBW_BAND_LANES") ? atoi(getenv("PBW_BAND_LANES")) : 8;
  if (2 * band_max + 2 <= 16) launch_band_c<2, 8>(a, num_sms, st);
  else if (2 * band_max + 2 <= 32) launch_band_c<4, 8>(a, num_sms, st);
  else if (lanes == 16) launch_band_c<4, 16>(a, num_sms, st);
  else launch_band_c<8, 8>(a, num_sms, st);
}

}  // namespace pbw
