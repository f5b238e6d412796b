// align_window.cu -- K3w: whole-window DP with one block of 8 warps per job.
//
// Used for bands wider than 31: the mate-rescue and shortlist
// cross-alignments of the paired path (SingleEndMapper::align_at_window,
// src/mapper/single.rs:220-275, which bands the aligner to the full window),
// seeded DP with --max-indel-len > 31, and explicit problems of that width.
// The recurrences, tie rules and traceback are those of
// SmithWatermanAligner::align (src/align/smith_waterman.rs:113-255).
//
// A window of n columns is cut into tiles of 32C columns (C = 4 or 8 columns
// per lane); tile k belongs to warp k mod 8. Inside a tile lane l owns the C
// columns j = 32Ck + Cl + 1 .. 32Ck + Cl + C and lags lane l-1 by one row: at
// step t it computes row i = R0 + t - l of its columns from left to right. The left
// and diagonal cells of its first column come from lane l-1's last column by
// __shfl_up_sync; every other input is in the lane's registers (its previous
// row). Lane 0 reads the left column from the boundary buffer that tile
// k-1's lane 31 writes row by row into shared memory, so the eight warps run
// as a wavefront over the tiles: warp w follows warp w-1 at a distance of
// about 40 rows, and a window of n columns takes about n/(32C) * 40 + m steps
// (C columns per lane put C cells of work behind each step's shuffles,
// boundary loads and progress checks). Every step is free of divergent
// branches: the ramps at both ends of a tile, partial and banded tiles
// compute each cell and select its output by predicates. The producer publishes its progress
// every 8 rows (fence, then a volatile store); the consumer polls it with a
// bounded spin.
//
// Per job the window symbols, gap-open costs, traceback ops and the 4-bit
// traceback nibbles live in shared memory when they fit the block's budget,
// otherwise in the block's global slab. One thread then runs the traceback
// and the per-alignment bookkeeping (align_finish.cuh).
#include <algorithm>

#include "align_finish.cuh"
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

constexpr int WIN_WARPS = 8;  // power of two
constexpr int WIN_THREADS = WIN_WARPS * 32;
constexpr int WIN_TAG = 4096;                 // > rows of any job
constexpr unsigned WIN_SPIN_LIMIT = 1u << 22;  // polls before a wait gives up
constexpr size_t WIN_SMEM_CAP = 110 * 1024;    // two blocks per SM

static __host__ __device__ inline size_t w16(size_t x) { return (x + 15) & ~(size_t)15; }

// qs, qq (bytes), per-row mismatch penalty, WIN_WARPS boundary buffers (M, I, D)
__host__ __device__ inline size_t win_fixed_bytes(int lmax) {
  return 2 * w16((size_t)lmax) + w16(4 * (size_t)lmax) + (size_t)WIN_WARPS * 3 * w16(4 * ((size_t)lmax + 2));
}
// window symbols, gap opens, traceback ops and (tbs words per column) nibbles of one job
__host__ __device__ inline size_t win_var_bytes(int m, int n, int tbs) {
  return w16((size_t)n) + w16(4 * (size_t)n) + w16((size_t)m + n + 2) + 4 * ((size_t)n + 1) * tbs;
}
size_t window_smem_bytes(int lmax, int nmax) {
  const size_t fixed = win_fixed_bytes(lmax);
  const size_t want = fixed + win_var_bytes(lmax, nmax, (lmax + 7) / 8);
  return std::min(want, std::max(WIN_SMEM_CAP, fixed + 16 * 1024));
}


struct XBand {
  long long hint, band;
  int n;
  __device__ __forceinline__ int js(int i) const {
    long long v = (long long)i + hint - band;
    return v < 1 ? 1 : (int)v;
  }
  __device__ __forceinline__ int je(int i) const {
    long long v = (long long)i + hint + band;
    if (v > n) v = n;
    if (v < 0) v = 0;
    return (int)v;
  }
};

// WIN_C window columns per lane; MINB resident blocks per SM the registers allow.
template <int WIN_C, int MINB>
__global__ void __launch_bounds__(WIN_THREADS, MINB) k_align_window(AlignArgs p, unsigned int smem_total) {
  constexpr int WIN_TILE = 32 * WIN_C;  // columns per tile (one warp)
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ unsigned int s_jid;
  __shared__ unsigned long long s_best;
  __shared__ volatile int s_pub[WIN_WARPS];
  __shared__ volatile int s_abort;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  uint8_t* qs = sm;
  uint8_t* qq = qs + w16((size_t)p.lmax);
  int32_t* pen = (int32_t*)(qq + w16((size_t)p.lmax));
  int32_t* bufs = (int32_t*)((unsigned char*)pen + w16(4 * (size_t)p.lmax));
  const size_t bstride = w16(4 * ((size_t)p.lmax + 2)) / 4;
  unsigned char* var_smem = sm + win_fixed_bytes(p.lmax);
  const size_t var_avail = (size_t)smem_total - win_fixed_bytes(p.lmax);
  unsigned char* slab = p.tb_global ? p.tb_global + p.tb_global_per_warp * blockIdx.x : nullptr;
  const unsigned int njobs = *p.n_jobs;
  const unsigned int spin_limit = p.wait_polls ? p.wait_polls : WIN_SPIN_LIMIT;
  unsigned long long cells_acc = 0, jobs_acc = 0;

  while (true) {
    if (tid == 0) s_jid = atomicAdd(p.next_job, 1u);
    __syncthreads();
    const unsigned int jid = s_jid;
    if (jid >= njobs) break;
    const AlnJob J = p.jobs[jid];
    AlnOut* O = p.out + J.slot;
    const uint8_t* bases = J.mate ? p.bases2 : p.bases;
    const uint8_t* quals = J.mate ? p.quals2 : p.quals;
    const uint64_t* offs = J.mate ? p.offs2 : p.offs;
    const uint64_t qo = J.valid ? offs[J.read] : 0;
    const int m = J.valid ? (int)(offs[J.read + 1] - qo) : 0;
    const int n = (int)(J.ref_end - J.ref_start);
    const long long r0l = 1 - J.hint - (long long)J.band;
    const int R0 = r0l > 1 ? (int)min(r0l, (long long)m + 1) : 1;
    const long long r1l = (long long)n + J.band - J.hint;
    const int R1 = r1l < (long long)m ? (int)max(r1l, 0ll) : m;
    const int nrows = R1 >= R0 ? R1 - R0 + 1 : 0;
    const int TBS = (nrows + 7) >> 3;
    const bool fits = n <= p.nmax && m <= p.lmax;
    const bool in_smem = win_var_bytes(m, n, TBS) <= var_avail;
    unsigned char* vb = in_smem ? var_smem : slab;
    if (!J.valid || !fits || !vb) {
      if (tid == 0 && J.valid) {
        atomicExch(p.err, 4);
        O->n_ops = 0;
      }
      __syncthreads();
      continue;
    }
    if (tid == 0) jobs_acc++;
    uint8_t* rs = vb;
    int32_t* go = (int32_t*)(vb + w16((size_t)n));
    uint8_t* ops = vb + w16((size_t)n) + w16(4 * (size_t)n);
    uint32_t* tb = (uint32_t*)(ops + w16((size_t)m + n + 2));
    for (int i = tid; i < m; i += WIN_THREADS) {
      uint8_t b, q;
      if (p.ref_bytes) {
        b = bases[qo + i];
        q = quals[qo + i];
      } else if (!J.rev) {
        b = up_ascii(bases[qo + i]);
        q = quals[qo + i];
      } else {
        b = comp_ascii(up_ascii(bases[qo + m - 1 - i]));
        q = quals[qo + m - 1 - i];
      }
      qs[i] = b;
      qq[i] = q;
      pen[i] = __ldg(&p.tab->mmpen[q]) * 256 | (int32_t)b;  // mismatch penalty << 8 | read symbol
    }
    if (p.ref_bytes) {
      for (int j = tid; j < n; j += WIN_THREADS) rs[j] = p.ref_bytes[J.ref_start + j];
    } else {
      const uint64_t gb = __ldg(&p.G.cbase[J.contig]) + J.ref_start;
      for (int j = tid; j < n; j += WIN_THREADS) rs[j] = code_ascii(gcode(p.G, gb + j));
    }
    if (tid == 0) {
      s_best = 0;
      s_abort = 0;
    }
    if (tid < WIN_WARPS) s_pub[tid] = 0;
    __syncthreads();
    if (m == 0 || n == 0) {
      if (tid == 0) finish_empty(m, J.ref_start, O);
      __syncthreads();
      continue;
    }
    // gap open per column from the window's homopolymer runs (smith_waterman.rs:288-291, 348-363)
    if (wid == 0) {
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
    }
    __syncthreads();
    const int32_t ge = J.gap_extend;
    unsigned long long bestKey = 0;  // (value + 2^31) << 32 | j << 1 | state; 0 = none
    if (nrows > 0) {
      const int NT = (n + WIN_TILE - 1) / WIN_TILE;
      for (int k = wid; k < NT; k += WIN_WARPS) {
        const int j0 = 1 + WIN_TILE * k + WIN_C * lane;  // the lane's first column
        uint32_t rsc[WIN_C];   // window symbols of the lane's columns
        int32_t goc[WIN_C];    // gap open of each column
        int ilo[WIN_C], sp[WIN_C];   // rows ilo .. ilo + sp of each column inside the band: js(i) <= j <= je(i)
        bool con[WIN_C];
        bool all_full = true;
#pragma unroll
        for (int c = 0; c < WIN_C; c++) {
          const int j = j0 + c;
          con[c] = j <= n;
          rsc[c] = con[c] ? rs[j - 1] : 0u;
          goc[c] = con[c] ? go[j - 1] : 0;
          ilo[c] = 1 << 30;  // empty: (unsigned)(i - ilo) is never <= sp
          sp[c] = 0;
          if (con[c]) {
            const long long lo = (long long)j - J.hint - (long long)J.band;
            const long long hi = (long long)j - J.hint + (long long)J.band;
            const int a = (int)min(max((long long)R0, lo), (long long)R1 + 1);
            const int b = (int)max(min((long long)R1, hi), (long long)R0 - 1);
            if (b >= a) {
              ilo[c] = a;
              sp[c] = b - a;
              cells_acc += (unsigned long long)(b - a + 1);
            }
          }
          all_full = all_full && con[c] && ilo[c] == R0 && ilo[c] + sp[c] == R1;
        }
        const int bin = (k - 1) & (WIN_WARPS - 1), bout = k & (WIN_WARPS - 1);
        const int32_t* inM = bufs + (size_t)(3 * bin) * bstride;
        const int32_t* inI = inM + bstride;
        const int32_t* inD = inI + bstride;
        int32_t* outM = bufs + (size_t)(3 * bout) * bstride;
        int32_t* outI = outM + bstride;
        int32_t* outD = outI + bstride;
        const bool has_next = k + 1 < NT;
        const int tag_in = (k - 1) * WIN_TAG;
        // the lane's previous row per column (up and, one column right, diagonal);
        // before row R0 it is the initial row (smith_waterman.rs:174-176)
        int32_t PM[WIN_C], PI[WIN_C], PD[WIN_C];
        uint32_t acc[WIN_C];
#pragma unroll
        for (int c = 0; c < WIN_C; c++) {
          PM[c] = con[c] ? 0 : NEG;
          PI[c] = NEG;
          PD[c] = NEG;
          acc[c] = 0;
        }
        int32_t rM = con[0] ? 0 : NEG, rI = NEG, rD = NEG;     // received from lane - 1
        int32_t qM = lane == 0 ? 0 : NEG, qI = NEG, qD = NEG;  // diagonal of the first column
        uint32_t* tbc = tb + (size_t)j0 * TBS;                 // column j0 + c at tbc + c * TBS
        const int T = nrows + 31;
        // Steps where every lane's row is inside [R0, R1 - 1] and all of the
        // tile's columns are in the window and the band take the branch-free
        // form below; the ramps at both ends (and tiles with a partial or
        // banded column) take the general form.
        const bool full_tile = __all_sync(0xffffffffu, all_full);
        const int f0 = full_tile ? 31 : T, f1 = full_tile ? max(31, nrows - 1) : T;
        auto poll = [&](int t) {
          if (k > 0 && (t & 7) == 0 && t < nrows) {
            const int target = tag_in + min(t + 8, nrows);
            unsigned int spins = 0;
            while (s_pub[bin] < target) {
              if (s_abort) break;
              if (++spins > spin_limit) {
                if (lane == 0) {
                  s_abort = 1;
                  atomicExch(p.err, 9);
                }
                break;
              }
            }
            __threadfence_block();
          }
        };
        auto publish = [&](int t, int i) {
          if (has_next) {
            if (lane == 31 && i >= R0 && i <= R1) {
              outM[i] = PM[WIN_C - 1];
              outI[i] = PI[WIN_C - 1];
              outD[i] = PD[WIN_C - 1];
            }
            const int done = t - 30;  // rows R0 .. R0 + done - 1 written by lane 31
            if (done > 0 && ((done & 7) == 0 || done == nrows) && lane == 31) {
              __threadfence_block();
              s_pub[bout] = k * WIN_TAG + done;
            }
          }
        };
        // Ramps, partial and banded tiles: every cell is computed and the
        // output is selected (in the band: the cell; row R0 - 1 of a window
        // column: the initial row; else NEG_INF), so that lanes at different
        // rows take no divergent branches.
        auto general = [&](int t) {
          const int i = R0 + t - lane;
          const int i0 = R0 + t;  // lane 0's row
          poll(t);
          int32_t bM = NEG, bI = NEG, bD = NEG;
          if (k > 0 && i0 <= R1) {
            bM = inM[i0];
            bI = inI[i0];
            bD = inD[i0];
          }
          int32_t lM = lane == 0 ? bM : rM;  // (i, j0 - 1)
          int32_t lD = lane == 0 ? bD : rD;
          const int32_t nqM = lM, nqI = lane == 0 ? bI : rI, nqD = lD;
          int32_t dgM = qM, dgI = qI, dgD = qD;  // (i - 1, j0 - 1)
          const int32_t pv = pen[min(max(i - 1, 0), m - 1)];
          const uint32_t qsym = (uint32_t)pv & 0xFFu;
          const int32_t mp = pv >> 8;
          const int rr = i - R0;
          const int sh = (rr & 7) * 4;
          const bool init_row = i == R0 - 1;
          const bool last_row = i == R1;
#pragma unroll
          for (int c = 0; c < WIN_C; c++) {
            const int32_t uM = PM[c], uI = PI[c], uD = PD[c];
            const bool on = (unsigned)(i - ilo[c]) <= (unsigned)sp[c];
            const int32_t sc = rsc[c] == qsym ? 20 : mp;
            const int32_t m2 = max(max(dgM, dgI), dgD);
            const int32_t Mv = m2 + sc;
            const uint32_t tm = dgM == m2 ? 0u : (dgI == m2 ? 1u : 2u);
            const int32_t io = uM + goc[c], ie = uI + ge;
            const int32_t Iv = max(io, ie);
            const int32_t dop = lM + goc[c], dex = lD + ge;
            const int32_t Dv = max(dop, dex);
            const uint32_t nib = tm | (io >= ie ? 0u : 4u) | (dop >= dex ? 0u : 8u);
            acc[c] |= on ? nib << sh : 0u;
            if (on && ((rr & 7) == 7 || i == ilo[c] + sp[c])) {
              tbc[(size_t)c * TBS + (rr >> 3)] = acc[c];
              acc[c] = 0;
            }
            if (on && last_row) {
              const unsigned long long jj = (unsigned long long)(j0 + c);
              const unsigned long long kM = ((unsigned long long)((long long)Mv + 2147483648LL) << 32) | (jj << 1);
              const unsigned long long kI =
                  ((unsigned long long)((long long)Iv + 2147483648LL) << 32) | (jj << 1) | 1ull;
              bestKey = max(bestKey, max(kM, kI));
            }
            const int32_t oM = on ? Mv : ((init_row && con[c]) ? 0 : NEG);
            const int32_t oI = on ? Iv : NEG;
            const int32_t oD = on ? Dv : NEG;
            PM[c] = oM;
            PI[c] = oI;
            PD[c] = oD;
            dgM = uM;
            dgI = uI;
            dgD = uD;
            lM = oM;
            lD = oD;
          }
          publish(t, i);
          qM = nqM;
          qI = nqI;
          qD = nqD;
          rM = __shfl_up_sync(0xffffffffu, PM[WIN_C - 1], 1);
          rI = __shfl_up_sync(0xffffffffu, PI[WIN_C - 1], 1);
          rD = __shfl_up_sync(0xffffffffu, PD[WIN_C - 1], 1);
        };
        int t = 0;
        for (; t < f0; t++) general(t);
        for (; t < f1; t++) {
          // every lane in rows [R0, R1 - 1], every column in the window and the band
          const int i = R0 + t - lane;
          poll(t);
          int32_t lM = rM, lI = rI, lD = rD;
          if (k > 0) {
            const int32_t bM = inM[R0 + t], bI = inI[R0 + t], bD = inD[R0 + t];
            if (lane == 0) {
              lM = bM;
              lI = bI;
              lD = bD;
            }
          } else if (lane == 0) {
            lM = NEG;
            lI = NEG;
            lD = NEG;
          }
          const int32_t nqM = lM, nqI = lI, nqD = lD;
          int32_t dgM = qM, dgI = qI, dgD = qD;
          const int32_t pv = pen[i - 1];
          const uint32_t qsym = (uint32_t)pv & 0xFFu;
          const int32_t mp = pv >> 8;
          const int rr = i - R0;
          const int sh = (rr & 7) * 4;
#pragma unroll
          for (int c = 0; c < WIN_C; c++) {
            const int32_t uM = PM[c], uI = PI[c], uD = PD[c];
            const int32_t sc = rsc[c] == qsym ? 20 : mp;
            const int32_t m2 = max(max(dgM, dgI), dgD);
            const int32_t Mv = m2 + sc;
            const uint32_t tm = dgM == m2 ? 0u : (dgI == m2 ? 1u : 2u);
            const int32_t io = uM + goc[c], ie = uI + ge;
            const int32_t Iv = max(io, ie);
            const int32_t dop = lM + goc[c], dex = lD + ge;
            const int32_t Dv = max(dop, dex);
            acc[c] |= (tm | (io >= ie ? 0u : 4u) | (dop >= dex ? 0u : 8u)) << sh;
            PM[c] = Mv;
            PI[c] = Iv;
            PD[c] = Dv;
            dgM = uM;
            dgI = uI;
            dgD = uD;
            lM = Mv;
            lD = Dv;
          }
          rM = __shfl_up_sync(0xffffffffu, PM[WIN_C - 1], 1);
          rI = __shfl_up_sync(0xffffffffu, PI[WIN_C - 1], 1);
          rD = __shfl_up_sync(0xffffffffu, PD[WIN_C - 1], 1);
          if ((rr & 7) == 7) {
#pragma unroll
            for (int c = 0; c < WIN_C; c++) {
              tbc[(size_t)c * TBS + (rr >> 3)] = acc[c];
              acc[c] = 0;
            }
          }
          publish(t, i);
          qM = nqM;
          qI = nqI;
          qD = nqD;
        }
        for (; t < T; t++) general(t);
      }
    }
    for (int d = 16; d >= 1; d >>= 1) bestKey = max(bestKey, __shfl_xor_sync(0xffffffffu, bestKey, d));
    if (lane == 0 && bestKey) atomicMax(&s_best, bestKey);
    __syncthreads();
    if (tid == 0) {
      const XBand B{J.hint, (long long)J.band, n};
      int endV, endJ, endS;
      if (R1 < R0) {
        endV = 0;
        endJ = n;
        endS = 0;
      } else {
        const unsigned long long best = s_best;
        if (best == 0) {
          endV = NEG;
          endJ = -1;
          endS = 0;
        } else {
          endV = (int)((long long)(best >> 32) - 2147483648LL);
          endJ = (int)((best >> 1) & 0x7FFFFFFFull);
          endS = (int)(best & 1ull);
        }
        resolve_endpoint(endV, endJ, endS, B.js(R1), B.je(R1), n);
      }
      auto tbr = [&](int i, int j) -> uint32_t {
        if (i < R0 || i > R1 || j < 1 || j < B.js(i) || j > B.je(i)) return 0u;
        const int rr = i - R0;
        return (tb[(size_t)j * TBS + (rr >> 3)] >> ((rr & 7) * 4)) & 15u;
      };
      traceback_cigar(m, endV, endJ, endS, ops, tbr, J.ref_start, O, p.cig_pool, p.cig_pool_used, p.cig_pool_cap,
                      p.err);
    }
    __syncthreads();
  }
  if (p.counters) {
    for (int d = 16; d >= 1; d >>= 1) cells_acc += __shfl_down_sync(0xffffffffu, cells_acc, d);
    if (lane == 0) atomicAdd(&p.counters[1], cells_acc);
    if (tid == 0) atomicAdd(&p.counters[0], jobs_acc);
  }
}

// wide: 8 columns per lane, one block per SM (the paired path's ~1,000
// column windows, fewer jobs per batch than SMs: the job's latency is the
// batch's); else 4 columns per lane and two blocks per SM (many narrower
// windows: throughput).
void launch_align_window(const AlignArgs& a, int grid, cudaStream_t st, bool wide) {
  const size_t sm = window_smem_bytes(a.lmax, a.nmax);
  if (wide) {
    smem_ceiling(k_align_window<8, 1>);
    k_align_window<8, 1><<<std::max(1, grid / 2), WIN_THREADS, sm, st>>>(a, (unsigned int)sm);
  } else {
    smem_ceiling(k_align_window<4, 2>);
    k_align_window<4, 2><<<grid, WIN_THREADS, sm, st>>>(a, (unsigned int)sm);
  }
}

}  // namespace pbw
