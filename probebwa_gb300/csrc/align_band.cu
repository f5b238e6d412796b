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
// mismatch penalty), the window as (gap open, symbol) pairs, a two-chunk ring
// of traceback rows and the CIGAR run stack. The traceback itself (4 bits per
// cell, G*C/2 bytes per row) goes to a per-alignment global slab, which stays
// in L2: keeping it out of shared memory more than doubles the warps an SM
// holds, which the DP's short dependency chains need. The alignment's lanes
// then walk the traceback together, streaming its rows back into the ring
// with cp.async one 16-row chunk ahead of the walk.
//
// Cells outside the band, outside [1, n] or outside rows [R0, R1] hold
// NEG_INF exactly as in the reference; rows before R0 hold the initial row
// (M = 0 at every window column, smith_waterman.rs:174-176).
#include <algorithm>
#include <type_traits>

#include "align_finish.cuh"
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

constexpr int B_PADC = 16;   // window padding (columns) on each side, >= C
constexpr int B_PADR = 16;   // read padding (rows) on each side, >= lanes per alignment

static __host__ __device__ inline size_t b16(size_t x) { return (x + 15) & ~(size_t)15; }

constexpr int TB_CH = 16;    // traceback rows per prefetched chunk

struct BandLayout {
  size_t o_col, o_ring, o_runs, bytes;  // shared memory of one alignment
  size_t tb_job;                        // global traceback bytes of one alignment
};
// Offsets inside one alignment's shared area (traceback rows of row_bytes);
// the areas of one warp start 32 bytes apart modulo 128 so that the
// alignments of a warp use different banks.
__host__ __device__ inline BandLayout band_layout(int lmax, int nmax, int row_bytes) {
  BandLayout L;
  // The read rows and window columns are dead once the DP is done: the
  // traceback's chunk ring and CIGAR run stack reuse their space.
  L.o_col = b16(4 * ((size_t)lmax + 2 * B_PADR));
  const size_t dp_bytes = L.o_col + b16(8 * ((size_t)nmax + 2 * B_PADC));
  L.o_ring = 0;
  L.o_runs = 2 * TB_CH * (size_t)row_bytes;
  const size_t tb_bytes = L.o_runs + b16(2 * ((size_t)lmax + nmax + 2));
  const size_t s = std::max(dp_bytes, tb_bytes);
  L.bytes = ((s + 127) & ~(size_t)127) + 32;
  L.tb_job = (((size_t)lmax + 1 + TB_CH - 1) / TB_CH) * TB_CH * row_bytes;
  return L;
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}


// One lane's traceback nibbles of a row: C cells of 4 bits.
template <int C>
using TbWord = typename std::conditional<(C > 8), unsigned long long, uint32_t>::type;

template <int C>
__device__ __forceinline__ void store_tb(unsigned char* row, int k, TbWord<C> word) {
  if (C == 16) ((unsigned long long*)row)[k] = word;
  else if (C == 8) ((uint32_t*)row)[k] = (uint32_t)word;
  else if (C == 4) ((uint16_t*)row)[k] = (uint16_t)word;
  else row[k] = (uint8_t)word;
}

// Traceback (smith_waterman.rs:299-344) over the band's traceback rows, in
// band coordinates c = j - (i + base): M keeps c and moves up a row, I moves
// up a row and right a column, D moves left a column; j == 0 emits I.
// Nibbles outside rows [R0, R1], the band or the window read as 0. Runs of
// equal operations (collapse_cigar, :365-381) are pushed on a 16-bit stack as
// they end, so no per-operation array is kept; the CIGAR is then written in
// forward order.
//
// All G lanes of the alignment run the same walk (the leader, k == 0, writes
// the results). The rows come from the global slab through the shared ring:
// chunk q holds rows R0 + 16q .. R0 + 16q + 15; the walk only moves up, so
// while it reads chunk q from one ring slot, chunk q-1 is already in flight
// into the other, and entering chunk q-1 starts the copy of q-2. Every wait
// is a cp.async.wait_group, which ends when the thread's own copies land.
template <int ROWB, int G>
__device__ void band_traceback(int k, unsigned gmask, int m, int n, int B, int R0, int R1, long long basel, int endV,
                               int endJ, int endS, const unsigned char* tbg, unsigned char* ring, uint16_t* runs,
                               unsigned long long ref_start, AlnOut* O, uint32_t* cig_pool,
                               unsigned int* cig_pool_used, uint32_t cig_pool_cap, int* err) {
  constexpr int PIECES = TB_CH * ROWB / 16;  // 16-byte copies per chunk
  auto fetch = [&](int q) {
    if (q >= 0) {
      const unsigned char* src = tbg + (size_t)q * TB_CH * ROWB;
      unsigned char* dst = ring + (size_t)(q & 1) * TB_CH * ROWB;
      for (int x = k; x < PIECES; x += G) cp_async16(dst + 16 * x, src + 16 * x);
    }
    cp_async_commit();
  };
  const bool base_ok = basel >= -(long long)(1 << 29) && basel <= (long long)(1 << 29);
  const int base = base_ok ? (int)basel : 0;
  int cur_q = -1;
  if (R1 >= R0) {
    cur_q = (R1 - R0) / TB_CH;
    fetch(cur_q);
    fetch(cur_q - 1);
    cp_async_wait<1>();
    __syncwarp(gmask);
  }
  int i = m, j = endJ, st = endS;
  int c = j - i - base;
  int nruns = 0, run = 0, cur = -1, span = 0;
  while (i > 0) {
    const bool j0 = j == 0;
    const bool inb = base_ok && i >= R0 && i <= R1 && j >= 1 && j <= n && c >= 0 && c <= 2 * B;
    uint32_t nib = 0;
    if (inb) {
      const int rr = i - R0;
      if (rr / TB_CH < cur_q) {  // the walk entered the next chunk down
        cp_async_wait<0>();
        __syncwarp(gmask);
        fetch(cur_q - 2);
        cur_q--;
      }
      const uint32_t byte = ring[(size_t)(cur_q & 1) * TB_CH * ROWB + (size_t)(rr % TB_CH) * ROWB + (c >> 1)];
      nib = (byte >> ((c & 1) * 4)) & 15u;
    }
    const int op = j0 ? 1 : st;
    const int from_m = (int)(nib & 3u), from_i = (int)((nib >> 2) & 1u), from_d = (int)((nib >> 2) & 2u);
    st = j0 ? st : (st == 0 ? from_m : (st == 1 ? from_i : from_d));
    const bool brk = op != cur && cur >= 0;
    if (brk && k == 0) runs[nruns] = (uint16_t)((run << 2) | cur);
    nruns += brk ? 1 : 0;
    run = op != cur ? 1 : run + 1;
    cur = op;
    span += op != 1 ? 1 : 0;
    i -= op != 2 ? 1 : 0;
    j -= op != 1 ? 1 : 0;
    c += op == 1 ? 1 : (op == 2 ? -1 : 0);
  }
  cp_async_wait<0>();
  if (k != 0) return;
  if (cur >= 0) runs[nruns++] = (uint16_t)((run << 2) | cur);
  const uint32_t ncig = (uint32_t)nruns;
  uint32_t pool_base = 0xFFFFFFFFu;
  if (ncig > CIG_INLINE) {
    pool_base = atomicAdd(cig_pool_used, ncig);
    if (pool_base + ncig > cig_pool_cap) {
      atomicExch(err, 3);
      pool_base = 0xFFFFFFFFu;
    }
  }
  uint32_t* cdst = ncig > CIG_INLINE ? (pool_base != 0xFFFFFFFFu ? cig_pool + pool_base : nullptr) : O->cig;
  if (cdst) {
    for (uint32_t q = 0; q < ncig; q++) {
      const uint32_t r = runs[ncig - 1 - q];
      cdst[q] = ((r >> 2) << 4) | (r & 3u);
    }
  }
  O->pos = ref_start + (unsigned long long)j;
  O->score = endV;
  O->span = (uint32_t)span;
  O->n_ops = ncig;
  O->cig_pool = pool_base;
}

// One step of C cells of row i for one lane (see the file comment). GENERAL
// applies the exact masks of every cell: outside the band, the window or
// rows [R0, R1] a cell is NEG_INF, and rows before R0 keep the initial row.
// The fast form is used once every lane of the warp is past the window's
// left edge and row R0: then no cell an in-band cell reads is outside the
// window or the rows, so the only cell that must be forced to NEG_INF is
// column 2*band + 1 (M and I; its up value feeds column 2*band), at lane
// kstar, position TSTAR.
template <int C, int G, int TSTAR, bool GENERAL>
__device__ __forceinline__ TbWord<C> band_step(int32_t (&PM)[C], int32_t (&PI)[C], int32_t (&PD)[C], const int (&lo)[C],
                                              const int (&sp)[C], int k, int i, int R0, int kstar, int32_t qsym,
                                              int32_t pen, int32_t ge, const int2* cols) {
  constexpr unsigned FULL = 0xffffffffu;
  const int32_t sLM = __shfl_up_sync(FULL, PM[C - 1], 1, G);
  const int32_t sLD = __shfl_up_sync(FULL, PD[C - 1], 1, G);
  int32_t lM = k ? sLM : NEG, lD = k ? sLD : NEG;
  const bool pre = i < R0;
  const bool kill = k == kstar;
  TbWord<C> word = 0;
  int32_t upM = NEG, upI = NEG;
#pragma unroll
  for (int t = 0; t < C; t++) {
    const int2 cv = cols[t];
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
    word |= (TbWord<C>)(tm | (io >= ie ? 0u : 4u) | (dop >= dex ? 0u : 8u)) << (4 * t);
    int32_t nM, nI, nD;
    if (GENERAL) {
      const bool on = (unsigned)(i - lo[t]) <= (unsigned)sp[t];
      nM = on ? Mv : (pre ? dM : NEG);
      nI = on ? Iv : NEG;
      nD = on ? Dv : NEG;
    } else if (t == TSTAR) {
      nM = kill ? NEG : Mv;
      nI = kill ? NEG : Iv;
      nD = Dv;
    } else {
      nM = Mv;
      nI = Iv;
      nD = Dv;
    }
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
  return word;
}

template <bool B>
struct BoolConst {
  static constexpr bool value = B;
};

template <int C, int G, int TSTAR>
// The 4-lane form keeps 16 columns of state per lane; its shared memory
// (8 alignments per warp) already holds it to a few blocks per SM, so its
// register bound is looser.
__global__ void __launch_bounds__(32, G == 4 ? 4 : 16) k_align_band(AlignArgs p, BandLayout LY) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int BJ = 32 / G;         // alignments per warp
  constexpr int ROWB = G * C / 2;    // traceback bytes per row
  const int lane = threadIdx.x & 31;
  const int g = lane / G, k = lane % G;
  unsigned char* my = smem_raw + (size_t)g * LY.bytes;
  int32_t* rowi = (int32_t*)my + B_PADR;         // rowi[i - 1] describes read row i
  int2* coli = (int2*)(my + LY.o_col) + B_PADC;  // coli[j - 1] = (gap open, symbol) of window column j
  unsigned char* ring = my + LY.o_ring;
  uint16_t* runs = (uint16_t*)(my + LY.o_runs);
  unsigned char* tbg = p.tb_global + ((size_t)blockIdx.x * BJ + g) * LY.tb_job;
  const unsigned gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (g * G);
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
          s = up_ascii(qbases[qo + i]);
          q = qquals[qo + i];
        } else {
          s = comp_ascii(up_ascii(qbases[qo + m - 1 - i]));
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
        for (int j = k; j < n; j += G) coli[j] = make_int2(0, (int)code_ascii(gcode(p.G, gb + j)));
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
    // first step of the fast form: every lane past row R0 (s >= k) and with
    // all its columns at j >= 1; only when column 2*band + 1 sits at TSTAR
    const int cstar = 2 * B + 1;
    const int kstar = cstar < G * C ? cstar / C : G;
    const bool fast_ok = !dp || cstar >= G * C || cstar % C == TSTAR;
    int S0 = dp ? max(k, 1 - base - k * C - R0 + k) : 0;
    S0 = fast_ok ? S0 : T;
    for (int d = 16; d >= 1; d >>= 1) S0 = max(S0, __shfl_xor_sync(FULL, S0, d));
    S0 = min(S0, T);
    unsigned long long bestKey = 0;  // (value + 2^31) << 32 | j << 1 | state; 0 = none
    // one step: row i = R0 + s - k of this lane's columns, its traceback
    // word, and on row R1 the endpoint candidates. The masked steps (s < S0)
    // and the fast ones run as two loops, so neither carries the other's
    // selects.
    auto row = [&](int s, auto general) {
      constexpr bool GEN = decltype(general)::value;
      const int i = R0 + s - k;
      const int ri = min(max(i - 1, -B_PADR), m - 1 + B_PADR);
      const int32_t rw = rowi[ri];
      const int32_t qsym = rw & 0xFF;
      const int32_t pen = rw >> 16;
      const int jb = min(max(i + base + k * C - 1, -B_PADC), n + B_PADC - C);
      const TbWord<C> word = band_step<C, G, TSTAR, GEN>(PM, PI, PD, lo, sp, k, i, R0, kstar, qsym, pen, ge, coli + jb);
      if (i >= R0 && i <= R1) {
        store_tb<C>(tbg + (size_t)(i - R0) * ROWB, k, word);
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
    };
    int s = 0;
    for (; s < S0; s++) row(s, BoolConst<true>{});
    for (; s < T; s++) row(s, BoolConst<false>{});
    for (int d = G / 2; d >= 1; d >>= 1) bestKey = max(bestKey, __shfl_xor_sync(FULL, bestKey, d, G));
    // the traceback rows written above, by every lane, are read back through
    // cp.async by the lanes of the same alignment
    __threadfence_block();
    __syncwarp();
    if (act) {
      AlnOut* O = p.out + J.slot;
      if (m == 0 || n == 0) {
        if (k == 0) finish_empty(m, J.ref_start, O);
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
        band_traceback<ROWB, G>(k, gmask, m, n, B, R0, R1, basel, endV, endJ, endS, tbg, ring, runs, J.ref_start,
                                O, p.cig_pool, p.cig_pool_used, p.cig_pool_cap, p.err);
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
static int band_grid(const BandLayout& LY, int num_sms) {
  const size_t sm = LY.bytes * (32 / G);
  return num_sms * (int)std::max<size_t>(1, std::min<size_t>(32, (226 * 1024) / (sm + 1024)));
}

static int band_c(int band_max) { return 2 * band_max + 2 <= 16 ? 2 : (2 * band_max + 2 <= 32 ? 4 : 8); }

template <int C, int G, int TSTAR>
static void launch_band_c(const AlignArgs& a, int num_sms, cudaStream_t st) {
  const BandLayout LY = band_layout(a.lmax, a.nmax, G * C / 2);
  const size_t sm = LY.bytes * (32 / G);
  smem_ceiling(k_align_band<C, G, TSTAR>);
  k_align_band<C, G, TSTAR><<<band_grid<C, G>(LY, num_sms), 32, sm, st>>>(a, LY);
}

// Global traceback slab that launch_align_band needs in AlignArgs::tb_global:
// enough for either lane count (8 or 16 lanes per alignment).
size_t band_tb_slab_bytes(int lmax, int nmax, int num_sms, int band_max) {
  const int C = band_c(band_max);
  const BandLayout L8 = band_layout(lmax, nmax, 8 * C / 2);
  const int g8 = C == 2 ? band_grid<2, 8>(L8, num_sms) : (C == 4 ? band_grid<4, 8>(L8, num_sms) : band_grid<8, 8>(L8, num_sms));
  size_t need = (size_t)g8 * 4 * L8.tb_job;
  if (C >= 4) {
    // 16 lanes with half the columns per lane
    const BandLayout L16 = band_layout(lmax, nmax, 16 * (C / 2) / 2);
    const int g16 = C == 4 ? band_grid<2, 16>(L16, num_sms) : band_grid<4, 16>(L16, num_sms);
    need = std::max(need, (size_t)g16 * 2 * L16.tb_job);
  }
  if (C == 8) {
    // 4 lanes with twice the columns per lane
    const BandLayout L4 = band_layout(lmax, nmax, 4 * 16 / 2);
    need = std::max(need, (size_t)band_grid<16, 4>(L4, num_sms) * 8 * L4.tb_job);
  }
  return need;
}

// Whether a 16-lane form exists for the band (a band of at least 8 columns
// per 8 lanes, i.e. C >= 4).
bool band_has_lanes16(int band_max) { return band_c(band_max) >= 4; }
// Whether a 4-lane form exists for the band (16 columns per lane: bands of
// 16 to 31).
bool band_has_lanes4(int band_max) { return band_c(band_max) == 8; }

// lanes lanes per alignment, C columns per lane with lanes*C > 2*band_max + 1;
// the fast form is compiled for column 2*band_max + 1 at lane position TSTAR
// (odd, as 2*band + 1 is odd and C even); alignments of other bands in the
// same launch use the masked form throughout. lanes 16 halves C (bands with
// C >= 4 only); lanes 4 doubles it (C == 8 only).
void launch_align_band_lanes(const AlignArgs& a, int num_sms, int band_max, int lanes, cudaStream_t st) {
  const int cstar = 2 * band_max + 1;
  const int C = band_c(band_max);
  if (lanes == 4 && C == 8) {
    switch (cstar % 16) {
      case 1: launch_band_c<16, 4, 1>(a, num_sms, st); break;
      case 3: launch_band_c<16, 4, 3>(a, num_sms, st); break;
      case 5: launch_band_c<16, 4, 5>(a, num_sms, st); break;
      case 7: launch_band_c<16, 4, 7>(a, num_sms, st); break;
      case 9: launch_band_c<16, 4, 9>(a, num_sms, st); break;
      case 11: launch_band_c<16, 4, 11>(a, num_sms, st); break;
      case 13: launch_band_c<16, 4, 13>(a, num_sms, st); break;
      default: launch_band_c<16, 4, 15>(a, num_sms, st); break;
    }
    return;
  }
  if (lanes == 16 && C >= 4) {
    if (C == 4) {
      launch_band_c<2, 16, 1>(a, num_sms, st);
    } else if (cstar % 4 == 1) {
      launch_band_c<4, 16, 1>(a, num_sms, st);
    } else {
      launch_band_c<4, 16, 3>(a, num_sms, st);
    }
    return;
  }
  if (C == 2) {
    launch_band_c<2, 8, 1>(a, num_sms, st);
  } else if (C == 4) {
    if (cstar % 4 == 1) launch_band_c<4, 8, 1>(a, num_sms, st);
    else launch_band_c<4, 8, 3>(a, num_sms, st);
  } else {
    switch (cstar % 8) {
      case 1: launch_band_c<8, 8, 1>(a, num_sms, st); break;
      case 3: launch_band_c<8, 8, 3>(a, num_sms, st); break;
      case 5: launch_band_c<8, 8, 5>(a, num_sms, st); break;
      default: launch_band_c<8, 8, 7>(a, num_sms, st); break;
    }
  }
}

void launch_align_band(const AlignArgs& a, int num_sms, int band_max, cudaStream_t st) {
  launch_align_band_lanes(a, num_sms, band_max, 8, st);
}

}  // namespace pbw
