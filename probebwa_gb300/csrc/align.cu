// align.cu -- K3: banded affine-gap DP with traceback
// (SmithWatermanAligner::align, src/align/smith_waterman.rs:163-345), one
// warp per alignment, fed by a device work queue.
//
// Wavefront: the warp walks the DP rows in strips of 32; lane l owns row
// i = s0 + l and lags lane l-1 by one column, so at step t lane l computes
// cell (i, j = jlo + t - l) -- all 32 cells of a step lie on one
// anti-diagonal of the strip and are independent. The three values of the
// cell above travel from lane l-1 by __shfl_up_sync; the cell to the left is
// the lane's own previous output; the diagonal is what arrived one step
// earlier. Lane 0 reads the row above from a shared-memory row buffer that
// lane 31 of the previous strip filled. Integer arithmetic and tie rules are
// those of the reference, including the NEG_INF = i32::MIN/2 sentinel of
// cells outside the band, rows whose band is empty being skipped without a
// reset, and the "last maximum" endpoint over (M, I) of the final row.
//
// Traceback pointers (tb_m 2 bits, tb_i 1, tb_d 1 per cell) are kept as
// nibbles in shared memory (band coordinates when the band is <= 31, full
// rows otherwise) or, for windows too wide for shared memory, in a per-warp
// global scratch slab. Lane 0 then walks the traceback and derives the CIGAR,
// the alignment log-likelihood (bayesian.rs:142-179), the log_entropy inputs
// (bayesian.rs:306-357) and the edit distance.
#include "pbw_common.cuh"
#include "pbw_kernels.h"
#include "align_finish.cuh"

namespace pbw {

struct AlnSmem {
  uint8_t* qs;    // query symbols (lmax)
  uint8_t* qq;    // query qualities (lmax)
  uint8_t* rs;    // reference symbols (nmax)
  int32_t* go;    // gap open per column (nmax)
  int32_t* bufM;  // row buffer (nmax + 1)
  int32_t* bufI;
  int32_t* bufD;
  uint8_t* ops;   // traceback ops, reversed (lmax + nmax + 2)
  uint32_t* tb;   // shared traceback (tb_smem bytes)
};

static __host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t align_smem_bytes(int lmax, int nmax, size_t tb_smem) {
  return al16(lmax) + al16(lmax) + al16(nmax) + al16(4 * (size_t)nmax) + 3 * al16(4 * ((size_t)nmax + 1)) +
         al16((size_t)lmax + nmax + 2) + al16(tb_smem);
}
size_t align_smem_per_warp(int lmax, int nmax, size_t tb_smem) { return align_smem_bytes(lmax, nmax, tb_smem); }

__device__ inline void carve(AlnSmem& s, unsigned char* base, int lmax, int nmax) {
  size_t o = 0;
  s.qs = base + o; o += al16(lmax);
  s.qq = base + o; o += al16(lmax);
  s.rs = base + o; o += al16(nmax);
  s.go = (int32_t*)(base + o); o += al16(4 * (size_t)nmax);
  s.bufM = (int32_t*)(base + o); o += al16(4 * ((size_t)nmax + 1));
  s.bufI = (int32_t*)(base + o); o += al16(4 * ((size_t)nmax + 1));
  s.bufD = (int32_t*)(base + o); o += al16(4 * ((size_t)nmax + 1));
  s.ops = base + o; o += al16((size_t)lmax + nmax + 2);
  s.tb = (uint32_t*)(base + o);
}

// Uppercase ASCII (DnaSeq::from_ascii, src/types.rs:12-15).
__device__ __forceinline__ uint8_t up_ascii(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }
// Complement used by DnaSeq::reverse_complement (src/types.rs:34-48).
__device__ __forceinline__ uint8_t comp_ascii(uint8_t b) {
  switch (b) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'C': return 'G';
    case 'G': return 'C';
    default: return 'N';
  }
}

struct Band {
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

__global__ void __launch_bounds__(128) k_align(AlignArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const size_t per_warp = align_smem_bytes(p.lmax, p.nmax, p.tb_smem);
  AlnSmem S;
  carve(S, smem_raw + per_warp * wib, p.lmax, p.nmax);
  const unsigned int gwarp = blockIdx.x * (blockDim.x >> 5) + wib;
  uint32_t* tb_glob = p.tb_global ? (uint32_t*)(p.tb_global + p.tb_global_per_warp * gwarp) : nullptr;
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
    // ---- stage query and reference ----
    const uint8_t* qbases = J.mate ? p.bases2 : p.bases;
    const uint8_t* qquals = J.mate ? p.quals2 : p.quals;
    const uint64_t* qoffs = J.mate ? p.offs2 : p.offs;
    const uint64_t qo = qoffs[J.read];
    const int m = (int)(qoffs[J.read + 1] - qo);
    const int n = (int)(J.ref_end - J.ref_start);
    for (int i = lane; i < m; i += 32) {
      if (p.ref_bytes) {
        S.qs[i] = qbases[qo + i];
        S.qq[i] = qquals[qo + i];
      } else if (!J.rev) {
        S.qs[i] = up_ascii(qbases[qo + i]);
        S.qq[i] = qquals[qo + i];
      } else {
        S.qs[i] = comp_ascii(up_ascii(qbases[qo + m - 1 - i]));
        S.qq[i] = qquals[qo + m - 1 - i];
      }
    }
    if (p.ref_bytes) {
      for (int j = lane; j < n; j += 32) S.rs[j] = p.ref_bytes[J.ref_start + j];
    } else {
      const uint64_t gb = __ldg(&p.G.cbase[J.contig]) + J.ref_start;
      for (int j = lane; j < n; j += 32) {
        uint8_t c = gcode(p.G, gb + j);
        S.rs[j] = (uint8_t)"ACGTN"[c];
      }
    }
    __syncwarp();
    if (m == 0 || n == 0) {
      if (lane == 0) finish_empty(m, J.ref_start, O);
      continue;
    }
    // homopolymer run length per position (smith_waterman.rs:348-363) and
    // the discounted gap open (smith_waterman.rs:288-291): run start by a
    // warp prefix-max, run end by a suffix-min, 32 columns at a time.
    {
      int carry = 0;
      for (int c0 = 0; c0 < n; c0 += 32) {
        const int j = c0 + lane;
        int v = (j < n && (j == 0 || S.rs[j] != S.rs[j - 1])) ? j : -1;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, v, d);
          if (lane >= d) v = max(v, y);
        }
        v = max(v, carry);
        if (j < n) S.go[j] = v;  // run start, temporarily
        carry = __shfl_sync(0xffffffffu, v, 31);
      }
      __syncwarp();
      int carry_e = n - 1;
      for (int c0 = ((n - 1) >> 5) << 5; c0 >= 0; c0 -= 32) {
        const int j = c0 + lane;
        int v = (j < n && (j == n - 1 || S.rs[j + 1] != S.rs[j])) ? j : INT32_MAX;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          int y = __shfl_down_sync(0xffffffffu, v, d);
          if (lane + d < 32) v = min(v, y);
        }
        v = min(v, carry_e);
        if (j < n) {
          int run = v - S.go[j] + 1;
          if (run > 65535) run = 65535;
          long long g = (long long)J.gap_open + (run - 1);
          S.go[j] = g > -1 ? -1 : (int32_t)g;
        }
        carry_e = __shfl_sync(0xffffffffu, v, 0);
      }
      __syncwarp();
    }
    const int32_t ge = J.gap_extend;
    const Band B{J.hint, (long long)J.band, n};
    long long r0l = 1 - J.hint - (long long)J.band;
    const int R0 = r0l > 1 ? (int)min(r0l, (long long)m + 1) : 1;
    long long r1l = (long long)n + J.band - J.hint;
    const int R1 = r1l < (long long)m ? (int)max(r1l, 0ll) : m;
    // traceback layout
    const bool band_mode = J.band <= 31;
    const int width = band_mode ? (int)(2 * J.band + 1) : n + 1;
    const int stride_w = (width + 7) >> 3;
    const int nrows = R1 >= R0 ? R1 - R0 + 1 : 0;
    uint32_t* tb = S.tb;
    if ((size_t)nrows * stride_w * 4 > p.tb_smem) {
      tb = tb_glob;
      if (!tb || (size_t)nrows * stride_w * 4 > p.tb_global_per_warp) {
        if (lane == 0) atomicExch(p.err, 2);
        continue;
      }
    }
    // initial row buffer: row 0 of the reference (M = 0, I = D = NEG_INF)
    for (int j = lane; j <= n; j += 32) {
      S.bufM[j] = 0;
      S.bufI[j] = NEG;
      S.bufD[j] = NEG;
    }
    __syncwarp();
    // best endpoint candidates of the final row (held by its lane)
    int bestV = NEG, bestJ = -1, bestS = 0;
    unsigned long long cells = 0;
    for (int s0 = R0; s0 <= R1; s0 += 32) {
      const int i = s0 + lane;
      const bool row_on = i <= R1;
      const int jlo = B.js(s0);
      const int slast = min(s0 + 31, R1);
      const int jhi = B.je(slast);
      const int my_js = row_on ? B.js(i) : 1, my_je = row_on ? B.je(i) : 0;
      // previous row band (row s0-1) for lane 0's reads
      const bool prev_init = (s0 == R0);
      const int pjs = prev_init ? 0 : B.js(s0 - 1), pje = prev_init ? n : B.je(s0 - 1);
      const uint8_t qsym = row_on ? S.qs[i - 1] : 0;
      const int32_t mmp = row_on ? __ldg(&p.tab->mmpen[S.qq[i - 1]]) : 0;
      int32_t lM = NEG, lD = NEG;                 // left (own previous output)
      int32_t uM = NEG, uI = NEG, uD = NEG;       // up (row above, same column)
      int32_t dM = NEG, dI = NEG, dD = NEG;       // diagonal
      if (lane == 0) {
        int jd = jlo - 1;
        if (jd >= pjs && jd <= pje) { dM = S.bufM[jd]; dI = S.bufI[jd]; dD = S.bufD[jd]; }
        if (jlo >= pjs && jlo <= pje) { uM = S.bufM[jlo]; uI = S.bufI[jlo]; uD = S.bufD[jlo]; }
      }
      uint32_t acc = 0;
      int acc_word = -1;
      const int T = jhi - jlo + 32;
      const int rowbase = (i - R0) * stride_w;
      for (int t = 0; t < T; t++) {
        const int j = jlo + t - lane;
        const bool on = row_on && j >= my_js && j <= my_je;
        int32_t oM = NEG, oI = NEG, oD = NEG;
        if (on) {
          const uint8_t rsym = S.rs[j - 1];
          const int32_t go = S.go[j - 1];
          const int32_t sc = qsym == rsym ? 20 : mmp;  // MATCH_SCORE (smith_waterman.rs:81)
          const int32_t fm = dM + sc, fi = dI + sc, fd = dD + sc;
          const int32_t Mv = max(max(fm, fi), fd);
          const uint32_t tm = Mv == fm ? 0u : (Mv == fi ? 1u : 2u);
          const int32_t io = uM + go, ie = uI + ge;
          const int32_t Iv = max(io, ie);
          const uint32_t ti = Iv == io ? 0u : 1u;
          const int32_t dop = lM + go, dex = lD + ge;
          const int32_t Dv = max(dop, dex);
          const uint32_t td = Dv == dop ? 0u : 1u;
          oM = Mv; oI = Iv; oD = Dv;
          const uint32_t nib = tm | (ti << 2) | (td << 3);
          const int c = band_mode ? (int)((long long)j - ((long long)i + J.hint - J.band)) : j;
          const int w = c >> 3;
          if (w != acc_word) {
            if (acc_word >= 0) tb[rowbase + acc_word] = acc;
            acc_word = w;
            acc = 0;
          }
          acc |= nib << ((c & 7) * 4);
          cells++;
          if (i == R1) {
            // last-maximum endpoint over (j, M), (j, I) in increasing j
            if (Mv >= bestV) { bestV = Mv; bestJ = j; bestS = 0; }
            if (Iv >= bestV) { bestV = Iv; bestJ = j; bestS = 1; }
          }
          if (lane == 31) { S.bufM[j] = Mv; S.bufI[j] = Iv; S.bufD[j] = Dv; }
        }
        lM = oM;
        lD = oD;
        // shift the row above down the warp
        int32_t nM = __shfl_up_sync(0xffffffffu, oM, 1);
        int32_t nI = __shfl_up_sync(0xffffffffu, oI, 1);
        int32_t nD = __shfl_up_sync(0xffffffffu, oD, 1);
        if (lane == 0) {
          int jn = jlo + t + 1;
          if (jn >= pjs && jn <= pje && jn <= n) { nM = S.bufM[jn]; nI = S.bufI[jn]; nD = S.bufD[jn]; }
          else { nM = NEG; nI = NEG; nD = NEG; }
        }
        dM = uM; dI = uI; dD = uD;
        uM = nM; uI = nI; uD = nD;
      }
      if (acc_word >= 0) tb[rowbase + acc_word] = acc;
      __syncwarp();
    }
    cells_acc += cells;
    // ---- endpoint (smith_waterman.rs:248-251) ----
    int endV, endJ, endS;
    if (R1 < R0) {
      endV = 0; endJ = n; endS = 0;  // no processed row: row 0 has M = 0 everywhere
    } else {
      const int holder = (R1 - R0) & 31;
      endV = __shfl_sync(0xffffffffu, bestV, holder);
      endJ = __shfl_sync(0xffffffffu, bestJ, holder);
      endS = __shfl_sync(0xffffffffu, bestS, holder);
      resolve_endpoint(endV, endJ, endS, B.js(R1), B.je(R1), n);
    }
    // ---- traceback and bookkeeping, lane 0 ----
    if (lane == 0) {
      const uint8_t* rs = S.rs;
      auto tbr = [&](int i, int j) -> uint32_t {
        if (i < R0 || i > R1 || j < B.js(i) || j > B.je(i)) return 0u;
        const int c = band_mode ? (int)((long long)j - ((long long)i + J.hint - J.band)) : j;
        return (tb[(i - R0) * stride_w + (c >> 3)] >> ((c & 7) * 4)) & 15u;
      };
      auto rsym = [&](int j) -> uint8_t { return rs[j]; };
      finish_alignment(m, endV, endJ, endS, S.qs, S.qq, S.ops, tbr, rsym, J.ref_start, p.tab, O, p.cig_pool,
                       p.cig_pool_used, p.cig_pool_cap, p.err);
    }
    __syncwarp();
  }
  for (int d = 16; d >= 1; d >>= 1) {
    cells_acc += __shfl_down_sync(0xffffffffu, cells_acc, d);
    jobs_acc += __shfl_down_sync(0xffffffffu, jobs_acc, d);
  }
  if (lane == 0 && p.counters) {
    atomicAdd(&p.counters[0], jobs_acc / 32);
    atomicAdd(&p.counters[1], cells_acc);
  }
}

void launch_align(const AlignArgs& a, int grid, cudaStream_t st) {
  const int threads = 128;
  size_t sm = align_smem_bytes(a.lmax, a.nmax, a.tb_smem) * (threads / 32);
  cudaFuncSetAttribute(k_align, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_align<<<grid, threads, sm, st>>>(a);
}

}  // namespace pbw
