// align_wide.cu -- K3w: the same DP as align.cu for wide bands, i.e. the
// whole-window alignments of mate rescue and shortlist cross-alignment
// (SingleEndMapper::align_at_window, src/mapper/single.rs:220-275, which bands
// the aligner to the full window length) and any band wider than 31.
//
// Orientation is transposed: the warp walks the window in tiles of 32
// columns; lane l owns column j = j0 + l and lags lane l-1 by one row, so at
// step t lane l computes cell (i = R0 + t - l, j). The cell to the left and the
// diagonal arrive from lane l-1 by __shfl_up_sync, the cell above is the
// lane's own previous output, and lane 0 reads the previous tile's last
// column from a shared-memory column buffer. Shared memory therefore grows
// with the read length, not with the window (windows reach thousands of
// columns), and the traceback nibbles go to a per-warp global slab in
// column-major order.
#include "align_finish.cuh"
#include "pbw_common.cuh"
#include "pbw_kernels.h"

namespace pbw {

static __host__ __device__ inline size_t a16(size_t x) { return (x + 15) & ~(size_t)15; }

__host__ __device__ inline size_t wide_smem_bytes(int lmax) {
  return 3 * a16(4 * ((size_t)lmax + 2)) + 2 * a16((size_t)lmax);
}
__host__ __device__ inline size_t wide_tbs(int lmax) { return ((size_t)lmax + 8) / 8; }
size_t wide_slab_bytes(int lmax, int nmax) {
  return a16(4 * (size_t)nmax) + a16(4 * ((size_t)nmax + 1) * wide_tbs(lmax)) + a16((size_t)lmax + nmax + 2);
}

__device__ __forceinline__ uint8_t up_ascii_w(uint8_t b) { return (b >= 'a' && b <= 'z') ? (uint8_t)(b - 32) : b; }
__device__ __forceinline__ uint8_t comp_ascii_w(uint8_t b) {
  switch (b) {
    case 'A': return 'T';
    case 'T': return 'A';
    case 'C': return 'G';
    case 'G': return 'C';
    default: return 'N';
  }
}

struct WBand {
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

__global__ void __launch_bounds__(128) k_align_wide(AlignArgs p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const size_t per_warp = wide_smem_bytes(p.lmax);
  unsigned char* my = smem_raw + per_warp * wib;
  int32_t* colM = (int32_t*)my;
  int32_t* colI = (int32_t*)(my + a16(4 * ((size_t)p.lmax + 2)));
  int32_t* colD = (int32_t*)(my + 2 * a16(4 * ((size_t)p.lmax + 2)));
  uint8_t* qs = my + 3 * a16(4 * ((size_t)p.lmax + 2));
  uint8_t* qq = qs + a16((size_t)p.lmax);
  const unsigned int gwarp = blockIdx.x * (blockDim.x >> 5) + wib;
  unsigned char* slab = p.tb_global + p.tb_global_per_warp * gwarp;
  int32_t* go = (int32_t*)slab;
  uint32_t* tb = (uint32_t*)(slab + a16(4 * (size_t)p.nmax));
  uint8_t* ops = slab + a16(4 * (size_t)p.nmax) + a16(4 * ((size_t)p.nmax + 1) * wide_tbs(p.lmax));
  const int TBS = (int)wide_tbs(p.lmax);
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
    const uint8_t* bases = J.mate ? p.bases2 : p.bases;
    const uint8_t* quals = J.mate ? p.quals2 : p.quals;
    const uint64_t* offs = J.mate ? p.offs2 : p.offs;
    const uint64_t qo = offs[J.read];
    const int m = (int)(offs[J.read + 1] - qo);
    const int n = (int)(J.ref_end - J.ref_start);
    if (n > p.nmax || m > p.lmax) {
      if (lane == 0) {
        atomicExch(p.err, 4);
        O->n_ops = 0;
      }
      continue;
    }
    for (int i = lane; i < m; i += 32) {
      if (p.ref_bytes) {
        qs[i] = bases[qo + i];
        qq[i] = quals[qo + i];
      } else if (!J.rev) {
        qs[i] = up_ascii_w(bases[qo + i]);
        qq[i] = quals[qo + i];
      } else {
        qs[i] = comp_ascii_w(up_ascii_w(bases[qo + m - 1 - i]));
        qq[i] = quals[qo + m - 1 - i];
      }
    }
    const uint64_t gb = p.ref_bytes ? 0 : __ldg(&p.G.cbase[J.contig]) + J.ref_start;
    auto rsym = [&](int j) -> uint8_t {
      if (p.ref_bytes) return p.ref_bytes[J.ref_start + j];
      return (uint8_t)"ACGTN"[gcode(p.G, gb + j)];
    };
    __syncwarp();
    if (m == 0 || n == 0) {
      if (lane == 0) finish_empty(m, J.ref_start, O);
      continue;
    }
    // gap open per column from the window's homopolymer runs (smith_waterman.rs:288-291, 348-363)
    {
      int carry = 0;
      for (int c0 = 0; c0 < n; c0 += 32) {
        const int j = c0 + lane;
        int v = (j < n && (j == 0 || rsym(j) != rsym(j - 1))) ? j : -1;
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
        int v = (j < n && (j == n - 1 || rsym(j + 1) != rsym(j))) ? j : INT32_MAX;
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
    const WBand B{J.hint, (long long)J.band, n};
    long long r0l = 1 - J.hint - (long long)J.band;
    const int R0 = r0l > 1 ? (int)min(r0l, (long long)m + 1) : 1;
    long long r1l = (long long)n + J.band - J.hint;
    const int R1 = r1l < (long long)m ? (int)max(r1l, 0ll) : m;
    // column buffer: column 0; row R0-1 is the initial row (M = 0)
    for (int i = lane; i <= m + 1; i += 32) {
      colM[i] = (i == R0 - 1) ? 0 : NEG;
      colI[i] = NEG;
      colD[i] = NEG;
    }
    __syncwarp();
    unsigned long long bestKey = 0;  // (value + 2^31) << 32 | j << 1 | state; 0 = none
    unsigned long long cells = 0;
    if (R1 >= R0) {
      const int nrows = R1 - R0 + 1;
      for (int j0 = 1; j0 <= n; j0 += 32) {
        const int j = j0 + lane;
        const bool col_on = j <= n;
        const uint8_t rs_j = col_on ? rsym(j - 1) : 0;
        const int32_t go_j = col_on ? go[j - 1] : 0;
        int32_t uM = col_on ? 0 : NEG, uI = NEG;   // cell above (own previous output)
        // left received at the previous step; before the first step that is
        // the initial row (M = 0), the diagonal of row R0 in lane 1
        int32_t rM = col_on ? 0 : NEG, rI = NEG, rD = NEG;
        int32_t qM = NEG, qI = NEG, qD = NEG;      // left of the previous step = diagonal
        uint32_t acc = 0;
        int acc_word = -1;
        uint32_t* tbcol = tb + (size_t)j * TBS;
        const int T = nrows + 31;
        for (int t = 0; t < T; t++) {
          const int i = R0 + t - lane;
          int32_t lM, lD, dM, dI, dD;
          if (lane == 0) {
            const bool ir = i >= R0 && i <= R1;
            lM = ir ? colM[i] : NEG;
            lD = ir ? colD[i] : NEG;
            const int id = i - 1;
            const bool dr = id >= R0 - 1 && id <= R1;
            dM = dr ? colM[id] : NEG;
            dI = dr ? colI[id] : NEG;
            dD = dr ? colD[id] : NEG;
          } else {
            lM = rM;
            lD = rD;
            dM = qM;
            dI = qI;
            dD = qD;
          }
          const bool on = col_on && i >= R0 && i <= R1 && j >= B.js(i) && j <= B.je(i);
          int32_t oM, oI, oD;
          if (on) {
            const uint8_t qsym = qs[i - 1];
            const int32_t sc = qsym == rs_j ? 20 : __ldg(&p.tab->mmpen[qq[i - 1]]);
            const int32_t fm = dM + sc, fi = dI + sc, fd = dD + sc;
            const int32_t Mv = max(max(fm, fi), fd);
            const uint32_t tm = Mv == fm ? 0u : (Mv == fi ? 1u : 2u);
            const int32_t io = uM + go_j, ie = uI + ge;
            const int32_t Iv = max(io, ie);
            const uint32_t ti = Iv == io ? 0u : 1u;
            const int32_t dop = lM + go_j, dex = lD + ge;
            const int32_t Dv = max(dop, dex);
            const uint32_t td = Dv == dop ? 0u : 1u;
            oM = Mv;
            oI = Iv;
            oD = Dv;
            const int rr = i - R0;
            const int w = rr >> 3;
            if (w != acc_word) {
              if (acc_word >= 0) tbcol[acc_word] = acc;
              acc_word = w;
              acc = 0;
            }
            acc |= (tm | (ti << 2) | (td << 3)) << ((rr & 7) * 4);
            cells++;
            if (i == R1) {
              const unsigned long long kM = ((unsigned long long)((long long)Mv + 2147483648LL) << 32) |
                                            ((unsigned long long)j << 1);
              const unsigned long long kI = ((unsigned long long)((long long)Iv + 2147483648LL) << 32) |
                                            ((unsigned long long)j << 1) | 1ull;
              bestKey = max(bestKey, max(kM, kI));
            }
          } else if (i == R0 - 1 && col_on) {
            oM = 0;  // initial row (smith_waterman.rs:174-176)
            oI = NEG;
            oD = NEG;
          } else {
            oM = NEG;
            oI = NEG;
            oD = NEG;
          }
          if (lane == 31 && i >= R0 && i <= R1) {
            colM[i] = oM;
            colI[i] = oI;
            colD[i] = oD;
          }
          uM = oM;
          uI = oI;
          qM = lane == 0 ? NEG : lM;
          qI = lane == 0 ? NEG : rI;
          qD = lane == 0 ? NEG : lD;
          rM = __shfl_up_sync(0xffffffffu, oM, 1);
          rI = __shfl_up_sync(0xffffffffu, oI, 1);
          rD = __shfl_up_sync(0xffffffffu, oD, 1);
        }
        if (acc_word >= 0) tbcol[acc_word] = acc;
        __syncwarp();
      }
    }
    cells_acc += cells;
    for (int d = 16; d >= 1; d >>= 1) bestKey = max(bestKey, __shfl_xor_sync(0xffffffffu, bestKey, d));
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
      resolve_endpoint(endV, endJ, endS, B.js(R1), B.je(R1), n);
    }
    if (lane == 0) {
      auto tbr = [&](int i, int j) -> uint32_t {
        if (i < R0 || i > R1 || j < 1 || j < B.js(i) || j > B.je(i)) return 0u;
        const int rr = i - R0;
        return (tb[(size_t)j * TBS + (rr >> 3)] >> ((rr & 7) * 4)) & 15u;
      };
      finish_alignment(m, endV, endJ, endS, qs, qq, ops, tbr, rsym, J.ref_start, p.tab, O, p.cig_pool,
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

void launch_align_wide(const AlignArgs& a, int grid, cudaStream_t st) {
  const int threads = 128;
  size_t sm = wide_smem_bytes(a.lmax) * (threads / 32);
  cudaFuncSetAttribute(k_align_wide, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_align_wide<<<grid, threads, sm, st>>>(a);
}

}  // namespace pbw
