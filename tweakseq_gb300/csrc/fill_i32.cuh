// fill_i32.cuh -- group-striped Gotoh fill in int32 (score, identity or
// traceback planes; global or local).
//
// Recurrences (Gotoh 1982, with the tie-breaks the CPU oracle fixes):
//   E(i,j) = max(E(i,j-1) - ext, H(i,j-1) - open - ext)   open wins ties
//   F(i,j) = max(F(i-1,j) - ext, H(i-1,j) - open - ext)   open wins ties
//   H(i,j) = max(H(i-1,j-1) + s, E, F [, 0])              diag > E > F
//
// Work split.  A group of G consecutive lanes of a warp owns one pair.  The
// rows (residues of a) are cut into bands of G*R rows; lane t of the group
// holds rows t*R .. t*R+R-1 of the band in registers and sweeps the columns
// (residues of b) one per step, lagging lane t-1 by one step.  So at step s
// the group works on the anti-diagonal s of the band: lane t computes column
// s - t.  The bottom row of lane t (H and F) reaches lane t+1 by a warp
// shuffle; the bottom row of the band (lane G-1) goes to a scratch row in
// HBM and is the top row of the next band, read back by lane 0.
//
// Scores come from a per-lane query profile in shared memory: for each of
// the 26 letters, the R int8 scores of the lane's rows, laid out
// [letter][thread][R bytes] so that the 32 lanes of a warp read one
// conflict-free 8-byte word each whatever letters they look up.
//
// Every group of a warp walks the same number of bands and steps (the
// warp-wide maximum), with per-group masks, so the warp never diverges
// across its shuffles; the planner sorts pairs so that the groups of a warp
// get pairs of nearly equal shape.
#pragma once

#include <cstdint>

#include "tsq_internal.h"

namespace tsq {
namespace fill {

constexpr int kThreads = 256;   // 8 warps per block
constexpr int kMatBytes = 704;  // 26*26 int8 rounded up to a 64-byte multiple

// Sign-extends byte K of w to 32 bits with one PRMT (selector bit 3 of each
// nibble replicates the sign of the chosen byte).
template <int K>
__device__ __forceinline__ int32_t sbyte(uint32_t w) {
  uint32_t d;
  asm("prmt.b32 %0, %1, 0, %2;" : "=r"(d) : "r"(w), "n"(K | ((K | 8) << 4) | ((K | 8) << 8) | ((K | 8) << 12)));
  return int32_t(d);
}

template <int R>
struct ProfWord;
template <>
struct ProfWord<4> {
  using T = uint32_t;
  __device__ static uint32_t word(T v, int k) { return v; }
};
template <>
struct ProfWord<8> {
  using T = uint2;
  __device__ static uint32_t word(T v, int k) { return k == 0 ? v.x : v.y; }
};

// Global-mode boundary value H(i,0) = H(0,i) = -(open + i*ext), H(0,0) = 0.
__device__ __forceinline__ int32_t edge_h(int i, int32_t go, int32_t ge, bool local) {
  return (local || i == 0) ? 0 : -(go + i * ge);
}

// Packed path counts for identity mode: (identical columns << 16) | columns.
constexpr uint32_t kCol = 1u, kIdentCol = 0x10001u;

template <int G>
__device__ __forceinline__ unsigned group_mask(int lane) {
  return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((lane / G) * G));
}

template <int G, typename T>
__device__ __forceinline__ T group_max(T v) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o, G);
    v = w > v ? w : v;
  }
  return v;
}

template <int G, int R, bool LOCAL, int OUT>
__global__ void __launch_bounds__(kThreads) fill_i32_kernel(const FillArgs A) {
  extern __shared__ __align__(16) uint8_t smem[];
  int8_t *s_mat = reinterpret_cast<int8_t *>(smem);
  uint8_t *s_prof = smem + kMatBytes;
  using PW = ProfWord<R>;
  using PT = typename PW::T;

  for (int k = threadIdx.x; k < kLetters * kLetters; k += blockDim.x) s_mat[k] = A.matrix[k];
  __syncthreads();

  constexpr int GPW = 32 / G;  // groups per warp
  constexpr int P = G * R;     // rows per band
  const int lane = threadIdx.x & 31;
  const int t = lane % G;
  const int gw = lane / G;
  const int32_t go = A.gap_open, ge = A.gap_extend, oe = go + ge;
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int slot = warp_id * GPW + gw;
  // Boundary scratch: one row of (H, F[, cH, cF]) per group.  Lane 0 of
  // band k+1 reads column j before lane G-1 of the same band overwrites it:
  // lane G-1's value for column j is computed from data lane 0 derived from
  // that read, G-1 shuffles later, so one row suffices.
  constexpr int BW = OUT == kOutIdent ? 4 : 2;
  int32_t *bnd = A.bnd + (int64_t)slot * BW * A.bnd_cols;
  PT *prof = reinterpret_cast<PT *>(s_prof) + threadIdx.x;  // + c * kThreads

  for (;;) {
    int base_task = 0;
    if (lane == 0) base_task = atomicAdd(A.counter, GPW);
    base_task = __shfl_sync(0xffffffffu, base_task, 0);
    if (base_task >= A.n_tasks) break;
    const int task = base_task + gw;
    const bool have = task < A.n_tasks;
    const int pid = have ? A.tasks[task] : 0;
    PairDev pr;
    if (have) {
      pr = A.pairs[pid];
    } else {
      pr.a_off = pr.b_off = 0;
      pr.a_len = pr.b_len = 0;
    }
    const int m = pr.a_len, n = pr.b_len;
    const uint8_t *qa_codes = A.codes + pr.a_off;
    const uint8_t *qb_codes = A.codes + pr.b_off;
    const bool trivial = (m == 0 || n == 0);
    const int passes = trivial ? 0 : (m + P - 1) / P;
    const int steps = trivial ? 0 : n + G - 1;
    int max_passes = passes, max_steps = steps;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      max_passes = max(max_passes, __shfl_xor_sync(0xffffffffu, max_passes, o));
      max_steps = max(max_steps, __shfl_xor_sync(0xffffffffu, max_steps, o));
    }
    uint8_t *planes = nullptr;
    if constexpr (OUT == kOutTrace) planes = A.planes + (have ? A.plane_off[pid] : 0);

    bool bad = false;
    if (have && trivial) {
      // No DP cells, but every residue is still validated.
      for (int k = t; k < m; k += G) bad |= qa_codes[k] == kBadCode;
      for (int k = t; k < n; k += G) bad |= qb_codes[k] == kBadCode;
    }
    // Local: best cell so far of this lane (value, 1-based row, 1-based col).
    int32_t lbest = 0, lrow = 0, lcol = 0;
    uint32_t lcnt = 0;
    int32_t last_h = 0;
    uint32_t last_c = 0;

    for (int pass = 0; pass < max_passes; ++pass) {
      const bool gact = pass < passes;
      const int row0 = pass * P + t * R;  // rows row0+1 .. row0+R (1-based)
      // Query codes and the lane's profile for this band.
      int qa[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = row0 + r;
        int c = (gact && i < m) ? qa_codes[i] : 0;
        if (gact && i < m && c == kBadCode) bad = true;
        qa[r] = (gact && i < m && c != kBadCode) ? c : -1;
      }
#pragma unroll 2
      for (int c = 0; c < kLetters; ++c) {
        uint32_t w[R / 4];
#pragma unroll
        for (int q = 0; q < R / 4; ++q) {
          uint32_t v = 0;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int a = qa[q * 4 + k];
            const uint32_t sc = a >= 0 ? uint8_t(s_mat[a * kLetters + c]) : 0u;
            v |= sc << (8 * k);
          }
          w[q] = v;
        }
        if constexpr (R == 8)
          prof[c * kThreads] = make_uint2(w[0], w[1]);
        else
          prof[c * kThreads] = w[0];
      }

      int32_t H[R], E[R];
      uint32_t cH[R], cE[R];
      int32_t best[R], bcol[R];
      uint32_t bcnt[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        H[r] = edge_h(row0 + r + 1, go, ge, LOCAL);
        E[r] = kNegInf;
        cH[r] = LOCAL ? 0u : uint32_t(row0 + r + 1);
        cE[r] = 0u;
        best[r] = 0;
        bcol[r] = 0;
        bcnt[r] = 0;
      }
      int32_t hdiag = edge_h(row0, go, ge, LOCAL);
      uint32_t cdiag = LOCAL ? 0u : uint32_t(row0);
      int32_t outH = 0, outF = kNegInf;
      uint32_t outCH = 0, outCF = 0;
      int bc_next = 0;
      {
        const int jj = -t;
        if (gact && jj >= 0 && jj < n) bc_next = qb_codes[jj];
      }

      for (int s = 0; s < max_steps; ++s) {
        int32_t upH = __shfl_up_sync(0xffffffffu, outH, 1, G);
        int32_t upF = __shfl_up_sync(0xffffffffu, outF, 1, G);
        uint32_t upCH = 0, upCF = 0;
        if constexpr (OUT == kOutIdent) {
          upCH = __shfl_up_sync(0xffffffffu, outCH, 1, G);
          upCF = __shfl_up_sync(0xffffffffu, outCF, 1, G);
        }
        const int jj = s - t;
        const bool valid = gact && jj >= 0 && jj < n;
        int bc = bc_next;
        if (gact && jj + 1 >= 0 && jj + 1 < n) bc_next = qb_codes[jj + 1];
        if (valid) {
          if (bc == kBadCode) {
            bad = true;
            bc = 0;
          }
          if (t == 0) {
            if (pass == 0) {
              upH = edge_h(jj + 1, go, ge, LOCAL);
              upF = kNegInf;
              upCH = LOCAL ? 0u : uint32_t(jj + 1);
              upCF = 0u;
            } else {
              upH = bnd[(jj + 1) * BW + 0];
              upF = bnd[(jj + 1) * BW + 1];
              if constexpr (OUT == kOutIdent) {
                upCH = uint32_t(bnd[(jj + 1) * BW + 2]);
                upCF = uint32_t(bnd[(jj + 1) * BW + 3]);
              }
            }
          }
          const PT pw = prof[bc * kThreads];
          int32_t hu = upH, fv = upF, d = hdiag;
          uint32_t chu = upCH, cfv = upCF, cd = cdiag;
          hdiag = upH;
          cdiag = upCH;
          uint32_t tw = 0;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const uint32_t wq = PW::word(pw, r / 4);
            int32_t sc;
            switch (r & 3) {
              case 0: sc = sbyte<0>(wq); break;
              case 1: sc = sbyte<1>(wq); break;
              case 2: sc = sbyte<2>(wq); break;
              default: sc = sbyte<3>(wq); break;
            }
            const int32_t eo = H[r] - oe, ee = E[r] - ge;
            const int32_t fo = hu - oe, fe = fv - ge;
            const int32_t e = max(eo, ee);
            const int32_t f = max(fo, fe);
            const int32_t dd = d + sc;
            int32_t h;
            if constexpr (OUT == kOutScore) {
              h = LOCAL ? __vimax3_s32_relu(dd, e, f) : __vimax3_s32(dd, e, f);
              if constexpr (LOCAL) {
                if (h > best[r]) {
                  best[r] = h;
                  bcol[r] = jj + 1;
                }
              }
            } else {
              const bool eopen = eo >= ee, fopen = fo >= fe;
              int dir = kDirDiag;
              h = dd;
              if (e > h) {
                h = e;
                dir = kDirE;
              }
              if (f > h) {
                h = f;
                dir = kDirF;
              }
              if (LOCAL && h <= 0) {
                h = 0;
                dir = kDirStop;
              }
              if constexpr (OUT == kOutIdent) {
                const uint32_t ce = (eopen ? cH[r] : cE[r]) + kCol;
                const uint32_t cf = (fopen ? chu : cfv) + kCol;
                const uint32_t cdd = cd + (qa[r] == bc ? kIdentCol : kCol);
                uint32_t ch = dir == kDirDiag ? cdd : (dir == kDirE ? ce : cf);
                if (LOCAL && dir == kDirStop) ch = 0u;
                cd = cH[r];
                cH[r] = ch;
                cE[r] = ce;
                chu = ch;
                cfv = cf;
                if constexpr (LOCAL) {
                  if (h > best[r]) {
                    best[r] = h;
                    bcol[r] = jj + 1;
                    bcnt[r] = ch;
                  }
                }
              } else {
                tw |= uint32_t(dir | (eopen ? 4 : 0) | (fopen ? 8 : 0)) << (4 * r);
                if constexpr (LOCAL) {
                  if (h > best[r]) {
                    best[r] = h;
                    bcol[r] = jj + 1;
                  }
                }
              }
            }
            d = H[r];
            H[r] = h;
            E[r] = e;
            hu = h;
            fv = f;
          }
          outH = hu;
          outF = fv;
          outCH = chu;
          outCF = cfv;
          if (t == G - 1) {
            bnd[(jj + 1) * BW + 0] = outH;
            bnd[(jj + 1) * BW + 1] = outF;
            if constexpr (OUT == kOutIdent) {
              bnd[(jj + 1) * BW + 2] = int32_t(outCH);
              bnd[(jj + 1) * BW + 3] = int32_t(outCF);
            }
          }
          if constexpr (OUT == kOutTrace) {
            const int64_t entry = ((int64_t)pass * (n + G - 1) + s) * G + t;
            if constexpr (R == 8)
              reinterpret_cast<uint32_t *>(planes)[entry] = tw;
            else
              reinterpret_cast<uint16_t *>(planes)[entry] = uint16_t(tw);
          }
        }
      }
      __syncwarp();

      if (gact) {
        if constexpr (LOCAL) {
          // Rows of a lane increase with r and with the band, so a strict
          // comparison keeps the first row holding the lane's maximum.
#pragma unroll
          for (int r = 0; r < R; ++r) {
            if (row0 + r < m && best[r] > lbest) {
              lbest = best[r];
              lrow = row0 + r + 1;
              lcol = bcol[r];
              lcnt = bcnt[r];
            }
          }
        } else if (pass == passes - 1) {
          // The lane holding row m keeps H(m, n) (and its counts).
          const int lr = (m - 1) - row0;
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (r == lr) {
              last_h = H[r];
              last_c = cH[r];
            }
        }
      }
    }

    // ---- results ------------------------------------------------------
    const unsigned gm = group_mask<G>(lane);
    const bool gbad = (__ballot_sync(0xffffffffu, bad) & gm) != 0;
    if constexpr (LOCAL) {
      // First cell in row-major order holding the maximum: largest value,
      // then smallest row, then smallest column.
      uint64_t key = (uint64_t(uint32_t(lbest)) << 40) | (uint64_t(0xFFFFFu - uint32_t(lrow)) << 20) |
                     uint64_t(0xFFFFFu - uint32_t(lcol));
      const uint64_t gkey = group_max<G>(key);
      const bool owner = (key == gkey) && lbest > 0;
      // Counts of the winning cell travel with the owner.
      const unsigned own = __ballot_sync(0xffffffffu, owner) & gm;
      const int src = own ? (__ffs(own) - 1) : (gw * G);
      const uint32_t wcnt = __shfl_sync(0xffffffffu, lcnt, src);
      if (have && t == 0) {
        ResultDev &o = A.res[pid];
        o.status = gbad ? TSQ_E_INVALID_RESIDUE : TSQ_OK;
        const int32_t sc = int32_t(gkey >> 40);
        // An empty local alignment (no positive cell) sits at (0, 0).
        o.score = sc;
        o.a_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t((gkey >> 20) & 0xFFFFFu)) : 0;
        o.b_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t(gkey & 0xFFFFFu)) : 0;
        o.a_begin = o.b_begin = sc > 0 ? -1 : 0;
        if (OUT == kOutIdent) {
          o.n_ident = sc > 0 ? int32_t(wcnt >> 16) : 0;
          o.n_cols = sc > 0 ? int32_t(wcnt & 0xFFFFu) : 0;
        } else {
          o.n_ident = o.n_cols = -1;
        }
      }
    } else {
      const int owner_t = trivial ? 0 : ((m - 1) % P) / R;
      const int32_t h = __shfl_sync(0xffffffffu, last_h, gw * G + owner_t);
      const uint32_t c = __shfl_sync(0xffffffffu, last_c, gw * G + owner_t);
      if (have && t == 0) {
        ResultDev &o = A.res[pid];
        o.status = gbad ? TSQ_E_INVALID_RESIDUE : TSQ_OK;
        o.a_begin = 0;
        o.a_end = m;
        o.b_begin = 0;
        o.b_end = n;
        if (trivial) {
          o.score = (m + n == 0) ? 0 : -(go + (m + n) * ge);
          o.n_ident = OUT == kOutScore ? -1 : 0;
          o.n_cols = OUT == kOutScore ? -1 : m + n;
        } else {
          o.score = h;
          if (OUT == kOutIdent) {
            o.n_ident = int32_t(c >> 16);
            o.n_cols = int32_t(c & 0xFFFFu);
          } else {
            o.n_ident = o.n_cols = -1;
          }
        }
      }
    }
    __syncwarp();
  }
}

}  // namespace fill
}  // namespace tsq
