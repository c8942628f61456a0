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
// HBM and is the top row of the next band, read back by lane 0.  Row 0 of
// the matrix is written into that scratch row before the first band, so
// every band reads its top row the same way.
//
// Latency hiding.  The top row and b's residue codes are staged per group in
// shared-memory rings by cp.async one 32-column chunk ahead; each step reads
// the next step's code, profile word and (lane 0) top entry from shared
// memory, so no global load sits on the step's dependency chain.
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

#include "fill_common.cuh"

namespace tsq {
namespace fill {

// One warp task: the warp's 32/G groups each take one pair (or idle).
// The group rings sit in the block's ring area at the warp's slots; with
// warp_rings set they sit there instead, in a layout private to the warp
// (the top rings of its groups, then their code rings), so that warps of
// one block may run different output modes at once.
template <int G, int R, bool LOCAL, int OUT>
__device__ __forceinline__ void fill_warp_task(const FillArgs &A, const int8_t *s_mat, uint2 *s_prof,
                                               uint8_t *s_rings, int begin, int count, int warp_id,
                                               uint8_t *warp_rings = nullptr) {
  static_assert(R == 8, "the profile word layout assumes 8 rows per lane");
  using Top = typename TopT<OUT>::T;
  constexpr int GPW = 32 / G;  // groups per warp
  constexpr int P = G * R;     // rows per band
  const int lane = threadIdx.x & 31;
  const int t = lane % G;
  const int gw = lane / G;
  const int32_t go = A.gap_open, ge = A.gap_extend, oe = go + ge;
  // One top row per group.  Lane 0 of a band reads column j several steps
  // before lane G-1 of the same band overwrites it, and lane G-1's value is
  // computed from data derived from that read, so one row suffices.
  Top *top = reinterpret_cast<Top *>(A.bnd) + ((int64_t)warp_id * 8 + gw) * A.bnd_cols;
  const uint2 *prof = s_prof + threadIdx.x;  // + c * kThreads
  (void)GPW;
  // This group's staging rings.
  const int gslot = (threadIdx.x >> 5) * 8 + gw;
  constexpr int kTopStride = kTopRing * int(sizeof(Top)) + kRingPad;  // bytes
  Top *top_ring = reinterpret_cast<Top *>(warp_rings ? warp_rings + gw * kTopStride : s_rings + gslot * kTopStride);
  uint8_t *code_ring = warp_rings ? warp_rings + GPW * kTopStride + gw * (kCodeRing + kRingPad)
                                  : s_rings + kSlotsPerBlock * kTopStride + gslot * (kCodeRing + kRingPad);

  {
    const bool have = gw < count;
    const int pid = have ? A.tasks[begin + gw] : 0;
    int m = 0, n = 0;
    const uint8_t *qa_codes = A.codes, *qb_codes = A.codes;
    int64_t boff = 0;
    if (have) {
      const PairDev pr = A.pairs[pid];
      m = pr.a_len;
      n = pr.b_len;
      qa_codes = A.codes + pr.a_off;
      qb_codes = A.codes + pr.b_off;
      boff = pr.b_off;
    }
    // Residues are validated once per pair; a pair with an invalid residue
    // is reported and not filled.
    bool bad = false;
    for (int k = t; k < m; k += G) bad |= qa_codes[k] >= kLetters;
    for (int k = t; k < n; k += G) bad |= qb_codes[k] >= kLetters;
    const unsigned gm = group_mask<G>(lane);
    const bool gbad = (__ballot_sync(0xffffffffu, bad) & gm) != 0;
    const bool trivial = (m == 0 || n == 0 || gbad);
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

    // Row 0 of the matrix becomes the first top row.
    if (!trivial) {
      for (int j = t; j < n; j += G) {
        Top v;
        v.x = edge_h(j + 1, go, ge, LOCAL);
        v.y = kNegInf;
        if constexpr (OUT == kOutIdent) {
          v.z = LOCAL ? 0 : j + 1;
          v.w = 0;
        }
        top[j] = v;
      }
    }
    __syncwarp();

    // Local: best cell so far of this lane (value, 1-based row, 1-based col).
    int32_t lbest = 0, lrow = 0, lcol = 0;
    uint32_t lcnt = 0;
    int32_t last_h = 0;
    uint32_t last_c = 0;

    for (int pass = 0; pass < max_passes; ++pass) {
      const bool gact = pass < passes;
      const int nact = gact ? n : 0;
      const int row0 = pass * P + t * R;  // rows row0+1 .. row0+R (1-based)
      // Query codes and the lane's profile for this band (padding rows: 0).
      int qa[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = row0 + r;
        qa[r] = (gact && i < m) ? int(qa_codes[i]) : -1;
      }
      __syncwarp();
#pragma unroll 2
      for (int c = 0; c < kLetters; ++c) {
        uint32_t w[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          uint32_t v = 0;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int a = qa[q * 4 + k];
            const uint32_t sc = a >= 0 ? uint8_t(s_mat[a * kLetters + c]) : 0u;
            v |= sc << (8 * k);
          }
          w[q] = v;
        }
        s_prof[c * kThreads + threadIdx.x] = make_uint2(w[0], w[1]);
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

      // Stage chunk 0 (and wait for it), then put chunk 1 in flight.
      cp_async_wait_all();
      __syncwarp();
      stage_chunk<G>(0, t, nact, top, top_ring, A.codes, boff, code_ring);
      cp_async_commit();
      cp_async_wait_all();
      __syncwarp();
      stage_chunk<G>(1, t, nact, top, top_ring, A.codes, boff, code_ring);
      cp_async_commit();

      // Double-buffered per-step operands: slot (s & 1) holds what step s
      // uses; step s loads slot ((s + 1) & 1) from the rings.
      int cb[2];
      uint2 pw[2];
      Top tv[2];
      cb[0] = min(int(code_ring[(boff - t) & (kCodeRing - 1)]), kLetters - 1);
      pw[0] = prof[cb[0] * kThreads];
      tv[0] = top_ring[0];

      // Steps run in groups of kAhead (the count padded up; padding steps
      // have every column out of range).  Steps [G, n_min) -- n_min the
      // shortest column count of the warp's groups this band, 0 when one of
      // them is idle -- have every lane in range: no range test there.
      const int steps_pad = (max_steps + kAhead - 1) / kAhead * kAhead;
      int n_min = nact;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) n_min = min(n_min, __shfl_xor_sync(0xffffffffu, n_min, o));
      const int i0 = min(G, steps_pad);
      const int i1 = max(i0, n_min / kAhead * kAhead);
      auto step = [&](const int s, auto k_tag, auto interior_tag) {
        constexpr int k = decltype(k_tag)::value;
        constexpr bool INTERIOR = decltype(interior_tag)::value;
        if (k == kAhead - 1 && ((s + 1) & (kChunk - 1)) == 0) {
          // Last step of a chunk: the next chunk (issued 32 steps ago) must
          // have landed before this step reads its first column.
          cp_async_wait_all();
          __syncwarp();
          stage_chunk<G>((s + 1) / kChunk + 1, t, nact, top, top_ring, A.codes, boff, code_ring);
          cp_async_commit();
        }
        int32_t upH = __shfl_up_sync(0xffffffffu, outH, 1, G);
        int32_t upF = __shfl_up_sync(0xffffffffu, outF, 1, G);
        uint32_t upCH = 0, upCF = 0;
        if constexpr (OUT == kOutIdent) {
          upCH = __shfl_up_sync(0xffffffffu, outCH, 1, G);
          upCF = __shfl_up_sync(0xffffffffu, outCF, 1, G);
        }
        const int jj = s - t;
        const bool valid = INTERIOR || (unsigned)jj < (unsigned)nact;
        const int bc = cb[k & 1];
        const uint2 pcur = pw[k & 1];
        // Operands of the next step.  Codes outside the pair are clamped
        // into the table; those steps are masked anyway.
        cb[(k + 1) & 1] = min(int(code_ring[(boff + jj + 1) & (kCodeRing - 1)]), kLetters - 1);
        pw[(k + 1) & 1] = prof[cb[(k + 1) & 1] * kThreads];
        // Lane 0 takes the staged top row (selects, not a branch); every
        // lane of a group reads lane 0's ring entry (one address per group).
        if (t == 0) {
          upH = tv[k & 1].x;
          upF = tv[k & 1].y;
          if constexpr (OUT == kOutIdent) {
            upCH = uint32_t(tv[k & 1].z);
            upCF = uint32_t(tv[k & 1].w);
          }
        }
        tv[(k + 1) & 1] = top_ring[(s + 1) & (kTopRing - 1)];
        if (valid) {
          int32_t hu = upH, fv = upF, d = hdiag;
          uint32_t chu = upCH, cfv = upCF, cd = cdiag;
          hdiag = upH;
          cdiag = upCH;
          uint32_t tw = 0;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int32_t sc = sbyte_dyn(r < 4 ? pcur.x : pcur.y, r);
            // E and F: opening beats extending on ties (a max that also reports
            // which operand won, max_pred).
            bool eopen, fopen;
            const int32_t e = max_pred(H[r] - oe, E[r] - ge, &eopen);
            const int32_t f = max_pred(hu - oe, fv - ge, &fopen);
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
              // H: diagonal beats E beats F on ties: pde = (diag >= E),
              // pxf = (max(diag, E) >= F).
              bool pde, pxf;
              const int32_t x = max_pred(dd, e, &pde);
              h = max_pred(x, f, &pxf);
              int dir = pxf ? (pde ? int(kDirDiag) : int(kDirE)) : int(kDirF);
              if (LOCAL && h <= 0) {
                h = 0;
                dir = kDirStop;
              }
              if constexpr (OUT == kOutIdent) {
                const uint32_t ce = (eopen ? cH[r] : cE[r]) + kCol;
                const uint32_t cfn = (fopen ? chu : cfv) + kCol;
                const uint32_t cdd = cd + (qa[r] == bc ? kIdentCol : kCol);
                uint32_t ch = pxf ? (pde ? cdd : ce) : cfn;
                if (LOCAL && h <= 0) ch = 0u;
                cd = cH[r];
                cH[r] = ch;
                cE[r] = ce;
                chu = ch;
                cfv = cfn;
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
            Top v;
            v.x = outH;
            v.y = outF;
            if constexpr (OUT == kOutIdent) {
              v.z = int32_t(outCH);
              v.w = int32_t(outCF);
            }
            top[jj] = v;
          }
          if constexpr (OUT == kOutTrace) {
            const int64_t entry = ((int64_t)pass * (n + G - 1) + s) * G + t;
            reinterpret_cast<uint32_t *>(planes)[entry] = tw;
          }
        }
      };
      auto run = [&](int from, int to, auto interior_tag) {
        for (int s0 = from; s0 < to; s0 += kAhead) {
          step(s0, IntTag<0>{}, interior_tag);
          step(s0 + 1, IntTag<1>{}, interior_tag);
          step(s0 + 2, IntTag<2>{}, interior_tag);
          step(s0 + 3, IntTag<3>{}, interior_tag);
        }
      };
      static_assert(kAhead == 4, "the step runs below are unrolled by 4");
      // One copy of each body: the ramp-up and ramp-down segments share the
      // general one.
#pragma unroll 1
      for (int seg = 0; seg < 3; ++seg) {
        if (seg == 1)
          run(i0, i1, BoolTag<true>{});
        else
          run(seg == 0 ? 0 : i1, seg == 0 ? i0 : steps_pad, BoolTag<false>{});
      }
      cp_async_wait_all();
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
    if constexpr (LOCAL) {
      // First cell in row-major order holding the maximum: largest value,
      // then smallest row, then smallest column.
      const uint64_t key = (uint64_t(uint32_t(lbest)) << 40) | (uint64_t(0xFFFFFu - uint32_t(lrow)) << 20) |
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
      const int owner_t = (m > 0) ? ((m - 1) % P) / R : 0;
      const int32_t h = __shfl_sync(0xffffffffu, last_h, gw * G + owner_t);
      const uint32_t c = __shfl_sync(0xffffffffu, last_c, gw * G + owner_t);
      if (have && t == 0) {
        ResultDev &o = A.res[pid];
        o.status = gbad ? TSQ_E_INVALID_RESIDUE : TSQ_OK;
        o.a_begin = 0;
        o.a_end = m;
        o.b_begin = 0;
        o.b_end = n;
        if (m == 0 || n == 0) {
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

// Residency target per SM: 4 blocks (16 warps) for score and traceback
// fills (128 registers); identity fills carry path counts: 3 blocks (12
// warps, 170 registers).
template <int OUT>
struct MinBlocks {
  static constexpr int value = OUT == kOutIdent ? 3 : 4;
};

template <int R, bool LOCAL, int OUT>
__global__ void __launch_bounds__(kThreads, MinBlocks<OUT>::value) fill_i32_kernel(const FillArgs A) {
  extern __shared__ __align__(16) uint8_t smem[];
  int8_t *s_mat = reinterpret_cast<int8_t *>(smem);
  uint2 *s_prof = reinterpret_cast<uint2 *>(smem + kMatBytes);
  uint8_t *s_rings = smem + kMatBytes + kLetters * kThreads * sizeof(uint2);
  for (int k = threadIdx.x; k < kLetters * kLetters; k += blockDim.x) s_mat[k] = A.matrix[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int n_wtasks = A.n_wtasks_dev ? *A.n_wtasks_dev : A.n_wtasks;
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(A.counter, 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= n_wtasks) break;
    const int2 w = A.wtasks[idx];
    const int G = w.y >> 16, count = w.y & 0xFFFF;
    switch (G) {
      case 4: fill_warp_task<4, R, LOCAL, OUT>(A, s_mat, s_prof, s_rings, w.x, count, warp_id); break;
      case 8: fill_warp_task<8, R, LOCAL, OUT>(A, s_mat, s_prof, s_rings, w.x, count, warp_id); break;
      case 16: fill_warp_task<16, R, LOCAL, OUT>(A, s_mat, s_prof, s_rings, w.x, count, warp_id); break;
      default: fill_warp_task<32, R, LOCAL, OUT>(A, s_mat, s_prof, s_rings, w.x, count, warp_id); break;
    }
  }
}

}  // namespace fill
}  // namespace tsq
