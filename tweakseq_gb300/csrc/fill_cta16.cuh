// fill_cta16.cuh -- one long pair per CTA in int16x2 lanes with rebased
// values (global or local alignment; score or traceback output).
//
// Rows go in passes of 512.  Lane t of a warp holds rows 512p + 8t .. +7
// (band A, low halves) and 512p + 256 + 8t .. +7 (band B, high halves),
// band B 32 steps behind band A: the cell arithmetic, decision nibbles and
// plane layout of the int16x2 warp fill with 32 lanes per pair
// (fill_i16.cuh).  Pass p runs on warp p mod W, and consecutive passes run
// at the same time, each a few chunks of columns behind the one above.  The
// passes are joined as in the int32 CTA fill (fill_cta.cuh): shared-memory
// rings with flow control both ways between warps w and w+1, a full-width
// row in global memory from warp W-1 back to warp 0, absolute int32 (H, F)
// in both.
//
// Values.  A long pair's scores leave the int16 range; the cells a warp
// holds at one time do not.  |H(i,j) - H(i-1,j)| and |H(i,j) - H(i,j-1)|
// are at most open + ext + max_score (a gap of one costs open + ext, and a
// diagonal step gains at most max_score on top of one), and a warp's live
// cells span at most 512 rows and 64 columns.  So each warp keeps its
// values relative to a base, an int32 shared by its lanes, and at every
// 32nd step moves the base to its lane 0's first row, shifting every live
// value by the difference (entries at minus infinity stay at the floor).
// With open + ext + max_score <= kMaxStep16 the live values stay within
// +-26,000 of the base.  Ring entries are converted to the warp's base as
// lane 0 reads them, and the bottom row back to absolute values as lane 31
// writes it.
//
// Local mode.  H's floor, 0, is -base on a warp's scale (held at the int16
// floor when the base is higher: the live values are then all positive).
// A local maximum may lie far from the current base, so the per-row maxima
// of the last 32 steps are folded into one absolute (score, row, column)
// key per lane at every move of the base, and then start again; the keys of
// all lanes and warps give the pair's maximum, first in row-major order on
// ties, as the other fills do.
//
// Every wait is bounded, as in the int32 CTA fill: a wait that runs out
// marks the pair TSQ_E_TIMEOUT and makes every other wait of the CTA give
// up, so the kernel always finishes.
#pragma once

#include <algorithm>
#include <cstdint>

#include "fill_cta.cuh"
#include "fill_i16.cuh"

namespace tsq {
namespace fill {

// Largest open + ext + max_score the rebased int16x2 lanes take.
constexpr int kMaxStep16 = 40;

// Shared memory of the int16x2 CTA fill with W warps and nclasses score
// classes.
__host__ __device__ constexpr size_t cta16_smem_bytes(int W, int nclasses) {
  return size_t(kMatBytes16) + size_t(2 * nclasses) * W * 32 * sizeof(uint2) +  // class matrix, profile
         size_t(kTopRing) * sizeof(int2) + kRingPad +                           // warp 0's staging ring
         size_t(W) * (kCodeRing16 + kRingPad) +                                 // code rings
         size_t(W - 1) * kCtaRing * sizeof(int2) +                              // inter-warp rings
         cta_ctl_bytes(W);                                                      // counters
}

// Class codes of chunk k for a warp whose top row comes from a ring: three
// 16-byte copies by lanes 0..2, the ring's head mirrored past its end.
__device__ __forceinline__ void stage_codes16(int k, int t, int n, const uint8_t *codes, int64_t boff,
                                              uint8_t *code_ring) {
  const int c0 = kChunk * k;
  if (c0 >= n || t >= 3) return;
  const int64_t a = ((boff + c0) & ~int64_t(15)) + 16 * t;
  cp_async16(code_ring + (a & (kCodeRing16 - 1)), codes + a);
  if ((a & (kCodeRing16 - 1)) == 0) cp_async16(code_ring + kCodeRing16, codes + a);
}

template <int OUT, int W, bool LOCAL>
__global__ void __launch_bounds__(W * 32, 1) fill_cta16_kernel(const FillArgs A) {
  static_assert(OUT == kOutScore || OUT == kOutTrace, "score and traceback output");
  constexpr int G = 32, R = 8, P = G * R, P2 = 2 * P;
  constexpr int kThr = W * 32;
  extern __shared__ __align__(16) uint8_t smem[];
  int8_t *s_mat = reinterpret_cast<int8_t *>(smem);
  uint2 *s_prof = reinterpret_cast<uint2 *>(smem + kMatBytes16);
  uint8_t *p = smem + kMatBytes16 + size_t(2 * A.nclasses) * kThr * sizeof(uint2);
  int2 *stage_ring = reinterpret_cast<int2 *>(p);  // warp 0: staged global row
  p += kTopRing * sizeof(int2) + kRingPad;
  uint8_t *code_rings = p;
  p += W * (kCodeRing16 + kRingPad);
  int2 *rings = reinterpret_cast<int2 *>(p);  // ring w (w = 1..W-1) at rings + (w-1)*kCtaRing
  p += (W - 1) * kCtaRing * sizeof(int2);
  volatile int *prod = reinterpret_cast<volatile int *>(p);  // [W]
  volatile int *cons = prod + W;                              // [W]
  volatile int *fail = cons + W;
  int *s_misc = const_cast<int *>(fail) + 1;  // task index
  uint64_t *s_keys = reinterpret_cast<uint64_t *>(p + cta_keys_offset(W));  // [W] local maxima

  for (int k = threadIdx.x; k < kMatBytes16; k += blockDim.x) {
    const int x = k / kMatRow16, c = k % kMatRow16;
    s_mat[k] = (x < A.nclasses && c < A.nclasses) ? A.cmatrix[x * A.nclasses + c] : int8_t(0);
  }
  // The code rings start as class 0: positions a lane reads before its
  // columns are staged (it is out of range there) index the profile.
  for (int k = threadIdx.x; k < W * (kCodeRing16 + kRingPad); k += blockDim.x) code_rings[k] = 0;
  __syncthreads();

  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, t = lane;
  const int32_t go = A.gap_open, ge = A.gap_extend, oe = go + ge;
  const uint32_t nge2 = pack2(-ge, -ge), noe2 = pack2(-oe, -oe);
  const uint32_t one = A.one;
  const uint32_t neg_oe2 = 0u - ((uint32_t(oe) << 16) | uint32_t(oe));
  const uint32_t minus_one = 0u - one, k1 = one * 0x00010001u;
  const uint32_t m4 = 0u - 4u * one, m8 = 0u - 8u * one;
  const uint32_t k16 = one << 4, k256 = one << 8, k4096 = one << 12;
  (void)minus_one, (void)k1, (void)m4, (void)m8, (void)k16, (void)k256, (void)k4096;
  int2 *grow = reinterpret_cast<int2 *>(A.bnd) + int64_t(blockIdx.x) * A.bnd_cols;  // the wrap-around row
  uint8_t *code_ring = code_rings + w * (kCodeRing16 + kRingPad);
  const uint2 *profA = s_prof + threadIdx.x;        // + (2c) * kThr
  const uint2 *profB = s_prof + kThr + threadIdx.x;  // + (2c) * kThr
  const int src_lane = (t + G - 1) & (G - 1);        // rotate within the warp
  const uint32_t selH = t == 0 ? 0x5410u : 0x7654u;  // (top H, rotated band-A H) or the shuffled word
  const uint32_t selF = t == 0 ? 0x5432u : 0x7654u;
  const int ncls = A.nclasses;
  const int n_tasks = A.n_wtasks;
  const int spin = A.spin_limit > 0 ? A.spin_limit : kSpinLimit;

  for (;;) {
    if (threadIdx.x == 0) s_misc[0] = atomicAdd(A.counter, 1);
    __syncthreads();
    const int task = s_misc[0];
    __syncthreads();
    if (task >= n_tasks) break;
    const int pid = A.tasks[task];
    const PairDev pr = A.pairs[pid];
    const int m = pr.a_len, n = pr.b_len;
    const uint8_t *qa_cls = A.ccodes + pr.a_off;
    const int64_t boff = pr.b_off;
    bool bad = false;
    for (int k = threadIdx.x; k < m; k += blockDim.x) bad |= A.codes[pr.a_off + k] >= kLetters;
    for (int k = threadIdx.x; k < n; k += blockDim.x) bad |= A.codes[boff + k] >= kLetters;
    const bool gbad = __syncthreads_or(bad) != 0;
    const bool trivial = (m == 0 || n == 0 || gbad);
    const int passes = trivial ? 0 : (m + P2 - 1) / P2;
    const int nbands = (m + P - 1) / P;
    uint32_t *planes = nullptr;
    if constexpr (OUT == kOutTrace) planes = reinterpret_cast<uint32_t *>(A.planes + A.plane_off[pid]);
    (void)planes, (void)nbands;
    if (!trivial)
      for (int j = threadIdx.x; j < n; j += blockDim.x) grow[j] = make_int2(edge_h(j + 1, go, ge, LOCAL), kNegInf);
    if (threadIdx.x < W) {
      prod[threadIdx.x] = 0;
      cons[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) *fail = 0;
    __syncthreads();

    int32_t last_h = 0;
    uint64_t lkey = 0;  // local: this lane's maximum so far, as (score, -row, -column)
    const int2 *ring_in = w > 0 ? rings + (w - 1) * kCtaRing : nullptr;  // written by warp w-1
    int2 *ring_out = w < W - 1 ? rings + w * kCtaRing : nullptr;         // read by warp w+1

    for (int pass = w; pass < passes; pass += W) {
      const int i = pass / W;  // this warp's i-th pass
      const int base = i * n;  // cumulative column position of the pass in its rings
      // The last pass's bottom row has no reader.
      int2 *const out_ring = pass + 1 < passes ? ring_out : nullptr;
      const int rowA = pass * P2 + t * R;  // band A rows rowA+1 .. rowA+R (1-based)
      const int rowB = rowA + P;           // band B rows rowB+1 .. rowB+R
      // Profile of this lane's 16 rows, as in the int16x2 warp fill.
      {
        int xa[R], xb[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          xa[r] = kMatRow16 * (rowA + r < m ? int(qa_cls[rowA + r]) : ncls);
          xb[r] = kMatRow16 * (rowB + r < m ? int(qa_cls[rowB + r]) : ncls);
        }
#pragma unroll 1
        for (int cb = 0; cb < ncls; cb += 4) {
          uint32_t a[R], b[R];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            a[r] = *reinterpret_cast<const uint32_t *>(s_mat + xa[r] + cb);
            b[r] = *reinterpret_cast<const uint32_t *>(s_mat + xb[r] + cb);
          }
          uint32_t a0[4], a1[4], b0[4], b1[4];
          transpose4x4(a[0], a[1], a[2], a[3], a0);
          transpose4x4(a[4], a[5], a[6], a[7], a1);
          transpose4x4(b[0], b[1], b[2], b[3], b0);
          transpose4x4(b[4], b[5], b[6], b[7], b1);
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int c = cb + k;
            if (c < ncls) {
              s_prof[(2 * c) * kThr + threadIdx.x] = make_uint2(a0[k], a1[k]);
              s_prof[(2 * c + 1) * kThr + threadIdx.x] = make_uint2(b0[k], b1[k]);
            }
          }
        }
      }

      // The warp's values are relative to bw (absolute); it starts at the
      // pass's top-left cell H(512p, 0).
      int32_t bw = edge_h(pass * P2, go, ge, LOCAL);
      // Local: H's floor 0, and 0 - open - ext, on the warp's scale.
      uint32_t zero2 = 0u, zero_oe2 = 0u;
      auto set_zero = [&]() {
        const uint32_t z = uint32_t(max(-bw, kNeg16) + kBias16), zo = uint32_t(max(-bw - oe, kNeg16) + kBias16);
        zero2 = (z << 16) | z;
        zero_oe2 = (zo << 16) | zo;
      };
      if constexpr (LOCAL) set_zero();
      uint32_t H[R], E[R], T[R];
      uint32_t best[R], bstep[R];  // local: per row, the best H of this window and its step (offset in the window)
      (void)best, (void)bstep;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        H[r] = pack2b(edge_h(rowA + r + 1, go, ge, LOCAL) - bw, edge_h(rowB + r + 1, go, ge, LOCAL) - bw);
        T[r] = __viaddmax_u16x2(H[r], noe2, kNeg2);
        E[r] = kNeg2;
        if constexpr (LOCAL) {
          best[r] = zero2;
          bstep[r] = 0u;
        }
      }
      uint32_t hdiag = pack2b(edge_h(rowA, go, ge, LOCAL) - bw, edge_h(rowB, go, ge, LOCAL) - bw);
      int sw = 0;  // local: first step of the current window
      // Local: folds the window's row maxima (above 0, in rows of a) into
      // the lane's key; columns from the step, 1-based.
      auto fold = [&]() {
        if constexpr (LOCAL) {
#pragma unroll
          for (int half = 0; half < 2; ++half) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const int row = (half ? rowB : rowA) + r;  // 0-based
              const int32_t v = (half ? hi16b(best[r]) : lo16b(best[r])) + bw;
              const int32_t col = sw + int32_t(half ? bstep[r] >> 16 : bstep[r] & 0xFFFFu) - t - (half ? G : 0) + 1;
              if (row < m && v > 0) {
                const uint64_t key = (uint64_t(uint32_t(v)) << 40) | (uint64_t(0xFFFFFu - uint32_t(row + 1)) << 20) |
                                     uint64_t(0xFFFFFu - uint32_t(col));
                lkey = key > lkey ? key : lkey;
              }
            }
          }
        }
      };
      uint32_t outH = kBias2, outF = kNeg2;
      const int nS = n + G - 1;
      const int64_t wordA = ((int64_t)(2 * pass) * nS) * G + t;
      const int64_t wordB = ((int64_t)(2 * pass + 1) * nS - G) * G + t;
      const bool hasB = 2 * pass + 1 < nbands;
      (void)wordA, (void)wordB, (void)hasB;

      // Codes (and, for warp 0, the global row's entries) of chunk c.
      auto stage = [&](int chunk) {
        if (w == 0) {
          if (pass > 0) cta_wait_geq(&prod[0], (i - 1) * n + min(kChunk * (chunk + 1), n), fail, spin);
          stage_chunk_rt<int2, kCodeRing16>(G, chunk, t, n, grow, stage_ring, A.ccodes, boff, code_ring);
        } else {
          stage_codes16(chunk, t, n, A.ccodes, boff, code_ring);
        }
      };
      cp_async_wait_all();
      __syncwarp();
      stage(0);
      if (w > 0) cta_wait_geq(&prod[w], base + min(kChunk + 1, n), fail, spin);
      cp_async_commit();
      cp_async_wait_all();
      __syncwarp();
      stage(1);
      cp_async_commit();
      // Producer side: room for the first chunk of this pass's bottom row.
      if (out_ring) cta_wait_geq(&cons[w + 1], base + kChunk - kCtaRing, fail, spin);

      // Top entry of column col (absolute (H, F)) as a packed word on the
      // warp's base: biased H low, biased F high; F may be minus infinity.
      auto top_word = [&](int col) -> uint32_t {
        const int2 v = w == 0 ? stage_ring[col & (kTopRing - 1)] : ring_in[(base + col) % kCtaRing];
        const uint32_t h = uint32_t(v.x - bw + kBias16);
        const uint32_t f = uint32_t(max(v.y - bw, kNeg16) + kBias16);
        return imad(f, 0x10000u * one, h);
      };

      uint2 pa[2], pb[2];
      uint32_t tv[2];
      {
        const int ca = code_ring[(boff - t) & (kCodeRing16 - 1)];
        const int cbb = code_ring[(boff - t - G) & (kCodeRing16 - 1)];
        pa[0] = profA[(2 * ca) * kThr];
        pb[0] = profB[(2 * cbb) * kThr];
        tv[0] = top_word(0);
      }
      const int max_steps = n + 2 * G - 1;
      const int steps_pad = (max_steps + 1) & ~1;
      const int i0 = min(2 * G, steps_pad);
      const int i1 = max(i0, n & ~3);
      const int cA0 = int(boff & (kCodeRing16 - 1)) - t + 1 + kCodeRing16;  // code of column jA + 1, positive
      const int cB0 = cA0 - G;                                               // code of column jB + 1

      auto step = [&](const int s, auto k_tag, auto interior_tag, auto last_tag, const uint8_t *codeA,
                      const uint8_t *codeB) {
        constexpr int k = decltype(k_tag)::value;
        constexpr int cur = k & 1, nxt = cur ^ 1;
        constexpr bool INTERIOR = decltype(interior_tag)::value;
        // Chunk boundaries fall on the last step of a unit only.
        if (decltype(last_tag)::value && ((s + 1) & (kChunk - 1)) == 0) {
          // Producer: publish the columns lane 31's band B finished, then
          // wait for room for the chunk it starts.
          const int done = min(max(s - (2 * G - 1), 0), n);
          if (lane == G - 1) {
            __threadfence_block();
            if (w == W - 1)
              prod[0] = base + done;
            else
              prod[w + 1] = base + done;
          }
          if (out_ring && done < n) cta_wait_geq(&cons[w + 1], base + done + kChunk - kCtaRing, fail, spin);
          // Consumer: the next chunk must be there before lane 0 reads its
          // first column; report what was read.
          cp_async_wait_all();
          __syncwarp();
          stage((s + 1) / kChunk + 1);
          if (w > 0) {
            if (lane == 0) {
              __threadfence_block();  // the entries read so far are in registers
              cons[w] = base + min(s + 2, n);
            }
            cta_wait_geq(&prod[w], base + min(s + 1 + kChunk + 1, n), fail, spin);
          }
          cp_async_commit();
          // Rebase: lane 0's first row (band A) becomes 0.  Values move by
          // -delta; entries at the floor stay there.
          // (-delta in both halves as one 32-bit addend: for delta > 0 a
          // subtraction that never borrows, every half being at least
          // floor + delta after the max; for delta <= 0 an addition that
          // never carries, the live values being far below the top.)
          fold();
          const int32_t delta = __shfl_sync(0xffffffffu, lo16b(H[0]), 0);
          const uint32_t nd2 = uint32_t(-delta) * 0x10001u;
          const uint32_t lift = uint32_t(kNeg16 + kBias16 + max(delta, 0));
          const uint32_t lift2 = (lift << 16) | lift;
          auto shift = [&](uint32_t x) { return imad(__vimax3_u16x2(x, lift2, lift2), one, nd2); };
#pragma unroll
          for (int r = 0; r < R; ++r) {
            H[r] = shift(H[r]);
            E[r] = shift(E[r]);
            T[r] = shift(T[r]);
          }
          hdiag = shift(hdiag);
          outH = shift(outH);
          outF = shift(outF);
          tv[cur] = shift(tv[cur]);
          bw += delta;
          if constexpr (LOCAL) {
            set_zero();
#pragma unroll
            for (int r = 0; r < R; ++r) {
              best[r] = zero2;
              bstep[r] = 0u;
            }
            sw = s;
          }
        }
        const uint32_t rH = __shfl_sync(0xffffffffu, outH, src_lane);
        const uint32_t rF = __shfl_sync(0xffffffffu, outF, src_lane);
        const int jA = s - t, jB = jA - G;
        const uint2 wa = pa[cur], wb = pb[cur];
        {
          const int ca = codeA[k];
          const int cbb = codeB[k];
          pa[nxt] = profA[(2 * ca) * kThr];
          pb[nxt] = profB[(2 * cbb) * kThr];
        }
        const uint32_t upH = prmt(tv[cur], rH, selH);
        const uint32_t upF = prmt(tv[cur], rF, selF);
        // Lane 0's next top entry (column s + 1); every lane reads the same
        // address.
        if (s + 1 < n) tv[nxt] = top_word(s + 1);
        const bool vA = INTERIOR || (unsigned)jA < (unsigned)n;
        const bool vB = INTERIOR || (unsigned)jB < (unsigned)n;
        if (vA || vB) {
          uint32_t d = hdiag;
          const uint32_t xo0 = INTERIOR ? sub2_imad(upH, one, neg_oe2) : __viaddmax_u16x2(upH, noe2, kNeg2);
          uint32_t fv = __viaddmax_u16x2(upF, nge2, xo0);
          uint32_t xo = 0u;
          uint32_t acc1 = 0xCCCCCCCCu, acc2 = 0xCCCCCCCCu;
          uint32_t nz1 = 0u, nz2w = 0u;  // local: rows whose H is above 0
          (void)acc1, (void)acc2, (void)nz1, (void)nz2w;
          const uint32_t step2 = uint32_t(s - sw) * 0x10001u;  // local: the step in both halves
          (void)step2;
          auto sweep = [&](auto masked_tag, uint32_t keep) {
            constexpr bool MASKED = decltype(masked_tag)::value;
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const uint32_t sc = score2_dyn(r < 4 ? wa.x : wa.y, r < 4 ? wb.x : wb.y, r);
              uint32_t e = __viaddmax_u16x2(E[r], nge2, T[r]);
              uint32_t x, dd = 0u;
              (void)dd;
              if constexpr (OUT == kOutScore) {
                x = __viaddmax_u16x2(d, sc, e);
              } else {
                dd = __viaddmax_u16x2(d, sc, 0u);  // D + s per half
                x = __vimax3_u16x2(dd, e, e);
              }
              const uint32_t fo = r == 0 ? xo0 : xo;  // F's open candidate
              const uint32_t f = r == 0 ? fv : __viaddmax_u16x2(fv, nge2, xo);
              uint32_t h = LOCAL ? __vimax3_u16x2(x, f, zero2) : __vimax3_u16x2(x, f, f);
              uint32_t tn = sub2_imad(h, one, neg_oe2);
              xo = LOCAL ? __viaddmax_u16x2(x, noe2, zero_oe2) : sub2_imad(x, one, neg_oe2);
              (void)fo;
              if constexpr (OUT == kOutTrace) {
                // dir = [h > dd] + [h > x]; bits 2 and 3 clear when E / F
                // extended.
                uint32_t c = imad(nz2(h, x, minus_one, k1), one, nz2(h, dd, minus_one, k1));
                c = imad(nz2(e, T[r], minus_one, k1), m4, c);
                c = imad(nz2(f, fo, minus_one, k1), m8, c);
                const uint32_t wgt = (r & 3) == 0 ? one : (r & 3) == 1 ? k16 : (r & 3) == 2 ? k256 : k4096;
                if (r < 4)
                  acc1 = imad(c, wgt, acc1);
                else
                  acc2 = imad(c, wgt, acc2);
                if constexpr (LOCAL) {
                  const uint32_t z = nz2(h, zero2, minus_one, k1);
                  if (r < 4)
                    nz1 = imad(z, wgt, nz1);
                  else
                    nz2w = imad(z, wgt, nz2w);
                }
              }
              if constexpr (MASKED) {
                h = (h & ~keep) | (H[r] & keep);
                tn = (tn & ~keep) | (T[r] & keep);
                e = (e & ~keep) | (E[r] & keep);
              }
              if constexpr (LOCAL) {
                // Halves where this cell beats the row's best of the window
                // (strictly: the first column of a maximum is kept); a half
                // outside its column range keeps an old value and records
                // nothing.
                const uint32_t nb = __vimax3_u16x2(best[r], h, h);
                uint32_t cm = imad(nz2(nb, best[r], minus_one, k1), 0xFFFFu * one, 0u);
                if constexpr (MASKED) cm &= ~keep;
                best[r] = (nb & cm) | (best[r] & ~cm);
                bstep[r] = (bstep[r] & ~cm) | (step2 & cm);
              }
              d = H[r];
              H[r] = h;
              T[r] = tn;
              E[r] = e;
              fv = f;
            }
          };
          if (INTERIOR || (OUT == kOutScore && vA && vB)) {
            hdiag = upH;
            sweep(BoolTag<false>{}, 0u);
          } else {
            // Halves outside their column range keep their old values; a
            // half that has not started keeps its left-boundary diagonal.
            const uint32_t keep = (vA ? 0u : 0x0000FFFFu) | (vB ? 0u : 0xFFFF0000u);
            hdiag = (upH & ~keep) | (hdiag & keep);
            sweep(BoolTag<true>{}, keep);
          }
          outH = H[R - 1];
          outF = fv;
          if (t == G - 1 && vB) {
            // Band B's bottom row, absolute, for the next pass.
            const int2 v = make_int2(hi16b(outH) + bw, hi16b(outF) + bw);
            if (w == W - 1)
              grow[jB] = v;
            else if (out_ring)
              out_ring[(base + jB) % kCtaRing] = v;
          }
          if constexpr (OUT == kOutTrace) {
            if constexpr (LOCAL) {
              // A local stop (H = 0) has direction 3.
              acc1 |= (0x11111111u - nz1) * 3u;
              acc2 |= (0x11111111u - nz2w) * 3u;
            }
            if (vA) planes[wordA + (int64_t)s * G] = prmt(acc1, acc2, 0x5410u);
            if (vB && hasB) planes[wordB + (int64_t)s * G] = prmt(acc1, acc2, 0x7632u);
          }
        }
      };
      int s0 = 0;
      auto pair_of_steps = [&]() {
        const uint8_t *codeA = code_ring + ((cA0 + s0) & (kCodeRing16 - 1));
        const uint8_t *codeB = code_ring + ((cB0 + s0) & (kCodeRing16 - 1));
        step(s0, IntTag<0>{}, BoolTag<false>{}, BoolTag<false>{}, codeA, codeB);
        step(s0 + 1, IntTag<1>{}, BoolTag<false>{}, BoolTag<true>{}, codeA, codeB);
      };
      auto quad_of_steps = [&]() {
        const uint8_t *codeA = code_ring + ((cA0 + s0) & (kCodeRing16 - 1));
        const uint8_t *codeB = code_ring + ((cB0 + s0) & (kCodeRing16 - 1));
        step(s0, IntTag<0>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB);
        step(s0 + 1, IntTag<1>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB);
        step(s0 + 2, IntTag<2>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB);
        step(s0 + 3, IntTag<3>{}, BoolTag<true>{}, BoolTag<true>{}, codeA, codeB);
      };
      if constexpr (OUT == kOutScore) {
        for (; s0 < i0; s0 += 2) pair_of_steps();
        for (; s0 < i1; s0 += 4) quad_of_steps();
        for (; s0 < steps_pad; s0 += 2) pair_of_steps();
      } else {
        // Traceback: units of two steps in the interior too (code size).
        auto pair_interior = [&]() {
          const uint8_t *codeA = code_ring + ((cA0 + s0) & (kCodeRing16 - 1));
          const uint8_t *codeB = code_ring + ((cB0 + s0) & (kCodeRing16 - 1));
          step(s0, IntTag<0>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB);
          step(s0 + 1, IntTag<1>{}, BoolTag<true>{}, BoolTag<true>{}, codeA, codeB);
        };
#pragma unroll 1
        for (; s0 < i0; s0 += 2) pair_of_steps();
#pragma unroll 1
        for (; s0 < i1; s0 += 2) pair_interior();
#pragma unroll 1
        for (; s0 < steps_pad; s0 += 2) pair_of_steps();
      }
      cp_async_wait_all();
      __syncwarp();
      // The whole bottom row is out; everything of the input ring was read.
      if (lane == G - 1) {
        __threadfence_block();
        if (w == W - 1)
          prod[0] = base + n;
        else
          prod[w + 1] = base + n;
      }
      if (lane == 0 && w > 0) {
        __threadfence_block();
        cons[w] = base + n;
      }
      fold();
      if (!LOCAL && pass == passes - 1) {
        const int wr = (m - 1) - pass * P2;  // row m within this pass
        const int half = wr >= P ? 1 : 0;
        const int lr = (wr - half * P) - t * R;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (r == lr) last_h = (half ? hi16b(H[r]) : lo16b(H[r])) + bw;
      }
    }

    // ---- result (every warp has finished its passes) --------------------
    __syncthreads();
    if constexpr (LOCAL) {
      const uint64_t wkey = group_max<32>(lkey);
      if (lane == 0) s_keys[w] = wkey;
      __syncthreads();
      if (threadIdx.x == 0) {
        uint64_t gkey = 0;
        for (int q = 0; q < W; ++q) gkey = s_keys[q] > gkey ? s_keys[q] : gkey;
        ResultDev &o = A.res[pid];
        o.status = gbad ? TSQ_E_INVALID_RESIDUE : (*fail ? TSQ_E_TIMEOUT : TSQ_OK);
        const int32_t sc = int32_t(gkey >> 40);
        o.score = sc;
        o.a_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t((gkey >> 20) & 0xFFFFFu)) : 0;
        o.b_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t(gkey & 0xFFFFFu)) : 0;
        o.a_begin = o.b_begin = sc > 0 ? -1 : 0;
        o.n_ident = o.n_cols = -1;
      }
      __syncthreads();
      continue;
    }
    const int last_w = passes > 0 ? (passes - 1) % W : 0;
    const int wr = m > 0 ? (m - 1) % P2 : 0;
    const int owner_t = (wr % P) / R;
    if (w == last_w && lane == owner_t) {
      ResultDev &o = A.res[pid];
      o.status = gbad ? TSQ_E_INVALID_RESIDUE : (*fail ? TSQ_E_TIMEOUT : TSQ_OK);
      o.a_begin = 0;
      o.a_end = m;
      o.b_begin = 0;
      o.b_end = n;
      o.score = (m == 0 || n == 0) ? ((m + n == 0) ? 0 : -(go + (m + n) * ge)) : last_h;
      o.n_ident = OUT == kOutScore ? -1 : (m == 0 || n == 0 ? 0 : -1);
      o.n_cols = OUT == kOutScore ? -1 : (m == 0 || n == 0 ? m + n : -1);
    }
    __syncthreads();
  }
}

}  // namespace fill
}  // namespace tsq
