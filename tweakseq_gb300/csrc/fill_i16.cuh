// fill_i16.cuh -- group-striped Gotoh fill in packed int16x2 with DPX
// instructions (two cells per instruction): score, traceback planes, or
// identity counts (global).
//
// Same recurrences and work split as the int32 fill (fill_i32.cuh), with two
// row bands per pass packed into the two 16-bit halves of every register:
// lane t holds rows t*R .. t*R+R-1 of band A in the low halves and the same
// rows of band B (the G*R rows below band A) in the high halves.  Band B
// runs G columns behind band A, so at step s lane t computes column s - t of
// band A and column s - t - G of band B.  One rotate-shuffle per value
// carries each lane's bottom row to the next lane; lane 0 gets band A's top
// row from the staged top-row ring and band B's top row from lane G-1's
// band-A bottom row, which is exactly one step old.  Only the bottom row of
// band B goes back to HBM.
//
// Per packed cell the fill issues 7 instructions: the profile PRMT that
// builds the two int16 scores, four DPX add/max forms -- E = max(E - ext,
// T), X = max(D + s, E), F = max(F_above - ext, XO_above), H = max(X, F) --
// and two subtractions, T = H - (open + ext) for the next column's E and
// XO = X - (open + ext) (X clamped at 0 first in local mode) for the next
// row's F.  F can take X instead of H from the row above because open >= 0
// makes the F - open - ext candidate redundant, so rows depend on each other
// through one add-max only.
//
// Biased halves.  Every value v is held as v + 32768 in an unsigned 16-bit
// half, compared with the unsigned DPX forms; the proven range keeps every
// half inside [0, 65535] and every subtrahend below it, so a packed
// subtraction is one plain 32-bit subtraction (no borrow crosses the
// halves).  Those two subtractions are issued as integer multiply-adds,
// which run on the FMA pipe beside the DPX instructions' ALU pipe (the
// kernel is ALU-pipe bound).  Adds of signed amounts (scores, -ext) stay in
// the DPX add-max forms, whose per-half addition is modulo 2^16.
//
// Range.  The planner only sends a pair here when every value of its matrix
// fits int16: H <= max_score * min(m, n) and every H, E, F >= -(3*open +
// (rows + n + 1)*ext + 128), checked on the host against kNeg16.  Pairs
// whose upper bound is not proven run the CHECK variant, which keeps the
// running maximum of H and flags the pair for an exact int32 re-run when it
// comes within max_score of 32767 (an overflow must pass through such a
// value first, since one diagonal step adds at most max_score).
//
// Decisions (traceback and identity fills).  Every decision of the
// recurrences is a zero test of a difference between a maximum and one of
// its operands: E opened iff e - T = 0, F opened iff f - XO = 0, H from the
// diagonal iff h - dd = 0, from E iff h - x = 0 < x - dd.  A DPX maximum is
// taken per half, so each such difference is >= 0 in both halves whatever
// the values (even in halves outside their column range), and one 32-bit
// subtraction computes both without a borrow crossing the halves;
// min(difference, 1) per half is then the decision bit of each cell.  With
// open >= 0 the F decision taken from X instead of H differs from the
// int32 fill's only when open = 0 and F beats X strictly; both then walk
// through the same cells and count the same columns.
//
// Traceback: per row, the nibble dir | E-open << 2 | F-open << 3 (dir =
// [h > dd] + [h > x], or 3 for a local stop) is summed into two words by
// integer multiply-adds (rows 0-3 and 4-7, band A in the low halves, band
// B in the high halves), and two PRMTs give each band's 32-bit plane word.
// The planes have the int32 fill's layout -- band A of pass p is band 2p,
// band B band 2p+1, step index column + lane -- so the walker reads either.
//
// Identity (global): each cell carries two packed counts along its
// optimal path, identical columns I and diagonal columns D (columns =
// m + n - D); E, F and H pick theirs with the decision masks (0xFFFF per
// half) by LOP3 selects, and the diagonal adds the match bit and 1.  The
// profile is indexed by letter (every letter its own class), and a second
// per-thread table holds, for each letter, the rows of the lane it matches.
#pragma once

#include <algorithm>
#include <cstdint>

#include "fill_common.cuh"

namespace tsq {
namespace fill {

// 4 warps per block; shared memory (each thread's profile rows, each
// group's rings) allows 3 blocks per SM, 2 for the identity fill (26-letter
// profile, match table, 16-byte ring entries).  (2-warp blocks, 14 warps per
// SM instead of 12, measured no faster: the ALU pipe is the limit.)  No
// minimum-blocks bound: with one, ptxas gives the score fill 128 registers
// instead of 96.
constexpr int kThreads16 = 128;
constexpr int kSlots16 = kThreads16 / 32 * 8;
constexpr int kCodeRing16 = 256;  // band B reads codes up to 2G columns behind band A
constexpr int32_t kNeg16 = -32000;
constexpr int32_t kBias16 = 32768;
constexpr uint32_t kBias2 = 0x80008000u;  // value 0 in both (biased) halves
constexpr uint32_t kNeg2 = 0x03000300u;   // kNeg16 in both (biased) halves
// The class matrix is staged with one 32-byte row per class, plus a row of
// zeros that padding rows (past the end of a) read, so that a lane's
// profile is built from whole rows (four classes per word).
constexpr int kMatRow16 = 32;
constexpr int kMatBytes16 = (kLetters + 1) * kMatRow16 + 32;  // 896, a 64-byte multiple

// Top-row entry carried from pass to pass: (H, F) of band B's bottom row as
// biased halves; identity fills add the path counts (I, D) of that H and of
// that F.
template <int OUT>
struct Top16 {
  using T = uint32_t;
};
template <>
struct Top16<kOutIdent> {
  using T = uint4;
};

__device__ __forceinline__ uint32_t pack2(int32_t lo, int32_t hi) {
  return (uint32_t(lo) & 0xFFFFu) | (uint32_t(hi) << 16);
}

// Values as biased halves.
__device__ __forceinline__ uint32_t pack2b(int32_t lo, int32_t hi) { return pack2(lo + kBias16, hi + kBias16); }
__device__ __forceinline__ int32_t lo16b(uint32_t v) { return int32_t(v & 0xFFFFu) - kBias16; }
__device__ __forceinline__ int32_t hi16b(uint32_t v) { return int32_t(v >> 16) - kBias16; }

// a - sub2 for biased packed halves (each half of a >= its subtrahend),
// issued as an integer multiply-add by the opaque 1.
__device__ __forceinline__ uint32_t sub2_imad(uint32_t a, uint32_t one, uint32_t neg_sub2) {
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(one), "r"(neg_sub2));
  return d;
}

// a * b + c on the FMA pipe (b an opaque run-time value, so that the
// multiply-add is not turned into shifts and adds on the ALU pipe).
__device__ __forceinline__ uint32_t imad(uint32_t a, uint32_t b, uint32_t c) {
  uint32_t d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

// Decision bits: 1 in each half where the difference hi - lo (>= 0 in
// both halves, so the subtraction never borrows across them) is not zero.
// minus_one is the opaque -1; k1 is 0x00010001.
__device__ __forceinline__ uint32_t nz2(uint32_t hi, uint32_t lo, uint32_t minus_one, uint32_t k1) {
  return __vimin3_u16x2(imad(lo, minus_one, hi), k1, k1);
}

// (sign-extended byte K of a, sign-extended byte K of b) as int16x2.
template <int K>
__device__ __forceinline__ uint32_t score2(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "n"(K | ((K | 8) << 4) | ((4 + K) << 8) | ((12 + K) << 12)));
  return d;
}

__device__ __forceinline__ uint32_t score2_dyn(uint32_t a, uint32_t b, int k) {
  switch (k & 3) {
    case 0: return score2<0>(a, b);
    case 1: return score2<1>(a, b);
    case 2: return score2<2>(a, b);
    default: return score2<3>(a, b);
  }
}

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel) {
  uint32_t d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
  return d;
}

// The (H, F) word of a top-row entry.
__device__ __forceinline__ uint32_t top_hf(uint32_t v) { return v; }
__device__ __forceinline__ uint32_t top_hf(const uint4 &v) { return v.x; }


// 4x4 byte transpose: w[i] holds bytes (x_i0, x_i1, x_i2, x_i3); o[k]
// receives (x_0k, x_1k, x_2k, x_3k).
__device__ __forceinline__ void transpose4x4(const uint32_t w0, const uint32_t w1, const uint32_t w2,
                                             const uint32_t w3, uint32_t o[4]) {
  const uint32_t t0 = prmt(w0, w1, 0x5140u), t1 = prmt(w2, w3, 0x5140u);
  const uint32_t t2 = prmt(w0, w1, 0x7362u), t3 = prmt(w2, w3, 0x7362u);
  o[0] = prmt(t0, t1, 0x5410u);
  o[1] = prmt(t0, t1, 0x7632u);
  o[2] = prmt(t2, t3, 0x5410u);
  o[3] = prmt(t2, t3, 0x7632u);
}

// True when any of the len letter codes at p is invalid (>= kLetters).  The
// lanes of a group read the 16-byte aligned chunks covering the range, four
// loads in flight per lane; bytes of a chunk outside the range are masked
// off.  The codes buffer is padded past its end, so the last chunk is in
// bounds.
__device__ __forceinline__ bool range_has_bad(const uint8_t *p, int len, int t, int G) {
  if (len <= 0) return false;
  const uintptr_t a = reinterpret_cast<uintptr_t>(p);
  const uintptr_t a0 = a & ~uintptr_t(15);
  const int head = int(a - a0);
  const int nch = (head + len + 15) >> 4;
  uint32_t any = 0;
#pragma unroll 4
  for (int c = t; c < nch; c += G) {
    const uint4 w = *reinterpret_cast<const uint4 *>(a0 + 16 * uintptr_t(c));
    const int s = head - 16 * c, e = head + len - 16 * c;  // bytes [s, e) of this chunk are in range
    const uint32_t ww[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int lo = min(max(s - 4 * q, 0), 4), hi = min(max(e - 4 * q, 0), 4);
      const uint32_t mlo = lo >= 4 ? 0u : (0xFFFFFFFFu << (8 * lo));
      const uint32_t mhi = hi >= 4 ? 0xFFFFFFFFu : ((1u << (8 * hi)) - 1u);
      any |= __vcmpgeu4(ww[q], 0x1A1A1A1Au) & mlo & mhi;
    }
  }
  return any != 0;
}

// The lane width G is a run-time value: one code path serves every width,
// which keeps the kernel small enough for the instruction cache.  With
// warp_rings set (one 32-lane group per warp), the group's rings sit there
// -- the top ring, then the code ring -- instead of in the block's ring
// area.
template <bool LOCAL, bool CHECK, int OUT>
__device__ __forceinline__ void fill16_warp_task(const FillArgs &A, const int8_t *s_mat, uint2 *s_prof,
                                                 uint32_t *s_match, uint8_t *s_rings, int begin, int count,
                                                 int warp_id, int G, int lg, uint8_t *warp_rings = nullptr) {
  static_assert(!(OUT == kOutIdent && LOCAL), "the int16x2 identity fill is global only");
  using Top = typename Top16<OUT>::T;
  constexpr int R = 8;
  const int P = G * R;   // rows per band
  const int P2 = 2 * P;  // rows per pass (bands A and B)
  const int lane = threadIdx.x & 31;
  const int t = lane & (G - 1);
  const int gw = lane >> lg;
  const int32_t go = A.gap_open, ge = A.gap_extend, oe = go + ge;
  const uint32_t nge2 = pack2(-ge, -ge), noe2 = pack2(-oe, -oe);
  const uint32_t one = A.one;
  const uint32_t neg_oe2 = 0u - ((uint32_t(oe) << 16) | uint32_t(oe));  // adds -(oe, oe) without borrows
  const uint32_t zero_oe2 = pack2b(-oe, -oe);                          // max(x, 0) - oe floor, local
  // Opaque constants of the decision arithmetic (multipliers of the FMA
  // pipe's multiply-adds).
  const uint32_t minus_one = 0u - one, k1 = one * 0x00010001u;
  const uint32_t m4 = 0u - 4u * one, m8 = 0u - 8u * one;  // traceback: -4, -8
  const uint32_t k16 = one << 4, k256 = one << 8, k4096 = one << 12;
  const uint32_t kffff = one * 0xFFFFu;  // identity: decision bits to half masks
  (void)minus_one, (void)k1, (void)m4, (void)m8, (void)k16, (void)k256, (void)k4096, (void)kffff, (void)s_match;
  Top *top = reinterpret_cast<Top *>(A.bnd) + ((int64_t)warp_id * 8 + gw) * A.bnd_cols;
  const int gslot = (threadIdx.x >> 5) * 8 + gw;
  constexpr int kTopStride = kTopRing * int(sizeof(Top)) + kRingPad;  // bytes
  Top *top_ring = reinterpret_cast<Top *>(warp_rings ? warp_rings : s_rings + gslot * kTopStride);
  uint8_t *code_ring = warp_rings ? warp_rings + kTopStride
                                  : s_rings + kSlots16 * kTopStride + gslot * (kCodeRing16 + kRingPad);
  const uint2 *profA = s_prof + threadIdx.x;                // + (2c) * kThreads16
  const uint2 *profB = s_prof + kThreads16 + threadIdx.x;   // + (2c) * kThreads16
  const int src_lane = (lane & ~(G - 1)) | ((t + G - 1) & (G - 1));  // rotate within the group
  const uint32_t selH = t == 0 ? 0x5410u : 0x7654u;  // (top H, rotated band-A H) or the shuffled word
  const uint32_t selF = t == 0 ? 0x5432u : 0x7654u;

  const bool have = gw < count;
  const int pid = have ? A.tasks[begin + gw] : 0;
  int m = 0, n = 0;
  // Residues as score classes (the profile is indexed by class).
  const int ncls = A.nclasses;
  const uint8_t *qa_codes = A.ccodes;
  int64_t boff = 0;
  if (have) {
    const PairDev pr = A.pairs[pid];
    m = pr.a_len;
    n = pr.b_len;
    qa_codes = A.ccodes + pr.a_off;
    boff = pr.b_off;
  }
  // Invalid residues: their letter codes (class codes of invalid letters
  // are 0, a valid profile index).
  bool bad = false;
  if (have) {
    const uint8_t *la = A.codes + A.pairs[pid].a_off, *lb = A.codes + boff;
    bad = range_has_bad(la, m, t, G) || range_has_bad(lb, n, t, G);
  }
  const unsigned gm = group_mask_rt(lane, G);
  const bool gbad = (__ballot_sync(0xffffffffu, bad) & gm) != 0;
  const bool trivial = (m == 0 || n == 0 || gbad);
  const int passes = trivial ? 0 : (m + P2 - 1) / P2;
  const int steps = trivial ? 0 : n + 2 * G - 1;
  int max_passes = passes, max_steps = steps;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    max_passes = max(max_passes, __shfl_xor_sync(0xffffffffu, max_passes, o));
    max_steps = max(max_steps, __shfl_xor_sync(0xffffffffu, max_steps, o));
  }

  // Row 0 of the matrix becomes the first top row: (H, F) as int16 halves
  // (path counts 0).
  if (!trivial) {
    for (int j = t; j < n; j += G) {
      const uint32_t hf = pack2b(edge_h(j + 1, go, ge, LOCAL), kNeg16);
      if constexpr (OUT == kOutIdent)
        top[j] = make_uint4(hf, 0u, 0u, 0u);
      else
        top[j] = hf;
    }
  }
  __syncwarp();
  // Traceback planes of the pair: band b, step s (column + lane), lane t
  // at word (b * (n + G - 1) + s) * G + t; bands past the last real row
  // have no words.
  uint32_t *planes = nullptr;
  const int nbands = (m + P - 1) / P;
  if constexpr (OUT == kOutTrace) planes = reinterpret_cast<uint32_t *>(A.planes + (have ? A.plane_off[pid] : 0));
  (void)planes, (void)nbands;

  int32_t lbest = 0, lrow = 0, lcol = 0;
  int32_t last_h = 0;
  uint32_t last_i = 0, last_d = 0;  // identity: counts of H(m, n)
  uint32_t hmax = LOCAL ? kBias2 : kNeg2;

  for (int pass = 0; pass < max_passes; ++pass) {
    const bool gact = pass < passes;
    const int nact = gact ? n : 0;
    const int rowA = pass * P2 + t * R;  // band A rows rowA+1 .. rowA+R (1-based)
    const int rowB = rowA + P;           // band B rows rowB+1 .. rowB+R
    // Profile of this lane's 16 rows (padding rows read the zero row and
    // score 0): each row's class row is read four classes per word and the
    // words of four rows are transposed into per-class words.
    {
      int xa[R], xb[R];  // byte offsets of the rows' class rows in s_mat
#pragma unroll
      for (int r = 0; r < R; ++r) {
        xa[r] = kMatRow16 * ((gact && rowA + r < m) ? int(qa_codes[rowA + r]) : ncls);
        xb[r] = kMatRow16 * ((gact && rowB + r < m) ? int(qa_codes[rowB + r]) : ncls);
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
            s_prof[(2 * c) * kThreads16 + threadIdx.x] = make_uint2(a0[k], a1[k]);
            s_prof[(2 * c + 1) * kThreads16 + threadIdx.x] = make_uint2(b0[k], b1[k]);
          }
        }
      }
      if constexpr (OUT == kOutIdent) {
        // Match table: for each letter, bit r (band A) and bit 16 + r
        // (band B) set where row r of the lane holds that letter.  Padding
        // rows (class ncls) match nothing.
        for (int c = 0; c < ncls; ++c) s_match[c * kThreads16 + threadIdx.x] = 0u;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int ca = xa[r] / kMatRow16, cb2 = xb[r] / kMatRow16;
          if (ca < ncls) s_match[ca * kThreads16 + threadIdx.x] |= 1u << r;
          if (cb2 < ncls) s_match[cb2 * kThreads16 + threadIdx.x] |= 1u << (16 + r);
        }
      }
    }

    uint32_t H[R], E[R], T[R];
    uint32_t best[R], bcol[R];
    // Identity: counts (I, D) of H and E per row.
    uint32_t IH[R], DH[R], IE[R], DE[R];
    (void)IH, (void)DH, (void)IE, (void)DE;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      H[r] = pack2b(edge_h(rowA + r + 1, go, ge, LOCAL), edge_h(rowB + r + 1, go, ge, LOCAL));
      T[r] = __viaddmax_u16x2(H[r], noe2, kNeg2);
      E[r] = kNeg2;
      best[r] = kBias2;
      bcol[r] = 0u;
      if constexpr (OUT == kOutIdent) IH[r] = DH[r] = IE[r] = DE[r] = 0u;
    }
    uint32_t hdiag = pack2b(edge_h(rowA, go, ge, LOCAL), edge_h(rowB, go, ge, LOCAL));
    uint32_t outH = kBias2, outF = kNeg2;
    // Identity: counts of the diagonal H and of the bottom row's H and F.
    uint32_t gdI = 0u, gdD = 0u, outIH = 0u, outDH = 0u, outIF = 0u, outDF = 0u;
    (void)gdI, (void)gdD, (void)outIH, (void)outDH, (void)outIF, (void)outDF;
    // Traceback: plane words of this lane at step 0 of bands 2p and 2p+1
    // (band B's step index is s - G); a step adds G words.
    const int nS = n + G - 1;
    const int64_t wordA = ((int64_t)(2 * pass) * nS) * G + t;
    const int64_t wordB = ((int64_t)(2 * pass + 1) * nS - G) * G + t;
    const bool hasB = 2 * pass + 1 < nbands;
    (void)nS, (void)wordA, (void)wordB, (void)hasB;

    cp_async_wait_all();
    __syncwarp();
    stage_chunk_rt<Top, kCodeRing16>(G, 0, t, nact, top, top_ring, A.ccodes, boff, code_ring);
    cp_async_commit();
    cp_async_wait_all();
    __syncwarp();
    stage_chunk_rt<Top, kCodeRing16>(G, 1, t, nact, top, top_ring, A.ccodes, boff, code_ring);
    cp_async_commit();

    uint2 pa[2], pb[2];
    Top tv[2];
    uint32_t ma[2] = {0u, 0u}, mb[2] = {0u, 0u};  // identity: match words of the columns
    (void)ma, (void)mb;
    {
      const int ca = code_ring[(boff - t) & (kCodeRing16 - 1)];
      const int cb = code_ring[(boff - t - G) & (kCodeRing16 - 1)];
      pa[0] = profA[(2 * ca) * kThreads16];
      pb[0] = profB[(2 * cb) * kThreads16];
      if constexpr (OUT == kOutIdent) {
        ma[0] = s_match[ca * kThreads16 + threadIdx.x];
        mb[0] = s_match[cb * kThreads16 + threadIdx.x];
      }
      tv[0] = top_ring[0];
    }

    // Steps run in units of two (the ramps) or four (the interior); an odd
    // count gets one padding step, in which every lane's columns are out of
    // range (s - t >= n + G).  Steps [2G, n_min) -- n_min the shortest
    // column count of the warp's groups this pass, 0 when one of them is
    // idle -- have both halves of every lane in range: they run without
    // range tests or masks, four per unit.
    const int steps_pad = (max_steps + 1) & ~1;
    int n_min = nact;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) n_min = min(n_min, __shfl_xor_sync(0xffffffffu, n_min, o));
    const int i0 = min(2 * G, steps_pad);  // a multiple of 4 whenever the interior is not empty
    const int i1 = max(i0, n_min & ~3);

    // Ring positions of a unit's first step: step k of the unit reads k
    // entries further, into the mirrored head past the ring's end when the
    // unit starts near it (the mirrors hold 16 bytes: 16 codes, 4 top-row
    // entries), so a unit computes its ring addresses once.
    const int cA0 = int(boff & (kCodeRing16 - 1)) - t + 1 + kCodeRing16;  // code of column jA + 1, positive
    const int cB0 = cA0 - G;                                               // code of column jB + 1
    auto step = [&](const int s, auto k_tag, auto interior_tag, auto last_tag, const uint8_t *codeA,
                    const uint8_t *codeB, const Top *topp) {
      constexpr int k = decltype(k_tag)::value;
      constexpr int cur = k & 1, nxt = cur ^ 1;
      constexpr bool INTERIOR = decltype(interior_tag)::value;
      // Chunk boundaries fall on the last step of a unit only (units start
      // on steps that are multiples of their size).
      if (decltype(last_tag)::value && ((s + 1) & (kChunk - 1)) == 0) {
        cp_async_wait_all();
        __syncwarp();
        stage_chunk_rt<Top, kCodeRing16>(G, (s + 1) / kChunk + 1, t, nact, top, top_ring, A.ccodes, boff,
                                              code_ring);
        cp_async_commit();
      }
      const uint32_t rH = __shfl_sync(0xffffffffu, outH, src_lane);
      const uint32_t rF = __shfl_sync(0xffffffffu, outF, src_lane);
      uint32_t rIH = 0u, rDH = 0u, rIF = 0u, rDF = 0u;
      (void)rIH, (void)rDH, (void)rIF, (void)rDF;
      if constexpr (OUT == kOutIdent) {
        rIH = __shfl_sync(0xffffffffu, outIH, src_lane);
        rDH = __shfl_sync(0xffffffffu, outDH, src_lane);
        rIF = __shfl_sync(0xffffffffu, outIF, src_lane);
        rDF = __shfl_sync(0xffffffffu, outDF, src_lane);
      }
      const int jA = s - t, jB = jA - G;
      const uint2 wa = pa[cur], wb = pb[cur];
      uint32_t mw = 0u;  // identity: match bits of this step's columns
      (void)mw;
      if constexpr (OUT == kOutIdent) mw = (ma[cur] & 0x0000FFFFu) | (mb[cur] & 0xFFFF0000u);
      {
        const int ca = codeA[k];
        const int cb = codeB[k];
        pa[nxt] = profA[(2 * ca) * kThreads16];
        pb[nxt] = profB[(2 * cb) * kThreads16];
        if constexpr (OUT == kOutIdent) {
          ma[nxt] = s_match[ca * kThreads16 + threadIdx.x];
          mb[nxt] = s_match[cb * kThreads16 + threadIdx.x];
        }
      }
      // Lane 0: band A from the staged top row, band B from lane G-1's
      // band-A bottom; other lanes take the shuffled values whole.  Lane-
      // dependent PRMT selectors instead of a branch; every lane of a group
      // reads lane 0's ring entry (one broadcast address per group).
      const uint32_t upH = prmt(top_hf(tv[cur]), rH, selH);
      const uint32_t upF = prmt(top_hf(tv[cur]), rF, selF);
      uint32_t upIH = 0u, upDH = 0u, upIF = 0u, upDF = 0u;
      if constexpr (OUT == kOutIdent) {
        // Ring entry: (I, D) of H in .y, of F in .z.
        upIH = prmt(tv[cur].y, rIH, selH);
        upDH = prmt(tv[cur].y, rDH, selF);
        upIF = prmt(tv[cur].z, rIF, selH);
        upDF = prmt(tv[cur].z, rDF, selF);
      }
      tv[nxt] = topp[k];
      const bool vA = INTERIOR || (unsigned)jA < (unsigned)nact;
      const bool vB = INTERIOR || (unsigned)jB < (unsigned)nact;
      if (vA || vB) {
        uint32_t d = hdiag;
        // F of the lane's first row from the row above it: max(F - ext,
        // H - open - ext) with the true H above.
        // (In the interior every upH is a real cell, far above the floor, so
        // the subtraction runs as an IMAD on the FMA pipe.)
        const uint32_t xo0 = INTERIOR ? sub2_imad(upH, one, neg_oe2) : __viaddmax_u16x2(upH, noe2, kNeg2);
        uint32_t fv = __viaddmax_u16x2(upF, nge2, xo0);
        uint32_t xo = 0u;
        // Traceback: the nibbles of rows 0-3 and 4-7 (12 in each nibble
        // stands for both opened; the decisions subtract from it).
        uint32_t acc1 = 0xCCCCCCCCu, acc2 = 0xCCCCCCCCu;
        uint32_t nz1 = 0u, nz2w = 0u;  // local: rows whose H is above 0
        // Identity: counts of the cell above (H and F) and of the diagonal.
        uint32_t ciH = upIH, cdH = upDH, ciF = upIF, cdF = upDF;
        uint32_t gI = gdI, gD = gdD;
        (void)acc1, (void)acc2, (void)nz1, (void)nz2w, (void)ciH, (void)cdH, (void)ciF, (void)cdF, (void)gI, (void)gD;
        // Rows in order.  Since open >= 0, F(i+1,j) = max(F(i,j) - ext,
        // max(X(i,j) [, 0]) - open - ext) with X = max(D + s, E): the only
        // dependence between rows is one add-max on F.
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
            uint32_t h = LOCAL ? __vimax3_u16x2(x, f, kBias2) : __vimax3_u16x2(x, f, f);
            uint32_t tn = sub2_imad(h, one, neg_oe2);
            xo = LOCAL ? __viaddmax_u16x2(x, noe2, zero_oe2) : sub2_imad(x, one, neg_oe2);
            (void)fo;
            if constexpr (OUT == kOutTrace) {
              // dir = [h > dd] + [h > x]; bits 2 and 3 clear when E / F
              // extended.
              uint32_t c = imad(nz2(h, x, minus_one, k1), one, nz2(h, dd, minus_one, k1));
              c = imad(nz2(e, T[r], minus_one, k1), m4, c);
              c = imad(nz2(f, fo, minus_one, k1), m8, c);
              const uint32_t w = (r & 3) == 0 ? one : (r & 3) == 1 ? k16 : (r & 3) == 2 ? k256 : k4096;
              if (r < 4)
                acc1 = imad(c, w, acc1);
              else
                acc2 = imad(c, w, acc2);
              if constexpr (LOCAL) {
                const uint32_t z = nz2(h, kBias2, minus_one, k1);
                if (r < 4)
                  nz1 = imad(z, w, nz1);
                else
                  nz2w = imad(z, w, nz2w);
              }
            }
            if constexpr (OUT == kOutIdent) {
              // Masks (0xFFFF per half): E extended, F extended, X from E,
              // H from F.
              const uint32_t mE = imad(nz2(e, T[r], minus_one, k1), kffff, 0u);
              const uint32_t mF = imad(nz2(f, fo, minus_one, k1), kffff, 0u);
              const uint32_t mX = imad(nz2(x, dd, minus_one, k1), kffff, 0u);
              const uint32_t mH = imad(nz2(h, x, minus_one, k1), kffff, 0u);
              uint32_t ie = (IE[r] & mE) | (IH[r] & ~mE);
              uint32_t de = (DE[r] & mE) | (DH[r] & ~mE);
              const uint32_t iF = (ciF & mF) | (ciH & ~mF);
              const uint32_t dF = (cdF & mF) | (cdH & ~mF);
              // Diagonal: + match bit of row r (bit r, bit 16 + r of mw),
              // + 1 diagonal column in each half.
              const uint32_t id = imad((mw >> r) & 0x00010001u, one, gI);
              const uint32_t dg = imad(k1, one, gD);
              uint32_t ih = (((ie & mX) | (id & ~mX)) & ~mH) | (iF & mH);
              uint32_t dh = (((de & mX) | (dg & ~mX)) & ~mH) | (dF & mH);
              if constexpr (MASKED) {
                ih = (ih & ~keep) | (IH[r] & keep);
                dh = (dh & ~keep) | (DH[r] & keep);
                ie = (ie & ~keep) | (IE[r] & keep);
                de = (de & ~keep) | (DE[r] & keep);
              }
              gI = IH[r];
              gD = DH[r];
              IH[r] = ih;
              DH[r] = dh;
              IE[r] = ie;
              DE[r] = de;
              ciH = ih;
              cdH = dh;
              ciF = iF;
              cdF = dF;
            }
            if constexpr (MASKED) {
              h = (h & ~keep) | (H[r] & keep);
              tn = (tn & ~keep) | (T[r] & keep);
              e = (e & ~keep) | (E[r] & keep);
            }
            if constexpr (CHECK) hmax = __vimax3_u16x2(hmax, h, h);
            if constexpr (LOCAL) {
              if constexpr (OUT == kOutScore) {
                // Halves where this cell beats the row's best so far
                // (strictly, so the first column of a maximum is kept).
                const uint32_t cm = __vcmpgtu2(h, best[r]);
                best[r] = __vimax3_u16x2(best[r], h, h);
                bcol[r] = (bcol[r] & ~cm) | (pack2(jA + 1, jB + 1) & cm);
              } else {
                // The same with the decision arithmetic: the new best
                // differs from the old one exactly where h beat it.
                const uint32_t nb = __vimax3_u16x2(best[r], h, h);
                const uint32_t cm = imad(nz2(nb, best[r], minus_one, k1), kffff, 0u);
                best[r] = nb;
                bcol[r] = (bcol[r] & ~cm) | (pack2(jA + 1, jB + 1) & cm);
              }
            }
            d = H[r];
            H[r] = h;
            T[r] = tn;
            E[r] = e;
            fv = f;
          }
        };
        // (Outside the interior the traceback and identity fills run the
        // masked sweep alone, whose keep mask is 0 when both halves are in
        // range: their sweeps are large, and fewer copies of them keep the
        // kernel within the instruction cache.)
        if (INTERIOR || (OUT == kOutScore && vA && vB)) {
          hdiag = upH;
          if constexpr (OUT == kOutIdent) {
            gdI = upIH;
            gdD = upDH;
          }
          sweep(BoolTag<false>{}, 0u);
        } else {
          // Halves outside their column range keep their old values; a
          // half that has not started keeps its left-boundary diagonal.
          const uint32_t keep = (vA ? 0u : 0x0000FFFFu) | (vB ? 0u : 0xFFFF0000u);
          hdiag = (upH & ~keep) | (hdiag & keep);
          if constexpr (OUT == kOutIdent) {
            gdI = (upIH & ~keep) | (gdI & keep);
            gdD = (upDH & ~keep) | (gdD & keep);
          }
          sweep(BoolTag<true>{}, keep);
        }
        outH = H[R - 1];
        outF = fv;
        if constexpr (OUT == kOutIdent) {
          outIH = IH[R - 1];
          outDH = DH[R - 1];
          outIF = ciF;
          outDF = cdF;
          if (t == G - 1 && vB)
            top[jB] = make_uint4(prmt(outH, outF, 0x7632u), prmt(outIH, outDH, 0x7632u),
                                 prmt(outIF, outDF, 0x7632u), 0u);
        } else {
          if (t == G - 1 && vB) top[jB] = prmt(outH, outF, 0x7632u);
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
      const Top *topp = top_ring + ((s0 + 1) & (kTopRing - 1));
      step(s0, IntTag<0>{}, BoolTag<false>{}, BoolTag<false>{}, codeA, codeB, topp);
      step(s0 + 1, IntTag<1>{}, BoolTag<false>{}, BoolTag<true>{}, codeA, codeB, topp);
    };
    auto quad_of_steps = [&]() {
      const uint8_t *codeA = code_ring + ((cA0 + s0) & (kCodeRing16 - 1));
      const uint8_t *codeB = code_ring + ((cB0 + s0) & (kCodeRing16 - 1));
      const Top *topp = top_ring + ((s0 + 1) & (kTopRing - 1));
      step(s0, IntTag<0>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB, topp);
      step(s0 + 1, IntTag<1>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB, topp);
      step(s0 + 2, IntTag<2>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB, topp);
      step(s0 + 3, IntTag<3>{}, BoolTag<true>{}, BoolTag<true>{}, codeA, codeB, topp);
    };
    if constexpr (OUT == kOutScore) {
      for (; s0 < i0; s0 += 2) pair_of_steps();
      for (; s0 < i1; s0 += 4) quad_of_steps();
      for (; s0 < steps_pad; s0 += 2) pair_of_steps();
    } else {
      // Traceback and identity: units of two steps in the interior too
      // (code size, as above).
      auto pair_interior = [&]() {
        const uint8_t *codeA = code_ring + ((cA0 + s0) & (kCodeRing16 - 1));
        const uint8_t *codeB = code_ring + ((cB0 + s0) & (kCodeRing16 - 1));
        const Top *topp = top_ring + ((s0 + 1) & (kTopRing - 1));
        step(s0, IntTag<0>{}, BoolTag<true>{}, BoolTag<false>{}, codeA, codeB, topp);
        step(s0 + 1, IntTag<1>{}, BoolTag<true>{}, BoolTag<true>{}, codeA, codeB, topp);
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

    if (gact) {
      if constexpr (LOCAL) {
        // Band A rows of this pass precede band B rows; within a band rows
        // increase with r, so strict comparisons keep the first maximum.
#pragma unroll
        for (int half = 0; half < 2; ++half) {
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int row = (half ? rowB : rowA) + r;
            const int32_t v = half ? hi16b(best[r]) : lo16b(best[r]);
            const int32_t c = half ? int32_t(bcol[r] >> 16) : int32_t(bcol[r] & 0xFFFFu);
            if (row < m && v > lbest) {
              lbest = v;
              lrow = row + 1;
              lcol = c;
            }
          }
        }
      } else if (pass == passes - 1) {
        const int w = (m - 1) - pass * P2;  // row m within this pass
        const int half = w >= P ? 1 : 0;
        const int lr = (w - half * P) - t * R;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (r == lr) {
            last_h = half ? hi16b(H[r]) : lo16b(H[r]);
            if constexpr (OUT == kOutIdent) {
              last_i = half ? IH[r] >> 16 : IH[r] & 0xFFFFu;
              last_d = half ? DH[r] >> 16 : DH[r] & 0xFFFFu;
            }
          }
      }
    }
  }

  // ---- results ---------------------------------------------------------
  bool overflow = false;
  if constexpr (CHECK) {
    const int32_t lim = 32767 - A.max_score;
    overflow = lo16b(hmax) > lim || hi16b(hmax) > lim;
  }
  const bool goverflow = (__ballot_sync(0xffffffffu, overflow) & gm) != 0;
  if constexpr (LOCAL) {
    const uint64_t key = (uint64_t(uint32_t(lbest)) << 40) | (uint64_t(0xFFFFFu - uint32_t(lrow)) << 20) |
                         uint64_t(0xFFFFFu - uint32_t(lcol));
    const uint64_t gkey = group_max_rt(key, G);
    if (have && t == 0) {
      ResultDev &o = A.res[pid];
      o.status = gbad ? TSQ_E_INVALID_RESIDUE : TSQ_OK;
      const int32_t sc = int32_t(gkey >> 40);
      o.score = sc;
      o.a_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t((gkey >> 20) & 0xFFFFFu)) : 0;
      o.b_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t(gkey & 0xFFFFFu)) : 0;
      o.a_begin = o.b_begin = sc > 0 ? -1 : 0;
      o.n_ident = o.n_cols = -1;
      if (CHECK) A.overflow[pid] = goverflow ? 1 : 0;
    }
  } else {
    int owner = 0;
    if (m > 0) {
      const int w = (m - 1) % P2;
      owner = (w % P) / R;
    }
    const int32_t h = __shfl_sync(0xffffffffu, last_h, gw * G + owner);
    uint32_t ci = 0u, cd = 0u;
    if constexpr (OUT == kOutIdent) {
      ci = __shfl_sync(0xffffffffu, last_i, gw * G + owner);
      cd = __shfl_sync(0xffffffffu, last_d, gw * G + owner);
    }
    if (have && t == 0) {
      ResultDev &o = A.res[pid];
      o.status = gbad ? TSQ_E_INVALID_RESIDUE : TSQ_OK;
      o.a_begin = 0;
      o.a_end = m;
      o.b_begin = 0;
      o.b_end = n;
      o.score = (m == 0 || n == 0) ? ((m + n == 0) ? 0 : -(go + (m + n) * ge)) : h;
      if (OUT != kOutScore && (m == 0 || n == 0)) {
        o.n_ident = 0;
        o.n_cols = m + n;
      } else if (OUT == kOutIdent) {
        o.n_ident = int32_t(ci);
        o.n_cols = m + n - int32_t(cd);
      } else {
        o.n_ident = o.n_cols = -1;
      }
      if (CHECK) A.overflow[pid] = goverflow ? 1 : 0;
    }
  }
  __syncwarp();
}

// Shared memory of the int16x2 fills: class matrix, per-thread profile
// (two words of 8 rows per class), identity's match table, group rings.
__host__ __device__ constexpr size_t smem16_prof_bytes(int nclasses) {
  return size_t(2 * nclasses) * kThreads16 * sizeof(uint2);
}
__host__ __device__ constexpr size_t smem16_match_bytes(int out_mode, int nclasses) {
  return out_mode == kOutIdent ? size_t(nclasses) * kThreads16 * sizeof(uint32_t) : 0;
}
__host__ __device__ constexpr size_t smem16_top_stride(int out_mode) {
  return size_t(kTopRing) * (out_mode == kOutIdent ? 16 : 4) + kRingPad;
}
// Bytes of one group's private rings (the warp_rings layout).
__host__ __device__ constexpr size_t warp_rings16_bytes(int out_mode) {
  return smem16_top_stride(out_mode) + kCodeRing16 + kRingPad;
}

template <bool LOCAL, bool CHECK, int OUT>
__global__ void __launch_bounds__(kThreads16) fill_i16_kernel(const FillArgs A) {
  extern __shared__ __align__(16) uint8_t smem[];
  // Class scores, one 32-byte row per class, then a zero row (index
  // nclasses) for padding rows.
  int8_t *s_mat = reinterpret_cast<int8_t *>(smem);
  uint2 *s_prof = reinterpret_cast<uint2 *>(smem + kMatBytes16);
  uint32_t *s_match = reinterpret_cast<uint32_t *>(smem + kMatBytes16 + smem16_prof_bytes(A.nclasses));
  uint8_t *s_rings = smem + kMatBytes16 + smem16_prof_bytes(A.nclasses) + smem16_match_bytes(OUT, A.nclasses);
  for (int k = threadIdx.x; k < kMatBytes16; k += blockDim.x) {
    const int x = k / kMatRow16, c = k % kMatRow16;
    s_mat[k] = (x < A.nclasses && c < A.nclasses) ? A.cmatrix[x * A.nclasses + c] : int8_t(0);
  }
  // Code rings start as class 0: a group without a pair still reads its
  // ring, and the step uses what it reads as a profile index unchecked
  // (every class code the rings receive is below nclasses).
  {
    uint8_t *code_rings = s_rings + kSlots16 * smem16_top_stride(OUT);
    for (int k = threadIdx.x; k < kSlots16 * (kCodeRing16 + kRingPad); k += blockDim.x) code_rings[k] = 0;
  }
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
    const int lg = G == 4 ? 2 : (G == 8 ? 3 : (G == 16 ? 4 : 5));
    fill16_warp_task<LOCAL, CHECK, OUT>(A, s_mat, s_prof, s_match, s_rings, w.x, count, warp_id, 1 << lg, lg);
  }
}

size_t smem_i16(int out_mode, int nclasses);

// Launch and residency of the int16x2 fill of one output mode (each mode
// is instantiated in its own translation unit).
template <int OUT>
cudaError_t launch_i16(bool check, bool local, const FillArgs &args, int blocks, size_t smem, cudaStream_t st) {
  FillArgs a = args;
  a.one = 1u;
  if constexpr (OUT == kOutIdent) {
    if (local) return cudaErrorInvalidValue;
    if (check)
      fill_i16_kernel<false, true, OUT><<<blocks, kThreads16, smem, st>>>(a);
    else
      fill_i16_kernel<false, false, OUT><<<blocks, kThreads16, smem, st>>>(a);
  } else {
    if (check) {
      if (local)
        fill_i16_kernel<true, true, OUT><<<blocks, kThreads16, smem, st>>>(a);
      else
        fill_i16_kernel<false, true, OUT><<<blocks, kThreads16, smem, st>>>(a);
    } else {
      if (local)
        fill_i16_kernel<true, false, OUT><<<blocks, kThreads16, smem, st>>>(a);
      else
        fill_i16_kernel<false, false, OUT><<<blocks, kThreads16, smem, st>>>(a);
    }
  }
  return cudaGetLastError();
}

template <int OUT>
int occupancy_i16(bool check, bool local, size_t smem) {
  void (*k)(const FillArgs);
  if constexpr (OUT == kOutIdent) {
    if (local) return 0;
    k = check ? fill_i16_kernel<false, true, OUT> : fill_i16_kernel<false, false, OUT>;
  } else {
    k = check ? (local ? fill_i16_kernel<true, true, OUT> : fill_i16_kernel<false, true, OUT>)
              : (local ? fill_i16_kernel<true, false, OUT> : fill_i16_kernel<false, false, OUT>);
  }
  // The attribute allows the largest profile (26 classes), so that every
  // scheme's launch fits whatever scheme was sized first.
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           int(std::max(smem, smem_i16(OUT, kLetters)))) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads16, smem) != cudaSuccess) return 0;
  return nb;
}

}  // namespace fill
}  // namespace tsq
