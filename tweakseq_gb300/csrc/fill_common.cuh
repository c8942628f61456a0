// fill_common.cuh -- pieces shared by the int32 and int16x2 fill kernels:
// profile-byte extraction, boundary values, group reductions and the
// cp.async staging of the top row and of b's residue codes.
#pragma once

#include <cstdint>

#include "tsq_internal.h"

namespace tsq {
namespace fill {

constexpr int kThreads = 128;   // 4 warps per block
constexpr int kMatBytes = 704;  // 26*26 int8 rounded up to a 64-byte multiple
constexpr int kAhead = 4;       // step-loop unroll

// Compile-time flags for the step bodies.
template <bool B>
struct BoolTag {
  static constexpr bool value = B;
};
template <int K>
struct IntTag {
  static constexpr int value = K;
};

// Sign-extends byte K of w to 32 bits with one PRMT (selector bit 3 of each
// nibble replicates the sign of the chosen byte).
template <int K>
__device__ __forceinline__ int32_t sbyte(uint32_t w) {
  uint32_t d;
  asm("prmt.b32 %0, %1, 0, %2;" : "=r"(d) : "r"(w), "n"(K | ((K | 8) << 4) | ((K | 8) << 8) | ((K | 8) << 12)));
  return int32_t(d);
}

__device__ __forceinline__ int32_t sbyte_dyn(uint32_t w, int k) {
  switch (k & 3) {
    case 0: return sbyte<0>(w);
    case 1: return sbyte<1>(w);
    case 2: return sbyte<2>(w);
    default: return sbyte<3>(w);
  }
}

// max(a, b) and whether a won (a >= b, so a wins ties): one compare and one
// select.  (The predicated DPX max, __vibmax_s32, costs four instructions --
// three on the ALU pipe -- on sm_103a.)
__device__ __forceinline__ int32_t max_pred(int32_t a, int32_t b, bool *a_won) {
  const bool p = a >= b;
  *a_won = p;
  return p ? a : b;
}

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

// Top-row entry carried from band to band: H and F, plus the path counts of
// both in identity mode.
template <int OUT>
struct TopT {
  using T = int2;
};
template <>
struct TopT<kOutIdent> {
  using T = int4;
};

// ---- staging rings --------------------------------------------------------
// Each group keeps, in shared memory, a 64-column ring of its top row and a
// 128-byte ring of b's residue codes.  They are filled by cp.async 32
// columns ahead of use (one chunk in flight while the group sweeps the
// previous one), so the step loop reads only shared memory.
constexpr int kChunk = 32;       // columns per staged chunk
constexpr int kTopRing = 64;     // top-row ring entries per group
constexpr int kCodeRing = 128;   // code ring bytes per group
constexpr int kSlotsPerBlock = kThreads / 32 * 8;  // 8 group slots per warp
// Ring slots are padded by 16 bytes so that the rings of a warp's groups,
// read at the same index in the same step, start in different banks.
constexpr int kRingPad = 16;

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
  const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Issues the copies of chunk k (columns [32k, 32k+32) of the top row and the
// code bytes of columns [32k, 32k+32]) for one group; lane t of the group
// takes copies t, t+G, ...  Nothing is copied past the pair's columns.
template <int G, typename Top, int CODE_RING = kCodeRing>
__device__ __forceinline__ void stage_chunk(int k, int t, int nact, const Top *top_g, Top *top_ring,
                                            const uint8_t *codes, int64_t boff, uint8_t *code_ring) {
  constexpr int kPer = 16 / int(sizeof(Top));                  // entries per 16-byte copy
  constexpr int kTopCopies = kChunk / kPer;
  constexpr int kCopies = kTopCopies + 3;
  const int c0 = kChunk * k;
  if (c0 >= nact) return;
  const int64_t a0 = (boff + c0) & ~int64_t(15);
#pragma unroll
  for (int q0 = 0; q0 < kCopies; q0 += G) {
    const int q = q0 + t;
    if (q < kTopCopies) {
      const int e = c0 + q * kPer;
      cp_async16(top_ring + (e & (kTopRing - 1)), top_g + e);
    } else if (q < kCopies) {
      const int64_t a = a0 + 16 * (q - kTopCopies);
      cp_async16(code_ring + (a & (CODE_RING - 1)), codes + a);
    }
  }
}

// Only the code bytes of chunk k (for groups whose top row comes from
// elsewhere): three 16-byte copies by lanes 0..2.
template <int CODE_RING = kCodeRing>
__device__ __forceinline__ void stage_codes(int k, int t, int nact, const uint8_t *codes, int64_t boff,
                                            uint8_t *code_ring) {
  const int c0 = kChunk * k;
  if (c0 >= nact || t >= 3) return;
  const int64_t a = ((boff + c0) & ~int64_t(15)) + 16 * t;
  cp_async16(code_ring + (a & (CODE_RING - 1)), codes + a);
}

// ---- runtime lane width ----------------------------------------------------
__device__ __forceinline__ unsigned group_mask_rt(int lane, int G) {
  return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << (lane & ~(G - 1)));
}

template <typename T>
__device__ __forceinline__ T group_max_rt(T v, int G) {
  for (int o = G >> 1; o > 0; o >>= 1) {
    T w = __shfl_xor_sync(0xffffffffu, v, o, G);
    v = w > v ? w : v;
  }
  return v;
}

// stage_chunk with the group width G known only at run time; ring slots of
// TOP_STRIDE entries and CODE_STRIDE bytes.
template <typename Top, int CODE_RING>
__device__ __forceinline__ void stage_chunk_rt(int G, int k, int t, int nact, const Top *top_g, Top *top_ring,
                                               const uint8_t *codes, int64_t boff, uint8_t *code_ring) {
  constexpr int kPer = 16 / int(sizeof(Top));
  constexpr int kTopCopies = kChunk / kPer;
  constexpr int kCopies = kTopCopies + 3;
  const int c0 = kChunk * k;
  if (c0 >= nact) return;
  const int64_t a0 = (boff + c0) & ~int64_t(15);
  for (int q = t; q < kCopies; q += G) {
    if (q < kTopCopies) {
      const int e = c0 + q * kPer;
      cp_async16(top_ring + (e & (kTopRing - 1)), top_g + e);
      // The first 16 bytes of each ring are mirrored past its end (into the
      // ring's padding), so a read at index + 1 needs no wrap.
      if ((e & (kTopRing - 1)) == 0) cp_async16(top_ring + kTopRing, top_g + e);
    } else {
      const int64_t a = a0 + 16 * (q - kTopCopies);
      cp_async16(code_ring + (a & (CODE_RING - 1)), codes + a);
      if ((a & (CODE_RING - 1)) == 0) cp_async16(code_ring + CODE_RING, codes + a);
    }
  }
}

}  // namespace fill
}  // namespace tsq
