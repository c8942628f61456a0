// fill_cta.cuh -- one long pair per CTA: the pair's row bands are striped
// over the CTA's W warps (band b runs on warp b mod W), each warp a 32-lane
// group of the int32 fill of fill_i32.cuh.  Consecutive bands run at the
// same time, each a few chunks of columns behind the one above it, so a
// pair of 50 kb sweeps with W warps instead of 1.  W is 16 where the
// kernel fits 128 registers (global score and traceback: one CTA fills an
// SM's 16 warps with one pair, halving a long pair's time against two
// 8-warp CTAs), 8 otherwise (local mode, identity).
//
// Band-to-band rows.  The bottom row of a band is the top row of the next.
// Between warps w and w+1 (w < W-1) it goes through a shared-memory ring of
// kCtaRing columns with flow control both ways (the producer waits for
// room, the consumer for data), published in 32-column chunks.  The wrap
// from warp W-1 back to warp 0 goes through a full-width row in global memory
// (the same row the warp-per-pair fill uses), whose producer never waits:
// that breaks the cycle of waits, so the pipeline cannot deadlock.  Warp 0
// stages that row with cp.async as the warp-per-pair fill does, after
// checking warp W-1's progress counter.
//
// Every wait is bounded (FillArgs::spin_limit polls, kSpinLimit when it is
// 0); a wait that runs out marks the pair TSQ_E_TIMEOUT and makes every
// other wait of the CTA give up, so the kernel always finishes.  A warp
// whose wait gave up carries on without waiting: every index it uses stays
// inside its rings, its rows and its pair's planes, and the pair's results
// are discarded through its status.
#pragma once

#include <algorithm>
#include <cstdint>

#include "fill_common.cuh"

namespace tsq {
namespace fill {

constexpr int kCtaRing = 256;               // inter-warp ring, columns (a multiple of kChunk)
constexpr int kSpinLimit = 1 << 22;         // polls per wait before giving up

template <int OUT>
struct CtaTop {
  using T = int2;
};
template <>
struct CtaTop<kOutIdent> {
  using T = int4;
};

// Warps per CTA for an output mode and alignment mode.
__host__ __device__ constexpr int cta_warps(int out_mode, bool local) {
  return (out_mode != kOutIdent && !local) ? 16 : 8;
}

// Control block after the rings: progress counters prod[W], cons[W], the
// fail flag and two ints (task index, spare), then W reduction keys and W
// counts.
__host__ __device__ constexpr int cta_keys_offset(int W) { return (4 * (2 * W + 3) + 15) & ~15; }
__host__ __device__ constexpr int cta_ctl_bytes(int W) { return (cta_keys_offset(W) + 12 * W + 15) & ~15; }

// Shared-memory bytes of the CTA fill for an output mode.
__host__ __device__ constexpr size_t cta_smem_bytes(int out_mode, int W) {
  return size_t(kMatBytes) + size_t(kLetters) * W * 32 * 8 +                           // matrix, profile
         size_t(kTopRing) * (out_mode == kOutIdent ? 16 : 8) + kRingPad +              // warp 0's staging ring
         size_t(W) * (kCodeRing + kRingPad) +                                          // code rings
         size_t(W - 1) * kCtaRing * (out_mode == kOutIdent ? 16 : 8) +                 // inter-warp rings
         cta_ctl_bytes(W);                                                             // counters
}

// Warp-uniform poll of a shared counter until it reaches target.  False if
// the wait ran out (or another wait of the CTA did).
__device__ __forceinline__ bool cta_wait_geq(const volatile int *ctr, int target, volatile int *fail, int limit) {
  const int lane = threadIdx.x & 31;
  for (int it = 0; it < limit; ++it) {
    int v = 0, f = 0;
    if (lane == 0) {
      v = *ctr;
      f = *fail;
    }
    v = __shfl_sync(0xffffffffu, v, 0);
    f = __shfl_sync(0xffffffffu, f, 0);
    if (v >= target) {
      __threadfence_block();
      return true;
    }
    if (f) return false;
    __nanosleep(64);
  }
  if (lane == 0) *fail = 1;
  return false;
}

template <bool LOCAL, int OUT, int W>
__global__ void __launch_bounds__(W * 32, 1) fill_cta_kernel(const FillArgs A) {
  constexpr int G = 32, R = 8, P = G * R;
  constexpr int kCtaWarps = W, kCtaThreads = W * 32;
  using Top = typename CtaTop<OUT>::T;
  extern __shared__ __align__(16) uint8_t smem[];
  int8_t *s_mat = reinterpret_cast<int8_t *>(smem);
  uint2 *s_prof = reinterpret_cast<uint2 *>(smem + kMatBytes);
  uint8_t *p = smem + kMatBytes + size_t(kLetters) * kCtaThreads * 8;
  Top *stage_ring = reinterpret_cast<Top *>(p);  // warp 0: staged global row
  p += kTopRing * sizeof(Top) + kRingPad;
  uint8_t *code_rings = p;
  p += kCtaWarps * (kCodeRing + kRingPad);
  Top *rings = reinterpret_cast<Top *>(p);  // ring w (w = 1..W-1) at rings + (w-1)*kCtaRing
  p += (kCtaWarps - 1) * kCtaRing * sizeof(Top);
  volatile int *prod = reinterpret_cast<volatile int *>(p);       // [kCtaWarps]
  volatile int *cons = prod + kCtaWarps;                           // [kCtaWarps]
  volatile int *fail = cons + kCtaWarps;
  int *s_misc = const_cast<int *>(fail) + 1;                       // task index, bad flag
  int64_t *s_keys = reinterpret_cast<int64_t *>(p + cta_keys_offset(W));           // [W] local reductions
  uint32_t *s_cnt = reinterpret_cast<uint32_t *>(p + cta_keys_offset(W) + 8 * W);  // [W]

  for (int k = threadIdx.x; k < kLetters * kLetters; k += blockDim.x) s_mat[k] = A.matrix[k];
  __syncthreads();

  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, t = lane;
  const int32_t go = A.gap_open, ge = A.gap_extend, oe = go + ge;
  Top *grow = reinterpret_cast<Top *>(A.bnd) + int64_t(blockIdx.x) * A.bnd_cols;  // the wrap-around row
  uint8_t *code_ring = code_rings + w * (kCodeRing + kRingPad);
  const uint2 *prof = s_prof + threadIdx.x;
  const int n_tasks = A.n_wtasks_dev ? *A.n_wtasks_dev : A.n_wtasks;
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
    const uint8_t *qa_codes = A.codes + pr.a_off, *qb_codes = A.codes + pr.b_off;
    const int64_t boff = pr.b_off;
    bool bad = false;
    for (int k = threadIdx.x; k < m; k += blockDim.x) bad |= qa_codes[k] >= kLetters;
    for (int k = threadIdx.x; k < n; k += blockDim.x) bad |= qb_codes[k] >= kLetters;
    const bool gbad = __syncthreads_or(bad) != 0;
    const bool trivial = (m == 0 || n == 0 || gbad);
    const int passes = trivial ? 0 : (m + P - 1) / P;
    uint8_t *planes = nullptr;
    if constexpr (OUT == kOutTrace) planes = A.planes + A.plane_off[pid];
    if (!trivial)
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        Top v;
        v.x = edge_h(j + 1, go, ge, LOCAL);
        v.y = kNegInf;
        if constexpr (OUT == kOutIdent) {
          v.z = LOCAL ? 0 : j + 1;
          v.w = 0;
        }
        grow[j] = v;
      }
    if (threadIdx.x < kCtaWarps) {
      prod[threadIdx.x] = 0;
      cons[threadIdx.x] = 0;
    }
    if (threadIdx.x == 0) *fail = 0;
    __syncthreads();

    int32_t lbest = 0, lrow = 0, lcol = 0;
    uint32_t lcnt = 0;
    int32_t last_h = 0;
    uint32_t last_c = 0;
    Top *ring_in = w > 0 ? rings + (w - 1) * kCtaRing : nullptr;             // written by warp w-1
    Top *ring_out = w < kCtaWarps - 1 ? rings + w * kCtaRing : nullptr;      // read by warp w+1

    for (int band = w; band < passes; band += kCtaWarps) {
      const int i = band / kCtaWarps;        // this warp's i-th band
      const int base = i * n;                // cumulative column position of the band in its rings
      // The last band's bottom row has no reader: it is neither written to
      // the next warp's ring nor waited on (nobody would make room).
      Top *const out_ring = band + 1 < passes ? ring_out : nullptr;
      const int row0 = band * P + t * R;
      int qa[R];
#pragma unroll
      for (int r = 0; r < R; ++r) qa[r] = (row0 + r < m) ? int(qa_codes[row0 + r]) : -1;
#pragma unroll 2
      for (int c = 0; c < kLetters; ++c) {
        uint32_t wv[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          uint32_t v = 0;
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            const int a = qa[q * 4 + k];
            v |= (a >= 0 ? uint32_t(uint8_t(s_mat[a * kLetters + c])) : 0u) << (8 * k);
          }
          wv[q] = v;
        }
        s_prof[c * kCtaThreads + threadIdx.x] = make_uint2(wv[0], wv[1]);
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

      // Where this band's top row comes from.  Warp 0: the global row (row
      // 0, or warp W-1's previous band, whose progress it checks first).
      auto stage_global = [&](int chunk) {
        if (band > 0) cta_wait_geq(&prod[0], (i - 1) * n + min(kChunk * (chunk + 1), n), fail, spin);
        stage_chunk<G, Top>(chunk, t, n, grow, stage_ring, A.codes, boff, code_ring);
      };
      cp_async_wait_all();
      __syncwarp();
      if (w == 0) {
        stage_global(0);
      } else {
        stage_codes(0, t, n, A.codes, boff, code_ring);
        cta_wait_geq(&prod[w], base + min(kChunk + 1, n), fail, spin);
      }
      cp_async_commit();
      cp_async_wait_all();
      __syncwarp();
      if (w == 0)
        stage_global(1);
      else
        stage_codes(1, t, n, A.codes, boff, code_ring);
      cp_async_commit();
      // Producer side: room for the first chunk of this band's bottom row.
      if (out_ring) cta_wait_geq(&cons[w + 1], base + kChunk - kCtaRing, fail, spin);

      auto top_at = [&](int col) -> Top {
        return w == 0 ? stage_ring[col & (kTopRing - 1)] : ring_in[(base + col) % kCtaRing];
      };
      int cb[2];
      uint2 pw[2];
      Top tv[2];
      cb[0] = min(int(code_ring[(boff - t) & (kCodeRing - 1)]), kLetters - 1);
      pw[0] = prof[cb[0] * kCtaThreads];
      tv[0] = top_at(0);
      const int max_steps = n + G - 1;

      // Steps [G, n_int) have every lane in range (and lane 0's next top
      // entry inside the row): no range tests there.  Both ends even, so
      // the double-buffer slot of a step is its parity in every segment.
      const int i0 = min(G, max_steps & ~1);
      const int i1 = max(i0, (n - 1) & ~1);
      auto step = [&](const int s, auto k_tag, auto interior_tag) {
        constexpr int k = decltype(k_tag)::value;
        constexpr bool INTERIOR = decltype(interior_tag)::value;
        if (((s + 1) & (kChunk - 1)) == 0) {
          // Consumer: the next chunk must be there before lane 0
          // prefetches its first column; report what was read.
          cp_async_wait_all();
          __syncwarp();
          if (w == 0) {
            stage_global((s + 1) / kChunk + 1);
          } else {
            stage_codes((s + 1) / kChunk + 1, t, n, A.codes, boff, code_ring);
            if (lane == 0) {
              __threadfence_block();  // the entries read so far are in registers
              cons[w] = base + min(s + 2, n);
            }
            cta_wait_geq(&prod[w], base + min(s + 1 + kChunk + 1, n), fail, spin);
          }
          cp_async_commit();
        }
        if ((s & (kChunk - 1)) == kChunk - 1) {
          // Producer: publish the chunk lane 31 finished, then wait for
          // room for the one it starts (column s - 31).
          const int done = min(max(s - (G - 1), 0), n);
          if (lane == G - 1) {
            __threadfence_block();
            if (w == kCtaWarps - 1)
              prod[0] = base + done;
            else
              prod[w + 1] = base + done;
          }
          if (out_ring && done < n) cta_wait_geq(&cons[w + 1], base + done + kChunk - kCtaRing, fail, spin);
        }
        int32_t upH = __shfl_up_sync(0xffffffffu, outH, 1);
        int32_t upF = __shfl_up_sync(0xffffffffu, outF, 1);
        uint32_t upCH = 0, upCF = 0;
        if constexpr (OUT == kOutIdent) {
          upCH = __shfl_up_sync(0xffffffffu, outCH, 1);
          upCF = __shfl_up_sync(0xffffffffu, outCF, 1);
        }
        const int jj = s - t;
        const bool valid = INTERIOR || (unsigned)jj < (unsigned)n;
        const int bc = cb[k & 1];
        const uint2 pcur = pw[k & 1];
        cb[(k + 1) & 1] = min(int(code_ring[(boff + jj + 1) & (kCodeRing - 1)]), kLetters - 1);
        pw[(k + 1) & 1] = prof[cb[(k + 1) & 1] * kCtaThreads];
        if (t == 0) {
          upH = tv[k & 1].x;
          upF = tv[k & 1].y;
          if constexpr (OUT == kOutIdent) {
            upCH = uint32_t(tv[k & 1].z);
            upCF = uint32_t(tv[k & 1].w);
          }
          if (INTERIOR || jj + 1 < n) tv[(k + 1) & 1] = top_at(jj + 1);
        }
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
            if (w == kCtaWarps - 1)
              grow[jj] = v;
            else if (out_ring)
              out_ring[(base + jj) % kCtaRing] = v;
          }
          if constexpr (OUT == kOutTrace) {
            const int64_t entry = ((int64_t)band * (n + G - 1) + s) * G + t;
            reinterpret_cast<uint32_t *>(planes)[entry] = tw;
          }
        }
      };
      int s0 = 0;
      for (; s0 < i0; s0 += 2) {
        step(s0, IntTag<0>{}, BoolTag<false>{});
        if (s0 + 1 < max_steps) step(s0 + 1, IntTag<1>{}, BoolTag<false>{});
      }
      for (; s0 < i1; s0 += 2) {
        step(s0, IntTag<0>{}, BoolTag<true>{});
        step(s0 + 1, IntTag<1>{}, BoolTag<true>{});
      }
      for (; s0 < max_steps; s0 += 2) {
        step(s0, IntTag<0>{}, BoolTag<false>{});
        if (s0 + 1 < max_steps) step(s0 + 1, IntTag<1>{}, BoolTag<false>{});
      }
      cp_async_wait_all();
      __syncwarp();
      // The whole bottom row is out; everything of the input ring was read.
      if (lane == G - 1) {
        __threadfence_block();
        if (w == kCtaWarps - 1)
          prod[0] = base + n;
        else
          prod[w + 1] = base + n;
      }
      if (lane == 0 && w > 0) {
        __threadfence_block();
        cons[w] = base + n;
      }

      if constexpr (LOCAL) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (row0 + r < m && best[r] > lbest) {
            lbest = best[r];
            lrow = row0 + r + 1;
            lcol = bcol[r];
            lcnt = bcnt[r];
          }
      } else if (band == passes - 1) {
        const int lr = (m - 1) - row0;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (r == lr) {
            last_h = H[r];
            last_c = cH[r];
          }
      }
    }

    // ---- results (every warp has finished its bands) -------------------
    __syncthreads();
    if constexpr (LOCAL) {
      const uint64_t key = (uint64_t(uint32_t(lbest)) << 40) | (uint64_t(0xFFFFFu - uint32_t(lrow)) << 20) |
                           uint64_t(0xFFFFFu - uint32_t(lcol));
      const uint64_t wkey = group_max<32>(key);
      const unsigned own = __ballot_sync(0xffffffffu, key == wkey && lbest > 0);
      const uint32_t wcnt = __shfl_sync(0xffffffffu, lcnt, own ? (__ffs(own) - 1) : 0);
      if (lane == 0) {
        s_keys[w] = int64_t(wkey);
        s_cnt[w] = wcnt;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        uint64_t gkey = 0;
        uint32_t cnt = 0;
        for (int q = 0; q < kCtaWarps; ++q)
          if (uint64_t(s_keys[q]) > gkey) {
            gkey = uint64_t(s_keys[q]);
            cnt = s_cnt[q];
          }
        ResultDev &o = A.res[pid];
        o.status = gbad ? TSQ_E_INVALID_RESIDUE : (*fail ? TSQ_E_TIMEOUT : TSQ_OK);
        const int32_t sc = int32_t(gkey >> 40);
        o.score = sc;
        o.a_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t((gkey >> 20) & 0xFFFFFu)) : 0;
        o.b_end = sc > 0 ? int32_t(0xFFFFFu - uint32_t(gkey & 0xFFFFFu)) : 0;
        o.a_begin = o.b_begin = sc > 0 ? -1 : 0;
        if (OUT == kOutIdent) {
          o.n_ident = sc > 0 ? int32_t(cnt >> 16) : 0;
          o.n_cols = sc > 0 ? int32_t(cnt & 0xFFFFu) : 0;
        } else {
          o.n_ident = o.n_cols = -1;
        }
      }
    } else {
      const int last_w = passes > 0 ? (passes - 1) % kCtaWarps : 0;
      const int owner_t = (m > 0) ? ((m - 1) % P) / R : 0;
      if (w == last_w && lane == owner_t) {
        ResultDev &o = A.res[pid];
        o.status = gbad ? TSQ_E_INVALID_RESIDUE : (*fail ? TSQ_E_TIMEOUT : TSQ_OK);
        o.a_begin = 0;
        o.a_end = m;
        o.b_begin = 0;
        o.b_end = n;
        if (m == 0 || n == 0) {
          o.score = (m + n == 0) ? 0 : -(go + (m + n) * ge);
          o.n_ident = OUT == kOutScore ? -1 : 0;
          o.n_cols = OUT == kOutScore ? -1 : m + n;
        } else {
          o.score = last_h;
          o.n_ident = OUT == kOutIdent ? int32_t(last_c >> 16) : -1;
          o.n_cols = OUT == kOutIdent ? int32_t(last_c & 0xFFFFu) : -1;
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace fill
}  // namespace tsq
