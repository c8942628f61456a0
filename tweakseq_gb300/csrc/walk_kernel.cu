// walk_kernel.cu -- traceback walker and residue encoder.
//
// The walker follows the 4-bit direction planes written by the fill from the
// end cell back to the start, exactly as the CPU oracle's walk does (state
// machine over H, E and F; E and F runs end where the "opened" bit is set;
// global rows/columns 0 are single gap runs; local stops on a STOP cell or
// row/column 0).  It emits the two gapped rows backwards into the pair's
// output slot, so the aligned strings end at slot + cap and start at
// slot + cap - n_cols, and records identity, column count and the begin
// coordinates.
#include <algorithm>

#include "tsq_internal.h"

namespace tsq {
namespace {

// The walk of one pair, from its end cell back to its start, through a
// plane reader and two sequence readers.  Every lane of the pair's warp runs
// it with the same values (warp-uniform branches); only `writer` (lane 0)
// stores, except in a run of diagonal moves, where lane k writes the k-th
// column of the run.
template <class Plane, class Seq>
__device__ __forceinline__ void walk_pair(const WalkArgs &A, const PairDev &pr, ResultDev &res, Plane &pl, Seq &a,
                                          Seq &b, char *out_a, char *out_b, int64_t cap, int lane) {
  const bool writer = lane == 0;
  const int m = pr.a_len, n = pr.b_len;
  int i, j;
  if (A.local) {
    if (res.score <= 0) {
      if (writer) {
        res.a_begin = res.a_end = res.b_begin = res.b_end = 0;
        res.n_ident = res.n_cols = 0;
      }
      return;
    }
    i = res.a_end;
    j = res.b_end;
  } else {
    i = m;
    j = n;
  }
  if (i > 0) pl.set_row(i);
  int state = 0;  // 0 = H, 1 = E, 2 = F
  int64_t L = 0;
  int ident = 0;
  for (;;) {
    if (L >= cap && (i > 0 || j > 0)) {  // cannot happen with valid planes
      if (writer) res.status = TSQ_E_CUDA;
      return;
    }
    if (state == 0) {
      if (A.local) {
        if (i == 0 || j == 0 || (pl.nib(j) & 3) == kDirStop) break;
      } else if (i == 0 && j == 0) {
        break;
      }
      if (i > 0 && j > 0) {
        // A run of diagonal moves at once: lane k tests the cell k steps back
        // along the diagonal, inside the plane window loaded around the
        // current cell (a cell outside it ends the run); the leading run of
        // diagonal cells becomes p aligned columns, lane k writing the k-th.
        (void)pl.nib(j);
        const uint32_t dm = pl.diag_mask(i, j);
        const int p = dm == 0xffffffffu ? 32 : __ffs(~dm) - 1;
        if (p > 1) {
          a.cover(i - 1);
          b.cover(j - 1);
          uint8_t ca = 0, cb = 0;
          if (lane < p) {
            ca = a.get(i - 1 - lane);
            cb = b.get(j - 1 - lane);
            out_a[cap - L - 1 - lane] = char(ca);
            out_b[cap - L - 1 - lane] = char(cb);
          }
          ident += __popc(__ballot_sync(0xffffffffu, lane < p && ca == cb));
          L += p;
          i -= p;
          j -= p;
          if (i > 0) pl.set_row(i);
          continue;
        }
      }
      if (i == 0) {  // global top row: one horizontal gap run
        ++L;
        const char cb = char(b.at(j - 1));
        if (writer) {
          out_a[cap - L] = '-';
          out_b[cap - L] = cb;
        }
        --j;
        continue;
      }
      if (j == 0) {  // global left column: one vertical gap run
        ++L;
        const char ca = char(a.at(i - 1));
        if (writer) {
          out_a[cap - L] = ca;
          out_b[cap - L] = '-';
        }
        --i;
        if (i > 0) pl.up();
        continue;
      }
      const int hd = pl.nib(j) & 3;
      if (hd == kDirDiag) {
        ++L;
        const uint8_t ca = a.at(i - 1), cb = b.at(j - 1);
        if (writer) {
          out_a[cap - L] = char(ca);
          out_b[cap - L] = char(cb);
        }
        ident += ca == cb;
        --i;
        --j;
        if (i > 0) pl.up();
      } else {
        state = hd;
      }
    } else if (state == 1) {
      // An E run always ends inside the matrix (E(i,0) is minus infinity);
      // if the planes say otherwise, stop instead of leaving the matrix.
      if (j <= 0 || i <= 0) {
        if (writer) res.status = TSQ_E_CUDA;
        return;
      }
      const int d = pl.nib(j);
      ++L;
      const char cb = char(b.at(j - 1));
      if (writer) {
        out_a[cap - L] = '-';
        out_b[cap - L] = cb;
      }
      --j;
      if (d & 4) state = 0;
    } else {
      if (i <= 0 || j <= 0) {
        if (writer) res.status = TSQ_E_CUDA;
        return;
      }
      const int d = pl.nib(j);
      ++L;
      const char ca = char(a.at(i - 1));
      if (writer) {
        out_a[cap - L] = ca;
        out_b[cap - L] = '-';
      }
      --i;
      if (i > 0) pl.up();
      if (d & 8) state = 0;
    }
  }
  if (!writer) return;
  res.a_begin = i;
  res.b_begin = j;
  if (!A.local) {
    res.a_end = m;
    res.b_end = n;
  }
  res.n_cols = int32_t(L);
  res.n_ident = ident;
}

// One warp per pair, every lane running the pair's walk with the same
// values, so a window refill costs the warp one coalesced load per lane and
// the warp waits only for its own pair's refills.  (A thread per pair made
// each warp wait for all 32 of its pairs' refills in turn: 0.77 against
// 0.14 ms on 2,016 protein pairs, 18.3 against 3.2 ms on 32 long DNA pairs,
// 3.8 against 3.6 ms on 100,000 pairs.)
constexpr int kWarpWalkWarps = 4;
constexpr int kWS = 32, kWL = 4;  // plane window: 32 steps x 4 lanes of one band
constexpr int kSeqWin = 128;      // residues per sequence window

struct WarpPlane {
  const uint32_t *words;
  uint32_t *win;  // kWS * kWL words of this warp
  int n, G, P, lane;
  int band, t, r;
  int wband = -1, wt = -1, ws = -1;
  __device__ void set_row(int i) {
    const int row0 = i - 1;
    band = row0 / P;
    const int w = row0 - band * P;
    t = w >> 3;
    r = w & 7;
  }
  __device__ void up() {
    if (--r < 0) {
      r = 7;
      if (--t < 0) {
        t = G - 1;
        --band;
      }
    }
  }
  // Steps s-kWS+1..s of lanes t-kWL+1..t (clamped into the band).
  __device__ void refill(int s) {
    wband = band;
    wt = t;
    ws = s;
    const int64_t row = (int64_t)band * (n + G - 1);
    uint32_t v[kWS * kWL / 32];
#pragma unroll
    for (int q = 0; q < kWS * kWL / 32; ++q) {
      const int w = lane + 32 * q;
      const int ss = max(s - w / kWL, 0), tt = max(t - w % kWL, 0);
      v[q] = __ldg(words + (row + ss) * G + tt);
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < kWS * kWL / 32; ++q) win[lane + 32 * q] = v[q];
    __syncwarp();
  }
  __device__ int nib(int j) {
    const int s = j - 1 + t;
    if (band != wband || t > wt || t <= wt - kWL || s > ws || s <= ws - kWS) refill(s);
    return int(win[(ws - s) * kWL + (wt - t)] >> (4 * r)) & 15;
  }
  // Lanes whose cell (i - lane, j - lane) lies inside the matrix and the
  // current window and takes H from the diagonal.
  __device__ uint32_t diag_mask(int i, int j) const {
    const int ik = i - lane, jk = j - lane;
    bool d = false;
    if (ik >= 1 && jk >= 1) {
      const int row0 = ik - 1;
      const int bk = row0 / P;
      const int w = row0 - bk * P;
      const int tk = w >> 3, rk = w & 7;
      const int sk = jk - 1 + tk;
      if (bk == wband && tk <= wt && tk > wt - kWL && sk <= ws && sk > ws - kWS)
        d = ((win[(ws - sk) * kWL + (wt - tk)] >> (4 * rk)) & 3) == uint32_t(kDirDiag);
    }
    return __ballot_sync(0xffffffffu, d);
  }
};

// One sequence read backwards through a shared window of kSeqWin residues.
struct WarpSeq {
  const uint8_t *base;
  int len;
  uint8_t *win;
  int lane;
  int lo = 1 << 30;
  // The window ending at idx.
  __device__ void refill_to(int idx) {
    lo = max(0, idx - kSeqWin + 1);
    uint8_t v[kSeqWin / 32];
#pragma unroll
    for (int q = 0; q < kSeqWin / 32; ++q) {
      const int k = lo + lane + 32 * q;
      v[q] = k < len ? base[k] : uint8_t(0);
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < kSeqWin / 32; ++q) win[lane + 32 * q] = v[q];
    __syncwarp();
  }
  __device__ uint8_t at(int idx) {
    if (idx < lo || idx >= lo + kSeqWin) refill_to(idx);
    return win[idx - lo];
  }
  // Makes residues idx-31..idx (those >= 0) readable with get().
  __device__ void cover(int idx) {
    if (max(0, idx - 31) < lo || idx >= lo + kSeqWin) refill_to(idx);
  }
  __device__ uint8_t get(int idx) const { return win[idx - lo]; }
};

__global__ void __launch_bounds__(kWarpWalkWarps * 32) walk_warp_kernel(const WalkArgs A) {
  __shared__ uint32_t s_plane[kWarpWalkWarps][kWS * kWL];
  __shared__ uint8_t s_seq[kWarpWalkWarps][2][kSeqWin];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int k = blockIdx.x * kWarpWalkWarps + w;
  if (k >= A.n_tasks) return;
  const int p = A.tasks[k];
  const PairDev pr = A.pairs[p];
  ResultDev &res = A.res[p];
  if (res.status != TSQ_OK) return;
  WarpSeq a{A.seqs + pr.a_off, pr.a_len, s_seq[w][0], lane}, b{A.seqs + pr.b_off, pr.b_len, s_seq[w][1], lane};
  const int64_t cap = (int64_t)pr.a_len + pr.b_len;
  char *out_a = A.aln + A.aln_off[p];
  const int G = A.shape_G[p];
  WarpPlane pl{reinterpret_cast<const uint32_t *>(A.planes + A.plane_off[p]), s_plane[w], pr.b_len, G,
               G * A.shape_R[p], lane};
  walk_pair(A, pr, res, pl, a, b, out_a, out_a + cap, cap, lane);
}

// ASCII -> letter codes, and (when clut is set) -> score classes for the
// int16x2 fill, through shared-memory tables.
__global__ void encode_kernel(const uint8_t *__restrict__ seqs, int64_t len, const uint8_t *__restrict__ lut,
                              uint8_t *__restrict__ codes, const uint8_t *__restrict__ clut,
                              uint8_t *__restrict__ ccodes) {
  __shared__ uint8_t s_lut[256], s_clut[256];
  s_lut[threadIdx.x] = lut[threadIdx.x];
  s_clut[threadIdx.x] = clut ? clut[threadIdx.x] : uint8_t(0);
  __syncthreads();
  // 16 residues per thread per iteration through 128-bit loads where the
  // buffer allows it; the tail goes byte by byte.
  const int64_t nvec = len / 16;
  const uint4 *src = reinterpret_cast<const uint4 *>(seqs);
  uint4 *dst = reinterpret_cast<uint4 *>(codes);
  uint4 *cdst = reinterpret_cast<uint4 *>(ccodes);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < nvec; v += stride) {
    const uint4 w0 = src[v];
    uint4 w = w0, c = w0;
    uint32_t *x = reinterpret_cast<uint32_t *>(&w);
    uint32_t *y = reinterpret_cast<uint32_t *>(&c);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const uint32_t u = x[q];
      x[q] = uint32_t(s_lut[u & 0xFF]) | (uint32_t(s_lut[(u >> 8) & 0xFF]) << 8) |
             (uint32_t(s_lut[(u >> 16) & 0xFF]) << 16) | (uint32_t(s_lut[u >> 24]) << 24);
      y[q] = uint32_t(s_clut[u & 0xFF]) | (uint32_t(s_clut[(u >> 8) & 0xFF]) << 8) |
             (uint32_t(s_clut[(u >> 16) & 0xFF]) << 16) | (uint32_t(s_clut[u >> 24]) << 24);
    }
    dst[v] = w;
    if (ccodes) cdst[v] = c;
  }
  for (int64_t k = nvec * 16 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < len; k += stride) {
    codes[k] = s_lut[seqs[k]];
    if (ccodes) ccodes[k] = s_clut[seqs[k]];
  }
}

}  // namespace

cudaError_t launch_walk(const WalkArgs &a, cudaStream_t st) {
  if (a.n_tasks <= 0) return cudaSuccess;
  const int blocks = (a.n_tasks + kWarpWalkWarps - 1) / kWarpWalkWarps;
  walk_warp_kernel<<<blocks, kWarpWalkWarps * 32, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_encode(const uint8_t *seqs, int64_t len, const uint8_t *lut_dev, uint8_t *codes,
                          const uint8_t *clut_dev, uint8_t *ccodes, cudaStream_t st) {
  if (len <= 0) return cudaSuccess;
  int dev = 0, sms = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t work = (len + 15) / 16;
  int blocks = int(std::min<int64_t>((work + 255) / 256, (int64_t)sms * 8));
  if (blocks < 1) blocks = 1;
  encode_kernel<<<blocks, 256, 0, st>>>(seqs, len, lut_dev, codes, clut_dev, ccodes);
  return cudaGetLastError();
}

}  // namespace tsq
