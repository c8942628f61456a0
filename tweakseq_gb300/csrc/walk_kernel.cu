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

constexpr int kWalkThreads = 128;
constexpr int kWin = 16;  // steps per plane window

// Direction nibbles of one pair, read through a window: the words of steps
// ws-15..ws for lanes wt-1 and wt of one band, loaded together into this
// thread's shared-memory slots.  A walk moves one step left or one row up
// at a time, so most nibbles come from the window and the window's 32 loads
// are independent of each other (one global-memory latency per refill
// instead of one per step).  Row i is tracked as (band, lane t, row r).
struct PlaneWalk {
  const uint32_t *words;  // planes as 32-bit entries: 8 rows x 4 bits
  uint32_t *win;          // 2 * kWin shared words of this thread
  int n, G, P;
  int band, t, r;                       // position of row i (1-based i >= 1)
  int wband = -1, wt = -1, ws = -1;     // the window
  __device__ void set_row(int i) {
    const int row0 = i - 1;
    band = row0 / P;
    const int w = row0 - band * P;
    t = w >> 3;
    r = w & 7;
  }
  __device__ void up() {  // i -> i - 1
    if (--r < 0) {
      r = 7;
      if (--t < 0) {
        t = G - 1;
        --band;
      }
    }
  }
  __device__ void refill(int s) {
    wband = band;
    wt = t;
    ws = s;
    const int64_t row = (int64_t)band * (n + G - 1);
    // All loads first (addresses clamped into the band, unused slots read a
    // valid word), then the stores: the loads overlap instead of each
    // waiting for the previous store.
    uint32_t v[2 * kWin];
#pragma unroll
    for (int k = 0; k < kWin; ++k) {
      const int64_t e = (row + max(s - k, 0)) * G + t;
      v[2 * k + 1] = __ldg(words + e);
      v[2 * k] = __ldg(words + (t > 0 ? e - 1 : e));
    }
#pragma unroll
    for (int k = 0; k < 2 * kWin; ++k) win[k] = v[k];
  }
  // Nibble of cell (i, j), i the current row, j >= 1.
  __device__ int nib(int j) {
    const int s = j - 1 + t;
    if (band != wband || (t != wt && t != wt - 1) || s > ws || s <= ws - kWin) refill(s);
    const uint32_t w = win[2 * (ws - s) + (t == wt ? 1 : 0)];
    return int(w >> (4 * r)) & 15;
  }
};

// One sequence read backwards through a 16-byte window.
struct SeqWalk {
  const uint8_t *base;
  uintptr_t blk = ~uintptr_t(0);
  uint4 v;
  __device__ uint8_t at(int idx) {
    const uintptr_t addr = reinterpret_cast<uintptr_t>(base) + uintptr_t(idx);
    const uintptr_t b = addr & ~uintptr_t(15);
    if (b != blk) {
      v = *reinterpret_cast<const uint4 *>(b);
      blk = b;
    }
    const int o = int(addr - b);
    const uint32_t w = o < 8 ? (o < 4 ? v.x : v.y) : (o < 12 ? v.z : v.w);
    return uint8_t(w >> (8 * (o & 3)));
  }
};

__global__ void __launch_bounds__(kWalkThreads) walk_kernel(const WalkArgs A) {
  __shared__ uint32_t s_win[kWalkThreads * 2 * kWin];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= A.n_tasks) return;
  const int p = A.tasks[k];
  const PairDev pr = A.pairs[p];
  ResultDev &res = A.res[p];
  if (res.status != TSQ_OK) return;
  const int m = pr.a_len, n = pr.b_len;
  SeqWalk a{A.seqs + pr.a_off}, b{A.seqs + pr.b_off};
  const int64_t cap = (int64_t)m + n;
  char *out_a = A.aln + A.aln_off[p];
  char *out_b = out_a + cap;
  const int G = A.shape_G[p];
  PlaneWalk pl{reinterpret_cast<const uint32_t *>(A.planes + A.plane_off[p]), s_win + threadIdx.x * 2 * kWin, n, G,
               G * A.shape_R[p]};

  int i, j;
  if (A.local) {
    if (res.score <= 0) {
      res.a_begin = res.a_end = res.b_begin = res.b_end = 0;
      res.n_ident = res.n_cols = 0;
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
      res.status = TSQ_E_CUDA;
      return;
    }
    if (state == 0) {
      if (A.local) {
        if (i == 0 || j == 0 || (pl.nib(j) & 3) == kDirStop) break;
      } else if (i == 0 && j == 0) {
        break;
      }
      if (i == 0) {  // global top row: one horizontal gap run
        ++L;
        out_a[cap - L] = '-';
        out_b[cap - L] = char(b.at(j - 1));
        --j;
        continue;
      }
      if (j == 0) {  // global left column: one vertical gap run
        ++L;
        out_a[cap - L] = char(a.at(i - 1));
        out_b[cap - L] = '-';
        --i;
        if (i > 0) pl.up();
        continue;
      }
      const int hd = pl.nib(j) & 3;
      if (hd == kDirDiag) {
        ++L;
        const uint8_t ca = a.at(i - 1), cb = b.at(j - 1);
        out_a[cap - L] = char(ca);
        out_b[cap - L] = char(cb);
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
        res.status = TSQ_E_CUDA;
        return;
      }
      const int d = pl.nib(j);
      ++L;
      out_a[cap - L] = '-';
      out_b[cap - L] = char(b.at(j - 1));
      --j;
      if (d & 4) state = 0;
    } else {
      if (i <= 0 || j <= 0) {
        res.status = TSQ_E_CUDA;
        return;
      }
      const int d = pl.nib(j);
      ++L;
      out_a[cap - L] = char(a.at(i - 1));
      out_b[cap - L] = '-';
      --i;
      if (i > 0) pl.up();
      if (d & 8) state = 0;
    }
  }
  res.a_begin = i;
  res.b_begin = j;
  if (!A.local) {
    res.a_end = m;
    res.b_end = n;
  }
  res.n_cols = int32_t(L);
  res.n_ident = ident;
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
  const int blocks = (a.n_tasks + kWalkThreads - 1) / kWalkThreads;
  walk_kernel<<<blocks, kWalkThreads, 0, st>>>(a);
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
