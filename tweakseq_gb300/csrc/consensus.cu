// consensus.cu -- consensus line of a gapped alignment on the GPU.
//
// Same result as Consensus::calculate (tweakseq/Core/Annotations/
// Consensus.cpp:80-161), which for every column scores each row against
// every other row (O(nseq^2) per column): +1 for two "gap" bytes (anything
// outside 'A'..'Z', :96-106), -4 for one, BLOSUM62 otherwise; a pair counts as
// a match when its score is positive.  The first row with the highest sum
// wins, and the column shows that row's byte when its match count reaches
// the plurality (default nseq / 2, :163-172), else '?'.
//
// A row's sum depends only on its class (23 BLOSUM62 rows + the gap class),
// so the kernel counts bytes per column in 27 bins ('A'..'Z' and everything
// else; one pass over the bytes), and the finishing kernel folds the bins
// into the 24 classes, evaluates the class sums from the counts:
// score(x) = sum_y count(y) S(x,y) - S(x,x), then scans the column from the
// first row for the first row whose class holds the best sum.  All terms are
// integers, so this equals the reference's double sums exactly, and the row
// found is the first row with the best score, as there.
#include <climits>
#include <cstring>

#include "engine.h"

namespace tsq {
namespace {

constexpr int kClasses = 24;  // BLOSUM62 rows 0..22, 23 = gap class
constexpr int kGapClass = 23;
constexpr int kBins = 27;  // counted per column: 'A'..'Z', then every other byte
constexpr int kOtherBin = 26;
constexpr int kCountWarps = 8;
constexpr int kCountThreads = kCountWarps * 32;
constexpr int kTile = 128;  // columns per block

__constant__ int8_t c_pair[kClasses][kClasses];  // class-vs-class pair scores
__constant__ uint8_t c_class[256];                // byte -> class
__constant__ uint8_t c_bin_class[kBins];          // counting bin -> class

// Counting bin of each byte of a word, four at a time: 'A'..'Z' -> 0..25,
// every other byte -> 26 (per-byte SIMD subtract and compare).
__device__ __forceinline__ uint32_t bins4(uint32_t v) {
  const uint32_t d = __vsub4(v, 0x41414141u);
  const uint32_t lt = __vcmpltu4(d, 0x1a1a1a1au);  // 0xff in the letter bytes
  return (d & lt) | (0x1a1a1a1au & ~lt);
}

// A block covers 128 columns (lane t holds columns t, t+32, t+64, t+96 of
// the tile, so that its counters fall in bank t) and one slice of the rows,
// striped over its 8 warps.  With 4-byte-aligned rows a lane reads its 4
// columns of a row with one 32-bit load, eight rows' loads in flight, bins
// the four bytes with two SIMD instructions and adds each to its column's
// bin with one shared-memory atomic -- the one shared-memory operation per
// byte, which sets the pace.  The counts go to one shared histogram per
// block, then into the column totals with global atomics.  Only counts: the
// first row of a class is needed for the winning classes alone and is found
// afterwards.
template <bool kVec>
__global__ void __launch_bounds__(kCountThreads) consensus_count_kernel(const uint8_t *__restrict__ rows, int32_t nseq,
                                                                        int32_t ncols, int64_t stride,
                                                                        int32_t rows_per_slice, uint32_t *cnt) {
  __shared__ uint32_t h[kBins][kTile];
  for (int k = threadIdx.x; k < kBins * kTile; k += kCountThreads) (&h[0][0])[k] = 0u;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t c0 = blockIdx.x * kTile;
  const int32_t r0 = blockIdx.y * rows_per_slice;
  const int32_t r1 = min(nseq, r0 + rows_per_slice);
  // This lane's columns: c0 + 4*lane .. +3 in memory, tile slots lane + 32u.
  const int32_t mc = c0 + 4 * lane;
  const int nvalid = max(0, min(4, ncols - mc));
  if (nvalid > 0) {
    const uint8_t *p = rows + mc;
    uint32_t *hb = &h[0][lane];
    constexpr int kRows = 8;
    int32_t r = r0 + w;
    if (kVec && nvalid == 4) {
      auto count4 = [&](uint32_t v) {
        const uint32_t b = bins4(v);
        atomicAdd(hb + __byte_perm(b, 0u, 0x4440u) * kTile, 1u);
        atomicAdd(hb + 32 + __byte_perm(b, 0u, 0x4441u) * kTile, 1u);
        atomicAdd(hb + 64 + __byte_perm(b, 0u, 0x4442u) * kTile, 1u);
        atomicAdd(hb + 96 + __byte_perm(b, 0u, 0x4443u) * kTile, 1u);
      };
      const uint32_t *pw = reinterpret_cast<const uint32_t *>(p);
      const int64_t wstride = stride / 4;
      for (; r + (kRows - 1) * kCountWarps < r1; r += kRows * kCountWarps) {
        uint32_t v[kRows];
#pragma unroll
        for (int q = 0; q < kRows; ++q) v[q] = __ldg(pw + int64_t(r + q * kCountWarps) * wstride);
#pragma unroll
        for (int q = 0; q < kRows; ++q) count4(v[q]);
      }
      for (; r < r1; r += kCountWarps) count4(__ldg(pw + int64_t(r) * wstride));
    } else {
      // Ragged last columns or unaligned rows: byte loads.
      for (; r < r1; r += kCountWarps) {
        uint32_t v = 0;
        for (int u = 0; u < nvalid; ++u) v |= uint32_t(__ldg(p + int64_t(r) * stride + u)) << (8 * u);
        const uint32_t b = bins4(v);
        for (int u = 0; u < nvalid; ++u) atomicAdd(hb + 32 * u + ((b >> (8 * u)) & 0xffu) * kTile, 1u);
      }
    }
  }
  __syncthreads();
  for (int e = threadIdx.x; e < kBins * kTile; e += kCountThreads) {
    const int bin = e / kTile, slot = e % kTile;
    const uint32_t s = h[bin][slot];
    // Tile slot lane + 32u holds memory column c0 + 4*lane + u.
    const int32_t col = c0 + 4 * (slot & 31) + (slot >> 5);
    if (s != 0u && col < ncols) atomicAdd(&cnt[int64_t(col) * kBins + bin], s);
  }
}

__global__ void consensus_init_kernel(uint32_t *cnt, int64_t n) {
  for (int64_t k = blockIdx.x * int64_t(blockDim.x) + threadIdx.x; k < n; k += int64_t(gridDim.x) * blockDim.x)
    cnt[k] = 0u;
}

// One warp per column: lane x < 24 forms class x's sum of pair scores
// against the column's counts (less the row's own pair) and its count of
// positive pairs; the warp takes the best sum over the classes present, and
// then the first row (in row order) whose class holds it -- the row the
// reference's loop settles on -- scanning 32 rows per ballot.  The scan
// usually ends in the first ballot (a winning class is a frequent one).
constexpr int kFinishWarps = 8;
__global__ void __launch_bounds__(kFinishWarps * 32)
    consensus_finish_kernel(const uint8_t *__restrict__ rows, int32_t nseq, int32_t ncols, int64_t stride,
                            double plurality, const uint32_t *__restrict__ cnt, uint8_t *out, int32_t *best_score,
                            int32_t *best_matches) {
  __shared__ uint8_t cls[256];
  __shared__ int8_t pair[kClasses][kClasses + 1];
  __shared__ uint32_t n_s[kFinishWarps][kClasses];
  for (int k = threadIdx.x; k < 256; k += blockDim.x) cls[k] = c_class[k];
  for (int k = threadIdx.x; k < kClasses * kClasses; k += blockDim.x)
    pair[k / kClasses][k % kClasses] = c_pair[k / kClasses][k % kClasses];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int32_t col = blockIdx.x * kFinishWarps + w;
  __shared__ uint32_t bin_s[kFinishWarps][kBins];
  if (col < ncols && lane < kBins) bin_s[w][lane] = cnt[int64_t(col) * kBins + lane];
  __syncwarp();
  if (col < ncols && lane < kClasses) {  // fold the bins into the classes
    uint32_t c = 0u;
    for (int b = 0; b < kBins; ++b) c += c_bin_class[b] == lane ? bin_s[w][b] : 0u;
    n_s[w][lane] = c;
  }
  __syncthreads();
  if (col >= ncols) return;
  const int x = lane < kClasses ? lane : 0;
  int64_t sx = 0, mt = 0;
#pragma unroll 8
  for (int y = 0; y < kClasses; ++y) {
    const int64_t ny = n_s[w][y];
    const int v = pair[x][y];
    sx += ny * v;
    if (v > 0) mt += ny;
  }
  // A row does not score against itself.
  sx -= pair[x][x];
  if (pair[x][x] > 0) mt -= 1;
  const bool present = lane < kClasses && n_s[w][x] != 0u;
  int64_t bs = present ? sx : INT64_MIN;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const int64_t other = __shfl_xor_sync(0xffffffffu, bs, o);
    bs = other > bs ? other : bs;
  }
  const uint32_t winners = __ballot_sync(0xffffffffu, present && sx == bs);  // classes holding the best sum
  int32_t r = -1;
  int c = 0;
  for (int32_t r0 = 0; r0 < nseq; r0 += 32) {
    const int32_t rr = r0 + lane;
    const int cl = rr < nseq ? int(cls[rows[int64_t(rr) * stride + col]]) : 0;
    const uint32_t hit = __ballot_sync(0xffffffffu, rr < nseq && ((winners >> cl) & 1u));
    if (hit) {
      const int first = __ffs(hit) - 1;
      r = r0 + first;
      c = __shfl_sync(0xffffffffu, cl, first);
      break;
    }
  }
  if (r < 0) {  // (a winning class always occurs; stays in bounds regardless)
    r = nseq - 1;
    c = cls[rows[int64_t(r) * stride + col]];
  }
  const int64_t bm = __shfl_sync(0xffffffffu, mt, c);
  if (lane == 0) {
    out[col] = double(bm) >= plurality ? rows[int64_t(r) * stride + col] : uint8_t('?');
    if (best_score) best_score[col] = int32_t(bs);
    if (best_matches) best_matches[col] = int32_t(bm);
  }
}

// BLOSUM62 row of each letter 'A'..'Z' (J, O, U, X share the X row), as the
// reference's letter map; everything else is the gap class.
void class_tables(int8_t pair[kClasses][kClasses], uint8_t cls[256], uint8_t bin_class[kBins]) {
  static const char kOrder[23] = {'A', 'R', 'N', 'D', 'C', 'Q', 'E', 'G', 'H', 'I', 'L', 'K',
                                  'M', 'F', 'P', 'S', 'T', 'W', 'Y', 'V', 'B', 'Z', 'X'};
  for (int b = 0; b < 256; ++b) cls[b] = kGapClass;
  for (int k = 0; k < 23; ++k) cls[uint8_t(kOrder[k])] = uint8_t(k);
  cls[uint8_t('J')] = cls[uint8_t('O')] = cls[uint8_t('U')] = 22;
  for (int b = 0; b < 26; ++b) bin_class[b] = cls[uint8_t('A' + b)];
  bin_class[kOtherBin] = kGapClass;
  for (int x = 0; x < kClasses; ++x)
    for (int y = 0; y < kClasses; ++y) {
      if (x == kGapClass && y == kGapClass)
        pair[x][y] = 1;
      else if (x == kGapClass || y == kGapClass)
        pair[x][y] = -4;
      else
        pair[x][y] = blosum62_by_row(x, y);
    }
}

cudaError_t upload_tables() {
  // The constant tables are per device; upload them once per device.
  static thread_local int done_dev = -1;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || done_dev == dev) return e;
  int8_t pair[kClasses][kClasses];
  uint8_t cls[256], bin_class[kBins];
  class_tables(pair, cls, bin_class);
  e = cudaMemcpyToSymbol(c_pair, pair, sizeof(pair));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_class, cls, sizeof(cls));
  if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_bin_class, bin_class, sizeof(bin_class));
  if (e == cudaSuccess) done_dev = dev;
  return e;
}

int sm_count() {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms;
}

int check_args(int32_t nseq, int32_t ncols, int64_t stride) {
  if (nseq <= 0 || nseq > (1 << 27) || ncols < 0 || stride < ncols) return TSQ_E_INVALID_ARG;
  return TSQ_OK;
}

// Launches on `stream`: counts, then the per-column decision.
cudaError_t consensus_enqueue(const uint8_t *d_rows, int32_t nseq, int32_t ncols, int64_t stride, double plurality,
                              uint8_t *d_out, int32_t *d_score, int32_t *d_matches, void *scratch,
                              cudaStream_t stream) {
  if (ncols == 0) return cudaSuccess;
  cudaError_t e = upload_tables();
  if (e != cudaSuccess) return e;
  uint32_t *cnt = static_cast<uint32_t *>(scratch);
  const int64_t entries = int64_t(ncols) * kBins;
  consensus_init_kernel<<<int(std::min<int64_t>((entries + 255) / 256, 4096)), 256, 0, stream>>>(cnt, entries);
  // Enough blocks for every SM several times over: split the rows into
  // slices when the columns alone do not give them.
  const int32_t col_tiles = (ncols + kTile - 1) / kTile;
  const int64_t want = int64_t(sm_count()) * 8;
  int32_t slices = int32_t(std::max<int64_t>(1, std::min<int64_t>((want + col_tiles - 1) / col_tiles, 65535)));
  int32_t per = (nseq + slices - 1) / slices;
  per = std::max(per, 8 * kCountWarps);
  slices = (nseq + per - 1) / per;
  const bool vec = stride % 4 == 0 && reinterpret_cast<uintptr_t>(d_rows) % 4 == 0;
  if (vec)
    consensus_count_kernel<true><<<dim3(col_tiles, slices), kCountThreads, 0, stream>>>(d_rows, nseq, ncols, stride,
                                                                                      per, cnt);
  else
    consensus_count_kernel<false><<<dim3(col_tiles, slices), kCountThreads, 0, stream>>>(d_rows, nseq, ncols, stride,
                                                                                       per, cnt);
  consensus_finish_kernel<<<(ncols + kFinishWarps - 1) / kFinishWarps, kFinishWarps * 32, 0, stream>>>(
      d_rows, nseq, ncols, stride, plurality, cnt, d_out, d_score, d_matches);
  return cudaGetLastError();
}

struct ConsensusCache {
  DevBuf rows, scratch, out;
  cudaStream_t stream = nullptr;
  int dev = -1;
  ~ConsensusCache() {
    if (stream) cudaStreamDestroy(stream);
  }
};

}  // namespace

size_t consensus_scratch_bytes(int32_t ncols) { return size_t(ncols > 0 ? ncols : 0) * kBins * 4; }

}  // namespace tsq

extern "C" {

size_t tsq_consensus_scratch_bytes(int32_t ncols) { return tsq::consensus_scratch_bytes(ncols); }

int tsq_consensus_device(const uint8_t *d_rows, int32_t nseq, int32_t ncols, int64_t stride, double plurality,
                         uint8_t *d_consensus, int32_t *d_best_score, int32_t *d_best_matches, void *d_scratch,
                         size_t scratch_bytes, void *stream) {
  if (int rc = tsq::check_args(nseq, ncols, stride)) return rc;
  if (ncols > 0 && (!d_rows || !d_consensus || !d_scratch || scratch_bytes < tsq::consensus_scratch_bytes(ncols)))
    return TSQ_E_INVALID_ARG;
  if (plurality < 0) plurality = nseq / 2.0;
  return tsq::cuda_status(tsq::consensus_enqueue(d_rows, nseq, ncols, stride, plurality, d_consensus, d_best_score,
                                                 d_best_matches, d_scratch, static_cast<cudaStream_t>(stream)));
}

int tsq_consensus(const uint8_t *rows, int32_t nseq, int32_t ncols, int64_t stride, double plurality,
                  uint8_t *consensus, int32_t *best_score, int32_t *best_matches) {
  if (int rc = tsq::check_args(nseq, ncols, stride)) return rc;
  if (ncols > 0 && (!rows || !consensus)) return TSQ_E_INVALID_ARG;
  if (ncols == 0) return TSQ_OK;
  if (plurality < 0) plurality = nseq / 2.0;
  try {
    thread_local tsq::ConsensusCache c;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return TSQ_E_CUDA;
    if (c.dev != dev) {
      c.rows.release();
      c.scratch.release();
      c.out.release();
      if (c.stream) cudaStreamDestroy(c.stream);
      c.stream = nullptr;
      if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) return TSQ_E_CUDA;
      c.dev = dev;
    }
    // Rows go up packed (pitch = ncols rounded up to 16 bytes).
    const int64_t pitch = (int64_t(ncols) + 15) / 16 * 16;
    cudaError_t e = c.rows.ensure(size_t(pitch) * size_t(nseq));
    if (e == cudaSuccess) e = c.scratch.ensure(tsq::consensus_scratch_bytes(ncols));
    if (e == cudaSuccess) e = c.out.ensure(size_t(ncols) * 9);
    if (e == cudaSuccess)
      e = cudaMemcpy2DAsync(c.rows.p, size_t(pitch), rows, size_t(stride), size_t(ncols), size_t(nseq),
                            cudaMemcpyHostToDevice, c.stream);
    uint8_t *d_out = c.out.as<uint8_t>();
    int32_t *d_score = reinterpret_cast<int32_t *>(d_out + (int64_t(ncols) + 15) / 16 * 16);
    int32_t *d_match = d_score + ncols;
    if (e == cudaSuccess)
      e = tsq::consensus_enqueue(c.rows.as<uint8_t>(), nseq, ncols, pitch, plurality, d_out, d_score, d_match,
                                 c.scratch.p, c.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(consensus, d_out, size_t(ncols), cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess && best_score)
      e = cudaMemcpyAsync(best_score, d_score, size_t(ncols) * 4, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess && best_matches)
      e = cudaMemcpyAsync(best_matches, d_match, size_t(ncols) * 4, cudaMemcpyDeviceToHost, c.stream);
    const cudaError_t s = cudaStreamSynchronize(c.stream);
    return tsq::cuda_status(e != cudaSuccess ? e : s);
  } catch (const std::bad_alloc &) {
    return TSQ_E_NOMEM;
  }
}

}  // extern "C"
