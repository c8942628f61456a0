// noalloc.cu -- score-only batch alignment that allocates no memory.
//
// For callers that cannot allocate device memory themselves: code that runs
// while another allocator owns the device's free memory, real-time paths
// that must not block in cudaMalloc, or hosts whose allocations must all be
// accounted up front.  They hand over device buffers they already own (the
// residues, the pair table and the result array) plus a stream; every
// intermediate the fill needs -- encoded residues, the pair list, the band
// boundary rows and the work counters -- lives in one file-scope
// __device__ array of fixed size (kScratchBytes, 32 MiB), which every GPU
// that loads this library keeps until the process exits.
//
// Limits (larger inputs are rejected with TSQ_E_TOO_LARGE):
//   total residue bytes  <= kMaxResidues   (8 MiB)
//   pairs per call       <= kMaxPairs      (1,048,576)
//   sequence length      <= kMaxLen        (2,048)
//
// The fill is the int32 score kernel body (fill_i32.cuh) with 32 lanes per
// pair and one boundary row per warp; pairs are taken in input order.
//
// Every call shares the array and leaves its contents behind: each call
// clears its counters and rewrites everything else it reads before reading
// it.  Two calls whose work overlaps on the GPU (different streams, or
// different host threads) race on the array and corrupt each other.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (the host-side symbol is a stand-in, never a
// device address) and opts the fill kernel into its shared memory; that
// first call should come before any stream capture.  The set-up is kept per
// device for the life of the process: it is not redone after
// cudaDeviceReset, so a process that resets a device must not call this
// entry point on it again.
//
// Alignment: d_seqs must be 16-byte aligned, d_pairs 8-byte and d_out
// 4-byte aligned; other pointers are refused with TSQ_E_INVALID_ARG.
#include <cstdint>
#include <cstring>
#include <mutex>

#include "fill_i32.cuh"

namespace tsq {
namespace {

constexpr int64_t kMaxResidues = int64_t(8) << 20;
constexpr int64_t kMaxPairs = int64_t(1) << 20;
constexpr int32_t kMaxLen = 2048;
constexpr int32_t kBndCols = ((kMaxLen + 31) / 32 + 1) * 32;  // one staged chunk past the longest row
constexpr size_t kBndRowBytes = size_t(kBndCols) * sizeof(int2);

// Layout of the scratch array (byte offsets, 256-aligned).
constexpr size_t kOffCodes = 0;
constexpr size_t kOffMatrix = kOffCodes + size_t(kMaxResidues) + 256;
constexpr size_t kOffLut = kOffMatrix + 1024;
constexpr size_t kOffCounts = kOffLut + 256;  // [0] valid pairs, [1] next pair to fill
constexpr size_t kOffTasks = kOffCounts + 256;
constexpr size_t kOffBnd = kOffTasks + size_t(kMaxPairs) * sizeof(int32_t);
constexpr size_t kScratchBytes = size_t(32) << 20;
constexpr size_t kBndBytes = kScratchBytes - kOffBnd;
static_assert(kOffBnd % 256 == 0, "boundary rows must stay 256-aligned");
static_assert(kBndBytes >= size_t(64) * 8 * kBndRowBytes, "room for at least 64 blocks of boundary rows");

static __device__ __align__(256) uint8_t g_scratch[kScratchBytes];

static_assert(sizeof(tsq_device_result) == sizeof(ResultDev), "result layouts must match");
static_assert(sizeof(tsq_pair_desc) == sizeof(PairDev), "pair layouts must match");

struct Tables {
  int8_t matrix[kLetters * kLetters];
  uint8_t lut[256];
};

// Writes the scheme tables into the scratch array and clears the counters.
__global__ void na_prepare_kernel(const Tables tab, uint8_t *scratch) {
  for (int k = threadIdx.x; k < kLetters * kLetters; k += blockDim.x)
    reinterpret_cast<int8_t *>(scratch + kOffMatrix)[k] = tab.matrix[k];
  scratch[kOffLut + threadIdx.x] = tab.lut[threadIdx.x];
  if (threadIdx.x < 2) reinterpret_cast<int32_t *>(scratch + kOffCounts)[threadIdx.x] = 0;
}

// Rejects pairs outside the residue buffer or longer than max_len (status in
// the caller's result) and lists the others for the fill.
__global__ void na_validate_kernel(const PairDev *pairs, int32_t n, int64_t seqs_len, int32_t max_len,
                                   ResultDev *out, uint8_t *scratch) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const PairDev p = pairs[k];
  int32_t st = TSQ_OK;
  if (p.a_len < 0 || p.b_len < 0 || p.a_off < 0 || p.b_off < 0 || p.a_off > seqs_len - p.a_len ||
      p.b_off > seqs_len - p.b_len)
    st = TSQ_E_INVALID_ARG;
  else if (p.a_len > max_len || p.b_len > max_len)
    st = TSQ_E_TOO_LARGE;
  if (st != TSQ_OK) {
    ResultDev r;
    r.score = r.a_begin = r.a_end = r.b_begin = r.b_end = r.n_ident = r.n_cols = -1;
    r.status = st;
    out[k] = r;
    return;
  }
  int32_t *counts = reinterpret_cast<int32_t *>(scratch + kOffCounts);
  reinterpret_cast<int32_t *>(scratch + kOffTasks)[atomicAdd(&counts[0], 1)] = k;
}

// One pair per warp (32 lanes), one boundary row per warp.
template <bool LOCAL>
__global__ void __launch_bounds__(fill::kThreads) na_fill_kernel(const FillArgs base, uint8_t *scratch) {
  extern __shared__ __align__(16) uint8_t smem[];
  int8_t *s_mat = reinterpret_cast<int8_t *>(smem);
  uint2 *s_prof = reinterpret_cast<uint2 *>(smem + fill::kMatBytes);
  uint8_t *s_rings = smem + fill::kMatBytes + kLetters * fill::kThreads * sizeof(uint2);
  for (int k = threadIdx.x; k < kLetters * kLetters; k += blockDim.x) s_mat[k] = base.matrix[k];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int32_t *counts = reinterpret_cast<int32_t *>(scratch + kOffCounts);
  const int32_t n_valid = *reinterpret_cast<volatile int32_t *>(&counts[0]);
  FillArgs a = base;
  a.bnd = reinterpret_cast<int32_t *>(scratch + kOffBnd + size_t(warp) * kBndRowBytes);
  for (;;) {
    int idx = 0;
    if (lane == 0) idx = atomicAdd(&counts[1], 1);
    idx = __shfl_sync(0xffffffffu, idx, 0);
    if (idx >= n_valid) break;
    fill::fill_warp_task<32, 8, LOCAL, kOutScore>(a, s_mat, s_prof, s_rings, idx, 1, 0);
  }
}

struct DeviceSetup {
  uint8_t *scratch = nullptr;
  int blocks = 0;
  bool ready = false;
};

std::mutex g_setup_mu;
DeviceSetup g_setup[64];

int device_setup(int dev, DeviceSetup **out) {
  if (dev < 0 || dev >= 64) return TSQ_E_CUDA;
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup &s = g_setup[dev];
  if (!s.ready) {
    void *ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess) return TSQ_E_CUDA;
    const size_t smem = fill_smem_bytes(8, 0, kOutScore);
    if (cudaFuncSetAttribute(na_fill_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) !=
            cudaSuccess ||
        cudaFuncSetAttribute(na_fill_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) !=
            cudaSuccess)
      return TSQ_E_CUDA;
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, na_fill_kernel<false>, fill::kThreads, smem) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return TSQ_E_CUDA;
    const int warps_per_block = fill::kThreads / 32;
    const int fit = int(kBndBytes / (kBndRowBytes * warps_per_block));
    s.blocks = std::max(1, std::min(per_sm * sms, fit));
    s.scratch = static_cast<uint8_t *>(ptr);
    s.ready = true;
  }
  *out = &s;
  return TSQ_OK;
}

}  // namespace
}  // namespace tsq

extern "C" int tsq_align_score_noalloc(const uint8_t *d_seqs, int64_t seqs_len, const tsq_pair_desc *d_pairs,
                                       int32_t n, int32_t max_len, const tsq_params *p, tsq_device_result *d_out,
                                       void *stream) {
  using namespace tsq;
  if (!p || n < 0 || seqs_len < 0 || max_len < 0) return TSQ_E_INVALID_ARG;
  if (seqs_len > kMaxResidues || int64_t(n) > kMaxPairs || max_len > kMaxLen) return TSQ_E_TOO_LARGE;
  if ((seqs_len > 0 && !d_seqs) || (n > 0 && (!d_pairs || !d_out))) return TSQ_E_INVALID_ARG;
  // The encoder reads the residues 16 bytes at a time, the pair table holds
  // 8-byte offsets and the results are 4-byte fields: a misaligned caller
  // pointer (an offset into the caller's own buffer, say) is refused here,
  // before anything is launched, instead of faulting on the device.
  if ((seqs_len > 0 && (reinterpret_cast<uintptr_t>(d_seqs) & 15u) != 0) ||
      (n > 0 && ((reinterpret_cast<uintptr_t>(d_pairs) & 7u) != 0 || (reinterpret_cast<uintptr_t>(d_out) & 3u) != 0)))
    return TSQ_E_INVALID_ARG;
  if (p->output != TSQ_OUT_SCORE || (p->mode != TSQ_GLOBAL && p->mode != TSQ_LOCAL)) return TSQ_E_INVALID_ARG;
  if (p->gap_open < 0 || p->gap_extend < 0 || p->gap_open > 1000000 || p->gap_extend > 1000000)
    return TSQ_E_INVALID_ARG;
  // The int32 value range: every H, E, F stays above -(3*open + (2*max_len +
  // 1)*ext + 128), far from the kernel's minus infinity.
  if (3 * int64_t(p->gap_open) + (2 * int64_t(max_len) + 1) * p->gap_extend + 128 >= (int64_t(1) << 28))
    return TSQ_E_TOO_LARGE;
  Scheme sc;
  int rc = build_scheme(p, &sc);
  if (rc) return rc;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TSQ_E_CUDA;
  DeviceSetup *ds = nullptr;
  if ((rc = device_setup(dev, &ds))) return rc;
  if (n == 0) return TSQ_OK;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  Tables tab;
  std::memcpy(tab.matrix, sc.score, sizeof(tab.matrix));
  build_lut(sc, tab.lut);
  uint8_t *scratch = ds->scratch;
  na_prepare_kernel<<<1, 256, 0, st>>>(tab, scratch);
  if (cudaGetLastError() != cudaSuccess) return TSQ_E_CUDA;
  if (launch_encode(d_seqs, seqs_len, scratch + kOffLut, scratch + kOffCodes, nullptr, nullptr, st) != cudaSuccess) return TSQ_E_CUDA;
  na_validate_kernel<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const PairDev *>(d_pairs), n, seqs_len,
                                                       max_len, reinterpret_cast<ResultDev *>(d_out), scratch);
  if (cudaGetLastError() != cudaSuccess) return TSQ_E_CUDA;

  FillArgs a{};
  a.codes = scratch + kOffCodes;
  a.pairs = reinterpret_cast<const PairDev *>(d_pairs);
  a.tasks = reinterpret_cast<const int32_t *>(scratch + kOffTasks);
  a.matrix = reinterpret_cast<const int8_t *>(scratch + kOffMatrix);
  a.gap_open = p->gap_open;
  a.gap_extend = p->gap_extend;
  a.res = reinterpret_cast<ResultDev *>(d_out);
  a.bnd_cols = kBndCols;
  a.max_score = sc.max_score;
  const size_t smem = fill_smem_bytes(8, 0, kOutScore);
  if (p->mode == TSQ_LOCAL)
    na_fill_kernel<true><<<ds->blocks, fill::kThreads, smem, st>>>(a, scratch);
  else
    na_fill_kernel<false><<<ds->blocks, fill::kThreads, smem, st>>>(a, scratch);
  return cudaGetLastError() == cudaSuccess ? TSQ_OK : TSQ_E_CUDA;
}
