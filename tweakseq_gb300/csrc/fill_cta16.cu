// fill_cta16.cu -- instantiations and launcher of the int16x2 CTA fill.
#include <map>
#include <mutex>
#include <tuple>

#include "fill_cta16.cuh"

namespace tsq {
namespace fill {
namespace {

// Warps per CTA: 16 when the profile of the scheme's classes fits, else 8.
int cta16_warps(int nclasses) {
  return cta16_smem_bytes(16, nclasses) <= size_t(227) * 1024 ? 16 : 8;
}

template <int OUT, int W>
int occ16(int nclasses) {
  const size_t smem = cta16_smem_bytes(W, nclasses);
  auto k = fill_cta16_kernel<OUT, W>;
  // The attribute allows the largest profile this W takes, so that a launch
  // fits whatever scheme was sized first.
  const size_t most = W == 16 ? size_t(227) * 1024 : cta16_smem_bytes(W, kLetters);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(most)) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, W * 32, smem) != cudaSuccess) return 0;
  return nb;
}

template <int OUT>
int occ16_any(int nclasses) {
  return cta16_warps(nclasses) == 16 ? occ16<OUT, 16>(nclasses) : occ16<OUT, 8>(nclasses);
}

}  // namespace
}  // namespace fill

bool cta16_supported(int out_mode, bool local, const Scheme &sc, int32_t gap_open, int32_t gap_extend) {
  if (local || (out_mode != kOutScore && out_mode != kOutTrace)) return false;
  const int64_t step = int64_t(gap_open) + gap_extend + std::max(sc.max_score, 0);
  return step <= fill::kMaxStep16 && sc.min_score >= -128 && sc.nclasses >= 1 && sc.nclasses <= kLetters;
}

int cta16_blocks(int out_mode, int nclasses) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<std::tuple<int, int, int>, int> known;
  const auto key = std::make_tuple(dev, out_mode, nclasses);
  {
    std::lock_guard<std::mutex> g(mu);
    const auto it = known.find(key);
    if (it != known.end()) return it->second;
  }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = out_mode == kOutTrace ? fill::occ16_any<kOutTrace>(nclasses) : fill::occ16_any<kOutScore>(nclasses);
  if (per_sm * sms > 0) {
    std::lock_guard<std::mutex> g(mu);
    known[key] = per_sm * sms;
  }
  return per_sm * sms;
}

cudaError_t launch_cta16(int out_mode, const FillArgs &args, int blocks, cudaStream_t st) {
  FillArgs a = args;
  a.one = 1u;
  const int W = fill::cta16_warps(a.nclasses);
  const size_t smem = fill::cta16_smem_bytes(W, a.nclasses);
  if (out_mode == kOutTrace) {
    if (W == 16)
      fill::fill_cta16_kernel<kOutTrace, 16><<<blocks, 16 * 32, smem, st>>>(a);
    else
      fill::fill_cta16_kernel<kOutTrace, 8><<<blocks, 8 * 32, smem, st>>>(a);
  } else if (out_mode == kOutScore) {
    if (W == 16)
      fill::fill_cta16_kernel<kOutScore, 16><<<blocks, 16 * 32, smem, st>>>(a);
    else
      fill::fill_cta16_kernel<kOutScore, 8><<<blocks, 8 * 32, smem, st>>>(a);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tsq
