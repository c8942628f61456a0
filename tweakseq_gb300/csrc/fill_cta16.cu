// fill_cta16.cu -- instantiations and launcher of the int16x2 CTA fill.
#include <map>
#include <mutex>
#include <tuple>

#include "fill_cta16.cuh"

namespace tsq {
namespace fill {
namespace {

// Warps per CTA: 16 when the profile of the scheme's classes fits and the
// kernel fits 128 registers (global mode), else 8.
int cta16_warps(int nclasses, bool local) {
  return !local && cta16_smem_bytes(16, nclasses) <= size_t(227) * 1024 ? 16 : 8;
}

template <int OUT, int W, bool LOCAL>
int occ16(int nclasses) {
  const size_t smem = cta16_smem_bytes(W, nclasses);
  auto k = fill_cta16_kernel<OUT, W, LOCAL>;
  // The attribute allows the largest profile this W takes, so that a launch
  // fits whatever scheme was sized first.
  const size_t most = W == 16 ? size_t(227) * 1024 : cta16_smem_bytes(W, kLetters);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(most)) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, W * 32, smem) != cudaSuccess) return 0;
  return nb;
}

template <int OUT>
int occ16_any(int nclasses, bool local) {
  if (local) return occ16<OUT, 8, true>(nclasses);
  return cta16_warps(nclasses, false) == 16 ? occ16<OUT, 16, false>(nclasses) : occ16<OUT, 8, false>(nclasses);
}

template <int OUT>
void go16(bool local, const FillArgs &a, int blocks, cudaStream_t st) {
  const int W = cta16_warps(a.nclasses, local);
  const size_t smem = cta16_smem_bytes(W, a.nclasses);
  if (local)
    fill_cta16_kernel<OUT, 8, true><<<blocks, 8 * 32, smem, st>>>(a);
  else if (W == 16)
    fill_cta16_kernel<OUT, 16, false><<<blocks, 16 * 32, smem, st>>>(a);
  else
    fill_cta16_kernel<OUT, 8, false><<<blocks, 8 * 32, smem, st>>>(a);
}

}  // namespace
}  // namespace fill

bool cta16_supported(int out_mode, bool local, const Scheme &sc, int32_t gap_open, int32_t gap_extend) {
  (void)local;
  if (out_mode != kOutScore && out_mode != kOutTrace) return false;
  const int64_t step = int64_t(gap_open) + gap_extend + std::max(sc.max_score, 0);
  return step <= fill::kMaxStep16 && sc.min_score >= -128 && sc.nclasses >= 1 && sc.nclasses <= kLetters;
}

int cta16_blocks(int out_mode, bool local, int nclasses) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int>, int> known;
  const auto key = std::make_tuple(dev, out_mode, int(local), nclasses);
  {
    std::lock_guard<std::mutex> g(mu);
    const auto it = known.find(key);
    if (it != known.end()) return it->second;
  }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int per_sm = out_mode == kOutTrace ? fill::occ16_any<kOutTrace>(nclasses, local)
                                           : fill::occ16_any<kOutScore>(nclasses, local);
  if (per_sm * sms > 0) {
    std::lock_guard<std::mutex> g(mu);
    known[key] = per_sm * sms;
  }
  return per_sm * sms;
}

cudaError_t launch_cta16(int out_mode, bool local, const FillArgs &args, int blocks, cudaStream_t st) {
  FillArgs a = args;
  a.one = 1u;
  if (out_mode == kOutTrace)
    fill::go16<kOutTrace>(local, a, blocks, st);
  else if (out_mode == kOutScore)
    fill::go16<kOutScore>(local, a, blocks, st);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace tsq
