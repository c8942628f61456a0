// fill_cta.cu -- instantiations of the CTA-per-pair int32 fill.
#include <map>
#include <mutex>
#include <tuple>

#include "fill_cta.cuh"

namespace tsq {
namespace fill {

namespace {
template <bool LOCAL, int OUT>
constexpr int kW = cta_warps(OUT, LOCAL);

template <int OUT>
cudaError_t go(bool local, const FillArgs &a, int blocks, cudaStream_t st) {
  if (local)
    fill_cta_kernel<true, OUT, kW<true, OUT>><<<blocks, kW<true, OUT> * 32, cta_smem_bytes(OUT, kW<true, OUT>), st>>>(a);
  else
    fill_cta_kernel<false, OUT, kW<false, OUT>>
        <<<blocks, kW<false, OUT> * 32, cta_smem_bytes(OUT, kW<false, OUT>), st>>>(a);
  return cudaGetLastError();
}

template <int OUT>
int occ(bool local) {
  const int W = cta_warps(OUT, local);
  const size_t smem = cta_smem_bytes(OUT, W);
  auto k = local ? fill_cta_kernel<true, OUT, kW<true, OUT>> : fill_cta_kernel<false, OUT, kW<false, OUT>>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, W * 32, smem) != cudaSuccess) return 0;
  return nb;
}
}  // namespace

}  // namespace fill

// Resident CTAs of the long-pair fill on the current device (occupancy
// queries cached per device and kernel, as for the warp fills).
int cta_blocks(int out_mode, bool local) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<std::tuple<int, int, int>, int> known;
  const auto key = std::make_tuple(dev, out_mode, int(local));
  {
    std::lock_guard<std::mutex> g(mu);
    const auto it = known.find(key);
    if (it != known.end()) return it->second;
  }
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int per_sm = 0;
  switch (out_mode) {
    case kOutScore: per_sm = fill::occ<kOutScore>(local); break;
    case kOutIdent: per_sm = fill::occ<kOutIdent>(local); break;
    case kOutTrace: per_sm = fill::occ<kOutTrace>(local); break;
  }
  if (per_sm * sms > 0) {
    std::lock_guard<std::mutex> g(mu);
    known[key] = per_sm * sms;
  }
  return per_sm * sms;
}

size_t cta_bnd_entry_bytes(int out_mode) { return out_mode == kOutIdent ? 16 : 8; }

cudaError_t launch_cta(int out_mode, bool local, const FillArgs &a, int blocks, cudaStream_t st) {
  switch (out_mode) {
    case kOutScore: return fill::go<kOutScore>(local, a, blocks, st);
    case kOutIdent: return fill::go<kOutIdent>(local, a, blocks, st);
    case kOutTrace: return fill::go<kOutTrace>(local, a, blocks, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tsq
