// fill_dispatch.cu -- picks the fill kernel for an output mode and lane type.
#include <map>
#include <mutex>
#include <tuple>

#include "fill_i16.cuh"
#include "fill_i32.cuh"

namespace tsq {
namespace fill {
template <int OUT>
cudaError_t launch_i32(bool local, const FillArgs &a, int blocks, size_t smem, cudaStream_t st);
template <int OUT>
int occupancy_i32(bool local, size_t smem);
// The int16x2 fills are instantiated in their own translation units.
extern template cudaError_t launch_i16<kOutScore>(bool, bool, const FillArgs &, int, size_t, cudaStream_t);
extern template cudaError_t launch_i16<kOutTrace>(bool, bool, const FillArgs &, int, size_t, cudaStream_t);
extern template cudaError_t launch_i16<kOutIdent>(bool, bool, const FillArgs &, int, size_t, cudaStream_t);
extern template int occupancy_i16<kOutScore>(bool, bool, size_t);
extern template int occupancy_i16<kOutTrace>(bool, bool, size_t);
extern template int occupancy_i16<kOutIdent>(bool, bool, size_t);
}  // namespace fill

int fill_threads() { return fill::kThreads; }

size_t fill_smem_bytes(int R, int i16, int out_mode, int nclasses) {
  if (i16) return fill::smem_i16(out_mode, nclasses);
  const size_t top = out_mode == kOutIdent ? 16 : 8;
  return size_t(fill::kMatBytes) + size_t(kLetters) * fill::kThreads * size_t(R) +
         size_t(fill::kSlotsPerBlock) * (fill::kTopRing * top + fill::kCodeRing + 2 * fill::kRingPad);
}

size_t fill_bnd_entry_bytes(int i16, int out_mode) {
  if (i16) return out_mode == kOutIdent ? 16 : 4;
  return out_mode == kOutIdent ? 16 : 8;
}

int fill_threads_for(int i16) { return i16 ? fill::kThreads16 : fill::kThreads; }

bool shape_supported(const Shape &sh, int out_mode, bool local) {
  if (sh.R != 8) return false;
  if (sh.i16 && out_mode == kOutIdent && local) return false;
  return sh.G == 4 || sh.G == 8 || sh.G == 16 || sh.G == 32;
}

namespace {
int fill_blocks_uncached(int R, int i16, int out_mode, bool local, int nclasses);
}

// Resident blocks of a fill launch on the current device.  The occupancy
// queries (and the shared-memory attribute they set) cost far more than a
// plan's host work, so each answer is kept per device and kernel.
int fill_blocks(int R, int i16, int out_mode, bool local, int nclasses) {
  int dev = 0;
  cudaGetDevice(&dev);
  static std::mutex mu;
  static std::map<std::tuple<int, int, int, int, int, int>, int> known;
  const auto key = std::make_tuple(dev, R, i16, out_mode, int(local), i16 ? nclasses : 0);
  {
    std::lock_guard<std::mutex> g(mu);
    const auto it = known.find(key);
    if (it != known.end()) return it->second;
  }
  const int v = fill_blocks_uncached(R, i16, out_mode, local, nclasses);
  if (v > 0) {
    std::lock_guard<std::mutex> g(mu);
    known[key] = v;
  }
  return v;
}

namespace {
int fill_blocks_uncached(int R, int i16, int out_mode, bool local, int nclasses) {
  if (R != 8) return 0;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = fill_smem_bytes(R, i16, out_mode, nclasses);
  if (i16) {
    switch (out_mode) {
      case kOutScore: return fill::occupancy_i16<kOutScore>(i16 == 2, local, smem) * sms;
      case kOutTrace: return fill::occupancy_i16<kOutTrace>(i16 == 2, local, smem) * sms;
      case kOutIdent: return fill::occupancy_i16<kOutIdent>(i16 == 2, local, smem) * sms;
    }
    return 0;
  }
  int per_sm = 0;
  switch (out_mode) {
    case kOutScore: per_sm = fill::occupancy_i32<kOutScore>(local, smem); break;
    case kOutIdent: per_sm = fill::occupancy_i32<kOutIdent>(local, smem); break;
    case kOutTrace: per_sm = fill::occupancy_i32<kOutTrace>(local, smem); break;
  }
  return per_sm * sms;
}
}  // namespace

cudaError_t launch_fill(int R, int i16, int out_mode, bool local, const FillArgs &a, int blocks,
                        cudaStream_t st) {
  if (R != 8) return cudaErrorInvalidValue;
  const size_t smem = fill_smem_bytes(R, i16, out_mode, i16 ? a.nclasses : kLetters);
  if (i16) {
    switch (out_mode) {
      case kOutScore: return fill::launch_i16<kOutScore>(i16 == 2, local, a, blocks, smem, st);
      case kOutTrace: return fill::launch_i16<kOutTrace>(i16 == 2, local, a, blocks, smem, st);
      case kOutIdent: return fill::launch_i16<kOutIdent>(i16 == 2, local, a, blocks, smem, st);
    }
    return cudaErrorInvalidValue;
  }
  switch (out_mode) {
    case kOutScore: return fill::launch_i32<kOutScore>(local, a, blocks, smem, st);
    case kOutIdent: return fill::launch_i32<kOutIdent>(local, a, blocks, smem, st);
    case kOutTrace: return fill::launch_i32<kOutTrace>(local, a, blocks, smem, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tsq
