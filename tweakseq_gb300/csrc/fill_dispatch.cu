// fill_dispatch.cu -- picks the fill kernel instantiation for a shape.
#include "fill_i32.cuh"

namespace tsq {
namespace fill {
template <int OUT>
cudaError_t launch_i32(const Shape &sh, bool local, const FillArgs &a, int blocks, size_t smem, cudaStream_t st);
template <int OUT>
int occupancy_i32(const Shape &sh, bool local, size_t smem);
template <int OUT>
bool has_i32(const Shape &sh);
}  // namespace fill

int fill_threads() { return fill::kThreads; }

size_t fill_smem_bytes(const Shape &sh) {
  return size_t(fill::kMatBytes) + size_t(kLetters) * fill::kThreads * sh.R;
}

bool shape_supported(const Shape &sh, int out_mode, bool local) {
  (void)local;
  if (sh.i16) return false;
  switch (out_mode) {
    case kOutScore: return fill::has_i32<kOutScore>(sh);
    case kOutIdent: return fill::has_i32<kOutIdent>(sh);
    case kOutTrace: return fill::has_i32<kOutTrace>(sh);
  }
  return false;
}

int fill_blocks(const Shape &sh, int out_mode, bool local) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = fill_smem_bytes(sh);
  int per_sm = 0;
  switch (out_mode) {
    case kOutScore: per_sm = fill::occupancy_i32<kOutScore>(sh, local, smem); break;
    case kOutIdent: per_sm = fill::occupancy_i32<kOutIdent>(sh, local, smem); break;
    case kOutTrace: per_sm = fill::occupancy_i32<kOutTrace>(sh, local, smem); break;
  }
  return per_sm * sms;
}

cudaError_t launch_fill(const Shape &sh, int out_mode, bool local, const FillArgs &a, int blocks,
                        cudaStream_t st) {
  const size_t smem = fill_smem_bytes(sh);
  switch (out_mode) {
    case kOutScore: return fill::launch_i32<kOutScore>(sh, local, a, blocks, smem, st);
    case kOutIdent: return fill::launch_i32<kOutIdent>(sh, local, a, blocks, smem, st);
    case kOutTrace: return fill::launch_i32<kOutTrace>(sh, local, a, blocks, smem, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tsq
