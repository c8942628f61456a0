// fill_i32_score.cu -- instantiations of the int32 fill for kOutScore
// (one translation unit per output mode so they compile in parallel).
#include "fill_i32.cuh"

namespace tsq {
namespace fill {

#define TSQ_I32_SHAPES(X) X(4, 8) X(8, 8) X(16, 8) X(32, 8)

template <int OUT>
cudaError_t launch_i32(const Shape &sh, bool local, const FillArgs &a, int blocks, size_t smem, cudaStream_t st);
template <int OUT>
int occupancy_i32(const Shape &sh, bool local, size_t smem);
template <int OUT>
bool has_i32(const Shape &sh);

template <int G, int R, bool L, int OUT>
static cudaError_t go(const FillArgs &a, int blocks, size_t smem, cudaStream_t st) {
  // The shared-memory opt-in is set by occ(), which the planner calls
  // before any launch (and outside stream capture).
  fill_i32_kernel<G, R, L, OUT><<<blocks, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

template <int G, int R, bool L, int OUT>
static int occ(size_t smem) {
  auto k = fill_i32_kernel<G, R, L, OUT>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, smem) != cudaSuccess) return 0;
  return nb;
}

template <>
cudaError_t launch_i32<kOutScore>(const Shape &sh, bool local, const FillArgs &a, int blocks, size_t smem,
                                    cudaStream_t st) {
#define X(G_, R_)                                                                 \
  if (sh.G == G_ && sh.R == R_)                                                   \
    return local ? go<G_, R_, true, kOutScore>(a, blocks, smem, st)             \
                 : go<G_, R_, false, kOutScore>(a, blocks, smem, st);
  TSQ_I32_SHAPES(X)
#undef X
  return cudaErrorInvalidValue;
}

template <>
int occupancy_i32<kOutScore>(const Shape &sh, bool local, size_t smem) {
#define X(G_, R_) \
  if (sh.G == G_ && sh.R == R_) return local ? occ<G_, R_, true, kOutScore>(smem) : occ<G_, R_, false, kOutScore>(smem);
  TSQ_I32_SHAPES(X)
#undef X
  return 0;
}

template <>
bool has_i32<kOutScore>(const Shape &sh) {
#define X(G_, R_) \
  if (sh.G == G_ && sh.R == R_) return true;
  TSQ_I32_SHAPES(X)
#undef X
  return false;
}

}  // namespace fill
}  // namespace tsq
