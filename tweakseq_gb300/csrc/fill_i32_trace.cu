// fill_i32_trace.cu -- the int32 fill for kOutTrace (one translation
// unit per output mode so they compile in parallel).
#include "fill_i32.cuh"

namespace tsq {
namespace fill {

template <int OUT>
cudaError_t launch_i32(bool local, const FillArgs &a, int blocks, size_t smem, cudaStream_t st);
template <int OUT>
int occupancy_i32(bool local, size_t smem);

template <>
cudaError_t launch_i32<kOutTrace>(bool local, const FillArgs &a, int blocks, size_t smem, cudaStream_t st) {
  // The shared-memory opt-in is set by occupancy_i32, which the planner
  // calls before any launch (and outside stream capture).
  if (local)
    fill_i32_kernel<8, true, kOutTrace><<<blocks, kThreads, smem, st>>>(a);
  else
    fill_i32_kernel<8, false, kOutTrace><<<blocks, kThreads, smem, st>>>(a);
  return cudaGetLastError();
}

template <>
int occupancy_i32<kOutTrace>(bool local, size_t smem) {
  auto k = local ? fill_i32_kernel<8, true, kOutTrace> : fill_i32_kernel<8, false, kOutTrace>;
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, smem) != cudaSuccess) return 0;
  return nb;
}

}  // namespace fill
}  // namespace tsq
