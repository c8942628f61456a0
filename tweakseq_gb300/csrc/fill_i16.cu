// fill_i16.cu -- the int16x2 score fills (plain and overflow-checked) and
// the overflow collector of the int32 re-run.
#include <algorithm>

#include "fill_i16.cuh"

namespace tsq {
namespace fill {

cudaError_t launch_i16(bool check, bool local, const FillArgs &args, int blocks, size_t smem, cudaStream_t st) {
  FillArgs a = args;
  a.one = 1u;
  if (check) {
    if (local)
      fill_i16_kernel<true, true><<<blocks, kThreads16, smem, st>>>(a);
    else
      fill_i16_kernel<false, true><<<blocks, kThreads16, smem, st>>>(a);
  } else {
    if (local)
      fill_i16_kernel<true, false><<<blocks, kThreads16, smem, st>>>(a);
    else
      fill_i16_kernel<false, false><<<blocks, kThreads16, smem, st>>>(a);
  }
  return cudaGetLastError();
}

size_t smem_i16(int nclasses);

int occupancy_i16(bool check, bool local, size_t smem) {
  auto k = check ? (local ? fill_i16_kernel<true, true> : fill_i16_kernel<false, true>)
                 : (local ? fill_i16_kernel<true, false> : fill_i16_kernel<false, false>);
  // The attribute allows the largest profile (26 classes), so that every
  // scheme's launch fits whatever scheme was sized first.
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(std::max(smem, smem_i16(kLetters)))) !=
      cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads16, smem) != cudaSuccess) return 0;
  return nb;
}

size_t smem_i16(int nclasses) {
  return size_t(kMatBytes16) + size_t(2 * nclasses) * kThreads16 * sizeof(uint2) +
         size_t(kSlots16) * (kTopRing * sizeof(uint32_t) + kCodeRing16 + 2 * kRingPad);
}

namespace {
__global__ void collect_overflow_kernel(const int32_t *checked, int32_t n_checked, const int32_t *overflow,
                                        const int32_t *pair_g, int32_t *rerun_tasks, int2 *rerun_wtasks,
                                        int32_t *rerun_count) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n_checked) return;
  const int32_t pid = checked[k];
  if (!overflow[pid]) return;
  const int32_t slot = atomicAdd(rerun_count, 1);
  rerun_tasks[slot] = pid;
  rerun_wtasks[slot] = make_int2(slot, (pair_g[pid] << 16) | 1);
}
}  // namespace

}  // namespace fill

cudaError_t launch_collect_overflow(const int32_t *checked, int32_t n_checked, const int32_t *overflow,
                                    const int32_t *pair_g, int32_t *rerun_tasks, int2 *rerun_wtasks,
                                    int32_t *rerun_count, cudaStream_t st) {
  if (n_checked <= 0) return cudaSuccess;
  fill::collect_overflow_kernel<<<(n_checked + 255) / 256, 256, 0, st>>>(checked, n_checked, overflow, pair_g,
                                                                          rerun_tasks, rerun_wtasks, rerun_count);
  return cudaGetLastError();
}

}  // namespace tsq
