// fill_i16.cu -- the int16x2 score fills (plain and overflow-checked), the
// shared-memory size of every int16x2 fill and the overflow collector of
// the int32 re-run.
#include <algorithm>

#include "fill_i16.cuh"

namespace tsq {
namespace fill {

template cudaError_t launch_i16<kOutScore>(bool, bool, const FillArgs &, int, size_t, cudaStream_t);
template int occupancy_i16<kOutScore>(bool, bool, size_t);

size_t smem_i16(int out_mode, int nclasses) {
  return size_t(kMatBytes16) + smem16_prof_bytes(nclasses) + smem16_match_bytes(out_mode, nclasses) +
         size_t(kSlots16) * (smem16_top_stride(out_mode) + kCodeRing16 + kRingPad);
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
