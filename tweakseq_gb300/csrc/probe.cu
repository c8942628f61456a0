// probe.cu -- measured integer/DPX throughput of the device, the roofline
// denominator for the DP fill (which is bound by integer max/add issue, not
// by HBM or tensor cores).
//
// The probe runs the fill's inner operation mix -- add-then-max and
// three-way max, the two DPX forms a Gotoh cell needs -- on 8 independent
// chains per thread across a full grid, and reports instructions per second
// per lane.  Peak cells/s follows as rate * lanes_per_instruction / 4 (a
// cell is 4 DPX-class instructions: the E and F add-max, the diagonal add and
// the three-way max).
#include "tsq_internal.h"

namespace tsq {
namespace {

template <bool PACKED>
__global__ void dpx_probe_kernel(int iters, int32_t seed, int32_t *sink) {
  int32_t a[8], b = seed ^ threadIdx.x, c = seed + blockIdx.x;
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed * (k + 1) + threadIdx.x;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (PACKED) {
        a[k] = int32_t(__viaddmax_s16x2(uint32_t(a[k]), uint32_t(b), uint32_t(c)));
        a[k] = int32_t(__vimax3_s16x2(uint32_t(a[k]), uint32_t(c), uint32_t(b)));
      } else {
        a[k] = __viaddmax_s32(a[k], b, c);
        a[k] = __vimax3_s32(a[k], c, b);
      }
    }
  }
  int32_t x = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) x ^= a[k];
  if (x == 0x7fffffff) sink[threadIdx.x] = x;  // keeps the chains alive
}

}  // namespace
}  // namespace tsq

extern "C" int tsq_probe_dpx(int32_t packed, double *instr_per_s) {
  using namespace tsq;
  if (!instr_per_s) return TSQ_E_INVALID_ARG;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return TSQ_E_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return TSQ_E_CUDA;
  int32_t *sink = nullptr;
  if (cudaMalloc(&sink, 1024 * sizeof(int32_t)) != cudaSuccess) return TSQ_E_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int threads = 256, blocks = sms * 8, iters = 4096;
  float best = 1e30f;
  cudaError_t err = cudaSuccess;
  for (int rep = 0; rep < 4 && err == cudaSuccess; ++rep) {
    cudaEventRecord(e0);
    if (packed)
      dpx_probe_kernel<true><<<blocks, threads>>>(iters, 12345 + rep, sink);
    else
      dpx_probe_kernel<false><<<blocks, threads>>>(iters, 12345 + rep, sink);
    cudaEventRecord(e1);
    err = cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(sink);
  if (err != cudaSuccess) return TSQ_E_CUDA;
  const double instr = double(blocks) * threads * iters * 8 * 2;
  *instr_per_s = instr / (double(best) * 1e-3);
  return TSQ_OK;
}
