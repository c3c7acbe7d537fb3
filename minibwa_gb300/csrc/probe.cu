// probe.cu -- measured integer-pipe peak used as the roofline denominator of
// the DP kernels (the measured peaks cover HBM copy and bf16 GEMM only).
//
// Each thread runs 8 independent chains of (IADD3, LOP3) pairs, so the SMs
// issue back-to-back integer instructions without dependency stalls; the
// result is written out so nothing is optimised away.
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ksw2_gb300.h"

namespace {
constexpr int kChains = 8;
constexpr int kIters = 4096;

__global__ void __launch_bounds__(256) int_peak_kernel(uint32_t seed, uint32_t *out) {
  uint32_t a[kChains], b[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) a[i] = seed ^ (threadIdx.x * 2654435761u + i), b[i] = seed + i * 97u;
#pragma unroll 4
  for (int it = 0; it < kIters; ++it) {
#pragma unroll
    for (int i = 0; i < kChains; ++i) {
      a[i] = a[i] + b[i] + 0x9e3779b9u;  // IADD3
      b[i] = (a[i] & 0x5bd1e995u) ^ b[i];  // LOP3
    }
  }
  uint32_t r = 0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) r ^= a[i] + b[i];
  if (r == 0x12345678u) out[blockIdx.x] = r;
}
}  // namespace

// Integer instructions per second (thread-level: one 32-bit op per lane per
// instruction) sustained by the device, best of 3 runs.
extern "C" int ksw2g_probe_int32_peak(int device, double *ops_per_s) {
  if (!ops_per_s) return KSW2G_E_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return KSW2G_E_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  uint32_t *out = nullptr;
  if (cudaMalloc(&out, sizeof(uint32_t) * sms * 64) != cudaSuccess) return KSW2G_E_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int blocks = sms * 8, threads = 256;
  int_peak_kernel<<<blocks, threads>>>(1u, out);  // warm-up
  double best = 0;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    int_peak_kernel<<<blocks, threads>>>(rep + 2u, out);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    // 2 instructions (IADD3 + LOP3) per chain per iteration per thread
    const double ops = (double)blocks * threads * kIters * kChains * 2.0;
    if (ms > 0 && ops / (ms * 1e-3) > best) best = ops / (ms * 1e-3);
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return KSW2G_E_CUDA;
  *ops_per_s = best;
  return 0;
}
