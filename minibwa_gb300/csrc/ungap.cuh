// ungap.cuh -- mb_ungap (pe.c:209-247) on the device: the 7-mer Hough transform
// that mate rescue runs on every candidate window before ksw_ll.  Included by
// rescue.cu and by the CPU emulator of the tests.
#pragma once
#include <stdint.h>

#ifndef KSW2G_BLOCK_SHARED  // block-shared variables (statics in the host emulation)
#ifdef KSW2G_EMU
#define KSW2G_BLOCK_SHARED static
#else
#define KSW2G_BLOCK_SHARED __shared__
#endif
#endif

namespace ksw2g {

constexpr int kUngapThreads = 128;
constexpr int kUngapK = 7, kUngapCap = 1 << (2 * kUngapK);
constexpr size_t kUngapTable = (size_t)kUngapCap * 2;  // bytes of the k-mer table
constexpr size_t kUngapSmemMax = 200 * 1024;           // shared histogram up to (this - table) / 4 diagonals

struct UngapJob {
  int64_t qoff, toff;  // read in the read arena; window in the window arena
  int32_t qlen, tlen, meth, pad;
};
struct UngapRes {
  int32_t max, max_i, n_good, n_kmer;
};

__device__ __forceinline__ uint32_t meth_base(int mt, uint32_t c) {
  // c2t = {0, 3, 2, 3}, g2a = {0, 1, 0, 3} (pe.c:211-212)
  return mt == 1 ? (c == 1 ? 3 : c) : mt == 2 ? (c == 2 ? 0 : c) : c;
}

// Persistent over candidates, one block at a time.  Dynamic shared memory: the
// k-mer table, then (when ghist is null) the diagonal histogram of the window;
// with ghist each block uses its own hist_cap slice of it.
__global__ void __launch_bounds__(kUngapThreads)
ungap_kernel(int n, const UngapJob *__restrict__ jobs, const uint8_t *__restrict__ qarena,
             const uint8_t *__restrict__ tarena, UngapRes *__restrict__ res, int *__restrict__ counter,
             int32_t *__restrict__ ghist, int64_t hist_cap) {
  extern __shared__ uint32_t ug_smem[];
  uint16_t *h = (uint16_t *)ug_smem;
  int32_t *a = ghist ? ghist + (size_t)blockIdx.x * hist_cap : (int32_t *)(ug_smem + kUngapCap / 2);
  KSW2G_BLOCK_SHARED int s_job, s_nk, s_max, s_mi, s_ng;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_job = atomicAdd(counter, 1);
    __syncthreads();
    const int j = s_job;
    __syncthreads();
    if (j >= n) return;
    const UngapJob J = jobs[j];
    const uint8_t *q = qarena + J.qoff, *t = tarena + J.toff;
    const int mt = J.meth, tl = J.tlen;
    if (J.qlen >= 65535) {  // positions no longer fit the uint16 table
      if (tid == 0) res[j] = UngapRes{0, -1, 0, 0};
      continue;
    }
    for (int i = tid; i < kUngapCap / 2; i += kUngapThreads) ug_smem[i] = 0;
    for (int i = tid; i < tl; i += kUngapThreads) a[i] = 0;
    __syncthreads();
    if (tid == 0) {
      int l = 0, nk = 0;
      uint32_t x = 0;
      for (int i = 0; i < J.qlen; ++i) {
        const uint32_t c0 = q[i];
        if (c0 < 4) {
          x = ((x << 2) | meth_base(mt, c0)) & (kUngapCap - 1);
          if (++l >= kUngapK) {
            if (h[x] == 0) ++nk;
            h[x] = (uint16_t)i;
          }
        } else x = 0, l = 0;
      }
      s_nk = nk, s_max = 0, s_mi = 0x7fffffff, s_ng = 0;
    }
    __syncthreads();
    // target position i closes a k-mer when bases i-6..i are all A/C/G/T
    for (int i = kUngapK - 1 + tid; i < tl; i += kUngapThreads) {
      uint32_t x = 0;
      bool ok = true;
#pragma unroll
      for (int k = kUngapK - 1; k >= 0; --k) {
        const uint32_t c0 = t[i - k];
        ok &= c0 < 4;
        x = (x << 2) | meth_base(mt, c0 & 3);
      }
      if (!ok) continue;
      const int hx = h[x];
      if (hx > 0 && i >= hx) atomicAdd(&a[i - hx], 1);
    }
    __syncthreads();
    int lm = 0, li = 0x7fffffff;
    for (int i = tid; i < tl; i += kUngapThreads)
      if (a[i] > lm) lm = a[i], li = i;  // this thread's first index of its maximum
    atomicMax(&s_max, lm);
    __syncthreads();
    const int mx = s_max;
    if (mx > 0 && lm == mx) atomicMin(&s_mi, li);
    int ng = 0;
    for (int i = tid; i < tl; i += kUngapThreads) ng += a[i] > (mx >> 1);
    atomicAdd(&s_ng, ng);
    __syncthreads();
    if (tid == 0) res[j] = UngapRes{mx, mx > 0 ? s_mi : -1, s_ng, s_nk};
    __syncthreads();
  }
}

}  // namespace ksw2g
