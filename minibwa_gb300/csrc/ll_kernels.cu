// ll_kernels.cu -- instantiations and launcher of the striped local-alignment kernel.
#include <cuda_runtime.h>
#include <atomic>
#include <map>
#include <mutex>
#include <utility>
#include "launch.h"
#include "ll.cuh"

namespace ksw2g {

typedef void (*ll_fn)(const ksw2g_ll_job *, int, const uint8_t *, const int8_t *, int, int, int, ksw2g_ll_result *,
                      uint64_t *, const int64_t *, int *);

static const int kSlen[] = {8, 16, 32, 64};
static const ll_fn kLL[2][4] = {{ll_kernel<1, 8>, ll_kernel<1, 16>, ll_kernel<1, 32>, ll_kernel<1, 64>},
                                {ll_kernel<2, 8>, ll_kernel<2, 16>, ll_kernel<2, 32>, ll_kernel<2, 64>}};
static const int kSlenD[] = {8, 16, 20, 24, 32, 48};
static const int kNumSlenD = 6;
static const ll_fn kLLD[2][kNumSlenD] = {
    {ll_dpx_kernel<1, 8>, ll_dpx_kernel<1, 16>, ll_dpx_kernel<1, 20>, ll_dpx_kernel<1, 24>, ll_dpx_kernel<1, 32>,
     ll_dpx_kernel<1, 48>},
    {ll_dpx_kernel<2, 8>, ll_dpx_kernel<2, 16>, ll_dpx_kernel<2, 20>, ll_dpx_kernel<2, 24>, ll_dpx_kernel<2, 32>,
     ll_dpx_kernel<2, 48>}};

// Segments of the longest query: the register-resident kernels hold 64; the
// shared-memory kernel holds as many as fit its block's shared memory.
static int wide_smem_cap() {
  static int cap = 0;
  if (!cap) {
    int d = 0, v = 0;
    cudaGetDevice(&d);
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, d) != cudaSuccess || v <= 0) v = 48 * 1024;
    cap = v;
  }
  return cap;
}
cudaError_t raise_smem_cap(const void *fn, size_t bytes) {
  static std::mutex mu;
  static std::map<std::pair<int, const void *>, size_t> cap;  // (device, kernel) -> cap set so far
  int d = 0;
  cudaError_t e = cudaGetDevice(&d);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  size_t &c = cap[std::make_pair(d, fn)];
  if (bytes <= c) return cudaSuccess;
  e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) c = bytes;
  return e;
}

static size_t wide_smem_bytes(int size, int m, int slen) {
  const int lanes = size == 1 ? 16 : 8;
  return (size_t)(m + 3) * slen * lanes * sizeof(int16_t);
}
int ll_slen_class(int slen) {
  for (int i = 0; i < kNumSlenD; ++i)
    if (slen <= kSlenD[i]) return i;
  return kNumSlenD;
}

int ll_slen_cap(int size, int m) {
  const size_t per = wide_smem_bytes(size, m, 1);  // bytes per segment
  const int s = (int)((size_t)wide_smem_cap() / (per ? per : 1));
  return s > 64 ? s : 64;
}

static cudaError_t launch_wide(int size, int slen_max, const LLLaunch &L, int max_blocks, cudaStream_t st) {
  typedef void (*wide_fn)(const ksw2g_ll_job *, int, const uint8_t *, const int8_t *, int, int, int,
                          ksw2g_ll_result *, uint64_t *, const int64_t *, int *, int);
  const wide_fn fn = size == 1 ? ll_wide_kernel<1> : ll_wide_kernel<2>;
  const size_t smem = wide_smem_bytes(size, L.m, slen_max);
  if (smem > (size_t)wide_smem_cap()) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_cap((const void *)fn, smem);
  if (e != cudaSuccess) return e;
  const int lanes = size == 1 ? 16 : 8;
  int occ = 0, sms = 0, d = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, lanes, smem);
  cudaGetDevice(&d);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
  int blocks = L.n_jobs;
  const int cap = sms * (occ > 0 ? occ : 1);
  if (blocks > cap) blocks = cap;
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  fn<<<blocks, lanes, smem, st>>>(L.jobs, L.n_jobs, L.arena, L.mat, L.m, L.gapo, L.gape, L.res, L.blist,
                                  L.blist_off, L.job_counter, slen_max);
  return cudaGetLastError();
}

bool ll_dpx_exact(int size, const LLLaunch &L) {
  if (size == 1) return true;
  const int goe = L.gapo + L.gape;
  if (L.gape < 0 || goe < 0 || goe > 32767) return false;
  const long long mpos = L.mat_max > 0 ? L.mat_max : 0;
  return ((long long)L.qlen_max + 1) * mpos <= 32767;
}

static cudaError_t launch_dpx(int size, int slen_max, const LLLaunch &L, int max_blocks, cudaStream_t st, bool &done) {
  done = false;
  int si = -1;
  for (int i = 0; i < kNumSlenD; ++i)
    if (slen_max <= kSlenD[i]) {
      si = i;
      break;
    }
  if (si < 0) return cudaSuccess;
  const ll_fn fn = kLLD[size - 1][si];
  const int T = size == 1 ? 8 : 4, groups = 128 / T;
  const size_t smem = ll_dpx_smem_bytes(L.m, kSlenD[si], T);
  if (smem > 200 * 1024) return cudaSuccess;
  if (smem > 48 * 1024) {
    cudaError_t e = raise_smem_cap((const void *)fn, smem);
    if (e != cudaSuccess) return e;
  }
  int occ = 0, sms = 0, d = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 128, smem);
  cudaGetDevice(&d);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
  int blocks = (L.n_jobs + groups - 1) / groups;
  const int cap = sms * (occ > 0 ? occ : 1);
  if (blocks > cap) blocks = cap;
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  fn<<<blocks, 128, smem, st>>>(L.jobs, L.n_jobs, L.arena, L.mat, L.m, L.gapo, L.gape, L.res, L.blist, L.blist_off,
                                L.job_counter);
  done = true;
  return cudaGetLastError();
}

cudaError_t launch_ll(int size, int slen_max, const LLLaunch &L, int max_blocks, cudaStream_t st, int force) {
  if (L.n_jobs <= 0) return cudaSuccess;
  if (force != 1 && (size == 1 || size == 2) && ll_dpx_exact(size, L)) {
    bool done = false;
    cudaError_t e = launch_dpx(size, slen_max, L, max_blocks, st, done);
    if (e != cudaSuccess || done) return e;
  }
  if (size != 1 && size != 2) return cudaErrorInvalidValue;
  int si = -1;
  for (int i = 0; i < 4; ++i)
    if (slen_max <= kSlen[i]) {
      si = i;
      break;
    }
  if (si < 0) return launch_wide(size, slen_max, L, max_blocks, st);
  const ll_fn fn = kLL[size - 1][si];
  const int lanes = size == 1 ? 16 : 8, groups = 128 / lanes;
  const size_t smem = (size_t)groups * (L.m * kSlen[si] * lanes + 8) * sizeof(int16_t);
  static std::atomic<int> occ[2][4][17] = {};  // computed once, by whichever thread comes first
  static std::atomic<int> sms_seen{0};
  const int mi = L.m < 16 ? L.m : 16;
  if (smem > 48 * 1024) {
    cudaError_t e = raise_smem_cap((const void *)fn, smem);
    if (e != cudaSuccess) return e;
  }
  if (!occ[size - 1][si][mi].load(std::memory_order_relaxed)) {
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, 128, smem);
    occ[size - 1][si][mi].store(o > 0 ? o : 1, std::memory_order_relaxed);
  }
  int sms = sms_seen.load(std::memory_order_relaxed);
  if (!sms) {
    int d = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
    sms_seen.store(sms, std::memory_order_relaxed);
  }
  int blocks = (L.n_jobs + groups - 1) / groups;
  const int cap = sms * occ[size - 1][si][mi];
  if (blocks > cap) blocks = cap;
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  fn<<<blocks, 128, smem, st>>>(L.jobs, L.n_jobs, L.arena, L.mat, L.m, L.gapo, L.gape, L.res, L.blist, L.blist_off,
                                L.job_counter);
  return cudaGetLastError();
}

}  // namespace ksw2g
