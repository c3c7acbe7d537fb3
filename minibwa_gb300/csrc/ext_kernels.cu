// ext_kernels.cu -- instantiations and launchers of the extension kernels.
// Compiled once per (VAR) via -DKSW2G_EXT_VAR=0/1 so the two halves build in parallel.
#include <cuda_runtime.h>
#include <atomic>

#include "ext_dp.cuh"
#include "ext_split.cuh"
#include "launch.h"
#include "shapes.h"

#ifndef KSW2G_EXT_VAR
#define KSW2G_EXT_VAR 0
#endif
#if KSW2G_EXT_VAR == 0
#include "ext_bt.cuh"    // the backtrack and packing kernels live in the extz2 half only
#include "ext_wide.cuh"  // and so does the block-wide kernel (both variants, runtime dual)
#endif

namespace ksw2g {


typedef void (*ext_fn)(const ksw2g_job *, const int32_t *, int, const uint8_t *, const ksw2g_ext_params,
                       ksw2g_ext_result *, ksw2g_bt *, uint8_t *, const int64_t *, int *);

#define KSW2G_ROW(i, G, K) \
  {ext_dp_kernel<KSW2G_EXT_VAR, 0, G, K>, ext_dp_kernel<KSW2G_EXT_VAR, 1, G, K>, ext_dp_kernel<KSW2G_EXT_VAR, 2, G, K>},
static const ext_fn kTable[kNumExtShapes][3] = {KSW2G_SHAPES(KSW2G_ROW)};
#undef KSW2G_ROW

#if KSW2G_EXT_VAR == 0
#define KSW2G_SHAPE(i, G, K) {G, K},
const ExtShape kExtShapes[kNumExtShapes] = {KSW2G_SHAPES(KSW2G_SHAPE)};
const SplitShape kSplitShapes[kNumSplitShapes] = {KSW2G_SPLIT_SHAPES(KSW2G_SHAPE)};
#undef KSW2G_SHAPE

int ext_split_for(int n_col) {
  for (int i = 0; i < kNumSplitShapes; ++i)
    if (32 * kSplitShapes[i].NW * kSplitShapes[i].K >= 4 * n_col) return i;
  return -1;
}

int ext_shape_for(int n_col) {
  for (int i = 0; i < kNumExtShapes; ++i)
    if (kExtShapes[i].G * kExtShapes[i].K >= 4 * n_col) return i;
  return -1;
}

cudaError_t launch_ext_bt(const ksw2g_job *jobs, const int32_t *order, int n_jobs, const ksw2g_bt *bts,
                          uint8_t *tb_pool, const int64_t *tb_off, ksw2g_ext_result *res, uint32_t *cigar_out,
                          unsigned long long *cursor, long long cigar_cap, int *err, cudaStream_t st) {
  if (n_jobs <= 0) return cudaSuccess;
  const int bs = 128;
  ext_bt_kernel<<<(n_jobs + bs - 1) / bs, bs, 0, st>>>(jobs, order, n_jobs, bts, tb_pool, tb_off, res, cigar_out,
                                                        cursor, cigar_cap, err);
  return cudaGetLastError();
}

cudaError_t launch_pack(int n, const uint8_t *raw, const int64_t *raw_off, const int32_t *len, uint8_t *arena,
                        const int64_t *dst_off, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int bs = 256;
  int blocks = (int)(((int64_t)n * 32 + bs - 1) / bs);
  if (blocks > 65535 * 8) blocks = 65535 * 8;
  pack_seqs_kernel<<<blocks, bs, 0, st>>>(n, raw, raw_off, len, arena, dst_off);
  return cudaGetLastError();
}

int64_t ext_wide_scratch(int qlen, int tlen) { return (ext_wide_scratch_bytes(qlen, tlen) + 255) & ~(int64_t)255; }

cudaError_t launch_ext_wide(const ksw2g_ext_params &P, const ExtLaunch &L, cudaStream_t st) {
  if (L.n_jobs <= 0) return cudaSuccess;
  if (!L.wide_scratch || L.wide_blocks <= 0) return cudaErrorInvalidValue;
  const int blocks = L.n_jobs < L.wide_blocks ? L.n_jobs : L.wide_blocks;
  ext_wide_kernel<<<blocks, kWideThreads, 0, st>>>(L.jobs, L.order, L.n_jobs, L.arena, P, L.res, L.bts, L.tb_pool,
                                                   L.tb_off, L.job_counter, L.wide_scratch, L.wide_stride);
  return cudaGetLastError();
}

int num_sms(int device) {
  int v = 0;
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
  return v;
}
#endif

#if KSW2G_EXT_VAR == 0
cudaError_t launch_ext_dp_z2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                             cudaStream_t st)
#else
cudaError_t launch_ext_dp_d2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                             cudaStream_t st)
#endif
{
  if (L.n_jobs <= 0) return cudaSuccess;
  if (shape < 0 || shape >= kNumExtShapes || mode < 0 || mode > 2) return cudaErrorInvalidValue;
  const ext_fn fn = kTable[shape][mode];
  static int occ[kNumExtShapes][3] = {};
  static int dev_sms = 0;
  if (!occ[shape][mode]) {
    int o = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, 128, 0);
    occ[shape][mode] = o > 0 ? o : 1;
  }
  if (!dev_sms) {
    int d = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, d);
  }
  const int G = kExtShapes[shape].G;
  const int groups_per_block = 128 / G;
  int blocks = (L.n_jobs + groups_per_block - 1) / groups_per_block;
  const int cap = dev_sms * occ[shape][mode];
  if (blocks > cap) blocks = cap;
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  fn<<<blocks, 128, 0, st>>>(L.jobs, L.order, L.n_jobs, L.arena, P, L.res, L.bts, L.tb_pool, L.tb_off,
                             L.job_counter);
  return cudaGetLastError();
}

// block-split kernel, one instance per words a thread; the block's warps come from the launch
static const ext_fn kSplitTable[3][3] = {
    {ext_split_kernel<KSW2G_EXT_VAR, 0, 1>, ext_split_kernel<KSW2G_EXT_VAR, 1, 1>, ext_split_kernel<KSW2G_EXT_VAR, 2, 1>},
    {ext_split_kernel<KSW2G_EXT_VAR, 0, 2>, ext_split_kernel<KSW2G_EXT_VAR, 1, 2>, ext_split_kernel<KSW2G_EXT_VAR, 2, 2>},
    {ext_split_kernel<KSW2G_EXT_VAR, 0, 4>, ext_split_kernel<KSW2G_EXT_VAR, 1, 4>, ext_split_kernel<KSW2G_EXT_VAR, 2, 4>}};

#if KSW2G_EXT_VAR == 0
cudaError_t launch_ext_split_z2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                                cudaStream_t st)
#else
cudaError_t launch_ext_split_d2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                                cudaStream_t st)
#endif
{
  if (L.n_jobs <= 0) return cudaSuccess;
  if (shape < 0 || shape >= kNumSplitShapes || mode < 0 || mode > 2) return cudaErrorInvalidValue;
  const int NW = kSplitShapes[shape].NW, K = kSplitShapes[shape].K;
  const int ki = K == 1 ? 0 : K == 2 ? 1 : 2;
  if (NW < 1 || NW > kSplitMaxWarps || (K != 1 && K != 2 && K != 4)) return cudaErrorInvalidValue;
  const ext_fn fn = kSplitTable[ki][mode];
  // resident blocks per SM of every (shape, mode), and the device's SMs, found once (callers
  // on several host threads may race here; they store the same values)
  static std::atomic<int> occ[kNumSplitShapes][3];
  static std::atomic<int> dev_sms{0};
  int o = occ[shape][mode].load(std::memory_order_relaxed);
  if (!o) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, fn, 32 * NW, 0);
    o = o > 0 ? o : 1;
    occ[shape][mode].store(o, std::memory_order_relaxed);
  }
  int sms = dev_sms.load(std::memory_order_relaxed);
  if (!sms) {
    int d = 0;
    cudaGetDevice(&d);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d);
    dev_sms.store(sms, std::memory_order_relaxed);
  }
  int blocks = L.n_jobs;
  if (blocks > sms * o) blocks = sms * o;
  if (max_blocks > 0 && blocks > max_blocks) blocks = max_blocks;
  fn<<<blocks, 32 * NW, 0, st>>>(L.jobs, L.order, L.n_jobs, L.arena, P, L.res, L.bts, L.tb_pool, L.tb_off,
                                 L.job_counter);
  return cudaGetLastError();
}

}  // namespace ksw2g
