// ext16_kernels.cu -- instantiations and launchers of the 16-bit-lane (DPX) extension kernels.
// Compiled once per (VAR) via -DKSW2G_EXT_VAR=0/1 so the two halves build in parallel.
#include <cuda_runtime.h>
#include "ext16_dp.cuh"
#include "launch.h"
#include "shapes.h"

#ifndef KSW2G_EXT_VAR
#define KSW2G_EXT_VAR 0
#endif

namespace ksw2g {

typedef void (*ext16_fn)(const ksw2g_job *, const int32_t *, int, const uint8_t *, const ksw2g_ext_params,
                         ksw2g_ext_result *, ksw2g_bt *, uint8_t *, const int64_t *, int *);

#define KSW2G_ROW(i, G, K)                                                                      \
  {ext16_dp_kernel<KSW2G_EXT_VAR, 0, G, K>, ext16_dp_kernel<KSW2G_EXT_VAR, 1, G, K>,             \
   ext16_dp_kernel<KSW2G_EXT_VAR, 2, G, K>},
static const ext16_fn kTable16[kNumExtShapes][3] = {KSW2G_SHAPES(KSW2G_ROW)};
#undef KSW2G_ROW

#if KSW2G_EXT_VAR == 0
cudaError_t launch_ext16_dp_z2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                               cudaStream_t st)
#else
cudaError_t launch_ext16_dp_d2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                               cudaStream_t st)
#endif
{
  if (L.n_jobs <= 0) return cudaSuccess;
  if (shape < 0 || shape >= kNumExtShapes || mode < 0 || mode > 2) return cudaErrorInvalidValue;
  const ext16_fn fn = kTable16[shape][mode];
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

}  // namespace ksw2g
