// launch.h -- host-side entry points of the kernels (C++; used by the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "ksw2g.h"
#include "shapes.h"

namespace ksw2g {

// Raises a kernel's dynamic shared-memory cap on the current device to at least `bytes` and
// never lowers it.  The attribute belongs to the function, process-wide: a launch that set it
// to its own need could lower it under a concurrent launch of the same kernel from another
// thread (the per-call drop-in runs one stream per caller thread), which then fails with an
// invalid argument.
cudaError_t raise_smem_cap(const void *fn, size_t bytes);

// Thread-group shapes instantiated for the extension DP kernel.  A pair with
// n_col_ 16-byte blocks per anti-diagonal needs G*K >= 4*n_col_ words.
struct ExtShape {
  int G, K;
};
constexpr int kNumExtShapes = KSW2G_NUM_SHAPES;
extern const ExtShape kExtShapes[kNumExtShapes];

// Smallest instantiated shape index able to hold n_col_ blocks, or -1.
int ext_shape_for(int n_col);
// Autotuner preference for n_col_: a shape code, where codes kNumExtShapes + s select the
// 16-bit-lane kernel of shape s (ksw2g_ext_set_shape).
void ext_shape_set_pref(int dual, int mode, int n_col_lo, int n_col_hi, int code);

struct ExtLaunch {
  const ksw2g_job *jobs;
  const int32_t *order;
  int n_jobs;
  const uint8_t *arena;
  ksw2g_ext_result *res;
  ksw2g_bt *bts;
  uint8_t *tb_pool;
  const int64_t *tb_off;
  int *job_counter;
  // wide-band bins only: wide_blocks per-block scratch areas of wide_stride bytes
  uint8_t *wide_scratch = nullptr;
  int64_t wide_stride = 0;
  int wide_blocks = 0;
};
// Bands wider than the widest thread-group shape run on the block-wide kernel
// (ext_wide.cuh); bins and launches use this virtual shape index for them.
constexpr int kWideShape = KSW2G_NUM_SHAPES;

cudaError_t launch_ext_wide(const ksw2g_ext_params &P, const ExtLaunch &L, cudaStream_t st);
int64_t ext_wide_scratch(int qlen, int tlen);

// The 16-bit-lane (DPX) kernels of the same (G, K) shapes have the shape ids kExt16Base + s.
constexpr int kExt16Base = KSW2G_NUM_SHAPES + 1;
// The block-split kernel's shapes (ext_split.cuh) have the shape ids kSplitBase + s.
struct SplitShape {
  int NW, K;
};
constexpr int kNumSplitShapes = KSW2G_NUM_SPLIT_SHAPES;
extern const SplitShape kSplitShapes[kNumSplitShapes];
constexpr int kSplitBase = 2 * KSW2G_NUM_SHAPES + 1;
constexpr int kNumShapeIds = kSplitBase + KSW2G_NUM_SPLIT_SHAPES;
// Smallest split shape able to hold n_col_ blocks, or -1.
int ext_split_for(int n_col);
cudaError_t launch_ext_split_z2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                                cudaStream_t st);
cudaError_t launch_ext_split_d2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                                cudaStream_t st);
cudaError_t launch_ext16_dp_z2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                               cudaStream_t st);
cudaError_t launch_ext16_dp_d2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                               cudaStream_t st);
// Shape id of a job of n_col_ blocks under scoring P: the autotuner's preference (or the
// smallest byte-lane shape that holds the band), the lane width forced by
// ksw2g_ext_set_family if any, 16-bit lanes only where ext16_params_ok; kWideShape for
// bands wider than every shape.
int ext_shape_id(int dual, int mode, int n_col, const ksw2g_ext_params &P);

// Launch the DP kernel of (dual, mode, shape id) as a persistent grid.
cudaError_t launch_ext_dp(int dual, int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L,
                          int max_blocks, cudaStream_t st);
cudaError_t launch_ext_bt(const ksw2g_job *jobs, const int32_t *order, int n_jobs, const ksw2g_bt *bts,
                          uint8_t *tb_pool,
                          const int64_t *tb_off, ksw2g_ext_result *res, uint32_t *cigar_out,
                          unsigned long long *cursor, long long cigar_cap, int *err, cudaStream_t st);
// Index of the smallest segment count instantiated for the DPX ksw_ll kernels that holds `slen`
// segments (6 classes; 6 = beyond them).  Jobs of one class share a kernel instance.
int ll_slen_class(int slen);
cudaError_t launch_pack(int n, const uint8_t *raw, const int64_t *raw_off, const int32_t *len, uint8_t *arena,
                        const int64_t *dst_off, cudaStream_t st);

// ksw_ll (striped local SW)
struct LLLaunch {
  const ksw2g_ll_job *jobs;
  int n_jobs;
  const uint8_t *arena;
  const int8_t *mat;
  int m;
  int gapo, gape;
  ksw2g_ll_result *res;
  uint64_t *blist;          // per-job second-best scratch (KSW_LL_SUBO), may be null
  const int64_t *blist_off;
  int *job_counter;
  int qlen_max;             // longest query of the launch
  int mat_max;              // largest matrix entry
};
// Picks the DPX kernel (two lanes per thread) when it is exact for the
// launch -- always for u8; for i16 when no H value can reach 32767 and the gap
// costs are in [0, 32767] -- else the one-lane-per-thread kernel.
// force: 0 automatic, 1 one lane per thread, 2 DPX (only where exact).
cudaError_t launch_ll(int size, int slen_max, const LLLaunch &L, int max_blocks, cudaStream_t st, int force = 0);
bool ll_dpx_exact(int size, const LLLaunch &L);
// Longest ksw_ll query, in segments, the kernels take for an alphabet of m.
int ll_slen_cap(int size, int m);

int num_sms(int device);

}  // namespace ksw2g
