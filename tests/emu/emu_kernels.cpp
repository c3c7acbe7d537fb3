// emu_kernels.cpp -- the CUDA kernels of minibwa_gb300/csrc compiled for the
// host through cuda_emu.h (TEST INFRASTRUCTURE).  Lets the CPU test suite run
// the exact device code paths -- window sliding, shuffles, votes, lockstep
// groups, the work counter -- on small inputs without a GPU.
#include <chrono>
#include <thread>
#include <vector>

#include "cuda_emu.h"

thread_local emu_dim3 threadIdx, blockIdx;
emu_dim3 blockDim, gridDim;
namespace emu {
Warp *g_warps = nullptr;
Barrier *g_block = nullptr;
LaneState g_lane_state[1024];
}

#include "../../minibwa_gb300/csrc/ext_bt.cuh"
#include "../../minibwa_gb300/csrc/ext_dp.cuh"
#include "../../minibwa_gb300/csrc/ext16_dp.cuh"
#include "../../minibwa_gb300/csrc/ext_split.cuh"
#include "../../minibwa_gb300/csrc/ext_wide.cuh"
#include "../../minibwa_gb300/csrc/host_common.h"
#include "../../minibwa_gb300/csrc/ll.cuh"
#include "../../minibwa_gb300/csrc/shapes.h"
#include "../../minibwa_gb300/csrc/ungap.cuh"

namespace ksw2g {
alignas(16) int16_t ll_smem[1 << 20];
alignas(16) uint32_t lld_smem[1 << 20];
alignas(16) int16_t llw_smem[1 << 22];
alignas(16) uint32_t ug_smem[kUngapSmemMax / 4];
}

using namespace ksw2g;

template <class F>
static void run_block(int nthreads, F f) {
  blockDim.x = nthreads;
  gridDim.x = 1;
  std::vector<emu::Warp> warps((nthreads + 31) / 32);
  for (size_t w = 0; w < warps.size(); ++w) {
    const int n = std::min(32, nthreads - (int)w * 32);
    warps[w].present = n == 32 ? 0xffffffffu : ((1u << n) - 1u);
  }
  emu::g_warps = warps.data();
  emu::Barrier block_bar;
  block_bar.need = nthreads;
  emu::g_block = &block_bar;
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([=] {
      threadIdx.x = t;
      blockIdx.x = 0;
      f();
    });
  std::atomic<bool> fin{false};
  std::thread dog([&] {
    for (int i = 0; i < 100 && !fin; ++i) std::this_thread::sleep_for(std::chrono::milliseconds(50));
    if (fin) return;
    for (int t = 0; t < nthreads; ++t)
      fprintf(stderr, "[emu watchdog] thread %d last mask %08x calls %ld\n", t, emu::g_lane_state[t].mask.load(),
              emu::g_lane_state[t].calls.load());
  });
  for (auto &x : th) x.join();
  fin = true;
  dog.join();
}

typedef void (*ext_fn)(const ksw2g_job *, const int32_t *, int, const uint8_t *, const ksw2g_ext_params,
                       ksw2g_ext_result *, ksw2g_bt *, uint8_t *, const int64_t *, int *);
#define ROW(i, G, K) {{ext_dp_kernel<0, 0, G, K>, ext_dp_kernel<0, 1, G, K>, ext_dp_kernel<0, 2, G, K>}, \
                      {ext_dp_kernel<1, 0, G, K>, ext_dp_kernel<1, 1, G, K>, ext_dp_kernel<1, 2, G, K>}},
static const ext_fn kTab[KSW2G_NUM_SHAPES][2][3] = {KSW2G_SHAPES(ROW)};
#undef ROW
#define ROW(i, G, K) {{ext16_dp_kernel<0, 0, G, K>, ext16_dp_kernel<0, 1, G, K>, ext16_dp_kernel<0, 2, G, K>}, \
                      {ext16_dp_kernel<1, 0, G, K>, ext16_dp_kernel<1, 1, G, K>, ext16_dp_kernel<1, 2, G, K>}},
static const ext_fn kTab16[KSW2G_NUM_SHAPES][2][3] = {KSW2G_SHAPES(ROW)};
#undef ROW
#define SH(i, G, K) {G, K},
static const int kShape[KSW2G_NUM_SHAPES][2] = {KSW2G_SHAPES(SH)};
#undef SH

extern "C" {

int emu_num_shapes(void) { return KSW2G_NUM_SHAPES; }
int emu_shape_words(int s) { return kShape[s][0] * kShape[s][1]; }
int emu_shape_threads(int s) { return kShape[s][0]; }

void emu_derive_params(int dual, int m, const int8_t *mat, int q, int e, int q2, int e2, ksw2g_ext_params *P) {
  derive_ext_params(dual, (int8_t)m, mat, (int8_t)q, (int8_t)e, (int8_t)q2, (int8_t)e2, *P);
}

// Run the DP kernel of (dual, mode, shape) over all jobs with one emulated warp
// (`threads` lanes), then the backtrack kernel.  The arena must already be padded
// as the device arena is (32 zero bytes around every sequence).
int emu_ext(int dual, int mode, int shape, const ksw2g_ext_params *P, int n, const ksw2g_job *jobs,
            const uint8_t *arena, ksw2g_ext_result *res, ksw2g_bt *bts, uint8_t *tb_pool, const int64_t *tb_off,
            uint32_t *cigar, long long cap, int threads, int family) {
  if (shape < 0 || shape > KSW2G_NUM_SHAPES) return -1;
  int counter = 0;
  const ksw2g_ext_params Pc = *P;
  if (shape == KSW2G_NUM_SHAPES) {  // the block-wide kernel, one emulated block
    int64_t stride = 0;
    for (int j = 0; j < n; ++j) stride = std::max(stride, ext_wide_scratch_bytes(jobs[j].qlen, jobs[j].tlen));
    std::vector<uint8_t> scratch((size_t)stride + 256);
    uint8_t *sp = (uint8_t *)(((uintptr_t)scratch.data() + 255) & ~(uintptr_t)255);
    run_block(kWideThreads, [&] {
      ext_wide_kernel(jobs, nullptr, n, arena, Pc, res, bts, tb_pool, tb_off, &counter, sp, stride);
    });
  } else {
    const ext_fn f = family ? kTab16[shape][dual][mode] : kTab[shape][dual][mode];
    run_block(threads, [&] { f(jobs, nullptr, n, arena, Pc, res, bts, tb_pool, tb_off, &counter); });
  }
  if (mode != 0) {
    unsigned long long cursor = 0;
    int err = 0;
    blockDim.x = 1;
    for (int j = 0; j < n; ++j) {
      threadIdx.x = 0;
      blockIdx.x = j;
      ext_bt_kernel(jobs, nullptr, n, bts, tb_pool, tb_off, res, cigar, &cursor, cap, &err);
    }
    if (err) return -2;
  }
  return 0;
}

// The block-split kernel (ext_split.cuh) with one emulated block of 32*nw threads, k words a
// thread, then the backtrack kernel.
int emu_ext_split(int dual, int mode, int nw, int k, const ksw2g_ext_params *P, int n, const ksw2g_job *jobs,
                  const uint8_t *arena, ksw2g_ext_result *res, ksw2g_bt *bts, uint8_t *tb_pool,
                  const int64_t *tb_off, uint32_t *cigar, long long cap) {
  if (nw < 1 || nw > kSplitMaxWarps || (k != 1 && k != 2 && k != 4) || mode < 0 || mode > 2) return -1;
  static const ext_fn tab[2][3][3] = {
      {{ext_split_kernel<0, 0, 1>, ext_split_kernel<0, 1, 1>, ext_split_kernel<0, 2, 1>},
       {ext_split_kernel<0, 0, 2>, ext_split_kernel<0, 1, 2>, ext_split_kernel<0, 2, 2>},
       {ext_split_kernel<0, 0, 4>, ext_split_kernel<0, 1, 4>, ext_split_kernel<0, 2, 4>}},
      {{ext_split_kernel<1, 0, 1>, ext_split_kernel<1, 1, 1>, ext_split_kernel<1, 2, 1>},
       {ext_split_kernel<1, 0, 2>, ext_split_kernel<1, 1, 2>, ext_split_kernel<1, 2, 2>},
       {ext_split_kernel<1, 0, 4>, ext_split_kernel<1, 1, 4>, ext_split_kernel<1, 2, 4>}}};
  const ext_fn f = tab[dual ? 1 : 0][k == 1 ? 0 : k == 2 ? 1 : 2][mode];
  int counter = 0;
  const ksw2g_ext_params Pc = *P;
  run_block(32 * nw, [&] { f(jobs, nullptr, n, arena, Pc, res, bts, tb_pool, tb_off, &counter); });
  if (mode != 0) {
    unsigned long long cursor = 0;
    int err = 0;
    blockDim.x = 1;
    for (int j = 0; j < n; ++j) {
      threadIdx.x = 0;
      blockIdx.x = j;
      ext_bt_kernel(jobs, nullptr, n, bts, tb_pool, tb_off, res, cigar, &cursor, cap, &err);
    }
    if (err) return -2;
  }
  return 0;
}

int emu_ll(int size, int slen_max, int n, const ksw2g_ll_job *jobs, const uint8_t *arena, const int8_t *mat, int m,
           int gapo, int gape, ksw2g_ll_result *res, uint64_t *blist, const int64_t *blist_off, int threads,
           int dpx) {
  int counter = 0;
  typedef void (*ll_fn)(const ksw2g_ll_job *, int, const uint8_t *, const int8_t *, int, int, int,
                        ksw2g_ll_result *, uint64_t *, const int64_t *, int *);
  ll_fn f = nullptr;
  const int sl[] = {8, 16, 32, 64};
  const ll_fn t1[] = {ll_kernel<1, 8>, ll_kernel<1, 16>, ll_kernel<1, 32>, ll_kernel<1, 64>};
  const ll_fn t2[] = {ll_kernel<2, 8>, ll_kernel<2, 16>, ll_kernel<2, 32>, ll_kernel<2, 64>};
  for (int i = 0; i < 4; ++i)
    if (slen_max <= sl[i]) {
      f = size == 1 ? t1[i] : t2[i];
      break;
    }
  if (dpx) {
    const int sd[] = {8, 16, 20, 24, 32, 48};
    const ll_fn d1[] = {ll_dpx_kernel<1, 8>,  ll_dpx_kernel<1, 16>, ll_dpx_kernel<1, 20>,
                        ll_dpx_kernel<1, 24>, ll_dpx_kernel<1, 32>, ll_dpx_kernel<1, 48>};
    const ll_fn d2[] = {ll_dpx_kernel<2, 8>,  ll_dpx_kernel<2, 16>, ll_dpx_kernel<2, 20>,
                        ll_dpx_kernel<2, 24>, ll_dpx_kernel<2, 32>, ll_dpx_kernel<2, 48>};
    f = nullptr;
    for (int i = 0; i < 6; ++i)
      if (slen_max <= sd[i]) {
        f = size == 1 ? d1[i] : d2[i];
        break;
      }
    threads = (size == 1 ? 8 : 4) * (threads / (size == 1 ? 16 : 8));
  }
  if (!f && !dpx && slen_max > 64) {  // long queries: the shared-memory kernel, one job per LANES threads
    const int lanes = size == 1 ? 16 : 8;
    if ((size_t)(m + 3) * slen_max * lanes > sizeof(llw_smem) / sizeof(int16_t)) return -3;
    run_block(lanes, [&] {
      if (size == 1) ll_wide_kernel<1>(jobs, n, arena, mat, m, gapo, gape, res, blist, blist_off, &counter, slen_max);
      else ll_wide_kernel<2>(jobs, n, arena, mat, m, gapo, gape, res, blist, blist_off, &counter, slen_max);
    });
    return 0;
  }
  if (!f) return -1;
  run_block(threads, [&] { f(jobs, n, arena, mat, m, gapo, gape, res, blist, blist_off, &counter); });
  return 0;
}

// mb_ungap of every job with one emulated block (shared-memory histogram when
// ghist is null, else ghist[0, hist_cap)).
int emu_ungap(int n, const UngapJob *jobs, const uint8_t *qarena, const uint8_t *tarena, UngapRes *res,
              int32_t *ghist, long long hist_cap) {
  int counter = 0;
  run_block(kUngapThreads, [&] { ungap_kernel(n, jobs, qarena, tarena, res, &counter, ghist, hist_cap); });
  return 0;
}
}
