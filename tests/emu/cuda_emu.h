// cuda_emu.h -- host emulation of the CUDA built-ins used by the kernels in
// minibwa_gb300/csrc, so the same kernel source can be compiled with g++ and
// run on the CPU by the tests (TEST INFRASTRUCTURE: the product never does this).
//
// One emulated block = blockDim.x std::threads.  Warp collectives
// (__shfl*_sync, __all_sync, __ballot_sync, __syncwarp) synchronise exactly the
// lanes named in their mask, through a per-(warp, mask) barrier, with the
// semantics of the CUDA C++ programming guide.  __byte_perm uses only the
// documented selector bits (2:0 of each nibble), so device code that relies on
// anything else shows up here as a wrong result.
#pragma once
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <condition_variable>
#include <map>
#include <memory>
#include <mutex>
#include <sched.h>

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __restrict__
#define __shared__
#define KSW2G_EMU 1

struct uint4 {
  uint32_t x, y, z, w;
};
inline uint4 make_uint4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) { return uint4{x, y, z, w}; }

struct emu_dim3 {
  unsigned x = 0, y = 0, z = 0;
};
extern thread_local emu_dim3 threadIdx, blockIdx;
extern emu_dim3 blockDim, gridDim;

using std::max;
using std::min;

namespace emu {

// Spin barrier over the lanes of one mask.  Lanes that do not exist in the
// emulated warp (blocks smaller than 32 threads) are left out of the count.
struct Barrier {
  std::atomic<int> count{0};
  std::atomic<long> gen{0};
  int need = 0;
  uint64_t slot[32];
  void arrive() {
    const long g = gen.load(std::memory_order_acquire);
    if (count.fetch_add(1, std::memory_order_acq_rel) + 1 == need) {
      count.store(0, std::memory_order_relaxed);
      gen.fetch_add(1, std::memory_order_acq_rel);
    } else {
      int spins = 0;
      long total = 0;
      while (gen.load(std::memory_order_acquire) == g) {
        if (++spins > 64) sched_yield(), spins = 0;
        if (++total == 200000000L) fprintf(stderr, "[emu] barrier %p stuck: need %d count %d\n", (void *)this, need, count.load());
      }
    }
  }
};

struct Warp {
  std::mutex mu;
  unsigned present = 0xffffffffu;
  std::map<unsigned, std::unique_ptr<Barrier>> bars;
  Barrier &get(unsigned mask) {
    std::lock_guard<std::mutex> g(mu);
    auto &p = bars[mask];
    if (!p) {
      p.reset(new Barrier);
      p->need = __builtin_popcount(mask & present);
    }
    return *p;
  }
};

extern Warp *g_warps;  // one per warp of the emulated block
extern Barrier *g_block;  // all threads of the emulated block (__syncthreads)

// last collective of each emulated thread, for the watchdog of run_block
struct LaneState {
  std::atomic<unsigned> mask{0};
  std::atomic<long> calls{0};
  std::atomic<int> waiting{0};
};
extern LaneState g_lane_state[1024];

inline int lane() { return threadIdx.x & 31; }
inline Warp &warp() { return g_warps[threadIdx.x >> 5]; }
inline Barrier &enter(unsigned mask) {
  LaneState &ls = g_lane_state[threadIdx.x];
  ls.mask = mask;
  ls.calls++;
  return warp().get(mask);
}

inline Barrier &enter(unsigned mask);

template <typename T>
inline T exchange(unsigned mask, T v, int src_lane) {
  Barrier &b = enter(mask);
  uint64_t raw = 0;
  memcpy(&raw, &v, sizeof(T));
  b.slot[lane()] = raw;
  b.arrive();
  uint64_t got = b.slot[src_lane & 31];
  b.arrive();
  T out;
  memcpy(&out, &got, sizeof(T));
  return out;
}

}  // namespace emu

template <typename T>
inline T __shfl_sync(unsigned mask, T v, int src, int width = 32) {
  const int base = emu::lane() & ~(width - 1);
  return emu::exchange(mask, v, base + (src & (width - 1)));
}
template <typename T>
inline T __shfl_up_sync(unsigned mask, T v, unsigned d, int width = 32) {
  const int l = emu::lane(), base = l & ~(width - 1), r = l - base;
  const int src = (int)r - (int)d >= 0 ? l - (int)d : l;
  return emu::exchange(mask, v, src);
}
template <typename T>
inline T __shfl_xor_sync(unsigned mask, T v, int x, int width = 32) {
  const int l = emu::lane(), base = l & ~(width - 1);
  const int src = base + (((l - base) ^ x) & (width - 1));
  return emu::exchange(mask, v, src);
}
inline unsigned __ballot_sync(unsigned mask, int pred) {
  emu::Barrier &b = emu::enter(mask);
  b.slot[emu::lane()] = pred ? 1 : 0;
  b.arrive();
  unsigned r = 0;
  mask &= emu::warp().present;
  for (int i = 0; i < 32; ++i)
    if ((mask >> i) & 1) r |= (b.slot[i] ? 1u : 0u) << i;
  b.arrive();
  return r;
}
// __reduce_*_sync over the lanes named in mask (sm_80+ warp reductions)
inline uint64_t emu_reduce(unsigned mask, uint64_t v, int op) {  // op 0: max s32, 1: min u32, 2: add u32, 3: max u32, 4: and
  emu::Barrier &b = emu::enter(mask);
  b.slot[emu::lane()] = v;
  b.arrive();
  mask &= emu::warp().present;
  int64_t smax = INT64_MIN;
  uint64_t umin = UINT64_MAX, umax = 0, sum = 0, band = 0xffffffffu;
  for (int i = 0; i < 32; ++i)
    if ((mask >> i) & 1) {
      const uint32_t x = (uint32_t)b.slot[i];
      band &= x;
      smax = std::max<int64_t>(smax, (int32_t)x);
      umin = std::min<uint64_t>(umin, x);
      umax = std::max<uint64_t>(umax, x);
      sum += x;
    }
  b.arrive();
  return op == 0 ? (uint64_t)(uint32_t)(int32_t)smax : op == 1 ? umin : op == 2 ? (uint32_t)sum : op == 3 ? umax : band;
}
inline int __reduce_max_sync(unsigned mask, int v) { return (int)(uint32_t)emu_reduce(mask, (uint32_t)v, 0); }
inline unsigned __reduce_min_sync(unsigned mask, unsigned v) { return (unsigned)emu_reduce(mask, v, 1); }
inline unsigned __reduce_add_sync(unsigned mask, unsigned v) { return (unsigned)emu_reduce(mask, v, 2); }
inline unsigned __reduce_max_sync(unsigned mask, unsigned v) { return (unsigned)emu_reduce(mask, v, 3); }
inline unsigned __reduce_and_sync(unsigned mask, unsigned v) { return (unsigned)emu_reduce(mask, v, 4); }
inline int __ffs(unsigned x) { return x ? __builtin_ctz(x) + 1 : 0; }
inline int __popc(unsigned x) { return __builtin_popcount(x); }
inline int __all_sync(unsigned mask, int pred) { return __ballot_sync(mask, pred) == (mask & emu::warp().present); }
inline int __any_sync(unsigned mask, int pred) { return __ballot_sync(mask, pred) != 0; }
inline void __syncwarp(unsigned mask = 0xffffffffu) { (void)__ballot_sync(mask, 1); }
inline void __syncthreads() { emu::g_block->arrive(); }

inline uint32_t __byte_perm(uint32_t x, uint32_t y, uint32_t s) {
  uint8_t b[8];
  for (int i = 0; i < 4; ++i) b[i] = (uint8_t)(x >> (8 * i)), b[4 + i] = (uint8_t)(y >> (8 * i));
  uint32_t r = 0;
  for (int i = 0; i < 4; ++i) {
    const unsigned nib = (s >> (4 * i)) & 0xf;
    r |= (uint32_t)b[nib & 7] << (8 * i);
  }
  return r;
}
inline uint32_t __funnelshift_l(uint32_t lo, uint32_t hi, uint32_t sh) {
  const uint64_t v = ((uint64_t)hi << 32) | lo;
  return (uint32_t)((v << (sh & 31)) >> 32);
}
// 16x2 SIMD / DPX built-ins: per halfword, signed 16-bit, additions wrap
namespace emu {
inline int16_t lo16(uint32_t x) { return (int16_t)(uint16_t)x; }
inline int16_t hi16(uint32_t x) { return (int16_t)(uint16_t)(x >> 16); }
inline uint32_t pk16(int lo, int hi) { return (uint32_t)(uint16_t)lo | ((uint32_t)(uint16_t)hi << 16); }
template <class F>
inline uint32_t map16(uint32_t a, uint32_t b, uint32_t c, F f) {
  return pk16(f(lo16(a), lo16(b), lo16(c)), f(hi16(a), hi16(b), hi16(c)));
}
}  // namespace emu
inline uint32_t __vadd2(uint32_t a, uint32_t b) {
  return emu::map16(a, b, 0, [](int x, int y, int) { return (int16_t)(x + y); });
}
inline int __vimax3_s32(int a, int b, int c) { return std::max(a, std::max(b, c)); }
inline uint32_t __vmaxs2(uint32_t a, uint32_t b) {
  return emu::map16(a, b, 0, [](int x, int y, int) { return x > y ? x : y; });
}
inline uint32_t __viaddmax_s16x2(uint32_t a, uint32_t b, uint32_t c) {
  return emu::map16(a, b, c, [](int x, int y, int z) { const int s = (int16_t)(x + y); return s > z ? s : z; });
}
inline uint32_t __viaddmin_s16x2(uint32_t a, uint32_t b, uint32_t c) {
  return emu::map16(a, b, c, [](int x, int y, int z) { const int s = (int16_t)(x + y); return s < z ? s : z; });
}
inline uint32_t __vimax3_s16x2(uint32_t a, uint32_t b, uint32_t c) {
  return emu::map16(a, b, c, [](int x, int y, int z) { return std::max(x, std::max(y, z)); });
}
// unsigned halves
namespace emu {
template <class F>
inline uint32_t map16u(uint32_t a, uint32_t b, uint32_t c, F f) {
  return (uint32_t)(uint16_t)f(a & 0xffffu, b & 0xffffu, c & 0xffffu) |
         ((uint32_t)(uint16_t)f(a >> 16, b >> 16, c >> 16) << 16);
}
}  // namespace emu
inline uint32_t __vimax3_u16x2(uint32_t a, uint32_t b, uint32_t c) {
  return emu::map16u(a, b, c, [](uint32_t x, uint32_t y, uint32_t z) { return std::max(x, std::max(y, z)); });
}
inline uint32_t __vmaxu2(uint32_t a, uint32_t b) {
  return emu::map16u(a, b, 0, [](uint32_t x, uint32_t y, uint32_t) { return std::max(x, y); });
}
inline uint32_t __vminu2(uint32_t a, uint32_t b) {
  return emu::map16u(a, b, 0, [](uint32_t x, uint32_t y, uint32_t) { return std::min(x, y); });
}
// funnel shifts with the count clamped at 32
inline uint32_t __funnelshift_rc(uint32_t lo, uint32_t hi, uint32_t s) {
  const uint64_t v = ((uint64_t)hi << 32) | lo;
  return (uint32_t)(v >> (s > 32 ? 32 : s));
}
inline uint32_t __funnelshift_lc(uint32_t lo, uint32_t hi, uint32_t s) {
  const uint64_t v = ((uint64_t)hi << 32) | lo;
  return (uint32_t)((v << (s > 32 ? 32 : s)) >> 32);
}
template <typename T>
inline T __ldg(const T *p) { return *p; }
inline int atomicAdd(int *p, int v) { return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST); }
inline unsigned long long atomicAdd(unsigned long long *p, unsigned long long v) {
  return __atomic_fetch_add(p, v, __ATOMIC_SEQ_CST);
}
inline int atomicOr(int *p, int v) { return __atomic_fetch_or(p, v, __ATOMIC_SEQ_CST); }
inline int atomicMax(int *p, int v) {
  int o = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (o < v && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return o;
}
inline int atomicMin(int *p, int v) {
  int o = __atomic_load_n(p, __ATOMIC_SEQ_CST);
  while (o > v && !__atomic_compare_exchange_n(p, &o, v, false, __ATOMIC_SEQ_CST, __ATOMIC_SEQ_CST)) {
  }
  return o;
}
