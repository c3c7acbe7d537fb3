// swar.cuh -- four int8 lanes per 32-bit register.
//
// Each helper reproduces one SSE byte-lane operation of the ksw2 kernels
// (_mm_add_epi8 / _mm_sub_epi8 wrap, _mm_cmpgt_epi8 / _mm_max_epi8 signed,
// _mm_max_epu8 / _mm_min_epu8 unsigned) on four lanes at once with plain
// integer instructions.  Comparisons produce an "msb mask" (bit 7 of each lane
// set where the predicate holds); bmask() widens it to a 0x00/0xff lane mask
// with one PTX prmt in sign-replicate mode.
#pragma once
#include <stdint.h>

namespace ksw2g {

static constexpr uint32_t kHi = 0x80808080u;
static constexpr uint32_t kLo = 0x7f7f7f7fu;

__device__ __forceinline__ uint32_t splat8(uint32_t b) { return (b & 0xffu) * 0x01010101u; }

// 0xff in every lane whose bit 7 is set: PTX prmt in its default mode, where
// bit 3 of a selector nibble replicates the sign bit of the selected byte
// (__byte_perm documents only selector bits 2:0, so it is not used here).
__device__ __forceinline__ uint32_t bmask(uint32_t m) {
#if defined(__CUDA_ARCH__)
  uint32_t r;
  asm("prmt.b32 %0, %1, 0, 0xba98;" : "=r"(r) : "r"(m));
  return r;
#else
  return ((m >> 7) & 0x01010101u) * 0xffu;
#endif
}

// lane-wise a + b (mod 256)
__device__ __forceinline__ uint32_t add8(uint32_t a, uint32_t b) {
  return ((a & kLo) + (b & kLo)) ^ ((a ^ b) & kHi);
}
// lane-wise a - b (mod 256)
__device__ __forceinline__ uint32_t sub8(uint32_t a, uint32_t b) {
  return ((a | kHi) - (b & kLo)) ^ ((a ^ ~b) & kHi);
}
// lane-wise r - c (mod 256) for lanes r in [0, 127], given rh = r | 0x80 in every lane: the
// biased lanes r + 128 - (c & 127) never borrow, and the msb is fixed up from c's msb
__device__ __forceinline__ uint32_t sub8_nn(uint32_t rh, uint32_t c) { return (rh - (c & kLo)) ^ (~c & kHi); }
// msb mask of (int8)a > (int8)b
__device__ __forceinline__ uint32_t gts8(uint32_t a, uint32_t b) {
  uint32_t c = (b | kHi) - (a & kLo);            // bit7: b_lo >= a_lo
  // a7 == b7 ? !c7 : b7   (on bit 7)
  return ((~(a ^ b)) & ~c) | ((a ^ b) & b);
}
// msb mask of (uint8)a > (uint8)b
__device__ __forceinline__ uint32_t gtu8(uint32_t a, uint32_t b) {
  uint32_t c = (b | kHi) - (a & kLo);
  return ((~(a ^ b)) & ~c) | ((a ^ b) & a);
}
// msb mask of (int8)a > 0
__device__ __forceinline__ uint32_t gt0s8(uint32_t a) { return ((a & kLo) + kLo) & ~a; }
// msb mask of (int8)a < 0
__device__ __forceinline__ uint32_t lt0s8(uint32_t a) { return a; }
// m ? a : b with a full 0x00/0xff lane mask
__device__ __forceinline__ uint32_t sel(uint32_t m, uint32_t a, uint32_t b) { return (a & m) | (b & ~m); }

__device__ __forceinline__ uint32_t maxs8(uint32_t a, uint32_t b) { return sel(bmask(gts8(a, b)), a, b); }
__device__ __forceinline__ uint32_t mins8(uint32_t a, uint32_t b) { return sel(bmask(gts8(a, b)), b, a); }
__device__ __forceinline__ uint32_t maxu8(uint32_t a, uint32_t b) { return sel(bmask(gtu8(a, b)), a, b); }
__device__ __forceinline__ uint32_t minu8(uint32_t a, uint32_t b) { return sel(bmask(gtu8(a, b)), b, a); }
// max((int8)a, 0)
__device__ __forceinline__ uint32_t relu8(uint32_t a) { return a & ~bmask(a); }
// msb mask of lanes equal to zero
__device__ __forceinline__ uint32_t eqz8(uint32_t x) { return ~(((x & kLo) + kLo) | x) & kHi; }

// one byte of a word, zero- or sign-extended
__device__ __forceinline__ int32_t ubyte(uint32_t w, int i) { return (int32_t)((w >> (8 * i)) & 0xffu); }
__device__ __forceinline__ int32_t sbyte(uint32_t w, int i) { return (int32_t)(int8_t)(uint8_t)(w >> (8 * i)); }

}  // namespace ksw2g
