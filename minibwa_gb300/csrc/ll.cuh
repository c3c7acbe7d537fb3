// ll.cuh -- striped local Smith-Waterman of ksw2_ll_sse.c on sm_103a.
//
// The reference's result depends on its stripe layout (Farrar's striping
// with a lazy-F pass that does not feed E, ksw2_ll_sse.c:174-186), so the
// kernel keeps that layout: a group of LANES threads (16 for the u8 core,
// 8 for the i16 core) processes one job, thread l being SSE lane l.  Lane l
// owns query positions l*slen .. l*slen+slen-1; its H, E and Hmax segments
// live in registers (SLEN >= slen, unrolled).  Cross-lane steps of the
// reference -- the one-lane shift of H at the start of a target row
// (ksw2_ll_sse.c:146-147), the one-lane shift of F before every lazy-F pass
// (ksw2_ll_sse.c:176), the all-lanes exit test (ksw2_ll_sse.c:183), the row
// maximum (ksw2_ll_sse.c:187) -- are warp shuffles and votes inside the group.
// The striped query profile of ksw_ll_qinit (ksw2_ll_sse.c:77-95) is built
// per job in shared memory.
#pragma once
#include "ksw2g.h"

#ifndef KSW2G_LL_LZC
#define KSW2G_LL_LZC 4
#endif

namespace ksw2g {

template <int LANES>
__device__ __forceinline__ unsigned ll_group_mask() {
  const int lane = threadIdx.x & 31;
  return ((1u << LANES) - 1u) << (lane & ~(LANES - 1));
}

// SIZE 1: unsigned saturating bytes with bias `shift`; SIZE 2: signed 16-bit.
template <int SIZE, int SLEN>
__global__ void __launch_bounds__(128)
ll_kernel(const ksw2g_ll_job *__restrict__ jobs, int n_jobs, const uint8_t *__restrict__ arena,
          const int8_t *__restrict__ mat_g, int m, int gapo, int gape, ksw2g_ll_result *__restrict__ res,
          uint64_t *__restrict__ blist, const int64_t *__restrict__ blist_off, int *__restrict__ job_counter) {
  constexpr int LANES = SIZE == 1 ? 16 : 8;
  constexpr int GROUPS = 128 / LANES;
  const int lane = threadIdx.x & 31;
  const int l = lane & (LANES - 1);
  const int grp = threadIdx.x / LANES;
  const unsigned gm = ll_group_mask<LANES>();
  extern __shared__ int16_t ll_smem[];
  // per group: profile [m][SLEN][LANES] int16, plus 16 bytes so the groups' regions fall on different banks
  const int prof_stride = m * SLEN * LANES + 8;
  int16_t *prof = ll_smem + grp * prof_stride;

  // scoring constants (ksw2_ll_sse.c:66-74)
  int shift = 127, mdiff = 0;
  for (int a = 0; a < m * m; ++a) {
    const int v = mat_g[a];
    if (v < (int)(int8_t)(uint8_t)shift) shift = (uint8_t)v;
    if (v > (int)(int8_t)(uint8_t)mdiff) mdiff = (uint8_t)v;
  }
  const int qmax = mdiff;
  shift = (256 - shift) & 0xff;
  const int goe = SIZE == 1 ? ((gapo + gape) & 0xff) : (int)(int16_t)(gapo + gape);
  const int ge = SIZE == 1 ? (gape & 0xff) : (int)(int16_t)gape;

  int32_t H[SLEN], E[SLEN], HM[SLEN];
  int jid = -1, slen = 0, qlen = 0, tlen = 0, xtra = 0, i = 0, te = -1, gmax = 0, n_b = 0, minsc = 0, endsc = 0;
  const uint8_t *tp = nullptr;
  uint64_t *bl = nullptr;
  bool active = false, need = true;

  // saturating lane ops (s2n-lite.h / SSE semantics)
  auto adds = [&](int a, int b) -> int {
    if (SIZE == 1) { const int s = a + b; return s > 255 ? 255 : s; }
    const int s = a + b; return s > 32767 ? 32767 : s < -32768 ? -32768 : s;
  };
  auto subsu = [&](int a, int b) -> int {  // unsigned saturating subtract on the lane width
    if (SIZE == 1) return a > b ? a - b : 0;
    const unsigned x = (uint16_t)a, y = (uint16_t)b;
    return (int)(int16_t)(uint16_t)(x > y ? x - y : 0u);
  };
  auto vmax = [&](int a, int b) -> int { return a > b ? a : b; };  // max_epu8 on 0..255 / max_epi16

  for (;;) {
    if (need) {
      int j = 0;
      if (l == 0) j = atomicAdd(job_counter, 1);
      j = __shfl_sync(gm, j, 0, LANES);
      need = false;
      active = j < n_jobs;
      if (active) {
        jid = j;
        const ksw2g_ll_job J = jobs[jid];
        jid = J.slot;
        qlen = J.qlen, tlen = J.tlen, xtra = J.xtra;
        slen = (qlen + LANES - 1) / LANES;
        tp = arena + J.toff;
        const uint8_t *qp = arena + J.qoff;
        // striped profile: lane l of segment s scores query position s + l*slen
        __syncwarp(gm);
        for (int a = 0; a < m; ++a)
#pragma unroll
          for (int s = 0; s < SLEN; ++s) {
            if (s < slen) {
              const int k = s + l * slen;
              const int qc = k >= qlen ? 0 : qp[k];
              const int v = k >= qlen ? -1 : mat_g[a * m + (qc < m ? qc : m - 1)];  // codes must be < m
              prof[(a * SLEN + s) * LANES + l] = (int16_t)(SIZE == 1 ? ((v + shift) & 0xff) : v);
            }
          }
        __syncwarp(gm);
        minsc = (xtra & KSW2G_LL_SUBO) ? (xtra & 0xffff) : 0x10000;
        endsc = (xtra & KSW2G_LL_STOP) ? (xtra & 0xffff) : 0x10000;
        bl = (blist && (xtra & KSW2G_LL_SUBO)) ? blist + blist_off[jid] : nullptr;
#pragma unroll
        for (int s = 0; s < SLEN; ++s) H[s] = 0, E[s] = 0, HM[s] = 0;
        i = 0, te = -1, gmax = 0, n_b = 0;
        if (tlen <= 0) {
          // no rows: fall through to the result with gmax = 0
        }
      }
    }
    if (__all_sync(0xffffffffu, !active)) break;
    if (!active) continue;

    bool done = i >= tlen;
    if (!done) {
      // ---- target row i (ksw2_ll_sse.c:142-201) ----
      const int a = tp[i] < m ? tp[i] : m - 1;  // codes must be < m; clamp keeps the read inside the profile
      const int16_t *S = prof + a * SLEN * LANES + l;
      int hlast = H[0];
#pragma unroll
      for (int s = 1; s < SLEN; ++s) hlast = (s == slen - 1) ? H[s] : hlast;
      int h = __shfl_up_sync(gm, hlast, 1, LANES);
      if (l == 0) h = 0;
      int f = 0, mx = 0;
#pragma unroll
      for (int s = 0; s < SLEN; ++s) {
        if (s < slen) {
          int sc = S[s * LANES];
          int hv;
          if (SIZE == 1) hv = subsu(adds(h, sc & 0xff), shift);
          else hv = adds(h, sc);
          const int ev = E[s];
          hv = vmax(hv, ev);
          hv = vmax(hv, f);
          mx = vmax(mx, hv);
          h = H[s];  // H(i-1, s): diagonal predecessor of segment s+1
          H[s] = hv;
          E[s] = vmax(subsu(ev, ge), subsu(hv, goe));
          f = vmax(subsu(f, ge), subsu(hv, goe));
        }
      }
      // lazy-F (ksw2_ll_sse.c:175-185 / 287-297)
      bool fin = false;
      for (int kk = 0; kk < 16 && !fin; ++kk) {
        int fs = __shfl_up_sync(gm, f, 1, LANES);
        f = l == 0 ? 0 : fs;
#pragma unroll
        for (int s = 0; s < SLEN; ++s) {
          if (s < slen && !fin) {
            const int hv = vmax(H[s], f);
            H[s] = hv;
            const int hh = subsu(hv, goe);
            f = subsu(f, ge);
            const bool ok = SIZE == 1 ? (f <= hh) : !(f > hh);
            fin = __all_sync(gm, ok);
          }
        }
      }
      int imax = mx;
#pragma unroll
      for (int off = LANES / 2; off > 0; off >>= 1) imax = vmax(imax, __shfl_xor_sync(gm, imax, off, LANES));
      if (imax >= minsc && bl != nullptr && l == 0) {  // second-best bookkeeping (ksw2_ll_sse.c:188-193)
        if (n_b == 0 || (int32_t)bl[n_b - 1] + 1 != i) bl[n_b++] = (uint64_t)imax << 32 | (uint32_t)i;
        else if ((int)(bl[n_b - 1] >> 32) < imax) bl[n_b - 1] = (uint64_t)imax << 32 | (uint32_t)i;
      }
      if (imax >= minsc && bl != nullptr) n_b = __shfl_sync(gm, n_b, 0, LANES);
      if (imax > gmax) {
        gmax = imax, te = i;
#pragma unroll
        for (int s = 0; s < SLEN; ++s) HM[s] = H[s];
        if ((SIZE == 1 && gmax + shift >= 255) || gmax >= endsc) done = true;
      }
      ++i;
      if (i >= tlen) done = true;
    }
    if (done) {
      // ---- result (ksw2_ll_sse.c:202-219 / 314-330) ----
      ksw2g_ll_result o;
      o.score = SIZE == 1 ? (gmax + shift < 255 ? gmax : 255) : gmax;
      o.te = te, o.qe = -1, o.score2 = -1, o.te2 = -1, o.rows = i;
      if (SIZE == 2 || o.score != 255) {
        // max over Hmax in memory order, ties to the smallest query index
        uint32_t best = 0;
        bool any = false;
#pragma unroll
        for (int s = 0; s < SLEN; ++s) {
          if (s < slen) {
            const uint32_t v = SIZE == 1 ? (uint32_t)HM[s] : (uint32_t)(uint16_t)HM[s];
            const uint32_t key = (v << 16) | (uint32_t)(0xffff - (s + l * slen));
            if (!any || key > best) best = key, any = true;
          }
        }
#pragma unroll
        for (int off = LANES / 2; off > 0; off >>= 1) best = max(best, __shfl_xor_sync(gm, best, off, LANES));
        if (slen > 0) o.qe = 0xffff - (int)(best & 0xffff);
        if (bl != nullptr && l == 0 && n_b > 0) {
          const int c = qmax > 0 ? (o.score + qmax - 1) / qmax : 0;
          const int low = te - c, high = te + c;
          for (int b = 0; b < n_b; ++b) {
            const int e = (int32_t)bl[b];
            if ((e < low || e > high) && (int)(bl[b] >> 32) > o.score2) o.score2 = (int)(bl[b] >> 32), o.te2 = e;
          }
        }
      }
      if (l == 0) res[jid] = o;
      need = true;
    }
  }
}


// Queries of more segments than the register-resident kernels hold: the same
// one-lane-per-thread recurrences, with the striped profile, H, E and the
// best-row copy of H in shared memory (int16 entries, [segment][lane]), one job
// per block of LANES threads and dynamic segment loops.  slen_cap is the
// number of segments the block's shared memory was sized for.
template <int SIZE>
__global__ void __launch_bounds__(16)
ll_wide_kernel(const ksw2g_ll_job *__restrict__ jobs, int n_jobs, const uint8_t *__restrict__ arena,
          const int8_t *__restrict__ mat_g, int m, int gapo, int gape, ksw2g_ll_result *__restrict__ res,
          uint64_t *__restrict__ blist, const int64_t *__restrict__ blist_off, int *__restrict__ job_counter,
          int slen_cap) {
  constexpr int LANES = SIZE == 1 ? 16 : 8;
  const int l = threadIdx.x;
  const unsigned gm = (1u << LANES) - 1u;
  extern __shared__ int16_t llw_smem[];
  int16_t *prof = llw_smem;                           // [m][slen_cap][LANES]
  int16_t *Hs = prof + (size_t)m * slen_cap * LANES;  // [slen_cap][LANES]
  int16_t *Es = Hs + (size_t)slen_cap * LANES;
  int16_t *HMs = Es + (size_t)slen_cap * LANES;

  // scoring constants (ksw2_ll_sse.c:66-74)
  int shift = 127, mdiff = 0;
  for (int a = 0; a < m * m; ++a) {
    const int v = mat_g[a];
    if (v < (int)(int8_t)(uint8_t)shift) shift = (uint8_t)v;
    if (v > (int)(int8_t)(uint8_t)mdiff) mdiff = (uint8_t)v;
  }
  const int qmax = mdiff;
  shift = (256 - shift) & 0xff;
  const int goe = SIZE == 1 ? ((gapo + gape) & 0xff) : (int)(int16_t)(gapo + gape);
  const int ge = SIZE == 1 ? (gape & 0xff) : (int)(int16_t)gape;

  int jid = -1, slen = 0, qlen = 0, tlen = 0, xtra = 0, i = 0, te = -1, gmax = 0, n_b = 0, minsc = 0, endsc = 0;
  const uint8_t *tp = nullptr;
  uint64_t *bl = nullptr;
  bool active = false, need = true;

  // saturating lane ops (s2n-lite.h / SSE semantics)
  auto adds = [&](int a, int b) -> int {
    if (SIZE == 1) { const int s = a + b; return s > 255 ? 255 : s; }
    const int s = a + b; return s > 32767 ? 32767 : s < -32768 ? -32768 : s;
  };
  auto subsu = [&](int a, int b) -> int {  // unsigned saturating subtract on the lane width
    if (SIZE == 1) return a > b ? a - b : 0;
    const unsigned x = (uint16_t)a, y = (uint16_t)b;
    return (int)(int16_t)(uint16_t)(x > y ? x - y : 0u);
  };
  auto vmax = [&](int a, int b) -> int { return a > b ? a : b; };  // max_epu8 on 0..255 / max_epi16

  for (;;) {
    if (need) {
      int j = 0;
      if (l == 0) j = atomicAdd(job_counter, 1);
      j = __shfl_sync(gm, j, 0, LANES);
      need = false;
      active = j < n_jobs;
      if (active) {
        jid = j;
        const ksw2g_ll_job J = jobs[jid];
        jid = J.slot;
        qlen = J.qlen, tlen = J.tlen, xtra = J.xtra;
        slen = (qlen + LANES - 1) / LANES;
        tp = arena + J.toff;
        const uint8_t *qp = arena + J.qoff;
        // striped profile: lane l of segment s scores query position s + l*slen
        __syncwarp(gm);
        for (int a = 0; a < m; ++a)
          for (int s = 0; s < slen; ++s) {
            const int k = s + l * slen;
            const int qc = k >= qlen ? 0 : qp[k];
            const int v = k >= qlen ? -1 : mat_g[a * m + (qc < m ? qc : m - 1)];  // codes must be < m
            prof[(a * slen_cap + s) * LANES + l] = (int16_t)(SIZE == 1 ? ((v + shift) & 0xff) : v);
          }
        __syncwarp(gm);
        minsc = (xtra & KSW2G_LL_SUBO) ? (xtra & 0xffff) : 0x10000;
        endsc = (xtra & KSW2G_LL_STOP) ? (xtra & 0xffff) : 0x10000;
        bl = (blist && (xtra & KSW2G_LL_SUBO)) ? blist + blist_off[jid] : nullptr;
        for (int s = 0; s < slen; ++s) Hs[s * LANES + l] = 0, Es[s * LANES + l] = 0, HMs[s * LANES + l] = 0;
        i = 0, te = -1, gmax = 0, n_b = 0;
        if (tlen <= 0) {
          // no rows: fall through to the result with gmax = 0
        }
      }
    }
    if (!active) break;  // one job per block: active is uniform


    bool done = i >= tlen;
    if (!done) {
      // ---- target row i (ksw2_ll_sse.c:142-201) ----
      const int a = tp[i] < m ? tp[i] : m - 1;  // codes must be < m; clamp keeps the read inside the profile
      const int16_t *S = prof + a * slen_cap * LANES + l;
      int hlast = slen > 0 ? Hs[(slen - 1) * LANES + l] : 0;
      int h = __shfl_up_sync(gm, hlast, 1, LANES);
      if (l == 0) h = 0;
      int f = 0, mx = 0;
      for (int s = 0; s < slen; ++s) {
        const int sc = S[s * LANES];
        int hv;
        if (SIZE == 1) hv = subsu(adds(h, sc & 0xff), shift);
        else hv = adds(h, sc);
        const int ev = Es[s * LANES + l];
        hv = vmax(hv, ev);
        hv = vmax(hv, f);
        mx = vmax(mx, hv);
        h = Hs[s * LANES + l];  // H(i-1, s): diagonal predecessor of segment s+1
        Hs[s * LANES + l] = (int16_t)hv;
        Es[s * LANES + l] = (int16_t)vmax(subsu(ev, ge), subsu(hv, goe));
        f = vmax(subsu(f, ge), subsu(hv, goe));
      }
      // lazy-F (ksw2_ll_sse.c:175-185 / 287-297)
      bool fin = false;
      for (int kk = 0; kk < 16 && !fin; ++kk) {
        int fs = __shfl_up_sync(gm, f, 1, LANES);
        f = l == 0 ? 0 : fs;
        for (int s = 0; s < slen && !fin; ++s) {
          const int hv = vmax(Hs[s * LANES + l], f);
          Hs[s * LANES + l] = (int16_t)hv;
          const int hh = subsu(hv, goe);
          f = subsu(f, ge);
          const bool ok = SIZE == 1 ? (f <= hh) : !(f > hh);
          fin = __all_sync(gm, ok);
        }
      }
      int imax = mx;
#pragma unroll
      for (int off = LANES / 2; off > 0; off >>= 1) imax = vmax(imax, __shfl_xor_sync(gm, imax, off, LANES));
      if (imax >= minsc && bl != nullptr && l == 0) {  // second-best bookkeeping (ksw2_ll_sse.c:188-193)
        if (n_b == 0 || (int32_t)bl[n_b - 1] + 1 != i) bl[n_b++] = (uint64_t)imax << 32 | (uint32_t)i;
        else if ((int)(bl[n_b - 1] >> 32) < imax) bl[n_b - 1] = (uint64_t)imax << 32 | (uint32_t)i;
      }
      if (imax >= minsc && bl != nullptr) n_b = __shfl_sync(gm, n_b, 0, LANES);
      if (imax > gmax) {
        gmax = imax, te = i;
        for (int s = 0; s < slen; ++s) HMs[s * LANES + l] = Hs[s * LANES + l];
        if ((SIZE == 1 && gmax + shift >= 255) || gmax >= endsc) done = true;
      }
      ++i;
      if (i >= tlen) done = true;
    }
    if (done) {
      // ---- result (ksw2_ll_sse.c:202-219 / 314-330) ----
      ksw2g_ll_result o;
      o.score = SIZE == 1 ? (gmax + shift < 255 ? gmax : 255) : gmax;
      o.te = te, o.qe = -1, o.score2 = -1, o.te2 = -1, o.rows = i;
      if (SIZE == 2 || o.score != 255) {
        // max over Hmax in memory order, ties to the smallest query index
        uint32_t best = 0;
        bool any = false;
        for (int s = 0; s < slen; ++s) {
          const int hmv = HMs[s * LANES + l];
          const uint32_t v = SIZE == 1 ? (uint32_t)hmv : (uint32_t)(uint16_t)hmv;
          const uint32_t key = (v << 16) | (uint32_t)(0xffff - (s + l * slen));
          if (!any || key > best) best = key, any = true;
        }
#pragma unroll
        for (int off = LANES / 2; off > 0; off >>= 1) best = max(best, __shfl_xor_sync(gm, best, off, LANES));
        if (slen > 0) o.qe = 0xffff - (int)(best & 0xffff);
        if (bl != nullptr && l == 0 && n_b > 0) {
          const int c = qmax > 0 ? (o.score + qmax - 1) / qmax : 0;
          const int low = te - c, high = te + c;
          for (int b = 0; b < n_b; ++b) {
            const int e = (int32_t)bl[b];
            if ((e < low || e > high) && (int)(bl[b] >> 32) > o.score2) o.score2 = (int)(bl[b] >> 32), o.te2 = e;
          }
        }
      }
      if (l == 0) res[jid] = o;
      need = true;
    }
  }
}

}  // namespace ksw2g

namespace ksw2g {

// Bytes 2H and 2H+1 of x into the low and high halfwords, sign-extended when
// SIGNED (PTX prmt, default mode: selector bit 3 replicates the selected byte's sign).
template <bool SIGNED, int H>
__device__ __forceinline__ uint32_t widen2(uint32_t x) {
#if defined(__CUDA_ARCH__)
  uint32_t r;
  if (SIGNED && H == 0) asm("prmt.b32 %0, %1, 0, 0x9180;" : "=r"(r) : "r"(x));
  else if (SIGNED) asm("prmt.b32 %0, %1, 0, 0xb3a2;" : "=r"(r) : "r"(x));
  else if (H == 0) asm("prmt.b32 %0, %1, 0, 0x4140;" : "=r"(r) : "r"(x));
  else asm("prmt.b32 %0, %1, 0, 0x4342;" : "=r"(r) : "r"(x));
  return r;
#else
  const uint32_t b0 = (x >> (16 * H)) & 0xffu, b1 = (x >> (16 * H + 8)) & 0xffu;
  if (SIGNED) return (uint32_t)(uint16_t)(int16_t)(int8_t)b0 | ((uint32_t)(uint16_t)(int16_t)(int8_t)b1 << 16);
  return b0 | (b1 << 16);
#endif
}

// Shared-memory layout of the DPX kernel.  Each thread's profile row (one residue, all
// its segments, two lane bytes per segment) is contiguous and padded to SP segments,
// SP = 8 (mod 16), so a 16-byte load brings 8 segments and the rows of the threads of
// a quarter-warp start on different banks; a group's rows are followed by padding that
// puts the next group's on the other half of the banks.  The per-thread Hmax columns
// follow all the profiles.
__host__ __device__ constexpr int ll_dpx_sp(int slen) { return ((slen + 7) / 16) * 16 + 8; }
__host__ __device__ inline int ll_dpx_group_words(int m, int slen, int T) {
  const int w = m * T * ll_dpx_sp(slen) / 2;
  return w + (16 - w % 32 + 32) % 32;
}
__host__ __device__ inline int ll_dpx_hm_offset(int m, int slen, int T) {
  return (128 / T) * ll_dpx_group_words(m, slen, T);
}
// Dynamic shared memory of one 128-thread block of the DPX kernel.
inline size_t ll_dpx_smem_bytes(int m, int slen, int T) {
  return (size_t)ll_dpx_hm_offset(m, slen, T) * 4 + (size_t)128 * slen * 4;
}

// Two SSE lanes per thread, in the two halfwords of every register, on the DPX
// 16x2 instructions: thread t of a group of T = LANES/2 threads holds lanes t
// (low half) and t+T (high half) of one job.  Every step of the reference's
// recurrences is one instruction for both lanes:
//   u8 :  h = max(max(min(h + S, 255) - shift, 0), e, f)     (adds/subs_epu8)
//   i16:  h = max(h + S, e, f)                                (adds_epi16 without saturation)
//   t = max(h - goe, 0);  e = max(e - ge, t);  f = max(f - ge, t)  (subs_epu*, max_ep*)
// The u8 form is exact for every input.  The i16 form is exact when the host
// has checked that no H value can reach 32767 and that 0 <= gape, gapo+gape
// <= 32767; otherwise the host launches ll_kernel above.
// Resident blocks asked per SM: six up to 16 segments and five up to 24 fit the
// registers without spilling (config 3's 19 segments: 970 -> 1,131 GCUPS
// going from four blocks to five).
template <int SIZE, int SLEN>
__global__ void __launch_bounds__(128, SLEN <= 16 ? 6 : SLEN <= 24 ? 5 : (SLEN <= 32 ? 3 : 2))
ll_dpx_kernel(const ksw2g_ll_job *__restrict__ jobs, int n_jobs, const uint8_t *__restrict__ arena,
              const int8_t *__restrict__ mat_g, int m, int gapo, int gape, ksw2g_ll_result *__restrict__ res,
              uint64_t *__restrict__ blist, const int64_t *__restrict__ blist_off, int *__restrict__ job_counter) {
  constexpr int LANES = SIZE == 1 ? 16 : 8;
  constexpr int T = LANES / 2;
  const int lane = threadIdx.x & 31;
  const int t = lane & (T - 1);
  const int grp = threadIdx.x / T;
  const unsigned gm = ((1u << T) - 1u) << (lane & ~(T - 1));
  // Shared memory: the groups' striped profiles, one byte per SSE lane (two per 16-bit
  // entry: lanes t and t+T), then the best-row copy of H of every thread (Hmax of the
  // reference) in a thread-interleaved column, which is written only when the maximum grows.
  extern __shared__ uint32_t lld_smem[];
  constexpr int SP = ll_dpx_sp(SLEN);
  constexpr int LZC = KSW2G_LL_LZC;  // lazy-F segments per exit test
  uint16_t *prof = (uint16_t *)(lld_smem + grp * ll_dpx_group_words(m, SLEN, T));
  uint32_t *hm = lld_smem + ll_dpx_hm_offset(m, SLEN, T) + threadIdx.x;  // hm[s * 128]

  int shift = 127, mdiff = 0;  // ksw2_ll_sse.c:66-74
  for (int a = 0; a < m * m; ++a) {
    const int v = mat_g[a];
    if (v < (int)(int8_t)(uint8_t)shift) shift = (uint8_t)v;
    if (v > (int)(int8_t)(uint8_t)mdiff) mdiff = (uint8_t)v;
  }
  const int qmax = mdiff;
  shift = (256 - shift) & 0xff;
  const int goe = SIZE == 1 ? ((gapo + gape) & 0xff) : (gapo + gape);
  const int ge = SIZE == 1 ? (gape & 0xff) : gape;
  auto pk = [](int lo, int hi) -> uint32_t { return (uint32_t)(uint16_t)lo | ((uint32_t)(uint16_t)hi << 16); };
  const uint32_t NGOE = pk(-goe, -goe), NGE = pk(-ge, -ge), NSHIFT = pk(-shift, -shift), C255 = pk(255, 255);

  uint32_t H[SLEN], E[SLEN];
  uint32_t hl = 0;  // H[slen-1], the segment the next row's one-lane shift reads
  int jid = -1, slen = 0, qlen = 0, tlen = 0, xtra = 0, i = 0, te = -1, gmax = 0, n_b = 0, minsc = 0, endsc = 0;
  const uint8_t *tp = nullptr;
  uint64_t *bl = nullptr;
  bool active = false, need = true;

  for (;;) {
    if (need) {
      int j = 0;
      if (t == 0) j = atomicAdd(job_counter, 1);
      j = __shfl_sync(gm, j, 0, T);
      need = false;
      active = j < n_jobs;
      if (active) {
        jid = j;
        const ksw2g_ll_job J = jobs[jid];
        jid = J.slot;
        qlen = J.qlen, tlen = J.tlen, xtra = J.xtra;
        slen = (qlen + LANES - 1) / LANES;
        tp = arena + J.toff;
        const uint8_t *qp = arena + J.qoff;
        // striped profile (ksw2_ll_sse.c:77-95): lane l of segment s scores query position s + l*slen
        for (int a = 0; a < m; ++a)
#pragma unroll
          for (int s = 0; s < SLEN; ++s) {
            if (s < slen) {
              int v2[2];
#pragma unroll
              for (int h = 0; h < 2; ++h) {
                const int k = s + (t + h * T) * slen;
                const int qc = k >= qlen ? 0 : qp[k];
                const int v = k >= qlen ? -1 : mat_g[a * m + (qc < m ? qc : m - 1)];  // codes must be < m
                v2[h] = SIZE == 1 ? ((v + shift) & 0xff) : v;  // u8: 0..255; i16: an int8 score
              }
              prof[(a * T + t) * SP + s] = (uint16_t)((v2[0] & 0xff) | ((v2[1] & 0xff) << 8));
            }
          }
        __syncwarp(gm);
        minsc = (xtra & KSW2G_LL_SUBO) ? (xtra & 0xffff) : 0x10000;
        endsc = (xtra & KSW2G_LL_STOP) ? (xtra & 0xffff) : 0x10000;
        bl = (blist && (xtra & KSW2G_LL_SUBO)) ? blist + blist_off[jid] : nullptr;
#pragma unroll
        for (int s = 0; s < SLEN; ++s) H[s] = 0, E[s] = 0, hm[s * 128] = 0;
        hl = 0;
        i = 0, te = -1, gmax = 0, n_b = 0;
      }
    }
    if (__all_sync(0xffffffffu, !active)) break;
    if (!active) continue;

    bool done = i >= tlen;
    if (!done) {
      const int a = tp[i] < m ? tp[i] : m - 1;
      const uint4 *S4 = (const uint4 *)(prof + (a * T + t) * SP);  // 8 segments per 16-byte load
      // one-lane shift of the last segment (ksw2_ll_sse.c:146-147): lane l <- lane l-1, lane 0 <- 0
      const uint32_t up = __shfl_up_sync(gm, hl, 1, T), wrap = __shfl_sync(gm, hl, T - 1, T);
      uint32_t h = t ? up : (wrap << 16);
      uint32_t f = 0, mx = 0;
      uint4 q8 = make_uint4(0, 0, 0, 0);
#pragma unroll
      for (int s = 0; s < SLEN; ++s) {
        if ((s & 7) == 0 && s < slen) q8 = S4[s >> 3];
        if (s < slen) {
          // widen the segment's two bytes to the two halfwords: zero-extended (u8) or sign-extended (i16)
          const uint32_t qw = (s & 7) < 2 ? q8.x : (s & 7) < 4 ? q8.y : (s & 7) < 6 ? q8.z : q8.w;
          const uint32_t sc = (s & 1) ? widen2<SIZE == 2, 1>(qw) : widen2<SIZE == 2, 0>(qw);
          uint32_t hv;
          if (SIZE == 1) hv = __viaddmax_s16x2(__viaddmin_s16x2(h, sc, C255), NSHIFT, 0u);
          else hv = __vadd2(h, sc);
          hv = __vimax3_s16x2(hv, E[s], f);
          mx = __vmaxs2(mx, hv);
          h = H[s];
          H[s] = hv;
          hl = hv;  // the last segment processed is slen-1
          const uint32_t tt = __viaddmax_s16x2(hv, NGOE, 0u);
          E[s] = __viaddmax_s16x2(E[s], NGE, tt);
          f = __viaddmax_s16x2(f, NGE, tt);
        }
      }
      // lazy-F (ksw2_ll_sse.c:175-185 / 287-297): the reference stops after the first segment
      // at which f <= H - gapoe holds in every lane.  Segments go in chunks of LZC: each
      // chunk's candidate H values and exit tests are computed, one group-wide AND of the
      // tests finds the first exiting segment, and H is kept only up to it.
      bool fin = false;
      for (int kk = 0; kk < 16 && !fin; ++kk) {
        const uint32_t fu = __shfl_up_sync(gm, f, 1, T), fw = __shfl_sync(gm, f, T - 1, T);
        f = t ? fu : (fw << 16);
#pragma unroll
        for (int c = 0; c < SLEN; c += LZC) {
          if (c < slen && !fin) {
            uint32_t nh[LZC];
            unsigned ok = 0;
#pragma unroll
            for (int u = 0; u < LZC; ++u) {
              nh[u] = 0;
              if (c + u < SLEN && c + u < slen) {
                nh[u] = __vmaxs2(H[c + u], f);
                const uint32_t hh = __viaddmax_s16x2(nh[u], NGOE, 0u);
                f = __viaddmax_s16x2(f, NGE, 0u);
                if ((__vmaxs2(f, hh) ^ hh) == 0u) ok |= 1u << u;  // f <= hh in this thread's lanes
              }
            }
            const unsigned all = __reduce_and_sync(gm, ok);
            const int last = all ? __ffs(all) - 1 : LZC - 1;  // the last segment of the chunk that is kept
            fin = all != 0;
#pragma unroll
            for (int u = 0; u < LZC; ++u) {
              if (c + u < SLEN && c + u < slen && u <= last) {
                H[c + u] = nh[u];
                if (c + u == slen - 1) hl = nh[u];
              }
            }
          }
        }
      }
      int m2 = max((int)(int16_t)(uint16_t)mx, (int)(int16_t)(uint16_t)(mx >> 16));
      const int imax = __reduce_max_sync(gm, m2);
      if (imax >= minsc && bl != nullptr && t == 0) {  // second best (ksw2_ll_sse.c:188-193)
        if (n_b == 0 || (int32_t)bl[n_b - 1] + 1 != i) bl[n_b++] = (uint64_t)imax << 32 | (uint32_t)i;
        else if ((int)(bl[n_b - 1] >> 32) < imax) bl[n_b - 1] = (uint64_t)imax << 32 | (uint32_t)i;
      }
      if (imax >= minsc && bl != nullptr) n_b = __shfl_sync(gm, n_b, 0, T);
      if (imax > gmax) {
        gmax = imax, te = i;
#pragma unroll
        for (int s = 0; s < SLEN; ++s) hm[s * 128] = H[s];
        if ((SIZE == 1 && gmax + shift >= 255) || gmax >= endsc) done = true;
      }
      ++i;
      if (i >= tlen) done = true;
    }
    if (done) {
      ksw2g_ll_result o;
      o.score = SIZE == 1 ? (gmax + shift < 255 ? gmax : 255) : gmax;
      o.te = te, o.qe = -1, o.score2 = -1, o.te2 = -1, o.rows = i;
      if (SIZE == 2 || o.score != 255) {
        uint32_t best = 0;
        bool any = false;
#pragma unroll
        for (int s = 0; s < SLEN; ++s) {
          if (s < slen) {
#pragma unroll
            for (int hf = 0; hf < 2; ++hf) {
              const uint32_t v = (hm[s * 128] >> (16 * hf)) & 0xffffu;
              const uint32_t key = (v << 16) | (uint32_t)(0xffff - (s + (t + hf * T) * slen));
              if (!any || key > best) best = key, any = true;
            }
          }
        }
        best = __reduce_max_sync(gm, best);
        if (slen > 0) o.qe = 0xffff - (int)(best & 0xffff);
        if (bl != nullptr && t == 0 && n_b > 0) {
          const int c = qmax > 0 ? (o.score + qmax - 1) / qmax : 0;
          const int low = te - c, high = te + c;
          for (int b = 0; b < n_b; ++b) {
            const int e = (int32_t)bl[b];
            if ((e < low || e > high) && (int)(bl[b] >> 32) > o.score2) o.score2 = (int)(bl[b] >> 32), o.te2 = e;
          }
        }
      }
      if (t == 0) res[jid] = o;
      need = true;
    }
  }
}

}  // namespace ksw2g
