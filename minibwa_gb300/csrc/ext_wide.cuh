// ext_wide.cuh -- extension DP for bands wider than the register-resident
// kernel's widest thread group (more than 64 blocks of 16 cells per
// anti-diagonal: long reads' end extension with w up to bw_long).
//
// One block of kWideThreads threads owns one pair at a time.  The state lives
// in the block's global scratch in the reference's own flat layout (one byte
// per target position for u, v, x, y[, x2, y2], the score row s, the target
// and the reversed query; int32 H), indexed by target position exactly as
// ksw2_extz2_sse.c / ksw2_extd2_sse.c index their arrays.  The cells of an
// anti-diagonal are split over the block's threads; the only order the
// reference's sequential block loop imposes -- cell t reads x, v (and x2) of
// cell t-1 from the previous anti-diagonal -- is kept by double-buffering x,
// v and x2, so a thread never reads a value another thread of the same
// anti-diagonal has already overwritten.  u, y and y2 are read and written at
// the same position by the same thread.  The maximum of an anti-diagonal and
// its tie-break are a block reduction of (H, key) pairs with the key order of
// the register kernel (en0 first, then the four int32 lanes over [st0, en1),
// then the scalar tail).  Traceback rows go to the pair's rows of the
// traceback pool in the layout ext_bt_kernel reads.
#pragma once
#include "ksw2g.h"

namespace ksw2g {

#ifndef KSW2G_WIDE_THREADS
#define KSW2G_WIDE_THREADS 256
#endif
constexpr int kWideThreads = KSW2G_WIDE_THREADS;  // a multiple of 32

// block-shared variables (the host emulation of the kernels shares them as statics)
#ifndef KSW2G_BLOCK_SHARED
#ifdef KSW2G_EMU
#define KSW2G_BLOCK_SHARED static
#else
#define KSW2G_BLOCK_SHARED __shared__
#endif
#endif

// Bytes of one block's scratch for a pair (the 16 bytes of slack after every
// row array absorb the reference's 16-byte score stores that run past tlen).
__host__ __device__ inline int64_t ext_wide_scratch_bytes(int qlen, int tlen) {
  const int64_t T = (((int64_t)tlen + 15) & ~(int64_t)15) + 32;
  const int64_t QR = (((int64_t)qlen + 15) & ~(int64_t)15) + 64;
  return 11 * T + QR + 4 * T + 64;
}

__device__ __forceinline__ int32_t wide_vv(int dual, uint8_t b, int qe) {
  return dual ? (int32_t)(int8_t)b : (int32_t)b - qe;
}
__device__ __forceinline__ uint8_t wb_sub(uint8_t a, uint8_t b) { return (uint8_t)(a - b); }
__device__ __forceinline__ uint8_t wb_add(uint8_t a, uint8_t b) { return (uint8_t)(a + b); }
__device__ __forceinline__ int wb_gt(uint8_t a, uint8_t b) { return (int8_t)a > (int8_t)b; }
__device__ __forceinline__ uint8_t wb_max(uint8_t a, uint8_t b) { return wb_gt(a, b) ? a : b; }
__device__ __forceinline__ uint8_t wb_min(uint8_t a, uint8_t b) { return wb_gt(a, b) ? b : a; }
__device__ __forceinline__ uint8_t wu_max(uint8_t a, uint8_t b) { return a > b ? a : b; }
__device__ __forceinline__ uint8_t wu_min(uint8_t a, uint8_t b) { return a < b ? a : b; }

// Largest H, then smallest key, over the block; every thread gets the result.
__device__ __forceinline__ uint64_t wide_reduce(uint64_t v, uint64_t *red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u > v ? u : v;
  }
  __syncthreads();  // red may still be read from the previous reduction
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  uint64_t b = red[0];
  for (int w = 1; w < kWideThreads / 32; ++w) b = red[w] > b ? red[w] : b;
  return b;
}
// (H, key) packed so that the unsigned maximum is the largest H with the smallest key
__device__ __forceinline__ uint64_t wide_pack(int32_t h, uint32_t key) {
  return ((uint64_t)((uint32_t)h ^ 0x80000000u) << 32) | (uint64_t)(0xffffffffu - key);
}

__global__ void __launch_bounds__(kWideThreads)
ext_wide_kernel(const ksw2g_job *__restrict__ jobs, const int32_t *__restrict__ order, int n_jobs,
                const uint8_t *__restrict__ arena, const ksw2g_ext_params P, ksw2g_ext_result *__restrict__ res,
                ksw2g_bt *__restrict__ bts, uint8_t *__restrict__ tb_pool, const int64_t *__restrict__ tb_off,
                int *__restrict__ job_counter, uint8_t *__restrict__ scratch, int64_t scratch_stride) {
  KSW2G_BLOCK_SHARED uint64_t red[kWideThreads / 32];
  KSW2G_BLOCK_SHARED int s_job;
  const int tid = threadIdx.x, NT = kWideThreads;
  const int dual = P.dual;
  uint8_t *base = scratch + (int64_t)blockIdx.x * scratch_stride;
  const uint8_t init1 = dual ? (uint8_t)(-P.q - P.e) : 0, init2 = dual ? (uint8_t)(-P.q2 - P.e2) : 0;
  const int qe = P.qe_scalar;
  const int ez_e = dual ? P.e2 : P.e;

  for (;;) {
    if (tid == 0) s_job = atomicAdd(job_counter, 1);
    __syncthreads();
    const int j = s_job;
    __syncthreads();
    if (j >= n_jobs) return;
    const int jid = order ? order[j] : j;
    const ksw2g_job J = jobs[jid];
    const int qlen = J.qlen, tlen = J.tlen, zdrop = J.zdrop, end_bonus = J.end_bonus, flag = J.flag;
    int w = J.w;
    int32_t ez_max = 0, max_q = -1, max_t = -1, mqe = KSW2G_NEG_INF, mqe_t = -1, mte = KSW2G_NEG_INF, mte_q = -1;
    int32_t score = KSW2G_NEG_INF, zdropped = 0, n_diag = 0;
    int64_t cells = 0;
    if (P.skip_all || qlen <= 0 || tlen <= 0 || P.m <= dual) {
      if (tid == 0) {
        ksw2g_ext_result o;
        o.score = score, o.max = 0, o.max_q = -1, o.max_t = -1, o.mqe = mqe, o.mqe_t = -1, o.mte = mte, o.mte_q = -1;
        o.zdropped = 0, o.reach_end = 0, o.n_cigar = 0, o.n_diag = 0, o.cigar_off = 0, o.cells = 0;
        res[jid] = o;
        bts[jid] = ksw2g_bt{-1, -1, 0, 0};
      }
      continue;
    }
    if (w < 0) w = tlen > qlen ? tlen : qlen;
    const int with_cigar = !(flag & KSW2G_SCORE_ONLY), right = !!(flag & KSW2G_RIGHT);
    const int approx = !!(flag & KSW2G_APPROX_MAX), generic = !!(flag & KSW2G_GENERIC_SC);
    int ncol = qlen < tlen ? qlen : tlen;
    ncol = ((ncol < w + 1 ? ncol : w + 1) + 15) / 16 + 1;
    const int64_t ncol16 = (int64_t)ncol * 16;
    uint8_t *tb = tb_pool + tb_off[jid];

    // scratch arrays, same indexing as the reference's
    const int64_t T = (((int64_t)tlen + 15) & ~(int64_t)15) + 32;
    uint8_t *U = base, *Y = U + T, *Y2 = Y + T, *S = Y2 + T, *SF = S + T;
    uint8_t *Xb[2] = {SF + T, SF + 2 * T}, *Vb[2] = {SF + 3 * T, SF + 4 * T}, *X2b[2] = {SF + 5 * T, SF + 6 * T};
    uint8_t *QR = SF + 7 * T;
    const int64_t QRn = (((int64_t)qlen + 15) & ~(int64_t)15) + 64;
    int32_t *H = (int32_t *)(((uintptr_t)(QR + QRn) + 15) & ~(uintptr_t)15);
    const uint8_t *qp = arena + J.qoff, *tp = arena + J.toff;
    for (int64_t t = tid; t < T; t += NT) {
      U[t] = Y[t] = Xb[0][t] = Xb[1][t] = Vb[0][t] = Vb[1][t] = init1;
      Y2[t] = X2b[0][t] = X2b[1][t] = init2;
      S[t] = 0;
      SF[t] = t < tlen ? tp[t] : 0;
      H[t] = KSW2G_NEG_INF;
    }
    for (int64_t t = tid; t < QRn; t += NT) QR[t] = t < qlen ? qp[qlen - 1 - t] : 0;
    __syncthreads();

    int cur = 0, last_st = -1, last_en = -1;
    int32_t H0 = 0, last_H0_t = 0, last_max_H = 0;
    bool stop = false;
    for (int r = 0; r < qlen + tlen - 1 && !stop; ++r) {
      int st = 0, en = tlen - 1;
      if (st < r - qlen + 1) st = r - qlen + 1;
      if (en > r) en = r;
      if (st < (r - w + 1) >> 1) st = (r - w + 1) >> 1;
      if (en > (r + w) >> 1) en = (r + w) >> 1;
      if (st > en) {  // ksw2_extz2_sse.c:103-106
        zdropped = 1;
        break;
      }
      const int st0 = st, en0 = en;
      st = st / 16 * 16, en = (en + 16) / 16 * 16 - 1;  // ksw2_extz2_sse.c:108
      ++n_diag;
      cells += en0 - st0 + 1;
      const uint8_t *Xp = Xb[cur ^ 1], *Vp = Vb[cur ^ 1], *X2p = X2b[cur ^ 1];
      uint8_t *Xc = Xb[cur], *Vc = Vb[cur], *X2c = X2b[cur];
      // boundary values (ksw2_extz2_sse.c:110-115, ksw2_extd2_sse.c:141-155)
      uint8_t x1, v1, x21 = 0, extx = 0, extv = 0;
      if (!dual) {
        if (st > 0) {
          if (st - 1 >= last_st && st - 1 <= last_en) x1 = Xp[st - 1], v1 = Vp[st - 1];
          else x1 = v1 = 0;
        } else x1 = 0, v1 = r ? (uint8_t)P.c_q : 0;
        extx = (x1 & 0x80) ? 0xff : 0;  // _mm_cvtsi32_si128 of an int8_t (ksw2_extz2_sse.c:138-139)
        extv = (v1 & 0x80) ? 0xff : 0;
      } else {
        const uint8_t vb = r == 0 ? (uint8_t)(-P.q - P.e)
                                  : r < P.long_thres ? (uint8_t)(-P.e)
                                  : r == P.long_thres ? (uint8_t)P.long_diff : (uint8_t)(-P.e2);
        if (st > 0) {
          if (st - 1 >= last_st && st - 1 <= last_en) x1 = Xp[st - 1], x21 = X2p[st - 1], v1 = Vp[st - 1];
          else x1 = init1, x21 = init2, v1 = init1;
        } else x1 = init1, x21 = init2, v1 = vb;
        if (en >= r && tid == 0) Y[r] = init1, Y2[r] = init2, U[r] = vb;
      }
      if (!dual && en >= r && tid == 0) Y[r] = 0, U[r] = r ? (uint8_t)P.c_q : 0;
      // substitution scores: the reference's 16-byte stores from st0 (ksw2_extz2_sse.c:117-136)
      const uint8_t *qrr = QR + (qlen - 1 - r);
      if (!generic) {
        for (int t = st0 + 16 * tid; t <= en0; t += 16 * NT)
          for (int k = 0; k < 16; ++k) {
            const uint8_t sq = SF[t + k], sr = qrr[t + k];
            const uint8_t sc = sq == sr ? (uint8_t)P.c_mch : (uint8_t)P.c_mis;
            S[t + k] = (sq == (uint8_t)P.c_m1 || sr == (uint8_t)P.c_m1) ? (uint8_t)P.c_N : sc;
          }
      } else {
        for (int t = st0 + tid; t <= en0; t += NT) S[t] = (uint8_t)P.mat[(SF[t] * P.m + qrr[t]) & 255];
      }
      __syncthreads();
      // cells st..en (ksw2_extz2_sse.c:142-215, ksw2_extd2_sse.c:183-314)
      uint8_t *row = with_cigar ? tb + (int64_t)r * ncol16 : nullptr;
      for (int t = st + tid; t <= en; t += NT) {
        uint8_t xp = t == st ? x1 : Xp[t - 1], vp = t == st ? v1 : Vp[t - 1];
        const uint8_t x2p = t == st ? x21 : X2p[t - 1];
        if (!dual && t > st && t <= st + 3) xp |= extx, vp |= extv;
        const uint8_t up = U[t];
        uint8_t z, a, b, d = 0;
        if (!dual) {
          z = wb_add(S[t], (uint8_t)P.c_qe2);
          a = wb_add(xp, vp);
          b = wb_add(Y[t], up);
          if (!with_cigar) {
            z = wb_max(z, a), z = wu_max(z, b), z = wu_min(z, (uint8_t)P.c_maxsc);
          } else if (!right) {
            d = wb_gt(a, z) ? 1 : 0;
            z = wb_max(z, a);
            if (wb_gt(b, z)) d = 2;
            z = wu_max(z, b), z = wu_min(z, (uint8_t)P.c_maxsc);
          } else {
            d = wb_gt(z, a) ? 0 : 1;
            z = wb_max(z, a);
            if (!wb_gt(z, b)) d = 2;
            z = wu_max(z, b), z = wu_min(z, (uint8_t)P.c_maxsc);
          }
          U[t] = wb_sub(z, vp);
          Vc[t] = wb_sub(z, up);
          z = wb_sub(z, (uint8_t)P.c_q);
          a = wb_sub(a, z), b = wb_sub(b, z);
          if (!with_cigar) {
            Xc[t] = wb_max(a, 0), Y[t] = wb_max(b, 0);
          } else if (!right) {
            if (wb_gt(a, 0)) Xc[t] = a, d |= 0x08; else Xc[t] = 0;
            if (wb_gt(b, 0)) Y[t] = b, d |= 0x10; else Y[t] = 0;
          } else {
            if (wb_gt(0, a)) Xc[t] = 0; else Xc[t] = a, d |= 0x08;
            if (wb_gt(0, b)) Y[t] = 0; else Y[t] = b, d |= 0x10;
          }
        } else {
          z = S[t];
          a = wb_add(xp, vp), b = wb_add(Y[t], up);
          uint8_t a2 = wb_add(x2p, vp), b2 = wb_add(Y2[t], up);
          if (!with_cigar) {
            z = wb_max(z, a), z = wb_max(z, b), z = wb_max(z, a2), z = wb_max(z, b2);
            z = wb_min(z, (uint8_t)P.c_mch);
          } else if (!right) {
            d = wb_gt(a, z) ? 1 : 0;
            z = wb_max(z, a);
            if (wb_gt(b, z)) d = 2;
            z = wb_max(z, b);
            if (wb_gt(a2, z)) d = 3;
            z = wb_max(z, a2);
            if (wb_gt(b2, z)) d = 4;
            z = wb_max(z, b2), z = wb_min(z, (uint8_t)P.c_mch);
          } else {
            d = wb_gt(z, a) ? 0 : 1;
            z = wb_max(z, a);
            if (!wb_gt(z, b)) d = 2;
            z = wb_max(z, b);
            if (!wb_gt(z, a2)) d = 3;
            z = wb_max(z, a2);
            if (!wb_gt(z, b2)) d = 4;
            z = wb_max(z, b2), z = wb_min(z, (uint8_t)P.c_mch);
          }
          U[t] = wb_sub(z, vp);
          Vc[t] = wb_sub(z, up);
          uint8_t tmp = wb_sub(z, (uint8_t)P.c_q);
          a = wb_sub(a, tmp), b = wb_sub(b, tmp);
          tmp = wb_sub(z, (uint8_t)P.c_q2);
          a2 = wb_sub(a2, tmp), b2 = wb_sub(b2, tmp);
          const uint8_t cqe = (uint8_t)P.c_qe, cqe2 = (uint8_t)P.c_qe2;
          if (!with_cigar) {
            Xc[t] = wb_sub(wb_max(a, 0), cqe), Y[t] = wb_sub(wb_max(b, 0), cqe);
            X2c[t] = wb_sub(wb_max(a2, 0), cqe2), Y2[t] = wb_sub(wb_max(b2, 0), cqe2);
          } else if (!right) {
            if (wb_gt(a, 0)) Xc[t] = wb_sub(a, cqe), d |= 0x08; else Xc[t] = wb_sub(0, cqe);
            if (wb_gt(b, 0)) Y[t] = wb_sub(b, cqe), d |= 0x10; else Y[t] = wb_sub(0, cqe);
            if (wb_gt(a2, 0)) X2c[t] = wb_sub(a2, cqe2), d |= 0x20; else X2c[t] = wb_sub(0, cqe2);
            if (wb_gt(b2, 0)) Y2[t] = wb_sub(b2, cqe2), d |= 0x40; else Y2[t] = wb_sub(0, cqe2);
          } else {
            if (wb_gt(0, a)) Xc[t] = wb_sub(0, cqe); else Xc[t] = wb_sub(a, cqe), d |= 0x08;
            if (wb_gt(0, b)) Y[t] = wb_sub(0, cqe); else Y[t] = wb_sub(b, cqe), d |= 0x10;
            if (wb_gt(0, a2)) X2c[t] = wb_sub(0, cqe2); else X2c[t] = wb_sub(a2, cqe2), d |= 0x20;
            if (wb_gt(0, b2)) Y2[t] = wb_sub(0, cqe2); else Y2[t] = wb_sub(b2, cqe2), d |= 0x40;
          }
        }
        if (with_cigar) row[t - st] = d;
      }
      __syncthreads();
      if (!approx) {  // exact max (ksw2_extz2_sse.c:216-261, ksw2_extd2_sse.c:315-368)
        int32_t hen0;
        if (r > 0) hen0 = en0 > 0 ? H[en0 - 1] + wide_vv(dual, U[en0], qe) : H[en0] + wide_vv(dual, Vc[en0], qe);
        else hen0 = wide_vv(dual, Vc[0], qe) - qe;
        __syncthreads();  // every thread has read H[en0-1] before it is updated
        uint64_t best = 0;
        if (r > 0) {
          const int en1 = st0 + (en0 - st0) / 4 * 4;
          for (int t = st0 + tid; t < en0; t += NT) {
            const int32_t h = H[t] + wide_vv(dual, Vc[t], qe);
            H[t] = h;
            const uint32_t c = t < en1 ? (uint32_t)(1 + ((t - st0) & 3)) : 5u;
            const uint64_t k = wide_pack(h, (c << 24) | (uint32_t)(t - st0));
            best = k > best ? k : best;
          }
        }
        if (tid == 0) {
          H[en0] = hen0;
          const uint64_t k = wide_pack(hen0, 0u);
          best = k > best ? k : best;
        }
        best = wide_reduce(best, red);  // also orders the H updates before the reads below
        const int32_t max_H = (int32_t)((uint32_t)(best >> 32) ^ 0x80000000u);
        const uint32_t key = 0xffffffffu - (uint32_t)best;
        const int mt = key == 0 ? en0 : st0 + (int)(key & 0xffffffu);
        if (en0 == tlen - 1 && H[en0] > mte) mte = H[en0], mte_q = r - en0;
        if (r - st0 == qlen - 1 && H[st0] > mqe) mqe = H[st0], mqe_t = st0;
        if (max_H > ez_max) {  // ksw_apply_zdrop (ksw2.h:181-197)
          ez_max = max_H, max_t = mt, max_q = r - mt;
        } else if (mt >= max_t && r - mt >= max_q) {
          const int tl = mt - max_t, ql = (r - mt) - max_q, l = tl > ql ? tl - ql : ql - tl;
          if (zdrop >= 0 && ez_max - max_H > zdrop + l * ez_e) zdropped = 1, stop = true;
        }
        if (!stop) {
          if (r == qlen + tlen - 2 && en0 == tlen - 1) score = H[tlen - 1];
          if (dual) {
            if (flag & KSW2G_EXTZ_ONLY) {  // ksw2_extd2_sse.c:361-367
              const int32_t rH = last_max_H > max_H ? last_max_H : max_H;
              const int32_t rq = qlen - (r - st0), rt = tlen - en0;
              const int32_t rm = rq >= tlen - st0 ? tlen - st0
                                 : rt >= qlen - (r - en0) ? qlen - (r - en0)
                                                          : tlen + qlen - 1 - r;
              if (rH + rm * P.max_sc + end_bonus < ez_max) stop = true;
            }
            last_max_H = max_H;
          }
        }
      } else {  // approximate max (ksw2_extz2_sse.c:262-278, ksw2_extd2_sse.c:369-385)
        auto VV = [&](int t) { return wide_vv(dual, Vc[t], qe); };
        auto UU = [&](int t) { return wide_vv(dual, U[t], qe); };
        bool zd = false;
        if (r > 0) {
          if (last_H0_t >= st0 && last_H0_t <= en0 && last_H0_t + 1 >= st0 && last_H0_t + 1 <= en0) {
            const int32_t d0 = VV(last_H0_t), d1 = UU(last_H0_t + 1);
            if (d0 > d1) H0 += d0;
            else H0 += d1, ++last_H0_t;
          } else if (last_H0_t >= st0 && last_H0_t <= en0) {
            H0 += VV(last_H0_t);
          } else {
            ++last_H0_t, H0 += UU(last_H0_t);
          }
          if (!dual) zd = true;
        } else {
          H0 = VV(0) - qe, last_H0_t = 0;
        }
        if (dual) zd = true;
        if (zd && (flag & KSW2G_APPROX_DROP)) {
          if (H0 > ez_max) {
            ez_max = H0, max_t = last_H0_t, max_q = r - last_H0_t;
          } else if (last_H0_t >= max_t && r - last_H0_t >= max_q) {
            const int tl = last_H0_t - max_t, ql = (r - last_H0_t) - max_q, l = tl > ql ? tl - ql : ql - tl;
            if (zdrop >= 0 && ez_max - H0 > zdrop + l * ez_e) zdropped = 1, stop = true;
          }
        }
        if (!stop && r == qlen + tlen - 2 && en0 == tlen - 1) score = H0;
        __syncthreads();  // every read of this anti-diagonal's state precedes the next one's writes
      }
      last_st = st, last_en = en;
      cur ^= 1;
    }
    // backtrack start (ksw2_extz2_sse.c:284-295)
    int reach_end = 0, i0 = -1, j0 = -1;
    if (with_cigar) {
      if (!zdropped && !(flag & KSW2G_EXTZ_ONLY)) i0 = tlen - 1, j0 = qlen - 1;
      else if ((flag & KSW2G_EXTZ_ONLY) && mqe + end_bonus > ez_max) reach_end = 1, i0 = mqe_t, j0 = qlen - 1;
      else if (max_t >= 0 && max_q >= 0) i0 = max_t, j0 = max_q;
    }
    if (tid == 0) {
      ksw2g_ext_result o;
      o.score = score, o.max = ez_max, o.max_q = max_q, o.max_t = max_t, o.mqe = mqe, o.mqe_t = mqe_t;
      o.mte = mte, o.mte_q = mte_q, o.zdropped = zdropped, o.reach_end = reach_end, o.n_cigar = 0;
      o.n_diag = n_diag, o.cigar_off = 0, o.cells = cells;
      res[jid] = o;
      bts[jid] = with_cigar ? ksw2g_bt{i0, j0, n_diag, 0} : ksw2g_bt{-1, -1, 0, 0};
    }
    __syncthreads();  // the scratch is reused by the block's next pair
  }
}

}  // namespace ksw2g
