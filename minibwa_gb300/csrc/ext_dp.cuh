// ext_dp.cuh -- banded anti-diagonal DP for ksw_extz2_sse / ksw_extd2_sse on sm_103a.
//
// Mapping.  A group of G threads (4 <= G <= 32, inside one warp) owns one
// pair at a time.  The group keeps a window of W = G*K 32-bit words of every
// per-position state array of the reference (u, v, x, y[, x2, y2], s and the
// 32-bit H of the exact max) in registers: word i of the window covers
// absolute target positions 16*wb + 4*i .. +3, and thread k owns words
// k, k+G, k+2G, ... so that one store instruction of the group writes G
// consecutive traceback words.  The window base wb always equals the
// reference's first padded 16-byte block of the current anti-diagonal
// (st_ in ksw2_extz2_sse.c:140), which moves right by at most one block per
// anti-diagonal; when it moves, all state shifts down by four words.  W is at
// least 4*n_col_ words, the n_col_ blocks the reference computes per
// anti-diagonal (ksw2_extz2_sse.c:68,141).  One more slot of G words holds only
// the substitution scores, for the 16-byte score stores that run past en0
// into the next block (ksw2_extz2_sse.c:118-132).
//
// Per anti-diagonal each thread first exchanges, in one packed shuffle per
// slot, the last bytes of its x, v (and x2) words with its neighbour, then
// computes all its slots back to back (independent chains).  Words past the
// band's last padded block are skipped and hold stale state, never read; a block
// that enters the band is reset to the reference's initial state first.  The maximum and
// its tie-break use single-instruction warp reductions.
//
// Every cell operation reproduces the reference's byte-lane semantics
// (swar.cuh), including the cells of the 16-byte padding outside the nominal
// band, because those are read back as neighbours.  The groups of a warp
// step their anti-diagonals in lockstep; a group whose pair ends (last
// anti-diagonal, z-drop, or the extd2 early stop) takes the next job from a
// device work counter at once.
#pragma once
#include "ksw2g.h"
#include "swar.cuh"

#ifndef KSW2G_TRACE
#define KSW2G_TRACE(...)
#endif

namespace ksw2g {

template <int G>
__device__ __forceinline__ unsigned group_mask() {
  if (G == 32) return 0xffffffffu;
  const int lane = threadIdx.x & 31;
  return ((1u << G) - 1u) << (lane & ~(G - 1));
}

template <int K>
__device__ __forceinline__ uint32_t pick(const uint32_t (&a)[K], int j) {  // a[j], j uniform
  uint32_t v = a[0];
#pragma unroll
  for (int i = 1; i < K; ++i) v = (j == i) ? a[i] : v;
  return v;
}
// shift a per-slot array down by four words (word i <- word i+4)
template <int G, int K, typename T>
__device__ __forceinline__ void shift4(T (&a)[K], T fill, int k, unsigned gm) {
#pragma unroll
  for (int j = 0; j < K; ++j) {
    T send = (k < 4) ? (j + 1 < K ? a[j + 1] : fill) : a[j];
    a[j] = __shfl_sync(gm, send, (k + 4) & (G - 1), G);
  }
}

__device__ __forceinline__ uint32_t ld_tw(const uint8_t *tp, int p, int tlen) {
  return p < tlen ? __ldg((const uint32_t *)(tp + p)) : 0u;
}
// Byte lanes j of a word with from <= j <= to set to 0xff, the others 0 (from, to relative to
// the word's first cell; the funnel shifts clamp their counts at 32, so any range works).
__device__ __forceinline__ uint32_t lanes_upto(int to) {
  return __funnelshift_rc(0xffffffffu, 0u, (uint32_t)max(24 - 8 * to, 0));
}
__device__ __forceinline__ uint32_t lanes_from(int from) {
  return __funnelshift_lc(0u, 0xffffffffu, (uint32_t)max(8 * from, 0));
}
// query bytes of four consecutive cells: lane j = query[hi - j], 0 outside [0, qlen) (the
// 16-bit kernel carries them from anti-diagonal to anti-diagonal)
__device__ __forceinline__ uint32_t ld_qw(const uint8_t *qp, int hi, int qlen) {
  uint32_t w = 0;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int i = hi - j;
    w |= (i >= 0 && i < qlen ? (uint32_t)__ldg(qp + i) : 0u) << (8 * j);
  }
  return w;
}

// Batch constants of the cell recurrence and the score lookup, in byte lanes.
struct ExtConsts {
  uint32_t q4, q24, qe4, qe24, mch4, mis4, N4, m14, maxsc4, mchraw4, sc_lo, sc_hi;
  uint32_t initb, init2b, init4, init24, s_init4;
  bool nt4;
};
template <int VAR>
__device__ __forceinline__ ExtConsts ext_consts(const ksw2g_ext_params &P) {
  constexpr bool D2 = VAR == 1;
  ExtConsts c;
  c.q4 = splat8(P.c_q), c.q24 = splat8(P.c_q2), c.qe4 = splat8(P.c_qe), c.qe24 = splat8(P.c_qe2);
  c.mch4 = splat8(D2 ? P.c_mch : P.c_mch + P.c_qe2);  // extz2 stores s + 2(q+e)
  c.mis4 = splat8(D2 ? P.c_mis : P.c_mis + P.c_qe2);
  c.N4 = splat8(D2 ? P.c_N : P.c_N + P.c_qe2);
  c.m14 = splat8(P.c_m1), c.maxsc4 = splat8(P.c_maxsc), c.mchraw4 = splat8(P.c_mch);
  // score table of the byte-permute lookup: lane index 0 = match, 1-3 = mismatch, 4-7 = N
  c.nt4 = P.c_m1 == 4;
  c.sc_lo = (c.mch4 & 0xffu) | (c.mis4 & 0xffffff00u), c.sc_hi = c.N4;
  c.initb = D2 ? (uint32_t)(uint8_t)(-P.q - P.e) : 0u;
  c.init2b = D2 ? (uint32_t)(uint8_t)(-P.q2 - P.e2) : 0u;
  c.init4 = splat8(c.initb), c.init24 = splat8(c.init2b);
  c.s_init4 = D2 ? 0u : splat8(P.c_qe2);
  return c;
}
// H increment of one byte of u or v: extd2 stores it signed, extz2 biased by q+e
template <int VAR>
__device__ __forceinline__ int32_t ext_vv(uint32_t byte, int qe) {
  return VAR ? (int32_t)(int8_t)(uint8_t)byte : (int32_t)(byte & 0xffu) - qe;
}

// The four query bytes of a word whose lowest query index is idx0 (lane j = query[idx0 + 3 - j]
// after the permute qsel of the anti-diagonal).
__device__ __forceinline__ uint32_t ld_qword(const uint8_t *qp, int idx0, uint32_t qsel) {
  const uint32_t *qa = (const uint32_t *)(qp + (idx0 & ~3));
  return __byte_perm(__ldg(qa), __ldg(qa + 1), qsel);
}
// Scores of four lanes by one byte-permute lookup, exact for m = 5 (N = 4) where every lane has
// t | q <= 4: the lane index (t ^ q) & 3 | (t | q) & 4 is 0 for a match, 1-3 for a mismatch and 4
// for N.  A lane with t | q >= 5 sets bits 3-7 of its byte in bad.
__device__ __forceinline__ uint32_t score_lookup(uint32_t Tw, uint32_t Qw, const ExtConsts &c, uint32_t &bad) {
  const uint32_t tq = Tw | Qw;
  const uint32_t ix = ((Tw ^ Qw) & 0x03030303u) | (tq & 0x04040404u);
  bad |= tq | (tq + 0x03030303u);
  return __byte_perm(c.sc_lo, c.sc_hi, __byte_perm(ix | (ix >> 4), 0u, 0x4420));
}
// Scores of four lanes by the general comparisons (ksw2_extz2_sse.c:117-136), or from the
// matrix under KSW_EZ_GENERIC_SC.
template <int VAR>
__device__ __forceinline__ uint32_t score_exact(uint32_t Tw, uint32_t Qw, bool generic, const ksw2g_ext_params &P,
                                                const ExtConsts &c) {
  uint32_t sn;
  if (!generic) {
    const uint32_t eq = eqz8(Tw ^ Qw);
    const uint32_t nn = eqz8(Tw ^ c.m14) | eqz8(Qw ^ c.m14);
    sn = sel(bmask(eq), c.mch4, c.mis4);
    sn = sel(bmask(nn), c.N4, sn);
  } else {
    sn = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int tc = (Tw >> (8 * b)) & 0xff, qc = (Qw >> (8 * b)) & 0xff;
      uint32_t v = (uint32_t)(uint8_t)P.mat[(tc * P.m + qc) & 255];
      if (!VAR) v = (v + P.c_qe2) & 0xffu;
      sn |= v << (8 * b);
    }
  }
  return sn;
}

// One word (four cells) of an anti-diagonal (ksw2_extz2_sse.c:142-215, ksw2_extd2_sse.c:183-314):
// xt1, vt1, x2t1 are x, v, x2 of the cells t-1 .. t+2 on the anti-diagonal before, s the scores;
// u, v, x, y (x2, y2) are updated in place and the traceback byte lanes returned.
template <int VAR, int MODE>
__device__ __forceinline__ uint32_t ext_cell(uint32_t xt1, uint32_t vt1, uint32_t x2t1, uint32_t s, uint32_t &U,
                                             uint32_t &V, uint32_t &X, uint32_t &Y, uint32_t &X2, uint32_t &Y2,
                                             const ExtConsts &c) {
  const uint32_t ut = U;
  uint32_t z = s, a = add8(xt1, vt1), b = add8(Y, ut), d = 0;
  uint32_t nu, nv, nx, ny, nx2 = 0, ny2 = 0;
  if (!VAR) {
    if (MODE == 0) {
      z = maxs8(z, a);
    } else if (MODE == 1) {
      const uint32_t M = bmask(gts8(a, z));
      d = M & 0x01010101u;
      z = sel(M, a, z);
      d = sel(bmask(gts8(b, z)), 0x02020202u, d);
    } else {
      const uint32_t M = bmask(gts8(z, a));
      d = ~M & 0x01010101u;
      z = sel(M, z, a);
      d = sel(bmask(gts8(z, b)), d, 0x02020202u);
    }
    z = maxu8(z, b);
    z = minu8(z, c.maxsc4);
    nu = sub8(z, vt1);
    nv = sub8(z, ut);
    z = sub8(z, c.q4);
    a = sub8(a, z);
    b = sub8(b, z);
    if (MODE == 1) {
      const uint32_t ga = gt0s8(a) & kHi, gb = gt0s8(b) & kHi;
      nx = a & bmask(ga);
      ny = b & bmask(gb);
      d |= (ga >> 4) | (gb >> 3);
    } else {
      nx = relu8(a);
      ny = relu8(b);
      if (MODE == 2) d |= ((~a & kHi) >> 4) | ((~b & kHi) >> 3);
    }
  } else {
    uint32_t a2 = add8(x2t1, vt1), b2 = add8(Y2, ut);
    if (MODE == 0) {
      z = maxs8(z, a);
      z = maxs8(z, b);
      z = maxs8(z, a2);
      z = maxs8(z, b2);
    } else if (MODE == 1) {
      uint32_t M = bmask(gts8(a, z));
      d = M & 0x01010101u;
      z = sel(M, a, z);
      M = bmask(gts8(b, z));
      d = sel(M, 0x02020202u, d);
      z = sel(M, b, z);
      M = bmask(gts8(a2, z));
      d = sel(M, 0x03030303u, d);
      z = sel(M, a2, z);
      M = bmask(gts8(b2, z));
      d = sel(M, 0x04040404u, d);
      z = sel(M, b2, z);
    } else {
      uint32_t M = bmask(gts8(z, a));
      d = ~M & 0x01010101u;
      z = sel(M, z, a);
      M = bmask(gts8(z, b));
      d = sel(M, d, 0x02020202u);
      z = sel(M, z, b);
      M = bmask(gts8(z, a2));
      d = sel(M, d, 0x03030303u);
      z = sel(M, z, a2);
      M = bmask(gts8(z, b2));
      d = sel(M, d, 0x04040404u);
      z = sel(M, z, b2);
    }
    z = mins8(z, c.mchraw4);
    nu = sub8(z, vt1);
    nv = sub8(z, ut);
    uint32_t tq = sub8(z, c.q4);
    a = sub8(a, tq);
    b = sub8(b, tq);
    tq = sub8(z, c.q24);
    a2 = sub8(a2, tq);
    b2 = sub8(b2, tq);
    if (MODE == 1) {
      const uint32_t ga = gt0s8(a) & kHi, gb = gt0s8(b) & kHi, ga2 = gt0s8(a2) & kHi, gb2 = gt0s8(b2) & kHi;
      nx = sub8_nn((a & bmask(ga)) | kHi, c.qe4);
      ny = sub8_nn((b & bmask(gb)) | kHi, c.qe4);
      nx2 = sub8_nn((a2 & bmask(ga2)) | kHi, c.qe24);
      ny2 = sub8_nn((b2 & bmask(gb2)) | kHi, c.qe24);
      d |= (ga >> 4) | (gb >> 3) | (ga2 >> 2) | (gb2 >> 1);
    } else {
      nx = sub8_nn(relu8(a) | kHi, c.qe4);
      ny = sub8_nn(relu8(b) | kHi, c.qe4);
      nx2 = sub8_nn(relu8(a2) | kHi, c.qe24);
      ny2 = sub8_nn(relu8(b2) | kHi, c.qe24);
      if (MODE == 2) d |= ((~a & kHi) >> 4) | ((~b & kHi) >> 3) | ((~a2 & kHi) >> 2) | ((~b2 & kHi) >> 1);
    }
  }
  U = nu, V = nv, X = nx, Y = ny;
  if (VAR) X2 = nx2, Y2 = ny2;
  return d;
}

// Tie-break key of the reference's exact max (ksw2_extz2_sse.c:216-261) for the cell at offset
// o = t - st0 of an anti-diagonal whose band is [st0, st0 + E]: en0 first (key 0), then the four
// int32 lanes over [st0, en1) -- lowest lane, then lowest t --, then the scalar tail [en1, en0).
__device__ __forceinline__ uint32_t max_key(int o, int E) {
  const int L4 = E & ~3;
  return o == E ? 0u : o < L4 ? ((uint32_t)(1 + (o & 3)) << 24) | (uint32_t)o : (5u << 24) | (uint32_t)o;
}

// VAR: 0 = extz2 (affine), 1 = extd2 (dual affine)
// MODE: 0 = score only, 1 = left-aligned gaps with traceback, 2 = right-aligned gaps with traceback
#ifndef KSW2G_EXT_MINB4
#define KSW2G_EXT_MINB4 4  // resident blocks per SM asked of shapes with K <= 4
#endif
// resident blocks per SM asked of a shape: two-word shapes fit five (extd2) or six (extz2)
// blocks of 128 threads without spilling
template <int VAR, int K>
constexpr int ext_min_blocks() {
  return K <= 2 ? (VAR ? 5 : 6) : K <= 4 ? KSW2G_EXT_MINB4 : K <= 5 ? 3 : 2;
}
template <int VAR, int MODE, int G, int K>
__global__ void __launch_bounds__(128, ext_min_blocks<VAR, K>())
ext_dp_kernel(const ksw2g_job *__restrict__ jobs, const int32_t *__restrict__ order, int n_jobs,
              const uint8_t *__restrict__ arena, const ksw2g_ext_params P, ksw2g_ext_result *__restrict__ res,
              ksw2g_bt *__restrict__ bts, uint8_t *__restrict__ tb_pool, const int64_t *__restrict__ tb_off,
              int *__restrict__ job_counter) {
  constexpr bool D2 = VAR == 1;
  constexpr bool CIG = MODE != 0;
  const int lane = threadIdx.x & 31;
  const int k = lane & (G - 1);
  const unsigned gm = group_mask<G>();

  // batch constants (byte lanes)
  const ExtConsts C = ext_consts<VAR>(P);
  const uint32_t initb = C.initb, init2b = C.init2b, init4 = C.init4, init24 = C.init24, s_init4 = C.s_init4;
  // extz2: q+e; extd2: q+e as declared before the swap (ksw2_extd2_sse.c:60,70), used only at r == 0
  const int qe = P.qe_scalar;
  const int ez_e = D2 ? P.e2 : P.e;

  // per-slot state
  uint32_t U[K], V[K], X[K], Y[K], X2[K], Y2[K], S[K + 1], TW[K + 1];
  int32_t H0[K], H1[K], H2[K], H3[K];

  // per-group state (identical in every thread of the group)
  int jid = -1, qlen = 0, tlen = 0, w = 0, zdrop = 0, end_bonus = 0, flag = 0;
  int r = 0, wb = 0, top = 0, ncol16 = 0, n_diag = 0;
  int64_t cells = 0;
  const uint8_t *qp = nullptr, *tp = nullptr;
  uint8_t *tb = nullptr;
  int32_t ez_max = 0, max_q = -1, max_t = -1, mqe = KSW2G_NEG_INF, mqe_t = -1, mte = KSW2G_NEG_INF, mte_q = -1;
  int32_t score = KSW2G_NEG_INF, zdropped = 0, last_max_H = 0, Hz = 0, last_H0_t = 0;
  int32_t hA = 0, hB = 0, last_en0 = 0;  // H[en0] and H[en0 - 1] after the last anti-diagonal
  bool active = false, need = true;

  auto vv = [&](uint32_t byte) -> int32_t { return ext_vv<VAR>(byte, qe); };

  for (;;) {
    // ---------------- take the next job ----------------
    if (need) {
      int j = 0;
      if (k == 0) j = atomicAdd(job_counter, 1);
      j = __shfl_sync(gm, j, 0, G);
      need = false;
      active = j < n_jobs;
      if (active) {
        jid = order ? order[j] : j;
        const ksw2g_job J = jobs[jid];
        qlen = J.qlen, tlen = J.tlen, w = J.w, zdrop = J.zdrop, end_bonus = J.end_bonus, flag = J.flag;
        ez_max = 0, max_q = max_t = mqe_t = mte_q = -1;
        score = mqe = mte = KSW2G_NEG_INF;
        zdropped = 0, n_diag = 0, cells = 0;
        if (P.skip_all || qlen <= 0 || tlen <= 0 || P.m <= VAR) {
          // degenerate input: the reference returns right after ksw_reset_extz
          if (k == 0) {
            ksw2g_ext_result o;
            o.score = score, o.max = 0, o.max_q = -1, o.max_t = -1, o.mqe = mqe, o.mqe_t = -1, o.mte = mte, o.mte_q = -1;
            o.zdropped = 0, o.reach_end = 0, o.n_cigar = 0, o.n_diag = 0, o.cigar_off = 0, o.cells = 0;
            res[jid] = o;
            if (CIG) bts[jid] = ksw2g_bt{-1, -1, 0, 0};
          }
          need = true;
          continue;
        }
        if (w < 0) w = tlen > qlen ? tlen : qlen;
        {
          int nc = qlen < tlen ? qlen : tlen;
          nc = ((nc < w + 1 ? nc : w + 1) + 15) / 16 + 1;
          ncol16 = nc * 16;
        }
        qp = arena + J.qoff, tp = arena + J.toff;
        if (CIG) tb = tb_pool + tb_off[jid];
        r = 0, wb = 0, top = 0, last_max_H = 0, Hz = 0, last_H0_t = 0, hA = hB = 0, last_en0 = 0;
#pragma unroll
        for (int i = 0; i < K; ++i) {
          U[i] = V[i] = X[i] = Y[i] = init4;
          X2[i] = Y2[i] = init24;
          H0[i] = H1[i] = H2[i] = H3[i] = KSW2G_NEG_INF;
        }
#pragma unroll
        for (int i = 0; i <= K; ++i) S[i] = s_init4, TW[i] = ld_tw(tp, 4 * (k + G * i), tlen);
      }
    }
    if (__all_sync(0xffffffffu, !active)) break;
    if (!active) continue;

    // ---------------- one anti-diagonal ----------------
    bool done = false;
    {
      int st0 = r - qlen + 1 > 0 ? r - qlen + 1 : 0;
      int en0 = r < tlen - 1 ? r : tlen - 1;
      {
        const int a = (r - w + 1) >> 1, b = (r + w) >> 1;
        if (st0 < a) st0 = a;
        if (en0 > b) en0 = b;
      }
      KSW2G_TRACE("lane %d job %d r %d st0 %d en0 %d wb %d\n", lane, jid, r, st0, en0, wb);
      if (st0 > en0) {  // ksw2_extz2_sse.c:103-106
        zdropped = 1;
        done = true;
      } else {
        const int stb = st0 >> 4, enb = en0 >> 4;
        uint32_t x1, v1, x21 = 0;
        if (stb != wb) {  // the first padded block moved right by one: slide the window
          const uint32_t xr = __shfl_sync(gm, X[0], 3, G) >> 24;
          const uint32_t vr = __shfl_sync(gm, V[0], 3, G) >> 24;
          uint32_t x2r = 0;
          if (D2) x2r = __shfl_sync(gm, X2[0], 3, G) >> 24;
          shift4<G, K>(U, init4, k, gm);
          shift4<G, K>(V, init4, k, gm);
          shift4<G, K>(X, init4, k, gm);
          shift4<G, K>(Y, init4, k, gm);
          if (D2) {
            shift4<G, K>(X2, init24, k, gm);
            shift4<G, K>(Y2, init24, k, gm);
          }
          shift4<G, K + 1>(S, s_init4, k, gm);
          shift4<G, K + 1>(TW, 0u, k, gm);
          shift4<G, K>(H0, (int32_t)KSW2G_NEG_INF, k, gm);
          shift4<G, K>(H1, (int32_t)KSW2G_NEG_INF, k, gm);
          shift4<G, K>(H2, (int32_t)KSW2G_NEG_INF, k, gm);
          shift4<G, K>(H3, (int32_t)KSW2G_NEG_INF, k, gm);
          wb = stb;
          if (k >= G - 4) TW[K] = ld_tw(tp, (wb << 4) + 4 * (k + G * K), tlen);
          x1 = xr, v1 = vr, x21 = x2r;  // (r-1, st-1) was computed on the last anti-diagonal
        } else {
          x1 = initb, v1 = initb, x21 = init2b;
        }
        const uint32_t vb = D2 ? (r == 0 ? (uint32_t)(uint8_t)(-P.q - P.e)
                                  : r < P.long_thres ? (uint32_t)(uint8_t)(-P.e)
                                  : r == P.long_thres ? (uint32_t)(uint8_t)P.long_diff
                                                      : (uint32_t)(uint8_t)(-P.e2))
                               : (r ? P.c_q : 0u);
        if (stb == 0) x1 = initb, x21 = init2b, v1 = vb;  // ksw2_extz2_sse.c:114, ksw2_extd2_sse.c:148-151
        const int base = wb << 4;
        const int en = (enb << 4) + 15;
        if (enb > top) {
          // A 16-byte block enters the band (at most one per anti-diagonal).  Words past
          // the last live block hold stale state, so the entering block gets the state the
          // reference's untouched memory holds.
          top = enb;
          const int wtop = (enb - wb) << 2;
#pragma unroll
          for (int i = 0; i < K; ++i) {  // selects, not a conditional store: no slot is indexed at run time
            const bool e = ((k + G * i) & ~3) == wtop;
            U[i] = e ? init4 : U[i], V[i] = e ? init4 : V[i], X[i] = e ? init4 : X[i], Y[i] = e ? init4 : Y[i];
            if (D2) X2[i] = e ? init24 : X2[i], Y2[i] = e ? init24 : Y2[i];
          }
        }
        if (en >= r) {  // top row boundary (ksw2_extz2_sse.c:115, ksw2_extd2_sse.c:152-155)
          const int pr = r - base, wr = pr >> 2, sh = (pr & 3) * 8;
          const uint32_t keep = ~(0xffu << sh);
#pragma unroll
          for (int i = 0; i < K; ++i) {
            const bool e = k + G * i == wr;
            Y[i] = e ? (Y[i] & keep) | (initb << sh) : Y[i];
            U[i] = e ? (U[i] & keep) | (vb << sh) : U[i];
            if (D2) Y2[i] = e ? (Y2[i] & keep) | (init2b << sh) : Y2[i];
          }
        }
        // ---- substitution scores written by the 16-byte stores from st0 (ksw2_extz2_sse.c:117-136) ----
        {
          const bool generic = flag & KSW2G_GENERIC_SC;
          const int fend = generic ? en0 : st0 + (((en0 - st0) >> 4) << 4) + 15;
          const int o = (r + 1) & 3;
          const uint32_t qsel = (uint32_t)((o + 3) | ((o + 2) << 4) | ((o + 1) << 8) | (o << 12));
          // Bytes of a word outside [st0, fend] keep their old scores (the reference does not
          // store them).  The scores are first taken by a byte-permute lookup, exact for m = 5
          // (N = 4) when in every lane t | q <= 4; otherwise the thread runs the loop again with
          // the general comparisons (or the matrix), over the same byte masks.
          uint32_t bad = generic || !C.nt4 ? 0xffffffffu : 0u;
#pragma unroll
          for (int i = 0; i <= K; ++i) {
            const int p0 = base + 4 * (k + G * i);
            // Slots 0..K-1 run without a branch: a word outside [st0, fend] reads the query
            // at an index clamped into the range the words inside read, and its byte mask is 0.
            // The extra slot K is mostly outside and keeps the branch.
            if (i < K || (p0 + 3 >= st0 && p0 <= fend)) {
              // words of slots 1.. start above st0 (the window starts at st0's 16-cell block)
              const int idx0 = i == 0 ? min(max(r - p0 - 3, r - fend - 3), r - st0) : max(r - p0 - 3, r - fend - 3);
              const uint32_t sn = score_lookup(TW[i], ld_qword(qp, idx0, qsel), C, bad);
              const uint32_t wm = i == 0 ? lanes_from(st0 - p0) & lanes_upto(fend - p0) : lanes_upto(fend - p0);
              S[i] = (S[i] & ~wm) | (sn & wm);
            }
          }
          if (bad & 0xf8f8f8f8u) {  // group-divergent only on inputs with other codes
#pragma unroll
            for (int i = 0; i <= K; ++i) {
              const int p0 = base + 4 * (k + G * i);
              if (p0 + 3 >= st0 && p0 <= fend) {
                const uint32_t sn = score_exact<VAR>(TW[i], ld_qword(qp, r - p0 - 3, qsel), generic, P, C);
                const uint32_t wm = lanes_from(st0 - p0) & lanes_upto(fend - p0);
                S[i] = (S[i] & ~wm) | (sn & wm);
              }
            }
          }
        }
        // ---- cells st..en of the anti-diagonal (ksw2_extz2_sse.c:142-215, ksw2_extd2_sse.c:183-314) ----
        const int nlive = (enb - wb + 1) << 2;
        const uint32_t extx = (!D2 && (x1 & 0x80)) ? 0xffffff00u : 0u;  // sign-extended _mm_cvtsi32_si128
        const uint32_t extv = (!D2 && (v1 & 0x80)) ? 0xffffff00u : 0u;
        uint32_t *row = CIG ? (uint32_t *)(tb + (size_t)r * ncol16) : nullptr;
        // last bytes of x, v, x2 of every word, packed, and handed to the next word's owner
        uint32_t rv[K];
        {
          uint32_t pk[K];
#pragma unroll
          for (int i = 0; i < K; ++i) {
            pk[i] = __byte_perm(X[i], V[i], 0x0073);
            if (D2) pk[i] = __byte_perm(pk[i], X2[i], 0x0710);
          }
#pragma unroll
          for (int i = 0; i < K; ++i) {
            const uint32_t send = (k == G - 1) ? (i > 0 ? pk[i > 0 ? i - 1 : 0] : 0u) : pk[i];
            rv[i] = __shfl_sync(gm, send, (k - 1) & (G - 1), G);
          }
          if (k == 0) rv[0] = x1 | (v1 << 8) | (x21 << 16);
        }
#pragma unroll
        for (int i = 0; i < K; ++i) {
          const int wi = k + G * i;
          // A word past the last live block is never read before its block enters the band
          // and is reset, so it is not computed; a slot dead in every group of the warp costs
          // nothing (the groups of a warp mostly run pairs of equal length in step).
          if (wi >= nlive) continue;
          uint32_t xt1 = __byte_perm(rv[i], X[i], 0x6540);  // x[r-1][t-1 .. t+2]
          uint32_t vt1 = __byte_perm(rv[i], V[i], 0x6541);
          if (!D2 && i == 0 && k == 0) xt1 |= extx, vt1 |= extv;
          const uint32_t x2t1 = D2 ? __byte_perm(rv[i], X2[i], 0x6542) : 0u;
          const uint32_t d = ext_cell<VAR, MODE>(xt1, vt1, x2t1, S[i], U[i], V[i], X[i], Y[i], X2[i], Y2[i], C);
          if (CIG) row[wi] = d;
        }
        ++n_diag;
        cells += en0 - st0 + 1;
        // ---- exact or approximate max, z-drop (ksw2_extz2_sse.c:216-278, ksw2_extd2_sse.c:315-385) ----
        if (!(flag & KSW2G_APPROX_MAX)) {
          const int pe = en0 - base, ws = pe >> 2, bs = pe & 3;
          int32_t Hen0;
          if (r == 0) {
            Hen0 = vv(__shfl_sync(gm, V[0], 0, G) & 0xff) - qe;
          } else if (en0 > 0) {
            // H[en0 - 1] of the anti-diagonal before: its H[en0] when en0 moved up by one,
            // else its H[en0 - 1] (hA and hB carry the two from one anti-diagonal to the next;
            // the second may be a cell that already left the band, as in the reference's array)
            const int32_t hm1 = en0 > last_en0 ? hA : hB;
            const uint32_t uw = __shfl_sync(gm, pick<K>(U, ws / G), ws & (G - 1), G);
            Hen0 = hm1 + vv(uw >> (8 * bs));
            hB = hm1;
            if (en0 - 1 >= st0) {  // H[en0 - 1] takes this anti-diagonal's v (pe - 1 >= st0 - base >= 0)
              const int pm = pe - 1;
              const uint32_t vw = __shfl_sync(gm, pick<K>(V, (pm >> 2) / G), (pm >> 2) & (G - 1), G);
              hB += vv(vw >> (8 * (pm & 3)));
            }
          } else {
            const uint32_t vw = __shfl_sync(gm, pick<K>(V, ws / G), ws & (G - 1), G);
            Hen0 = hA + vv(vw >> (8 * bs));
          }
          hA = Hen0, last_en0 = en0;
          // Update H over [st0, en0) and set H[en0]; then the local maximum.  Cells past en0
          // take the additions too: they start at KSW2G_NEG_INF, stay far below any score, and
          // are set when en0 reaches them.  Cells below st0 keep their value (the reference
          // reads one back through H[en0 - 1] above); only window words 0-3 -- threads 0-3 of
          // slot 0 -- can lie below st0, since the window starts at st0's 16-cell block.
          const int se = ws / G;  // slot and thread of H[en0]
          const bool own = k == (ws & (G - 1));
          const int lo = st0 - base - 4 * k;  // slot 0: bytes b >= lo are at or above st0
          int32_t lmax = INT32_MIN;
#pragma unroll
          for (int i = 0; i < K; ++i) {
            const uint32_t vw = V[i];
            if (i == 0) {
              H0[0] += lo <= 0 ? vv(vw) : 0;
              H1[0] += lo <= 1 ? vv(vw >> 8) : 0;
              H2[0] += lo <= 2 ? vv(vw >> 16) : 0;
              H3[0] += lo <= 3 ? vv(vw >> 24) : 0;
            } else {
              H0[i] += vv(vw), H1[i] += vv(vw >> 8), H2[i] += vv(vw >> 16), H3[i] += vv(vw >> 24);
            }
            if (i == se) {  // group-uniform
              H0[i] = own && bs == 0 ? Hen0 : H0[i];
              H1[i] = own && bs == 1 ? Hen0 : H1[i];
              H2[i] = own && bs == 2 ? Hen0 : H2[i];
              H3[i] = own && bs == 3 ? Hen0 : H3[i];
            }
            if (i == 0) {
              lmax = max(max(lo <= 0 ? H0[0] : INT32_MIN, lo <= 1 ? H1[0] : INT32_MIN),
                         max(lo <= 2 ? H2[0] : INT32_MIN, lo <= 3 ? H3[0] : INT32_MIN));
            } else {
              lmax = max(lmax, max(max(H0[i], H1[i]), max(H2[i], H3[i])));
            }
          }
          const int32_t gmax = __reduce_max_sync(gm, lmax);
          // tie-break of the reference: en0 first, then four int32 lanes over
          // [st0, en1) (lowest lane, then lowest t), then the scalar tail [en1, en0)
          // The position of the maximum is used only when this anti-diagonal sets a new
          // maximum or may z-drop (ksw_apply_zdrop, ksw2.h:181-197); otherwise it is skipped.
          const bool need_mt = ez_e < 0 || gmax > ez_max || (zdrop >= 0 && ez_max - gmax > zdrop);
          uint32_t key = 0xffffffffu;
          if (need_mt && lmax == gmax) {
            // cells holding the maximum: one bit per cell of the thread's words (cells past en0
            // never hold it; cells below st0 are masked), then the key of each, usually one
            const int E = en0 - st0;
            uint32_t mm = 0;
#pragma unroll
            for (int i = 0; i < K; ++i) {
              mm |= (H0[i] == gmax ? 1u : 0u) << (4 * i);
              mm |= (H1[i] == gmax ? 2u : 0u) << (4 * i);
              mm |= (H2[i] == gmax ? 4u : 0u) << (4 * i);
              mm |= (H3[i] == gmax ? 8u : 0u) << (4 * i);
            }
            if (lo > 0) mm &= lo >= 4 ? ~0xfu : ~((1u << lo) - 1u);
            while (mm) {
              const int j = __ffs(mm) - 1;
              mm &= mm - 1;
              key = min(key, max_key(base + 4 * (k + G * (j >> 2)) + (j & 3) - st0, E));
            }
          }
          if (need_mt) key = __reduce_min_sync(gm, key);
          const int32_t max_H = gmax;
          const int mt = key == 0 ? en0 : st0 + (int)(key & 0xffffffu);
          if (en0 == tlen - 1 && Hen0 > mte) mte = Hen0, mte_q = r - en0;
          if (r - st0 == qlen - 1) {
            const int ps = st0 - base, bsel = ps & 3;  // H[st0]: slot 0 of thread ps / 4
            const int32_t h0 = bsel == 0 ? H0[0] : bsel == 1 ? H1[0] : bsel == 2 ? H2[0] : H3[0];
            const int32_t hs = __shfl_sync(gm, h0, ps >> 2, G);
            if (hs > mqe) mqe = hs, mqe_t = st0;
          }
          // ksw_apply_zdrop (ksw2.h:181-197)
          if (max_H > ez_max) {
            ez_max = max_H, max_t = mt, max_q = r - mt;
          } else if (need_mt && mt >= max_t && r - mt >= max_q) {
            const int tl = mt - max_t, ql = (r - mt) - max_q, l = tl > ql ? tl - ql : ql - tl;
            if (zdrop >= 0 && ez_max - max_H > zdrop + l * ez_e) zdropped = 1, done = true;
          }
          if (!done) {
            if (r == qlen + tlen - 2 && en0 == tlen - 1) score = Hen0;
            if (D2) {
              if (flag & KSW2G_EXTZ_ONLY) {  // early stop, ksw2_extd2_sse.c:361-367
                const int32_t rH = last_max_H > max_H ? last_max_H : max_H;
                const int32_t rq = qlen - (r - st0), rt = tlen - en0;
                const int32_t rm = rq >= tlen - st0 ? tlen - st0
                                   : rt >= qlen - (r - en0) ? qlen - (r - en0)
                                                            : tlen + qlen - 1 - r;
                if (rH + rm * P.max_sc + end_bonus < ez_max) done = true;
              }
              last_max_H = max_H;
            }
          }
        } else {
          // approximate max: follow one cell per anti-diagonal
          auto bytev = [&](const uint32_t(&A)[K], int p) -> uint32_t {
            const int pp = p - base, ws = pp >> 2;
            return (__shfl_sync(gm, pick<K>(A, ws / G), ws & (G - 1), G) >> (8 * (pp & 3))) & 0xffu;
          };
          bool zd = false;
          if (r > 0) {
            const bool in1 = last_H0_t >= st0 && last_H0_t <= en0, in2 = last_H0_t + 1 >= st0 && last_H0_t + 1 <= en0;
            if (in1 && in2) {
              const int32_t d0 = vv(bytev(V, last_H0_t)), d1 = vv(bytev(U, last_H0_t + 1));
              if (d0 > d1) Hz += d0;
              else Hz += d1, ++last_H0_t;
            } else if (in1) {
              Hz += vv(bytev(V, last_H0_t));
            } else {
              ++last_H0_t;
              Hz += vv(bytev(U, last_H0_t));
            }
            if (!D2) zd = true;
          } else {
            Hz = vv(bytev(V, 0)) - qe, last_H0_t = 0;
          }
          if (D2) zd = true;
          if (zd && (flag & KSW2G_APPROX_DROP)) {
            if (Hz > ez_max) {
              ez_max = Hz, max_t = last_H0_t, max_q = r - last_H0_t;
            } else if (last_H0_t >= max_t && r - last_H0_t >= max_q) {
              const int tl = last_H0_t - max_t, ql = (r - last_H0_t) - max_q, l = tl > ql ? tl - ql : ql - tl;
              if (zdrop >= 0 && ez_max - Hz > zdrop + l * ez_e) zdropped = 1, done = true;
            }
          }
          if (!done && r == qlen + tlen - 2 && en0 == tlen - 1) score = Hz;
        }
        ++r;
        if (r == qlen + tlen - 1) done = true;
      }
    }
    if (done) {
      // ---------------- finish the pair: choose the backtrack start (ksw2_extz2_sse.c:284-295) ----------------
      int reach_end = 0, i0 = -1, j0 = -1;
      if (CIG) {
        if (!zdropped && !(flag & KSW2G_EXTZ_ONLY)) i0 = tlen - 1, j0 = qlen - 1;
        else if ((flag & KSW2G_EXTZ_ONLY) && mqe + end_bonus > ez_max) reach_end = 1, i0 = mqe_t, j0 = qlen - 1;
        else if (max_t >= 0 && max_q >= 0) i0 = max_t, j0 = max_q;
      }
      if (k == 0) {
        ksw2g_ext_result o;
        o.score = score, o.max = ez_max, o.max_q = max_q, o.max_t = max_t, o.mqe = mqe, o.mqe_t = mqe_t;
        o.mte = mte, o.mte_q = mte_q, o.zdropped = zdropped, o.reach_end = reach_end, o.n_cigar = 0;
        o.n_diag = n_diag, o.cigar_off = 0, o.cells = cells;
        res[jid] = o;
        if (CIG) bts[jid] = ksw2g_bt{i0, j0, n_diag, 0};
      }
      need = true;
    }
  }
}

}  // namespace ksw2g
