// ext_split.cuh -- the extension DP of one pair on a whole block, for batches whose few long
// pairs would otherwise each run on one thread group and set the batch's duration.
//
// Mapping.  The NT = 32 NW threads of a block (NW warps, 1 <= NW <= kSplitMaxWarps, set by the
// launch) own one pair at a time.  The window of W = NT*K 32-bit words of every state array of
// the reference (u, v, x, y[, x2, y2], s and the 32-bit H of the exact max) is laid out as in
// ext_dp_kernel over a group: word i covers target positions 16*wb + 4*i .. +3 and belongs to
// thread i % NT, slot i / NT, so that one store of a warp writes 32 consecutive traceback
// words; one more slot holds only scores.  The cell recurrence, the scores and the tie-break
// keys are ext_dp.cuh's.
//
// Per anti-diagonal the block meets at one barrier.  Before it, every thread computes its
// words and writes to shared memory what another warp needs from it:
//  - lane 31 the last bytes of x, v (x2) of its words, the left neighbours of the next warp's
//    lane 0 on the next anti-diagonal;
//  - lane 0 the warp's largest H with the smallest tie-break key among its cells holding it;
//  - the thread holding cell en0 the new H[en0], the one holding en0 - 1 its v byte, the one
//    holding st0 H[st0] when the reference reads it, and under the approximate max the holders
//    of the followed cell its v and u bytes.
// After it, every thread reads the same values and takes the same decisions (maximum, z-drop,
// the extd2 early stop), so control flow stays uniform over the block.  Shared buffers
// alternate between two copies by anti-diagonal parity, so the next anti-diagonal's writes
// never meet this one's reads.  When the band's first 16-cell block moves right (the window
// slides by four words), lanes 0-3 of every warp pass their words through shared memory to
// lanes 28-31 of the warp before, with two more barriers.
#pragma once
#include "ext_dp.cuh"

namespace ksw2g {

constexpr int kSplitMaxWarps = 16;
constexpr int kSplitMaxK = 4;
constexpr int kSplitSlideWords = 12 * kSplitMaxK + 2;  // u v x y x2 y2 h0-h3 (K each), s tw (K + 1 each)

#ifndef KSW2G_BLOCK_SHARED
#ifdef KSW2G_EMU
#define KSW2G_BLOCK_SHARED static
#else
#define KSW2G_BLOCK_SHARED __shared__
#endif
#endif

struct SplitXchg {
  uint32_t nb[2][kSplitMaxWarps][kSplitMaxK];  // [parity][warp][slot]: lane 31's packed x | v << 8 | x2 << 16
  uint64_t wmk[2][kSplitMaxWarps];             // [parity][warp]: (H, key) packed by split_pack
  int32_t pub[2][4];                           // [parity]: H[en0], v at en0 - 1, H[st0]; approximate max: v, u
  int job;
};
// (H, key) packed so that the unsigned maximum is the largest H with the smallest key
__device__ __forceinline__ uint64_t split_pack(int32_t h, uint32_t key) {
  return ((uint64_t)((uint32_t)h ^ 0x80000000u) << 32) | (uint64_t)(0xffffffffu - key);
}

template <int N, typename T>
__device__ __forceinline__ void slide_put(uint32_t *sb, int &o, const T (&a)[N]) {
#pragma unroll
  for (int j = 0; j < N; ++j) sb[o + j] = (uint32_t)a[j];
  o += N;
}
// word i takes word i + 4: lanes 0-27 from lane + 4 of the warp, lanes 28-31 from lanes 0-3 of
// the next warp (nx), the last warp's from warp 0's next slot, or fill past the last slot
template <int N, typename T>
__device__ __forceinline__ void slide_take(const uint32_t *nx, bool lastw, int &o, T (&a)[N], T fill, int lane) {
#pragma unroll
  for (int j = 0; j < N; ++j) {
    T v = __shfl_sync(0xffffffffu, a[j], (lane + 4) & 31);
    if (lane >= 28) v = !lastw ? (T)nx[o + j] : (j + 1 < N ? (T)nx[o + j + 1] : fill);
    a[j] = v;
  }
  o += N;
}
// thread and slot holding window word ws of a block of nt threads
template <int K>
__device__ __forceinline__ int split_slot(int ws, int nt) {
  int s = 0;
#pragma unroll
  for (int i = 1; i < K; ++i) s += ws >= nt * i;
  return s;
}

template <int VAR, int MODE, int K>
__global__ void __launch_bounds__(32 * kSplitMaxWarps, 1)
ext_split_kernel(const ksw2g_job *__restrict__ jobs, const int32_t *__restrict__ order, int n_jobs,
                 const uint8_t *__restrict__ arena, const ksw2g_ext_params P, ksw2g_ext_result *__restrict__ res,
                 ksw2g_bt *__restrict__ bts, uint8_t *__restrict__ tb_pool, const int64_t *__restrict__ tb_off,
                 int *__restrict__ job_counter) {
  constexpr bool D2 = VAR == 1;
  constexpr bool CIG = MODE != 0;
  KSW2G_BLOCK_SHARED SplitXchg xs;
  KSW2G_BLOCK_SHARED uint32_t sbuf[kSplitMaxWarps][4][kSplitSlideWords];
  const int NT = blockDim.x, NW = NT >> 5;
  const int k = threadIdx.x, lane = k & 31, wp = k >> 5;
  const unsigned full = 0xffffffffu;

  const ExtConsts C = ext_consts<VAR>(P);
  const uint32_t initb = C.initb, init2b = C.init2b, init4 = C.init4, init24 = C.init24, s_init4 = C.s_init4;
  const uint32_t pk_init = initb | (initb << 8) | (init2b << 16);
  const int qe = P.qe_scalar;
  const int ez_e = D2 ? P.e2 : P.e;
  auto vv = [&](uint32_t byte) -> int32_t { return ext_vv<VAR>(byte, qe); };

  uint32_t U[K], V[K], X[K], Y[K], X2[K], Y2[K], S[K + 1], TW[K + 1];
  int32_t H0[K], H1[K], H2[K], H3[K];

  for (;;) {
    // ---------------- take the next job (the same for the whole block) ----------------
    if (k == 0) xs.job = atomicAdd(job_counter, 1);
    __syncthreads();
    const int j = xs.job;
    __syncthreads();  // every thread has read it before thread 0 may take the next
    if (j >= n_jobs) return;
    const int jid = order ? order[j] : j;
    const ksw2g_job J = jobs[jid];
    const int qlen = J.qlen, tlen = J.tlen, zdrop = J.zdrop, end_bonus = J.end_bonus, flag = J.flag;
    int w = J.w;
    int32_t ez_max = 0, max_q = -1, max_t = -1, mqe = KSW2G_NEG_INF, mqe_t = -1, mte = KSW2G_NEG_INF, mte_q = -1;
    int32_t score = KSW2G_NEG_INF, zdropped = 0, n_diag = 0;
    int64_t cells = 0;
    if (P.skip_all || qlen <= 0 || tlen <= 0 || P.m <= VAR) {
      // degenerate input: the reference returns right after ksw_reset_extz
      if (k == 0) {
        ksw2g_ext_result o;
        o.score = score, o.max = 0, o.max_q = -1, o.max_t = -1, o.mqe = mqe, o.mqe_t = -1, o.mte = mte, o.mte_q = -1;
        o.zdropped = 0, o.reach_end = 0, o.n_cigar = 0, o.n_diag = 0, o.cigar_off = 0, o.cells = 0;
        res[jid] = o;
        if (CIG) bts[jid] = ksw2g_bt{-1, -1, 0, 0};
      }
      continue;
    }
    if (w < 0) w = tlen > qlen ? tlen : qlen;
    int ncol16;
    {
      int nc = qlen < tlen ? qlen : tlen;
      nc = ((nc < w + 1 ? nc : w + 1) + 15) / 16 + 1;
      ncol16 = nc * 16;
    }
    const uint8_t *qp = arena + J.qoff, *tp = arena + J.toff;
    uint8_t *tb = CIG ? tb_pool + tb_off[jid] : nullptr;
    int r = 0, wb = 0, top = 0;
    int32_t last_max_H = 0, Hz = 0, last_H0_t = 0, hA = 0, hB = 0, last_en0 = 0;
#pragma unroll
    for (int i = 0; i < K; ++i) {
      U[i] = V[i] = X[i] = Y[i] = init4;
      X2[i] = Y2[i] = init24;
      H0[i] = H1[i] = H2[i] = H3[i] = KSW2G_NEG_INF;
    }
#pragma unroll
    for (int i = 0; i <= K; ++i) S[i] = s_init4, TW[i] = ld_tw(tp, 4 * (k + NT * i), tlen);
    // band [s0, e0] of anti-diagonal rr (ksw2_extz2_sse.c:99-102)
    auto band = [&](int rr, int &s0, int &e0) {
      s0 = rr - qlen + 1 > 0 ? rr - qlen + 1 : 0;
      e0 = rr < tlen - 1 ? rr : tlen - 1;
      const int a = (rr - w + 1) >> 1, b = (rr + w) >> 1;
      if (s0 < a) s0 = a;
      if (e0 > b) e0 = b;
    };
    // substitution scores of anti-diagonal rr written by the reference's 16-byte stores from s0
    // (ksw2_extz2_sse.c:117-136), into the window with base bs
    auto scores = [&](int rr, int s0, int e0, int bs) {
      const bool generic = flag & KSW2G_GENERIC_SC;
      const int fend = generic ? e0 : s0 + (((e0 - s0) >> 4) << 4) + 15;
      const int o = (rr + 1) & 3;
      const uint32_t qsel = (uint32_t)((o + 3) | ((o + 2) << 4) | ((o + 1) << 8) | (o << 12));
      uint32_t bad = generic || !C.nt4 ? 0xffffffffu : 0u;
#pragma unroll
      for (int i = 0; i <= K; ++i) {
        const int p0 = bs + 4 * (k + NT * i);
        if (p0 + 3 >= s0 && p0 <= fend) {
          const uint32_t sn = score_lookup(TW[i], ld_qword(qp, rr - p0 - 3, qsel), C, bad);
          const uint32_t wm = lanes_from(s0 - p0) & lanes_upto(fend - p0);
          S[i] = (S[i] & ~wm) | (sn & wm);
        }
      }
      if (bad & 0xf8f8f8f8u) {
#pragma unroll
        for (int i = 0; i <= K; ++i) {
          const int p0 = bs + 4 * (k + NT * i);
          if (p0 + 3 >= s0 && p0 <= fend) {
            const uint32_t sn = score_exact<VAR>(TW[i], ld_qword(qp, rr - p0 - 3, qsel), generic, P, C);
            const uint32_t wm = lanes_from(s0 - p0) & lanes_upto(fend - p0);
            S[i] = (S[i] & ~wm) | (sn & wm);
          }
        }
      }
    };

    // ---------------- anti-diagonals ----------------
    for (bool done = false; !done;) {
      const int p = r & 1;
      int st0, en0;
      band(r, st0, en0);
      if (st0 > en0) {  // ksw2_extz2_sse.c:103-106
        zdropped = 1;
        break;
      }
      const int stb = st0 >> 4, enb = en0 >> 4;
      uint32_t x1, v1, x21 = 0;
      if (stb != wb) {  // the first padded block moved right by one: slide the window
        const uint32_t xr = __shfl_sync(full, X[0], 3) >> 24;
        const uint32_t vr = __shfl_sync(full, V[0], 3) >> 24;
        const uint32_t x2r = D2 ? __shfl_sync(full, X2[0], 3) >> 24 : 0u;
        if (lane < 4) {
          uint32_t *sb = sbuf[wp][lane];
          int o = 0;
          slide_put<K>(sb, o, U), slide_put<K>(sb, o, V), slide_put<K>(sb, o, X), slide_put<K>(sb, o, Y);
          if (D2) slide_put<K>(sb, o, X2), slide_put<K>(sb, o, Y2);
          slide_put<K + 1>(sb, o, S), slide_put<K + 1>(sb, o, TW);
          slide_put<K>(sb, o, H0), slide_put<K>(sb, o, H1), slide_put<K>(sb, o, H2), slide_put<K>(sb, o, H3);
        }
        __syncthreads();
        {
          const bool lastw = wp == NW - 1;
          const uint32_t *nx = sbuf[lastw ? 0 : wp + 1][lane & 3];
          int o = 0;
          slide_take<K>(nx, lastw, o, U, init4, lane), slide_take<K>(nx, lastw, o, V, init4, lane);
          slide_take<K>(nx, lastw, o, X, init4, lane), slide_take<K>(nx, lastw, o, Y, init4, lane);
          if (D2) slide_take<K>(nx, lastw, o, X2, init24, lane), slide_take<K>(nx, lastw, o, Y2, init24, lane);
          slide_take<K + 1>(nx, lastw, o, S, s_init4, lane), slide_take<K + 1>(nx, lastw, o, TW, 0u, lane);
          const int32_t ninf = KSW2G_NEG_INF;
          slide_take<K>(nx, lastw, o, H0, ninf, lane), slide_take<K>(nx, lastw, o, H1, ninf, lane);
          slide_take<K>(nx, lastw, o, H2, ninf, lane), slide_take<K>(nx, lastw, o, H3, ninf, lane);
        }
        wb = stb;
        if (k >= NT - 4) TW[K] = ld_tw(tp, (wb << 4) + 4 * (k + NT * K), tlen);
        x1 = xr, v1 = vr, x21 = x2r;  // (r-1, st-1) was computed on the last anti-diagonal
        // the left neighbours lane 0 reads below, renumbered with the window
        if (lane == 31) {
#pragma unroll
          for (int i = 0; i < K; ++i) {
            uint32_t pk = __byte_perm(X[i], V[i], 0x0073);
            if (D2) pk = __byte_perm(pk, X2[i], 0x0710);
            xs.nb[p ^ 1][wp][i] = pk;
          }
        }
        __syncthreads();
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
      if (enb > top) {  // a 16-byte block enters the band: the state of the reference's untouched memory
        top = enb;
        const int wtop = (enb - wb) << 2;
#pragma unroll
        for (int i = 0; i < K; ++i) {
          const bool e = ((k + NT * i) & ~3) == wtop;
          U[i] = e ? init4 : U[i], V[i] = e ? init4 : V[i], X[i] = e ? init4 : X[i], Y[i] = e ? init4 : Y[i];
          if (D2) X2[i] = e ? init24 : X2[i], Y2[i] = e ? init24 : Y2[i];
        }
      }
      if (en >= r) {  // top row boundary (ksw2_extz2_sse.c:115, ksw2_extd2_sse.c:152-155)
        const int pr = r - base, wr = pr >> 2, sh = (pr & 3) * 8;
        const uint32_t keep = ~(0xffu << sh);
#pragma unroll
        for (int i = 0; i < K; ++i) {
          const bool e = k + NT * i == wr;
          Y[i] = e ? (Y[i] & keep) | (initb << sh) : Y[i];
          U[i] = e ? (U[i] & keep) | (vb << sh) : U[i];
          if (D2) Y2[i] = e ? (Y2[i] & keep) | (init2b << sh) : Y2[i];
        }
      }
      scores(r, st0, en0, base);
      // ---- cells st..en of the anti-diagonal (ksw2_extz2_sse.c:142-215, ksw2_extd2_sse.c:183-314) ----
      const int nlive = (enb - wb + 1) << 2;
      const uint32_t extx = (!D2 && (x1 & 0x80)) ? 0xffffff00u : 0u;  // sign-extended _mm_cvtsi32_si128
      const uint32_t extv = (!D2 && (v1 & 0x80)) ? 0xffffff00u : 0u;
      uint32_t *row = CIG ? (uint32_t *)(tb + (size_t)r * ncol16) : nullptr;
      uint32_t rv[K];
#pragma unroll
      for (int i = 0; i < K; ++i) {
        uint32_t pk = __byte_perm(X[i], V[i], 0x0073);
        if (D2) pk = __byte_perm(pk, X2[i], 0x0710);
        rv[i] = __shfl_up_sync(full, pk, 1);
        if (lane == 0)  // the word before lies in the warp before, or in the last warp's slot before
          rv[i] = r == 0 ? pk_init : wp > 0 ? xs.nb[p ^ 1][wp - 1][i] : i > 0 ? xs.nb[p ^ 1][NW - 1][i - 1] : 0u;
      }
      if (k == 0) rv[0] = x1 | (v1 << 8) | (x21 << 16);
#pragma unroll
      for (int i = 0; i < K; ++i) {
        const int wi = k + NT * i;
        if (wi >= nlive) continue;  // past the last live block: reset before it is first read
        uint32_t xt1 = __byte_perm(rv[i], X[i], 0x6540);  // x[r-1][t-1 .. t+2]
        uint32_t vt1 = __byte_perm(rv[i], V[i], 0x6541);
        if (!D2 && k == 0 && i == 0) xt1 |= extx, vt1 |= extv;
        const uint32_t x2t1 = D2 ? __byte_perm(rv[i], X2[i], 0x6542) : 0u;
        const uint32_t d = ext_cell<VAR, MODE>(xt1, vt1, x2t1, S[i], U[i], V[i], X[i], Y[i], X2[i], Y2[i], C);
        if (CIG) row[wi] = d;
      }
      if (lane == 31) {
#pragma unroll
        for (int i = 0; i < K; ++i) {
          uint32_t pk = __byte_perm(X[i], V[i], 0x0073);
          if (D2) pk = __byte_perm(pk, X2[i], 0x0710);
          xs.nb[p][wp][i] = pk;
        }
      }
      ++n_diag;
      cells += en0 - st0 + 1;
      const bool approx = flag & KSW2G_APPROX_MAX;
      const int pe = en0 - base;
      int32_t hm1 = 0;
      if (!approx) {
        // ---- exact max: H, the warp's maximum and its key (ksw2_extz2_sse.c:216-261) ----
        const int ws = pe >> 2, bs = pe & 3;
        const int se = split_slot<K>(ws, NT);
        const bool own = k == ws - NT * se;
        hm1 = en0 > last_en0 ? hA : hB;  // H[en0 - 1] of the anti-diagonal before
        int32_t Hen0 = 0;
        if (own) {
          if (r == 0) Hen0 = vv(V[0] & 0xff) - qe;
          else if (en0 > 0) Hen0 = hm1 + vv(pick<K>(U, se) >> (8 * bs));
          else Hen0 = hA + vv(pick<K>(V, se) >> (8 * bs));
          xs.pub[p][0] = Hen0;
        }
        if (r > 0 && en0 > 0 && en0 - 1 >= st0) {  // v at en0 - 1, for H[en0 - 1]
          const int pm = pe - 1, wm = pm >> 2, sm = split_slot<K>(wm, NT);
          if (k == wm - NT * sm) xs.pub[p][1] = vv(pick<K>(V, sm) >> (8 * (pm & 3)));
        }
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
          if (i == se) {
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
        if (r - st0 == qlen - 1) {  // H[st0]: slot 0 of thread (st0 - base) / 4
          const int ps = st0 - base, bsel = ps & 3;
          if (k == (ps >> 2)) xs.pub[p][2] = bsel == 0 ? H0[0] : bsel == 1 ? H1[0] : bsel == 2 ? H2[0] : H3[0];
        }
        if (K == 1) {
          // One word a thread: every thread finds the key of its own maximum without a branch,
          // and two warp reductions of the packed (H, key) give the warp's; the cells holding
          // the warp's maximum are those at their thread's maximum where it equals the warp's.
          const int E = en0 - st0, o0 = base + 4 * k - st0;
          uint32_t lkey = 0xffffffffu;
#pragma unroll
          for (int b = 0; b < 4; ++b) {
            const int32_t h = b == 0 ? H0[0] : b == 1 ? H1[0] : b == 2 ? H2[0] : H3[0];
            lkey = h == lmax && b >= lo ? min(lkey, max_key(o0 + b, E)) : lkey;
          }
          const uint32_t hi = (uint32_t)lmax ^ 0x80000000u, lw = 0xffffffffu - lkey;
          const uint32_t mh = __reduce_max_sync(full, hi);
          const uint32_t ml = __reduce_max_sync(full, hi == mh ? lw : 0u);
          if (lane == 0) xs.wmk[p][wp] = ((uint64_t)mh << 32) | ml;
        } else {
          const int32_t wmax = __reduce_max_sync(full, lmax);
          // The key is wanted only where the block's maximum may set a new maximum or z-drop
          // (ksw_apply_zdrop, ksw2.h:181-197); a warp whose own maximum rules both out cannot
          // hold the block's maximum on an anti-diagonal that does.
          const bool need_w = ez_e < 0 || wmax > ez_max || (zdrop >= 0 && ez_max - wmax > zdrop);
          uint32_t key = 0xffffffffu;
          if (need_w) {
            if (lmax == wmax) {
              const int E = en0 - st0;
              uint32_t mm = 0;
#pragma unroll
              for (int i = 0; i < K; ++i) {
                mm |= (H0[i] == wmax ? 1u : 0u) << (4 * i);
                mm |= (H1[i] == wmax ? 2u : 0u) << (4 * i);
                mm |= (H2[i] == wmax ? 4u : 0u) << (4 * i);
                mm |= (H3[i] == wmax ? 8u : 0u) << (4 * i);
              }
              if (lo > 0) mm &= lo >= 4 ? ~0xfu : ~((1u << lo) - 1u);
              while (mm) {
                const int b = __ffs(mm) - 1;
                mm &= mm - 1;
                key = min(key, max_key(base + 4 * (k + NT * (b >> 2)) + (b & 3) - st0, E));
              }
            }
            key = __reduce_min_sync(full, key);
          }
          if (lane == 0) xs.wmk[p][wp] = split_pack(wmax, key);
        }
      } else {
        // ---- approximate max: the followed cell's v and u (ksw2_extz2_sse.c:262-278) ----
        const int ta = r == 0 ? 0 : last_H0_t, tbb = last_H0_t + 1;
        if (ta >= st0 && ta <= en0) {
          const int pa = ta - base, wa = pa >> 2, sa = split_slot<K>(wa, NT);
          if (k == wa - NT * sa) xs.pub[p][0] = (int32_t)((pick<K>(V, sa) >> (8 * (pa & 3))) & 0xffu);
        }
        if (r > 0 && tbb >= st0 && tbb <= en0) {
          const int pb = tbb - base, wb2 = pb >> 2, sb2 = split_slot<K>(wb2, NT);
          if (k == wb2 - NT * sb2) xs.pub[p][1] = (int32_t)((pick<K>(U, sb2) >> (8 * (pb & 3))) & 0xffu);
        }
      }
      __syncthreads();
      // ---- the same decisions in every thread (ksw2_extz2_sse.c:216-278, ksw2_extd2_sse.c:315-385) ----
      if (!approx) {
        uint64_t best;
        {  // the warps' packed maxima, reduced across the lanes of every warp at once
          const uint64_t e = lane < NW ? xs.wmk[p][lane] : 0ull;
          const uint32_t hi = (uint32_t)(e >> 32), lw = (uint32_t)e;
          const uint32_t mh = __reduce_max_sync(full, hi);
          best = ((uint64_t)mh << 32) | __reduce_max_sync(full, hi == mh ? lw : 0u);
        }
        const int32_t max_H = (int32_t)((uint32_t)(best >> 32) ^ 0x80000000u);
        const uint32_t key = 0xffffffffu - (uint32_t)best;
        const int32_t Hen0 = xs.pub[p][0];
        if (r > 0 && en0 > 0) hB = hm1 + (en0 - 1 >= st0 ? xs.pub[p][1] : 0);
        hA = Hen0, last_en0 = en0;
        const bool need_mt = ez_e < 0 || max_H > ez_max || (zdrop >= 0 && ez_max - max_H > zdrop);
        const int mt = key == 0 ? en0 : st0 + (int)(key & 0xffffffu);
        if (en0 == tlen - 1 && Hen0 > mte) mte = Hen0, mte_q = r - en0;
        if (r - st0 == qlen - 1) {
          const int32_t hs = xs.pub[p][2];
          if (hs > mqe) mqe = hs, mqe_t = st0;
        }
        if (max_H > ez_max) {  // ksw_apply_zdrop (ksw2.h:181-197)
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
        bool zd = false;
        if (r > 0) {
          const bool in1 = last_H0_t >= st0 && last_H0_t <= en0, in2 = last_H0_t + 1 >= st0 && last_H0_t + 1 <= en0;
          if (in1 && in2) {
            const int32_t d0 = vv(xs.pub[p][0]), d1 = vv(xs.pub[p][1]);
            if (d0 > d1) Hz += d0;
            else Hz += d1, ++last_H0_t;
          } else if (in1) {
            Hz += vv(xs.pub[p][0]);
          } else {
            ++last_H0_t;
            Hz += vv(xs.pub[p][1]);
          }
          if (!D2) zd = true;
        } else {
          Hz = vv(xs.pub[p][0]) - qe, last_H0_t = 0;
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
    // ---------------- finish the pair: choose the backtrack start (ksw2_extz2_sse.c:284-295) ----------------
    if (k == 0) {
      int reach_end = 0, i0 = -1, j0 = -1;
      if (CIG) {
        if (!zdropped && !(flag & KSW2G_EXTZ_ONLY)) i0 = tlen - 1, j0 = qlen - 1;
        else if ((flag & KSW2G_EXTZ_ONLY) && mqe + end_bonus > ez_max) reach_end = 1, i0 = mqe_t, j0 = qlen - 1;
        else if (max_t >= 0 && max_q >= 0) i0 = max_t, j0 = max_q;
      }
      ksw2g_ext_result o;
      o.score = score, o.max = ez_max, o.max_q = max_q, o.max_t = max_t, o.mqe = mqe, o.mqe_t = mqe_t;
      o.mte = mte, o.mte_q = mte_q, o.zdropped = zdropped, o.reach_end = reach_end, o.n_cigar = 0;
      o.n_diag = n_diag, o.cigar_off = 0, o.cells = cells;
      res[jid] = o;
      if (CIG) bts[jid] = ksw2g_bt{i0, j0, n_diag, 0};
    }
  }
}

}  // namespace ksw2g
