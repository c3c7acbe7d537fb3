// ext16_dp.cuh -- banded anti-diagonal DP for ksw_extz2_sse / ksw_extd2_sse on sm_103a,
// with the reference's byte lanes held in 16-bit halves and the DP step on DPX instructions.
//
// Representation.  Every byte b of the reference's arrays (u, v, x, y[, x2, y2], the score
// row) lives in one 16-bit half of a register as a multiple of 8 in [0, 2040]:
//   K form  K(b) = ((b + 128) mod 256) << 3   -- unsigned order of K(b) = signed order of b
//   R form  R(b) = (b mod 256) << 3           -- unsigned order of R(b) = unsigned order of b
// A wrapping byte addition is one 32-bit add of the two halves plus a constant, then a mask
// of bits 3-10 (the halves never carry into each other: every sum stays below 65536), so
// the int8 wrap-around of the reference -- which does occur, in the padding cells of the
// band -- is reproduced exactly.  The three low bits are free: the candidates of the cell
// maximum (score, x+v, y+u[, x2+v, y2+u]) carry a code there, so one unsigned 16x2 max
// (__vimax3_u16x2) returns both the reference's maximum and the candidate its strict
// (left-aligned gaps) or non-strict (right-aligned gaps) comparison chain picks, which is
// the traceback state (ksw2_extd2_sse.c:227-235, 274-282; ksw2_extz2_sse.c:169-179,
// 195-205).  Gap-state updates max(a, 0) - qe are one __viaddmax_s16x2, their traceback
// flags one __viaddmin_s16x2 each, and the flag bits are merged with multiply-adds on the
// FMA pipe.
//
// extd2 holds everything in K form (all its comparisons are signed).  extz2 mixes signed and
// unsigned comparisons (ksw2_extz2_sse.c:18-39: max_epi8 with a, max_epu8 with b, min_epu8
// with the score cap), so its z runs in K form up to the signed step and in R form after it;
// its v is kept in R form, the form ksw2 reads it in for H (uint8_t - qe).
//
// Mapping, window, boundaries, the query bytes handed from unit to unit, the exact maximum
// and the job loop are those of ext_dp_kernel (ext_dp.cuh): a group of G threads owns a
// pair, thread k holds units k, k+G, ... of 4 cells (two registers per array and unit:
// cells 0-1 and 2-3), the window slides by 16 cells with the reference's first padded
// block, units past the last live block are skipped, and the traceback of a unit is one
// 32-bit store.  Per unit this kernel issues about as many instructions as the byte-lane
// kernel and holds twice the registers, so it is the second lane width of the shape
// autotuner rather than the default.
#pragma once
#include "ext_dp.cuh"

namespace ksw2g {

namespace x16 {
constexpr uint32_t kM = 0x07f807f8u;  // the byte field of both halves
__device__ __forceinline__ uint32_t dup(uint32_t h) { return (h & 0xffffu) | (h << 16); }
// K form of a raw byte (one half)
__device__ __forceinline__ uint32_t kf(uint32_t raw) { return ((raw ^ 0x80u) & 0xffu) << 3; }
// R form of a raw byte (one half)
__device__ __forceinline__ uint32_t rf(uint32_t raw) { return (raw & 0xffu) << 3; }
// the byte field of the low / high half, zero-extended
__device__ __forceinline__ int32_t lo8(uint32_t w) { return (int32_t)__byte_perm(w >> 3, 0u, 0x4440); }
__device__ __forceinline__ int32_t hi8(uint32_t w) { return (int32_t)__byte_perm(w >> 3, 0u, 0x4442); }
// replace the half of cell c (0..3) of (L, H) with the 16-bit value h
__device__ __forceinline__ void set_cell(uint32_t &L, uint32_t &H, int c, uint32_t h) {
  const int sh = 16 * (c & 1);
  const uint32_t keep = ~(0xffffu << sh);
  if (c < 2) L = (L & keep) | (h << sh);
  else H = (H & keep) | (h << sh);
}
}  // namespace x16

// resident blocks per SM asked of a shape (two registers per array and unit)
template <int VAR, int K>
constexpr int ext16_min_blocks() {
  return K <= 1 ? 6 : K <= 3 ? 4 : K <= 5 ? 3 : 2;
}

// VAR: 0 = extz2 (affine), 1 = extd2 (dual affine)
// MODE: 0 = score only, 1 = left-aligned gaps with traceback, 2 = right-aligned gaps with traceback
// Exact for 0 <= q, e, q2, e2 and q+e, q2+e2 <= 128 (ext16_params_ok), where x = max(a,0) - qe
// cannot wrap; every other operation wraps as the reference's bytes do.
template <int VAR, int MODE, int G, int K>
__global__ void __launch_bounds__(128, ext16_min_blocks<VAR, K>())
ext16_dp_kernel(const ksw2g_job *__restrict__ jobs, const int32_t *__restrict__ order, int n_jobs,
                const uint8_t *__restrict__ arena, const ksw2g_ext_params P, ksw2g_ext_result *__restrict__ res,
                ksw2g_bt *__restrict__ bts, uint8_t *__restrict__ tb_pool, const int64_t *__restrict__ tb_off,
                int *__restrict__ job_counter) {
  using namespace x16;
  constexpr bool D2 = VAR == 1;
  constexpr bool CIG = MODE != 0;
  const int lane = threadIdx.x & 31;
  const int k = lane & (G - 1);
  const unsigned gm = group_mask<G>();

  // ---- batch constants ----
  // score bytes are kept XOR 0x80 (the K form's bias): extd2 s, extz2 s + 2(q+e) (ksw2_extz2_sse.c:19)
  const uint32_t mch4 = splat8(D2 ? P.c_mch : P.c_mch + P.c_qe2) ^ 0x80808080u;
  const uint32_t mis4 = splat8(D2 ? P.c_mis : P.c_mis + P.c_qe2) ^ 0x80808080u;
  const uint32_t N4 = splat8(D2 ? P.c_N : P.c_N + P.c_qe2) ^ 0x80808080u;
  const uint32_t m14 = splat8(P.c_m1);
  const bool nt4 = P.c_m1 == 4;
  const uint32_t sc_lo = (mch4 & 0xffu) | (mis4 & 0xffffff00u), sc_hi = N4;
  const uint32_t initb = D2 ? (uint32_t)(uint8_t)(-P.q - P.e) : 0u;
  const uint32_t init2b = D2 ? (uint32_t)(uint8_t)(-P.q2 - P.e2) : 0u;
  const uint32_t s_init4 = (D2 ? 0u : splat8(P.c_qe2)) ^ 0x80808080u;
  // initial halves: u, x, y (x2, y2) in K form; v in K form (extd2) or R form (extz2)
  const uint32_t iK = dup(kf(initb)), iK2 = dup(kf(init2b)), iV = D2 ? iK : dup(rf(0u));
  // candidate codes in the low three bits: left-aligned gaps take the first maximum of
  // (score, a, b, a2, b2) -- codes 7..3, d = 7 - code; right-aligned the last -- codes 0..4, d = code
  constexpr uint32_t cS = MODE == 1 ? 7u : 0u, cA = MODE == 1 ? 6u : MODE == 2 ? 1u : 0u,
                     cB = MODE == 1 ? 5u : MODE == 2 ? 2u : 0u, cA2 = MODE == 1 ? 4u : MODE == 2 ? 3u : 0u,
                     cB2 = MODE == 1 ? 3u : MODE == 2 ? 4u : 0u;
  const uint32_t qK = (uint32_t)P.q << 3, q2K = (uint32_t)P.q2 << 3;
  const uint32_t qeK = (uint32_t)(P.q + P.e) << 3, qe2K = (uint32_t)(P.q2 + P.e2) << 3;
  // extd2: z = min_epi8(z, mat[0]) (ksw2_extd2_sse.c:192); extz2: min_epu8(z, mat[0] + 2(q+e)) (extz2:34, R form)
  const uint32_t zcap = D2 ? dup(kf(P.c_mch) | (MODE ? 7u : 0u)) : dup(rf(P.c_maxsc) | (MODE ? 7u : 0u));
  // extz2 reads u, v through uint8_t and subtracts q+e; extd2 through int8_t
  const int qe = P.qe_scalar;
  const int ez_e = D2 ? P.e2 : P.e;
  const int vbias = D2 ? 128 : P.qe_scalar;  // v = field - vbias
  auto vv_l = [&](uint32_t w) -> int32_t { return lo8(w) - vbias; };
  auto vv_h = [&](uint32_t w) -> int32_t { return hi8(w) - vbias; };
  auto uu = [&](int32_t field) -> int32_t { return D2 ? field - 128 : (int32_t)((uint32_t)field ^ 0x80u) - qe; };
  auto vvf = [&](int32_t field) -> int32_t { return field - vbias; };

  // ---- per-unit state ----
  uint32_t UL[K], UH[K], VL[K], VH[K], XL[K], XH[K], YL[K], YH[K], X2L[K], X2H[K], Y2L[K], Y2H[K];
  uint32_t S[K + 1], TW[K + 1];
  uint32_t QW[K];  // query bytes of every unit's cells on this anti-diagonal (as in ext_dp_kernel)
  int32_t H0[K], H1[K], H2[K], H3[K];

  // ---- per-group state (identical in every thread of the group) ----
  int jid = -1, qlen = 0, tlen = 0, w = 0, zdrop = 0, end_bonus = 0, flag = 0;
  int r = 0, wb = 0, top = 0, ncol16 = 0, n_diag = 0;
  int64_t cells = 0;
  const uint8_t *qp = nullptr, *tp = nullptr;
  uint8_t *tb = nullptr;
  int32_t ez_max = 0, max_q = -1, max_t = -1, mqe = KSW2G_NEG_INF, mqe_t = -1, mte = KSW2G_NEG_INF, mte_q = -1;
  int32_t score = KSW2G_NEG_INF, zdropped = 0, last_max_H = 0, Hz = 0, last_H0_t = 0;
  int32_t hA = 0, hB = 0, last_en0 = 0;
  bool active = false, need = true;

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
          UL[i] = UH[i] = XL[i] = XH[i] = YL[i] = YH[i] = iK;
          VL[i] = VH[i] = iV;
          X2L[i] = X2H[i] = Y2L[i] = Y2H[i] = iK2;
          H0[i] = H1[i] = H2[i] = H3[i] = KSW2G_NEG_INF;
          QW[i] = 0u;
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
      if (st0 > en0) {  // ksw2_extz2_sse.c:103-106
        zdropped = 1;
        done = true;
      } else {
        const int stb = st0 >> 4, enb = en0 >> 4;
        uint32_t x1, v1, x21 = 0;  // halves of the cell before the band start (K form; extz2 v1 R form)
        if (stb != wb) {  // the first padded block moved right by one: slide the window by four units
          const uint32_t xr = __shfl_sync(gm, XH[0], 3, G) >> 16;
          const uint32_t vr = __shfl_sync(gm, VH[0], 3, G) >> 16;
          uint32_t x2r = 0;
          if (D2) x2r = __shfl_sync(gm, X2H[0], 3, G) >> 16;
          shift4<G, K>(UL, iK, k, gm), shift4<G, K>(UH, iK, k, gm);
          shift4<G, K>(VL, iV, k, gm), shift4<G, K>(VH, iV, k, gm);
          shift4<G, K>(XL, iK, k, gm), shift4<G, K>(XH, iK, k, gm);
          shift4<G, K>(YL, iK, k, gm), shift4<G, K>(YH, iK, k, gm);
          if (D2) {
            shift4<G, K>(X2L, iK2, k, gm), shift4<G, K>(X2H, iK2, k, gm);
            shift4<G, K>(Y2L, iK2, k, gm), shift4<G, K>(Y2H, iK2, k, gm);
          }
          shift4<G, K + 1>(S, s_init4, k, gm);
          shift4<G, K + 1>(TW, 0u, k, gm);
          shift4<G, K>(QW, 0u, k, gm);
          shift4<G, K>(H0, (int32_t)KSW2G_NEG_INF, k, gm);
          shift4<G, K>(H1, (int32_t)KSW2G_NEG_INF, k, gm);
          shift4<G, K>(H2, (int32_t)KSW2G_NEG_INF, k, gm);
          shift4<G, K>(H3, (int32_t)KSW2G_NEG_INF, k, gm);
          wb = stb;
          if (k >= G - 4) {
            TW[K] = ld_tw(tp, (wb << 4) + 4 * (k + G * K), tlen);
            QW[K - 1] = ld_qw(qp, r - 1 - ((wb << 4) + 4 * (k + G * (K - 1))), qlen);
          }
          x1 = xr, v1 = vr, x21 = x2r;  // (r-1, st-1) was computed on the last anti-diagonal
        } else {
          x1 = kf(initb), v1 = D2 ? kf(initb) : rf(0u), x21 = kf(init2b);
        }
        const uint32_t vb = D2 ? (r == 0 ? (uint32_t)(uint8_t)(-P.q - P.e)
                                  : r < P.long_thres ? (uint32_t)(uint8_t)(-P.e)
                                  : r == P.long_thres ? (uint32_t)(uint8_t)P.long_diff
                                                      : (uint32_t)(uint8_t)(-P.e2))
                               : (r ? P.c_q : 0u);
        if (stb == 0) x1 = kf(initb), x21 = kf(init2b), v1 = D2 ? kf(vb) : rf(vb);  // extz2:114, extd2:148-151
        const int base = wb << 4;
        const int en = (enb << 4) + 15;
        if (enb > top) {
          // a 16-cell block enters the band: it gets the state the reference's untouched memory holds
          top = enb;
          const int wtop = (enb - wb) << 2;
#pragma unroll
          for (int i = 0; i < K; ++i) {
            const bool e = ((k + G * i) & ~3) == wtop;
            UL[i] = e ? iK : UL[i], UH[i] = e ? iK : UH[i], VL[i] = e ? iV : VL[i], VH[i] = e ? iV : VH[i];
            XL[i] = e ? iK : XL[i], XH[i] = e ? iK : XH[i], YL[i] = e ? iK : YL[i], YH[i] = e ? iK : YH[i];
            if (D2) {
              X2L[i] = e ? iK2 : X2L[i], X2H[i] = e ? iK2 : X2H[i];
              Y2L[i] = e ? iK2 : Y2L[i], Y2H[i] = e ? iK2 : Y2H[i];
            }
          }
        }
        if (en >= r) {  // top row boundary (ksw2_extz2_sse.c:115, ksw2_extd2_sse.c:152-155)
          const int pr = r - base, wr = pr >> 2, c = pr & 3;
#pragma unroll
          for (int i = 0; i < K; ++i) {
            if (k + G * i == wr) {
              set_cell(YL[i], YH[i], c, kf(initb));
              set_cell(UL[i], UH[i], c, kf(vb));
              if (D2) set_cell(Y2L[i], Y2H[i], c, kf(init2b));
            }
          }
        }
        // the last cell of x, v (and x2) and the last query byte of every unit go to the next
        // unit's owner: [x(t+3), v(t+3)] and [query byte, -, x2(t+3)]
        uint32_t rv[K], rv2[K];
        {
          uint32_t pk[K], pk2[K];
#pragma unroll
          for (int i = 0; i < K; ++i) {
            pk[i] = __byte_perm(XH[i], VH[i], 0x7632);
            pk2[i] = __byte_perm(D2 ? X2H[i] : 0u, QW[i], 0x3247);
          }
#pragma unroll
          for (int i = 0; i < K; ++i) {
            const uint32_t send = (k == G - 1) ? (i > 0 ? pk[i > 0 ? i - 1 : 0] : 0u) : pk[i];
            rv[i] = __shfl_sync(gm, send, (k - 1) & (G - 1), G);
            const uint32_t send2 = (k == G - 1) ? (i > 0 ? pk2[i > 0 ? i - 1 : 0] : 0u) : pk2[i];
            rv2[i] = __shfl_sync(gm, send2, (k - 1) & (G - 1), G);
          }
          if (k == 0) {
            const int qi = r - base;
            const uint32_t qin = qi >= 0 && qi < qlen ? (uint32_t)__ldg(qp + qi) : 0u;
            rv[0] = x1 | (v1 << 16), rv2[0] = (x21 << 16) | qin;
          }
#pragma unroll
          for (int i = 0; i < K; ++i) QW[i] = __byte_perm(rv2[i], QW[i], 0x6540);
        }
        // ---- substitution scores written by the 16-byte stores from st0 (ksw2_extz2_sse.c:117-136) ----
        {
          const bool generic = flag & KSW2G_GENERIC_SC;
          const int fend = generic ? en0 : st0 + (((en0 - st0) >> 4) << 4) + 15;
          const int o = (r + 1) & 3;
          const uint32_t qsel = (uint32_t)((o + 3) | ((o + 2) << 4) | ((o + 1) << 8) | (o << 12));
          uint32_t bad = generic || !nt4 ? 0xffffffffu : 0u;
#pragma unroll
          for (int i = 0; i <= K; ++i) {
            const int p0 = base + 4 * (k + G * i);
            if (i < K || (p0 + 3 >= st0 && p0 <= fend)) {
              uint32_t Qw;
              if (i < K) {
                Qw = QW[i];
              } else {
                const int idx0 = max(r - p0 - 3, r - fend - 3);
                const uint32_t *qa = (const uint32_t *)(qp + (idx0 & ~3));
                Qw = __byte_perm(__ldg(qa), __ldg(qa + 1), qsel);
              }
              const uint32_t Tw = TW[i];
              const uint32_t tq = Tw | Qw;
              const uint32_t ix = ((Tw ^ Qw) & 0x03030303u) | (tq & 0x04040404u);
              const uint32_t sn = __byte_perm(sc_lo, sc_hi, __byte_perm(ix | (ix >> 4), 0u, 0x4420));
              bad |= tq | (tq + 0x03030303u);
              // slots above 0 start above st0 (the window starts at st0's 16-cell block)
              const uint32_t wm = i == 0 ? lanes_from(st0 - p0) & lanes_upto(fend - p0) : lanes_upto(fend - p0);
              S[i] = (S[i] & ~wm) | (sn & wm);
            }
          }
          if (bad & 0xf8f8f8f8u) {
#pragma unroll
            for (int i = 0; i <= K; ++i) {
              const int p0 = base + 4 * (k + G * i);
              if (p0 + 3 >= st0 && p0 <= fend) {
                uint32_t Qw;
                if (i < K) {
                  Qw = QW[i];
                } else {
                  const int idx0 = r - p0 - 3;
                  const uint32_t *qa = (const uint32_t *)(qp + (idx0 & ~3));
                  Qw = __byte_perm(__ldg(qa), __ldg(qa + 1), qsel);
                }
                const uint32_t Tw = TW[i];
                uint32_t sn;
                if (!generic) {
                  const uint32_t eq = eqz8(Tw ^ Qw);
                  const uint32_t nn = eqz8(Tw ^ m14) | eqz8(Qw ^ m14);
                  sn = sel(bmask(eq), mch4, mis4);
                  sn = sel(bmask(nn), N4, sn);
                } else {
                  sn = 0;
#pragma unroll
                  for (int b = 0; b < 4; ++b) {
                    const int tc = (Tw >> (8 * b)) & 0xff, qc = (Qw >> (8 * b)) & 0xff;
                    uint32_t v = (uint32_t)(uint8_t)P.mat[(tc * P.m + qc) & 255];
                    if (!D2) v = (v + P.c_qe2) & 0xffu;
                    sn |= (v ^ 0x80u) << (8 * b);
                  }
                }
                const uint32_t wm = lanes_from(st0 - p0) & lanes_upto(fend - p0);
                S[i] = (S[i] & ~wm) | (sn & wm);
              }
            }
          }
        }
        // ---- cells st..en of the anti-diagonal (ksw2_extz2_sse.c:142-215, ksw2_extd2_sse.c:183-314) ----
        const int nlive = (enb - wb + 1) << 2;
        uint32_t *row = CIG ? (uint32_t *)(tb + (size_t)r * ncol16) : nullptr;
        const bool extq = !D2 && k == 0 && (x1 < 0x400u || v1 >= 0x400u);  // extz2:138-139 sign extension
#pragma unroll
        for (int i = 0; i < K; ++i) {
          const int wi = k + G * i;
          if (wi >= nlive) continue;  // past the last live block: never read before it is reset
          // neighbours: x, v at t-1 .. t+2 of the last anti-diagonal
          uint32_t xL = __byte_perm(rv[i], XL[i], 0x5410), xH = __byte_perm(XL[i], XH[i], 0x5432);
          uint32_t vL = __byte_perm(rv[i], VL[i], 0x5432), vH = __byte_perm(VL[i], VH[i], 0x5432);
          if (!D2 && i == 0 && extq) {
            // _mm_cvtsi32_si128 of a negative int8 fills lanes 1-3 of the first block with 0xff
            if (x1 < 0x400u) xL = (xL & 0xffffu) | (kf(0xffu) << 16), xH = dup(kf(0xffu));
            if (v1 >= 0x400u) vL = (vL & 0xffffu) | (rf(0xffu) << 16), vH = dup(rf(0xffu));
          }
          // score keys of the four cells
          const uint32_t sL = __byte_perm(S[i], 0u, 0x4140) * 8u + cS * 0x10001u;
          const uint32_t sH = __byte_perm(S[i], 0u, 0x4342) * 8u + cS * 0x10001u;
          const uint32_t uL = UL[i], uH = UH[i];
          uint32_t dL = 0, dH = 0;  // traceback bytes in the low byte of each half
          if (D2) {
            const uint32_t x2L = __byte_perm(rv2[i], X2L[i], 0x5432), x2H = __byte_perm(X2L[i], X2H[i], 0x5432);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint32_t xt = h ? xH : xL, vt = h ? vH : vL, x2t = h ? x2H : x2L, ut = h ? uH : uL;
              const uint32_t yt = h ? YH[i] : YL[i], y2t = h ? Y2H[i] : Y2L[i], st = h ? sH : sL;
              const uint32_t a = ((xt + vt + 0x04000400u) & kM) | (cA * 0x10001u);
              const uint32_t b = ((yt + ut + 0x04000400u) & kM) | (cB * 0x10001u);
              const uint32_t a2 = ((x2t + vt + 0x04000400u) & kM) | (cA2 * 0x10001u);
              const uint32_t b2 = ((y2t + ut + 0x04000400u) & kM) | (cB2 * 0x10001u);
              const uint32_t zk = __vimax3_u16x2(__vimax3_u16x2(st, a, b), a2, b2);
              const uint32_t z = __vminu2(zk, zcap) & kM;  // min_epi8(z, mat[0])
              const uint32_t nu = z - vt + 0x0c000c00u;     // u = z - v(t-1); unmasked, below 5113
              const uint32_t nv = (z - ut + 0x1c001c00u) & kM;  // v = z - u(t)
              // a - (z - q) etc., then x = max(a, 0) - (q+e)
              const uint32_t aa = (a - z + (qK + 0x0c00u - cA) * 0x10001u) & kM;
              const uint32_t bb = (b - z + (qK + 0x0c00u - cB) * 0x10001u) & kM;
              const uint32_t aa2 = (a2 - z + (q2K + 0x0c00u - cA2) * 0x10001u) & kM;
              const uint32_t bb2 = (b2 - z + (q2K + 0x0c00u - cB2) * 0x10001u) & kM;
              const uint32_t nqe = dup(0u - qeK), nqe2 = dup(0u - qe2K);
              const uint32_t fl = dup(0x400u - qeK), fl2 = dup(0x400u - qe2K);
              const uint32_t nx = __viaddmax_s16x2(aa, nqe, fl), ny = __viaddmax_s16x2(bb, nqe, fl);
              const uint32_t nx2 = __viaddmax_s16x2(aa2, nqe2, fl2), ny2 = __viaddmax_s16x2(bb2, nqe2, fl2);
              if (MODE != 0) {
                uint32_t fx, fy, fx2, fy2;
                if (MODE == 1) {  // a > 0 etc. (ksw2_extd2_sse.c:253-264)
                  const uint32_t nfl = dup(0u - (0x400u - qeK)), nfl2 = dup(0u - (0x400u - qe2K));
                  fx = __viaddmin_s16x2(nx, nfl, 0x00080008u), fy = __viaddmin_s16x2(ny, nfl, 0x00080008u);
                  fx2 = __viaddmin_s16x2(nx2, nfl2, 0x00080008u), fy2 = __viaddmin_s16x2(ny2, nfl2, 0x00080008u);
                } else {  // !(0 > a) etc. (ksw2_extd2_sse.c:300-311)
                  fx = __vminu2(__viaddmax_s16x2(aa, 0xfc08fc08u, 0u), 0x00080008u);
                  fy = __vminu2(__viaddmax_s16x2(bb, 0xfc08fc08u, 0u), 0x00080008u);
                  fx2 = __vminu2(__viaddmax_s16x2(aa2, 0xfc08fc08u, 0u), 0x00080008u);
                  fy2 = __vminu2(__viaddmax_s16x2(bb2, 0xfc08fc08u, 0u), 0x00080008u);
                }
                uint32_t d = MODE == 1 ? ((~zk & 0x00070007u) | fx) : ((zk & 0x00070007u) | fx);
                d += fy * 2u + fx2 * 4u + fy2 * 8u;
                if (h) dH = d;
                else dL = d;
              }
              if (h) UH[i] = nu, VH[i] = nv, XH[i] = nx, YH[i] = ny, X2H[i] = nx2, Y2H[i] = ny2;
              else UL[i] = nu, VL[i] = nv, XL[i] = nx, YL[i] = ny, X2L[i] = nx2, Y2L[i] = ny2;
            }
          } else {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              const uint32_t xt = h ? xH : xL, vt = h ? vH : vL, ut = h ? uH : uL;
              const uint32_t yt = h ? YH[i] : YL[i], st = h ? sH : sL;
              // a = x + v (K + R -> K); b = y + u (K + K -> R)
              const uint32_t a = ((xt + vt) & kM) | (cA * 0x10001u);
              const uint32_t bR = (yt + ut) & kM;
              const uint32_t b = bR ^ ((0x400u | cB) * 0x10001u);
              const uint32_t z1 = __vmaxu2(st, a);  // max_epi8(z, a)
              uint32_t dk = 0;
              if (MODE != 0) dk = __vmaxu2(z1, b);  // b > z (signed) picks the state
              // max_epu8(z, b), min_epu8(z, max_sc) in R form
              const uint32_t z = __vminu2(__vmaxu2(z1 ^ 0x04000400u, bR), zcap) & kM;
              const uint32_t nu = z - vt + 0x0c000c00u;           // K form, unmasked, below 5113
              const uint32_t nv = (z - ut + 0x1c001c00u) & kM;    // R form
              const uint32_t aa = (a - z + (qK + 0x0800u - cA) * 0x10001u) & kM;
              const uint32_t bb = (b - z + (qK + 0x0800u - cB) * 0x10001u) & kM;
              const uint32_t nx = __vmaxu2(aa, 0x04000400u), ny = __vmaxu2(bb, 0x04000400u);  // max_epi8(a, 0)
              if (MODE != 0) {
                uint32_t fx, fy;
                if (MODE == 1) {  // ksw2_extz2_sse.c:181-187
                  fx = __viaddmin_s16x2(nx, 0xfc00fc00u, 0x00080008u);
                  fy = __viaddmin_s16x2(ny, 0xfc00fc00u, 0x00080008u);
                } else {  // ksw2_extz2_sse.c:207-213
                  fx = __vminu2(__viaddmax_s16x2(aa, 0xfc08fc08u, 0u), 0x00080008u);
                  fy = __vminu2(__viaddmax_s16x2(bb, 0xfc08fc08u, 0u), 0x00080008u);
                }
                uint32_t d = MODE == 1 ? ((~dk & 0x00070007u) | fx) : ((dk & 0x00070007u) | fx);
                d += fy * 2u;
                if (h) dH = d;
                else dL = d;
              }
              if (h) UH[i] = nu, VH[i] = nv, XH[i] = nx, YH[i] = ny;
              else UL[i] = nu, VL[i] = nv, XL[i] = nx, YL[i] = ny;
            }
          }
          if (CIG) row[wi] = __byte_perm(dL, dH, 0x6420);
        }
        ++n_diag;
        cells += en0 - st0 + 1;
        // ---- exact or approximate max, z-drop (ksw2_extz2_sse.c:216-278, ksw2_extd2_sse.c:315-385) ----
        if (!(flag & KSW2G_APPROX_MAX)) {
          const int pe = en0 - base, ws = pe >> 2, bs = pe & 3;
          int32_t Hen0;
          if (r == 0) {
            Hen0 = vvf(__shfl_sync(gm, (int32_t)lo8(VL[0]), 0, G)) - qe;
          } else if (en0 > 0) {
            // H[en0] = H[en0 - 1] + u[en0]: H[en0 - 1] is the last anti-diagonal's H[en0] when en0
            // moved up, else its H[en0 - 1] (hA, hB carry them)
            const int32_t hm1 = en0 > last_en0 ? hA : hB;
            const uint32_t uw = __shfl_sync(gm, bs < 2 ? pick<K>(UL, ws / G) : pick<K>(UH, ws / G), ws & (G - 1), G);
            Hen0 = hm1 + uu((int32_t)((uw >> (3 + 16 * (bs & 1))) & 0xffu));
            hB = hm1;
            if (en0 - 1 >= st0) {
              const int pm = pe - 1, cm = pm & 3;
              const uint32_t vw =
                  __shfl_sync(gm, cm < 2 ? pick<K>(VL, (pm >> 2) / G) : pick<K>(VH, (pm >> 2) / G), (pm >> 2) & (G - 1), G);
              hB += vvf((int32_t)((vw >> (3 + 16 * (cm & 1))) & 0xffu));
            }
          } else {
            const uint32_t vw = __shfl_sync(gm, bs < 2 ? pick<K>(VL, ws / G) : pick<K>(VH, ws / G), ws & (G - 1), G);
            Hen0 = hA + vvf((int32_t)((vw >> (3 + 16 * (bs & 1))) & 0xffu));
          }
          hA = Hen0, last_en0 = en0;
          const int se = ws / G;
          const bool own = k == (ws & (G - 1));
          const int lo = st0 - base - 4 * k;
          int32_t lmax = INT32_MIN;
#pragma unroll
          for (int i = 0; i < K; ++i) {
            if (i == 0) {
              H0[0] += lo <= 0 ? vv_l(VL[0]) : 0;
              H1[0] += lo <= 1 ? vv_h(VL[0]) : 0;
              H2[0] += lo <= 2 ? vv_l(VH[0]) : 0;
              H3[0] += lo <= 3 ? vv_h(VH[0]) : 0;
            } else {
              H0[i] += vv_l(VL[i]), H1[i] += vv_h(VL[i]), H2[i] += vv_l(VH[i]), H3[i] += vv_h(VH[i]);
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
              lmax = __vimax3_s32(lmax, max(H0[i], H1[i]), max(H2[i], H3[i]));
            }
          }
          const int32_t gmax = __reduce_max_sync(gm, lmax);
          const bool need_mt = ez_e < 0 || gmax > ez_max || (zdrop >= 0 && ez_max - gmax > zdrop);
          uint32_t key = 0xffffffffu;
          if (need_mt && lmax == gmax) {
            const int E = en0 - st0, L4 = E & ~3;
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
              const int o = base + 4 * (k + G * (j >> 2)) + (j & 3) - st0;
              const uint32_t kk = o == E  ? 0u
                                  : o < L4 ? ((uint32_t)(1 + (o & 3)) << 24) | (uint32_t)o
                                           : (5u << 24) | (uint32_t)o;
              key = min(key, kk);
            }
          }
          if (need_mt) key = __reduce_min_sync(gm, key);
          const int32_t max_H = gmax;
          const int mt = key == 0 ? en0 : st0 + (int)(key & 0xffffffu);
          if (en0 == tlen - 1 && Hen0 > mte) mte = Hen0, mte_q = r - en0;
          if (r - st0 == qlen - 1) {
            const int ps = st0 - base, bsel = ps & 3;
            const int32_t h0 = bsel == 0 ? H0[0] : bsel == 1 ? H1[0] : bsel == 2 ? H2[0] : H3[0];
            const int32_t hs = __shfl_sync(gm, h0, ps >> 2, G);
            if (hs > mqe) mqe = hs, mqe_t = st0;
          }
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
          auto field = [&](const uint32_t(&AL)[K], const uint32_t(&AH)[K], int p) -> int32_t {
            const int pp = p - base, ws = pp >> 2, c = pp & 3;
            const uint32_t wv = __shfl_sync(gm, c < 2 ? pick<K>(AL, ws / G) : pick<K>(AH, ws / G), ws & (G - 1), G);
            return (int32_t)((wv >> (3 + 16 * (c & 1))) & 0xffu);
          };
          bool zd = false;
          if (r > 0) {
            const bool in1 = last_H0_t >= st0 && last_H0_t <= en0, in2 = last_H0_t + 1 >= st0 && last_H0_t + 1 <= en0;
            if (in1 && in2) {
              const int32_t d0 = vvf(field(VL, VH, last_H0_t)), d1 = uu(field(UL, UH, last_H0_t + 1));
              if (d0 > d1) Hz += d0;
              else Hz += d1, ++last_H0_t;
            } else if (in1) {
              Hz += vvf(field(VL, VH, last_H0_t));
            } else {
              ++last_H0_t;
              Hz += uu(field(UL, UH, last_H0_t));
            }
            if (!D2) zd = true;
          } else {
            Hz = vvf(field(VL, VH, 0)) - qe, last_H0_t = 0;
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
