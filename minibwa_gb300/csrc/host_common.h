// host_common.h -- host-side derivations shared by the C ABI and the tests'
// CPU emulation of the kernels.
#pragma once
#include <string.h>
#include <algorithm>
#include "ksw2g.h"

namespace ksw2g {

// Scoring constants, derived exactly as the reference does at the top of
// ksw_extz2_sse (ksw2_extz2_sse.c:48-74) and ksw_extd2_sse (ksw2_extd2_sse.c:67-97).
inline void derive_ext_params(int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2,
                              ksw2g_ext_params &P) {
  memset(&P, 0, sizeof P);
  P.dual = dual, P.m = m;
  if (m <= dual) {
    P.skip_all = 1;
    return;
  }
  P.qe_scalar = q + e;  // extd2 declares qe = q + e before swapping (ksw2_extd2_sse.c:60,70)
  if (dual && q2 + e2 < q + e) std::swap(q, q2), std::swap(e, e2);
  if (!dual) q2 = q, e2 = e;
  P.q = q, P.e = e, P.q2 = q2, P.e2 = e2;
  int max_sc = mat[0], min_sc = mat[1];
  for (int t = 1; t < m * m; ++t) max_sc = std::max(max_sc, (int)mat[t]), min_sc = std::min(min_sc, (int)mat[t]);
  P.max_sc = max_sc, P.min_sc = min_sc;
  if (-min_sc > 2 * (q + e)) P.skip_all = 1;
  P.c_q = (uint8_t)q, P.c_q2 = (uint8_t)q2, P.c_qe = (uint8_t)(q + e);
  P.c_mch = (uint8_t)mat[0], P.c_mis = (uint8_t)mat[1], P.c_m1 = (uint8_t)(m - 1);
  if (!dual) {
    P.c_qe2 = (uint8_t)((q + e) * 2);
    P.c_N = mat[m * m - 1] == 0 ? (uint8_t)(-e) : (uint8_t)mat[m * m - 1];
    P.c_maxsc = (uint8_t)(mat[0] + (q + e) * 2);
  } else {
    P.c_qe2 = (uint8_t)(q2 + e2);
    P.c_N = mat[m * m - 1] == 0 ? (uint8_t)(-e2) : (uint8_t)mat[m * m - 1];
    int lt = e != e2 ? (q2 - q) / (e - e2) - 1 : 0;
    if (q2 + e2 + lt * e2 > q + e + lt * e) ++lt;
    P.long_thres = lt;
    P.long_diff = lt * (e - e2) - (q2 - q) - e2;
  }
  if (m * m <= 256) memcpy(P.mat, mat, m * m);
}

// The 16-bit-lane kernels (ext16_dp.cuh) reproduce every byte operation of the reference with
// its wrap-around, except x = max(a, 0) - (q+e), which they compute without wrapping: exact
// when the gap costs after the extd2 swap are non-negative and q+e, q2+e2 <= 128.
inline bool ext16_params_ok(const ksw2g_ext_params &P) {
  return P.q >= 0 && P.e >= 0 && P.q2 >= 0 && P.e2 >= 0 && P.q + P.e <= 128 && P.q2 + P.e2 <= 128;
}

// the reference's n_col_: 16-byte blocks of one traceback row (ksw2_extz2_sse.c:64-68)
inline int ext_ncol(int qlen, int tlen, int w) {
  if (w < 0) w = tlen > qlen ? tlen : qlen;
  int nc = qlen < tlen ? qlen : tlen;
  return ((nc < w + 1 ? nc : w + 1) + 15) / 16 + 1;
}
// kernel mode of a flag: 0 score only, 1 left-aligned gaps, 2 right-aligned gaps
inline int ext_mode(int flag) { return (flag & KSW2G_SCORE_ONLY) ? 0 : (flag & KSW2G_RIGHT) ? 2 : 1; }
// bytes of one padded sequence slot of the device arena
inline int64_t slot_bytes(int len) { return 32 + (((int64_t)len + 15) & ~(int64_t)15) + 32; }

}  // namespace ksw2g
