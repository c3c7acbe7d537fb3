// align_pairs.cu -- align.c's mb_align_pair (align.c:329-390) over a batch of pairs.
//
// mb_align1 (align.c:548-757) calls mb_align_pair for every left extension,
// chain gap fill and right extension of a hit; mb_align_pair first tries the
// ungapped shortcuts (an extension whose ungapped score reaches the end with at
// most three mismatches; a gap fill of equal lengths with at most four
// mismatches or a score above any gapped one), shrinks the band of short pairs
// to what their mismatches allow, skips pairs over the DP memory cap, and only
// then calls ksw_extz2_sse or ksw_extd2_sse.  Here the shortcuts and the band
// shrink run on the host while the pairs are read, and every pair that needs
// DP goes into one extz2 or extd2 batch on the device, so a caller can hand
// over all pairs of many reads at once.  Results are those of mb_align_pair:
// the ksw_extz_t fields and the CIGAR, exactly.
#include <cuda_runtime.h>
#include <string.h>

#include <vector>

#include "../../include/ksw2.h"
#include "../../include/ksw2_gb300.h"
#include "batch.h"
#include "host_parallel.h"

using namespace ksw2g;

namespace {

constexpr int32_t kNegInf = -0x40000000;  // KSW_NEG_INF (ksw2.h:8)
constexpr int kMaxBwAdjLen = 100;         // align.c:332

void reset_extz(ksw2g_ext_result_t &r) {  // ksw_reset_extz (ksw2.h:174-179)
  r.max_q = r.max_t = r.mqe_t = r.mte_q = -1;
  r.max = 0, r.score = r.mqe = r.mte = kNegInf;
  r.n_cigar = 0, r.zdropped = 0, r.reach_end = 0;
  r.n_diag = 0, r.cigar_off = 0, r.cells = 0;
}

int32_t max_bw_from_mm(const ksw2g_align_opt_t &o, int32_t mm) {  // align.c:320-326
  const int32_t x = mm * (o.a + o.b);
  int32_t max1 = 0, max2 = 0;
  if (x >= o.q + o.e) max1 = (x - o.q + o.e - 1) / o.e;
  if (x >= o.q2 + o.e2) max2 = (x - o.q2 + o.e2 - 1) / o.e2;
  return max1 > max2 ? max1 : max2;
}

}  // namespace

extern "C" int ksw2g_align_pairs(ksw2g_ctx_t *c, const ksw2g_align_opt_t *opt, const int8_t *mat, int n,
                                 const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
                                 int64_t tbuf_len, ksw2g_ext_result_t *res, uint32_t *cigar, int64_t cigar_cap,
                                 int64_t *cigar_used) {
  if (!c || !opt || !mat || n < 0 || (n > 0 && (!jobs || !res)))
    return report_error(KSW2G_E_ARG, "align_pairs: bad arguments");
  if (opt->e <= 0 || opt->e2 <= 0) return report_error(KSW2G_E_ARG, "align_pairs: gap extensions must be positive");
  if (cigar_used) *cigar_used = 0;
  const ksw2g_align_opt_t &o = *opt;
  const bool dual = !(o.q == o.q2 && o.e == o.e2);
  const int extra_flag = ((o.b_ts != 0 && o.b != o.b_ts) || o.meth) ? KSW_EZ_GENERIC_SC : 0;
  std::vector<uint8_t> shortcut(n, 0);  // 1: ungapped CIGAR of qlen M, 2: no CIGAR, 3: DP, 4: out of bounds
  std::vector<int32_t> band(n, 0);       // the DP band after the shrink of short pairs
  int64_t used = 0;
  // the shortcuts, the band shrink and the memory cap, pair by pair over the host threads
  parallel_for(n, 2048, [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      const ksw2g_job_t &J = jobs[i];
      if (J.qlen < 0 || J.tlen < 0 || J.qoff < 0 || J.toff < 0 || J.qoff + J.qlen > qbuf_len ||
          J.toff + J.tlen > tbuf_len || (J.qlen > 0 && !qbuf) || (J.tlen > 0 && !tbuf)) {
        shortcut[i] = 4;
        continue;
      }
      const uint8_t *qs = qbuf + J.qoff, *ts = tbuf + J.toff;
      const int flag = J.flag | extra_flag;
      int w = J.w;
      int32_t n_mm = -1;
      ksw2g_ext_result_t &R = res[i];
      reset_extz(R);
      if ((flag & KSW_EZ_EXTZ_ONLY) && J.tlen >= J.qlen) {  // ungapped extension (align.c:335-349)
        int32_t score = 0, mx = 0;
        for (int j = 0; j < J.qlen; ++j) {
          const int8_t s = mat[ts[j] * 5 + qs[j]];
          score += s;
          n_mm += (ts[j] > 3 || qs[j] > 3 || s < 0);
          if (mx < score) mx = score, R.max_q = R.max_t = j;
        }
        R.score = score, R.max = mx;
        if (n_mm <= 2) {
          R.mqe = score, R.mqe_t = J.qlen - 1;
          if (R.mqe + J.end_bonus >= R.max) {
            R.reach_end = 1;
            shortcut[i] = 1;
            continue;
          }
        }
      } else if (J.qlen == J.tlen && !(flag & KSW_EZ_EXTZ_ONLY)) {  // ungapped alignment (align.c:350-360)
        const int32_t max_gapped = (J.qlen - 2) * o.a - 2 * (o.q + o.e);
        int32_t score = 0;
        for (int j = 0; j < J.qlen; ++j) {
          const int8_t s = mat[ts[j] * 5 + qs[j]];
          score += s;
          n_mm += (ts[j] > 3 || qs[j] > 3 || s < 0);
        }
        R.score = score;
        if (n_mm <= 3 || score > max_gapped) {
          shortcut[i] = 1;
          continue;
        }
      }
      if (n_mm >= 0 && (J.qlen < J.tlen ? J.qlen : J.tlen) < kMaxBwAdjLen) {  // align.c:362-366
        const int32_t max_bw = max_bw_from_mm(o, n_mm);
        if (w > max_bw + 4) w = max_bw + 4;
      }
      if (o.max_sw_mat > 0 && (int64_t)J.tlen * J.qlen > o.max_sw_mat) {  // align.c:368-370
        reset_extz(R);
        R.zdropped = 1;
        shortcut[i] = 2;
        continue;
      }
      band[i] = w, shortcut[i] = 3;
    }
  });
  std::vector<ksw2g_job_t> dp;
  std::vector<int> dp_idx;
  for (int i = 0; i < n; ++i) {
    if (shortcut[i] == 4) return report_error(KSW2G_E_ARG, "align_pairs: pair out of buffer bounds");
    if (shortcut[i] != 3) continue;
    const ksw2g_job_t &J = jobs[i];
    dp.push_back(ksw2g_job_t{J.qoff, J.toff, J.qlen, J.tlen, band[i], J.zdrop * o.a, J.end_bonus, J.flag | extra_flag});
    dp_idx.push_back(i);
  }
  // DP of the remaining pairs: CIGARs land in the caller's buffer first, the shortcuts' runs after them
  if (!dp.empty()) {
    std::vector<ksw2g_ext_result_t> er(dp.size());
    int64_t u = 0;
    int rc = ksw2g_ext_batch(c, dual, 5, mat, (int8_t)o.q, (int8_t)o.e, (int8_t)o.q2, (int8_t)o.e2, (int)dp.size(),
                             dp.data(), qbuf, qbuf_len, tbuf, tbuf_len, er.data(), cigar, cigar ? cigar_cap : 0, &u);
    if (rc) return rc;
    for (size_t k = 0; k < dp.size(); ++k) res[dp_idx[k]] = er[k];
    if (cigar) used = u;
  }
  for (int i = 0; i < n; ++i) {
    if (shortcut[i] != 1) continue;
    // ksw_push_cigar(MB_CIGAR_MATCH, qlen) onto an empty CIGAR: one run, even of length 0
    res[i].n_cigar = 1;
    if (cigar) {
      if (used + 1 > cigar_cap) return report_error(KSW2G_E_CAPACITY, "align_pairs: CIGAR buffer too small");
      cigar[used] = (uint32_t)jobs[i].qlen << 4 | 0u;
      res[i].cigar_off = used++;
    }
  }
  if (cigar_used) *cigar_used = used;
  return 0;
}
