// align_chains.cu -- whole chains of align.c's mb_align1 (align.c:548-757) with every DP job
// of every chain issued at once.
//
// mb_align1 walks a hit's anchors and runs one DP call after another: a left extension, one
// gap fill between consecutive anchors, a right extension.  The coordinates of all of them
// follow from the anchors alone -- the loop advances from anchor end to anchor end whatever
// the DP returns (align.c:668-740) -- except that the first gap fill that z-drops ends the
// walk and cancels everything behind it (align.c:698-720).  So the host derives every job of
// every chain up front, sends them to the device in one batch (through ksw2g_align_pairs,
// which keeps mb_align_pair's shortcuts and band shrink), tests the gap fills' first-pass
// CIGARs for a z-drop as mm_test_zdrop does (align.c:26-68; its inversion check, a ksw_ll_i16
// of the reverse complement, runs as one more device batch), reruns the gap fills that need
// the exact second pass (align.c:690-693) in a second batch, and assembles each chain in order,
// discarding the speculative jobs behind a z-drop.  The hit then holds what mb_align1 leaves
// in it before mb_update_extra (align.c:753), which the caller runs.
// The host stages -- deriving the jobs, copying the sequences into the batches, the z-drop
// scans and the assembly -- run over the host threads (host_parallel.h), one chain per item;
// results do not depend on the thread count.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <memory>
#include <vector>

#include "../../include/ksw2.h"
#include "../../include/ksw2_gb300.h"
#include "batch.h"
#include "host_common.h"
#include "host_parallel.h"

using namespace ksw2g;

namespace {

constexpr uint32_t kSeedLongJoin = 0x1, kSeedIgnore = 0x2;  // MB_SEED_* (mbpriv.h:16-17)
constexpr uint32_t kOpM = 0, kOpI = 1, kOpD = 2, kOpN = 3;    // MB_CIGAR_* (minibwa.h:27-30)

inline int32_t min32(int32_t a, int32_t b) { return a < b ? a : b; }

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ksw_gen_nt4_mat (ksw2.h:199-219)
void gen_mat(int8_t *mat, int a, int b, int b_ts, int b_ambi, int mt) {
  const int m = 5;
  a = a < 0 ? -a : a, b = b > 0 ? -b : b, b_ambi = b_ambi > 0 ? -b_ambi : b_ambi;
  for (int i = 0; i < m - 1; ++i) {
    for (int j = 0; j < m - 1; ++j) mat[i * m + j] = (int8_t)(i == j ? a : b);
    mat[i * m + m - 1] = (int8_t)b_ambi;
  }
  for (int j = 0; j < m; ++j) mat[(m - 1) * m + j] = (int8_t)b_ambi;
  if (b_ts != 0 && b_ts != b) {
    b_ts = b_ts > 0 ? -b_ts : b_ts;
    mat[0 * m + 2] = mat[1 * m + 3] = mat[2 * m + 0] = mat[3 * m + 1] = (int8_t)b_ts;
  }
  if (mt == 1) mat[1 * m + 3] = (int8_t)a;
  else if (mt == 2) mat[2 * m + 0] = (int8_t)a;
}

// mb_max_stretch (align.c:522-546): the run of anchors without a gap with the most matches
void max_stretch(const ksw2g_anchor_t *a, int as, int cnt, int &as1, int &cnt1) {
  as1 = as, cnt1 = cnt;
  if (cnt < 2) return;
  int32_t best = -1, best_i = -1, best_len = 0, score = a[as].len, len = 1, i;
  for (i = as + 1; i < as + cnt; ++i) {
    const int32_t lr = (int32_t)(a[i].tpos - a[i - 1].tpos), lq = a[i].qpos - a[i - 1].qpos;
    if (lq == lr) {
      score += lq < a[i].len ? lq : a[i].len, ++len;
    } else {
      if (score > best) best = score, best_len = len, best_i = i - len;
      score = a[i].len, len = 1;
    }
  }
  if (score > best) best = score, best_len = len, best_i = i - len;
  as1 = best_i, cnt1 = best_len;
}

inline int64_t diag_gap(const ksw2g_anchor_t *a, int i) {  // insertion > 0, deletion < 0
  return (int64_t)(a[i].qpos - a[i - 1].qpos) - (a[i].tpos - a[i - 1].tpos);
}

// indices i (relative to as1) of the gaps longer than min_gap; empty unless there are two or more
std::vector<int> long_gaps(const ksw2g_anchor_t *a, int as1, int cnt1, int min_gap) {
  std::vector<int> k;
  for (int i = 1; i < cnt1; ++i) {
    const int64_t g = diag_gap(a + as1, i);
    if (g < -min_gap || g > min_gap) k.push_back(i);
  }
  if (k.size() <= 1) k.clear();
  return k;
}

// mm_filter_bad_seeds (align.c:411-447): anchors between a long insertion and a long deletion
// that nearly cancel (e.g. 1000I20M1000D) are ignored by the gap fill
void filter_bad_seeds(ksw2g_anchor_t *a, int as1, int cnt1, int min_gap, int diff_thres, int max_ext_len,
                      int max_ext_cnt) {
  const std::vector<int> K = long_gaps(a, as1, cnt1, min_gap);
  if (K.empty()) return;
  const int n = (int)K.size();
  ksw2g_anchor_t *b = a + as1;
  int max = 0, max_st = -1, max_en = -1;
  for (int k = 0;; ++k) {
    if (k == n || k >= max_en) {
      if (max_en > 0)
        for (int i = K[max_st]; i < K[max_en]; ++i) b[i].flag |= kSeedIgnore;
      max = 0, max_st = max_en = -1;
      if (k == n) break;
    }
    const int i = K[k];
    int n_ins = 0, n_del = 0, max_diff = 0, max_diff_l = -1;
    int gap = (int)diag_gap(b, i);
    if (gap > 0) n_ins += gap;
    else n_del -= gap;
    const int qs = b[i - 1].qpos;
    const int64_t ts = b[i - 1].tpos;
    for (int l = k + 1; l < n && l <= k + max_ext_cnt; ++l) {
      const int j = K[l];
      if (b[j].qpos - b[j].len - qs > max_ext_len || b[j].tpos - b[j].len - ts > max_ext_len) break;
      gap = (int)diag_gap(b, j);
      if (gap > 0) n_ins += gap;
      else n_del -= gap;
      const int diff = n_ins + n_del - abs(n_ins - n_del);
      if (max_diff < diff) max_diff = diff, max_diff_l = l;
    }
    if (max_diff > diff_thres && max_diff > max) max = max_diff, max_st = k, max_en = max_diff_l;
  }
}

// mm_filter_bad_seeds_alt (align.c:449-484): runs of long gaps in one direction (e.g.
// 1000I20M2000I) are joined into one gap fill over their last anchor
void filter_bad_seeds_alt(ksw2g_anchor_t *a, int as1, int cnt1, int min_gap, int max_ext) {
  const std::vector<int> K = long_gaps(a, as1, cnt1, min_gap);
  if (K.empty()) return;
  const int n = (int)K.size();
  ksw2g_anchor_t *b = a + as1;
  for (int k = 0; k < n;) {
    const int i = K[k];
    int gap1 = (int)diag_gap(b, i);
    int64_t te1 = b[i].tpos;
    int32_t qe1 = b[i].qpos, left_len = b[i].len;
    gap1 = gap1 > 0 ? gap1 : -gap1;
    int l;
    for (l = k + 1; l < n; ++l) {
      const int j = K[l];
      if (b[j].qpos - qe1 > max_ext || b[j].tpos - te1 > max_ext) break;
      int gap2 = (int)diag_gap(b, j);
      const int64_t m_t = b[j - 1].tpos - te1 + left_len;
      const int32_t m_q = b[j - 1].qpos - qe1 + left_len;
      const int m = (int)(m_t < m_q ? m_t : m_q);
      gap2 = gap2 > 0 ? gap2 : -gap2;
      if (m > gap1 + gap2) break;
      te1 = b[j].tpos, qe1 = b[j].qpos, left_len = b[j].len, gap1 = gap2;
    }
    if (l > k + 1) {
      const int end = K[l - 1];
      for (int j = K[k]; j < end; ++j) b[j].flag |= kSeedIgnore;
      b[end].flag |= kSeedLongJoin;
    }
    k = l;
  }
}

// mm_fix_bad_ends (align.c:486-520): drop the anchors at either end of a long-read chain that
// leave its diagonal by more than half the matched length before them
void fix_bad_ends(const ksw2g_anchor_t *a, int as, int cnt, int mlen, int bw, int min_match, int &as1, int &cnt1) {
  as1 = as, cnt1 = cnt;
  if (cnt < 3) return;
  int32_t l, m;
  m = l = a[as].len;
  for (int i = as + 1; i < as + cnt - 1; ++i) {
    if (a[i].flag & kSeedLongJoin) break;
    const int32_t lr = (int32_t)(a[i].tpos - a[i - 1].tpos), lq = a[i].qpos - a[i - 1].qpos, span = a[i].len;
    const int32_t mn = lr < lq ? lr : lq, mx = lr > lq ? lr : lq;
    if (mx - mn > l >> 1) as1 = i;
    l += mn, m += mn < span ? mn : span;
    if (l >= bw << 1 || (m >= min_match && m >= bw) || m >= mlen >> 1) break;
  }
  cnt1 = as + cnt - as1;
  m = l = a[as + cnt - 1].len;
  for (int i = as + cnt - 2; i > as1; --i) {
    if (a[i + 1].flag & kSeedLongJoin) break;
    const int32_t lr = (int32_t)(a[i + 1].tpos - a[i].tpos - a[i + 1].len + a[i].len);
    const int32_t lq = a[i + 1].qpos - a[i].qpos - a[i + 1].len + a[i].len, span = a[i].len;
    const int32_t mn = lr < lq ? lr : lq, mx = lr > lq ? lr : lq;
    if (mx - mn > l >> 1) cnt1 = i + 1 - as1;
    l += mn, m += mn < span ? mn : span;
    if (l >= bw << 1 || (m >= min_match && m >= bw) || m >= mlen >> 1) break;
  }
}

// mb_cal_mblen (map-algo.c:133-150): matched bases of n anchors
int32_t cal_mlen(int n, const ksw2g_anchor_t *a) {
  if (n <= 0) return 0;
  int64_t mlen = a[0].len;
  for (int i = 1; i < n; ++i) {
    const int span = a[i].len, tl = (int32_t)a[i].tpos - (int32_t)a[i - 1].tpos, ql = a[i].qpos - a[i - 1].qpos;
    mlen += tl > span && ql > span ? span : tl < ql ? tl : ql;
  }
  return (int32_t)mlen;
}

// mb_append_cigar (align.c:300-314): a run of the same op as the last one is merged into it
void append_cigar(std::vector<uint32_t> &c, const uint32_t *add, int n) {
  if (n <= 0) return;
  if (!c.empty() && (c.back() & 0xf) == (add[0] & 0xf)) {
    c.back() += add[0] >> 4 << 4;
    c.insert(c.end(), add + 1, add + n);
  } else {
    c.insert(c.end(), add, add + n);
  }
}

// The CIGAR scan of mm_test_zdrop (align.c:26-49): the largest drop of the running score below
// its maximum, less e per diagonal shift, and where it lies (pos[0] target, pos[1] query).
int32_t cigar_zdrop(const ksw2g_chain_opt_t &o, const uint8_t *qseq, const uint8_t *tseq, const uint32_t *cig, int n,
                    const int8_t *mat, int pos[2][2]) {
  int32_t score = 0, max = INT32_MIN, max_zdrop = 0;
  int max_i = -1, max_j = -1, i = 0, j = 0;
  pos[0][0] = pos[0][1] = pos[1][0] = pos[1][1] = -1;
  auto update = [&](int32_t s, int ii, int jj) {  // update_max_zdrop (align.c:11-24)
    if (s < max) {
      const int li = ii - max_i, lj = jj - max_j, diff = li > lj ? li - lj : lj - li;
      const int z = max - s - diff * o.e;
      if (z > max_zdrop) max_zdrop = z, pos[0][0] = max_i, pos[0][1] = ii, pos[1][0] = max_j, pos[1][1] = jj;
    } else {
      max = s, max_i = ii, max_j = jj;
    }
  };
  for (int k = 0; k < n; ++k) {
    const uint32_t op = cig[k] & 0xf, len = cig[k] >> 4;
    if (op == kOpM) {
      for (uint32_t l = 0; l < len; ++l) {
        score += mat[tseq[i + l] * 5 + qseq[j + l]];
        update(score, i + (int)l, j + (int)l);
      }
      i += (int)len, j += (int)len;
    } else if (op == kOpI || op == kOpD || op == kOpN) {
      score -= o.q + o.e * (int32_t)len;
      if (op == kOpI) j += (int)len;
      else i += (int)len;
      update(score, i, j);
    }
  }
  return max_zdrop;
}

// One DP job of a chain.
struct Job {
  int kind;         // 0 left extension, 1 gap fill, 2 right extension
  int anchor;       // gap fills: index i of the anchor they end at (relative to as1)
  int64_t ts, te;   // target window (contig coordinates)
  int32_t qs, qe;   // query window (read coordinates in the aligned orientation)
  int32_t w, end_bonus, zdrop, flag;
  int64_t d1;       // gap fills: matches trimmed off the anchor's end (align.c:676-683)
  int64_t te1;      // gap fills: the anchor end the walk moves to
  int32_t qe1;
  int pass1, pass2;  // index in the first / second batch (-1: none)
  int zcode;        // mm_test_zdrop's result on the first pass
};

struct ChainWork {
  const ksw2g_chain_opt_t *o = nullptr;  // the hit's options
  int as1 = 0, cnt1 = 0, is_sr = 1, rev = 0, mt = 0;
  int64_t tid = 0, ts0 = 0, te0 = 0;
  int32_t qs0 = 0, qe0 = 0;
  int64_t ts_first = 0, te_first = 0;  // chain start after the left-extension region; end of the first anchor
  int32_t qs_first = 0, qe_first = 0;
  int64_t te_last = 0;                 // te1 / qe1 after the walk when no gap fill drops
  int32_t qe_last = 0;
  std::vector<ksw2g_anchor_t> a;       // the hit's anchors, flags as the long-read filters leave them
  std::vector<Job> jobs;
  int64_t win_off = 0;                 // target window [ts0, te0) at tbuf + win_off
};

}  // namespace

// the scores every option set of one call must share: they fix the matrix and the DP batches
bool same_scoring(const ksw2g_chain_opt_t &x, const ksw2g_chain_opt_t &y) {
  return x.a == y.a && x.b == y.b && x.b_ts == y.b_ts && x.b_ambi == y.b_ambi && x.q == y.q && x.e == y.e &&
         x.q2 == y.q2 && x.e2 == y.e2 && x.meth == y.meth && x.max_sw_mat == y.max_sw_mat;
}

extern "C" int ksw2g_align_chains(ksw2g_ctx_t *c, const ksw2g_ref_t *ref, int n_opts, const ksw2g_chain_opt_t *opts,
                                  int n, const ksw2g_chain_t *chains, ksw2g_anchor_t *anchors, int64_t n_anchors,
                                  const uint8_t *qbuf, int64_t qbuf_len, ksw2g_chain_result_t *res, uint32_t *cigar,
                                  int64_t cigar_cap, int64_t *cigar_used) {
  if (!c || !ref || n < 0 || n_anchors < 0 || n_opts <= 0 || !opts || (n > 0 && (!chains || !res || !qbuf || !anchors)))
    return report_error(KSW2G_E_ARG, "align_chains: bad arguments");
  if (cigar_used) *cigar_used = 0;
  if (n == 0) return 0;
  const ksw2g_chain_opt_t &S = opts[0];  // scoring
  if (S.e <= 0 || S.e2 <= 0 || S.a <= 0) return report_error(KSW2G_E_ARG, "align_chains: a, e and e2 must be positive");
  for (int k = 1; k < n_opts; ++k)
    if (!same_scoring(S, opts[k])) return report_error(KSW2G_E_ARG, "align_chains: option sets differ in scoring");
  int rc;
  double t0 = now_ms(), t1;
  for (double &x : c->ch_ms) x = 0;
  for (int64_t &x : c->ch_n) x = 0;
  c->ch_n[0] = n;
  std::vector<ChainWork> W(n);
  int64_t tbuf_len = 0;
  // ---- jobs of every chain, as mb_align1 would issue them if no gap fill z-dropped; chains in
  // parallel, each on its own copy of its anchors (chains of one call must not share anchors)
  std::vector<int> bad(n, 0);
  std::vector<const char *> why(n, nullptr);
  auto derive = [&](int ci) -> int {
    auto fail = [&](const char *msg) { why[ci] = msg; return KSW2G_E_ARG; };
    const ksw2g_chain_t &h = chains[ci];
    ChainWork &cw = W[ci];
    res[ci] = ksw2g_chain_result_t{};
    res[ci].cigar_off = -1, res[ci].cnt = h.cnt, res[ci].score = h.score;
    if (h.cnt <= 0) return 0;
    if (h.as < 0 || h.as + (int64_t)h.cnt > n_anchors || h.qoff < 0 || h.qlen < 0 || h.qoff + (int64_t)h.qlen > qbuf_len ||
        h.meth < 0 || h.meth > 2 || h.opt < 0 || h.opt >= n_opts)
      return fail("align_chains: chain out of bounds");
    const ksw2g_chain_opt_t &o = opts[h.opt];
    cw.o = &o;
    cw.a.assign(anchors + h.as, anchors + h.as + h.cnt);
    ksw2g_anchor_t *a = cw.a.data();  // indices relative to the hit's first anchor
    const int qlen = h.qlen;
    cw.rev = a[0].sid & 1;
    cw.tid = a[0].sid >> 1;
    cw.mt = cw.rev && h.meth ? 3 - h.meth : h.meth;  // l2b_meth_rev
    cw.is_sr = !(o.long_reads || (o.adaptive && qlen > o.max_sr_len));
    const int32_t max_back = cw.is_sr ? 0 : 10;
    const int32_t bw = (int32_t)(o.bw * 1.5 + 1.);
    int32_t bw_long = bw;
    if (!cw.is_sr) {
      bw_long = (int32_t)(o.bw_long * 1.5 + 1.);
      if (bw_long < bw) bw_long = bw;
    }
    const int64_t ctg_len = ref_ctg_len(ref, cw.tid);
    if (ctg_len < 0) return fail("align_chains: anchor contig out of range");
    if (cw.is_sr) {
      max_stretch(a, 0, h.cnt, cw.as1, cw.cnt1);
    } else {
      fix_bad_ends(a, 0, h.cnt, h.mlen, o.bw, o.min_chain_score * 2, cw.as1, cw.cnt1);
      filter_bad_seeds(a, cw.as1, cw.cnt1, 10, 40, o.max_gap >> 1, 10);
      filter_bad_seeds_alt(a, cw.as1, cw.cnt1, 30, o.max_gap >> 1);
    }
    const ksw2g_anchor_t &f = a[cw.as1], &g = a[cw.as1 + cw.cnt1 - 1];
    int64_t ts = f.tpos + 1 - f.len + min32(f.len >> 1, max_back);
    int32_t qs = f.qpos + 1 - f.len + min32(f.len >> 1, max_back);
    int64_t te = g.tpos + 1 - min32(g.len >> 1, max_back);
    int32_t qe = g.qpos + 1 - min32(g.len >> 1, max_back);
    // the DP region (align.c:594-644)
    if (cw.is_sr) {
      cw.qs0 = 0, cw.qe0 = qlen;
      int64_t l = qs;
      l += l * o.a + o.end_bonus > o.q ? (l * o.a + o.end_bonus - o.q) / o.e : 0;
      cw.ts0 = ts - l > 0 ? ts - l : 0;
      l = qlen - qe;
      l += l * o.a + o.end_bonus > o.q ? (l * o.a + o.end_bonus - o.q) / o.e : 0;
      cw.te0 = te + l < ctg_len ? te + l : ctg_len;
    } else {
      cw.ts0 = a[0].tpos + 1 - a[0].len;
      cw.qs0 = a[0].qpos + 1 - a[0].len;
      if (cw.ts0 < 0) cw.ts0 = 0;
      if (cw.qs0 < 0) return fail("align_chains: anchor starts before the read");
      int64_t ts1 = 0;
      int32_t qs1 = 0;
      if (qs > 0 && ts > 0) {
        int64_t l = qs < o.max_gap ? qs : o.max_gap;
        qs1 = qs1 > qs - l ? qs1 : (int32_t)(qs - l);
        cw.qs0 = cw.qs0 < qs1 ? cw.qs0 : qs1;
        l += l * o.a > o.q ? (l * o.a - o.q) / o.e : 0;
        l = l < o.max_gap ? l : o.max_gap;
        l = l < ts ? l : ts;
        ts1 = ts1 > ts - l ? ts1 : ts - l;
        cw.ts0 = cw.ts0 < ts1 ? cw.ts0 : ts1;
        cw.ts0 = cw.ts0 < ts ? cw.ts0 : ts;
      } else {
        cw.ts0 = ts, cw.qs0 = qs;
      }
      cw.te0 = a[h.cnt - 1].tpos + 1;
      cw.qe0 = a[h.cnt - 1].qpos + 1;
      int64_t te1 = ctg_len;
      int32_t qe1 = qlen;
      if (qe < qlen && te < ctg_len) {
        int64_t l = qlen - qe < o.max_gap ? qlen - qe : o.max_gap;
        qe1 = qe1 < qe + l ? qe1 : (int32_t)(qe + l);
        cw.qe0 = cw.qe0 > qe1 ? cw.qe0 : qe1;
        l += l * o.a > o.q ? (l * o.a - o.q) / o.e : 0;
        l = l < o.max_gap ? l : o.max_gap;
        l = l < ctg_len - te ? l : ctg_len - te;
        te1 = te1 < te + l ? te1 : te + l;
        cw.te0 = cw.te0 > te1 ? cw.te0 : te1;
      } else {
        cw.te0 = te, cw.qe0 = qe;
      }
    }
    if (!(cw.te0 > cw.ts0) || cw.qs0 < 0 || cw.qe0 > qlen || cw.te0 > ctg_len)
      return fail("align_chains: anchors outside the read or the contig");
    // left extension (align.c:647-659)
    if (qs > 0 && ts > 0) {
      Job j{};
      j.kind = 0, j.ts = cw.ts0, j.te = ts, j.qs = cw.qs0, j.qe = qs;
      j.w = bw, j.end_bonus = o.end_bonus, j.zdrop = h.split_inv ? o.zdrop_inv : o.zdrop;
      j.flag = KSW_EZ_EXTZ_ONLY | KSW_EZ_RIGHT | KSW_EZ_REV_CIGAR;
      cw.jobs.push_back(j);
    }
    cw.ts_first = ts, cw.qs_first = qs;
    // the first anchor's exact match (align.c:663-671)
    te = f.tpos + 1 - min32(f.len >> 1, max_back);
    qe = f.qpos + 1 - min32(f.len >> 1, max_back);
    if (te - ts != qe - qs || te < ts) return fail("align_chains: first anchor is not a match");
    cw.te_first = te, cw.qe_first = qe;
    ts = te, qs = qe;
    int64_t te1 = te;
    int32_t qe1 = qe;
    // gap fills (align.c:673-740), walking as if none z-dropped
    for (int i = 1; i < cw.cnt1; ++i) {
      const ksw2g_anchor_t &ai = a[cw.as1 + i];
      if ((ai.flag & kSeedIgnore) && i != cw.cnt1 - 1) continue;
      te1 = ai.tpos + 1 - min32(ai.len >> 1, max_back);
      qe1 = ai.qpos + 1 - min32(ai.len >> 1, max_back);
      if (i == cw.cnt1 - 1 || (ai.flag & kSeedLongJoin) || (qe1 - qs >= o.min_ksw_len && te1 - ts >= o.min_ksw_len)) {
        int64_t d1 = 0;
        if (ai.len > o.min_len * 2) {
          d1 = te1 - (ai.tpos + 1 - ai.len);
          d1 = d1 < qe1 - qs ? d1 : qe1 - qs;
          d1 = d1 < te1 - ts ? d1 : te1 - ts;
          d1 -= o.min_len;
          if (d1 < o.min_len) d1 = 0;
        }
        te = te1 - d1, qe = (int32_t)(qe1 - d1);
        int32_t bw1 = bw_long;
        if (ai.flag & kSeedLongJoin) bw1 = (int32_t)(qe - qs > te - ts ? qe - qs : te - ts);
        Job j{};
        j.kind = 1, j.anchor = i, j.ts = ts, j.te = te, j.qs = qs, j.qe = qe;
        j.w = bw1, j.end_bonus = -1, j.zdrop = o.zdrop, j.flag = KSW_EZ_APPROX_MAX;
        j.d1 = d1, j.te1 = te1, j.qe1 = qe1;
        if (te < ts || qe < qs) return fail("align_chains: anchors out of order");
        cw.jobs.push_back(j);
        if (d1 > 0) te = te1, qe = qe1;
        ts = te, qs = qe;
      }
    }
    cw.te_last = te1, cw.qe_last = qe1;
    // right extension (align.c:742-751), issued speculatively
    if (qe < cw.qe0 && te < cw.te0) {
      Job j{};
      j.kind = 2, j.ts = te, j.te = cw.te0, j.qs = qe, j.qe = cw.qe0;
      j.w = bw, j.end_bonus = o.end_bonus, j.zdrop = o.zdrop, j.flag = KSW_EZ_EXTZ_ONLY;
      cw.jobs.push_back(j);
    }
    return 0;
  };
  parallel_for(n, 256, [&](int64_t lo, int64_t hi) {
    for (int64_t ci = lo; ci < hi; ++ci) bad[ci] = derive((int)ci);
  });
  for (int ci = 0; ci < n; ++ci) {
    if (bad[ci]) return report_error(bad[ci], why[ci]);
    const ksw2g_chain_t &h = chains[ci];
    ChainWork &cw = W[ci];
    if (h.cnt <= 0) continue;
    if (!cw.is_sr)  // mb_align1 filters the caller's anchors (align.c:571-573)
      for (int k = 0; k < h.cnt; ++k) anchors[h.as + k].flag = cw.a[k].flag;
    if ((rc = ref_check_window(ref, cw.tid, cw.ts0, cw.te0 - cw.ts0))) return rc;
    cw.win_off = tbuf_len;
    tbuf_len += cw.te0 - cw.ts0;
  }
  t1 = now_ms(), c->ch_ms[0] = t1 - t0, t0 = t1;
  // ---- the target windows, decoded from the resident reference and brought to the host
  std::vector<uint8_t> tbuf((size_t)std::max<int64_t>(tbuf_len, 1));
  {
    std::vector<int32_t> tid, len, fl;
    std::vector<int64_t> st, dst;
    int64_t arena = 0;
    for (int ci = 0; ci < n; ++ci)
      if (W[ci].te0 > W[ci].ts0 && chains[ci].cnt > 0) {
        tid.push_back((int32_t)W[ci].tid), st.push_back(W[ci].ts0), len.push_back((int32_t)(W[ci].te0 - W[ci].ts0));
        fl.push_back(0), dst.push_back(arena + 32);
        arena += slot_bytes(len.back());
      }
    const int nw = (int)tid.size();
    if (nw > 0) {
      if (cudaSetDevice(c->device) != cudaSuccess) return report_error(KSW2G_E_CUDA, "align_chains: bad device");
      DevBuf darena, dmeta;
      darena.st = dmeta.st = c->st;
      const size_t mb = (size_t)nw * (8 + 8 + 4 + 4 + 4);
      if ((rc = darena.ensure((size_t)arena + 64)) || (rc = dmeta.ensure(mb))) return rc;
      std::vector<uint8_t> hm(mb);
      memcpy(hm.data(), st.data(), 8 * (size_t)nw);
      memcpy(hm.data() + 8 * (size_t)nw, dst.data(), 8 * (size_t)nw);
      memcpy(hm.data() + 16 * (size_t)nw, tid.data(), 4 * (size_t)nw);
      memcpy(hm.data() + 20 * (size_t)nw, len.data(), 4 * (size_t)nw);
      memcpy(hm.data() + 24 * (size_t)nw, fl.data(), 4 * (size_t)nw);
      std::vector<uint8_t> harena((size_t)arena + 64);
      uint8_t *dm = dmeta.as<uint8_t>();
      if (cudaMemcpyAsync(dm, hm.data(), mb, cudaMemcpyHostToDevice, c->st) != cudaSuccess ||
          launch_ref_gather(nw, (const int32_t *)(dm + 16 * (size_t)nw), (const int64_t *)dm,
                            (const int32_t *)(dm + 20 * (size_t)nw), (const int32_t *)(dm + 24 * (size_t)nw),
                            (const int64_t *)(dm + 8 * (size_t)nw), darena.as<uint8_t>(), ref, c->st) != cudaSuccess ||
          cudaMemcpyAsync(harena.data(), darena.p, (size_t)arena + 64, cudaMemcpyDeviceToHost, c->st) != cudaSuccess ||
          cudaStreamSynchronize(c->st) != cudaSuccess)
        return report_error(KSW2G_E_CUDA, "align_chains: window gather failed");
      darena.release(), dmeta.release();
      std::vector<int> wk(n, -1);  // window of each chain
      for (int ci = 0, k = 0; ci < n; ++ci)
        if (W[ci].te0 > W[ci].ts0 && chains[ci].cnt > 0) wk[ci] = k++;
      parallel_for(n, 1024, [&](int64_t lo, int64_t hi) {
        for (int64_t ci = lo; ci < hi; ++ci)
          if (wk[ci] >= 0) memcpy(tbuf.data() + W[ci].win_off, harena.data() + dst[wk[ci]], (size_t)len[wk[ci]]);
      });
    }
  }
  t1 = now_ms(), c->ch_ms[1] = t1 - t0, t0 = t1;
  // ---- one mb_align_pair batch per (pass, methylation mode); left extensions run on reversed sequences
  ksw2g_align_opt_t ao{S.a, S.b, S.b_ts, S.b_ambi, S.q, S.e, S.q2, S.e2, S.meth ? 1 : 0, 0, S.max_sw_mat};
  struct Out {
    std::vector<ksw2g_ext_result_t> res;
    std::vector<uint32_t> cig;
  };
  Out pass[2][3];
  auto run_pass = [&](int p) -> int {
    for (int mt = 0; mt < 3; ++mt) {
      // job records and buffer offsets in chain order, then the sequences copied over the threads
      std::vector<ksw2g_job_t> jobs;
      int64_t qn = 0, tn = 0, cap = 0;
      for (int ci = 0; ci < n; ++ci) {
        ChainWork &cw = W[ci];
        if (cw.mt != mt) continue;
        for (Job &j : cw.jobs) {
          if (p == 1 && !(j.kind == 1 && j.zcode != 0)) continue;
          const int32_t ql = j.qe - j.qs, tl = (int32_t)(j.te - j.ts);
          int zd = j.zdrop, fl = j.flag;
          if (p == 1) zd = j.zcode == 2 ? cw.o->zdrop_inv : cw.o->zdrop, fl = 0;  // exact maximum (align.c:693)
          (p == 0 ? j.pass1 : j.pass2) = (int)jobs.size();
          jobs.push_back(ksw2g_job_t{qn, tn, ql, tl, j.w, zd, j.end_bonus, fl});
          qn += ql, tn += tl, cap += ql + tl + 1;
        }
      }
      c->ch_n[1 + p] += (int64_t)jobs.size();
      Out &out = pass[p][mt];
      out.res.assign(jobs.size(), ksw2g_ext_result_t{});
      out.cig.assign((size_t)cap + 16, 0);
      if (jobs.empty()) continue;
      std::unique_ptr<uint8_t[]> qb(new uint8_t[qn + 1]), tb(new uint8_t[tn + 1]);
      parallel_for(n, 512, [&](int64_t lo, int64_t hi) {
        for (int64_t ci = lo; ci < hi; ++ci) {
          const ChainWork &cw = W[ci];
          if (cw.mt != mt) continue;
          const uint8_t *q = qbuf + chains[ci].qoff, *t = tbuf.data() + cw.win_off;
          for (const Job &j : cw.jobs) {
            const int idx = p == 0 ? j.pass1 : j.pass2;
            if (idx < 0) continue;
            const ksw2g_job_t &J = jobs[idx];
            const uint8_t *qsrc = q + j.qs, *tsrc = t + (j.ts - cw.ts0);
            uint8_t *qd = qb.get() + J.qoff, *td = tb.get() + J.toff;
            if (j.kind == 0) {  // mb_seq_rev of both (align.c:650-652)
              for (int32_t x = 0; x < J.qlen; ++x) qd[x] = qsrc[J.qlen - 1 - x];
              for (int32_t x = 0; x < J.tlen; ++x) td[x] = tsrc[J.tlen - 1 - x];
            } else {
              memcpy(qd, qsrc, (size_t)J.qlen), memcpy(td, tsrc, (size_t)J.tlen);
            }
          }
        }
      });
      int8_t mat[25];
      gen_mat(mat, S.a, S.b, S.b_ts, S.b_ambi, mt);
      int64_t used = 0;
      const int r = ksw2g_align_pairs(c, &ao, mat, (int)jobs.size(), jobs.data(), qb.get(), qn + 1, tb.get(), tn + 1,
                                      out.res.data(), out.cig.data(), (int64_t)out.cig.size(), &used);
      if (r) return r;
    }
    return 0;
  };
  for (ChainWork &cw : W)
    for (Job &j : cw.jobs) j.pass1 = j.pass2 = -1, j.zcode = 0;
  if ((rc = run_pass(0))) return rc;
  t1 = now_ms(), c->ch_ms[2] = t1 - t0, t0 = t1;
  // ---- mm_test_zdrop on the first pass of every gap fill; the inversion checks as one ksw_ll batch per mode
  {
    struct Inv {
      int ci, ji;
      int32_t tlen;
      int64_t toff_t;  // offset of the target piece in tbuf
      std::vector<uint8_t> q;
    };
    std::vector<std::vector<Inv>> invc(n);  // per chain, then gathered in chain order
    parallel_for(n, 512, [&](int64_t lo, int64_t hi) {
     for (int64_t ci = lo; ci < hi; ++ci) {
      ChainWork &cw = W[ci];
      if (cw.jobs.empty()) continue;
      const ksw2g_chain_opt_t &o = *cw.o;
      int8_t mat[25];
      gen_mat(mat, S.a, S.b, S.b_ts, S.b_ambi, cw.mt);
      for (size_t ji = 0; ji < cw.jobs.size(); ++ji) {
        Job &j = cw.jobs[ji];
        if (j.kind != 1) continue;
        const ksw2g_ext_result_t &E = pass[0][cw.mt].res[j.pass1];
        const uint8_t *qs = qbuf + chains[ci].qoff + j.qs, *ts = tbuf.data() + cw.win_off + (j.ts - cw.ts0);
        int pos[2][2];
        const int32_t mz = cigar_zdrop(S, qs, ts, pass[0][cw.mt].cig.data() + (E.n_cigar > 0 ? E.cigar_off : 0),
                                       E.n_cigar > 0 ? E.n_cigar : 0, mat, pos);
        j.zcode = mz > o.zdrop ? 1 : 0;
        const int q_len = pos[1][1] - pos[1][0], t_len = pos[0][1] - pos[0][0];
        if (!cw.is_sr && mz > o.zdrop_inv && q_len < o.max_gap && t_len < o.max_gap) {
          Inv v{(int)ci, (int)ji, t_len, cw.win_off + (j.ts - cw.ts0) + pos[0][0], {}};
          v.q.resize((size_t)std::max(q_len, 0));
          for (int x = 0; x < q_len; ++x) {  // reverse complement of the dropped query stretch (align.c:55-58)
            const int b = qs[pos[1][1] - x - 1];
            v.q[x] = (uint8_t)(b >= 4 ? 4 : 3 - b);
          }
          invc[ci].push_back(std::move(v));
        }
      }
     }
    });
    std::vector<Inv> inv[3];
    for (int ci = 0; ci < n; ++ci)
      for (Inv &v : invc[ci]) inv[W[ci].mt].push_back(std::move(v));
    for (int mt = 0; mt < 3; ++mt) {
      if (inv[mt].empty()) continue;
      int8_t mat[25];
      gen_mat(mat, S.a, S.b, S.b_ts, S.b_ambi, mt);
      std::vector<ksw2g_ll_job_t> lj;
      std::vector<uint8_t> qb, tb;
      for (const Inv &v : inv[mt]) {
        lj.push_back(ksw2g_ll_job_t{(int64_t)qb.size(), (int64_t)tb.size(), (int32_t)v.q.size(), v.tlen, 0, 0});
        qb.insert(qb.end(), v.q.begin(), v.q.end());
        tb.insert(tb.end(), tbuf.data() + v.toff_t, tbuf.data() + v.toff_t + std::max(v.tlen, 0));
      }
      std::vector<ksw2g_ll_result_t> lr(lj.size());
      c->ch_n[3] += (int64_t)lj.size();
      if (qb.empty()) qb.push_back(0);
      if (tb.empty()) tb.push_back(0);
      if ((rc = ksw2g_ll_batch(c, 2, 5, mat, S.q, S.e, (int)lj.size(), lj.data(), qb.data(), (int64_t)qb.size(),
                               tb.data(), (int64_t)tb.size(), lr.data())))
        return rc;
      for (size_t k = 0; k < lj.size(); ++k) {  // ksw_ll_i16's score (align.c:63-65)
        const int32_t s = lr[k].score;
        const ksw2g_chain_opt_t &o = *W[inv[mt][k].ci].o;
        if (s >= o.min_chain_score * o.a && s >= o.min_dp_max * o.a) W[inv[mt][k].ci].jobs[inv[mt][k].ji].zcode = 2;
      }
    }
  }
  t1 = now_ms(), c->ch_ms[3] = t1 - t0, t0 = t1;
  if ((rc = run_pass(1))) return rc;
  t1 = now_ms(), c->ch_ms[4] = t1 - t0, t0 = t1;
  // ---- assemble every chain in order (align.c:647-757), chains over the threads
  std::vector<std::vector<uint32_t>> cgs(n);
  parallel_for(n, 512, [&](int64_t lo, int64_t hi) {
   for (int64_t ci = lo; ci < hi; ++ci) {
    const ksw2g_chain_t &h = chains[ci];
    ChainWork &cw = W[ci];
    ksw2g_chain_result_t &R = res[ci];
    if (h.cnt <= 0) continue;
    const ksw2g_chain_opt_t &o = *cw.o;
    std::vector<uint32_t> &cg = cgs[ci];
    int32_t dp_score = 0;
    int n_dp = 0;
    size_t ji = 0;
    const ksw2g_anchor_t *a = cw.a.data();
    auto result = [&](const Job &j, const uint32_t *&cig) -> const ksw2g_ext_result_t & {
      const Out &out = j.pass2 >= 0 ? pass[1][cw.mt] : pass[0][cw.mt];
      const ksw2g_ext_result_t &E = out.res[j.pass2 >= 0 ? j.pass2 : j.pass1];
      cig = out.cig.data() + (E.n_cigar > 0 ? E.cigar_off : 0);
      n_dp += j.pass2 >= 0 ? 2 : 1;
      return E;
    };
    int64_t ts1 = cw.ts_first, te1;
    int32_t qs1 = cw.qs_first, qe1;
    if (ji < cw.jobs.size() && cw.jobs[ji].kind == 0) {
      const Job &j = cw.jobs[ji++];
      const uint32_t *cig;
      const ksw2g_ext_result_t &E = result(j, cig);
      if (E.n_cigar > 0) append_cigar(cg, cig, E.n_cigar), dp_score += E.reach_end ? E.mqe : E.max;
      ts1 = j.te - (E.reach_end ? E.mqe_t + 1 : E.max_t + 1);
      qs1 = j.qe - (E.reach_end ? j.qe - j.qs : E.max_q + 1);
    }
    {
      const uint32_t m = (uint32_t)(cw.te_first - cw.ts_first) << 4 | kOpM;
      append_cigar(cg, &m, 1);
      dp_score += o.a * (int32_t)(cw.te_first - cw.ts_first);
    }
    te1 = cw.te_last, qe1 = cw.qe_last;
    bool dropped = false;
    for (; ji < cw.jobs.size() && cw.jobs[ji].kind == 1; ++ji) {
      const Job &j = cw.jobs[ji];
      const uint32_t *cig;
      const ksw2g_ext_result_t &E = result(j, cig);
      if (E.n_cigar > 0) append_cigar(cg, cig, E.n_cigar);
      if (E.zdropped) {  // align.c:698-720: the walk ends here; the jobs behind are discarded
        int k;
        for (k = j.anchor - 1; k >= 0; --k)
          if (a[cw.as1 + k].tpos <= j.ts + E.max_t) break;
        if (k < 0) k = 0;
        dropped = true;
        dp_score += E.max;
        te1 = j.ts + (E.max_t + 1);
        qe1 = j.qs + (E.max_q + 1);
        const int32_t mlen = cal_mlen(cw.cnt1 - (k + 1), a + cw.as1 + k + 1);
        const int split_n = cw.as1 + k + 1;  // mb_split_hit's n, relative to the hit's first anchor
        if (mlen >= o.min_chain_score && split_n > 0 && split_n < h.cnt) {
          const int cnt2 = h.cnt - split_n;  // mb_split_hit (map-algo.c:247-265)
          const int32_t score2 = (int32_t)(h.score * ((float)cnt2 / h.cnt) + .499);
          R.split_n = split_n, R.cnt = h.cnt - cnt2, R.score = h.score - score2;
          R.split_inv2 = j.zcode == 2 ? 1 : 0;
        }
        ++ji;
        break;
      }
      dp_score += E.score;
      if (j.d1 > 0) {
        const uint32_t m = (uint32_t)j.d1 << 4 | kOpM;
        append_cigar(cg, &m, 1);
        dp_score += o.a * (int32_t)j.d1;
      }
    }
    while (ji < cw.jobs.size() && cw.jobs[ji].kind == 1) ++ji;  // gap fills behind a z-drop: discarded
    if (!dropped && ji < cw.jobs.size() && cw.jobs[ji].kind == 2) {
      const Job &j = cw.jobs[ji];
      const uint32_t *cig;
      const ksw2g_ext_result_t &E = result(j, cig);
      if (E.n_cigar > 0) append_cigar(cg, cig, E.n_cigar), dp_score += E.reach_end ? E.mqe : E.max;
      te1 = j.ts + (E.reach_end ? E.mqe_t + 1 : E.max_t + 1);
      qe1 = j.qs + (E.reach_end ? j.qe - j.qs : E.max_q + 1);
    }
    R.ts = ts1, R.te = te1;
    if (!cw.rev) R.qs = qs1, R.qe = qe1;
    else R.qs = h.qlen - qe1, R.qe = h.qlen - qs1;
    R.dp_score = dp_score;
    R.n_cigar = (int32_t)cg.size();
    R.n_dp = n_dp;
    R.n_dp_issued = 0;
    for (const Job &j : cw.jobs) R.n_dp_issued += j.pass2 >= 0 ? 2 : 1;
   }
  });
  int64_t used = 0;
  for (int ci = 0; ci < n; ++ci) {
    if (chains[ci].cnt <= 0) continue;
    if (cigar) {
      if (used + (int64_t)cgs[ci].size() > cigar_cap)
        return report_error(KSW2G_E_CAPACITY, "align_chains: CIGAR buffer too small");
      res[ci].cigar_off = used;
    }
    used += (int64_t)cgs[ci].size();
  }
  if (cigar)
    parallel_for(n, 2048, [&](int64_t lo, int64_t hi) {
      for (int64_t ci = lo; ci < hi; ++ci)
        if (res[ci].cigar_off >= 0) memcpy(cigar + res[ci].cigar_off, cgs[ci].data(), cgs[ci].size() * 4);
    });
  if (cigar_used) *cigar_used = used;
  c->ch_ms[5] = now_ms() - t0;
  return 0;
}

extern "C" int ksw2g_align_chains_last_stats(const ksw2g_ctx_t *c, double *ms, int64_t *counts) {
  if (!c) return report_error(KSW2G_E_ARG, "align_chains: null ctx");
  for (int k = 0; k < 6; ++k)
    if (ms) ms[k] = c->ch_ms[k];
  for (int k = 0; k < 4; ++k)
    if (counts) counts[k] = c->ch_n[k];
  return 0;
}
