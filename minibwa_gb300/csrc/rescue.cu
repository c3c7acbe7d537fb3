// rescue.cu -- pe.c's mate rescue on the device: the 7-mer Hough prefilter
// (mb_ungap, pe.c:209-247), the window narrowing and thresholds of
// mb_matesw_core (pe.c:347-353), then ksw_ll and the reverse extension of
// mb_matesw_align (pe.c:249-300) as batches over the resident reference.
//
// The caller computes each candidate window from the insert-size statistics as
// pe.c:336-339 does and passes the read in the orientation pe.c aligns
// (seq[is_rev]) with the window's methylation mode.  Stage 1 decodes the
// windows on the device (plain l2b_getseq: pe.c converts bases only inside
// mb_ungap and through the scoring matrix) and votes the read's 7-mers along
// diagonals, one block per candidate: the query's table of last positions
// (4^7 uint16, the reference's direct table) is built in shared memory in the
// reference's sequential order, so the last occurrence wins as it does there;
// the target's votes are parallel atomic adds into a diagonal histogram in
// shared memory (global memory for windows too long for it).  Stage 2 runs
// ksw_ll on the narrowed windows (u8 or i16 by pe.c:263's rule, matrix scaled by
// a), stage 3 extends the reversed prefixes ending at ksw_ll's end with extz2
// (EXTZ_ONLY | RIGHT | REV_CIGAR, plus GENERIC_SC for methylation modes).
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <vector>

#include "../../include/ksw2.h"
#include "../../include/ksw2_gb300.h"
#include "batch.h"
#include "host_parallel.h"
#include "host_common.h"
#include "launch.h"
#include "ungap.cuh"

using namespace ksw2g;

namespace {

// ksw_gen_nt4_mat (ksw2.h:199-219) with its int8 arguments
void gen_nt4(int8_t *mat, int8_t a, int8_t b, int8_t b_ts, int8_t b_ambi, int mt) {
  const int m = 5;
  a = a < 0 ? -a : a;
  b = b > 0 ? -b : b;
  b_ambi = b_ambi > 0 ? -b_ambi : b_ambi;
  for (int i = 0; i < m - 1; ++i) {
    for (int j = 0; j < m - 1; ++j) mat[i * m + j] = i == j ? a : b;
    mat[i * m + m - 1] = b_ambi;
  }
  for (int j = 0; j < m; ++j) mat[(m - 1) * m + j] = b_ambi;
  if (b_ts != 0 && b_ts != b) {  // compared after b is made negative, as there
    b_ts = b_ts > 0 ? -b_ts : b_ts;
    mat[0 * m + 2] = mat[1 * m + 3] = mat[2 * m + 0] = mat[3 * m + 1] = b_ts;
  }
  if (mt == 1) mat[1 * m + 3] = a;
  else if (mt == 2) mat[2 * m + 0] = a;
}

inline int64_t al16(int64_t x) { return (x + 15) & ~(int64_t)15; }

// mb_seq_rev of the read prefixes ksw_ll ends at (pe.c:283), from the reads the prefilter
// uploaded: one block per prefix
__global__ void rev_prefix_kernel(int n, const uint8_t *__restrict__ src, const int64_t *__restrict__ soff,
                                  const int32_t *__restrict__ len, uint8_t *__restrict__ dst,
                                  const int64_t *__restrict__ doff) {
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const uint8_t *s = src + soff[i];
    uint8_t *d = dst + doff[i];
    const int L = len[i];
    for (int p = threadIdx.x; p < L; p += blockDim.x) d[p] = s[L - 1 - p];
  }
}

double ms_since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

extern "C" int ksw2g_rescue_batch(ksw2g_ctx_t *c, const ksw2g_ref_t *ref, const ksw2g_rescue_opt_t *opt, int n,
                                  const ksw2g_rescue_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
                                  ksw2g_rescue_result_t *res, uint32_t *cigar, int64_t cigar_cap,
                                  int64_t *cigar_used) {
  if (!c || !ref || !opt || n < 0 || qbuf_len < 0 || (n > 0 && (!jobs || !res || !qbuf)))
    return report_error(KSW2G_E_ARG, "rescue: bad arguments");
  if (opt->a <= 0) return report_error(KSW2G_E_ARG, "rescue: the match score must be positive");
  if (cigar_used) *cigar_used = 0;
  c->rs_launches = 0, c->rs_ms[0] = c->rs_ms[1] = c->rs_ms[2] = 0, c->rs_dev_ms[0] = c->rs_dev_ms[1] = 0;
  if (n == 0) return 0;
  if (cudaSetDevice(c->device) != cudaSuccess) return report_error(KSW2G_E_CUDA, "rescue: bad device");
  const ksw2g_rescue_opt_t &o = *opt;
  auto t0 = std::chrono::steady_clock::now();
  int rc;
  for (int i = 0; i < n; ++i) {
    const ksw2g_rescue_job_t &J = jobs[i];
    if (J.qlen < 0 || J.qoff < 0 || J.qoff + J.qlen > qbuf_len || J.te < J.ts || J.te - J.ts > INT32_MAX / 2 ||
        J.meth < 0 || J.meth > 2)
      return report_error(KSW2G_E_ARG, "rescue: candidate out of bounds");
    if ((rc = ref_check_window(ref, J.tid, J.ts, J.te - J.ts))) return rc;
  }
  // ---- stage 1: the windows decoded on the device, then mb_ungap's votes
  // device records: st int64[n] | dst int64[n] | tid, len, flags int32[n] | UngapJob[n] | counter
  const int64_t o_dst = 8 * (int64_t)n, o_tid = 16 * (int64_t)n, o_len = 20 * (int64_t)n, o_fl = 24 * (int64_t)n;
  const int64_t o_uj = al16(28 * (int64_t)n), o_cnt = o_uj + (int64_t)sizeof(UngapJob) * n, meta = o_cnt + 16;
  const int64_t o_ur = al16(meta);
  if ((rc = c->rs_h.ensure((size_t)(o_ur + (int64_t)sizeof(UngapRes) * n)))) return rc;
  uint8_t *hm = (uint8_t *)c->rs_h.p;
  int64_t tarena = 0;
  int tmax = 1;
  for (int i = 0; i < n; ++i) {
    const ksw2g_rescue_job_t &J = jobs[i];
    const int len = (int)(J.te - J.ts);
    ((int64_t *)hm)[i] = J.ts;
    ((int64_t *)(hm + o_dst))[i] = tarena + 32;
    ((int32_t *)(hm + o_tid))[i] = J.tid;
    ((int32_t *)(hm + o_len))[i] = len;
    ((int32_t *)(hm + o_fl))[i] = 0;
    ((UngapJob *)(hm + o_uj))[i] = UngapJob{J.qoff, tarena + 32, J.qlen, len, J.meth, 0};
    tarena += slot_bytes(len);
    tmax = std::max(tmax, len);
  }
  memset(hm + o_cnt, 0, 16);
  if (!c->nsm) c->nsm = num_sms(c->device);
  const int blocks = std::min(n, c->nsm * 8);
  const bool shared_hist = kUngapTable + (size_t)tmax * 4 <= kUngapSmemMax;
  const size_t smem = shared_hist ? kUngapTable + (size_t)tmax * 4 : kUngapTable;
  if ((rc = c->rs_q.ensure((size_t)qbuf_len + 16)) || (rc = c->rs_t.ensure((size_t)tarena + 64)) ||
      (rc = c->rs_meta.ensure((size_t)meta)) || (rc = c->rs_res.ensure(sizeof(UngapRes) * (size_t)n)) ||
      (!shared_hist && (rc = c->rs_hist.ensure((size_t)blocks * tmax * 4))))
    return rc;
  cudaStream_t st = c->st;
  uint8_t *dm = c->rs_meta.as<uint8_t>();
  if ((qbuf_len && cudaMemcpyAsync(c->rs_q.p, qbuf, (size_t)qbuf_len, cudaMemcpyHostToDevice, st) != cudaSuccess) ||
      cudaMemcpyAsync(dm, hm, (size_t)meta, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "rescue: upload failed");
  if (launch_ref_gather(n, (const int32_t *)(dm + o_tid), (const int64_t *)dm, (const int32_t *)(dm + o_len),
                        (const int32_t *)(dm + o_fl), (const int64_t *)(dm + o_dst), c->rs_t.as<uint8_t>(), ref,
                        st) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "rescue: window gather failed");
  if (smem > 48 * 1024 && raise_smem_cap((const void *)ungap_kernel, smem) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "rescue: shared memory attribute");
  ungap_kernel<<<blocks, kUngapThreads, smem, st>>>(
      n, (const UngapJob *)(dm + o_uj), c->rs_q.as<uint8_t>(), c->rs_t.as<uint8_t>(), c->rs_res.as<UngapRes>(),
      (int *)(dm + o_cnt), shared_hist ? nullptr : c->rs_hist.as<int32_t>(), shared_hist ? 0 : (int64_t)tmax);
  const UngapRes *ur = (const UngapRes *)(hm + o_ur);
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync((void *)ur, c->rs_res.p, sizeof(UngapRes) * (size_t)n, cudaMemcpyDeviceToHost, st) !=
          cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "rescue: prefilter failed");
  c->rs_launches += 2;
  c->rs_ms[0] = ms_since(t0);
  t0 = std::chrono::steady_clock::now();

  // ---- stage 2: narrowing and thresholds (pe.c:347-353), then ksw_ll per (size, methylation) group
  const int b_mm = (o.b + o.a - 1) / o.a, b_ts = (o.b_ts + o.a - 1) / o.a, b_ambi = (o.b_ambi + o.a - 1) / o.a;
  const int gapo = (o.q + o.a - 1) / o.a, gape = (o.e + o.a - 1) / o.a;
  std::vector<int> ll_size(n, 0);
  for (int i = 0; i < n; ++i) {
    const ksw2g_rescue_job_t &J = jobs[i];
    ksw2g_rescue_result_t &R = res[i];
    memset(&R, 0, sizeof R);
    R.ext.cigar_off = -1;
    R.max_ug = ur[i].max, R.max_i = ur[i].max_i, R.n_good = ur[i].n_good, R.n_kmer = ur[i].n_kmer;
    int64_t ts2 = J.ts, te2 = J.te;
    if (R.max_ug >= 10 && R.max_ug >= J.qlen >> 1 && R.n_good == 1) {
      ts2 = J.ts + R.max_i - J.qlen / 2;
      te2 = ts2 + (int64_t)J.qlen * 2;
      if (ts2 < J.ts) ts2 = J.ts;
      if (te2 > J.te) te2 = J.te;
    }
    R.ts2 = ts2, R.te2 = te2;
    if (!(R.max_ug >= 10 || R.max_ug >= R.n_kmer * 0.33)) continue;
    const int64_t tl2 = te2 - ts2, max_sc = J.qlen < tl2 ? J.qlen : tl2;
    if (max_sc >= 32767) continue;  // mb_matesw_align returns before ksw_ll
    ll_size[i] = max_sc < 255 - b_mm ? 1 : 2;
  }
  // one batch per (size, methylation mode); all are prepared, then run on the context's two
  // streams at once, the largest alone on the first, so the few i16 jobs overlap the u8 ones
  struct LLGroup {
    int slot, size;
    std::vector<int> idx;
  };
  std::vector<LLGroup> groups;
  for (int size = 1; size <= 2; ++size)
    for (int mt = 0; mt <= 2; ++mt) {
      LLGroup g{(size - 1) * 3 + mt, size, {}};
      for (int i = 0; i < n; ++i)
        if (ll_size[i] == size && jobs[i].meth == mt) g.idx.push_back(i);
      if (g.idx.empty()) continue;
      int8_t mat[25];
      gen_nt4(mat, 1, (int8_t)b_mm, (int8_t)b_ts, (int8_t)b_ambi, mt);
      std::vector<ksw2g_ll_job_t> lj(g.idx.size());
      std::vector<int32_t> tids(g.idx.size());
      for (size_t k = 0; k < g.idx.size(); ++k) {
        const int i = g.idx[k];
        lj[k] = ksw2g_ll_job_t{jobs[i].qoff, res[i].ts2, jobs[i].qlen, (int32_t)(res[i].te2 - res[i].ts2),
                               KSW_LL_SUBO | o.min_len, 0};
        tids[k] = jobs[i].tid;
      }
      if (!c->rs_ll[g.slot]) c->rs_ll[g.slot] = new ksw2g_batch;
      // the reads the prefilter uploaded stay on the device
      const SeqSeg seg{lj.data(), (int)lj.size(), qbuf, qbuf_len, nullptr, 0, c->rs_q.as<uint8_t>()};
      const RefTargets rt{ref, tids.data(), nullptr};
      if ((rc = ll_prepare_segs(c, c->rs_ll[g.slot], size, 5, mat, gapo, gape, 1, &seg, &rt))) return rc;
      groups.push_back(std::move(g));
    }
  if (groups.size() > 1 && !c->aux && cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "rescue: stream creation failed");
  std::sort(groups.begin(), groups.end(), [](const LLGroup &x, const LLGroup &y) { return x.idx.size() > y.idx.size(); });
  for (size_t gi = 0; gi < groups.size(); ++gi) {
    ksw2g_batch *b = c->rs_ll[groups[gi].slot];
    ksw2g_batch_set_timing(b, 1);
    if ((rc = ll_run_on(b, gi == 0 ? c->st : c->aux))) return rc;
    c->rs_launches += 2 + b->launches;  // query packing and window gather, then the DP
  }
  if (groups.size() > 1 && cudaStreamSynchronize(c->aux) != cudaSuccess)
    return report_error(KSW2G_E_CUDA, "rescue: ksw_ll failed");
  for (const LLGroup &g : groups) {
    std::vector<ksw2g_ll_result_t> lr(g.idx.size());
    if ((rc = ksw2g_ll_fetch(c, c->rs_ll[g.slot], lr.data()))) return rc;
    double dp = 0, bt = 0;
    if (ksw2g_batch_kernel_ms(c->rs_ll[g.slot], &dp, &bt, nullptr, nullptr) == 0) c->rs_dev_ms[0] += dp + bt;
    for (size_t k = 0; k < g.idx.size(); ++k) {
      ksw2g_rescue_result_t &R = res[g.idx[k]];
      R.ll_done = 1, R.ll_score = lr[k].score, R.ll_te = lr[k].te, R.ll_qe = lr[k].qe;
      R.ll_score2 = lr[k].score2, R.ll_te2 = lr[k].te2;
    }
  }
  c->rs_ms[1] = ms_since(t0);
  t0 = std::chrono::steady_clock::now();
  // ---- stage 3: extz2 on the reversed prefixes ending at ksw_ll's end (pe.c:283-300)
  int64_t used = 0;
  std::vector<int> by_mt[3];  // the candidates that go on to extz2, per methylation mode
  for (int i = 0; i < n; ++i) {
    const ksw2g_rescue_result_t &R = res[i];
    if (R.ll_done && jobs[i].meth >= 0 && jobs[i].meth <= 2 && R.ll_score >= o.min_dp_max &&
        R.ll_score >= jobs[i].min_sc)
      by_mt[jobs[i].meth].push_back(i);
  }
  for (int mt = 0; mt <= 2; ++mt) {
    const std::vector<int> &idx = by_mt[mt];
    if (idx.empty()) continue;
    int8_t mat[25];
    gen_nt4(mat, (int8_t)o.a, (int8_t)o.b, (int8_t)o.b_ts, (int8_t)o.b_ambi, mt);
    const int flag = KSW_EZ_EXTZ_ONLY | KSW_EZ_RIGHT | KSW_EZ_REV_CIGAR | (mt ? KSW_EZ_GENERIC_SC : 0);
    std::vector<ksw2g_job_t> ej(idx.size());
    std::vector<int32_t> tids(idx.size()), tfl(idx.size(), KSW2G_REF_REVERSE);
    // the reversed prefixes are cut from the device copy of the reads (no host byte touched)
    const int m = (int)idx.size();
    const size_t o_len = (size_t)8 * m, o_dof = (o_len + (size_t)4 * m + 7) & ~(size_t)7, rm = o_dof + (size_t)8 * m;
    std::vector<uint8_t> hr(rm);
    int64_t *hso = (int64_t *)hr.data(), *hdo = (int64_t *)(hr.data() + o_dof);
    int32_t *hln = (int32_t *)(hr.data() + o_len);
    int64_t qo = 0;
    for (int k = 0; k < m; ++k) {
      const int i = idx[k];
      const int qe = res[i].ll_qe + 1, te = res[i].ll_te + 1;
      hso[k] = jobs[i].qoff, hln[k] = qe, hdo[k] = qo;
      ej[k] = ksw2g_job_t{qo, res[i].ts2, qe, te, o.bw, o.zdrop, o.end_bonus, flag};
      tids[k] = jobs[i].tid;
      qo += qe;
    }
    const int64_t rq_len = qo;
    if ((rc = c->rs_rq.ensure((size_t)std::max<int64_t>(rq_len, 1) + 16)) || (rc = c->rs_rmeta.ensure(rm))) return rc;
    uint8_t *drm = c->rs_rmeta.as<uint8_t>();
    if (cudaMemcpyAsync(drm, hr.data(), rm, cudaMemcpyHostToDevice, st) != cudaSuccess)
      return report_error(KSW2G_E_CUDA, "rescue: prefix records upload failed");
    rev_prefix_kernel<<<std::min(m, c->nsm * 16), 64, 0, st>>>(m, c->rs_q.as<uint8_t>(), (const int64_t *)drm,
                                                               (const int32_t *)(drm + o_len), c->rs_rq.as<uint8_t>(),
                                                               (const int64_t *)(drm + o_dof));
    if (cudaGetLastError() != cudaSuccess) return report_error(KSW2G_E_CUDA, "rescue: prefix kernel failed");
    std::vector<ksw2g_ext_result_t> er(idx.size());
    int64_t u = 0;
    if (!c->rs_ext[mt]) c->rs_ext[mt] = new ksw2g_batch;
    ksw2g_batch *eb = c->rs_ext[mt];
    const SeqSeg seg{ej.data(), m, qbuf, rq_len, nullptr, 0, c->rs_rq.as<uint8_t>()};
    const RefTargets rt{ref, tids.data(), tfl.data()};
    // CIGARs go straight into the caller's buffer behind those of earlier groups
    if ((rc = ext_prepare_segs(c, eb, 0, 5, mat, (int8_t)o.q, (int8_t)o.e, (int8_t)o.q, (int8_t)o.e, 1, &seg, &rt)) ||
        (rc = ksw2g_batch_set_timing(eb, 1)) || (rc = ksw2g_batch_run(c, eb)) ||
        (rc = ksw2g_ext_fetch(c, eb, er.data(), cigar ? cigar + used : nullptr, cigar ? cigar_cap - used : 0, &u)))
      return rc;
    c->rs_launches += 2 + eb->launches;  // prefix records and kernel, then packing, gather and the DP
    {
      double dp = 0, bt = 0;
      if (ksw2g_batch_kernel_ms(eb, &dp, &bt, nullptr, nullptr) == 0) c->rs_dev_ms[1] += dp + bt;
    }

    parallel_for((int64_t)idx.size(), 16384, [&](int64_t lo, int64_t hi) {
    for (int64_t k = lo; k < hi; ++k) {
      const int i = idx[k];
      ksw2g_rescue_result_t &R = res[i];
      const ksw2g_ext_result_t &E = er[k];
      R.ext_done = 1;
      R.ext = E;
      R.ext.cigar_off = E.n_cigar > 0 && cigar ? E.cigar_off + used : -1;
      if (E.n_cigar > 0 && E.max >= o.min_dp_max * o.a) {  // the hit of pe.c:291-304 and 361-368
        const int qe = ej[k].qlen, te = ej[k].tlen;
        int qs = qe - (E.reach_end ? qe : E.max_q + 1), qe2 = qe;
        R.rescued = 1;
        R.ts = res[i].ts2 + te - (E.reach_end ? E.mqe_t + 1 : E.max_t + 1);
        R.te = res[i].ts2 + te;
        const int32_t d2 = (int32_t)((double)E.max / R.ll_score * R.ll_score2 + .499);
        R.dp_max2 = d2 < 0 ? 0 : d2;
        if (jobs[i].rev) {
          const int t = qs;
          qs = jobs[i].qlen - qe2, qe2 = jobs[i].qlen - t;
        }
        R.qs = qs, R.qe = qe2;
      }
    }
    });
    if (cigar) used += u;
  }
  if (cigar_used) *cigar_used = used;
  c->rs_ms[2] = ms_since(t0);
  return 0;
}

extern "C" int ksw2g_rescue_last_device_ms(const ksw2g_ctx_t *c, double *ms) {
  if (!c || !ms) return report_error(KSW2G_E_ARG, "rescue: null argument");
  ms[0] = c->rs_dev_ms[0], ms[1] = c->rs_dev_ms[1];
  return 0;
}

extern "C" int ksw2g_rescue_last_stats(const ksw2g_ctx_t *c, int *launches, double *ms) {
  if (!c) return report_error(KSW2G_E_ARG, "rescue: null ctx");
  if (launches) *launches = c->rs_launches;
  if (ms) ms[0] = c->rs_ms[0], ms[1] = c->rs_ms[1], ms[2] = c->rs_ms[2];
  return 0;
}
