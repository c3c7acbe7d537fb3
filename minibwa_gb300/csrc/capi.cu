// capi.cu -- C ABI of libksw2gpu.so: contexts, batches, and the per-call
// drop-in replacements of the reference's ksw2 entry points.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ksw2.h"
#include "../../include/ksw2_gb300.h"
#include "ksw2g.h"
#include "launch.h"
#include "host_common.h"
#include "batch.h"
#include "host_parallel.h"

static_assert(sizeof(ksw2g_job_t) == sizeof(ksw2g_job), "job layout");
static_assert(sizeof(ksw2g_ext_result_t) == sizeof(ksw2g_ext_result), "result layout");
static_assert(sizeof(ksw2g_ll_job_t) == sizeof(ksw2g_ll_job), "ll job layout");
static_assert(sizeof(ksw2g_ll_result_t) == sizeof(ksw2g_ll_result), "ll result layout");

namespace ksw2g {
cudaError_t launch_ext_dp_z2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                             cudaStream_t st);
cudaError_t launch_ext_dp_d2(int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L, int max_blocks,
                             cudaStream_t st);
cudaError_t launch_ext_dp(int dual, int mode, int shape, const ksw2g_ext_params &P, const ExtLaunch &L,
                          int max_blocks, cudaStream_t st) {
  if (shape == kWideShape) return launch_ext_wide(P, L, st);
  if (shape >= kSplitBase)
    return dual ? launch_ext_split_d2(mode, shape - kSplitBase, P, L, max_blocks, st)
                : launch_ext_split_z2(mode, shape - kSplitBase, P, L, max_blocks, st);
  if (shape >= kExt16Base)
    return dual ? launch_ext16_dp_d2(mode, shape - kExt16Base, P, L, max_blocks, st)
                : launch_ext16_dp_z2(mode, shape - kExt16Base, P, L, max_blocks, st);
  return dual ? launch_ext_dp_d2(mode, shape, P, L, max_blocks, st)
              : launch_ext_dp_z2(mode, shape, P, L, max_blocks, st);
}

static const int64_t kWaveTarget = (int64_t)1 << 30;  // traceback bytes per wave of short pairs
static const double kLongCells = 200000.0;             // mean band cells above which pairs count as long

// shape preference per (dual, mode, n_col): shape code + 1 (codes from kNumExtShapes on are
// the 16-bit-lane kernels); 0 = the smallest byte-lane shape that holds the band
static const int kMaxPrefCol = 512;
static int g_pref[2][3][kMaxPrefCol + 1];
static std::mutex g_pref_mu;
// lane width forced on every batch: -1 none (preferences decide), 0 bytes, 1 16-bit halves
static std::atomic<int> g_family{-1};
// block-split kernel (ksw2g_ext_set_split): -1 the batch decides, 0 never, 1 wherever a split
// shape holds the band; the environment variable KSW2G_SPLIT sets the initial value
static int split_from_env() {
  const char *v = getenv("KSW2G_SPLIT");
  const int m = v && *v ? atoi(v) : -1;
  return m >= -1 && m <= 1 ? m : -1;
}
static std::atomic<int> g_split{split_from_env()};
// Which jobs a batch runs on the block-split kernel.  Bands wider than every thread-group shape
// always do: one 10 kb extd2 pair at w=1100 takes 1.25 us per anti-diagonal there against 3.75
// on the block-wide kernel (ext_wide.cuh), and 608 such pairs 6.0 against 8.9 us.  The jobs of
// a thread-group (mode, shape) class do when they number at most kSplitMaxJobs and their
// bands span at least kSplitMinCol 16-cell blocks (w above about 250): a group computes a pair's anti-diagonals
// one after another (1.41 us each at w=100 and at w=500, the same with up to 608 such pairs at
// once), so a batch of few long pairs lasts as long as its longest pair on one group, while a
// block takes 0.95 us at w=100 and 1.00 us at w=500.  With more pairs the groups' throughput
// wins (608 pairs at w=500: 1.42 us on groups, 2.25 on blocks).
static const int kSplitMinCol = 17;
static const int kSplitMaxJobs = 304;

static bool use_split(int n_col, int count, bool wide) {
  const int m = g_split.load(std::memory_order_relaxed);
  if (m == 0 || (m < 0 && !wide && (n_col < kSplitMinCol || count > kSplitMaxJobs))) return false;
  return ext_split_for(n_col) >= 0;
}

static bool shape_holds(int s, int n_col) {
  return s >= 0 && s < kNumExtShapes && kExtShapes[s].G * kExtShapes[s].K >= 4 * n_col;
}

int ext_shape_id(int dual, int mode, int n_col, const ksw2g_ext_params &P) {
  const int fit = ext_shape_for(n_col);
  if (fit < 0) return kWideShape;
  int s = fit;
  bool w16 = false;
  if (n_col >= 0 && n_col <= kMaxPrefCol) {
    const int p = g_pref[dual & 1][mode][n_col] - 1;
    if (p >= 0 && shape_holds(p % kNumExtShapes, n_col)) s = p % kNumExtShapes, w16 = p >= kNumExtShapes;
  }
  const int fam = g_family.load(std::memory_order_relaxed);
  if (fam >= 0) w16 = fam == 1;
  return w16 && ext16_params_ok(P) ? kExt16Base + s : s;
}
void ext_shape_set_pref(int dual, int mode, int lo, int hi, int code) {
  std::lock_guard<std::mutex> g(g_pref_mu);
  for (int c = lo < 0 ? 0 : lo; c <= hi && c <= kMaxPrefCol; ++c) g_pref[dual & 1][mode][c] = code + 1;
}
}  // namespace ksw2g

using namespace ksw2g;

// ---------------------------------------------------------------- errors
static thread_local std::string tl_err;
static int set_err(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
static int set_err(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  tl_err = buf;
  return code;
}
#define CK(x)                                                                                          \
  do {                                                                                                 \
    cudaError_t e_ = (x);                                                                              \
    if (e_ != cudaSuccess) return set_err(KSW2G_E_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), \
                                          __FILE__, __LINE__);                                         \
  } while (0)

extern "C" const char *ksw2g_last_error(void) { return tl_err.c_str(); }

namespace ksw2g {
int report_error(int code, const char *msg) { return set_err(code, "%s", msg); }

static std::atomic<int> g_fail_alloc{0};
bool take_injected_alloc_failure() {
  int n = g_fail_alloc.load(std::memory_order_relaxed);
  while (n > 0)
    if (g_fail_alloc.compare_exchange_weak(n, n - 1)) return n == 1;
  return false;
}
}  // namespace ksw2g

extern "C" void ksw2g_debug_fail_device_alloc(int nth) { ksw2g::g_fail_alloc.store(nth > 0 ? nth : 0); }

extern "C" int ksw2g_ctx_create(int device, ksw2g_ctx_t **out) {
  if (!out) return set_err(KSW2G_E_ARG, "null output");
  int ndev = 0;
  CK(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return set_err(KSW2G_E_ARG, "device %d not present (%d devices)", device, ndev);
  CK(cudaSetDevice(device));
  ksw2g_ctx *c = new ksw2g_ctx;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return set_err(KSW2G_E_CUDA, "cudaStreamCreate failed");
  }
  c->nsm = num_sms(device);
  *out = c;
  return 0;
}

extern "C" void ksw2g_batch_free(ksw2g_batch_t *b);

extern "C" void ksw2g_ctx_destroy(ksw2g_ctx_t *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->st);
  if (c->scratch) ksw2g_batch_free(c->scratch);
  for (ksw2g_ctx *sc : c->sub)
    if (sc) ksw2g_ctx_destroy(sc);
  if (c->aux) {
    cudaStreamSynchronize(c->aux);
    cudaStreamDestroy(c->aux);
  }
  c->tb_pool.release();
  c->one.release();
  c->one_h.release();
  for (DevBuf *d : {&c->rs_q, &c->rs_t, &c->rs_meta, &c->rs_res, &c->rs_hist, &c->rs_rq, &c->rs_rmeta}) d->release();
  for (ksw2g_batch *b : c->rs_ll)
    if (b) ksw2g_batch_free(b);
  for (ksw2g_batch *b : c->rs_ext)
    if (b) ksw2g_batch_free(b);
  c->rs_h.release();
  cudaStreamDestroy(c->st);
  delete c;
}
extern "C" void *ksw2g_ctx_stream(ksw2g_ctx_t *c) { return c ? (void *)c->st : nullptr; }
extern "C" int ksw2g_ctx_sync(ksw2g_ctx_t *c) {
  if (!c) return set_err(KSW2G_E_ARG, "null ctx");
  CK(cudaStreamSynchronize(c->st));
  return 0;
}
extern "C" int ksw2g_ctx_set_tb_budget(ksw2g_ctx_t *c, int64_t bytes) {
  if (!c || bytes < (1 << 20)) return set_err(KSW2G_E_ARG, "budget must be >= 1 MiB");
  c->tb_budget = bytes;
  return 0;
}

extern "C" void ksw2g_batch_free(ksw2g_batch_t *b) {
  if (!b) return;
  for (DevBuf *d : {&b->raw, &b->rawmeta, &b->arena, &b->jobs, &b->order, &b->sorted, &b->tb_off, &b->res, &b->bts, &b->cigar,
                    &b->counters, &b->llmat, &b->blist, &b->blist_off, &b->wide})
    d->release();
  batch_release_streams(b);
  delete b;
}
extern "C" int ksw2g_batch_launches(const ksw2g_batch_t *b) { return b ? b->launches : 0; }

extern "C" int ksw2g_batch_set_timing(ksw2g_batch_t *b, int on) {
  if (!b) return set_err(KSW2G_E_ARG, "null batch");
  b->timing = on != 0;
  b->n_timed = 0;
  return 0;
}

extern "C" int ksw2g_batch_kernel_ms(ksw2g_batch_t *b, double *dp_ms, double *bt_ms, int *n_dp, int *n_bt) {
  if (!b) return set_err(KSW2G_E_ARG, "null batch");
  // Launches of a two-stream run overlap: report, per kernel kind, the length of the
  // union of the launches' intervals (the plain sum when they run one after another).
  double t[2] = {0, 0};
  int c[2] = {0, 0};
  std::vector<std::pair<double, double>> iv[2];
  for (int i = 0; i < b->n_timed; ++i) {
    float a = 0, z = 0;
    CK(cudaEventSynchronize(b->tev[2 * i + 1]));
    CK(cudaEventElapsedTime(&a, b->tev[0], b->tev[2 * i]));
    CK(cudaEventElapsedTime(&z, b->tev[0], b->tev[2 * i + 1]));
    iv[b->tkind[i]].push_back({a, z});
    ++c[b->tkind[i]];
  }
  for (int k = 0; k < 2; ++k) {
    std::sort(iv[k].begin(), iv[k].end());
    double end = -1e300;
    for (auto &x : iv[k]) {
      if (x.first > end) t[k] += x.second - x.first, end = x.second;
      else if (x.second > end) t[k] += x.second - end, end = x.second;
    }
  }
  if (dp_ms) *dp_ms = t[0];
  if (bt_ms) *bt_ms = t[1];
  if (n_dp) *n_dp = c[0];
  if (n_bt) *n_bt = c[1];
  return 0;
}

// Upload raw sequences and pack them into the padded arena.  Writes the padded
// offsets of query s and target s to qpad[s], tpad[s].
// qoff/toff index the concatenation of the segments' query / target buffers.
int upload_and_pack(ksw2g_ctx *c, ksw2g_batch *b, int n, const int64_t *qoff, const int32_t *qlen,
                           const int64_t *toff, const int32_t *tlen, int nseg, const SeqSeg *segs,
                           std::vector<int64_t> &qpad, std::vector<int64_t> &tpad, const RefTargets *rt) {
  int64_t qbuf_len = 0, tbuf_len = 0;
  for (int k = 0; k < nseg; ++k) qbuf_len += segs[k].qlen, tbuf_len += rt ? 0 : segs[k].tlen;
  const uint8_t *qdev = nseg == 1 ? segs[0].qdev : nullptr;  // queries already on the device
  const int64_t qraw = qdev ? 0 : qbuf_len;                      // query bytes uploaded into raw
  qpad.resize(n), tpad.resize(n);
  int64_t a = 0;
  for (int i = 0; i < n; ++i) {
    qpad[i] = a + 32, a += slot_bytes(qlen[i]);
    tpad[i] = a + 32, a += slot_bytes(tlen[i]);
  }
  const int64_t arena_bytes = a + 64;
  int rc;
  if ((rc = b->arena.ensure(arena_bytes))) return rc;
  if ((rc = b->raw.ensure(qraw + tbuf_len + 16))) return rc;
  // metadata of the packed sequences (queries, then targets unless they come from the
  // device reference): raw offsets (int64), lengths (int32), arena offsets (int64)
  const int npack = rt ? n : 2 * n;
  const size_t o_ln = (size_t)8 * npack, o_dof = (o_ln + (size_t)4 * npack + 7) & ~(size_t)7;
  const size_t meta = o_dof + (size_t)8 * npack;
  if ((rc = b->rawmeta.ensure(meta))) return rc;
  std::vector<uint8_t> hm(meta);
  int64_t *ro = (int64_t *)hm.data();
  int32_t *ln = (int32_t *)(hm.data() + o_ln);
  int64_t *dof = (int64_t *)(hm.data() + o_dof);
  for (int i = 0; i < n; ++i) {
    ro[i] = qoff[i], ln[i] = qlen[i], dof[i] = qpad[i];
    if (!rt) ro[n + i] = qraw + toff[i], ln[n + i] = tlen[i], dof[n + i] = tpad[i];
  }
  uint8_t *raw = b->raw.as<uint8_t>();
  {
    int64_t qa = 0, ta = qraw;
    for (int k = 0; k < nseg; ++k) {
      if (segs[k].qlen && !qdev) CK(cudaMemcpyAsync(raw + qa, segs[k].qbuf, segs[k].qlen, cudaMemcpyHostToDevice, c->st));
      if (!rt && segs[k].tlen) CK(cudaMemcpyAsync(raw + ta, segs[k].tbuf, segs[k].tlen, cudaMemcpyHostToDevice, c->st));
      qa += segs[k].qlen, ta += rt ? 0 : segs[k].tlen;
    }
  }
  CK(cudaMemcpyAsync(b->rawmeta.p, hm.data(), meta, cudaMemcpyHostToDevice, c->st));
  const int64_t *dro = b->rawmeta.as<int64_t>();
  const int32_t *dln = (const int32_t *)(b->rawmeta.as<uint8_t>() + o_ln);
  const int64_t *ddof = (const int64_t *)(b->rawmeta.as<uint8_t>() + o_dof);
  if (qdev) {  // queries from their device copy, targets (unless from the reference) from raw
    CK(launch_pack(n, qdev, dro, dln, b->arena.as<uint8_t>(), ddof, c->st));
    if (!rt) CK(launch_pack(n, raw, dro + n, dln + n, b->arena.as<uint8_t>(), ddof + n, c->st));
  } else {
    CK(launch_pack(npack, raw, dro, dln, b->arena.as<uint8_t>(), ddof, c->st));
  }
  if (rt) {  // targets: windows of the device reference, decoded into their arena slots
    // layout: start (int64), arena offset (int64), contig (int32), length (int32), flags (int32)
    const size_t rm = (size_t)n * (8 + 8 + 4 + 4 + 4);
    if ((rc = b->refmeta.ensure(rm))) return rc;
    std::vector<uint8_t> h(rm);
    int64_t *hst = (int64_t *)h.data(), *hdst = hst + n;
    int32_t *htid = (int32_t *)(hdst + n), *hlen = htid + n, *hfl = hlen + n;
    for (int i = 0; i < n; ++i)
      hst[i] = toff[i], hdst[i] = tpad[i], htid[i] = rt->tid[i], hlen[i] = tlen[i],
      hfl[i] = rt->flags ? rt->flags[i] : 0;
    CK(cudaMemcpyAsync(b->refmeta.p, h.data(), rm, cudaMemcpyHostToDevice, c->st));
    const int64_t *dst = b->refmeta.as<int64_t>(), *ddst = dst + n;
    const int32_t *dtid = (const int32_t *)(ddst + n), *dlen = dtid + n, *dfl = dlen + n;
    CK(launch_ref_gather(n, dtid, dst, dlen, dfl, ddst, b->arena.as<uint8_t>(), rt->ref, c->st));
  }
  // the H2D source buffers may be reused by the caller after return
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

// Jobs of all segments with offsets rebased onto the concatenated buffers; each
// job must stay inside its own segment's buffers.
template <typename J>
static int flatten_segs(int nseg, const SeqSeg *segs, std::vector<J> &flat, const J *&jobs, int &n,
                        int64_t &qtot, int64_t &ttot) {
  n = 0, qtot = 0, ttot = 0;
  for (int k = 0; k < nseg; ++k) {
    if (segs[k].n < 0 || (segs[k].n > 0 && !segs[k].jobs) || segs[k].qlen < 0 || segs[k].tlen < 0)
      return set_err(KSW2G_E_ARG, "bad batch segment %d", k);
    n += segs[k].n;
  }
  if (nseg == 1) {
    jobs = (const J *)segs[0].jobs, qtot = segs[0].qlen, ttot = segs[0].tlen;
    return 0;
  }
  flat.resize(n);
  int at = 0;
  for (int k = 0; k < nseg; ++k) {
    const J *src = (const J *)segs[k].jobs;
    for (int i = 0; i < segs[k].n; ++i, ++at) {
      J j = src[i];
      if (j.qlen < 0 || j.tlen < 0 || j.qoff < 0 || j.toff < 0 || j.qoff + j.qlen > segs[k].qlen ||
          j.toff + j.tlen > segs[k].tlen)
        return set_err(KSW2G_E_ARG, "segment %d job %d: sequence out of buffer bounds", k, i);
      j.qoff += qtot, j.toff += ttot;
      flat[at] = j;
    }
    qtot += segs[k].qlen, ttot += segs[k].tlen;
  }
  jobs = flat.data();
  return 0;
}

int ext_prepare_into(ksw2g_ctx *c, ksw2g_batch *b, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e,
                     int8_t q2, int8_t e2, int n, const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
                     const uint8_t *tbuf, int64_t tbuf_len) {
  if (n < 0 || (n > 0 && !jobs)) return set_err(KSW2G_E_ARG, "bad batch arguments");
  const SeqSeg seg{jobs, n, qbuf, qbuf_len, tbuf, tbuf_len};
  return ext_prepare_segs(c, b, dual, m, mat, q, e, q2, e2, 1, &seg);
}

// Rough device time of a bin in cycles, to spread the bins of a wave over streams: its
// longest pair's anti-diagonals at one pair's latency plus its anti-diagonal words (diag_words)
// at the whole device's rate.  Measured on a GB300 with one 10 kb extd2 pair: about 2,200 + 140 K
// cycles per anti-diagonal on a group of K words a thread, 1,750 + 85 NW K on a block of NW
// warps, 8,000 on the block-wide kernel; 1,000,000 config-1 pairs run at about 0.02 cycles per
// anti-diagonal word on groups, and blocks take about three times the groups' device time per
// word.
static double bin_cost(int shape, int64_t max_diag, double diag_words) {
  double lat = 8000.0, per_word = 0.06;
  if (shape >= kSplitBase) {
    const SplitShape &b = kSplitShapes[shape - kSplitBase];
    lat = 1750.0 + 85.0 * b.NW * b.K;
  } else if (shape != kWideShape) {
    lat = 2200.0 + 140.0 * kExtShapes[shape >= kExt16Base ? shape - kExt16Base : shape].K, per_word = 0.02;
  }
  return (double)max_diag * lat + per_word * diag_words;
}
// Assign the bins of a wave to its streams, costliest first, each to the stream with the least
// cost so far (the longest-processing-time rule), and order them that way for launching.  The
// block-wide kernel's bins share one stream, because they share the wave's scratch.
// KSW2G_SIDE_STREAMS (0 to kSideStreams) sets how many side streams a wave may use.
static int side_streams() {
  static const int n = [] {
    const char *v = getenv("KSW2G_SIDE_STREAMS");
    const int k = v && *v ? atoi(v) : kSideStreams;
    return k < 0 ? 0 : k > kSideStreams ? kSideStreams : k;
  }();
  return n;
}
static void spread_bins(std::vector<Bin> &bins) {
  std::stable_sort(bins.begin(), bins.end(), [](const Bin &a, const Bin &b) { return a.cost > b.cost; });
  double load[1 + kSideStreams] = {};
  int wide_sub = -1;
  const int ns = side_streams();
  for (Bin &bn : bins) {
    int s = 0;
    if (bn.shape == kWideShape && wide_sub >= 0) s = wide_sub;
    else
      for (int i = 1; i <= ns; ++i)
        if (load[i] < load[s]) s = i;
    if (bn.shape == kWideShape) wide_sub = s;
    load[s] += bn.cost;
    bn.sub = s;
  }
}

int ext_prepare_segs(ksw2g_ctx *c, ksw2g_batch *b, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e,
                     int8_t q2, int8_t e2, int nseg, const SeqSeg *segs, const RefTargets *rt) {
  if (rt && (nseg != 1 || !rt->ref || (segs[0].n > 0 && !rt->tid)))
    return set_err(KSW2G_E_ARG, "reference targets need one segment and a contig id per job");
  std::vector<ksw2g_job_t> flat;
  const ksw2g_job_t *jobs = nullptr;
  int n = 0;
  int64_t qbuf_len = 0, tbuf_len = 0;
  {
    const int rc0 = flatten_segs(nseg, segs, flat, jobs, n, qbuf_len, tbuf_len);
    if (rc0) return rc0;
  }
  if (n < 0 || (n > 0 && !jobs) || !mat) return set_err(KSW2G_E_ARG, "bad batch arguments");
  CK(cudaSetDevice(c->device));
  b->kind = dual ? 1 : 0;
  b->n = n;
  b->launches = 0;
  derive_ext_params(dual, m, mat, q, e, q2, e2, b->P);
  std::vector<int64_t> qo(n), to(n);
  std::vector<int32_t> ql(n), tl(n);
  std::vector<int> shape(n), mode(n), ncol(n);
  std::vector<double> dwords(n);  // anti-diagonals x window words of every job (bin costs)
  std::vector<int64_t> foot(n);
  int64_t cig = 0, wide_max = 0;
  int64_t band_cells = 0;  // sum of (qlen + tlen) x band width: the batch's size class
  int n_wide = 0;
  {
    // One job's checks and plan; returns nonzero at the first failing check, with the error
    // set on the calling thread.
    auto plan = [&](int i, int64_t &cg, int64_t &bc) -> int {
      const ksw2g_job_t &J = jobs[i];
      if (J.qlen < 0 || J.tlen < 0 || J.qoff < 0 || J.toff < 0 || J.qoff + J.qlen > qbuf_len ||
          (!rt && J.toff + J.tlen > tbuf_len))
        return set_err(KSW2G_E_ARG, "job %d: sequence out of buffer bounds", i);
      if (rt && ref_check_window(rt->ref, rt->tid[i], J.toff, J.tlen)) return KSW2G_E_ARG;
      if ((J.flag & KSW_EZ_GENERIC_SC) && m > 16)
        return set_err(KSW2G_E_UNSUPPORTED, "job %d: GENERIC_SC needs m <= 16 on the device (m=%d)", i, m);
      qo[i] = J.qoff, to[i] = J.toff, ql[i] = J.qlen, tl[i] = J.tlen;
      mode[i] = ext_mode(J.flag);
      const bool live = J.qlen > 0 && J.tlen > 0 && !b->P.skip_all;
      const int nc = live ? ext_ncol(J.qlen, J.tlen, J.w) : 1;
      shape[i] = ext_shape_id(dual, mode[i], nc, b->P);
      ncol[i] = nc;
      dwords[i] = (double)std::max(J.qlen + J.tlen - 1, 0) * 4.0 * nc;
      foot[i] = (live && mode[i] != 0) ? (((int64_t)(J.qlen + J.tlen - 1) * nc * 16 + 15) & ~(int64_t)15) : 0;
      if (foot[i] > c->tb_budget)
        return set_err(KSW2G_E_CAPACITY, "job %d: traceback needs %lld bytes, budget %lld", i, (long long)foot[i],
                       (long long)c->tb_budget);
      if (mode[i] != 0) cg += J.qlen + J.tlen + 1;
      bc += (int64_t)(J.qlen + J.tlen) * (nc > 1 ? 16 * (nc - 1) : 0);
      return 0;
    };
    // over threads in ranges; a range stops at its first failing job, and the first failing job
    // of the batch is planned again on this thread, which reports it
    const int64_t grain = 16384;
    const int nr = (int)std::max<int64_t>(1, std::min<int64_t>(host_threads(), (n + grain - 1) / grain));
    std::vector<int64_t> rcg(nr, 0), rbc(nr, 0);
    std::vector<int> rfail(nr, -1);
    parallel_for(nr, 1, [&](int64_t lo, int64_t hi) {
      for (int64_t t = lo; t < hi; ++t)
        for (int i = (int)(n * t / nr), e = (int)(n * (t + 1) / nr); i < e; ++i)
          if (plan(i, rcg[t], rbc[t])) {
            rfail[t] = i;
            break;
          }
    });
    for (int t = 0; t < nr; ++t) {
      if (rfail[t] >= 0) {
        int64_t a = 0, bb = 0;
        return plan(rfail[t], a, bb);
      }
      cig += rcg[t], band_cells += rbc[t];
    }
  }
  {  // jobs of the (mode, shape) classes that hold few of them move to the block-split kernel
    std::vector<int> cnt(3 * kNumShapeIds, 0);
    for (int i = 0; i < n; ++i) ++cnt[mode[i] * kNumShapeIds + shape[i]];
    for (int i = 0; i < n; ++i)
      if (jobs[i].qlen > 0 && jobs[i].tlen > 0 &&
          use_split(ncol[i], cnt[mode[i] * kNumShapeIds + shape[i]], shape[i] == kWideShape))
        shape[i] = kSplitBase + ext_split_for(ncol[i]);
  }
  for (int i = 0; i < n; ++i)
    if (shape[i] == kWideShape) ++n_wide, wide_max = std::max(wide_max, ext_wide_scratch(jobs[i].qlen, jobs[i].tlen));
  std::vector<int64_t> qpad, tpad;
  int rc = upload_and_pack(c, b, n, qo.data(), ql.data(), to.data(), tl.data(), nseg, segs, qpad, tpad, rt);
  if (rc) return rc;
  // device job table
  std::vector<ksw2g_job> dj(n);
  for (int i = 0; i < n; ++i) {
    dj[i] = ksw2g_job{qpad[i], tpad[i], jobs[i].qlen, jobs[i].tlen, jobs[i].w, jobs[i].zdrop, jobs[i].end_bonus,
                      jobs[i].flag};
  }
  // Longest jobs first: the persistent kernels then finish with short jobs and
  // the waves (traceback budget) are cut from that order, so no wave waits on
  // one long pair.  Bins by (mode, shape) inside each wave.
  // counting sort by qlen+tlen, longest first (stable)
  std::vector<int32_t> srt(n);
  {
    int64_t maxkey = 0;
    for (int i = 0; i < n; ++i) maxkey = std::max<int64_t>(maxkey, (int64_t)ql[i] + tl[i]);
    std::vector<int32_t> cnt((size_t)maxkey + 2, 0);
    for (int i = 0; i < n; ++i) ++cnt[(size_t)(maxkey - ((int64_t)ql[i] + tl[i]))];
    int32_t acc = 0;
    for (auto &c : cnt) { const int32_t t = c; c = acc; acc += t; }
    for (int i = 0; i < n; ++i) srt[cnt[(size_t)(maxkey - ((int64_t)ql[i] + tl[i]))]++] = i;
  }
  b->waves.clear();
  // Runs that alternate waves between two streams cut batches of short pairs into waves
  // of at most 1 GiB of traceback rows (a single larger job still gets a wave of its
  // own, up to the budget): on 1,000,000 config-1 pairs a step takes 187.8 ms with 1 GiB
  // waves, 190.1 with 4 GiB and 192.5 with 8 GiB.  Batches of long pairs keep the largest
  // waves, because every wave ends with the tail of its longest pair (config 2's long
  // pairs ran 3.6x slower in 1 GiB waves).
  int64_t wave_cap = std::max<int64_t>(c->tb_budget / std::max(c->wave_div, 1), 16);
  if (c->wave_div >= 2 && n > 0 && (double)band_cells / n < kLongCells) wave_cap = std::min<int64_t>(wave_cap, kWaveTarget);
  std::vector<int64_t> tbo(n);
  std::vector<int32_t> ord(n);
  int64_t ordp = 0;
  const int nshp = kNumShapeIds;  // both lane widths' shapes and the block-wide kernel
  const int nbins = 3 * nshp;
  std::vector<int32_t> bcount(nbins), bpos(nbins);
  std::vector<double> bwords(nbins);
  for (int i = 0; i < n;) {
    Wave wv;
    wv.w0 = i;
    wv.any_cig = false;
    int64_t acc = 0;
    while (i < n && (acc + foot[srt[i]] <= wave_cap || i == wv.w0)) tbo[srt[i]] = acc, acc += foot[srt[i]], ++i;
    wv.w1 = i;
    wv.tb_bytes = acc;
    std::fill(bcount.begin(), bcount.end(), 0);
    std::fill(bwords.begin(), bwords.end(), 0.0);
    for (int k = wv.w0; k < wv.w1; ++k) {
      const int j = srt[k], bi = mode[j] * nshp + shape[j];
      ++bcount[bi], bwords[bi] += dwords[j];
    }
    for (int bi = 0; bi < nbins; ++bi) {
      bpos[bi] = (int32_t)ordp;
      if (bcount[bi]) {
        wv.bins.push_back(Bin{bi / nshp, bi % nshp, ordp, bcount[bi], 0.0, 0});
        wv.any_cig |= bi / nshp != 0;
      }
      ordp += bcount[bi];
    }
    for (int k = wv.w0; k < wv.w1; ++k) ord[bpos[mode[srt[k]] * nshp + shape[srt[k]]]++] = srt[k];
    if (wv.bins.size() > 1) {
      for (Bin &bn : wv.bins) {  // a bin's first job is its longest (the order is longest first)
        const int j = ord[bn.order_off];
        bn.cost = bin_cost(bn.shape, std::max<int64_t>((int64_t)ql[j] + tl[j] - 1, 0), bwords[bn.mode * nshp + bn.shape]);
      }
      spread_bins(wv.bins);
    }
    b->waves.push_back(wv);
  }
  b->n_counters = 0;
  for (auto &wv : b->waves) b->n_counters += (int)wv.bins.size();
  if ((rc = b->jobs.ensure(sizeof(ksw2g_job) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->order.ensure(sizeof(int32_t) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->sorted.ensure(sizeof(int32_t) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->tb_off.ensure(sizeof(int64_t) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->res.ensure(sizeof(ksw2g_ext_result) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->bts.ensure(sizeof(ksw2g_bt) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->counters.ensure(16 + sizeof(int) * (size_t)std::max(b->n_counters, 1)))) return rc;
  // block scratch of the wide-band jobs: one area per resident block, in two halves for two-stream runs
  b->wide_blocks = 0, b->wide_stride = 0;
  if (n_wide) {
    if (!c->nsm) c->nsm = num_sms(c->device);
    b->wide_blocks = std::min(n_wide, std::max(c->nsm, 1) * 2);
    b->wide_stride = wide_max;
    if ((rc = b->wide.ensure((size_t)(2 * b->wide_blocks) * (size_t)wide_max))) return rc;
  }
  b->cigar_cap = std::max<int64_t>(cig, 16);
  if ((rc = b->cigar.ensure(sizeof(uint32_t) * (size_t)b->cigar_cap))) return rc;
  if (n) {
    CK(cudaMemcpyAsync(b->jobs.p, dj.data(), sizeof(ksw2g_job) * n, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(b->order.p, ord.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(b->sorted.p, srt.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(b->tb_off.p, tbo.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

extern "C" int ksw2g_ext_prepare(ksw2g_ctx_t *c, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e,
                                 int8_t q2, int8_t e2, int n_jobs, const ksw2g_job_t *jobs, const uint8_t *qbuf,
                                 int64_t qbuf_len, const uint8_t *tbuf, int64_t tbuf_len, ksw2g_batch_t **out) {
  if (!c || !out) return set_err(KSW2G_E_ARG, "null ctx/out");
  ksw2g_batch *b = new ksw2g_batch;
  int rc = ext_prepare_into(c, b, dual, m, mat, q, e, q2, e2, n_jobs, jobs, qbuf, qbuf_len, tbuf, tbuf_len);
  if (rc) {
    ksw2g_batch_free(b);
    return rc;
  }
  *out = b;
  return 0;
}

// Per-launch timing (ksw2g_batch_set_timing): an event pair on the launching
// stream around each kernel.
static cudaError_t timed_begin(ksw2g_batch *b, int kind, cudaStream_t st) {
  if (!b->timing) return cudaSuccess;
  const size_t need = 2 * (size_t)(b->n_timed + 1);
  while (b->tev.size() < need) {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return r;
    b->tev.push_back(e);
  }
  if (b->tkind.size() < (size_t)b->n_timed + 1) b->tkind.resize(b->n_timed + 1);
  b->tkind[b->n_timed] = kind;
  return cudaEventRecord(b->tev[2 * b->n_timed], st);
}
static cudaError_t timed_end(ksw2g_batch *b, cudaStream_t st) {
  if (!b->timing) return cudaSuccess;
  const cudaError_t r = cudaEventRecord(b->tev[2 * b->n_timed + 1], st);
  ++b->n_timed;
  return r;
}

int64_t ext_max_wave(const ksw2g_batch *b) {
  int64_t m = 16;
  for (const Wave &wv : b->waves) m = std::max(m, wv.tb_bytes);
  return m;
}

int ext_run_on(ksw2g_batch *b, cudaStream_t st, uint8_t *tb, int64_t tb_cap) {
  return ext_run_on2(b, st, nullptr, tb, nullptr, tb_cap);
}

int ext_run_on2(ksw2g_batch *b, cudaStream_t s0, cudaStream_t s1, uint8_t *tb0, uint8_t *tb1, int64_t tb_cap) {
  b->launches = 0;
  if (b->n == 0) return 0;
  for (auto &wv : b->waves)
    if (wv.tb_bytes > tb_cap) return set_err(KSW2G_E_CAPACITY, "traceback wave exceeds the pool");
  const bool two = s1 && tb1 && b->waves.size() >= 2;
  if (two && !b->ev_fork) {
    CK(cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming));
    CK(cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming));
  }
  cudaStream_t st = s0;
  uint8_t *tb = tb0;
  int *cnt = b->counters.as<int>();
  unsigned long long *cursor = (unsigned long long *)cnt;  // bytes 0..7
  int *err = cnt + 2;                                      // bytes 8..11
  int *jc = cnt + 4;                                       // per-bin job counters
  CK(cudaMemsetAsync(b->counters.p, 0, 16 + sizeof(int) * (size_t)b->n_counters, s0));
  if (two) {
    CK(cudaEventRecord(b->ev_fork, s0));
    CK(cudaStreamWaitEvent(s1, b->ev_fork, 0));
  }
  const ksw2g_job *dj = b->jobs.as<ksw2g_job>();
  ksw2g_ext_result *dr = b->res.as<ksw2g_ext_result>();
  ksw2g_bt *db = b->bts.as<ksw2g_bt>();
  const int64_t *dto = b->tb_off.as<int64_t>();
  const int32_t *dord = b->order.as<int32_t>();
  const int32_t *dsrt = b->sorted.as<int32_t>();
  int ci = 0;
  for (size_t w = 0; w < b->waves.size(); ++w) {
    const Wave &wv = b->waves[w];
    const int par = two && (w & 1) ? 1 : 0;
    st = par ? s1 : s0;
    tb = par ? tb1 : tb0;
    int nside = 0;
    for (auto &bn : wv.bins) nside = std::max(nside, bn.sub);
    if (nside) {  // fork the side streams from the wave's stream (after its previous wave's backtrack)
      if (!b->ev_wfork[par]) CK(cudaEventCreateWithFlags(&b->ev_wfork[par], cudaEventDisableTiming));
      for (int i = 0; i < nside; ++i) {
        if (!b->side[par][i]) CK(cudaStreamCreateWithFlags(&b->side[par][i], cudaStreamNonBlocking));
        if (!b->ev_wjoin[par][i]) CK(cudaEventCreateWithFlags(&b->ev_wjoin[par][i], cudaEventDisableTiming));
      }
      CK(cudaEventRecord(b->ev_wfork[par], st));
      for (int i = 0; i < nside; ++i) CK(cudaStreamWaitEvent(b->side[par][i], b->ev_wfork[par], 0));
    }
    for (auto &bn : wv.bins) {
      const cudaStream_t bs = bn.sub ? b->side[par][bn.sub - 1] : st;
      ExtLaunch L{dj, dord + bn.order_off, bn.count, b->arena.as<uint8_t>(), dr, db, tb, dto,
                  jc + ci++};
      if (bn.shape == kWideShape)  // each stream of a two-stream run has its own half of the scratch
        L.wide_scratch = b->wide.as<uint8_t>() + (size_t)par * b->wide_blocks * b->wide_stride,
        L.wide_stride = b->wide_stride, L.wide_blocks = b->wide_blocks;
      CK(timed_begin(b, 0, bs));
      CK(launch_ext_dp(b->kind, bn.mode, bn.shape, b->P, L, 0, bs));
      CK(timed_end(b, bs));
      ++b->launches;
    }
    for (int i = 0; i < nside; ++i) {
      CK(cudaEventRecord(b->ev_wjoin[par][i], b->side[par][i]));
      CK(cudaStreamWaitEvent(st, b->ev_wjoin[par][i], 0));
    }
    if (wv.any_cig) {
      CK(timed_begin(b, 1, st));
      CK(launch_ext_bt(dj, dsrt + wv.w0, wv.w1 - wv.w0, db, tb, dto, dr,
                       b->cigar.as<uint32_t>(), cursor, (long long)b->cigar_cap, err, st));
      CK(timed_end(b, st));
      ++b->launches;
    }
  }
  if (two) {
    CK(cudaEventRecord(b->ev_join, s1));
    CK(cudaStreamWaitEvent(s0, b->ev_join, 0));
  }
  return 0;
}

static int ext_run(ksw2g_ctx *c, ksw2g_batch *b) {
  CK(cudaSetDevice(c->device));
  const int64_t maxtb = ext_max_wave(b), al = (maxtb + 255) & ~(int64_t)255;
  int rc;
  if (b->waves.size() >= 2 && 2 * maxtb <= c->tb_budget + 512 && c->wave_div >= 2) {
    if (!c->aux && cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking) != cudaSuccess)
      return set_err(KSW2G_E_CUDA, "cudaStreamCreate failed");
    if ((rc = c->tb_pool.ensure((size_t)(2 * al)))) return rc;
    uint8_t *tb = c->tb_pool.as<uint8_t>();
    return ext_run_on2(b, c->st, c->aux, tb, tb + al, maxtb);
  }
  if ((rc = c->tb_pool.ensure((size_t)maxtb))) return rc;
  return ext_run_on(b, c->st, c->tb_pool.as<uint8_t>(), (int64_t)c->tb_pool.cap);
}

extern "C" int ksw2g_batch_run(ksw2g_ctx_t *c, ksw2g_batch_t *b) {
  if (!c || !b) return set_err(KSW2G_E_ARG, "null ctx/batch");
  if (b->kind <= 1) return ext_run(c, b);
  extern int ll_run(ksw2g_ctx * c, ksw2g_batch * b);
  return ll_run(c, b);
}

extern "C" int ksw2g_ext_fetch(ksw2g_ctx_t *c, ksw2g_batch_t *b, ksw2g_ext_result_t *res, uint32_t *cigar,
                               int64_t cigar_cap, int64_t *cigar_used) {
  if (!c || !b || b->kind > 1) return set_err(KSW2G_E_ARG, "not an extension batch");
  CK(cudaSetDevice(c->device));
  struct {
    unsigned long long cursor;
    int err, pad;
  } hdr = {0, 0, 0};
  if (b->n) {
    if (res) CK(cudaMemcpyAsync(res, b->res.p, sizeof(ksw2g_ext_result) * b->n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(&hdr, b->counters.p, sizeof hdr, cudaMemcpyDeviceToHost, c->st));
  }
  CK(cudaStreamSynchronize(c->st));
  if (hdr.err) return set_err(KSW2G_E_CAPACITY, "device CIGAR arena overflow");
  if (cigar_used) *cigar_used = (int64_t)hdr.cursor;
  if (hdr.cursor > 0 && cigar) {
    if ((int64_t)hdr.cursor > cigar_cap)
      return set_err(KSW2G_E_CAPACITY, "CIGAR buffer holds %lld words, %llu needed", (long long)cigar_cap,
                     hdr.cursor);
    CK(cudaMemcpyAsync(cigar, b->cigar.p, sizeof(uint32_t) * hdr.cursor, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
  }
  return 0;
}

// One-shot extension batches of more than kChunkJobs jobs run as chunks that
// rotate through kOneShotDepth sub-contexts: while the device runs chunks i and i+1,
// the host prepares chunk i+2 (job table, wave plan, uploads) on a third stream.
// Each chunk's CIGARs are appended to the caller's buffer as the chunk
// completes, and its results' cigar_off are shifted to match.  Small chunks keep
// the gaps between them short: on 1,000,000 pairs of 100-300 nt the call takes
// 136.7 ms with chunks of 16,384 jobs and 143.2 ms with 32,768.
// Long pairs want larger chunks, because every chunk ends with the tail of its own
// longest pair: 200,000 pairs of 0.5-30 kb at w=500 run 14% slower in chunks of
// 32,768 than of 131,072.  So batches whose pairs average more than kLongCells
// band cells use the larger chunk.
static const int kChunkJobs = 16384, kChunkJobsLong = 131072;

static int chunk_jobs(int n, const ksw2g_job_t *jobs) {
  double cells = 0;
  for (int i = 0; i < n; ++i) {
    const ksw2g_job_t &J = jobs[i];
    const int64_t mn = J.qlen < J.tlen ? J.qlen : J.tlen;
    const int64_t band = J.w < 0 || J.w + 1 > mn ? mn : J.w + 1;
    cells += (double)(J.qlen + J.tlen) * (double)band;
  }
  return n > 0 && cells / n > kLongCells ? kChunkJobsLong : kChunkJobs;
}

// Chunk boundaries of a one-shot call of n jobs in chunks of about `per` jobs.  With `early`
// the first chunk is an eighth of that (at least 1,024 jobs), so that the device starts on it
// while the host still prepares the second.  Chunks of long pairs keep one size: every chunk
// ends with the tail of its own longest pair, and one more chunk is one more tail (config 2
// end to end: 624 k aln/s with a small first chunk, 676 k without).
static std::vector<int> chunk_starts(int n, int per, bool early) {
  std::vector<int> st{0};
  const int first = early ? std::min(per, std::max(1024, per / 8)) : per;
  for (int64_t j = first; j < n; j += per) st.push_back((int)j);
  st.push_back(n);
  return st;
}

static int sub_ctx(ksw2g_ctx *c, int i, ksw2g_ctx **out) {
  if (!c->sub[i]) {
    int rc = ksw2g_ctx_create(c->device, &c->sub[i]);
    if (rc) return rc;
    c->sub[i]->scratch = new ksw2g_batch;
  }
  c->sub[i]->tb_budget = std::max<int64_t>(c->tb_budget / 2, 1 << 20);
  c->sub[i]->wave_div = 1;  // each sub-context runs one stream; the chunks rotate through them
  *out = c->sub[i];
  return 0;
}

// With rt the targets are windows of the device-resident reference (toff is the
// window start on contig rt->tid[i]) and only the queries are uploaded.
static int ext_batch_chunked(ksw2g_ctx *c, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e, int8_t q2,
                             int8_t e2, int n, const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
                             const uint8_t *tbuf, int64_t tbuf_len, ksw2g_ext_result_t *res, uint32_t *cigar,
                             int64_t cigar_cap, int64_t *cigar_used, const RefTargets *rt = nullptr) {
  const int cj_jobs = chunk_jobs(n, jobs);
  const std::vector<int> cst = chunk_starts(n, cj_jobs, cj_jobs == kChunkJobs);
  const int nch = (int)cst.size() - 1;
  ksw2g_ctx *sc[kOneShotDepth];
  int rc;
  for (int i = 0; i < kOneShotDepth; ++i)
    if ((rc = sub_ctx(c, i, &sc[i]))) return rc;
  int64_t used = 0;
  int pending[kOneShotDepth];  // chunk index in flight on each sub-context
  std::fill(pending, pending + kOneShotDepth, -1);
  c->oneshot_launches = 0;
  auto finish = [&](int s) -> int {
    const int ch = pending[s];
    if (ch < 0) return 0;
    pending[s] = -1;
    ksw2g_ctx *x = sc[s];
    ksw2g_batch *b = x->scratch;
    const int j0 = cst[ch];
    struct {
      unsigned long long cursor;
      int err, pad;
    } hdr = {0, 0, 0};
    CK(cudaMemcpyAsync(&hdr, b->counters.p, sizeof hdr, cudaMemcpyDeviceToHost, x->st));
    CK(cudaStreamSynchronize(x->st));  // the chunk's results are in res by now
    if (hdr.err) return set_err(KSW2G_E_CAPACITY, "device CIGAR arena overflow");
    if (hdr.cursor) {
      if (!cigar || used + (int64_t)hdr.cursor > cigar_cap)
        return set_err(KSW2G_E_CAPACITY, "CIGAR buffer holds %lld words, more needed", (long long)cigar_cap);
      CK(cudaMemcpyAsync(cigar + used, b->cigar.p, sizeof(uint32_t) * hdr.cursor, cudaMemcpyDeviceToHost, x->st));
      if (res)
        for (int i = 0; i < b->n; ++i) res[j0 + i].cigar_off += used;
      used += (int64_t)hdr.cursor;
      CK(cudaStreamSynchronize(x->st));
    }
    return 0;
  };
  for (int ch = 0; ch < nch && !rc; ++ch) {
    const int s = ch % kOneShotDepth;
    if ((rc = finish(s))) break;
    const int j0 = cst[ch], nj = cst[ch + 1] - j0;
    ksw2g_ctx *x = sc[s];
    ksw2g_batch *b = x->scratch;
    // upload only the part of the sequence buffers this chunk's jobs read
    int64_t qlo = qbuf_len, qhi = 0, tlo = tbuf_len, thi = 0;
    for (int i = j0; i < j0 + nj; ++i) {
      const ksw2g_job_t &J = jobs[i];
      if (J.qoff < 0 || J.toff < 0 || J.qlen < 0 || J.tlen < 0 || J.qoff + J.qlen > qbuf_len ||
          (!rt && J.toff + J.tlen > tbuf_len)) {
        rc = set_err(KSW2G_E_ARG, "job %d: sequence out of buffer bounds", i);
        break;
      }
      qlo = std::min(qlo, J.qoff), qhi = std::max<int64_t>(qhi, J.qoff + J.qlen);
      if (!rt) tlo = std::min(tlo, J.toff), thi = std::max<int64_t>(thi, J.toff + J.tlen);
    }
    if (rc) break;
    if (qlo > qhi) qlo = qhi = 0;
    if (rt || tlo > thi) tlo = thi = 0;
    std::vector<ksw2g_job_t> cj(jobs + j0, jobs + j0 + nj);
    for (auto &J : cj) J.qoff -= qlo, J.toff -= tlo;
    if (rt) {
      const SeqSeg seg{cj.data(), nj, qbuf + qlo, qhi - qlo, nullptr, 0};
      const RefTargets crt{rt->ref, rt->tid + j0, rt->flags ? rt->flags + j0 : nullptr};
      rc = ext_prepare_segs(x, b, dual, m, mat, q, e, q2, e2, 1, &seg, &crt);
    } else {
      rc = ext_prepare_into(x, b, dual, m, mat, q, e, q2, e2, nj, cj.data(), qbuf + qlo, qhi - qlo, tbuf + tlo,
                            thi - tlo);
    }
    if (rc) break;
    if ((rc = ext_run(x, b))) break;
    c->oneshot_launches += b->launches + (rt ? 1 : 0) + (nj ? 1 : 0);  // DP and backtrack, window gather, packing
    if (res && nj)
      CK(cudaMemcpyAsync(res + j0, b->res.p, sizeof(ksw2g_ext_result) * nj, cudaMemcpyDeviceToHost, x->st));
    pending[s] = ch;
  }
  // drain in chunk order (the CIGAR buffer is filled in chunk order)
  for (int ch = nch - kOneShotDepth; ch < nch && !rc; ++ch)
    if (ch >= 0) rc = finish(ch % kOneShotDepth);
  if (rc) {
    for (int s = 0; s < kOneShotDepth; ++s) cudaStreamSynchronize(sc[s]->st);
    return rc;
  }
  if (cigar_used) *cigar_used = used;
  return 0;
}

extern "C" int ksw2g_ext_batch(ksw2g_ctx_t *c, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e,
                               int8_t q2, int8_t e2, int n_jobs, const ksw2g_job_t *jobs, const uint8_t *qbuf,
                               int64_t qbuf_len, const uint8_t *tbuf, int64_t tbuf_len, ksw2g_ext_result_t *res,
                               uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_used) {
  if (!c) return set_err(KSW2G_E_ARG, "null ctx");
  CK(cudaSetDevice(c->device));
  if (n_jobs > kChunkJobs)
    return ext_batch_chunked(c, dual, m, mat, q, e, q2, e2, n_jobs, jobs, qbuf, qbuf_len, tbuf, tbuf_len, res, cigar,
                             cigar_cap, cigar_used);
  if (!c->scratch) c->scratch = new ksw2g_batch;
  int rc = ext_prepare_into(c, c->scratch, dual, m, mat, q, e, q2, e2, n_jobs, jobs, qbuf, qbuf_len, tbuf, tbuf_len);
  if (rc) return rc;
  if ((rc = ext_run(c, c->scratch))) return rc;
  return ksw2g_ext_fetch(c, c->scratch, res, cigar, cigar_cap, cigar_used);
}

int ll_run(ksw2g_ctx *c, ksw2g_batch *b);

// ---- batches whose targets are windows of a device-resident reference
extern "C" int ksw2g_ext_prepare_ref(ksw2g_ctx_t *c, const ksw2g_ref_t *ref, int dual, int8_t m, const int8_t *mat,
                                     int8_t q, int8_t e, int8_t q2, int8_t e2, int n_jobs, const ksw2g_job_t *jobs,
                                     const int32_t *tid, const int32_t *tflags, const uint8_t *qbuf,
                                     int64_t qbuf_len, ksw2g_batch_t **out) {
  if (!c || !out || !ref) return set_err(KSW2G_E_ARG, "null ctx/ref/out");
  ksw2g_batch *b = new ksw2g_batch;
  const SeqSeg seg{jobs, n_jobs, qbuf, qbuf_len, nullptr, 0};
  const RefTargets rt{ref, tid, tflags};
  int rc = ext_prepare_segs(c, b, dual, m, mat, q, e, q2, e2, 1, &seg, &rt);
  if (rc) {
    ksw2g_batch_free(b);
    return rc;
  }
  *out = b;
  return 0;
}

extern "C" int ksw2g_ext_batch_ref(ksw2g_ctx_t *c, const ksw2g_ref_t *ref, int dual, int8_t m, const int8_t *mat,
                                   int8_t q, int8_t e, int8_t q2, int8_t e2, int n_jobs, const ksw2g_job_t *jobs,
                                   const int32_t *tid, const int32_t *tflags, const uint8_t *qbuf, int64_t qbuf_len,
                                   ksw2g_ext_result_t *res, uint32_t *cigar, int64_t cigar_cap, int64_t *cigar_used) {
  if (!c || !ref) return set_err(KSW2G_E_ARG, "null ctx/ref");
  CK(cudaSetDevice(c->device));
  const RefTargets rt{ref, tid, tflags};
  if (n_jobs > kChunkJobs) {
    if (!tid) return set_err(KSW2G_E_ARG, "reference targets need a contig id per job");
    return ext_batch_chunked(c, dual, m, mat, q, e, q2, e2, n_jobs, jobs, qbuf, qbuf_len, nullptr, 0, res, cigar,
                             cigar_cap, cigar_used, &rt);
  }
  if (!c->scratch) c->scratch = new ksw2g_batch;
  const SeqSeg seg{jobs, n_jobs, qbuf, qbuf_len, nullptr, 0};
  int rc = ext_prepare_segs(c, c->scratch, dual, m, mat, q, e, q2, e2, 1, &seg, &rt);
  if (rc) return rc;
  if ((rc = ext_run(c, c->scratch))) return rc;
  c->oneshot_launches = c->scratch->launches + 1 + (n_jobs ? 1 : 0);
  return ksw2g_ext_fetch(c, c->scratch, res, cigar, cigar_cap, cigar_used);
}

extern "C" int ksw2g_ll_batch_ref(ksw2g_ctx_t *c, const ksw2g_ref_t *ref, int size, int m, const int8_t *mat, int gapo,
                                  int gape, int n_jobs, const ksw2g_ll_job_t *jobs, const int32_t *tid,
                                  const int32_t *tflags, const uint8_t *qbuf, int64_t qbuf_len,
                                  ksw2g_ll_result_t *res) {
  if (!c || !ref) return set_err(KSW2G_E_ARG, "null ctx/ref");
  CK(cudaSetDevice(c->device));
  if (!c->scratch) c->scratch = new ksw2g_batch;
  const SeqSeg seg{jobs, n_jobs, qbuf, qbuf_len, nullptr, 0};
  const RefTargets rt{ref, tid, tflags};
  int rc = ll_prepare_segs(c, c->scratch, size, m, mat, gapo, gape, 1, &seg, &rt);
  if (rc) return rc;
  if ((rc = ll_run(c, c->scratch))) return rc;
  return ksw2g_ll_fetch(c, c->scratch, res);
}

extern "C" int ksw2g_ext_num_shapes(void) { return kNumExtShapes; }
extern "C" int ksw2g_ext_shape_info(int shape, int *g, int *k) {
  if (shape < 0 || shape >= kNumExtShapes) return set_err(KSW2G_E_ARG, "bad shape");
  if (g) *g = kExtShapes[shape].G;
  if (k) *k = kExtShapes[shape].K;
  return 0;
}
extern "C" int ksw2g_ext_set_shape(int dual, int mode, int lo, int hi, int shape) {
  if (shape < 0 || shape >= 2 * kNumExtShapes || mode < 0 || mode > 2) return set_err(KSW2G_E_ARG, "bad shape/mode");
  ext_shape_set_pref(dual, mode, lo, hi, shape);
  return 0;
}
extern "C" int ksw2g_ext_set_family(int family) {
  if (family < -1 || family > 1) return set_err(KSW2G_E_ARG, "lane width must be -1 (tuned), 0 (bytes) or 1 (16-bit)");
  g_family.store(family);
  return 0;
}
extern "C" int ksw2g_ext_get_family(void) { return g_family.load(); }
extern "C" int ksw2g_ext_set_split(int mode) {
  if (mode < -1 || mode > 1) return set_err(KSW2G_E_ARG, "split mode must be -1 (batch decides), 0 (never) or 1 (always)");
  g_split.store(mode);
  return 0;
}
extern "C" int ksw2g_ext_get_split(void) { return g_split.load(); }

// ---------------------------------------------------------------- per-call drop-in
// Allocation of ez->cigar and of the ksw_ll_qinit block follows the caller's
// allocator: when the process exports kalloc's krealloc/kmalloc (minibwa built
// with mimalloc=0, i.e. HAVE_KALLOC, and linked with -rdynamic), they are used
// with the caller's km exactly as ksw2.h:114-122 does; kalloc itself falls back
// to libc for km == NULL (kalloc.c:128-185).  Otherwise libc realloc/malloc.
extern "C" void *krealloc(void *km, void *ptr, size_t size) __attribute__((weak));
extern "C" void *kmalloc(void *km, size_t size) __attribute__((weak));
static void *caller_realloc(void *km, void *p, size_t n) { return krealloc ? krealloc(km, p, n) : realloc(p, n); }
static void *caller_malloc(void *km, size_t n) { return kmalloc ? kmalloc(km, n) : malloc(n); }

// Each host thread gets its own context (stream + scratch) on the current
// device, so concurrent kt_for workers never share a stream.
static void die(const char *what, cudaError_t e) {
  fprintf(stderr, "[ksw2gpu] fatal: %s: %s\n", what, cudaGetErrorString(e));
  abort();
}
#define DIE_ON(x)                          \
  do {                                     \
    cudaError_t e_ = (x);                  \
    if (e_ != cudaSuccess) die(#x, e_);    \
  } while (0)

struct TlsCtx {
  ksw2g_ctx *c = nullptr;
  ~TlsCtx() {
    if (c) ksw2g_ctx_destroy(c);
  }
};
static thread_local TlsCtx tls;

static ksw2g_ctx *thread_ctx() {
  int dev = 0;
  DIE_ON(cudaGetDevice(&dev));
  if (tls.c && tls.c->device != dev) {
    ksw2g_ctx_destroy(tls.c);
    tls.c = nullptr;
  }
  if (!tls.c) {
    if (ksw2g_ctx_create(dev, &tls.c) != 0) {
      fprintf(stderr, "[ksw2gpu] fatal: %s\n", tl_err.c_str());
      abort();
    }
  }
  return tls.c;
}

// Device scratch layout of one call (all 16-byte aligned):
//   [0,16) cursor/err | [16,32) job counter | job | tb_off | bt | res | cigar | arena | traceback
static void ext_one(void *km, int dual, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
                    const int8_t *mat, int8_t q, int8_t e, int8_t q2, int8_t e2, int w, int zdrop, int end_bonus,
                    int flag, ksw_extz_t *ez) {
  // ksw_reset_extz (ksw2.h:174-179): cigar and m_cigar are left alone
  ez->max_q = ez->max_t = ez->mqe_t = ez->mte_q = -1;
  ez->max = 0, ez->score = ez->mqe = ez->mte = KSW_NEG_INF;
  ez->n_cigar = 0, ez->zdropped = 0, ez->reach_end = 0;
  if (m <= dual || qlen <= 0 || tlen <= 0) return;
  ksw2g_ext_params P;
  derive_ext_params(dual, m, mat, q, e, q2, e2, P);
  if (P.skip_all) return;
  if ((flag & KSW_EZ_GENERIC_SC) && m > 16) {
    fprintf(stderr, "[ksw2gpu] fatal: GENERIC_SC with m=%d > 16 is not supported on the device\n", m);
    abort();
  }
  ksw2g_ctx *c = thread_ctx();
  const int mode = ext_mode(flag);
  const int nc = ext_ncol(qlen, tlen, w);
  int shape = ext_shape_id(dual, mode, nc, P);
  if (use_split(nc, 1, shape == kWideShape)) shape = kSplitBase + ext_split_for(nc);
  const int64_t ncig = mode ? (int64_t)qlen + tlen + 1 : 0;
  const int64_t foot = mode ? (int64_t)(qlen + tlen - 1) * nc * 16 : 0;
  const size_t o_job = 32, o_tbo = o_job + 48, o_bt = o_tbo + 16, o_res = o_bt + 16;
  const size_t o_cig = o_res + 64;
  const size_t o_arena = (o_cig + ncig * 4 + 15) & ~(size_t)15;
  const size_t arena_bytes = slot_bytes(qlen) + slot_bytes(tlen);
  const size_t o_tb = (o_arena + arena_bytes + 255) & ~(size_t)255;
  const int64_t wide = shape == kWideShape ? ext_wide_scratch(qlen, tlen) : 0;  // block scratch of a wide band
  const size_t o_wide = (o_tb + foot + 255) & ~(size_t)255;
  const size_t total = o_wide + wide + 16;
  if (c->one.ensure(total) || c->one_h.ensure(o_tb)) {
    fprintf(stderr, "[ksw2gpu] fatal: %s\n", tl_err.c_str());
    abort();
  }
  uint8_t *h = (uint8_t *)c->one_h.p;
  uint8_t *d = (uint8_t *)c->one.p;
  memset(h, 0, o_job);
  const int64_t qpad = (int64_t)(o_arena - o_arena) + 32, tpad = slot_bytes(qlen) + 32;
  ksw2g_job J{qpad, tpad, qlen, tlen, w, zdrop, end_bonus, flag};
  memcpy(h + o_job, &J, sizeof J);
  memset(h + o_tbo, 0, 16);
  memset(h + o_arena, 0, arena_bytes);
  memcpy(h + o_arena + qpad, query, qlen);
  memcpy(h + o_arena + tpad, target, tlen);
  // upload counters + job + tb offset, and the arena, in two copies from one pinned block
  DIE_ON(cudaMemcpyAsync(d, h, o_bt, cudaMemcpyHostToDevice, c->st));
  DIE_ON(cudaMemcpyAsync(d + o_arena, h + o_arena, arena_bytes, cudaMemcpyHostToDevice, c->st));
  ExtLaunch L{(const ksw2g_job *)(d + o_job), nullptr, 1, d + o_arena, (ksw2g_ext_result *)(d + o_res),
              (ksw2g_bt *)(d + o_bt), d + o_tb, (const int64_t *)(d + o_tbo), (int *)(d + 16)};
  if (wide) L.wide_scratch = d + o_wide, L.wide_stride = wide, L.wide_blocks = 1;
  DIE_ON(launch_ext_dp(dual, mode, shape, P, L, 1, c->st));
  if (mode)
    DIE_ON(launch_ext_bt((const ksw2g_job *)(d + o_job), nullptr, 1, (const ksw2g_bt *)(d + o_bt), d + o_tb,
                         (const int64_t *)(d + o_tbo), (ksw2g_ext_result *)(d + o_res), (uint32_t *)(d + o_cig),
                         (unsigned long long *)d, (long long)ncig, (int *)(d + 8), c->st));
  DIE_ON(cudaMemcpyAsync(h + o_res, d + o_res, 64 + ncig * 4, cudaMemcpyDeviceToHost, c->st));
  DIE_ON(cudaStreamSynchronize(c->st));
  ksw2g_ext_result R;
  memcpy(&R, h + o_res, sizeof R);
  ez->max = (uint32_t)R.max, ez->zdropped = R.zdropped ? 1 : 0;
  ez->max_q = R.max_q, ez->max_t = R.max_t, ez->mqe = R.mqe, ez->mqe_t = R.mqe_t;
  ez->mte = R.mte, ez->mte_q = R.mte_q, ez->score = R.score, ez->reach_end = R.reach_end;
  if (R.n_cigar > 0) {
    // grow like ksw_push_cigar (ksw2.h:127-129): doubling from 4
    int mc = ez->m_cigar;
    while (mc < R.n_cigar) mc = mc ? mc << 1 : 4;
    if (mc != ez->m_cigar || !ez->cigar) {
      ez->cigar = (uint32_t *)caller_realloc(km, ez->cigar, (size_t)mc * 4);
      ez->m_cigar = mc;
    }
    memcpy(ez->cigar, h + o_cig, (size_t)R.n_cigar * 4);
    ez->n_cigar = R.n_cigar;
  }
}

extern "C" void ksw_extz2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
                              const int8_t *mat, int8_t q, int8_t e, int w, int zdrop, int end_bonus, int flag,
                              ksw_extz_t *ez) {
  ext_one(km, 0, qlen, query, tlen, target, m, mat, q, e, q, e, w, zdrop, end_bonus, flag, ez);
}

extern "C" void ksw_extd2_sse(void *km, int qlen, const uint8_t *query, int tlen, const uint8_t *target, int8_t m,
                              const int8_t *mat, int8_t gapo, int8_t gape, int8_t gapo2, int8_t gape2, int w,
                              int zdrop, int end_bonus, int flag, ksw_extz_t *ez) {
  ext_one(km, 1, qlen, query, tlen, target, m, mat, gapo, gape, gapo2, gape2, w, zdrop, end_bonus, flag, ez);
}

// ================================================================ ksw_ll
int ll_prepare_into(ksw2g_ctx *c, ksw2g_batch *b, int size, int m, const int8_t *mat, int gapo, int gape, int n,
                    const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
                    int64_t tbuf_len) {
  if (n < 0 || (n > 0 && !jobs)) return set_err(KSW2G_E_ARG, "bad ll batch arguments");
  const SeqSeg seg{jobs, n, qbuf, qbuf_len, tbuf, tbuf_len};
  return ll_prepare_segs(c, b, size, m, mat, gapo, gape, 1, &seg);
}

int ll_prepare_segs(ksw2g_ctx *c, ksw2g_batch *b, int size, int m, const int8_t *mat, int gapo, int gape, int nseg,
                    const SeqSeg *segs, const RefTargets *rt) {
  if (rt && (nseg != 1 || !rt->ref || (segs[0].n > 0 && !rt->tid)))
    return set_err(KSW2G_E_ARG, "reference targets need one segment and a contig id per job");
  std::vector<ksw2g_ll_job_t> flat;
  const ksw2g_ll_job_t *jobs = nullptr;
  int n = 0;
  int64_t qbuf_len = 0, tbuf_len = 0;
  {
    const int rc0 = flatten_segs(nseg, segs, flat, jobs, n, qbuf_len, tbuf_len);
    if (rc0) return rc0;
  }
  if (n < 0 || (n > 0 && !jobs) || !mat || m <= 0 || m > 64) return set_err(KSW2G_E_ARG, "bad ll batch arguments");
  CK(cudaSetDevice(c->device));
  size = size > 1 ? 2 : 1;
  b->kind = size == 1 ? 2 : 3;
  b->ll_size = size, b->ll_m = m, b->ll_gapo = gapo, b->ll_gape = gape;
  b->n = n;
  b->launches = 0;
  const int lanes = size == 1 ? 16 : 8;
  std::vector<int64_t> qo(n), to(n), blo(n);
  std::vector<int32_t> ql(n), tl(n);
  int slen = 1;
  int64_t nbl = 0;
  for (int i = 0; i < n; ++i) {
    const ksw2g_ll_job_t &J = jobs[i];
    if (J.qlen < 0 || J.tlen < 0 || J.qoff < 0 || J.toff < 0 || J.qoff + J.qlen > qbuf_len ||
        (!rt && J.toff + J.tlen > tbuf_len))
      return set_err(KSW2G_E_ARG, "ll job %d: sequence out of buffer bounds", i);
    if (rt && ref_check_window(rt->ref, rt->tid[i], J.toff, J.tlen)) return KSW2G_E_ARG;
    qo[i] = J.qoff, to[i] = J.toff, ql[i] = J.qlen, tl[i] = J.tlen;
    slen = std::max(slen, (J.qlen + lanes - 1) / lanes);
    blo[i] = nbl;
    if (J.xtra & KSW_LL_SUBO) nbl += J.tlen;
  }
  if (slen > ll_slen_cap(size, m))
    return set_err(KSW2G_E_BAND, "ll query of %d segments exceeds the kernel's %d", slen, ll_slen_cap(size, m));
  b->ll_slen = slen;
  b->ll_qlen_max = 0;
  for (int i = 0; i < n; ++i) b->ll_qlen_max = std::max(b->ll_qlen_max, (int)jobs[i].qlen);
  b->ll_mat_max = mat[0];
  for (int a = 1; a < m * m; ++a) b->ll_mat_max = std::max(b->ll_mat_max, (int)mat[a]);
  std::vector<int64_t> qpad, tpad;
  int rc = upload_and_pack(c, b, n, qo.data(), ql.data(), to.data(), tl.data(), nseg, segs, qpad, tpad, rt);
  if (rc) return rc;
  // Jobs in the device table by segment count, longest first (counting sort, stable): the
  // groups of a warp then run queries of similar length side by side, so the segments
  // one group skips are not computed for another, and the longest jobs start first.
  std::vector<ksw2g_ll_job> dj(n);
  {
    std::vector<int32_t> cnt((size_t)slen + 2, 0);
    auto key = [&](int i) { return slen - (jobs[i].qlen + lanes - 1) / lanes; };
    for (int i = 0; i < n; ++i) ++cnt[(size_t)key(i)];
    int32_t acc = 0;
    for (auto &x : cnt) { const int32_t t = x; x = acc; acc += t; }
    for (int i = 0; i < n; ++i)
      dj[cnt[(size_t)key(i)]++] = ksw2g_ll_job{qpad[i], tpad[i], jobs[i].qlen, jobs[i].tlen, jobs[i].xtra, i};
  }
  if ((rc = b->jobs.ensure(sizeof(ksw2g_ll_job) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->res.ensure(sizeof(ksw2g_ll_result) * (size_t)std::max(n, 1)))) return rc;
  if ((rc = b->counters.ensure(16))) return rc;
  if ((rc = b->llmat.ensure((size_t)m * m + 16))) return rc;
  if ((rc = b->blist.ensure(sizeof(uint64_t) * (size_t)std::max<int64_t>(nbl, 1)))) return rc;
  if ((rc = b->blist_off.ensure(sizeof(int64_t) * (size_t)std::max(n, 1)))) return rc;
  if (n) {
    CK(cudaMemcpyAsync(b->jobs.p, dj.data(), sizeof(ksw2g_ll_job) * n, cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(b->blist_off.p, blo.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, c->st));
  }
  CK(cudaMemcpyAsync(b->llmat.p, mat, (size_t)m * m, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

int ll_run_on(ksw2g_batch *b, cudaStream_t st) {
  {
    const char *f = getenv("KSW2G_LL_KERNEL");  // "lane" or "dpx": pin one kernel family (tests)
    b->ll_force = f ? (strcmp(f, "lane") == 0 ? 1 : strcmp(f, "dpx") == 0 ? 2 : 0) : 0;
  }
  b->launches = 0;
  if (b->n == 0) return 0;
  CK(cudaMemsetAsync(b->counters.p, 0, 16, st));
  LLLaunch L{b->jobs.as<ksw2g_ll_job>(), b->n, b->arena.as<uint8_t>(), b->llmat.as<int8_t>(), b->ll_m, b->ll_gapo,
             b->ll_gape, b->res.as<ksw2g_ll_result>(), b->blist.as<uint64_t>(), b->blist_off.as<int64_t>(),
             b->counters.as<int>(), b->ll_qlen_max, b->ll_mat_max};
  CK(timed_begin(b, 0, st));
  CK(launch_ll(b->ll_size, b->ll_slen, L, 0, st, b->ll_force));
  CK(timed_end(b, st));
  ++b->launches;
  return 0;
}

int ll_run(ksw2g_ctx *c, ksw2g_batch *b) {
  CK(cudaSetDevice(c->device));
  return ll_run_on(b, c->st);
}

extern "C" int ksw2g_ll_prepare(ksw2g_ctx_t *c, int size, int m, const int8_t *mat, int gapo, int gape, int n_jobs,
                                const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
                                const uint8_t *tbuf, int64_t tbuf_len, ksw2g_batch_t **out) {
  if (!c || !out) return set_err(KSW2G_E_ARG, "null ctx/out");
  ksw2g_batch *b = new ksw2g_batch;
  int rc = ll_prepare_into(c, b, size, m, mat, gapo, gape, n_jobs, jobs, qbuf, qbuf_len, tbuf, tbuf_len);
  if (rc) {
    ksw2g_batch_free(b);
    return rc;
  }
  *out = b;
  return 0;
}

extern "C" int ksw2g_ll_fetch(ksw2g_ctx_t *c, ksw2g_batch_t *b, ksw2g_ll_result_t *res) {
  if (!c || !b || b->kind < 2) return set_err(KSW2G_E_ARG, "not an ll batch");
  CK(cudaSetDevice(c->device));
  if (b->n && res) CK(cudaMemcpyAsync(res, b->res.p, sizeof(ksw2g_ll_result) * b->n, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return 0;
}

// One-shot ksw_ll batches of more than kLLChunkJobs jobs run as chunks that rotate
// through the sub-contexts, so each chunk's uploads overlap the earlier chunks' DP.
static const int kLLChunkJobs = 262144;

static int ll_batch_chunked(ksw2g_ctx *c, int size, int m, const int8_t *mat, int gapo, int gape, int n,
                            const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
                            int64_t tbuf_len, ksw2g_ll_result_t *res) {
  const std::vector<int> cst = chunk_starts(n, kLLChunkJobs, true);
  const int nch = (int)cst.size() - 1;
  ksw2g_ctx *sc[kOneShotDepth];
  int rc;
  for (int i = 0; i < kOneShotDepth; ++i)
    if ((rc = sub_ctx(c, i, &sc[i]))) return rc;
  int pending[kOneShotDepth];
  std::fill(pending, pending + kOneShotDepth, -1);
  auto finish = [&](int s) -> int {
    const int ch = pending[s];
    if (ch < 0) return 0;
    pending[s] = -1;
    return ksw2g_ll_fetch(sc[s], sc[s]->scratch, res ? res + cst[ch] : nullptr);
  };
  for (int ch = 0; ch < nch && !rc; ++ch) {
    const int s = ch % kOneShotDepth;
    if ((rc = finish(s))) break;
    const int j0 = cst[ch], nj = cst[ch + 1] - j0;
    int64_t qlo = qbuf_len, qhi = 0, tlo = tbuf_len, thi = 0;
    for (int i = j0; i < j0 + nj; ++i) {
      const ksw2g_ll_job_t &J = jobs[i];
      if (J.qoff < 0 || J.toff < 0 || J.qlen < 0 || J.tlen < 0 || J.qoff + J.qlen > qbuf_len ||
          J.toff + J.tlen > tbuf_len) {
        rc = set_err(KSW2G_E_ARG, "ll job %d: sequence out of buffer bounds", i);
        break;
      }
      qlo = std::min(qlo, J.qoff), qhi = std::max<int64_t>(qhi, J.qoff + J.qlen);
      tlo = std::min(tlo, J.toff), thi = std::max<int64_t>(thi, J.toff + J.tlen);
    }
    if (rc) break;
    if (qlo > qhi) qlo = qhi = 0;
    if (tlo > thi) tlo = thi = 0;
    std::vector<ksw2g_ll_job_t> cj(jobs + j0, jobs + j0 + nj);
    for (auto &J : cj) J.qoff -= qlo, J.toff -= tlo;
    ksw2g_ctx *x = sc[s];
    if ((rc = ll_prepare_into(x, x->scratch, size, m, mat, gapo, gape, nj, cj.data(), qbuf + qlo, qhi - qlo,
                              tbuf + tlo, thi - tlo)))
      break;
    if ((rc = ll_run(x, x->scratch))) break;
    pending[s] = ch;
  }
  for (int ch = nch - kOneShotDepth; ch < nch && !rc; ++ch)
    if (ch >= 0) rc = finish(ch % kOneShotDepth);
  if (rc)
    for (int s = 0; s < kOneShotDepth; ++s) cudaStreamSynchronize(sc[s]->st);
  return rc;
}

extern "C" int ksw2g_ll_batch(ksw2g_ctx_t *c, int size, int m, const int8_t *mat, int gapo, int gape, int n_jobs,
                              const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
                              int64_t tbuf_len, ksw2g_ll_result_t *res) {
  if (!c) return set_err(KSW2G_E_ARG, "null ctx");
  CK(cudaSetDevice(c->device));
  if (n_jobs > kLLChunkJobs && jobs && mat)
    return ll_batch_chunked(c, size, m, mat, gapo, gape, n_jobs, jobs, qbuf, qbuf_len, tbuf, tbuf_len, res);
  if (!c->scratch) c->scratch = new ksw2g_batch;
  int rc = ll_prepare_into(c, c->scratch, size, m, mat, gapo, gape, n_jobs, jobs, qbuf, qbuf_len, tbuf, tbuf_len);
  if (rc) return rc;
  if ((rc = ll_run(c, c->scratch))) return rc;
  return ksw2g_ll_fetch(c, c->scratch, res);
}

// ---- per-call drop-ins of ksw_ll_qinit / ksw_ll_u8_core / ksw_ll_i16_core / ksw_ll_i16
// The "profile" returned by ksw_ll_qinit is one malloc() block holding the
// query and the matrix; the striped profile itself is built on the device
// by every core call.  Callers only pass the block back and free() it.
struct LLQ {
  uint32_t magic;
  int32_t size, qlen, m;
};
static const uint32_t kLLQMagic = 0x6b73776cu;

extern "C" void *ksw_ll_qinit(void *km, int size, int qlen, const uint8_t *query, int m, const int8_t *mat) {
  if (qlen < 0) qlen = 0;
  LLQ *h = (LLQ *)caller_malloc(km, sizeof(LLQ) + (size_t)m * m + qlen + 16);
  h->magic = kLLQMagic, h->size = size > 1 ? 2 : 1, h->qlen = qlen, h->m = m;
  memcpy((uint8_t *)(h + 1), mat, (size_t)m * m);
  if (qlen) memcpy((uint8_t *)(h + 1) + m * m, query, qlen);
  return h;
}

static ksw_llrst_t ll_one(void *q_, int tlen, const uint8_t *target, int gapo, int gape, int xtra, int want_size) {
  LLQ *h = (LLQ *)q_;
  if (!h || h->magic != kLLQMagic) {
    fprintf(stderr, "[ksw2gpu] fatal: ksw_ll core called with a block not made by ksw_ll_qinit\n");
    abort();
  }
  (void)want_size;  // the reference runs the core it is asked for, whatever size qinit used
  const int m = h->m, qlen = h->qlen, size = want_size;
  const int lanes = size == 1 ? 16 : 8;
  const int slen = (qlen + lanes - 1) / lanes;
  if (slen > ll_slen_cap(size, m)) {
    fprintf(stderr, "[ksw2gpu] fatal: ksw_ll query of %d nt exceeds the kernel limit\n", qlen);
    abort();
  }
  if (tlen < 0) tlen = 0;
  ksw2g_ctx *c = thread_ctx();
  const int64_t nbl = (xtra & KSW_LL_SUBO) ? tlen : 0;
  const size_t o_job = 16, o_blo = o_job + 32, o_res = o_blo + 16, o_mat = o_res + 32;
  const size_t o_arena = (o_mat + (size_t)m * m + 15) & ~(size_t)15;
  const size_t arena_bytes = slot_bytes(qlen) + slot_bytes(tlen);
  const size_t o_bl = (o_arena + arena_bytes + 15) & ~(size_t)15;
  const size_t total = o_bl + nbl * 8 + 16;
  if (c->one.ensure(total) || c->one_h.ensure(o_bl)) {
    fprintf(stderr, "[ksw2gpu] fatal: %s\n", tl_err.c_str());
    abort();
  }
  uint8_t *hb = (uint8_t *)c->one_h.p, *d = (uint8_t *)c->one.p;
  memset(hb, 0, o_arena);
  ksw2g_ll_job J{32, slot_bytes(qlen) + 32, qlen, tlen, xtra, 0};  // slot 0: the one result
  memcpy(hb + o_job, &J, sizeof J);
  memcpy(hb + o_mat, (uint8_t *)(h + 1), (size_t)m * m);
  memset(hb + o_arena, 0, arena_bytes);
  if (qlen) memcpy(hb + o_arena + J.qoff, (uint8_t *)(h + 1) + m * m, qlen);
  if (tlen) memcpy(hb + o_arena + J.toff, target, tlen);
  DIE_ON(cudaMemcpyAsync(d, hb, o_arena + arena_bytes, cudaMemcpyHostToDevice, c->st));
  int mat_max = m > 0 ? ((const int8_t *)(h + 1))[0] : 0;
  for (int a = 1; a < m * m; ++a) mat_max = std::max(mat_max, (int)((const int8_t *)(h + 1))[a]);
  LLLaunch L{(const ksw2g_ll_job *)(d + o_job), 1, d + o_arena, (const int8_t *)(d + o_mat), m, gapo, gape,
             (ksw2g_ll_result *)(d + o_res), (uint64_t *)(d + o_bl), (const int64_t *)(d + o_blo), (int *)d, qlen,
             mat_max};
  DIE_ON(launch_ll(size, slen < 1 ? 1 : slen, L, 1, c->st));
  DIE_ON(cudaMemcpyAsync(hb + o_res, d + o_res, sizeof(ksw2g_ll_result), cudaMemcpyDeviceToHost, c->st));
  DIE_ON(cudaStreamSynchronize(c->st));
  ksw2g_ll_result R;
  memcpy(&R, hb + o_res, sizeof R);
  ksw_llrst_t r;
  r.score = R.score, r.te = R.te, r.qe = R.qe, r.score2 = R.score2, r.te2 = R.te2;
  return r;
}

extern "C" ksw_llrst_t ksw_ll_u8_core(void *q, int tlen, const uint8_t *target, int gapo, int gape, int xtra) {
  return ll_one(q, tlen, target, gapo, gape, xtra, 1);
}
extern "C" ksw_llrst_t ksw_ll_i16_core(void *q, int tlen, const uint8_t *target, int gapo, int gape, int xtra) {
  return ll_one(q, tlen, target, gapo, gape, xtra, 2);
}
extern "C" int ksw_ll_i16(void *q, int tlen, const uint8_t *target, int gapo, int gape, int *qe, int *te) {
  ksw_llrst_t r = ll_one(q, tlen, target, gapo, gape, 0, 2);
  *qe = r.qe, *te = r.te;
  return r.score;
}
