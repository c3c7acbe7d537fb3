// batch.h -- internal host-side structures of libksw2gpu.so (contexts, device
// buffers, prepared batches), shared by the C ABI (capi.cu) and the serving
// engine (server.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "../../include/ksw2_gb300.h"
#include "ksw2g.h"

namespace ksw2g {
int report_error(int code, const char *msg);
// Failure injection for host-side tests: when positive, the n-th next device buffer growth
// fails as if the allocator had no memory left (ksw2g_debug_fail_device_alloc).
bool take_injected_alloc_failure();
}

// ---------------------------------------------------------------- buffers
struct DevBuf {
  void *p = nullptr;
  size_t cap = 0;
  // With a stream, growth is stream-ordered (cudaMallocAsync / cudaFreeAsync from the
  // device's memory pool) and does not synchronise the device; otherwise cudaMalloc.
  cudaStream_t st = nullptr;
  cudaError_t alloc_(void **q, size_t c) { return st ? cudaMallocAsync(q, c, st) : cudaMalloc(q, c); }
  void free_(void *q) {
    if (st) cudaFreeAsync(q, st);
    else cudaFree(q);
  }
  int ensure(size_t n) {
    if (n <= cap) return 0;
    if (p) free_(p);
    p = nullptr, cap = 0;
    size_t c = n < 4096 ? 4096 : n + (st ? n / 2 : n / 8);
    if (ksw2g::take_injected_alloc_failure()) return ksw2g::report_error(KSW2G_E_NOMEM, "device allocation failed (injected)");
    if (alloc_(&p, c) != cudaSuccess) {
      cudaGetLastError();
      if (alloc_(&p, n) != cudaSuccess) {
        cudaGetLastError();
        p = nullptr;
        return ksw2g::report_error(KSW2G_E_NOMEM, "device allocation failed");
      }
      c = n;
    }
    cap = c;
    return 0;
  }
  void release() {
    if (p) free_(p);
    p = nullptr, cap = 0;
  }
  template <typename T>
  T *as() const { return (T *)p; }
};
struct PinBuf {
  void *p = nullptr;
  size_t cap = 0;
  int ensure(size_t n) {
    if (n <= cap) return 0;
    if (p) cudaFreeHost(p);
    p = nullptr, cap = 0;
    size_t c = n < 4096 ? 4096 : n + n / 2;
    if (cudaMallocHost(&p, c) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return ksw2g::report_error(KSW2G_E_NOMEM, "cudaMallocHost failed");
    }
    cap = c;
    return 0;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr, cap = 0;
  }
};

// ---------------------------------------------------------------- context
// Chunks of a one-shot call in flight at once.  Preparing a chunk on the host takes about as
// long as the device runs one, and with two in flight the host waited on the previous chunk
// of the same sub-context: 1,000,000 pairs of 100-300 nt took 150.7 ms end to end in chunks of
// 32,768 two deep, 143.2 ms three deep and 136.7 ms in chunks of 16,384 three deep (the device
// alone: 133.6 ms).
static const int kOneShotDepth = 3;

struct ksw2g_ctx {
  int device = 0;
  cudaStream_t st = nullptr;
  int nsm = 0;
  int64_t tb_budget = (int64_t)16 << 30;
  // Waves are cut at tb_budget / wave_div.  With 2, two waves fit the budget at
  // once, and ksw2g_batch_run alternates them between st and aux so that one
  // wave's tail overlaps the next wave's start.
  int wave_div = 2;
  cudaStream_t aux = nullptr;
  DevBuf tb_pool;       // traceback rows of the running wave
  DevBuf one;           // per-call drop-in scratch (device)
  PinBuf one_h;         // per-call drop-in staging (pinned)
  DevBuf rs_q, rs_t, rs_meta, rs_res, rs_hist;  // mate-rescue prefilter: reads, windows, records, votes
  PinBuf rs_h;                                  // mate-rescue staging (pinned)
  int oneshot_launches = 0;                     // kernels the last one-shot extension call launched
  ksw2g_batch *rs_ll[6 * 7] = {};               // mate-rescue ksw_ll batches, one per (size, methylation,
                                                // query-segment class)
  ksw2g_batch *rs_ext[3] = {};                  // mate-rescue extz2 batches, one per methylation mode
  DevBuf rs_rq, rs_rmeta;                       // reversed read prefixes on the device and their records
  int rs_launches = 0;                          // kernels the last rescue call launched
  double rs_ms[3] = {0, 0, 0};                  // its stages' wall time: prefilter, ksw_ll, extz2
  double rs_dev_ms[2] = {0, 0};                 // device time of its ksw_ll and extz2 kernels
  double ch_ms[6] = {};      // the last ksw2g_align_chains call's stages (host wall time)
  int64_t ch_n[4] = {};      // its hits, first-pass jobs, second-pass jobs, inversion checks
  ksw2g_batch *scratch = nullptr;  // reused by the one-shot batch calls
  // sub-contexts (own stream and traceback pool, half the budget each) that the
  // one-shot calls rotate their chunks through, so the host prepares the next chunks
  // while the device runs the earlier ones
  ksw2g_ctx *sub[kOneShotDepth] = {};
};

// ---------------------------------------------------------------- batches
struct Bin {
  int mode, shape;
  int64_t order_off;
  int count;
  double cost;  // rough device cycles (bin_cost in capi.cu)
  int sub;      // stream of the wave it runs on: 0 the wave's own, s > 0 side stream s - 1
};
// Bins of one wave run at once on the wave's stream and up to kSideStreams side streams,
// which fork from it at the wave's start and join it before the wave's backtrack.
constexpr int kSideStreams = 3;
struct Wave {
  int w0, w1;            // range of the longest-first job order (batch->sorted)
  int64_t tb_bytes;
  bool any_cig;
  std::vector<Bin> bins;
};

struct ksw2g_batch {
  int kind = 0;          // 0 extz2, 1 extd2, 2 ll u8, 3 ll i16
  int n = 0;
  ksw2g_ext_params P;
  int ll_m = 0, ll_gapo = 0, ll_gape = 0, ll_size = 1, ll_slen = 0, ll_qlen_max = 0, ll_mat_max = 0, ll_force = 0;
  DevBuf raw, rawmeta, arena, jobs, order, sorted, tb_off, res, bts, cigar, counters, llmat, blist, blist_off;
  DevBuf refmeta;         // per-job reference windows of a batch whose targets come from the device reference
  DevBuf wide;            // block scratch of wide-band jobs: two halves of wide_blocks x wide_stride
  int64_t wide_stride = 0;
  int wide_blocks = 0;
  int64_t cigar_cap = 0;
  int n_counters = 0;
  std::vector<Wave> waves;
  int launches = 0;
  int64_t total_cells_hint = 0;
  // optional per-launch timing: an event pair around every kernel of a run
  bool timing = false;
  std::vector<cudaEvent_t> tev;  // 2 per timed launch
  std::vector<int> tkind;        // 0 DP kernel, 1 backtrack kernel, per timed launch
  int n_timed = 0;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  // two-stream runs
  // side streams of multi-bin waves and their fork and join events, one set per stream
  // parity of a two-stream run; created on first use
  cudaStream_t side[2][kSideStreams] = {};
  cudaEvent_t ev_wfork[2] = {}, ev_wjoin[2][kSideStreams] = {};
};

// Destroy the batch's events and side streams (work already enqueued on them completes).
inline void batch_release_streams(ksw2g_batch *b) {
  for (cudaEvent_t e : b->tev) cudaEventDestroy(e);
  b->tev.clear();
  b->n_timed = 0;
  for (cudaEvent_t *e : {&b->ev_fork, &b->ev_join, &b->ev_wfork[0], &b->ev_wfork[1]})
    if (*e) cudaEventDestroy(*e), *e = nullptr;
  for (int p = 0; p < 2; ++p)
    for (int i = 0; i < kSideStreams; ++i) {
      if (b->ev_wjoin[p][i]) cudaEventDestroy(b->ev_wjoin[p][i]), b->ev_wjoin[p][i] = nullptr;
      if (b->side[p][i]) cudaStreamDestroy(b->side[p][i]), b->side[p][i] = nullptr;
    }
}


// Make every device buffer of the batch grow in stream order on st.
inline void batch_bind_stream(ksw2g_batch *b, cudaStream_t st) {
  for (DevBuf *d : {&b->raw, &b->rawmeta, &b->arena, &b->jobs, &b->order, &b->sorted, &b->tb_off, &b->res, &b->bts,
                    &b->cigar, &b->counters, &b->llmat, &b->blist, &b->blist_off, &b->wide, &b->refmeta})
    d->st = st;
}

// A run of jobs whose qoff/toff index their own query and target buffers.  A
// batch may be prepared from several segments (the serving engine merges the
// requests of one scoring scheme this way); job offsets are rebased onto the
// concatenation of the segments' buffers.
struct SeqSeg {
  const void *jobs;  // ksw2g_job_t[] or ksw2g_ll_job_t[]
  int n;
  const uint8_t *qbuf;
  int64_t qlen;
  const uint8_t *tbuf;
  int64_t tlen;
  // device copy of qbuf (qlen bytes) already on the context's stream: the queries are packed
  // from it and qbuf is not read (single-segment batches only)
  const uint8_t *qdev = nullptr;
};
// Targets read from a device-resident reference instead of host buffers: job
// k's target is the window [toff, toff+tlen) of contig tid[k], decoded with
// flags[k] (KSW2G_REF_*; flags may be null).  Used with a single segment whose
// tbuf is unused.
struct ksw2g_ref;
struct RefTargets {
  const ksw2g_ref *ref;
  const int32_t *tid;
  const int32_t *flags;
};
int ext_prepare_segs(ksw2g_ctx *c, ksw2g_batch *b, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e,
                     int8_t q2, int8_t e2, int nseg, const SeqSeg *segs, const RefTargets *rt = nullptr);
int ll_prepare_segs(ksw2g_ctx *c, ksw2g_batch *b, int size, int m, const int8_t *mat, int gapo, int gape, int nseg,
                    const SeqSeg *segs, const RefTargets *rt = nullptr);
namespace ksw2g {
cudaError_t launch_ref_gather(int n, const int32_t *tid, const int64_t *st, const int32_t *len, const int32_t *flags,
                              const int64_t *dst_off, uint8_t *arena, const ksw2g_ref *R, cudaStream_t stream);
int ref_check_window(const ksw2g_ref *R, int64_t tid, int64_t st, int64_t len);
int64_t ref_ctg_len(const ksw2g_ref *R, int64_t tid);  // -1 for a bad contig id
}  // namespace ksw2g

// Upload + pack the sequences and build the device job table and the wave plan
// (synchronous on c->st, so the host buffers may be reused on return).
int ext_prepare_into(ksw2g_ctx *c, ksw2g_batch *b, int dual, int8_t m, const int8_t *mat, int8_t q, int8_t e,
                     int8_t q2, int8_t e2, int n, const ksw2g_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len,
                     const uint8_t *tbuf, int64_t tbuf_len);
int ll_prepare_into(ksw2g_ctx *c, ksw2g_batch *b, int size, int m, const int8_t *mat, int gapo, int gape, int n,
                    const ksw2g_ll_job_t *jobs, const uint8_t *qbuf, int64_t qbuf_len, const uint8_t *tbuf,
                    int64_t tbuf_len);
// Enqueue the DP (+ backtrack) of a prepared extension batch on st, with tb (tb_cap bytes)
// holding the traceback rows of one wave at a time.
int ext_run_on(ksw2g_batch *b, cudaStream_t st, uint8_t *tb, int64_t tb_cap);
// The same with the waves alternating between s0 (region tb0) and s1 (region
// tb1); s1 joins s0's order at the start and s0 waits for s1 at the end.  With
// s1 null, or fewer than two waves, everything runs on s0 in tb0.
int ext_run_on2(ksw2g_batch *b, cudaStream_t s0, cudaStream_t s1, uint8_t *tb0, uint8_t *tb1, int64_t tb_cap);
// Largest wave of a prepared extension batch (bytes, at least 16).
int64_t ext_max_wave(const ksw2g_batch *b);
int ll_run_on(ksw2g_batch *b, cudaStream_t st);
