// loadgen.cc -- open-loop load generator for the serving benchmark.
//
// One trace (request batches with arrival times, each made of up to one
// sub-request per job set) is replayed either against the serving engine
// (ksw2g_server_*) or against the plain per-call drop-in (ksw_extz2_sse,
// ksw_extd2_sse, ksw_ll_qinit + ksw_ll_{u8,i16}_core) driven by a pool of host
// worker threads taking jobs in arrival order, the way a kt_for loop in the
// aligner would call them.  Latency of a request batch is measured from its
// scheduled arrival to the moment its last result is in host memory, so a
// generator that falls behind is charged to the system under test.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <memory>
#include <thread>
#include <vector>

#include "../../include/ksw2.h"
#include "../../include/ksw2_gb300.h"

extern "C" {

typedef struct {
  int kind;  // 0 extz2, 1 extd2, 2 ll u8, 3 ll i16
  int m;
  const int8_t *mat;
  int q, e, q2, e2;  // extension gap costs
  int gapo, gape;    // ll gap costs
  int n_jobs;
  const void *jobs;  // ksw2g_job_t[] (kinds 0,1) or ksw2g_ll_job_t[] (kinds 2,3)
  const uint8_t *qbuf, *tbuf;
  void *res;  // out (server runs): results indexed like jobs
} lg_set_t;

typedef struct {
  int n_groups;
  const double *t_arrive;  // seconds from the start, non-decreasing
  const int *sub_start;    // n_groups + 1 prefix offsets into the sub-request arrays
  const int *sub_set, *sub_j0, *sub_n;
} lg_trace_t;

}  // extern "C"

namespace {

using clk = std::chrono::steady_clock;

double secs(clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); }

void wait_until(clk::time_point t) {
  for (;;) {
    const auto now = clk::now();
    if (now >= t) return;
    const double left = secs(now, t);
    if (left > 2e-4) std::this_thread::sleep_for(std::chrono::duration<double>(left - 1e-4));
    else std::this_thread::yield();
  }
}

uint64_t fnv(uint64_t h, const uint32_t *w, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    for (int b = 0; b < 4; ++b) h = (h ^ ((w[i] >> (8 * b)) & 0xffu)) * 0x100000001b3ull;
  return h;
}

// A sub-request's jobs re-based onto its own contiguous slice of the sequence buffers.
struct Prepared {
  std::vector<uint8_t> jobs;
  const uint8_t *q = nullptr, *t = nullptr;
  int64_t qlen = 0, tlen = 0, cig_cap = 0;
};

template <class J>
void rebase(const J *src, int n, const uint8_t *qb, const uint8_t *tb, Prepared &p) {
  int64_t q0 = INT64_MAX, q1 = 0, t0 = INT64_MAX, t1 = 0;
  for (int i = 0; i < n; ++i) {
    q0 = std::min(q0, src[i].qoff), q1 = std::max<int64_t>(q1, src[i].qoff + src[i].qlen);
    t0 = std::min(t0, src[i].toff), t1 = std::max<int64_t>(t1, src[i].toff + src[i].tlen);
  }
  if (n == 0) q0 = q1 = t0 = t1 = 0;
  p.jobs.resize(sizeof(J) * (size_t)n);
  J *d = (J *)p.jobs.data();
  for (int i = 0; i < n; ++i) {
    d[i] = src[i];
    d[i].qoff -= q0, d[i].toff -= t0;
    p.cig_cap += (int64_t)src[i].qlen + src[i].tlen + 1;
  }
  p.q = qb + q0, p.t = tb + t0, p.qlen = q1 - q0, p.tlen = t1 - t0;
}

}  // namespace

extern "C" uint64_t lg_cigar_hash(const ksw2g_ext_result_t *res, const uint32_t *cigar, int n) {
  uint64_t h = 0xcbf29ce484222325ull;
  for (int i = 0; i < n; ++i) h = fnv(h, cigar + res[i].cigar_off, res[i].n_cigar);
  return h;
}

// Replays the trace against a server.  Per sub-request: latency (scheduled
// arrival to results in host memory) and time queued in the engine, the CIGAR
// hash of its results, and its status.  Returns 0, or the first error.
extern "C" int lg_run_server(ksw2g_server_t *srv, const lg_set_t *sets, const lg_trace_t *tr, double *sub_lat_ms,
                             double *sub_queue_ms, uint64_t *sub_hash, int *sub_status, double *wall_s) {
  const int ns = tr->sub_start[tr->n_groups];
  std::vector<Prepared> prep(ns);
  for (int s = 0; s < ns; ++s) {
    const lg_set_t &S = sets[tr->sub_set[s]];
    if (S.kind <= 1)
      rebase((const ksw2g_job_t *)S.jobs + tr->sub_j0[s], tr->sub_n[s], S.qbuf, S.tbuf, prep[s]);
    else
      rebase((const ksw2g_ll_job_t *)S.jobs + tr->sub_j0[s], tr->sub_n[s], S.qbuf, S.tbuf, prep[s]);
  }
  std::vector<int64_t> ids(ns, 0);
  std::vector<double> lag(ns, 0);
  // Uninitialised result buffers: zero-filling a large CIGAR buffer would delay the submitter.
  std::vector<std::unique_ptr<uint8_t[]>> res(ns);
  std::vector<std::unique_ptr<uint32_t[]>> cig(ns);
  std::atomic<int> published{0};
  std::atomic<bool> failed{false};
  const auto t0 = clk::now() + std::chrono::milliseconds(20);
  double t_last = 0;

  std::thread waiter([&] {
    for (int s = 0; s < ns; ++s) {
      while (published.load(std::memory_order_acquire) <= s) {
        if (failed.load()) return;
        std::this_thread::sleep_for(std::chrono::microseconds(20));
      }
      double lat = 0, que = 0;
      int64_t used = 0;
      const int st = ids[s] > 0 ? ksw2g_server_wait(srv, ids[s], &lat, &que, &used) : (int)ids[s];
      sub_status[s] = st;
      sub_lat_ms[s] = lag[s] * 1e3 + lat, sub_queue_ms[s] = que;
      t_last = std::max(t_last, secs(t0, clk::now()));
      const lg_set_t &S = sets[tr->sub_set[s]];
      const int n = tr->sub_n[s];
      if (S.kind <= 1) {
        const ksw2g_ext_result_t *r = (const ksw2g_ext_result_t *)res[s].get();
        sub_hash[s] = st == 0 ? lg_cigar_hash(r, cig[s].get(), n) : 0;
        if (st == 0 && S.res) memcpy((ksw2g_ext_result_t *)S.res + tr->sub_j0[s], r, sizeof(*r) * (size_t)n);
      } else {
        sub_hash[s] = 0;
        if (st == 0 && S.res)
          memcpy((ksw2g_ll_result_t *)S.res + tr->sub_j0[s], res[s].get(), sizeof(ksw2g_ll_result_t) * (size_t)n);
      }
      res[s].reset();
      cig[s].reset();
    }
  });

  for (int g = 0; g < tr->n_groups; ++g) {
    const auto ta = t0 + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(tr->t_arrive[g]));
    wait_until(ta);
    for (int s = tr->sub_start[g]; s < tr->sub_start[g + 1]; ++s) {
      const lg_set_t &S = sets[tr->sub_set[s]];
      const Prepared &P = prep[s];
      const int n = tr->sub_n[s];
      int64_t id;
      lag[s] = secs(ta, clk::now());
      if (S.kind <= 1) {
        const int64_t cap = std::max<int64_t>(P.cig_cap, 1);
        res[s].reset(new uint8_t[sizeof(ksw2g_ext_result_t) * (size_t)std::max(n, 1)]);
        cig[s].reset(new uint32_t[(size_t)cap]);
        id = ksw2g_server_submit_ext(srv, S.kind, (int8_t)S.m, S.mat, (int8_t)S.q, (int8_t)S.e, (int8_t)S.q2,
                                     (int8_t)S.e2, n, (const ksw2g_job_t *)P.jobs.data(), P.q, P.qlen, P.t, P.tlen,
                                     (ksw2g_ext_result_t *)res[s].get(), cig[s].get(), cap);
      } else {
        res[s].reset(new uint8_t[sizeof(ksw2g_ll_result_t) * (size_t)std::max(n, 1)]);
        id = ksw2g_server_submit_ll(srv, S.kind == 2 ? 1 : 2, S.m, S.mat, S.gapo, S.gape, n,
                                    (const ksw2g_ll_job_t *)P.jobs.data(), P.q, P.qlen, P.t, P.tlen,
                                    (ksw2g_ll_result_t *)res[s].get());
      }
      ids[s] = id;
      published.store(s + 1, std::memory_order_release);
    }
  }
  waiter.join();
  *wall_s = t_last;
  for (int s = 0; s < ns; ++s)
    if (sub_status[s]) return sub_status[s];
  return 0;
}

// Replays the trace against the per-call drop-in with n_threads host workers.
// Workers take jobs in arrival order; a job is started no earlier than its
// request's arrival.  Jobs not started within deadline_s of the start are
// skipped and their requests reported with latency -1.  Returns the number of
// jobs completed; *wall_s is the time of the last completion.
extern "C" int64_t lg_run_percall(const lg_set_t *sets, const lg_trace_t *tr, int n_threads, double deadline_s,
                                  double *group_lat_ms, double *wall_s, int64_t *score_sum) {
  struct Item {
    int g, set, j;
  };
  std::vector<Item> items;
  for (int g = 0; g < tr->n_groups; ++g)
    for (int s = tr->sub_start[g]; s < tr->sub_start[g + 1]; ++s)
      for (int k = 0; k < tr->sub_n[s]; ++k) items.push_back(Item{g, tr->sub_set[s], tr->sub_j0[s] + k});
  std::vector<std::atomic<int>> left(tr->n_groups);
  std::vector<std::atomic<int64_t>> done_ns(tr->n_groups);
  for (int g = 0; g < tr->n_groups; ++g) {
    left[g].store(0);
    done_ns[g].store(0);
  }
  for (auto &it : items) left[it.g].fetch_add(1);
  std::atomic<int64_t> next{0}, n_done{0}, ssum{0};
  const auto t0 = clk::now() + std::chrono::milliseconds(20);
  auto worker = [&] {
    ksw_extz_t ez;
    memset(&ez, 0, sizeof ez);
    int64_t local = 0;
    for (;;) {
      const int64_t i = next.fetch_add(1);
      if (i >= (int64_t)items.size()) break;
      const Item &it = items[(size_t)i];
      const auto ta =
          t0 + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(tr->t_arrive[it.g]));
      wait_until(ta);
      if (secs(t0, clk::now()) > deadline_s) break;
      const lg_set_t &S = sets[it.set];
      if (S.kind <= 1) {
        const ksw2g_job_t &J = ((const ksw2g_job_t *)S.jobs)[it.j];
        if (S.kind == 0)
          ksw_extz2_sse(0, J.qlen, S.qbuf + J.qoff, J.tlen, S.tbuf + J.toff, (int8_t)S.m, S.mat, (int8_t)S.q,
                        (int8_t)S.e, J.w, J.zdrop, J.end_bonus, J.flag, &ez);
        else
          ksw_extd2_sse(0, J.qlen, S.qbuf + J.qoff, J.tlen, S.tbuf + J.toff, (int8_t)S.m, S.mat, (int8_t)S.q,
                        (int8_t)S.e, (int8_t)S.q2, (int8_t)S.e2, J.w, J.zdrop, J.end_bonus, J.flag, &ez);
        local += ez.score;
      } else {
        const ksw2g_ll_job_t &J = ((const ksw2g_ll_job_t *)S.jobs)[it.j];
        const int size = S.kind == 2 ? 1 : 2;
        void *qp = ksw_ll_qinit(0, size, J.qlen, S.qbuf + J.qoff, S.m, S.mat);
        const ksw_llrst_t r = size == 1 ? ksw_ll_u8_core(qp, J.tlen, S.tbuf + J.toff, S.gapo, S.gape, J.xtra)
                                        : ksw_ll_i16_core(qp, J.tlen, S.tbuf + J.toff, S.gapo, S.gape, J.xtra);
        free(qp);
        local += r.score;
      }
      const int64_t t = std::chrono::duration_cast<std::chrono::nanoseconds>(clk::now() - t0).count();
      int64_t prev = done_ns[it.g].load();
      while (prev < t && !done_ns[it.g].compare_exchange_weak(prev, t)) {
      }
      left[it.g].fetch_sub(1);
      n_done.fetch_add(1);
    }
    free(ez.cigar);
    ssum.fetch_add(local);
  };
  std::vector<std::thread> th;
  for (int k = 0; k < n_threads; ++k) th.emplace_back(worker);
  for (auto &t : th) t.join();
  double last = 0;
  for (int g = 0; g < tr->n_groups; ++g) {
    if (left[g].load() > 0) {
      group_lat_ms[g] = -1;
      continue;
    }
    const double td = done_ns[g].load() * 1e-9;
    last = std::max(last, td);
    group_lat_ms[g] = std::max(0.0, td - tr->t_arrive[g]) * 1e3;
  }
  *wall_s = last;
  *score_sum = ssum.load();
  return n_done.load();
}
