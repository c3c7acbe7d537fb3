"""Serving benchmark: the mixed extension / rescue workload replayed open-loop.

Request batches arrive as a Poisson process; each carries 1-4096 jobs (log-uniform) split
70% short extz2 (150 nt, w=25), 20% long extd2 (log-normal 1-10 kb, w=500) and 10% ksw_ll
i16 rescue jobs (150 nt vs 500-1000 nt), one sub-request per job kind.  The same trace is
replayed against

  * the serving engine (ksw2g_server_*: continuous batching, traceback admission against a
    fixed HBM budget, several streams), and
  * the plain per-call drop-in (ksw_extz2_sse / ksw_extd2_sse / ksw_ll_*), called by a pool
    of host threads in arrival order, one job per call,

by the C load generator in libksw2loadgen.so.  Latency is measured from a request's
scheduled arrival to its last result in host memory.  Arrival rates are fractions of the
engine's measured peak (all requests queued at time 0).

    python -m minibwa_gb300.serving [--duration 3] [--fracs 0.1,0.5,0.8,1.0] [--percall-threads 16]
"""
import argparse
import ctypes as C
import json
import os
import sys

import numpy as np

from . import synth
from .lib import EXT_RESULT, LL_RESULT, load_library

_PKG = os.path.dirname(os.path.abspath(__file__))

SPEC_LONG_1_10KB = dict(lognorm_median=3162.0, lognorm_sigma=0.58, clip_lo=1000, clip_hi=10000, sub_rate=0.005,
                        indel_rate=0.003, indel_p=0.5, indel_max=5, flank=100)
MIX = (0.7, 0.2, 0.1)  # extz2 short, extd2 long, ll rescue
MAX_REQ = 4096


class LGSet(C.Structure):
    _fields_ = [("kind", C.c_int), ("m", C.c_int), ("mat", C.c_void_p), ("q", C.c_int), ("e", C.c_int),
                ("q2", C.c_int), ("e2", C.c_int), ("gapo", C.c_int), ("gape", C.c_int), ("n_jobs", C.c_int),
                ("jobs", C.c_void_p), ("qbuf", C.c_void_p), ("tbuf", C.c_void_p), ("res", C.c_void_p)]


class LGTrace(C.Structure):
    _fields_ = [("n_groups", C.c_int), ("t_arrive", C.c_void_p), ("sub_start", C.c_void_p), ("sub_set", C.c_void_p),
                ("sub_j0", C.c_void_p), ("sub_n", C.c_void_p)]


_LG = None


def _lg():
    global _LG
    if _LG is None:
        load_library()
        p = os.path.join(_PKG, "libksw2loadgen.so")
        if not os.path.exists(p):
            raise RuntimeError("libksw2loadgen.so missing: run `python -m minibwa_gb300.build`")
        L = C.CDLL(p)
        vp, dp = C.c_void_p, C.POINTER(C.c_double)
        L.lg_run_server.restype = C.c_int
        L.lg_run_server.argtypes = [vp, vp, C.POINTER(LGTrace), vp, vp, vp, vp, dp]
        L.lg_run_percall.restype = C.c_int64
        L.lg_run_percall.argtypes = [vp, C.POINTER(LGTrace), C.c_int, C.c_double, vp, dp, C.POINTER(C.c_int64)]
        L.lg_cigar_hash.restype = C.c_uint64
        L.lg_cigar_hash.argtypes = [vp, vp, C.c_int]
        _LG = L
    return _LG


class JobSets:
    """The three job pools of the mixed workload; requests take contiguous ranges of them."""

    def __init__(self, n_short=200000, n_long=20000, n_ll=40000, seed=synth.SEED + 40):
        self.short = synth.ext_pairs(n_short, synth.SPEC_SHORT, 25, 100, 10, dual=False, seed=seed,
                                     name="extz2-150nt-w25")
        self.long = synth.ext_pairs(n_long, SPEC_LONG_1_10KB, 500, 400, -1, dual=True, seed=seed + 1,
                                    name="extd2-lognorm-1-10kb-w500")
        self.ll = synth.ll_jobs(n_ll, seed=seed + 2, name="ll-i16-150vs500-1000")
        self.pools = [self.short, self.long, self.ll]
        self.res = [np.zeros(len(self.short), EXT_RESULT), np.zeros(len(self.long), EXT_RESULT),
                    np.zeros(len(self.ll), LL_RESULT)]
        self._mk()

    def _mk(self):
        arr = (LGSet * 3)()
        for k, (p, r) in enumerate(zip(self.pools, self.res)):
            s = arr[k]
            if k < 2:
                s.kind, s.q, s.e, s.q2, s.e2 = int(p.dual), p.q, p.e, p.q2, p.e2
            else:
                s.kind, s.gapo, s.gape = 3 if p.size == 2 else 2, p.gapo, p.gape
            s.m, s.mat, s.n_jobs = 5, p.mat.ctypes.data, len(p)
            s.jobs, s.qbuf, s.tbuf, s.res = p.jobs.ctypes.data, p.qbuf.ctypes.data, p.tbuf.ctypes.data, r.ctypes.data
        self.c = arr

    def clear_results(self):
        for r in self.res:
            r[...] = 0


class Trace:
    """Request batches: arrival times and, per batch, up to three sub-requests."""

    def __init__(self, sets, n_jobs_target, rate_jobs_s, seed=7, sizes=None):
        rng = np.random.default_rng(seed)
        pools = [len(p) for p in sets.pools]
        cursor = [0, 0, 0]
        t, ta, start, sset, sj0, sn = 0.0, [], [0], [], [], []
        mean_req = (MAX_REQ - 1) / np.log(MAX_REQ)
        total = 0
        while total < n_jobs_target:
            n = int(sizes.pop(0)) if sizes else int(min(MAX_REQ, np.floor(np.exp(rng.uniform(0, np.log(MAX_REQ + 1))))))
            n = max(n, 1)
            parts = rng.multinomial(n, MIX)
            if rate_jobs_s is not None:
                t += rng.exponential(mean_req / rate_jobs_s)
            ta.append(t)
            for k in range(3):
                c = int(parts[k])
                if c == 0:
                    continue
                if cursor[k] + c > pools[k]:
                    cursor[k] = 0
                sset.append(k), sj0.append(cursor[k]), sn.append(c)
                cursor[k] += c
            start.append(len(sset))
            total += n
        self.t = np.array(ta, np.float64)
        self.start = np.array(start, np.int32)
        self.set = np.array(sset, np.int32)
        self.j0 = np.array(sj0, np.int32)
        self.n = np.array(sn, np.int32)
        self.n_jobs = int(self.n.sum())
        self.c = LGTrace(len(self.t), self.t.ctypes.data, self.start.ctypes.data, self.set.ctypes.data,
                         self.j0.ctypes.data, self.n.ctypes.data)

    def group_of_sub(self):
        return np.repeat(np.arange(len(self.t)), np.diff(self.start))


def run_server(server, sets, trace):
    """Replays the trace against a Server.  Returns per-request latency (ms), the run's wall time,
    per-sub-request queue times and CIGAR hashes."""
    ns = len(trace.set)
    lat, que = np.zeros(ns), np.zeros(ns)
    h, st = np.zeros(ns, np.uint64), np.zeros(ns, np.int32)
    wall = C.c_double()
    rc = _lg().lg_run_server(server.h, C.addressof(sets.c), C.byref(trace.c), lat.ctypes.data, que.ctypes.data,
                             h.ctypes.data, st.ctypes.data, C.byref(wall))
    if rc != 0:
        raise RuntimeError(f"serving run failed: status {rc}")
    g = trace.group_of_sub()
    glat = np.zeros(len(trace.t))
    np.maximum.at(glat, g, lat)
    return dict(lat=glat, wall=wall.value, queue=que, hash=h)


def run_percall(sets, trace, threads, deadline_s):
    glat = np.zeros(len(trace.t))
    wall, ssum = C.c_double(), C.c_int64()
    done = _lg().lg_run_percall(C.addressof(sets.c), C.byref(trace.c), threads, deadline_s, glat.ctypes.data,
                                C.byref(wall), C.byref(ssum))
    return dict(lat=glat, wall=wall.value, done=int(done))


def check_against_batches(ctx, sets, trace, sub_hash):
    """Every job the trace touched must equal the same job run alone in a plain batch; every
    extension sub-request's CIGAR hash must equal the hash of the batch CIGARs of its jobs."""
    L = _lg()
    bad = 0
    for k, p in enumerate(sets.pools):
        used = np.zeros(len(p), bool)
        for j0, n in zip(trace.j0[trace.set == k], trace.n[trace.set == k]):
            used[j0:j0 + n] = True
        if k < 2:
            ref, cig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
            for f in ("score", "max", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "zdropped", "reach_end",
                      "n_cigar"):
                bad += int((sets.res[k][f][used] != ref[f][used]).sum())
            for s in np.nonzero(trace.set == k)[0]:
                j0, n = int(trace.j0[s]), int(trace.n[s])
                hh = L.lg_cigar_hash(ref[j0:].ctypes.data, cig.ctypes.data, n)
                bad += int(hh != int(sub_hash[s]))
        else:
            ref = ctx.ll_batch(p.size, 5, p.mat, p.gapo, p.gape, p.jobs, p.qbuf, p.tbuf)
            for f in ("score", "te", "qe", "score2", "te2"):
                bad += int((sets.res[k][f][used] != ref[f][used]).sum())
    return bad


def pct(a, q):
    a = a[a >= 0]
    return float(np.percentile(a, q)) if len(a) else None


def sweep(duration=3.0, fracs=(0.1, 0.25, 0.5, 0.8, 1.0), slots=8, budget=40 << 30, percall_threads=16,
          percall_deadline=4.0, check=True, log=sys.stderr, max_merge=None, percall_peak_jobs=20000,
          percall_peak_only=False):
    from .lib import Context, Server
    sets = JobSets()
    srv = Server(0, slots=slots, tb_budget=budget, max_merge=max_merge)
    warm = Trace(sets, 20000, None, seed=1)
    run_server(srv, sets, warm)
    # peak: everything queued at time 0
    peak_tr = Trace(sets, 300000, None, seed=2)
    pk = run_server(srv, sets, peak_tr)
    peak = peak_tr.n_jobs / pk["wall"]
    print(f"peak: {peak_tr.n_jobs} jobs in {len(peak_tr.t)} requests, {pk['wall']:.3f} s, {peak:.0f} jobs/s",
          file=log, flush=True)
    out = dict(peak_jobs_s=peak, peak_requests=len(peak_tr.t), rates=[])
    bad = 0
    for fr in fracs:
        rate = fr * peak
        tr = Trace(sets, int(rate * duration), rate, seed=int(fr * 1000) + 3)
        sets.clear_results()
        r = run_server(srv, sets, tr)
        if check:
            ctx = Context(0)
            bad += check_against_batches(ctx, sets, tr, r["hash"])
            ctx.close()
        row = dict(frac=fr, offered_jobs_s=rate, requests=len(tr.t), jobs=tr.n_jobs,
                   served_jobs_s=tr.n_jobs / r["wall"], p50_ms=pct(r["lat"], 50), p99_ms=pct(r["lat"], 99),
                   max_ms=float(r["lat"].max()))
        print(json.dumps(row), file=log, flush=True)
        out["rates"].append(row)
    out["mismatches_vs_alone"] = bad
    out["server_stats"] = srv.stats()
    srv.close()
    # per-call drop-in: closed-loop peak, then the same open-loop rates under a deadline
    if percall_threads > 0:
        tr = Trace(sets, percall_peak_jobs, None, seed=5)
        pc = run_percall(sets, tr, percall_threads, percall_deadline * 4)
        out["percall_peak_jobs_s"] = pc["done"] / pc["wall"] if pc["wall"] > 0 else None
        out["percall_threads"] = percall_threads
        print(f"per-call peak: {pc['done']} jobs in {pc['wall']:.3f} s", file=log, flush=True)
        out["percall_rates"] = []
        for fr in (() if percall_peak_only else fracs):
            rate = fr * peak
            tr = Trace(sets, int(rate * min(duration, 1.0)), rate, seed=int(fr * 1000) + 3)
            pc = run_percall(sets, tr, percall_threads, percall_deadline)
            fin = pc["lat"] >= 0
            row = dict(frac=fr, offered_jobs_s=rate, requests=len(tr.t), completed_requests=int(fin.sum()),
                       jobs=tr.n_jobs, done_jobs=pc["done"], served_jobs_s=pc["done"] / max(pc["wall"], 1e-9),
                       p50_ms=pct(pc["lat"], 50), p99_ms=pct(pc["lat"], 99))
            print(json.dumps(row), file=log, flush=True)
            out["percall_rates"].append(row)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--duration", type=float, default=3.0)
    ap.add_argument("--fracs", default="0.1,0.25,0.5,0.8,0.9,1.0")
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--budget-gb", type=float, default=40)
    ap.add_argument("--percall-threads", type=int, default=16)
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--max-merge", type=int, default=None, help="jobs per merged launch (1: no merging)")
    a = ap.parse_args(argv)
    out = sweep(a.duration, tuple(float(x) for x in a.fracs.split(",")), a.slots, int(a.budget_gb * (1 << 30)),
                a.percall_threads, check=not a.no_check, max_merge=a.max_merge)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
