"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is named for this path; these generators stand in for real
reads.  Config numbering follows the benchmark definition:

  0  extz2, 150 nt, 0.1% N, 1% subst, 0.2% indels (1-3), +30 flank, w=25   (20,000 pairs)
  1  extd2, 100-300 nt, 2% subst, 0.5% indels (geom p=.5, <=20), +50 flank,
     1% with a 200-nt junk query suffix, w=100                             (1,000,000 pairs)
  2  mixed: long extd2 (log-normal median 2 kb, 500 nt-30 kb, 0.5% subst,
     0.3% indels 1-5, +100 flank, w=500, zdrop=400) + short extz2 as config 0
  3  ksw_ll i16 rescue: 150 nt vs 500-1000 nt, 30% with a planted copy
     (2% subst, 0.3% indels)                                               (2,000,000 jobs)
Scoring everywhere: match +2, mismatch -8, N -1 (ksw_gen_nt4_mat(2,8,0,1)), q=12, e=2
(q2=24, e2=1 for extd2).  RNG: splitmix64, seed 11.
"""
import ctypes as C
import os

import numpy as np

from .lib import EXT_JOB, LL_JOB, RESCUE_JOB, KSW_EZ_EXTZ_ONLY, gen_nt4_mat

_PKG = os.path.dirname(os.path.abspath(__file__))
SEED = 11


class ExtSpec(C.Structure):
    _fields_ = [("qlen_lo", C.c_int), ("qlen_hi", C.c_int), ("lognorm_median", C.c_double),
                ("lognorm_sigma", C.c_double), ("clip_lo", C.c_int), ("clip_hi", C.c_int),
                ("n_rate", C.c_double), ("sub_rate", C.c_double), ("indel_rate", C.c_double),
                ("indel_p", C.c_double), ("indel_max", C.c_int), ("flank", C.c_int),
                ("junk_frac", C.c_double), ("junk_len", C.c_int)]


class RescueSpec(C.Structure):
    _fields_ = [("qlen_lo", C.c_int), ("qlen_hi", C.c_int), ("lo", C.c_int), ("hi", C.c_int),
                ("p_random", C.c_double), ("p_meth", C.c_double), ("sub_rate", C.c_double),
                ("indel_rate", C.c_double), ("min_sc_hi", C.c_int)]


class LLSpec(C.Structure):
    _fields_ = [("qlen", C.c_int), ("tlen_lo", C.c_int), ("tlen_hi", C.c_int), ("plant_frac", C.c_double),
                ("sub_rate", C.c_double), ("indel_rate", C.c_double), ("indel_p", C.c_double),
                ("indel_max", C.c_int)]


_L = None


def _lib():
    global _L
    if _L is None:
        p = os.path.join(_PKG, "libksw2synth.so")
        if not os.path.exists(p):
            raise RuntimeError("libksw2synth.so missing: run `python -m minibwa_gb300.build`")
        _L = C.CDLL(p)
        args = [C.c_void_p, C.c_uint64, C.c_int] + [C.c_void_p] * 6 + [C.c_int64, C.c_void_p, C.c_int64,
                                                                          C.c_void_p, C.c_void_p]
        for f in (_L.synth_ext, _L.synth_ll):
            f.restype = C.c_int
        _L.synth_ext.argtypes = [C.POINTER(ExtSpec), C.c_uint64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        _L.synth_rescue.restype = C.c_int
        _L.synth_rescue.argtypes = [C.POINTER(RescueSpec), C.c_uint64, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
        _L.synth_ll.argtypes = [C.POINTER(LLSpec), C.c_uint64, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        del args
    return _L


SPEC_SHORT = dict(qlen_lo=150, qlen_hi=150, n_rate=0.001, sub_rate=0.01, indel_rate=0.002, indel_p=0.5,
                  indel_max=3, flank=30)
SPEC_MID = dict(qlen_lo=100, qlen_hi=300, sub_rate=0.02, indel_rate=0.005, indel_p=0.5, indel_max=20, flank=50,
                junk_frac=0.01, junk_len=200)
SPEC_LONG = dict(lognorm_median=2000.0, lognorm_sigma=0.8, clip_lo=500, clip_hi=30000, sub_rate=0.005,
                 indel_rate=0.003, indel_p=0.5, indel_max=5, flank=100)


class Pairs:
    """A set of extension jobs with back-to-back sequence buffers."""

    def __init__(self, jobs, qbuf, tbuf, dual, mat, q, e, q2, e2, name):
        self.jobs, self.qbuf, self.tbuf = jobs, qbuf, tbuf
        self.dual, self.mat, self.q, self.e, self.q2, self.e2 = dual, mat, q, e, q2, e2
        self.name = name

    def __len__(self):
        return len(self.jobs)

    def subset(self, idx):
        """Jobs idx re-packed into compact buffers."""
        idx = np.asarray(idx)
        j = self.jobs[idx].copy()
        qparts = [self.qbuf[o:o + n] for o, n in zip(j["qoff"], j["qlen"])]
        tparts = [self.tbuf[o:o + n] for o, n in zip(j["toff"], j["tlen"])]
        j["qoff"] = np.concatenate([[0], np.cumsum([len(x) for x in qparts])[:-1]]) if len(qparts) else []
        j["toff"] = np.concatenate([[0], np.cumsum([len(x) for x in tparts])[:-1]]) if len(tparts) else []
        qb = np.concatenate(qparts) if qparts else np.zeros(0, np.uint8)
        tb = np.concatenate(tparts) if tparts else np.zeros(0, np.uint8)
        return Pairs(j, qb, tb, self.dual, self.mat, self.q, self.e, self.q2, self.e2, self.name)

    def query(self, i):
        j = self.jobs[i]
        return self.qbuf[j["qoff"]:j["qoff"] + j["qlen"]]

    def target(self, i):
        j = self.jobs[i]
        return self.tbuf[j["toff"]:j["toff"] + j["tlen"]]


def ext_pairs(n, spec, w, zdrop, end_bonus, flag=KSW_EZ_EXTZ_ONLY, dual=False, seed=SEED, name="pairs"):
    s = ExtSpec(**{**dict(qlen_lo=0, qlen_hi=0, lognorm_median=0.0, lognorm_sigma=0.0, clip_lo=0, clip_hi=0,
                          n_rate=0.0, sub_rate=0.0, indel_rate=0.0, indel_p=0.5, indel_max=1, flank=0,
                          junk_frac=0.0, junk_len=0), **spec})
    qmax = max(s.qlen_hi, s.clip_hi) + s.junk_len
    qcap = int(n) * qmax + 64
    tcap = int(n) * (int(qmax * (1 + 2 * s.indel_rate * s.indel_max)) + s.flank + 64) + 64
    jobs = np.zeros(n, EXT_JOB)
    qoff, toff = np.zeros(n, np.int64), np.zeros(n, np.int64)
    qlen, tlen = np.zeros(n, np.int32), np.zeros(n, np.int32)
    qbuf, tbuf = np.zeros(qcap, np.uint8), np.zeros(tcap, np.uint8)
    qu, tu = C.c_int64(), C.c_int64()
    rc = _lib().synth_ext(C.byref(s), seed, n, qoff.ctypes.data, qlen.ctypes.data, toff.ctypes.data,
                          tlen.ctypes.data, qbuf.ctypes.data, qcap, tbuf.ctypes.data, tcap, C.byref(qu), C.byref(tu))
    if rc != 0:
        raise RuntimeError("synth_ext: buffer capacity exceeded")
    jobs["qoff"], jobs["toff"], jobs["qlen"], jobs["tlen"] = qoff, toff, qlen, tlen
    jobs["w"], jobs["zdrop"], jobs["end_bonus"], jobs["flag"] = w, zdrop, end_bonus, flag
    mat = gen_nt4_mat(2, 8, 0, 1)
    q2, e2 = (24, 1) if dual else (12, 2)
    return Pairs(jobs, qbuf[:qu.value].copy(), tbuf[:tu.value].copy(), dual, mat, 12, 2, q2, e2, name)


def config0(n=20000, seed=SEED):
    return ext_pairs(n, SPEC_SHORT, 25, 100, 10, KSW_EZ_EXTZ_ONLY, False, seed, "cfg0-extz2-150nt-w25")


def config1(n=1000000, seed=SEED + 1):
    return ext_pairs(n, SPEC_MID, 100, 100, 10, KSW_EZ_EXTZ_ONLY, True, seed, "cfg1-extd2-100-300nt-w100")


def config2_long(n=200000, seed=SEED + 2):
    return ext_pairs(n, SPEC_LONG, 500, 400, -1, KSW_EZ_EXTZ_ONLY, True, seed, "cfg2-extd2-lognorm2kb-w500")


def config2_short(n=1000000, seed=SEED + 3):
    return ext_pairs(n, SPEC_SHORT, 25, 100, 10, KSW_EZ_EXTZ_ONLY, False, seed, "cfg2-extz2-150nt-w25")


class Rescue:
    """A set of ksw_ll jobs."""

    def __init__(self, jobs, qbuf, tbuf, size, mat, gapo, gape, name):
        self.jobs, self.qbuf, self.tbuf = jobs, qbuf, tbuf
        self.size, self.mat, self.gapo, self.gape, self.name = size, mat, gapo, gape, name

    def __len__(self):
        return len(self.jobs)

    def subset(self, idx):
        idx = np.asarray(idx)
        j = self.jobs[idx].copy()
        qparts = [self.qbuf[o:o + n] for o, n in zip(j["qoff"], j["qlen"])]
        tparts = [self.tbuf[o:o + n] for o, n in zip(j["toff"], j["tlen"])]
        j["qoff"] = np.concatenate([[0], np.cumsum([len(x) for x in qparts])[:-1]])
        j["toff"] = np.concatenate([[0], np.cumsum([len(x) for x in tparts])[:-1]])
        return Rescue(j, np.concatenate(qparts), np.concatenate(tparts), self.size, self.mat, self.gapo,
                      self.gape, self.name)


def ll_jobs(n, qlen=150, tlen_lo=500, tlen_hi=1000, plant=0.3, size=2, xtra=0, mat=None, gapo=12, gape=2,
            seed=SEED + 4, name="rescue"):
    s = LLSpec(qlen=qlen, tlen_lo=tlen_lo, tlen_hi=tlen_hi, plant_frac=plant, sub_rate=0.02, indel_rate=0.003,
               indel_p=0.5, indel_max=3)
    qcap, tcap = int(n) * qlen + 64, int(n) * tlen_hi + 64
    qoff, toff = np.zeros(n, np.int64), np.zeros(n, np.int64)
    ql, tl = np.zeros(n, np.int32), np.zeros(n, np.int32)
    qbuf, tbuf = np.zeros(qcap, np.uint8), np.zeros(tcap, np.uint8)
    qu, tu = C.c_int64(), C.c_int64()
    rc = _lib().synth_ll(C.byref(s), seed, n, qoff.ctypes.data, ql.ctypes.data, toff.ctypes.data, tl.ctypes.data,
                         qbuf.ctypes.data, qcap, tbuf.ctypes.data, tcap, C.byref(qu), C.byref(tu))
    if rc != 0:
        raise RuntimeError("synth_ll: buffer capacity exceeded")
    jobs = np.zeros(n, LL_JOB)
    jobs["qoff"], jobs["toff"], jobs["qlen"], jobs["tlen"], jobs["xtra"] = qoff, toff, ql, tl, xtra
    mat = gen_nt4_mat(2, 8, 0, 1) if mat is None else mat
    return Rescue(jobs, qbuf[:qu.value].copy(), tbuf[:tu.value].copy(), size, mat, gapo, gape, name)


def config3(n=2000000, seed=SEED + 4):
    return ll_jobs(n, seed=seed, name="cfg3-ll-i16-150vs500-1000")


def config3_pe(n=200000, seed=SEED + 5):
    """pe.c rescue variant (pe.c:252-271): matrix scaled by a=2 (match 1, mismatch 4, N 1), gapo=6,
    gape=1, u8 core with KSW_LL_SUBO | min_len(19)."""
    from .lib import KSW_LL_SUBO
    mat = gen_nt4_mat(1, 4, 0, 1)
    return ll_jobs(n, size=1, xtra=KSW_LL_SUBO | 19, mat=mat, gapo=6, gape=1, seed=seed, name="cfg3-ll-u8-pe")


class Reference2b:
    """A synthetic reference in minibwa's l2b layout: 2-bit packed bases (32 per uint64, base i
    at bits 2*(i%32)), contigs back to back, and sorted [st, en) runs of N.  N positions hold a
    random 2-bit base in pac, as l2b_import stores them."""

    def __init__(self, ctg_len, n_runs=20, run_max=200, seed=SEED + 50, n_repeats=0):
        rng = np.random.default_rng(seed)
        self.ctg_len = np.asarray(ctg_len, np.uint64)
        self.ctg_off = np.concatenate([[0], np.cumsum(self.ctg_len)[:-1]]).astype(np.uint64)
        tot = int(self.ctg_len.sum())
        self.bases = rng.integers(0, 4, tot).astype(np.uint8)
        for _ in range(n_repeats):  # near-tandem copies (1% substitutions) 100-700 bases downstream
            ln = int(rng.integers(100, 400))
            src = int(rng.integers(0, max(tot - ln - 800, 1)))
            dst = src + ln + int(rng.integers(0, 400))
            if dst + ln <= tot:
                cp = self.bases[src:src + ln].copy()
                s = rng.random(ln) < 0.01
                cp[s] = rng.integers(0, 4, int(s.sum()))
                self.bases[dst:dst + ln] = cp
        starts = np.sort(rng.choice(max(tot - run_max, 1), n_runs, replace=False)) if n_runs else np.zeros(0, int)
        runs = []
        for st in starts:
            en = int(st) + int(rng.integers(1, run_max + 1))
            if runs and st <= runs[-1][1]:
                runs[-1][1] = max(runs[-1][1], en)
            else:
                runs.append([int(st), en])
        self.ambi = np.array(runs, np.uint64).reshape(-1, 2)
        n_pac = (tot + 31) // 32
        b = np.zeros(n_pac * 32, np.uint8)
        b[:tot] = self.bases
        b = b.reshape(n_pac, 32)
        self.pac = np.zeros(n_pac, np.uint64)
        for k in range(32):
            self.pac |= b[:, k].astype(np.uint64) << np.uint64(2 * k)

    def decoded(self):
        """All contigs as codes 0..4 (N runs applied)."""
        g = self.bases.copy()
        for s0, e0 in self.ambi:
            g[int(s0):int(e0)] = 4
        return g

    def window(self, tid, st, length, flags=0):
        """The decoded window, computed here with numpy (an independent cross-check)."""
        g0 = int(self.ctg_off[tid]) + int(st)
        w = self.bases[g0:g0 + length].copy()
        for s0, e0 in self.ambi:
            s1, e1 = max(int(s0), g0), min(int(e0), g0 + length)
            if s1 < e1:
                w[s1 - g0:e1 - g0] = 4
        if flags & 2:
            w[w == 1] = 3
        elif flags & 4:
            w[w == 2] = 0
        return w[::-1].copy() if flags & 1 else w


def ref_pairs(ref, n, qlen_lo=100, qlen_hi=300, flank=50, w=100, dual=True, flag=KSW_EZ_EXTZ_ONLY, flags=None,
              seed=SEED + 51):
    """Extension jobs whose targets are windows of `ref`: the query is the window (as the job's
    flags decode it) with 2% substitutions and 0.5% indels, the window `flank` bases longer.
    Returns (Pairs with host target bytes, contig ids, window flags)."""
    rng = np.random.default_rng(seed)
    jobs = np.zeros(n, EXT_JOB)
    tids = np.zeros(n, np.int32)
    tfl = np.zeros(n, np.int32) if flags is None else np.asarray(flags, np.int32)
    qparts, tparts = [], []
    for i in range(n):
        ql = int(rng.integers(qlen_lo, qlen_hi + 1))
        k = int(rng.integers(0, len(ref.ctg_len)))
        tl = min(ql + flank, int(ref.ctg_len[k]))
        st = int(rng.integers(0, int(ref.ctg_len[k]) - tl + 1))
        t = ref.window(k, st, tl, int(tfl[i]))
        q = t[:min(ql, tl)].copy()
        sub = rng.random(len(q)) < 0.02
        q[sub] = rng.integers(0, 4, int(sub.sum()))
        if rng.random() < 0.3 and len(q) > 20:
            p = int(rng.integers(5, len(q) - 5))
            q = np.concatenate([q[:p], q[p + int(rng.integers(1, 4)):]])
        jobs[i]["qlen"], jobs[i]["tlen"], jobs[i]["toff"] = len(q), tl, st
        tids[i] = k
        qparts.append(q), tparts.append(t)
    jobs["qoff"] = np.concatenate([[0], np.cumsum([len(x) for x in qparts])[:-1]])
    jobs["w"], jobs["zdrop"], jobs["end_bonus"], jobs["flag"] = w, 100, 10, flag
    mat = gen_nt4_mat(2, 8, 0, 1)
    q2, e2 = (24, 1) if dual else (12, 2)
    host = jobs.copy()
    host["toff"] = np.concatenate([[0], np.cumsum([len(x) for x in tparts])[:-1]])
    pairs = Pairs(host, np.concatenate(qparts), np.concatenate(tparts), dual, mat, 12, 2, q2, e2, "ref-windows")
    pairs.ref_toff = jobs["toff"].copy()
    return pairs, tids, tfl


# minibwa's short-read defaults (options.c mb_opt_init / the "sr" preset)
RESCUE_OPT_SR = dict(a=2, b=8, b_ts=0, b_ambi=1, q=12, e=2, bw=100, zdrop=80, end_bonus=10, min_len=19,
                     min_dp_max=30)


def _revcomp(x):
    x = np.asarray(x, np.uint8)[::-1]
    return np.where(x < 4, 3 - x, x).astype(np.uint8)


class RescueCases:
    """Mate-rescue candidates over a Reference2b: for each, an anchor hit (contig, ts, te, rev,
    r0), one permitted orientation dir with insert bounds [lo, hi], the mate as sequenced and
    its reverse complement (seq[0], seq[1]) and the library's methylation mode mt0.  window()
    gives the candidate window and the read orientation of pe.c:330-339; jobs/qbuf are the
    device call's inputs (the read in the orientation pe.c aligns, mt after l2b_meth_rev)."""

    def __init__(self, ref, n, qlen_lo=100, qlen_hi=250, lo=50, hi=800, p_random=0.2, p_meth=0.25,
                 p_edge=0.05, sub=0.02, indel=0.005, min_sc_hi=40, seed=SEED + 52):
        rng = np.random.default_rng(seed)
        self.ref, self.cases = ref, []
        parts, jobs = [], []
        off = 0
        while len(self.cases) < n:
            k = int(rng.integers(0, len(ref.ctg_len)))
            clen = int(ref.ctg_len[k])
            qlen = int(rng.integers(qlen_lo, qlen_hi + 1))
            l0 = int(rng.integers(qlen_lo, qlen_hi + 1))
            if clen < 3 * (hi + qlen + l0):
                continue
            if rng.random() < p_edge:
                h_ts = int(rng.integers(0, 2 * hi)) if rng.random() < 0.5 else int(rng.integers(clen - 2 * hi, clen - l0))
            else:
                h_ts = int(rng.integers(0, clen - l0))
            h_te, h_rev, r0, d = h_ts + l0, int(rng.integers(0, 2)), int(rng.integers(0, 2)), int(rng.integers(0, 4))
            mt0 = int(rng.integers(1, 3)) if rng.random() < p_meth else 0
            ts, te, is_rev = rescue_window(d, lo, hi, h_ts, h_te, h_rev, r0, qlen, clen)
            if te - ts <= qlen:
                continue
            mt = meth_rev(mt0) if is_rev else mt0
            if rng.random() < p_random:
                m = rng.integers(0, 4, qlen).astype(np.uint8)
            else:
                ms = int(rng.integers(ts, te - qlen + 1))
                m = ref.window(k, ms, qlen).copy()
                m = _mutate(rng, m, sub, indel)
                if mt:
                    conv = rng.random(len(m)) < 0.9
                    if mt == 1:
                        m[(m == 1) & conv] = 3
                    else:
                        m[(m == 2) & conv] = 0
            # the window follows the read's final length, as pe.c computes it from len
            ts, te, is_rev = rescue_window(d, lo, hi, h_ts, h_te, h_rev, r0, len(m), clen)
            if te - ts <= len(m):
                continue
            seq = [None, None]
            seq[is_rev] = m
            seq[1 - is_rev] = _revcomp(m)
            min_sc = int(rng.integers(0, min_sc_hi + 1))
            self.cases.append(dict(tid=k, h_ts=h_ts, h_te=h_te, h_rev=h_rev, r0=r0, dir=d, lo=lo, hi=hi, mt0=mt0,
                                   seq=seq, min_sc=min_sc, ts=ts, te=te, is_rev=is_rev, mt=mt))
            j = np.zeros(1, RESCUE_JOB)
            j["qoff"], j["ts"], j["te"], j["qlen"], j["tid"] = off, ts, te, len(m), k
            j["meth"], j["min_sc"], j["rev"] = mt, min_sc, is_rev
            jobs.append(j), parts.append(m)
            off += len(m)
        self.jobs = np.concatenate(jobs)
        self.qbuf = np.concatenate(parts)


def rescue_window(dir, lo, hi, h_ts, h_te, h_rev, r0, qlen, ctg_len):
    """The candidate window [ts, te) and read orientation of one orientation dir
    (pe.c:330-339)."""
    pos5 = h_te if h_rev else h_ts
    is_rev = int((dir >> 1) != (dir & 1)) ^ h_rev
    if (dir >> 1) != (dir & 1):
        is_larger = (dir >> 1) ^ is_rev
    else:
        is_larger = (dir >> 1) ^ r0 ^ h_rev
    ts = (pos5 + lo if is_larger else pos5 - hi) - (0 if not is_rev else qlen)
    te = (pos5 + hi if is_larger else pos5 - lo) + (qlen if not is_rev else 0)
    return max(ts, 0), min(te, int(ctg_len)), is_rev


def meth_rev(mt):
    """l2b_meth_rev (l2bit.h:63-66)."""
    return 0 if mt == 0 else 2 if mt == 1 else 1


def _mutate(rng, m, sub, indel):
    m = m.copy()
    s = rng.random(len(m)) < sub
    m[s] = rng.integers(0, 4, int(s.sum()))
    out, i = [], 0
    while i < len(m):
        u = rng.random()
        if u < indel / 2:
            i += int(rng.integers(1, 4))
            continue
        if u < indel:
            out.extend(rng.integers(0, 4, int(rng.integers(1, 4))).tolist())
        out.append(int(m[i]))
        i += 1
    return np.array(out, np.uint8)


RESCUE_SPEC = dict(qlen_lo=100, qlen_hi=250, lo=50, hi=800, p_random=0.2, p_meth=0.0, sub_rate=0.02,
                   indel_rate=0.005, min_sc_hi=40)


def rescue_workload(n, ctg_len=(40_000_000, 25_000_000, 15_000_000), spec=None, seed=SEED + 60, ref=None):
    """n mate-rescue candidates (the C generator) over a Reference2b of the given contigs:
    anchors uniform on the contigs, insert bounds [50, 800] (minibwa's pe_lo / pe_hi), reads of
    100-250 nt with 2% substitutions and 0.5% indels, 20% unrelated reads.
    Returns (reference, RESCUE_JOB array, read buffer)."""
    sp = RescueSpec(**{**RESCUE_SPEC, **(spec or {})})
    if ref is None:
        ref = Reference2b(list(ctg_len), n_runs=200, run_max=500, seed=seed, n_repeats=2000)
    g = ref.decoded()
    jobs = np.zeros(n, RESCUE_JOB)
    qbuf = np.zeros(int(n) * (sp.qlen_hi * 2 + 8) + 64, np.uint8)
    used = C.c_int64()
    off = np.ascontiguousarray(ref.ctg_off, np.uint64)
    ln = np.ascontiguousarray(ref.ctg_len, np.uint64)
    rc = _lib().synth_rescue(C.byref(sp), seed, g.ctypes.data, len(off), off.ctypes.data, ln.ctypes.data, int(n),
                             jobs.ctypes.data, qbuf.ctypes.data, len(qbuf), C.byref(used))
    if rc != 0:
        raise RuntimeError(f"synth_rescue failed ({rc})")
    return ref, jobs, qbuf[:used.value].copy()


# minibwa's option presets the chain cases are aligned with (options.c:53-83): "sr"/"adap" and "lr"
CHAIN_OPT_SR = dict(a=2, b=8, b_ts=0, b_ambi=1, q=12, e=2, q2=23, e2=1, bw=100, bw_long=20000, max_gap=100,
                    end_bonus=10, zdrop=80, zdrop_inv=80, min_ksw_len=20, min_len=19, min_chain_score=25,
                    min_dp_max=30, long_reads=0, adaptive=1, max_sr_len=325, meth=0, max_sw_mat=100000000)
CHAIN_OPT_LR = dict(CHAIN_OPT_SR, bw=500, max_gap=5000, end_bonus=-1, zdrop=400, zdrop_inv=240, min_ksw_len=200,
                    min_chain_score=40, min_dp_max=50, long_reads=1, adaptive=0)


class ChainCases:
    """Hits (chains of exact-match anchors) of simulated reads over a Reference2b, shaped like the
    chains minibwa hands to mb_align1: for each read, the sequence in the orientation aligned
    (seq[rev]) and its anchors -- the maximal runs of at least min_len bases that match the
    reference on one diagonal, ordered along the read -- with mlen and a chaining score.
    Reads carry substitutions and short indels, and each draws one event (`kind`):
      0 none; 1 a block of random bases of unchanged length (a gap fill that z-drops);
      2 a chimeric junction to a region downstream on the contig; 3 one long insertion or
      deletion; 4 an inverted segment (the inversion test of the z-drop check); 5 two long gaps,
      opposite (mm_filter_bad_seeds) or in one direction (mm_filter_bad_seeds_alt); 6 a mid-size
      indel near either end (mm_fix_bad_ends); 7 a read at a contig's start or end.
    Bisulfite reads (meth=True) read C as T (mode 1) or G as A (mode 2) on their forward strand;
    some hits carry split_inv (the z-drop of their left extension uses zdrop_inv)."""

    N_KINDS = 8

    def __init__(self, ref, n, long_reads=False, seed=SEED + 70, min_len=19, meth=False, p_split_inv=0.2):
        rng = np.random.default_rng(seed)
        g = ref.decoded()
        self.ref = ref
        anchors, chains, reads = [], [], []
        self.fwd, self.rc, self.kind = [], [], []
        qoff = 0
        big = (lambda lo, hi: int(rng.integers(lo * 5, hi * 5))) if long_reads else (lambda lo, hi: int(rng.integers(lo, hi)))
        while len(chains) < n:
            k = int(rng.integers(0, len(ref.ctg_len)))
            clen, c0 = int(ref.ctg_len[k]), int(ref.ctg_off[k])
            L = int(rng.integers(1000, 6000)) if long_reads else int(rng.integers(100, 251))
            kind = len(chains) % self.N_KINDS
            if clen < 4 * L + 20000:
                continue
            if kind == 7:
                st = int(rng.integers(0, 40)) if rng.random() < 0.5 else clen - L - int(rng.integers(0, 40))
            else:
                st = int(rng.integers(0, clen - 2 * L - 12000))
            mt = int(rng.integers(1, 3)) if meth and rng.random() < 0.7 else 0
            sub, ind = (0.05, 0.02) if long_reads else (0.02, 0.005)
            at = int(rng.integers(L // 4, 3 * L // 4))
            ev = []  # (read position, event) to apply
            if kind == 1:
                ev = [(at, ("junk", big(20, 80)))]
            elif kind == 2:
                ev = [(at, ("jump", big(60, 1600)))]
            elif kind == 3:
                ev = [(at, ("ins" if rng.random() < 0.5 else "del", big(30, 120)))]
            elif kind == 4:
                ev = [(at, ("inv", big(40, 200)))]
            elif kind == 5:
                l1 = big(30, 120)
                same = rng.random() < 0.5
                l2 = big(30, 120) if same else l1 + int(rng.integers(-10, 11))
                op1 = "ins" if rng.random() < 0.5 else "del"
                op2 = op1 if same else ("del" if op1 == "ins" else "ins")
                ev = [(at, (op1, l1)), (at + int(rng.integers(20, 60)) * (5 if long_reads else 1), (op2, max(l2, 1)))]
            elif kind == 6:
                p6 = int(rng.integers(25, 90)) if rng.random() < 0.5 else L - int(rng.integers(25, 90))
                ev = [(p6, ("ins" if rng.random() < 0.5 else "del", int(rng.integers(15, 60))))]
            seq, pos = [], []  # the read in the aligned orientation and its reference position (-1: inserted)
            t = st
            while len(seq) < L and t < clen - 1:
                if ev and len(seq) >= ev[0][0]:
                    op, ln = ev.pop(0)[1]
                    if op == "junk":
                        seq += [int(x) for x in rng.integers(0, 4, ln)]
                        pos += [-1] * ln
                        t += ln
                    elif op == "jump" or op == "del":
                        t += ln
                    elif op == "ins":
                        seq += [int(x) for x in rng.integers(0, 4, ln)]
                        pos += [-1] * ln
                    elif op == "inv":
                        ln = min(ln, clen - 1 - t)
                        piece = g[c0 + t:c0 + t + ln]
                        seq += [int(x) for x in _revcomp(piece)]
                        pos += [-1] * ln
                        t += ln
                    continue
                u = rng.random()
                if u < ind / 2:
                    t += int(rng.integers(1, 4))
                    continue
                if u < ind:
                    for _ in range(int(rng.integers(1, 4))):
                        seq.append(int(rng.integers(0, 4))), pos.append(-1)
                    continue
                b = int(g[c0 + t])
                if b < 4 and rng.random() < sub:
                    b = (b + int(rng.integers(1, 4))) % 4
                if mt == 1 and b == 1 and rng.random() < 0.95:
                    b = 3
                elif mt == 2 and b == 2 and rng.random() < 0.95:
                    b = 0
                seq.append(b), pos.append(t)
                t += 1
            s = np.array(seq, np.uint8)
            p = np.array(pos, np.int64)
            if len(s) < 60:
                continue
            # maximal exact runs on one diagonal (bisulfite pairs match through the conversion)
            ok = p >= 0
            gb = np.where(ok, g[c0 + np.maximum(p, 0)], 255)
            eq = ok & ((s == gb) | ((mt == 1) & (gb == 1) & (s == 3)) | ((mt == 2) & (gb == 2) & (s == 0)))
            runs, i = [], 0
            while i < len(s):
                if not eq[i]:
                    i += 1
                    continue
                j = i
                while j + 1 < len(s) and eq[j + 1] and p[j + 1] == p[j] + 1:
                    j += 1
                if j - i + 1 >= min_len:
                    runs.append((i, j))
                i = j + 1
            if not runs:
                continue
            rev = int(rng.random() < 0.5)
            mt_read = (3 - mt if mt else 0) if rev else mt  # the mode of the read's own forward strand
            a0 = len(anchors)
            for i, j in runs:
                anchors.append((k << 1 | rev, j - i + 1, j, 0, int(p[j])))
            cnt = len(runs)
            tp = np.array([x[4] for x in anchors[a0:]], np.int64)
            qp = np.array([x[2] for x in anchors[a0:]], np.int64)
            lens = np.array([x[1] for x in anchors[a0:]], np.int64)
            mlen = int(lens[0])
            for i in range(1, cnt):  # mb_cal_mblen (map-algo.c:133-150)
                tl, ql, sp = int(tp[i] - tp[i - 1]), int(qp[i] - qp[i - 1]), int(lens[i])
                mlen += sp if (tl > sp and ql > sp) else min(tl, ql)
            split_inv = int(rng.random() < p_split_inv)
            chains.append((a0, cnt, mlen, int(lens.sum()), qoff, len(s), mt_read, split_inv))
            reads.append(s)
            fwd = _revcomp(s) if rev else s
            self.fwd.append(fwd), self.rc.append(_revcomp(fwd)), self.kind.append(kind)
            qoff += len(s)
        self.anchors = np.array(anchors, dtype=[("sid", "<i4"), ("len", "<i4"), ("qpos", "<i4"), ("flag", "<u4"),
                                                ("tpos", "<i8")])
        self.chains = np.array(chains, dtype=[(x, "<i4") for x in ("as", "cnt", "mlen", "score", "qoff", "qlen",
                                                                     "meth", "split_inv")])
        self.qbuf = np.concatenate(reads)

    def __len__(self):
        return len(self.chains)

    def read(self, i):
        c = self.chains[i]
        return self.qbuf[c["qoff"]:c["qoff"] + c["qlen"]]


# ---- genomes and reads for whole-mapper runs (FASTA in, SAM out)

_ACGTN = np.frombuffer(b"ACGTN", np.uint8)


def _mutate_fast(rng, s, sub, indel):
    """Substitutions at rate sub, then indels of 1-3 bases at rate indel (half insertions),
    without a per-base Python loop."""
    s = s.copy()
    m = rng.random(len(s)) < sub
    s[m] = (s[m] + rng.integers(1, 4, int(m.sum()))).astype(np.uint8) % 4
    ev = np.nonzero(rng.random(len(s)) < indel)[0]
    if len(ev) == 0:
        return s
    keep = np.ones(len(s), bool)
    ins_at, ins = [], []
    for p in ev:
        ln = int(rng.integers(1, 4))
        if rng.random() < 0.5:
            keep[p:p + ln] = False
        else:
            ins_at.append(p), ins.append(rng.integers(0, 4, ln).astype(np.uint8))
    if ins:
        s = np.insert(s, np.repeat(ins_at, [len(x) for x in ins]), np.concatenate(ins))
        keep = np.insert(keep, np.repeat(ins_at, [len(x) for x in ins]), True)
    return s[keep]


def mapper_genome(ctg_len=(2_000_000, 1_200_000, 800_000), seed=SEED + 80, n_repeats=300, n_runs=20):
    """Contigs of random bases with near-copies of segments (300 of 200-3000 bases, 2%
    diverged) and runs of N; returns a list of (name, uint8 codes 0-4)."""
    rng = np.random.default_rng(seed)
    ctgs = [rng.integers(0, 4, n).astype(np.uint8) for n in ctg_len]
    for _ in range(n_repeats):
        a, b = (int(x) for x in rng.integers(0, len(ctgs), 2))
        ln = int(rng.integers(200, 3000))
        sa, sb = int(rng.integers(0, len(ctgs[a]) - ln)), int(rng.integers(0, len(ctgs[b]) - ln))
        seg = _mutate_fast(rng, ctgs[a][sa:sa + ln], 0.02, 0.0)
        ctgs[b][sb:sb + ln] = seg[:ln]
    for _ in range(n_runs):
        k = int(rng.integers(0, len(ctgs)))
        ln, st = int(rng.integers(1, 400)), int(rng.integers(0, len(ctgs[k]) - 400))
        ctgs[k][st:st + ln] = 4
    return [(f"ctg{k + 1}", c) for k, c in enumerate(ctgs)]


def write_fasta(fn, seqs, width=0):
    with open(fn, "w") as f:
        for name, s in seqs:
            f.write(f">{name}\n{_ACGTN[s].tobytes().decode()}\n")


def mapper_pairs(genome, n, rl=150, ins_mean=350, ins_sd=50, seed=SEED + 81, sub=0.015, indel=0.002,
                 p_noisy=0.08, p_junk=0.04, p_chimera=0.03):
    """n read pairs (FR orientation) from the genome: substitutions and short indels, some mates
    noisy (12% substitutions: mate rescue), some with a random tail (z-drop) or a chimeric
    second half.  Returns (reads 1, reads 2) as lists of (name, codes)."""
    rng = np.random.default_rng(seed)
    lens = np.array([len(c) for _, c in genome], np.float64)
    r1, r2 = [], []
    while len(r1) < n:
        k = int(rng.choice(len(genome), p=lens / lens.sum()))
        g = genome[k][1]
        ins = max(rl + 20, int(rng.normal(ins_mean, ins_sd)))
        if len(g) < ins + 200:
            continue
        st = int(rng.integers(0, len(g) - ins - 50))
        frag = g[st:st + ins + 40]
        if rng.random() < 0.5:
            frag = _revcomp(frag)
        a = _mutate_fast(rng, frag[:rl + 20], sub, indel)[:rl]
        b = _revcomp(_mutate_fast(rng, frag[ins - rl - 20:ins], sub, indel)[-rl:])
        u = rng.random()
        if u < p_noisy:
            b = _mutate_fast(rng, b, 0.12, 0.0)
        elif u < p_noisy + p_junk:
            t = int(rng.integers(20, 70))
            a = np.concatenate([a[:rl - t], rng.integers(0, 4, t).astype(np.uint8)])
        elif u < p_noisy + p_junk + p_chimera:
            k2 = int(rng.integers(0, len(genome)))
            g2 = genome[k2][1]
            s2 = int(rng.integers(0, len(g2) - rl))
            a = np.concatenate([a[:rl // 2], g2[s2:s2 + rl - rl // 2]])
        if len(a) < 30 or len(b) < 30:
            continue
        nm = f"p{len(r1)}"
        r1.append((nm + "/1", a)), r2.append((nm + "/2", b))
    return r1, r2


def mapper_long_reads(genome, n, lo=1000, hi=8000, seed=SEED + 82, sub=0.05, indel=0.03, p_inv=0.15, p_junk=0.1,
                      p_chimera=0.05):
    """n long reads: 5% substitutions and 3% indels, some with an inverted segment (the
    inversion check), a random block (a z-drop inside the chain) or a chimeric junction."""
    rng = np.random.default_rng(seed)
    lens = np.array([len(c) for _, c in genome], np.float64)
    out = []
    while len(out) < n:
        k = int(rng.choice(len(genome), p=lens / lens.sum()))
        g = genome[k][1]
        L = int(rng.integers(lo, hi))
        if len(g) < L + 100:
            continue
        st = int(rng.integers(0, len(g) - L))
        s = g[st:st + L].copy()
        u = rng.random()
        if u < p_inv:
            a, ln = int(rng.integers(L // 4, L // 2)), int(rng.integers(150, min(1500, L // 3)))
            s[a:a + ln] = _revcomp(s[a:a + ln])
        elif u < p_inv + p_junk:
            a, ln = int(rng.integers(L // 4, L // 2)), int(rng.integers(100, 600))
            s[a:a + ln] = rng.integers(0, 4, len(s[a:a + ln]))
        elif u < p_inv + p_junk + p_chimera:
            k2 = int(rng.integers(0, len(genome)))
            g2 = genome[k2][1]
            s2 = int(rng.integers(0, len(g2) - L // 2))
            s = np.concatenate([s[:L // 2], g2[s2:s2 + L // 2]])
        s = _mutate_fast(rng, s, sub, indel)
        if rng.random() < 0.5:
            s = _revcomp(s)
        out.append((f"l{len(out)}", s))
    return out
