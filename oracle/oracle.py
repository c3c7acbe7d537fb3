"""ctypes binding of the checker libraries (TEST INFRASTRUCTURE ONLY).

  liboracle.so        scalar C restatement of the reference (ksw2_oracle.c), builds anywhere
  _ref/libksw2ref.so  the reference's own ksw2 SSE sources, built here from the reference
                      tree when it is present (never on a machine without it)
  _ref/libmbpe.so     the reference's mate rescue (pe.c) behind ref_pe.c, same conditions

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module,
and only as the checker / the timed CPU baseline -- never as a product code path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# The reference's sources as `make stage` copies them (git-ignored; they travel with the working
# tree to machines where the reference tree itself does not exist).
STAGED_TREE = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "src")
LIB_ORACLE = os.path.join(HERE, "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libksw2ref.so")
LIB_MBPE = os.path.join(HERE, "_ref", "libmbpe.so")

ORC_JOB = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"),
                    ("w", "<i4"), ("zdrop", "<i4"), ("end_bonus", "<i4"), ("flag", "<i4")])
ORC_RES = np.dtype([("score", "<i4"), ("max", "<i4"), ("max_q", "<i4"), ("max_t", "<i4"),
                    ("mqe", "<i4"), ("mqe_t", "<i4"), ("mte", "<i4"), ("mte_q", "<i4"),
                    ("zdropped", "<i4"), ("reach_end", "<i4"), ("n_cigar", "<i4"), ("n_diag", "<i4"),
                    ("cigar_off", "<i8")])
ORC_RESCUE_JOB = np.dtype([("qoff", "<i8"), ("ts", "<i8"), ("te", "<i8"), ("qlen", "<i4"), ("tid", "<i4"),
                           ("meth", "<i4"), ("min_sc", "<i4"), ("rev", "<i4"), ("pad", "<i4")])
ORC_RESCUE_RES = np.dtype([("max_ug", "<i4"), ("max_i", "<i4"), ("n_good", "<i4"), ("n_kmer", "<i4"),
                           ("ts2", "<i8"), ("te2", "<i8"),
                           ("ll_done", "<i4"), ("ll_score", "<i4"), ("ll_te", "<i4"), ("ll_qe", "<i4"),
                           ("ll_score2", "<i4"), ("ll_te2", "<i4"), ("ext_done", "<i4"), ("rescued", "<i4"),
                           ("qs", "<i4"), ("qe", "<i4"), ("dp_max2", "<i4"), ("pad", "<i4"),
                           ("ts", "<i8"), ("te", "<i8"),
                           ("ext", [(k, "<i4") for k in ("score", "max", "max_q", "max_t", "mqe", "mqe_t", "mte",
                                                          "mte_q", "zdropped", "reach_end", "n_cigar", "n_diag")]
                            + [("cigar_off", "<i8"), ("cells", "<i8")])])
ORC_LLRES = np.dtype([("score", "<i4"), ("te", "<i4"), ("qe", "<i4"), ("score2", "<i4"), ("te2", "<i4")])


class OrcExtz(C.Structure):
    _fields_ = [("max", C.c_uint32, 31), ("zdropped", C.c_uint32, 1),
                ("max_q", C.c_int), ("max_t", C.c_int), ("mqe", C.c_int), ("mqe_t", C.c_int),
                ("mte", C.c_int), ("mte_q", C.c_int), ("score", C.c_int),
                ("m_cigar", C.c_int), ("n_cigar", C.c_int), ("reach_end", C.c_int),
                ("cigar", C.POINTER(C.c_uint32))]

    def fields(self):
        return dict(max=self.max, zdropped=self.zdropped, max_q=self.max_q, max_t=self.max_t, mqe=self.mqe,
                    mqe_t=self.mqe_t, mte=self.mte, mte_q=self.mte_q, score=self.score,
                    reach_end=self.reach_end, n_cigar=self.n_cigar,
                    cigar=[self.cigar[i] for i in range(self.n_cigar)])


class OrcStats(C.Structure):
    _fields_ = [("cells", C.c_int64), ("padded_cells", C.c_int64), ("n_diag", C.c_int32)]


class OrcLL(C.Structure):
    _fields_ = [("score", C.c_int), ("te", C.c_int), ("qe", C.c_int), ("score2", C.c_int), ("te2", C.c_int)]


def ref_tree():
    """The reference source tree to compile: $KSW2_REF_TREE, else the staged copy, else None."""
    t = os.environ.get("KSW2_REF_TREE")
    if t and os.path.isdir(t):
        return t
    return STAGED_TREE if os.path.isfile(os.path.join(STAGED_TREE, "ksw2.h")) else None


def stage(tree):
    """Copy the reference's sources and test reads from `tree` into the staged folder."""
    subprocess.check_call(["make", "-s", "-C", HERE, "stage", f"REF={tree}"])


def build(ref=True):
    """Compile liboracle.so, and _ref/libksw2ref.so and _ref/libmbpe.so when a reference tree
    (ref_tree()) exists."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    t = ref_tree() if ref else None
    if t:
        subprocess.check_call(["make", "-s", "-C", HERE, "-j8", "ref", f"REF={t}"])


def build_minibwa(gpulib_dir):
    """Compile the reference's minibwa stock and relinked against libksw2gpu.so in gpulib_dir
    (oracle/_ref/minibwa_{stock,gpu}{,_km}); needs a reference tree."""
    t = ref_tree()
    if not t:
        raise RuntimeError("no reference tree: set KSW2_REF_TREE or stage one (make -C oracle stage REF=...)")
    subprocess.check_call(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", "minibwa", f"REF={t}",
                           f"GPULIB={gpulib_dir}"])
    return {k: os.path.join(HERE, "_ref", "minibwa_" + k) for k in ("stock", "gpu", "stock_km", "gpu_km")}


def have_ref():
    return os.path.exists(LIB_REF)


_libs = {}


def _load(path, prefix):
    if path in _libs:
        return _libs[path]
    L = C.CDLL(path)
    vp, i32, i64, i8 = C.c_void_p, C.c_int, C.c_int64, C.c_int8
    f = getattr(L, prefix + "ext_batch")
    f.restype = i64
    f.argtypes = [i32, i32, vp, vp, vp, i8, vp, i8, i8, i8, i8, vp, vp, i64, i32, vp]
    f = getattr(L, prefix + "ll_batch")
    f.restype = None
    f.argtypes = [i32, i32, vp, vp, vp, i32, vp, i32, i32, i32, vp, i32, vp]
    if prefix == "orc_":
        L.orc_extz2.restype = None
        L.orc_extz2.argtypes = [i32, vp, i32, vp, i8, vp, i8, i8, i32, i32, i32, i32, C.POINTER(OrcExtz),
                                C.POINTER(OrcStats)]
        L.orc_extd2.restype = None
        L.orc_extd2.argtypes = [i32, vp, i32, vp, i8, vp, i8, i8, i8, i8, i32, i32, i32, i32, C.POINTER(OrcExtz),
                                C.POINTER(OrcStats)]
        L.orc_ll_qinit.restype = vp
        L.orc_ll_qinit.argtypes = [i32, i32, vp, i32, vp]
        L.orc_ll_u8_core.restype = OrcLL
        L.orc_ll_u8_core.argtypes = [vp, i32, vp, i32, i32, i32]
        L.orc_ll_i16_core.restype = OrcLL
        L.orc_ll_i16_core.argtypes = [vp, i32, vp, i32, i32, i32]
        L.orc_ll_rows.restype = i32
        L.orc_ll_rows.argtypes = [vp]
        L.orc_l2b_getseq.restype = None
        L.orc_l2b_getseq.argtypes = [vp, vp, i64, vp, i64, i64, i64, i32, vp]
        L.orc_ungap.restype = i32
        L.orc_rescue_batch.restype = i64
        L.orc_rescue_batch.argtypes = [vp, i32, vp, vp, vp, vp, i64, vp, vp, vp, i64, i32]
        L.orc_ungap.argtypes = [i32, vp, i32, vp, i32, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]
    _libs[path] = L
    return L


def oracle_lib():
    if not os.path.exists(LIB_ORACLE):
        build(ref=False)
    return _load(LIB_ORACLE, "orc_")


def have_ref_pe():
    return os.path.exists(LIB_MBPE)


def refpe_lib():
    if not have_ref_pe():
        raise RuntimeError("reference rescue build not available (oracle/_ref)")
    if LIB_MBPE not in _libs:
        L = C.CDLL(LIB_MBPE)
        vp, i32, i64 = C.c_void_p, C.c_int, C.c_int64
        L.refpe_ungap.restype = i32
        L.refpe_ungap.argtypes = [i32, vp, i32, vp, i32, i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]
        L.refpe_matesw.restype = i32
        L.refpe_matesw.argtypes = [i64, vp, vp, vp, i64, i64, vp, vp, i32, i32, i32, i64, i64, i64, i32, i32, i32,
                                   vp, vp, i32, i32, vp, vp, i32]
        L.refpe_getseq.restype = i64
        L.refpe_getseq.argtypes = [i64, vp, vp, vp, i64, i64, vp, i64, i64, i64, vp]
        _libs[LIB_MBPE] = L
    return _libs[LIB_MBPE]


def ref_lib():
    if not have_ref():
        raise RuntimeError("reference build not available (oracle/_ref)")
    return _load(LIB_REF, "ref_")


def _p(a):
    return a.ctypes.data


def ext_batch(which, dual, m, mat, q, e, q2, e2, jobs, qbuf, tbuf, nthreads=1):
    """Run extension jobs on the oracle ('orc') or the reference build ('ref').
    Returns (results ORC_RES, cigar words)."""
    L = oracle_lib() if which == "orc" else ref_lib()
    f = getattr(L, ("orc_" if which == "orc" else "ref_") + "ext_batch")
    jobs = np.ascontiguousarray(np.asarray(jobs).astype(ORC_JOB))
    qbuf = np.ascontiguousarray(qbuf, np.uint8)
    tbuf = np.ascontiguousarray(tbuf, np.uint8)
    mat = np.ascontiguousarray(mat, np.int8)
    n = len(jobs)
    res = np.zeros(n, ORC_RES)
    cap = int((jobs["qlen"].astype(np.int64) + jobs["tlen"] + 1).sum()) + 16
    cig = np.zeros(cap, np.uint32)
    tot = f(int(dual), n, _p(jobs), _p(qbuf), _p(tbuf), m, _p(mat), q, e, q2, e2, _p(res), _p(cig), cap,
            nthreads, None)
    if tot < 0:
        raise RuntimeError("cigar capacity")
    return res, cig


def ll_batch(which, size, m, mat, gapo, gape, jobs, qbuf, tbuf, nthreads=1, xtra=None):
    L = oracle_lib() if which == "orc" else ref_lib()
    f = getattr(L, ("orc_" if which == "orc" else "ref_") + "ll_batch")
    jobs = np.ascontiguousarray(jobs)
    j = np.zeros(len(jobs), ORC_JOB)
    j["qoff"], j["toff"], j["qlen"], j["tlen"] = jobs["qoff"], jobs["toff"], jobs["qlen"], jobs["tlen"]
    xt = int(jobs["xtra"][0]) if xtra is None and len(jobs) else (xtra or 0)
    if len(jobs) and not np.all(jobs["xtra"] == xt):
        raise ValueError("the CPU ll batch takes one xtra for all jobs")
    res = np.zeros(len(jobs), ORC_LLRES)
    f(size, len(jobs), _p(j), _p(np.ascontiguousarray(qbuf, np.uint8)), _p(np.ascontiguousarray(tbuf, np.uint8)),
      m, _p(np.ascontiguousarray(mat, np.int8)), gapo, gape, xt, _p(res), nthreads, None)
    return res


def extz(dual, query, target, m, mat, q, e, q2, e2, w, zdrop, end_bonus, flag, m_cigar0=0):
    """One oracle call; returns (fields dict, stats)."""
    L = oracle_lib()
    qa = np.ascontiguousarray(query, np.uint8)
    ta = np.ascontiguousarray(target, np.uint8)
    ma = np.ascontiguousarray(mat, np.int8)
    ez, st = OrcExtz(), OrcStats()
    if dual:
        L.orc_extd2(len(qa), _p(qa), len(ta), _p(ta), m, _p(ma), q, e, q2, e2, w, zdrop, end_bonus, flag,
                    C.byref(ez), C.byref(st))
    else:
        L.orc_extz2(len(qa), _p(qa), len(ta), _p(ta), m, _p(ma), q, e, w, zdrop, end_bonus, flag, C.byref(ez),
                    C.byref(st))
    out = ez.fields()
    out["m_cigar"] = ez.m_cigar
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    if ez.cigar:
        libc.free(C.cast(ez.cigar, C.c_void_p))
    return out, dict(cells=st.cells, padded_cells=st.padded_cells, n_diag=st.n_diag)


def ll(size, query, target, m, mat, gapo, gape, xtra):
    """One oracle ll call; returns (dict, rows processed)."""
    L = oracle_lib()
    qa = np.ascontiguousarray(query, np.uint8)
    ta = np.ascontiguousarray(target, np.uint8)
    ma = np.ascontiguousarray(mat, np.int8)
    qp = L.orc_ll_qinit(size, len(qa), _p(qa), m, _p(ma))
    r = (L.orc_ll_u8_core if size == 1 else L.orc_ll_i16_core)(qp, len(ta), _p(ta), gapo, gape, xtra)
    rows = L.orc_ll_rows(qp)
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    libc.free(qp)
    return dict(score=r.score, te=r.te, qe=r.qe, score2=r.score2, te2=r.te2), rows


def l2b_getseq(ref, tid, st, length, flags=0):
    """A window of a 2-bit reference (an object with pac, ctg_off and ambi arrays, ambi as
    (n, 2) [st, en) rows), decoded as the reference's l2b_getseq / l2b_meth_convert / mb_seq_rev
    sequence; flags 1 reverse, 2 C2T, 4 G2A."""
    L = oracle_lib()
    out = np.zeros(max(int(length), 1), np.uint8)
    amb = np.ascontiguousarray(ref.ambi, np.uint64).reshape(-1)
    L.orc_l2b_getseq(_p(np.ascontiguousarray(ref.pac, np.uint64)), _p(np.ascontiguousarray(ref.ctg_off, np.uint64)),
                     len(amb) // 2, _p(amb) if len(amb) else None, int(tid), int(st), int(length), int(flags),
                     _p(out))
    return out[:int(length)]


def ungap(query, target, kmer=7, mt=0):
    """mb_ungap (pe.c:209-247); returns (max, max_i, n_good, n_kmer)."""
    L = oracle_lib()
    q = np.ascontiguousarray(query, np.uint8)
    t = np.ascontiguousarray(target, np.uint8)
    mi, ng, nk = C.c_int(), C.c_int(), C.c_int()
    mx = L.orc_ungap(len(q), _p(q) if len(q) else None, len(t), _p(t) if len(t) else None, kmer, mt, C.byref(mi),
                     C.byref(ng), C.byref(nk))
    return mx, mi.value, ng.value, nk.value


def ref_ungap(query, target, kmer=7, mt=0):
    """The reference's own mb_ungap (through _ref/libmbpe.so)."""
    L = refpe_lib()
    q = np.ascontiguousarray(query, np.uint8)
    t = np.ascontiguousarray(target, np.uint8)
    mi, ng, nk = C.c_int(), C.c_int(), C.c_int()
    mx = L.refpe_ungap(len(q), _p(q) if len(q) else None, len(t), _p(t) if len(t) else None, kmer, mt, C.byref(mi),
                       C.byref(ng), C.byref(nk))
    return mx, mi.value, ng.value, nk.value


def _l2b_args(ref):
    off = np.ascontiguousarray(ref.ctg_off, np.uint64)
    ln = np.ascontiguousarray(ref.ctg_len, np.uint64)
    pac = np.ascontiguousarray(ref.pac, np.uint64)
    amb = np.ascontiguousarray(ref.ambi, np.uint64).reshape(-1)
    return (off, ln, pac, amb), (len(off), _p(off), _p(ln), _p(pac), len(pac), len(amb) // 2,
                                 _p(amb) if len(amb) else None)


def ref_getseq(ref, tid, st, en):
    """The reference's own l2b_getseq (l2bit.c:52-77) on [st, en) of contig tid."""
    L = refpe_lib()
    keep, args = _l2b_args(ref)
    out = np.zeros(max(int(en) - int(st), 1), np.uint8)
    n = L.refpe_getseq(*args, int(tid), int(st), int(en), _p(out))
    return out[:max(int(n), 0)]


RESCUE_SC = ("a", "b", "b_ts", "b_ambi", "q", "e", "bw", "zdrop", "end_bonus", "min_len", "min_dp_max")
HIT_FIELDS = ("rescued", "ts", "te", "qs", "qe", "rev", "dp_max", "dp_max2", "score", "subsc", "n_cigar")


def ref_matesw(ref, opt, dir, lo, hi, tid, h_ts, h_te, h_rev, r0, seq_fwd, seq_rc, mt0, min_sc):
    """The reference's own mb_matesw_core for one permitted orientation (pe.c:323-377), with
    mb_update_extra left out; returns None (no hit) or the hit's fields and CIGAR."""
    L = refpe_lib()
    sc = np.array([opt[k] for k in RESCUE_SC], np.int32)
    keep, args = _l2b_args(ref)
    f = np.ascontiguousarray(seq_fwd, np.uint8).copy()
    r = np.ascontiguousarray(seq_rc, np.uint8).copy()
    out = np.zeros(11, np.int64)
    cig = np.zeros(len(f) * 2 + 16, np.uint32)
    rc = L.refpe_matesw(*args, _p(sc), dir, lo, hi, tid, h_ts, h_te, h_rev, r0, len(f), _p(f), _p(r), mt0, min_sc, _p(out),
                        _p(cig), len(cig))
    if rc != 0:
        raise RuntimeError("CIGAR buffer too small")
    if out[10] == 0 and out[0] == 0:
        return None
    d = {k: int(v) for k, v in zip(HIT_FIELDS, out)}
    d["cigar"] = [int(x) for x in cig[:d["n_cigar"]]]
    return d


def rescue_window(dir, lo, hi, h_ts, h_te, h_rev, r0, qlen, ctg_len):
    """The candidate window and read orientation of one orientation dir (pe.c:330-339)."""
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


def gen_nt4_mat(a, b, b_ts, b_ambi, mt=0):
    """ksw_gen_nt4_mat (ksw2.h:199-219), int8 arguments as there."""
    a, b, b_ts, b_ambi = (int(np.int8(x)) for x in (a, b, b_ts, b_ambi))
    a, b, b_ambi = abs(a), -abs(b), -abs(b_ambi)
    mat = np.zeros(25, np.int8)
    for i in range(4):
        for j in range(4):
            mat[i * 5 + j] = a if i == j else b
        mat[i * 5 + 4] = b_ambi
    mat[20:25] = b_ambi
    if b_ts != 0 and b_ts != b:
        mat[2] = mat[8] = mat[10] = mat[16] = -abs(b_ts)
    if mt == 1:
        mat[8] = a
    elif mt == 2:
        mat[10] = a
    return mat


def rescue(ref, opt, tid, ts, te, query, meth, min_sc, rev):
    """One rescue candidate through the oracle's restatements: l2b_getseq, mb_ungap, the
    narrowing and thresholds of pe.c:347-353, ksw_ll with the matrix scaled by a and extz2 on
    the reversed prefixes (pe.c:249-300), the hit as pe.c:291-304 and 361-368 derive it.
    Returns the fields of ksw2g_rescue_result_t that the device pipeline fills, and the CIGAR."""
    o = opt
    q = np.ascontiguousarray(query, np.uint8)
    qlen = len(q)
    ref_seq = l2b_getseq(ref, tid, ts, te - ts)
    max_ug, max_i, n_good, n_kmer = ungap(q, ref_seq, 7, meth)
    out = dict(max_ug=max_ug, max_i=max_i, n_good=n_good, n_kmer=n_kmer, ts2=ts, te2=te, ll_done=0, ext_done=0,
               rescued=0, cigar=[])
    ts2, te2 = ts, te
    if max_ug >= 10 and max_ug >= qlen >> 1 and n_good == 1:
        ts2 = ts + max_i - qlen // 2
        te2 = ts2 + qlen * 2
        ts2, te2 = max(ts2, ts), min(te2, te)
    out["ts2"], out["te2"] = ts2, te2
    if not (max_ug >= 10 or max_ug >= n_kmer * 0.33):
        return out
    t = ref_seq[ts2 - ts:te2 - ts]
    max_sc = min(qlen, len(t))
    if max_sc >= 32767:
        return out
    a = o["a"]
    b_mm = (o["b"] + a - 1) // a
    mat = gen_nt4_mat(1, b_mm, (o["b_ts"] + a - 1) // a, (o["b_ambi"] + a - 1) // a, meth)
    size = 1 if max_sc < 255 - b_mm else 2
    r, _ = ll(size, q, t, 5, mat, (o["q"] + a - 1) // a, (o["e"] + a - 1) // a, 0x40000 | o["min_len"])
    out.update(ll_done=1, ll_score=r["score"], ll_te=r["te"], ll_qe=r["qe"], ll_score2=r["score2"], ll_te2=r["te2"])
    if not (r["score"] >= o["min_dp_max"] and r["score"] >= min_sc):
        return out
    qe, te_ = r["qe"] + 1, r["te"] + 1
    flag = 0x40 | 0x02 | 0x80 | (0x04 if meth else 0)  # EXTZ_ONLY | RIGHT | REV_CIGAR (| GENERIC_SC)
    mat = gen_nt4_mat(a, o["b"], o["b_ts"], o["b_ambi"], meth)
    ez, _ = extz(0, q[:qe][::-1], t[:te_][::-1], 5, mat, o["q"], o["e"], o["q"], o["e"], o["bw"], o["zdrop"],
                 o["end_bonus"], flag)
    out["ext_done"] = 1
    out["ext"] = ez
    out["cigar"] = ez["cigar"]
    if ez["n_cigar"] > 0 and ez["max"] >= o["min_dp_max"] * a:
        qs = qe - (qe if ez["reach_end"] else ez["max_q"] + 1)
        qe2 = qe
        hts = ts2 + te_ - (ez["mqe_t"] + 1 if ez["reach_end"] else ez["max_t"] + 1)
        d2 = int(np.int32(int(np.float64(ez["max"]) / r["score"] * r["score2"] + .499)))
        if rev:
            qs, qe2 = qlen - qe2, qlen - qs
        out.update(rescued=1, ts=hts, te=ts2 + te_, qs=qs, qe=qe2, dp_max2=max(d2, 0))
    return out


def rescue_batch(ref, opt, jobs, qbuf, nthreads=1):
    """The C restatement of the rescue (rescue_cpu.c) over a batch of candidates on nthreads
    threads; returns (results in the ksw2g_rescue_result_t layout, CIGAR words)."""
    L = oracle_lib()
    o = np.array([opt[k] for k in RESCUE_SC], np.int32)
    jobs = np.ascontiguousarray(jobs).view(ORC_RESCUE_JOB) if len(jobs) else np.zeros(0, ORC_RESCUE_JOB)
    res = np.zeros(len(jobs), ORC_RESCUE_RES)
    cap = int((jobs["qlen"].astype(np.int64) + jobs["te"] - jobs["ts"] + 1).sum()) + 1
    cig = np.zeros(cap, np.uint32)
    amb = np.ascontiguousarray(ref.ambi, np.uint64).reshape(-1)
    q = np.ascontiguousarray(qbuf, np.uint8)
    pac = np.ascontiguousarray(ref.pac, np.uint64)
    off = np.ascontiguousarray(ref.ctg_off, np.uint64)
    rc = L.orc_rescue_batch(_p(o), len(jobs), _p(jobs), _p(q), _p(pac), _p(off), len(amb) // 2,
                            _p(amb) if len(amb) else None, _p(res), _p(cig), cap, int(nthreads))
    if rc < 0:
        raise RuntimeError("CIGAR buffer too small")
    return res, cig


ALIGN_SC = ("a", "b", "b_ts", "b_ambi", "q", "e", "q2", "e2", "meth")
ALIGN_OUT = ("max", "zdropped", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "score", "n_cigar", "reach_end")


def ref_align_pair(opt, mat, query, target, w, end_bonus, zdrop, flag):
    """The reference's own mb_align_pair (align.c:329-390) through _ref/libmbpe.so."""
    L = refpe_lib()
    if not hasattr(L, "_refal"):
        L.refal_align_pair.restype = C.c_int
        L.refal_align_pair.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        L._refal = True
    sc = np.array([int(opt[k]) for k in ALIGN_SC], np.int32)
    q = np.ascontiguousarray(query, np.uint8)
    t = np.ascontiguousarray(target, np.uint8)
    m = np.ascontiguousarray(mat, np.int8)
    out = np.zeros(11, np.int32)
    cig = np.zeros(len(q) + len(t) + 8, np.uint32)
    rc = L.refal_align_pair(_p(sc), int(opt.get("max_sw_mat", 0)), len(q), _p(q) if len(q) else None, len(t),
                            _p(t) if len(t) else None, _p(m), w, end_bonus, zdrop, flag, _p(out), _p(cig), len(cig))
    if rc:
        raise RuntimeError("CIGAR buffer too small")
    d = {k: int(v) for k, v in zip(ALIGN_OUT, out)}
    d["cigar"] = [int(x) for x in cig[:d["n_cigar"]]]
    return d


def align_pair(opt, mat, query, target, w, end_bonus, zdrop, flag):
    """mb_align_pair (align.c:329-390) restated over the oracle's extz2/extd2: the ungapped
    shortcuts, the band shrink of short pairs, the memory cap, then the DP call."""
    a, b, b_ts, q, e, q2, e2 = (int(opt[k]) for k in ("a", "b", "b_ts", "q", "e", "q2", "e2"))
    qs = np.ascontiguousarray(query, np.uint8)
    ts = np.ascontiguousarray(target, np.uint8)
    mat = np.ascontiguousarray(mat, np.int8)
    qlen, tlen = len(qs), len(ts)
    if (b_ts != 0 and b != b_ts) or opt.get("meth", 0):
        flag |= 0x04
    neg = -0x40000000
    reset = dict(max=0, zdropped=0, max_q=-1, max_t=-1, mqe=neg, mqe_t=-1, mte=neg, mte_q=-1, score=neg, n_cigar=0,
                 reach_end=0, cigar=[])
    n_mm = -1
    if (flag & 0x40) and tlen >= qlen:
        r = dict(reset)
        score = mx = 0
        for j in range(qlen):
            s = int(mat[ts[j] * 5 + qs[j]])
            score += s
            n_mm += int(ts[j] > 3 or qs[j] > 3 or s < 0)
            if mx < score:
                mx, r["max_q"], r["max_t"] = score, j, j
        r["score"], r["max"] = score, mx
        if n_mm <= 2:
            r["mqe"], r["mqe_t"] = score, qlen - 1
            if r["mqe"] + end_bonus >= r["max"]:
                r.update(reach_end=1, n_cigar=1, cigar=[qlen << 4])
                return r
    elif qlen == tlen and not (flag & 0x40):
        r = dict(reset)
        score = 0
        for j in range(qlen):
            s = int(mat[ts[j] * 5 + qs[j]])
            score += s
            n_mm += int(ts[j] > 3 or qs[j] > 3 or s < 0)
        r["score"] = score
        if n_mm <= 3 or score > (qlen - 2) * a - 2 * (q + e):
            r.update(n_cigar=1, cigar=[qlen << 4])
            return r
    if n_mm >= 0 and min(qlen, tlen) < 100:
        x = n_mm * (a + b)
        max1 = (x - q + e - 1) // e if x >= q + e else 0
        max2 = (x - q2 + e2 - 1) // e2 if x >= q2 + e2 else 0
        w = min(w, max(max1, max2) + 4)
    msm = int(opt.get("max_sw_mat", 0))
    if msm > 0 and tlen * qlen > msm:
        r = dict(reset)
        r["zdropped"] = 1
        return r
    dual = not (q == q2 and e == e2)
    ez, _ = extz(int(dual), qs, ts, 5, mat, q, e, q2, e2, w, zdrop * a, end_bonus, flag)
    return {k: ez[k] for k in ALIGN_OUT + ("cigar",)}
