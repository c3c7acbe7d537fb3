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


def build_minibwa_stock():
    """Compile the reference's minibwa from its sources, stock (oracle/_ref/minibwa_stock); needs a
    reference tree."""
    t = ref_tree()
    if not t:
        raise RuntimeError("no reference tree: set KSW2_REF_TREE or stage one (make -C oracle stage REF=...)")
    subprocess.check_call(["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", "_ref/minibwa_stock", f"REF={t}"])
    return os.path.join(HERE, "_ref", "minibwa_stock")


def build_mbgstub():
    """Compile the batched minibwa against _ref/libmbgstub.so (ksw2g_align_chains by the
    reference's own mb_align1 on the CPU) and the stock minibwa; needs a reference tree.
    Returns the paths of both (libc builds)."""
    t = ref_tree()
    if not t:
        raise RuntimeError("no reference tree: set KSW2_REF_TREE or stage one (make -C oracle stage REF=...)")
    j = f"-j{os.cpu_count() or 4}"
    subprocess.check_call(["make", "-s", "-C", HERE, j, "mbgstub", "_ref/minibwa_stock", f"REF={t}"])
    return dict(stock=os.path.join(HERE, "_ref", "minibwa_stock"),
                batch=os.path.join(HERE, "_ref", "mbgstub", "minibwa_batch"))


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


CHAIN_OPT = ("a", "b", "b_ts", "b_ambi", "q", "e", "q2", "e2", "bw", "bw_long", "max_gap", "end_bonus", "zdrop",
             "zdrop_inv", "min_ksw_len", "min_len", "min_chain_score", "min_dp_max", "long_reads", "adaptive",
             "max_sr_len", "meth", "max_sw_mat")
ALIGN1_OUT = ("ts", "te", "qs", "qe", "dp_score", "n_cigar", "cnt", "score", "r2_cnt", "r2_as", "r2_split_inv",
              "r2_score")


def ref_align1(ref, opt, anchors, chain, seq_fwd, seq_rc):
    """The reference's own mb_align1 (align.c:548-760) on one hit through _ref/libmbpe.so, with
    mb_update_extra left out; `anchors` is the whole anchor array (mb_align1 filters a copy of
    the hit's range in place), `chain` one ksw2g_chain_t-shaped record."""
    L = refpe_lib()
    if not hasattr(L, "_refal1"):
        L.refal_align1.restype = C.c_int
        L.refal_align1.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int64, C.c_void_p,
                                   C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                   C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_int]
        L._refal1 = True
    keep, args = _l2b_args(ref)
    optv = np.array([int(opt[k]) for k in CHAIN_OPT], np.int64)
    a = np.ascontiguousarray(anchors)
    ai = np.ascontiguousarray(np.stack([a["sid"], a["len"], a["qpos"], a["flag"].astype(np.int32)], 1), np.int32)
    at = np.ascontiguousarray(a["tpos"], np.int64)
    f = np.ascontiguousarray(seq_fwd, np.uint8).copy()
    r = np.ascontiguousarray(seq_rc, np.uint8).copy()
    out = np.zeros(len(ALIGN1_OUT), np.int64)
    cig = np.zeros(2 * len(f) + 64 + 4 * int(chain["cnt"]), np.uint32)
    rc = L.refal_align1(*args, _p(optv), len(f), _p(f), _p(r), int(chain["meth"]), len(a), _p(ai), _p(at),
                        int(chain["as"]), int(chain["cnt"]), int(chain["mlen"]), int(chain["score"]),
                        int(chain["split_inv"]), _p(out), _p(cig), len(cig))
    if rc:
        raise RuntimeError("CIGAR buffer too small")
    d = {k: int(v) for k, v in zip(ALIGN1_OUT, out)}
    d["cigar"] = [int(x) for x in cig[:d["n_cigar"]]]
    return d


def _max_stretch(a):
    """mb_max_stretch (align.c:522-546) over the hit's anchors a[0..cnt)."""
    if len(a) < 2:
        return 0, len(a)
    best, best_i, best_len, score, ln = -1, -1, 0, int(a[0]["len"]), 1
    for i in range(1, len(a)):
        lr, lq = int(a[i]["tpos"] - a[i - 1]["tpos"]), int(a[i]["qpos"] - a[i - 1]["qpos"])
        if lq == lr:
            score += min(lq, int(a[i]["len"]))
            ln += 1
        else:
            if score > best:
                best, best_len, best_i = score, ln, i - ln
            score, ln = int(a[i]["len"]), 1
    if score > best:
        best, best_len, best_i = score, ln, len(a) - ln
    return best_i, best_len


def _gap(a, i):
    return int(a[i]["qpos"] - a[i - 1]["qpos"]) - int(a[i]["tpos"] - a[i - 1]["tpos"])


def _fix_bad_ends(a, mlen, bw, min_match):
    """mm_fix_bad_ends (align.c:486-520)."""
    cnt = len(a)
    if cnt < 3:
        return 0, cnt
    as1 = 0
    m = l = int(a[0]["len"])
    for i in range(1, cnt - 1):
        if a[i]["flag"] & 1:
            break
        lr, lq, span = int(a[i]["tpos"] - a[i - 1]["tpos"]), int(a[i]["qpos"] - a[i - 1]["qpos"]), int(a[i]["len"])
        mn, mx = min(lr, lq), max(lr, lq)
        if mx - mn > l >> 1:
            as1 = i
        l += mn
        m += min(mn, span)
        if l >= bw << 1 or (m >= min_match and m >= bw) or m >= mlen >> 1:
            break
    cnt1 = cnt - as1
    m = l = int(a[cnt - 1]["len"])
    for i in range(cnt - 2, as1, -1):
        if a[i + 1]["flag"] & 1:
            break
        lr = int(a[i + 1]["tpos"] - a[i]["tpos"] - a[i + 1]["len"] + a[i]["len"])
        lq = int(a[i + 1]["qpos"] - a[i]["qpos"] - a[i + 1]["len"] + a[i]["len"])
        mn, mx, span = min(lr, lq), max(lr, lq), int(a[i]["len"])
        if mx - mn > l >> 1:
            cnt1 = i + 1 - as1
        l += mn
        m += min(mn, span)
        if l >= bw << 1 or (m >= min_match and m >= bw) or m >= mlen >> 1:
            break
    return as1, cnt1


def _long_gaps(b, min_gap):
    k = [i for i in range(1, len(b)) if abs(_gap(b, i)) > min_gap]
    return k if len(k) > 1 else []


def _filter_bad_seeds(b, min_gap, diff_thres, max_ext_len, max_ext_cnt):
    """mm_filter_bad_seeds (align.c:411-447) on the view b = a[as1:as1+cnt1] (flags set in place)."""
    K = _long_gaps(b, min_gap)
    n, mx, st, en, k = len(K), 0, -1, -1, 0
    if not K:
        return
    while True:
        if k == n or k >= en:
            if en > 0:
                for i in range(K[st], K[en]):
                    b[i]["flag"] |= 2
            mx, st, en = 0, -1, -1
            if k == n:
                break
        i = K[k]
        n_ins = n_del = max_diff = 0
        max_diff_l = -1
        g = _gap(b, i)
        n_ins, n_del = (g, 0) if g > 0 else (0, -g)
        qs, ts = int(b[i - 1]["qpos"]), int(b[i - 1]["tpos"])
        for l in range(k + 1, min(n, k + max_ext_cnt + 1)):
            j = K[l]
            if int(b[j]["qpos"] - b[j]["len"]) - qs > max_ext_len or int(b[j]["tpos"] - b[j]["len"]) - ts > max_ext_len:
                break
            g = _gap(b, j)
            if g > 0:
                n_ins += g
            else:
                n_del -= g
            diff = n_ins + n_del - abs(n_ins - n_del)
            if max_diff < diff:
                max_diff, max_diff_l = diff, l
        if max_diff > diff_thres and max_diff > mx:
            mx, st, en = max_diff, k, max_diff_l
        k += 1


def _filter_bad_seeds_alt(b, min_gap, max_ext):
    """mm_filter_bad_seeds_alt (align.c:449-484) on the view b."""
    K = _long_gaps(b, min_gap)
    n, k = len(K), 0
    while k < n:
        i = K[k]
        gap1 = abs(_gap(b, i))
        te1, qe1, left = int(b[i]["tpos"]), int(b[i]["qpos"]), int(b[i]["len"])
        l = k + 1
        while l < n:
            j = K[l]
            if int(b[j]["qpos"]) - qe1 > max_ext or int(b[j]["tpos"]) - te1 > max_ext:
                break
            gap2 = abs(_gap(b, j))
            m = min(int(b[j - 1]["tpos"]) - te1 + left, int(b[j - 1]["qpos"]) - qe1 + left)
            if m > gap1 + gap2:
                break
            te1, qe1, left, gap1 = int(b[j]["tpos"]), int(b[j]["qpos"]), int(b[j]["len"]), gap2
            l += 1
        if l > k + 1:
            for j in range(K[k], K[l - 1]):
                b[j]["flag"] |= 2
            b[K[l - 1]]["flag"] |= 1
        k = l


def _cal_mlen(a):
    """mb_cal_mblen (map-algo.c:133-150), its first value."""
    if len(a) == 0:
        return 0
    mlen = int(a[0]["len"])
    for i in range(1, len(a)):
        sp, tl, ql = int(a[i]["len"]), int(np.int32(a[i]["tpos"]) - np.int32(a[i - 1]["tpos"])), int(a[i]["qpos"] - a[i - 1]["qpos"])
        mlen += sp if tl > sp and ql > sp else min(tl, ql)
    return mlen


def _test_zdrop(opt, qseq, tseq, cigar, mat, is_sr):
    """mm_test_zdrop (align.c:26-68)."""
    score, mx, mi, mj, i, j, mz = 0, -(1 << 31), -1, -1, 0, 0, 0
    pos = [[-1, -1], [-1, -1]]

    def upd(s, ii, jj):
        nonlocal mx, mi, mj, mz
        if s < mx:
            z = mx - s - abs((ii - mi) - (jj - mj)) * opt["e"]
            if z > mz:
                mz, pos[0][0], pos[0][1], pos[1][0], pos[1][1] = z, mi, ii, mj, jj
        else:
            mx, mi, mj = s, ii, jj
    for c in cigar:
        op, ln = c & 0xf, c >> 4
        if op == 0:
            for l in range(ln):
                score += int(mat[int(tseq[i + l]) * 5 + int(qseq[j + l])])
                upd(score, i + l, j + l)
            i += ln
            j += ln
        elif op in (1, 2, 3):
            score -= opt["q"] + opt["e"] * ln
            if op == 1:
                j += ln
            else:
                i += ln
            upd(score, i, j)
    q_len, t_len = pos[1][1] - pos[1][0], pos[0][1] - pos[0][0]
    if not is_sr and mz > opt["zdrop_inv"] and q_len < opt["max_gap"] and t_len < opt["max_gap"]:
        q2 = np.array([4 if qseq[pos[1][1] - x - 1] >= 4 else 3 - qseq[pos[1][1] - x - 1] for x in range(q_len)],
                      np.uint8)
        r, _ = ll(2, q2, tseq[pos[0][0]:pos[0][0] + t_len], 5, mat, opt["q"], opt["e"], 0)
        if r["score"] >= opt["min_chain_score"] * opt["a"] and r["score"] >= opt["min_dp_max"] * opt["a"]:
            return 2
    return 1 if mz > opt["zdrop"] else 0


def _append(cg, add):
    """mb_append_cigar (align.c:300-314)."""
    if not add:
        return
    if cg and (cg[-1] & 0xf) == (add[0] & 0xf):
        cg[-1] += add[0] >> 4 << 4
        cg.extend(add[1:])
    else:
        cg.extend(add)


def align1(ref, opt, anchors, chain, seq):
    """mb_align1 (align.c:548-757) restated over the oracle's mb_align_pair and ksw_ll, up to
    mb_update_extra: `seq` is the read in the orientation aligned (seq[rev]), `anchors` the
    whole anchor array.  Returns the dict ref_align1 returns."""
    opt = {k: int(v) for k, v in opt.items()}
    a = np.array(anchors[int(chain["as"]):int(chain["as"]) + int(chain["cnt"])], copy=True)
    qseq = np.ascontiguousarray(seq, np.uint8)
    qlen, cnt = len(qseq), int(chain["cnt"])
    rev, tid = int(a[0]["sid"]) & 1, int(a[0]["sid"]) >> 1
    ctg_len = int(ref.ctg_len[tid])
    mt = int(chain["meth"])
    mt = meth_rev(mt) if rev else mt
    is_sr = not (opt["long_reads"] or (opt["adaptive"] and qlen > opt["max_sr_len"]))
    max_back = 0 if is_sr else 10
    mat = gen_nt4_mat(opt["a"], opt["b"], opt["b_ts"], opt["b_ambi"], mt)
    bw = int(opt["bw"] * 1.5 + 1.)
    bw_long = max(int(opt["bw_long"] * 1.5 + 1.), bw) if not is_sr else bw
    if is_sr:
        as1, cnt1 = _max_stretch(a)
    else:
        as1, cnt1 = _fix_bad_ends(a, int(chain["mlen"]), opt["bw"], opt["min_chain_score"] * 2)
        _filter_bad_seeds(a[as1:as1 + cnt1], 10, 40, opt["max_gap"] >> 1, 10)
        _filter_bad_seeds_alt(a[as1:as1 + cnt1], 30, opt["max_gap"] >> 1)
    A = lambda i: (int(a[i]["tpos"]), int(a[i]["qpos"]), int(a[i]["len"]), int(a[i]["flag"]))  # noqa: E731
    tp, qp, ln, _ = A(as1)
    ts, qs = tp + 1 - ln + min(ln >> 1, max_back), qp + 1 - ln + min(ln >> 1, max_back)
    tp, qp, ln, _ = A(as1 + cnt1 - 1)
    te, qe = tp + 1 - min(ln >> 1, max_back), qp + 1 - min(ln >> 1, max_back)
    ea = lambda l, bonus: l + ((l * opt["a"] + bonus - opt["q"]) // opt["e"] if l * opt["a"] + bonus > opt["q"] else 0)  # noqa: E731
    if is_sr:
        qs0, qe0 = 0, qlen
        ts0 = max(ts - ea(qs, opt["end_bonus"]), 0)
        te0 = min(te + ea(qlen - qe, opt["end_bonus"]), ctg_len)
    else:
        ts0, qs0 = max(A(0)[0] + 1 - A(0)[2], 0), A(0)[1] + 1 - A(0)[2]
        if qs > 0 and ts > 0:
            l = min(qs, opt["max_gap"])
            qs0 = min(qs0, max(0, qs - l))
            l = min(ea(l, 0), opt["max_gap"], ts)
            ts0 = min(ts0, max(0, ts - l), ts)
        else:
            ts0, qs0 = ts, qs
        te0, qe0 = A(cnt - 1)[0] + 1, A(cnt - 1)[1] + 1
        if qe < qlen and te < ctg_len:
            l = min(qlen - qe, opt["max_gap"])
            qe0 = max(qe0, min(qlen, qe + l))
            l = min(ea(l, 0), opt["max_gap"], ctg_len - te)
            te0 = max(te0, min(ctg_len, te + l))
        else:
            te0, qe0 = te, qe
    tgt = lambda s, e: l2b_getseq(ref, tid, s, e - s)  # noqa: E731
    cg, dp, dropped = [], 0, False
    out = dict(r2_cnt=0, r2_as=0, r2_split_inv=0, r2_score=0, cnt=cnt, score=int(chain["score"]))
    if qs > 0 and ts > 0:
        ez = align_pair(opt, mat, qseq[qs0:qs][::-1], tgt(ts0, ts)[::-1], bw, opt["end_bonus"],
                        opt["zdrop_inv"] if chain["split_inv"] else opt["zdrop"], 0x40 | 0x02 | 0x80)
        if ez["n_cigar"] > 0:
            _append(cg, ez["cigar"])
            dp += ez["mqe"] if ez["reach_end"] else ez["max"]
        ts1 = ts - (ez["mqe_t"] + 1 if ez["reach_end"] else ez["max_t"] + 1)
        qs1 = qs - (qs - qs0 if ez["reach_end"] else ez["max_q"] + 1)
    else:
        ts1, qs1 = ts, qs
    tp, qp, ln, _ = A(as1)
    te = te1 = tp + 1 - min(ln >> 1, max_back)
    qe = qe1 = qp + 1 - min(ln >> 1, max_back)
    _append(cg, [(te - ts) << 4])
    dp += opt["a"] * (te - ts)
    ts, qs = te, qe
    for i in range(1, cnt1):
        tp, qp, ln, fl = A(as1 + i)
        if (fl & 2) and i != cnt1 - 1:
            continue
        te1, qe1 = tp + 1 - min(ln >> 1, max_back), qp + 1 - min(ln >> 1, max_back)
        if not (i == cnt1 - 1 or (fl & 1) or (qe1 - qs >= opt["min_ksw_len"] and te1 - ts >= opt["min_ksw_len"])):
            continue
        d1 = 0
        if ln > opt["min_len"] * 2:
            d1 = min(te1 - (tp + 1 - ln), qe1 - qs, te1 - ts) - opt["min_len"]
            d1 = 0 if d1 < opt["min_len"] else d1
        te, qe = te1 - d1, qe1 - d1
        bw1 = max(qe - qs, te - ts) if fl & 1 else bw_long
        qg, tg = qseq[qs:qe], tgt(ts, te)
        ez = align_pair(opt, mat, qg, tg, bw1, -1, opt["zdrop"], 0x08)  # first pass: approximate maximum
        code = _test_zdrop(opt, qg, tg, ez["cigar"], mat, is_sr)
        if code:
            ez = align_pair(opt, mat, qg, tg, bw1, -1, opt["zdrop_inv"] if code == 2 else opt["zdrop"], 0)
        if ez["n_cigar"] > 0:
            _append(cg, ez["cigar"])
        if ez["zdropped"]:
            j = i - 1
            while j >= 0 and int(a[as1 + j]["tpos"]) > ts + ez["max_t"]:
                j -= 1
            j = max(j, 0)
            dropped = True
            dp += ez["max"]
            te1, qe1 = ts + ez["max_t"] + 1, qs + ez["max_q"] + 1
            if _cal_mlen(a[as1 + j + 1:as1 + cnt1]) >= opt["min_chain_score"]:
                n = as1 + j + 1  # mb_split_hit (map-algo.c:247-264)
                if 0 < n < cnt:
                    c2 = cnt - n
                    s2 = int(float(np.float32(np.float32(chain["score"]) * (np.float32(c2) / np.float32(cnt)))) + .499)
                    out.update(r2_cnt=c2, r2_as=int(chain["as"]) + n, r2_score=s2, cnt=cnt - c2,
                               score=int(chain["score"]) - s2, r2_split_inv=int(code == 2))
            break
        dp += ez["score"]
        if d1 > 0:
            _append(cg, [d1 << 4])
            dp += opt["a"] * d1
            te, qe = te1, qe1
        ts, qs = te, qe
    if not dropped and qe < qe0 and te < te0:
        ez = align_pair(opt, mat, qseq[qe:qe0], tgt(te, te0), bw, opt["end_bonus"], opt["zdrop"], 0x40)
        if ez["n_cigar"] > 0:
            _append(cg, ez["cigar"])
            dp += ez["mqe"] if ez["reach_end"] else ez["max"]
        te1 = te + (ez["mqe_t"] + 1 if ez["reach_end"] else ez["max_t"] + 1)
        qe1 = qe + (qe0 - qe if ez["reach_end"] else ez["max_q"] + 1)
    out.update(ts=ts1, te=te1, dp_score=dp, n_cigar=len(cg), cigar=cg)
    out.update(qs=qlen - qe1 if rev else qs1, qe=qlen - qs1 if rev else qe1)
    return out
