"""ctypes binding of the checker libraries (TEST INFRASTRUCTURE ONLY).

  liboracle.so        scalar C restatement of the reference (ksw2_oracle.c), builds anywhere
  _ref/libksw2ref.so  the reference's own ksw2 SSE sources, built here from the reference
                      tree when it is present (never on a machine without it)

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this module,
and only as the checker / the timed CPU baseline -- never as a product code path.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_TREE = os.environ.get("KSW2_REF_TREE", "/root/reference")
LIB_ORACLE = os.path.join(HERE, "liboracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libksw2ref.so")

ORC_JOB = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"),
                    ("w", "<i4"), ("zdrop", "<i4"), ("end_bonus", "<i4"), ("flag", "<i4")])
ORC_RES = np.dtype([("score", "<i4"), ("max", "<i4"), ("max_q", "<i4"), ("max_t", "<i4"),
                    ("mqe", "<i4"), ("mqe_t", "<i4"), ("mte", "<i4"), ("mte_q", "<i4"),
                    ("zdropped", "<i4"), ("reach_end", "<i4"), ("n_cigar", "<i4"), ("n_diag", "<i4"),
                    ("cigar_off", "<i8")])
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


def build(ref=True):
    """Compile liboracle.so (and _ref/libksw2ref.so when the reference tree exists)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    if ref and os.path.isdir(REF_TREE):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", f"REF={REF_TREE}"])


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
    _libs[path] = L
    return L


def oracle_lib():
    if not os.path.exists(LIB_ORACLE):
        build(ref=False)
    return _load(LIB_ORACLE, "orc_")


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
