"""ctypes binding of libksw2gpu.so.

Two surfaces:
  * the reference-shaped per-call functions (ksw_extz2_sse, ksw_extd2_sse, ksw_ll_*),
    with the same argument meaning and results as ksw2.h of the reference;
  * the batched API (Context, ExtBatch, LLBatch) over include/ksw2_gb300.h.
"""
import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))

KSW_NEG_INF = -0x40000000
KSW_EZ_SCORE_ONLY = 0x01
KSW_EZ_RIGHT = 0x02
KSW_EZ_GENERIC_SC = 0x04
KSW_EZ_APPROX_MAX = 0x08
KSW_EZ_APPROX_DROP = 0x10
KSW_EZ_EXTZ_ONLY = 0x40
KSW_EZ_REV_CIGAR = 0x80
KSW_LL_STOP = 0x20000
KSW_LL_SUBO = 0x40000

# include/ksw2_gb300.h layouts
KSW2G_E_CAPACITY = -5  # caller's output buffer too small (include/ksw2_gb300.h)

EXT_JOB = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"),
                    ("w", "<i4"), ("zdrop", "<i4"), ("end_bonus", "<i4"), ("flag", "<i4")])
EXT_RESULT = np.dtype([("score", "<i4"), ("max", "<i4"), ("max_q", "<i4"), ("max_t", "<i4"),
                       ("mqe", "<i4"), ("mqe_t", "<i4"), ("mte", "<i4"), ("mte_q", "<i4"),
                       ("zdropped", "<i4"), ("reach_end", "<i4"), ("n_cigar", "<i4"), ("n_diag", "<i4"),
                       ("cigar_off", "<i8"), ("cells", "<i8")])
LL_JOB = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"),
                   ("xtra", "<i4"), ("pad", "<i4")])
LL_RESULT = np.dtype([("score", "<i4"), ("te", "<i4"), ("qe", "<i4"), ("score2", "<i4"),
                      ("te2", "<i4"), ("rows", "<i4")])
assert EXT_JOB.itemsize == 40 and EXT_RESULT.itemsize == 64 and LL_JOB.itemsize == 32 and LL_RESULT.itemsize == 24
ALIGN_OPT = np.dtype([(k, "<i4") for k in ("a", "b", "b_ts", "b_ambi", "q", "e", "q2", "e2", "meth", "pad")]
                     + [("max_sw_mat", "<i8")])
RESCUE_OPT = np.dtype([(k, "<i4") for k in ("a", "b", "b_ts", "b_ambi", "q", "e", "bw", "zdrop", "end_bonus",
                                            "min_len", "min_dp_max")])
RESCUE_JOB = np.dtype([("qoff", "<i8"), ("ts", "<i8"), ("te", "<i8"), ("qlen", "<i4"), ("tid", "<i4"),
                       ("meth", "<i4"), ("min_sc", "<i4"), ("rev", "<i4"), ("pad", "<i4")])
RESCUE_RESULT = np.dtype([("max_ug", "<i4"), ("max_i", "<i4"), ("n_good", "<i4"), ("n_kmer", "<i4"),
                          ("ts2", "<i8"), ("te2", "<i8"),
                          ("ll_done", "<i4"), ("ll_score", "<i4"), ("ll_te", "<i4"), ("ll_qe", "<i4"),
                          ("ll_score2", "<i4"), ("ll_te2", "<i4"), ("ext_done", "<i4"), ("rescued", "<i4"),
                          ("qs", "<i4"), ("qe", "<i4"), ("dp_max2", "<i4"), ("pad", "<i4"),
                          ("ts", "<i8"), ("te", "<i8"), ("ext", EXT_RESULT)])
assert RESCUE_OPT.itemsize == 44 and RESCUE_JOB.itemsize == 48 and RESCUE_RESULT.itemsize == 160


# ksw2g_anchor_t / ksw2g_chain_t / ksw2g_chain_opt_t / ksw2g_chain_result_t (include/ksw2_gb300.h)
ANCHOR = np.dtype([("sid", "<i4"), ("len", "<i4"), ("qpos", "<i4"), ("flag", "<u4"), ("tpos", "<i8")])
CHAIN = np.dtype([("as", "<i8"), ("qoff", "<i8")] + [(k, "<i4") for k in ("cnt", "mlen", "score", "qlen", "meth",
                                                                          "split_inv", "opt", "pad")])
CHAIN_OPT = np.dtype([(k, "<i4") for k in ("a", "b", "b_ts", "b_ambi", "q", "e", "q2", "e2", "bw", "bw_long",
                                             "max_gap", "end_bonus", "zdrop", "zdrop_inv", "min_ksw_len", "min_len",
                                             "min_chain_score", "min_dp_max", "long_reads", "adaptive", "max_sr_len",
                                             "meth")] + [("max_sw_mat", "<i8")], align=True)
CHAIN_RESULT = np.dtype([("ts", "<i8"), ("te", "<i8"), ("qs", "<i4"), ("qe", "<i4"), ("dp_score", "<i4"),
                         ("n_cigar", "<i4"), ("cigar_off", "<i8"), ("cnt", "<i4"), ("score", "<i4"),
                         ("split_n", "<i4"), ("split_inv2", "<i4"), ("n_dp", "<i4"), ("n_dp_issued", "<i4")])


class KswExtz(C.Structure):
    """ksw_extz_t (ksw2.h:36-45)."""
    _fields_ = [("max", C.c_uint32, 31), ("zdropped", C.c_uint32, 1),
                ("max_q", C.c_int), ("max_t", C.c_int), ("mqe", C.c_int), ("mqe_t", C.c_int),
                ("mte", C.c_int), ("mte_q", C.c_int), ("score", C.c_int),
                ("m_cigar", C.c_int), ("n_cigar", C.c_int), ("reach_end", C.c_int),
                ("cigar", C.POINTER(C.c_uint32))]

    def cigar_list(self):
        return [self.cigar[i] for i in range(self.n_cigar)]

    def fields(self):
        return dict(max=self.max, zdropped=self.zdropped, max_q=self.max_q, max_t=self.max_t, mqe=self.mqe,
                    mqe_t=self.mqe_t, mte=self.mte, mte_q=self.mte_q, score=self.score,
                    reach_end=self.reach_end, n_cigar=self.n_cigar, cigar=self.cigar_list())


class KswLLRst(C.Structure):
    """ksw_llrst_t (ksw2.h:47-51)."""
    _fields_ = [("score", C.c_int), ("te", C.c_int), ("qe", C.c_int), ("score2", C.c_int), ("te2", C.c_int)]


def lib_path():
    return os.environ.get("KSW2GPU_LIB", os.path.join(_PKG, "libksw2gpu.so"))


_lib = None


def load_library():
    """Load libksw2gpu.so; raises if it is missing (there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not os.path.exists(p):
        raise RuntimeError(f"libksw2gpu.so not found at {p}: build it with `python -m minibwa_gb300.build`")
    L = C.CDLL(p)
    vp, i32, i64, u8p, i8 = C.c_void_p, C.c_int, C.c_int64, C.c_void_p, C.c_int8
    sig = {
        "ksw2g_ctx_create": (i32, [i32, C.POINTER(vp)]),
        "ksw2g_ctx_destroy": (None, [vp]),
        "ksw2g_ctx_stream": (vp, [vp]),
        "ksw2g_ctx_sync": (i32, [vp]),
        "ksw2g_ctx_set_tb_budget": (i32, [vp, i64]),
        "ksw2g_last_error": (C.c_char_p, []),
        "ksw2g_ext_batch": (i32, [vp, i32, i8, vp, i8, i8, i8, i8, i32, vp, u8p, i64, u8p, i64, vp, vp, i64,
                                  C.POINTER(i64)]),
        "ksw2g_ll_batch": (i32, [vp, i32, i32, vp, i32, i32, i32, vp, u8p, i64, u8p, i64, vp]),
        "ksw2g_ext_prepare": (i32, [vp, i32, i8, vp, i8, i8, i8, i8, i32, vp, u8p, i64, u8p, i64, C.POINTER(vp)]),
        "ksw2g_ll_prepare": (i32, [vp, i32, i32, vp, i32, i32, i32, vp, u8p, i64, u8p, i64, C.POINTER(vp)]),
        "ksw2g_batch_run": (i32, [vp, vp]),
        "ksw2g_ext_fetch": (i32, [vp, vp, vp, vp, i64, C.POINTER(i64)]),
        "ksw2g_ll_fetch": (i32, [vp, vp, vp]),
        "ksw2g_batch_launches": (i32, [vp]),
        "ksw2g_batch_free": (None, [vp]),
        "ksw2g_ext_num_shapes": (i32, []),
        "ksw2g_ext_shape_info": (i32, [i32, C.POINTER(i32), C.POINTER(i32)]),
        "ksw2g_ext_set_shape": (i32, [i32, i32, i32, i32, i32]),
        "ksw2g_ext_set_family": (i32, [i32]),
        "ksw2g_ext_get_family": (i32, []),
        "ksw2g_ext_set_split": (i32, [i32]),
        "ksw2g_ext_get_split": (i32, []),
        "ksw2g_debug_fail_device_alloc": (None, [i32]),
        "ksw2g_probe_int32_peak": (i32, [i32, C.POINTER(C.c_double)]),
        "ksw2g_batch_set_timing": (i32, [vp, i32]),
        "ksw2g_batch_kernel_ms": (i32, [vp, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(i32),
                                        C.POINTER(i32)]),
        "ksw2g_ref_create": (i32, [vp, i64, vp, vp, vp, i64, i64, vp, C.POINTER(vp)]),
        "ksw2g_ref_destroy": (None, [vp]),
        "ksw2g_ref_getseq": (i32, [vp, vp, i64, i64, i64, i32, u8p]),
        "ksw2g_ext_batch_ref": (i32, [vp, vp, i32, i8, vp, i8, i8, i8, i8, i32, vp, vp, vp, u8p, i64, vp, vp, i64,
                                      C.POINTER(i64)]),
        "ksw2g_ext_prepare_ref": (i32, [vp, vp, i32, i8, vp, i8, i8, i8, i8, i32, vp, vp, vp, u8p, i64,
                                        C.POINTER(vp)]),
        "ksw2g_ll_batch_ref": (i32, [vp, vp, i32, i32, vp, i32, i32, i32, vp, vp, vp, u8p, i64, vp]),
        "ksw2g_rescue_batch": (i32, [vp, vp, vp, i32, vp, u8p, i64, vp, vp, i64, vp]),
        "ksw2g_rescue_last_stats": (i32, [vp, vp, vp]),
        "ksw2g_rescue_last_device_ms": (i32, [vp, vp]),
        "ksw2g_align_chains_last_stats": (i32, [vp, vp, vp]),
        "ksw2g_align_chains": (i32, [vp, vp, i32, vp, i32, vp, vp, i64, u8p, i64, vp, vp, i64, C.POINTER(i64)]),
        "ksw2g_align_pairs": (i32, [vp, vp, vp, i32, vp, u8p, i64, u8p, i64, vp, vp, i64, vp]),
        "ksw2g_graph_create": (i32, [vp, i32, C.POINTER(vp), C.POINTER(vp)]),
        "ksw2g_graph_launch": (i32, [vp, vp]),
        "ksw2g_graph_launches": (i32, [vp]),
        "ksw2g_graph_destroy": (None, [vp]),
        "ksw2g_server_create": (i32, [i32, i32, i64, C.POINTER(vp)]),
        "ksw2g_server_destroy": (None, [vp]),
        "ksw2g_server_submit_ext": (i64, [vp, i32, i8, vp, i8, i8, i8, i8, i32, vp, u8p, i64, u8p, i64, vp, vp, i64]),
        "ksw2g_server_submit_ll": (i64, [vp, i32, i32, vp, i32, i32, i32, vp, u8p, i64, u8p, i64, vp]),
        "ksw2g_server_wait": (i32, [vp, i64, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(i64)]),
        "ksw2g_server_stats": (i32, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]),
        "ksw2g_server_launch_stats": (i32, [vp, C.POINTER(i64), C.POINTER(i64)]),
        "ksw2g_server_set_merge": (i32, [vp, i32]),
        "ksw_extz2_sse": (None, [vp, i32, u8p, i32, u8p, i8, vp, i8, i8, i32, i32, i32, i32, C.POINTER(KswExtz)]),
        "ksw_extd2_sse": (None, [vp, i32, u8p, i32, u8p, i8, vp, i8, i8, i8, i8, i32, i32, i32, i32,
                                 C.POINTER(KswExtz)]),
        "ksw_ll_qinit": (vp, [vp, i32, i32, u8p, i32, vp]),
        "ksw_ll_u8_core": (KswLLRst, [vp, i32, u8p, i32, i32, i32]),
        "ksw_ll_i16_core": (KswLLRst, [vp, i32, u8p, i32, i32, i32]),
        "ksw_ll_i16": (i32, [vp, i32, u8p, i32, i32, C.POINTER(i32), C.POINTER(i32)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise RuntimeError(f"ksw2gpu error {rc}: {_lib.ksw2g_last_error().decode()}")


def _ptr(a):
    return a.ctypes.data if a is not None else None


_libc = C.CDLL(None)
_libc.free.argtypes = [C.c_void_p]


def gen_nt4_mat(a=2, b=8, b_ts=0, b_ambi=1, mt=0):
    """ksw_gen_nt4_mat (ksw2.h:199-219) as an int8 numpy array of 25."""
    m = 5
    a = abs(a)
    b = -abs(b)
    b_ambi = -abs(b_ambi)
    mat = np.zeros(25, np.int8)
    for i in range(m - 1):
        for j in range(m - 1):
            mat[i * m + j] = a if i == j else b
        mat[i * m + m - 1] = b_ambi
    for j in range(m):
        mat[(m - 1) * m + j] = b_ambi
    if b_ts != 0 and -abs(b_ts) != b:
        bt = -abs(b_ts)
        mat[0 * m + 2] = mat[1 * m + 3] = mat[2 * m + 0] = mat[3 * m + 1] = bt
    if mt == 1:
        mat[1 * m + 3] = a
    elif mt == 2:
        mat[2 * m + 0] = a
    return mat


# ------------------------------------------------------------------ per-call (reference-shaped)
def _u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


def ksw_extz2_sse(query, target, m, mat, q, e, w, zdrop, end_bonus, flag, ez=None):
    L = load_library()
    q_, t_, mat_ = _u8(query), _u8(target), np.ascontiguousarray(mat, np.int8)
    ez = ez if ez is not None else KswExtz()
    L.ksw_extz2_sse(None, len(q_), _ptr(q_), len(t_), _ptr(t_), m, _ptr(mat_), q, e, w, zdrop, end_bonus, flag,
                    C.byref(ez))
    return ez


def ksw_extd2_sse(query, target, m, mat, q, e, q2, e2, w, zdrop, end_bonus, flag, ez=None):
    L = load_library()
    q_, t_, mat_ = _u8(query), _u8(target), np.ascontiguousarray(mat, np.int8)
    ez = ez if ez is not None else KswExtz()
    L.ksw_extd2_sse(None, len(q_), _ptr(q_), len(t_), _ptr(t_), m, _ptr(mat_), q, e, q2, e2, w, zdrop, end_bonus,
                    flag, C.byref(ez))
    return ez


def free_extz(ez):
    if ez.cigar:
        _libc.free(C.cast(ez.cigar, C.c_void_p))
        ez.cigar = None
        ez.m_cigar = 0


def ksw_ll_qinit(size, query, m, mat):
    L = load_library()
    q_, mat_ = _u8(query), np.ascontiguousarray(mat, np.int8)
    return L.ksw_ll_qinit(None, size, len(q_), _ptr(q_), m, _ptr(mat_))


def ll_free(qp):
    _libc.free(qp)


def ksw_ll_u8_core(qp, target, gapo, gape, xtra):
    t_ = _u8(target)
    return load_library().ksw_ll_u8_core(qp, len(t_), _ptr(t_), gapo, gape, xtra)


def ksw_ll_i16_core(qp, target, gapo, gape, xtra):
    t_ = _u8(target)
    return load_library().ksw_ll_i16_core(qp, len(t_), _ptr(t_), gapo, gape, xtra)


def ksw_ll_i16(qp, target, gapo, gape):
    t_ = _u8(target)
    qe, te = C.c_int(), C.c_int()
    s = load_library().ksw_ll_i16(qp, len(t_), _ptr(t_), gapo, gape, C.byref(qe), C.byref(te))
    return s, qe.value, te.value


# ------------------------------------------------------------------ batched API
class Context:
    """One CUDA stream and its device pools (ksw2g_ctx_t)."""

    def __init__(self, device=0, tb_budget=None):
        self.L = load_library()
        h = C.c_void_p()
        _check(self.L.ksw2g_ctx_create(device, C.byref(h)))
        self.h = h
        if tb_budget:
            _check(self.L.ksw2g_ctx_set_tb_budget(self.h, int(tb_budget)))

    @property
    def stream(self):
        return self.L.ksw2g_ctx_stream(self.h)

    def sync(self):
        _check(self.L.ksw2g_ctx_sync(self.h))

    def close(self):
        if self.h:
            self.L.ksw2g_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def ext_batch(self, dual, m, mat, q, e, q2, e2, jobs, qbuf, tbuf):
        """One-shot batch of extension jobs; returns (results, cigar words)."""
        jobs = np.ascontiguousarray(jobs, EXT_JOB)
        qbuf, tbuf, mat = _u8(qbuf), _u8(tbuf), np.ascontiguousarray(mat, np.int8)
        n = len(jobs)
        res = np.zeros(n, EXT_RESULT)
        cap = int(((jobs["qlen"].astype(np.int64) + jobs["tlen"] + 1)).sum()) + 16
        cig = np.zeros(cap, np.uint32)
        used = C.c_int64()
        _check(self.L.ksw2g_ext_batch(self.h, int(dual), m, _ptr(mat), q, e, q2, e2, n, _ptr(jobs), _ptr(qbuf),
                                      len(qbuf), _ptr(tbuf), len(tbuf), _ptr(res), _ptr(cig), cap, C.byref(used)))
        return res, cig[:used.value]

    def align_pairs(self, opt, mat, jobs, qbuf, tbuf):
        """align.c's mb_align_pair over a batch (ksw2g_align_pairs): opt is a dict or ALIGN_OPT
        record; returns (results, cigar words)."""
        if isinstance(opt, dict):
            o = np.zeros(1, ALIGN_OPT)
            for k, v in opt.items():
                o[k] = v
            opt = o
        opt = np.ascontiguousarray(opt, ALIGN_OPT)
        jobs = np.ascontiguousarray(jobs, EXT_JOB)
        qbuf, tbuf, mat = _u8(qbuf), _u8(tbuf), np.ascontiguousarray(mat, np.int8)
        res = np.zeros(len(jobs), EXT_RESULT)
        cap = int(((jobs["qlen"].astype(np.int64) + jobs["tlen"] + 1)).sum()) + 16
        cig = np.zeros(cap, np.uint32)
        used = C.c_int64()
        _check(self.L.ksw2g_align_pairs(self.h, _ptr(opt), _ptr(mat), len(jobs), _ptr(jobs), _ptr(qbuf), len(qbuf),
                                        _ptr(tbuf), len(tbuf), _ptr(res), _ptr(cig), cap, C.byref(used)))
        return res, cig[:used.value]

    def ll_batch(self, size, m, mat, gapo, gape, jobs, qbuf, tbuf):
        jobs = np.ascontiguousarray(jobs, LL_JOB)
        qbuf, tbuf, mat = _u8(qbuf), _u8(tbuf), np.ascontiguousarray(mat, np.int8)
        res = np.zeros(len(jobs), LL_RESULT)
        _check(self.L.ksw2g_ll_batch(self.h, size, m, _ptr(mat), gapo, gape, len(jobs), _ptr(jobs), _ptr(qbuf),
                                     len(qbuf), _ptr(tbuf), len(tbuf), _ptr(res)))
        return res


def set_ext_family(family):
    """Lane width of extension batches prepared from now on: 1 = 16-bit lanes (DPX), 0 = byte
    lanes, -1 = the shape preferences decide.  Returns the previous setting."""
    L = load_library()
    prev = L.ksw2g_ext_get_family()
    _check(L.ksw2g_ext_set_family(int(family)))
    return prev


def set_ext_split(mode):
    """Block-split kernel use for extension batches prepared from now on: -1 the batch decides,
    0 never, 1 wherever a block holds the band.  Returns the previous setting."""
    L = load_library()
    prev = L.ksw2g_ext_get_split()
    _check(L.ksw2g_ext_set_split(int(mode)))
    return prev


def probe_int32_peak(device=0):
    """Measured 32-bit integer lane-ops per second of the device."""
    v = C.c_double()
    _check(load_library().ksw2g_probe_int32_peak(device, C.byref(v)))
    return v.value


class _Batch:
    def __init__(self, ctx):
        self.ctx, self.L, self.h = ctx, ctx.L, C.c_void_p()

    def run(self):
        _check(self.L.ksw2g_batch_run(self.ctx.h, self.h))

    @property
    def launches(self):
        return self.L.ksw2g_batch_launches(self.h)

    def set_timing(self, on=True):
        _check(self.L.ksw2g_batch_set_timing(self.h, int(on)))

    def kernel_ms(self):
        """(DP-kernel ms, backtrack-kernel ms, DP launches, backtrack launches), summed over the runs
        since set_timing(True)."""
        dp, bt, ndp, nbt = C.c_double(), C.c_double(), C.c_int(), C.c_int()
        _check(self.L.ksw2g_batch_kernel_ms(self.h, C.byref(dp), C.byref(bt), C.byref(ndp), C.byref(nbt)))
        return dp.value, bt.value, ndp.value, nbt.value

    def free(self):
        if self.h:
            self.L.ksw2g_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class ExtBatch(_Batch):
    """Resident extension batch: inputs uploaded once, run() enqueues the DP asynchronously."""

    def __init__(self, ctx, dual, m, mat, q, e, q2, e2, jobs, qbuf, tbuf):
        super().__init__(ctx)
        jobs = np.ascontiguousarray(jobs, EXT_JOB)
        qbuf, tbuf, mat = _u8(qbuf), _u8(tbuf), np.ascontiguousarray(mat, np.int8)
        self.n = len(jobs)
        self.cap = int(((jobs["qlen"].astype(np.int64) + jobs["tlen"] + 1)).sum()) + 16
        _check(self.L.ksw2g_ext_prepare(ctx.h, int(dual), m, _ptr(mat), q, e, q2, e2, self.n, _ptr(jobs),
                                        _ptr(qbuf), len(qbuf), _ptr(tbuf), len(tbuf), C.byref(self.h)))

    def fetch(self, res=None, cig=None):
        res = res if res is not None else np.zeros(self.n, EXT_RESULT)
        cig = cig if cig is not None else np.zeros(self.cap, np.uint32)
        used = C.c_int64()
        _check(self.L.ksw2g_ext_fetch(self.ctx.h, self.h, _ptr(res), _ptr(cig), len(cig), C.byref(used)))
        return res, cig[:used.value]


class LLBatch(_Batch):
    def __init__(self, ctx, size, m, mat, gapo, gape, jobs, qbuf, tbuf):
        super().__init__(ctx)
        jobs = np.ascontiguousarray(jobs, LL_JOB)
        qbuf, tbuf, mat = _u8(qbuf), _u8(tbuf), np.ascontiguousarray(mat, np.int8)
        self.n = len(jobs)
        _check(self.L.ksw2g_ll_prepare(ctx.h, size, m, _ptr(mat), gapo, gape, self.n, _ptr(jobs), _ptr(qbuf),
                                       len(qbuf), _ptr(tbuf), len(tbuf), C.byref(self.h)))

    def fetch(self, res=None):
        res = res if res is not None else np.zeros(self.n, LL_RESULT)
        _check(self.L.ksw2g_ll_fetch(self.ctx.h, self.h, _ptr(res)))
        return res


class Reference:
    """A 2-bit reference resident on the device (ksw2g_ref_t), from l2b arrays: pac (uint64, 32
    bases each), contig offsets and lengths, and (n, 2) [st, en) runs of N."""

    def __init__(self, ctx, pac, ctg_off, ctg_len, ambi):
        self.L, self.ctx = ctx.L, ctx
        self._pac = np.ascontiguousarray(pac, np.uint64)
        self._off = np.ascontiguousarray(ctg_off, np.uint64)
        self._len = np.ascontiguousarray(ctg_len, np.uint64)
        self._amb = np.ascontiguousarray(ambi, np.uint64).reshape(-1)
        self.h = C.c_void_p()
        _check(self.L.ksw2g_ref_create(ctx.h, len(self._off), _ptr(self._off), _ptr(self._len), _ptr(self._pac),
                                       len(self._pac), len(self._amb) // 2, _ptr(self._amb) if len(self._amb) else None,
                                       C.byref(self.h)))

    def getseq(self, tid, st, length, flags=0):
        out = np.zeros(max(int(length), 1), np.uint8)
        _check(self.L.ksw2g_ref_getseq(self.ctx.h, self.h, int(tid), int(st), int(length), int(flags), _ptr(out)))
        return out[:int(length)]

    def ext_batch(self, dual, m, mat, q, e, q2, e2, jobs, tid, tflags, qbuf):
        """Extension jobs whose targets are windows (jobs['toff'], jobs['tlen'] of contig tid)."""
        jobs = np.ascontiguousarray(jobs, EXT_JOB)
        tid = np.ascontiguousarray(tid, np.int32)
        tflags = None if tflags is None else np.ascontiguousarray(tflags, np.int32)
        qbuf, mat = _u8(qbuf), np.ascontiguousarray(mat, np.int8)
        res = np.zeros(len(jobs), EXT_RESULT)
        cap = int((jobs["qlen"].astype(np.int64) + jobs["tlen"] + 1).sum()) + 16
        cig = np.zeros(cap, np.uint32)
        used = C.c_int64()
        _check(self.L.ksw2g_ext_batch_ref(self.ctx.h, self.h, int(dual), m, _ptr(mat), q, e, q2, e2, len(jobs),
                                          _ptr(jobs), _ptr(tid), _ptr(tflags), _ptr(qbuf), len(qbuf), _ptr(res),
                                          _ptr(cig), cap, C.byref(used)))
        return res, cig[:used.value]

    def ll_batch(self, size, m, mat, gapo, gape, jobs, tid, tflags, qbuf):
        jobs = np.ascontiguousarray(jobs, LL_JOB)
        tid = np.ascontiguousarray(tid, np.int32)
        tflags = None if tflags is None else np.ascontiguousarray(tflags, np.int32)
        qbuf, mat = _u8(qbuf), np.ascontiguousarray(mat, np.int8)
        res = np.zeros(len(jobs), LL_RESULT)
        _check(self.L.ksw2g_ll_batch_ref(self.ctx.h, self.h, size, m, _ptr(mat), gapo, gape, len(jobs), _ptr(jobs),
                                         _ptr(tid), _ptr(tflags), _ptr(qbuf), len(qbuf), _ptr(res)))
        return res

    def rescue_batch(self, opt, jobs, qbuf):
        """Mate rescue of candidate windows (ksw2g_rescue_batch): opt is a dict or RESCUE_OPT
        record of mb_opt_t scores, jobs a RESCUE_JOB array.  Returns (results, cigar words)."""
        if isinstance(opt, dict):
            o = np.zeros(1, RESCUE_OPT)
            for k, v in opt.items():
                o[k] = v
            opt = o
        opt = np.ascontiguousarray(opt, RESCUE_OPT)
        jobs = np.ascontiguousarray(jobs, RESCUE_JOB)
        qbuf = _u8(qbuf)
        res = np.zeros(len(jobs), RESCUE_RESULT)
        cap = int((jobs["qlen"].astype(np.int64) + jobs["te"] - jobs["ts"] + 1).sum()) + 16
        cig = np.zeros(cap, np.uint32)
        used = C.c_int64()
        _check(self.L.ksw2g_rescue_batch(self.ctx.h, self.h, _ptr(opt), len(jobs), _ptr(jobs), _ptr(qbuf), len(qbuf),
                                         _ptr(res), _ptr(cig), cap, C.byref(used)))
        return res, cig[:used.value]

    def align_chains(self, opts, chains, anchors, qbuf, cigar_cap=None):
        """mb_align1 over many hits at once (ksw2g_align_chains): opts one option set (a dict or
        CHAIN_OPT record) or a list of them that chains["opt"] indexes, chains records with the
        CHAIN fields (extra fields are ignored, missing ones are 0) indexing anchors (ANCHOR; their
        flags are updated in place when it is an ANCHOR array) and qbuf (each read in the
        orientation it aligns in).  Returns (CHAIN_RESULT array, CIGAR words)."""
        if isinstance(opts, dict) or (isinstance(opts, np.ndarray) and opts.dtype == CHAIN_OPT and opts.ndim == 0):
            opts = [opts]
        o = np.zeros(len(opts), CHAIN_OPT)
        for i, x in enumerate(opts):
            for k in CHAIN_OPT.names:
                o[i][k] = x[k]
        ch = np.zeros(len(chains), CHAIN)
        for k in CHAIN.names:
            if chains.dtype.names and k in chains.dtype.names:
                ch[k] = chains[k]
        if not (isinstance(anchors, np.ndarray) and anchors.dtype == ANCHOR and anchors.flags.c_contiguous):
            anchors = np.ascontiguousarray(anchors, ANCHOR)
        qbuf = _u8(qbuf)
        res = np.zeros(len(ch), CHAIN_RESULT)
        grow = cigar_cap is None  # the default bound is a guess: grow it when a hit's CIGAR needs more
        if cigar_cap is None:
            cigar_cap = int(2 * ch["qlen"].astype(np.int64).sum() + 4 * ch["cnt"].astype(np.int64).sum()) + 64
        used = C.c_int64()
        while True:
            cig = np.zeros(max(int(cigar_cap), 1), np.uint32)
            flags = anchors["flag"].copy()
            rc = self.L.ksw2g_align_chains(self.ctx.h, self.h, len(o), _ptr(o), len(ch), _ptr(ch), _ptr(anchors),
                                           len(anchors), _ptr(qbuf), len(qbuf), _ptr(res), _ptr(cig),
                                           int(cigar_cap), C.byref(used))
            if rc != KSW2G_E_CAPACITY or not grow:
                break
            anchors["flag"] = flags  # the call is repeated on the anchors as they were
            cigar_cap *= 2
        _check(rc)
        return res, cig[:used.value]

    def chains_stats(self):
        """(stage ms [derive, gather, pass 1, z-drop tests, pass 2, assembly], counts [hits, pass-1
        jobs, pass-2 jobs, inversion checks]) of the context's last align_chains call."""
        ms = (C.c_double * 6)()
        n = (C.c_int64 * 4)()
        _check(self.L.ksw2g_align_chains_last_stats(self.ctx.h, ms, n))
        return list(ms), list(n)

    def rescue_device_ms(self):
        """[ksw_ll, extz2] kernel time (ms) of the context's last rescue call."""
        ms = (C.c_double * 2)()
        _check(self.L.ksw2g_rescue_last_device_ms(self.ctx.h, ms))
        return list(ms)

    def rescue_stats(self):
        """(kernel launches, [prefilter, ksw_ll, extz2] stage ms) of the context's last rescue call."""
        n = C.c_int()
        ms = (C.c_double * 3)()
        _check(self.L.ksw2g_rescue_last_stats(self.ctx.h, C.byref(n), ms))
        return n.value, list(ms)

    def close(self):
        if self.h:
            self.L.ksw2g_ref_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Graph:
    """One CUDA graph over several prepared batches (ksw2g_graph_t); every batch is a branch,
    so one launch runs them all concurrently.  Fetch results from the batches afterwards."""

    def __init__(self, ctx, batches):
        self.L, self.ctx, self.batches = ctx.L, ctx, list(batches)
        arr = (C.c_void_p * len(self.batches))(*[b.h.value for b in self.batches])
        self.h = C.c_void_p()
        _check(self.L.ksw2g_graph_create(ctx.h, len(self.batches), arr, C.byref(self.h)))

    @property
    def launches(self):
        return self.L.ksw2g_graph_launches(self.h)

    def launch(self):
        _check(self.L.ksw2g_graph_launch(self.ctx.h, self.h))

    def close(self):
        if self.h:
            self.L.ksw2g_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Request:
    """A request in flight on a Server; keeps its buffers alive until wait()."""

    def __init__(self, server, rid, kind, keep, res, cig):
        self.server, self.id, self.kind, self._keep, self.res, self.cig = server, rid, kind, keep, res, cig

    def wait(self):
        """Returns (results, cigar words, latency_ms, queue_ms)."""
        lat, que, used = C.c_double(), C.c_double(), C.c_int64()
        rc = self.server.L.ksw2g_server_wait(self.server.h, self.id, C.byref(lat), C.byref(que), C.byref(used))
        _check(rc)
        cig = self.cig[:used.value] if self.cig is not None else None
        return self.res, cig, lat.value, que.value


class Server:
    """Continuous-batching serving engine (ksw2g_server_t): requests admitted by traceback
    footprint against a fixed device budget, run concurrently on `slots` streams."""

    def __init__(self, device=0, slots=8, tb_budget=40 << 30, max_merge=None):
        self.L = load_library()
        h = C.c_void_p()
        _check(self.L.ksw2g_server_create(device, slots, int(tb_budget), C.byref(h)))
        self.h = h
        if max_merge is not None:
            _check(self.L.ksw2g_server_set_merge(self.h, int(max_merge)))

    def submit_ext(self, dual, m, mat, q, e, q2, e2, jobs, qbuf, tbuf):
        jobs = np.ascontiguousarray(jobs, EXT_JOB)
        qbuf, tbuf, mat = _u8(qbuf), _u8(tbuf), np.ascontiguousarray(mat, np.int8)
        res = np.zeros(len(jobs), EXT_RESULT)
        cap = int((jobs["qlen"].astype(np.int64) + jobs["tlen"] + 1).sum()) + 16
        cig = np.zeros(cap, np.uint32)
        rid = self.L.ksw2g_server_submit_ext(self.h, int(dual), m, _ptr(mat), q, e, q2, e2, len(jobs), _ptr(jobs),
                                             _ptr(qbuf), len(qbuf), _ptr(tbuf), len(tbuf), _ptr(res), _ptr(cig), cap)
        if rid < 0:
            _check(int(rid))
        return Request(self, rid, "ext", (jobs, qbuf, tbuf, mat), res, cig)

    def submit_ll(self, size, m, mat, gapo, gape, jobs, qbuf, tbuf):
        jobs = np.ascontiguousarray(jobs, LL_JOB)
        qbuf, tbuf, mat = _u8(qbuf), _u8(tbuf), np.ascontiguousarray(mat, np.int8)
        res = np.zeros(len(jobs), LL_RESULT)
        rid = self.L.ksw2g_server_submit_ll(self.h, size, m, _ptr(mat), gapo, gape, len(jobs), _ptr(jobs),
                                            _ptr(qbuf), len(qbuf), _ptr(tbuf), len(tbuf), _ptr(res))
        if rid < 0:
            _check(int(rid))
        return Request(self, rid, "ll", (jobs, qbuf, tbuf, mat), res, None)

    def stats(self):
        a, d, p, b = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        _check(self.L.ksw2g_server_stats(self.h, C.byref(a), C.byref(d), C.byref(p), C.byref(b)))
        nl, mg = C.c_int64(), C.c_int64()
        _check(self.L.ksw2g_server_launch_stats(self.h, C.byref(nl), C.byref(mg)))
        return dict(admitted=a.value, done=d.value, peak_inflight=p.value, peak_pool_bytes=b.value,
                    launches=nl.value, max_merged=mg.value)

    def close(self):
        if self.h:
            self.L.ksw2g_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
