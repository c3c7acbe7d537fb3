"""The ksw2 calls of real minibwa runs (tests/golden/minibwa_trace.npz, recorded from the
reference's own minibwa by tests/golden/make_trace.py) replayed on the GPU: through the per-call
drop-in with the caller's ez state as the reference run had it, and through the batch API grouped
by scoring scheme.  Every field, the CIGAR and m_cigar must equal the recorded call."""
import ctypes as C

import numpy as np
import pytest

from conftest import LL_FIELDS, TRACE_OUT, trace_ext_calls, trace_ll_calls

pytestmark = pytest.mark.gpu

_libc = C.CDLL(None)
_libc.malloc.restype = C.c_void_p


def test_traced_extension_calls_per_call(built, trace):
    import minibwa_gb300.lib as K
    n = 0
    for c in trace_ext_calls(trace):
        ez = K.KswExtz()
        if c["m_cigar_in"] > 0:  # the caller's buffer as the reference run had it (align.c:908, pe.c:435)
            ez.m_cigar = c["m_cigar_in"]
            ez.cigar = C.cast(_libc.malloc(4 * c["m_cigar_in"]), C.POINTER(C.c_uint32))
        if c["dual"]:
            K.ksw_extd2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"], c["w"],
                            c["zdrop"], c["end_bonus"], c["flag"], ez)
        else:
            K.ksw_extz2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["w"], c["zdrop"],
                            c["end_bonus"], c["flag"], ez)
        got = ez.fields()
        got["m_cigar"] = ez.m_cigar
        for f in TRACE_OUT:
            assert got[f] == c["out"][f], (n, f, got[f], c["out"][f])
        assert got["cigar"] == c["cigar"], n
        K.free_extz(ez)
        n += 1
    assert n > 5000


def test_traced_extension_calls_batched(built, trace):
    from minibwa_gb300 import Context
    from minibwa_gb300.lib import EXT_JOB
    calls = list(trace_ext_calls(trace))
    groups = {}
    for i, c in enumerate(calls):
        groups.setdefault((c["dual"], c["m"], c["mat"].tobytes(), c["q"], c["e"], c["q2"], c["e2"]), []).append(i)
    ctx = Context(0)
    try:
        for (dual, m, matb, q, e, q2, e2), idx in groups.items():
            jobs = np.zeros(len(idx), EXT_JOB)
            qs = [calls[i]["query"] for i in idx]
            ts = [calls[i]["target"] for i in idx]
            jobs["qlen"], jobs["tlen"] = [len(x) for x in qs], [len(x) for x in ts]
            jobs["qoff"] = np.concatenate([[0], np.cumsum(jobs["qlen"])[:-1]])
            jobs["toff"] = np.concatenate([[0], np.cumsum(jobs["tlen"])[:-1]])
            for f in ("w", "zdrop", "end_bonus", "flag"):
                jobs[f] = [calls[i][f] for i in idx]
            res, cig = ctx.ext_batch(int(dual), m, np.frombuffer(matb, np.int8), q, e, q2, e2, jobs,
                                     np.concatenate(qs), np.concatenate(ts))
            for j, i in enumerate(idx):
                for f in TRACE_OUT:
                    if f != "m_cigar":
                        assert int(res[f][j]) == calls[i]["out"][f], (i, f)
                k = int(res["n_cigar"][j])
                assert cig[res["cigar_off"][j]:res["cigar_off"][j] + k].tolist() == calls[i]["cigar"], i
    finally:
        ctx.close()


def test_traced_ll_calls(built, trace):
    import minibwa_gb300.lib as K
    from minibwa_gb300 import Context
    from minibwa_gb300.lib import LL_JOB
    calls = list(trace_ll_calls(trace))
    for n, c in enumerate(calls):  # per call: ksw_ll_qinit + the core pe.c:266-271 calls
        qp = K.ksw_ll_qinit(c["size"], c["query"], c["m"], c["mat"])
        core = K.ksw_ll_u8_core if c["size"] == 1 else K.ksw_ll_i16_core
        r = core(qp, c["target"], c["gapo"], c["gape"], c["xtra"])
        K.ll_free(qp)
        got = dict(score=r.score, te=r.te, qe=r.qe, score2=r.score2, te2=r.te2)
        assert got == c["out"], (n, got, c["out"])
    groups = {}
    for i, c in enumerate(calls):
        groups.setdefault((c["size"], c["m"], c["mat"].tobytes(), c["gapo"], c["gape"]), []).append(i)
    ctx = Context(0)
    try:
        for (size, m, matb, gapo, gape), idx in groups.items():
            jobs = np.zeros(len(idx), LL_JOB)
            qs = [calls[i]["query"] for i in idx]
            ts = [calls[i]["target"] for i in idx]
            jobs["qlen"], jobs["tlen"] = [len(x) for x in qs], [len(x) for x in ts]
            jobs["qoff"] = np.concatenate([[0], np.cumsum(jobs["qlen"])[:-1]])
            jobs["toff"] = np.concatenate([[0], np.cumsum(jobs["tlen"])[:-1]])
            jobs["xtra"] = [calls[i]["xtra"] for i in idx]
            res = ctx.ll_batch(size, m, np.frombuffer(matb, np.int8), gapo, gape, jobs, np.concatenate(qs),
                               np.concatenate(ts))
            for j, i in enumerate(idx):
                for f in LL_FIELDS:
                    assert int(res[f][j]) == calls[i]["out"][f], (i, f)
    finally:
        ctx.close()
