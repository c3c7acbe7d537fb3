"""The per-call drop-in from many host threads at once, as minibwa's kt_for workers call it
(map-main.c:179,191): every thread gets its own stream and scratch, so concurrent calls give each
call's own result.  The traced calls of real minibwa runs are split over eight threads that call
ksw_extz2_sse / ksw_extd2_sse / ksw_ll_* concurrently, and each result must equal the recorded
one; contexts of the batch API used from several threads at once must not interfere either."""
import threading

import numpy as np
import pytest

from conftest import TRACE_OUT, trace_ext_calls, trace_ll_calls

pytestmark = pytest.mark.gpu


def _run_threads(n, fn):
    errors = []

    def wrap(t):
        try:
            fn(t)
        except BaseException as e:  # reported on the main thread
            errors.append(e)

    th = [threading.Thread(target=wrap, args=(t,)) for t in range(n)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    if errors:
        raise errors[0]


def test_per_call_dropin_from_eight_threads(built, trace):
    import minibwa_gb300.lib as K
    calls = list(trace_ext_calls(trace))[:2400]
    lls = list(trace_ll_calls(trace))
    n_threads = 8

    def work(t):
        for c in calls[t::n_threads]:
            if c["dual"]:
                ez = K.ksw_extd2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"],
                                     c["w"], c["zdrop"], c["end_bonus"], c["flag"])
            else:
                ez = K.ksw_extz2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["w"], c["zdrop"],
                                     c["end_bonus"], c["flag"])
            got = ez.fields()
            for f in TRACE_OUT:
                if f != "m_cigar":
                    assert got[f] == c["out"][f], (t, f)
            assert got["cigar"] == c["cigar"]
            K.free_extz(ez)
        for c in lls[t::n_threads]:
            qp = K.ksw_ll_qinit(c["size"], c["query"], c["m"], c["mat"])
            r = (K.ksw_ll_u8_core if c["size"] == 1 else K.ksw_ll_i16_core)(qp, c["target"], c["gapo"], c["gape"],
                                                                                c["xtra"])
            K.ll_free(qp)
            assert dict(score=r.score, te=r.te, qe=r.qe, score2=r.score2, te2=r.te2) == c["out"]

    _run_threads(n_threads, work)


def test_batch_contexts_from_four_threads(built):
    from minibwa_gb300 import Context, synth
    from oracle import oracle as O
    sets = [synth.config1(3000, seed=600 + t) for t in range(4)]
    expected = [O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 4) for p in sets]

    def work(t):
        p = sets[t]
        ctx = Context(0)
        try:
            for _ in range(3):
                res, cig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
                ores, ocig = expected[t]
                for f in ("score", "max", "max_q", "max_t", "mqe", "mqe_t", "zdropped", "reach_end", "n_cigar"):
                    assert np.array_equal(res[f], ores[f]), (t, f)
                for i in range(0, len(p), 97):
                    k = int(res["n_cigar"][i])
                    assert np.array_equal(cig[res["cigar_off"][i]:res["cigar_off"][i] + k],
                                          ocig[ores["cigar_off"][i]:ores["cigar_off"][i] + k])
        finally:
            ctx.close()

    _run_threads(4, work)


def test_long_ll_queries_from_sixteen_threads(built):
    """ksw_ll_i16 on queries of 520-4,000 nt (align.c's inversion check, up to max_gap) from 16
    threads at once: the block-wide ksw_ll kernel takes a different amount of shared memory for
    every query length, and a call must never lower the kernel's shared-memory cap under a
    concurrent launch of another thread (that launch failed with an invalid argument)."""
    import minibwa_gb300.lib as K
    from oracle import oracle as O
    rng = np.random.default_rng(77)
    mat = K.gen_nt4_mat(2, 8, 0, 1)
    cases = []
    for _ in range(160):
        ql, tl = int(rng.integers(520, 4000)), int(rng.integers(300, 4000))
        q = rng.integers(0, 4, ql).astype(np.uint8)
        t = rng.integers(0, 4, tl).astype(np.uint8)
        if rng.random() < 0.5:  # a stretch of the query in the target
            a, ln = int(rng.integers(0, ql // 2)), int(rng.integers(50, 300))
            b = int(rng.integers(0, max(tl - ln, 1)))
            piece = q[a:a + ln][: tl - b]
            t[b:b + len(piece)] = piece
        cases.append((q, t, O.ll(2, q, t, 5, mat, 12, 2, 0)[0]))
    n_threads = 16

    def work(t):
        for q, tg, exp in cases[t::n_threads]:
            qp = K.ksw_ll_qinit(2, q, 5, mat)
            r = K.ksw_ll_i16_core(qp, tg, 12, 2, 0)
            K.ll_free(qp)
            assert dict(score=r.score, te=r.te, qe=r.qe, score2=r.score2, te2=r.te2) == exp
    _run_threads(n_threads, work)
