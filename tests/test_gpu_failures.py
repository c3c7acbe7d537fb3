"""Failure handling of the batch and serving APIs.  Every failure is made on the host -- a
poisoned job descriptor, a request whose traceback cannot fit the engine's pool, a device
allocation that an injection hook makes fail -- and must come back as an error code before any
kernel of the failing call runs, with the context (or engine) still usable and later results
still bit-exact.  Nothing here faults, traps or hangs a GPU."""
import ctypes as C

import numpy as np
import pytest

from conftest import compare_ext, compare_ll

pytestmark = pytest.mark.gpu

E_ARG, E_NOMEM, E_CAPACITY = -2, -4, -5


def _code(fn):
    try:
        fn()
    except RuntimeError as e:
        msg = str(e)
        assert msg.startswith("ksw2gpu error "), msg
        return int(msg.split()[2].rstrip(":"))
    return 0


@pytest.fixture(scope="module")
def ctx(built):
    from minibwa_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _ext_ok(ctx, p):
    from oracle import oracle as O
    res, cig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    ores, ocig = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 8)
    compare_ext(res, cig, ores, ocig)


def test_poisoned_extension_descriptors(ctx):
    from minibwa_gb300 import synth
    p = synth.config1(300, seed=901)
    poisons = [("qoff", len(p.qbuf)), ("toff", len(p.tbuf) - 3), ("qlen", -1), ("tlen", -7), ("qoff", -16),
               ("qlen", 1 << 30)]
    for field, value in poisons:
        jobs = p.jobs.copy()
        jobs[field][157] = value
        rc = _code(lambda: ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, jobs, p.qbuf, p.tbuf))
        assert rc == E_ARG, (field, value, rc)
    _ext_ok(ctx, p)  # the context is unharmed


def test_poisoned_ll_descriptors(ctx):
    from minibwa_gb300 import synth
    from oracle import oracle as O
    r = synth.config3(300, seed=902)
    for field, value in (("toff", len(r.tbuf)), ("tlen", -1), ("qoff", len(r.qbuf) - 10)):
        jobs = r.jobs.copy()
        jobs[field][42] = value
        rc = _code(lambda: ctx.ll_batch(r.size, 5, r.mat, r.gapo, r.gape, jobs, r.qbuf, r.tbuf))
        assert rc == E_ARG, (field, value, rc)
    res = ctx.ll_batch(r.size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf)
    compare_ll(res, O.ll_batch("orc", r.size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf, 8))


def _footprint(jobs):
    q, t = jobs["qlen"].astype(np.int64), jobs["tlen"].astype(np.int64)
    w = np.where(jobs["w"] < 0, np.maximum(q, t), jobs["w"]).astype(np.int64)
    nc = (np.minimum(np.minimum(q, t), w + 1) + 15) // 16 + 1
    return ((q + t - 1) * nc * 16 + 15) & ~15


def test_server_refuses_a_request_beyond_its_pool_and_serves_the_rest(built, ctx):
    from minibwa_gb300 import Server, synth
    budget = 1 << 20
    big = synth.config2_long(40, seed=903)
    k = int(np.argmax(_footprint(big.jobs)))
    assert _footprint(big.jobs)[k] > budget
    bad = big.subset([k])
    good = [synth.config1(12, seed=904 + i) for i in range(6)]
    srv = Server(0, slots=2, tb_budget=budget)
    try:
        reqs = []
        for i, p in enumerate(good):
            reqs.append((p, srv.submit_ext(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)))
            if i == 2:  # in the middle of the stream of requests
                rc = _code(lambda: srv.submit_ext(bad.dual, 5, bad.mat, bad.q, bad.e, bad.q2, bad.e2, bad.jobs,
                                                  bad.qbuf, bad.tbuf))
                assert rc == E_CAPACITY, rc
                jobs = p.jobs.copy()
                jobs["toff"][0] = len(p.tbuf)
                rc = _code(lambda: srv.submit_ext(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, jobs, p.qbuf, p.tbuf))
                assert rc == E_ARG, rc
        for p, r in reqs:
            res, cig, _, _ = r.wait()
            exp, ecig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
            compare_ext(res, cig, exp, ecig)
    finally:
        srv.close()


def test_injected_allocation_failure(built):
    import torch
    from minibwa_gb300 import Context, synth
    from minibwa_gb300.lib import load_library
    L = load_library()
    L.ksw2g_debug_fail_device_alloc.argtypes = [C.c_int]
    L.ksw2g_debug_fail_device_alloc.restype = None
    p = synth.config1(500, seed=905)
    c = Context(0)
    try:
        _ext_ok(c, p)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        for nth in (1, 2, 3, 1, 2, 3):
            fresh = Context(0)  # its buffers are still empty, so the call must grow them
            try:
                L.ksw2g_debug_fail_device_alloc(nth)
                rc = _code(lambda: fresh.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf))
                L.ksw2g_debug_fail_device_alloc(0)
                assert rc == E_NOMEM, (nth, rc)
                _ext_ok(fresh, p)  # the same context recovers on the next call
            finally:
                L.ksw2g_debug_fail_device_alloc(0)
                fresh.close()
        torch.cuda.synchronize()
        assert free0 - torch.cuda.mem_get_info()[0] < (256 << 20)  # nothing left behind by the failed calls
    finally:
        c.close()
