"""The serving engine: requests admitted by traceback footprint, run concurrently on
several streams.  Every request's results must be exactly those of the same request
run alone (continuous batching may not change any result)."""
import threading

import numpy as np
import pytest

from conftest import EXT_FIELDS, LL_FIELDS

pytestmark = pytest.mark.gpu


def _requests():
    from minibwa_gb300 import synth
    out = []
    for i in range(6):
        out.append(("ext", synth.config0(200 + 50 * i, seed=100 + i)))
        out.append(("ext", synth.config1(120 + 30 * i, seed=200 + i)))
        out.append(("ll", synth.config3(300, seed=300 + i)))
        out.append(("ll", synth.config3_pe(200, seed=400 + i)))
    out.append(("ext", synth.config2_long(12, seed=500)))
    return out


def _alone(ctx, kind, p):
    if kind == "ext":
        return ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    return ctx.ll_batch(p.size, 5, p.mat, p.gapo, p.gape, p.jobs, p.qbuf, p.tbuf), None


def _submit(srv, kind, p):
    if kind == "ext":
        return srv.submit_ext(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    return srv.submit_ll(p.size, 5, p.mat, p.gapo, p.gape, p.jobs, p.qbuf, p.tbuf)


def _same(kind, a, ca, b, cb):
    for f in (EXT_FIELDS if kind == "ext" else LL_FIELDS):
        assert np.array_equal(a[f], b[f]), f
    if kind == "ext":
        for i in range(len(a)):
            k = int(a["n_cigar"][i])
            assert np.array_equal(ca[a["cigar_off"][i]:a["cigar_off"][i] + k], cb[b["cigar_off"][i]:b["cigar_off"][i] + k])


@pytest.mark.parametrize("slots,budget", [(1, 4 << 30), (4, 64 << 20), (8, 4 << 30)])
def test_results_same_alone_and_in_the_mix(built, slots, budget):
    from minibwa_gb300 import Context, Server
    reqs = _requests()
    ctx = Context(0)
    alone = [_alone(ctx, k, p) for k, p in reqs]
    ctx.close()
    srv = Server(0, slots=slots, tb_budget=budget)
    got = [None] * len(reqs)

    def worker(idxs):
        handles = [(i, _submit(srv, *reqs[i])) for i in idxs]
        for i, h in handles:
            got[i] = h.wait()

    ths = [threading.Thread(target=worker, args=(list(range(t, len(reqs), 3)),)) for t in range(3)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    st = srv.stats()
    srv.close()
    assert st["done"] == len(reqs) and st["admitted"] == len(reqs)
    assert st["peak_inflight"] >= 2  # requests overlapped on the device (merged or on separate slots)
    if slots == 1:
        assert st["max_merged"] >= 2 and st["launches"] < len(reqs)  # queued requests were merged
    assert st["peak_pool_bytes"] <= budget
    for (kind, p), (res, cig), (r2, c2, lat, que) in zip(reqs, alone, got):
        _same(kind, r2, c2, res, cig)
        assert lat >= que >= 0
