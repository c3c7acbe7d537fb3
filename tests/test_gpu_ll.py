"""GPU parity of the striped local alignment (ksw_ll_*) through the C ABI."""
import numpy as np
import pytest

from conftest import LL_FIELDS, compare_ll, golden_ll_cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built):
    from minibwa_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def test_golden_vectors_per_call(built, golden):
    import minibwa_gb300.lib as K
    for i, c in enumerate(golden_ll_cases(golden)):
        qp = K.ksw_ll_qinit(c["size"], c["query"], c["m"], c["mat"])
        if c["size"] == 1:
            r = K.ksw_ll_u8_core(qp, c["target"], c["gapo"], c["gape"], c["xtra"])
        else:
            r = K.ksw_ll_i16_core(qp, c["target"], c["gapo"], c["gape"], c["xtra"])
        K.ll_free(qp)
        got = dict(score=r.score, te=r.te, qe=r.qe, score2=r.score2, te2=r.te2)
        assert got == c["out"], (i, got, c["out"], c["size"], c["xtra"])


def test_ksw_ll_i16_wrapper(built, golden):
    import minibwa_gb300.lib as K
    n = 0
    for c in golden_ll_cases(golden):
        if c["size"] != 2 or c["xtra"] != 0:
            continue
        qp = K.ksw_ll_qinit(2, c["query"], c["m"], c["mat"])
        s, qe, te = K.ksw_ll_i16(qp, c["target"], c["gapo"], c["gape"])
        K.ll_free(qp)
        assert (s, qe, te) == (c["out"]["score"], c["out"]["qe"], c["out"]["te"])
        n += 1
    assert n > 10


def _batch(ctx, r):
    from minibwa_gb300.lib import LL_RESULT  # noqa: F401
    res = ctx.ll_batch(r.size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf)
    ores = O.ll_batch("orc", r.size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf, 8)
    compare_ll(res, ores)
    return res


def test_config3_i16(ctx):
    from minibwa_gb300 import synth
    res = _batch(ctx, synth.config3(20000))
    assert (res["score"] > 100).sum() > 1000  # planted copies were found


def test_config3_pe_u8_with_second_best(ctx):
    from minibwa_gb300 import synth
    res = _batch(ctx, synth.config3_pe(20000))
    assert (res["score2"] >= 0).sum() > 0


def test_random_ll_against_oracle(ctx):
    """Random lengths (slen up to 64 segments), scores, gaps and xtra flags."""
    from minibwa_gb300 import synth
    from minibwa_gb300.lib import gen_nt4_mat
    rng = np.random.default_rng(11)
    for it in range(40):
        size = 1 if it % 2 else 2
        lanes = 16 if size == 1 else 8
        ql = int(rng.integers(1, 64 * lanes))
        xtra = [0, 0x40000 | 19, 0x20000 | 60, 0x60000 | 30][it % 4]
        mat = gen_nt4_mat(int(rng.integers(1, 4)), int(rng.integers(1, 9)), 0, 1)
        r = synth.ll_jobs(200, qlen=ql, tlen_lo=1, tlen_hi=int(rng.integers(2, 1200)), plant=0.5, size=size,
                          xtra=xtra, mat=mat, gapo=int(rng.integers(0, 12)), gape=int(rng.integers(1, 4)),
                          seed=int(rng.integers(1, 1 << 30)))
        _batch(ctx, r)


def test_full_size_config3_sample(ctx):
    """2,000,000 jobs on the device; a random sample of 5,000 matches the checker."""
    from minibwa_gb300 import LLBatch, synth
    r = synth.config3()
    b = LLBatch(ctx, r.size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf)
    b.run()
    res = b.fetch()
    b.free()
    idx = np.sort(np.random.default_rng(5).choice(len(r), 5000, replace=False))
    s = r.subset(idx)
    ores = O.ll_batch("orc", s.size, 5, s.mat, s.gapo, s.gape, s.jobs, s.qbuf, s.tbuf, 8)
    compare_ll(res[idx], ores)
    assert (res["rows"] == r.jobs["tlen"]).all()


@pytest.mark.parametrize("family", ["lane", "dpx"])
def test_both_kernel_families(ctx, family, monkeypatch):
    """One lane per thread and the DPX two-lanes-per-thread kernel, pinned in turn, on
    i16 and u8 rescue jobs of several query lengths."""
    from minibwa_gb300 import synth
    from minibwa_gb300.lib import gen_nt4_mat
    monkeypatch.setenv("KSW2G_LL_KERNEL", family)
    for ql, size in ((37, 2), (150, 2), (300, 2), (150, 1), (400, 1)):
        r = synth.ll_jobs(1500, qlen=ql, tlen_lo=50, tlen_hi=900, size=size, seed=ql * 7 + size,
                          xtra=(0x40000 | 19) if size == 1 else 0,
                          mat=gen_nt4_mat(1, 4, 0, 1) if size == 1 else None, gapo=6 if size == 1 else 12,
                          gape=1 if size == 1 else 2)
        _batch(ctx, r)


def test_long_queries_shared_memory_kernel(ctx):
    """Queries beyond 64 segments (align.c's inversion check allows up to max_gap = 5000 nt)
    run on the shared-memory kernel; batched and per call."""
    from minibwa_gb300 import synth
    from minibwa_gb300.lib import gen_nt4_mat
    import minibwa_gb300.lib as K
    for size, ql, xtra in ((2, 600, 0), (2, 2000, 0), (2, 5000, 0), (1, 1100, 0x40000 | 19), (1, 3000, 0x40000 | 19)):
        mat = gen_nt4_mat(1, 4, 0, 1) if size == 1 else None
        r = synth.ll_jobs(40, qlen=ql, tlen_lo=ql // 2, tlen_hi=ql * 2, plant=0.6, size=size, xtra=xtra, mat=mat,
                          gapo=6 if size == 1 else 12, gape=1 if size == 1 else 2, seed=ql + size)
        _batch(ctx, r)
    r = synth.ll_jobs(3, qlen=3000, tlen_lo=2000, tlen_hi=4000, plant=1.0, seed=3)
    for k in range(len(r)):
        q = r.qbuf[r.jobs["qoff"][k]:r.jobs["qoff"][k] + r.jobs["qlen"][k]]
        t = r.tbuf[r.jobs["toff"][k]:r.jobs["toff"][k] + r.jobs["tlen"][k]]
        qp = K.ksw_ll_qinit(2, q, 5, r.mat)
        s, qe, te = K.ksw_ll_i16(qp, t, r.gapo, r.gape)
        K.ll_free(qp)
        want, _ = O.ll(2, q, t, 5, r.mat, r.gapo, r.gape, 0)
        assert (s, qe, te) == (want["score"], want["qe"], want["te"])


def test_one_shot_chunked_equals_resident(ctx):
    """Above 262,144 jobs the one-shot ksw_ll call runs in chunks on two sub-contexts; its
    results equal the resident batch's, with the pe.c u8 scoring and second-best lists."""
    from minibwa_gb300 import LLBatch, synth
    from minibwa_gb300.lib import KSW_LL_SUBO
    r = synth.config3(600000, seed=77)
    jobs = r.jobs.copy()
    jobs["xtra"] = np.where(np.arange(len(jobs)) % 2 == 0, KSW_LL_SUBO | 19, 0)
    b = LLBatch(ctx, r.size, 5, r.mat, r.gapo, r.gape, jobs, r.qbuf, r.tbuf)
    b.run()
    want = b.fetch()
    b.free()
    got = ctx.ll_batch(r.size, 5, r.mat, r.gapo, r.gape, jobs, r.qbuf, r.tbuf)
    compare_ll(got, want)
    assert np.array_equal(got["rows"], want["rows"])
