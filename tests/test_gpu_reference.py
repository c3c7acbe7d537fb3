"""Targets decoded on the device from a resident 2-bit reference: the windows equal the
oracle's l2b_getseq, and batches that name their targets as windows give exactly the results
of the same jobs with host target bytes."""
import numpy as np
import pytest

from conftest import EXT_FIELDS, LL_FIELDS

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_ctx(built):
    from minibwa_gb300 import Context, Reference, synth
    r = synth.Reference2b([50000, 1234, 200000, 77], n_runs=60, run_max=400)
    ctx = Context(0)
    dev = Reference(ctx, r.pac, r.ctg_off, r.ctg_len, r.ambi)
    yield r, ctx, dev
    dev.close()
    ctx.close()


def test_windows_match_oracle(ref_ctx):
    from oracle import oracle as O
    r, ctx, dev = ref_ctx
    rng = np.random.default_rng(3)
    for it in range(300):
        k = int(rng.integers(0, len(r.ctg_len)))
        L = min(int(rng.integers(0, 2000)), int(r.ctg_len[k]))
        st = int(rng.integers(0, int(r.ctg_len[k]) - L + 1))
        fl = int(rng.choice([0, 1, 2, 3, 4, 5]))
        assert np.array_equal(dev.getseq(k, st, L, fl), O.l2b_getseq(r, k, st, L, fl)), (it, k, st, L, fl)


@pytest.mark.parametrize("dual", [0, 1])
def test_ext_batch_with_reference_targets(ref_ctx, dual):
    from minibwa_gb300 import synth
    r, ctx, dev = ref_ctx
    flags = np.random.default_rng(5 + dual).choice([0, 1, 2, 4, 5], 3000)
    p, tids, tfl = synth.ref_pairs(r, 3000, dual=bool(dual), flags=flags, seed=40 + dual)
    want, wcig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    jobs = p.jobs.copy()
    jobs["toff"] = p.ref_toff
    got, gcig = dev.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, jobs, tids, tfl, p.qbuf)
    for f in EXT_FIELDS:
        assert np.array_equal(got[f], want[f]), f
    for i in range(len(p)):
        o, n, wo = int(got["cigar_off"][i]), int(got["n_cigar"][i]), int(want["cigar_off"][i])
        assert np.array_equal(gcig[o:o + n], wcig[wo:wo + n]), i


def test_chunked_ext_batch_with_reference_targets(ref_ctx):
    """Above 32,768 jobs the one-shot call runs in chunks on two sub-contexts; with reference
    targets each chunk gathers its own windows.  Results equal the same jobs with host targets."""
    from minibwa_gb300 import synth
    r, ctx, dev = ref_ctx
    flags = np.random.default_rng(9).choice([0, 1, 2, 5], 140000)
    p, tids, tfl = synth.ref_pairs(r, 140000, qlen_lo=60, qlen_hi=160, flags=flags, seed=90)
    want, wcig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    jobs = p.jobs.copy()
    jobs["toff"] = p.ref_toff
    got, gcig = dev.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, jobs, tids, tfl, p.qbuf)
    for f in EXT_FIELDS:
        assert np.array_equal(got[f], want[f]), f
    for i in range(0, len(p), 7):
        o, n, wo = int(got["cigar_off"][i]), int(got["n_cigar"][i]), int(want["cigar_off"][i])
        assert np.array_equal(gcig[o:o + n], wcig[wo:wo + n]), i


def test_ll_batch_with_reference_targets(ref_ctx):
    from minibwa_gb300 import synth
    from minibwa_gb300.lib import LL_JOB
    r, ctx, dev = ref_ctx
    p, tids, tfl = synth.ref_pairs(r, 2000, qlen_lo=150, qlen_hi=150, flank=700, seed=61)
    jobs = np.zeros(len(p), LL_JOB)
    jobs["qoff"], jobs["qlen"], jobs["tlen"] = p.jobs["qoff"], p.jobs["qlen"], p.jobs["tlen"]
    jobs["toff"] = p.jobs["toff"]
    want = ctx.ll_batch(2, 5, p.mat, 12, 2, jobs, p.qbuf, p.tbuf)
    jobs["toff"] = p.ref_toff
    got = dev.ll_batch(2, 5, p.mat, 12, 2, jobs, tids, tfl, p.qbuf)
    for f in LL_FIELDS:
        assert np.array_equal(got[f], want[f]), f
