"""CUDA-graph batched mode: several prepared batches captured into one graph (one
branch each) give exactly the results of the same batches run one by one."""
import numpy as np
import pytest

from conftest import EXT_FIELDS, LL_FIELDS

pytestmark = pytest.mark.gpu


def _cigars(res, cig):
    return [cig[o:o + n].tolist() for o, n in zip(res["cigar_off"], res["n_cigar"])]


@pytest.mark.parametrize("budget", [None, 48 << 20])  # 48 MiB: several waves, run on two streams
def test_mixed_graph_matches_plain_batches(built, budget):
    from minibwa_gb300 import Context, ExtBatch, Graph, LLBatch, synth
    long_, short, resc = synth.config2_long(60), synth.config2_short(3000), synth.config3(2000)
    ctx = Context(0, tb_budget=budget)
    want_l = ctx.ext_batch(long_.dual, 5, long_.mat, long_.q, long_.e, long_.q2, long_.e2, long_.jobs, long_.qbuf,
                           long_.tbuf)
    want_s = ctx.ext_batch(short.dual, 5, short.mat, short.q, short.e, short.q2, short.e2, short.jobs, short.qbuf,
                           short.tbuf)
    want_r = ctx.ll_batch(resc.size, 5, resc.mat, resc.gapo, resc.gape, resc.jobs, resc.qbuf, resc.tbuf)
    bl = ExtBatch(ctx, long_.dual, 5, long_.mat, long_.q, long_.e, long_.q2, long_.e2, long_.jobs, long_.qbuf,
                  long_.tbuf)
    bs = ExtBatch(ctx, short.dual, 5, short.mat, short.q, short.e, short.q2, short.e2, short.jobs, short.qbuf,
                  short.tbuf)
    br = LLBatch(ctx, resc.size, 5, resc.mat, resc.gapo, resc.gape, resc.jobs, resc.qbuf, resc.tbuf)
    g = Graph(ctx, [bl, bs, br])
    assert g.launches >= 3
    for _ in range(2):  # a graph is relaunched as is
        g.launch()
        ctx.sync()
        for b, (wres, wcig) in ((bl, want_l), (bs, want_s)):
            res, cig = b.fetch()
            for f in EXT_FIELDS:
                assert np.array_equal(res[f], wres[f]), f
            assert _cigars(res, cig) == _cigars(wres, wcig)
        rr = br.fetch()
        for f in LL_FIELDS:
            assert np.array_equal(rr[f], want_r[f]), f
    g.close()
    for b in (bl, bs, br):
        b.free()
    ctx.close()
