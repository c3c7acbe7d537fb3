"""The block-split extension kernel (ext_split.cuh): one pair per block, each anti-diagonal split
over the block's warps.  Forced on every job (ksw2g_ext_set_split(1)) it must give the results
of the thread-group kernels and of the checker, CIGARs included, in both variants, every
traceback mode, the approximate max, generic scoring, bands from a few cells up to the widest
block, many waves and the per-call drop-in; left to the batch (the default), the jobs of a
band class that are few and wide run on it."""
import numpy as np
import pytest

from conftest import EXT_FIELDS, compare_ext
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built):
    from minibwa_gb300 import Context
    c = Context(0)
    yield c
    c.close()


class _split:
    def __init__(self, mode):
        self.mode = mode

    def __enter__(self):
        import minibwa_gb300.lib as K
        self.prev = K.set_ext_split(self.mode)

    def __exit__(self, *a):
        import minibwa_gb300.lib as K
        K.set_ext_split(self.prev)


def _run(ctx, p, mode):
    with _split(mode):
        return ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)


def _check(ctx, p, nthreads=8):
    rs, cs = _run(ctx, p, 1)
    rg, cg = _run(ctx, p, 0)
    compare_ext(rs, cs, rg, cg)
    ores, ocig = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, nthreads)
    compare_ext(rs, cs, ores, ocig)
    return rs


@pytest.mark.parametrize("which", ["cfg0", "cfg1", "cfg2_long"])
def test_benchmark_shapes(ctx, which):
    from minibwa_gb300 import synth
    p = {"cfg0": lambda: synth.config0(3000, seed=81), "cfg1": lambda: synth.config1(3000, seed=82),
         "cfg2_long": lambda: synth.config2_long(30, seed=83)}[which]()
    _check(ctx, p)


def test_every_mode_and_band(ctx):
    """Every flag family x band width, both variants: one warp up to eight warps a block."""
    from minibwa_gb300 import synth
    base = synth.config1(300, seed=84)
    for dual in (0, 1):
        for flag in (0x40, 0xc2, 0x41, 0x08, 0x00, 0x58, 0x04, 0x18):
            for w in (5, 40, 100, 230, 480, 900):
                p = base.subset(np.arange(flag % 5, 300, 9))
                p.dual = dual
                p.q2, p.e2 = (24, 1) if dual else (12, 2)
                p.jobs["w"], p.jobs["flag"] = w, flag
                _check(ctx, p)


def test_random_scoring(ctx):
    from minibwa_gb300 import synth
    import minibwa_gb300.lib as K
    rng = np.random.default_rng(20261206)
    base = synth.config1(300, seed=85)
    for it in range(16):
        a, b = int(rng.integers(1, 7)), int(rng.integers(1, 13))
        p = base.subset(np.arange(it % 5, 300, 6))
        p.mat = K.gen_nt4_mat(a, b, 0, int(rng.integers(0, 3)))
        p.dual = it % 2
        p.q, p.e = int(rng.integers(0, 61)), int(rng.integers(0, 9))
        p.q2, p.e2 = (int(rng.integers(0, 80)), int(rng.integers(0, 4))) if p.dual else (p.q, p.e)
        if b > 2 * (p.q + p.e):
            p.q += b
        p.jobs["flag"] = int(rng.choice([0x40, 0xc2, 0x41, 0x08, 0x00, 0x58, 0x04, 0x80, 0x02]))
        p.jobs["w"] = int(rng.choice([3, 17, 40, 100, 230, 600]))
        p.jobs["zdrop"] = int(rng.choice([-1, 30, 100]))
        p.jobs["end_bonus"] = int(rng.choice([-1, 0, 10]))
        _check(ctx, p)


def _wide_pairs(n, lo, hi, w, flag, dual, seed):
    from minibwa_gb300 import synth
    return synth.ext_pairs(n, dict(synth.SPEC_LONG, clip_lo=lo, clip_hi=hi), w, 400, 10, flag, dual, seed=seed)


def test_wide_bands(ctx):
    """Bands of several hundred blocks (two and four words a thread, sixteen warps), alone and
    mixed with narrow pairs, and over many waves on two streams."""
    from minibwa_gb300 import Context
    for flag in (0x40, 0x00, 0xc2, 0x08):
        for dual in (0, 1):
            _check(ctx, _wide_pairs(5, 1500, 5000, -1, flag, dual, seed=flag + dual + 7))
    _check(ctx, _wide_pairs(40, 300, 3000, 1200, 0x40, 1, seed=4))
    c = Context(0, tb_budget=64 << 20)
    try:
        _check(c, _wide_pairs(12, 1500, 3000, 2500, 0x40, 1, seed=10))
    finally:
        c.close()


def test_per_call(built):
    """The per-call drop-in on one block, for long pairs and for short ones."""
    import minibwa_gb300.lib as K
    from minibwa_gb300 import synth
    p = _wide_pairs(3, 2000, 6000, 500, 0x40, 1, seed=22)
    s = synth.config0(40, seed=23)
    with _split(1):
        for i in range(len(p)):
            q, t = p.query(i), p.target(i)
            ez = K.ksw_extd2_sse(q, t, 5, p.mat, p.q, p.e, p.q2, p.e2, 500, 400, 10, 0x40)
            exp, _ = O.extz(1, q, t, 5, p.mat, p.q, p.e, p.q2, p.e2, 500, 400, 10, 0x40)
            got = ez.fields()
            for f in EXT_FIELDS + ["cigar"]:
                assert got[f] == exp[f], (i, f)
            K.free_extz(ez)
        for i in range(len(s)):
            q, t = s.query(i), s.target(i)
            ez = K.ksw_extz2_sse(q, t, 5, s.mat, s.q, s.e, 25, 100, 10, 0x40)
            exp, _ = O.extz(0, q, t, 5, s.mat, s.q, s.e, s.q, s.e, 25, 100, 10, 0x40)
            got = ez.fields()
            for f in EXT_FIELDS + ["cigar"]:
                assert got[f] == exp[f], (i, f)
            K.free_extz(ez)


def test_batch_decides(ctx):
    """Left to the batch, a few long pairs among many short ones run on blocks and the rest on
    thread groups; the results are the checker's either way."""
    from minibwa_gb300 import synth
    long = synth.config2_long(12, seed=86)
    short = synth.config1(2000, seed=87)
    for p in (long, short):
        with _split(-1):
            res, cig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
        ores, ocig = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 8)
        compare_ext(res, cig, ores, ocig)


def test_split_mode_argument(built):
    import minibwa_gb300.lib as K
    L = K.load_library()
    assert L.ksw2g_ext_set_split(2) != 0 and L.ksw2g_ext_set_split(-2) != 0
