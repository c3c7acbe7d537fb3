"""The two lane widths of the extension DP agree with each other and with the checker: the
16-bit-lane DPX kernels (ext16_dp.cuh) and the byte-lane kernels (ext_dp.cuh).  Scoring
schemes outside the 16-bit kernels' range (a gap cost above 128 after the extd2 swap) must run
on byte lanes and stay exact, whatever lane width is asked for."""
import numpy as np
import pytest

from conftest import compare_ext
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built):
    from minibwa_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _both(ctx, p):
    import minibwa_gb300.lib as K
    out = []
    for fam in (1, 0):
        prev = K.set_ext_family(fam)
        try:
            out.append(ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf))
        finally:
            K.set_ext_family(prev)
    return out


@pytest.mark.parametrize("which", ["cfg0", "cfg1", "cfg2_long", "cfg2_short"])
def test_lane_widths_agree_on_benchmark_shapes(ctx, which):
    from minibwa_gb300 import synth
    p = {"cfg0": lambda: synth.config0(4000, seed=71), "cfg1": lambda: synth.config1(4000, seed=72),
         "cfg2_long": lambda: synth.config2_long(40, seed=73),
         "cfg2_short": lambda: synth.config2_short(4000, seed=74)}[which]()
    (r16, c16), (r8, c8) = _both(ctx, p)
    compare_ext(r16, c16, r8, c8)
    ores, ocig = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 8)
    compare_ext(r16, c16, ores, ocig)


def test_random_scoring_every_mode(ctx):
    """Random scoring (match 1-6, mismatch 1-12, gap open 0-60, extend 0-8, long gaps, other N
    scores), every flag family and band width, both variants: batched against the checker."""
    from minibwa_gb300 import synth
    import minibwa_gb300.lib as K
    rng = np.random.default_rng(20261204)
    base = synth.config1(400, seed=75)
    for it in range(24):
        a, b = int(rng.integers(1, 7)), int(rng.integers(1, 13))
        p = base.subset(np.arange(it % 7, 400, 5))
        p.mat = K.gen_nt4_mat(a, b, 0, int(rng.integers(0, 3)))
        p.dual = it % 2
        p.q, p.e = int(rng.integers(0, 61)), int(rng.integers(0, 9))
        p.q2, p.e2 = (int(rng.integers(0, 80)), int(rng.integers(0, 4))) if p.dual else (p.q, p.e)
        if b > 2 * (p.q + p.e):  # the reference returns at once for such scoring; keep it meaningful
            p.q += b
        p.jobs["flag"] = int(rng.choice([0x40, 0xc2, 0x41, 0x08, 0x00, 0x58, 0x04, 0x80, 0x02]))
        p.jobs["w"] = int(rng.choice([3, 17, 40, 100, 230]))
        p.jobs["zdrop"] = int(rng.choice([-1, 30, 100]))
        p.jobs["end_bonus"] = int(rng.choice([-1, 0, 10]))
        (r16, c16), (r8, c8) = _both(ctx, p)
        ores, ocig = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 8)
        compare_ext(r16, c16, ores, ocig)
        compare_ext(r8, c8, ores, ocig)


def test_trace_calls_on_16bit_lanes(built, trace):
    """The extension calls of real minibwa runs, per call, with 16-bit lanes forced."""
    import minibwa_gb300.lib as K
    from conftest import TRACE_OUT, trace_ext_calls
    prev = K.set_ext_family(1)
    try:
        for n, c in enumerate(trace_ext_calls(trace)):
            if n % 4:
                continue
            if c["dual"]:
                ez = K.ksw_extd2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"],
                                     c["w"], c["zdrop"], c["end_bonus"], c["flag"])
            else:
                ez = K.ksw_extz2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["w"], c["zdrop"],
                                     c["end_bonus"], c["flag"])
            got = ez.fields()
            for f in TRACE_OUT:
                if f != "m_cigar":
                    assert got[f] == c["out"][f], (n, f, got[f], c["out"][f])
            assert got["cigar"] == c["cigar"], n
            K.free_extz(ez)
    finally:
        K.set_ext_family(prev)


def test_scoring_outside_the_16bit_range_runs_on_byte_lanes(ctx):
    from minibwa_gb300 import synth
    p = synth.config1(300, seed=76)
    p.q, p.e, p.q2, p.e2 = 100, 40, 110, 30  # q+e = 140 > 128
    (r16, c16), _ = _both(ctx, p)
    ores, ocig = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 8)
    compare_ext(r16, c16, ores, ocig)
