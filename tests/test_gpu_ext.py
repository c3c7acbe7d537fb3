"""GPU parity of the extension kernels (ksw_extz2_sse / ksw_extd2_sse) through the C ABI.

Bar: bit-exact equality with the checker on every field and the CIGAR.  The checker is the
scalar restatement (oracle/), itself pinned to the reference by the golden vectors."""
import numpy as np
import pytest

from conftest import EXT_FIELDS, compare_ext, expected_m_cigar, golden_ext_cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(built):
    from minibwa_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _dropin(c, ez=None):
    import minibwa_gb300.lib as K
    if c["dual"]:
        return K.ksw_extd2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"], c["w"],
                               c["zdrop"], c["end_bonus"], c["flag"], ez)
    return K.ksw_extz2_sse(c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["w"], c["zdrop"],
                           c["end_bonus"], c["flag"], ez)


def test_golden_vectors_per_call(built, golden):
    """Every golden case through the reference-shaped per-call entry points."""
    import minibwa_gb300.lib as K
    for i, c in enumerate(golden_ext_cases(golden)):
        ez = _dropin(c)
        got = ez.fields()
        for f in EXT_FIELDS:
            assert got[f] == c["out"][f], (i, f, got[f], c["out"][f], c["flag"], c["dual"])
        assert got["cigar"] == c["cigar"], (i, got["cigar"], c["cigar"])
        assert ez.m_cigar == expected_m_cigar(0, ez.n_cigar)
        K.free_extz(ez)


def test_golden_vectors_batched(ctx, golden):
    """Golden cases through the batch API, grouped by scoring scheme."""
    cases = list(golden_ext_cases(golden))
    groups = {}
    for i, c in enumerate(cases):
        key = (c["dual"], c["m"], c["mat"].tobytes(), c["q"], c["e"], c["q2"], c["e2"])
        groups.setdefault(key, []).append(i)
    from minibwa_gb300.lib import EXT_JOB
    for key, idx in groups.items():
        dual, m, matb, q, e, q2, e2 = key
        qs = [cases[i]["query"] for i in idx]
        ts = [cases[i]["target"] for i in idx]
        jobs = np.zeros(len(idx), EXT_JOB)
        jobs["qlen"] = [len(x) for x in qs]
        jobs["tlen"] = [len(x) for x in ts]
        jobs["qoff"] = np.concatenate([[0], np.cumsum(jobs["qlen"])[:-1]])
        jobs["toff"] = np.concatenate([[0], np.cumsum(jobs["tlen"])[:-1]])
        for f in ("w", "zdrop", "end_bonus", "flag"):
            jobs[f] = [cases[i][f] for i in idx]
        res, cig = ctx.ext_batch(dual, m, np.frombuffer(matb, np.int8), q, e, q2, e2, jobs, np.concatenate(qs),
                                 np.concatenate(ts))
        for j, i in enumerate(idx):
            for f in EXT_FIELDS:
                assert int(res[f][j]) == cases[i]["out"][f], (i, f)
            k = int(res["n_cigar"][j])
            assert cig[res["cigar_off"][j]:res["cigar_off"][j] + k].tolist() == cases[i]["cigar"], i


def test_caller_owned_cigar_buffer_is_grown_like_the_reference(built, golden):
    """pe.c:435-437 hands in m_cigar=16 with a malloc'ed buffer; align.c:908 reuses one ez."""
    import ctypes as C
    import minibwa_gb300.lib as K
    libc = C.CDLL(None)
    libc.malloc.restype = C.c_void_p
    ez = K.KswExtz()
    ez.m_cigar = 16
    ez.cigar = C.cast(libc.malloc(64), C.POINTER(C.c_uint32))
    m0 = 16
    for c in list(golden_ext_cases(golden))[:200]:
        _dropin(c, ez)
        assert ez.fields()["cigar"] == c["cigar"]
        m0 = expected_m_cigar(m0, ez.n_cigar)
        assert ez.m_cigar == m0
    K.free_extz(ez)


def _rand_case(rng):
    m = 5
    ql = int(rng.integers(1, 400))
    q = rng.integers(0, 4, ql).astype(np.uint8)
    q[rng.random(ql) < 0.01] = 4
    t = q.copy()
    if rng.random() < 0.3:
        t = rng.integers(0, 4, int(rng.integers(1, 400))).astype(np.uint8)
    else:
        sub = rng.random(len(t)) < rng.random() * 0.1
        t[sub] = rng.integers(0, 5, sub.sum())
        if rng.random() < 0.5:
            p = int(rng.integers(0, len(t)))
            t = np.concatenate([t[:p], rng.integers(0, 4, int(rng.integers(1, 8))).astype(np.uint8), t[p:]])
        t = np.concatenate([t, rng.integers(0, 4, int(rng.integers(0, 60))).astype(np.uint8)])
    a, b = int(rng.integers(1, 5)), int(rng.integers(2, 10))
    mat = np.array([a if i // m == i % m else -b for i in range(25)], np.int8)
    mat[20:25] = -1
    mat[4::5] = -1
    return dict(dual=int(rng.random() < 0.5), m=m, mat=mat, q=int(rng.integers(2, 20)), e=int(rng.integers(1, 4)),
                q2=int(rng.integers(10, 40)), e2=1, w=int(rng.choice([-1, 0, 3, 10, 25, 60, 100, 200, 500])),
                zdrop=int(rng.choice([-1, 20, 100, 400])), end_bonus=int(rng.choice([-1, 0, 10])),
                flag=int(rng.choice([0x40, 0xc2, 0x08, 0x00, 0x41, 0x02, 0x58, 0x18, 0x80, 0x04, 0x44])),
                query=q, target=t)


def test_random_cases_per_call_against_oracle(built):
    import minibwa_gb300.lib as K
    rng = np.random.default_rng(7)
    for it in range(1500):
        c = _rand_case(rng)
        if not c["dual"]:
            c["q2"], c["e2"] = c["q"], c["e"]
        ez = _dropin(c)
        got = ez.fields()
        exp, _ = O.extz(c["dual"], c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"],
                        c["w"], c["zdrop"], c["end_bonus"], c["flag"])
        for f in EXT_FIELDS + ["cigar"]:
            assert got[f] == exp[f], (it, f, got[f], exp[f], {k: v for k, v in c.items() if k not in ("query", "target")})
        K.free_extz(ez)


def test_codes_above_n_and_random_matrices(built):
    """Bytes 5-7 (neither a base nor N) compare by equality in the reference's non-generic scores
    (ksw2_extz2_sse.c:117-131); any matrix, not only match/mismatch/N ones."""
    import minibwa_gb300.lib as K
    rng = np.random.default_rng(17)
    for it in range(400):
        c = _rand_case(rng)
        if not c["dual"]:
            c["q2"], c["e2"] = c["q"], c["e"]
        if not c["flag"] & 0x04:
            for s in ("query", "target"):
                x = c[s]
                hit = rng.random(len(x)) < 0.1
                x[hit] = rng.integers(0, 8, hit.sum())
        if rng.random() < 0.5:
            a = int(c["mat"][0])
            mat = rng.integers(-8, a + 1, 25).astype(np.int8)
            mat[0] = a
            c["mat"] = mat
        ez = _dropin(c)
        got = ez.fields()
        exp, _ = O.extz(c["dual"], c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"],
                        c["w"], c["zdrop"], c["end_bonus"], c["flag"])
        for f in EXT_FIELDS + ["cigar"]:
            assert got[f] == exp[f], (it, f, got[f], exp[f])
        K.free_extz(ez)


def test_one_cell_bands(ctx):
    """Bands that pinch to one cell on consecutive anti-diagonals read H of a cell that already
    left the band; batched, against the checker."""
    rng = np.random.default_rng(29)
    mat = np.array([3 if i // 5 == i % 5 else -4 for i in range(25)], np.int8)
    mat[20:25] = -1
    mat[4::5] = -1
    qs = [rng.integers(0, 4, 46).astype(np.uint8) for _ in range(4)]
    ts = [q[:tl].copy() for q, tl in zip(qs, (1, 2, 3, 5))]
    qbuf, tbuf = np.concatenate(qs), np.concatenate(ts)
    for dual in (0, 1):
        for flag in (0x00, 0x01, 0x40, 0x42):
            for w in (2, 3, 4, 6, 10):
                jobs = np.zeros(4, O.ORC_JOB)
                jobs["qoff"] = np.cumsum([0] + [len(q) for q in qs[:-1]])
                jobs["toff"] = np.cumsum([0] + [len(t) for t in ts[:-1]])
                jobs["qlen"], jobs["tlen"] = [len(q) for q in qs], [len(t) for t in ts]
                jobs["w"], jobs["zdrop"], jobs["end_bonus"], jobs["flag"] = w, -1, 5, flag
                q2 = 20 if dual else 3
                res, cig = ctx.ext_batch(dual, 5, mat, 3, 1, q2, 1, jobs, qbuf, tbuf)
                ores, ocig = O.ext_batch("orc", dual, 5, mat, 3, 1, q2, 1, jobs, qbuf, tbuf, 1)
                compare_ext(res, cig, ores, ocig)


def _batch_vs_oracle(ctx, p, nthreads=8):
    res, cig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    ores, ocig = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, nthreads)
    compare_ext(res, cig, ores, ocig)
    return res


def test_config0_full_size(ctx):
    """20,000 extz2 pairs, 150 nt, w=25: the configuration the CPU reference is timed on."""
    from minibwa_gb300 import synth
    res = _batch_vs_oracle(ctx, synth.config0())
    assert (res["n_cigar"] > 0).all()


def test_config1_shapes(ctx):
    from minibwa_gb300 import synth
    res = _batch_vs_oracle(ctx, synth.config1(20000))
    assert res["zdropped"].sum() > 0 and res["reach_end"].sum() > 0


def test_config2_long_and_short(ctx):
    from minibwa_gb300 import synth
    _batch_vs_oracle(ctx, synth.config2_long(60))
    _batch_vs_oracle(ctx, synth.config2_short(4000))


def test_all_modes_and_shapes_batched(ctx):
    """Every flag family x band width (hence every kernel shape) on benchmark-like pairs."""
    from minibwa_gb300 import synth
    base = synth.config1(600, seed=99)
    for dual in (0, 1):
        for flag in (0x40, 0xc2, 0x41, 0x08, 0x00, 0x58, 0x04):
            for w in (5, 40, 100, 230, 480, 900):
                p = base.subset(np.arange(0, 600, 7))
                p.dual = dual
                p.q2, p.e2 = (24, 1) if dual else (12, 2)
                p.jobs["w"], p.jobs["flag"] = w, flag
                _batch_vs_oracle(ctx, p)


def test_tiny_traceback_budget_forces_many_waves(built):
    from minibwa_gb300 import Context, synth
    c = Context(0, tb_budget=2 << 20)
    try:
        _batch_vs_oracle(c, synth.config1(3000, seed=5))
    finally:
        c.close()


def test_full_size_config1_properties(ctx):
    """1,000,000 pairs: a resident batch run twice gives identical output, and a random
    sample of 3,000 pairs matches the checker exactly."""
    from minibwa_gb300 import ExtBatch, synth
    p = synth.config1()
    b = ExtBatch(ctx, p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    b.run()
    r1, c1 = b.fetch()
    b.run()
    r2, c2 = b.fetch()
    b.free()
    for f in EXT_FIELDS:
        assert np.array_equal(r1[f], r2[f])
    # CIGAR placement may differ between runs (atomic reservation); content may not
    k = r1["n_cigar"]
    assert np.array_equal(k, r2["n_cigar"])
    rng = np.random.default_rng(3)
    idx = np.sort(rng.choice(len(p), 3000, replace=False))
    sub = p.subset(idx)
    ores, ocig = O.ext_batch("orc", sub.dual, 5, sub.mat, sub.q, sub.e, sub.q2, sub.e2, sub.jobs, sub.qbuf, sub.tbuf, 8)
    g = r1[idx].copy()
    compare_ext(g, c1, ores, ocig)
    # CIGAR spans agree with the reported end points
    for i in idx[:500]:
        n = int(r1["n_cigar"][i])
        if n == 0:
            continue
        ops = c1[r1["cigar_off"][i]:r1["cigar_off"][i] + n]
        ql = sum(int(x >> 4) for x in ops if (x & 0xf) in (0, 1))
        tl = sum(int(x >> 4) for x in ops if (x & 0xf) in (0, 2))
        if r1["reach_end"][i]:
            assert ql == p.jobs["qlen"][i] and tl == r1["mqe_t"][i] + 1
        else:
            assert ql == r1["max_q"][i] + 1 and tl == r1["max_t"][i] + 1


def test_one_shot_chunked_equals_resident(built):
    """One-shot batches above the chunk size run as overlapped chunks on two streams; every
    result and CIGAR equals the resident single-launch run of the same jobs."""
    from minibwa_gb300 import Context, ExtBatch, synth
    from conftest import EXT_FIELDS
    p = synth.config0(300000, seed=77)
    ctx = Context(0)
    res, cig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    b = ExtBatch(ctx, p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    b.run()
    want, wcig = b.fetch()
    b.free()
    ctx.close()
    for f in EXT_FIELDS:
        assert np.array_equal(res[f], want[f]), f
    assert len(cig) == len(wcig)
    for i in range(0, len(p), 997):
        o, n = int(res["cigar_off"][i]), int(res["n_cigar"][i])
        wo = int(want["cigar_off"][i])
        assert np.array_equal(cig[o:o + n], wcig[wo:wo + n]), i
    # the CIGARs tile the used part of the buffer without overlap
    live = res["n_cigar"] > 0
    o = res["cigar_off"][live].astype(np.int64)
    n = res["n_cigar"][live].astype(np.int64)
    k = np.argsort(o, kind="stable")
    assert (o[k][1:] >= o[k][:-1] + n[k][:-1]).all() and o[k][-1] + n[k][-1] <= len(cig)


def _wide_pairs(n, lo, hi, w, flag, dual, seed):
    from minibwa_gb300 import synth
    spec = dict(synth.SPEC_LONG, clip_lo=lo, clip_hi=hi)
    p = synth.ext_pairs(n, spec, w, 400, 10, flag, dual, seed=seed)
    return p


def test_wide_bands_block_kernel(ctx):
    """Bands wider than the widest thread group (long reads' end extension with w up to
    bw_long) on the block-wide kernel (the block-split kernel, which takes such bands by
    default, is off here): batched alone, mixed with narrow pairs in one batch, with several
    traceback modes in one batch (their block-wide bins share the wave's scratch, so they run
    on one stream), and over many waves."""
    import minibwa_gb300.lib as K
    from minibwa_gb300 import Context
    prev = K.set_ext_split(0)
    try:
        for flag in (0x40, 0x00, 0xc2, 0x08, 0x41):
            for dual in (0, 1):
                _batch_vs_oracle(ctx, _wide_pairs(6, 1500, 4000, -1, flag, dual, seed=flag + dual))
        mixed = _wide_pairs(40, 300, 3000, 1200, 0x40, 1, seed=3)   # narrow and wide jobs in one batch
        _batch_vs_oracle(ctx, mixed)
        modes = _wide_pairs(12, 1500, 3000, -1, 0x40, 1, seed=5)    # score-only, left and right gaps
        modes.jobs["flag"] = np.array([0x40, 0x41, 0xc2] * 4, np.int32)
        _batch_vs_oracle(ctx, modes)
        c = Context(0, tb_budget=64 << 20)                           # many waves, two streams
        try:
            _batch_vs_oracle(c, _wide_pairs(12, 1500, 3000, 2500, 0x40, 1, seed=9))
        finally:
            c.close()
    finally:
        K.set_ext_split(prev)


def test_wide_band_per_call(built):
    import minibwa_gb300.lib as K
    p = _wide_pairs(3, 2000, 3000, 3000, 0x40, 1, seed=21)
    prev = K.set_ext_split(0)  # the block-wide kernel, not the block-split one
    try:
        _per_call_wide(K, p)
    finally:
        K.set_ext_split(prev)


def _per_call_wide(K, p):
    for i in range(len(p)):
        q, t = p.query(i), p.target(i)
        ez = K.ksw_extd2_sse(q, t, 5, p.mat, p.q, p.e, p.q2, p.e2, 3000, 400, 10, 0x40)
        exp, _ = O.extz(1, q, t, 5, p.mat, p.q, p.e, p.q2, p.e2, 3000, 400, 10, 0x40)
        got = ez.fields()
        for f in EXT_FIELDS + ["cigar"]:
            assert got[f] == exp[f], (i, f)
        K.free_extz(ez)
