"""The device kernels' source, compiled for the host with tests/emu/cuda_emu.h and run
on the CPU: the exact code paths of the CUDA kernels (window sliding, shuffles, votes,
lockstep groups, the device work counter, the backtrack) checked against the golden
vectors and the oracle without a GPU."""
import os
import sys

import numpy as np
import pytest

from conftest import EXT_FIELDS, LL_FIELDS, ROOT, golden_ext_cases, golden_ll_cases

sys.path.insert(0, os.path.join(ROOT, "tests", "emu"))


@pytest.fixture(scope="module")
def emu(built):
    import emu as E
    E.lib()
    return E


def test_emulated_kernels_match_golden_extension(emu, golden):
    cases = list(golden_ext_cases(golden))
    for i, c in enumerate(cases[::3]):  # 200 of the 600 cases keep the CPU suite short
        res, cig = emu.ext(c["dual"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"], [c["query"]], [c["target"]],
                           c["w"], c["zdrop"], c["end_bonus"], c["flag"])
        got = {f: int(res[0][f]) for f in EXT_FIELDS}
        assert got == c["out"], (i, got, c["out"])
        assert cig[0] == c["cigar"], i


def test_emulated_16bit_kernels_match_golden_extension(emu, golden):
    """The 16-bit-lane DPX kernels (ext16_dp.cuh) on the golden cases, every fourth one."""
    cases = list(golden_ext_cases(golden))
    for i, c in enumerate(cases[1::4]):
        res, cig = emu.ext(c["dual"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"], [c["query"]], [c["target"]],
                           c["w"], c["zdrop"], c["end_bonus"], c["flag"], family=1)
        got = {f: int(res[0][f]) for f in EXT_FIELDS}
        assert got == c["out"], (i, got, c["out"])
        assert cig[0] == c["cigar"], i


def test_emulated_kernels_match_golden_ll(emu, golden):
    cases = list(golden_ll_cases(golden))
    for i, c in enumerate(cases[::3]):
        r = emu.ll(c["size"], c["m"], c["mat"], c["gapo"], c["gape"], [c["query"]], [c["target"]], c["xtra"])[0]
        assert {f: int(r[f]) for f in LL_FIELDS} == c["out"], (i, c["size"], c["xtra"])


def test_emulated_lockstep_groups_and_work_counter(emu):
    """Several groups per warp take jobs of different lengths from the work counter;
    each result must still equal the oracle (exercises group divergence)."""
    from minibwa_gb300 import synth
    from oracle import oracle as O
    p = synth.config0(24, seed=3)
    qs = [p.query(i)[: 40 + 7 * i] for i in range(len(p))]
    ts = [p.target(i)[: 50 + 5 * i] for i in range(len(p))]
    for dual, flag in ((0, 0x40), (1, 0xc2), (1, 0x41), (0, 0x08)):
        q2, e2 = (24, 1) if dual else (12, 2)
        res, cig = emu.ext(dual, 5, p.mat, 12, 2, q2, e2, qs, ts, 25, 100, 10, flag, threads=32, shape=0)
        res3, cig3 = emu.ext(dual, 5, p.mat, 12, 2, q2, e2, qs, ts, 25, 100, 10, flag, threads=32, shape=1)
        assert np.array_equal(res, res3) and cig == cig3
        for i in range(len(qs)):
            exp, _ = O.extz(dual, qs[i], ts[i], 5, p.mat, 12, 2, q2, e2, 25, 100, 10, flag)
            assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, i)
            assert cig[i] == exp["cigar"], (dual, flag, i)
    r = synth.config3_pe(12, seed=4)
    qs = [r.qbuf[j["qoff"]:j["qoff"] + j["qlen"]] for j in r.jobs]
    ts = [r.tbuf[j["toff"]:j["toff"] + j["tlen"] // (1 + i % 3)] for i, j in enumerate(r.jobs)]
    res = emu.ll(1, 5, r.mat, r.gapo, r.gape, qs, ts, int(r.jobs["xtra"][0]), threads=32)
    for i in range(len(qs)):
        exp, _ = O.ll(1, qs[i], ts[i], 5, r.mat, r.gapo, r.gape, int(r.jobs["xtra"][0]))
        assert {f: int(res[i][f]) for f in LL_FIELDS} == exp, i


def test_emulated_codes_above_n(emu):
    """Bytes 5-7 in the sequences take the general score comparisons, not the nt4 lookup."""
    from oracle import oracle as O
    rng = np.random.default_rng(23)
    mat = np.array([2 if i // 5 == i % 5 else -4 for i in range(25)], np.int8)
    mat[20:25] = -1
    mat[4::5] = -1
    for dual, flag in ((0, 0x42), (1, 0x40), (0, 0x00)):
        qs, ts = [], []
        for _ in range(8):
            base = rng.integers(0, 4, 70).astype(np.uint8)
            q, t = base[: int(rng.integers(20, 70))].copy(), base[: int(rng.integers(20, 70))].copy()
            q[rng.random(len(q)) < 0.2] = rng.integers(4, 8)
            t[rng.random(len(t)) < 0.1] = rng.integers(4, 8)
            qs.append(q), ts.append(t)
        res, cig = emu.ext(dual, 5, mat, 6, 1, 20, 1, qs, ts, 7, 100, 5, flag)
        for i in range(len(qs)):
            exp, _ = O.extz(dual, qs[i], ts[i], 5, mat, 6, 1, 20 if dual else 6, 1, 7, 100, 5, flag)
            assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, i)
            assert cig[i] == exp["cigar"], (dual, flag, i)


def test_emulated_one_cell_bands(emu):
    """Narrow bands against short targets pinch to one cell on consecutive anti-diagonals; H[en0]
    then reads H[en0-1] of a cell that already left the band (its last value, as the reference's
    array holds it), which the kernel carries as a scalar."""
    from oracle import oracle as O
    rng = np.random.default_rng(29)
    mat = np.array([3 if i // 5 == i % 5 else -4 for i in range(25)], np.int8)
    mat[20:25] = -1
    mat[4::5] = -1
    qs = [rng.integers(0, 4, 46).astype(np.uint8) for _ in range(4)]
    ts = [q[:tl].copy() for q, tl in zip(qs, (1, 2, 3, 5))]
    for dual in (0, 1):
        for flag in (0x00, 0x01, 0x40, 0x42):
            for w in (2, 3, 4, 6, 10):
                res, cig = emu.ext(dual, 5, mat, 3, 1, 20, 1, qs, ts, w, -1, 5, flag)
                for i in range(len(qs)):
                    exp, _ = O.extz(dual, qs[i], ts[i], 5, mat, 3, 1, 20 if dual else 3, 1, w, -1, 5, flag)
                    got = {f: int(res[i][f]) for f in EXT_FIELDS}
                    assert got == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, w, i)
                    assert cig[i] == exp["cigar"], (dual, flag, w, i)


def test_emulated_wide_band_shapes(emu):
    """Wide bands select the 16- and 32-thread shapes."""
    from minibwa_gb300 import synth
    from oracle import oracle as O
    p = synth.config1(4, seed=9)
    qs = [p.query(i) for i in range(len(p))]
    ts = [p.target(i) for i in range(len(p))]
    L = emu.lib()
    index = {(L.emu_shape_threads(s), L.emu_shape_words(s) // L.emu_shape_threads(s)): s
             for s in range(L.emu_num_shapes())}
    for w, g, k in ((100, 16, 2), (100, 8, 4), (100, 4, 8), (180, 16, 4), (230, 16, 4), (480, 32, 4), (480, 32, 5),
                    (900, 32, 8)):
        res, cig = emu.ext(1, 5, p.mat, 12, 2, 24, 1, qs, ts, w, 100, 10, 0x40, shape=index[(g, k)])
        for i in range(len(qs)):
            exp, _ = O.extz(1, qs[i], ts[i], 5, p.mat, 12, 2, 24, 1, w, 100, 10, 0x40)
            assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (w, i)
            assert cig[i] == exp["cigar"]


def test_emulated_dpx_ll_kernel_matches_golden(emu, golden):
    """The two-lanes-per-thread DPX kernel, wherever the host would choose it."""
    n = 0
    for i, c in enumerate(golden_ll_cases(golden)):
        mat_max = int(c["mat"].max())
        exact = c["size"] == 1 or (c["gape"] >= 0 and 0 <= c["gapo"] + c["gape"] <= 32767 and
                                   (len(c["query"]) + 1) * max(mat_max, 0) <= 32767)
        lanes = 16 if c["size"] == 1 else 8
        if not exact or (len(c["query"]) + lanes - 1) // lanes > 48:
            continue
        r = emu.ll(c["size"], c["m"], c["mat"], c["gapo"], c["gape"], [c["query"]], [c["target"]], c["xtra"],
                   dpx=True)[0]
        assert {f: int(r[f]) for f in LL_FIELDS} == c["out"], (i, c["size"], c["xtra"])
        n += 1
    assert n > 200


def test_emulated_long_query_ll_kernel(emu):
    """Queries beyond the 64 register-resident segments run on the shared-memory kernel."""
    from oracle import oracle as O
    from minibwa_gb300 import synth
    from minibwa_gb300.lib import gen_nt4_mat
    for size, ql, xtra, mat, go, ge in ((2, 1200, 0, None, 12, 2), (1, 1500, 0x40000 | 19, gen_nt4_mat(1, 4, 0, 1), 6, 1)):
        r = synth.ll_jobs(6, qlen=ql, tlen_lo=ql, tlen_hi=ql + 600, plant=0.7, size=size, xtra=xtra, mat=mat, gapo=go,
                          gape=ge, seed=ql)
        qs = [r.qbuf[o:o + n] for o, n in zip(r.jobs["qoff"], r.jobs["qlen"])]
        ts = [r.tbuf[o:o + n] for o, n in zip(r.jobs["toff"], r.jobs["tlen"])]
        got = emu.ll(size, 5, r.mat, r.gapo, r.gape, qs, ts, xtra)
        want = O.ll_batch("orc", size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf, 4)
        for f in ("score", "te", "qe", "score2", "te2"):
            assert np.array_equal(got[f], want[f]), (size, f, got[f], want[f])


def test_emulated_block_wide_kernel(emu):
    """Bands wider than the widest thread group (here w=-1 on ~1.2 kb pairs: 76+ blocks) run
    on the block-wide kernel; every flag family against the oracle."""
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    for flag in (0x40, 0x00, 0xc2, 0x41, 0x08, 0x18, 0x04):
        for dual in (0, 1):
            qs, ts = [], []
            for _ in range(2):
                q = rng.integers(0, 4, int(rng.integers(1100, 1400))).astype(np.uint8)
                t = q.copy()
                sub = rng.random(len(t)) < 0.03
                t[sub] = rng.integers(0, 5, sub.sum())
                t = np.concatenate([t[:300], rng.integers(0, 4, 7).astype(np.uint8), t[300:],
                                    rng.integers(0, 4, int(rng.integers(0, 200))).astype(np.uint8)])
                qs.append(q), ts.append(t)
            mat = np.array([2 if i // 5 == i % 5 else -8 for i in range(25)], np.int8)
            mat[20:25] = -1
            mat[4::5] = -1
            q2, e2 = (24, 1) if dual else (12, 2)
            res, cig = emu.ext(dual, 5, mat, 12, 2, q2, e2, qs, ts, -1, 100, 10, flag)
            for k in range(len(qs)):
                exp, _ = O.extz(dual, qs[k], ts[k], 5, mat, 12, 2, q2, e2, -1, 100, 10, flag)
                got = {f: int(res[f][k]) for f in EXT_FIELDS if f in exp}
                for f in got:
                    assert got[f] == exp[f], (flag, dual, k, f, got[f], exp[f])
                assert cig[k] == exp["cigar"], (flag, dual, k)


@pytest.mark.parametrize("global_hist", [False, True])
def test_emulated_ungap_kernel(emu, global_hist):
    """The device mb_ungap (shared-memory or global vote histogram) against the oracle's
    restatement, on the golden rescue windows plus planted, N-rich and degenerate pairs."""
    from oracle import oracle as O
    from test_rescue import load_rescue_golden
    g, ref, opt = load_rescue_golden()
    pairs, meth = [], []
    for j in g["jobs"][:120]:
        pairs.append((g["qbuf"][j["qoff"]:j["qoff"] + j["qlen"]],
                      O.l2b_getseq(ref, int(j["tid"]), int(j["ts"]), int(j["te"] - j["ts"]))))
        meth.append(int(j["meth"]))
    rng = np.random.default_rng(17)
    for it in range(40):
        q = rng.integers(0, 4, int(rng.integers(0, 300))).astype(np.uint8)
        t = rng.integers(0, 4, int(rng.integers(0, 2000))).astype(np.uint8)
        if len(t) > len(q) and it % 2:
            p = int(rng.integers(0, len(t) - len(q) + 1))
            t[p:p + len(q)] = q
        if it % 3 == 0 and len(t):
            t[rng.random(len(t)) < 0.03] = 4
        pairs.append((q, t)), meth.append(it % 3)
    got = emu.ungap(pairs, meth, global_hist)
    for i, ((q, t), mt) in enumerate(zip(pairs, meth)):
        assert got[i] == O.ungap(q, t, 7, mt), i


SPLIT_SHAPES = ((1, 1), (2, 1), (3, 1), (1, 2), (2, 2), (1, 4))


def test_emulated_split_kernel_matches_golden(emu, golden):
    """The block-split kernel (ext_split.cuh) on the golden cases, every sixth one, in every block
    shape of up to three warps that holds the band."""
    cases = list(golden_ext_cases(golden))
    for i, c in enumerate(cases[2::6]):
        nc = emu.ncol(len(c["query"]), len(c["target"]), c["w"])
        for nw, k in SPLIT_SHAPES:
            if 32 * nw * k < 4 * nc:
                continue
            res, cig = emu.ext(c["dual"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"], [c["query"]],
                               [c["target"]], c["w"], c["zdrop"], c["end_bonus"], c["flag"], split=(nw, k))
            got = {f: int(res[0][f]) for f in EXT_FIELDS}
            assert got == c["out"], (i, nw, k, got, c["out"])
            assert cig[0] == c["cigar"], (i, nw, k)


def test_emulated_split_kernel_long_pairs(emu):
    """Pairs long enough for the window to slide many times across warp boundaries, with junk
    tails that z-drop, in both variants, every traceback mode and the approximate max, against
    the oracle; several pairs per block take jobs one after another."""
    from minibwa_gb300 import synth
    from oracle import oracle as O
    p = synth.config1(6, seed=41)
    qs = [p.query(i) for i in range(len(p))]
    ts = [p.target(i) for i in range(len(p))]
    for dual, flag, w, split in ((1, 0x40, 100, (2, 1)), (1, 0x42, 60, (1, 2)), (0, 0x00, 90, (3, 1)),
                                 (0, 0x41, 120, (2, 2)), (1, 0x18, 80, (2, 1)), (0, 0x58, 100, (1, 4)),
                                 (1, 0xc0, 200, (4, 1)), (0, 0x44, 100, (2, 1))):
        q2, e2 = (24, 1) if dual else (12, 2)
        res, cig = emu.ext(dual, 5, p.mat, 12, 2, q2, e2, qs, ts, w, 100, 10, flag, split=split)
        for i in range(len(qs)):
            exp, _ = O.extz(dual, qs[i], ts[i], 5, p.mat, 12, 2, q2, e2, w, 100, 10, flag)
            assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, w, i)
            assert cig[i] == exp["cigar"], (dual, flag, w, i)


def test_emulated_split_kernel_edges(emu):
    """One-cell bands, codes above N (the general score path) and empty sequences on the
    block-split kernel."""
    from oracle import oracle as O
    rng = np.random.default_rng(31)
    mat = np.array([3 if i // 5 == i % 5 else -4 for i in range(25)], np.int8)
    mat[20:25] = -1
    mat[4::5] = -1
    qs = [rng.integers(0, 4, 46).astype(np.uint8) for _ in range(4)]
    ts = [q[:tl].copy() for q, tl in zip(qs, (1, 2, 3, 5))]
    for dual in (0, 1):
        for flag in (0x00, 0x01, 0x40, 0x42):
            for w in (2, 6):
                res, cig = emu.ext(dual, 5, mat, 3, 1, 20, 1, qs, ts, w, -1, 5, flag, split=(2, 1))
                for i in range(len(qs)):
                    exp, _ = O.extz(dual, qs[i], ts[i], 5, mat, 3, 1, 20 if dual else 3, 1, w, -1, 5, flag)
                    assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, w)
                    assert cig[i] == exp["cigar"], (dual, flag, w, i)
    qs, ts = [], []
    for _ in range(6):
        base = rng.integers(0, 4, 160).astype(np.uint8)
        q, t = base[: int(rng.integers(60, 160))].copy(), base[: int(rng.integers(60, 160))].copy()
        q[rng.random(len(q)) < 0.1] = rng.integers(4, 8)
        t[rng.random(len(t)) < 0.05] = rng.integers(4, 8)
        qs.append(q), ts.append(t)
    qs.append(np.zeros(0, np.uint8)), ts.append(rng.integers(0, 4, 30).astype(np.uint8))
    for dual, flag in ((0, 0x42), (1, 0x40), (1, 0x01)):
        res, cig = emu.ext(dual, 5, mat, 6, 1, 20, 1, qs, ts, 40, 100, 5, flag, split=(2, 1))
        for i in range(len(qs)):
            exp, _ = O.extz(dual, qs[i], ts[i], 5, mat, 6, 1, 20 if dual else 6, 1, 40, 100, 5, flag)
            assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, i)
            assert cig[i] == exp["cigar"], (dual, flag, i)


def test_emulated_split_kernel_stops(emu):
    """Pairs stopped early -- z-drop under the exact and the approximate max, the extd2 early
    stop, bands that empty -- at every point of a pair, from the first anti-diagonals to just
    before the last, on one and two warps and one and two words a thread."""
    from oracle import oracle as O
    rng = np.random.default_rng(47)
    mat = np.array([2 if i // 5 == i % 5 else -4 for i in range(25)], np.int8)
    mat[20:25] = -1
    mat[4::5] = -1
    qs, ts = [], []
    for i in range(36):
        base = rng.integers(0, 4, 170).astype(np.uint8)
        q, t = base[: int(rng.integers(8, 150))].copy(), base[: int(rng.integers(8, 150))].copy()
        cut = int(rng.integers(0, max(len(q), 1)))
        q[cut:] = rng.integers(0, 4, len(q) - cut)  # a junk tail from a random point
        if i % 3 == 0:
            t = t[: max(1, len(q) // 3)]  # bands that empty early
        qs.append(q), ts.append(t)
    for dual, flag, w, zdrop, split in ((1, 0x40, 12, 8, (1, 1)), (0, 0x40, 30, 15, (2, 1)),
                                        (1, 0x00, 20, 5, (1, 2)), (0, 0x01, 6, 10, (2, 1)),
                                        (1, 0x18, 25, 12, (1, 1)), (0, 0x18, 40, 6, (2, 1)),
                                        (1, 0x41, 60, 30, (1, 2)), (0, 0x42, 3, 4, (1, 1))):
        q2, e2 = (24, 1) if dual else (4, 2)
        res, cig = emu.ext(dual, 5, mat, 4, 2, q2, e2, qs, ts, w, zdrop, 3, flag, split=split)
        for i in range(len(qs)):
            exp, _ = O.extz(dual, qs[i], ts[i], 5, mat, 4, 2, q2, e2, w, zdrop, 3, flag)
            assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, w, i)
            assert cig[i] == exp["cigar"], (dual, flag, w, i)


def test_emulated_split_kernel_wide_words(emu):
    """Two and four words a thread (the shapes of bands wider than the widest group), where
    each warp reduces its maximum first and only the warps that may hold the block's maximum
    look for its key; full-band extension (w < 0) of pairs of 100-300 bases."""
    from minibwa_gb300 import synth
    from oracle import oracle as O
    p = synth.config1(3, seed=43)
    qs = [p.query(i) for i in range(len(p))]
    ts = [p.target(i) for i in range(len(p))]
    for dual, flag, split in ((1, 0x40, (2, 4)), (0, 0x02, (3, 2)), (1, 0x01, (2, 2))):
        q2, e2 = (24, 1) if dual else (12, 2)
        nc = max(emu.ncol(len(a), len(b), -1) for a, b in zip(qs, ts))
        if 32 * split[0] * split[1] < 4 * nc:
            continue
        res, cig = emu.ext(dual, 5, p.mat, 12, 2, q2, e2, qs, ts, -1, 100, 10, flag, split=split)
        for i in range(len(qs)):
            exp, _ = O.extz(dual, qs[i], ts[i], 5, p.mat, 12, 2, q2, e2, -1, 100, 10, flag)
            assert {f: int(res[i][f]) for f in EXT_FIELDS} == {f: exp[f] for f in EXT_FIELDS}, (dual, flag, split, i)
            assert cig[i] == exp["cigar"], (dual, flag, split, i)
