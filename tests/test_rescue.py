"""Mate rescue (pe.c:209-372) on the CPU: the oracle's restatement of the pipeline against the
reference's own mb_ungap / l2b_getseq / mb_matesw_core, through the committed golden fixture
(always) and through the reference build itself (where the reference tree was built here)."""
import os
import types

import numpy as np
import pytest

from conftest import ROOT

GOLDEN_RESCUE = os.path.join(ROOT, "tests", "golden", "rescue_golden.npz")
CASE_COLS = ("tid", "h_ts", "h_te", "h_rev", "r0", "dir", "lo", "hi", "mt0", "min_sc")


def load_rescue_golden():
    from oracle import oracle as O
    g = dict(np.load(GOLDEN_RESCUE))
    ref = types.SimpleNamespace(pac=g["pac"], ctg_off=g["ctg_off"], ctg_len=g["ctg_len"], ambi=g["ambi"])
    opt = dict(zip(O.RESCUE_SC, [int(x) for x in g["opt"]]))
    return g, ref, opt


def expected_hits(g, i):
    """The reference's hit of golden candidate i as (fields, CIGAR), or None."""
    from oracle import oracle as O
    if not g["has_hit"][i]:
        return None
    d = dict(zip(O.HIT_FIELDS, [int(x) for x in g["hit"][i]]))
    return d, [int(x) for x in g["cigar"][g["cigar_off"][i]:g["cigar_off"][i + 1]]]


def oracle_as_hit(o, job):
    """The oracle's rescue result in the reference's hit fields (pe.c:291-304, 361-368)."""
    if not o["rescued"]:
        return None
    return dict(rescued=1, ts=o["ts"], te=o["te"], qs=o["qs"], qe=o["qe"], rev=int(job["rev"]), dp_max=o["ext"]["max"],
                dp_max2=o["dp_max2"], score=o["ll_score"], subsc=o["ll_score2"], n_cigar=len(o["cigar"])), o["cigar"]


@pytest.fixture(scope="module")
def rg():
    from oracle import oracle as O
    O.oracle_lib()
    return load_rescue_golden()


def test_oracle_ungap_matches_golden(rg):
    from oracle import oracle as O
    g, ref, opt = rg
    for i, j in enumerate(g["jobs"]):
        q = g["qbuf"][j["qoff"]:j["qoff"] + j["qlen"]]
        w = O.l2b_getseq(ref, int(j["tid"]), int(j["ts"]), int(j["te"] - j["ts"]))
        assert O.ungap(q, w, 7, int(j["meth"])) == tuple(int(x) for x in g["ungap"][i]), i


def test_oracle_rescue_matches_golden(rg):
    from oracle import oracle as O
    g, ref, opt = rg
    n_hit = 0
    for i, j in enumerate(g["jobs"]):
        q = g["qbuf"][j["qoff"]:j["qoff"] + j["qlen"]]
        o = O.rescue(ref, opt, int(j["tid"]), int(j["ts"]), int(j["te"]), q, int(j["meth"]), int(j["min_sc"]),
                     int(j["rev"]))
        assert oracle_as_hit(o, j) == expected_hits(g, i), i
        n_hit += o["rescued"]
    assert n_hit > 400  # the fixture exercises the extension stage, not only the filters


def test_golden_windows_follow_pe_geometry(rg):
    """The fixture's windows are pe.c:330-339's for the stored anchors and orientations."""
    from minibwa_gb300 import synth
    g, ref, opt = rg
    for i, j in enumerate(g["jobs"]):
        c = dict(zip(CASE_COLS, [int(x) for x in g["cases"][i]]))
        ts, te, is_rev = synth.rescue_window(c["dir"], c["lo"], c["hi"], c["h_ts"], c["h_te"], c["h_rev"], c["r0"],
                                             int(j["qlen"]), int(ref.ctg_len[c["tid"]]))
        assert (ts, te, is_rev) == (int(j["ts"]), int(j["te"]), int(j["rev"])), i
        assert int(j["meth"]) == (synth.meth_rev(c["mt0"]) if is_rev else c["mt0"])


def test_oracle_ungap_edges():
    from oracle import oracle as O
    rng = np.random.default_rng(9)
    q = rng.integers(0, 4, 150).astype(np.uint8)
    assert O.ungap(q[:6], q, 7, 0) == (0, -1, 0, 0)          # no 7-mer in the read
    assert O.ungap(q, np.zeros(0, np.uint8), 7, 0)[:2] == (0, -1)
    assert O.ungap(np.full(70000, 0, np.uint8), q, 7, 0) == (0, -1, 0, 0)  # positions past the uint16 table
    t = np.concatenate([rng.integers(0, 4, 300), q, rng.integers(0, 4, 300)]).astype(np.uint8)
    mx, mi, ng, nk = O.ungap(q, t, 7, 0)
    assert mx >= 130 and ng == 1 and mi == 300 and nk >= mx
    qn = q.copy()
    qn[::6] = 4                                             # an N in every 7-mer window
    assert O.ungap(qn, t, 7, 0)[0] == 0


@pytest.fixture(scope="module")
def refpe(built):
    from oracle import oracle as O
    if not O.have_ref_pe():
        pytest.skip("reference rescue build not available")
    return O


def test_ungap_restatement_matches_reference(refpe):
    O = refpe
    rng = np.random.default_rng(21)
    for it in range(400):
        ql, tl = int(rng.integers(0, 400)), int(rng.integers(0, 3000))
        q = rng.integers(0, 4, ql).astype(np.uint8)
        t = rng.integers(0, 4, tl).astype(np.uint8)
        if tl > ql and rng.random() < 0.7:                    # plant the read
            p = int(rng.integers(0, tl - ql + 1))
            t[p:p + ql] = q
        for a in (q, t):
            if len(a) and rng.random() < 0.3:
                a[rng.random(len(a)) < 0.02] = 4
        mt = int(rng.integers(0, 3))
        assert O.ungap(q, t, 7, mt) == O.ref_ungap(q, t, 7, mt), it


def test_getseq_restatement_matches_reference(refpe):
    O = refpe
    from minibwa_gb300 import synth
    r = synth.Reference2b([5000, 33, 20000], n_runs=40, run_max=300, seed=77)
    rng = np.random.default_rng(5)
    for it in range(300):
        k = int(rng.integers(0, 3))
        L = min(int(rng.integers(1, 1500)), int(r.ctg_len[k]))
        st = int(rng.integers(0, int(r.ctg_len[k]) - L + 1))
        assert np.array_equal(O.ref_getseq(r, k, st, st + L), O.l2b_getseq(r, k, st, L)), it


@pytest.mark.parametrize("kw", [dict(qlen_lo=40, qlen_hi=400, p_random=0.15, seed=201),
                                dict(qlen_lo=150, qlen_hi=350, lo=2000, hi=9000, p_meth=0.5, seed=202)])
def test_rescue_restatement_matches_reference(refpe, kw):
    O = refpe
    from minibwa_gb300 import synth
    ref = synth.Reference2b([90000, 70000], n_runs=20, n_repeats=200, seed=203)
    rc = synth.RescueCases(ref, 250, **kw)
    opt = synth.RESCUE_OPT_SR
    for i, (c, j) in enumerate(zip(rc.cases, rc.jobs)):
        o = O.rescue(ref, opt, c["tid"], c["ts"], c["te"], c["seq"][c["is_rev"]], c["mt"], c["min_sc"], c["is_rev"])
        r = O.ref_matesw(ref, opt, c["dir"], c["lo"], c["hi"], c["tid"], c["h_ts"], c["h_te"], c["h_rev"], c["r0"],
                         c["seq"][0], c["seq"][1], c["mt0"], c["min_sc"])
        exp = None if r is None else ({k: r[k] for k in O.HIT_FIELDS}, r["cigar"])
        assert oracle_as_hit(o, j) == exp, i
