"""Mate rescue on the device (ksw2g_rescue_batch): every stage's output equals the oracle's
restatement of pe.c (mb_ungap, the narrowing, ksw_ll, the reverse extz2 and the hit), and the
hits equal the reference's own mb_matesw_core through the golden fixture."""
import numpy as np
import pytest

from test_rescue import expected_hits, load_rescue_golden, oracle_as_hit

pytestmark = pytest.mark.gpu

EXT_KEYS = ("score", "max", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "zdropped", "reach_end", "n_cigar")


def compare_to_oracle(ref, opt, jobs, qbuf, res, cig):
    from oracle import oracle as O
    n_hit = 0
    for i, j in enumerate(jobs):
        q = qbuf[j["qoff"]:j["qoff"] + j["qlen"]]
        o = O.rescue(ref, opt, int(j["tid"]), int(j["ts"]), int(j["te"]), q, int(j["meth"]), int(j["min_sc"]),
                     int(j["rev"]))
        r = res[i]
        got = {k: int(r[k]) for k in ("max_ug", "max_i", "n_good", "n_kmer", "ts2", "te2", "ll_done", "ext_done",
                                      "rescued")}
        exp = {k: int(o[k]) for k in got}
        assert got == exp, (i, got, exp)
        if o["ll_done"]:
            got = {k: int(r["ll_" + k]) for k in ("score", "te", "qe", "score2", "te2")}
            exp = {k: int(o["ll_" + k]) for k in got}
            assert got == exp, (i, "ksw_ll", got, exp)
        if o["ext_done"]:
            got = {k: int(r["ext"][k]) for k in EXT_KEYS}
            exp = {k: int(o["ext"][k]) for k in EXT_KEYS}
            assert got == exp, (i, "extz2", got, exp)
            k = int(r["ext"]["n_cigar"])
            c = cig[r["ext"]["cigar_off"]:r["ext"]["cigar_off"] + k].tolist() if k else []
            assert c == o["cigar"], (i, "CIGAR")
        if o["rescued"]:
            n_hit += 1
            got = {k: int(r[k]) for k in ("ts", "te", "qs", "qe", "dp_max2")}
            exp = {k: int(o[k]) for k in got}
            assert got == exp, (i, "hit", got, exp)
    return n_hit


@pytest.fixture(scope="module")
def ctx(built):
    from minibwa_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def test_rescue_golden(ctx):
    from minibwa_gb300 import Reference
    g, ref, opt = load_rescue_golden()
    dev = Reference(ctx, ref.pac, ref.ctg_off, ref.ctg_len, ref.ambi)
    try:
        res, cig = dev.rescue_batch(opt, g["jobs"], g["qbuf"])
    finally:
        dev.close()
    assert compare_to_oracle(ref, opt, g["jobs"], g["qbuf"], res, cig) > 400
    for i, j in enumerate(g["jobs"]):   # the reference's own hits, CIGARs included
        r = res[i]
        got = None
        if r["rescued"]:
            k = int(r["ext"]["n_cigar"])
            got = (dict(rescued=1, ts=int(r["ts"]), te=int(r["te"]), qs=int(r["qs"]), qe=int(r["qe"]),
                        rev=int(j["rev"]), dp_max=int(r["ext"]["max"]), dp_max2=int(r["dp_max2"]),
                        score=int(r["ll_score"]), subsc=int(r["ll_score2"]), n_cigar=k),
                   cig[r["ext"]["cigar_off"]:r["ext"]["cigar_off"] + k].tolist())
        assert got == expected_hits(g, i), i
        assert tuple(int(r[k]) for k in ("max_ug", "max_i", "n_good", "n_kmer")) == tuple(g["ungap"][i])


@pytest.mark.parametrize("kw", [dict(qlen_lo=40, qlen_hi=400, p_random=0.15, seed=301),
                                dict(qlen_lo=100, qlen_hi=300, lo=1000, hi=20000, p_meth=0.5, seed=302)])
def test_rescue_generated(ctx, kw):
    from minibwa_gb300 import Reference, synth
    ref = synth.Reference2b([400000, 250000, 5000], n_runs=40, n_repeats=500, seed=300)
    rc = synth.RescueCases(ref, 2500, **kw)
    opt = synth.RESCUE_OPT_SR
    dev = Reference(ctx, ref.pac, ref.ctg_off, ref.ctg_len, ref.ambi)
    try:
        res, cig = dev.rescue_batch(opt, rc.jobs, rc.qbuf)
    finally:
        dev.close()
    assert compare_to_oracle(ref, opt, rc.jobs, rc.qbuf, res, cig) > 1000


def test_rescue_long_windows_and_reads(ctx):
    """Windows past the shared-memory histogram (global votes) and a read past the uint16
    position table, next to ordinary candidates in one call."""
    from minibwa_gb300 import Reference, synth
    from minibwa_gb300.lib import RESCUE_JOB
    ref = synth.Reference2b([300000], n_runs=10, seed=310)
    rng = np.random.default_rng(311)
    opt = synth.RESCUE_OPT_SR
    jobs, parts, off = [], [], 0
    for ts, te, ql in [(1000, 61000, 150), (200000, 290000, 250), (5000, 6000, 120), (0, 140000, 70000),
                       (100, 52000, 300)]:
        st = int(rng.integers(ts, te - ql))
        q = ref.window(0, st, ql).copy() if ql < 65535 else rng.integers(0, 4, ql).astype(np.uint8)
        j = np.zeros(1, RESCUE_JOB)
        j["qoff"], j["ts"], j["te"], j["qlen"], j["tid"], j["min_sc"] = off, ts, te, ql, 0, 20
        jobs.append(j), parts.append(q)
        off += ql
    jobs, qbuf = np.concatenate(jobs), np.concatenate(parts)
    dev = Reference(ctx, ref.pac, ref.ctg_off, ref.ctg_len, ref.ambi)
    try:
        res, cig = dev.rescue_batch(opt, jobs, qbuf)
    finally:
        dev.close()
    compare_to_oracle(ref, opt, jobs, qbuf, res, cig)
    assert tuple(res[3][["max_ug", "max_i", "n_good", "n_kmer"]].tolist()) == (0, -1, 0, 0)
    assert res[0]["rescued"] and res[1]["rescued"] and res[4]["rescued"]


def test_rescue_arguments(ctx):
    from minibwa_gb300 import Reference, synth
    from minibwa_gb300.lib import RESCUE_JOB
    ref = synth.Reference2b([20000], n_runs=0, seed=320)
    dev = Reference(ctx, ref.pac, ref.ctg_off, ref.ctg_len, ref.ambi)
    try:
        res, cig = dev.rescue_batch(synth.RESCUE_OPT_SR, np.zeros(0, RESCUE_JOB), np.zeros(1, np.uint8))
        assert len(res) == 0 and len(cig) == 0
        j = np.zeros(1, RESCUE_JOB)
        j["ts"], j["te"], j["qlen"] = 19000, 20001, 100   # past the contig's end
        with pytest.raises(RuntimeError):
            dev.rescue_batch(synth.RESCUE_OPT_SR, j, np.zeros(100, np.uint8))
        j["te"], j["meth"] = 20000, 3                      # no such methylation mode
        with pytest.raises(RuntimeError):
            dev.rescue_batch(synth.RESCUE_OPT_SR, j, np.zeros(100, np.uint8))
    finally:
        dev.close()
