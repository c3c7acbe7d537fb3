"""ksw2g_align_chains on the device: every hit's result -- coordinates, dp_score, CIGAR and the
z-drop split -- equals the reference's own mb_align1 through the golden fixture, and the
oracle's restatement on fresh seeds."""
import numpy as np
import pytest

from test_chains import chain_sets, expected, load_chains_golden, read_of

pytestmark = pytest.mark.gpu


def as_align1(chain, r, cig):
    """A CHAIN_RESULT record in the shape of the reference harness's output."""
    d = dict(ts=int(r["ts"]), te=int(r["te"]), qs=int(r["qs"]), qe=int(r["qe"]), dp_score=int(r["dp_score"]),
             n_cigar=int(r["n_cigar"]), cnt=int(r["cnt"]), score=int(r["score"]), r2_cnt=0, r2_as=0,
             r2_split_inv=0, r2_score=0)
    if r["split_n"] > 0:
        d.update(r2_cnt=int(chain["cnt"]) - int(r["split_n"]), r2_as=int(chain["as"]) + int(r["split_n"]),
                 r2_split_inv=int(r["split_inv2"]), r2_score=int(chain["score"]) - int(r["score"]))
    d["cigar"] = cig[r["cigar_off"]:r["cigar_off"] + r["n_cigar"]].tolist() if r["n_cigar"] else []
    return d


@pytest.fixture(scope="module")
def dev(built):
    from minibwa_gb300 import Context
    ctx = Context(0)
    yield ctx
    ctx.close()


def test_chains_golden(dev):
    from minibwa_gb300.lib import Reference
    z = load_chains_golden()
    ref = Reference(dev, z["pac"], z["ctg_off"], z["ctg_len"], z["ambi"])
    for name, opt, idx in chain_sets(z):
        ch = z["chains"][idx.start:idx.stop]
        res, cig = ref.align_chains(opt, ch, z["anchors"].copy(), z["qbuf"])
        for k, i in enumerate(idx):
            got = as_align1(ch[k], res[k], cig)
            assert got == expected(z, i), (name, i)
            assert res[k]["n_dp"] <= res[k]["n_dp_issued"]
    ref.close()


def test_chains_oracle_fresh_seeds(dev):
    from oracle import oracle as O
    from minibwa_gb300 import synth
    from minibwa_gb300.lib import Reference
    R = synth.Reference2b([400000, 250000, 120000], n_runs=12, seed=310)
    ref = Reference(dev, R.pac, R.ctg_off, R.ctg_len, R.ambi)
    for lr, n, opt, meth in ((False, 1200, synth.CHAIN_OPT_SR, False), (True, 48, synth.CHAIN_OPT_LR, False),
                             (False, 300, dict(synth.CHAIN_OPT_SR, meth=1, b_ts=4), True),
                             (True, 24, dict(synth.CHAIN_OPT_LR, meth=1), True)):
        cs = synth.ChainCases(R, n, long_reads=lr, seed=311 + n, meth=meth)
        res, cig = ref.align_chains(opt, cs.chains, cs.anchors.copy(), cs.qbuf)
        for i in range(len(cs)):
            exp = O.align1(R, opt, cs.anchors, cs.chains[i], cs.read(i))
            assert as_align1(cs.chains[i], res[i], cig) == exp, (lr, meth, i, cs.kind[i])
    ref.close()


def test_chains_several_option_sets(dev):
    """One call over hits of three option sets that share their scores (short-read preset,
    long-read preset, long reads under the short-read preset's adaptive switch)."""
    from minibwa_gb300.lib import CHAIN, Reference
    z = load_chains_golden()
    ref = Reference(dev, z["pac"], z["ctg_off"], z["ctg_len"], z["ambi"])
    sets = [s for s in chain_sets(z) if s[0] != "sr_meth"]
    opts = [s[1] for s in sets]
    idx = np.concatenate([np.arange(s[2].start, s[2].stop) for s in sets])
    ch = np.zeros(len(idx), CHAIN)
    for k in ("as", "qoff", "cnt", "mlen", "score", "qlen", "meth", "split_inv"):
        ch[k] = z["chains"][k][idx]
    ch["opt"] = np.concatenate([np.full(len(s[2]), i) for i, s in enumerate(sets)])
    perm = np.random.default_rng(5).permutation(len(ch))  # hits of the sets interleaved
    res, cig = ref.align_chains(opts, ch[perm], z["anchors"].copy(), z["qbuf"])
    for k, p in enumerate(perm):
        assert as_align1(ch[p], res[k], cig) == expected(z, int(idx[p])), int(idx[p])
    meth_opt = next(s[1] for s in chain_sets(z) if s[0] == "sr_meth")
    with pytest.raises(RuntimeError):  # option sets with other scores in one call
        ref.align_chains([opts[0], meth_opt], ch[:2], z["anchors"].copy(), z["qbuf"])
    ref.close()


def test_chains_edges(dev):
    from minibwa_gb300.lib import CHAIN, Reference
    z = load_chains_golden()
    ref = Reference(dev, z["pac"], z["ctg_off"], z["ctg_len"], z["ambi"])
    opt = next(chain_sets(z))[1]
    res, cig = ref.align_chains(opt, np.zeros(0, CHAIN), z["anchors"].copy(), z["qbuf"])
    assert len(res) == 0 and len(cig) == 0
    ch = z["chains"][:3].copy()
    ch[1]["cnt"] = 0  # mb_align1 returns at once for a hit without anchors
    res, cig = ref.align_chains(opt, ch, z["anchors"].copy(), z["qbuf"])
    assert res[1]["n_cigar"] == 0 and res[1]["cigar_off"] == -1 and res[1]["n_dp_issued"] == 0
    for k in (0, 2):
        assert as_align1(ch[k], res[k], cig) == expected(z, k)
    bad = z["chains"][:2].copy()
    bad[1]["as"] = len(z["anchors"])  # anchors out of range: refused before any device work
    with pytest.raises(RuntimeError):
        ref.align_chains(opt, bad, z["anchors"].copy(), z["qbuf"])
    with pytest.raises(RuntimeError):  # CIGAR buffer too small
        ref.align_chains(opt, z["chains"][:4], z["anchors"].copy(), z["qbuf"], cigar_cap=1)
    ref.close()


@pytest.mark.parametrize("threads", ["1", "3"])
def test_chains_host_thread_count(built, threads):
    """The host stages of ksw2g_align_chains split hits over threads (KSW2G_HOST_THREADS, read once
    per process): one and three threads give the fixture's results too."""
    import os
    import subprocess
    import sys
    from conftest import ROOT
    code = (
        "import sys; sys.path.insert(0, 'tests')\n"
        "from test_chains import chain_sets, expected, load_chains_golden\n"
        "from test_gpu_chains import as_align1\n"
        "from minibwa_gb300 import Context\n"
        "from minibwa_gb300.lib import Reference\n"
        "z = load_chains_golden(); ctx = Context(0)\n"
        "ref = Reference(ctx, z['pac'], z['ctg_off'], z['ctg_len'], z['ambi'])\n"
        "bad = 0\n"
        "for name, opt, idx in chain_sets(z):\n"
        "    ch = z['chains'][idx.start:idx.stop]\n"
        "    res, cig = ref.align_chains(opt, ch, z['anchors'].copy(), z['qbuf'])\n"
        "    bad += sum(as_align1(ch[k], res[k], cig) != expected(z, i) for k, i in enumerate(idx))\n"
        "print('mismatches', bad)\n")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                         env=dict(os.environ, KSW2G_HOST_THREADS=threads))
    assert out.returncode == 0, out.stderr[-2000:]
    assert "mismatches 0" in out.stdout, out.stdout
