"""mb_align1 over whole hits (speculative gap fill): the oracle's restatement of align.c:548-757
equals the reference's own mb_align1 through the golden fixture, and, where the reference tree
is present, the fixture equals a fresh run of the reference on the same inputs."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CHAINS_GOLDEN = os.path.join(ROOT, "tests", "golden", "chains_golden.npz")


class RefArrays:
    """The 2-bit reference of a fixture, in the attributes the oracle reads."""

    def __init__(self, z):
        self.pac, self.ctg_off, self.ctg_len, self.ambi = z["pac"], z["ctg_off"], z["ctg_len"], z["ambi"]


def load_chains_golden():
    z = dict(np.load(CHAINS_GOLDEN))
    z["ref"] = RefArrays(z)
    return z


def chain_sets(z):
    """(name, opt dict, index range) of every option set in the fixture."""
    from oracle import oracle as O
    for si in range(len(z["set_lo"]) - 1):
        yield (str(z["set_names"][si]), {k: int(v) for k, v in zip(O.CHAIN_OPT, z["opts"][si])},
               range(int(z["set_lo"][si]), int(z["set_lo"][si + 1])))


def expected(z, i):
    from oracle import oracle as O
    d = {k: int(v) for k, v in zip(O.ALIGN1_OUT, z["out"][i])}
    d["cigar"] = [int(x) for x in z["cigar"][z["cigar_off"][i]:z["cigar_off"][i + 1]]]
    return d


def read_of(z, i):
    c = z["chains"][i]
    return z["qbuf"][c["qoff"]:c["qoff"] + c["qlen"]]


def test_fixture_covers_the_paths():
    z = load_chains_golden()
    out = z["out"]
    names = [s[0] for s in chain_sets(z)]
    assert names == ["sr", "sr_meth", "lr", "adaptive"]
    assert (out[:, 8] > 0).sum() >= 10, "z-drop splits"
    assert (out[:, 10] > 0).sum() >= 3, "splits flagged as inversions"
    assert (z["chains"]["split_inv"] > 0).sum() >= 50
    assert (z["chains"]["meth"] > 0).sum() >= 40
    assert (z["anchors"]["sid"] & 1).sum() > len(z["anchors"]) // 4


def test_oracle_align1_matches_reference_fixture(built):
    from oracle import oracle as O
    z = load_chains_golden()
    for name, opt, idx in chain_sets(z):
        for i in idx:
            got = O.align1(z["ref"], opt, z["anchors"], z["chains"][i], read_of(z, i))
            exp = expected(z, i)
            assert {k: got[k] for k in exp} == exp, (name, i)


def test_fixture_matches_reference_run(built):
    from oracle import oracle as O
    from minibwa_gb300.synth import _revcomp
    if not O.have_ref_pe():
        pytest.skip("the reference tree is not present")
    z = load_chains_golden()
    for name, opt, idx in chain_sets(z):
        for i in list(idx)[::7]:
            c = z["chains"][i]
            s = read_of(z, i)
            fwd = _revcomp(s) if z["anchors"][c["as"]]["sid"] & 1 else s
            got = O.ref_align1(z["ref"], opt, z["anchors"], c, fwd, _revcomp(fwd))
            assert got == expected(z, i), (name, i)


def test_synthetic_hits_oracle_vs_reference(built):
    """Fresh seeds beyond the fixture: the restatement and the reference agree hit for hit."""
    from oracle import oracle as O
    from minibwa_gb300 import synth
    if not O.have_ref_pe():
        pytest.skip("the reference tree is not present")
    ref = synth.Reference2b([120000, 90000], n_runs=6, seed=300)
    for lr, n, opt in ((False, 160, synth.CHAIN_OPT_SR), (True, 24, synth.CHAIN_OPT_LR),
                       (False, 80, dict(synth.CHAIN_OPT_SR, meth=1, b_ts=4))):
        cs = synth.ChainCases(ref, n, long_reads=lr, seed=301 + n, meth=bool(opt["meth"]))
        for i in range(len(cs)):
            exp = O.ref_align1(ref, opt, cs.anchors, cs.chains[i], cs.fwd[i], cs.rc[i])
            got = O.align1(ref, opt, cs.anchors, cs.chains[i], cs.read(i))
            assert {k: got[k] for k in exp} == exp, (lr, i, cs.kind[i])
