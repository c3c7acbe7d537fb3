"""align.c's mb_align_pair (the ungapped shortcuts, band shrink and memory cap in front of every
DP call of mb_align1) on the CPU: the oracle's restatement against the reference's own function,
through the committed golden fixture and, where the reference was built here, directly."""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLDEN_ALIGN = os.path.join(ROOT, "tests", "golden", "align_golden.npz")


def align_cases():
    from oracle import oracle as O
    g = dict(np.load(GOLDEN_ALIGN))
    scorings = []
    for row in g["scoring"]:
        sc = dict(zip(O.ALIGN_SC, [int(x) for x in row[:len(O.ALIGN_SC)]]))
        sc["max_sw_mat"], sc["mt"] = int(row[-2]), int(row[-1])
        scorings.append(sc)
    for i, (si, w, eb, zd, fl) in enumerate(g["params"]):
        sc = scorings[si]
        out = dict(zip(O.ALIGN_OUT, [int(x) for x in g["out"][i]]))
        out["cigar"] = [int(x) for x in g["cigar"][g["cigar_off"][i]:g["cigar_off"][i + 1]]]
        yield dict(si=int(si), scoring=sc, mat=O.gen_nt4_mat(sc["a"], sc["b"], sc["b_ts"], sc["b_ambi"], sc["mt"]),
                   query=g["q"][g["qoff"][i]:g["qoff"][i + 1]], target=g["t"][g["toff"][i]:g["toff"][i + 1]],
                   w=int(w), end_bonus=int(eb), zdrop=int(zd), flag=int(fl), out=out)


def test_fixture_reaches_every_branch():
    cases = list(align_cases())
    outs = [c["out"] for c in cases]
    assert len(cases) == 1500
    assert sum(o["reach_end"] and o["n_cigar"] == 1 for o in outs) > 100          # ungapped extension
    assert sum(c["flag"] & 0x40 == 0 and c["out"]["n_cigar"] == 1 and c["out"]["max"] == 0 for c in cases) > 50
    assert sum(o["zdropped"] and o["max"] == 0 and o["n_cigar"] == 0 for o in outs) > 20   # memory cap
    assert len({c["si"] for c in cases}) == 5


def test_oracle_matches_golden_align_pairs(built):
    from oracle import oracle as O
    for n, c in enumerate(align_cases()):
        got = O.align_pair(c["scoring"], c["mat"], c["query"], c["target"], c["w"], c["end_bonus"], c["zdrop"],
                           c["flag"])
        assert got == c["out"], (n, got, c["out"])


def test_align_pair_restatement_matches_reference(built):
    from oracle import oracle as O
    if not O.have_ref_pe():
        pytest.skip("reference build not available")
    rng = np.random.default_rng(99)
    sc = dict(a=2, b=8, b_ts=0, b_ambi=1, q=12, e=2, q2=23, e2=1, meth=0, max_sw_mat=30000)
    mat = O.gen_nt4_mat(2, 8, 0, 1)
    for it in range(600):
        ql = int(rng.integers(0, 200))
        q = rng.integers(0, 4, ql).astype(np.uint8)
        t = np.concatenate([q, rng.integers(0, 4, int(rng.integers(0, 30))).astype(np.uint8)])
        t[rng.random(len(t)) < rng.random() * 0.05] = 3
        if it % 3 == 0:
            t = t[:ql]
        fl = int(rng.choice([0x40, 0xc2, 0x48, 0x00, 0x08]))
        args = (sc, mat, q, t, int(rng.choice([10, 100])), int(rng.choice([-1, 10])), 100, fl)
        assert O.align_pair(*args) == O.ref_align_pair(*args), it
