"""Generate tests/golden/rescue_golden.npz from the reference's own mate rescue.

Run where the reference tree is available (it builds oracle/_ref/libmbpe.so, the
reference's pe.c behind oracle/ref_pe.c, from the reference sources first):

    python tests/golden/make_golden_rescue.py

The fixture holds a seeded 2-bit reference (130 kb over three contigs, N runs and
near-tandem repeats), rescue candidates drawn over both read lengths of the u8 and
i16 ksw_ll paths, all four orientations, both anchor strands, methylation modes and
contig edges, the reference's mb_ungap outputs and l2b_getseq windows for them, and
the hit mb_matesw_core returns (mb_update_extra left out), with its CIGAR.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from minibwa_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "rescue_golden.npz")
OPT = synth.RESCUE_OPT_SR
SETS = [dict(n=500, qlen_lo=40, qlen_hi=400, p_random=0.15, seed=101),
        dict(n=60, qlen_lo=100, qlen_hi=300, lo=1000, hi=12000, seed=102),
        dict(n=40, qlen_lo=60, qlen_hi=200, p_meth=1.0, seed=103)]


def main():
    O.build(ref=True)
    if not O.have_ref_pe():
        raise SystemExit("the reference tree is needed to generate the rescue fixture")
    ref = synth.Reference2b([60000, 40000, 30000], n_runs=12, seed=100, n_repeats=150)
    cases, jobs, qparts = [], [], []
    off = 0
    for kw in SETS:
        kw = dict(kw)
        rc = synth.RescueCases(ref, kw.pop("n"), **kw)
        for c, j in zip(rc.cases, rc.jobs):
            j = j.copy()
            j["qoff"] = off
            off += int(j["qlen"])
            cases.append(c), jobs.append(j), qparts.append(c["seq"][c["is_rev"]])
    jobs = np.array(jobs, dtype=jobs[0].dtype)
    n = len(cases)
    case_arr = np.array([[c[k] for k in ("tid", "h_ts", "h_te", "h_rev", "r0", "dir", "lo", "hi", "mt0", "min_sc")]
                         for c in cases], np.int64)
    ug = np.zeros((n, 4), np.int64)
    hit = np.full((n, len(O.HIT_FIELDS)), 0, np.int64)
    has_hit = np.zeros(n, np.int8)
    cig, cig_off = [], np.zeros(n + 1, np.int64)
    for i, c in enumerate(cases):
        q = qparts[i]
        w = O.ref_getseq(ref, c["tid"], c["ts"], c["te"])
        assert np.array_equal(w, O.l2b_getseq(ref, c["tid"], c["ts"], c["te"] - c["ts"]))
        ug[i] = O.ref_ungap(q, w, 7, c["mt"])
        r = O.ref_matesw(ref, OPT, c["dir"], c["lo"], c["hi"], c["tid"], c["h_ts"], c["h_te"], c["h_rev"], c["r0"],
                         c["seq"][0], c["seq"][1], c["mt0"], c["min_sc"])
        if r is not None:
            has_hit[i] = 1
            hit[i] = [r[k] for k in O.HIT_FIELDS]
            cig.extend(r["cigar"])
        cig_off[i + 1] = len(cig)
    np.savez_compressed(OUT, pac=ref.pac, ctg_off=ref.ctg_off, ctg_len=ref.ctg_len, ambi=ref.ambi, jobs=jobs,
                        qbuf=np.concatenate(qparts), cases=case_arr, ungap=ug, has_hit=has_hit, hit=hit,
                        cigar=np.array(cig, np.uint32), cigar_off=cig_off,
                        opt=np.array([OPT[k] for k in O.RESCUE_SC], np.int32))
    print(f"{OUT}: {n} candidates, {int(has_hit.sum())} rescued, {len(cig)} CIGAR words")


if __name__ == "__main__":
    main()
