"""Generate tests/golden/chains_golden.npz from the reference's own mb_align1.

Run where the reference tree is available (it builds oracle/_ref/libmbpe.so, the
reference's align.c with its mb_update_extra call left out, behind oracle/ref_align.c):

    python tests/golden/make_golden_chains.py

The fixture holds a seeded 2-bit reference (two contigs, N runs), hits of simulated reads
over it (synth.ChainCases: every event kind, both strands, bisulfite modes, split_inv set on
some) in four option sets -- minibwa's short-read preset, the same with methylation, the
long-read preset, and long reads under the short-read preset's adaptive switch -- and, for
every hit, what mb_align1 leaves in it: ts, te, qs, qe, dp_score, the CIGAR, cnt and score
after a z-drop split, and the split-off hit's cnt, first anchor, split_inv and score.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from minibwa_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "chains_golden.npz")
SETS = [("sr", dict(n=400, seed=201), synth.CHAIN_OPT_SR),
        ("sr_meth", dict(n=120, seed=202, meth=True), dict(synth.CHAIN_OPT_SR, meth=1)),
        ("lr", dict(n=64, seed=203, long_reads=True), synth.CHAIN_OPT_LR),
        ("adaptive", dict(n=32, seed=204, long_reads=True), synth.CHAIN_OPT_SR)]


def main():
    O.build(ref=True)
    if not O.have_ref_pe():
        raise SystemExit("the reference tree is needed to generate the chain fixture")
    ref = synth.Reference2b([200000, 150000], n_runs=10, seed=200)
    opts, set_lo = [], []
    anchors, chains, qparts, outs, cig, cig_off = [], [], [], [], [], [0]
    qoff = 0
    for name, kw, opt in SETS:
        kw = dict(kw)
        cs = synth.ChainCases(ref, kw.pop("n"), **kw)
        opts.append([int(opt[k]) for k in O.CHAIN_OPT])
        set_lo.append(len(chains))
        a_base = sum(len(a) for a in anchors)
        for i in range(len(cs)):
            c = cs.chains[i].copy()
            d = O.ref_align1(ref, opt, cs.anchors, c, cs.fwd[i], cs.rc[i])
            if d["r2_cnt"]:
                d["r2_as"] += a_base  # into the concatenated anchor array
            outs.append([d[k] for k in O.ALIGN1_OUT])
            cig.extend(d["cigar"])
            cig_off.append(len(cig))
            c["as"] += a_base
            c["qoff"] = qoff + int(c["qoff"])
            chains.append(c)
        anchors.append(cs.anchors)
        qparts.append(cs.qbuf)
        qoff += len(cs.qbuf)
    set_lo.append(len(chains))
    np.savez_compressed(
        OUT, pac=ref.pac, ctg_off=ref.ctg_off, ctg_len=ref.ctg_len, ambi=np.asarray(ref.ambi, np.uint64).reshape(-1, 2),
        anchors=np.concatenate(anchors), chains=np.array(chains), qbuf=np.concatenate(qparts),
        opts=np.array(opts, np.int64), set_lo=np.array(set_lo, np.int64), set_names=np.array([s[0] for s in SETS]),
        out=np.array(outs, np.int64), cigar=np.array(cig, np.uint32), cigar_off=np.array(cig_off, np.int64))
    print(OUT, len(chains), "hits", len(cig), "CIGAR words", os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
