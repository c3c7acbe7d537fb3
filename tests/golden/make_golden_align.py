"""Generate tests/golden/align_golden.npz from the reference's own mb_align_pair (align.c:329-390).

Run where the reference tree is available (it builds oracle/_ref/libmbpe.so first):

    python tests/golden/make_golden_align.py

Pairs: the extension and gap-fill windows of the recorded minibwa calls
(tests/golden/minibwa_trace.npz), plus seeded pairs made to reach every branch of
mb_align_pair -- ungapped extensions with 0-6 mismatches or N (the reach-end shortcut and its
fall-through), equal-length gap fills (the ungapped-alignment shortcut), short pairs (the band
shrink), empty sequences and pairs over the DP memory cap -- under five scoring schemes:
minibwa's default dual-affine one, a single-affine one (extz2), transition scoring (GENERIC_SC),
methylation (GENERIC_SC with the C/T matrix) and a small memory cap.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from conftest import trace_ext_calls  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "align_golden.npz")
SCORING = [
    dict(a=2, b=8, b_ts=0, b_ambi=1, q=12, e=2, q2=23, e2=1, meth=0, max_sw_mat=100000000, mt=0),
    dict(a=1, b=4, b_ts=0, b_ambi=1, q=6, e=1, q2=6, e2=1, meth=0, max_sw_mat=100000000, mt=0),
    dict(a=2, b=8, b_ts=4, b_ambi=1, q=12, e=2, q2=23, e2=1, meth=0, max_sw_mat=100000000, mt=0),
    dict(a=2, b=8, b_ts=0, b_ambi=1, q=12, e=2, q2=23, e2=1, meth=1, max_sw_mat=100000000, mt=1),
    dict(a=2, b=8, b_ts=0, b_ambi=1, q=12, e=2, q2=23, e2=1, meth=0, max_sw_mat=20000, mt=0),
]
FLAGS_EXT = [0x40, 0x40 | 0x02 | 0x80, 0x40 | 0x08]
FLAGS_FILL = [0x00, 0x08]


def crafted(rng, n):
    out = []
    for k in range(n):
        kind = k % 5
        if kind in (0, 1):  # extension: target = query with a few changes + flank
            ql = int(rng.integers(0, 220)) if rng.random() < 0.95 else 0
            q = rng.integers(0, 4, ql).astype(np.uint8)
            t = q.copy()
            nm = int(rng.integers(0, 7))
            for p in rng.integers(0, max(ql, 1), nm if ql else 0):
                t[p] = (t[p] + 1 + int(rng.integers(0, 3))) % 4 if rng.random() < 0.8 else 4
            t = np.concatenate([t, rng.integers(0, 4, int(rng.integers(0, 40))).astype(np.uint8)])
            out.append((q, t, int(rng.choice([20, 100, 151])), int(rng.choice([-1, 10])), 100,
                        int(rng.choice(FLAGS_EXT))))
        elif kind in (2, 3):  # gap fill of equal lengths
            ql = int(rng.integers(1, 260))
            q = rng.integers(0, 4, ql).astype(np.uint8)
            t = q.copy()
            for p in rng.integers(0, ql, int(rng.integers(0, 9))):
                t[p] = (t[p] + 1) % 4
            if rng.random() < 0.3 and ql > 10:  # one indel, lengths kept equal
                p = int(rng.integers(1, ql - 1))
                t = np.concatenate([t[:p], t[p + 1:], rng.integers(0, 4, 1).astype(np.uint8)])
            out.append((q, t, int(rng.choice([10, 50, 100])), -1, 100, int(rng.choice(FLAGS_FILL))))
        else:  # unequal short fills and large pairs
            ql, tl = int(rng.integers(0, 150)), int(rng.integers(0, 150))
            if rng.random() < 0.2:
                ql, tl = int(rng.integers(150, 400)), int(rng.integers(150, 400))
            q = rng.integers(0, 4, ql).astype(np.uint8)
            t = q[:tl].copy() if tl <= ql else np.concatenate([q, rng.integers(0, 4, tl - ql).astype(np.uint8)])
            t = t.copy()
            if len(t):
                t[rng.random(len(t)) < 0.05] = 1
            out.append((q, t, int(rng.choice([5, 30, 100])), -1, 100, int(rng.choice(FLAGS_FILL + [0x40]))))
    return out


def main():
    O.build(ref=True)
    if not O.have_ref_pe():
        raise SystemExit("the reference tree is needed to generate the fixture")
    rng = np.random.default_rng(77)
    tr = dict(np.load(os.path.join(HERE, "minibwa_trace.npz")))
    calls = list(trace_ext_calls(tr))
    pick = rng.choice(len(calls), 500, replace=False)
    traced = [(calls[i]["query"], calls[i]["target"], calls[i]["w"], calls[i]["end_bonus"], 100,
               calls[i]["flag"] & ~0x04) for i in sorted(pick)]
    pairs = traced + crafted(rng, 1000)
    rows, qs, ts, outs, cigs, cig_off = [], [], [], [], [], [0]
    for i, (q, t, w, eb, zd, fl) in enumerate(pairs):
        si = i % len(SCORING)
        sc = SCORING[si]
        mat = O.gen_nt4_mat(sc["a"], sc["b"], sc["b_ts"], sc["b_ambi"], sc["mt"])
        r = O.ref_align_pair(sc, mat, q, t, w, eb, zd, fl)
        rows.append([si, w, eb, zd, fl])
        qs.append(np.asarray(q, np.uint8)), ts.append(np.asarray(t, np.uint8))
        outs.append([r[k] for k in O.ALIGN_OUT])
        cigs.extend(r["cigar"])
        cig_off.append(len(cigs))
    qoff = np.concatenate([[0], np.cumsum([len(x) for x in qs])])
    toff = np.concatenate([[0], np.cumsum([len(x) for x in ts])])
    sc_arr = np.array([[s[k] for k in O.ALIGN_SC] + [s["max_sw_mat"], s["mt"]] for s in SCORING], np.int64)
    np.savez_compressed(OUT, params=np.array(rows, np.int32), q=np.concatenate(qs), qoff=qoff,
                        t=np.concatenate(ts), toff=toff, out=np.array(outs, np.int32),
                        cigar=np.array(cigs, np.uint32), cigar_off=np.array(cig_off, np.int64), scoring=sc_arr)
    o = np.array(outs)
    print(f"{OUT}: {len(pairs)} pairs; {int((o[:, 9] == 1).sum())} with one CIGAR run, "
          f"{int(o[:, 1].sum())} zdropped")


if __name__ == "__main__":
    main()
