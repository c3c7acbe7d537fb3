"""Latency of long extension pairs: the device time per anti-diagonal of n seeded extd2 pairs
(default one 10 kb pair at w=500) run alone, on thread groups (split 0) and on the block-split
kernel (split 1), with the results of both compared job by job.  Bands wider than every
thread-group shape run on the block-wide kernel with split 0.

    python -m minibwa_gb300.latency [--w 500] [--qlen 10000] [--pairs 1] [--cigar] [--reps 3]

Prints one JSON line per kernel choice.  CUDA events around every DP and backtrack launch
(ksw2g_batch_set_timing) give the device time; the first run of each batch is untimed.
"""
import argparse
import json

import numpy as np

from . import lib, synth

FIELDS = ("score", "max", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "zdropped", "reach_end", "n_cigar")


def run(ctx, p, split, reps):
    prev = lib.set_ext_split(split)
    try:
        b = lib.ExtBatch(ctx, p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    finally:
        lib.set_ext_split(prev)
    try:
        b.run()
        ctx.sync()
        b.set_timing(True)
        for _ in range(reps):
            b.run()
        ctx.sync()
        dp, bt, _, _ = b.kernel_ms()
        res, cig = b.fetch()
    finally:
        b.free()
    return dp / reps, bt / reps, res, cig


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--w", type=int, default=500)
    ap.add_argument("--qlen", type=int, default=10000)
    ap.add_argument("--pairs", type=int, default=1)
    ap.add_argument("--cigar", action="store_true", help="left-aligned CIGAR (default: score only)")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--split", type=int, default=None, choices=[0, 1], help="one kernel choice only")
    a = ap.parse_args(argv)
    spec = dict(qlen_lo=a.qlen, qlen_hi=a.qlen, sub_rate=0.005, indel_rate=0.003, indel_p=0.5, indel_max=5,
                flank=100)
    flag = lib.KSW_EZ_EXTZ_ONLY | (0 if a.cigar else lib.KSW_EZ_SCORE_ONLY)
    p = synth.ext_pairs(a.pairs, spec, a.w, 400, 10, flag=flag, dual=True, seed=77)
    ctx = lib.Context(tb_budget=64 << 30)
    out = {}
    for split in ((0, 1) if a.split is None else (a.split,)):
        dp, bt, res, cig = run(ctx, p, split, a.reps)
        out[split] = (res, cig)
        nd = int(res["n_diag"].max())
        print(json.dumps({"kernel": "block-split" if split else "thread groups", "pairs": a.pairs, "qlen": a.qlen,
                          "w": a.w, "cigar": a.cigar, "dp_ms": round(dp, 3), "backtrack_ms": round(bt, 3),
                          "anti_diagonals": nd, "us_per_anti_diagonal": round(dp * 1e3 / max(nd, 1), 4)}),
              flush=True)
    if len(out) == 2:
        (r0, c0), (r1, c1) = out[0], out[1]
        same = all(np.array_equal(r0[f], r1[f]) for f in FIELDS)
        same = same and all(np.array_equal(c0[o0:o0 + n], c1[o1:o1 + n]) for o0, o1, n in
                            zip(r0["cigar_off"], r1["cigar_off"], r0["n_cigar"]))
        print(json.dumps({"same_results": bool(same)}), flush=True)
        if not same:
            raise SystemExit("the two kernel choices disagree")
    ctx.close()


if __name__ == "__main__":
    main()
