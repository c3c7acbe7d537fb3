"""align.c's mb_align_pair over a batch on the device (ksw2g_align_pairs): every pair of the golden
fixture, recorded from the reference's own mb_align_pair, grouped by scoring scheme into one call
each -- shortcuts settled on the host, the rest as one DP batch -- gives the reference's ksw_extz_t
fields and CIGAR."""
import numpy as np
import pytest

from test_align_pairs import align_cases

pytestmark = pytest.mark.gpu

FIELDS = ("max", "zdropped", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "score", "n_cigar", "reach_end")


def test_align_pairs_golden(built):
    from minibwa_gb300 import Context
    from minibwa_gb300.lib import EXT_JOB
    cases = list(align_cases())
    groups = {}
    for i, c in enumerate(cases):
        groups.setdefault(c["si"], []).append(i)
    ctx = Context(0)
    try:
        for si, idx in groups.items():
            sc = cases[idx[0]]["scoring"]
            opt = {k: sc[k] for k in ("a", "b", "b_ts", "b_ambi", "q", "e", "q2", "e2", "meth", "max_sw_mat")}
            jobs = np.zeros(len(idx), EXT_JOB)
            qs = [cases[i]["query"] for i in idx]
            ts = [cases[i]["target"] for i in idx]
            jobs["qlen"], jobs["tlen"] = [len(x) for x in qs], [len(x) for x in ts]
            jobs["qoff"] = np.concatenate([[0], np.cumsum(jobs["qlen"])[:-1]])
            jobs["toff"] = np.concatenate([[0], np.cumsum(jobs["tlen"])[:-1]])
            jobs["w"] = [cases[i]["w"] for i in idx]
            jobs["zdrop"] = [cases[i]["zdrop"] for i in idx]
            jobs["end_bonus"] = [cases[i]["end_bonus"] for i in idx]
            jobs["flag"] = [cases[i]["flag"] for i in idx]
            res, cig = ctx.align_pairs(opt, cases[idx[0]]["mat"], jobs, np.concatenate(qs), np.concatenate(ts))
            for j, i in enumerate(idx):
                got = {f: int(res[f][j]) for f in FIELDS}
                k = int(res["n_cigar"][j])
                got["cigar"] = cig[res["cigar_off"][j]:res["cigar_off"][j] + k].tolist() if k else []
                assert got == cases[i]["out"], (si, i, got, cases[i]["out"])
    finally:
        ctx.close()
