"""Generate tests/golden/ksw2_golden.npz from the reference's own ksw2 SSE code.

Run where the reference tree is available (it builds oracle/_ref/libksw2ref.so from the
reference sources first):

    python tests/golden/make_golden.py

Cases are seeded random draws over the parameter space the reference accepts (both
extension kernels, every flag combination used by minibwa plus the rest, band widths
from 0 to unbounded, small alphabets, N-rich sequences, ksw_ll u8/i16 with and without
KSW_LL_SUBO / KSW_LL_STOP), plus the benchmark-shaped pairs.  The fixture stores the
inputs and every output field, including the CIGAR.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

N_EXT, N_LL = 600, 300
FLAGS = [0x40, 0xc2, 0x08, 0x00, 0x41, 0x42, 0x02, 0x80, 0x01, 0x04, 0x44, 0x18, 0x58, 0x48, 0xc0, 0x46, 0x10,
         0x0a, 0x82, 0x5a]


def gen_nt4(a, b, b_ts, b_ambi, mt=0):
    m = 5
    mat = np.zeros(25, np.int8)
    a, b, b_ambi = abs(a), -abs(b), -abs(b_ambi)
    for i in range(4):
        for j in range(4):
            mat[i * m + j] = a if i == j else b
        mat[i * m + 4] = b_ambi
    mat[20:25] = b_ambi
    if b_ts and -abs(b_ts) != b:
        mat[2] = mat[8] = mat[10] = mat[16] = -abs(b_ts)
    if mt == 1:
        mat[8] = a
    elif mt == 2:
        mat[10] = a
    return mat


def mutate(rng, q, m, sub, ind):
    out = []
    i = 0
    while i < len(q):
        u = rng.random()
        if u < ind / 2:
            i += int(rng.integers(1, 5))
            continue
        if u < ind:
            out.extend(rng.integers(0, m - 1, int(rng.integers(1, 6))).tolist())
        c = int(q[i]) if q[i] < m - 1 else int(rng.integers(0, m - 1))
        if rng.random() < sub:
            c = int(rng.integers(0, m))
        out.append(c)
        i += 1
    return np.array(out if out else [0], np.uint8)


def rand_pair(rng, m, maxlen):
    ql = int(rng.integers(1, maxlen + 1))
    pn = rng.random() * 0.05 if rng.random() < 0.3 else 0.0
    q = np.where(rng.random(ql) < pn, m - 1, rng.integers(0, m - 1, ql)).astype(np.uint8)
    mode = int(rng.integers(0, 4))
    if mode == 0:
        tl = int(rng.integers(1, maxlen + 1))
        t = rng.integers(0, m - 1, tl).astype(np.uint8)
    else:
        t = mutate(rng, q, m, rng.random() * 0.15, rng.random() * 0.08)
        if mode >= 2:
            t = np.concatenate([t, rng.integers(0, m - 1, int(rng.integers(0, 41))).astype(np.uint8)])
    return q, t


def main():
    O.build(ref=True)
    if not O.have_ref():
        raise SystemExit("reference tree not available")
    rng = np.random.default_rng(20261203)
    P, MAT, QS, TS, OUT, CIG = [], [], [], [], [], []
    for it in range(N_EXT):
        m = 5 if rng.random() < 0.9 else int(rng.integers(2, 9))
        maxlen = int(rng.integers(1, 41)) if rng.random() < 0.6 else int(rng.integers(41, 400))
        q, t = rand_pair(rng, m, maxlen)
        a, b = int(rng.integers(1, 7)), int(rng.integers(1, 13))
        if m == 5:
            mat = gen_nt4(a, b, int(rng.integers(1, 13)) if rng.random() < 0.2 else 0, int(rng.integers(0, 4)),
                          int(rng.integers(1, 3)) if rng.random() < 0.1 else 0)
        else:
            mat = np.array([a if i // m == i % m else -b for i in range(m * m)], np.int8)
        if rng.random() < 0.05:
            mat[m * m - 1] = 0
        dual = int(rng.random() < 0.5)
        qo, eo = int(rng.integers(0, 31)), int(rng.integers(1, 7))
        q2, e2 = int(rng.integers(0, 51)), int(rng.integers(1, 7))
        w = -1 if rng.random() < 0.15 else int(rng.integers(0, 201))
        zdrop = -1 if rng.random() < 0.2 else int(rng.integers(0, 301))
        eb = -1 if rng.random() < 0.3 else int(rng.integers(0, 31))
        flag = FLAGS[it % len(FLAGS)] if rng.random() < 0.7 else int(rng.integers(0, 256)) & 0xdf
        if not dual:
            q2, e2 = qo, eo
        job = np.zeros(1, O.ORC_JOB)
        job["qlen"], job["tlen"], job["toff"] = len(q), len(t), 0
        job["w"], job["zdrop"], job["end_bonus"], job["flag"] = w, zdrop, eb, flag
        res, cig = O.ext_batch("ref", dual, m, mat, qo, eo, q2, e2, job, q, t)
        r = res[0]
        P.append([dual, m, qo, eo, q2, e2, w, zdrop, eb, flag, len(q), len(t)])
        mp = np.zeros(64, np.int8)
        mp[:m * m] = mat
        MAT.append(mp)
        QS.append(q)
        TS.append(t)
        OUT.append([r["score"], r["max"], r["max_q"], r["max_t"], r["mqe"], r["mqe_t"], r["mte"], r["mte_q"],
                    r["zdropped"], r["reach_end"], r["n_cigar"]])
        CIG.append(cig[r["cigar_off"]:r["cigar_off"] + r["n_cigar"]].copy())
    LP, LQ, LT, LO, LMAT = [], [], [], [], []
    for it in range(N_LL):
        m = 5
        maxlen = int(rng.integers(1, 60)) if rng.random() < 0.5 else int(rng.integers(60, 500))
        q, t = rand_pair(rng, m, maxlen)
        if rng.random() < 0.5:  # embed the query in a longer window
            pad = rng.integers(0, 4, int(rng.integers(0, 300))).astype(np.uint8)
            t = np.concatenate([pad, t, rng.integers(0, 4, int(rng.integers(0, 300))).astype(np.uint8)])
        size = 1 if rng.random() < 0.5 else 2
        a, b = int(rng.integers(1, 5)), int(rng.integers(1, 11))
        mat = gen_nt4(a, b, 0, int(rng.integers(0, 4)))
        gapo, gape = int(rng.integers(0, 13)), int(rng.integers(1, 5))
        xtra = 0
        if rng.random() < 0.5:
            xtra |= 0x40000 | int(rng.integers(0, 41))
        if rng.random() < 0.2:
            xtra |= 0x20000 | int(rng.integers(1, 201))
        job = np.zeros(1, dtype=[("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"),
                                 ("xtra", "<i4"), ("pad", "<i4")])
        job["qlen"], job["tlen"], job["xtra"] = len(q), len(t), xtra
        r = O.ll_batch("ref", size, m, mat, gapo, gape, job, q, t)[0]
        LP.append([size, m, gapo, gape, xtra, len(q), len(t)])
        LMAT.append(mat)
        LQ.append(q)
        LT.append(t)
        LO.append([r["score"], r["te"], r["qe"], r["score2"], r["te2"]])

    def cat(xs):
        off = np.concatenate([[0], np.cumsum([len(x) for x in xs])]).astype(np.int64)
        return np.concatenate(xs).astype(xs[0].dtype), off

    qs, qo_ = cat(QS)
    ts, to_ = cat(TS)
    cg, co_ = cat([c.astype(np.uint32) if len(c) else np.zeros(0, np.uint32) for c in CIG])
    lq, lqo = cat(LQ)
    lt, lto = cat(LT)
    out = os.path.join(HERE, "ksw2_golden.npz")
    np.savez_compressed(out, ext_params=np.array(P, np.int32), ext_mat=np.array(MAT, np.int8), ext_q=qs,
                        ext_qoff=qo_, ext_t=ts, ext_toff=to_, ext_out=np.array(OUT, np.int64), ext_cigar=cg,
                        ext_cigoff=co_, ll_params=np.array(LP, np.int32), ll_mat=np.array(LMAT, np.int8), ll_q=lq,
                        ll_qoff=lqo, ll_t=lt, ll_toff=lto, ll_out=np.array(LO, np.int32))
    print("wrote", out, os.path.getsize(out), "bytes;", N_EXT, "extension and", N_LL, "ll cases")


if __name__ == "__main__":
    main()
