"""Generate tests/golden/minibwa_trace.npz: the ksw2 calls the reference's own minibwa issues.

Run where the reference tree is available:

    python tests/golden/make_trace.py

It builds oracle/_ref/minibwa_trace (the reference's minibwa compiled from its sources, its
ksw2 entry points recorded by oracle/trace_shim.c), indexes the reference's test genome
(test/chrM-human.fa.gz, also with --meth), and maps:
  1. the reference's own test read pairs (test/chrM-read_{1,2}.fa.gz);
  2. seeded simulated pairs from chrM (3% substitutions, 0.6% indels, 10% of pairs with one
     mate at 12% substitutions so that mate rescue runs, 5% with a random tail for z-drop);
  3. the same pairs with other scoring (-A1 -B4 -O6 -E1) and with a narrow band (-w 30);
  4. seeded simulated long reads (1-6 kb, 5% substitutions, 2% indels, -x lr);
  5. seeded directional bisulfite pairs mapped with --meth.
Every call's inputs and outputs (the ksw_extz_t fields, m_cigar and the CIGAR; the ksw_llrst_t
fields) are stored.  Only simulated reads and the reference's own test files are used.
"""
import gzip
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "minibwa_trace.npz")
EXE = os.path.join(ROOT, "oracle", "_ref", "minibwa_trace")
COMP = np.array([3, 2, 1, 0, 4], np.uint8)
ACGT = np.frombuffer(b"ACGTN", np.uint8)


def read_fasta_gz(fn):
    seq = []
    for line in gzip.open(fn, "rt"):
        if not line.startswith(">"):
            seq.append(line.strip())
    s = "".join(seq).upper().encode()
    lut = np.full(256, 4, np.uint8)
    for i, c in enumerate(b"ACGT"):
        lut[c] = i
    return lut[np.frombuffer(s, np.uint8)]


def mutate(rng, s, sub, indel):
    s = s.copy()
    m = rng.random(len(s)) < sub
    s[m] = (s[m] + rng.integers(1, 4, int(m.sum()))) % 4
    out, i = [], 0
    while i < len(s):
        u = rng.random()
        if u < indel / 2:
            i += int(rng.integers(1, 4))
            continue
        if u < indel:
            out.extend(rng.integers(0, 4, int(rng.integers(1, 4))).tolist())
        out.append(int(s[i]))
        i += 1
    return np.array(out, np.uint8)


def revcomp(s):
    return COMP[s[::-1]]


def write_fa(fn, reads):
    with open(fn, "w") as f:
        for name, s in reads:
            f.write(f">{name}\n{ACGT[s].tobytes().decode()}\n")


def sim_pairs(rng, g, n, rl=150, ins=(250, 450), p_bad=0.1, p_junk=0.05, meth=False):
    r1, r2 = [], []
    for k in range(n):
        L = int(rng.integers(*ins))
        st = int(rng.integers(0, len(g) - L))
        f = g[st:st + L].copy()
        if rng.random() < 0.5:
            f = revcomp(f)
        if meth:  # bisulfite on the sequenced strand: unmethylated C reads as T
            c = (f == 1) & (rng.random(len(f)) < 0.95)
            f[c] = 3
        a = mutate(rng, f[:rl], 0.03, 0.006)
        b = mutate(rng, revcomp(f[-rl:]), 0.03, 0.006)
        if rng.random() < p_bad:
            if rng.random() < 0.5:
                a = mutate(rng, f[:rl], 0.12, 0.01)
            else:
                b = mutate(rng, revcomp(f[-rl:]), 0.12, 0.01)
        if rng.random() < p_junk:
            a = np.concatenate([a[:rl - 40], rng.integers(0, 4, 40).astype(np.uint8)])
        r1.append((f"p{k}/1", a)), r2.append((f"p{k}/2", b))
    return r1, r2


def sim_long(rng, g, n):
    out = []
    for k in range(n):
        L = int(rng.integers(1000, 6000))
        st = int(rng.integers(0, len(g) - L))
        s = g[st:st + L]
        if rng.random() < 0.5:
            s = revcomp(s)
        out.append((f"l{k}", mutate(rng, s, 0.05, 0.02)))
    return out


def run(args, trace, cwd):
    env = dict(os.environ, KSW2_TRACE=trace)
    subprocess.run([EXE] + args, cwd=cwd, env=env, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def parse(fn):
    b = open(fn, "rb").read()
    a = np.frombuffer(b, np.uint8)
    p = 0

    def i32(n):
        nonlocal p
        v = np.frombuffer(b, "<i4", n, p)
        p += 4 * n
        return [int(x) for x in v]

    def by(n):
        nonlocal p
        v = a[p:p + n].copy()
        p += (n + 3) & ~3
        return v

    ext, ll = [], []
    while p < len(b):
        kind = i32(1)[0]
        if kind in (1, 2):
            hdr = i32(12)
            qlen, tlen, m = hdr[0], hdr[1], hdr[2]
            mat, q, t = by(m * m), by(qlen), by(tlen)
            o = i32(12)
            cig = i32(o[10]) if o[10] > 0 else []
            ext.append((kind, hdr, mat, q, t, o, cig))
        else:
            hdr = i32(7)
            size, qlen, m, tlen = hdr[0], hdr[1], hdr[2], hdr[3]
            mat, q, t = by(m * m), by(qlen), by(tlen)
            ll.append((kind, hdr, mat, q, t, i32(5)))
    return ext, ll


def main():
    tree = O.ref_tree()
    if tree is None:
        raise SystemExit("the reference tree is needed to record the trace (set KSW2_REF_TREE)")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "trace", f"REF={tree}"])
    rng = np.random.default_rng(20241203)
    g = read_fasta_gz(os.path.join(tree, "test", "chrM-human.fa.gz"))
    with tempfile.TemporaryDirectory() as d:
        tr = os.path.join(d, "trace.bin")
        fa = os.path.join(tree, "test", "chrM-human.fa.gz")
        run(["index", fa, "chrM"], os.devnull, d)
        run(["index", "--meth", fa, "chrMm"], os.devnull, d)
        t1, t2 = (os.path.join(tree, "test", f"chrM-read_{i}.fa.gz") for i in (1, 2))
        run(["map", "chrM", t1, t2], tr, d)
        a, b = sim_pairs(rng, g, 1500)
        write_fa(os.path.join(d, "s1.fa"), a), write_fa(os.path.join(d, "s2.fa"), b)
        run(["map", "chrM", "s1.fa", "s2.fa"], tr, d)
        run(["map", "-A1", "-B4", "-O6", "-E1", "chrM", "s1.fa", "s2.fa"], tr, d)
        run(["map", "-w", "30", "chrM", "s1.fa", "s2.fa"], tr, d)
        write_fa(os.path.join(d, "long.fa"), sim_long(rng, g, 40))
        run(["map", "-x", "lr", "chrM", "long.fa"], tr, d)
        a, b = sim_pairs(rng, g, 600, meth=True)
        write_fa(os.path.join(d, "m1.fa"), a), write_fa(os.path.join(d, "m2.fa"), b)
        run(["map", "--meth", "chrMm", "m1.fa", "m2.fa"], tr, d)
        ext, ll = parse(tr)
    # store: one row of parameters and outputs per call, sequences back to back
    def pack(seqs):
        off = np.zeros(len(seqs) + 1, np.int64)
        off[1:] = np.cumsum([len(s) for s in seqs])
        return (np.concatenate(seqs) if seqs else np.zeros(0, np.uint8)), off
    eq, eqo = pack([e[3] for e in ext])
    et, eto = pack([e[4] for e in ext])
    em, emo = pack([e[2].astype(np.uint8) for e in ext])
    ec, eco = pack([np.array(e[6], np.uint32) for e in ext])
    lq, lqo = pack([x[3] for x in ll])
    lt, lto = pack([x[4] for x in ll])
    lm, lmo = pack([x[2].astype(np.uint8) for x in ll])
    np.savez_compressed(
        OUT,
        ext_kind=np.array([e[0] for e in ext], np.int32), ext_hdr=np.array([e[1] for e in ext], np.int32),
        ext_out=np.array([e[5] for e in ext], np.int32), ext_q=eq, ext_qoff=eqo, ext_t=et, ext_toff=eto,
        ext_mat=em, ext_matoff=emo, ext_cigar=ec, ext_cigoff=eco,
        ll_kind=np.array([x[0] for x in ll], np.int32), ll_hdr=np.array([x[1] for x in ll], np.int32).reshape(-1, 7),
        ll_out=np.array([x[5] for x in ll], np.int32).reshape(-1, 5), ll_q=lq, ll_qoff=lqo, ll_t=lt, ll_toff=lto,
        ll_mat=lm, ll_matoff=lmo)
    flags = sorted(set(int(e[1][10]) for e in ext))
    print(f"{OUT}: {len(ext)} extension calls (extz2 {sum(e[0] == 1 for e in ext)}, extd2 "
          f"{sum(e[0] == 2 for e in ext)}; flags {[hex(f) for f in flags]}; max qlen "
          f"{max(e[1][0] for e in ext)}), {len(ll)} ksw_ll calls (kinds {sorted(set(x[0] for x in ll))})")


if __name__ == "__main__":
    main()
