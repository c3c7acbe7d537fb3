"""The batched minibwa: the reference's mapper with the alignment of every hit of a mini-batch
handed to the GPU at once (minibwa_gb300/mapper) maps the same reads as the stock build,
byte for byte.

Stock minibwa is the reference compiled from its own sources (oracle/Makefile); the batched
build is the same sources with three lines of map-main.c and one of pe.c substituted (each
read's alignment deferred, the mini-batch's hits and mate-rescue windows aligned on the GPU),
and libksw2gpu.so in place of the three ksw2 objects.  Read sets: the
reference's own test pairs on chrM; 100,000 simulated pairs on a 4 Mb simulated genome with
repeats (noisy mates for rescue, junk tails, chimeras); simulated long reads with inversions,
junk blocks and chimeras (-x lr: z-drop splits, the inversion check, the long-read seed
filters); bisulfite pairs (--meth).  The reference tree comes from its staged copy; without
it the tests skip."""
import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mp(built, tmp_path_factory):
    from oracle import oracle as O
    from minibwa_gb300 import mapper, synth
    tree = O.ref_tree()
    if tree is None:
        pytest.skip("no reference tree staged (make -C oracle stage REF=...)")
    stock = O.build_minibwa(os.path.join(ROOT, "minibwa_gb300"))
    batch = mapper.build(tree)
    d = str(tmp_path_factory.mktemp("mapper"))
    fa = os.path.join(tree, "test", "chrM-human.fa.gz")
    mapper.index(stock["stock"], fa, "chrM", d)
    mapper.index(stock["stock"], fa, "chrMm", d, meth=True)
    g = synth.mapper_genome()
    synth.write_fasta(os.path.join(d, "g.fa"), g)
    mapper.index(stock["stock"], "g.fa", "g", d)
    a, b = synth.mapper_pairs(g, 100_000)
    synth.write_fasta(os.path.join(d, "p1.fa"), a), synth.write_fasta(os.path.join(d, "p2.fa"), b)
    synth.write_fasta(os.path.join(d, "long.fa"), synth.mapper_long_reads(g, 1500))
    return dict(stock=stock, batch=batch, dir=d, tree=tree)


def _same(mp, args, min_records, pairs=(("stock", "batch"),), threads=8):
    from minibwa_gb300 import mapper
    times = {}
    for s, b in pairs:
        sa, ts = mapper.map_reads(mp["stock"][s], args, mp["dir"], threads)
        sb, tb = mapper.map_reads(mp["batch"][b], args, mp["dir"], threads)
        n = sum(1 for ln in sa.splitlines() if not ln.startswith(b"@"))
        assert n >= min_records, (args, n)
        if sa != sb:
            la, lb = sa.splitlines(), sb.splitlines()
            bad = [i for i, (x, y) in enumerate(zip(la, lb)) if x != y]
            first = bad[0] if bad else min(len(la), len(lb))
            raise AssertionError(f"minibwa_{b} SAM differs from minibwa_{s} for {args}: {len(bad)} lines "
                                 f"({len(la)} vs {len(lb)}), first at {first}:\n"
                                 f"{la[first] if first < len(la) else b''!r}\n{lb[first] if first < len(lb) else b''!r}")
        times[(s, b)] = (ts, tb)
    return n, times


def test_reference_test_pairs(mp):
    t1, t2 = (os.path.join(mp["tree"], "test", f"chrM-read_{i}.fa.gz") for i in (1, 2))
    n, _ = _same(mp, ["chrM", t1, t2], 2013, pairs=(("stock", "batch"), ("stock_km", "batch_km")))
    assert n == 2013


def test_simulated_pairs_100k(mp):
    n, t = _same(mp, ["g", "p1.fa", "p2.fa"], 200_000, threads=16)
    ts, tb = t[("stock", "batch")]
    print(f"\n100k pairs, 16 threads: stock {ts:.2f} s, batched {tb:.2f} s")


def test_simulated_pairs_single_end(mp):
    _same(mp, ["g", "p1.fa"], 100_000, threads=16)


@pytest.mark.parametrize("opts", [["-A1", "-B4", "-O6", "-E1"], ["-w", "30"]], ids=["scoring", "w30"])
def test_simulated_pairs_options(mp, opts):
    from minibwa_gb300 import synth
    p = os.path.join(mp["dir"], "s1.fa")
    if not os.path.exists(p):
        g = synth.mapper_genome()
        a, b = synth.mapper_pairs(g, 10_000, seed=91)
        synth.write_fasta(p, a), synth.write_fasta(os.path.join(mp["dir"], "s2.fa"), b)
    _same(mp, opts + ["g", "s1.fa", "s2.fa"], 20_000)


def test_simulated_long_reads(mp):
    n, t = _same(mp, ["-x", "lr", "g", "long.fa"], 1500, pairs=(("stock", "batch"), ("stock_km", "batch_km")),
                 threads=16)
    ts, tb = t[("stock", "batch")]
    print(f"\n1,500 long reads, 16 threads: stock {ts:.2f} s, batched {tb:.2f} s")


def test_bisulfite_pairs(mp):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_trace import read_fasta_gz, sim_pairs, write_fa
    m1 = os.path.join(mp["dir"], "m1.fa")
    if not os.path.exists(m1):
        g = read_fasta_gz(os.path.join(mp["tree"], "test", "chrM-human.fa.gz"))
        a, b = sim_pairs(np.random.default_rng(20261205), g, 800, meth=True)
        write_fa(m1, a), write_fa(os.path.join(mp["dir"], "m2.fa"), b)
    _same(mp, ["--meth", "chrMm", "m1.fa", "m2.fa"], 1600)


def test_missing_device_fails_loudly(mp):
    """A GPU the batched mapper cannot open ends the run with an error and no SAM records,
    rather than aligning anywhere else (no CPU fallback)."""
    import subprocess
    t1 = os.path.join(mp["tree"], "test", "chrM-read_1.fa.gz")
    env = dict(os.environ, MBG_DEVICE="63")
    out = subprocess.run([mp["batch"]["batch"], "map", "-t", "4", "chrM", t1], cwd=mp["dir"], capture_output=True,
                         env=env)
    assert out.returncode != 0
    assert b"ksw2g_ctx_create" in out.stderr
    assert not any(ln and not ln.startswith(b"@") for ln in out.stdout.splitlines())


@pytest.mark.parametrize("split", ["0", "1"])
def test_long_reads_either_kernel_choice(mp, split):
    """The extension kernels a batch picks (KSW2G_SPLIT: 0 thread groups and the block-wide kernel
    only, 1 the block-split kernel for every band it holds) do not change the SAM."""
    from minibwa_gb300 import mapper
    args = ["-x", "lr", "g", "long.fa"]
    sa, _ = mapper.map_reads(mp["stock"]["stock"], args, mp["dir"], 16)
    sb, _ = mapper.map_reads(mp["batch"]["batch"], args, mp["dir"], 16, env=dict(os.environ, KSW2G_SPLIT=split))
    assert sa == sb
