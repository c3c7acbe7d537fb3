"""The drop-in, proven by relinking: the reference's minibwa is compiled from its own sources
twice, once with its three ksw2 objects (stock) and once against libksw2gpu.so in their place
(the link-line change of the reference's Makefile:6-7), and both map the same reads.  The SAM
output must be byte-identical.

This exercises the callers as they are: align.c's mb_align_pair (align.c:374,376) and the
two-pass gap fill, pe.c's mate rescue (pe.c:266-287), the per-thread CUDA streams of
concurrent kt_for workers (map-main.c:179,191, run with -t 8), and both allocator couplings:
the default build, where ksw2 allocates with libc (ksw2.h:117-121), and the HAVE_KALLOC build,
where it allocates from the caller's kalloc pool (the library finds krealloc/kmalloc exported
with -rdynamic).

The reference tree is read from its staged copy (baseline/_ref/src, made by `make -C oracle
stage`); without it the tests skip.  Reads: the reference's own test pairs (2,013 records)
and seeded simulated read sets of tests/golden/make_trace.py (noisy mates for rescue, junk
tails for z-drop, other scoring, a narrow band, long reads, bisulfite pairs)."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


@pytest.fixture(scope="module")
def mb(built, tmp_path_factory):
    from oracle import oracle as O
    tree = O.ref_tree()
    if tree is None:
        pytest.skip("no reference tree staged (make -C oracle stage REF=...)")
    exe = O.build_minibwa(os.path.join(ROOT, "minibwa_gb300"))
    d = tmp_path_factory.mktemp("minibwa")
    fa = os.path.join(tree, "test", "chrM-human.fa.gz")
    for args in (["index", fa, "chrM"], ["index", "--meth", fa, "chrMm"]):
        subprocess.run([exe["stock"]] + args, cwd=d, check=True, capture_output=True)
    return dict(exe=exe, dir=str(d), tree=tree)


def _map(mb, which, args):
    out = subprocess.run([mb["exe"][which], "map", "-t", "8"] + args, cwd=mb["dir"], capture_output=True)
    assert out.returncode == 0, (which, out.stderr.decode(errors="replace")[-2000:])
    return out.stdout


def _same(mb, args, min_records):
    for stock, gpu in (("stock", "gpu"), ("stock_km", "gpu_km")):
        a, b = _map(mb, stock, args), _map(mb, gpu, args)
        n = sum(1 for ln in a.splitlines() if not ln.startswith(b"@"))
        assert n >= min_records, (args, n)
        if a != b:
            la, lb = a.splitlines(), b.splitlines()
            bad = [i for i, (x, y) in enumerate(zip(la, lb)) if x != y]
            first = bad[0] if bad else min(len(la), len(lb))
            raise AssertionError(f"{gpu} SAM differs from {stock} for {args}: {len(bad)} lines, first at {first}:\n"
                                 f"{la[first] if first < len(la) else b''!r}\n{lb[first] if first < len(lb) else b''!r}")
    return n


def test_reference_test_pairs(mb):
    t1, t2 = (os.path.join(mb["tree"], "test", f"chrM-read_{i}.fa.gz") for i in (1, 2))
    assert _same(mb, ["chrM", t1, t2], 2013) == 2013


@pytest.fixture(scope="module")
def sim(mb):
    from make_trace import read_fasta_gz, sim_long, sim_pairs, write_fa
    rng = np.random.default_rng(20261204)
    g = read_fasta_gz(os.path.join(mb["tree"], "test", "chrM-human.fa.gz"))
    d = mb["dir"]
    a, b = sim_pairs(rng, g, 3000)
    write_fa(os.path.join(d, "s1.fa"), a), write_fa(os.path.join(d, "s2.fa"), b)
    write_fa(os.path.join(d, "long.fa"), sim_long(rng, g, 60))
    a, b = sim_pairs(rng, g, 800, meth=True)
    write_fa(os.path.join(d, "m1.fa"), a), write_fa(os.path.join(d, "m2.fa"), b)
    return d


@pytest.mark.parametrize("opts", [[], ["-A1", "-B4", "-O6", "-E1"], ["-w", "30"]], ids=["default", "scoring", "w30"])
def test_simulated_pairs(mb, sim, opts):
    _same(mb, opts + ["chrM", "s1.fa", "s2.fa"], 6000)


def test_simulated_long_reads(mb, sim):
    _same(mb, ["-x", "lr", "chrM", "long.fa"], 60)


def test_simulated_bisulfite_pairs(mb, sim):
    _same(mb, ["--meth", "chrMm", "m1.fa", "m2.fa"], 1600)
