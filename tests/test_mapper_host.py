"""The host side of the batched minibwa (minibwa_gb300/mapper), without a GPU: linked against
oracle/chains_stub.c, whose ksw2g_align_chains runs the reference's own mb_align1 on the CPU,
the batched mapper -- each read's alignment deferred, the hits of a mini-batch aligned in
rounds (hits split off at a z-drop in later rounds), the finishing pass with mb_update_extra,
the inversion check and the rest of mb_map_sai -- writes the same SAM as the stock minibwa,
byte for byte.  The device entry point is pinned to mb_align1 by tests/test_gpu_chains.py and
the whole GPU build by tests/test_gpu_mapper.py.  Needs the reference tree (staged copy);
skips without it."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def mp(built, tmp_path_factory):
    from oracle import oracle as O
    from minibwa_gb300 import mapper, synth
    tree = O.ref_tree()
    if tree is None:
        pytest.skip("no reference tree staged (make -C oracle stage REF=...)")
    exe = O.build_mbgstub()
    d = str(tmp_path_factory.mktemp("mapper_host"))
    fa = os.path.join(tree, "test", "chrM-human.fa.gz")
    mapper.index(exe["stock"], fa, "chrM", d)
    mapper.index(exe["stock"], fa, "chrMm", d, meth=True)
    g = synth.mapper_genome(seed=83)
    synth.write_fasta(os.path.join(d, "g.fa"), g)
    mapper.index(exe["stock"], "g.fa", "g", d)
    a, b = synth.mapper_pairs(g, 12_000, seed=84)
    synth.write_fasta(os.path.join(d, "p1.fa"), a), synth.write_fasta(os.path.join(d, "p2.fa"), b)
    synth.write_fasta(os.path.join(d, "long.fa"), synth.mapper_long_reads(g, 250, seed=85))
    return dict(exe=exe, dir=d, tree=tree)


def _same(mp, args, min_records):
    from minibwa_gb300 import mapper
    sa, _ = mapper.map_reads(mp["exe"]["stock"], args, mp["dir"], 4)
    sb, _ = mapper.map_reads(mp["exe"]["batch"], args, mp["dir"], 4)
    n = sum(1 for ln in sa.splitlines() if not ln.startswith(b"@"))
    assert n >= min_records, (args, n)
    if sa != sb:
        la, lb = sa.splitlines(), sb.splitlines()
        bad = [i for i, (x, y) in enumerate(zip(la, lb)) if x != y]
        first = bad[0] if bad else min(len(la), len(lb))
        raise AssertionError(f"batched SAM differs for {args}: {len(bad)} lines, first at {first}:\n"
                             f"{la[first] if first < len(la) else b''!r}\n{lb[first] if first < len(lb) else b''!r}")
    return n


def test_reference_test_pairs(mp):
    t1, t2 = (os.path.join(mp["tree"], "test", f"chrM-read_{i}.fa.gz") for i in (1, 2))
    assert _same(mp, ["chrM", t1, t2], 2013) == 2013


@pytest.mark.parametrize("opts", [[], ["-A1", "-B4", "-O6", "-E1"]], ids=["default", "scoring"])
def test_simulated_pairs(mp, opts):
    _same(mp, opts + ["g", "p1.fa", "p2.fa"], 24_000)


def test_single_end(mp):
    _same(mp, ["g", "p1.fa"], 12_000)


def test_long_reads(mp):
    _same(mp, ["-x", "lr", "g", "long.fa"], 250)


def test_bisulfite_pairs(mp):
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    from make_trace import read_fasta_gz, sim_pairs, write_fa
    g = read_fasta_gz(os.path.join(mp["tree"], "test", "chrM-human.fa.gz"))
    a, b = sim_pairs(np.random.default_rng(20261206), g, 400, meth=True)
    write_fa(os.path.join(mp["dir"], "m1.fa"), a), write_fa(os.path.join(mp["dir"], "m2.fa"), b)
    _same(mp, ["--meth", "chrMm", "m1.fa", "m2.fa"], 800)
