"""The checker itself: the scalar restatement against the reference's golden vectors
and, where the reference tree is present, against the reference's SSE code directly."""
import os
import subprocess

import numpy as np
import pytest

from conftest import EXT_FIELDS, LL_FIELDS, expected_m_cigar, golden_ext_cases, golden_ll_cases
from oracle import oracle as O


@pytest.fixture(scope="module")
def orc(built):
    return O.oracle_lib()


def test_oracle_matches_golden_extension(orc, golden):
    n = 0
    for c in golden_ext_cases(golden):
        got, st = O.extz(c["dual"], c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"],
                         c["w"], c["zdrop"], c["end_bonus"], c["flag"])
        for f in EXT_FIELDS:
            assert got[f] == c["out"][f], (n, f, got[f], c["out"][f])
        assert got["cigar"] == c["cigar"], n
        assert got["m_cigar"] == expected_m_cigar(0, got["n_cigar"])
        n += 1
    assert n == 600


def test_oracle_matches_golden_ll(orc, golden):
    n = 0
    for c in golden_ll_cases(golden):
        got, rows = O.ll(c["size"], c["query"], c["target"], c["m"], c["mat"], c["gapo"], c["gape"], c["xtra"])
        for f in LL_FIELDS:
            assert got[f] == c["out"][f], (n, f, got[f], c["out"][f])
        assert 0 <= rows <= len(c["target"])
        n += 1
    assert n == 300


def test_oracle_degenerate_inputs(orc):
    mat = np.array([2 if i // 5 == i % 5 else -8 for i in range(25)], np.int8)
    for dual in (0, 1):
        got, st = O.extz(dual, np.zeros(0, np.uint8), np.zeros(5, np.uint8), 5, mat, 12, 2, 24, 1, 10, 100, 10, 0x40)
        assert got["score"] == -0x40000000 and got["max"] == 0 and got["n_cigar"] == 0 and st["n_diag"] == 0
        got, st = O.extz(dual, np.zeros(5, np.uint8), np.zeros(0, np.uint8), 5, mat, 12, 2, 24, 1, 10, 100, 10, 0x40)
        assert got["max_q"] == -1 and got["mqe"] == -0x40000000 and st["n_diag"] == 0
    # -min_sc > 2(q+e): the reference returns right after reset
    got, st = O.extz(0, np.zeros(5, np.uint8), np.zeros(5, np.uint8), 5, mat, 1, 1, 1, 1, 10, 100, 10, 0)
    assert st["n_diag"] == 0 and got["n_cigar"] == 0


def test_cell_counter(orc):
    """nominal cells = sum over processed anti-diagonals of en0-st0+1 (band geometry only)."""
    mat = np.array([2 if i // 5 == i % 5 else -8 for i in range(25)], np.int8)
    q = np.zeros(40, np.uint8)
    t = np.zeros(40, np.uint8)
    got, st = O.extz(0, q, t, 5, mat, 12, 2, 12, 2, 5, -1, 0, 0)
    exp = 0
    for r in range(79):
        s0, e0 = max(0, r - 39, (r - 5 + 1) >> 1), min(39, r, (r + 5) >> 1)
        exp += e0 - s0 + 1
    assert st["cells"] == exp and st["n_diag"] == 79


needs_ref = pytest.mark.skipif(O.ref_tree() is None, reason="reference tree not present")


@needs_ref
def test_oracle_equals_reference_on_benchmark_shapes(built):
    from minibwa_gb300 import synth
    for p in (synth.config0(3000), synth.config1(3000), synth.config2_long(40), synth.config2_short(2000)):
        ro, co = O.ext_batch("orc", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 8)
        rr, cr = O.ext_batch("ref", p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, 8)
        assert np.array_equal(ro, rr), p.name
        assert np.array_equal(co, cr), p.name
    for r in (synth.config3(3000), synth.config3_pe(3000)):
        a = O.ll_batch("orc", r.size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf, 8)
        b = O.ll_batch("ref", r.size, 5, r.mat, r.gapo, r.gape, r.jobs, r.qbuf, r.tbuf, 8)
        assert np.array_equal(a, b), r.name


@needs_ref
def test_differential_fuzz_against_reference(built):
    subprocess.check_call(["make", "-s", "-C", O.HERE, "fuzz", f"REF={O.ref_tree()}"])
    out = subprocess.run([os.path.join(O.HERE, "_ref", "fuzz_vs_ref"), "30000", "7"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.startswith("OK")
