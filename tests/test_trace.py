"""The ksw2 calls of real minibwa runs (the reference's own minibwa mapping its test reads and
seeded simulated reads, recorded by oracle/trace_shim.c into tests/golden/minibwa_trace.npz):
the oracle reproduces every one of them, CIGAR and m_cigar included."""
import pytest

from conftest import LL_FIELDS, TRACE_OUT, expected_m_cigar, trace_ext_calls, trace_ll_calls
from oracle import oracle as O


@pytest.fixture(scope="module")
def orc(built):
    return O.oracle_lib()


def test_trace_covers_the_callers(trace):
    calls = list(trace_ext_calls(trace))
    flags = {c["flag"] for c in calls}
    assert len(calls) > 5000 and {0x40, 0xc2, 0x08}.issubset(flags)   # align.c:645,690,693,735 and pe.c:282
    assert any(c["flag"] & 0x04 for c in calls)                          # --meth: GENERIC_SC
    assert any(not c["dual"] for c in calls) and any(c["dual"] for c in calls)
    assert len(list(trace_ll_calls(trace))) > 100                        # pe.c rescue
    for c in calls:
        assert c["out"]["m_cigar"] == expected_m_cigar(c["m_cigar_in"], c["out"]["n_cigar"])


def test_oracle_matches_traced_extension_calls(orc, trace):
    for n, c in enumerate(trace_ext_calls(trace)):
        got, _ = O.extz(int(c["dual"]), c["query"], c["target"], c["m"], c["mat"], c["q"], c["e"], c["q2"], c["e2"],
                        c["w"], c["zdrop"], c["end_bonus"], c["flag"])
        for f in TRACE_OUT:
            if f != "m_cigar":
                assert got[f] == c["out"][f], (n, f, got[f], c["out"][f])
        assert got["cigar"] == c["cigar"], n


def test_oracle_matches_traced_ll_calls(orc, trace):
    for n, c in enumerate(trace_ll_calls(trace)):
        got, _ = O.ll(c["size"], c["query"], c["target"], c["m"], c["mat"], c["gapo"], c["gape"], c["xtra"])
        for f in LL_FIELDS:
            assert got[f] == c["out"][f], (n, f, got[f], c["out"][f])
