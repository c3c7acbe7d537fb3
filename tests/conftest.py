import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "ksw2_golden.npz")
EXT_FIELDS = ["score", "max", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "zdropped", "reach_end", "n_cigar"]
LL_FIELDS = ["score", "te", "qe", "score2", "te2"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def built():
    """Build the CUDA library, the synth helper and the oracle (once per session)."""
    from minibwa_gb300 import build as B
    from oracle import oracle as O
    B.build()
    O.build(ref=True)
    return True


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


def golden_ext_cases(g):
    P = g["ext_params"]
    for i in range(len(P)):
        dual, m, q, e, q2, e2, w, zdrop, eb, flag, ql, tl = [int(x) for x in P[i]]
        yield dict(dual=dual, m=m, mat=g["ext_mat"][i][:m * m].copy(), q=q, e=e, q2=q2, e2=e2, w=w, zdrop=zdrop,
                   end_bonus=eb, flag=flag, query=g["ext_q"][g["ext_qoff"][i]:g["ext_qoff"][i + 1]],
                   target=g["ext_t"][g["ext_toff"][i]:g["ext_toff"][i + 1]],
                   out=dict(zip(EXT_FIELDS, [int(x) for x in g["ext_out"][i]])),
                   cigar=[int(x) for x in g["ext_cigar"][g["ext_cigoff"][i]:g["ext_cigoff"][i + 1]]])


def golden_ll_cases(g):
    P = g["ll_params"]
    for i in range(len(P)):
        size, m, gapo, gape, xtra, ql, tl = [int(x) for x in P[i]]
        yield dict(size=size, m=m, mat=g["ll_mat"][i].copy(), gapo=gapo, gape=gape, xtra=xtra,
                   query=g["ll_q"][g["ll_qoff"][i]:g["ll_qoff"][i + 1]],
                   target=g["ll_t"][g["ll_toff"][i]:g["ll_toff"][i + 1]],
                   out=dict(zip(LL_FIELDS, [int(x) for x in g["ll_out"][i]])))


def expected_m_cigar(m0, n):
    """m_cigar after ksw_push_cigar growth (doubling from 4) starting from m0."""
    m = m0
    while m < n:
        m = m * 2 if m else 4
    return m


def compare_ext(gres, gcig, ores, ocig, idx=None):
    """Assert GPU batch results equal oracle/reference batch results, CIGARs included."""
    n = len(gres)
    for f in EXT_FIELDS:
        a, b = gres[f], ores[f]
        bad = np.nonzero(a != b)[0]
        assert len(bad) == 0, f"field {f}: {len(bad)} of {n} differ, first job {bad[0]}: gpu {a[bad[0]]} vs {b[bad[0]]}"
    for i in range(n):
        k = int(gres["n_cigar"][i])
        if k:
            ga = gcig[gres["cigar_off"][i]:gres["cigar_off"][i] + k]
            ob = ocig[ores["cigar_off"][i]:ores["cigar_off"][i] + k]
            assert np.array_equal(ga, ob), f"CIGAR of job {i} differs: {ga.tolist()} vs {ob.tolist()}"


def compare_ll(gres, ores):
    for f in LL_FIELDS:
        bad = np.nonzero(gres[f] != ores[f])[0]
        assert len(bad) == 0, f"ll field {f}: {len(bad)} differ, first {bad[0]}: gpu {gres[f][bad[0]]} vs {ores[f][bad[0]]}"


TRACE = os.path.join(ROOT, "tests", "golden", "minibwa_trace.npz")
TRACE_OUT = ["max", "zdropped", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "score", "m_cigar", "n_cigar",
             "reach_end"]


@pytest.fixture(scope="session")
def trace():
    return dict(np.load(TRACE))


def trace_ext_calls(g):
    """The extension calls the reference's minibwa issued (tests/golden/make_trace.py)."""
    for i in range(len(g["ext_kind"])):
        qlen, tlen, m, q, e, q2, e2, w, zdrop, eb, flag, m0 = [int(x) for x in g["ext_hdr"][i]]
        yield dict(dual=int(g["ext_kind"][i]) == 2, m=m, q=q, e=e, q2=q2, e2=e2, w=w, zdrop=zdrop, end_bonus=eb,
                   flag=flag, m_cigar_in=m0,
                   mat=g["ext_mat"][g["ext_matoff"][i]:g["ext_matoff"][i + 1]].view(np.int8).copy(),
                   query=g["ext_q"][g["ext_qoff"][i]:g["ext_qoff"][i + 1]],
                   target=g["ext_t"][g["ext_toff"][i]:g["ext_toff"][i + 1]],
                   out=dict(zip(TRACE_OUT, [int(x) for x in g["ext_out"][i]])),
                   cigar=[int(x) for x in g["ext_cigar"][g["ext_cigoff"][i]:g["ext_cigoff"][i + 1]]])


def trace_ll_calls(g):
    for i in range(len(g["ll_kind"])):
        size, qlen, m, tlen, gapo, gape, xtra = [int(x) for x in g["ll_hdr"][i]]
        yield dict(kind=int(g["ll_kind"][i]), size=size, m=m, gapo=gapo, gape=gape, xtra=xtra,
                   mat=g["ll_mat"][g["ll_matoff"][i]:g["ll_matoff"][i + 1]].view(np.int8).copy(),
                   query=g["ll_q"][g["ll_qoff"][i]:g["ll_qoff"][i + 1]],
                   target=g["ll_t"][g["ll_toff"][i]:g["ll_toff"][i + 1]],
                   out=dict(zip(LL_FIELDS, [int(x) for x in g["ll_out"][i]])))
