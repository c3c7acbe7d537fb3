"""ksw2g_ext_noalloc: the extension batch for callers that cannot let the library
allocate device memory (a framework whose caching allocator owns the device memory,
or a serving loop that cannot take the synchronisation of cudaMalloc/cudaFree).
The caller owns the sequence arena, results and CIGAR buffer; the library's scratch
is a fixed static device array.  Its results must equal ksw2g_ext_batch's exactly,
on consecutive calls that reuse that array.  Collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _padded(p):
    """Device-arena layout the entry point expects: 16-aligned starts, 32 zero bytes
    before each sequence, zeros after it up to the next 16-byte boundary plus 32."""
    from minibwa_gb300.lib import EXT_JOB

    def slot(n):
        return 32 + ((n + 15) & ~15) + 32

    jobs = np.zeros(len(p), EXT_JOB)
    jobs[:] = p.jobs
    arena = np.zeros(sum(slot(int(a)) + slot(int(b)) for a, b in zip(p.jobs["qlen"], p.jobs["tlen"])) + 64, np.uint8)
    off = 0
    for i in range(len(p)):
        q, t = p.query(i), p.target(i)
        jobs["qoff"][i] = off + 32
        arena[off + 32:off + 32 + len(q)] = q
        off += slot(len(q))
        jobs["toff"][i] = off + 32
        arena[off + 32:off + 32 + len(t)] = t
        off += slot(len(t))
    return jobs, arena


@pytest.fixture(scope="module")
def L(built):
    from minibwa_gb300.lib import load_library
    lib = load_library()
    lib.ksw2g_ext_noalloc.restype = C.c_int
    lib.ksw2g_ext_noalloc.argtypes = [C.c_int, C.c_int8, C.c_void_p, C.c_int8, C.c_int8, C.c_int8, C.c_int8, C.c_int,
                                      C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_int64,
                                      C.c_void_p]
    return lib


def _run_noalloc(L, p):
    import torch
    from minibwa_gb300.lib import EXT_RESULT
    jobs, arena = _padded(p)
    n = len(jobs)
    cap = int((p.jobs["qlen"].astype(np.int64) + p.jobs["tlen"] + 1).sum())
    d_arena = torch.from_numpy(arena).cuda()
    d_res = torch.zeros(n * EXT_RESULT.itemsize, dtype=torch.uint8, device="cuda")
    d_cig = torch.zeros(cap * 4, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.ksw2g_ext_noalloc(int(p.dual), 5, p.mat.ctypes.data, p.q, p.e, p.q2, p.e2, n, jobs.ctypes.data,
                             C.c_void_p(d_arena.data_ptr()), len(arena), C.c_void_p(d_res.data_ptr()),
                             C.c_void_p(d_cig.data_ptr()), cap, C.c_void_p(stream))
    assert rc == 0, L.ksw2g_last_error().decode()
    torch.cuda.synchronize()
    res = np.frombuffer(d_res.cpu().numpy().tobytes(), EXT_RESULT)
    cig = np.frombuffer(d_cig.cpu().numpy().tobytes(), np.uint32)
    return res, cig


def _check_equal(a, ca, b, cb):
    for f in ("score", "max", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "zdropped", "reach_end", "n_cigar",
              "n_diag", "cells"):
        assert np.array_equal(a[f], b[f]), f
    for i in range(len(a)):
        k = int(a["n_cigar"][i])
        assert np.array_equal(ca[a["cigar_off"][i]:a["cigar_off"][i] + k], cb[b["cigar_off"][i]:b["cigar_off"][i] + k]), i


def test_noalloc_matches_batch_on_consecutive_calls(L):
    from minibwa_gb300 import Context, synth
    ctx = Context(0)
    try:
        for p in (synth.config0(1500, seed=77), synth.config1(600, seed=78)):  # two calls in a row
            res, cig = _run_noalloc(L, p)
            ref, rcig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
            _check_equal(res, cig, ref, rcig)
            assert (res["n_cigar"] > 0).all()
    finally:
        ctx.close()


def test_noalloc_wide_bands(L):
    """Bands wider than the widest thread group run one pair per block, with no scratch beyond
    the traceback rows."""
    from minibwa_gb300 import Context, synth
    p = synth.ext_pairs(2, dict(synth.SPEC_LONG, clip_lo=1500, clip_hi=2500), -1, 400, 10, 0x40, True, seed=80)
    ctx = Context(0)
    try:
        res, cig = _run_noalloc(L, p)
        ref, rcig = ctx.ext_batch(p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
        _check_equal(res, cig, ref, rcig)
    finally:
        ctx.close()


def test_noalloc_rejects_oversized_batches(L):
    from minibwa_gb300 import synth
    p = synth.config1(3000, seed=79)  # about 170 MB of traceback rows: beyond the fixed scratch
    jobs, _ = _padded(p.subset(np.arange(3000)))
    rc = L.ksw2g_ext_noalloc(1, 5, p.mat.ctypes.data, 12, 2, 24, 1, len(jobs), jobs.ctypes.data, 16, 1 << 40, 16, 16,
                             1 << 30, None)
    assert rc == -5  # KSW2G_E_CAPACITY, before any device work
    assert b"scratch" in L.ksw2g_last_error()
