"""Python driver of the CPU emulation of the device kernels (TEST INFRASTRUCTURE).

Builds tests/emu/libkswemu.so (g++, the kernel sources of minibwa_gb300/csrc with
cuda_emu.h) and runs jobs through it with the same padded-arena layout, work-counter
scheduling, shape choice and result layout as the CUDA library.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(HERE, "libkswemu.so")

import sys  # noqa: E402

sys.path.insert(0, ROOT)
from minibwa_gb300.lib import EXT_JOB, EXT_RESULT, LL_JOB, LL_RESULT  # noqa: E402

PARAMS_SIZE = 4 * 21 + 256  # sizeof(ksw2g_ext_params)


def build():
    src = [os.path.join(HERE, "emu_kernels.cpp")]
    deps = src + [os.path.join(HERE, "cuda_emu.h")] + [os.path.join(ROOT, "minibwa_gb300", "csrc", f) for f in
                                                        os.listdir(os.path.join(ROOT, "minibwa_gb300", "csrc"))]
    if os.path.exists(LIB) and all(os.path.getmtime(d) <= os.path.getmtime(LIB) for d in deps):
        return
    subprocess.check_call(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-w",
                           "-DKSW2G_WIDE_THREADS=64", "-o", LIB] + src)


_L = None


def lib():
    global _L
    if _L is None:
        build()
        _L = C.CDLL(LIB)
        vp, i = C.c_void_p, C.c_int
        _L.emu_ext.restype = i
        _L.emu_ext.argtypes = [i, i, i, vp, i, vp, vp, vp, vp, vp, vp, vp, C.c_longlong, i, i]
        _L.emu_ext_split.restype = i
        _L.emu_ext_split.argtypes = [i, i, i, i, vp, i, vp, vp, vp, vp, vp, vp, vp, C.c_longlong]
        _L.emu_ll.restype = i
        _L.emu_ll.argtypes = [i, i, i, vp, vp, vp, i, i, i, vp, vp, vp, i, i]
        _L.emu_derive_params.restype = None
        _L.emu_derive_params.argtypes = [i, i, vp, i, i, i, i, vp]
        _L.emu_shape_words.restype = i
        _L.emu_shape_words.argtypes = [i]
        _L.emu_shape_threads.restype = i
        _L.emu_shape_threads.argtypes = [i]
        _L.emu_num_shapes.restype = i
        _L.emu_ungap.restype = i
        _L.emu_ungap.argtypes = [i, vp, vp, vp, vp, vp, C.c_longlong]
    return _L


def slot_bytes(n):
    return 32 + ((n + 15) & ~15) + 32


def pack(qs, ts):
    """Padded arena as the device builds it; returns (arena, qoff, toff)."""
    sizes = []
    for q, t in zip(qs, ts):
        sizes += [slot_bytes(len(q)), slot_bytes(len(t))]
    arena = np.zeros(sum(sizes) + 64, np.uint8)
    qo, to, a = [], [], 0
    for q, t in zip(qs, ts):
        qo.append(a + 32)
        arena[a + 32:a + 32 + len(q)] = q
        a += slot_bytes(len(q))
        to.append(a + 32)
        arena[a + 32:a + 32 + len(t)] = t
        a += slot_bytes(len(t))
    return arena, np.array(qo, np.int64), np.array(to, np.int64)


def ncol(ql, tl, w):
    if w < 0:
        w = max(ql, tl)
    nc = min(ql, tl)
    return (min(nc, w + 1) + 15) // 16 + 1


def shape_for(nc):
    L = lib()
    for s in range(L.emu_num_shapes()):
        if L.emu_shape_words(s) >= 4 * nc:
            return s
    return -1


def ext(dual, m, mat, q, e, q2, e2, qs, ts, w, zdrop, end_bonus, flag, threads=None, shape=None, family=0,
        split=None):
    """Run one batch (one flag/mode for all jobs) through the emulated kernels (family 0: byte
    lanes, ext_dp_kernel; 1: 16-bit lanes, ext16_dp_kernel; split=(warps, words a thread): the
    block-split kernel, ext_split_kernel).
    Returns (EXT_RESULT array, list of CIGAR lists)."""
    L = lib()
    n = len(qs)
    arena, qo, to = pack(qs, ts)
    jobs = np.zeros(n, EXT_JOB)
    jobs["qoff"], jobs["toff"] = qo, to
    jobs["qlen"] = [len(x) for x in qs]
    jobs["tlen"] = [len(x) for x in ts]
    jobs["w"], jobs["zdrop"], jobs["end_bonus"], jobs["flag"] = w, zdrop, end_bonus, flag
    P = np.zeros(PARAMS_SIZE, np.uint8)
    mat = np.ascontiguousarray(mat, np.int8)
    L.emu_derive_params(int(dual), m, mat.ctypes.data, q, e, q2, e2, P.ctypes.data)
    mode = 0 if flag & 1 else (2 if flag & 2 else 1)
    if split is not None:
        nw, k = split
        if any(32 * nw * k < 4 * ncol(len(a), len(b), w) for a, b in zip(qs, ts)):
            raise ValueError("block too small for the band")
        run = lambda *a: L.emu_ext_split(int(dual), mode, nw, k, *a)  # noqa: E731
    else:
        run = None
    wide = L.emu_num_shapes()  # index of the block-wide kernel
    need = max(shape_for(ncol(len(a), len(b), w)) for a, b in zip(qs, ts))
    if need < 0:
        need = wide
    if shape is None:
        shape = need
    if shape != wide and (need == wide or L.emu_shape_words(shape) < L.emu_shape_words(need)):
        raise ValueError("shape too small for the band")
    if threads is None:  # one thread group per emulated warp
        threads = L.emu_shape_threads(shape) if shape != wide else 0
    foot = [((len(a) + len(b) - 1) * ncol(len(a), len(b), w) * 16 + 15) & ~15 if mode else 0 for a, b in zip(qs, ts)]
    tb_off = np.concatenate([[0], np.cumsum(foot)[:-1]]).astype(np.int64)
    tb = np.zeros(max(sum(foot), 16), np.uint8)
    res = np.zeros(n, EXT_RESULT)
    bts = np.zeros(n * 16, np.uint8)
    cap = sum(len(a) + len(b) + 1 for a, b in zip(qs, ts)) + 16
    cig = np.zeros(cap, np.uint32)
    if run is not None:
        rc = run(P.ctypes.data, n, jobs.ctypes.data, arena.ctypes.data, res.ctypes.data, bts.ctypes.data,
                 tb.ctypes.data, tb_off.ctypes.data, cig.ctypes.data, cap)
    else:
        rc = L.emu_ext(int(dual), mode, shape, P.ctypes.data, n, jobs.ctypes.data, arena.ctypes.data,
                       res.ctypes.data, bts.ctypes.data, tb.ctypes.data, tb_off.ctypes.data, cig.ctypes.data, cap,
                       threads, family)
    if rc != 0:
        raise RuntimeError(f"emu_ext rc={rc}")
    cigars = [cig[r["cigar_off"]:r["cigar_off"] + r["n_cigar"]].tolist() if r["n_cigar"] > 0 else [] for r in res]
    return res, cigars


def ll(size, m, mat, gapo, gape, qs, ts, xtra, threads=None, dpx=False):
    L = lib()
    n = len(qs)
    arena, qo, to = pack(qs, ts)
    jobs = np.zeros(n, LL_JOB)
    jobs["qoff"], jobs["toff"] = qo, to
    jobs["qlen"] = [len(x) for x in qs]
    jobs["tlen"] = [len(x) for x in ts]
    jobs["xtra"] = xtra
    jobs["pad"] = np.arange(n)  # the result slot of each job
    lanes = 16 if size == 1 else 8
    threads = threads or lanes
    slen = max(1, max((len(x) + lanes - 1) // lanes for x in qs))
    res = np.zeros(n, LL_RESULT)
    blo = np.concatenate([[0], np.cumsum([len(t) for t in ts])[:-1]]).astype(np.int64)
    bl = np.zeros(max(1, sum(len(t) for t in ts)), np.uint64)
    mat = np.ascontiguousarray(mat, np.int8)
    rc = L.emu_ll(size, slen, n, jobs.ctypes.data, arena.ctypes.data, mat.ctypes.data, m, gapo, gape,
                  res.ctypes.data, bl.ctypes.data, blo.ctypes.data, threads, int(dpx))
    if rc != 0:
        raise RuntimeError(f"emu_ll rc={rc}")
    return res


UNGAP_JOB = np.dtype([("qoff", "<i8"), ("toff", "<i8"), ("qlen", "<i4"), ("tlen", "<i4"), ("meth", "<i4"),
                      ("pad", "<i4")])


def ungap(pairs, meth, global_hist=False):
    """mb_ungap of (query, target) pairs through the emulated device kernel; returns a list of
    (max, max_i, n_good, n_kmer).  Targets sit in a padded arena as the window gather leaves them."""
    L = lib()
    n = len(pairs)
    jobs = np.zeros(n, UNGAP_JOB)
    qs, ts, qo, to = [], [], 0, 0
    for i, (q, t) in enumerate(pairs):
        jobs[i]["qoff"], jobs[i]["qlen"], jobs[i]["toff"] = qo, len(q), to + 32
        jobs[i]["tlen"], jobs[i]["meth"] = len(t), meth[i]
        qs.append(np.asarray(q, np.uint8))
        qo += len(q)
        slot = np.zeros(slot_bytes(len(t)), np.uint8)
        slot[32:32 + len(t)] = t
        ts.append(slot)
        to += len(slot)
    qa = np.concatenate(qs + [np.zeros(16, np.uint8)])
    ta = np.concatenate(ts + [np.zeros(64, np.uint8)])
    res = np.zeros((n, 4), np.int32)
    cap = max([len(t) for _, t in pairs] + [1])
    hist = np.zeros(cap, np.int32) if global_hist else None
    L.emu_ungap(n, jobs.ctypes.data, qa.ctypes.data, ta.ctypes.data, res.ctypes.data,
                hist.ctypes.data if hist is not None else None, cap if global_hist else 0)
    return [tuple(int(x) for x in r) for r in res]
