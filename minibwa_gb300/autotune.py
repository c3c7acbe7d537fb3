"""Autotuner for the extension kernels' thread-group shape and lane width.

A pair whose reference n_col_ (16-byte blocks per anti-diagonal, ksw2_extz2_sse.c:68) is c
can run on every instantiated shape (G threads x K words) with G*K >= 4*c, on byte lanes or on
16-bit DPX lanes.  Fewer threads per pair mean more words per thread (more independent work
between the per-anti-diagonal reductions, more registers); more threads mean more pairs in
flight per SM is lower.  The tuner times every eligible (shape, lane width) on a sample of each
n_col_ class of a workload (device time, CUDA events on the library's stream) and installs the
fastest in the library's preference table (ksw2g_ext_set_shape).  Results are plain dicts, so
a caller can store and reapply them.
"""
import ctypes as C

import numpy as np

from .lib import EXT_JOB, ExtBatch, load_library


def shapes():
    L = load_library()
    out = []
    for s in range(L.ksw2g_ext_num_shapes()):
        g, k = C.c_int(), C.c_int()
        L.ksw2g_ext_shape_info(s, C.byref(g), C.byref(k))
        out.append((g.value, k.value))
    return out


def ncol(qlen, tlen, w):
    w = np.where(w < 0, np.maximum(qlen, tlen), w)
    nc = np.minimum(qlen, tlen)
    return (np.minimum(nc, w + 1) + 15) // 16 + 1


def mode_of(flag):
    return 0 if flag & 1 else (2 if flag & 2 else 1)


def _time_batch(ctx, b, reps):
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream)
    b.run()
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        b.run()
    e1.record(stream)
    ctx.sync()
    return e0.elapsed_time(e1) / reps


def tune_ext(ctx, pairs, sample=32768, reps=3, min_class=64, seed=1, lanes=True):
    """Tune the shape (and with `lanes` True the lane width; 0 or 1 keeps byte or 16-bit lanes) of
    every n_col_ class of `pairs` (a synth.Pairs or anything with the same fields).  Installs the
    winners and returns
    {(dual, mode, ncol): (G, K, w16, ms_per_pair_by_choice)}, choices keyed (G, K, w16); a
    scoring the 16-bit lanes cannot hold runs those choices on byte lanes, so they tie.

    The sample must fill the GPU the way the real batch does: on GB300 a 4,096-pair sample of
    150 nt pairs favours groups of 8 threads, while full batches of them run 30% faster in
    groups of 4, because a small sample leaves most SMs idle and rewards spreading each pair
    over more threads."""
    L = load_library()
    shp = shapes()
    jobs = pairs.jobs
    nc = ncol(jobs["qlen"].astype(np.int64), jobs["tlen"].astype(np.int64), jobs["w"].astype(np.int64))
    modes = np.array([mode_of(int(f)) for f in jobs["flag"]])
    rng = np.random.default_rng(seed)
    widths = (0, 1) if lanes is True else (int(lanes),)
    table = {}
    for md in np.unique(modes):
        for c in np.unique(nc[modes == md]):
            idx = np.nonzero((nc == c) & (modes == md))[0]
            if len(idx) < min_class:
                continue
            idx = np.sort(rng.choice(idx, min(sample, len(idx)), replace=False))
            sub = pairs.subset(idx)
            timings = {}
            for s, (g, k) in enumerate(shp):
                if g * k < 4 * int(c):
                    continue
                for w16 in widths:
                    L.ksw2g_ext_set_shape(int(pairs.dual), int(md), int(c), int(c), s + w16 * len(shp))
                    b = ExtBatch(ctx, sub.dual, 5, sub.mat, sub.q, sub.e, sub.q2, sub.e2, sub.jobs, sub.qbuf,
                                 sub.tbuf)
                    timings[(s, w16)] = _time_batch(ctx, b, reps)
                    b.free()
            best = min(timings, key=timings.get)
            L.ksw2g_ext_set_shape(int(pairs.dual), int(md), int(c), int(c), best[0] + best[1] * len(shp))
            table[(int(pairs.dual), int(md), int(c))] = (
                shp[best[0]][0], shp[best[0]][1], best[1],
                {(shp[s][0], shp[s][1], w): timings[(s, w)] / len(idx) for s, w in timings})
    return table


def apply(table):
    """Reinstall a table returned by tune_ext."""
    L = load_library()
    shp = shapes()
    for (dual, md, c), (g, k, w16, _) in table.items():
        L.ksw2g_ext_set_shape(dual, md, c, c, shp.index((g, k)) + w16 * len(shp))


def reset(table):
    """Put the classes of a table back on their default: the smallest byte-lane shape that holds
    the band."""
    L = load_library()
    shp = shapes()
    for (dual, md, c) in table:
        s = next(i for i, (g, k) in enumerate(shp) if g * k >= 4 * c)
        L.ksw2g_ext_set_shape(dual, md, c, c, s)


__all__ = ["tune_ext", "apply", "reset", "shapes", "EXT_JOB"]
