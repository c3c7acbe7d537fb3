"""Benchmark of the ksw2 extension hot path on GB300.

Workload (N=1): 1,000,000 seeded extd2 (dual-affine) extension pairs with CIGAR,
query 100-300 nt, target = query with 2% substitutions / 0.5% indels + 50 flanking bases,
1% with a 200-nt junk query suffix, band w=100, zdrop=100, end_bonus=10.
A step is one pass of DP + backtrack over all pairs.

  value   alignments/s with the inputs resident in HBM (CUDA events on the library's stream)
  e2e     the same metric through the C ABI one-shot batch call (ksw2g_ext_batch) with pinned
          host buffers: H2D of sequences + jobs and D2H of results + CIGARs inside the timed step

`--impl reference` times the reference's CPU implementation of the path on the host cores
(oracle/_ref when the reference could be built here, else the scalar restatement in oracle/).
Under torchrun every rank runs its own replica of the workload (pairs are independent, no
collective); value is the sum over ranks divided by the max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "alignments/s"
UNIT = "aln/s"
WORKLOAD = "cfg1: 1M extd2 extension pairs, 100-300 nt, w=100, CIGAR"
# Lane operations the reference SSE code spends per nominal cell of ksw_extd2_sse with CIGAR
# (ksw2_extd2_sse.c:30-58,226-265: 54 byte-lane ops per 16-byte block of 16 cells, plus 6 for the
# substitution scores, extd2:157-172), and int32 lane ops of the exact max (extd2:326-341: 5 per
# 4 cells).  One 32-bit instruction carries 4 byte lanes, so the algorithmic int32 work is
# (54 + 6) / 4 + 5 / 4 = 16.25 instructions per cell.
INT32_OPS_PER_CELL = (54 + 6) / 4 + 5 / 4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=1000000)
    ap.add_argument("--cpu-sample", type=int, default=40000, help="pairs in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_init(args):
    rank, world = int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(x, world):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return float(x)


def allsum(x, world):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())
    return float(x)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.p, self.lines = index, None, []

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None
        return self

    def _read(self):
        for ln in self.p.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(p, sample, reference_preferred=True):
    """Time the CPU implementation on a bounded sample of the same pairs with all host threads."""
    from oracle import oracle as O
    kind = "reference" if (reference_preferred and O.have_ref()) else "port"
    threads = os.cpu_count() or 1
    sub = p.subset(np.arange(min(sample, len(p))))
    t0 = time.perf_counter()
    O.ext_batch("ref" if kind == "reference" else "orc", sub.dual, 5, sub.mat, sub.q, sub.e, sub.q2, sub.e2,
                sub.jobs, sub.qbuf, sub.tbuf, threads)
    dt = time.perf_counter() - t0
    return {"value": len(sub) / dt, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"first {len(sub)} pairs of the workload, {threads} threads, {dt:.2f} s wall"}, dt


def run_reference(args, rank, world):
    from minibwa_gb300 import synth
    if rank != 0:
        return
    p = synth.config1(max(args.cpu_sample, 1000))
    for _ in range(args.warmup):
        cpu_baseline(p, min(args.cpu_sample, 2000))
    vals, times = [], []
    for _ in range(args.steps):
        cb, dt = cpu_baseline(p, args.cpu_sample)
        vals.append(cb["value"])
        times.append(dt)
    v = len(times) * args.cpu_sample / sum(times)
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8",
            "data": "synthetic (seeded splitmix64)", "config": {"workload": WORKLOAD, "pairs_per_step": args.cpu_sample},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    rank, world = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    from minibwa_gb300 import Context, ExtBatch, synth
    from minibwa_gb300 import lib as K
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    K.load_library()
    p = synth.config1(args.pairs, seed=synth.SEED + 1 + rank * 1000)
    n = len(p)
    ctx = Context(dev)
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)

    # ---------------- value: resident inputs, device timing
    b = ExtBatch(ctx, p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf)
    for _ in range(args.warmup):
        b.run()
    ctx.sync()
    res, cig = b.fetch()
    cells = int(res["cells"].sum())
    diags = res["n_diag"].astype(np.int64)
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(args.steps):
            b.run()
        e1.record(stream)
        ctx.sync()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1) / args.steps
    launches_per_step = b.launches
    ms_max = allmax(ms, world)
    tot_pairs = allsum(n, world)
    value = tot_pairs / (ms_max * 1e-3)

    # dominant kernel alone (the DP launch of the single bin), for the roofline
    # the batch of one bin = one DP kernel + one backtrack kernel per wave; time DP share via a DP-only clone
    int_peak = K.probe_int32_peak(dev)
    achieved_int = cells * INT32_OPS_PER_CELL / (ms * 1e-3)
    # algorithmic HBM bytes per pair: traceback rows written once + read back along the path,
    # inputs, result, CIGAR (SURVEY formula)
    ncol = ((np.minimum(np.minimum(p.jobs["qlen"], p.jobs["tlen"]), 101) + 15) // 16 + 1).astype(np.int64)
    tb_bytes = int((diags * ncol * 16).sum())
    in_bytes = int(p.jobs["qlen"].sum() + p.jobs["tlen"].sum())
    path_bytes = in_bytes
    alg_bytes = tb_bytes + path_bytes + in_bytes + 4 * int(res["n_cigar"].sum()) + 64 * n
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved_gbs = alg_bytes / (ms * 1e-3) / 1e9

    # ---------------- e2e through the C ABI with pinned host buffers
    def pinned(a):
        t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
        t.numpy()[:] = a.view(np.uint8).reshape(-1)
        return t

    jobs_h, q_h, t_h = pinned(p.jobs), pinned(p.qbuf), pinned(p.tbuf)
    res_h = torch.empty(n * K.EXT_RESULT.itemsize, dtype=torch.uint8, pin_memory=True)
    cap = int((p.jobs["qlen"].astype(np.int64) + p.jobs["tlen"] + 1).sum()) + 16
    cig_h = torch.empty(cap * 4, dtype=torch.uint8, pin_memory=True)
    import ctypes as C
    L = K.load_library()
    used = C.c_int64()

    def e2e_step():
        rc = L.ksw2g_ext_batch(ctx.h, int(p.dual), 5, p.mat.ctypes.data, p.q, p.e, p.q2, p.e2, n,
                               jobs_h.data_ptr(), q_h.data_ptr(), len(p.qbuf), t_h.data_ptr(), len(p.tbuf),
                               res_h.data_ptr(), cig_h.data_ptr(), cap, C.byref(used))
        if rc != 0:
            raise RuntimeError(L.ksw2g_last_error().decode())

    for _ in range(max(1, args.warmup)):
        e2e_step()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = allmax((time.perf_counter() - t0) / args.steps, world)
    barrier(world)
    e2e_value = tot_pairs / e2e_s
    # sanity: the e2e results equal the resident-run results
    r2 = np.frombuffer(res_h.numpy().tobytes(), K.EXT_RESULT)
    assert np.array_equal(r2["max"], res["max"]) and np.array_equal(r2["n_cigar"], res["n_cigar"])
    h2d = len(p.qbuf) + len(p.tbuf) + p.jobs.nbytes
    d2h = res.nbytes + 4 * int(used.value)

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb, _ = cpu_baseline(p, args.cpu_sample)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8", "data": "synthetic (seeded splitmix64, no public dataset)",
            "config": {"workload": WORKLOAD, "pairs_per_gpu": n, "kernel": "extd2 left-aligned with CIGAR",
                       "l2": "inputs (%.0f MB arena) and traceback rows (%.1f GB per step) exceed the 129 MB L2"
                             % ((in_bytes + 128 * n) / 1e6, tb_bytes / 1e9),
                       "parallelism": f"replicas x{world}"},
            "gcups": cells / (ms * 1e-3) / 1e9,
            "cells_per_step": cells,
            "gpu_launches": launches_per_step * args.steps,
            "roofline": {"bound": "int", "achieved": achieved_int / 1e12, "peak": int_peak / 1e12,
                         "unit": "Tops/s", "frac": achieved_int / int_peak, "traffic": None,
                         "ops_per_cell": INT32_OPS_PER_CELL,
                         "peak_source": "measured in-bench: IADD3+LOP3 chains on every SM (MEASURED_PEAKS.json "
                                        "has no integer figure)"},
            "roofline_hbm": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                             "frac": achieved_gbs / hbm_peak, "algorithmic_bytes_per_step": alg_bytes,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_s * 1e3},
            "clocks": clk.summary(),
        }
        if cb:
            line["cpu_baseline"] = cb
        print(json.dumps(line), flush=True)
    b.free()
    ctx.close()


if __name__ == "__main__":
    main()
