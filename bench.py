"""Benchmark of the ksw2 extension / rescue hot path on GB300.

Default workload (N=1), the one the headline metric is quoted on: 1,000,000 seeded extd2
(dual-affine) extension pairs with CIGAR, query 100-300 nt, target = query with 2%
substitutions / 0.5% indels + 50 flanking bases, 1% with a 200-nt junk query suffix, band
w=100, zdrop=100, end_bonus=10.  A step is one pass of DP + backtrack over all pairs.

  value     alignments/s with the inputs resident in HBM (CUDA events on the library's stream)
  e2e       the same metric through the C ABI one-shot batch call (ksw2g_ext_batch) with pinned
            host buffers: H2D of sequences + jobs and D2H of results + CIGARs inside the timed step
  roofline  the DP kernel alone: integer ops of the reference's SSE lane-op count per cell x cells,
            over the DP launches' summed duration (CUDA events around every launch, on the
            launching stream, during the timed steps); traffic = DRAM bytes per cell from ncu x cells

Other workloads (--workload): cfg0 (20k extz2 pairs), cfg2 (200k long extd2 + 1M short extz2 in one
CUDA graph, two branches), cfg3 (2M ksw_ll i16 rescue jobs).

`--impl reference` times the reference's CPU implementation of the path on the host cores
(oracle/_ref when the reference could be built here, else the scalar restatement in oracle/).
Under torchrun every rank runs its own replica of the workload (pairs are independent, no
collective); value is the sum over ranks divided by the max-over-ranks time.
"""
import argparse
import ctypes as C
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

# 32-bit integer operations per nominal cell, from the reference SSE code's lane operations:
# byte-lane ops count 1/4 (four byte lanes per 32-bit op), int16-lane ops 1/2, and int32-lane ops 1
# (one lane per 32-bit op):
#  extd2 with CIGAR: 54 byte-lane ops per cell of a 16-cell block (ksw2_extd2_sse.c:183-265) + 6 for
#    the substitution scores (extd2:157-172), and 6 int32 lane ops of the exact max (extd2:315-345):
#    60/4 + 6 = 21;
#  extz2 with CIGAR: 29 + 6 byte-lane ops (ksw2_extz2_sse.c:117-136,163-188) and 5 int32 (extz2:216-243):
#    35/4 + 5 = 13.75;
#  ksw_ll i16: 10 int16-lane ops per cell (ksw2_ll_sse.c:265-286), lazy-F passes not counted: 10/2 = 5.
OPS_PER_CELL = {
    "extd2": (54 + 6) / 4 + 6,
    "extz2": (29 + 6) / 4 + 5,
    "ll_i16": 10 / 2,
}
# DRAM bytes per nominal cell of the DP kernel, from ncu (dram__bytes_read.sum + dram__bytes_write.sum
# of one captured launch / its cells), scaled to the workload's launches by their cell counts.
# extd2: 188,659,200 + 791,366,144 B over 674,520,661 cells (ext_dp_kernel<1,1,8,4>, 20,000 config-1 pairs);
# extz2: 129,133,568 + 261,759,488 B over 146,499,977 cells (ext_dp_kernel<0,1,4,3>, 20,000 config-0 pairs);
# ll_i16: 111,992,832 B over 11,259,234,900 cells (ll_dpx_kernel<2,20>, 100,000 config-3 jobs).
# All grow with the cells a launch processes (traceback rows and sequences), so they scale.
DRAM_BYTES_PER_CELL = {"extd2": (188659200 + 791366144) / 674520661, "extz2": (129133568 + 261759488) / 146499977,
                       "ll_i16": 111992832 / 11259234900}

WORKLOADS = {
    "cfg1": "cfg1: 1M extd2 extension pairs, 100-300 nt, w=100, CIGAR",
    "cfg0": "cfg0: 20k extz2 extension pairs, 150 nt, w=25, CIGAR",
    "cfg2": "cfg2: 200k long extd2 (log-normal median 2 kb, w=500) + 1M short extz2 (150 nt, w=25), "
            "one CUDA graph, CIGAR",
    "cfg3": "cfg3: 2M ksw_ll i16 rescue jobs, 150 nt vs 500-1000 nt",
    "rescue": "rescue: 500k pe.c mate-rescue candidates (mb_ungap + ksw_ll + reverse extz2) over an "
              "80 Mb resident 2-bit reference, reads 100-250 nt, insert bounds [50, 800]",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cfg1", choices=sorted(WORKLOADS))
    ap.add_argument("--pairs", type=int, default=None, help="override the workload's unit count")
    ap.add_argument("--cpu-sample", type=int, default=None, help="units in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline workload only (by default a cfg1 run also measures cfg2, cfg3 and one "
                         "serving point)")
    ap.add_argument("--lanes", type=int, default=-1, choices=[-1, 0, 1],
                    help="extension DP lane width: -1 the library's choice, 0 bytes, 1 16-bit (DPX)")
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


def _reduce(x, world, op):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(x)], dtype=torch.float64)
        dist.all_reduce(t, op=op)
        return float(t.item())
    return float(x)


def allmax(x, world):
    if world > 1:
        import torch.distributed as dist
        return _reduce(x, world, dist.ReduceOp.MAX)
    return float(x)


def allsum(x, world):
    if world > 1:
        import torch.distributed as dist
        return _reduce(x, world, dist.ReduceOp.SUM)
    return float(x)


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region (started, and its first
    sample awaited, before the region begins)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.p, self.lines = index, None, []
        self.first = threading.Event()

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=5)
        except Exception:
            self.p = None
        return self

    def _read(self):
        for ln in self.p.stdout:
            self.lines.append(ln.strip())
            self.first.set()

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


# ------------------------------------------------------------------ workloads
class Workload:
    """The inputs of one benchmark configuration and how to run them."""

    def __init__(self, name, args, rank, sizes_only=False, prefix=None):
        from minibwa_gb300 import synth
        self.name, self.desc = name, WORKLOADS[name]
        seed_shift = rank * 1000
        n = args.pairs
        if name == "cfg1":
            spec = [(synth.config1, n or 1000000, synth.SEED + 1)]
        elif name == "cfg0":
            spec = [(synth.config0, n or 20000, synth.SEED)]
        elif name == "cfg2":
            nl = (n or 1200000) // 6
            spec = [(synth.config2_long, nl, synth.SEED + 2), (synth.config2_short, nl * 5, synth.SEED + 3)]
        else:
            spec = [(synth.config3, n or 2000000, synth.SEED + 4)]
        self.set_sizes = [k for _, k, _ in spec]
        self.ll = name == "cfg3"
        self.metric = "jobs/s" if self.ll else "alignments/s"
        self.unit = "jobs/s" if self.ll else "aln/s"
        if sizes_only:
            self.sets, self.n = [], sum(self.set_sizes)
            return
        if prefix is not None:  # the first units of every set (the generator is sequential per set)
            spec = [(f, p, sd) for (f, _, sd), p in zip(spec, prefix)]
        self.sets = [f(k, seed=sd + seed_shift) for f, k, sd in spec]
        self.kind = "ll_i16" if self.ll else ("extd2" if self.sets[0].dual else "extz2")
        self.n = sum(len(s) for s in self.sets)

    def kernel_kinds(self):
        return ["ll_i16" if self.ll else ("extd2" if s.dual else "extz2") for s in self.sets]


def prepare(ctx, s):
    from minibwa_gb300 import ExtBatch, LLBatch
    if hasattr(s, "size"):
        return LLBatch(ctx, s.size, 5, s.mat, s.gapo, s.gape, s.jobs, s.qbuf, s.tbuf)
    return ExtBatch(ctx, s.dual, 5, s.mat, s.q, s.e, s.q2, s.e2, s.jobs, s.qbuf, s.tbuf)


def cells_of(s, res):
    if hasattr(s, "size"):
        return int((res["rows"].astype(np.int64) * s.jobs["qlen"]).sum())
    return int(res["cells"].sum())


def cpu_baseline(w, sample, reference_preferred=True):
    """Time the CPU implementation on a bounded sample of the same units with all host threads:
    the reference's own ksw2 SIMD code (oracle/_ref, compiled from the reference's sources, jobs
    spread by its kt_for) when it could be built, else the scalar restatement.  Returns (baseline
    dict, seconds, per-set outputs), the outputs being (results, CIGAR words) of the first units of
    every set."""
    from oracle import oracle as O
    kind = "reference" if (reference_preferred and O.have_ref()) else "port"
    which = "ref" if kind == "reference" else "orc"
    threads = os.cpu_count() or 1
    # the sample keeps the workload's mix: the same fraction of every set
    frac = min(1.0, sample / w.n)
    subs = []
    for s in w.sets:
        k = max(1, int(round(len(s) * frac)))
        subs.append(s.subset(np.arange(k)))
    outs, n_done = [], 0
    t0 = time.perf_counter()
    for sub in subs:
        if hasattr(sub, "size"):
            outs.append((O.ll_batch(which, sub.size, 5, sub.mat, sub.gapo, sub.gape, sub.jobs, sub.qbuf, sub.tbuf,
                                    threads), None))
        else:
            outs.append(O.ext_batch(which, sub.dual, 5, sub.mat, sub.q, sub.e, sub.q2, sub.e2, sub.jobs, sub.qbuf,
                                    sub.tbuf, threads))
        n_done += len(sub)
    dt = time.perf_counter() - t0
    what = ("the reference's ksw2 SIMD functions (NEON via s2n-lite.h on Arm, SSE4 on x86-64) compiled from its "
            "sources, jobs spread over the threads by its kt_for" if kind == "reference" else
            "the scalar C restatement of the reference (the reference's sources were not available)")
    return ({"value": n_done / dt, "unit": w.unit, "cores": threads, "kind": kind,
             "sample": f"first {n_done} units of the benchmarked set (same seed, same mix), {threads} threads, "
                       f"{dt:.2f} s wall; {what}"}, dt, outs)


def parity_vs_cpu(w, results, outs, kind):
    """Compare the GPU's results on the first units of every set with the CPU run's outputs,
    field by field and CIGAR by CIGAR."""
    fields_ext = ("score", "max", "max_q", "max_t", "mqe", "mqe_t", "mte", "mte_q", "zdropped", "reach_end",
                  "n_cigar")
    n, bad = 0, 0
    for s, r, (cres, ccig) in zip(w.sets, results, outs):
        k = len(cres)
        n += k
        if hasattr(s, "size"):
            ok = np.ones(k, bool)
            for f in ("score", "te", "qe", "score2", "te2"):
                ok &= r[f][:k] == cres[f]
        else:
            gres, gcig = r
            ok = np.ones(k, bool)
            for f in fields_ext:
                ok &= gres[f][:k] == cres[f]
            for i in np.nonzero(ok)[0]:
                m = int(gres["n_cigar"][i])
                a, b = int(gres["cigar_off"][i]), int(cres["cigar_off"][i])
                if m and not np.array_equal(gcig[a:a + m], ccig[b:b + m]):
                    ok[i] = False
        bad += int((~ok).sum())
    return {"against": kind, "units": n, "mismatches": bad, "equal": bad == 0}


DEFAULT_SAMPLE = {"cfg1": 100000, "cfg0": 20000, "cfg2": 6000, "cfg3": 100000, "rescue": 60000}


def workload_config(name, n, world):
    """The config dict of a workload; both arms print the same one."""
    return {"workload": WORKLOADS[name], "units_per_gpu": n, "parallelism": f"replicas x{world}",
            "graph": name == "cfg2",
            "l2": "inputs and traceback rows exceed the 129 MB L2 on every step (no flush needed)"}


def rescue_cpu_baseline(ref, jobs, qbuf, sample):
    """The CPU restatement of the rescue (oracle/rescue_cpu.c) on the first `sample` candidates
    with all host threads; returns (baseline dict, its results, CIGAR words)."""
    from minibwa_gb300 import synth
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    k = min(sample, len(jobs))
    t0 = time.perf_counter()
    res, cig = O.rescue_batch(ref, synth.RESCUE_OPT_SR, jobs[:k], qbuf, threads)
    dt = time.perf_counter() - t0
    return ({"value": k / dt, "unit": "candidates/s", "cores": threads, "kind": "port",
             "sample": f"first {k} candidates of the workload, {threads} threads, {dt:.2f} s wall "
                       f"(scalar C restatement of pe.c's rescue over the oracle's ksw2 restatement)"},
            res, cig, dt)


def run_rescue(args, rank, world):
    """The mate-rescue workload: every step is one ksw2g_rescue_batch call over all candidates
    (reads and job records from pinned host memory, results and CIGARs back to the host); the
    2-bit reference stays resident in HBM.  The call's stages read one another's results on the
    host, so there is no device-only variant: value and e2e are the same timed call."""
    import torch
    from minibwa_gb300 import Context, Reference, synth
    from minibwa_gb300 import lib as K
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    L = K.load_library()
    n = args.pairs or 500000
    ref, jobs, qbuf = synth.rescue_workload(n, seed=synth.SEED + 60 + 1000 * rank)
    ctx = Context(dev)
    dref = Reference(ctx, ref.pac, ref.ctg_off, ref.ctg_len, ref.ambi)
    opt = np.zeros(1, K.RESCUE_OPT)
    for k_, v in synth.RESCUE_OPT_SR.items():
        opt[k_] = v

    def pinned(a):
        t = torch.empty(max(1, a.nbytes), dtype=torch.uint8, pin_memory=True)
        t.numpy()[:a.nbytes] = a.view(np.uint8).reshape(-1)
        return t

    hj, hq = pinned(jobs), pinned(qbuf)
    hres = torch.empty(n * K.RESCUE_RESULT.itemsize, dtype=torch.uint8, pin_memory=True)
    cap = int((jobs["qlen"].astype(np.int64) + jobs["te"] - jobs["ts"] + 1).sum()) + 16
    hcig = torch.empty(cap * 4, dtype=torch.uint8, pin_memory=True)
    used = C.c_int64()

    def step():
        rc = L.ksw2g_rescue_batch(ctx.h, dref.h, opt.ctypes.data, n, hj.data_ptr(), hq.data_ptr(), len(qbuf),
                                  hres.data_ptr(), hcig.data_ptr(), cap, C.byref(used))
        if rc != 0:
            raise RuntimeError(L.ksw2g_last_error().decode())

    for _ in range(args.warmup):
        step()
    barrier(world)
    torch.cuda.synchronize()
    stage_ms = np.zeros(3)
    dev_ms = np.zeros(2)
    launches = 0
    with ClockSampler(dev) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
            nl, ms3 = dref.rescue_stats()
            launches += nl
            stage_ms += ms3
            dev_ms += dref.rescue_device_ms()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / args.steps
    dt_max = allmax(dt, world)
    barrier(world)
    tot = allsum(n, world)
    value = tot / dt_max
    res = np.frombuffer(hres.numpy().tobytes(), K.RESCUE_RESULT)
    cig = np.frombuffer(hcig.numpy()[:4 * used.value].tobytes(), np.uint32)
    cb = None
    checked = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb, ores, ocig, _ = rescue_cpu_baseline(ref, jobs, qbuf, args.cpu_sample or DEFAULT_SAMPLE["rescue"])
        k = len(ores)
        same = all(np.array_equal(res[f][:k], ores[f]) for f in
                   ("max_ug", "max_i", "n_good", "n_kmer", "ts2", "te2", "ll_score", "ll_te", "ll_qe", "ll_score2",
                    "rescued", "qs", "qe", "ts", "te", "dp_max2"))
        for i in np.nonzero(ores["ext"]["n_cigar"] > 0)[0][:2000]:
            a, b = res[i]["ext"], ores[i]["ext"]
            same &= bool(np.array_equal(cig[a["cigar_off"]:a["cigar_off"] + a["n_cigar"]],
                                        ocig[b["cigar_off"]:b["cigar_off"] + b["n_cigar"]]))
        checked = f"first {k} candidates equal the CPU restatement field by field: {bool(same)}"
    if rank == 0:
        h2d = jobs.nbytes + len(qbuf)
        d2h = res.nbytes + 4 * used.value
        stage_ms /= args.steps
        dev_ms /= args.steps
        line = {
            "metric": "rescue candidates/s", "value": value, "unit": "candidates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt_max * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "int8/int16",
            "data": "synthetic (seeded splitmix64 candidates over a seeded reference, no public dataset)",
            "config": {"workload": WORKLOADS["rescue"], "units_per_gpu": n, "parallelism": f"replicas x{world}",
                       "value_is_e2e": "the stages read each other's results on the host; the reference is "
                                       "resident, reads and results cross PCIe/C2C every step",
                       "rescued_fraction": float(res["rescued"].mean()),
                       "ll_fraction": float(res["ll_done"].mean())},
            "stages_ms": {"gather_prefilter": stage_ms[0], "ksw_ll": stage_ms[1], "extz2": stage_ms[2]},
            "kernels_ms": {"ksw_ll": dev_ms[0], "extz2": dev_ms[1],
                           "note": "CUDA events around the stages' DP and backtrack launches; the rest of each "
                                   "stage is host work and copies"},
            "gpu_launches": launches,
            "roofline": None,
            "e2e": {"value": value, "unit": "candidates/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "ms_per_step": dt_max * 1e3},
            "clocks": clk.summary(),
        }
        if cb:
            line["cpu_baseline"] = cb
            line["parity"] = checked
        print(json.dumps(line), flush=True)
    dref.close()
    ctx.close()


def run_reference(args, rank, world):
    if rank != 0:
        return
    if args.workload == "rescue":
        from minibwa_gb300 import synth
        sample = args.cpu_sample or DEFAULT_SAMPLE["rescue"]
        ref, jobs, qbuf = synth.rescue_workload(sample)
        for _ in range(args.warmup):
            rescue_cpu_baseline(ref, jobs, qbuf, max(1, sample // 20))
        times = []
        for _ in range(args.steps):
            cb, _, _, dt = rescue_cpu_baseline(ref, jobs, qbuf, sample)
            times.append(dt)
        v = len(times) * sample / sum(times)
        cb["value"] = v
        print(json.dumps({"impl": "reference", "metric": "rescue candidates/s", "value": v, "unit": "candidates/s",
                          "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                          "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "int8/int16",
                          "data": "synthetic (seeded splitmix64)",
                          "config": {"workload": WORKLOADS["rescue"], "units_per_step": sample},
                          "cpu_baseline": cb, "e2e": {"value": v, "unit": "candidates/s", "h2d_bytes_per_step": 0,
                                                      "d2h_bytes_per_step": 0}}), flush=True)
        return
    # The benchmarked sets are generated by one sequential splitmix64 stream per set, so their first
    # units do not depend on the set size: generate only the sample's prefix of each set.
    sample = args.cpu_sample or DEFAULT_SAMPLE[args.workload]
    full = Workload(args.workload, args, 0, sizes_only=True)
    frac = min(1.0, sample / full.n)
    args_s = argparse.Namespace(**vars(args))
    w = Workload(args.workload, args_s, 0, prefix=[max(1, int(round(n * frac))) for n in full.set_sizes])
    for _ in range(args.warmup):
        cpu_baseline(w, max(1, w.n // 20))
    times = []
    for _ in range(args.steps):
        cb, dt, _ = cpu_baseline(w, w.n)
        times.append(dt)
    v = len(times) * w.n / sum(times)
    cb["value"] = v
    line = {"impl": "reference", "metric": w.metric, "value": v, "unit": w.unit, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16" if args.workload == "cfg3" else "int8",
            "data": "synthetic (seeded splitmix64, no public dataset)",
            "config": workload_config(args.workload, full.n, args.gpus),
            "cpu_baseline": cb, "e2e": {"value": v, "unit": w.unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# Traceback pool of config 2's own context.  Its 200k long pairs with CIGAR write about 420 GB
# of traceback rows a step, which the default 16 GiB pool takes in about 70 waves, each ending
# with its longest pair's tail.  48 GiB of the GPU's 288 GB (120 GiB with the three half-size
# sub-contexts of the end-to-end calls) measured 814 k against 734 k alignments/s resident and
# 742 k against 657 k end to end; 96 GiB added nothing resident.
CFG2_TB_BUDGET = 48 << 30


def measure(args, w, ctx, dev, rank, world, steps, warmup, int_peak, with_cpu, sample):
    """One workload: resident-input device timing, the DP kernel's roofline, end-to-end timing
    through the C ABI one-shot calls, and (rank 0, N=1) the CPU baseline and parity on a
    sample.  Returns the JSON fields of the workload.  Config 2 runs on a context of its own
    with a larger traceback pool, released afterwards."""
    if w.name != "cfg2":
        return _measure(args, w, ctx, dev, rank, world, steps, warmup, int_peak, with_cpu, sample)
    import gc
    from minibwa_gb300 import Context
    own = Context(dev, tb_budget=CFG2_TB_BUDGET)
    try:
        out = _measure(args, w, own, dev, rank, world, steps, warmup, int_peak, with_cpu, sample)
        out["tb_budget_gib"] = CFG2_TB_BUDGET >> 30
        return out
    finally:
        gc.collect()  # the workload's batches and graph go before their context
        own.close()


def _measure(args, w, ctx, dev, rank, world, steps, warmup, int_peak, with_cpu, sample):
    import torch
    from minibwa_gb300 import Graph
    from minibwa_gb300 import lib as K
    L = K.load_library()
    stream = torch.cuda.ExternalStream(ctx.stream, device=dev)

    # config 2 runs with an autotuned thread-group shape and lane width per band class: the tuner
    # times every eligible choice on a sample of each class first (not timed here); --lanes 0 or 1
    # keeps the tuner to that lane width
    tuned = {}
    if w.name == "cfg2":
        from minibwa_gb300 import autotune
        for s in w.sets:
            lanes = True if args.lanes < 0 else args.lanes
            tuned.update(autotune.tune_ext(ctx, s, sample=16384, reps=2, lanes=lanes))

    # ---------------- value: resident inputs, device timing
    batches = [prepare(ctx, s) for s in w.sets]
    graph = Graph(ctx, batches) if len(batches) > 1 else None

    def step():
        if graph is not None:
            graph.launch()
        else:
            batches[0].run()

    for _ in range(warmup):
        step()
    ctx.sync()
    results = [b.fetch() for b in batches]
    res_list = [r if w.ll else r[0] for r in results]
    cells = [cells_of(s, r) for s, r in zip(w.sets, res_list)]
    if graph is None:
        batches[0].set_timing(True)
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        e0.record(stream)
        for _ in range(steps):
            step()
        e1.record(stream)
        ctx.sync()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1) / steps
    launches_per_step = graph.launches if graph is not None else batches[0].launches
    ms_max = allmax(ms, world)
    tot = allsum(w.n, world)
    value = tot / (ms_max * 1e-3)
    tot_cells = sum(cells)

    # ---------------- roofline of the dominant kernel (the DP kernel)
    kinds = w.kernel_kinds()
    ops = sum(c * OPS_PER_CELL[k] for c, k in zip(cells, kinds))
    n_dp = 1
    if graph is None:
        dp_ms, bt_ms, n_dp, n_bt = batches[0].kernel_ms()
        n_dp = max(1, n_dp // steps)
        dp_ms_step = dp_ms / steps
        kernel_note = (f"DP kernel: {n_dp} launches per step, busy {dp_ms_step:.2f} ms per step "
                       f"(backtrack {bt_ms / steps:.2f} ms); CUDA events around each launch, the "
                       f"union of their intervals (waves alternate between two streams)")
    else:
        dp_ms_step = ms  # branches overlap inside the graph: the whole graph is the timed unit
        kernel_note = "whole graph (DP branches overlap); CUDA events around each graph launch"
    achieved = ops / (dp_ms_step * 1e-3)
    bpc = [DRAM_BYTES_PER_CELL.get(k) for k in kinds]
    # per DP launch (per graph launch for a graph), like achieved
    traffic = sum(c * b for c, b in zip(cells, bpc)) / n_dp if all(b is not None for b in bpc) else None
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    # algorithmic HBM bytes per step (traceback rows written once and read along the path,
    # inputs, results and CIGARs)
    alg_bytes = 0
    for s, r in zip(w.sets, res_list):
        if hasattr(s, "size"):
            alg_bytes += int(s.jobs["qlen"].sum() + s.jobs["tlen"].sum()) + 24 * len(s)
        else:
            jq, jt = s.jobs["qlen"].astype(np.int64), s.jobs["tlen"].astype(np.int64)
            ww = np.where(s.jobs["w"] < 0, np.maximum(jq, jt), s.jobs["w"]).astype(np.int64)
            ncol = (np.minimum(np.minimum(jq, jt), ww + 1) + 15) // 16 + 1
            tb = int((r["n_diag"].astype(np.int64) * ncol * 16).sum())
            alg_bytes += tb + 2 * int(jq.sum() + jt.sum()) + 4 * int(r["n_cigar"].sum()) + 64 * len(s)
    achieved_gbs = alg_bytes / (ms * 1e-3) / 1e9
    if graph is not None:
        graph.close()
    for b in batches:
        b.free()

    # ---------------- e2e through the C ABI one-shot calls with pinned host buffers
    def pinned(a):
        t = torch.empty(max(1, a.nbytes), dtype=torch.uint8, pin_memory=True)
        t.numpy()[:a.nbytes] = a.view(np.uint8).reshape(-1)
        return t

    host = []
    for s in w.sets:
        d = {"jobs": pinned(s.jobs), "q": pinned(s.qbuf), "t": pinned(s.tbuf)}
        if hasattr(s, "size"):
            d["res"] = torch.empty(len(s) * K.LL_RESULT.itemsize, dtype=torch.uint8, pin_memory=True)
        else:
            d["res"] = torch.empty(len(s) * K.EXT_RESULT.itemsize, dtype=torch.uint8, pin_memory=True)
            d["cap"] = int((s.jobs["qlen"].astype(np.int64) + s.jobs["tlen"] + 1).sum()) + 16
            d["cig"] = torch.empty(d["cap"] * 4, dtype=torch.uint8, pin_memory=True)
        host.append(d)
    used = [C.c_int64() for _ in w.sets]

    def e2e_step():
        for s, d, u in zip(w.sets, host, used):
            if hasattr(s, "size"):
                rc = L.ksw2g_ll_batch(ctx.h, s.size, 5, s.mat.ctypes.data, s.gapo, s.gape, len(s),
                                      d["jobs"].data_ptr(), d["q"].data_ptr(), len(s.qbuf), d["t"].data_ptr(),
                                      len(s.tbuf), d["res"].data_ptr())
            else:
                rc = L.ksw2g_ext_batch(ctx.h, int(s.dual), 5, s.mat.ctypes.data, s.q, s.e, s.q2, s.e2, len(s),
                                       d["jobs"].data_ptr(), d["q"].data_ptr(), len(s.qbuf), d["t"].data_ptr(),
                                       len(s.tbuf), d["res"].data_ptr(), d["cig"].data_ptr(), d["cap"],
                                       C.byref(u))
            if rc != 0:
                raise RuntimeError(L.ksw2g_last_error().decode())

    for _ in range(max(1, min(warmup, 2))):
        e2e_step()
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = allmax((time.perf_counter() - t0) / steps, world)
    barrier(world)
    e2e_value = tot / e2e_s
    # the e2e results equal the resident-run results
    h2d = d2h = 0
    for s, d, r, u in zip(w.sets, host, res_list, used):
        dt = K.LL_RESULT if hasattr(s, "size") else K.EXT_RESULT
        r2 = np.frombuffer(d["res"].numpy().tobytes(), dt)
        assert np.array_equal(r2["score"], r["score"])
        h2d += len(s.qbuf) + len(s.tbuf) + s.jobs.nbytes
        d2h += r.nbytes + 4 * int(u.value)

    out = {
        "value": value, "unit": w.unit, "ms_per_step": ms_max, "steps": steps, "warmup": warmup,
        "gcups": tot_cells / (ms * 1e-3) / 1e9, "cells_per_step": tot_cells, "bytes_per_step": alg_bytes,
        "gpu_launches": launches_per_step * steps,
        "roofline": {"bound": "int", "achieved": achieved / 1e12, "peak": int_peak / 1e12, "unit": "Tops/s",
                     "frac": achieved / int_peak, "traffic": traffic,
                     "ops_per_cell": {k: OPS_PER_CELL[k] for k in sorted(set(kinds))},
                     "kernel": kernel_note,
                     "peak_source": "measured in-bench: IADD3+LOP3 chains on every SM (MEASURED_PEAKS.json "
                                    "has no integer figure)"},
        "roofline_hbm": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved_gbs / hbm_peak, "algorithmic_bytes_per_step": alg_bytes,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
        "e2e": {"value": e2e_value, "unit": w.unit, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": e2e_s * 1e3},
        "clocks": clk.summary(),
    }
    if with_cpu and rank == 0 and world == 1:
        cb, _, outs = cpu_baseline(w, sample)
        out["cpu_baseline"] = cb
        out["parity_vs_cpu"] = parity_vs_cpu(w, results, outs, cb["kind"])
    if tuned:
        from minibwa_gb300 import autotune
        out["autotuned"] = {f"{'extd2' if d else 'extz2'} mode {md} n_col {c}":
                            f"{g}x{k} {'16-bit' if w16 else 'byte'} lanes" for (d, md, c), (g, k, w16, _) in tuned.items()}
        autotune.reset(tuned)  # later workloads of the run start from the default shapes
    return out


def serving_point(frac=0.8, duration=3.0):
    """Config 4 at one offered load: the continuous-batching engine's p50 / p99 latency and served
    rate at `frac` of its measured peak (every job checked against the same job run alone), and
    the reference CPU implementation's rate on a sample of the same mix."""
    from minibwa_gb300 import serving
    from oracle import oracle as O
    # the per-call drop-in's closed-loop rate on the same mix (16 caller threads, about 4 s at most)
    out = serving.sweep(duration=duration, fracs=(frac,), percall_threads=16, check=True, log=open(os.devnull, "w"),
                        percall_peak_jobs=6000, percall_deadline=1.0, percall_peak_only=True)
    row = out["rates"][0]
    line = {"metric": "served jobs/s at %d%% of peak, p50/p99 latency" % round(frac * 100),
            "value": row["served_jobs_s"], "unit": "jobs/s", "p50_ms": row["p50_ms"], "p99_ms": row["p99_ms"],
            "max_ms": row["max_ms"], "offered_jobs_s": row["offered_jobs_s"], "peak_jobs_s": out["peak_jobs_s"],
            "requests": row["requests"], "duration_s": duration,
            "mismatches_vs_alone": out["mismatches_vs_alone"],
            "percall_dropin_jobs_s": out.get("percall_peak_jobs_s"),
            "engine_peak_over_percall": (out["peak_jobs_s"] / out["percall_peak_jobs_s"]
                                         if out.get("percall_peak_jobs_s") else None),
            "mix": "70% extz2 150 nt w=25, 20% extd2 log-normal 1-10 kb w=500, 10% ksw_ll i16; request batches "
                   "of 1-4096 jobs, Poisson arrivals; 8 slots, 40 GB traceback budget"}
    # CPU: the reference's functions over a sample of the three pools in the mix's proportions
    sets = serving.JobSets(n_short=7000, n_long=400, n_ll=1000)
    kind = "reference" if O.have_ref() else "port"
    which = "ref" if kind == "reference" else "orc"
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    for p in sets.pools[:2]:
        O.ext_batch(which, p.dual, 5, p.mat, p.q, p.e, p.q2, p.e2, p.jobs, p.qbuf, p.tbuf, threads)
    p = sets.pools[2]
    O.ll_batch(which, p.size, 5, p.mat, p.gapo, p.gape, p.jobs, p.qbuf, p.tbuf, threads)
    dt = time.perf_counter() - t0
    n = sum(len(p) for p in sets.pools)
    line["cpu_baseline"] = {"value": n / dt, "unit": "jobs/s", "cores": threads, "kind": kind,
                            "sample": f"{n} jobs of the mix (7000 extz2, 400 long extd2, 1000 ksw_ll), "
                                      f"{threads} threads, {dt:.2f} s wall"}
    return line


def _timed_run(cmd, cwd, env=None):
    """(completed process, wall s, CPU s of the child: user + system)"""
    import resource
    r0 = resource.getrusage(resource.RUSAGE_CHILDREN)
    t0 = time.perf_counter()
    out = subprocess.run(cmd, cwd=cwd, capture_output=True, env=env)
    dt = time.perf_counter() - t0
    r1 = resource.getrusage(resource.RUSAGE_CHILDREN)
    return out, dt, (r1.ru_utime - r0.ru_utime) + (r1.ru_stime - r0.ru_stime)


def mapper_point(n_pairs=100_000, n_long=16_000):
    """The batched minibwa (minibwa_gb300/mapper) against the stock build of the same reference
    sources on the same simulated reads, all with all host threads: reads mapped per second of
    wall time and the host CPU time each spent, whether their SAM outputs are byte-identical, and
    the batched run's stages.  Pairs (the short-read preset) and long reads (-x lr).  The
    relinked build (the stock sources with libksw2gpu.so in place of the ksw2 objects, every DP
    call one per-call drop-in call) is timed beside them on the first 2,000 pairs and 200 long
    reads, with the stock build on the same subsets: one pair's DP on the device takes about as
    long as hundreds of them on a host core, so the full sets would take minutes."""
    import shutil
    import tempfile
    from minibwa_gb300 import mapper, synth
    from oracle import oracle as O
    tree = O.ref_tree()
    if tree is None:
        return {"unavailable": "the reference's sources are not staged (make -C oracle stage REF=...)"}
    builds = O.build_minibwa(os.path.join(ROOT, "minibwa_gb300"))
    stock, relinked = builds["stock"], builds["gpu"]
    batch = mapper.build(tree)["batch"]
    d = tempfile.mkdtemp(prefix="mapper_point_")
    threads = os.cpu_count() or 1
    runs = {}
    try:
        g = synth.mapper_genome(ctg_len=(6_000_000, 4_000_000, 2_000_000), n_repeats=800)
        synth.write_fasta(os.path.join(d, "g.fa"), g)
        mapper.index(stock, "g.fa", "g", d)
        a, b = synth.mapper_pairs(g, n_pairs)
        synth.write_fasta(os.path.join(d, "p1.fa"), a), synth.write_fasta(os.path.join(d, "p2.fa"), b)
        long_reads = synth.mapper_long_reads(g, n_long)
        synth.write_fasta(os.path.join(d, "long.fa"), long_reads)
        synth.write_fasta(os.path.join(d, "p1s.fa"), a[:2000]), synth.write_fasta(os.path.join(d, "p2s.fa"), b[:2000])
        synth.write_fasta(os.path.join(d, "longs.fa"), long_reads[:200])
        env = dict(os.environ, MBG_TIMING="1")
        for name, args, n, small, n_small in (
                ("pairs", ["g", "p1.fa", "p2.fa"], 2 * n_pairs, ["g", "p1s.fa", "p2s.fa"], 4000),
                ("long_reads", ["-x", "lr", "g", "long.fa"], n_long, ["-x", "lr", "g", "longs.fa"], 200)):
            mapper.map_reads(stock, args, d, threads)  # page in the index and the binary
            so, ts, cs = _timed_run([stock, "map", "-t", str(threads)] + args, d)
            bo, tb, cb = _timed_run([batch, "map", "-t", str(threads)] + args, d, env)
            ro, tr, cr = _timed_run([relinked, "map", "-t", str(threads)] + small, d)
            so2, ts2, cs2 = _timed_run([stock, "map", "-t", str(threads)] + small, d)
            if so.returncode != 0 or bo.returncode != 0 or ro.returncode != 0 or so2.returncode != 0:
                return {"unavailable": "minibwa failed: " +
                        (bo.stderr or ro.stderr or so.stderr).decode(errors="replace")[-300:]}
            runs[name] = {"reads": n, "batched_reads_s": n / tb, "stock_reads_s": n / ts, "batched_wall_s": tb,
                          "stock_wall_s": ts, "batched_cpu_s": cb, "stock_cpu_s": cs,
                          "relinked": {"reads": n_small, "relinked_reads_s": n_small / tr, "relinked_wall_s": tr,
                                       "relinked_cpu_s": cr, "stock_reads_s": n_small / ts2, "stock_wall_s": ts2,
                                       "sam_identical_to_stock": ro.stdout == so2.stdout},
                          "sam_identical_to_stock": bo.stdout == so.stdout and ro.stdout == so2.stdout,
                          "stages": [ln.split("] ", 1)[1] for ln in bo.stderr.decode().splitlines()
                                     if ln.startswith("[M::mbg]")]}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    p = runs["pairs"]
    return {"metric": "reads mapped/s, whole minibwa run (index loaded, SAM written)", "value": p["batched_reads_s"],
            "unit": "reads/s", "sam_identical_to_stock": all(r["sam_identical_to_stock"] for r in runs.values()),
            "workload": f"{n_pairs} simulated 150 nt pairs and {n_long} long reads (1-8 kb, -x lr) from synth on a "
                        f"12 Mb simulated genome with 800 near-repeats, minibwa map -t {threads}; the relinked "
                        f"per-call build on the first 2,000 pairs and 200 long reads",
            "runs": runs,
            "cpu_baseline": {"value": p["stock_reads_s"], "unit": "reads/s", "cores": threads, "kind": "reference",
                             "sample": f"the stock minibwa built from the reference's sources, same pairs, "
                                       f"{threads} threads, {p['stock_wall_s']:.2f} s wall"}}


def main():
    args = parse()
    rank, world = dist_init(args)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload == "rescue":
        run_rescue(args, rank, world)
        return
    import torch
    from minibwa_gb300 import Context
    from minibwa_gb300 import lib as K
    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    K.load_library()
    K.set_ext_family(args.lanes)
    int_peak = K.probe_int32_peak(dev)
    ctx = Context(dev)
    w = Workload(args.workload, args, rank)
    m = measure(args, w, ctx, dev, rank, world, args.steps, args.warmup, int_peak, not args.no_cpu_baseline,
                args.cpu_sample or DEFAULT_SAMPLE[args.workload])
    del w
    extra = {}
    if args.workload == "cfg1" and not args.no_extras and world == 1:
        # the other configurations, measured in the same run with fixed short step counts
        for name in ("cfg2", "cfg3"):
            wx = Workload(name, argparse.Namespace(pairs=None), rank)
            mx = measure(args, wx, ctx, dev, rank, world, 3, 1, int_peak, not args.no_cpu_baseline,
                         DEFAULT_SAMPLE[name])
            mx["metric"] = wx.metric
            mx["config"] = workload_config(name, wx.n, world)
            extra[name] = mx
            del wx
        extra["cfg4"] = serving_point()
        extra["mapper"] = mapper_point()
    if rank == 0:
        line = {
            "metric": Workload(args.workload, args, rank, sizes_only=True).metric, "value": m["value"],
            "unit": m["unit"], "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16" if args.workload == "cfg3" else "int8",
            "data": "synthetic (seeded splitmix64, no public dataset)",
            "config": workload_config(args.workload, sum(Workload(args.workload, args, rank,
                                                                  sizes_only=True).set_sizes), world),
        }
        for k in ("bytes_per_step", "gcups", "cells_per_step", "gpu_launches", "roofline", "roofline_hbm", "e2e",
                  "clocks", "cpu_baseline", "parity_vs_cpu", "autotuned", "tb_budget_gib"):
            if k in m:
                line[k] = m[k]
        if extra:
            line["extra"] = extra
        print(json.dumps(line), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
