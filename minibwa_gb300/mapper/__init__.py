"""The batched minibwa: the reference's mapper with mb_align1 of every hit of a mini-batch on
the GPU (mbg_map.c, mbg_align.c, the map-main.c substitutions in the Makefile).

build(tree) compiles it from a reference source tree against the in-tree libksw2gpu.so;
map_reads() runs a minibwa binary and returns its SAM output and wall time."""
import os
import subprocess
import time

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")


def build(tree, jobs=None):
    """Compile minibwa_batch and minibwa_batch_km from the reference tree `tree`; returns their paths."""
    subprocess.check_call(["make", "-s", "-C", HERE, f"-j{jobs or os.cpu_count() or 4}", f"REF={tree}",
                           f"GPULIB={PKG}", f"INC={os.path.join(os.path.dirname(PKG), 'include')}", f"OUT={OUT}"])
    return {k: os.path.join(OUT, "minibwa_" + k) for k in ("batch", "batch_km")}


def map_reads(exe, args, cwd, threads=8, env=None):
    """`exe map -t threads args...` in cwd; returns (SAM bytes, seconds)."""
    t0 = time.perf_counter()
    out = subprocess.run([exe, "map", "-t", str(threads)] + list(args), cwd=cwd, capture_output=True, env=env)
    dt = time.perf_counter() - t0
    if out.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} map {' '.join(args)} failed: "
                           + out.stderr.decode(errors="replace")[-2000:])
    return out.stdout, dt


def index(exe, fasta, prefix, cwd, meth=False):
    subprocess.run([exe, "index"] + (["--meth"] if meth else []) + [fasta, prefix], cwd=cwd, check=True,
                   capture_output=True)
