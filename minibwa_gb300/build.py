"""Build recipe for the native parts of minibwa_gb300 (in-tree, no cmake).

    python -m minibwa_gb300.build            # libksw2gpu.so + libksw2synth.so

libksw2gpu.so   CUDA kernels for sm_103a + the C ABI (include/ksw2.h, include/ksw2_gb300.h)
libksw2synth.so host-only synthetic workload generator (gcc)
libksw2loadgen.so open-loop load generator of the serving benchmark (g++, links libksw2gpu.so)

Objects go to minibwa_gb300/_build/; the translation units compile in parallel.
"""
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB_GPU = os.path.join(PKG, "libksw2gpu.so")
LIB_SYNTH = os.path.join(PKG, "libksw2synth.so")
LIB_LOADGEN = os.path.join(PKG, "libksw2loadgen.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(os.path.dirname(PKG), "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    units = [
        ("ext_kernels.cu", "ext_z2.o", ["-DKSW2G_EXT_VAR=0"]),
        ("ext_kernels.cu", "ext_d2.o", ["-DKSW2G_EXT_VAR=1"]),
        ("ext16_kernels.cu", "ext16_z2.o", ["-DKSW2G_EXT_VAR=0"]),
        ("ext16_kernels.cu", "ext16_d2.o", ["-DKSW2G_EXT_VAR=1"]),
        ("ll_kernels.cu", "ll.o", []),
        ("capi.cu", "capi.o", []),
        ("probe.cu", "probe.o", []),
        ("noalloc.cu", "noalloc.o", []),
        ("server.cu", "server.o", []),
        ("graph.cu", "graph.o", []),
        ("ref.cu", "ref.o", []),
        ("rescue.cu", "rescue.o", []),
        ("align_pairs.cu", "align_pairs.o", []),
        ("align_chains.cu", "align_chains.o", []),
    ]
    hdrs = _headers()
    procs, objs = [], []
    for src, obj, extra in units:
        s, o = os.path.join(CSRC, src), os.path.join(BUILD, obj)
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", s, "-o", o]
            if verbose:
                print(" ".join(cmd), flush=True)
            procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or _stale(LIB_GPU, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB_GPU] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    src = os.path.join(CSRC, "synth.c")
    if force or _stale(LIB_SYNTH, [src]):
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-o", LIB_SYNTH, src, "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    src = os.path.join(CSRC, "loadgen.cc")
    if force or _stale(LIB_LOADGEN, [src, LIB_GPU] + hdrs):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-o", LIB_LOADGEN, src, "-L" + PKG, "-lksw2gpu",
               "-Wl,-rpath,$ORIGIN", "-lpthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.check_call(cmd)
    return LIB_GPU


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)
