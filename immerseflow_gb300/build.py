"""Build the CUDA library (libimmerseflow_gb300.so) and the CLI in-tree.

One -gencode for sm_103a, translation units compiled in parallel.  The
immersed-boundary files (set-up, and the per-step geometry of moving bodies)
are compiled with -fmad=false so that tagging, image-point weights and the
body pose are reproducible bit for bit on the CPU.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libimmerseflow_gb300.so")
CLI = os.path.join(HERE, "bin", "immerseflow_gb300")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall",
          "-I" + os.path.join(HERE, "..", "include")]

SOURCES = [
    ("kernels_method.cu", []),
    ("kernels_persist.cu", []),
    ("kernels_cluster.cu", []),
    ("kernels_ibm.cu", ["-fmad=false"]),
    ("kernels_move.cu", ["-fmad=false"]),
    ("kernels_ref.cu", []),
    ("solver.cu", []),
    ("io.cpp", ["-x", "cu"]),
    ("noalloc.cu", []),
    ("server.cpp", ["-x", "cu"]),
    ("state_io.cpp", ["-x", "cu"]),
]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, ptxas_info=False):
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(os.path.dirname(CLI), exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "immerseflow_gb300.h"))
    jobs = []
    objs = []
    for src, extra in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if _stale(o, [s] + headers) or ptxas_info:
            cmd = [NVCC] + GENCODE + COMMON + extra + ["-c", s, "-o", o]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if _stale(LIB, objs):
        _run([NVCC] + GENCODE + ["-shared", "-o", LIB] + objs + ["-cudart", "static"])
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and _stale(CLI, [cli_src, LIB]):
        _run([NVCC] + GENCODE + ["-O2", "-std=c++17", "-x", "cu", cli_src, "-o", CLI,
                                 "-I" + os.path.join(HERE, "..", "include"),
                                 "-L" + HERE, "-limmerseflow_gb300",
                                 "-Xlinker", "-rpath,$ORIGIN/.."])
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print("built", LIB)
