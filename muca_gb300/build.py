"""Build the GB300 engine in-tree: muca_gb300/_build/libmuca.so and the
drop-in executables muca_gb300/_build/{multigpu_weight,produce_gpu}.

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, without fast-math
(the sweep kernels call the IEEE logf and need exactly rounded FP32/FP64).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
CLI = os.path.join(HERE, "cli")
OUT = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "-I", INCLUDE,
                     "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
CU_SOURCES = ["k_sweep.cu", "k_sweep_random.cu", "k_lattice.cu", "k_weights.cu", "k_observables.cu", "k_bench.cu", "k_batch.cu",
              "k_mlp.cu", "muca_api.cu", "muca_batch.cu", "muca_mlp.cu"]
CLI_SOURCES = {"multigpu_weight": "multigpu_weight.cpp", "produce_gpu": "produce_gpu.cpp"}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nv = nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "muca.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src.replace(".cu", ".o"))
        objs.append(o)
        if ptxas_info or _stale(o, [s] + headers):
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nv] + NVCC_FLAGS + extra + ["-c", s, "-o", o])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        for out in ex.map(_run, jobs):
            logs.append(out)
    lib = os.path.join(OUT, "libmuca.so")
    if jobs or not os.path.exists(lib):
        _run([nv] + ARCH + ["-shared", "-o", lib] + objs)
    # drop-in executables (host C++ over the C ABI)
    for exe, src in CLI_SOURCES.items():
        s = os.path.join(CLI, src)
        if not os.path.exists(s):
            continue
        t = os.path.join(OUT, exe)
        if _stale(t, [s, lib, os.path.join(INCLUDE, "muca.h"), os.path.join(CLI, "cli_common.h")]
                  if os.path.exists(os.path.join(CLI, "cli_common.h")) else [s, lib]):
            _run(["g++", "-O2", "-std=c++17", "-I", INCLUDE, "-o", t, s, "-L", OUT, "-lmuca",
                  "-Wl,-rpath,$ORIGIN"])
    if verbose:
        sys.stdout.write("".join(logs))
    return lib


if __name__ == "__main__":
    build(verbose=True, ptxas_info="-v" in sys.argv)
