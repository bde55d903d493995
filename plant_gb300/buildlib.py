"""Compile the engine: libchl.so (C ABI, CUDA for sm_103a) and the `hhl` CLI.

Each translation unit is compiled by its own nvcc process, in parallel, then
linked.  Objects go to plant_gb300/_build/; the library and the CLI are
written next to this file.  Nothing here imports torch.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libchl.so")
CLI = os.path.join(HERE, "hhl")

SOURCES = [
    "chl_graph.cpp",
    "chl_host.cpp",
    "chl_prims.cu",
    "chl_build.cu",
    "chl_labels.cu",
    "chl_order.cu",
    "chl_server.cu",
    "chl_gnn.cu",
    "chl_labelio.cu",
    "chl_ingest.cu",
    "chl_tune.cpp",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp,-ffp-contract=off",
          "-I" + os.path.join(HERE, "..", "include")]


# extra nvcc flags for diagnostic builds, e.g. CHL_NVCC_FLAGS=-DCHL_PHASE_TIMING=1
EXTRA = os.environ.get("CHL_NVCC_FLAGS", "").split()


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(OUT, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "chl.h"))
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc] + ARCH + COMMON + EXTRA + ["-c", s, "-o", o]
            if src.endswith(".cu") and verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(_run, jobs))
        if verbose:
            for o in outs:
                sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lgomp"])
    cli_src = os.path.join(CSRC, "hhl_main.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB])):
        _run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(HERE, "..", "include"), cli_src,
              "-o", CLI, "-L" + HERE, "-lchl", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
