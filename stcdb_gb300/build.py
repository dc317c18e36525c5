"""Builds the native libraries in-tree (no pip install, no cmake).

  lib/libstctrace.so  host C: seeded synthetic trace generator (the device
                      generator in libstc.so shares its per-object code)
  lib/libstc.so       CUDA sm_103a kernels + C++ host runtime behind the C ABI
                      declared in include/stc.h

Sources compile in parallel; nvcc emits exactly one -gencode target.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
OBJ_DIR = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = [
    "stc_context.cu",
    "stc_partition.cu",
    "stc_refine.cu",
    "stc_meetings.cu",
    "stc_schema.cu",
    "stc_sort.cu",
    "stc_util.cu",
    "stc_lsm.cu",
    "stc_query.cu",
    "stc_tracegen.cu",
    "stc_compact.cu",
    "stc_tune.cu",
    "stc_serve.cu",
]


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("build failed: " + " ".join(cmd))
    if r.stdout.strip():
        sys.stderr.write(r.stdout)


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def build_tracegen() -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    out = os.path.join(LIB_DIR, "libstctrace.so")
    src = os.path.join(CSRC, "tracegen.c")
    deps = [src, os.path.join(CSRC, "tracegen.h"), os.path.join(CSRC, "tracegen_walk.h"),
            os.path.join(INCLUDE, "stc_trace.h"), os.path.join(INCLUDE, "stc.h")]
    if _stale(out, deps):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
              "-I" + INCLUDE, "-I" + CSRC, "-o", out, src, "-lm"])
    return out


def build_cuda(verbose_ptxas: bool = False) -> str:
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    out = os.path.join(LIB_DIR, "libstc.so")
    hdrs = _headers()
    flags = [NVCC, GENCODE, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
             "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE, "-I" + CSRC]
    if verbose_ptxas:
        flags.append("-Xptxas=-v")
    objs = []
    jobs = []
    for s in CU_SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ_DIR, s.replace(".cu", ".o"))
        objs.append(obj)
        if verbose_ptxas or _stale(obj, [src] + hdrs):
            jobs.append(flags + ["-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    if jobs or _stale(out, objs):
        _run([NVCC, GENCODE, "-shared", "-o", out] + objs + ["-lcudart", "-lpthread"])
    return out


def build_all(verbose_ptxas: bool = False) -> None:
    build_tracegen()
    build_cuda(verbose_ptxas=verbose_ptxas)


if __name__ == "__main__":
    build_all(verbose_ptxas="-v" in sys.argv)
