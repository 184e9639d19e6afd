"""Builds libhbx.so and run_hyperblocker_exec in-tree for sm_103a.

CUDA sources compile with nvcc for ``-gencode arch=compute_103a,code=sm_103a``
only; host sources with g++ (C++17, -ffp-contract=off so host arithmetic is
the same on x86-64 and aarch64).  Translation units compile in parallel; the
outputs go to ``hyperblocker_gb300/_build`` (git-ignored).

    python -m hyperblocker_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libhbx.so")
PROBE_LIB = os.path.join(OUT, "libhbx_probe.so")  # measurement probes (bench.py only)
EXE = os.path.join(OUT, "run_hyperblocker_exec")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

CU_SOURCES = ["kernels.cu", "engine.cu", "ingest.cu", "serve.cu", "stream.cu", "static_scratch.cu",
              "writer.cu", "csv_gpu.cu", "sort.cu"]
CPP_SOURCES = ["csv.cpp", "rules.cpp", "planner.cpp", "encode.cpp", "capi.cpp", "cli.cpp"]
PROBE_SOURCES = ["probe.cu"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _needs(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(HERE, "..", "include", "hbx.h"))
    return hs


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stderr


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    objs = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + hdrs):
            jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "--expt-relaxed-constexpr",
                         "-c", src, "-o", obj])
    probe_objs = []
    for f in PROBE_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        probe_objs.append(obj)
        if force or _needs(obj, [src] + hdrs):
            jobs.append([nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xptxas", "-v" if verbose else "-O3", "-c", src, "-o", obj])
    for f in CPP_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-Wno-unused-function", "-I", "/usr/local/cuda/include",
                         "-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            for err in ex.map(_compile, jobs):
                if verbose and err:
                    sys.stderr.write(err)
    if force or jobs or _needs(LIB, objs):
        _compile([nvcc, ARCH, "-shared", "-o", LIB + ".tmp"] + objs +
                 ["-lpthread", "-ldl", "-lrt"])
        os.replace(LIB + ".tmp", LIB)
    if force or _needs(PROBE_LIB, probe_objs):
        _compile([nvcc, ARCH, "-shared", "-o", PROBE_LIB + ".tmp"] + probe_objs)
        os.replace(PROBE_LIB + ".tmp", PROBE_LIB)
    exe_src = os.path.join(CSRC, "run_hyperblocker_exec.cpp")
    if force or _needs(EXE, [LIB, exe_src]):
        _compile(["g++", "-std=c++17", "-O2", exe_src, "-o", EXE + ".tmp", "-L", OUT, "-lhbx",
                  "-Wl,-rpath,$ORIGIN"])
        os.replace(EXE + ".tmp", EXE)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
