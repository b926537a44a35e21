"""Build recipe of libpolgraw_gb300.so and the gwsearch-gb300,
coincidences-gb300 and gridgen-gb300 programs.

nvcc compiles the CUDA translation units for sm_103a only
(-gencode arch=compute_103a,code=sm_103a); gcc compiles the C host.  Host
code is built with -ffp-contract=off so that the FP64 record fields match
the reference bit for bit on both x86-64 and aarch64.  Translation units are
compiled in parallel; outputs go to polgraw-allsky_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpolgraw_gb300.so")
EXE = os.path.join(BUILD, "gwsearch-gb300")
COINC_EXE = os.path.join(BUILD, "coincidences-gb300")
GRIDGEN_EXE = os.path.join(BUILD, "gridgen-gb300")
INCLUDE = os.path.join(ROOT, "include")

CU_SOURCES = ["csrc/pa_engine_f32.cu", "csrc/pa_engine_f32_f64phase.cu", "csrc/pa_engine_f32_ffphase.cu",
              "csrc/pa_engine_f64.cu", "csrc/pa_api.cu", "csrc/pa_followup.cu", "csrc/pa_coinc.cu"]
C_SOURCES = ["host/pa_host.c", "host/pa_coinc_host.c", "host/pa_grid.c", "host/pa_lattice.c"]
HEADERS = ["csrc/pa_fft.cuh", "csrc/pa_engine.cuh", "csrc/pa_engine.h", "csrc/pa_trace.h"]
NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3", "-std=c++17",
              "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE]
CC_FLAGS = ["-std=gnu11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-result",
            "-I" + INCLUDE]


def _nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    for c in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


TRACE_BUILD = os.path.join(HERE, "_build_trace")
TRACE_LIB = os.path.join(TRACE_BUILD, "libpolgraw_gb300.so")


def build(force: bool = False, verbose: bool = False, trace: bool = False) -> str:
    """Builds the library (and the programs) into _build/.  trace=True builds
    the diagnostic variant with the per-CTA trace compiled in
    (-DPA_CTA_TRACE) into _build_trace/ instead (library only); it is used
    only by the benchmark's --cta-trace measurement."""
    out_dir = TRACE_BUILD if trace else BUILD
    lib_path = TRACE_LIB if trace else LIB
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    nvcc_flags = NVCC_FLAGS + (["-DPA_CTA_TRACE"] if trace else [])
    headers = [os.path.join(HERE, h) for h in HEADERS] + [
        os.path.join(INCLUDE, "polgraw_gb300.h"), os.path.join(INCLUDE, "polgraw_gb300_host.h")]
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src = os.path.join(HERE, s)
        obj = os.path.join(out_dir, os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc] + nvcc_flags + ["-c", src, "-o", obj])
    for s in C_SOURCES:
        src = os.path.join(HERE, s)
        obj = os.path.join(out_dir, os.path.basename(s) + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["gcc"] + CC_FLAGS + ["-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    if force or _stale(lib_path, objs):
        tmp = lib_path + ".tmp%d" % os.getpid()
        _run([nvcc, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", "-o", tmp] + objs + ["-lpthread"])
        os.replace(tmp, lib_path)
    if trace:
        return lib_path
    for exe, main in ((EXE, "gwsearch_gb300.c"), (COINC_EXE, "coincidences_gb300.c"),
                      (GRIDGEN_EXE, "gridgen_gb300.c")):
        main_src = os.path.join(HERE, "host", main)
        if force or _stale(exe, [LIB, main_src]):
            _run(["gcc"] + CC_FLAGS + ["-o", exe, main_src, "-L" + BUILD, "-lpolgraw_gb300",
                                        "-Wl,-rpath,$ORIGIN", "-lm"])
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    import sys
    build(force="--force" in sys.argv, verbose=True)
