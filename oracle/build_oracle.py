"""Build recipe for the CPU oracle (test infrastructure only).

Two things are built here:

* ``oracle/_build/liboracle.so`` -- the all-FP64 C restatement of the
  reference hot path (oracle.c + fft.c), OpenMP-parallel over spindowns.  It is
  the parity reference for the CUDA library and the timed CPU baseline ("port")
  of bench.py.  Built from this repository's sources on any machine.

* ``oracle/_ref/`` -- the UNMODIFIED reference search compiled from its own
  sources where they lie (search/network/src-cpu and src-openmp under the
  reference checkout), linked against the FFTW3/GSL shims in ``oracle/shim``
  because neither library is installed here.  Built only where the reference
  checkout exists; nothing of it is committed (``oracle/_ref`` is
  git-ignored).  Its outputs pin the oracle through the golden fixtures in
  ``tests/golden``.

Flags: ``-ffp-contract=off`` everywhere so that no FMA contraction changes
roundings between x86-64 and aarch64 builds of the oracle; ``-fcommon``
because the reference defines ``ifo[]`` in a header (struct.h:177);
``-DGNUSINCOS`` selects glibc sincos (jobcore.c:528) instead of the
prebuilt vector libraries.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# location of the reference checkout; override with POLGRAW_REFERENCE
REFERENCE_ROOT = os.environ.get("POLGRAW_REFERENCE", "/root/reference")
NETWORK = os.path.join(REFERENCE_ROOT, "search", "network")

ORACLE_LIB = os.path.join(BUILD, "liboracle.so")
REF_SERIAL = os.path.join(REF_OUT, "gwsearch-ref")
REF_OMP = os.path.join(REF_OUT, "gwsearch-ref-omp")

_CC = os.environ.get("CC", "gcc")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("oracle.c", "fft.c", "oracle_coinc.c", "shim/gsl_shim.c")]
    deps = srcs + [os.path.join(HERE, f) for f in ("oracle.h", "fft.h", "shim/gsl/pa_gsl_shim.h")] + [
        os.path.join(HERE, "..", "include", "polgraw_gb300.h")]
    if force or _newer(ORACLE_LIB, deps):
        tmp = ORACLE_LIB + ".tmp%d" % os.getpid()
        _run([_CC, "-std=gnu11", "-O2", "-fPIC", "-shared", "-fopenmp",
              "-ffp-contract=off", "-Wall", "-Wno-unused", "-I" + os.path.join(HERE, "shim"),
              "-o", tmp] + srcs + ["-lm"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


ORACLE_FAST_LIB = os.path.join(BUILD, "liboracle_fast.so")


def build_oracle_fast(force: bool = False) -> str:
    """The same oracle sources with the reference's timing flags
    (search/network/src-openmp/Makefile:13-18: -O3 -funroll-loops
    -ffast-math with OpenMP; its -march=haswell/-mavx2/-mfma are x86 only
    and left out so that the build runs on both host architectures): the
    timed CPU baseline of bench.py, never a parity reference."""
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("oracle.c", "fft.c", "oracle_coinc.c", "shim/gsl_shim.c")]
    deps = srcs + [os.path.join(HERE, f) for f in ("oracle.h", "fft.h", "shim/gsl/pa_gsl_shim.h")] + [
        os.path.join(HERE, "..", "include", "polgraw_gb300.h")]
    if force or _newer(ORACLE_FAST_LIB, deps):
        tmp = ORACLE_FAST_LIB + ".tmp%d" % os.getpid()
        _run([_CC, "-std=gnu11", "-O3", "-funroll-loops", "-ffast-math", "-fPIC", "-shared", "-fopenmp",
              "-Wall", "-Wno-unused", "-I" + os.path.join(HERE, "shim"), "-o", tmp] + srcs + ["-lm"])
        os.replace(tmp, ORACLE_FAST_LIB)
    return ORACLE_FAST_LIB


def reference_available() -> bool:
    return os.path.isdir(os.path.join(NETWORK, "src-cpu"))


def _build_ref_variant(subdir: str, out: str, extra: list[str]) -> str:
    src_dir = os.path.join(NETWORK, subdir)
    names = ["main.c", "jobcore.c", "timer.c", "settings.c", "auxi.c", "init.c"]
    srcs = [os.path.join(src_dir, n) for n in names]
    shims = [os.path.join(HERE, "shim", "fftw_shim.c"), os.path.join(HERE, "shim", "gsl_shim.c"),
             os.path.join(HERE, "fft.c")]
    if not _newer(out, srcs + shims):
        return out
    os.makedirs(REF_OUT, exist_ok=True)
    objdir = os.path.join(REF_OUT, "obj_" + subdir)
    os.makedirs(objdir, exist_ok=True)
    cflags = ["-std=gnu11", "-fcommon", "-DGNUSINCOS", "-DPREFIX=./candidates",
              "-DCODEVER=reference", "-I" + os.path.join(HERE, "shim"), "-w"] + extra
    objs = []
    for s in srcs + shims:
        o = os.path.join(objdir, os.path.basename(s).replace(".c", ".o"))
        inc = ["-I" + src_dir] if s in srcs else ["-I" + os.path.join(HERE, "shim")]
        _run([_CC] + cflags + inc + ["-c", s, "-o", o])
        objs.append(o)
    _run([_CC] + [f for f in extra if f.startswith("-f")] + ["-o", out] + objs + ["-lm", "-lpthread"])
    shutil.rmtree(objdir, ignore_errors=True)
    return out


REF_FOLLOWUP = os.path.join(REF_OUT, "libfollowup_ref.so")


def _build_ref_followup() -> str:
    """The reference followup program's own Fstatnet/evaluate_simplex/amoeba
    (followup/src/followup.c, followup/src/settings.c and the network
    search's auxi.c for lin2ast/ast2lin), unmodified, as a shared library
    driven by oracle/ref_followup_driver.c.  Yeppp! cos/sin come from
    oracle/shim/yeppp_shim.c (the C library's cos and sin)."""
    fu = os.path.join(REFERENCE_ROOT, "followup", "src")
    srcs = [os.path.join(fu, "followup.c"), os.path.join(fu, "settings.c"),
            os.path.join(NETWORK, "src-cpu", "auxi.c")]
    mine = [os.path.join(HERE, "ref_followup_driver.c"), os.path.join(HERE, "shim", "yeppp_shim.c"),
            os.path.join(HERE, "shim", "gsl_shim.c")]
    if not _newer(REF_FOLLOWUP, srcs + mine):
        return REF_FOLLOWUP
    os.makedirs(REF_OUT, exist_ok=True)
    objdir = os.path.join(REF_OUT, "obj_followup")
    os.makedirs(objdir, exist_ok=True)
    inc = ["-I" + os.path.join(HERE, "shim"), "-I" + fu, "-I" + os.path.join(NETWORK, "src-cpu"),
           "-I" + os.path.join(HERE, "..", "include")]
    # parity build: no fast-math; -fno-builtin as for the search build
    cflags = ["-std=gnu11", "-fcommon", "-fPIC", "-O2", "-ffp-contract=off", "-fno-builtin", "-DYEPPP",
              "-Dmain=followup_reference_main", "-w"] + inc
    objs = []
    for k, src in enumerate(srcs + mine):
        o = os.path.join(objdir, "%d_%s" % (k, os.path.basename(src).replace(".c", ".o")))
        _run([_CC] + cflags + ["-c", src, "-o", o])
        objs.append(o)
    _run([_CC, "-shared", "-o", REF_FOLLOWUP] + objs + ["-lm"])
    shutil.rmtree(objdir, ignore_errors=True)
    return REF_FOLLOWUP


REF_COINC = os.path.join(REF_OUT, "coincidences-ref")


def _build_ref_coinc() -> str:
    """The reference coincidence program (coincidences/src/coincidences.c
    with the network search's settings.c, auxi.c and init.c, as its Makefile
    links them), unmodified, against the FFTW/GSL shims (the eigensystem of
    manage_grid_matrix comes from oracle/shim/gsl_shim.c)."""
    co = os.path.join(REFERENCE_ROOT, "coincidences", "src")
    sd = os.path.join(NETWORK, "src-cpu")
    srcs = [os.path.join(co, "coincidences.c")] + [os.path.join(sd, n) for n in ("settings.c", "auxi.c", "init.c")]
    mine = [os.path.join(HERE, "shim", "fftw_shim.c"), os.path.join(HERE, "shim", "gsl_shim.c"),
            os.path.join(HERE, "fft.c")]
    if not _newer(REF_COINC, srcs + mine):
        return REF_COINC
    os.makedirs(REF_OUT, exist_ok=True)
    objdir = os.path.join(REF_OUT, "obj_coinc")
    os.makedirs(objdir, exist_ok=True)
    cflags = ["-std=gnu11", "-fcommon", "-O2", "-ffp-contract=off", "-fno-builtin", "-DGNUSINCOS",
              "-DPREFIX=./coinc-results", "-DDTAPREFIX=./candidates", "-DCODEVER=reference",
              "-I" + os.path.join(HERE, "shim"), "-I" + sd, "-w"]
    objs = []
    for k, src in enumerate(srcs + mine):
        o = os.path.join(objdir, "%d_%s" % (k, os.path.basename(src).replace(".c", ".o")))
        _run([_CC] + cflags + ["-c", src, "-o", o])
        objs.append(o)
    _run([_CC, "-o", REF_COINC] + objs + ["-lm"])
    shutil.rmtree(objdir, ignore_errors=True)
    return REF_COINC


REF_GRIDGEN = os.path.join(REF_OUT, "gridgen")
GRIDGEN_DIR = os.path.join(REFERENCE_ROOT, "gridgen")


def _build_ref_gridgen() -> str:
    """The reference grid generator (gridgen/main.cpp and gridgen/src/*.cpp,
    C++11 and the standard library only), unmodified, with its own Makefile's
    language level and no fast-math."""
    srcs = [os.path.join(GRIDGEN_DIR, "main.cpp")] + sorted(
        os.path.join(GRIDGEN_DIR, "src", f) for f in os.listdir(os.path.join(GRIDGEN_DIR, "src"))
        if f.endswith(".cpp"))
    if not _newer(REF_GRIDGEN, srcs):
        return REF_GRIDGEN
    os.makedirs(REF_OUT, exist_ok=True)
    objdir = os.path.join(REF_OUT, "obj_gridgen")
    os.makedirs(objdir, exist_ok=True)
    objs = []
    for k, src in enumerate(srcs):
        o = os.path.join(objdir, "%d_%s" % (k, os.path.basename(src).replace(".cpp", ".o")))
        _run(["g++", "-std=c++11", "-O2", "-ffp-contract=off", "-w", "-I" + os.path.join(GRIDGEN_DIR, "include"),
              "-c", src, "-o", o])
        objs.append(o)
    _run(["g++", "-o", REF_GRIDGEN] + objs)
    shutil.rmtree(objdir, ignore_errors=True)
    return REF_GRIDGEN


def run_ref_gridgen(ephemeris_dir: str, nfft_exp: int, match: float = 0.75) -> tuple[bytes, str]:
    """Runs the reference grid generator on a directory holding rSSB.bin,
    rDet.bin and DetSSB.bin (-m <match> -p dfg -d <dir>/ -n <nfft_exp>).  It
    reads its covering table dataS2.txt from the working directory, so it
    runs in a scratch directory holding a copy of the reference's table.
    Returns (grid.bin bytes, its standard output)."""
    import tempfile
    exe = _build_ref_gridgen()
    with tempfile.TemporaryDirectory() as tmp:
        shutil.copy(os.path.join(GRIDGEN_DIR, "dataS2.txt"), tmp)
        r = subprocess.run([exe, "-m", repr(match), "-p", "dfg", "-d", ephemeris_dir.rstrip("/") + "/",
                            "-n", str(nfft_exp)], cwd=tmp, capture_output=True, text=True,
                           stdin=subprocess.DEVNULL, timeout=600)
        if r.returncode != 0:
            raise RuntimeError("gridgen failed:\n" + r.stdout + r.stderr)
    with open(os.path.join(ephemeris_dir, "grid.bin"), "rb") as f:
        return f.read(), r.stdout


REF_BINDING = os.path.join(REF_OUT, "gwsearch-ref-gb300")
BINDING_DIR = os.path.join(HERE, "ref_binding")
REPO_INCLUDE = os.path.join(HERE, "..", "include")


def patch_jobcore(src: str) -> str:
    """The reference's search/network/src-cpu/jobcore.c with the GB300
    job_core binding spliced in: ref_binding/file_scope.c after the
    include of timer.h (jobcore.c:18), and ref_binding/call_site.c in place
    of the job_core() call of search() (jobcore.c:107-120)."""
    import re
    with open(os.path.join(BINDING_DIR, "file_scope.c")) as f:
        decls = f.read()
    with open(os.path.join(BINDING_DIR, "call_site.c")) as f:
        call = f.read()
    anchor = '#include "timer.h"\n'
    if src.count(anchor) != 1:
        raise RuntimeError("jobcore.c: include anchor not found once")
    out = src.replace(anchor, anchor + decls, 1)
    pat = re.compile(r"\n[ \t]*status = job_core\(.*?FNum\);[^\n]*\n", re.S)
    m = pat.search(out)
    if not m or "search(" not in out[:m.start()]:
        raise RuntimeError("jobcore.c: the job_core() call of search() not found")
    return out[:m.start()] + "\n" + call + out[m.end():]


def build_ref_binding(lib_dir: str) -> str | None:
    """The reference search program with job_core() swapped for the GB300
    library's pa_job_core() (the maintainer's patch of the reference host):
    a copy of src-cpu/jobcore.c patched by patch_jobcore() under
    oracle/_ref/binding/ (never committed), compiled with the reference's
    other sources against its own headers and the FFTW/GSL shims, and
    linked to libpolgraw_gb300.so in lib_dir.  Returns None where the
    reference checkout is absent."""
    if not reference_available():
        return None
    sd = os.path.join(NETWORK, "src-cpu")
    bdir = os.path.join(REF_OUT, "binding")
    os.makedirs(bdir, exist_ok=True)
    with open(os.path.join(sd, "jobcore.c")) as f:
        patched = patch_jobcore(f.read())
    pj = os.path.join(bdir, "jobcore.c")
    with open(pj, "w") as f:
        f.write(patched)
    srcs = [pj] + [os.path.join(sd, n) for n in ("main.c", "timer.c", "settings.c", "auxi.c", "init.c")]
    shims = [os.path.join(HERE, "shim", "fftw_shim.c"), os.path.join(HERE, "shim", "gsl_shim.c"),
             os.path.join(HERE, "fft.c")]
    cflags = ["-std=gnu11", "-fcommon", "-O2", "-ffp-contract=off", "-fno-builtin", "-DGNUSINCOS",
              "-DPREFIX=./candidates", "-DCODEVER=reference-gb300", "-I" + os.path.join(HERE, "shim"),
              "-I" + sd, "-I" + REPO_INCLUDE]
    objs = []
    for k, src in enumerate(srcs + shims):
        o = os.path.join(bdir, "%d_%s" % (k, os.path.basename(src).replace(".c", ".o")))
        # the patched file compiles with warnings as errors; the reference's own files as they are
        warn = ["-Wall", "-Werror", "-Wno-unused-variable", "-Wno-unused-but-set-variable",
                "-Wno-unused-function", "-Wno-unused-result", "-Wno-maybe-uninitialized",
                "-Wno-format", "-Wno-misleading-indentation", "-Wno-pointer-sign",
                "-Wno-implicit-function-declaration", "-Wno-unused-label",
                "-Wno-stringop-overflow", "-Wno-format-overflow"] if k == 0 else ["-w"]
        _run([_CC] + cflags + warn + ["-c", src, "-o", o])
        objs.append(o)
    _run([_CC, "-o", REF_BINDING] + objs + ["-L" + lib_dir, "-lpolgraw_gb300", "-Wl,-rpath," + lib_dir,
                                             "-lm", "-lpthread"])
    return REF_BINDING


def build_reference() -> dict:
    """Compile the reference search (serial parity build and OpenMP timing
    build).  Returns {} when the reference checkout is absent."""
    if not reference_available():
        return {}
    out = {}
    # parity build: no fast-math, verbose candidate lines, spindown timers.
    # -fno-builtin: add_signal reads "snr"/"amp" into char amporsnr[3]
    # (init.c:475,486), a one-byte overflow after which GCC folds
    # strcmp(amporsnr, "snr") to "different" and the injection is refused;
    # without the builtin the comparison behaves as the authors intended.
    out["serial"] = _build_ref_variant(
        "src-cpu", REF_SERIAL, ["-O2", "-ffp-contract=off", "-fno-builtin", "-DTIMERS=3", "-DVERBOSE"])
    # timing build: the reference's own optimisation flags (src-openmp/Makefile)
    out["omp"] = _build_ref_variant(
        "src-openmp", REF_OMP, ["-O3", "-ffast-math", "-fopenmp", "-fno-builtin", "-DTIMERS=3"])
    out["followup"] = _build_ref_followup()
    out["coinc"] = _build_ref_coinc()
    out["gridgen"] = _build_ref_gridgen()
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_oracle_fast(force="--force" in sys.argv))
    print(build_reference())
