"""Calibration of the timed CPU baseline against the reference's own OpenMP
search (TEST INFRASTRUCTURE).

The benchmark's CPU baseline and reference arm time the oracle (a C
restatement of job_core) on the GPU machine's host cores, because the
reference's sources, and so its build, exist only where the goldens are
made.  This script measures, on one host, the reference's own
search/network/src-openmp build (oracle/_ref/gwsearch-ref-omp: its
Makefile's -O3 -ffast-math with OpenMP, FFTW replaced by the shim over the
oracle's FFT) and the oracle's two builds (the timing build
liboracle_fast.so with the same flags, and the parity build liboracle.so)
on the same sample of the benchmark's network workload (H1+L1, N=86164,
nfft=131072): a 2 x 2 block of sky points x 200 spindowns, all host threads,
best of `repeats`.  The reference's time is its own "Time elapsed" line
(the sky loop of search(), jobcore.c:178-182); the oracle's is the same
loop of job_core() calls.  It writes oracle/cpu_calibration.json, whose
port_over_reference (oracle timing build / reference build, templates/s)
bench.py reports beside the CPU baseline.

Run where the reference checkout exists:  python oracle/calibrate_cpu.py
"""
from __future__ import annotations

import importlib.util
import json
import os
import platform
import re
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
OUT = os.path.join(HERE, "cpu_calibration.json")


def _pkg():
    d = os.path.join(ROOT, "polgraw-allsky_gb300")
    spec = importlib.util.spec_from_file_location("polgraw_gb300", os.path.join(d, "__init__.py"),
                                                  submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules["polgraw_gb300"] = m
    spec.loader.exec_module(m)


def _cpu_model() -> str:
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or "unknown"


def measure(repeats: int = 3, threads: int = 0) -> dict:
    _pkg()
    import build_oracle
    import oracle_setup
    from polgraw_gb300 import synth, workloads
    from pyoracle import Oracle
    exe = build_oracle.build_reference().get("omp")
    if not exe:
        raise SystemExit("reference checkout not found")
    nth = threads or os.cpu_count() or 1
    nspin = 200
    with tempfile.TemporaryDirectory() as tmp:
        argv, _ = workloads.network(tmp, nspin)
        rpath = os.path.join(tmp, "calib_range.txt")
        synth.write_range(rpath, [0, nspin - 1], [0, 1], [0, 1], [1, 1])
        inp = oracle_setup.Inputs(tmp, ident=1, band=666, dt=2.0, nod=2, range_file=rpath)
        s = inp.settings
        bins = s.nmax - s.nmin
        tasks = inp.sky_points()
        templates = len(tasks) * nspin * bins
        env = dict(os.environ, OMP_NUM_THREADS=str(nth))
        ref_t = []
        for _ in range(repeats):
            out = os.path.join(tmp, "out")
            os.makedirs(out, exist_ok=True)
            r = subprocess.run(["bash", "-c", 'ulimit -s unlimited; exec "$0" "$@"', exe, "-data", tmp, "-ident", "1",
                                "-band", "666", "-dt", "2", "-nod", "2", "-range", rpath, "-output", out,
                                "--nocheckpoint"], cwd=tmp, env=env, capture_output=True, text=True, timeout=3600)
            if r.returncode != 0:
                raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
            m = re.search(r"Time elapsed: ([-+.eE\d]+) s", r.stdout)
            ref_t.append(float(m.group(1)))
        res = {}
        for name, fast in (("port_timing_build", True), ("port_parity_build", False)):
            ts = []
            for _ in range(repeats):
                dets, nifo = inp.detectors()
                orc = Oracle(s, dets, nifo, nthreads=nth, fast=fast)
                opts, rng = inp.opts(), inp.range
                t0 = time.perf_counter()
                for pm, mm, nn in tasks:
                    rng.sst = rng.spndr[0]
                    orc.job_core(pm, mm, nn, opts, rng)
                ts.append(time.perf_counter() - t0)
                orc.close()
            res[name] = {"templates_s": templates / min(ts), "seconds": min(ts)}
    ref = {"templates_s": templates / min(ref_t), "seconds": min(ref_t),
           "build": "search/network/src-openmp, -O3 -ffast-math -fopenmp (its Makefile without the x86 "
                    "-march flags), FFTW shim over the oracle FFT"}
    return {"host": platform.machine(), "cpu": _cpu_model(), "threads": nth,
            "sample": "network workload (H1+L1, N=86164, nfft=131072): %d sky points x %d spindowns x %d bins, "
                      "best of %d" % (len(tasks), nspin, bins, repeats),
            "reference_omp": ref, **res,
            "port_over_reference": res["port_timing_build"]["templates_s"] / ref["templates_s"]}


if __name__ == "__main__":
    d = measure()
    with open(OUT, "w") as f:
        json.dump(d, f, indent=1)
    print(json.dumps(d, indent=1))
