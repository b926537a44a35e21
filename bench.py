"""Benchmark of the coherent-search hot path (job_core) on one GB300.

Workload (the H1+L1 network configuration): two detectors, N = 86164
samples at dt = 2 s (2 sidereal days), nfft = 131072, fftpad = 1,
interpftpad = 2, Gaussian-like noise sigma 1.0 (H1) and 1.3 (L1), five
injected signals (SNR 8-15, seed 2002), ~2000 sky points on the lattice of
one hemisphere x 200 spindowns.  Inputs are synthetic (deterministic
generator polgraw_gb300.synth); no dataset is read.

A step is one pass of the search over the sky points (pa_search_batch via
the C-ABI).  `value` = templates (sky x spindown x frequency bin) per second
with the inputs resident in HBM, timed with CUDA events on the context's
stream; `e2e` = the same metric through the C-ABI with host buffers, the
host->device upload of the data and the device->host candidates inside the
timed region.  The L2 is flushed (256 MB write) before every timed step.
"""
from __future__ import annotations

import argparse
import hashlib
import ctypes as C
import importlib.util
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))


def load_package():
    name = "polgraw_gb300"
    if name in sys.modules:
        return sys.modules[name]
    d = os.path.join(ROOT, "polgraw-allsky_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(d, "__init__.py"),
                                                  submodule_search_locations=[d])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()
from polgraw_gb300 import workloads  # noqa: E402

METRIC = "templates/sec (sky x spindown x bin) mixed vs all-FP64 on GB300 at 1e-4 F-stat err"
UNIT = "templates/s"
WORKLOAD = "network H1+L1, N=86164 dt=2s, nfft=131072, 2000 sky x 200 spindowns, 5 injections"
NSKY_DEFAULT = 2000
NSPIN_DEFAULT = 200


def make_workload(root: str, nspin: int, npoints: int = NSKY_DEFAULT):
    """Writes the data set and returns the search command line."""
    return workloads.network(root, nspin, npoints)[0]


def sky_tasks(host, limit: int):
    s = host.settings
    out = []
    for (pm, mm, nn) in host.sky_points():
        al1 = nn * s.M[10] + mm * s.M[14]
        al2 = nn * s.M[11] + mm * s.M[15]
        if (al1 * al1 + al2 * al2) / (s.oms * s.oms) <= 1.0:
            out.append((pm, mm, nn))
    return out[:limit]


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, reasons)."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.p = None
        self.path = tempfile.mktemp(suffix=".csv")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def l2_flush():
    import torch
    buf = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
    buf.zero_()
    torch.cuda.synchronize()
    del buf


# DRAM bytes (read + write) per spindown of the spindown pass A (H1+L1,
# N=86164, nfftf=131072) from an ncu capture of the current kernel, per
# schedule (spindowns per launch, FFT split); scaled by the spindowns of a
# launch.  Schedules without a capture of the current kernel report null.
PASS_A_TRAFFIC_PER_SPINDOWN = {(32, 1): 14.21e6 / 32}


def peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def cpu_calibration() -> dict | None:
    """The committed same-host calibration of the oracle's timing build
    against the reference's own OpenMP search build (oracle/calibrate_cpu.py):
    port_over_reference > 1 means the timed port is faster than the
    reference build, i.e. the baseline is not understated."""
    p = os.path.join(ROOT, "oracle", "cpu_calibration.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return {"port_over_reference": d["port_over_reference"], "host": "%s, %s" % (d["host"], d["cpu"]),
            "threads": d["threads"], "reference_templates_s": d["reference_omp"]["templates_s"],
            "port_templates_s": d["port_timing_build"]["templates_s"], "sample": d["sample"],
            "reference_build": d["reference_omp"]["build"]}


def cpu_baseline(host, tasks, nsky_sample: int, nthreads: int, keep=None, fast: bool = True):
    """The CPU oracle (all-FP64 C restatement, OpenMP over spindowns; by
    default its build with the reference's timing flags) on a bounded sample
    of the same sky points: templates/s.  `host` is the oracle-side input
    set-up (oracle_setup.Inputs) or the product host (same interface).  With
    `keep`, the oracle's candidates are appended to it as
    {(pm,mm,nn,ss,ii): F}."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import Oracle
    dets, nifo = host.detectors()
    orc = Oracle(host.settings, dets, nifo, nthreads=nthreads, fast=fast)
    opts, rng = host.opts(), host.range
    s = host.settings
    bins = s.nmax - s.nmin
    nspin = rng.spndr[1] - rng.spndr[0] + 1
    sample = tasks[:nsky_sample]
    t0 = time.perf_counter()
    for (pm, mm, nn) in sample:
        rng.sst = rng.spndr[0]
        o = orc.job_core(pm, mm, nn, opts, rng)
        if keep is not None:
            for x, r in zip(o["idx"], o["records"]):
                keep[tuple(int(x[f]) for f in ("pm", "mm", "nn", "ss", "ii"))] = r[4] * r[4] / 2 + 2
    dt = time.perf_counter() - t0
    orc.close()
    return len(sample) * nspin * bins / dt, dt, len(sample)


def run_stress(args, L):
    """Precision-stress workload (H1+L1, N=258492, nfftf=524288, fdot in
    [-1e-7, 1e-7)): templates/s of every precision form and the relative
    F-statistic error of each form on every candidate the all-FP64 CPU oracle
    finds at the sky points of the three injections (400 spindowns each)."""
    tmp = tempfile.mkdtemp(prefix="pa_stress_")
    argv, inj = workloads.stress(tmp, 400)
    host = L.Host(argv)
    s = host.settings
    dets, nifo = host.detectors()
    opts, rng = host.opts(), host.range
    bins = s.nmax - s.nmin
    nspin = rng.spndr[1] - rng.spndr[0] + 1
    tasks = sky_tasks(host, args.sky if args.sky != NSKY_DEFAULT else 500)
    inj_sky = [workloads.nearest_sky(host, j) for j in inj]
    forms = [("mixed-fixed", L.PA_PREC_MIXED, L.PA_PHASE_FIXED), ("mixed-f64phase", L.PA_PREC_MIXED, L.PA_PHASE_F64),
             ("mixed-ffphase", L.PA_PREC_MIXED, L.PA_PHASE_FF), ("fp64", L.PA_PREC_FP64, L.PA_PHASE_F64)]
    res, cands = {}, {}
    for name, prec, ph in forms:
        ctx = L.Context(s, dets, nifo, precision=prec, phase_mode=ph, device=0)
        sub = tasks if prec == L.PA_PREC_MIXED else tasks[:args.fp64_sky // 3]
        for _ in range(max(1, args.warmup)):
            ctx.search_batch(sub[:4], opts, rng)
        ms = 0.0
        for _ in range(args.steps):
            l2_flush()
            ctx.search_batch(sub, opts, rng)
            ms += ctx.last_call_ms()
        res[name] = {"value": len(sub) * nspin * bins * args.steps / (ms / 1e3), "sky_points": len(sub)}
        rec, idx, _ = ctx.search_batch(inj_sky, opts, rng)
        # F from the records' SNR (FP64), as the oracle's
        cands[name] = {tuple(int(x[f]) for f in ("pm", "mm", "nn", "ss", "ii")): float(r[4] * r[4] / 2 + 2)
                       for x, r in zip(idx, rec)}
        ctx.close()
    keep = {}
    t_cpu = time.perf_counter()
    # the checker: the oracle's parity build (the timing build's -ffast-math
    # moves F by up to ~2e-3 on some of these sky points)
    cpu_baseline(host, inj_sky, len(inj_sky), os.cpu_count() or 1, keep=keep, fast=False)
    t_cpu = time.perf_counter() - t_cpu
    per = []
    for k in sorted(keep):
        row = {"key": list(k), "F_oracle": keep[k]}
        for name in cands:
            row[name] = abs(cands[name][k] - keep[k]) / keep[k] if k in cands[name] else None
        per.append(row)
    summary = {}
    for name in cands:
        e = [r[name] for r in per if r[name] is not None]
        summary[name] = {"templates_per_s": res[name]["value"], "sky_points_timed": res[name]["sky_points"],
                         "rel_err_max": max(e) if e else None, "rel_err_median": statistics.median(e) if e else None,
                         "candidates_matched": len(e), "candidates_missing": sum(r[name] is None for r in per)}
    line = {"metric": "templates/sec per precision form and relative F-stat error vs the all-FP64 oracle",
            "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
            "config": {"workload": "precision stress H1+L1, N=258492 dt=2s, nfft=262144, fftpad=2 (nfftf=524288), "
                                   "%d sky x %d spindowns, fdot in [-1e-7,1e-7), 3 injections" % (len(tasks), nspin),
                       "l2": "flushed (256 MB write) before each timed step"},
            "forms": summary, "oracle_sample": "%d injection sky points x %d spindowns (%.1f s, parity build)" %
                                              (len(inj_sky), nspin, t_cpu),
            "per_candidate": per}
    emit(line)


def run_followup(args, L):
    """Followup workload (H1+L1+V1, N=86164, 4096 candidates offset by up to
    half a peak width from 4 injections): demodulated F-statistic and
    adjoint-gradient throughput in both forms, gradient ascent of all
    candidates, the batched reference simplex on the GPU, and the reference
    simplex (the pinned CPU oracle) on a bounded sample."""
    tmp = tempfile.mkdtemp(prefix="pa_followup_")
    argv, inj = workloads.followup(tmp)
    host = L.Host(argv)
    s = host.settings
    dets, nifo = host.detectors()
    ncand = args.candidates
    pts, ws, which = workloads.candidates_around(host, inj, ncand)
    scale = np.median(ws, axis=0)
    res = {}
    for name, prec, ph in (("mixed", L.PA_PREC_MIXED, L.PA_PHASE_F64),
                           ("mixed_ffphase", L.PA_PREC_MIXED, L.PA_PHASE_FF),
                           ("fp64", L.PA_PREC_FP64, L.PA_PHASE_F64)):
        fu = L.Followup(s, dets, nifo, precision=prec, phase_mode=ph)
        for _ in range(max(1, args.warmup)):
            fu.fstatnet(pts)
        ms = 0.0
        for _ in range(args.steps):
            l2_flush()
            fu.fstatnet(pts)
            ms += fu.last_call_ms()
        gms = 0.0
        for _ in range(args.steps):
            l2_flush()
            F, g = fu.fstatnet_grad(pts)
            gms += fu.last_call_ms()
        res[name] = {"fstat_evals_per_s": ncand * args.steps / (ms / 1e3),
                     "grad_evals_per_s": ncand * args.steps / (gms / 1e3),
                     "ms_per_batch": ms / args.steps, "grad_ms_per_batch": gms / args.steps,
                     "F": F, "grad": g}
        fu.close()
    # mixed-form gradient against the FP64 form, in peak-width units
    gm, g64, gff = res["mixed"].pop("grad"), res["fp64"].pop("grad"), res["mixed_ffphase"].pop("grad")
    Fm, F64, Fff = res["mixed"].pop("F"), res["fp64"].pop("F"), res["mixed_ffphase"].pop("F")
    gscale = np.abs(scale * g64).max(axis=1)
    grad_err = float((np.abs(scale * (gm - g64)).max(axis=1) / gscale).max())
    F_err = float((np.abs(Fm - F64) / F64).max())
    res["mixed_ffphase"]["F_rel_err_max_vs_fp64"] = float((np.abs(Fff - F64) / F64).max())
    res["mixed_ffphase"]["grad_rel_err_max_vs_fp64"] = float((np.abs(scale * (gff - g64)).max(axis=1) / gscale).max())
    fu = L.Followup(s, dets, nifo, precision=L.PA_PREC_MIXED)
    launches0 = fu.launches()
    t0 = time.perf_counter()
    p_asc, o_asc, it = fu.ascent(pts, scale, step0=0.25, min_step=1e-3, max_iter=100)
    t_asc = time.perf_counter() - t0
    asc_launches = fu.launches() - launches0
    F0 = -fu.fstatnet(pts)[:, 5]
    t0 = time.perf_counter()
    p_sx, o_sx, nev = fu.simplex(pts, 0.5 * scale, tol=1e-7, max_evals=2000)
    t_sx = time.perf_counter() - t0
    # the reference followup's flow with the ascent in place of the simplex:
    # a 3^4 grid of offsets (-1/3, 0, 1/3 peak widths) around every start,
    # evaluated in one batch, then the ascent from each candidate's best
    # grid point
    offs = np.array(np.meshgrid(*[[-1. / 3, 0., 1. / 3]] * 4, indexing="ij")).reshape(4, -1).T
    t0 = time.perf_counter()
    grid = (pts[:, None, :] + offs[None, :, :] * scale[None, None, :]).reshape(-1, 4)
    Fg = -fu.fstatnet(grid)[:, 5].reshape(ncand, len(offs))
    best = grid.reshape(ncand, len(offs), 4)[np.arange(ncand), Fg.argmax(axis=1)]
    p_ga, o_ga, it_ga = fu.ascent(best, scale, step0=0.25, min_step=1e-3, max_iter=100)
    t_ga = time.perf_counter() - t0
    F_asc, F_sx, F_ga = -o_asc[:, 5], -o_sx[:, 5], -o_ga[:, 5]
    peak = np.array([max(F_asc[which == j].max(), F_sx[which == j].max(), F_ga[which == j].max())
                     for j in range(len(inj))])
    reach = lambda Fv: float(np.mean(Fv >= (1 - 1e-3) * peak[which]))  # noqa: E731
    # the reference simplex on the CPU: the pinned oracle restatement of
    # followup.c amoeba, one core, on a bounded sample
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from pyoracle import FollowupOracle
    ora = FollowupOracle(s, dets, nifo, nthreads=1)
    ncpu = min(args.cpu_candidates, ncand)
    t0 = time.perf_counter()
    cpu_nev = 0
    for k in range(ncpu):
        _, _, ne = ora.amoeba(pts[k], 0.5 * scale, 1e-7, 2000)
        cpu_nev += ne
    t_cpu = time.perf_counter() - t0
    ora.close()
    value = ncand / t_asc
    line = {"metric": "followup candidates refined per second (gradient ascent, FP32 F-stat + FP64-phase adjoint)",
            "value": value, "unit": "candidates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "f32+f64phase", "data": "synthetic",
            "config": {"workload": "followup H1+L1+V1, N=86164 dt=2s, %d candidates offset by U(-0.5,0.5) peak "
                                   "widths from 4 injections (seed 2005)" % ncand,
                       "scale": scale.tolist(), "l2": "flushed (256 MB write) before each timed batch"},
            "forms": res, "mixed_vs_fp64": {"F_rel_err_max": F_err, "grad_rel_err_max_width_units": grad_err},
            "ascent": {"seconds": t_asc, "iters_mean": float(it.mean()), "F_gain_median": float(np.median(F_asc / F0)),
                       "reach_peak_frac": reach(F_asc), "gpu_launches": int(asc_launches)},
            "simplex_gpu": {"seconds": t_sx, "candidates_per_s": ncand / t_sx, "evals_mean": float(nev.mean()),
                            "reach_peak_frac": reach(F_sx)},
            "grid_then_ascent": {"seconds": t_ga, "candidates_per_s": ncand / t_ga, "grid_points": len(offs),
                                 "iters_mean": float(it_ga.mean()), "reach_peak_frac": reach(F_ga)},
            "cpu_baseline": {"value": ncpu / t_cpu, "unit": "candidates/s", "cores": 1, "kind": "port",
                             "sample": "reference simplex (oracle restatement of followup.c amoeba, pinned to it) "
                                       "on %d candidates, %d evaluations, %.1f s" % (ncpu, cpu_nev, t_cpu)}}
    fu.close()
    emit(line)


def run_segments(args, L):
    """Multi-segment workload: segments of uneven N (uniform in [60000,
    260000], seed 2004), H1+L1, fftpad=2, 300 sky x 150 spindowns each.
    Timed three ways on the same contexts: one segment after another
    (pa_search_batch each, default schedule); all segments at once on their
    own streams (pa_segments_search, default schedule, no graph); and all
    at once as one CUDA graph after pa_autotune of every segment."""
    segs = workloads.segments(args.segments, nsky=300, nspin=150)
    ctxs = [L.Context(g["settings"], g["dets"], 2, precision=L.PA_PREC_MIXED, phase_mode=L.PA_PHASE_FIXED)
            for g in segs]
    nspin = 150
    templates = sum(len(g["tasks"]) * nspin * (g["settings"].nmax - g["settings"].nmin) for g in segs)
    tl = [g["tasks"] for g in segs]
    ol = [g["opts"] for g in segs]
    rl = [g["range"] for g in segs]

    def serial():
        ms = 0.0
        for c, g in zip(ctxs, segs):
            c.search_batch(g["tasks"], g["opts"], g["range"])
            ms += c.last_call_ms()
        return ms

    for _ in range(args.warmup):
        serial()
    t_serial = 0.0
    for _ in range(args.steps):
        l2_flush()
        t_serial += serial()
    seg = L.Segments(ctxs, graph=False)
    for _ in range(args.warmup):
        seg.search(tl, ol, rl)
    t_fixed = 0.0
    for _ in range(args.steps):
        l2_flush()
        res_fixed = seg.search(tl, ol, rl)
        t_fixed += seg.last_call_ms()
    t0 = time.perf_counter()
    sched = [c.autotune(g["tasks"][:4], g["opts"], g["range"]) + (c.lanes(),) for c, g in zip(ctxs, segs)]
    t_tune = time.perf_counter() - t0
    seg.set_graph(True)
    for _ in range(args.warmup):
        seg.search(tl, ol, rl)
    launches0 = sum(c.launches() for c in ctxs)
    clocks = ClockSampler(0)
    t_tuned = 0.0
    for _ in range(args.steps):
        l2_flush()
        res_tuned = seg.search(tl, ol, rl)
        t_tuned += seg.last_call_ms()
    clk = clocks.stop()
    launches = (sum(c.launches() for c in ctxs) - launches0) // max(1, args.steps)
    # the schedules may differ in FFT rounding only: same candidate indices
    same = all(sorted(map(tuple, r1[1][["pm", "mm", "nn", "ss", "ii"]].tolist())) ==
               sorted(map(tuple, r2[1][["pm", "mm", "nn", "ss", "ii"]].tolist()))
               for r1, r2 in zip(res_fixed, res_tuned))
    value = templates * args.steps / (t_tuned / 1e3)
    Ns = [g["N"] for g in segs]
    line = {"metric": "templates/sec (sky x spindown x bin), multi-segment batch",
            "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_tuned / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64phase", "data": "synthetic",
            "config": {"workload": "%d segments, N uniform in [60000, 260000] (seed 2004), dt=2s, H1+L1, fftpad=2, "
                                   "300 sky x 150 spindowns per segment" % len(segs),
                       "N_min": min(Ns), "N_max": max(Ns), "nfftf": sorted({g["settings"].nfftf for g in segs}),
                       "l2": "flushed (256 MB write) before each timed step"},
            "clocks": clk, "gpu_launches": int(launches),
            "serial_templates_per_s": templates * args.steps / (t_serial / 1e3),
            "fixed_schedule_templates_per_s": templates * args.steps / (t_fixed / 1e3),
            "tuned_graph_templates_per_s": value,
            "autotune": {"seconds": t_tune, "schedules": [list(x) for x in sched]},
            "candidates_identical_fixed_vs_tuned": bool(same)}
    seg.close()
    emit(line)


def run_coinc(args, L):
    """Coincidence workload (consumer of the trigger files): 24 frames x
    2^20 trigger records (25.2 M records, 1.0 GB), N=86164 band 666, 64
    frequency lines x 256 sky positions, 1000 signals, mincoin 4.  A step is
    one pa_coinc_run over the resident records (cells, per-frame duplicate
    removal, coincidences, records); `e2e` adds the upload of every frame
    from pinned host memory and the read-back of the coincidence records."""
    import torch
    w = workloads.coincidences(args.coinc_frames, args.coinc_records)
    cfg = L.coinc_cfg(N=w["N"], oms=w["oms"], vedva_m=L.vedva(w["fisher"]), refr=w["refr"], mincoin=w["mincoin"])
    frames = w["frames"]
    # pinned host copies of the trigger records
    pinned = {}
    for f in frames:
        t = torch.empty((len(w["recs"][f]), 5), dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = w["recs"][f]
        pinned[f] = t.numpy()
    nrec = sum(len(v) for v in w["recs"].values())
    cc = L.Coinc(cfg)
    for f in frames:
        cc.add_frame(f, pinned[f])
    for _ in range(args.warmup):
        cc.run()
    l0 = cc.launches()
    clocks = ClockSampler(0)
    ms = 0.0
    for _ in range(args.steps):
        l2_flush()
        res = cc.run()
        ms += cc.last_call_ms()
    clk = clocks.stop()
    launches = (cc.launches() - l0) // max(1, args.steps)
    value = nrec * args.steps / (ms / 1e3)
    # per-kernel CUDA-event profile of separate runs (not the timed number)
    cc.set_profiling(True)
    for _ in range(args.steps):
        l2_flush()
        cc.run()
    prof = cc.profile()
    cc.set_profiling(False)
    # dominant kernel: the cells of every record (reads the 40-byte record,
    # writes 16 bytes of cells and a 1-byte flag)
    pk = peaks()
    cells_ms, cells_n = prof["coinc_cells"]
    per_launch = cells_ms / max(1, cells_n)
    achieved = 57.0 * nrec / (per_launch / 1e3) / 1e9
    tot = sum(v[0] for v in prof.values())
    roof = {"bound": "hbm", "kernel": "coinc_cells", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": achieved / pk["hbm_gbs"], "traffic": None,
            "note": "57 B per record; the kernel is bound by the FP64 pipe (frequency and spindown terms and "
                    "the rounding test in FP64, sky terms in FP32 with an FP64 recomputation near cell edges), "
                    "not by HBM",
            "peak_source": pk["source"] + " (MEASURED_PEAKS.json hbm_gbs)", "avg_launch_ms": per_launch,
            "units_per_launch": nrec}
    # end to end: upload, run, results back
    t_e2e = 0.0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        cc.reset()
        for f in frames:
            cc.add_frame(f, pinned[f])
        res = cc.run()
        t_e2e += time.perf_counter() - t0
    s = res.summary
    d2h = int(s.ncoin) * 48 + int(s.nmembers) * 8 + 12 * len(frames)
    # the CPU oracle on a bounded sample (the first records of every frame),
    # and the device on the same sample
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    sub = {f: np.ascontiguousarray(w["recs"][f][:args.coinc_cpu_records]) for f in frames}
    t0 = time.perf_counter()
    ora = pyoracle.coinc(cfg, frames, [sub[f] for f in frames])
    t_cpu = time.perf_counter() - t0
    nsub = sum(len(v) for v in sub.values())
    cs = L.Coinc(cfg)
    for f in frames:
        cs.add_frame(f, sub[f])
    dev = cs.run()
    cs.close()
    same = dev.coi_bytes() == ora.coi_bytes() and dev.frameinfo.tolist() == ora.frameinfo.tolist()
    line = {"metric": "trigger records/s through the coincidence step (cells, duplicate removal, coincidences)",
            "value": value, "unit": "records/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64 cells, u64 keys", "data": "synthetic",
            "config": {"workload": "%d frames x %d trigger records, N=86164, 64 lines x 256 sky, 1000 signals, "
                                   "mincoin 4" % (len(frames), args.coinc_records),
                       "records": nrec, "inband": int(s.inband), "unique": int(s.unique), "coincidences": int(s.ncoin),
                       "fp64_cells": int(s.fp64_cells),
                       "maxcoin": int(s.maxcoin),
                       "l2": "flushed (256 MB write) before each timed step; records 1.0 GB > L2"},
            "clocks": clk, "gpu_launches": int(launches),
            "e2e": {"value": nrec * args.steps / t_e2e, "unit": "records/s", "h2d_bytes_per_step": 40 * nrec,
                    "d2h_bytes_per_step": d2h},
            "cpu_baseline": {"value": nsub / t_cpu, "unit": "records/s", "cores": 1, "kind": "port",
                             "sample": "first %d records of each of the %d frames (CPU oracle, one thread, %.1f s)" %
                                       (args.coinc_cpu_records, len(frames), t_cpu)},
            "roofline": roof,
            "kernel_share": {k: round(v[0] / tot, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])
                             if v[1]},
            "matches_oracle_on_sample": bool(same)}
    cc.close()
    emit(line)


def coinc_extra(L, steps: int = 3) -> dict:
    """The coincidence step (trigger-file consumer) on a smaller workload than
    --workload coincidences: 24 frames x 2^18 records, device time per run."""
    w = workloads.coincidences(24, 1 << 18)
    cfg = L.coinc_cfg(N=w["N"], oms=w["oms"], vedva_m=L.vedva(w["fisher"]), refr=w["refr"], mincoin=w["mincoin"])
    cc = L.Coinc(cfg)
    for f in w["frames"]:
        cc.add_frame(f, w["recs"][f])
    for _ in range(2):
        cc.run()
    ms = 0.0
    for _ in range(steps):
        l2_flush()
        res = cc.run()
        ms += cc.last_call_ms()
    cc.close()
    nrec = int(res.summary.raw)
    return {"metric": "trigger records/s through the coincidence step", "value": nrec * steps / (ms / 1e3),
            "unit": "records/s", "ms_per_run": ms / steps, "records": nrec,
            "coincidences": int(res.summary.ncoin),
            "workload": "24 frames x 262144 trigger records, N=86164, 64 lines x 256 sky, 1000 signals, mincoin 4 "
                        "(bench.py --workload coincidences: 24 x 2^20)"}


def followup_extra(L, steps: int = 3) -> dict:
    """The followup F-statistic (demodulated; H1+L1+V1, N=86164, 4096
    candidates) and its adjoint gradient, device time per batch
    in the default mixed form (FP64 phase) and with the two-float phase."""
    tmp = tempfile.mkdtemp(prefix="pa_followup_")
    argv, inj = workloads.followup(tmp)
    host = L.Host(argv)
    dets, nifo = host.detectors()
    pts, ws, which = workloads.candidates_around(host, inj, 4096)
    out = {"metric": "demodulated F-statistic evaluations/s (followup)", "unit": "evals/s", "candidates": len(pts),
           "workload": "H1+L1+V1, N=86164 dt=2s, 4096 candidates around 4 injections "
                       "(bench.py --workload followup has the ascent, the simplex and the CPU baseline)"}
    for name, ph in (("mixed", L.PA_PHASE_F64), ("mixed_ffphase", L.PA_PHASE_FF)):
        fu = L.Followup(host.settings, dets, nifo, precision=L.PA_PREC_MIXED, phase_mode=ph)
        fu.fstatnet(pts)
        fu.fstatnet_grad(pts)
        ms = gms = 0.0
        for _ in range(steps):
            l2_flush()
            fu.fstatnet(pts)
            ms += fu.last_call_ms()
            l2_flush()
            fu.fstatnet_grad(pts)
            gms += fu.last_call_ms()
        out[name] = {"fstat_evals_per_s": len(pts) * steps / (ms / 1e3),
                     "grad_evals_per_s": len(pts) * steps / (gms / 1e3)}
        fu.close()
    return out


_JSON_FD = 1


def run_cta_trace(ctx, tasks, opts, rng, cfg, templates_per_sky) -> dict:
    """One step with the per-CTA trace on (diagnostic build): how much of the
    step the GPU runs no CTA at all (gaps between kernels and launch
    latency), how busy the SMs are (partial waves, tails), and the CTA time
    of each kernel kind.  All times from %globaltimer of the CTAs' first and
    last instruction of thread 0."""
    import torch
    REC = np.dtype([("t0", "<u8"), ("t1", "<u8"), ("c0", "<u8"), ("c1", "<u8"), ("kind", "<u4"),
                    ("smid", "<u4"), ("p0", "<u4"), ("p1", "<u4")])
    cap = 1 << 23
    buf = torch.zeros(cap * REC.itemsize, dtype=torch.uint8, device="cuda")
    ctx.set_cta_trace(buf.data_ptr(), cap)
    l2_flush()
    ctx.search_batch(tasks, opts, rng)
    step_ms = ctx.last_call_ms()
    n = ctx.cta_trace_count()
    ctx.set_cta_trace(0, 0)
    r = np.frombuffer(buf[:min(n, cap) * REC.itemsize].cpu().numpy().tobytes(), dtype=REC)
    r = r[r["t1"] > 0]
    t0 = r["t0"].astype(np.int64)
    t1 = r["t1"].astype(np.int64)
    base = t0.min()
    t0 -= base
    t1 -= base
    span = int(t1.max())

    def union(a, b):
        o = np.argsort(a, kind="stable")
        a, b = a[o], b[o]
        busy, cur_a, cur_b, gaps = 0, a[0], b[0], []
        for x, y in zip(a[1:], b[1:]):
            if x > cur_b:
                busy += cur_b - cur_a
                gaps.append(x - cur_b)
                cur_a, cur_b = x, y
            elif y > cur_b:
                cur_b = y
        busy += cur_b - cur_a
        return int(busy), np.array(gaps, dtype=np.int64)

    busy, gaps = union(t0, t1)
    nsm = int(r["smid"].max()) + 1
    sm_busy = []
    for sm in range(nsm):
        m = r["smid"] == sm
        sm_busy.append(union(t0[m], t1[m])[0] if m.any() else 0)
    names = {k: L_kind for k, L_kind in enumerate(
        ["prelude_mod", "fft_fwd_a", "fft_fwd_b", "fft_inv_a", "fft_inv_b", "spline_fwd", "spline_bwd",
         "splint", "spindown_pass_a", "spindown_pass_b_fstat", "threshold"])}
    kinds = {}
    cta_ns = (t1 - t0).astype(np.float64)
    for k in np.unique(r["kind"]):
        m = r["kind"] == k
        kinds[names.get(int(k), str(int(k)))] = {"ctas": int(m.sum()), "cta_ms": float(cta_ns[m].sum() / 1e6),
                                                "mean_cta_us": float(cta_ns[m].mean() / 1e3)}
    ut = np.unique(np.concatenate([t0, t1]))
    return {"cta_trace": {
        "workload": cfg["workload"], "sky_points": len(tasks), "step_ms_events": step_ms,
        "span_ms": span / 1e6, "ctas": int(len(r)), "dropped": int(max(0, n - cap)),
        "gpu_idle_frac": 1.0 - busy / span, "gaps": int(len(gaps)),
        "gaps_over_1us": int((gaps > 1000).sum()), "gap_ms_total": float(gaps.sum() / 1e6),
        "gap_us_median": float(np.median(gaps) / 1e3) if len(gaps) else 0.0,
        "sm_busy_frac_mean": float(np.mean(sm_busy) / span), "sm_busy_frac_min": float(np.min(sm_busy) / span),
        "cta_slots_mean": float(cta_ns.sum() / (nsm * span)), "sms": nsm,
        "timer_resolution_ns": int(np.diff(ut).min()) if len(ut) > 1 else 0,
        "templates_per_s_traced": len(tasks) * templates_per_sky / (step_ms / 1e3),
        "kinds": kinds}}


def run_reference(args) -> None:
    """The reference arm: the CPU implementation of the path (the oracle's
    build with the reference's timing flags, OpenMP on every host thread) on
    the same workload and metric, each step a bounded sample of the sky
    points.  Its inputs are read by the oracle-side set-up
    (oracle/oracle_setup.py), so this process loads no library of the
    product; no GPU is used."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_setup
    tmp = tempfile.mkdtemp(prefix="pa_bench_ref_")
    make_workload(tmp, args.spindowns)
    inp = oracle_setup.Inputs(tmp, ident=1, band=666, dt=2.0, nod=2, range_file=os.path.join(tmp, "range.txt"))
    tasks = sky_tasks(inp, args.sky)
    s = inp.settings
    bins = s.nmax - s.nmin
    nspin = args.spindowns
    cfg = {"workload": WORKLOAD, "sky_points": len(tasks), "spindowns": nspin, "bins": bins,
           "nifo": inp.nifo, "N": s.N, "nfftf": s.nfftf, "parallelism": "host CPU, OpenMP"}
    nth = os.cpu_count() or 1
    for _ in range(min(1, args.warmup)):
        cpu_baseline(inp, tasks, 1, nth)
    t_all = 0.0
    ntempl = 0
    for _ in range(args.steps):
        v, dt, ns = cpu_baseline(inp, tasks, args.cpu_sky, nth)
        t_all += dt
        ntempl += ns * nspin * bins
    value = ntempl / t_all
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_all / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": "%d sky points x %d spindowns per step (CPU oracle, timing build, "
                                       "OpenMP)" % (min(args.cpu_sky, len(tasks)), nspin),
                             "calibration": cpu_calibration()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0, "libraries_loaded": repo_libraries()}
    emit(line)


def repo_libraries() -> list[str]:
    """Shared libraries of this repository mapped into the process."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                p = line.split()[-1]
                if p.startswith(ROOT) and ".so" in os.path.basename(p):
                    out.add(os.path.relpath(p, ROOT))
    except OSError:
        pass
    return sorted(out)


def emit(line: dict) -> None:
    """The one JSON result line, on the original standard output."""
    os.write(_JSON_FD, (json.dumps(line) + "\n").encode())


def main():
    # the C host library reports its set-up on standard output, as the
    # reference program does; send that to standard error so that standard
    # output carries the JSON line only
    global _JSON_FD
    sys.stdout.flush()
    _JSON_FD = os.dup(1)
    os.dup2(2, 1)
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sky", type=int, default=NSKY_DEFAULT)
    ap.add_argument("--spindowns", type=int, default=NSPIN_DEFAULT)
    ap.add_argument("--phase", default="fixed", choices=["fixed", "f64", "ff"])
    ap.add_argument("--fp64-sky", type=int, default=48, help="sky points timed in the all-FP64 form")
    ap.add_argument("--cpu-sky", type=int, default=48, help="sky points in the CPU-baseline sample")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--schedule", default="",
                    help="fixed spindown schedule 'sbatch,split[,lanes]' (lanes 1 when omitted; skips the autotuner)")
    ap.add_argument("--segments", type=int, default=24, help="segments workload: number of segments")
    ap.add_argument("--coinc-frames", type=int, default=24, help="coincidences workload: frames")
    ap.add_argument("--coinc-records", type=int, default=1 << 20, help="coincidences workload: records per frame")
    ap.add_argument("--coinc-cpu-records", type=int, default=100000,
                    help="coincidences workload: records per frame in the CPU-oracle sample")
    ap.add_argument("--workload", default="network",
                    choices=["network", "stress", "followup", "segments", "coincidences"],
                    help="stress: the N=258492 precision-stress workload, every precision form; "
                         "followup: demodulated F-statistic, adjoint, ascent and simplex on 4096 candidates")
    ap.add_argument("--candidates", type=int, default=4096, help="followup workload: candidates")
    ap.add_argument("--graphs", type=int, default=1, help="capture each batch into a CUDA graph (1) or not (0)")
    ap.add_argument("--autotune", type=int, default=1,
                    help="tune the spindown schedule (pa_autotune) on 8 sky points before timing (1) or not (0)")
    ap.add_argument("--cpu-candidates", type=int, default=4, help="followup: CPU simplex sample")
    ap.add_argument("--cta-trace", type=int, default=0,
                    help="network workload: instead of the timed steps, one step of the diagnostic build "
                         "with the per-CTA trace on; prints the launch-structure summary (idle fraction, "
                         "gaps, SM busy fraction, CTA time per kernel)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    from polgraw_gb300 import build as pbuild, lib as L
    pbuild.build()
    if args.cta_trace:
        # the diagnostic build with the per-CTA trace compiled in
        L.load(pbuild.build(trace=True))
    if args.workload == "stress":
        if rank == 0:
            run_stress(args, L)
        return
    if args.workload == "followup":
        if rank == 0:
            run_followup(args, L)
        return
    if args.workload == "segments":
        if rank == 0:
            run_segments(args, L)
        return
    if args.workload == "coincidences":
        if rank == 0:
            run_coinc(args, L)
        return
    tmp = tempfile.mkdtemp(prefix="pa_bench_")
    # N > 1: the sky partitioned over the GPUs (weak scaling: a lattice of
    # about args.sky x N points, each rank a contiguous block of args.sky of
    # them; sky points are independent, nothing is exchanged); the step time
    # is the maximum over ranks and the work the sum
    from polgraw_gb300 import shards
    argv = make_workload(tmp, args.spindowns, args.sky if world == 1 else int(args.sky * world * 1.03) + 1)
    host = L.Host(argv)
    tasks = shards.shard(sky_tasks(host, args.sky * world), rank, world, args.sky)
    s = host.settings
    bins = s.nmax - s.nmin
    nspin = args.spindowns
    cfg = {"workload": WORKLOAD, "sky_points": len(tasks), "spindowns": nspin, "bins": bins,
           "graphs": bool(args.graphs),
           "nifo": 2, "N": s.N, "nfftf": s.nfftf, "phase": args.phase,
           "l2": "flushed (256 MB write) before each timed step",
           "parallelism": ("sky partitioned over %d GPUs, %d sky points each, no collective in the search"
                           % (world, args.sky)) if world > 1 else "1 GPU"}

    shards.init()
    local = shards.world()[2]
    device = local if world > 1 else 0
    if world > 1:
        import torch
        torch.cuda.set_device(device)
    dets, nifo = host.detectors()
    phase = L.PHASE_NAMES[args.phase]
    ctx = L.Context(s, dets, nifo, precision=L.PA_PREC_MIXED, phase_mode=phase, device=device)
    opts, rng = host.opts(), host.range
    templates = len(tasks) * nspin * bins
    if args.schedule:
        sv = [int(v) for v in args.schedule.split(",")]
        ctx.set_lanes(1)
        ctx.set_schedule(sv[0], sv[1])
        ctx.set_lanes(sv[2] if len(sv) > 2 else 1)
    elif args.autotune:
        # 32 sky points: large enough that the pipeline's start and end do
        # not decide between schedules a few per cent apart
        ctx.autotune(tasks[:32], opts, rng)
    ctx.set_graphs(bool(args.graphs))
    sched = ctx.schedule()
    lanes = ctx.lanes()
    for _ in range(args.warmup):
        ctx.search_batch(tasks, opts, rng)
    if args.cta_trace:
        if rank == 0:
            emit(run_cta_trace(ctx, tasks, opts, rng, cfg, nspin * bins))
        ctx.close()
        shards.shutdown()
        return
    launches0 = ctx.launches()
    shards.barrier()
    clocks = ClockSampler(device)
    dev_ms = []
    ncand = 0
    for _ in range(args.steps):
        l2_flush()
        rec, idx, fnum = ctx.search_batch(tasks, opts, rng)
        dev_ms.append(ctx.last_call_ms())
        ncand = len(rec)
    shards.barrier()
    clk = clocks.stop()
    launches = (ctx.launches() - launches0) // max(1, args.steps)
    t_dev, templates_all = shards.reduce_step(sum(dev_ms) / 1e3, float(templates))
    value = templates_all * args.steps / t_dev

    # end to end: host buffers in, candidates out, through the C-ABI
    e2e_t = 0.0
    shards.barrier()
    for _ in range(args.steps):
        l2_flush()
        t0 = time.perf_counter()
        ctx.set_data(dets, nifo)
        rec, idx, fnum = ctx.search_batch(tasks, opts, rng)
        e2e_t += time.perf_counter() - t0
    e2e_t, _ = shards.reduce_step(e2e_t, 0.0)
    e2e = templates_all * args.steps / e2e_t
    h2d = nifo * s.N * 8 * 4
    d2h = 4 + len(rec) * 24

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64phase", "data": "synthetic", "config": cfg,
           "clocks": clk, "gpu_launches": int(launches),
           "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
           "candidates_per_step": ncand,
           # digest of the last step's candidate records and indices: equal
           # across runs, and across code changes that keep the arithmetic,
           # for one schedule (the FFT split changes rounding)
           "candidates_sha1": hashlib.sha1(np.ascontiguousarray(rec).tobytes()
                                           + np.ascontiguousarray(idx).tobytes()).hexdigest()[:16],
           "schedule": {"spindown_batch": sched[0], "fft_split": sched[1], "lanes": lanes,
                        "autotuned": bool(args.autotune) and not args.schedule}}

    if not args.no_extras and rank == 0:
        # per-kernel CUDA-event profile of one step (not the timed number; the
        # context runs its kernels one at a time while profiling, so that each
        # launch's events time that kernel alone, as ncu's serialised list)
        ctx.set_profiling(True)
        ctx.profile_reset()
        l2_flush()
        ctx.search_batch(tasks, opts, rng)
        prof = ctx.profile()
        ctx.set_profiling(False)
        tot = sum(v[0] for v in prof.values())
        top = max(prof.items(), key=lambda kv: kv[1][0])
        name, (ms, nl, items) = top
        pk = peaks()
        # algorithmic bytes of the spindown loop: xDatm{a,b} (2 x 8 B FP32
        # complex) + one 8-B phase coefficient per detector and sample
        per_unit = nifo * s.N * 24
        achieved = per_unit * items / (ms / 1e3) / 1e9 if name == "spindown_pass_a" else None
        out["roofline"] = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": pk["hbm_gbs"],
                           "unit": "GB/s", "frac": (achieved / pk["hbm_gbs"]) if achieved else None,
                           "traffic": PASS_A_TRAFFIC_PER_SPINDOWN[tuple(sched[:2])] * items / max(1, nl)
                           if (name == "spindown_pass_a" and s.N == 86164 and nifo == 2
                               and tuple(sched[:2]) in PASS_A_TRAFFIC_PER_SPINDOWN) else None,
                           "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch "
                                             "(profiles/spindown_pass_a_network_n86164.md)",
                           "peak_source": pk["source"] + " (MEASURED_PEAKS.json hbm_gbs)",
                           "avg_launch_ms": ms / max(1, nl), "units_per_launch": items / max(1, nl)}
        out["kernel_share"] = {k: round(v[0] / tot, 4) for k, v in sorted(prof.items(), key=lambda kv: -kv[1][0])}

        # all-FP64 form of the same kernels on a subset, and candidate agreement
        sub = tasks[:args.fp64_sky]
        c64 = L.Context(s, dets, nifo, precision=L.PA_PREC_FP64, device=0)
        c64.search_batch(sub[:2], opts, rng)
        l2_flush()
        r64, i64, _ = c64.search_batch(sub, opts, rng)
        ms64 = c64.last_call_ms()
        v64 = len(sub) * nspin * bins / (ms64 / 1e3)
        rmx, imx, _ = ctx.search_batch(sub, opts, rng)
        msmx = ctx.last_call_ms()
        vmx = len(sub) * nspin * bins / (msmx / 1e3)
        k64 = {tuple(int(x[f]) for f in ("pm", "mm", "nn", "ss", "ii")): r[4] for x, r in zip(i64, r64)}
        kmx = {tuple(int(x[f]) for f in ("pm", "mm", "nn", "ss", "ii")): r[4] for x, r in zip(imx, rmx)}
        F = lambda snr: snr * snr / 2 + 2  # noqa: E731
        common = [k for k in k64 if k in kmx]
        err = max([abs(F(kmx[k]) - F(k64[k])) / F(k64[k]) for k in common], default=0.0)
        edge = lambda k, d: abs(F(d[k]) - opts.trl) <= 1e-4 * opts.trl  # noqa: E731
        only64 = [k for k in k64 if k not in kmx and not edge(k, k64)]
        onlymx = [k for k in kmx if k not in k64 and not edge(k, kmx)]
        out["fp64_form"] = {"value": v64, "unit": UNIT, "sky_points": len(sub), "mixed_same_subset": vmx,
                            "mixed_over_fp64": vmx / v64, "fstat_rel_err_max": err,
                            "candidates": len(k64), "index_mismatches": len(only64) + len(onlymx)}
        c64.close()
        if rank == 0:
            nth = os.cpu_count() or 1
            cv, cdt, cn = cpu_baseline(host, tasks, args.cpu_sky, nth)
            out["cpu_baseline"] = {"value": cv, "unit": UNIT, "cores": nth, "kind": "port",
                                   "sample": "%d sky points x %d spindowns (CPU oracle, timing build, OpenMP, "
                                             "%.1f s)" % (cn, nspin, cdt),
                                   "calibration": cpu_calibration()}
            # and the serial form on one core (the reference's src-cpu build)
            c1v, c1dt, c1n = cpu_baseline(host, tasks, 1, 1)
            out["cpu_baseline_1core"] = {"value": c1v, "unit": UNIT, "cores": 1, "kind": "port",
                                         "sample": "1 sky point x %d spindowns (CPU oracle, timing build, one "
                                                   "thread, %.1f s)" % (nspin, c1dt)}
            # relative F-statistic error of the mixed form against the FP64 CPU
            # oracle (its parity build: the timing build's -ffast-math moves F
            # by up to ~1e-3)
            ref = {}
            _, _, cn = cpu_baseline(host, tasks, 24, nth, keep=ref, fast=False)
            rg, ig, _ = ctx.search_batch(tasks[:cn], opts, rng)
            got = {tuple(int(x[f]) for f in ("pm", "mm", "nn", "ss", "ii")): r[4] * r[4] / 2 + 2
                   for x, r in zip(ig, rg)}
            common = [k for k in ref if k in got]
            edge = lambda F: abs(F - opts.trl) <= 1e-4 * opts.trl  # noqa: E731
            out["vs_oracle"] = {"sky_points": cn, "candidates": len(ref), "oracle": "parity build",
                                "fstat_rel_err_max": max([abs(got[k] - ref[k]) / ref[k] for k in common],
                                                         default=0.0),
                                "index_mismatches": sum(1 for k in ref if k not in got and not edge(ref[k])) +
                                sum(1 for k in got if k not in ref and not edge(got[k]))}
    if not args.no_extras and rank == 0:
        out["coincidences"] = coinc_extra(L)
        out["followup"] = followup_extra(L)
    if rank == 0:
        emit(out)
    ctx.close()
    shards.shutdown()


if __name__ == "__main__":
    main()
