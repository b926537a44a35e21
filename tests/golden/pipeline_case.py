"""End-to-end pipeline case, the shape of the reference's sensitivity scripts
(sensitivity-scripts/dummy.sh: inject, search, coincidences, check): five
consecutive segments (frames) of H1+L1 data, one day at dt = 8 s each, with
the same continuous-wave signal injected in every segment (its frequency
advanced by the spindown from segment to segment), the network search of
each segment around the injection, and the coincidence step over the
segments' trigger files with the Fisher matrix of the grid generator's grid
for this data length (grid_pipeline.bin, made by make_gridgen_grids.py).

make_pipeline_golden.py runs the reference programs (oracle/_ref: the search
and the coincidence program) on it; tests/test_gpu_pipeline.py runs
gwsearch-gb300 and coincidences-gb300.
"""
from __future__ import annotations

import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

PIPELINE = dict(name="pipeline_h1l1", dets=["H1", "L1"], dt=8.0, nod=1, band=100, frames=[1, 2, 3, 4, 5], refr=3,
                grid=dict(m5=-2e-8, sky_scale=0.05), fisher_grid="grid_pipeline.bin", nfft_exp=14,
                inject=dict(f=1.0, fdot=-6e-8, delta=0.3, alpha=1.2, snr=16.0),
                threshold=12.0, mincoin=3, snrcutoff=4.5, narrowdown=0.5, spin=(1, 5))


def settings(case: dict = PIPELINE) -> dict:
    from polgraw_gb300 import synth
    N = synth.nsamples(case["nod"], case["dt"])
    fpo = synth.fpo_default(case["band"], case["dt"])
    return dict(N=N, fpo=fpo, oms=2. * math.pi * fpo * case["dt"])


def search_grid(case: dict = PIPELINE) -> list[float]:
    from polgraw_gb300 import synth
    st = settings(case)
    nfft = 1 << int(math.ceil(math.log(st["N"]) / math.log(2.)))
    g = dict(case["grid"])
    d = g.pop("sky_scale") * st["oms"]
    return synth.grid_matrix(nfft, st["oms"], sky=(d, 0.0, 0.0, d), **g)


def injection_cell(case: dict = PIPELINE) -> tuple[int, int, int]:
    """(pm, nn, mm) of the grid point nearest to the injection."""
    from polgraw_gb300 import synth
    st = settings(case)
    M = search_grid(case)
    inj = case["inject"]
    be, pm = synth.ast2lin(inj["alpha"], inj["delta"])
    A = np.array([[M[10], M[14]], [M[11], M[15]]])
    nn, mm = np.linalg.solve(A, [st["oms"] * be[0], st["oms"] * be[1]])
    return pm, int(round(nn)), int(round(mm))


def write_segments(root: str, case: dict = PIPELINE) -> dict:
    """Writes every frame's data set (ident = frame number, noise seeds offset
    by 100 per frame), injects the signal with f_k = f + 2 fdot N (k - refr)
    (the frequency the coincidence step shifts back to the reference frame,
    coincidences.c:235) and a range file around the injection.  Returns the
    search command line per frame (without -output) and the input hashes."""
    from polgraw_gb300 import synth
    st = settings(case)
    M = search_grid(case)
    pm, nn, mm = injection_cell(case)
    rng = os.path.join(root, "range.txt")
    synth.write_range(rng, case["spin"], (nn - 1, nn + 1), (mm - 1, mm + 1), (pm, pm))
    inj = case["inject"]
    args, files = {}, {}
    for k in case["frames"]:
        ds = synth.write_dataset(root, ident=k, band=case["band"], dt=case["dt"], nod=case["nod"], fftpad=1,
                                 dets=case["dets"], M=M, seed_offset=100 * k)
        fk = inj["f"] + 2. * inj["fdot"] * st["N"] * (k - case["refr"])
        synth.inject(ds, f=fk, fdot=inj["fdot"], delta=inj["delta"], alpha=inj["alpha"], snr=inj["snr"])
        files.update({"%03d/%s" % (k, n): v for n, v in ds.files.items()})
        args[k] = ["-data", root, "-ident", str(k), "-band", str(case["band"]), "-dt", repr(case["dt"]),
                   "-nod", str(case["nod"]), "-range", rng, "-threshold", repr(case["threshold"])]
    return dict(args=args, files=files, settings=st)


def coinc_args(cand_dir: str, grid_dir: str, out_dir: str, case: dict = PIPELINE) -> list[str]:
    """The coincidence program's command line over the collected trigger files."""
    st = settings(case)
    return ["-data", cand_dir, "-output", out_dir, "-refr", str(case["refr"]), "-fpo", repr(st["fpo"]),
            "-dt", repr(case["dt"]), "-trigname", "%04d" % case["band"], "-refloc", grid_dir,
            "-mincoin", str(case["mincoin"]), "-nod", str(case["nod"]), "-snrcutoff", repr(case["snrcutoff"]),
            "-narrowdown", repr(case["narrowdown"])]


def write_fisher_grid(grid_dir: str, case: dict = PIPELINE) -> None:
    os.makedirs(grid_dir, exist_ok=True)
    raw = open(os.path.join(HERE, case["fisher_grid"]), "rb").read()
    with open(os.path.join(grid_dir, "grid.bin"), "wb") as f:
        f.write(raw)
