"""Materialises a coincidence case of tests/golden/cases.py (COINC_CASES):
trigger files of every frame and grid.bin under a directory, from the
deterministic generator polgraw_gb300.synth.coinc_triggers.

The crafted case (craft=True) edits the generated frames with the CPU oracle
(oracle/pyoracle.py) as the tool that tells which cell sorts first or last:
* frame 1 starts with three records in one cell with SNRs 9, 7, 8 (its
  first in-band record is the best of the run: the reference keeps the 8);
  frame 2 carries two records in one cell with equal SNR (the later one is
  kept, coincidences.c:385);
* every frame holds the same base set with s = 0 (identical cells in all
  frames), and frames 3 and 4 lack the base set's first-sorted record, so
  that their last row meets the row one past it left over from the frame
  before (coincidences.c:338-352) unless they are read first;
* the base set's last-sorted cell is therefore a coincidence of every frame
  that keeps it, the last group of the sorted table, which the reference
  counts but writes with multiplicity 0 (coincidences.c:455-541).
"""
from __future__ import annotations

import math
import os

import numpy as np


def case_settings(case: dict) -> dict:
    from polgraw_gb300 import synth
    N = synth.nsamples(case["nod"], case["dt"])
    fpo = synth.fpo_default(case["band"], case["dt"])
    return dict(N=N, fpo=fpo, oms=2. * math.pi * fpo * case["dt"])


def _records(case: dict, st: dict) -> dict:
    from polgraw_gb300 import synth
    if not case.get("craft"):
        return synth.coinc_triggers(case["frames"], case["per_frame"], N=st["N"], refr=case["refr"],
                                    seed=case["seed"])
    import pyoracle
    base = synth.coinc_triggers([1], case["per_frame"], N=st["N"], refr=case["refr"], seed=case["seed"],
                                lines=2, sky=3, signals=0)[1]
    base = base.copy()
    base[:, 1] = 0.0                                       # same cells in every frame
    cfg = oracle_cfg(case)
    one = pyoracle.coinc(cfg, [1], [base])
    inb = np.nonzero(_inband(base, case, st))[0]           # in-band rows in read order
    cells = one.cells
    order = sorted(range(len(inb)), key=lambda i: tuple(-cells[i]))   # descending, stable
    first_sorted = inb[order[0]]
    recs = {}
    for fr in case["frames"]:
        r = base
        if fr in (3, 4):
            r = np.delete(base, first_sorted, axis=0)
        if fr == 1:
            x = base[inb[order[len(order) // 2]]].copy()
            trio = np.stack([x, x, x])
            trio[:, 4] = [9.0, 7.0, 8.0]
            r = np.concatenate([trio[:1], r, trio[1:]], axis=0)
        if fr == 2:
            x = base[inb[order[len(order) // 3]]].copy()
            pair = np.stack([x, x])
            pair[:, 4] = [8.5, 8.5]
            r = np.concatenate([r[:5], pair[:1], r[5:], pair[1:]], axis=0)
        recs[fr] = np.ascontiguousarray(r)
    return recs


def _inband(r: np.ndarray, case: dict, st: dict) -> np.ndarray:
    nd = case["narrowdown"] * math.pi
    f = r[:, 0]
    # every crafted frame uses s = 0, so the frame shift is zero
    ok = (f > math.pi / 2 - nd) & (f < math.pi / 2 + nd)
    return ok & (f > 0) & (f < math.pi) & (r[:, 4] > case["snrcutoff"])


def _oracle_vedva(fis):
    import pyoracle
    return pyoracle.coinc_vedva(fis)


def case_fisher(case: dict, st: dict):
    from polgraw_gb300 import synth
    if "grid" in case:
        raw = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), case["grid"]), "rb").read()
        return np.frombuffer(raw[4 + 128:4 + 256], dtype="<f8").reshape(4, 4).copy()
    return synth.fisher_matrix(st["N"], st["oms"])


def oracle_cfg(case: dict):
    """pa_coinc_cfg of the case with the oracle's (GSL shim) vedva."""
    from polgraw_gb300 import lib as L
    st = case_settings(case)
    fis = case_fisher(case, st)
    return L.coinc_cfg(N=st["N"], oms=st["oms"], vedva_m=_oracle_vedva(fis), shift=case["shift"],
                       scale=case["scale"], refr=case["refr"], narrowdown=case["narrowdown"],
                       snrcutoff=case["snrcutoff"], mincoin=case["mincoin"])


def materialize(case: dict, root: str) -> dict:
    """Writes <root>/cand/triggers_*.bin and <root>/grid/grid.bin; returns the
    settings, the records per frame, file hashes and the command line of the
    coincidence program (without its executable)."""
    from polgraw_gb300 import synth
    st = case_settings(case)
    recs = _records(case, st)
    files = synth.write_triggers(os.path.join(root, "cand"), recs, band=case["band"])
    if "grid" in case:
        # a grid.bin made by the reference grid generator (make_gridgen_grids.py)
        raw = open(os.path.join(os.path.dirname(os.path.abspath(__file__)), case["grid"]), "rb").read()
        os.makedirs(os.path.join(root, "grid"), exist_ok=True)
        gp = os.path.join(root, "grid", "grid.bin")
        with open(gp, "wb") as f:
            f.write(raw)
        fis = np.frombuffer(raw[4 + 128:4 + 256], dtype="<f8").reshape(4, 4).copy()
        import hashlib
        files["grid.bin"] = hashlib.sha256(raw).hexdigest()
    else:
        fis = synth.fisher_matrix(st["N"], st["oms"])
        files["grid.bin"] = synth.write_coinc_grid(os.path.join(root, "grid", "grid.bin"), fis)
    os.makedirs(os.path.join(root, "out"), exist_ok=True)
    args = ["-data", os.path.join(root, "cand"), "-output", os.path.join(root, "out"),
            "-refr", str(case["refr"]), "-fpo", repr(st["fpo"]), "-dt", repr(case["dt"]),
            "-trigname", "%04d" % case["band"], "-refloc", os.path.join(root, "grid"),
            "-mincoin", str(case["mincoin"]), "-nod", str(case["nod"]),
            "-shift", "%04d" % case["shift"], "-scale", "%04d" % case["scale"],
            "-narrowdown", repr(case["narrowdown"]), "-snrcutoff", repr(case["snrcutoff"])]
    coi = os.path.join(root, "out", "%04d_%04d_%04d.coi" % (case["shift"], case["scale"], case["band"]))
    return dict(settings=st, recs=recs, files=files, args=args, coi=coi, fisher=fis)
