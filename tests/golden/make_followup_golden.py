"""Generates the followup golden fixtures tests/golden/<case>.json for the
cases in FOLLOWUP_CASES (tests/golden/cases.py) by running the reference
followup program's own functions -- followup/src/followup.c compiled from its
own sources by oracle/build_oracle.py into oracle/_ref/libfollowup_ref.so and
driven by oracle/ref_followup_driver.c:

* fstatnet: evaluate_simplex() of one point (sky set-up + modvir + Fstatnet,
  followup.c:986-1009, 413-535) at the injection and at 16 points offset
  from it by up to 0.5 peak widths in each of (f, s, delta, alpha); the 11
  values of fstat_out per point;
* amoeba: the reference simplex (followup.c:1126-1174, tol 1e-7) from three
  offset starting points with initial steps of one peak width; the final
  point, its fstat_out and the number of F-statistic evaluations.

Peak widths: 2 pi/N (f), 2 pi/N^2 (s), and for the sky the angle that turns
the phase by 2 pi across the data, 2 pi / (oms * spread of dshft/dangle).

Run here (where the reference checkout exists):
    python tests/golden/make_followup_golden.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def _load_pkg():
    import importlib.util
    d = os.path.join(ROOT, "polgraw-allsky_gb300")
    spec = importlib.util.spec_from_file_location("polgraw_gb300", os.path.join(d, "__init__.py"),
                                                  submodule_search_locations=[d])
    m = importlib.util.module_from_spec(spec)
    sys.modules["polgraw_gb300"] = m
    spec.loader.exec_module(m)


_load_pkg()
import build_oracle  # noqa: E402
from cases import FOLLOWUP_CASES  # noqa: E402
from casegen import materialize  # noqa: E402


def peak_widths(settings, dets, nifo, delta, alpha):
    from polgraw_gb300 import workloads
    return workloads.peak_widths(settings, dets, nifo, delta, alpha)


def followup_points(case, settings, dets, nifo, seed=2005, n=16):
    inj = case["inject"]
    c = [inj["f"], inj["fdot"], inj["delta"], inj["alpha"]]
    w = peak_widths(settings, dets, nifo, inj["delta"], inj["alpha"])
    rng = np.random.default_rng(seed)
    pts = [c] + [[c[j] + float(rng.uniform(-0.5, 0.5)) * w[j] for j in range(4)] for _ in range(n)]
    return pts, w


def run_case(case: dict) -> dict:
    from polgraw_gb300.lib import Host
    lib = C.CDLL(build_oracle.build_reference()["followup"])
    P = C.POINTER(C.c_double)
    lib.ref_fu_init.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
    lib.ref_fu_fstatnet.argtypes = [P, P]
    lib.ref_fu_fstatnet.restype = None
    lib.ref_fu_amoeba.argtypes = [P, P, C.c_double, P]
    lib.ref_fu_amoeba.restype = C.c_long
    with tempfile.TemporaryDirectory() as tmp:
        data = os.path.join(tmp, "data")
        os.makedirs(data)
        m = materialize(case, data)
        host = Host(m["args"] + ["-output", os.path.join(tmp, "out"), "--nocheckpoint"])
        s = host.settings
        dets, nifo = host.detectors()
        assert lib.ref_fu_init(C.addressof(s), C.cast(dets, C.c_void_p), nifo) == 0
        pts, w = followup_points(case, s, dets, nifo)
        fst = []
        for p in pts:
            a = np.array(p, dtype=np.float64)
            out = np.zeros(11)
            lib.ref_fu_fstatnet(a.ctypes.data_as(P), out.ctypes.data_as(P))
            fst.append(out.tolist())
        am = []
        for k in (1, 2, 3):
            start = np.array(pts[k], dtype=np.float64)
            pc2 = np.array(w, dtype=np.float64)
            out = np.zeros(11)
            pt = start.copy()
            nev = lib.ref_fu_amoeba(pt.ctypes.data_as(P), pc2.ctypes.data_as(P), 1e-7, out.ctypes.data_as(P))
            am.append({"start": start.tolist(), "pc2": pc2.tolist(), "tol": 1e-7, "point": pt.tolist(),
                       "out": out.tolist(), "nevals": int(nev)})
        args = [a.replace(data, "<data>") for a in m["args"]]
        return {"case": case["name"], "inputs": m["ds"].files, "args": args, "N": s.N, "nifo": nifo,
                "widths": w, "points": pts, "fstatnet": fst, "amoeba": am,
                "generator": "followup/src/followup.c evaluate_simplex(dim=0) and amoeba(), "
                             "built by oracle/build_oracle.py"}


def main(names=None):
    for case in FOLLOWUP_CASES:
        if names and case["name"] not in names:
            continue
        g = run_case(case)
        path = os.path.join(HERE, case["name"] + ".json")
        with open(path, "w") as f:
            json.dump(g, f, indent=1)
        print(path, "F at injection %.6g" % -g["fstatnet"][0][5],
              "amoeba evals", [a["nevals"] for a in g["amoeba"]])


if __name__ == "__main__":
    main(sys.argv[1:] or None)
