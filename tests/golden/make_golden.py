"""Generates the golden fixtures tests/golden/<case>.json by running the
reference search -- search/network/src-cpu compiled from its own sources by
oracle/build_oracle.py into oracle/_ref/gwsearch-ref (-DVERBOSE) -- on the
synthetic inputs of tests/golden/cases.py.

Each fixture records the input hashes, the command line, the per-sky-point
spindown ranges the reference printed (">>FNum mm nn [smin..smax]",
jobcore.c:441), and every candidate: the indices of its VERBOSE line
("Signal k: pm mm nn ss ii snr", jobcore.c:689-692) and the five doubles of
its trigger-file record (jobcore.c:686-687, 141), in file order.

Run here (where the reference checkout exists):  python tests/golden/make_golden.py
"""
from __future__ import annotations

import glob
import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


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
from cases import CASES  # noqa: E402
from casegen import materialize  # noqa: E402

SIG_RE = re.compile(r"Signal (\d+): (-?\d+) (-?\d+) (-?\d+) (-?\d+) (-?\d+) snr=([-\d.naif]+)")
RANGE_RE = re.compile(r">>(\d+)\s+(-?\d+)\s+(-?\d+)\s+\[(-?\d+)\.\.(-?\d+)\]")


def run_case(case: dict, exe: str) -> dict:
    with tempfile.TemporaryDirectory() as tmp:
        data = os.path.join(tmp, "data")
        os.makedirs(data)
        m = materialize(case, data)
        out = os.path.join(tmp, "out")
        args = m["args"] + ["-output", out]
        r = subprocess.run([exe] + args, cwd=tmp, capture_output=True, text=True, timeout=3600)
        if r.returncode != 0:
            raise RuntimeError("reference failed on %s:\n%s\n%s" % (case["name"], r.stdout[-3000:], r.stderr[-3000:]))
        sigs = [tuple(int(g) for g in mm.groups()[1:6]) for mm in SIG_RE.finditer(r.stdout)]
        ranges = [tuple(int(g) for g in mm.groups()) for mm in RANGE_RE.finditer(r.stdout)]
        recs = []
        for pm in (1, 2):
            lbl = "_" + case["label"] if case.get("label") else ""
            f = os.path.join(out, "triggers_001_%04d%s_%d.bin" % (case["data"]["band"], lbl, pm))
            if os.path.exists(f):
                recs.append((pm, np.fromfile(f, dtype="<f8").reshape(-1, 5)))
        allrec = np.concatenate([x[1] for x in recs]) if recs else np.zeros((0, 5))
        if len(allrec) != len(sigs):
            raise RuntimeError("%s: %d records vs %d VERBOSE lines" % (case["name"], len(allrec), len(sigs)))
        files = sorted(os.path.basename(p) for p in glob.glob(os.path.join(out, "*")))
        cands = [list(s) + [float(v) for v in rec] for s, rec in zip(sigs, allrec)]
        return {"name": case["name"], "args": [a for a in case.get("args", [])], "inputs": m["ds"].files,
                "spindown_ranges": ranges, "trigger_files": files,
                "candidates": cands,
                "fields": ["pm", "mm", "nn", "ss", "ii", "f", "s1", "delta", "alpha", "snr"]}


def main(names=None):
    exes = build_oracle.build_reference()
    if not exes:
        raise SystemExit("reference checkout not found; goldens can only be generated where it exists")
    for case in CASES:
        if names and case["name"] not in names:
            continue
        g = run_case(case, exes["serial"])
        with open(os.path.join(HERE, case["name"] + ".json"), "w") as f:
            json.dump(g, f, indent=1)
        print("%-16s %5d candidates, %3d sky points" % (case["name"], len(g["candidates"]), len(g["spindown_ranges"])))


if __name__ == "__main__":
    main(sys.argv[1:] or None)
