"""Generates tests/golden/pipeline_h1l1.json: the reference pipeline on the
pipeline case of pipeline_case.py -- the reference network search
(oracle/_ref/gwsearch-ref, built from search/network/src-cpu) on every
segment, then the reference coincidence program (oracle/_ref/coincidences-ref,
built from coincidences/src/coincidences.c) over the segments' trigger files.

Recorded: the input hashes, every trigger file's records, the order in which
the coincidence program read the files, its per-frame counts, the .coi file
(base64) and its stderr summary line.

Run here (where the reference checkout exists), after make_gridgen_grids.py:
    python tests/golden/make_pipeline_golden.py
"""
from __future__ import annotations

import base64
import hashlib
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
from pipeline_case import PIPELINE, coinc_args, write_fisher_grid, write_segments  # noqa: E402


def main() -> None:
    exes = build_oracle.build_reference()
    case = PIPELINE
    with tempfile.TemporaryDirectory() as tmp:
        data = os.path.join(tmp, "data")
        os.makedirs(data)
        seg = write_segments(data, case)
        cand = os.path.join(tmp, "cand")
        for k in case["frames"]:
            r = subprocess.run([exes["serial"]] + seg["args"][k] + ["-output", cand, "--nocheckpoint"], cwd=tmp,
                               capture_output=True, text=True, timeout=3600)
            if r.returncode != 0:
                raise RuntimeError("reference search failed on frame %d:\n%s%s" % (k, r.stdout[-2000:], r.stderr))
        trig = {}
        for p in sorted(os.listdir(cand)):
            trig[p] = np.fromfile(os.path.join(cand, p), dtype="<f8").reshape(-1, 5).tolist()
        grid = os.path.join(tmp, "grid")
        write_fisher_grid(grid, case)
        out = os.path.join(tmp, "coinc")
        r = subprocess.run([exes["coinc"]] + coinc_args(cand, grid, out, case), cwd=tmp, capture_output=True,
                           text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError("reference coincidences failed:\n" + r.stdout + r.stderr)
        lines = re.findall(r"Frame (\d+): (\d+)/(\d+)", r.stdout)
        coi = open(os.path.join(out, "0000_1111_%04d.coi" % case["band"]), "rb").read()
        g = dict(name=case["name"], inputs=seg["files"], trigger_files=trig,
                 order=[int(a) for a, _, _ in lines], frameinfo=[[int(a), int(c), int(b)] for a, b, c in lines],
                 coi_b64=base64.b64encode(coi).decode(), coi_sha256=hashlib.sha256(coi).hexdigest(),
                 stderr=r.stderr)
    with open(os.path.join(HERE, case["name"] + ".json"), "w") as f:
        json.dump(g, f, indent=1)
    print(case["name"], {k: len(v) for k, v in g["trigger_files"].items()}, "order", g["order"],
          "coi", len(coi), "bytes;", g["stderr"][:120])


if __name__ == "__main__":
    main()
