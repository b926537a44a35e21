"""Generates the coincidence golden fixtures tests/golden/<case>.json for
COINC_CASES (tests/golden/cases.py) by running the reference coincidence
program -- coincidences/src/coincidences.c with the network search's
settings.c, auxi.c and init.c, compiled from their own sources by
oracle/build_oracle.py into oracle/_ref/coincidences-ref -- on the trigger
files of coinc_casegen.materialize().

Recorded per case: the input hashes, the frames in the order the program
read its directory (its "Frame <n>:" lines), per-frame counts, the .coi file
(base64) and the stderr summary line.

Run here (where the reference checkout exists):
    python tests/golden/make_coinc_golden.py
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
from cases import COINC_CASES  # noqa: E402
from helpers import canon_coi  # noqa: E402
from coinc_casegen import materialize  # noqa: E402


def main() -> None:
    exe = build_oracle.build_reference()["coinc"]
    for case in COINC_CASES:
        with tempfile.TemporaryDirectory() as tmp:
            m = materialize(case, tmp)
            r = subprocess.run([exe] + m["args"], capture_output=True, text=True, cwd=tmp)
            if r.returncode != 0:
                raise RuntimeError("%s: reference failed\n%s%s" % (case["name"], r.stdout, r.stderr))
            lines = re.findall(r"Frame (\d+): (\d+)/(\d+)", r.stdout)
            coi = open(m["coi"], "rb").read()
            g = dict(name=case["name"], files=m["files"],
                     order=[int(a) for a, _, _ in lines],
                     frameinfo=[[int(a), int(c), int(b)] for a, b, c in lines],
                     total=int(re.search(r"Total number of candidates from all frames: (\d+)", r.stdout).group(1)),
                     coi_sha256=hashlib.sha256(coi).hexdigest(), coi_size=len(coi),
                     coi_canon_sha256=hashlib.sha256(canon_coi(coi)).hexdigest(),
                     coi_b64=base64.b64encode(coi).decode() if len(coi) <= 65536 else None,
                     stderr=r.stderr)
            with open(os.path.join(HERE, case["name"] + ".json"), "w") as f:
                json.dump(g, f, indent=1)
            print(case["name"], "frames", g["order"], "coi", len(coi), "bytes", "summary:", r.stderr[:80])


if __name__ == "__main__":
    main()
