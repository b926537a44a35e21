"""Makes the grid.bin fixtures tests/golden/grid_<case>.bin with the
reference grid generator (gridgen/, compiled from its own sources by
oracle/build_oracle.py into oracle/_ref/gridgen) from the synthetic
ephemeris of each case that names one (cases.py: a search case with
data.grid.gridgen, a coincidence case with "grid"; the pipeline case's Fisher
matrix, pipeline_case.py): rSSB.bin, rDet.bin and
DetSSB.bin of the case's first detector (polgraw_gb300.synth.detssb_parts),
`gridgen -m 0.75 -p dfg -d <dir>/ -n <log2 nfft>`.  The ephemeris files are
regenerated bit for bit from the case parameters, so only the 388-byte grids
are committed; gridgen_grids.json records their hashes.

Run here (where the reference checkout exists), before make_golden.py and
make_coinc_golden.py:
    python tests/golden/make_gridgen_grids.py
"""
from __future__ import annotations

import hashlib
import json
import os
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
from cases import CASES, COINC_CASES  # noqa: E402
from polgraw_gb300 import synth  # noqa: E402


def gridgen_specs() -> list[dict]:
    """(fixture name, detector, dt, nod, band, nfft exponent) of every case
    that runs on a grid generator's grid."""
    out = []
    for c in CASES:
        g = c["data"].get("grid", {})
        if "gridgen" in g:
            d = c["data"]
            out.append(dict(file=g["gridgen"], det=d["dets"][0], dt=d["dt"], nod=d["nod"], band=d["band"],
                            nfft_exp=g["nfft_exp"]))
    for c in COINC_CASES:
        if "grid" in c:
            out.append(dict(file=c["grid"], det="H1", dt=c["dt"], nod=c["nod"], band=c["band"],
                            nfft_exp=c["nfft_exp"]))
    from pipeline_case import PIPELINE as P
    out.append(dict(file=P["fisher_grid"], det=P["dets"][0], dt=P["dt"], nod=P["nod"], band=P["band"],
                    nfft_exp=P["nfft_exp"]))
    return out


def main() -> None:
    record = {}
    for sp in gridgen_specs():
        with tempfile.TemporaryDirectory() as tmp:
            ds = synth.write_dataset(tmp, ident=1, band=sp["band"], dt=sp["dt"], nod=sp["nod"], dets=[sp["det"]],
                                     ephemeris_parts=True)
            eph = os.path.join(tmp, "%03d" % ds.ident, sp["det"])
            raw, out = build_oracle.run_ref_gridgen(eph, sp["nfft_exp"])
        assert len(raw) == 388, len(raw)
        with open(os.path.join(HERE, sp["file"]), "wb") as f:
            f.write(raw)
        record[sp["file"]] = dict(spec=sp, sha256=hashlib.sha256(raw).hexdigest(),
                                  ephemeris={k: v for k, v in ds.files.items() if "/" in k})
        print(sp["file"], record[sp["file"]]["sha256"])
    with open(os.path.join(HERE, "gridgen_grids.json"), "w") as f:
        json.dump(record, f, indent=1)


if __name__ == "__main__":
    main()
