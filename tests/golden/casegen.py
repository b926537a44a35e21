"""Materialises a golden case (tests/golden/cases.py) into a data directory:
synthetic inputs, grid, optional range and injection files, and the
reference-style command line.  Used by make_golden.py (to run the reference)
and by the tests (to run the GPU search and the oracle on the same inputs).
"""
from __future__ import annotations

import math
import os

from polgraw_gb300 import synth


def _grid(data: dict, ds_probe) -> list[float]:
    g = dict(data.get("grid", {}))
    nfftf = ds_probe.fftpad * ds_probe.nfft
    oms = ds_probe.oms
    if "sky_point" in g:
        delta, alpha = g.pop("sky_point")
        be, _ = synth.ast2lin(alpha, delta)
        sky = (be[0] * oms, 0.0, 0.0, be[1] * oms)
    else:
        d = g.pop("sky_scale", 0.05) * oms
        k = g.pop("skew", 0.0)
        sky = (d, k * d, -k * d, d)
    g.pop("sky_scale", None)
    g.pop("skew", None)
    return synth.grid_matrix(nfftf, oms, sky=sky, **g)


def materialize(case: dict, root: str) -> dict:
    """Writes the case's inputs under root and returns
    {"args": [...], "ds": Dataset, "pm": hemisphere of a sky-point case}."""
    data = case["data"]
    probe = synth.Dataset(root=root, ident=1, band=data["band"], dt=data["dt"], nod=data["nod"],
                          fftpad=data["fftpad"], M=[], dets=list(data["dets"]),
                          N=synth.nsamples(data["nod"], data["dt"]))
    g = data.get("grid", {})
    if data.get("fixture"):
        # the reference's own input files (testdata_fixture.py)
        import testdata_fixture
        ds = synth.Dataset(root=root, ident=1, band=data["band"], dt=data["dt"], nod=data["nod"],
                           fftpad=data["fftpad"], M=[], dets=list(data["dets"]),
                           N=synth.nsamples(data["nod"], data["dt"]))
        ds.files = testdata_fixture.unpack(root)
    elif "gridgen" in g:
        # a grid.bin made by the reference grid generator from this case's
        # synthetic ephemeris (make_gridgen_grids.py)
        ds = synth.write_dataset(root, ident=1, band=data["band"], dt=data["dt"], nod=data["nod"],
                                 fftpad=data["fftpad"], dets=data["dets"], gaps=data.get("gaps", 0.0),
                                 ephemeris_parts=True,
                                 grid_file=os.path.join(os.path.dirname(os.path.abspath(__file__)), g["gridgen"]))
    else:
        M = _grid(data, probe)
        ds = synth.write_dataset(root, ident=1, band=data["band"], dt=data["dt"], nod=data["nod"],
                                 fftpad=data["fftpad"], dets=data["dets"], M=M, gaps=data.get("gaps", 0.0))
    args = ["-data", root, "-ident", "1", "-band", str(data["band"]), "-dt", repr(data["dt"]),
            "-nod", str(data["nod"])]
    pm = None
    if "inject" in case:
        synth.inject(ds, **case["inject"])
        _, pm = synth.ast2lin(case["inject"]["alpha"], case["inject"]["delta"])
    if "addsig" in case:
        a = dict(case["addsig"])
        path = os.path.join(root, "addsig.txt")
        synth.write_addsig(path, f=a["f"], fdot=a["fdot"], delta=a["delta"], alpha=a["alpha"], snr=a.get("snr"),
                           amp=a.get("amp"), gsize=a.get("gsize", 2), reffr=1)
        args += ["-addsig", path]
    if "range" in case:
        r = list(case["range"])
        if r[6] is None:
            r[6] = r[7] = pm
        path = os.path.join(root, "range.txt")
        synth.write_range(path, r[0:2], r[2:4], r[4:6], r[6:8])
        args += ["-range", path]
    for det, rows in case.get("lines", {}).items():
        # known-lines file read by read_lines() (settings.c:327-400): '%'
        # comment lines, then frequency, type, offset, first and last comb
        # index (and two unused columns) per line
        with open(os.path.join(root, "O1LinesToBeCleaned_%s_v1.txt" % det), "w") as fh:
            fh.write("%% known lines of %s\n" % det)
            for r in rows:
                fh.write("\t".join(repr(float(x)) if i in (0, 2) else str(int(x)) for i, x in enumerate(r)) + "\n")
    if case.get("label"):
        # -label: the reference reads xdatc_<ident>_<band>_<label>.bin
        # (init.c:174-175, settings.c:134) and names its outputs with the label
        for det in data["dets"]:
            dd = os.path.join(root, "%03d" % 1, det)
            os.rename(os.path.join(dd, "xdatc_%03d_%04d.bin" % (1, data["band"])),
                      os.path.join(dd, "xdatc_%03d_%04d_%s.bin" % (1, data["band"], case["label"])))
        args += ["-label", case["label"]]
    args += list(case.get("args", []))
    return {"args": args, "ds": ds, "pm": pm}
