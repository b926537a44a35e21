"""The grid generator's lattice (pa_gridgen, host/pa_lattice.c) and the
gridgen-gb300 program against the reference grid generator (gridgen/,
compiled from its own sources by oracle/build_oracle.py): grid.bin equal
byte for byte.

* the committed grids of the golden cases (tests/golden/grid_*.bin, made by
  make_gridgen_grids.py from the synthetic ephemeris): the two on the common
  Polgraw configuration (N/nfft = 86164/131072, minimal match 0.75) take the
  S2 cell from the generator's table dataS2.txt, which exists only with the
  reference checkout; the third (N = 10771) computes the S2 cell;
* where the reference checkout exists, a sweep of seeded random segments
  (detector, N, nfft = 2^ceil(log2 N) or twice that, minimal match 0.60 to
  0.92) through the reference program and pa_gridgen, covering both
  methods, table hits and misses, fftpad 1 and 2;
* the program gridgen-gb300 with the reference's command line.
"""
import json
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

import build_oracle
from polgraw_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TABLE = os.path.join(build_oracle.GRIDGEN_DIR, "dataS2.txt")
HAVE_REF = os.path.exists(TABLE)


def _ephemeris(tmp, det, N, dt):
    ssb, rdet, phir, epsm = synth.detssb_parts(det, N, dt)
    d = os.path.join(str(tmp), "eph") + "/"
    os.makedirs(d, exist_ok=True)
    ssb.astype("<f8").tofile(d + "rSSB.bin")
    rdet.astype("<f8").tofile(d + "rDet.bin")
    with open(d + "DetSSB.bin", "wb") as f:
        f.write((ssb + rdet).astype("<f8").tobytes())
        f.write(np.array([phir, epsm], dtype="<f8").tobytes())
    return d, ssb, rdet, epsm


def _c0(mm):
    return float("%f" % (mm * mm))   # -m as the generator reads it


with open(os.path.join(GOLDEN, "gridgen_grids.json")) as _f:
    GRIDS = json.load(_f)


@pytest.mark.parametrize("name", sorted(GRIDS))
def test_committed_grids(name, tmp_path, lib):
    from polgraw_gb300.lib import gridgen
    sp = GRIDS[name]["spec"]
    N = synth.nsamples(sp["nod"], sp["dt"])
    d, ssb, rdet, epsm = _ephemeris(tmp_path, sp["det"], N, sp["dt"])
    want = open(os.path.join(GOLDEN, name), "rb").read()
    g = gridgen(ssb, rdet, epsm, sp["nfft_exp"], c0=_c0(0.75), table=TABLE if HAVE_REF else None)
    got = g.grid_bin()
    if got != want and not HAVE_REF:
        pytest.skip("this grid's S2 cell comes from the generator's dataS2.txt (reference checkout absent)")
    assert got == want
    assert len(got) == 388


def _sweep_cases(n=10, seed=7):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        det = ["H1", "L1", "V1"][int(rng.integers(3))]
        N = int(rng.integers(12000, 140000))
        e = int(math.ceil(math.log2(N))) + int(rng.integers(0, 2))
        mm = round(float(rng.uniform(0.6, 0.92)), 2)
        out.append((det, N, e, mm))
    # the common configuration (table hit) and an S1 case with tied vectors
    out += [("H1", 86164, 17, 0.75), ("H1", 80000, 17, 0.75), ("L1", 86164, 17, 0.8)]
    return out


@pytest.mark.skipif(not HAVE_REF, reason="reference checkout absent")
@pytest.mark.parametrize("case", _sweep_cases(), ids=lambda c: "%s-N%d-n%d-m%.2f" % c)
def test_matches_reference_program(case, tmp_path, lib):
    from polgraw_gb300.lib import gridgen
    det, N, e, mm = case
    d, ssb, rdet, epsm = _ephemeris(tmp_path, det, N, 2.0 * 86164.0905 / N)
    raw, _ = build_oracle.run_ref_gridgen(d, e, mm)
    g = gridgen(ssb, rdet, epsm, e, c0=_c0(mm), table=TABLE)
    assert g.grid_bin() == raw, (g.method, g.alpha)


def test_program(tmp_path, lib):
    from polgraw_gb300 import build
    from polgraw_gb300.lib import gridgen
    d, ssb, rdet, epsm = _ephemeris(tmp_path, "L1", 86164, 2.0)
    run = tmp_path / "run"
    run.mkdir()
    if HAVE_REF:
        shutil.copy(TABLE, str(run))
    r = subprocess.run([build.GRIDGEN_EXE, "-m", "0.75", "-p", "dfg", "-d", d, "-n", "17"], cwd=str(run),
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    got = open(d + "grid.bin", "rb").read()
    want = gridgen(ssb, rdet, epsm, 17, c0=_c0(0.75), table=TABLE if HAVE_REF else None).grid_bin()
    assert got == want
    if HAVE_REF:
        os.remove(d + "grid.bin")
        raw, _ = build_oracle.run_ref_gridgen(d, 17, 0.75)
        assert got == raw
    assert "fftpad: 1" in r.stdout
