"""The CPU oracle of the coincidence step (oracle/oracle_coinc.c) against the
reference coincidence program's own outputs (tests/golden/coinc_*.json, made
by tests/golden/make_coinc_golden.py from coincidences/src/coincidences.c):
the .coi file byte for byte (NaN means of a multiplicity-0 record compared
without their sign bit), the per-frame counts and the stderr summary line.
Also the library's host-side transformation matrix (pa_coinc_vedva) against
the oracle's."""
import base64
import hashlib
import os
import platform
import struct

import numpy as np
import pytest

from cases import COINC_CASES
from coinc_casegen import materialize, oracle_cfg
from helpers import GOLDEN_DIR, canon_coi, golden, parse_coi


@pytest.fixture(scope="module", params=[c["name"] for c in COINC_CASES])
def coinc_case(request, tmp_path_factory):
    case = [c for c in COINC_CASES if c["name"] == request.param][0]
    g = golden(case["name"])
    m = materialize(case, str(tmp_path_factory.mktemp(case["name"])))
    assert m["files"] == g["files"], "synthetic inputs differ from the golden run's"
    return case, g, m


def test_oracle_matches_reference_coincidences(coinc_case):
    import pyoracle
    case, g, m = coinc_case
    order = g["order"]
    res = pyoracle.coinc(oracle_cfg(case), order, [m["recs"][f] for f in order])
    assert res.frameinfo.tolist() == g["frameinfo"]
    assert res.summary.unique == g["total"]
    coi = res.coi_bytes()
    assert len(coi) == g["coi_size"]
    assert hashlib.sha256(canon_coi(coi)).hexdigest() == g["coi_canon_sha256"]
    if platform.machine() in ("x86_64", "AMD64"):
        assert hashlib.sha256(coi).hexdigest() == g["coi_sha256"]
    st = m["settings"]
    assert res.summary_line("%04d" % case["band"], case["shift"], st["fpo"]) == g["stderr"]


def test_crafted_quirks_are_exercised():
    """The crafted case really takes the reference's unusual branches."""
    g = golden("coinc_quirks")
    recs = parse_coi(base64.b64decode(g["coi_b64"]))
    fi = {f: (n, u) for f, n, u in g["frameinfo"]}
    # frames 3 and 4 lose one cell (the removed first-sorted record) and their
    # last run (the row left over from the frame read before them)
    assert fi[3][1] == fi[1][1] - 2 and fi[4][1] == fi[1][1] - 2
    # the last sorted cell is counted but written with multiplicity 0
    w, mean = recs[-1][0], recs[-1][1]
    assert w == 0 and np.isnan(mean[:4]).all() and mean[4] == 0
    assert all(r[0] > 0 for r in recs[:-1])


def test_vedva_host_matches_oracle(lib):
    import pyoracle
    from polgraw_gb300 import lib as L, synth
    for case in COINC_CASES[:1]:
        N = synth.nsamples(case["nod"], case["dt"])
        oms = 2 * np.pi * synth.fpo_default(case["band"], case["dt"]) * case["dt"]
        fis = synth.fisher_matrix(N, oms)
        a = L.vedva(fis)
        b = pyoracle.coinc_vedva(fis)
        assert np.array_equal(a, b)
        # columns are eigenvectors of the Fisher matrix scaled by sqrt(eigenvalue)
        for j in range(4):
            v = a[:, j]
            lam = v @ v
            assert np.allclose(fis @ (v / np.sqrt(lam)), lam * v / np.sqrt(lam), rtol=1e-10, atol=1e-20)


def test_digits_and_cfg():
    from polgraw_gb300 import lib as L
    assert L.digits4(1011, 0) == [1, 0, 1, 1]
    assert L.digits4(2412, 1) == [2, 4, 1, 2]
    assert L.digits4(1001, 1) == [1, 1, 1, 1]
    assert L.digits4(0, 0) == [0, 0, 0, 0]
    assert L.digits4(111, 1) == [1, 1, 1, 1]
    c = L.coinc_cfg(N=10, oms=1.0, vedva_m=np.eye(4), shift=1011, scale=2402, narrowdown=0.25)
    assert list(c.shift) == [1, 0, 1, 1] and list(c.scale) == [2, 4, 1, 2]
    assert c.narrowdown == 0.25 * np.pi


def test_fisher_reduced_matches_grid_generator(lib):
    """pa_fisher_reduced from the synthetic ephemeris parts equals, bit for
    bit, the reduced Fisher matrix that the reference grid generator wrote
    into each committed grid fixture (make_gridgen_grids.py)."""
    import json
    import os
    import tempfile
    from polgraw_gb300 import lib as L, synth
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    rec = json.load(open(os.path.join(here, "gridgen_grids.json")))
    assert rec
    for name, r in rec.items():
        sp = r["spec"]
        raw = open(os.path.join(here, name), "rb").read()
        assert hashlib.sha256(raw).hexdigest() == r["sha256"]
        N = synth.nsamples(sp["nod"], sp["dt"])
        ssb, rdet, phir, epsm = synth.detssb_parts(sp["det"], N, sp["dt"])
        with tempfile.TemporaryDirectory() as tmp:
            ds = synth.write_dataset(tmp, ident=1, band=sp["band"], dt=sp["dt"], nod=sp["nod"], dets=[sp["det"]],
                                     ephemeris_parts=True)
            assert {k: v for k, v in ds.files.items() if "/" in k} == r["ephemeris"]
        F = L.fisher_reduced(ssb, rdet, epsm)
        G = np.frombuffer(raw[4 + 128:4 + 256], dtype="<f8").reshape(4, 4)
        assert np.array_equal(F, G), (name, F - G)
        # and the grid's fftpad is the one the search derives for this length
        assert struct.unpack("<i", raw[:4])[0] == sp["nfft_exp"] - int(np.ceil(np.log2(N))) + 1


def test_oracle_on_reference_pipeline_triggers():
    """The coincidence oracle over the trigger files the reference search
    wrote for the pipeline case (tests/golden/pipeline_h1l1.json), in the
    order the reference coincidence program read them, reproduces that
    program's .coi file and summary line."""
    import re
    import pyoracle
    from pipeline_case import PIPELINE, settings
    from polgraw_gb300 import lib as L
    g = golden("pipeline_h1l1")
    st = settings(PIPELINE)
    raw = open(os.path.join(GOLDEN_DIR, PIPELINE["fisher_grid"]), "rb").read()
    fis = np.frombuffer(raw[132:260], dtype="<f8").reshape(4, 4)
    cfg = L.coinc_cfg(N=st["N"], oms=st["oms"], vedva_m=pyoracle.coinc_vedva(fis), refr=PIPELINE["refr"],
                      mincoin=PIPELINE["mincoin"], snrcutoff=PIPELINE["snrcutoff"],
                      narrowdown=PIPELINE["narrowdown"])
    by_frame = {int(re.match(r"triggers_(\d+)_", n).group(1)): np.array(r).reshape(-1, 5)
                for n, r in g["trigger_files"].items()}
    res = pyoracle.coinc(cfg, g["order"], [by_frame[f] for f in g["order"]])
    assert res.frameinfo.tolist() == g["frameinfo"]
    coi = base64.b64decode(g["coi_b64"])
    assert canon_coi(res.coi_bytes()) == canon_coi(coi)
    assert res.summary_line("%04d" % PIPELINE["band"], 0, st["fpo"]) == g["stderr"]
    # the injection is found in every segment
    assert res.summary.maxcoin == len(PIPELINE["frames"])
