"""The pipeline end to end on the GPU, against the reference pipeline
(tests/golden/pipeline_h1l1.json, make_pipeline_golden.py): gwsearch-gb300 on
five segments with the same injected signal, then the coincidence step over
their trigger files.

* FP64 form of the search: every trigger record equal to the reference's
  (f, s1, delta, alpha bit for bit; SNR to 1e-9 relative), and the
  coincidence records computed from our trigger files equal to the reference
  program's .coi (multiplicities, frames, positions, f/s/delta/alpha means;
  SNR means to 1e-6 relative), frames taken in the reference's directory
  order;
* default mixed form: the injection is found in every segment (the largest
  coincidence has multiplicity 5, at the reference's cell), and
  coincidences-gb300 over the trigger directory reports it on stderr."""
import base64
import os
import re
import subprocess

import numpy as np
import pytest

from helpers import GOLDEN_DIR, golden, parse_coi
from pipeline_case import PIPELINE, coinc_args, settings, write_fisher_grid, write_segments

pytestmark = pytest.mark.gpu


def _search(tmp_path, precision):
    from polgraw_gb300 import build
    data = str(tmp_path / "data")
    os.makedirs(data, exist_ok=True)
    seg = write_segments(data, PIPELINE)
    cand = str(tmp_path / ("cand_" + precision))
    for k in PIPELINE["frames"]:
        r = subprocess.run([build.EXE] + seg["args"][k] + ["-output", cand, "--nocheckpoint", "-precision", precision],
                           cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return seg, cand


def _coinc_cfg():
    from polgraw_gb300 import lib as L
    st = settings(PIPELINE)
    raw = open(os.path.join(GOLDEN_DIR, PIPELINE["fisher_grid"]), "rb").read()
    fis = np.frombuffer(raw[132:260], dtype="<f8").reshape(4, 4)
    return L.coinc_cfg(N=st["N"], oms=st["oms"], vedva_m=L.vedva(fis), refr=PIPELINE["refr"],
                       mincoin=PIPELINE["mincoin"], snrcutoff=PIPELINE["snrcutoff"], narrowdown=PIPELINE["narrowdown"])


def test_pipeline_fp64_matches_reference(tmp_path, gpu_ok):
    from polgraw_gb300 import lib as L
    g = golden("pipeline_h1l1")
    seg, cand = _search(tmp_path, "fp64")
    assert seg["files"] == g["inputs"], "synthetic inputs differ from the golden run's"
    assert sorted(os.listdir(cand)) == sorted(g["trigger_files"])
    by_frame = {}
    for name, ref in g["trigger_files"].items():
        ours = np.fromfile(os.path.join(cand, name), dtype="<f8").reshape(-1, 5)
        ref = np.array(ref).reshape(-1, 5)
        assert ours.shape == ref.shape, name
        assert np.array_equal(ours[:, :4], ref[:, :4]), name
        assert np.abs(ours[:, 4] - ref[:, 4]).max() <= 1e-9 * ref[:, 4].max(), name
        by_frame[int(re.match(r"triggers_(\d+)_", name).group(1))] = ours
    cc = L.Coinc(_coinc_cfg())
    for f in g["order"]:
        cc.add_frame(f, by_frame[f])
    res = cc.run()
    cc.close()
    assert res.frameinfo.tolist() == g["frameinfo"]
    mine = parse_coi(res.coi_bytes())
    ref = parse_coi(base64.b64decode(g["coi_b64"]))
    assert len(mine) == len(ref)
    for (w1, m1, f1, o1), (w2, m2, f2, o2) in zip(mine, ref):
        assert w1 == w2 and np.array_equal(f1, f2) and np.array_equal(o1, o2)
        if w1:
            assert np.array_equal(m1[:4], m2[:4])
            assert abs(m1[4] - m2[4]) <= 1e-6 * abs(m2[4])
    assert res.summary.maxcoin == len(PIPELINE["frames"])


def test_pipeline_mixed_finds_the_injection(tmp_path, gpu_ok):
    from polgraw_gb300 import build
    g = golden("pipeline_h1l1")
    seg, cand = _search(tmp_path, "mixed")
    grid = str(tmp_path / "grid")
    write_fisher_grid(grid, PIPELINE)
    out = str(tmp_path / "coinc")
    r = subprocess.run([build.COINC_EXE] + coinc_args(cand, grid, out, PIPELINE), capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ours, ref = r.stderr.split(), g["stderr"].split()
    # multiplicity (field 5) and the means of f, s, delta, alpha (fields 6-9)
    assert int(ours[4]) == int(ref[4]) == len(PIPELINE["frames"])
    for j in range(5, 9):
        assert abs(float(ours[j]) - float(ref[j])) <= 1e-6 * max(1.0, abs(float(ref[j]))), (j, ours[j], ref[j])
    assert abs(float(ours[9]) - float(ref[9])) <= 1e-4 * float(ref[9])
    # the participating frames, as a set (the directory order may differ)
    nf = len(PIPELINE["frames"])
    assert sorted(int(x) for x in ours[-int(ours[4]):]) == sorted(int(x) for x in ref[-int(ref[4]):])
    assert int(ours[3]) == nf
