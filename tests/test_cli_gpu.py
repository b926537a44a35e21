"""The drop-in program gwsearch-gb300 end to end on the GPU: same command
line as the reference search, trigger files compared with the reference's
(golden) records."""
import glob
import os
import subprocess

import numpy as np
import pytest

from helpers import case_by_name, golden, compare_candidates
from casegen import materialize

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["h1_addsig", "h1l1_gaps_veto", "h1_fullgrid", "h1l1v1_addsig",
                                  "h1v1_lines_usedet", "h1l1_label_pm2",
                                  "h1l1_amp_fpo", "ref_testdata_001", "ref_testdata_001_l1"])
@pytest.mark.parametrize("skybatch", ["1", "7", "7g"])
def test_cli_trigger_files(name, skybatch, tmp_path, lib, gpu_ok):
    """'7g': 7 sky points per batch, each batch captured as a CUDA graph."""
    from polgraw_gb300 import build
    g = golden(name)
    data = str(tmp_path / "data")
    os.makedirs(data)
    m = materialize(case_by_name(name), data)
    out = str(tmp_path / "out")
    cmd = [build.EXE] + m["args"] + ["-output", out, "-skybatch", skybatch.rstrip("g")]
    if skybatch.endswith("g"):
        cmd += ["-graphs", "1"]
    r = subprocess.run(cmd, cwd=str(tmp_path), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert sorted(os.path.basename(p) for p in glob.glob(out + "/*")) == g["trigger_files"]
    recs = np.concatenate([np.fromfile(p, dtype="<f8").reshape(-1, 5) for p in sorted(glob.glob(out + "/*"))]) \
        if g["trigger_files"] else np.zeros((0, 5))
    ref = np.array([c[5:] for c in g["candidates"]]).reshape(-1, 5)
    # match records by (f, s1, delta, alpha), which encode the indices exactly
    rk = [tuple(x) for x in ref[:, :4]]
    gk = [tuple(x) for x in recs[:, :4]]
    rF = list(ref[:, 4] ** 2 / 2 + 2)
    gF = list(recs[:, 4] ** 2 / 2 + 2)
    trl = float(g["args"][g["args"].index("-threshold") + 1]) if "-threshold" in g["args"] else 20.0
    # keys here are record tuples; compare as sets with threshold-edge slack
    missing = [(k, F) for k, F in zip(rk, rF) if k not in set(gk) and abs(F - trl) > 1e-4 * trl]
    extra = [(k, F) for k, F in zip(gk, gF) if k not in set(rk) and abs(F - trl) > 1e-4 * trl]
    assert len(missing) <= 0 and len(extra) <= 0, (missing[:5], extra[:5])
    common = {k: F for k, F in zip(rk, rF)}
    err = max([abs(F - common[k]) / common[k] for k, F in zip(gk, gF) if k in common], default=0)
    assert err < 1e-4
    # state file emptied at the end (main.c:142-147)
    st = glob.glob(str(tmp_path / "state_*.dat"))
    assert st and all(os.path.getsize(p) == 0 for p in st)
