"""The coincidence step on the GPU (pa_coinc_*) and the coincidences-gb300
program against the reference coincidence program's outputs
(tests/golden/coinc_*.json) and the CPU oracle (oracle/oracle_coinc.c).

Bar: bit-exact.  Cells, the records each frame's duplicate removal keeps,
per-frame counts, every .coi byte (NaN means of a multiplicity-0 record
compared without their sign bit, which is the machine's) and the stderr
summary line.  The frame order is the reference's directory order recorded
in the golden file, or any other order checked against the oracle run in
that same order."""
import hashlib
import os
import re
import subprocess

import numpy as np
import pytest

from cases import COINC_CASES
from coinc_casegen import materialize, oracle_cfg
from helpers import canon_coi, golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", params=[c["name"] for c in COINC_CASES])
def coinc_case(request, tmp_path_factory, gpu_ok):
    case = [c for c in COINC_CASES if c["name"] == request.param][0]
    g = golden(case["name"])
    root = str(tmp_path_factory.mktemp(case["name"]))
    m = materialize(case, root)
    assert m["files"] == g["files"], "synthetic inputs differ from the golden run's"
    return case, g, m, root


def _device(cfg, order, recs):
    from polgraw_gb300 import lib as L
    cc = L.Coinc(cfg)
    for f in order:
        cc.add_frame(f, recs[f])
    res = cc.run(cells=True)
    assert cc.launches() > 0 or res.summary.raw == 0
    cc.close()
    return res


def _same(a, b):
    """Two results agree in every output the reference writes."""
    assert a.frameinfo.tolist() == b.frameinfo.tolist()
    assert a.summary.inband == b.summary.inband and a.summary.unique == b.summary.unique
    assert a.summary.ncoin == b.summary.ncoin and a.summary.nmembers == b.summary.nmembers
    assert a.summary.maxcoin == b.summary.maxcoin and a.summary.maxcoin_index == b.summary.maxcoin_index
    assert np.array_equal(a.cells, b.cells)
    assert np.array_equal(a.keep, b.keep)
    assert np.array_equal(a.w, b.w) and np.array_equal(a.first, b.first)
    assert np.array_equal(a.fra, b.fra) and np.array_equal(a.ops, b.ops)
    assert canon_coi(a.coi_bytes()) == canon_coi(b.coi_bytes())


def test_device_matches_reference(coinc_case):
    case, g, m, _ = coinc_case
    order = g["order"]
    res = _device(oracle_cfg(case), order, m["recs"])
    assert res.frameinfo.tolist() == g["frameinfo"]
    assert res.summary.unique == g["total"]
    coi = res.coi_bytes()
    assert len(coi) == g["coi_size"]
    assert hashlib.sha256(canon_coi(coi)).hexdigest() == g["coi_canon_sha256"]
    assert res.summary_line("%04d" % case["band"], case["shift"], m["settings"]["fpo"]) == g["stderr"]


def test_device_matches_oracle_any_order(coinc_case):
    """Frame order changes the output (tie order, the rows left over between
    frames); device and oracle agree in every order tried."""
    import pyoracle
    case, g, m, _ = coinc_case
    cfg = oracle_cfg(case)
    frames = sorted(m["recs"])
    for order in (frames, frames[::-1], g["order"][1:] + g["order"][:1]):
        dev = _device(cfg, order, m["recs"])
        ora = pyoracle.coinc(cfg, order, [m["recs"][f] for f in order])
        _same(dev, ora)


def test_cli_matches_oracle(coinc_case):
    """coincidences-gb300 over the trigger directory: its .coi file and
    summary line equal the oracle's for the order it read the directory in."""
    import pyoracle
    from polgraw_gb300 import build
    case, g, m, root = coinc_case
    out = os.path.join(root, "out_gb300")
    args = list(m["args"])
    args[args.index("-output") + 1] = out
    r = subprocess.run([build.COINC_EXE] + args, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    order = [int(x) for x in re.findall(r"Frame (\d+):", r.stdout)]
    assert sorted(order) == sorted(m["recs"])
    ora = pyoracle.coinc(oracle_cfg(case), order, [m["recs"][f] for f in order])
    coi = open(os.path.join(out, os.path.basename(m["coi"])), "rb").read()
    assert canon_coi(coi) == canon_coi(ora.coi_bytes())
    assert r.stderr == ora.summary_line("%04d" % case["band"], case["shift"], m["settings"]["fpo"])
    lines = re.findall(r"Frame (\d+): (\d+)/(\d+)", r.stdout)
    assert [[int(a), int(c), int(b)] for a, b, c in lines] == ora.frameinfo.tolist()


def test_context_reuse_and_reset(gpu_ok):
    from polgraw_gb300 import lib as L
    case = COINC_CASES[0]
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        m = materialize(case, tmp)
    cfg = oracle_cfg(case)
    cc = L.Coinc(cfg)
    outs = []
    for _ in range(2):
        cc.reset()
        for f in sorted(m["recs"]):
            cc.add_frame(f, m["recs"][f])
        outs.append(cc.run(cells=True))
    _same(outs[0], outs[1])
    # a smaller set after a larger one: buffers are reused, nothing leaks over
    cc.reset()
    f0 = sorted(m["recs"])[0]
    cc.add_frame(f0, m["recs"][f0][:100])
    small = cc.run(cells=True)
    import pyoracle
    _same(small, pyoracle.coinc(cfg, [f0], [m["recs"][f0][:100]]))
    cc.close()


def _edge_frames(N, refr):
    from polgraw_gb300 import synth
    recs = synth.coinc_triggers([1, 2, 3], 300, N=N, refr=refr, seed=21, lines=1, sky=2, signals=4)
    out = {1: recs[1], 2: np.zeros((0, 5)), 3: recs[3], 4: np.array([[0.01, 0.0, 0.1, 0.1, 5.0]]),
           5: recs[2][:7]}
    return out


@pytest.mark.parametrize("variant", ["empty_and_cut_frames", "single_frame", "one_cell", "wide_keys",
                                     "no_records"])
def test_edges_match_oracle(variant, gpu_ok):
    """Empty frames, a frame whose records all fail the cuts, one frame, all
    records in one cell (zero key bits), cells spread so far that the key
    needs more than 64 bits, and no records at all."""
    import math
    import pyoracle
    from polgraw_gb300 import lib as L, synth
    case = dict(COINC_CASES[0])
    cfg = oracle_cfg(case)
    N = cfg.N
    recs = _edge_frames(N, case["refr"])
    order = [1, 2, 3, 4, 5]
    if variant == "single_frame":
        order = [3]
    elif variant == "one_cell":
        base = np.array([2.0, 0.0, 0.4, 1.1, 7.0])
        recs = {f: np.stack([base] * (3 + f)) for f in (1, 2, 3)}
        for f in recs:
            recs[f][:, 4] = 6.5 + 0.25 * np.arange(len(recs[f]))[::-1]
        order = [2, 1, 3]
    elif variant == "wide_keys":
        v = np.array(cfg.vedva[:]).reshape(4, 4) * 3.0e4
        cfg = L.coinc_cfg(N=N, oms=cfg.oms, vedva_m=v, shift=0, scale=1111, refr=case["refr"],
                          mincoin=2, narrowdown=0.5, snrcutoff=6.0)
    elif variant == "no_records":
        recs = {1: np.zeros((0, 5)), 2: np.zeros((0, 5))}
        order = [1, 2]
    dev = _device(cfg, order, recs)
    ora = pyoracle.coinc(cfg, order, [recs[f] for f in order])
    _same(dev, ora)
    if variant == "wide_keys":
        c = dev.cells.astype(np.int64)
        bits = sum(int(math.ceil(math.log2(max(2, int(c[:, j].max() - c[:, j].min()) + 1)))) for j in range(4))
        assert bits > 64, bits
    del synth


def test_rejects_bad_config(gpu_ok):
    from polgraw_gb300 import lib as L
    case = COINC_CASES[0]
    cfg = oracle_cfg(case)
    cfg.mincoin = 1
    with pytest.raises(L.SearchError):
        L.Coinc(cfg)
    cfg = oracle_cfg(case)
    cc = L.Coinc(cfg)
    for k in range(255):
        cc.add_frame(k + 1, np.zeros((0, 5)))
    with pytest.raises(L.SearchError):
        cc.add_frame(999, np.zeros((0, 5)))
    cc.close()
