"""The followup oracle (demodulated F-statistic, FP64 gradient, simplex)
against the reference followup program's own outputs (fixtures made by
tests/golden/make_followup_golden.py from followup/src/followup.c), and the
oracle's analytic gradient against central finite differences of its own
F-statistic.  CPU only."""
import numpy as np
import pytest

from casegen import materialize
from cases import FOLLOWUP_CASES
from helpers import golden


@pytest.fixture(scope="module", params=[c["name"] for c in FOLLOWUP_CASES])
def fu(tmp_path_factory, request):
    from polgraw_gb300.lib import Host
    from pyoracle import FollowupOracle
    case = [c for c in FOLLOWUP_CASES if c["name"] == request.param][0]
    g = golden(case["name"])
    tmp = tmp_path_factory.mktemp("fu")
    data = tmp / "data"
    data.mkdir()
    m = materialize(case, str(data))
    assert m["ds"].files == g["inputs"], "synthetic inputs differ from the golden run's"
    host = Host(m["args"] + ["-output", str(tmp / "out"), "--nocheckpoint"])
    dets, nifo = host.detectors()
    ora = FollowupOracle(host.settings, dets, nifo)
    return host, ora, g


def test_fstatnet_matches_reference(fu):
    _, ora, g = fu
    for p, ref in zip(g["points"], g["fstatnet"]):
        out = ora.fstatnet(p)
        ref = np.array(ref)
        # all 11 values of fstat_out; same expressions and order -> ~exact
        assert np.allclose(out, ref, rtol=1e-12, atol=0), (p, out - ref)


def test_amoeba_matches_reference(fu):
    _, ora, g = fu
    for a in g["amoeba"]:
        pt, out, nev = ora.amoeba(a["start"], a["pc2"], a["tol"])
        assert nev == a["nevals"]
        assert np.allclose(pt, a["point"], rtol=1e-12, atol=0)
        assert np.allclose(out, a["out"], rtol=1e-12, atol=0)
        # the simplex ends above the F-statistic of its start
        assert -out[5] >= -ora.fstatnet(a["start"])[5]


def test_gradient_matches_finite_differences(fu):
    _, ora, g = fu
    w = np.array(g["widths"])
    for p in g["points"][:8]:
        p = np.array(p)
        F, grad = ora.fstatnet_grad(p)
        assert abs(F + ora.fstatnet(p)[5]) <= 1e-9 * F
        fd = np.zeros(4)
        for j in range(4):
            h = np.zeros(4)
            h[j] = 1e-4 * w[j]
            fd[j] = (-ora.fstatnet(p + h)[5] + ora.fstatnet(p - h)[5]) / (2 * h[j])
        # compare the gradients in peak-width units (w * dF/dtheta)
        scale = np.linalg.norm(w * grad) + 1e-3 * F
        assert np.abs(w * (grad - fd)).max() <= 1e-5 * scale, (p, grad, fd)
