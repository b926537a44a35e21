"""Followup on the GPU: the demodulated network F-statistic (pa_fstatnet),
its adjoint gradient (pa_fstatnet_grad), gradient ascent and the batched
reference simplex, checked against the reference followup program's own
outputs (tests/golden/fu_h1l1v1.json, made from followup/src/followup.c) and
the FP64 oracle gradient.

Tolerances: F within 1e-4 relative (mixed: FP32 data with the FP64 phase or
the compensated two-float phase) and 1e-10 (FP64 form); gradients compared in peak-width units, w_j dF/dtheta_j, to
2e-3 (mixed) and 1e-8 (FP64) of the largest component at the point.
"""
import numpy as np
import pytest

from casegen import materialize
from cases import FOLLOWUP_CASES
from helpers import golden

pytestmark = pytest.mark.gpu

# (precision, F tolerance, gradient tolerance, phase form)
FORMS = {"mixed": (0, 1e-4, 2e-3, 0), "mixed-ffphase": (0, 1e-4, 2e-3, 2), "fp64": (1, 1e-10, 1e-8, 0)}


def _load_case(case, tmp_path_factory):
    from polgraw_gb300.lib import Host
    from pyoracle import FollowupOracle
    g = golden(case["name"])
    tmp = tmp_path_factory.mktemp("fu")
    data = tmp / "data"
    data.mkdir()
    m = materialize(case, str(data))
    assert m["ds"].files == g["inputs"], "synthetic inputs differ from the golden run's"
    host = Host(m["args"] + ["-output", str(tmp / "out"), "--nocheckpoint"])
    dets, nifo = host.detectors()
    return host, dets, nifo, g, FollowupOracle(host.settings, dets, nifo), case


@pytest.fixture(scope="module", params=[c["name"] for c in FOLLOWUP_CASES])
def fu_case(tmp_path_factory, request):
    return _load_case([c for c in FOLLOWUP_CASES if c["name"] == request.param][0], tmp_path_factory)


@pytest.fixture(scope="module")
def fu_first_case(tmp_path_factory):
    return _load_case(FOLLOWUP_CASES[0], tmp_path_factory)


def _fu(fu_case, form):
    from polgraw_gb300.lib import Followup
    host, dets, nifo, g = fu_case[:4]
    return Followup(host.settings, dets, nifo, precision=FORMS[form][0], phase_mode=FORMS[form][3])


@pytest.mark.parametrize("form", list(FORMS))
def test_fstatnet_matches_reference(form, fu_case, gpu_ok):
    g = fu_case[3]
    fu = _fu(fu_case, form)
    out = fu.fstatnet(g["points"])
    ref = np.array(g["fstatnet"])
    tol = FORMS[form][1]
    F, Fr = -out[:, 5], -ref[:, 5]
    assert np.abs(F - Fr).max() / Fr.max() < tol, np.abs(F - Fr) / Fr.max()
    # amplitude estimates and SNRs, relative to their scale at each point
    amp = np.abs(ref[:, :4]).max(axis=1, keepdims=True)
    assert np.abs(out[:, :4] - ref[:, :4]).max() <= 10 * tol * amp.max()
    assert np.allclose(out[:, 6:10], ref[:, 6:10], rtol=0, atol=0)
    assert np.abs(out[:, 10] - ref[:, 10]).max() / ref[:, 10].max() < 10 * tol


@pytest.mark.parametrize("form", list(FORMS))
def test_batch_independent(form, fu_case, gpu_ok):
    g = fu_case[3]
    fu = _fu(fu_case, form)
    pts = np.array(g["points"])
    whole = fu.fstatnet(pts)
    for k in (0, 5, len(pts) - 1):
        one = fu.fstatnet(pts[k:k + 1])
        assert np.array_equal(one[0], whole[k])


@pytest.mark.parametrize("form", list(FORMS))
def test_adjoint_gradient_matches_fp64_oracle(form, fu_case, gpu_ok):
    g, ora = fu_case[3], fu_case[4]
    fu = _fu(fu_case, form)
    w = np.array(g["widths"])
    pts = np.array(g["points"])
    F, grad = fu.fstatnet_grad(pts)
    out = fu.fstatnet(pts)
    assert np.allclose(F, -out[:, 5], rtol=1e-12, atol=0)
    tol = FORMS[form][2]
    for k, p in enumerate(pts):
        Fo, go = ora.fstatnet_grad(p)
        scale = np.abs(w * go).max()
        err = np.abs(w * (grad[k] - go)).max()
        assert err <= tol * scale, (k, w * grad[k], w * go)
    # seeds scale the gradient
    seed = np.linspace(0.5, 2.0, len(pts))
    _, gs = fu.fstatnet_grad(pts, seed=seed)
    want = w * grad * seed[:, None]
    rel = np.abs(w * gs - want).max(axis=1) / np.abs(want).max(axis=1)
    assert rel.max() <= (FORMS[form][2] if form != "fp64" else 1e-12), rel


def test_adjoint_matches_finite_differences_fp64(fu_case, gpu_ok):
    """Central differences of the GPU's own FP64 F against its adjoint."""
    g = fu_case[3]
    fu = _fu(fu_case, "fp64")
    w = np.array(g["widths"])
    for p in np.array(g["points"])[1:5]:
        F, grad = fu.fstatnet_grad(p)
        fd = np.zeros(4)
        for j in range(4):
            h = np.zeros(4)
            h[j] = 1e-4 * w[j]
            o = fu.fstatnet(np.stack([p + h, p - h]))
            fd[j] = (-o[0, 5] + o[1, 5]) / (2 * h[j])
        scale = np.abs(w * grad[0]).max()
        assert np.abs(w * (grad[0] - fd)).max() <= 1e-5 * scale


def test_autograd_function(fu_first_case, gpu_ok):
    """The adjoint behind a torch.autograd.Function (test harness only; the
    wrapper's plumbing, checked on the first followup case): the backward
    pass returns grad_output * dF/dtheta, the directional derivative matches a
    central difference, and an optimiser step in peak-width units raises F."""
    torch = pytest.importorskip("torch")
    g = fu_first_case[3]
    fu = _fu(fu_first_case, "mixed")
    w = torch.tensor(g["widths"], dtype=torch.float64)

    class Fstat(torch.autograd.Function):
        @staticmethod
        def forward(ctx, theta):
            F, grad = fu.fstatnet_grad(theta.detach().cpu().numpy())
            ctx.save_for_backward(torch.from_numpy(grad))
            return torch.from_numpy(F)

        @staticmethod
        def backward(ctx, gout):
            (grad,) = ctx.saved_tensors
            return gout[:, None] * grad

    pts = torch.tensor(g["points"][1:9], dtype=torch.float64)
    u = (pts / w).clone().requires_grad_(True)   # peak-width units
    F0 = Fstat.apply(u * w)
    F0.sum().backward()
    # the gradient at the points the forward pass evaluated ((pts / w) * w can
    # differ from pts in the last bit, which moves a mixed-form gradient)
    _, grad = fu.fstatnet_grad((u.detach() * w).numpy())
    assert torch.allclose(u.grad, torch.from_numpy(grad) * w, rtol=1e-12, atol=0)
    # the directional derivative along the gradient matches a central
    # difference of F (curvature cancels; tolerance covers the FP32 noise of F)
    d = u.grad / u.grad.norm(dim=1, keepdim=True)
    h = 1e-3
    with torch.no_grad():
        Fp = Fstat.apply((u + h * d) * w)
        Fm = Fstat.apply((u - h * d) * w)
    fd = (Fp - Fm) / (2 * h)
    slope = (u.grad * d).sum(dim=1)
    assert torch.allclose(fd, slope, rtol=2e-2, atol=0), (fd, slope)
    # one optimiser step of 0.01 peak widths along the normalised gradient
    # raises the summed F
    u.grad = d.clone()
    opt = torch.optim.SGD([u], lr=1e-2, maximize=True)
    opt.step()
    with torch.no_grad():
        F1 = Fstat.apply(u * w)
    assert float(F1.sum()) > float(F0.detach().sum())


@pytest.mark.parametrize("form", list(FORMS))
def test_simplex_matches_reference(form, fu_case, gpu_ok):
    g = fu_case[3]
    fu = _fu(fu_case, form)
    am = g["amoeba"]
    starts = np.array([a["start"] for a in am])
    pts, out, nev = fu.simplex(starts, am[0]["pc2"], tol=am[0]["tol"], max_evals=5000)
    w = np.array(g["widths"])
    Fr_all = [-a["out"][5] for a in am]
    for k, a in enumerate(am):
        Fr = -a["out"][5]
        # F of the reference's maximum within 10x the F tolerance; in the FP64
        # form also its point (0.05 widths).  The simplex path is chaotic:
        # rounding-level F differences of the mixed forms can turn a
        # comparison and end it on a side maximum of the same F level, or at
        # another point of a ridge along which the reference's own runs stop
        # at different heights (fu_h1l1v1_n86164: 172.19 to 172.40); a mixed
        # run must then still end as high as the lowest of the reference's
        # runs, and the best mixed run at the reference's best.
        if form == "fp64":
            assert -out[k, 5] >= Fr * (1 - 10 * FORMS[form][1]), (k, -out[k, 5], Fr)
        else:
            assert -out[k, 5] >= min(Fr_all) * (1 - 10 * FORMS[form][1]), (k, -out[k, 5], Fr_all)
        if form == "fp64":
            assert np.abs((pts[k] - np.array(a["point"])) / w).max() < 0.05
        if form == "fp64":
            assert abs(int(nev[k]) - a["nevals"]) <= 0.2 * a["nevals"]
    assert (-out[:, 5]).max() >= max(Fr_all) * (1 - 10 * FORMS[form][1]), (-out[:, 5], Fr_all)
    # the batch of three and each start alone give the same result
    p1, o1, n1 = fu.simplex(starts[1:2], am[0]["pc2"], tol=am[0]["tol"], max_evals=5000)
    assert np.array_equal(p1[0], pts[1]) and n1[0] == nev[1]


def _oracle_ascent(orc, start, w, step0, min_step, max_iter):
    """The ascent of pa_followup_ascent (BFGS on -F in peak-width units
    u = theta / w, backtracking line search with the sufficient-increase
    factor 1e-4, inverse-Hessian update when y.s > 0, stop when the step
    falls below min_step, the slope is not positive, or after max_iter
    accepted steps) restated in FP64 on the oracle's F and gradient.
    Returns (end point, F there, accepted steps)."""
    theta = np.array(start, dtype=np.float64)
    F, g = orc.fstatnet_grad(theta)
    gu = w * g
    nrm = np.linalg.norm(gu)
    if not nrm > 0:
        return theta, F, 0
    H = np.eye(4) * (step0 / nrm)
    t, iters = 1.0, 0
    while iters < max_iter:
        p = H @ gu
        slope = float(p @ gu)
        if not slope > 0 or t * np.linalg.norm(p) < min_step:
            break
        trial = theta + w * t * p
        Ft = -orc.fstatnet(trial)[5]
        if Ft >= F + 1e-4 * t * slope and Ft > F:
            s = t * p
            gold = gu
            theta, F = trial, Ft
            _, g = orc.fstatnet_grad(theta)
            gu = w * g
            y = gold - gu
            ys = float(y @ s)
            if ys > 0:
                r = 1.0 / ys
                Hy = H @ y
                H = H - r * (np.outer(s, Hy) + np.outer(Hy, s)) + (r * r * float(y @ Hy) + r) * np.outer(s, s)
            t = 1.0
            iters += 1
        else:
            t *= 0.5
    return theta, F, iters


@pytest.mark.parametrize("form", list(FORMS))
def test_ascent_reaches_simplex_maximum(form, fu_case, gpu_ok):
    g, orc = fu_case[3], fu_case[4]
    fu = _fu(fu_case, form)
    w = np.array(g["widths"])
    starts = np.array(g["points"][1:])
    F0 = -fu.fstatnet(starts)[:, 5]
    pts, out, it = fu.ascent(starts, w, step0=0.25, min_step=1e-4, max_iter=200)
    F1 = -out[:, 5]
    assert np.all(F1 >= F0)
    Fmax = max(-a["out"][5] for a in g["amoeba"])
    # the best start reaches the peak the reference simplex found
    assert F1.max() >= Fmax * (1 - 1e-3), (F1, Fmax)
    if fu_case[5].get("unimodal"):
        # no other maximum within 0.5 widths of the injection: every start
        # reaches its peak
        assert np.all(F1 >= Fmax * (1 - 1e-3)), (F1, Fmax)
    # every path, not only the best: the same ascent in FP64 on the oracle
    # from each start.  Every start off a stationary point takes at least one
    # step; every end point is a stationary point of the oracle's F, not
    # below the start; in the FP64 form each path ends where the oracle's
    # does (F and point).  A mixed-precision path may part from the FP64 one
    # where several stationary points lie within half a width (fu_h1l1_dt2:
    # maxima near 151.6 and 152.1, and flat saddles between them, where the
    # rounding noise of the FP32 gradient can end the ascent): it must then
    # still end on a stationary point of the oracle's F within 1 % of the
    # oracle path's F.  On fu_h1l1v1, whose F has no other stationary point
    # within half a width of the peak, no path may part.
    ftol = FORMS[form][1]
    worst_f = worst_p = worst_g = 0.0
    parted = []
    for k, st in enumerate(starts):
        Fs, gs = orc.fstatnet_grad(st)
        if np.abs(w * gs).max() > 1e-2 * Fs:
            assert it[k] > 0, (k, np.abs(w * gs).max() / Fs)
        pe, Fe, ie = _oracle_ascent(orc, st, w, 0.25, 1e-4, 200)
        Fg, gg = orc.fstatnet_grad(pts[k])
        assert Fg >= Fs * (1 - ftol), (k, Fg, Fs)
        worst_g = max(worst_g, float(np.abs(w * gg).max() / Fg))
        # stationary: the gradient (width units) below 2e-3 of F in the FP64
        # form; the mixed forms' FP32 gradient carries noise of a few 1e-3
        # of F per width, where their ascent may stop
        gtol = 2e-3 if form == "fp64" else 1e-2
        assert np.abs(w * gg).max() <= gtol * Fg, (k, np.abs(w * gg).max() / Fg)
        if abs(Fg - Fe) > 1e-3 * Fe:
            assert form != "fp64", (k, Fg, Fe)
            assert abs(Fg - Fe) <= 1e-2 * Fe, (k, Fg, Fe)
            parted.append((k, round(Fg, 3), round(Fe, 3)))
            continue
        worst_f = max(worst_f, abs(Fg - Fe) / Fe)
        worst_p = max(worst_p, float(np.abs((pts[k] - pe) / w).max()))
        if form == "fp64":
            assert np.abs((pts[k] - pe) / w).max() < 1e-2, (k, (pts[k] - pe) / w)
    if fu_case[5].get("unimodal"):
        assert not parted, parted
    print("\nascent %s %s: vs FP64-oracle ascent max rel F diff %.2e, max point diff %.2e widths, "
          "max |w grad|/F at the end %.2e, paths ending on another maximum %s"
          % (form, fu_case[5]["name"], worst_f, worst_p, worst_g, parted))
