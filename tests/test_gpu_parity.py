"""GPU parity: the CUDA path through the C-ABI against the reference's
golden candidates and the CPU oracle.

Tolerances (relative F-statistic error, the bar of the mixed form):
  mixed precision  : 1e-4 on candidate F, indices identical except at the
                     threshold edge (|F - trl| <= 1e-4 trl) and at argmax
                     ties within 1e-4
  all-FP64 form    : 1e-9 on candidate F
Record fields f, s1, delta, alpha are computed on the host from the indices
with the reference's FP64 expressions and must be bit-identical.
"""
import numpy as np
import pytest

from helpers import (CASES, case_by_name, compare_candidates, golden, key_of, make_host, run_sky_loop)

pytestmark = pytest.mark.gpu

RTOL_MIXED = 1e-4
RTOL_FP64 = 1e-9
FORMS = [("mixed", 0, 1), ("mixed", 0, 0), ("mixed", 0, 2), ("fp64", 1, 0)]
FORM_IDS = ["mixed-fixed", "mixed-f64phase", "mixed-ffphase", "fp64"]


def _ctx(host, precision, phase):
    from polgraw_gb300.lib import Context
    dets, nifo = host.detectors()
    return Context(host.settings, dets, nifo, precision=precision, phase_mode=phase)


def _golden_check(name, tmp_path, precision, phase):
    g = golden(name)
    host, m = make_host(case_by_name(name), str(tmp_path))
    assert m["ds"].files == g["inputs"], "synthetic inputs differ from the golden run's"
    ctx = _ctx(host, precision, phase)
    rec, idx, fnum = run_sky_loop(ctx.job_core, host)
    ref = g["candidates"]
    rkeys = [tuple(c[:5]) for c in ref]
    rF = [c[9] ** 2 / 2 + 2 for c in ref]
    gkeys = key_of(idx)
    gF = list(rec[:, 4] ** 2 / 2 + 2) if len(rec) else []
    trl = host.opts().trl
    rtol = RTOL_FP64 if precision == 1 else RTOL_MIXED
    matched, err, bad = compare_candidates(rkeys, rF, gkeys, gF, trl, rtol)
    assert not bad, bad[:10]
    assert err <= rtol, err
    # records of matched candidates: host-side FP64 fields bit-identical
    R = {k: c[5:9] for k, c in zip(rkeys, ref)}
    for k, r in zip(gkeys, rec):
        if k in R:
            assert list(r[:4]) == R[k], (k, list(r[:4]), R[k])
    per = [1 if host.opts().s0_flag else r[4] - r[3] + 1 for r in g["spindown_ranges"]]
    assert fnum == sum(per)
    return matched, err


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
@pytest.mark.parametrize("name", [c["name"] for c in CASES])
def test_gpu_matches_reference_goldens(name, form, tmp_path, gpu_ok):
    _, precision, phase = form
    matched, err = _golden_check(name, tmp_path, precision, phase)
    assert matched > 0 or not golden(name)["candidates"]


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
def test_gpu_prelude_matches_oracle(form, tmp_path, gpu_ok):
    """Resampled, weighted xDatma/xDatmb and aa, bb (jobcore.c:270-393)."""
    from pyoracle import Oracle
    _, precision, phase = form
    host, _ = make_host(case_by_name("h1l1_gaps_veto"), str(tmp_path))
    dets, nifo = host.detectors()
    ctx = _ctx(host, precision, phase)
    orc = Oracle(host.settings, dets, nifo)
    pm, mm, nn = host.sky_points()[4]
    xa, xb, aa, bb = ctx.prelude(pm, mm, nn)
    o = orc.job_core(pm, mm, nn, host.opts(), host.range, want_prelude=True)
    tol = 1e-12 if precision == 1 else 2e-6
    for got, ref in ((xa, o["pre_a"]), (xb, o["pre_b"])):
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() / scale < tol
    assert abs(aa - o["aa"]) / o["aa"] < (1e-13 if precision == 1 else 1e-6)
    assert abs(bb - o["bb"]) / o["bb"] < (1e-13 if precision == 1 else 1e-6)


@pytest.mark.parametrize("form", FORMS, ids=FORM_IDS)
@pytest.mark.parametrize("white", [0, 1])
def test_gpu_fstat_matches_oracle(form, white, tmp_path, gpu_ok):
    """Normalised F over every bin of one spindown (jobcore.c:635-651)."""
    from pyoracle import Oracle
    _, precision, phase = form
    extra = ["--whitenoise"] if white else []
    host, _ = make_host(case_by_name("h1l1_gaps_veto"), str(tmp_path), extra=extra)
    dets, nifo = host.detectors()
    ctx = _ctx(host, precision, phase)
    orc = Oracle(host.settings, dets, nifo)
    pm, mm, nn = host.sky_points()[4]
    opts, rng = host.opts(), host.range
    ss = rng.spndr[0] + 3
    F = ctx.fstat(pm, mm, nn, ss, opts)
    Fo = orc.job_core(pm, mm, nn, opts, rng, F_ss=ss)["F"]
    # error relative to the mean F level (2 for noise) and on strong bins
    lvl = np.mean(Fo)
    tol = 1e-10 if precision == 1 else 1e-4
    assert np.abs(F - Fo).max() / lvl < tol
    strong = Fo > 8 * lvl
    if strong.any():
        assert (np.abs(F - Fo)[strong] / Fo[strong]).max() < tol


def test_gpu_batch_equals_single(tmp_path, gpu_ok):
    """pa_search_batch over the sky loop == pa_job_core per sky point."""
    host, _ = make_host(case_by_name("h1l1_gaps_veto"), str(tmp_path))
    ctx = _ctx(host, 0, 1)
    rec1, idx1, f1 = run_sky_loop(ctx.job_core, host)
    rng = host.range
    rec2, idx2, f2 = ctx.search_batch(host.sky_points(), host.opts(), rng)
    assert f1 == f2
    assert key_of(idx1) == key_of(idx2)
    np.testing.assert_array_equal(rec1, rec2)


def test_gpu_deterministic(tmp_path, gpu_ok):
    host, _ = make_host(case_by_name("h1_addsig"), str(tmp_path))
    ctx = _ctx(host, 0, 1)
    a = run_sky_loop(ctx.job_core, host)
    b = run_sky_loop(ctx.job_core, host)
    np.testing.assert_array_equal(a[0], b[0])


@pytest.mark.parametrize("sbatch", [1, 3, 64])
def test_gpu_spindown_batch_sizes(sbatch, tmp_path, gpu_ok):
    """The spindown batching of the fused launches does not change results."""
    from polgraw_gb300.lib import Context
    host, _ = make_host(case_by_name("h1l1_gaps_veto"), str(tmp_path))
    dets, nifo = host.detectors()
    ref = run_sky_loop(_ctx(host, 0, 1).job_core, host)
    ctx = Context(host.settings, dets, nifo, precision=0, phase_mode=1, spindown_batch=sbatch)
    got = run_sky_loop(ctx.job_core, host)
    assert key_of(ref[1]) == key_of(got[1])
    np.testing.assert_array_equal(ref[0], got[0])
