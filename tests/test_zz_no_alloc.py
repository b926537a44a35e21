"""pa_fstat_noalloc: the F-statistic entry point for callers that cannot
allocate device memory (for example a plugin inside an application that owns
the GPU memory budget).  It keeps every device buffer in one static array
inside the library instead of calling cudaMalloc.

The test calls it through the C-ABI twice in a row (two spindowns of one sky
point, so the second call runs on the contents the first one left behind)
and compares each result with pa_debug_fstat() of an ordinary context of the
same form (mixed precision, fixed-point phase), within the F-statistic
tolerance the other GPU tests use (1e-4 of the mean F level).  This file is
collected last so that a failure here comes after every other test has run.
"""
import numpy as np
import pytest

from helpers import case_by_name, make_host

pytestmark = pytest.mark.gpu

TOL = 1e-4


def test_fstat_noalloc_matches_context(tmp_path, gpu_ok):
    from polgraw_gb300.lib import Context, fstat_noalloc, PA_PREC_MIXED, PA_PHASE_FIXED
    host, _ = make_host(case_by_name("h1_addsig"), str(tmp_path))
    dets, nifo = host.detectors()
    s = host.settings
    opts, rng = host.opts(), host.range
    ctx = Context(s, dets, nifo, precision=PA_PREC_MIXED, phase_mode=PA_PHASE_FIXED)
    # a sky point inside the grid disk
    pm, mm, nn = next(p for p in host.sky_points()
                      if ((p[2] * s.M[10] + p[1] * s.M[14]) ** 2 + (p[2] * s.M[11] + p[1] * s.M[15]) ** 2)
                      / s.oms ** 2 <= 1.0)
    for ss in (rng.spndr[0], rng.spndr[0] + 2):
        want = ctx.fstat(pm, mm, nn, ss, opts)
        got = fstat_noalloc(s, dets, nifo, pm, mm, nn, ss, opts)
        lvl = float(np.mean(want))
        assert np.all(np.isfinite(got))
        assert np.abs(got - want).max() / lvl < TOL, (ss, np.abs(got - want).max() / lvl)
