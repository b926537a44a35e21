"""pa_fstat_noalloc: the F-statistic entry point for callers that cannot
allocate device memory (for example a plugin inside an application that owns
the GPU memory budget, or code that must not grow its footprint after
start-up).  It keeps every device buffer in one static array inside the
library instead of calling cudaMalloc.

The test calls it through the C-ABI several times in a row, on inputs of
different sizes (one, three and two detectors; the last with fftpad 2, so
that nfftf = 2^15 takes the two-detector radix-16 spindown kernel), so that
each call runs on what the previous, differently laid out call left in the
array.  Each result must equal pa_debug_fstat() of an ordinary context of the
same form (mixed precision, fixed-point phase, the same default FFT split)
bit for bit: both run the same kernels on the same inputs, so any difference
would be a stale or aliased buffer in the static layout.  Device free memory
must not change across warmed calls, and sizes beyond the array's limits are
rejected with PA_ERR_ARG.  This file is collected last so that a failure here
comes after every other test has run.
"""
import numpy as np
import pytest

from helpers import case_by_name, make_host

pytestmark = pytest.mark.gpu

# two detectors, N = 10771, nfft = 16384, fftpad 2: nfftf = 32768
H1L1_PAD2 = dict(name="noalloc_h1l1_pad2",
                 data=dict(dets=["H1", "L1"], dt=8.0, nod=1, band=90, fftpad=2,
                           grid=dict(m5=-1.2e-8, m4=2.1e-4, sky_scale=0.05)),
                 range=[-3, 3, -1, 1, -1, 1, 1, 1],
                 args=["-threshold", "11"])


def _inside(s, p):
    return ((p[2] * s.M[10] + p[1] * s.M[14]) ** 2 + (p[2] * s.M[11] + p[1] * s.M[15]) ** 2) / s.oms ** 2 <= 1.0


def _setups(tmp_path):
    from polgraw_gb300.lib import Context, PA_PREC_MIXED, PA_PHASE_FIXED
    out = []
    for case in (case_by_name("h1l1v1_addsig"), case_by_name("h1_addsig"), H1L1_PAD2):
        host, _ = make_host(case, str(tmp_path / case["name"]))
        dets, nifo = host.detectors()
        s = host.settings
        ctx = Context(s, dets, nifo, precision=PA_PREC_MIXED, phase_mode=PA_PHASE_FIXED)
        pts = [p for p in host.sky_points() if _inside(s, p)]
        out.append(dict(host=host, dets=dets, nifo=nifo, ctx=ctx, pts=pts))
    assert [o["nifo"] for o in out] == [3, 1, 2]
    assert out[2]["host"].settings.nfftf == 1 << 15
    return out


def test_fstat_noalloc_matches_context(tmp_path, gpu_ok):
    from polgraw_gb300.lib import fstat_noalloc
    setups = _setups(tmp_path)
    # two calls in a row per input, alternating sizes so that every call runs
    # on the array as a differently laid out call left it
    for rep in range(2):
        for k, su in enumerate(setups):
            host, s = su["host"], su["host"].settings
            opts, rng = host.opts(), host.range
            pm, mm, nn = su["pts"][(rep * 3 + k) % len(su["pts"])]
            for ss in (rng.spndr[0] + rep, rng.spndr[1] - rep):
                want = su["ctx"].fstat(pm, mm, nn, ss, opts)
                got = fstat_noalloc(s, su["dets"], su["nifo"], pm, mm, nn, ss, opts)
                assert np.all(np.isfinite(got))
                assert np.array_equal(got, want), (su["nifo"], ss, np.abs(got - want).max() / np.mean(want))
    for su in setups:
        su["ctx"].close()


def test_fstat_noalloc_allocates_nothing(tmp_path, gpu_ok):
    """Free device memory is the same before and after warmed calls (the
    first call loaded the kernels)."""
    torch = pytest.importorskip("torch")
    from polgraw_gb300.lib import fstat_noalloc
    host, _ = make_host(case_by_name("h1_addsig"), str(tmp_path))
    dets, nifo = host.detectors()
    s, opts, rng = host.settings, host.opts(), host.range
    pm, mm, nn = next(p for p in host.sky_points() if _inside(s, p))
    fstat_noalloc(s, dets, nifo, pm, mm, nn, rng.spndr[0], opts)
    torch.cuda.synchronize(0)
    free0, _ = torch.cuda.mem_get_info(0)
    for ss in (rng.spndr[0], rng.spndr[0] + 1, rng.spndr[0] + 2):
        fstat_noalloc(s, dets, nifo, pm, mm, nn, ss, opts)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)


def test_fstat_noalloc_rejects_large_sizes(tmp_path, gpu_ok):
    from polgraw_gb300.lib import SearchError, fstat_noalloc, load
    host, _ = make_host(case_by_name("h1l1_white_pm2"), str(tmp_path))   # N = 21541
    dets, nifo = host.detectors()
    s, opts, rng = host.settings, host.opts(), host.range
    assert s.N > 16384
    pm, mm, nn = next(p for p in host.sky_points() if _inside(s, p))
    with pytest.raises(SearchError, match="beyond the no-allocation limits"):
        fstat_noalloc(s, dets, nifo, pm, mm, nn, rng.spndr[0], opts)
    assert "N <= 16384" in load().pa_last_error(None).decode()
