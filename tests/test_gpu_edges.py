"""Edge cases of the search boundary on the GPU:

* the caller's record buffer too small: PA_ERR_CAPACITY with *needed, the
  buffer and counters untouched, the same call with room succeeds;
* the device candidate buffer (2^18 candidates) overflowing: the context
  grows it and re-runs the batch, with the same records as a later run;
* an empty batch and sky points outside the grid disk (jobcore.c:248): no
  records, FNum unchanged;
* a crash between sky points (host-side fault injection) and the restart
  from the state file.
"""
import ctypes as C
import os

import numpy as np
import pytest

from casegen import materialize
from helpers import case_by_name, key_of, make_host

pytestmark = pytest.mark.gpu


def _ctx(host, **kw):
    from polgraw_gb300.lib import Context
    dets, nifo = host.detectors()
    return Context(host.settings, dets, nifo, **kw)


def test_caller_capacity(tmp_path, gpu_ok):
    from polgraw_gb300 import lib as L
    host, _ = make_host(case_by_name("h1l1_gaps_veto"), str(tmp_path))
    ctx = _ctx(host)
    tasks = list(host.sky_points())
    rec, idx, fnum = ctx.search_batch(tasks, host.opts(), host.range)
    n = len(rec)
    assert n > 2
    arr = (L.Sky * len(tasks))(*[L.Sky(*t) for t in tasks])
    sgnlc, fn, needed = C.c_int(0), C.c_int(0), C.c_int(0)
    cap = n - 1
    buf = np.full((cap, L.PA_NPAR), -7.0)
    ids = (L.CandIdx * cap)()
    rc = ctx.lib.pa_search_batch(ctx.ctx, arr, len(tasks), C.byref(host.opts()), C.byref(host.range),
                                 C.byref(sgnlc), buf.ctypes.data_as(C.POINTER(C.c_double)), cap, ids,
                                 C.byref(fn), C.byref(needed))
    assert rc == L.PA_ERR_CAPACITY
    assert needed.value == n and sgnlc.value == 0 and fn.value == 0
    assert np.all(buf == -7.0)
    rec2, idx2, fnum2 = ctx.search_batch(tasks, host.opts(), host.range, cap=n)
    assert np.array_equal(rec, rec2) and key_of(idx) == key_of(idx2) and fnum == fnum2


def test_device_candidate_overflow_regrows(tmp_path, gpu_ok):
    # threshold 5 on the N=258492, nfftf=524288 data: runs above it start at
    # ~2% of the 258048 bins of a spindown, more than the 2^18 candidates the
    # device buffer starts with for 7 sky points x 13 spindowns
    from polgraw_gb300 import workloads
    from polgraw_gb300.lib import Host
    root = str(tmp_path / "stress")
    cmd, inj = workloads.stress(root, 400)
    host = Host(cmd + ["-threshold", "5"])
    rng = host.range
    rng.spndr[0], rng.spndr[1], rng.sst = -6, 6, -6
    tasks = [workloads.nearest_sky(host, j) for j in inj]
    tasks += [(1, 0, 0), (1, 1, 1), (1, 2, 2), (1, -1, 1)]
    ctx = _ctx(host)
    rec1, idx1, f1 = ctx.search_batch(tasks, host.opts(), rng, cap=1 << 21)
    assert len(rec1) > (1 << 18)
    rec2, idx2, f2 = ctx.search_batch(tasks, host.opts(), rng, cap=1 << 21)
    assert np.array_equal(rec1, rec2) and key_of(idx1) == key_of(idx2) and f1 == f2 == 13 * len(tasks)


def test_empty_batch_and_outside_disk(tmp_path, gpu_ok):
    host, _ = make_host(case_by_name("h1_addsig"), str(tmp_path))
    ctx = _ctx(host)
    rec, idx, fnum = ctx.search_batch([], host.opts(), host.range)
    assert len(rec) == 0 and fnum == 0
    s = host.settings
    # a lattice point far outside the disk (al1^2 + al2^2 > oms^2)
    far = int(3 * s.oms / max(abs(s.M[10]), abs(s.M[15]))) + 1
    rec, idx, fnum = ctx.job_core(1, far, far, host.opts(), host.range)
    assert len(rec) == 0 and fnum == 0


def test_crash_and_resume(tmp_path, gpu_ok):
    """Host-side fault injection: gwsearch-gb300 stopped like a crash after
    writing the state file of its 4th sky point (PA_HOST_STOP_AT_SKY), then
    restarted with the same command.  As in the reference (jobcore.c:100-104,
    init.c:885-907, and the candidates it admits losing at jobcore.c:171):
    the candidates buffered before the crash are lost, the run resumes at the
    recorded sky point, and the final trigger file equals the uninterrupted
    run's records from that sky point on; the state file is emptied at the
    end."""
    import subprocess
    from polgraw_gb300 import build
    data = str(tmp_path / "data")
    os.makedirs(data)
    m = materialize(case_by_name("h1l1_gaps_veto"), data)
    name = "triggers_001_0200_1.bin"

    def run(cwd, env=None):
        os.makedirs(cwd, exist_ok=True)
        e = dict(os.environ)
        e.update(env or {})
        return subprocess.run([build.EXE] + m["args"] + ["-output", os.path.join(cwd, "out")], cwd=cwd,
                              capture_output=True, text=True, timeout=600, env=e)

    full = str(tmp_path / "full")
    r = run(full)
    assert r.returncode == 0, r.stderr[-2000:]
    A = np.fromfile(os.path.join(full, "out", name), dtype="<f8").reshape(-1, 5)
    crash = str(tmp_path / "crash")
    r = run(crash, {"PA_HOST_STOP_AT_SKY": "4"})
    assert r.returncode == 3, (r.returncode, r.stderr[-2000:])
    st = open(os.path.join(crash, "state_001_0200.dat")).read().split()
    assert len(st) == 5                                   # pm mm nn sst FNum of the 4th sky point
    assert not os.path.exists(os.path.join(crash, "out", name))   # nothing flushed before the crash
    r = run(crash)                                        # restart: resumes from the state file
    assert r.returncode == 0, r.stderr[-2000:]
    C = np.fromfile(os.path.join(crash, "out", name), dtype="<f8").reshape(-1, 5)
    assert 0 < len(C) < len(A)
    assert np.array_equal(C, A[len(A) - len(C):])        # the tail of the uninterrupted run
    lost = A[:len(A) - len(C)]
    assert not ({tuple(x) for x in lost[:, 2:4]} & {tuple(x) for x in C[:, 2:4]})   # whole sky points lost
    assert os.path.getsize(os.path.join(crash, "state_001_0200.dat")) == 0
