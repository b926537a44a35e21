"""Parity at the benchmark's own sizes, against the all-FP64 CPU oracle.

* Network search (H1+L1, N=86164, nfftf=131072, 63488 bins, the benchmark
  workload): 200 sky points of the 2000-point lattice -- the five injections'
  sky points and every tenth lattice point inside the disk -- x the full 200
  spindowns, at the default threshold 20.  Every precision form through
  pa_search_batch with its default (autotuned-size) schedule.
* Multi-segment search at real segment lengths: four H1+L1 segments of
  N = 60000, 120000, 160000 and 260000 (nfft 65536 .. 262144, fftpad 2, so
  nfftf = 131072, 262144, 524288, 524288 >= 2N), 4 sky points x 150
  spindowns each, through one pa_segments_search call (one CUDA graph over
  the four contexts), each segment compared with the oracle run on that
  segment's own inputs.

Bar (the same as the golden tests): candidate indices identical except at
the threshold edge (|F - trl| <= rtol trl) and argmax ties within rtol; F
within 1e-4 relative for the mixed forms, 1e-9 for the FP64 form.  The
largest errors are printed (pytest -s).
"""
import numpy as np
import pytest

from helpers import compare_candidates, key_of

pytestmark = pytest.mark.gpu

FORMS = {"mixed-fixed": (0, 1, 1e-4), "mixed-f64phase": (0, 0, 1e-4), "mixed-ffphase": (0, 2, 1e-4),
         "fp64": (1, 0, 1e-9)}


def _F(rec):
    return list(rec[:, 4] ** 2 / 2 + 2) if len(rec) else []


def _oracle_loop(ora, tasks, opts, rng):
    recs, idxs, fnum = [], [], 0
    for pm, mm, nn in tasks:
        rng.sst = rng.spndr[0]
        o = ora.job_core(pm, mm, nn, opts, rng)
        recs.append(o["records"])
        idxs.append(o["idx"])
        fnum += o["FNum"]
    return np.concatenate(recs), np.concatenate(idxs), fnum


def _in_disk(s, pm, mm, nn):
    al1 = nn * s.M[10] + mm * s.M[14]
    al2 = nn * s.M[11] + mm * s.M[15]
    return (al1 * al1 + al2 * al2) / (s.oms * s.oms) <= 1.0


@pytest.fixture(scope="module")
def network(tmp_path_factory, lib):
    from polgraw_gb300 import workloads
    from polgraw_gb300.lib import Host
    from pyoracle import Oracle
    root = str(tmp_path_factory.mktemp("network"))
    cmd, inj = workloads.network(root, 200)
    host = Host(cmd)
    s = host.settings
    assert (s.N, s.nfftf, s.nmax - s.nmin) == (86164, 131072, 63488)
    inside = [p for p in host.sky_points() if _in_disk(s, *p)]
    assert len(inside) >= 1900
    tasks = []
    for j in inj:
        t = workloads.nearest_sky(host, j)
        if t not in tasks:
            tasks.append(t)
    for t in inside[::10]:
        if t not in tasks:
            tasks.append(t)
    assert len(tasks) >= 200
    dets, nifo = host.detectors()
    opts, rng = host.opts(), host.range
    assert (rng.spndr[0], rng.spndr[1]) == (0, 199) and opts.trl == 20.0
    ora = Oracle(s, dets, nifo)
    ref = _oracle_loop(ora, tasks, opts, rng)
    ora.close()
    assert len(ref[0]) > 500
    return dict(host=host, tasks=tasks, ref=ref, dets=dets, nifo=nifo)


@pytest.mark.parametrize("form", list(FORMS))
def test_network_200_sky_points_vs_oracle(form, network):
    from polgraw_gb300.lib import Context
    precision, phase, rtol = FORMS[form]
    host = network["host"]
    ctx = Context(host.settings, network["dets"], network["nifo"], precision=precision, phase_mode=phase)
    ctx.set_graphs(True)
    rng = host.range
    rng.sst = rng.spndr[0]
    rec, idx, fnum = ctx.search_batch(network["tasks"], host.opts(), rng)
    ctx.close()
    rrec, ridx, rfnum = network["ref"]
    assert fnum == rfnum == 200 * len(network["tasks"])
    matched, err, bad = compare_candidates(key_of(ridx), _F(rrec), key_of(idx), _F(rec), host.opts().trl, rtol)
    print("\n%s: %d sky points, %d of %d oracle candidates matched, max rel F err %.2e, %d edge cases"
          % (form, len(network["tasks"]), matched, len(rrec), err, len(rrec) - matched))
    assert not bad, bad[:10]
    assert err <= rtol
    assert matched >= len(rrec) - 5
    # the host-side record fields of matched candidates are bit-identical
    R = {k: r[:4] for k, r in zip(key_of(ridx), rrec)}
    for k, r in zip(key_of(idx), rec):
        if k in R:
            assert list(r[:4]) == list(R[k])


SEG_N = (60000, 120000, 160000, 260000)


@pytest.fixture(scope="module")
def segments(lib):
    import math
    from polgraw_gb300 import workloads
    from polgraw_gb300.lib import Opts, Range
    from pyoracle import Oracle
    out = []
    for k, N in enumerate(SEG_N):
        s = workloads.segment_settings(N)
        assert s.fftpad == 2 and s.nfftf >= 2 * N
        dets, keep = workloads.segment_detectors(N, k)
        half = int(math.ceil(math.sqrt(2000 / math.pi))) + 1
        inside = [(1, mm, nn) for mm in range(-half, half + 1) for nn in range(-half, half + 1)
                  if _in_disk(s, 1, mm, nn)]
        tasks = inside[::len(inside) // 4][:4]
        o = Opts()
        o.trl = 14.0            # noise-only data: a lowered threshold gives candidates
        o.white_flag = 0
        o.s0_flag = 0
        o.use_range = 1
        r = Range()
        r.spndr[0], r.spndr[1] = 0, 149
        r.nr[0], r.nr[1] = -half, half
        r.mr[0], r.mr[1] = -half, half
        r.pmr[0], r.pmr[1] = 1, 1
        r.sst = 0
        ora = Oracle(s, dets, 2)
        ref = _oracle_loop(ora, tasks, o, r)
        ora.close()
        assert len(ref[0]) > 50
        out.append(dict(N=N, settings=s, dets=dets, keep=keep, tasks=tasks, opts=o, range=r, ref=ref))
    return out


@pytest.mark.parametrize("form", list(FORMS))
def test_segments_real_lengths_vs_oracle(form, segments):
    from polgraw_gb300.lib import Context, Segments
    precision, phase, rtol = FORMS[form]
    ctxs = [Context(g["settings"], g["dets"], 2, precision=precision, phase_mode=phase) for g in segments]
    seg = Segments(ctxs, graph=True)
    for g in segments:
        g["range"].sst = g["range"].spndr[0]
    res = seg.search([g["tasks"] for g in segments], [g["opts"] for g in segments],
                     [g["range"] for g in segments])
    seg.close()
    for c in ctxs:
        c.close()
    for g, (rec, idx, fnum) in zip(segments, res):
        rrec, ridx, rfnum = g["ref"]
        assert fnum == rfnum == 150 * len(g["tasks"])
        matched, err, bad = compare_candidates(key_of(ridx), _F(rrec), key_of(idx), _F(rec), g["opts"].trl, rtol)
        print("\n%s N=%d nfftf=%d: %d of %d oracle candidates matched, max rel F err %.2e"
              % (form, g["N"], g["settings"].nfftf, matched, len(rrec), err))
        assert not bad, (g["N"], bad[:10])
        assert err <= rtol
        assert matched >= len(rrec) - 5
