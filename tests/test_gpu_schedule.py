"""Launch schedules, CUDA graphs and the multi-segment front-end: none of
them may change the search's results.

* graphs on/off: identical records and indices, also when the graph is
  updated in place for a second batch of the same shape;
* spindown batch sizes: identical results; two spindown lanes (launches
  alternating between two streams): identical results, with and without
  graphs, and the lane/batch limits rejected; the swapped FFT factor split
  (odd log2(nfftf)): the reference's candidates within the usual tolerance;
* pa_autotune: picks a valid schedule, results still match the reference;
* pa_segments_search over contexts of different N (one per golden case),
  with and without the single CUDA graph: each segment's records equal
  that context's own pa_search_batch.
"""
import numpy as np
import pytest

from helpers import (case_by_name, compare_candidates, golden, key_of, make_host)

pytestmark = pytest.mark.gpu


def _ctx(host, **kw):
    from polgraw_gb300.lib import Context
    dets, nifo = host.detectors()
    return Context(host.settings, dets, nifo, **kw)


def _batch(ctx, host, tasks=None):
    tasks = list(host.sky_points()) if tasks is None else tasks
    rng = host.range
    return ctx.search_batch(tasks, host.opts(), rng)


def _same(a, b):
    assert np.array_equal(a[0], b[0])
    assert key_of(a[1]) == key_of(b[1])
    assert a[2] == b[2]


@pytest.mark.parametrize("name", ["h1l1_gaps_veto", "h1_fullgrid", "cfg1_h1"])
def test_graphs_identical(name, tmp_path, gpu_ok):
    host, _ = make_host(case_by_name(name), str(tmp_path))
    ctx = _ctx(host)
    ref = _batch(ctx, host)
    ctx.set_graphs(True)
    g1 = _batch(ctx, host)
    g2 = _batch(ctx, host)          # replay through an in-place update
    _same(ref, g1)
    _same(ref, g2)
    pts = list(host.sky_points())
    if len(pts) >= 4:
        half = len(pts) // 2
        ctx.set_graphs(False)
        a = _batch(ctx, host, pts[half:2 * half])
        ctx.set_graphs(True)
        _batch(ctx, host, pts[:half])
        b = _batch(ctx, host, pts[half:2 * half])   # same shape, new sky points
        _same(a, b)


def test_spindown_batch_sizes_identical(tmp_path, gpu_ok):
    host, _ = make_host(case_by_name("h1l1_gaps_veto"), str(tmp_path))
    ctx = _ctx(host)
    sb, split, sbmax = ctx.schedule()
    ref = _batch(ctx, host)
    for b in sorted({1, max(1, sb // 2), sbmax}):
        ctx.set_schedule(b, split)
        _same(ref, _batch(ctx, host))


@pytest.mark.parametrize("graphs", [False, True])
def test_two_lanes_identical(graphs, tmp_path, gpu_ok):
    from polgraw_gb300.lib import SearchError
    host, _ = make_host(case_by_name("h1l1_gaps_veto"), str(tmp_path))
    ctx = _ctx(host)
    sb, split, sbmax = ctx.schedule()
    assert ctx.lanes() == 2            # the default when the batch fits a lane
    ctx.set_lanes(1)
    ref = _batch(ctx, host)
    ctx.set_graphs(graphs)
    ctx.set_schedule(sbmax, split)
    with pytest.raises(SearchError):
        ctx.set_lanes(2)               # the batch is larger than one lane
    assert ctx.lanes() == 1
    for b in sorted({1, 3, sbmax // 2}):
        ctx.set_schedule(b, split)
        ctx.set_lanes(2)
        assert ctx.lanes() == 2
        _same(ref, _batch(ctx, host))
        _same(ref, _batch(ctx, host))  # graph replay / second call
        ctx.set_lanes(1)
    ctx.set_lanes(2)
    ctx.set_schedule(sbmax, split)     # too large for a lane: one lane
    assert ctx.lanes() == 1
    _same(ref, _batch(ctx, host))
    with pytest.raises(SearchError):
        ctx.set_lanes(3)
    # the per-launch profile runs one lane and still gives the same records
    ctx.set_profiling(True)
    _same(ref, _batch(ctx, host))
    ctx.set_profiling(False)


@pytest.mark.parametrize("name", ["h1l1_gaps_veto", "h1l1_white_pm2", "h1l1_gridgen"])
def test_pass_a_radix16_agrees_with_radix8(name, tmp_path, gpu_ok, monkeypatch):
    """Two detectors with L1 = 256 take the two-stage radix-16 spindown pass A;
    the generic radix-4/8 kernel (PA_SPIN_PASS_A=radix8) gives the same
    candidates, F within FP32 rounding."""
    host, _ = make_host(case_by_name(name), str(tmp_path))
    monkeypatch.setenv("PA_SPIN_PASS_A", "radix8")
    c8 = _ctx(host)
    monkeypatch.delenv("PA_SPIN_PASS_A")
    c16 = _ctx(host)
    for split in (0, 1):
        c8.set_schedule(c8.schedule()[0], split)
        c16.set_schedule(c16.schedule()[0], split)
        r8, i8, f8 = _batch(c8, host)
        r16, i16, f16 = _batch(c16, host)
        assert f8 == f16
        F = lambda snr: snr * snr / 2 + 2  # noqa: E731
        matched, err, bad = compare_candidates(key_of(i8), [F(r[4]) for r in r8], key_of(i16),
                                               [F(r[4]) for r in r16], host.opts().trl, 1e-5)
        assert not bad and err <= 1e-5 and matched > 0, (split, bad[:5], err)
    c8.close()
    c16.close()


def _golden_match(name, rec, idx, host, rtol=1e-4):
    g = golden(name)
    ref = g["candidates"]
    rkeys = [tuple(c[:5]) for c in ref]
    rF = [c[9] ** 2 / 2 + 2 for c in ref]
    gF = [r[4] ** 2 / 2 + 2 for r in rec]
    matched, err, bad = compare_candidates(rkeys, rF, key_of(idx), gF, host.opts().trl, rtol)
    assert not bad, bad[:10]
    assert err <= rtol
    return matched


@pytest.mark.parametrize("name", ["h1l1_white_pm2", "cfg1_h1"])
def test_swapped_split_matches_reference(name, tmp_path, gpu_ok):
    host, _ = make_host(case_by_name(name), str(tmp_path))
    assert host.settings.nfftf.bit_length() % 2 == 0   # odd log2(nfftf)
    ctx = _ctx(host)
    sb, _, _ = ctx.schedule()
    ctx.set_schedule(sb, 1)
    assert ctx.schedule()[1] == 1
    rec, idx, fnum = _batch(ctx, host)
    assert _golden_match(name, rec, idx, host) > 0


def test_autotune(tmp_path, gpu_ok):
    name = "cfg1_h1"
    host, _ = make_host(case_by_name(name), str(tmp_path))
    ctx = _ctx(host)
    pts = list(host.sky_points())
    sb, split = ctx.autotune(pts, host.opts(), host.range)
    s2, sp2, smax = ctx.schedule()
    assert (sb, split) == (s2, sp2) and 1 <= sb <= smax and split in (0, 1)
    assert ctx.lanes() in (1, 2) and (ctx.lanes() == 1 or sb <= smax // 2)
    rec, idx, _ = _batch(ctx, host)
    assert _golden_match(name, rec, idx, host) > 0


@pytest.mark.parametrize("graph", [True, False])
def test_segments_equal_per_context(graph, tmp_path, gpu_ok):
    from polgraw_gb300.lib import Segments
    names = ["h1_addsig", "h1l1_gaps_veto", "h1l1_white_pm2", "cfg1_h1"]
    hosts = [make_host(case_by_name(n), str(tmp_path / n))[0] for n in names]
    assert len({h.settings.N for h in hosts}) >= 3    # uneven segment lengths
    ctxs = [_ctx(h) for h in hosts]
    for c in ctxs:
        c.set_graphs(False)
    own = [_batch(c, h) for c, h in zip(ctxs, hosts)]
    seg = Segments(ctxs, graph=graph)
    for rep in range(2):   # the second call replays the updated graph
        res = seg.search([list(h.sky_points()) for h in hosts], [h.opts() for h in hosts],
                         [h.range for h in hosts])
        for k in range(len(hosts)):
            _same(own[k], res[k])
    assert seg.last_call_ms() > 0
    for n, h, r in zip(names, hosts, res):
        _golden_match(n, r[0], r[1], h)
