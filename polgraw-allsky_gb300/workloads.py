"""Synthetic workloads of the benchmark and the large parity cases, written
in the reference's on-disk layout by polgraw_gb300.synth.

* network(): H1+L1, N=86164 (2 sidereal days at dt=2 s), nfft=131072,
  fftpad=1, a sky lattice of spacing oms*sqrt(pi/2000) (~2000 points on one
  hemisphere), 5 injections (SNR 8-15, seed 2002).
* stress(): H1+L1, N=258492 (6 sidereal days), nfft=262144, fftpad=2
  (nfftf=524288), spindown step M5=5e-10 over ss in [-nspin/2, nspin/2) so
  that 400 spindowns span fdot in [-1e-7, 1e-7) (largest spindown phase
  s1*i^2 ~ 6.7e3 rad), sky lattice of spacing oms*sqrt(pi/500) (~500
  points), 3 injections (SNR 10-15, seed 2003).

Each returns (command line of the search, list of injections).
"""
from __future__ import annotations

import math
import os

import numpy as np

from . import synth


def _inject_random(ds, rng, n, *, fdot_lo, fdot_hi, snr_lo, snr_hi, f_lo=0.2, f_hi=2.9):
    out = []
    for _ in range(n):
        while True:
            delta = float(rng.uniform(-1.2, 1.2))
            alpha = float(rng.uniform(0, 2 * math.pi))
            _, pm = synth.ast2lin(alpha, delta)
            if pm == 1:
                break
        inj = dict(f=float(rng.uniform(f_lo, f_hi)), fdot=float(rng.uniform(fdot_lo, fdot_hi)),
                   delta=delta, alpha=alpha, snr=float(rng.uniform(snr_lo, snr_hi)))
        synth.inject(ds, **inj)
        out.append(inj)
    return out


def _lattice(root, *, dt, nod, band, fftpad, m5, npoints, dets=("H1", "L1")):
    N = synth.nsamples(nod, dt)
    probe = synth.Dataset(root=root, ident=1, band=band, dt=dt, nod=nod, fftpad=fftpad, M=[],
                          dets=list(dets), N=N)
    spacing = probe.oms * math.sqrt(math.pi / npoints)
    M = synth.grid_matrix(fftpad * probe.nfft, probe.oms, m5=m5, sky=(spacing, 0.0, 0.0, spacing))
    ds = synth.write_dataset(root, ident=1, band=band, dt=dt, nod=nod, fftpad=fftpad, dets=list(dets), M=M)
    nmax = int(math.ceil(1.0 / math.sqrt(math.pi / npoints))) + 1
    return ds, nmax


def network(root: str, nspin: int = 200, npoints: int = 2000):
    """The H1+L1 N=86164 network workload (a lattice of about `npoints` sky
    points on one hemisphere, 2000 by default, x `nspin` spindowns)."""
    ds, nmax = _lattice(root, dt=2.0, nod=2, band=666, fftpad=1, m5=-1e-9, npoints=npoints)
    inj = _inject_random(ds, np.random.default_rng(2002), 5, fdot_lo=-1.9e-7, fdot_hi=0.0,
                         snr_lo=8, snr_hi=15)
    rpath = os.path.join(root, "range.txt")
    synth.write_range(rpath, [0, nspin - 1], [-nmax, nmax], [-nmax, nmax], [1, 1])
    return ["-data", root, "-ident", "1", "-band", "666", "-dt", "2", "-nod", "2", "-range", rpath,
            "-output", os.path.join(root, "out"), "--nocheckpoint"], inj


def stress(root: str, nspin: int = 400):
    """The precision-stress workload: N=258492, nfftf=524288, fdot +-1e-7."""
    ds, nmax = _lattice(root, dt=2.0, nod=6, band=666, fftpad=2, m5=5e-10, npoints=500)
    inj = _inject_random(ds, np.random.default_rng(2003), 3, fdot_lo=-0.9e-7, fdot_hi=0.9e-7,
                         snr_lo=10, snr_hi=15)
    rpath = os.path.join(root, "range.txt")
    synth.write_range(rpath, [-(nspin // 2), nspin - nspin // 2 - 1], [-nmax, nmax], [-nmax, nmax], [1, 1])
    return ["-data", root, "-ident", "1", "-band", "666", "-dt", "2", "-nod", "6", "-range", rpath,
            "-output", os.path.join(root, "out"), "--nocheckpoint"], inj


def nearest_sky(host, inj):
    """Lattice sky point (pm, mm, nn) nearest to an injection's (delta,
    alpha), the point where its candidates appear."""
    s = host.settings
    be, pm = synth.ast2lin(inj["alpha"], inj["delta"])
    # al1 = nn M10 + mm M14, al2 = nn M11 + mm M15, with al = be * oms
    a = np.array([[s.M[10], s.M[14]], [s.M[11], s.M[15]]])
    nn, mm = np.linalg.solve(a, np.array(be) * s.oms)
    return (pm, int(round(mm)), int(round(nn)))


def peak_widths(settings, dets, nifo, delta, alpha):
    """Widths of the demodulated F-statistic peak in (f, s, delta, alpha):
    2 pi/N, 2 pi/N^2, and for each sky angle the step that turns the phase
    by 2 pi across the data, 2 pi / (oms * spread of d shft/d angle)."""
    N = settings.N
    sd, cd, sa, ca = np.sin(delta), np.cos(delta), np.sin(alpha), np.cos(alpha)
    spread_d, spread_a = 0.0, 0.0
    for n in range(nifo):
        R = np.ctypeslib.as_array(dets[n].DetSSB, shape=(3 * N,)).reshape(N, 3)
        dd = R @ np.array([-ca * sd, -sa * sd, cd])
        da = R @ np.array([-sa * cd, ca * cd, 0.0])
        spread_d = max(spread_d, float(dd.max() - dd.min()))
        spread_a = max(spread_a, float(da.max() - da.min()))
    oms = settings.oms
    return [2 * np.pi / N, 2 * np.pi / float(N) ** 2, 2 * np.pi / (oms * spread_d), 2 * np.pi / (oms * spread_a)]


def followup(root: str):
    """The followup workload: H1+L1+V1, N=86164 (2 sidereal days at dt=2 s),
    4 injected signals (SNR 10-15, seed 2005).  Returns (command line,
    injections); candidates_around() makes the starting points."""
    ds = synth.write_dataset(root, ident=1, band=666, dt=2.0, nod=2, fftpad=1, dets=["H1", "L1", "V1"],
                             M=None)
    inj = _inject_random(ds, np.random.default_rng(2005), 4, fdot_lo=-1e-8, fdot_hi=1e-8,
                         snr_lo=10, snr_hi=15)
    return ["-data", root, "-ident", "1", "-band", "666", "-dt", "2", "-nod", "2",
            "-output", os.path.join(root, "out"), "--nocheckpoint"], inj


def candidates_around(host, inj, n: int, seed: int = 2005):
    """n starting points spread over the injections, each offset from its
    injection by U(-0.5, 0.5) peak widths in every parameter; returns
    (points [n, 4], widths [n, 4], index of the injection per point)."""
    dets, nifo = host.detectors()
    rng = np.random.default_rng(seed)
    pts, ws, which = [], [], []
    for k in range(n):
        j = k % len(inj)
        c = inj[j]
        w = peak_widths(host.settings, dets, nifo, c["delta"], c["alpha"])
        base = [c["f"], c["fdot"], c["delta"], c["alpha"]]
        pts.append([base[t] + float(rng.uniform(-0.5, 0.5)) * w[t] for t in range(4)])
        ws.append(w)
        which.append(j)
    return np.array(pts), np.array(ws), np.array(which)


def segment_settings(N: int, *, dt: float = 2.0, band: int = 666, fftpad: int = 2, nifo: int = 2,
                     m5: float = -1e-9, npoints: int = 2000):
    """pa_settings of a data segment of arbitrary length N, as
    search_settings() (settings.c:16-81) and plan_fftw() (init.c:835-844)
    would set them, with a sky lattice of spacing oms*sqrt(pi/npoints)."""
    from .lib import Settings
    s = Settings()
    s.dt = dt
    s.fpo = synth.fpo_default(band, dt)
    s.B = 0.5 / dt
    s.oms = 2. * math.pi * s.fpo * dt
    s.omr = synth.C_OMEGA_R * dt
    s.N = int(N)
    s.nod = max(1, int(round(N * dt / synth.C_SIDDAY)))
    s.nfft = 1 << int(math.ceil(math.log(N) / math.log(2.)))
    s.s = 1
    s.Smax = 2. * math.pi * 0.5e-8 * dt * dt
    s.Smin = 2. * math.pi * 0.5e-9 * dt * dt
    s.nd = 2
    s.interpftpad = 2
    s.fftpad = fftpad
    s.nmin = int(fftpad * 4096 * s.B)
    s.nmax = int((s.nfft // 2 - 4096 * s.B) * fftpad)
    s.Ninterp = 2 * s.nfft
    s.nfftf = fftpad * s.nfft
    s.sepsm = math.sin(synth.C_EPSMA)
    s.cepsm = math.cos(synth.C_EPSMA)
    s.nifo = nifo
    spacing = s.oms * math.sqrt(math.pi / npoints)
    M = synth.grid_matrix(s.nfftf, s.oms, m5=m5, sky=(spacing, 0.0, 0.0, spacing))
    for k in range(16):
        s.M[k] = M[k]
    s.numlines_band = 0
    return s


def segment_detectors(N: int, k: int, dets=("H1", "L1"), dt: float = 2.0):
    """Noise-only data of segment k (seeds of the detector + 100 k) with the
    synthetic ephemeris, as a pa_detector array (and the arrays it points
    to, which must stay alive)."""
    from .lib import make_detectors
    xs, ps, s2, sph, cph, am = [], [], [], [], [], []
    for d in dets:
        x = synth.gauss_ih(synth.DEFAULT_SEED[d] + 100 * k, N) * synth.DEFAULT_SIGMA[d]
        pos, phir, _ = synth.detssb(d, N, dt)
        mean = x.sum() / N
        var = ((x - mean) ** 2).sum() / (N - 1)          # var() of auxi.c:124-139
        xs.append(x)
        ps.append(pos)
        s2.append(float(var))                            # no zeros: crf0 = 1
        sph.append(math.sin(phir))
        cph.append(math.cos(phir))
        site = synth.SITES[d]
        am.append(synth.rogcvir(site["ephi"], site["egam"]))
    return make_detectors(xs, ps, s2, sph, cph, am)


def segments(nseg: int = 24, *, nsky: int = 300, nspin: int = 150, seed: int = 2004,
             nmin_len: int = 60000, nmax_len: int = 260000):
    """The multi-segment workload: nseg segments of N uniform in
    [nmin_len, nmax_len] (seed), dt=2 s, H1+L1, fftpad=2 (nfftf = 2 nfft >=
    2N), nsky lattice sky points x nspin spindowns each.  Returns a list of
    dicts {N, settings, dets, keep, tasks, opts, range}."""
    from .lib import Opts, Range
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nseg):
        N = int(rng.integers(nmin_len, nmax_len + 1))
        s = segment_settings(N)
        dets, keep = segment_detectors(N, k)
        # lattice points inside the disk (jobcore.c:248), first nsky of them
        half = int(math.ceil(math.sqrt(2000 / math.pi))) + 1
        tasks = []
        for mm in range(-half, half + 1):
            for nn in range(-half, half + 1):
                al1, al2 = nn * s.M[10] + mm * s.M[14], nn * s.M[11] + mm * s.M[15]
                if (al1 * al1 + al2 * al2) / (s.oms * s.oms) <= 1.0:
                    tasks.append((1, mm, nn))
        tasks = tasks[:nsky]
        o = Opts()
        o.trl = 20.0
        o.white_flag = 0
        o.s0_flag = 0
        o.use_range = 1
        r = Range()
        r.spndr[0], r.spndr[1] = 0, nspin - 1
        r.nr[0], r.nr[1] = -half, half
        r.mr[0], r.mr[1] = -half, half
        r.pmr[0], r.pmr[1] = 1, 1
        r.sst = 0
        out.append(dict(N=N, settings=s, dets=dets, keep=keep, tasks=tasks, opts=o, range=r))
    return out


def coincidences(frames: int = 24, per_frame: int = 1 << 20, seed: int = 31) -> dict:
    """Coincidence workload: trigger records of `frames` frames (segments
    1..frames, reference frame in the middle), N = 86164 (2 days at dt = 2 s)
    band 666, spread over 64 frequency lines x 256 sky positions with 1000
    signals present in most frames; cells from the grid Fisher matrix of
    synth.fisher_matrix.  Returns the settings, the records per frame and
    the pa_coinc_cfg inputs (mincoin 4, no shift/scale, default cuts)."""
    from . import synth
    nod, dt, band = 2, 2.0, 666
    N = synth.nsamples(nod, dt)
    fpo = synth.fpo_default(band, dt)
    oms = 2. * math.pi * fpo * dt
    refr = (frames + 1) // 2
    fr = list(range(1, frames + 1))
    recs = synth.coinc_triggers(fr, per_frame, N=N, refr=refr, seed=seed, lines=64, sky=256, signals=1000)
    return dict(N=N, fpo=fpo, oms=oms, refr=refr, frames=fr, recs=recs, fisher=synth.fisher_matrix(N, oms),
                mincoin=4, band=band)
