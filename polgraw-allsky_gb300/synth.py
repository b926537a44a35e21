"""Synthetic inputs in the reference search's on-disk layout.

Writes, under ``<root>/<ident:03d>/``:

* ``grid.bin``: int32 fftpad + 16 doubles M (column-major grid generator) +
  32 filler doubles, 388 bytes like the reference's fixture (read_grid,
  search/network/src-cpu/init.c:287-321 reads the first 4+128 bytes);
* ``<DET>/xdatc_<ident:03d>_<band:04d>.bin``: N doubles of noise
  (detectors_settings, settings.c:134-136; init_arrays, init.c:339-352);
* ``<DET>/DetSSB.bin``: 3N doubles detector position (x, y, z interleaved,
  units of c*dt) + phir + epsm (init.c:381-397);

plus optional range files (8 ints, init.c:679-683) and injection files
(``snr|amp`` value, gsize, reffr, then f, fdot, delta, alpha and the four
amplitudes; init.c:486-505 with the amplitude formulas of sigen.c:348-357).

Determinism: every value is produced with IEEE-exact or correctly rounded
elementwise operations only (integer splitmix64 counters, sums of 32-bit
uniforms, + - * / and rint), and sin/cos are evaluated by a Cody-Waite
reduction and a Taylor polynomial written here.  The same call therefore
writes byte-identical files on x86-64 and aarch64, so fixtures generated on
one machine can be regenerated on the other.  The noise is Irwin-Hall(12)
(sum of twelve uniforms minus six): mean 0, variance 1, support +-6.
"""
from __future__ import annotations

import hashlib
import math
import os
import struct
from dataclasses import dataclass, field

import numpy as np

C_OMEGA_R = 7.2921151467064e-5                      # settings.h:31
C_SIDDAY = 2.0 * math.pi / C_OMEGA_R                # settings.h:32
C_EPSMA = 84381.448 / 3600.0 / (180.0 / math.pi)    # settings.h:20
C_SPEED_OF_LIGHT = 299792.458                       # km/s, settings.h:16
C_AU = 1.49597870691e8                              # km, settings.h:17
C_EARTH_R = 6378.140                                # km, settings.h:25
C_YEARSEC = 365.25 * 86400.0                        # settings.h:36

RAD_TO_DEG = 180.0 / math.pi
# Site latitude/longitude/orientation as in detectors_settings (settings.c:172-222)
SITES = {
    "H1": dict(ephi=(46 + (27 + 18.528 / 60.) / 60.) / RAD_TO_DEG,
               elam=-(119 + (24 + 27.5657 / 60.) / 60.) / RAD_TO_DEG,
               egam=170.9994 / RAD_TO_DEG),
    "L1": dict(ephi=(30 + (33 + 46.4196 / 60.) / 60.) / RAD_TO_DEG,
               elam=-(90 + (46 + 27.2654 / 60.) / 60.) / RAD_TO_DEG,
               egam=242.7165 / RAD_TO_DEG),
    "V1": dict(ephi=(43. + 37. / 60. + 53.0880 / 3600.) / RAD_TO_DEG,
               elam=(10. + 30. / 60. + 16.1885 / 3600.) / RAD_TO_DEG,
               egam=(135. - (19.0 + 25. / 60.0 + 57.96 / 3600.)) / RAD_TO_DEG),
}
DEFAULT_SIGMA = {"H1": 1.0, "L1": 1.3, "V1": 1.0}
DEFAULT_SEED = {"H1": 1001, "L1": 1002, "V1": 1003}

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(counter: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser of a uint64 counter array (wrapping arithmetic)."""
    with np.errstate(over="ignore"):
        z = counter + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return z


def uniform32(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n uniforms in [0, 1) with 32-bit resolution (exact doubles)."""
    base = np.uint64((seed * 0x100000001B3 + stream * 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        ctr = base + np.arange(n, dtype=np.uint64) * np.uint64(0xD1B54A32D192ED03)
    z = _splitmix64(ctr)
    return (z >> np.uint64(32)).astype(np.float64) * (2.0 ** -32)


def gauss_ih(seed: int, n: int) -> np.ndarray:
    """Irwin-Hall(12) noise: sum of 12 exact 32-bit uniforms minus 6 (exact)."""
    acc = np.zeros(n)
    for k in range(12):
        acc = acc + uniform32(seed, n, stream=k + 1)
    return acc - 6.0


_PIO2_HI = 1.5707963267341256      # pi/2 split: hi has 33 significant bits
_PIO2_LO = 6.077100506506192e-11   # pi/2 - hi


def det_sincos(x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """sin and cos with only + - * and rint: Cody-Waite reduction by pi/2
    (two-term constant) and Taylor series to x^19 on |r| <= pi/4 (truncation
    error < 1e-18).  Deterministic across IEEE-754 platforms."""
    x = np.asarray(x, dtype=np.float64)
    k = np.rint(x * (2.0 / math.pi))
    r = (x - k * _PIO2_HI) - k * _PIO2_LO
    r2 = r * r
    # sin r = r (1 - r2/3! (1 - r2/(4*5) (1 - ...)))  -- nested Horner form
    s = np.ones_like(r)
    for n in range(19, 1, -2):            # n = 19, 17, ..., 3
        s = 1.0 - s * r2 / (n * (n - 1))
    s = s * r
    c = np.ones_like(r)
    for n in range(20, 0, -2):            # n = 20, 18, ..., 2
        c = 1.0 - c * r2 / (n * (n - 1))
    q = (k.astype(np.int64)) & 3
    sin_x = np.where(q == 0, s, np.where(q == 1, c, np.where(q == 2, -s, -c)))
    cos_x = np.where(q == 0, c, np.where(q == 1, -s, np.where(q == 2, -c, s)))
    return sin_x, cos_x


def nsamples(nod: int, dt: float) -> int:
    """N = round(nod * C_SIDDAY / dt) (settings.c:32, round macro auxi.h:14)."""
    return int(math.floor(nod * C_SIDDAY / dt + 0.5))


def detssb_parts(det: str, N: int, dt: float, gmst0: float = 1.0,
                 orbit0: float = 0.7) -> tuple[np.ndarray, np.ndarray, float, float]:
    """The two parts of the detector position in units of c*dt, 3N doubles
    each (x, y, z interleaved, equatorial): the Earth's centre w.r.t. the SSB
    (circular 1 AU orbit in the ecliptic, rotated by the obliquity) and the
    site w.r.t. the Earth's centre (spherical Earth rotating at C_OMEGA_R).
    The layout of the ephemeris files rSSB.bin and rDet.bin that the grid
    generator reads (gridgen/src/ReadEphemeris.cpp:24-100).  Returns (rSSB,
    rDet, phir, epsm); phir is the site's local sidereal angle at t=0
    (gen2day/ExtractBand.c:336)."""
    site = SITES[det]
    t = np.arange(N, dtype=np.float64) * dt
    unit = C_SPEED_OF_LIGHT * dt                       # km per (c*dt)
    om_orb = 2.0 * math.pi / C_YEARSEC
    so, co = det_sincos(orbit0 + om_orb * t)
    se, ce = det_sincos(np.array([C_EPSMA]))
    r_au = C_AU / unit
    ssb = np.empty(3 * N)
    ssb[0::3] = r_au * co
    ssb[1::3] = r_au * so * ce[0]
    ssb[2::3] = r_au * so * se[0]
    phir = gmst0 + site["elam"]
    sp, cp = det_sincos(phir + C_OMEGA_R * t)
    sphi, cphi = det_sincos(np.array([site["ephi"]]))
    re = C_EARTH_R / unit
    rdet = np.empty(3 * N)
    rdet[0::3] = re * cphi[0] * cp
    rdet[1::3] = re * cphi[0] * sp
    rdet[2::3] = re * sphi[0]
    return ssb, rdet, float(phir), float(C_EPSMA)


def detssb(det: str, N: int, dt: float, gmst0: float = 1.0, orbit0: float = 0.7) -> tuple[np.ndarray, float, float]:
    """Detector position w.r.t. the SSB in units of c*dt (rSSB + rDet of
    detssb_parts).  Returns (3N array, phir, epsm)."""
    ssb, rdet, phir, epsm = detssb_parts(det, N, dt, gmst0, orbit0)
    return ssb + rdet, phir, epsm


def ast2lin(alfa: float, delta: float, epsm: float = C_EPSMA) -> tuple[list[float], int]:
    """Sky position -> linear coordinates and hemisphere (auxi.c:26-53)."""
    se, ce = (float(v[0]) for v in det_sincos(np.array([epsm])))
    sa, ca = (float(v[0]) for v in det_sincos(np.array([alfa])))
    sd, cd = (float(v[0]) for v in det_sincos(np.array([delta])))
    be0 = ce * sa * cd + se * sd
    be1 = ca * cd
    d1 = math.asin(be0 * math.sin(epsm) + math.sqrt(1. - be0 * be0 - be1 * be1) * math.cos(epsm)) - delta
    pm = 1 if abs(d1) < 10. * 2.220446049250313e-16 else 2
    return [be0, be1], pm


def sigen_amplitudes(psi: float, phi0: float, cosi: float) -> list[float]:
    """The four amplitudes a1..a4 of sigen.c:350-357."""
    hoc = cosi
    hop = (1. + hoc * hoc) / 2.
    s2, c2 = (float(v[0]) for v in det_sincos(np.array([2. * psi])))
    sp, cp = (float(v[0]) for v in det_sincos(np.array([phi0])))
    return [c2 * hop * cp - s2 * hoc * sp,
            s2 * hop * cp + c2 * hoc * sp,
            -c2 * hop * sp - s2 * hoc * cp,
            -s2 * hop * sp + c2 * hoc * cp]


def fpo_default(band: int, dt: float) -> float:
    """fpo = 10 + 0.96875 * band * (0.5/dt) (init.c:235-240)."""
    return 10. + 0.96875 * band * (0.5 / dt)


@dataclass
class Dataset:
    root: str
    ident: int
    band: int
    dt: float
    nod: int
    fftpad: int
    M: list[float]
    dets: list[str]
    N: int = 0
    files: dict = field(default_factory=dict)

    @property
    def nfft(self) -> int:
        return 1 << int(math.ceil(math.log(self.N) / math.log(2.)))

    @property
    def oms(self) -> float:
        return 2. * math.pi * fpo_default(self.band, self.dt) * self.dt


def grid_matrix(nfftf: int, oms: float, *, m4: float = 0.0, m5: float = -1e-9,
                sky: tuple[float, float, float, float] | None = None,
                m8: float = 0.0, m9: float = 0.0, m12: float = 0.0, m13: float = 0.0) -> list[float]:
    """Column-major 4x4 grid generator M (jobcore.c:219-240).  `sky` gives
    (M10, M11, M14, M15); default is a square lattice of spacing
    oms*sqrt(pi/2000) (about 2000 points per hemisphere)."""
    M = [0.0] * 16
    M[0] = 2. * math.pi / nfftf
    M[4] = m4
    M[5] = m5
    M[8] = m8
    M[9] = m9
    M[12] = m12
    M[13] = m13
    if sky is None:
        d = oms * math.sqrt(math.pi / 2000.)
        sky = (d, 0.0, 0.0, d)
    M[10], M[11], M[14], M[15] = sky
    return M


def _sha(path: str) -> str:
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def write_dataset(root: str, *, ident: int = 1, band: int = 666, dt: float = 2.0, nod: int = 2,
                  fftpad: int = 1, dets=("H1", "L1"), M: list[float] | None = None,
                  sigma: dict | None = None, seeds: dict | None = None,
                  gaps: float = 0.0, seed_offset: int = 0, ephemeris_parts: bool = False,
                  grid_file: str | None = None) -> Dataset:
    """Writes grid.bin, xdatc and DetSSB files.  `gaps` is the fraction of
    samples zeroed in runs (the reference treats exact zeros as gaps:
    init.c:359-367 and init.c:635).  `ephemeris_parts`: also rSSB.bin and
    rDet.bin per detector (the grid generator's inputs).  `grid_file`: copy
    this grid.bin (e.g. one made by the grid generator) instead of writing
    the synthetic one; M is then read from it."""
    N = nsamples(nod, dt)
    ds = Dataset(root=root, ident=ident, band=band, dt=dt, nod=nod, fftpad=fftpad,
                 M=list(M) if M is not None else [], dets=list(dets), N=N)
    if not ds.M:
        ds.M = grid_matrix(fftpad * ds.nfft, ds.oms)
    base = os.path.join(root, "%03d" % ident)
    os.makedirs(base, exist_ok=True)
    gpath = os.path.join(base, "grid.bin")
    if grid_file is not None:
        raw = open(grid_file, "rb").read()
        with open(gpath, "wb") as f:
            f.write(raw)
        ds.fftpad = struct.unpack("<i", raw[:4])[0]
        ds.M = list(np.frombuffer(raw[4:132], dtype="<f8"))
    else:
        with open(gpath, "wb") as f:
            f.write(struct.pack("<i", fftpad))
            f.write(np.asarray(ds.M, dtype="<f8").tobytes())
            f.write(np.zeros(32, dtype="<f8").tobytes())
    ds.files["grid.bin"] = _sha(gpath)
    sigma = dict(DEFAULT_SIGMA, **(sigma or {}))
    seeds = dict(DEFAULT_SEED, **(seeds or {}))
    for d in dets:
        dd = os.path.join(base, d)
        os.makedirs(dd, exist_ok=True)
        x = gauss_ih(seeds[d] + seed_offset, N) * sigma[d]
        if gaps > 0:
            # zero runs of ~N/40 samples at deterministic positions
            u = uniform32(seeds[d] + 7919, 64, stream=99)
            run = max(1, N // 40)
            nrun = int(round(gaps * N / run))
            for k in range(min(nrun, 64)):
                s0 = int(u[k] * (N - run))
                x[s0:s0 + run] = 0.0
        xp = os.path.join(dd, "xdatc_%03d_%04d.bin" % (ident, band))
        x.astype("<f8").tofile(xp)
        ds.files[d + "/xdat"] = _sha(xp)
        ssb, rdet, phir, epsm = detssb_parts(d, N, dt)
        pos = ssb + rdet
        if ephemeris_parts:
            for nm, arr in (("rSSB.bin", ssb), ("rDet.bin", rdet)):
                ep = os.path.join(dd, nm)
                arr.astype("<f8").tofile(ep)
                ds.files[d + "/" + nm[:-4]] = _sha(ep)
        sp_ = os.path.join(dd, "DetSSB.bin")
        with open(sp_, "wb") as f:
            f.write(pos.astype("<f8").tobytes())
            f.write(np.array([phir, epsm], dtype="<f8").tobytes())
        ds.files[d + "/DetSSB"] = _sha(sp_)
    return ds


def write_range(path: str, spndr, nr, mr, pmr) -> None:
    """Range file: 8 ints spndr0 spndr1 nr0 nr1 mr0 mr1 pm0 pm1 (init.c:679-683)."""
    with open(path, "w") as f:
        f.write("%d %d\n%d %d\n%d %d\n%d %d\n" % (spndr[0], spndr[1], nr[0], nr[1],
                                                  mr[0], mr[1], pmr[0], pmr[1]))


def write_addsig(path: str, *, f: float, fdot: float, delta: float, alpha: float,
                 snr: float | None = None, amp: float | None = None, gsize: int = 2,
                 reffr: int = 1, psi: float = 0.3, phi0: float = 1.0, cosi: float = 0.5) -> None:
    """Injection file read by add_signal (init.c:486-505)."""
    a = sigen_amplitudes(psi, phi0, cosi)
    with open(path, "w") as fh:
        if snr is not None:
            fh.write("snr %.16e\n%d\n%d\n" % (snr, gsize, reffr))
        else:
            fh.write("amp %.16e\n%d\n%d\n" % (amp, gsize, reffr))
        for v in [f, fdot, delta, alpha] + a:
            fh.write("%.16e\n" % v)


def rogcvir(ephi: float, egam: float) -> list[float]:
    """Amplitude-modulation coefficients c1..c9 (settings.c:264-272)."""
    s2g, c2g = math.sin(2. * egam), math.cos(2. * egam)
    sp, cp = math.sin(ephi), math.cos(ephi)
    return [.25 * s2g * (1 + sp * sp), -.5 * c2g * sp, .5 * s2g * math.sin(2. * ephi), -c2g * cp,
            .75 * s2g * cp * cp, c2g * sp, .5 * s2g * (1. + sp * sp), c2g * cp, .5 * s2g * math.sin(2. * ephi)]


def inject(ds: Dataset, *, f: float, fdot: float, delta: float, alpha: float, snr: float,
           psi: float = 0.3, phi0: float = 1.0, cosi: float = 0.5) -> None:
    """Adds a continuous-wave signal to the dataset's xdatc files, with the
    signal model of add_signal (init.c:575-642, reffr == ident): amplitude
    modulation a(t), b(t) of modvir, phase f i + fdot i^2 + (oms + f +
    2 fdot i) n.r_i, four amplitudes from (psi, phi0, cos iota), h0 scaled so
    that the network SNR is `snr` for unit noise, added where the data are
    non-zero.  Uses only deterministic arithmetic (see module docstring)."""
    N = ds.N
    a = sigen_amplitudes(psi, phi0, cosi)
    oms = ds.oms
    cof = oms + f
    omr = C_OMEGA_R * ds.dt
    i = np.arange(N, dtype=np.float64)
    sm, cm = det_sincos(omr * i)
    sd, cd = det_sincos(np.array([delta]))
    sa, ca = det_sincos(np.array([alpha]))
    sindel, cosdel, sinal, cosal = sd[0], cd[0], sa[0], ca[0]
    nS = (cosal * cosdel, sinal * cosdel, sindel)
    base = os.path.join(ds.root, "%03d" % ds.ident)
    sigs, xs, paths = [], [], []
    total = 0.0
    for d in ds.dets:
        site = SITES[d]
        k = rogcvir(site["ephi"], site["egam"])
        dp = os.path.join(base, d)
        raw = np.fromfile(os.path.join(dp, "DetSSB.bin"), dtype="<f8")
        pos, phir = raw[:3 * N], raw[3 * N]
        sph, cph = det_sincos(np.array([phir]))
        cosalfr = cosal * cph[0] + sinal * sph[0]
        sinalfr = sinal * cph[0] - cosal * sph[0]
        c = cosalfr * cm + sinalfr * sm
        s = sinalfr * cm - cosalfr * sm
        c2d = cosdel * cosdel
        c2sd = sindel * cosdel
        c2s = 2. * c * c
        cs = c * s
        aa = k[0] * (2. - c2d) * c2s + k[1] * (2. - c2d) * 2. * cs + k[2] * c2sd * c + k[3] * c2sd * s \
            - k[0] * (2. - c2d) + k[4] * c2d
        bb = k[5] * sindel * c2s + k[6] * sindel * 2. * cs + k[7] * cosdel * c + k[8] * cosdel * s - k[5] * sindel
        shift = nS[0] * pos[0::3] + nS[1] * pos[1::3] + nS[2] * pos[2::3]
        ph = f * i + fdot * (i * i) + (cof + 2. * fdot * i) * shift
        sp_, cp_ = det_sincos(ph)
        sig = a[0] * aa * cp_ + a[2] * aa * sp_ + a[1] * bb * cp_ + a[3] * bb * sp_
        total += float(np.sum(sig * sig))
        xp = os.path.join(dp, "xdatc_%03d_%04d.bin" % (ds.ident, ds.band))
        sigs.append(sig)
        xs.append(np.fromfile(xp, dtype="<f8"))
        paths.append(xp)
    h0 = snr / math.sqrt(total)
    for d, sig, x, xp in zip(ds.dets, sigs, xs, paths):
        x = np.where(x != 0.0, x + h0 * sig, x)
        x.astype("<f8").tofile(xp)
        ds.files[d + "/xdat"] = _sha(xp)


# ---------------------------------------------------------------------------
# Trigger files of several time frames, the input of the coincidence step
# (coincidences/src/coincidences.c:117-330), and the reference grid.bin that
# carries its Fisher matrix (init.c:1142-1172).
# ---------------------------------------------------------------------------

def fisher_matrix(N: int, oms: float, widths=(8.0, 16.0, 2.0e6, 2.0e6),
                  angles=(0.3, 0.5)) -> np.ndarray:
    """Symmetric positive-definite 4x4 matrix Q diag(1/w^2) Q^T (row-major)
    acting on the linear coordinates (f N, s N^2, oms N be0, oms N be1) of
    coincidences.c:251-263: cells are w wide along the columns of Q, two
    Givens rotations (f with s, the two sky coordinates) by `angles`."""
    del N, oms
    s0, c0 = (float(v[0]) for v in det_sincos(np.array([angles[0]])))
    s1, c1 = (float(v[0]) for v in det_sincos(np.array([angles[1]])))
    Q = np.array([[c0, -s0, 0., 0.], [s0, c0, 0., 0.], [0., 0., c1, -s1], [0., 0., s1, c1]])
    lam = np.array([1.0 / (w * w) for w in widths])
    G = np.zeros((4, 4))
    for i in range(4):
        for j in range(4):
            acc = 0.0
            for k in range(4):
                acc = acc + Q[i, k] * lam[k] * Q[j, k]
            G[i, j] = acc
    return G


def write_coinc_grid(path: str, fisher: np.ndarray, fftpad: int = 1) -> str:
    """grid.bin as the coincidence program reads it: int fftpad, the grid
    generator (16 doubles, unused there), the Fisher matrix (16 doubles,
    init.c:1162-1167), 16 filler doubles."""
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "wb") as f:
        f.write(struct.pack("<i", fftpad))
        f.write(np.zeros(16, dtype="<f8").tobytes())
        f.write(np.asarray(fisher, dtype="<f8").reshape(16).tobytes())
        f.write(np.zeros(16, dtype="<f8").tobytes())
    return _sha(path)


def trigger_name(frame: int, band: int, hemi: int = 2) -> str:
    """triggers_<frame>_<band><label>_<hemi>.bin (jobcore.c:92-93)."""
    return "triggers_%03d_%04d_%d.bin" % (frame, band, hemi)


def coinc_triggers(frames, per_frame: int, *, N: int, refr: int, seed: int = 7,
                   lines: int = 6, sky: int = 12, signals: int = 24,
                   f_lo: float = 0.3, f_hi: float = 2.8) -> dict:
    """Deterministic trigger records [f, s, delta, alpha, snr] per frame.

    A mix that exercises every branch of the coincidence step:
    * lattice triggers: f on a few lines with a step of half a frequency
      cell, s = 0 or a few spindown steps, sky from a small set, SNR from a
      small set (exact duplicates within and across frames, SNR ties, values
      under the SNR cut);
    * continuous triggers near the same lines (random cells);
    * signals: one record per frame whose f shifted to the reference frame
      (f + 2 s N (refr - frame), coincidences.c:235) is the same for every
      frame, so that they coincide;
    * records outside the band and far outside the narrowed band.
    Only exact uniforms and + - * / enter the values, so the files are
    byte-identical on every IEEE-754 machine."""
    frames = list(frames)
    out = {}
    step_f = 4.0 / N                       # half a frequency cell (width 8 in f N)
    step_s = 8.0 / (float(N) * float(N))   # half a spindown cell (width 16 in s N^2)
    uL = uniform32(seed, lines + 2 * sky + 6 * signals, stream=500)
    fl = f_lo + (f_hi - f_lo) * uL[:lines]
    sky_d = -1.3 + 2.6 * uL[lines:lines + sky]
    sky_a = 6.2 * uL[lines + sky:lines + 2 * sky]
    sg = uL[lines + 2 * sky:].reshape(signals, 6) if signals else np.zeros((0, 6))
    sig_f = f_lo + (f_hi - f_lo) * sg[:, 0]
    sig_s = (sg[:, 1] - 0.5) * 64.0 * step_s
    sig_d = -1.3 + 2.6 * sg[:, 2]
    sig_a = 6.2 * sg[:, 3]
    snr_set = np.array([5.5, 6.5, 7.0, 7.0, 8.25, 9.0])
    for k, fr in enumerate(frames):
        n_lat = per_frame // 2
        n_con = per_frame - n_lat
        u = uniform32(seed * 1000 + fr, 6 * per_frame + 4 * signals + 8, stream=501)
        pos = [0]

        def take(m, u=u, pos=pos):
            pos[0] += m
            return u[pos[0] - m:pos[0]]
        a = take(n_lat)
        li = np.floor(a * lines).astype(np.int64)
        fj = np.floor(take(n_lat) * 9.0) - 4.0
        f_lat = fl[li] + fj * step_f
        s_lat = np.floor(take(n_lat) * 3.0) * step_s * 2.0 - 2.0 * step_s
        si = np.floor(take(n_lat) * sky).astype(np.int64)
        snr_lat = snr_set[np.floor(take(n_lat) * snr_set.size).astype(np.int64)]
        li2 = np.floor(take(n_con) * lines).astype(np.int64)
        f_con = fl[li2] + (take(n_con) - 0.5) * 40.0 * step_f
        s_con = (take(n_con) - 0.5) * 16.0 * step_s
        si2 = np.floor(take(n_con) * sky).astype(np.int64)
        snr_con = 4.0 + 6.0 * take(n_con)
        rec = [np.stack([f_lat, s_lat, sky_d[si], sky_a[si], snr_lat], axis=1),
               np.stack([f_con, s_con, sky_d[si2] + (take(n_con) - 0.5) * 1e-4,
                         sky_a[si2] + (take(n_con) - 0.5) * 1e-4, snr_con], axis=1)]
        if signals:
            present = take(signals) < 0.8
            js = np.nonzero(present)[0]
            fs = sig_f[js] - 2.0 * sig_s[js] * N * (refr - fr)
            rec.append(np.stack([fs, sig_s[js], sig_d[js], sig_a[js], 7.0 + 3.0 * sg[js, 4]], axis=1))
        # outside the band (shift pushes below 0) and outside a narrowed band
        rec.append(np.array([[1e-7, 1e-9, 0.1, 0.2, 8.0], [0.05, 0.0, 0.3, 0.4, 9.0],
                             [3.1, 0.0, -0.2, 5.0, 9.5]]))
        r = np.concatenate(rec, axis=0)
        order = np.argsort(uniform32(seed * 7 + fr, r.shape[0], stream=502), kind="stable")
        out[fr] = np.ascontiguousarray(r[order])
    return out


def write_triggers(root: str, recs: dict, band: int = 666) -> dict:
    """Writes each frame's records as little-endian doubles, 5 per record
    (the search's trigger-file layout, jobcore.c:141).  Returns name -> sha256."""
    os.makedirs(root, exist_ok=True)
    files = {}
    for fr, r in recs.items():
        p = os.path.join(root, trigger_name(fr, band))
        np.asarray(r, dtype="<f8").tofile(p)
        files[os.path.basename(p)] = _sha(p)
    return files
