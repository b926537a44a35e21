"""Input set-up of the reference search for the CPU oracle, independent of
the product library (TEST INFRASTRUCTURE: used by the CPU baseline and the
reference arm of bench.py, so that the timed CPU path loads only oracle
code).

Reads a data directory in the reference's layout -- <data>/<ident>/grid.bin,
<data>/<ident>/<det>/xdatc_<ident>_<band>.bin and DetSSB.bin -- and a range
file, and fills the same pa_settings / pa_detector / pa_range / pa_opts
structs as the product's host set-up, following the reference:
  search_settings()     settings.c:16-81 (ora_search_settings)
  read_grid()           init.c:287-321 (fftpad and M from grid.bin)
  detectors_settings()  settings.c:92-246 (site latitude and orientation;
                        detectors in name order, as the product host)
  rogcvir()             settings.c:253-275 (ora_rogcvir)
  init_arrays()         init.c:339-412: xDat, crf0 and sig2 (ora_sig2),
                        DetSSB with phir and epsm, sin/cos of both
  set_search_range()    init.c:664-700 with a range file
  search()              jobcore.c:90-98: the sky-loop order
Only the case without lines, -addsig, -usedet or -label is covered: the
benchmark's workloads need no more.  tests/test_oracle_setup.py checks
every field against the product host on those workloads.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import struct

import numpy as np

import pyoracle

RAD_TO_DEG = 180 / math.pi
# settings.c:92-246: latitude ephi and orientation egam of each site
SITES = {
    "H1": ((46 + (27 + 18.528 / 60.) / 60.) / RAD_TO_DEG, 170.9994 / RAD_TO_DEG),
    "L1": ((30 + (33 + 46.4196 / 60.) / 60.) / RAD_TO_DEG, 242.7165 / RAD_TO_DEG),
    "V1": ((43. + 37. / 60. + 53.0880 / 3600.) / RAD_TO_DEG, (135. - (19.0 + 25. / 60.0 + 57.96 / 3600.)) / RAD_TO_DEG),
}


class Inputs:
    """Structs of one search (settings, detectors, range, opts) and the
    arrays they point to."""

    def __init__(self, data: str, *, ident: int, band: int, dt: float, nod: int, range_file: str,
                 trl: float = 20.0, fpo: float | None = None):
        from importlib import import_module
        L = import_module("polgraw_gb300.lib")    # the ctypes struct layouts only
        lib = pyoracle.load()
        lib.ora_sig2.restype = C.c_double
        base = os.path.join(data, "%03d" % ident)
        s = L.Settings()
        s.dt = dt
        s.nod = nod
        s.fpo = fpo if fpo is not None else 10. + 0.96875 * band * (0.5 / dt)
        with open(os.path.join(base, "grid.bin"), "rb") as f:
            raw = f.read(4 + 16 * 8)
        s.fftpad = struct.unpack("<i", raw[:4])[0]
        for k, v in enumerate(np.frombuffer(raw[4:], dtype="<f8")):
            s.M[k] = float(v)
        lib.ora_search_settings(C.byref(s))
        N = s.N
        dets = sorted(d for d in os.listdir(base) if d in SITES and
                      os.path.exists(os.path.join(base, d, "xdatc_%03d_%04d.bin" % (ident, band))))
        self.keep = []
        darr = (L.Detector * len(dets))()
        sepsm = None
        for n, d in enumerate(dets):
            x = np.zeros(N)
            xr = np.fromfile(os.path.join(base, d, "xdatc_%03d_%04d.bin" % (ident, band)), dtype="<f8")[:N]
            x[:len(xr)] = xr
            e = np.fromfile(os.path.join(base, d, "DetSSB.bin"), dtype="<f8")
            pos = np.ascontiguousarray(e[:3 * N])
            phir, epsm = float(e[3 * N]), float(e[3 * N + 1])
            self.keep += [x, pos]
            darr[n].xDat = x.ctypes.data_as(C.POINTER(C.c_double))
            darr[n].DetSSB = pos.ctypes.data_as(C.POINTER(C.c_double))
            darr[n].sig2 = lib.ora_sig2(x.ctypes.data_as(C.POINTER(C.c_double)), N)
            darr[n].sphir = math.sin(phir)
            darr[n].cphir = math.cos(phir)
            amod = (C.c_double * 9)()
            lib.ora_rogcvir(C.c_double(SITES[d][0]), C.c_double(SITES[d][1]), amod)
            for k in range(9):
                darr[n].amod[k] = amod[k]
            if sepsm is None:
                sepsm = (math.sin(epsm), math.cos(epsm))
        s.sepsm, s.cepsm = sepsm
        s.nifo = len(dets)
        s.numlines_band = 0
        with open(range_file) as f:
            v = [int(t) for t in f.read().split()[:8]]
        r = L.Range()
        r.spndr[0], r.spndr[1], r.nr[0], r.nr[1], r.mr[0], r.mr[1], r.pmr[0], r.pmr[1] = v
        r.pst, r.mst, r.nst, r.sst = r.pmr[0], r.mr[0], r.nr[0], r.spndr[0]
        o = L.Opts()
        o.trl = trl
        o.white_flag = 0
        o.s0_flag = 0
        o.use_range = 1
        self.settings, self.dets, self.nifo, self.range, self._opts = s, darr, len(dets), r, o
        self.det_names = dets

    def detectors(self):
        return self.dets, self.nifo

    def opts(self):
        return self._opts

    def sky_points(self) -> list[tuple[int, int, int]]:
        """(pm, mm, nn) in the sky-loop order of search() (jobcore.c:90-98)."""
        r = self.range
        return [(pm, mm, nn) for pm in range(r.pst, r.pmr[1] + 1) for mm in range(r.mst, r.mr[1] + 1)
                for nn in range(r.nst, r.nr[1] + 1)]
