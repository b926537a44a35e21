"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the parity reference.  The product never
uses it.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None
_lib_fast = None


def load(fast: bool = False):
    """The parity oracle (liboracle.so), or with fast=True its build with the
    reference's timing flags (liboracle_fast.so, the timed CPU baseline)."""
    global _lib, _lib_fast
    if fast and _lib_fast is not None:
        return _lib_fast
    if not fast and _lib is not None:
        return _lib
    path = build_oracle.build_oracle_fast() if fast else build_oracle.build_oracle()
    lib = C.CDLL(path)
    lib.ora_create.restype = C.c_void_p
    lib.ora_create.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    lib.ora_destroy.argtypes = [C.c_void_p]
    lib.ora_destroy.restype = None
    P = C.POINTER
    lib.ora_job_core.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, P(C.c_int),
                                 P(C.c_double), C.c_int, C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_double),
                                 P(C.c_double), P(C.c_double), P(C.c_double), C.c_int, P(C.c_double)]
    lib.ora_fft.argtypes = [C.c_int, C.c_int, P(C.c_double), P(C.c_double)]
    lib.ora_search_settings.argtypes = [C.c_void_p]
    lib.ora_search_settings.restype = None
    lib.ora_spindown_range.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, P(C.c_int), P(C.c_int)]
    if fast:
        _lib_fast = lib
    else:
        _lib = lib
    return lib


class Oracle:
    """All-FP64 CPU restatement of job_core() over the same pa_settings /
    pa_detector inputs as the GPU context."""

    def __init__(self, settings, dets, nifo: int, nthreads: int = 0, fast: bool = False):
        self.lib = load(fast)
        self.settings = settings
        self.nifo = nifo
        self.o = self.lib.ora_create(C.addressof(settings), C.cast(dets, C.c_void_p), nifo, nthreads)
        if not self.o:
            raise RuntimeError("ora_create failed")

    def job_core(self, pm, mm, nn, opts, rng, cap: int = 1 << 16, want_prelude=False, F_ss=None):
        from importlib import import_module
        pa_lib = import_module("polgraw_gb300.lib")
        N = self.settings.N
        sgnlc = C.c_int(0)
        fnum = C.c_int(0)
        needed = C.c_int(0)
        PD = C.POINTER(C.c_double)
        while True:
            buf = np.zeros((cap, 5))
            idx = (pa_lib.CandIdx * cap)()
            pre_a = np.zeros((self.nifo, N), np.complex128) if want_prelude else None
            pre_b = np.zeros((self.nifo, N), np.complex128) if want_prelude else None
            aa = C.c_double(0)
            bb = C.c_double(0)
            Fo = np.zeros(self.settings.nmax - self.settings.nmin) if F_ss is not None else None
            rc = self.lib.ora_job_core(
                self.o, pm, mm, nn, C.addressof(opts), C.addressof(rng), C.byref(sgnlc),
                buf.ctypes.data_as(PD), cap, C.addressof(idx), C.byref(fnum), C.byref(needed),
                pre_a.ctypes.data_as(PD) if want_prelude else None,
                pre_b.ctypes.data_as(PD) if want_prelude else None, C.byref(aa), C.byref(bb),
                int(F_ss) if F_ss is not None else -(1 << 30),
                Fo.ctypes.data_as(PD) if Fo is not None else None)
            if rc == -1:
                cap = needed.value + 16
                continue
            break
        n = sgnlc.value
        out = {"records": buf[:n].copy(), "idx": pa_lib.idx_to_array(idx, n), "FNum": fnum.value,
               "aa": aa.value, "bb": bb.value}
        if want_prelude:
            out["pre_a"], out["pre_b"] = pre_a, pre_b
        if Fo is not None:
            out["F"] = Fo
        return out

    def job_core3(self, pm, mm, nn, opts, rng):
        """(records, idx, FNum increment), the shape of lib.Context.job_core."""
        d = self.job_core(pm, mm, nn, opts, rng)
        return d["records"], d["idx"], d["FNum"]

    def close(self):
        if self.o:
            self.lib.ora_destroy(self.o)
            self.o = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fft(x: np.ndarray, sign: int) -> np.ndarray:
    lib = load()
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.empty_like(x)
    rc = lib.ora_fft(x.size, sign, x.ctypes.data_as(C.POINTER(C.c_double)),
                     out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc:
        raise ValueError("length must be a power of two")
    return out


def _fu_bind(lib):
    P = C.POINTER
    lib.ora_fstatnet.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
    lib.ora_fstatnet.restype = None
    lib.ora_fstatnet_grad.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double)]
    lib.ora_fstatnet_grad.restype = C.c_double
    lib.ora_amoeba.argtypes = [C.c_void_p, P(C.c_double), P(C.c_double), C.c_double, C.c_int, P(C.c_double)]
    lib.ora_amoeba.restype = C.c_int


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class FollowupOracle(Oracle):
    """The followup functions of the oracle (followup.c Fstatnet, the FP64
    gradient and the simplex) on the same inputs."""

    def __init__(self, settings, dets, nifo: int, nthreads: int = 0):
        super().__init__(settings, dets, nifo, nthreads)
        _fu_bind(self.lib)

    def fstatnet(self, sgnlo) -> np.ndarray:
        p = np.ascontiguousarray(sgnlo, dtype=np.float64)
        out = np.zeros(11)
        self.lib.ora_fstatnet(self.o, _dp(p), _dp(out))
        return out

    def fstatnet_grad(self, sgnlo):
        p = np.ascontiguousarray(sgnlo, dtype=np.float64)
        g = np.zeros(4)
        F = self.lib.ora_fstatnet_grad(self.o, _dp(p), _dp(g))
        return F, g

    def amoeba(self, point, pc2, tol: float = 1e-7, max_evals: int = 0):
        p = np.array(point, dtype=np.float64)
        st = np.ascontiguousarray(pc2, dtype=np.float64)
        out = np.zeros(11)
        nev = self.lib.ora_amoeba(self.o, _dp(p), _dp(st), tol, max_evals, _dp(out))
        return p, out, nev


def _coinc_bind(lib):
    if getattr(lib, "_coinc_bound", False):
        return lib
    P = C.POINTER
    lib.ora_coinc_vedva.argtypes = [P(C.c_double), P(C.c_double)]
    lib.ora_coinc_run.restype = C.c_void_p
    lib.ora_coinc_run.argtypes = [C.c_void_p, C.c_int, P(C.c_int), P(P(C.c_double)), P(C.c_longlong), C.c_void_p]
    lib.ora_coinc_get.argtypes = [C.c_void_p, P(C.c_int), C.c_void_p, P(C.c_int), P(C.c_int)]
    lib.ora_coinc_cells.argtypes = [C.c_void_p, P(C.c_int), P(C.c_ubyte)]
    lib.ora_coinc_free.argtypes = [C.c_void_p]
    lib.ora_coinc_free.restype = None
    lib._coinc_bound = True
    return lib


def coinc_vedva(fisher) -> np.ndarray:
    """manage_grid_matrix()'s vedva through the GSL shim's eigensystem."""
    lib = _coinc_bind(load())
    f = np.ascontiguousarray(np.asarray(fisher, dtype=np.float64).reshape(16))
    out = np.zeros(16)
    lib.ora_coinc_vedva(_dp(f), _dp(out))
    return out.reshape(4, 4)


def coinc(cfg, frames, recs) -> "object":
    """The coincidence step on the CPU over frames in the given order;
    returns the product's CoincResult type (cells included)."""
    from importlib import import_module
    L = import_module("polgraw_gb300.lib")
    lib = _coinc_bind(load())
    arrs = [np.ascontiguousarray(np.asarray(r, dtype=np.float64).reshape(-1, 5)) for r in recs]
    nf = len(arrs)
    fr = (C.c_int * max(1, nf))(*[int(x) for x in frames])
    ptrs = (C.POINTER(C.c_double) * max(1, nf))(*[_dp(a) for a in arrs])
    ns = (C.c_longlong * max(1, nf))(*[len(a) for a in arrs])
    s = L.CoincSummary()
    o = lib.ora_coinc_run(C.byref(cfg), nf, fr, ptrs, ns, C.byref(s))
    if not o:
        raise RuntimeError("ora_coinc_run: invalid arguments")
    try:
        IP = C.POINTER(C.c_int)
        fi = np.zeros((max(1, s.nframes), 3), dtype=np.int32)
        rr = (L.CoincRec * max(1, s.ncoin))()
        fra = np.zeros(max(1, s.nmembers), dtype=np.int32)
        ops = np.zeros(max(1, s.nmembers), dtype=np.int32)
        lib.ora_coinc_get(o, fi.ctypes.data_as(IP), rr, fra.ctypes.data_as(IP), ops.ctypes.data_as(IP))
        cl = np.zeros((max(1, s.inband), 4), dtype=np.int32)
        kp = np.zeros(max(1, s.inband), dtype=np.uint8)
        lib.ora_coinc_cells(o, cl.ctypes.data_as(IP), kp.ctypes.data_as(C.POINTER(C.c_ubyte)))
    finally:
        lib.ora_coinc_free(o)
    w, first, mean = L.coinc_recs(rr, s.ncoin)
    return L.CoincResult(s, fi[:s.nframes], w, first, mean, fra[:s.nmembers], ops[:s.nmembers],
                         cl[:s.inband], kp[:s.inband])
