"""ctypes binding of libpolgraw_gb300.so (include/polgraw_gb300.h and
include/polgraw_gb300_host.h).

This is the Python-side mirror that the tests and bench.py use to call the
C-ABI exactly as a C caller of job_core() would: plain structs, host
buffers, status codes.  The CUDA path is the only implementation behind it;
if the library or a GPU is missing the calls fail loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpolgraw_gb300.so")

PA_OK, PA_ERR_ARG, PA_ERR_CUDA, PA_ERR_CAPACITY, PA_ERR_TIMEOUT, PA_ERR_NOMEM, PA_ERR_NODEV = range(7)
PA_PREC_MIXED, PA_PREC_FP64 = 0, 1
PA_PHASE_F64, PA_PHASE_FIXED, PA_PHASE_FF = 0, 1, 2
PA_NPAR = 5
PHASE_NAMES = {"f64": PA_PHASE_F64, "fixed": PA_PHASE_FIXED, "ff": PA_PHASE_FF}

# Every exported entry point declared in include/*.h
EXPORTS = [
    "pa_version", "pa_device_count", "pa_create", "pa_set_data", "pa_destroy", "pa_last_error",
    "pa_job_core", "pa_search_batch", "pa_debug_prelude", "pa_debug_fstat", "pa_kernel_launches",
    "pa_last_call_ms", "pa_set_profiling", "pa_profile_reset", "pa_profile_get", "pa_fstat_noalloc",
    "pa_set_cta_trace", "pa_cta_trace_count",
    "pa_host_create", "pa_host_setup", "pa_host_search", "pa_host_main", "pa_host_destroy",
    "pa_host_settings", "pa_host_detectors", "pa_host_range", "pa_host_core_opts",
    "pa_host_config", "pa_host_detector_name",
    "pa_set_graphs", "pa_set_schedule", "pa_get_schedule", "pa_set_lanes", "pa_get_lanes", "pa_autotune",
    "pa_segments_create", "pa_segments_destroy", "pa_segments_last_error", "pa_segments_set_graph", "pa_segments_search",
    "pa_segments_last_call_ms",
    "pa_followup_create", "pa_followup_destroy", "pa_followup_last_error", "pa_fstatnet", "pa_fstatnet_grad",
    "pa_followup_ascent", "pa_followup_simplex", "pa_followup_last_call_ms", "pa_followup_kernel_launches",
    "pa_coinc_vedva", "pa_coinc_create", "pa_coinc_destroy", "pa_coinc_last_error", "pa_coinc_reset",
    "pa_coinc_add_frame", "pa_coinc_run", "pa_coinc_get", "pa_coinc_cells", "pa_coinc_last_call_ms",
    "pa_coinc_kernel_launches", "pa_coinc_main", "pa_coinc_set_profiling", "pa_coinc_profile_get",
    "pa_fisher_reduced", "pa_gridgen", "pa_gridgen_write",
]


class Settings(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("fpo", "dt", "B", "oms", "omr", "Smin", "Smax", "sepsm", "cepsm")] + \
               [(n, C.c_int) for n in ("nfft", "nod", "N", "nfftf", "nmax", "nmin", "s", "nd",
                                       "interpftpad", "fftpad", "Ninterp", "nifo")] + \
               [("M", C.c_double * 16), ("numlines_band", C.c_int), ("lines", C.POINTER(C.c_double))]


class Detector(C.Structure):
    _fields_ = [("xDat", C.POINTER(C.c_double)), ("DetSSB", C.POINTER(C.c_double)),
                ("sig2", C.c_double), ("sphir", C.c_double), ("cphir", C.c_double),
                ("amod", C.c_double * 9)]


class Opts(C.Structure):
    _fields_ = [("trl", C.c_double), ("white_flag", C.c_int), ("s0_flag", C.c_int), ("use_range", C.c_int)]


class Range(C.Structure):
    _fields_ = [("pmr", C.c_int * 2), ("mr", C.c_int * 2), ("nr", C.c_int * 2), ("spndr", C.c_int * 2),
                ("pst", C.c_int), ("mst", C.c_int), ("nst", C.c_int), ("sst", C.c_int)]


class CandIdx(C.Structure):
    _fields_ = [("pm", C.c_int), ("mm", C.c_int), ("nn", C.c_int), ("ss", C.c_int), ("ii", C.c_int),
                ("F", C.c_float)]


class Config(C.Structure):
    _fields_ = [("precision", C.c_int), ("phase_mode", C.c_int), ("spindown_batch", C.c_int), ("device", C.c_int)]


class Sky(C.Structure):
    _fields_ = [("pm", C.c_int), ("mm", C.c_int), ("nn", C.c_int)]


class CoincCfg(C.Structure):
    _fields_ = [("N", C.c_int), ("oms", C.c_double), ("vedva", C.c_double * 16), ("shift", C.c_int * 4),
                ("scale", C.c_int * 4), ("refr", C.c_int), ("narrowdown", C.c_double), ("snrcutoff", C.c_double),
                ("mincoin", C.c_int), ("device", C.c_int)]


class CoincRec(C.Structure):
    _fields_ = [("w", C.c_int), ("first", C.c_int), ("mean", C.c_double * 5)]


class CoincSummary(C.Structure):
    _fields_ = [("nframes", C.c_int), ("raw", C.c_longlong), ("inband", C.c_longlong), ("unique", C.c_longlong),
                ("ncoin", C.c_int), ("nmembers", C.c_longlong), ("maxcoin", C.c_int), ("maxcoin_index", C.c_int),
                ("fp64_cells", C.c_longlong)]


_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Loads the library (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        from . import build as _b
        _b.build()
    lib = C.CDLL(p)
    P = C.POINTER
    lib.pa_version.restype = C.c_char_p
    lib.pa_device_count.restype = C.c_int
    lib.pa_create.restype = C.c_void_p
    lib.pa_create.argtypes = [P(Settings), P(Detector), C.c_int, P(Config), P(C.c_int)]
    lib.pa_set_data.argtypes = [C.c_void_p, P(Detector), C.c_int]
    lib.pa_destroy.argtypes = [C.c_void_p]
    lib.pa_destroy.restype = None
    lib.pa_last_error.restype = C.c_char_p
    lib.pa_last_error.argtypes = [C.c_void_p]
    lib.pa_job_core.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P(Opts), P(Range), P(C.c_int),
                                P(C.c_double), C.c_int, P(CandIdx), P(C.c_int), P(C.c_int)]
    lib.pa_search_batch.argtypes = [C.c_void_p, P(Sky), C.c_int, P(Opts), P(Range), P(C.c_int),
                                    P(C.c_double), C.c_int, P(CandIdx), P(C.c_int), P(C.c_int)]
    lib.pa_debug_prelude.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, P(C.c_double), P(C.c_double),
                                     P(C.c_double), P(C.c_double)]
    lib.pa_debug_fstat.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, P(Opts), P(C.c_double)]
    lib.pa_kernel_launches.restype = C.c_longlong
    lib.pa_kernel_launches.argtypes = [C.c_void_p]
    lib.pa_last_call_ms.restype = C.c_double
    lib.pa_last_call_ms.argtypes = [C.c_void_p]
    lib.pa_set_profiling.argtypes = [C.c_void_p, C.c_int]
    lib.pa_set_cta_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_uint]
    lib.pa_cta_trace_count.argtypes = [C.c_void_p, P(C.c_uint)]
    lib.pa_profile_reset.argtypes = [C.c_void_p]
    lib.pa_profile_reset.restype = None
    lib.pa_profile_get.argtypes = [C.c_void_p, C.c_int, P(C.c_char_p), P(C.c_double), P(C.c_longlong),
                                   P(C.c_longlong)]
    lib.pa_fstat_noalloc.argtypes = [P(Settings), P(Detector), C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                     P(Opts), C.c_int, P(C.c_double)]
    lib.pa_set_graphs.argtypes = [C.c_void_p, C.c_int]
    lib.pa_set_schedule.argtypes = [C.c_void_p, C.c_int, C.c_int]
    lib.pa_get_schedule.argtypes = [C.c_void_p, P(C.c_int), P(C.c_int), P(C.c_int)]
    lib.pa_set_lanes.argtypes = [C.c_void_p, C.c_int]
    lib.pa_get_lanes.argtypes = [C.c_void_p, P(C.c_int)]
    lib.pa_autotune.argtypes = [C.c_void_p, P(Sky), C.c_int, P(Opts), P(Range), P(C.c_int), P(C.c_int)]
    lib.pa_segments_create.restype = C.c_void_p
    lib.pa_segments_create.argtypes = [P(C.c_void_p), C.c_int, P(C.c_int)]
    lib.pa_segments_destroy.argtypes = [C.c_void_p]
    lib.pa_segments_destroy.restype = None
    lib.pa_segments_last_error.restype = C.c_char_p
    lib.pa_segments_last_error.argtypes = [C.c_void_p]
    lib.pa_segments_set_graph.argtypes = [C.c_void_p, C.c_int]
    lib.pa_segments_search.argtypes = [C.c_void_p, P(SegmentJob), P(C.c_int)]
    lib.pa_segments_last_call_ms.restype = C.c_double
    lib.pa_segments_last_call_ms.argtypes = [C.c_void_p]
    lib.pa_followup_create.restype = C.c_void_p
    lib.pa_followup_create.argtypes = [P(Settings), P(Detector), C.c_int, P(Config), P(C.c_int)]
    lib.pa_followup_destroy.argtypes = [C.c_void_p]
    lib.pa_followup_destroy.restype = None
    lib.pa_followup_last_error.restype = C.c_char_p
    lib.pa_followup_last_error.argtypes = [C.c_void_p]
    lib.pa_fstatnet.argtypes = [C.c_void_p, P(C.c_double), C.c_int, P(C.c_double)]
    lib.pa_fstatnet_grad.argtypes = [C.c_void_p, P(C.c_double), C.c_int, P(C.c_double), P(C.c_double),
                                     P(C.c_double)]
    lib.pa_followup_ascent.argtypes = [C.c_void_p, P(C.c_double), C.c_int, P(AscentOpts), P(C.c_double),
                                       P(C.c_int)]
    lib.pa_followup_simplex.argtypes = [C.c_void_p, P(C.c_double), C.c_int, P(C.c_double), C.c_double, C.c_int,
                                        P(C.c_double), P(C.c_int)]
    lib.pa_followup_last_call_ms.restype = C.c_double
    lib.pa_followup_last_call_ms.argtypes = [C.c_void_p]
    lib.pa_followup_kernel_launches.restype = C.c_longlong
    lib.pa_followup_kernel_launches.argtypes = [C.c_void_p]
    lib.pa_coinc_vedva.argtypes = [P(C.c_double), P(C.c_double)]
    lib.pa_coinc_create.restype = C.c_void_p
    lib.pa_coinc_create.argtypes = [P(CoincCfg), P(C.c_int)]
    lib.pa_coinc_destroy.argtypes = [C.c_void_p]
    lib.pa_coinc_destroy.restype = None
    lib.pa_coinc_last_error.restype = C.c_char_p
    lib.pa_coinc_last_error.argtypes = [C.c_void_p]
    lib.pa_coinc_reset.argtypes = [C.c_void_p]
    lib.pa_coinc_add_frame.argtypes = [C.c_void_p, C.c_int, P(C.c_double), C.c_longlong]
    lib.pa_coinc_run.argtypes = [C.c_void_p, P(CoincSummary)]
    lib.pa_coinc_get.argtypes = [C.c_void_p, P(C.c_int), P(CoincRec), P(C.c_int), P(C.c_int)]
    lib.pa_coinc_cells.argtypes = [C.c_void_p, P(C.c_int), P(C.c_ubyte)]
    lib.pa_coinc_last_call_ms.restype = C.c_double
    lib.pa_coinc_last_call_ms.argtypes = [C.c_void_p]
    lib.pa_coinc_kernel_launches.restype = C.c_longlong
    lib.pa_coinc_kernel_launches.argtypes = [C.c_void_p]
    lib.pa_fisher_reduced.argtypes = [P(C.c_double), P(C.c_double), C.c_longlong, C.c_double, C.c_double,
                                      P(C.c_double)]
    lib.pa_gridgen.argtypes = [P(C.c_double), P(C.c_double), C.c_longlong, C.c_double, P(GridgenOpts),
                               P(GridgenOut)]
    lib.pa_gridgen_write.argtypes = [C.c_char_p, P(GridgenOut)]
    lib.pa_coinc_set_profiling.argtypes = [C.c_void_p, C.c_int]
    lib.pa_coinc_profile_get.argtypes = [C.c_void_p, C.c_int, P(C.c_char_p), P(C.c_double), P(C.c_longlong)]
    lib.pa_host_create.restype = C.c_void_p
    lib.pa_host_create.argtypes = [C.c_int, P(C.c_char_p), P(C.c_int)]
    lib.pa_host_setup.argtypes = [C.c_void_p]
    lib.pa_host_search.argtypes = [C.c_void_p, C.c_void_p]
    lib.pa_host_main.argtypes = [C.c_int, P(C.c_char_p)]
    lib.pa_host_destroy.argtypes = [C.c_void_p]
    lib.pa_host_destroy.restype = None
    lib.pa_host_settings.restype = P(Settings)
    lib.pa_host_settings.argtypes = [C.c_void_p]
    lib.pa_host_detectors.restype = P(Detector)
    lib.pa_host_detectors.argtypes = [C.c_void_p, P(C.c_int)]
    lib.pa_host_range.restype = P(Range)
    lib.pa_host_range.argtypes = [C.c_void_p]
    lib.pa_host_core_opts.argtypes = [C.c_void_p, P(Opts)]
    lib.pa_host_core_opts.restype = None
    lib.pa_host_config.argtypes = [C.c_void_p, P(Config)]
    lib.pa_host_config.restype = None
    lib.pa_host_detector_name.restype = C.c_char_p
    lib.pa_host_detector_name.argtypes = [C.c_void_p, C.c_int]
    _lib = lib
    return lib


def _argv(args: list[str]):
    arr = (C.c_char_p * (len(args) + 1))()
    arr[:-1] = [a.encode() for a in args]
    arr[-1] = None
    return arr


class Host:
    """Search set-up exactly as the drop-in program does it (handle_opts ...
    read_checkpoints), from a reference-style command line."""

    def __init__(self, args: list[str]):
        self.lib = load()
        argv = ["gwsearch-gb300"] + list(args)
        self._argv = _argv(argv)
        rc = C.c_int(0)
        h = self.lib.pa_host_create(len(argv), self._argv, C.byref(rc))
        if not h:
            raise RuntimeError("pa_host_create failed (%d)" % rc.value)
        self.h = h
        self.setup_rc = self.lib.pa_host_setup(h)
        if self.setup_rc == 101:
            raise RuntimeError("pa_host_setup failed")

    @property
    def settings(self) -> Settings:
        return self.lib.pa_host_settings(self.h).contents

    def detectors(self):
        n = C.c_int(0)
        p = self.lib.pa_host_detectors(self.h, C.byref(n))
        return p, n.value

    @property
    def range(self) -> Range:
        return self.lib.pa_host_range(self.h).contents

    def opts(self) -> Opts:
        o = Opts()
        self.lib.pa_host_core_opts(self.h, C.byref(o))
        return o

    def config(self) -> Config:
        c = Config()
        self.lib.pa_host_config(self.h, C.byref(c))
        return c

    def sky_points(self) -> list[tuple[int, int, int]]:
        """(pm, mm, nn) in the sky-loop order (jobcore.c:90-98)."""
        r = self.range
        out = []
        mst, nst = r.mst, r.nst
        for pm in range(r.pst, r.pmr[1] + 1):
            for mm in range(mst, r.mr[1] + 1):
                for nn in range(nst, r.nr[1] + 1):
                    out.append((pm, mm, nn))
                nst = r.nr[0]
            mst = r.mr[0]
        return out

    def close(self):
        if self.h:
            self.lib.pa_host_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SearchError(RuntimeError):
    pass


class Context:
    """A pa_ctx: GPU search context for one set of inputs."""

    def __init__(self, settings: Settings, dets, nifo: int, precision: int = PA_PREC_MIXED,
                 phase_mode: int = PA_PHASE_FIXED, spindown_batch: int = 0, device: int = 0):
        self.lib = load()
        self.cfg = Config(precision, phase_mode, spindown_batch, device)
        st = C.c_int(0)
        self.ctx = self.lib.pa_create(C.byref(settings), dets, nifo, C.byref(self.cfg), C.byref(st))
        if not self.ctx:
            raise SearchError("pa_create failed (%d): %s" % (st.value, self.lib.pa_last_error(None).decode()))
        self.settings = settings
        self.nifo = nifo
        # search_batch's output buffers, kept from call to call (the library
        # writes every field of the records and indices it returns)
        self._out_cap = 0
        self._out_buf = None
        self._out_idx = None

    def error(self) -> str:
        return self.lib.pa_last_error(self.ctx).decode()

    def job_core(self, pm, mm, nn, opts: Opts, rng: Range, cap: int = 1 << 16):
        """Returns (records [n,5], idx structured array, FNum increment)."""
        sgnlc = C.c_int(0)
        fnum = C.c_int(0)
        needed = C.c_int(0)
        while True:
            buf = np.zeros((cap, PA_NPAR))
            idx = (CandIdx * cap)()
            rc = self.lib.pa_job_core(self.ctx, pm, mm, nn, C.byref(opts), C.byref(rng), C.byref(sgnlc),
                                      buf.ctypes.data_as(C.POINTER(C.c_double)), cap, idx, C.byref(fnum),
                                      C.byref(needed))
            if rc == PA_ERR_CAPACITY:
                cap = needed.value + 16
                continue
            if rc != PA_OK:
                raise SearchError("pa_job_core failed (%d): %s" % (rc, self.error()))
            break
        n = sgnlc.value
        return buf[:n].copy(), idx_to_array(idx, n), fnum.value

    def search_batch(self, tasks, opts: Opts, rng: Range, cap: int = 1 << 18):
        # the sky points as the C array of {pm, mm, nn} ints
        sky = np.ascontiguousarray(np.asarray(tasks, dtype=np.int32).reshape(-1, 3))
        arr = sky.ctypes.data_as(C.POINTER(Sky))
        sgnlc = C.c_int(0)
        fnum = C.c_int(0)
        needed = C.c_int(0)
        while True:
            if self._out_cap != cap:
                self._out_buf = np.empty((cap, PA_NPAR))
                self._out_idx = (CandIdx * cap)()
                self._out_cap = cap
            buf, idx = self._out_buf, self._out_idx
            rc = self.lib.pa_search_batch(self.ctx, arr, len(sky), C.byref(opts), C.byref(rng),
                                          C.byref(sgnlc), buf.ctypes.data_as(C.POINTER(C.c_double)), cap, idx,
                                          C.byref(fnum), C.byref(needed))
            if rc == PA_ERR_CAPACITY:
                cap = needed.value + 16
                continue
            if rc != PA_OK:
                raise SearchError("pa_search_batch failed (%d): %s" % (rc, self.error()))
            break
        n = sgnlc.value
        return buf[:n].copy(), idx_to_array(idx, n), fnum.value

    def prelude(self, pm, mm, nn):
        N = self.settings.N
        xa = np.zeros((self.nifo, N), dtype=np.complex128)
        xb = np.zeros_like(xa)
        aa = C.c_double(0)
        bb = C.c_double(0)
        rc = self.lib.pa_debug_prelude(self.ctx, pm, mm, nn, xa.ctypes.data_as(C.POINTER(C.c_double)),
                                       xb.ctypes.data_as(C.POINTER(C.c_double)), C.byref(aa), C.byref(bb))
        if rc != PA_OK:
            raise SearchError("pa_debug_prelude failed (%d): %s" % (rc, self.error()))
        return xa, xb, aa.value, bb.value

    def fstat(self, pm, mm, nn, ss, opts: Opts):
        F = np.zeros(self.settings.nmax - self.settings.nmin)
        rc = self.lib.pa_debug_fstat(self.ctx, pm, mm, nn, ss, C.byref(opts),
                                     F.ctypes.data_as(C.POINTER(C.c_double)))
        if rc != PA_OK:
            raise SearchError("pa_debug_fstat failed (%d): %s" % (rc, self.error()))
        return F

    def set_data(self, dets, nifo):
        rc = self.lib.pa_set_data(self.ctx, dets, nifo)
        if rc != PA_OK:
            raise SearchError("pa_set_data failed (%d): %s" % (rc, self.error()))

    def launches(self) -> int:
        return int(self.lib.pa_kernel_launches(self.ctx))

    def last_call_ms(self) -> float:
        return float(self.lib.pa_last_call_ms(self.ctx))

    def set_graphs(self, on: bool):
        self.lib.pa_set_graphs(self.ctx, int(bool(on)))

    def set_schedule(self, sbatch: int, split: int = 0):
        rc = self.lib.pa_set_schedule(self.ctx, sbatch, split)
        if rc != PA_OK:
            raise SearchError("pa_set_schedule failed (%d): %s" % (rc, self.error()))

    def schedule(self):
        """(sbatch, split, max_sbatch)."""
        a, b, m = C.c_int(0), C.c_int(0), C.c_int(0)
        self.lib.pa_get_schedule(self.ctx, C.byref(a), C.byref(b), C.byref(m))
        return a.value, b.value, m.value

    def set_lanes(self, lanes: int):
        rc = self.lib.pa_set_lanes(self.ctx, lanes)
        if rc != PA_OK:
            raise SearchError("pa_set_lanes failed (%d): %s" % (rc, self.error()))

    def lanes(self) -> int:
        n = C.c_int(0)
        self.lib.pa_get_lanes(self.ctx, C.byref(n))
        return n.value

    def autotune(self, tasks, opts: Opts, rng: Range):
        arr = (Sky * len(tasks))(*[Sky(*t) for t in tasks])
        a, b = C.c_int(0), C.c_int(0)
        rc = self.lib.pa_autotune(self.ctx, arr, len(tasks), C.byref(opts), C.byref(rng), C.byref(a), C.byref(b))
        if rc != PA_OK:
            raise SearchError("pa_autotune failed (%d): %s" % (rc, self.error()))
        return a.value, b.value

    def set_profiling(self, on: bool):
        rc = self.lib.pa_set_profiling(self.ctx, 1 if on else 0)
        if rc != PA_OK:
            raise SearchError("pa_set_profiling failed: %s" % self.error())

    def profile_reset(self):
        self.lib.pa_profile_reset(self.ctx)

    def set_cta_trace(self, dev_ptr: int, cap: int):
        """Per-CTA trace into device memory at dev_ptr (cap 48-byte records);
        dev_ptr 0 switches it off."""
        rc = self.lib.pa_set_cta_trace(self.ctx, C.c_void_p(dev_ptr or None), cap)
        if rc != PA_OK:
            raise SearchError("pa_set_cta_trace failed: %s" % self.error())

    def cta_trace_count(self) -> int:
        n = C.c_uint(0)
        if self.lib.pa_cta_trace_count(self.ctx, C.byref(n)) != PA_OK:
            raise SearchError("pa_cta_trace_count failed: %s" % self.error())
        return n.value

    def profile(self) -> dict:
        """{kernel name: (total_ms, launches, items)}"""
        out = {}
        k = 0
        while True:
            name = C.c_char_p()
            ms = C.c_double()
            nl = C.c_longlong()
            it = C.c_longlong()
            if self.lib.pa_profile_get(self.ctx, k, C.byref(name), C.byref(ms), C.byref(nl), C.byref(it)) != PA_OK:
                break
            out[name.value.decode()] = (ms.value, nl.value, it.value)
            k += 1
        return out

    def close(self):
        if self.ctx:
            self.lib.pa_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SegmentJob(C.Structure):
    _fields_ = [("tasks", C.c_void_p), ("ntasks", C.c_int), ("opts", C.c_void_p), ("range", C.c_void_p),
                ("sgnlc", C.c_void_p), ("sgnlv", C.c_void_p), ("cap", C.c_int), ("idx", C.c_void_p),
                ("FNum", C.c_void_p), ("needed", C.c_void_p)]


class Segments:
    """pa_segments: several contexts (one per data segment) searched
    together, optionally as one CUDA graph."""

    def __init__(self, contexts, graph: bool = True):
        self.lib = load()
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c.ctx for c in self.contexts])
        st = C.c_int(0)
        self.seg = self.lib.pa_segments_create(arr, len(self.contexts), C.byref(st))
        if not self.seg:
            raise SearchError("pa_segments_create failed (%d): %s" %
                              (st.value, self.lib.pa_segments_last_error(None).decode()))
        self.lib.pa_segments_set_graph(self.seg, int(bool(graph)))

    def set_graph(self, on: bool):
        self.lib.pa_segments_set_graph(self.seg, int(bool(on)))

    def search(self, task_lists, opts_list, ranges, cap: int = 1 << 18):
        """Returns [(records, idx, FNum)] per segment."""
        n = len(self.contexts)
        while True:
            keep, jobs = [], (SegmentJob * n)()
            outs = []
            for k in range(n):
                tasks = task_lists[k]
                arr = (Sky * max(1, len(tasks)))(*[Sky(*t) for t in tasks])
                sgnlc, fnum, needed = C.c_int(0), C.c_int(0), C.c_int(0)
                buf = np.zeros((cap, PA_NPAR))
                idx = (CandIdx * cap)()
                keep += [arr, sgnlc, fnum, needed, buf, idx]
                jobs[k] = SegmentJob(C.cast(arr, C.c_void_p), len(tasks), C.addressof(opts_list[k]),
                                     C.addressof(ranges[k]), C.addressof(sgnlc), buf.ctypes.data, cap,
                                     C.addressof(idx), C.addressof(fnum), C.addressof(needed))
                outs.append((sgnlc, buf, idx, fnum, needed))
            status = (C.c_int * n)()
            rc = self.lib.pa_segments_search(self.seg, jobs, status)
            if rc == PA_ERR_CAPACITY:
                cap = max(o[4].value for o in outs) + 16
                continue
            if rc != PA_OK:
                raise SearchError("pa_segments_search failed (%d): %s" %
                                  (rc, self.lib.pa_segments_last_error(self.seg).decode()))
            return [(o[1][:o[0].value].copy(), idx_to_array(o[2], o[0].value), o[3].value) for o in outs]

    def last_call_ms(self) -> float:
        return self.lib.pa_segments_last_call_ms(self.seg)

    def close(self):
        if getattr(self, "seg", None):
            self.lib.pa_segments_destroy(self.seg)
            self.seg = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class AscentOpts(C.Structure):
    _fields_ = [("scale", C.c_double * 4), ("step0", C.c_double), ("min_step", C.c_double), ("max_iter", C.c_int)]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Followup:
    """pa_followup: the demodulated network F-statistic (followup.c
    Fstatnet), its adjoint gradient, gradient ascent and the batched
    reference simplex.  Points are rows (f, s, delta, alpha)."""

    def __init__(self, settings: Settings, dets, nifo: int, precision: int = PA_PREC_MIXED, device: int = 0,
                 phase_mode: int = PA_PHASE_F64):
        """phase_mode: PA_PHASE_F64 (FP64 phase, the default) or PA_PHASE_FF
        (compensated two-float phase) in the mixed precision."""
        self.lib = load()
        cfg = Config(precision, phase_mode, 0, device)
        st = C.c_int(0)
        self.fu = self.lib.pa_followup_create(C.byref(settings), dets, nifo, C.byref(cfg), C.byref(st))
        if not self.fu:
            raise SearchError("pa_followup_create failed (%d): %s" %
                              (st.value, self.lib.pa_followup_last_error(None).decode()))

    def _check(self, rc, what):
        if rc != PA_OK:
            raise SearchError("%s failed (%d): %s" % (what, rc, self.lib.pa_followup_last_error(self.fu).decode()))

    @staticmethod
    def _pts(sgnlo) -> np.ndarray:
        return np.ascontiguousarray(np.atleast_2d(np.asarray(sgnlo, dtype=np.float64)))

    def fstatnet(self, sgnlo) -> np.ndarray:
        """fstat_out rows [n, 11] (out[:, 5] = -F)."""
        p = self._pts(sgnlo)
        out = np.zeros((len(p), 11))
        self._check(self.lib.pa_fstatnet(self.fu, _dp(p), len(p), _dp(out)), "pa_fstatnet")
        return out

    def fstatnet_grad(self, sgnlo, seed=None):
        """(F [n], grad [n, 4]) with grad = seed * dF/d(f, s, delta, alpha)."""
        p = self._pts(sgnlo)
        n = len(p)
        F = np.zeros(n)
        g = np.zeros((n, 4))
        sd = None if seed is None else np.ascontiguousarray(seed, dtype=np.float64)
        self._check(self.lib.pa_fstatnet_grad(self.fu, _dp(p), n, None if sd is None else _dp(sd), _dp(F), _dp(g)),
                    "pa_fstatnet_grad")
        return F, g

    def ascent(self, sgnlo, scale, step0: float = 0.25, min_step: float = 1e-3, max_iter: int = 100):
        """Gradient ascent; returns (points [n, 4], fstat_out [n, 11], iters [n])."""
        p = self._pts(sgnlo).copy()
        n = len(p)
        out = np.zeros((n, 11))
        it = np.zeros(n, dtype=np.int32)
        o = AscentOpts((C.c_double * 4)(*[float(x) for x in scale]), step0, min_step, max_iter)
        self._check(self.lib.pa_followup_ascent(self.fu, _dp(p), n, C.byref(o), _dp(out),
                                                it.ctypes.data_as(C.POINTER(C.c_int))), "pa_followup_ascent")
        return p, out, it

    def simplex(self, sgnlo, pc2, tol: float = 1e-7, max_evals: int = 0):
        """The reference simplex; returns (points [n, 4], fstat_out [n, 11], nevals [n])."""
        p = self._pts(sgnlo).copy()
        n = len(p)
        out = np.zeros((n, 11))
        nev = np.zeros(n, dtype=np.int32)
        st = np.ascontiguousarray(pc2, dtype=np.float64)
        self._check(self.lib.pa_followup_simplex(self.fu, _dp(p), n, _dp(st), tol, max_evals, _dp(out),
                                                 nev.ctypes.data_as(C.POINTER(C.c_int))), "pa_followup_simplex")
        return p, out, nev

    def last_call_ms(self) -> float:
        return self.lib.pa_followup_last_call_ms(self.fu)

    def launches(self) -> int:
        return self.lib.pa_followup_kernel_launches(self.fu)

    def close(self):
        if getattr(self, "fu", None):
            self.lib.pa_followup_destroy(self.fu)
            self.fu = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fstat_noalloc(settings: Settings, dets, nifo: int, pm: int, mm: int, nn: int, ss: int, opts: Opts,
                  device: int = 0) -> np.ndarray:
    """pa_fstat_noalloc: normalised F of one template, no allocation."""
    lib = load()
    F = np.zeros(settings.nmax - settings.nmin)
    rc = lib.pa_fstat_noalloc(C.byref(settings), dets, nifo, pm, mm, nn, ss, C.byref(opts), device,
                              F.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != PA_OK:
        raise SearchError("pa_fstat_noalloc failed (%d): %s" % (rc, lib.pa_last_error(None).decode()))
    return F


IDX_DTYPE = np.dtype([("pm", "i4"), ("mm", "i4"), ("nn", "i4"), ("ss", "i4"), ("ii", "i4"), ("F", "f4")])


def idx_to_array(idx, n: int) -> np.ndarray:
    raw = np.frombuffer(C.string_at(C.addressof(idx), n * C.sizeof(CandIdx)), dtype=IDX_DTYPE) if n else \
        np.zeros(0, dtype=IDX_DTYPE)
    return raw.copy()


def make_detectors(xdats, detssbs, sig2s, sphirs, cphirs, amods):
    """Builds a pa_detector array from numpy inputs (arrays are kept alive by
    the returned tuple)."""
    n = len(xdats)
    arr = (Detector * n)()
    keep = []
    for i in range(n):
        x = np.ascontiguousarray(xdats[i], dtype=np.float64)
        d = np.ascontiguousarray(detssbs[i], dtype=np.float64)
        keep += [x, d]
        arr[i].xDat = x.ctypes.data_as(C.POINTER(C.c_double))
        arr[i].DetSSB = d.ctypes.data_as(C.POINTER(C.c_double))
        arr[i].sig2 = sig2s[i]
        arr[i].sphir = sphirs[i]
        arr[i].cphir = cphirs[i]
        for k in range(9):
            arr[i].amod[k] = amods[i][k]
    return arr, keep


# ---------------------------------------------------------------------------
# Coincidences among frames (pa_coinc_*, coincidences/src/coincidences.c)
# ---------------------------------------------------------------------------

def digits4(val: int, default: int) -> list[int]:
    """The four per-direction digits of -shift / -scale (coincidences.c:157-178):
    read from the right, a 0 digit keeps the default."""
    d = [default] * 4
    i = 3
    while val > 0 and i >= 0:
        if val % 10:
            d[i] = val % 10
        i -= 1
        val //= 10
    return d


def read_fisher(grid_path: str) -> np.ndarray:
    """The second 4x4 matrix of grid.bin (manage_grid_matrix, init.c:1155-1167)."""
    raw = open(grid_path, "rb").read()
    return np.frombuffer(raw[4 + 128:4 + 256], dtype="<f8").reshape(4, 4).copy()


def fisher_reduced(rssb, rdet, epsm: float, xi: float = 0.5) -> np.ndarray:
    """pa_fisher_reduced: the grid generator's reduced Fisher matrix from the
    ephemeris parts (n x 3 each)."""
    a = np.ascontiguousarray(np.asarray(rssb, dtype=np.float64).reshape(-1))
    b = np.ascontiguousarray(np.asarray(rdet, dtype=np.float64).reshape(-1))
    out = np.zeros(16)
    rc = load().pa_fisher_reduced(_dp(a), _dp(b), len(a) // 3, epsm, xi, _dp(out))
    if rc != PA_OK:
        raise SearchError("pa_fisher_reduced failed (%d)" % rc)
    return out.reshape(4, 4)


class GridgenOpts(C.Structure):
    _fields_ = [("c0", C.c_double), ("xi", C.c_double), ("nfft_exp", C.c_int), ("method", C.c_int),
                ("nalpha", C.c_int), ("nradius", C.c_int), ("table", C.c_char_p)]


class GridgenOut(C.Structure):
    _fields_ = [("fftpad", C.c_int), ("M", C.c_double * 16), ("fisher", C.c_double * 16), ("Mn", C.c_double * 16),
                ("method", C.c_int), ("alpha", C.c_double), ("alpha_from_table", C.c_int), ("density", C.c_double)]

    def grid_bin(self) -> bytes:
        """The 388 bytes of grid.bin."""
        import struct
        return struct.pack("<i", self.fftpad) + b"".join(
            np.array(list(m), dtype="<f8").tobytes() for m in (self.M, self.fisher, self.Mn))


def gridgen(rssb, rdet, epsm: float, nfft_exp: int, c0: float = 0.5625, xi: float = 0.5, method: int = 0,
            nalpha: int = 35, nradius: int = 20, table: str | None = None) -> GridgenOut:
    """pa_gridgen: the grid generator's grid.bin contents from the ephemeris
    parts (n x 3 each)."""
    a = np.ascontiguousarray(np.asarray(rssb, dtype=np.float64).reshape(-1))
    b = np.ascontiguousarray(np.asarray(rdet, dtype=np.float64).reshape(-1))
    o = GridgenOpts(c0, xi, nfft_exp, method, nalpha, nradius, table.encode() if table else None)
    out = GridgenOut()
    rc = load().pa_gridgen(_dp(a), _dp(b), len(a) // 3, epsm, C.byref(o), C.byref(out))
    if rc != PA_OK:
        raise SearchError("pa_gridgen failed (%d)" % rc)
    return out


def vedva(fisher) -> np.ndarray:
    """pa_coinc_vedva: eigenvectors x sqrt(eigenvalues) of the Fisher matrix."""
    f = np.ascontiguousarray(np.asarray(fisher, dtype=np.float64).reshape(16))
    out = np.zeros(16)
    rc = load().pa_coinc_vedva(_dp(f), _dp(out))
    if rc != PA_OK:
        raise SearchError("pa_coinc_vedva failed (%d)" % rc)
    return out.reshape(4, 4)


def coinc_cfg(*, N: int, oms: float, vedva_m, shift: int = 0, scale: int = 1111, refr: int = 1,
              narrowdown: float = 0.5, snrcutoff: float = 6.0, mincoin: int = 3, device: int = 0) -> CoincCfg:
    """pa_coinc_cfg from the coincidence program's options (handle_opts_coinc,
    init.c:972-1122): narrowdown in units of pi as on the command line."""
    import math
    c = CoincCfg()
    c.N = N
    c.oms = oms
    for i, v in enumerate(np.asarray(vedva_m, dtype=np.float64).reshape(16)):
        c.vedva[i] = float(v)
    for i, v in enumerate(digits4(int(shift), 0)):
        c.shift[i] = v
    for i, v in enumerate(digits4(int(scale), 1)):
        c.scale[i] = v
    c.refr = refr
    c.narrowdown = narrowdown * math.pi
    c.snrcutoff = snrcutoff
    c.mincoin = mincoin
    c.device = device
    return c


COINC_REC_DTYPE = np.dtype([("w", "<i4"), ("first", "<i4"), ("mean", "<f8", (5,))])


def coinc_recs(recs, n: int):
    """(w, first, mean[n, 5]) of a ctypes array of pa_coinc_rec."""
    a = np.frombuffer(recs, dtype=COINC_REC_DTYPE, count=n) if n else np.zeros(0, dtype=COINC_REC_DTYPE)
    return a["w"].astype(np.int32), a["first"].astype(np.int64), a["mean"].reshape(-1, 5).copy()


class CoincResult:
    """Output of a coincidence run: per-frame counts, the records in file
    order (multiplicity w, FP64 means), and their members."""

    def __init__(self, summary, frameinfo, w, first, mean, fra, ops, cells=None, keep=None):
        self.summary = summary
        self.frameinfo = frameinfo
        self.w = w
        self.first = first
        self.mean = mean
        self.fra = fra
        self.ops = ops
        self.cells = cells
        self.keep = keep

    def summary_line(self, trigname: str, shift: int, fpo: float) -> str:
        """The line the coincidence program writes to stderr for the largest
        coincidence with the largest mean SNR (coincidences.c:547-593), or ""
        when no coincidence reaches mincoin."""
        s = self.summary
        if s.ncoin == 0 or s.maxcoin < 1:
            return ""
        q = s.maxcoin_index
        m = self.mean[q]
        line = "%s %04d %5f %5d %5d %15.8e %5.8e %5.8e %5.8e %5e " % (
            trigname, shift, fpo, s.nframes & 0xFFFF, s.maxcoin, m[0], m[1], m[2], m[3], m[4])
        for fi in self.frameinfo:
            line += "%d %d %d " % tuple(int(x) for x in fi)
        a = int(self.first[q])
        for k in range(s.maxcoin):
            line += "%d " % int(self.fra[a + k])
        return line + "\n"

    def coi_bytes(self) -> bytes:
        """The .coi file (coincidences.c:529-533): per record unsigned short w,
        5 floats, w unsigned short frames, w int positions."""
        import struct
        out = bytearray()
        for q in range(len(self.w)):
            w = int(self.w[q])
            out += struct.pack("<H", w)
            out += np.asarray(self.mean[q], dtype=np.float64).astype("<f4").tobytes()
            a, b = int(self.first[q]), int(self.first[q]) + w
            out += np.asarray(self.fra[a:b], dtype="<u2").tobytes()
            out += np.asarray(self.ops[a:b], dtype="<i4").tobytes()
        return bytes(out)


class Coinc:
    """pa_coinc: the coincidence step on the device.  Frames are added in the
    reference's directory order; run() returns a CoincResult."""

    def __init__(self, cfg: CoincCfg):
        self.lib = load()
        st = C.c_int(0)
        self.cc = self.lib.pa_coinc_create(C.byref(cfg), C.byref(st))
        if not self.cc:
            raise SearchError("pa_coinc_create failed (%d): %s" % (st.value, self.lib.pa_coinc_last_error(None).decode()))

    def _check(self, rc, what):
        if rc != PA_OK:
            raise SearchError("%s failed (%d): %s" % (what, rc, self.lib.pa_coinc_last_error(self.cc).decode()))

    def reset(self):
        self._check(self.lib.pa_coinc_reset(self.cc), "pa_coinc_reset")

    def add_frame(self, frame: int, records: np.ndarray):
        r = np.ascontiguousarray(records, dtype=np.float64).reshape(-1, 5)
        self._check(self.lib.pa_coinc_add_frame(self.cc, int(frame), _dp(r), len(r)), "pa_coinc_add_frame")

    def run(self, cells: bool = False) -> CoincResult:
        s = CoincSummary()
        self._check(self.lib.pa_coinc_run(self.cc, C.byref(s)), "pa_coinc_run")
        fi = np.zeros((max(1, s.nframes), 3), dtype=np.int32)
        recs = np.empty(max(1, s.ncoin), dtype=COINC_REC_DTYPE)
        fra = np.empty(max(1, s.nmembers), dtype=np.int32)
        ops = np.empty(max(1, s.nmembers), dtype=np.int32)
        IP = C.POINTER(C.c_int)
        self._check(self.lib.pa_coinc_get(self.cc, fi.ctypes.data_as(IP), recs.ctypes.data_as(C.POINTER(CoincRec)),
                                          fra.ctypes.data_as(IP), ops.ctypes.data_as(IP)), "pa_coinc_get")
        recs = recs[:s.ncoin]
        w, first, mean = recs["w"], recs["first"], recs["mean"]
        cl = kp = None
        if cells:
            cl = np.zeros((max(1, s.inband), 4), dtype=np.int32)
            kp = np.zeros(max(1, s.inband), dtype=np.uint8)
            self._check(self.lib.pa_coinc_cells(self.cc, cl.ctypes.data_as(IP), kp.ctypes.data_as(C.POINTER(C.c_ubyte))),
                        "pa_coinc_cells")
            cl, kp = cl[:s.inband], kp[:s.inband]
        return CoincResult(s, fi[:s.nframes], w, first, mean, fra[:s.nmembers], ops[:s.nmembers], cl, kp)

    def last_call_ms(self) -> float:
        return self.lib.pa_coinc_last_call_ms(self.cc)

    def launches(self) -> int:
        return self.lib.pa_coinc_kernel_launches(self.cc)

    def set_profiling(self, on: bool):
        self._check(self.lib.pa_coinc_set_profiling(self.cc, int(on)), "pa_coinc_set_profiling")

    def profile(self) -> dict:
        """{kernel kind: (total ms, launches)} since profiling was switched on."""
        out, k = {}, 0
        while True:
            nm, ms, n = C.c_char_p(), C.c_double(), C.c_longlong()
            if self.lib.pa_coinc_profile_get(self.cc, k, C.byref(nm), C.byref(ms), C.byref(n)) != PA_OK:
                return out
            out[nm.value.decode()] = (ms.value, n.value)
            k += 1

    def close(self):
        if getattr(self, "cc", None):
            self.lib.pa_coinc_destroy(self.cc)
            self.cc = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
