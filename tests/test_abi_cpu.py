"""CPU-side checks of the C-ABI library: it loads, exports every entry point
that include/*.h declares, validates arguments without a GPU, and the C host
set-up follows the reference's command-line and file semantics."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in ("polgraw_gb300.h", "polgraw_gb300_host.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(pa_[a-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol(lib):
    from polgraw_gb300.lib import EXPORTS
    declared = _declared()
    assert declared == set(EXPORTS), declared ^ set(EXPORTS)
    for n in declared:
        assert hasattr(lib, n), n


def test_version_and_device_count(lib):
    assert b"sm_103a" in lib.pa_version()
    assert lib.pa_device_count() >= 0


def test_create_validates_arguments(lib):
    from polgraw_gb300.lib import Settings, Detector, Config, PA_ERR_ARG
    s = Settings()
    s.N, s.nfft, s.interpftpad, s.Ninterp, s.fftpad, s.nfftf = 1000, 1024, 2, 2048, 1, 1024
    s.nmin, s.nmax = 10, 500
    d = (Detector * 1)()
    st = C.c_int(0)
    ctx = lib.pa_create(C.byref(s), d, 1, C.byref(Config()), C.byref(st))
    assert not ctx and st.value == PA_ERR_ARG
    assert b"nfft" in lib.pa_last_error(None)
    ctx = lib.pa_create(C.byref(s), d, 0, C.byref(Config()), C.byref(st))
    assert not ctx and st.value == PA_ERR_ARG


def test_host_defaults_and_settings(tmp_path, lib):
    """handle_opts defaults (init.c:33-66) and search_settings (settings.c:16-81)."""
    import math
    from helpers import make_host, case_by_name
    host, m = make_host(case_by_name("cfg1_h1"), str(tmp_path))
    s = host.settings
    assert (s.N, s.nfft, s.nfftf, s.Ninterp, s.interpftpad, s.nd) == (86164, 131072, 131072, 262144, 2, 2)
    assert (s.nmin, s.nmax) == (1024, 64512)
    assert s.fpo == 10. + 0.96875 * 666 * 0.25
    assert s.oms == 2. * math.pi * s.fpo * 2.0
    o = host.opts()
    assert o.trl == 20 and o.use_range == 1 and o.white_flag == 0 and o.s0_flag == 0
    r = host.range
    assert (r.spndr[0], r.spndr[1], r.nr[0], r.nr[1], r.mr[0], r.mr[1]) == (-32, 31, 1, 1, 1, 1)
    assert host.config().phase_mode == 1 and host.config().precision == 0


def test_host_missing_nod_fails(lib):
    from polgraw_gb300.lib import _argv
    argv = ["x", "-data", "/nonexistent"]
    rc = C.c_int(0)
    h = lib.pa_host_create(len(argv), _argv(argv), C.byref(rc))
    assert not h and rc.value == 101


def test_host_getrange_writes_file(tmp_path, lib):
    from helpers import make_host, case_by_name
    path = str(tmp_path / "full_range.txt")
    from polgraw_gb300.lib import Host
    from casegen import materialize
    data = str(tmp_path / "data")
    os.makedirs(data)
    m = materialize(case_by_name("h1_fullgrid"), data)
    h = Host(m["args"] + ["-output", str(tmp_path / "out"), "-getrange", path, "--nocheckpoint"])
    assert h.setup_rc == 100  # reference exits after writing the range
    vals = [int(v) for v in open(path).read().split()]
    assert len(vals) == 8 and vals[0] <= vals[1] and vals[2] <= vals[3]


def test_host_fully_vetoed_band_exits(tmp_path, lib):
    from helpers import make_host, case_by_name
    host, _ = make_host(case_by_name("h1_addsig"), str(tmp_path), extra=["-narrowdown", "0"])
    assert host.setup_rc == 100


def test_host_checkpoint_resume(tmp_path, lib):
    """read_checkpoints (init.c:868-917): a state file restarts the sky loop at
    the recorded sky point and spindown, an empty one means nothing to do."""
    from polgraw_gb300.lib import Host
    from casegen import materialize
    from helpers import case_by_name
    data = str(tmp_path / "data")
    os.makedirs(data)
    m = materialize(case_by_name("h1l1_gaps_veto"), data)
    cwd = os.getcwd()
    os.chdir(str(tmp_path))
    try:
        with open("state_001_0200.dat", "w") as f:
            f.write("1 0 1 -3 40\n")
        h = Host(m["args"] + ["-output", str(tmp_path / "out")])
        r = h.range
        assert (r.pst, r.mst, r.nst, r.sst) == (1, 0, 1, -3)
        assert h.sky_points()[0] == (1, 0, 1)
        h.close()
        open("state_001_0200.dat", "w").close()
        h = Host(m["args"] + ["-output", str(tmp_path / "out")])
        assert h.setup_rc == 100
    finally:
        os.chdir(cwd)


def test_coinc_program_options_without_gpu(tmp_path, lib):
    """coincidences-gb300 parses the reference's options before touching a
    device: --help exits 0, a missing -nod fails like handle_opts_coinc
    (init.c:1112-1116), a missing grid.bin fails with its path."""
    import subprocess
    from polgraw_gb300 import build
    r = subprocess.run([build.COINC_EXE, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "-mincoin" in r.stdout and "-refloc" in r.stdout
    r = subprocess.run([build.COINC_EXE, "-data", str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "Number of days not set" in r.stdout
    out = tmp_path / "out"
    r = subprocess.run([build.COINC_EXE, "-nod", "2", "-output", str(out), "-refloc", str(tmp_path / "nogrid"),
                        "-snrcutoff", "4.5"], capture_output=True, text=True, timeout=60)
    assert r.returncode != 0 and "grid.bin" in r.stderr
    assert "corresponding to F-statistic value of 12.125000000000" in r.stdout
    assert out.is_dir()  # the output directory is created first, as the reference does


def test_coinc_create_validates_arguments(lib):
    from polgraw_gb300.lib import CoincCfg, PA_ERR_ARG, PA_ERR_NODEV
    cfg = CoincCfg()
    cfg.N, cfg.mincoin = 86164, 1
    for j in range(4):
        cfg.scale[j] = 1
    st = C.c_int(0)
    assert not lib.pa_coinc_create(C.byref(cfg), C.byref(st)) and st.value == PA_ERR_ARG
    assert b"mincoin" in lib.pa_coinc_last_error(None)
    cfg.mincoin, cfg.scale[2] = 3, 0
    assert not lib.pa_coinc_create(C.byref(cfg), C.byref(st)) and st.value == PA_ERR_ARG
    cfg.scale[2] = 1
    cc = lib.pa_coinc_create(C.byref(cfg), C.byref(st))
    if lib.pa_device_count() == 0:
        assert not cc and st.value == PA_ERR_NODEV
    elif cc:
        lib.pa_coinc_destroy(cc)
