"""The oracle-side input set-up (oracle/oracle_setup.py), which the CPU
baseline and the reference arm of the benchmark use instead of the product's
host library, against the product host (lib.Host): every settings field,
every detector constant and the data arrays bit for bit, the range and the
sky-loop order, on the benchmark's network workload and on the reference's
own input fixture (real gaps and ephemeris)."""
import os

import numpy as np
import pytest

import oracle_setup

SFIELDS = ["fpo", "dt", "B", "oms", "omr", "Smin", "Smax", "sepsm", "cepsm", "nfft", "nod", "N", "nfftf",
           "nmax", "nmin", "s", "nd", "interpftpad", "fftpad", "Ninterp", "nifo"]


def _compare(inp, host):
    a, b = inp.settings, host.settings
    for f in SFIELDS:
        assert getattr(a, f) == getattr(b, f), f
    assert list(a.M) == list(b.M)
    da, na = inp.detectors()
    db, nb = host.detectors()
    assert na == nb
    N = a.N
    for n in range(na):
        for f in ("sig2", "sphir", "cphir"):
            assert getattr(da[n], f) == getattr(db[n], f), (n, f)
        assert list(da[n].amod) == list(db[n].amod)
        assert np.array_equal(np.ctypeslib.as_array(da[n].xDat, (N,)), np.ctypeslib.as_array(db[n].xDat, (N,)))
        assert np.array_equal(np.ctypeslib.as_array(da[n].DetSSB, (3 * N,)),
                              np.ctypeslib.as_array(db[n].DetSSB, (3 * N,)))
    ra, rb = inp.range, host.range
    for f in ("pmr", "mr", "nr", "spndr"):
        assert list(getattr(ra, f)) == list(getattr(rb, f)), f
    for f in ("pst", "mst", "nst", "sst"):
        assert getattr(ra, f) == getattr(rb, f), f
    oa, ob = inp.opts(), host.opts()
    for f in ("trl", "white_flag", "s0_flag", "use_range"):
        assert getattr(oa, f) == getattr(ob, f), f
    assert inp.sky_points() == host.sky_points()


def test_setup_network_workload(tmp_path, lib):
    from polgraw_gb300 import workloads
    from polgraw_gb300.lib import Host
    root = str(tmp_path)
    argv, _ = workloads.network(root, 200)
    host = Host(argv)
    inp = oracle_setup.Inputs(root, ident=1, band=666, dt=2.0, nod=2, range_file=os.path.join(root, "range.txt"))
    _compare(inp, host)


def test_setup_reference_fixture(tmp_path, lib):
    from helpers import case_by_name, make_host
    case = case_by_name("ref_testdata_001")
    host, m = make_host(case, str(tmp_path))
    inp = oracle_setup.Inputs(str(tmp_path / "data"), ident=1, band=666, dt=2.0, nod=2,
                              range_file=str(tmp_path / "data" / "range.txt"))
    _compare(inp, host)
