"""The reference-side binding: the reference search program with its
job_core() call swapped for pa_job_core() by the patch kept in
oracle/ref_binding/ (file_scope.c after jobcore.c's includes, call_site.c in
place of the call at jobcore.c:107-120).

* The integration guide shows exactly those two files (its fenced C blocks
  equal them).
* oracle/build_oracle.py patches a copy of the reference's jobcore.c with
  them, compiles it against the reference's own struct.h / jobcore.h (the
  patch's _Static_asserts check that pa_range has Search_range's layout,
  that FLOAT_TYPE is double and NPAR is PA_NPAR) and links the program to
  libpolgraw_gb300.so.
* The program runs the reference's own set-up on the reference's input
  fixture; without a GPU it must stop at pa_create() with the library's
  "no CUDA device" error, with one its trigger records must equal the
  reference search's golden records (ref_testdata_001).

Runs where the reference checkout exists (it is not on the GPU machine).
"""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _guide_blocks():
    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        text = f.read()
    sec = text[text.index("## 2."):text.index("## 3.")]
    return re.findall(r"```c\n(.*?)```", sec, re.S)


def test_guide_shows_the_compiled_patch():
    blocks = _guide_blocks()
    files = [open(os.path.join(ROOT, "oracle", "ref_binding", n)).read() for n in ("file_scope.c", "call_site.c")]
    assert blocks == files


def test_patch_splices_into_jobcore():
    import build_oracle
    src = "#include \"timer.h\"\nvoid search(void) {\n\tint status;\n\tstatus = job_core(\n\t\t pm,\n\t\t FNum);  // x\n}\n"
    out = build_oracle.patch_jobcore(src)
    assert "status = job_core(" not in out
    assert out.index("static pa_ctx *make_ctx") < out.index("void search")
    assert "status = pa_job_core(pa_context" in out


def test_reference_program_with_gpu_job_core(tmp_path, lib):
    import build_oracle
    from polgraw_gb300 import build
    from casegen import materialize
    from helpers import case_by_name, golden
    if not build_oracle.reference_available():
        pytest.skip("reference checkout absent")
    exe = build_oracle.build_ref_binding(os.path.dirname(build.LIB))
    assert exe and os.path.exists(exe)
    nm = subprocess.run(["nm", "-D", "--undefined-only", exe], capture_output=True, text=True).stdout
    for sym in ("pa_create", "pa_job_core", "pa_last_error"):
        assert re.search(r"\b%s\b" % sym, nm), sym
    assert "job_core" not in re.sub(r"pa_job_core", "", nm)
    case = case_by_name("ref_testdata_001")
    data = str(tmp_path / "data")
    os.makedirs(data)
    m = materialize(case, data)
    out = str(tmp_path / "out")
    os.makedirs(out)
    r = subprocess.run(["bash", "-c", 'ulimit -s unlimited; exec "$0" "$@"', exe] + m["args"] +
                       ["-output", out, "--nocheckpoint"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=900)
    if lib.pa_device_count() < 1:
        assert r.returncode != 0
        assert "pa_create: no CUDA device" in r.stderr, r.stderr[-2000:]
        return
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    g = golden("ref_testdata_001")
    rec = np.fromfile(os.path.join(out, g["trigger_files"][0]), dtype="<f8").reshape(-1, 5)
    ref = np.array([c[5:] for c in g["candidates"]])
    assert rec.shape == ref.shape
    np.testing.assert_array_equal(rec[:, :4], ref[:, :4])
    np.testing.assert_allclose(rec[:, 4], ref[:, 4], rtol=1e-4)
