"""bench.py's reference arm on the CPU: one bounded step of the CPU oracle on
the H1+L1 N=86164 workload (1 sky point x 8 spindowns) prints exactly one JSON
line carrying the bench contract's keys, with the CPU baseline and an e2e
figure that moves no bytes to or from a device, having loaded no library of
the product (only the oracle's), and reports the committed
same-host calibration against the reference's own OpenMP build."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def test_reference_arm_prints_one_contract_line(lib):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-sky", "1", "--spindowns", "8"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, lines
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    for k in KEYS:
        assert k in d, k
    assert d["value"] > 0 and d["unit"] == "templates/s" and d["higher_is_better"] is True
    assert d["config"]["spindowns"] == 8 and d["config"]["N"] == 86164
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    # the CPU arm reads its inputs with the oracle's own set-up: no library
    # of the product is loaded, only the oracle's timing build
    libs = d["libraries_loaded"]
    assert "oracle/_build/liboracle_fast.so" in libs and all(x.startswith("oracle/") for x in libs), libs
    cal = cb["calibration"]
    assert cal is not None and cal["port_over_reference"] > 0
