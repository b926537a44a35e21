"""The fixed-point form's per-spindown het1 term is computed on the host and
passed with the launch parameters of the spindown pass A
(pa::het1_turns_fixed in csrc/pa_engine.cuh):
    het1 = fmod(ss M4, M0), wrapped into [0, M0) (jobcore.c:466-467),
    H = round-half-even(het1 2^64 / (2 pi)), saturated to [0, 2^64 - 1].
A host-only build of that function (nvcc, no GPU needed) against the same
formula in Python's IEEE doubles: fmod is exact and the two products are
single roundings, so every value must agree bit for bit, including ties
and the wrap of negative het1."""
import math
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "polgraw-allsky_gb300")
K = 2.9358905032820014e18  # 2^64 / (2 pi), as kTurnsPerRad64

SRC = r'''
#include <cstdio>
#include "pa_engine.cuh"
int main() {
  int ss;
  double M4, M0;
  while (scanf("%d %la %la", &ss, &M4, &M0) == 3)
    printf("%llu\n", (unsigned long long)pa::het1_turns_fixed(ss, M4, M0));
  return 0;
}
'''


def model(ss, m4, m0):
    het1 = math.fmod(float(ss) * m4, m0)
    if het1 < 0:
        het1 += m0
    x = het1 * K
    if not x > 0:
        return 0
    if x >= 2.0 ** 64:
        return 2 ** 64 - 1
    return round(x)  # Python rounds floats half to even


@pytest.fixture(scope="module")
def prog(tmp_path_factory):
    sys.path.insert(0, PKG)
    import build as pbuild
    try:
        nvcc = pbuild._nvcc()
    except RuntimeError:
        pytest.skip("nvcc not found")
    d = tmp_path_factory.mktemp("het1")
    src = d / "het1.cu"
    src.write_text(SRC)
    exe = d / "het1"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-std=c++17", "-O1",
                    "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(PKG, "csrc"),
                    "-I", os.path.join(ROOT, "include"), "-o", str(exe), str(src)], check=True)
    return str(exe)


def test_het1_constants_match_formula(prog):
    rng = np.random.default_rng(466)
    cases = []
    # the network workload's grid steps and spindown range, and random ones
    for m0, m4 in ((0.047936, -1.2e-9), (0.023968, 3.0e-7), (1.0, 0.5), (2 * math.pi, 1e-3)):
        cases += [(ss, m4, m0) for ss in range(-300, 301, 7)]
    for _ in range(3000):
        m0 = float(rng.uniform(1e-6, 6.0))
        m4 = float(rng.uniform(-1.0, 1.0)) * 10.0 ** float(rng.uniform(-9, 0))
        cases.append((int(rng.integers(-100000, 100000)), m4, m0))
    # het1 exactly 0, and M0 = 2 pi (x up to 2^64 - the saturation)
    cases += [(0, 0.3, 0.7), (5, 0.2, 1.0), (3, 2.0, 2 * math.pi), (-1, 1e-300, 2 * math.pi)]
    inp = "".join("%d %s %s\n" % (ss, m4.hex(), m0.hex()) for ss, m4, m0 in cases)
    out = subprocess.run([prog], input=inp, capture_output=True, text=True, check=True).stdout.split()
    assert len(out) == len(cases)
    bad = [(c, int(o), model(*c)) for c, o in zip(cases, out) if int(o) != model(*c)]
    assert not bad, bad[:5]
