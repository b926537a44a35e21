"""Packs the reference's search fixture testdata/test-gpu-cpu/001 (the input
of the reference's sample GPU run, search/network/src-gpu/runme) into
tests/golden/testdata_001.npz, losslessly (testdata_fixture.py gives the
encoding), with the SHA-256 of every original file.

Run here, where the reference checkout exists (its location is
POLGRAW_REFERENCE, default the build's reference root):
    python tests/golden/make_testdata_fixture.py
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import build_oracle  # noqa: E402
from testdata_fixture import DETS, FIXTURE, detssb_decode, detssb_encode  # noqa: E402

SRC = os.path.join(build_oracle.REFERENCE_ROOT, "testdata", "test-gpu-cpu", "001")


def main() -> None:
    if not os.path.isdir(SRC):
        raise SystemExit("reference fixture not found at " + SRC)
    out = {}
    grid = open(os.path.join(SRC, "grid.bin"), "rb").read()
    out["grid"] = np.frombuffer(grid, dtype=np.uint8)
    out["sha_grid"] = np.array(hashlib.sha256(grid).hexdigest())
    for d in DETS:
        x = open(os.path.join(SRC, d, "xdatc_001_0666.bin"), "rb").read()
        p = open(os.path.join(SRC, d, "DetSSB.bin"), "rb").read()
        # the per-detector grid.bin (read with -usedet of one detector,
        # init.c:299-301) differs from the network one
        gd = open(os.path.join(SRC, d, "grid.bin"), "rb").read()
        out[d + "_grid"] = np.frombuffer(gd, dtype=np.uint8)
        out["sha_%s_grid" % d] = np.array(hashlib.sha256(gd).hexdigest())
        enc, tail = detssb_encode(p)
        assert detssb_decode(enc, tail) == p
        out[d + "_xdat"] = np.frombuffer(x, dtype=np.uint8)
        out[d + "_detssb"] = enc
        out[d + "_tail"] = tail
        out["sha_%s_xdat" % d] = np.array(hashlib.sha256(x).hexdigest())
        out["sha_%s_DetSSB" % d] = np.array(hashlib.sha256(p).hexdigest())
    np.savez_compressed(FIXTURE, **out)
    print("%s: %d bytes" % (FIXTURE, os.path.getsize(FIXTURE)))


if __name__ == "__main__":
    main()
