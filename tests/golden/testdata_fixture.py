"""The reference's own search fixture testdata/test-gpu-cpu/001 (H1+L1,
N=86164 at dt=2 s, band 666: real-shaped Gaussian-noise data with gaps of
exact zeros, a barycentric ephemeris per detector and a grid.bin with
frequency-spindown and frequency-sky couplings), packed losslessly into
testdata_001.npz by make_testdata_fixture.py so that the tests can use it
where the reference checkout does not exist.

Packing: xdatc and grid.bin as raw bytes (zlib in the npz); DetSSB.bin's 3N
positions as the second differences, along time, of their IEEE-754 bit
patterns taken as 64-bit integers (wrap-around integer arithmetic, so the
inverse is exact), which compress six-fold against one and a half for the
raw doubles; the trailing phir, epsm doubles raw.  unpack() checks the
SHA-256 of every file it writes against the originals'.
"""
from __future__ import annotations

import hashlib
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "testdata_001.npz")
DETS = ("H1", "L1")
IDENT, BAND = 1, 666


def detssb_encode(raw: bytes) -> tuple[np.ndarray, np.ndarray]:
    d = np.frombuffer(raw, dtype="<f8")
    pos = d[:-2].view("<i8").reshape(-1, 3)
    enc = pos.copy()
    enc[1:] = pos[1:] - pos[:-1]
    enc[2:] = enc[2:] - enc[1:-1]
    return enc, d[-2:].copy()


def detssb_decode(enc: np.ndarray, tail: np.ndarray) -> bytes:
    # enc[0] = p_0, enc[1] = p_1 - p_0, enc[k] = (p_k - p_{k-1}) - (p_{k-1} - p_{k-2})
    e = np.asarray(enc, dtype="<i8")
    dif = np.cumsum(e[1:], axis=0, dtype="<i8")            # p_k - p_{k-1}, k >= 1
    pos = np.empty_like(e)
    pos[0] = e[0]
    pos[1:] = np.cumsum(dif, axis=0, dtype="<i8") + e[0]
    return pos.reshape(-1).view("<f8").tobytes() + np.asarray(tail, dtype="<f8").tobytes()


def _sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def unpack(root: str, dets=DETS) -> dict:
    """Writes <root>/001/grid.bin and <root>/001/<det>/{xdatc_001_0666.bin,
    DetSSB.bin, grid.bin}; returns {file key: sha256} in the key convention
    of polgraw_gb300.synth.write_dataset (grid.bin, <det>/xdat,
    <det>/DetSSB, and <det>/grid for the per-detector grid)."""
    z = np.load(FIXTURE)
    base = os.path.join(root, "%03d" % IDENT)
    os.makedirs(base, exist_ok=True)
    files = {}
    grid = z["grid"].tobytes()
    with open(os.path.join(base, "grid.bin"), "wb") as f:
        f.write(grid)
    files["grid.bin"] = _sha(grid)
    assert files["grid.bin"] == str(z["sha_grid"]), "grid.bin differs from the reference fixture"
    for d in dets:
        dd = os.path.join(base, d)
        os.makedirs(dd, exist_ok=True)
        x = z[d + "_xdat"].tobytes()
        p = detssb_decode(z[d + "_detssb"], z[d + "_tail"])
        gd = z[d + "_grid"].tobytes()
        for name, b, key in (("xdatc_%03d_%04d.bin" % (IDENT, BAND), x, d + "/xdat"),
                             ("DetSSB.bin", p, d + "/DetSSB"), ("grid.bin", gd, d + "/grid")):
            with open(os.path.join(dd, name), "wb") as f:
                f.write(b)
            files[key] = _sha(b)
            assert files[key] == str(z["sha_" + key.replace("/", "_")]), "%s differs from the reference fixture" % key
    return files
