"""Shared test helpers: materialise a golden case, build the host set-up and
compare candidate lists."""
from __future__ import annotations

import json
import os

import numpy as np

from casegen import materialize
from cases import CASES

GOLDEN_DIR = os.path.dirname(os.path.abspath(__file__)) + "/golden"


def case_by_name(name: str) -> dict:
    return [c for c in CASES if c["name"] == name][0]


def golden(name: str) -> dict:
    with open(os.path.join(GOLDEN_DIR, name + ".json")) as f:
        return json.load(f)


def make_host(case: dict, tmp: str, extra=()):
    from polgraw_gb300.lib import Host
    data = os.path.join(tmp, "data")
    os.makedirs(data, exist_ok=True)
    m = materialize(case, data)
    args = m["args"] + ["-output", os.path.join(tmp, "out"), "--nocheckpoint"] + list(extra)
    return Host(args), m


def run_sky_loop(job_core, host):
    """Runs job_core over the host's sky loop; returns (records, idx, FNum)."""
    recs, idxs, fnum = [], [], 0
    opts = host.opts()
    rng = host.range
    for k, (pm, mm, nn) in enumerate(host.sky_points()):
        if k > 0:
            rng.sst = rng.spndr[0]
        r, i, f = job_core(pm, mm, nn, opts, rng)
        recs.append(r)
        idxs.append(i)
        fnum += f
    rec = np.concatenate(recs) if recs else np.zeros((0, 5))
    idx = np.concatenate(idxs) if idxs else np.zeros(0)
    return rec, idx, fnum


def key_of(idx) -> list[tuple]:
    return [(int(x["pm"]), int(x["mm"]), int(x["nn"]), int(x["ss"]), int(x["ii"])) for x in idx]


def compare_candidates(ref_keys, ref_F, got_keys, got_F, trl, rtol):
    """Candidates must agree index for index except where the reference F
    lies within rtol of the threshold or an argmax tie is within rtol (the
    threshold edge).  Returns (matched, max relative F error, report)."""
    ref = dict(zip(ref_keys, ref_F))
    got = dict(zip(got_keys, got_F))
    bad = []
    for k, F in ref.items():
        if k not in got and abs(F - trl) > rtol * trl:
            # a tie inside the run: the other side reports a neighbour bin of
            # the same sky/spindown with F within rtol
            near = [g for g in got if g[:4] == k[:4] and abs(g[4] - k[4]) <= 4 and abs(got[g] - F) <= rtol * F]
            if not near:
                bad.append(("missing", k, F))
    for k, F in got.items():
        if k not in ref and abs(F - trl) > rtol * trl:
            near = [g for g in ref if g[:4] == k[:4] and abs(g[4] - k[4]) <= 4 and abs(ref[g] - F) <= rtol * F]
            if not near:
                bad.append(("extra", k, F))
    common = [k for k in ref if k in got]
    err = max([abs(got[k] - ref[k]) / ref[k] for k in common], default=0.0)
    return len(common), err, bad


def snr_to_F(snr: np.ndarray, nd: int = 2) -> np.ndarray:
    return snr * snr / 2.0 + nd


def parse_coi(b: bytes) -> list:
    """Records of a .coi file (coincidences.c:529-533): (w, 5 floats, frames,
    positions)."""
    import struct
    out, o = [], 0
    while o < len(b):
        w = struct.unpack_from("<H", b, o)[0]
        o += 2
        m = np.frombuffer(b[o:o + 20], dtype="<f4").copy()
        o += 20
        fra = np.frombuffer(b[o:o + 2 * w], dtype="<u2").copy()
        o += 2 * w
        ops = np.frombuffer(b[o:o + 4 * w], dtype="<i4").copy()
        o += 4 * w
        out.append((w, m, fra, ops))
    return out


def canon_coi(b: bytes) -> bytes:
    """The .coi bytes with every NaN mean written as 0x7fc00000: the
    multiplicity-0 record's means are 0/0, whose sign bit is the machine's
    (set on x86-64, clear on aarch64)."""
    out = bytearray(b)
    o = 0
    import struct
    while o < len(b):
        w = struct.unpack_from("<H", b, o)[0]
        for k in range(5):
            p = o + 2 + 4 * k
            v = np.frombuffer(b[p:p + 4], dtype="<f4")[0]
            if np.isnan(v):
                out[p:p + 4] = struct.pack("<I", 0x7FC00000)
        o += 22 + 6 * w
    return bytes(out)
