"""Golden-fixture cases: synthetic inputs (regenerated bit-identically from
the parameters below by polgraw_gb300.synth) and the reference search's
command line for each.  make_golden.py runs the reference search built from
its own sources (oracle/_ref/gwsearch-ref) on them and records its
candidates in <name>.json next to this file.

Coverage (reference file:line of the behaviour each case exercises):
  h1_addsig        -addsig injection and its grid range (init.c:462-651)
  h1l1_gaps_veto   two detectors, data gaps (init.c:359-367), grid with
                   M4, M8, M9, M12, M13 != 0 (het1 wrap, jobcore.c:466-467),
                   fftpad 2, lowered threshold (run clustering,
                   jobcore.c:659-669), -narrowdown band veto (settings.c:535-550)
  h1l1_white_pm2   --whitenoise (no FStat normalisation, jobcore.c:650),
                   second hemisphere (lin2ast pm = 2, auxi.c:19)
  h1_fullgrid      no -range/-addsig: gridr sky range (auxi.c:143-212) and the
                   Smin/Smax spindown range with trunc and swap (jobcore.c:424-439)
  h1_nospindown    --nospindown (jobcore.c:444, 456)
  cfg1_h1          the 1-detector N=86164 workload: 1 sky point (delta 0.3,
                   alpha 1.2) x 64 spindowns, injected f=0.1 fdot=-1e-8 SNR 12
"""
import math

CASES = [
    dict(name="h1_addsig",
         data=dict(dets=["H1"], dt=8.0, nod=1, band=100, fftpad=1,
                   grid=dict(m5=-2e-8, sky_scale=0.05)),
         addsig=dict(f=1.0, fdot=-6.6e-8, delta=0.3, alpha=1.2, snr=15.0, gsize=2),
         args=["-threshold", "20"]),
    dict(name="h1l1_gaps_veto",
         data=dict(dets=["H1", "L1"], dt=4.0, nod=1, band=200, fftpad=2, gaps=0.2,
                   grid=dict(m5=-3e-8, m4=3.7e-4, m8=2.1e-2, m9=1.7e-9, m12=-2.9e-2, m13=2.3e-9,
                             sky_scale=0.04, skew=0.3)),
         range=[-6, 6, -1, 1, -1, 1, 1, 1],
         args=["-threshold", "13", "-narrowdown", "0.35"]),
    dict(name="h1l1_white_pm2",
         data=dict(dets=["H1", "L1"], dt=8.0, nod=2, band=50, fftpad=1,
                   grid=dict(m5=-1.5e-8, sky_scale=0.06)),
         range=[0, 8, -1, 1, 0, 1, 2, 2],
         args=["-threshold", "12", "--whitenoise"]),
    dict(name="h1_fullgrid",
         data=dict(dets=["H1"], dt=8.0, nod=1, band=120, fftpad=1,
                   grid=dict(m5=-2e-7, sky_scale=0.55)),
         args=["-threshold", "14", "-hemisphere", "1"]),
    dict(name="h1_nospindown",
         data=dict(dets=["H1"], dt=8.0, nod=1, band=80, fftpad=1,
                   grid=dict(m5=-2e-8, sky_scale=0.05)),
         range=[0, 3, -2, 2, -1, 1, 1, 2],
         args=["-threshold", "10", "--nospindown", "--nocheckpoint"]),
    dict(name="cfg1_h1",
         data=dict(dets=["H1"], dt=2.0, nod=2, band=666, fftpad=1,
                   grid=dict(m5=-1e-9, sky_point=(0.3, 1.2))),
         inject=dict(f=0.1, fdot=-1e-8, delta=0.3, alpha=1.2, snr=12.0),
         range=[-32, 31, 1, 1, 1, 1, None, None],
         args=["-threshold", "20"]),
]


# Followup (demodulated F-statistic) cases: data with one injected signal;
# make_followup_golden.py evaluates the reference followup program's own
# Fstatnet() at points around the injection and runs its simplex (amoeba)
# from offset starting points.
#   fu_h1l1v1   three detectors (H1, L1, V1), N=10771 (1 day at dt=8 s)
FOLLOWUP_CASES = [
    dict(name="fu_h1l1v1",
         data=dict(dets=["H1", "L1", "V1"], dt=8.0, nod=1, band=100, fftpad=1,
                   grid=dict(m5=-2e-8, sky_scale=0.05)),
         inject=dict(f=1.0, fdot=-6e-8, delta=0.3, alpha=1.2, snr=25.0),
         range=[0, 0, 0, 0, 0, 0, None, None]),
]
