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
  h1l1_gridgen     a grid made by the reference grid generator (gridgen/) from
                   the synthetic ephemeris: lower-triangular M with frequency-
                   sky and frequency-spindown couplings (make_gridgen_grids.py)
  h1l1v1_addsig    three detectors (H1, L1, V1: the detector sum of
                   jobcore.c:471-623 and the weights of :374-393 over nifo=3),
                   -addsig network injection, M4 != 0, lowered threshold
  h1v1_lines_usedet  three detectors on disk, -usedet H1V1 (init.c:150-152,
                   detector selection), --vetolines (main.c:89-98) with
                   known-lines files per detector
                   (read_lines settings.c:327-400: types 0, 1 and 2, lines out
                   of band, the unused detector's file ignored) merged into
                   the band veto (lines_in_band, jobcore.c:675-684)
  h1l1_label_pm2   -label (input xdatc_<ident>_<band>_<label>.bin, trigger
                   and state file names, init.c:174-175, jobcore.c:92-93),
                   second hemisphere only
  h1l1_amp_fpo     -addsig in the amplitude form ("amp h0 gsize reffr",
                   init.c:488-490) with grid size 1; explicit -fpo, which
                   places the known line of L1 in the band (lines_in_band)
  cfg1_h1          the 1-detector N=86164 workload: 1 sky point (delta 0.3,
                   alpha 1.2) x 64 spindowns, injected f=0.1 fdot=-1e-8 SNR 12
  ref_testdata_001 the reference's own input fixture testdata/test-gpu-cpu/001
                   (H1+L1, N=86164, dt=2 s, band 666: real-shaped noise with
                   42 % / 53 % gaps of exact zeros, a barycentric ephemeris
                   and a grid with M4, M8, M9, M12, M13 != 0) with the
                   command line and range file of the reference's sample run
                   (search/network/src-gpu/runme, src-gpu/range.dat: 15 sky
                   points x 81 spindowns, -usedet H1L1, default threshold)
  ref_testdata_001_wide  the same fixture over 35 sky points x 138 spindowns,
                   the union of the Smin/Smax spindown ranges of those sky
                   points (jobcore.c:424-439), threshold 35
  ref_testdata_001_l1  the same fixture, -usedet L1: one detector and that
                   detector's own grid.bin (init.c:299-301), threshold 50
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
    dict(name="h1l1_gridgen",
         data=dict(dets=["H1", "L1"], dt=2.0, nod=1, band=666, fftpad=1,
                   grid=dict(gridgen="grid_h1l1_gridgen.bin", nfft_exp=16)),
         inject=dict(f=1.3, fdot=0.0, delta=0.5, alpha=2.1, snr=20.0),
         range=[-2, 2, 0, 1, -4, -3, None, None],
         args=["-threshold", "16"]),
    dict(name="h1l1v1_addsig",
         data=dict(dets=["H1", "L1", "V1"], dt=8.0, nod=1, band=150, fftpad=1,
                   grid=dict(m5=-2e-8, m4=2.9e-4, sky_scale=0.05)),
         addsig=dict(f=1.7, fdot=-4.0e-8, delta=0.3, alpha=1.2, snr=14.0, gsize=2),
         args=["-threshold", "12"]),
    dict(name="h1v1_lines_usedet",
         data=dict(dets=["H1", "L1", "V1"], dt=8.0, nod=1, band=120, fftpad=1,
                   grid=dict(m5=-1.5e-8, sky_scale=0.05)),
         # band 120 at dt=8: fpo = 17.265625 Hz, width 0.0625 Hz
         lines={"H1": [[17.28, 0, 0.0, 0, 0, 0, 0], [30.0, 0, 0.0, 0, 0, 0, 0]],
                "L1": [[17.30, 0, 0.0, 0, 0, 0, 0]],
                "V1": [[1.0, 1, 0.31, 15, 18, 0, 0], [8.6485, 2, 0.0, 2, 2, 0, 0]]},
         range=[-4, 4, -1, 1, -1, 1, 1, 1],
         args=["-threshold", "11", "-usedet", "H1V1", "--vetolines"]),
    dict(name="h1l1_label_pm2",
         data=dict(dets=["H1", "L1"], dt=8.0, nod=1, band=90, fftpad=1,
                   grid=dict(m5=-1.2e-8, sky_scale=0.05)),
         label="O3a",
         range=[-3, 3, -1, 1, -1, 0, 2, 2],
         args=["-threshold", "11"]),
    dict(name="h1l1_amp_fpo",
         data=dict(dets=["H1", "L1"], dt=8.0, nod=1, band=60, fftpad=1,
                   grid=dict(m5=-2e-8, sky_scale=0.05)),
         addsig=dict(f=2.2, fdot=-3e-8, delta=0.3, alpha=1.2, amp=0.25, gsize=1),
         # with -fpo 20.0 the band is [20.0, 20.0625] Hz
         lines={"L1": [[20.04, 0, 0.0, 0, 0, 0, 0]]},
         args=["-threshold", "12", "-fpo", "20.0", "--vetolines"]),
    dict(name="cfg1_h1",
         data=dict(dets=["H1"], dt=2.0, nod=2, band=666, fftpad=1,
                   grid=dict(m5=-1e-9, sky_point=(0.3, 1.2))),
         inject=dict(f=0.1, fdot=-1e-8, delta=0.3, alpha=1.2, snr=12.0),
         range=[-32, 31, 1, 1, 1, 1, None, None],
         args=["-threshold", "20"]),
    dict(name="ref_testdata_001",
         data=dict(fixture="testdata_001", dets=["H1", "L1"], dt=2.0, nod=2, band=666, fftpad=1),
         range=[-40, 40, -1, 1, -2, 2, 1, 1],
         args=["-usedet", "H1L1"]),
    dict(name="ref_testdata_001_wide",
         data=dict(fixture="testdata_001", dets=["H1", "L1"], dt=2.0, nod=2, band=666, fftpad=1),
         range=[-16, 121, -2, 2, -3, 3, 1, 1],
         args=["-threshold", "35"]),
    dict(name="ref_testdata_001_l1",
         data=dict(fixture="testdata_001", dets=["H1", "L1"], dt=2.0, nod=2, band=666, fftpad=1),
         range=[-40, 40, -1, 1, -2, 2, 1, 1],
         args=["-usedet", "L1", "-threshold", "50"]),
]


# Followup (demodulated F-statistic) cases: data with one injected signal;
# make_followup_golden.py evaluates the reference followup program's own
# Fstatnet() at points around the injection and runs its simplex (amoeba)
# from offset starting points.
#   fu_h1l1v1   three detectors (H1, L1, V1), N=10771 (1 day at dt=8 s)
#   fu_h1l1_dt2 two detectors (H1, L1), N=43082 (1 day at dt=2 s), southern sky
#   fu_h1l1v1_n86164 the followup configuration's size: three detectors
#               (H1, L1, V1), N=86164 (2 sidereal days at dt=2 s)
FOLLOWUP_CASES = [
    dict(name="fu_h1l1v1",
         data=dict(dets=["H1", "L1", "V1"], dt=8.0, nod=1, band=100, fftpad=1,
                   grid=dict(m5=-2e-8, sky_scale=0.05)),
         inject=dict(f=1.0, fdot=-6e-8, delta=0.3, alpha=1.2, snr=25.0),
         range=[0, 0, 0, 0, 0, 0, None, None],
         # no other maximum of F within 0.5 peak widths of the injection
         unimodal=True),
    dict(name="fu_h1l1_dt2",
         data=dict(dets=["H1", "L1"], dt=2.0, nod=1, band=666, fftpad=1,
                   grid=dict(m5=-1e-9, sky_scale=0.05)),
         inject=dict(f=2.0, fdot=-2e-8, delta=-0.5, alpha=4.0, snr=20.0),
         range=[0, 0, 0, 0, 0, 0, None, None],
         # local maxima of F (about 151.6 and 102) lie within 0.5 peak widths
         # of the peak (152.1): an ascent from a nearby start may stop there
         unimodal=False),
    dict(name="fu_h1l1v1_n86164",
         data=dict(dets=["H1", "L1", "V1"], dt=2.0, nod=2, band=666, fftpad=1,
                   grid=dict(m5=-1e-9, sky_scale=0.05)),
         inject=dict(f=1.5, fdot=-5e-9, delta=0.2, alpha=3.0, snr=20.0),
         range=[0, 0, 0, 0, 0, 0, None, None],
         # a long ridge through the peak (172.4: ascents from nearby starts
         # stall on it near 172.2) and a far side maximum near 46 reached
         # from a start at F = 3
         unimodal=False),
]

# Coincidence step (coincidences/src/coincidences.c) over synthetic trigger
# files of several frames (polgraw_gb300.synth.coinc_triggers) and a grid.bin
# with a Fisher matrix (synth.fisher_matrix).  make_coinc_golden.py runs the
# reference coincidence program built from its own sources
# (oracle/_ref/coincidences-ref) and records its .coi file, its stderr line
# and the directory order it read the frames in.
#   coinc_basic       defaults (mincoin 3, no shift/scale, narrowdown 0.5)
#   coinc_shift_scale cell shifts and scaling digits (coincidences.c:157-184),
#                     mincoin 2, narrowed band, higher SNR cut
#   coinc_quirks      crafted frames: SNR ties, a run whose best member is the
#                     frame's first record (index 0 doubles as the "no run"
#                     flag), frames whose last run meets the row left over from
#                     an earlier frame, and a coincidence in the last cell of
#                     the sorted table (written with multiplicity 0)
#   coinc_many        24 frames x 5000 records, mincoin 4
#   coinc_gridgen     the Fisher matrix of a grid made by the reference grid
#                     generator from the synthetic ephemeris (N=86164)
COINC_CASES = [
    dict(name="coinc_basic", nod=2, dt=2.0, band=666, frames=[1, 2, 3, 5, 8, 9], per_frame=2000, seed=7,
         refr=3, mincoin=3, shift=0, scale=1111, narrowdown=0.5, snrcutoff=6.0),
    dict(name="coinc_shift_scale", nod=2, dt=2.0, band=666, frames=[2, 4, 6, 7], per_frame=1500, seed=11,
         refr=4, mincoin=2, shift=1011, scale=2412, narrowdown=0.3, snrcutoff=6.5),
    dict(name="coinc_quirks", nod=2, dt=2.0, band=666, frames=[1, 2, 3, 4, 5, 6], per_frame=160, seed=5,
         refr=2, mincoin=3, shift=0, scale=1111, narrowdown=0.5, snrcutoff=6.0, craft=True),
    dict(name="coinc_many", nod=2, dt=2.0, band=666, frames=list(range(1, 25)), per_frame=5000, seed=3,
         refr=12, mincoin=4, shift=0, scale=1111, narrowdown=0.5, snrcutoff=6.0),
    dict(name="coinc_gridgen", nod=2, dt=2.0, band=666, frames=[1, 2, 3, 4, 5, 6, 7, 8], per_frame=3000, seed=13,
         refr=4, mincoin=3, shift=0, scale=1111, narrowdown=0.5, snrcutoff=6.0,
         grid="grid_coinc_gridgen.bin", nfft_exp=17),
]
