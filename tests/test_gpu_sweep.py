"""GPU parity of the CThmScan sweep (0_GEN/CThmScan.cpp) against the
reference's golden sweep results and the oracle, through the C ABI.

The bar (oracle/sweep_bar.py): the oracle notes every decision that steers
the search with its margin.  Where none is a tie (relative score margin
<= oracle.SWEEP_EPS = 1e-5, or a rounded offset within 1e-4 px of its
rounding boundary -- both far above the FP32 correlator's error) the GPU
must land on the identical angle, with the same err code, R within 1e-4
relative and X, Y within 0.01 px.  Where the oracle met a tie, the angle may
move by at most the bound the oracle derives for it (PeakHunt: the bracket
it held at its first tie).
"""
import concurrent.futures as cf

import numpy as np
import pytest

from conftest import load_golden
from oracle.sweep_bar import SweepStats, check

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    yield c
    c.close()


def _golden_search(orc, d):
    """The oracle's search on a golden case's inputs and parameters (with
    its decision margins); the oracle is pinned to the reference's numbers
    there, which is asserted again."""
    o = orc.thm_search(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]),
                       rthresh=float(d["rthresh"]), pretweak=int(d["pretweak"]),
                       disc=tuple(int(v) for v in d["disc"]), mode=int(d["mode"]),
                       ang0=float(d["ang0"]), hfang=float(d["hfang"]), step=float(d["step"]),
                       usecorrr=int(d["usecorrr"]) if "usecorrr" in d else 1)
    for k in ("A", "X", "Y", "R"):
        assert o[k] == float(d[k]), (k, o[k], float(d[k]))
    assert o["err"] == int(d["err"])
    return o


@pytest.mark.parametrize("case", sorted(load_golden("thm_scan")))
def test_sweep_golden(ctx, orc, case):
    import alignment_projects_gb300 as aln
    d = load_golden("thm_scan")[case]
    o = _golden_search(orc, d)
    T = aln.thumbs_from_points(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]))
    disc = tuple(int(v) for v in d["disc"])
    g = ctx.thm_search_batch([T], rthresh=float(d["rthresh"]), pretweak=int(d["pretweak"]),
                             disc=disc, mode=int(d["mode"]), ang0=float(d["ang0"]),
                             hfang=float(d["hfang"]), step=float(d["step"]))[0]
    check(g, o, case)


def _thumb_inputs(orc, seed, tile, dec):
    """Thumbnails of two tile x tile tiles (B rotated / shifted), binned by
    `dec` and normalised (MakeThumbs), as point lists."""
    import oracle
    from alignment_projects_gb300 import synth
    ta, tb, th, t = synth.thumb_pair(seed, tile=tile, dec=dec)
    n = tile // dec
    A, VA = oracle.image_to_points(ta)
    B, VB = oracle.image_to_points(tb)
    A, VA = orc.decimate_normalize(A, VA, n, n, 1)
    B, VB = orc.decimate_normalize(B, VB, n, n, 1)
    return A, VA, B, VB, th


def _sweep_vs_oracle(ctx, orc, seeds, tile, dec, req):
    import alignment_projects_gb300 as aln
    ins = [_thumb_inputs(orc, s, tile, dec) for s in seeds]
    with cf.ThreadPoolExecutor(max_workers=len(ins)) as ex:
        refs = list(ex.map(lambda t: orc.thm_search(t[0], t[1], t[2], t[3], req, mode=0,
                                                    ang0=0.0, hfang=10.0, step=0.5), ins))
    thumbs = [aln.thumbs_from_points(t[0], t[1], t[2], t[3], req) for t in ins]
    got = ctx.thm_search_batch(thumbs, mode=aln.THM_DENOVO, ang0=0.0, hfang=10.0, step=0.5)
    st = SweepStats()
    for k, (g, o) in enumerate(zip(got, refs)):
        st.add(check(g, o, f"seed {seeds[k]}"))
    return st, got, ins


def test_sweep_batch_of_pairs_matches_oracle(ctx, orc):
    """Several 96^2 thumbnail pairs in one call, against the oracle pair by pair."""
    st, _, _ = _sweep_vs_oracle(ctx, orc, [40, 41, 42, 43], tile=768, dec=8, req=195)
    assert st.table()["pairs"] == 4


def test_sweep_thumbnail_config_size(ctx, orc):
    """The cross-layer sweep at its production size: 256^2 thumbnails of
    2048^2 tiles (1024^2 transforms), DenovoBestAngle(0, 10, 0.5) with
    ApproximateMatch's settings (ConstXY, CorrImagesS, reqArea 3125), ~140
    correlator calls per pair, against the oracle pair by pair."""
    st, got, ins = _sweep_vs_oracle(ctx, orc, [301, 302, 303], tile=2048, dec=8, req=3125)
    t = st.table()
    assert t["pairs"] == 3
    # the synthetic rotation is recovered (B is A rotated by -theta)
    for g, i in zip(got, ins):
        assert g["err"] == 0 and abs(g["A"] + i[4]) < 0.5, (g, i[4])


@pytest.mark.parametrize("case", sorted(load_golden("thm_finish")))
def test_finish_golden(ctx, case):
    """PostTweaks / FinishAtFullRes from the reference's prior, against its
    golden results (the same bar as the sweep)."""
    import alignment_projects_gb300 as aln
    d = load_golden("thm_finish")[case]
    T = aln.thumbs_from_points(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]))
    prior = dict(zip("AXYR", (float(v) for v in d["prior"])))
    g = ctx.thm_finish_batch([T], int(d["mode"]), [prior], tptwk=[d["tptwk"]])[0]
    # both keep the prior's angle: it must come back unchanged
    assert g["A"] == float(d["A"]), (case, g)
    assert abs(g["R"] - float(d["R"])) <= 1e-4 * max(1.0, abs(float(d["R"]))), (case, g)
    assert abs(g["X"] - float(d["X"])) <= 0.01 and abs(g["Y"] - float(d["Y"])) <= 0.01, (case, g)
    assert np.abs(np.array(g["tptwk"]) - d["tptwk_out"]).max() <= 1e-6, (g, d["tptwk_out"])


@pytest.mark.parametrize("case", sorted(load_golden("thm_scan_f")))
def test_sweep_f_golden(ctx, orc, case):
    """useCorrR off: every correlator call is CorrImagesF."""
    import alignment_projects_gb300 as aln
    d = load_golden("thm_scan_f")[case]
    o = _golden_search(orc, dict(d, usecorrr=0, rthresh=0.3, pretweak=0,
                                 disc=np.array([0, 0, -1, -1])))
    T = aln.thumbs_from_points(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]))
    g = ctx.thm_search_batch([T], usecorrr=0, mode=int(d["mode"]), ang0=float(d["ang0"]),
                             hfang=float(d["hfang"]), step=float(d["step"]))[0]
    check(g, o, case)


def _golden_thumbs(case="thm_s0_denovo"):
    import alignment_projects_gb300 as aln
    d = load_golden("thm_scan")[case]
    return aln.thumbs_from_points(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"])), d


def test_call_ops_equal_search_modes(ctx):
    """CThmScan member functions through aln_thm_call_batch: DenovoBestAngle
    and UsePriorAngles from a fresh object give the search entry point's
    numbers exactly (the same engine), and a DenovoBestAngle result fed to
    PeakHunt keeps its record or improves it."""
    import alignment_projects_gb300 as aln
    T, d = _golden_thumbs()
    for op, mode, hf in ((aln.THMOP_DENOVO, aln.THM_DENOVO, 10.0),
                         (aln.THMOP_PRIOR, aln.THM_PRIOR, 1.0)):
        s = ctx.thm_search_batch([T], mode=mode, ang0=0.0, hfang=hf, step=0.5)[0]
        c = ctx.thm_call_batch([T], op, [0.0, hf, 0.5, 0.0])[0]
        for k in ("A", "X", "Y", "R", "err"):
            assert c[k] == s[k], (op, k, c, s)
        assert c["ret"] == (1.0 if s["err"] == 0 else 0.0)
    b = ctx.thm_call_batch([T], aln.THMOP_DENOVO, [0.0, 10.0, 0.5, 0.0])[0]
    h = ctx.thm_call_batch([T], aln.THMOP_PEAKHUNT, [0.0, 0.5 * 0.05 * 1.5, 0.0, 0.0],
                           best=[b])[0]
    assert h["R"] >= b["R"] and h["ret"] == h["R"]


def test_call_pretweaks_then_rfromangle(ctx, orc):
    """Pretweaks then RFromAngle (cross_thisblock's sequence) carries the
    pretweak transform from one call to the next, as the object does; the
    transform is a product of near-unity factors and the R it gives is at
    least the untweaked one."""
    import alignment_projects_gb300 as aln
    T, d = _golden_thumbs("thm_s2_denovo")
    ang = float(d["A"])
    r0 = ctx.thm_call_batch([T], aln.THMOP_RFROMANGLE, [ang, 0, 0, 0])[0]
    p = ctx.thm_call_batch([T], aln.THMOP_PRETWEAKS, [0.0, ang, 0, 0])[0]
    r1 = ctx.thm_call_batch([T], aln.THMOP_RFROMANGLE, [ang, 0, 0, 0], tptwk=[p["tptwk"]])[0]
    assert p["ret"] in (0.0, 1.0)
    tw = np.array(p["tptwk"])
    assert np.abs(tw - [1, 0, 0, 0, 1, 0]).max() < 0.2
    if p["ret"]:
        assert r1["R"] >= r0["R"] - 1e-9
    else:
        assert r1["R"] == r0["R"]


def test_disc_of_angle_callback(ctx):
    """newAngProc: a per-angle disc callback that returns the fixed disc gives
    the fixed-disc numbers; one that returns a disc around the answer gives
    the numbers of that fixed disc."""
    import alignment_projects_gb300 as aln
    T, d = _golden_thumbs()
    base = ctx.thm_call_batch([T], aln.THMOP_DENOVO, [0.0, 10.0, 0.5, 0.0])[0]
    cb = ctx.thm_call_batch([T], aln.THMOP_DENOVO, [0.0, 10.0, 0.5, 0.0],
                            disc_of_angle=lambda deg: (0, 0, -1, -1))[0]
    assert (cb["A"], cb["X"], cb["Y"], cb["R"]) == (base["A"], base["X"], base["Y"], base["R"])
    disc = (int(base["X"]), int(base["Y"]), 12, 12)
    fixed = ctx.thm_call_batch([T], aln.THMOP_DENOVO, [0.0, 10.0, 0.5, 0.0], disc=disc)[0]
    seen = []
    cb2 = ctx.thm_call_batch([T], aln.THMOP_DENOVO, [0.0, 10.0, 0.5, 0.0],
                             disc_of_angle=lambda deg: seen.append(deg) or disc)[0]
    assert (cb2["A"], cb2["X"], cb2["Y"], cb2["R"]) == (fixed["A"], fixed["X"], fixed["Y"],
                                                        fixed["R"])
    assert len(seen) == cb2["ncalls"]


def _points_raster(pa, va, w, h):
    """Raster-order point list (integer points, corner (0, 0)) -> image, mask."""
    img = np.zeros((h, w), np.float64)
    mask = np.zeros((h, w), np.uint8)
    x = pa[:, 0].astype(np.int64)
    y = pa[:, 1].astype(np.int64)
    img[y, x] = va
    mask[y, x] = 1
    return img, mask


def _check_decimated(g, xy, v):
    vals, pres, sd = g
    ys, xs = np.nonzero(pres)   # row-major: the reference's output order
    assert np.array_equal(np.stack([xs, ys], 1), xy.astype(np.int64))
    assert np.array_equal(vals[ys, xs], v)   # bit for bit


def test_decimate_golden(ctx):
    """MakeThumbs' DecimateVector + Normalize on the GPU against the
    reference's golden output (the same sums in the same order: bitwise)."""
    d = load_golden("decimate")["dec8"]
    w, h, lbin = int(d["w"]), int(d["h"]), int(d["lbin"])
    # the fixture's point list is in raster order
    order = np.lexsort((d["pa"][:, 0], d["pa"][:, 1]))
    assert np.array_equal(order, np.arange(len(order)))
    img, mask = _points_raster(d["pa"], d["va"], w, h)
    g = ctx.decimate([img], lbin, masks=[mask])[0]
    _check_decimated(g, d["xy"], d["v"])


@pytest.mark.parametrize("dt,lbin,masked", [(np.uint8, 8, False), (np.uint8, 8, True),
                                            (np.uint16, 4, True), (np.float32, 8, False),
                                            (np.float64, 5, True), (np.uint8, 16, False)])
def test_decimate_matches_oracle(ctx, orc, dt, lbin, masked):
    """Integer and float rasters, masks of any shape, ragged edge bins, and
    lbin 16 (a full bin's 256 points wrap the reference's uint8 counter to 0:
    the bin is dropped, as there)."""
    rng = np.random.default_rng(lbin * 10 + masked)
    h, w = 197, 261
    if dt in (np.uint8, np.uint16):
        img = rng.integers(0, 256 if dt == np.uint8 else 4096, (h, w)).astype(dt)
    else:
        img = rng.standard_normal((h, w)).astype(dt)
    mask = None
    if masked:
        yy, xx = np.mgrid[0:h, 0:w]
        mask = (((xx - 120) ** 2 + (yy - 90) ** 2) < 95 ** 2).astype(np.uint8)
    ys, xs = np.nonzero(mask if mask is not None else np.ones((h, w), np.uint8))
    pa = np.stack([xs, ys], 1).astype(np.float64)
    va = img[ys, xs].astype(np.float64)
    xy, v = orc.decimate_normalize(pa, va, w, h, lbin)
    g = ctx.decimate([img], lbin, masks=[mask])[0]
    _check_decimated(g, xy, v)
    # a batch of several images gives each its own numbers
    gb = ctx.decimate([img, img[:100, :150]], lbin, masks=None if mask is None
                      else [mask, mask[:100, :150]])
    assert np.array_equal(gb[0][0], g[0]) and np.array_equal(gb[0][1], g[1])
