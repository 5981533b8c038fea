"""GPU parity of the whole ApproximateMatch chain (1_DMesh/ApproximateMatch.cpp:
115-194: crop, MakeThumbs, sweep, PostTweaks, FinishAtFullRes, the change to
tile coordinates, the LIMXY test) through aln_approx_match_batch, against
the reference's own functions chained the same way (tests/golden/approx.npz,
made by refwrap's ref_approx_match).

The sweep inside is held to the sweep bar (oracle/sweep_bar.py): the oracle
runs the same search on the same thumbnails and bounds how far a tied
decision may move the angle; at the identical angle the full-resolution
offsets agree within 0.01 px and R within 1e-4.  The crop is integer
arithmetic and must be identical.
"""
import math

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

KEYS = ("xyconf", "olap1d", "olap2d", "thmdec", "mode_prior", "ang0", "hfangdn", "hfangpr",
        "rthresh", "nbmaxht", "pretweak", "tweaks", "limxy")


def _params(d):
    p = dict(zip(KEYS, (float(v) for v in d["params"])))
    for k in ("olap1d", "olap2d", "thmdec", "mode_prior", "pretweak", "tweaks", "limxy"):
        p[k] = int(p[k])
    return p


@pytest.fixture(scope="module")
def ctx():
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    yield c
    c.close()


def _oracle_sweep(orc, d, p):
    """The oracle's sweep (with its decision margins) on the thumbnails of
    the reference's crop."""
    import oracle
    x0, y0, bx0, by0, w, h = (int(v) for v in d["crop"])
    dec = p["thmdec"]
    thumbs = []
    for img, (ox, oy) in ((d["a"], (x0, y0)), (d["b"], (bx0, by0))):
        crop = np.asarray(img[oy:oy + h, ox:ox + w], np.float64)
        pts, vals = oracle.image_to_points(crop)
        thumbs += list(orc.decimate_normalize(pts, vals, w, h, dec))
    mode = 2 if p["mode_prior"] else 0
    return orc.thm_search(thumbs[0], thumbs[1], thumbs[2], thumbs[3],
                          p["olap2d"] // (dec * dec), p["olap1d"] // dec, p["rthresh"],
                          p["nbmaxht"], p["pretweak"], 1, 1, (0, 0, -1, -1), mode, p["ang0"],
                          p["hfangpr"] if p["mode_prior"] else p["hfangdn"], 0.5)


def test_approx_match_chain_golden(ctx, orc):
    cases = load_golden("approx")
    names = sorted(cases)
    # every case in one batch (each with its own settings would need one call
    # per setting: group by parameters)
    groups = {}
    for n in names:
        groups.setdefault(tuple(cases[n]["params"]), []).append(n)
    got = {}
    for key, ns in groups.items():
        p = _params(cases[ns[0]])
        res = ctx.approx_match_batch([(cases[n]["a"], cases[n]["b"], tuple(cases[n]["tab"]))
                                      for n in ns], **p)
        got.update(zip(ns, res))
    for n in names:
        d, g, p = cases[n], got[n], _params(cases[n])
        st = int(d["status"])
        if st == 1:   # crop too small: nothing else runs
            assert g["status"] == 1, (n, g)
            continue
        assert g["crop"] == [int(v) for v in d["crop"]], (n, g["crop"], d["crop"])
        o = _oracle_sweep(orc, d, p)
        assert o["A"] == float(d["sweep"][0]), (n, o["A"], d["sweep"])   # pinned oracle
        m = o["margins"]
        if not m["thr_tie"]:
            assert g["status"] == st and g["err"] == int(d["err"]), (n, g, st)
        dA = abs(g["A"] - float(d["A"]))
        assert dA <= m["tolA"] + 1e-9, (n, dA, m)
        if st not in (0, 4):
            continue
        # the final angle is the sweep's (PostTweaks and FinishAtFullRes keep it)
        assert g["A"] == g["sweep"][0], (n, g)
        if dA <= 1e-9:
            tol_xy = 0.01
            assert abs(g["R"] - float(d["R"])) <= 1e-4 * max(1.0, abs(float(d["R"]))), (n, g)
            assert np.abs(np.array(g["T"])[[0, 1, 3, 4]] - d["T"][[0, 1, 3, 4]]).max() <= 1e-6
        else:   # a tied bracket test: the same peak seen a whisker of angle apart
            r = math.hypot(*d["a"].shape)
            tol_xy = 0.01 + r * math.radians(dA)
        assert abs(g["X"] - float(d["X"])) <= tol_xy and abs(g["Y"] - float(d["Y"])) <= tol_xy, \
            (n, g, float(d["X"]), float(d["Y"]))
        assert abs(g["T"][2] - g["X"]) == 0.0 and abs(g["T"][5] - g["Y"]) == 0.0


def test_approx_match_finds_the_synthetic_transform(ctx):
    """On the golden tiles the guess lands near the transform that made them:
    angle within 0.5 deg, translation within 3 px."""
    cases = load_golden("approx")
    d = cases["approx_denovo"]
    g = ctx.approx_match_batch([(d["a"], d["b"], tuple(d["tab"]))], **_params(d))[0]
    t = d["truth"]
    assert g["status"] == 0
    assert abs(math.degrees(math.atan2(g["T"][3], g["T"][0]))
               - math.degrees(math.atan2(t[3], t[0]))) < 0.5
    assert abs(g["T"][2] - t[2]) < 3 and abs(g["T"][5] - t[5]) < 3


def test_approx_match_device_tiles_equal_host_tiles(ctx):
    """Tiles already in device memory give the host tiles' numbers bit for bit."""
    import torch
    cases = load_golden("approx")
    d = cases["approx_tweaks"]
    p = _params(d)
    h = ctx.approx_match_batch([(d["a"], d["b"], tuple(d["tab"]))], **p)[0]
    ta, tb = torch.from_numpy(d["a"]).cuda(), torch.from_numpy(d["b"]).cuda()
    g = ctx.approx_match_batch([(ta, tb, tuple(d["tab"]))], **p)[0]
    for k in ("status", "err", "A", "X", "Y", "R", "T", "sweep", "crop"):
        assert g[k] == h[k], (k, g[k], h[k])
