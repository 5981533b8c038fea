"""GPU parity of CorrImagesF / R / S (0_GEN/Correlation.cpp:3066-3290)
against the oracle and the reference's golden outputs, through the C ABI.

Tolerances: the integer peak equals the oracle's wherever the oracle's
top-two margin exceeds 1e-3 (in the returned units: R, or the S score);
the returned value within 1e-4 (R) or 1e-4 relative (S score); sub-pixel
offsets within 0.01 px.
"""
import numpy as np
import pytest

from conftest import legal_from, load_golden
from raster import splat_raster

pytestmark = pytest.mark.gpu

PX_TOL = 0.01
MARGIN = 1e-3


@pytest.fixture(scope="module")
def ctx():
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    yield c
    c.close()


def aln_legal(o):
    import alignment_projects_gb300 as aln
    return aln.legal(o.rgn_kind, o.rgn_a, o.rgn_b, o.rgn_area, o.cnt_kind, o.cnt_n)


def check(g, o, kind, msg):
    import alignment_projects_gb300 as aln
    if o["status"] == 1:
        assert g["status"] == aln.ALN_NO_PEAK, (msg, g, o)
        return
    assert g["status"] == aln.ALN_OK, (msg, g)
    tol = 1e-4 if kind == 1 else 1e-4 * max(1.0, abs(o["r"]))
    assert abs(g["r"] - o["r"]) <= tol, (msg, g["r"], o["r"])
    if o["r"] - o["second"] > MARGIN:
        assert (g["peak_x"], g["peak_y"]) == (o["bigx"], o["bigy"]), (msg, g, o)
        assert abs(g["dx"] - o["dx"]) <= PX_TOL and abs(g["dy"] - o["dy"]) <= PX_TOL, (msg, g, o)


def run_case(ctx, orc, kind, pa, va, pb, vb, lg, mincor, disc):
    a, ao = splat_raster(pa, va)
    b, bo = splat_raster(pb, vb)
    g = ctx.corr_images(kind, a, b, aln_legal(lg), mincor, 0.75, *disc, a_origin=ao,
                        b_origin=bo)
    o = orc.corr_images(kind, pa, va, pb, vb, lg, mincor, 0.75, *disc)
    return g, o


@pytest.mark.parametrize("case", sorted(load_golden("corr_images")))
def test_corr_images_golden(ctx, orc, case):
    d = load_golden("corr_images")[case]
    kind = int(d["kind"])
    lg = legal_from(d["legal"])
    disc = [int(v) for v in d["disc"]]
    g, o = run_case(ctx, orc, kind, d["pa"], d["va"], d["pb"], d["vb"], lg,
                    float(d["mincor"]), disc)
    # the oracle reproduces the reference (tests/test_oracle_golden.py)
    assert abs(o["r"] - float(d["r"])) < 1e-12
    check(g, o, kind, case)


def _thumbs(seed, deg):
    import oracle
    from alignment_projects_gb300 import synth
    ta, tb, th, t = synth.thumb_pair(seed, tile=768, dec=8)
    A, VA = oracle.image_to_points(ta)
    B, VB = oracle.image_to_points(tb)
    VA = (VA - VA.mean()) / VA.std(ddof=1)
    VB = (VB - VB.mean()) / VB.std(ddof=1)
    ang = np.deg2rad(deg)
    R = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
    return A @ R.T, VA, B, VB, th


@pytest.mark.parametrize("seed,kind", [(s, k) for s in range(6) for k in (0, 1, 2)])
def test_rotated_thumbnails(ctx, orc, seed, kind):
    import oracle
    pa, va, pb, vb, th = _thumbs(seed, -1.0 + 0.37 * seed)
    lg = oracle.legal(oracle.RGN_MIN, 0, 0, 200, oracle.CNT_GT, 200)
    g, o = run_case(ctx, orc, kind, pa, va, pb, vb, lg, 0.0, (0, 0, -1, -1))
    check(g, o, kind, f"seed {seed}")


@pytest.mark.parametrize("kind,mincor,disc", [(2, 0.05, (0, 0, -1, -1)), (2, 0.0, (4, -3, 15, 9)),
                                              (1, 0.1, (-6, 2, 12, 20)), (2, 0.0, (0, 0, 0, 5)),
                                              (0, 0.0, (0, 0, -1, -1)), (0, 0.2, (3, 3, 20, 16))])
def test_mincor_and_oval(ctx, orc, kind, mincor, disc):
    import oracle
    pa, va, pb, vb, th = _thumbs(3, 0.5)
    lg = oracle.legal(oracle.RGN_MIN, 10, 10, 100, oracle.CNT_GT, 100)
    g, o = run_case(ctx, orc, kind, pa, va, pb, vb, lg, mincor, disc)
    check(g, o, kind, f"{kind} {mincor} {disc}")


def test_too_small_is_no_peak(ctx):
    import alignment_projects_gb300 as aln
    a = np.random.default_rng(0).standard_normal((6, 20))
    b = np.random.default_rng(1).standard_normal((20, 20))
    g = ctx.corr_images(aln.CORR_S, a, b)
    assert g["status"] == aln.ALN_NO_PEAK and g["r"] == 0.0


def test_images_batch_equals_single(ctx):
    import alignment_projects_gb300 as aln
    jobs = []
    for s in range(4):
        pa, va, pb, vb, th = _thumbs(10 + s, 0.3 * s)
        a, ao = splat_raster(pa, va)
        b, bo = splat_raster(pb, vb)
        jobs.append(dict(kind=aln.CORR_S if s % 2 == 0 else aln.CORR_R, a=a, b=b, a_origin=ao,
                         b_origin=bo, legal=aln.legal(aln.RGN_MIN, 0, 0, 150, aln.CNT_GT, 150)))
    batch = ctx.corr_images_batch(jobs)
    for j, r in zip(jobs, batch):
        single = ctx.corr_images(j["kind"], j["a"], j["b"], j["legal"], a_origin=j["a_origin"],
                                 b_origin=j["b_origin"])
        assert r == single


# ---------------------------------------------------------------- CorrPatchToImage

@pytest.mark.parametrize("case", ["p2i_f0", "p2i_f1"])
def test_patch_to_image_golden(ctx, orc, case):
    d = load_golden("patch_to_image")[case]
    bf = bool(int(d["bfilter"]))
    g = ctx.corr_patch_to_image(d["pa"], d["va"], d["img2"], 0, 0, 4096, bf)
    o = orc.corr_patch_to_image(d["pa"], d["va"], d["img2"], 0, 0, 4096, bf)
    assert abs(o["r"] - float(d["r"])) < 1e-12
    assert g["status"] == 0
    assert (g["peak_x"], g["peak_y"]) == (o["bigx"], o["bigy"])
    # raw (unnormalised) correlation in FP32: 1e-5 relative
    assert abs(g["r"] - float(d["r"])) <= 1e-5 * abs(float(d["r"]))
    assert abs(g["dx"] - float(d["dx"])) <= PX_TOL and abs(g["dy"] - float(d["dy"])) <= PX_TOL


def test_patch_to_image_disc_and_offsets(ctx, orc):
    from alignment_projects_gb300 import synth
    import oracle
    p = synth.plain_pair(12, n=90, margin=8)
    A, VA = oracle.image_to_points(p.a, 20, 30)
    VA = (VA - VA.mean()) / VA.std() / 30
    img2 = np.zeros((256, 256))
    img2[30:120, 20:110] = (p.b - p.b.mean()) / p.b.std() / 30
    for (ox, oy, rad) in [(0, 0, 4096), (3, -2, 10)]:
        g = ctx.corr_patch_to_image(A, VA, img2, ox, oy, rad)
        o = orc.corr_patch_to_image(A, VA, img2, ox, oy, rad)
        assert (g["peak_x"], g["peak_y"]) == (o["bigx"], o["bigy"]), (g, o)
        assert abs(g["r"] - o["r"]) <= 1e-5 * abs(o["r"])
        assert abs(g["dx"] - o["dx"]) <= PX_TOL and abs(g["dy"] - o["dy"]) <= PX_TOL
