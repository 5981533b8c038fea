"""Point clouds to rasters on the device (aln_points_image:
ImageFromValuesAndPoints + DistributePixel, 0_GEN/Geometry.cpp:661-685,
0_GEN/Maths.h:236-276), and the C++ drop-in's fractional point lists through
it."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    yield c
    c.close()


def _rotated_cloud(seed, n=60, deg=7.0):
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:n, 0:n].astype(np.float64)
    c, s = math.cos(math.radians(deg)), math.sin(math.radians(deg))
    x = c * xx - s * yy + 3.3
    y = s * xx + c * yy - 1.7
    return np.stack([x.ravel(), y.ravel()], 1), rng.normal(100.0, 20.0, n * n)


def test_fractional_cloud_matches_oracle(ctx, orc):
    xy, v = _rotated_cloud(1)
    xmin, ymin = int(math.floor(xy[:, 0].min())), int(math.floor(xy[:, 1].min()))
    w = int(math.ceil(xy[:, 0].max())) - xmin + 1
    h = int(math.ceil(xy[:, 1].max())) - ymin + 1
    g, im = ctx.points_image(xy, v, xmin, ymin, w, h)
    o = orc.image_from_points(xy, v, xmin, ymin, w, h)
    assert np.abs(g - o).max() <= 1e-9 * np.abs(o).max()
    assert (im.w, im.h, im.x0, im.y0, im.on_device) == (w, h, xmin, ymin, 1)
    # the same cloud in another order gives the same raster bit for bit
    perm = np.random.default_rng(2).permutation(len(v))
    g2, _ = ctx.points_image(xy[perm], v[perm], xmin, ymin, w, h, slot=1)
    assert np.array_equal(g, g2)


def test_integer_cloud_is_exact(ctx, orc):
    rng = np.random.default_rng(3)
    pts = rng.integers(0, 40, (500, 2)).astype(np.float64)   # duplicates add
    v = rng.integers(0, 256, 500).astype(np.float64)
    g, _ = ctx.points_image(pts, v, 0, 0, 40, 40)
    assert np.array_equal(g, orc.image_from_points(pts, v, 0, 0, 40, 40))


def test_corr_patches_on_device_rasters(ctx, orc):
    """A fractional cloud splatted on the device feeds CorrPatches directly:
    the oracle's numbers on its own raster."""
    import oracle
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    p = synth.plain_pair(21, n=96, margin=12)
    ys, xs = np.nonzero(np.ones_like(p.a))
    xy = np.stack([xs + 0.25, ys + 0.5], 1).astype(np.float64)
    va = p.a[ys, xs].astype(np.float64)
    _, ia = ctx.points_image(xy, va, 0, 0, 97, 97, slot=0)
    _, ib = ctx.points_image(np.stack([xs, ys], 1), p.b[ys, xs].astype(np.float64),
                             0, 0, 96, 96, slot=1)
    from alignment_projects_gb300.native import AlnResult
    import ctypes as C
    lg = aln.legal(aln.RGN_MIN, 16, 16, 0)
    r = AlnResult()
    assert aln.lib().aln_corr_patches(ctx.h, C.byref(ia), C.byref(ib), 0, 0, 4096, C.byref(lg),
                                      C.byref(r)) >= 0
    o = orc.corr_patches(xy, va, np.stack([xs, ys], 1), p.b[ys, xs], 0, 0, 4096,
                         oracle.legal(oracle.RGN_MIN, 16, 16, 0))
    assert abs(r.r - o["r"]) <= 1e-4
    if o["r"] - o["second"] > 1e-3:
        assert (r.peak_x, r.peak_y) == (o["bigx"], o["bigy"])
        assert abs(r.dx - o["dx"]) <= 0.01 and abs(r.dy - o["dy"]) <= 0.01
