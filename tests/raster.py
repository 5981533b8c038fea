"""Point cloud -> raster helpers for the GPU tests (the host-side conversion a
caller of the raster ABI performs; ImageFromValuesAndPoints semantics,
0_GEN/Geometry.cpp:661-685 and the bilinear splat of 0_GEN/Maths.h:236-276)."""
import math

import numpy as np


def bbox(pts):
    xs, ys = pts[:, 0], pts[:, 1]
    return (int(math.floor(xs.min())), int(math.ceil(xs.max())),
            int(math.floor(ys.min())), int(math.ceil(ys.max())))


def splat_raster(pts, vals):
    """Bilinear forward splat of (pts, vals) into the points' bounding box.
    Returns (raster float64 [h][w], (x0, y0))."""
    pts = np.asarray(pts, np.float64)
    vals = np.asarray(vals, np.float64)
    L, R, B, T = bbox(pts)
    w, h = R - L + 1, T - B + 1
    img = np.zeros((h, w), np.float64)
    x = pts[:, 0] - L
    y = pts[:, 1] - B
    ix = np.floor(x).astype(np.int64)
    iy = np.floor(y).astype(np.int64)
    a = x - ix
    b = y - iy
    for dx, dy, wgt in ((0, 0, (1 - a) * (1 - b)), (0, 1, (1 - a) * b),
                        (1, 0, a * (1 - b)), (1, 1, a * b)):
        xx, yy = ix + dx, iy + dy
        m = (xx >= 0) & (xx < w) & (yy >= 0) & (yy < h)
        np.add.at(img, (yy[m], xx[m]), wgt[m] * vals[m])
    return img, (L, B)
