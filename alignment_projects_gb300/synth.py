"""Seeded synthetic EM-like tiles standing in for the Janelia data.

Field G(seed, H, W): Gaussian white noise shaped to a 1/f^1.5 power spectrum
(amplitude x f^-0.75, DC removed), rescaled to mean 128 / std 30, with dark
membrane ellipses (value 40, semi-axes U[4, 20] px, random orientation,
200 per 2048^2 px of area) painted over it.  Values stay FP64 until the final
quantisation.  Two implementations share the algorithm: numpy (small cases,
CPU tests) and torch (large batches generated on the device); they draw from
different random streams.

Pair builders follow the workloads the matcher is measured on:
  plain_pair       one 512^2 uint8 pair with an integer offset in [-64, 64]^2
  montage_pairs    W x 2048 (or 2048 x W) uint8 overlap strips, W in [164, 307],
                   +-40 px jitter, 2 % decoy pairs built from unrelated content
  uneven_pairs     uint16 patches, side log-uniform in [64, 1024], aspect 1-4
  thumb_pair       256^2 float thumbnails (8x box average of 2048^2 tiles),
                   B rotated by an angle in [-10, 10] deg and shifted
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


# ----------------------------------------------------------------------------
# numpy field
# ----------------------------------------------------------------------------

def _ellipse_params(rng, h, w, n):
    cy = rng.uniform(0, h, n)
    cx = rng.uniform(0, w, n)
    a = rng.uniform(4, 20, n)
    b = rng.uniform(4, 20, n)
    th = rng.uniform(0, math.pi, n)
    return cx, cy, a, b, th


def field_np(seed: int, h: int, w: int, mean=128.0, std=30.0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal((h, w))
    F = np.fft.rfft2(noise)
    fy = np.fft.fftfreq(h)[:, None]
    fx = np.fft.rfftfreq(w)[None, :]
    f = np.sqrt(fx * fx + fy * fy)
    with np.errstate(divide="ignore"):
        amp = np.where(f > 0, f ** -0.75, 0.0)
    img = np.fft.irfft2(F * amp, s=(h, w))
    img = (img - img.mean()) / img.std() * std + mean
    n = int(round(200.0 * h * w / (2048.0 * 2048.0)))
    cx, cy, a, b, th = _ellipse_params(rng, h, w, n)
    for i in range(n):
        r = int(math.ceil(max(a[i], b[i]))) + 1
        x0, x1 = max(0, int(cx[i]) - r), min(w, int(cx[i]) + r + 1)
        y0, y1 = max(0, int(cy[i]) - r), min(h, int(cy[i]) + r + 1)
        if x0 >= x1 or y0 >= y1:
            continue
        yy, xx = np.mgrid[y0:y1, x0:x1]
        dx, dy = xx - cx[i], yy - cy[i]
        c, s = math.cos(th[i]), math.sin(th[i])
        u = (c * dx + s * dy) / a[i]
        v = (-s * dx + c * dy) / b[i]
        m = u * u + v * v <= 1.0
        img[y0:y1, x0:x1][m] = 40.0
    return img


def to_u8(x: np.ndarray) -> np.ndarray:
    return np.clip(np.rint(x), 0, 255).astype(np.uint8)


def to_u16(x: np.ndarray, top=4095) -> np.ndarray:
    return np.clip(np.rint(x), 0, top).astype(np.uint16)


# ----------------------------------------------------------------------------
# pair builders (numpy)
# ----------------------------------------------------------------------------

@dataclass
class Pair:
    a: np.ndarray            # tile / strip 1 (row-major [h][w])
    b: np.ndarray            # tile / strip 2
    truth: tuple             # expected (dx, dy) placing a into b's frame
    ox: int = 0
    oy: int = 0
    radius: int = 4096
    decoy: bool = False


def plain_pair(seed: int = 1, n: int = 512, margin: int = 64, noise=8.0) -> Pair:
    """One n x n uint8 pair: A = field[m:m+n]^2, B = A's window shifted by t
    (t uniform in [-margin, margin]^2) plus N(0, noise^2).  Expected lag -t."""
    size = n + 2 * margin
    f = field_np(seed, size, size)
    rng = np.random.default_rng(seed + 1000003)
    tx, ty = (int(v) for v in rng.integers(-margin, margin + 1, 2))
    a = to_u8(f[margin:margin + n, margin:margin + n])
    bf = f[margin + ty:margin + ty + n, margin + tx:margin + tx + n]
    b = to_u8(bf + rng.normal(0.0, noise, bf.shape))
    return Pair(a, b, (-tx, -ty))


def montage_pair(seed: int, long_side: int = 2048, wmin: int = 164, wmax: int = 307,
                 jitter: int = 40, decoy_frac: float = 0.02, noise=8.0) -> Pair:
    """One same-layer montage overlap: strips of W x long_side (left-right) or
    long_side x W (top-bottom), B displaced by a jitter in [-40, 40]^2 from the
    nominal layout; a decoy pair takes B from an unrelated field."""
    rng = np.random.default_rng(seed)
    W = int(rng.integers(wmin, wmax + 1))
    lr = bool(rng.integers(0, 2))
    tx, ty = (int(v) for v in rng.integers(-jitter, jitter + 1, 2))
    decoy = bool(rng.random() < decoy_frac)
    m = 2 * jitter
    sw, sh = (W, long_side) if lr else (long_side, W)
    f = field_np(seed * 7 + 1, sh + 2 * m, sw + 2 * m)
    a = to_u8(f[m:m + sh, m:m + sw] + rng.normal(0.0, noise, (sh, sw)))
    if decoy:
        g = field_np(seed * 7 + 2, sh + 2 * m, sw + 2 * m)
        bf = g[m:m + sh, m:m + sw]
    else:
        bf = f[m + ty:m + ty + sh, m + tx:m + tx + sw]
    b = to_u8(bf + rng.normal(0.0, noise, (sh, sw)))
    return Pair(a, b, (-tx, -ty), 0, 0, 64, decoy)


def uneven_pair(seed: int, smin=64, smax=1024) -> Pair:
    """uint16 patches (values 0-4095, mean 2048 / std 480), long side
    log-uniform in [64, 1024], aspect 1-4, offset within a quarter of the
    short side; disc radius = short/2."""
    rng = np.random.default_rng(seed)
    s = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
    short = max(8, int(round(s / rng.uniform(1.0, 4.0))))
    wide = bool(rng.integers(0, 2))
    w, h = (s, short) if wide else (short, s)
    q = max(1, short // 4)
    tx, ty = (int(v) for v in rng.integers(-q, q + 1, 2))
    f = field_np(seed * 7 + 3, h + 2 * q, w + 2 * q, mean=2048.0, std=480.0)
    a = to_u16(f[q:q + h, q:q + w])
    bf = f[q + ty:q + ty + h, q + tx:q + tx + w]
    b = to_u16(bf + rng.normal(0.0, 30.0, bf.shape))
    return Pair(a, b, (-tx, -ty), 0, 0, max(1, short // 2))


def _bilinear(img: np.ndarray, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    h, w = img.shape
    x0 = np.clip(np.floor(x).astype(np.int64), 0, w - 2)
    y0 = np.clip(np.floor(y).astype(np.int64), 0, h - 2)
    ax = np.clip(x - x0, 0.0, 1.0)
    ay = np.clip(y - y0, 0.0, 1.0)
    return ((1 - ax) * (1 - ay) * img[y0, x0] + ax * (1 - ay) * img[y0, x0 + 1]
            + (1 - ax) * ay * img[y0 + 1, x0] + ax * ay * img[y0 + 1, x0 + 1])


def thumb_pair(seed: int, tile: int = 2048, dec: int = 8, max_deg=10.0, max_t=30.0,
               noise=5.0):
    """Cross-layer thumbnails: two tile x tile tiles of one field, B resampled
    at R(theta) p + t (bilinear), gain in [0.9, 1.1], N(0, noise^2); both
    box-averaged by `dec` into float thumbnails.  Returns (thumbA, thumbB,
    theta_deg, t) -- normalisation is left to the caller (MakeThumbs does it)."""
    rng = np.random.default_rng(seed)
    theta = float(rng.uniform(-max_deg, max_deg))
    t = rng.uniform(-max_t, max_t, 2)
    gain = float(rng.uniform(0.9, 1.1))
    pad = int(tile * 0.25) + int(max_t) + 4
    size = tile + 2 * pad
    f = field_np(seed * 7 + 5, size, size)
    a = f[pad:pad + tile, pad:pad + tile]
    yy, xx = np.mgrid[0:tile, 0:tile].astype(np.float64)
    c, s = math.cos(math.radians(theta)), math.sin(math.radians(theta))
    cx = cy = tile / 2.0
    X = c * (xx - cx) - s * (yy - cy) + cx + t[0] + pad
    Y = s * (xx - cx) + c * (yy - cy) + cy + t[1] + pad
    b = gain * _bilinear(f, X, Y) + rng.normal(0.0, noise, (tile, tile))
    ta = a.reshape(tile // dec, dec, tile // dec, dec).mean(axis=(1, 3))
    tb = b.reshape(tile // dec, dec, tile // dec, dec).mean(axis=(1, 3))
    return ta.astype(np.float32), tb.astype(np.float32), theta, (float(t[0]), float(t[1]))


# ----------------------------------------------------------------------------
# torch field (large batches on the device)
# ----------------------------------------------------------------------------

def field_torch(gen, h: int, w: int, device, mean=128.0, std=30.0, ellipses=True):
    """Same algorithm as field_np, drawing from torch generator `gen`."""
    import torch

    noise = torch.randn((h, w), generator=gen, device=device, dtype=torch.float64)
    F = torch.fft.rfft2(noise)
    fy = torch.fft.fftfreq(h, device=device, dtype=torch.float64)[:, None]
    fx = torch.fft.rfftfreq(w, device=device, dtype=torch.float64)[None, :]
    f = torch.sqrt(fx * fx + fy * fy)
    amp = torch.where(f > 0, f.clamp_min(1e-30) ** -0.75, torch.zeros_like(f))
    img = torch.fft.irfft2(F * amp, s=(h, w))
    img = (img - img.mean()) / img.std() * std + mean
    if ellipses:
        n = int(round(200.0 * h * w / (2048.0 * 2048.0)))
        if n > 0:
            u = torch.rand((n, 5), generator=gen, device=device, dtype=torch.float64)
            cx, cy = u[:, 0] * w, u[:, 1] * h
            a, b = 4 + 16 * u[:, 2], 4 + 16 * u[:, 3]
            th = u[:, 4] * math.pi
            # paint in tiles of 64 ellipses, each over its 41 x 41 window
            r = 21
            oy, ox = torch.meshgrid(torch.arange(-r, r + 1, device=device),
                                    torch.arange(-r, r + 1, device=device),
                                    indexing="ij")
            for s0 in range(0, n, 64):
                sl = slice(s0, min(n, s0 + 64))
                X = cx[sl].floor()[:, None, None] + ox
                Y = cy[sl].floor()[:, None, None] + oy
                dx = X - cx[sl][:, None, None]
                dy = Y - cy[sl][:, None, None]
                c = torch.cos(th[sl])[:, None, None]
                s = torch.sin(th[sl])[:, None, None]
                uu = (c * dx + s * dy) / a[sl][:, None, None]
                vv = (-s * dx + c * dy) / b[sl][:, None, None]
                m = (uu * uu + vv * vv <= 1.0) & (X >= 0) & (X < w) & (Y >= 0) & (Y < h)
                img[Y[m].long(), X[m].long()] = 40.0
    return img


def montage_batch_torch(seed: int, n: int, device, long_side: int = 2048, wmin: int = 164,
                        wmax: int = 307, jitter: int = 40, decoy_frac: float = 0.02,
                        noise: float = 8.0):
    """n montage overlap pairs (as montage_pair) generated with torch on
    `device`.  Pair i depends only on (seed, i).  Returns a list of dicts with
    uint8 tensors a, b, the expected lag `truth`, `decoy`, disc (0, 0, 64)."""
    import torch

    out = []
    m = 2 * jitter
    for i in range(n):
        s = seed * 1000003 + i
        rng = np.random.default_rng(s)
        W = int(rng.integers(wmin, wmax + 1))
        lr = bool(rng.integers(0, 2))
        tx, ty = (int(v) for v in rng.integers(-jitter, jitter + 1, 2))
        decoy = bool(rng.random() < decoy_frac)
        sw, sh = (W, long_side) if lr else (long_side, W)
        gen = torch.Generator(device=device)
        gen.manual_seed(s)
        f = field_torch(gen, sh + 2 * m, sw + 2 * m, device)
        na = torch.randn((sh, sw), generator=gen, device=device, dtype=torch.float64)
        nb = torch.randn((sh, sw), generator=gen, device=device, dtype=torch.float64)
        a = f[m:m + sh, m:m + sw] + noise * na
        if decoy:
            g = field_torch(gen, sh + 2 * m, sw + 2 * m, device)
            bf = g[m:m + sh, m:m + sw]
        else:
            bf = f[m + ty:m + ty + sh, m + tx:m + tx + sw]
        b = bf + noise * nb
        a8 = torch.clamp(torch.round(a), 0, 255).to(torch.uint8).contiguous()
        b8 = torch.clamp(torch.round(b), 0, 255).to(torch.uint8).contiguous()
        out.append(dict(a=a8, b=b8, truth=(-tx, -ty), decoy=decoy, ox=0, oy=0, radius=64,
                        lr=lr, W=W))
    return out


def thumb_batch_torch(seed: int, n: int, device, tile: int = 2048, dec: int = 8,
                      max_deg=10.0, max_t=30.0, noise=5.0):
    """n cross-layer thumbnail pairs (as thumb_pair) generated with torch on
    `device`: tile x tile tiles, B resampled at R(theta) p + t (bilinear),
    gain U[0.9, 1.1], N(0, noise^2), both box-averaged by `dec`, then each
    thumbnail normalised to mean 0, sample std 1 (MakeThumbs).  Pair i depends
    only on (seed, i).  Returns dicts with FP64 tensors ta, tb (on `device`),
    theta (deg) and t (full-resolution px)."""
    import torch

    out = []
    pad = int(tile * 0.25) + int(max_t) + 4
    size = tile + 2 * pad
    k = torch.arange(tile, device=device, dtype=torch.float64)
    yy, xx = torch.meshgrid(k, k, indexing="ij")
    cx = cy = tile / 2.0
    for i in range(n):
        s = seed * 1000003 + i
        rng = np.random.default_rng(s)
        theta = float(rng.uniform(-max_deg, max_deg))
        t = rng.uniform(-max_t, max_t, 2)
        gain = float(rng.uniform(0.9, 1.1))
        gen = torch.Generator(device=device)
        gen.manual_seed(s)
        f = field_torch(gen, size, size, device)
        a = f[pad:pad + tile, pad:pad + tile]
        c, sn = math.cos(math.radians(theta)), math.sin(math.radians(theta))
        X = c * (xx - cx) - sn * (yy - cy) + cx + float(t[0]) + pad
        Y = sn * (xx - cx) + c * (yy - cy) + cy + float(t[1]) + pad
        x0 = X.floor().long().clamp(0, size - 2)
        y0 = Y.floor().long().clamp(0, size - 2)
        ax = (X - x0).clamp(0.0, 1.0)
        ay = (Y - y0).clamp(0.0, 1.0)
        b = ((1 - ax) * (1 - ay) * f[y0, x0] + ax * (1 - ay) * f[y0, x0 + 1]
             + (1 - ax) * ay * f[y0 + 1, x0] + ax * ay * f[y0 + 1, x0 + 1])
        b = gain * b + noise * torch.randn((tile, tile), generator=gen, device=device,
                                           dtype=torch.float64)
        m = tile // dec
        ta = a.reshape(m, dec, m, dec).mean(dim=(1, 3)).float().double()
        tb = b.reshape(m, dec, m, dec).mean(dim=(1, 3)).float().double()
        ta = (ta - ta.mean()) / ta.std()
        tb = (tb - tb.mean()) / tb.std()
        out.append(dict(ta=ta.contiguous(), tb=tb.contiguous(), theta=theta,
                        t=(float(t[0]), float(t[1]))))
    return out


def neighbour_group_torch(seed: int, k: int, device, tile: int = 2048, dec: int = 8,
                          max_deg=10.0, max_t=30.0, noise=5.0):
    """One tile B and k neighbours A_1..A_k of it (different offsets of one
    field), as 256^2-class thumbnails: B is the field resampled at
    R(theta) p + t_B (bilinear, gain, noise), each A_i the field shifted by
    its own u_i in [-max_t, max_t]^2.  All box-averaged by `dec` and
    normalised (MakeThumbs).  Returns (tb, [ta_1..ta_k], theta) as FP64
    numpy arrays on the host."""
    import torch

    rng = np.random.default_rng(seed)
    theta = float(rng.uniform(-max_deg, max_deg))
    t = rng.uniform(-max_t, max_t, 2)
    u = rng.uniform(-max_t, max_t, (k, 2))
    gain = float(rng.uniform(0.9, 1.1))
    pad = int(tile * 0.25) + 2 * int(max_t) + 4
    size = tile + 2 * pad
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    f = field_torch(gen, size, size, device)
    kk = torch.arange(tile, device=device, dtype=torch.float64)
    yy, xx = torch.meshgrid(kk, kk, indexing="ij")
    c, sn = math.cos(math.radians(theta)), math.sin(math.radians(theta))
    cx = cy = tile / 2.0
    X = c * (xx - cx) - sn * (yy - cy) + cx + float(t[0]) + pad
    Y = sn * (xx - cx) + c * (yy - cy) + cy + float(t[1]) + pad
    x0 = X.floor().long().clamp(0, size - 2)
    y0 = Y.floor().long().clamp(0, size - 2)
    ax = (X - x0).clamp(0.0, 1.0)
    ay = (Y - y0).clamp(0.0, 1.0)
    b = ((1 - ax) * (1 - ay) * f[y0, x0] + ax * (1 - ay) * f[y0, x0 + 1]
         + (1 - ax) * ay * f[y0 + 1, x0] + ax * ay * f[y0 + 1, x0 + 1])
    b = gain * b + noise * torch.randn((tile, tile), generator=gen, device=device,
                                       dtype=torch.float64)
    m = tile // dec

    def thumb(img):
        th = img.reshape(m, dec, m, dec).mean(dim=(1, 3)).float().double()
        return ((th - th.mean()) / th.std()).cpu().numpy()

    tas = []
    for i in range(k):
        ox, oy = pad + int(round(u[i, 0])), pad + int(round(u[i, 1]))
        tas.append(thumb(f[oy:oy + tile, ox:ox + tile]))
    return thumb(b), tas, theta


def patch_group(seed: int, k: int, n: int = 512, margin: int = 64, noise=8.0):
    """One n x n uint8 tile B and k neighbours A_i (the field at offsets
    t_i in [-margin, margin]^2, plus noise).  Returns (b, [a_i], [truth_i])."""
    size = n + 2 * margin
    f = field_np(seed, size, size)
    rng = np.random.default_rng(seed + 1000003)
    b = to_u8(f[margin:margin + n, margin:margin + n] + rng.normal(0.0, noise, (n, n)))
    a_s, truths = [], []
    for _ in range(k):
        tx, ty = (int(v) for v in rng.integers(-margin, margin + 1, 2))
        af = f[margin + ty:margin + ty + n, margin + tx:margin + tx + n]
        a_s.append(to_u8(af + rng.normal(0.0, noise, af.shape)))
        truths.append((tx, ty))
    return b, a_s, truths


def uneven_batch_torch(seed: int, n: int, device, smin=64, smax=1024):
    """n uneven uint16 pairs (as uneven_pair: long side log-uniform in
    [smin, smax], aspect 1-4, orientation random, values 0-4095 with mean
    2048 / std 480, offset within a quarter of the short side, disc radius
    short/2), generated with torch on `device`.  Pair i depends only on
    (seed, i).  Returns dicts with tensors a, b stored as int16 (values
    0-4095: the same bits as uint16), the expected lag `truth` and the disc."""
    import torch

    out = []
    for i in range(n):
        s_ = seed * 1000003 + i
        rng = np.random.default_rng(s_)
        s = int(round(math.exp(rng.uniform(math.log(smin), math.log(smax)))))
        short = max(8, int(round(s / rng.uniform(1.0, 4.0))))
        wide = bool(rng.integers(0, 2))
        w, h = (s, short) if wide else (short, s)
        q = max(1, short // 4)
        tx, ty = (int(v) for v in rng.integers(-q, q + 1, 2))
        gen = torch.Generator(device=device)
        gen.manual_seed(s_)
        f = field_torch(gen, h + 2 * q, w + 2 * q, device, mean=2048.0, std=480.0)
        a = f[q:q + h, q:q + w]
        bf = f[q + ty:q + ty + h, q + tx:q + tx + w]
        b = bf + 30.0 * torch.randn(bf.shape, generator=gen, device=device, dtype=torch.float64)
        a16 = torch.clamp(torch.round(a), 0, 4095).to(torch.int32)
        b16 = torch.clamp(torch.round(b), 0, 4095).to(torch.int32)
        out.append(dict(a=a16.to(torch.int16).contiguous(), b=b16.to(torch.int16).contiguous(),
                        truth=(-tx, -ty), ox=0, oy=0, radius=max(1, short // 2)))
    return out


# ----------------------------------------------------------------------------
# mesh-optimizer cases (GradDescStep / ImproveControlPts)
# ----------------------------------------------------------------------------

def mesh_case(seed: int, box=(96, 80), cells=(2, 2), kind: str = "tri", field=200,
              warp=1.5, offset=(3.0, -2.0), noise=0.05):
    """A region-to-region mesh problem.  Region A is the integer points of a
    box; control points sit on a (cx+1) x (cy+1) lattice over the box, and
    each point's multipliers are the barycentric weights of its lattice
    triangle ("tri": 3 per point, cells split along the rising diagonal) or
    the bilinear weights of its cell ("quad": 4 per point).  B is a smooth
    synthetic field; A's values are B sampled at the point moved by a smooth
    warp (an offset plus up to `warp` px of bilinear deformation) with noise,
    then normalised to mean 0 / sd 1.  The control points start at the
    lattice moved by the offset alone (the optimiser has the warp to find).

    Returns dict(ac, am_idx, am_w, av, bimg, truth) -- am in compressed rows
    (indices ascending, -1 unused), ac / truth nc x 2 in B's frame."""
    rng = np.random.default_rng(seed)
    f = field_np(seed * 13 + 1, field, field)
    f = (f - f.mean()) / f.std()
    bw, bh = box
    x0 = (field - bw) // 2
    y0 = (field - bh) // 2
    gx, gy = cells
    lx = np.linspace(x0, x0 + bw - 1, gx + 1)
    ly = np.linspace(y0, y0 + bh - 1, gy + 1)
    cx, cy = np.meshgrid(lx, ly)
    ctl = np.stack([cx.ravel(), cy.ravel()], 1)            # j = iy * (gx + 1) + ix
    dwarp = rng.uniform(-warp, warp, (len(ctl), 2))
    truth = ctl + np.asarray(offset) + dwarp
    ys, xs = np.mgrid[y0:y0 + bh, x0:x0 + bw]
    px, py = xs.ravel().astype(np.float64), ys.ravel().astype(np.float64)
    ix = np.minimum(((px - x0) / (bw - 1) * gx).astype(int), gx - 1)
    iy = np.minimum(((py - y0) / (bh - 1) * gy).astype(int), gy - 1)
    u = (px - lx[ix]) / (lx[ix + 1] - lx[ix])
    v = (py - ly[iy]) / (ly[iy + 1] - ly[iy])
    j00 = iy * (gx + 1) + ix
    j10, j01, j11 = j00 + 1, j00 + gx + 1, j00 + gx + 2
    if kind == "quad":
        idx = np.stack([j00, j10, j01, j11], 1)
        wts = np.stack([(1 - u) * (1 - v), u * (1 - v), (1 - u) * v, u * v], 1)
    else:
        lower = u + v <= 1.0
        # lower triangle (00, 10, 01), upper (10, 01, 11): ascending indices
        idx = np.where(lower[:, None], np.stack([j00, j10, j01], 1),
                       np.stack([j10, j01, j11], 1))
        wts = np.where(lower[:, None], np.stack([1 - u - v, u, v], 1),
                       np.stack([1 - v, 1 - u, u + v - 1], 1))
    # true position of each point in B
    tx = (wts * truth[idx, 0]).sum(1)
    ty = (wts * truth[idx, 1]).sum(1)
    av = _bilinear(f, tx, ty) + rng.normal(0.0, noise, len(tx))
    av = (av - av.mean()) / av.std(ddof=1)
    ac = ctl + np.asarray(offset)
    return dict(ac=ac, am_idx=idx.astype(np.int32), am_w=wts, av=av, bimg=f, truth=truth)


# ----------------------------------------------------------------------------
# ApproximateMatch tile pairs
# ----------------------------------------------------------------------------

def approx_tile_pair(seed: int, tile: int = 512, max_deg=4.0, shift=(90.0, 30.0), jitter=6.0,
                     noise=6.0):
    """Two tile x tile uint8 tiles of one synthetic field, overlapping by most
    of their area: pixel p of A shows field point p + pad; pixel x of B
    shows field point R(theta)(x - c) + c + s + pad (c the tile centre, s the
    shift), with gain in [0.9, 1.1] and noise.  So A's pixel p sits in B at
    R(-theta)(p - c - s) + c: the true a -> b transform.  Tab (what the
    pipeline predicts) is its translation at the tile centre, -s, off by up
    to `jitter` px per axis.  Returns dict(a, b, tab, theta, truth T[6])."""
    rng = np.random.default_rng(seed)
    theta = float(rng.uniform(-max_deg, max_deg))
    s = np.asarray(shift, np.float64) * rng.choice([-1.0, 1.0], 2)
    gain = float(rng.uniform(0.9, 1.1))
    pad = int(tile * 0.3) + int(abs(s).max()) + 8
    size = tile + 2 * pad
    f = field_np(seed * 11 + 7, size, size)
    a = f[pad:pad + tile, pad:pad + tile]
    yy, xx = np.mgrid[0:tile, 0:tile].astype(np.float64)
    c_, s_ = math.cos(math.radians(theta)), math.sin(math.radians(theta))
    cx = cy = tile / 2.0
    X = c_ * (xx - cx) - s_ * (yy - cy) + cx + s[0] + pad
    Y = s_ * (xx - cx) + c_ * (yy - cy) + cy + s[1] + pad
    b = gain * _bilinear(f, X, Y) + rng.normal(0.0, noise, (tile, tile))
    # a -> b: x = R(-theta)(p - c - s) + c
    ci, si = c_, -s_
    t0 = -(ci * (cx + s[0]) - si * (cy + s[1])) + cx
    t1 = -(si * (cx + s[0]) + ci * (cy + s[1])) + cy
    truth = [ci, -si, t0, si, ci, t1]
    tab = (float(-s[0] + rng.uniform(-jitter, jitter)), float(-s[1] + rng.uniform(-jitter, jitter)))
    return dict(a=to_u8(a), b=to_u8(b), tab=tab, theta=theta, truth=truth)
