"""The transform plans CorrPatches uses, checked on the host in FP64 numpy
(no GPU): for the grid and column segments `aln_corr_patches_grid` reports,
the circular correlation the kernels compute -- row spectra, per column the
segments' spectral products summed and inverted (or one column transform),
the inverse row transform -- equals the direct linear correlation
sum_y,x a[y, x] b[y + dy, x + dx] at every lag of the disc window.  This is
the arithmetic of k2_rowfft / k2_corrseg / k2_corrcol / k2_lagrow restated
in numpy, so a planning rule that let wrap-around into the window would
fail here."""
import numpy as np
import pytest


def _pair(w0, h0, w1, h1, ox, oy, radius, keep):
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnPair
    a = np.zeros((h0, w0), np.uint8)
    b = np.zeros((h1, w1), np.uint8)
    keep += [a, b]
    P = AlnPair()
    P.a, P.b = aln.image(a), aln.image(b)
    P.ox, P.oy, P.radius = ox, oy, radius
    return P


def _window(w0, h0, w1, h1, ox, oy, rad):
    return (max(-(w0 - 1), ox - rad), min(w1 - 1, ox + rad),
            max(-(h0 - 1), oy - rad), min(h1 - 1, oy + rad))


def _plan_corr(a, b, nx, ny, nseg, ylo, yhi):
    """Correlation at lag rows ylo..yhi (all lag columns mod nx) the way the
    kernels form it: out[j, xs] for y = ylo + j."""
    h0, h1 = a.shape[0], b.shape[0]
    wy = yhi - ylo + 1
    A = np.fft.fft(a, n=nx, axis=1)   # row spectra T[y][kx] (complex form)
    B = np.fft.fft(b, n=nx, axis=1)
    Q = np.zeros((wy, nx), complex)
    if nseg:
        seg = -(-h0 // nseg)
        acc = np.zeros((ny, nx), complex)
        for s in range(nseg):
            y0 = s * seg
            asg = np.zeros((ny, nx), complex)
            n_a = max(0, min(seg, h0 - y0))
            asg[:n_a] = A[y0:y0 + n_a]
            bsg = np.zeros((ny, nx), complex)
            for j in range(seg + wy - 1):
                y = y0 + ylo + j
                if 0 <= y < h1:
                    bsg[j] = B[y]
            acc += np.fft.fft(bsg, axis=0) * np.conj(np.fft.fft(asg, axis=0))
        col = np.fft.ifft(acc, axis=0)
        Q[:] = col[:wy]
    else:
        Ac = np.fft.fft(A, n=ny, axis=0)
        Bc = np.fft.fft(B, n=ny, axis=0)
        col = np.fft.ifft(Bc * np.conj(Ac), axis=0)
        for j in range(wy):
            Q[j] = col[(ylo + j) % ny]
    return np.fft.ifft(Q, axis=1).real * 1.0   # the inverse row transform


def _direct(a, b, dx, dy):
    h0, w0 = a.shape
    h1, w1 = b.shape
    y0, y1 = max(0, -dy), min(h0, h1 - dy)
    x0, x1 = max(0, -dx), min(w0, w1 - dx)
    if y0 >= y1 or x0 >= x1:
        return 0.0
    return float((a[y0:y1, x0:x1] * b[y0 + dy:y1 + dy, x0 + dx:x1 + dx]).sum())


@pytest.mark.parametrize("seed", range(12))
def test_plan_equals_linear_correlation(seed):
    import alignment_projects_gb300 as aln
    rng = np.random.default_rng(seed)
    w0, w1 = (int(v) for v in rng.integers(20, 90, 2))
    h0, h1 = (int(v) for v in rng.integers(60, 400, 2))
    if seed % 3 == 0:   # montage-like: tall strips, a small disc
        w0 = w1 = int(rng.integers(20, 60))
        h0 = h1 = int(rng.integers(300, 600))
    ox, oy = (int(v) for v in rng.integers(-15, 16, 2))
    rad = int(rng.integers(4, 30))
    keep = []
    nx, ny, nseg, tr = aln.corr_patches_grid(_pair(w0, h0, w1, h1, ox, oy, rad, keep))
    if tr:   # solved transposed: exchange the axes here too
        w0, h0, w1, h1, ox, oy = h0, w0, h1, w1, oy, ox
    a = rng.standard_normal((h0, w0))
    b = rng.standard_normal((h1, w1))
    xlo, xhi, ylo, yhi = _window(w0, h0, w1, h1, ox, oy, rad)
    got = _plan_corr(a, b, nx, ny, nseg, ylo, yhi)
    for j, dy in enumerate(range(ylo, yhi + 1)):
        for dx in range(xlo, xhi + 1):
            if (dx - ox) ** 2 + (dy - oy) ** 2 > rad * rad:
                continue
            want = _direct(a, b, dx, dy)
            assert abs(got[j, dx % nx] - want) <= 1e-9 * max(1.0, abs(want)), \
                (seed, dx, dy, nx, ny, nseg)


SPLIT_L = (80, 96, 160, 192, 320, 384, 640, 768, 1280, 1536)


def _shortest_len(need):
    pow2 = max(2, 1 << (need - 1).bit_length())
    return min([pow2] + [2 * L for L in SPLIT_L if 2 * L >= need])


@pytest.mark.parametrize("W", [170, 193, 250, 256, 257, 300, 307])
def test_split_row_lengths_for_montage_strips(W):
    """Montage strips (W x 600 here, disc radius 64 at 0): the row axis
    takes the shortest alias-free length among powers of two and the split
    lengths 2L (L = 3 * 2^k, 5 * 2^k) -- W + 64 points are needed -- and
    that grid still gives the linear correlation at the disc's lags."""
    import alignment_projects_gb300 as aln
    keep = []
    h = 600
    nx, ny, nseg, tr = aln.corr_patches_grid(_pair(W, h, W, h, 0, 0, 64, keep))
    assert not tr
    assert nx == _shortest_len(W + 64), (W, nx)
    rng = np.random.default_rng(W)
    a = rng.standard_normal((h, W))
    b = rng.standard_normal((h, W))
    xlo, xhi, ylo, yhi = _window(W, h, W, h, 0, 0, 64)
    got = _plan_corr(a, b, nx, ny, nseg, ylo, yhi)
    for dy in (ylo, -17, 0, 5, yhi):
        for dx in (xlo, -63, -1, 0, 1, 40, xhi):
            if dx * dx + dy * dy > 64 * 64:
                continue
            want = _direct(a, b, dx, dy)
            assert abs(got[dy - ylo, dx % nx] - want) <= 1e-9 * max(1.0, abs(want)), (W, dx, dy)


def test_some_plans_are_segmented():
    import alignment_projects_gb300 as aln
    keep = []
    assert aln.corr_patches_grid(_pair(40, 500, 40, 500, 0, 0, 10, keep))[2] > 0


@pytest.mark.parametrize("seed", range(24))
def test_tie_order_matches_reference_raster(seed):
    """Ties between lags go to the first in the reference raster's row-major
    storage order (Correlation.cpp:1040-1070); the kernels key each lag by
    its storage index on the transform grid (ys * nx + xs, negative lags
    wrapped by the grid size, or the segment length).  Over the disc window
    both orders are the same."""
    import alignment_projects_gb300 as aln
    rng = np.random.default_rng(100 + seed)
    w0, w1 = (int(v) for v in rng.integers(10, 120, 2))
    h0, h1 = (int(v) for v in rng.integers(10, 600, 2))
    ox, oy = (int(v) for v in rng.integers(-40, 41, 2))
    if seed % 4 == 1:   # discs far from the zero lag (long strips, big offsets)
        oy = -int(rng.integers(h0 // 4 + 1, h0 // 2 + 2))
    if seed % 4 == 3:
        oy = int(rng.integers(h1 // 4 + 1, h1 // 2 + 2))
    rad = int(rng.integers(1, 60))
    keep = []
    nx, ny, nseg, tr = aln.corr_patches_grid(_pair(w0, h0, w1, h1, ox, oy, rad, keep))
    if nx == 0:
        return
    if tr:
        w0, h0, w1, h1, ox, oy = h0, w0, h1, w1, oy, ox
    rnx, rny = aln.lib().aln_fft_size(w0, w1), aln.lib().aln_fft_size(h0, h1)
    xlo, xhi, ylo, yhi = _window(w0, h0, w1, h1, ox, oy, rad)
    if xlo > xhi or ylo > yhi:
        return

    def key(x, y, mx, my):   # the kernels' form: one wrap of negative lags
        return ((y + my) if y < 0 else y) * mx + ((x + mx) if x < 0 else x)

    lags = [(x, y) for y in range(ylo, yhi + 1) for x in range(xlo, xhi + 1)]
    ours = np.array([key(x, y, nx, ny) for x, y in lags])
    ref = np.array([key(x, y, rnx, rny) for x, y in lags])
    assert ours.min() >= 0 and ref.min() >= 0
    assert np.array_equal(np.argsort(ours, kind="stable"), np.argsort(ref, kind="stable"))
    # k_final's decode of a storage index back to the lag
    for (x, y), k in zip(lags, ours):
        ys, xs = divmod(int(k), nx)
        assert ((xs - nx) if xs > xhi else xs, (ys - ny) if ys > yhi else ys) == (x, y)


@pytest.mark.parametrize("seed", range(24))
def test_column_rows_decode_to_window_lags(seed):
    """k2_corrcol (one column transform) keeps storage row ys as the lag
    y = ys - Ny when ys >= Ny - (h0 - 1), else y = ys, and stores it when y
    is in the window: on the plan's grid every window lag comes from exactly
    its own storage row."""
    import alignment_projects_gb300 as aln
    rng = np.random.default_rng(500 + seed)
    w0, w1 = (int(v) for v in rng.integers(10, 120, 2))
    h0, h1 = (int(v) for v in rng.integers(10, 600, 2))
    ox, oy = (int(v) for v in rng.integers(-40, 41, 2))
    if seed % 3 == 1:
        oy = -int(rng.integers(h0 // 4 + 1, h0 // 2 + 2))
    if seed % 3 == 2:
        oy = int(rng.integers(h1 // 4 + 1, h1 // 2 + 2))
    rad = int(rng.integers(1, 60))
    keep = []
    P = _pair(w0, h0, w1, h1, ox, oy, rad, keep)
    P.b_key = 7   # keyed: one column transform per column
    nx, ny, nseg, tr = aln.corr_patches_grid(P)
    assert nseg == 0
    if nx == 0:
        return
    if tr:
        w0, h0, w1, h1, ox, oy = h0, w0, h1, w1, oy, ox
    xlo, xhi, ylo, yhi = _window(w0, h0, w1, h1, ox, oy, rad)
    got = {}
    for ys in range(ny):
        y = ys - ny if ys >= ny - (h0 - 1) else ys
        if ylo <= y <= yhi:
            assert y not in got
            got[y] = ys
    assert sorted(got) == list(range(ylo, yhi + 1))
    for y, ys in got.items():
        assert ys == y % ny
