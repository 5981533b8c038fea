"""The C ABI library builds, loads and exports every symbol include/*.h declares
(no compute here: no GPU on this host)."""
import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(aln_[a-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    return syms


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("aln_ctx_create", "aln_corr_patches", "aln_corr_patches_batch",
              "aln_fft_2d", "aln_ift_2d", "aln_fft_size"):
        assert s in syms


def test_library_exports_all_declared_symbols():
    from alignment_projects_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [s for s in sorted(declared_symbols()) if not hasattr(lib, s)]
    assert not missing, missing


def test_fft_size_matches_reference_rule():
    from alignment_projects_gb300 import lib
    L = lib()
    import oracle
    orc = oracle.Oracle()
    for n1, n2 in [(1, 1), (5, 7), (512, 512), (300, 307), (2048, 2048), (64, 1000)]:
        assert L.aln_fft_size(n1, n2) == orc.lib.orc_fft_size(n1, n2)
    assert L.aln_fft_size_sqr(10, 20, 30, 5) == orc.lib.orc_fft_size_sqr(10, 20, 30, 5)


def test_parab_peak_fft_host_matches_oracle():
    import numpy as np
    import alignment_projects_gb300 as aln
    import oracle
    orc = oracle.Oracle()
    rng = np.random.default_rng(0)
    for _ in range(50):
        I = rng.random((16, 32))
        I[rng.random((16, 32)) < 0.2] = 0.0
        x, y = int(rng.integers(-15, 31)), int(rng.integers(-7, 15))
        gx, gy = aln.parab_peak_fft(x, y, 1, I)
        ox, oy = ctypes.c_double(x), ctypes.c_double(y)
        orc.lib.orc_parab_peak_fft(ctypes.byref(ox), ctypes.byref(oy), 1,
                                   I.ctypes.data_as(ctypes.c_void_p), 32, 16)
        assert (gx, gy) == (ox.value, oy.value)


def test_context_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        return
    import pytest
    import alignment_projects_gb300 as aln
    with pytest.raises(aln.AlnError):
        aln.Context(0)


def _pair(w0, h0, w1, h1, ox, oy, radius, buf):
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnImage, AlnPair
    P = AlnPair()
    P.a = AlnImage(buf.ctypes.data, aln.U8, w0, h0, w0, 0, 0, 0)
    P.b = AlnImage(buf.ctypes.data, aln.U8, w1, h1, w1, 0, 0, 0)
    P.ox, P.oy, P.radius = ox, oy, radius
    P.legal = aln.legal()
    return P


def test_corr_patches_grid_keeps_disc_lags_alias_free():
    """The CorrPatches transform grid: the shortest alias-free length -- a
    power of two, or on the row axis a split length 2L (L = 3 * 2^k,
    5 * 2^k) -- no larger than the reference's FFTSize grid, holding both
    images, and leaving every lag of the disc window free of wrap-around
    (x + m N outside the linear support [-(w0-1), w1-1] for m != 0).  Host
    planning only."""
    import numpy as np
    import alignment_projects_gb300 as aln
    buf = np.zeros(4096 * 4096, np.uint8)
    rng = np.random.default_rng(5)
    shrunk = segmented = split = 0
    split_lens = {2 * L for L in (80, 96, 160, 192, 320, 384, 640, 768, 1280, 1536)}
    cases = [(256, 2048, 256, 2048, 0, 0, 64), (200, 2048, 200, 2048, 0, 0, 64),
             (512, 512, 512, 512, 0, 0, 4096), (300, 120, 280, 100, 0, 0, 30),
             (64, 64, 64, 64, 40, -40, 10), (1, 1, 1, 1, 0, 0, 5)]
    for _ in range(400):
        w0, h0, w1, h1 = (int(v) for v in rng.integers(1, 700, 4))
        ox, oy = (int(v) for v in rng.integers(-300, 300, 2))
        cases.append((w0, h0, w1, h1, ox, oy, int(rng.integers(0, 400))))
    for (w0, h0, w1, h1, ox, oy, rad) in cases:
        nx, ny, nseg, tr = aln.corr_patches_grid(_pair(w0, h0, w1, h1, ox, oy, rad, buf))
        if tr:   # solved transposed: the grid is in the exchanged frame
            w0, h0, w1, h1, ox, oy = h0, w0, h1, w1, oy, ox
        xlo, xhi = max(-(w0 - 1), ox - rad), min(w1 - 1, ox + rad)
        ylo, yhi = max(-(h0 - 1), oy - rad), min(h1 - 1, oy + rad)
        if xlo > xhi or ylo > yhi:
            assert (nx, ny) == (0, 0)
            continue
        if nseg:
            # segmented columns: each segment of a's rows plus the window's
            # rows fits one transform, and the segments cover a's rows
            wy = yhi - ylo + 1
            seg_len = -(-h0 // nseg)
            assert ny & (ny - 1) == 0 and ny < aln.lib().aln_fft_size(h0, h1)
            assert seg_len + wy - 1 <= ny and nseg * seg_len >= h0
            segmented += 1
        # the row length: the shortest alias-free one of the powers of two
        # and the split lengths
        need = max(max(w0, w1), max(w1 - 1 - xlo, xhi + w0 - 1) + 1)
        cands = [c for c in split_lens | {max(2, 1 << (need - 1).bit_length())} if c >= need]
        assert nx == min(min(cands), max(2, aln.lib().aln_fft_size(w0, w1))), (nx, need)
        split += nx in split_lens
        for n, a0, a1, lo, hi in ((nx, w0, w1, xlo, xhi),) + (
                () if nseg else ((ny, h0, h1, ylo, yhi),)):
            ref = aln.lib().aln_fft_size(a0, a1)
            assert (n & (n - 1) == 0 or (n is nx and n in split_lens)) and n <= max(2, ref), \
                (n, ref)
            assert n >= max(a0, a1)
            for m in (-2, -1, 1, 2):
                for d in (lo, hi):
                    assert not (-(a0 - 1) <= d + m * n <= a1 - 1), (n, d, m)
            shrunk += n < ref
    assert shrunk > 50   # many discs allow a smaller grid
    assert segmented > 10
    assert split > 50    # and many a split row length
    # the montage strips (W x 2048, disc radius 64) are segmented
    assert aln.corr_patches_grid(_pair(200, 2048, 200, 2048, 0, 0, 64, buf))[2] > 0
