"""GPU parity: the CUDA CorrPatches / FFT path against the oracle and the
reference's golden outputs, through the C ABI.

Tolerances (FP32 FFTs, FP64 normalisation): the integer peak equals the
oracle's wherever the oracle's top-two margin exceeds 1e-3; r within 1e-4;
sub-pixel dx, dy within 0.01 px.
"""
import numpy as np
import pytest

from conftest import legal_from, load_golden

pytestmark = pytest.mark.gpu

R_TOL = 1e-4
PX_TOL = 0.01
MARGIN = 1e-3


@pytest.fixture(scope="module")
def ctx():
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    yield c
    c.close()


def aln_legal(o_legal):
    import alignment_projects_gb300 as aln
    return aln.legal(o_legal.rgn_kind, o_legal.rgn_a, o_legal.rgn_b, o_legal.rgn_area,
                     o_legal.cnt_kind, o_legal.cnt_n)


def points_to_raster(pts, vals):
    """Integer point cloud -> (raster, origin): ImageFromValuesAndPoints for
    integer coordinates (duplicates add)."""
    pts = np.asarray(pts)
    assert np.all(pts == np.round(pts))
    x = pts[:, 0].astype(np.int64)
    y = pts[:, 1].astype(np.int64)
    x0, y0 = x.min(), y.min()
    w, h = x.max() - x0 + 1, y.max() - y0 + 1
    img = np.zeros((h, w), np.float64)
    np.add.at(img, (y - y0, x - x0), vals)
    return img, (int(x0), int(y0))


def assert_parity(g, o, ctxmsg=""):
    import alignment_projects_gb300 as aln
    if o["status"] == 1:
        assert g["status"] == aln.ALN_NO_PEAK, (ctxmsg, g, o)
        return
    assert g["status"] == aln.ALN_OK, (ctxmsg, g)
    assert abs(g["r"] - o["r"]) <= R_TOL, (ctxmsg, g["r"], o["r"])
    if o["r"] - o["second"] > MARGIN:
        assert (g["peak_x"], g["peak_y"]) == (o["bigx"], o["bigy"]), (ctxmsg, g, o)
        assert abs(g["dx"] - o["dx"]) <= PX_TOL and abs(g["dy"] - o["dy"]) <= PX_TOL, (ctxmsg, g, o)


# ---------------------------------------------------------------- FFT_2D / IFT_2D

@pytest.mark.parametrize("shape", [(1, 2), (4, 8), (8, 16), (64, 32), (32, 128), (256, 512),
                                   (1024, 1024), (4096, 512), (512, 4096), (8192, 64)])
def test_fft_2d_matches_numpy(ctx, shape):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    x = rng.standard_normal(shape)
    F = ctx.fft_2d(x)
    ref = np.fft.rfft2(x)
    err = np.abs(F - ref).max() / np.abs(ref).max()
    assert err < 2e-6, err
    back = ctx.ift_2d(ref, shape[1])
    err2 = np.abs(back / x.size - x).max() / np.abs(x).max()
    assert err2 < 2e-6, err2


def test_fft_golden(ctx):
    for case, d in load_golden("fft").items():
        if "x" not in d:
            continue
        F = ctx.fft_2d(d["x"])
        assert np.abs(F - d["F"]).max() <= 2e-6 * np.abs(d["F"]).max(), case


def test_kat_time_fft(ctx):
    """Retired_Proj/4_Time_FFT: a copy shifted by index 2N+3 is recovered."""
    d = load_golden("fft")["kat_time_fft"]
    N = d["in1"].shape[0]
    G = ctx.ift_2d(ctx.fft_2d(d["in1"]) * np.conj(ctx.fft_2d(d["in2"])), N)
    assert int(np.argmax(G)) == int(d["argmax"])


# ---------------------------------------------------------------- CorrPatches golden

@pytest.mark.parametrize("case", sorted(load_golden("convolve")))
def test_convolve_golden(ctx, case):
    """Convolve (0_GEN/Correlation.cpp:371-457) against the reference's output:
    FP32 transforms, so within 1e-5 of the result's range."""
    d = load_golden("convolve")[case]
    g = ctx.convolve(d["src"], d["K"], sym=True, prenorm=True)
    ref = np.asarray(d["dst"])
    assert np.abs(g - ref).max() <= 1e-5 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("case", sorted(load_golden("corr_patches")))
def test_corr_patches_golden(ctx, orc, case):
    d = load_golden("corr_patches")[case]
    a, ao = points_to_raster(d["pa"], d["va"])
    b, bo = points_to_raster(d["pb"], d["vb"])
    lg = legal_from(d["legal"])
    g = ctx.corr_patches(a, b, int(d["ox"]), int(d["oy"]), int(d["radius"]), aln_legal(lg),
                         ao, bo)
    o = orc.corr_patches(d["pa"], d["va"], d["pb"], d["vb"], int(d["ox"]), int(d["oy"]),
                         int(d["radius"]), lg)
    # the oracle reproduces the reference bit-exactly (tests/test_oracle_golden.py)
    assert abs(o["r"] - float(d["r"])) < 1e-12
    assert_parity(g, o, case)
    if o["status"] == 0 and o["r"] - o["second"] > MARGIN:
        assert abs(g["dx"] - float(d["dx"])) <= PX_TOL and abs(g["dy"] - float(d["dy"])) <= PX_TOL


def test_kat_testnormcorr(ctx):
    """Retired_Proj/4_TestNormCorr: the exact copy is found with r = 1 at lag (-4, +2)."""
    import alignment_projects_gb300 as aln
    d = load_golden("corr_patches")["kat_testnormcorr"]
    a, ao = points_to_raster(d["pa"], d["va"])
    b, bo = points_to_raster(d["pb"], d["vb"])
    g = ctx.corr_patches(a, b, 0, 0, 4096, aln.legal(aln.RGN_MIN, 2, 2, 0), ao, bo)
    assert abs(g["r"] - 1.0) < 1e-5
    assert abs(g["dx"] - float(d["dx"])) < PX_TOL and g["dy"] == pytest.approx(2.0, abs=PX_TOL)


# ---------------------------------------------------------------- synthetic workloads

def _oracle_pair(orc, p, lg_o):
    import oracle
    A, VA = oracle.image_to_points(p.a)
    B, VB = oracle.image_to_points(p.b)
    return orc.corr_patches(A, VA, B, VB, p.ox, p.oy, p.radius, lg_o)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_plain_512_pair(ctx, orc, seed):
    """The 512^2 uint8 single-pair workload (FFT 1024^2), full lag window."""
    import oracle
    from alignment_projects_gb300 import synth
    p = synth.plain_pair(seed, n=512, margin=64)
    lg_o = oracle.legal(oracle.RGN_MIN, 32, 32, 0)
    g = ctx.corr_patches(p.a, p.b, 0, 0, 4096, aln_legal(lg_o))
    o = _oracle_pair(orc, p, lg_o)
    assert_parity(g, o, f"plain seed {seed}")
    assert (g["peak_x"], g["peak_y"]) == p.truth


@pytest.mark.parametrize("seed", [11, 12, 13, 14])
def test_montage_strips(ctx, orc, seed):
    """Montage overlap strips (W x 2048 / 2048 x W uint8), disc radius 64."""
    import oracle
    from alignment_projects_gb300 import synth
    p = synth.montage_pair(seed)
    lg_o = oracle.legal(oracle.RGN_SECTION, 1500, 1500, 30000)
    g = ctx.corr_patches(p.a, p.b, p.ox, p.oy, p.radius, aln_legal(lg_o))
    o = _oracle_pair(orc, p, lg_o)
    assert_parity(g, o, f"montage seed {seed}")
    if not p.decoy:
        assert (g["peak_x"], g["peak_y"]) == p.truth


@pytest.mark.parametrize("seed", range(20, 32))
def test_uneven_u16(ctx, orc, seed):
    """uint16 patches of uneven, non-square sizes with a disc."""
    import oracle
    from alignment_projects_gb300 import synth
    p = synth.uneven_pair(seed, smax=512)
    lg_o = oracle.legal(oracle.RGN_MIN, 8, 8, 0)
    g = ctx.corr_patches(p.a, p.b, p.ox, p.oy, p.radius, aln_legal(lg_o))
    o = _oracle_pair(orc, p, lg_o)
    assert_parity(g, o, f"uneven seed {seed}")


@pytest.mark.parametrize("seed", range(70, 76))
def test_uneven_u16_large(ctx, orc, seed):
    """The top of the uneven batch's size range: long sides 700-1024 px,
    i.e. 2048-point axes on the reference's FFTSize grid."""
    import oracle
    from alignment_projects_gb300 import synth
    p = synth.uneven_pair(seed, smin=700, smax=1024)
    assert max(p.a.shape) >= 700
    lg_o = oracle.legal(oracle.RGN_MIN, 8, 8, 0)
    g = ctx.corr_patches(p.a, p.b, p.ox, p.oy, p.radius, aln_legal(lg_o))
    o = _oracle_pair(orc, p, lg_o)
    assert o["nx"] == 2048 or o["ny"] == 2048, (o["nx"], o["ny"])
    assert_parity(g, o, f"uneven large seed {seed}")
    assert (g["peak_x"], g["peak_y"]) == p.truth


def _disc_case(seed):
    rng = np.random.default_rng(seed)
    w, h = int(rng.integers(24, 200)), int(rng.integers(24, 200))
    f = rng.normal(0.0, 1.0, (h + 100, w + 100))
    for ax in (0, 1):   # a few pixels of correlation length
        f = (f + np.roll(f, 1, ax) + np.roll(f, 2, ax)) / 3.0
    tx, ty = (int(v) for v in rng.integers(-30, 31, 2))
    a = f[50:50 + h, 50:50 + w]
    b = f[50 + ty:50 + ty + h, 50 + tx:50 + tx + w] + rng.normal(0.0, 0.1, (h, w))
    a8 = np.clip(np.round(128 + 40 * a), 0, 255).astype(np.uint8)
    b8 = np.clip(np.round(128 + 40 * b), 0, 255).astype(np.uint8)
    radius = int(rng.integers(3, 40))
    # the disc around a point near the truth: some truths lie outside it,
    # so the best lag sits on the rim
    ox, oy = -tx + int(rng.integers(-12, 13)), -ty + int(rng.integers(-12, 13))
    return a8, b8, ox, oy, radius


@pytest.mark.parametrize("seed", range(40, 64))
def test_disc_on_smaller_grid(ctx, orc, seed):
    """Discs that let CorrPatches transform on a grid smaller than the
    reference's FFTSize grid: the peak, r and the sub-pixel refinement
    (whose neighbours outside the disc read 0, by the reference raster's
    storage rules) equal the oracle's."""
    import oracle
    import alignment_projects_gb300 as aln
    a8, b8, ox, oy, radius = _disc_case(seed)
    lg_o = oracle.legal(oracle.RGN_MIN, 8, 8, 0)
    g = ctx.corr_patches(a8, b8, ox, oy, radius, aln_legal(lg_o))
    A, VA = oracle.image_to_points(a8)
    B, VB = oracle.image_to_points(b8)
    o = orc.corr_patches(A, VA, B, VB, ox, oy, radius, lg_o)
    assert_parity(g, o, f"disc seed {seed}")


@pytest.mark.parametrize("seed", range(8))
def test_disc_far_from_zero_lag(ctx, orc, seed):
    """Discs around large offsets (overlap strips cut with a big nominal
    shift): the window's lag rows lie far from the zero lag, where the
    storage rows of negative lags wrap; peaks and r equal the oracle's."""
    import oracle
    rng = np.random.default_rng(300 + seed)
    w, h = int(rng.integers(30, 70)), int(rng.integers(250, 420))
    f = rng.normal(0.0, 1.0, (3 * h, w + 40))
    for ax in (0, 1):
        f = (f + np.roll(f, 1, ax) + np.roll(f, 2, ax)) / 3.0
    ty = int(rng.integers(h // 4, h // 2)) * (1 if seed % 2 else -1)
    tx = int(rng.integers(-8, 9))
    y0 = h
    a = f[y0:y0 + h, 20:20 + w]
    b = f[y0 + ty:y0 + ty + h, 20 + tx:20 + tx + w] + rng.normal(0.0, 0.1, (h, w))
    a8 = np.clip(np.round(128 + 40 * a), 0, 255).astype(np.uint8)
    b8 = np.clip(np.round(128 + 40 * b), 0, 255).astype(np.uint8)
    ox, oy, radius = -tx + int(rng.integers(-4, 5)), -ty + int(rng.integers(-4, 5)), 12
    lg_o = oracle.legal(oracle.RGN_MIN, 8, 8, 0)
    g = ctx.corr_patches(a8, b8, ox, oy, radius, aln_legal(lg_o))
    A, VA = oracle.image_to_points(a8)
    B, VB = oracle.image_to_points(b8)
    o = orc.corr_patches(A, VA, B, VB, ox, oy, radius, lg_o)
    assert_parity(g, o, f"far disc seed {seed}")
    assert (g["peak_x"], g["peak_y"]) == (-tx, -ty)


def test_disc_grids_shrink_and_batch(ctx):
    """The same disc cases in one batch (several transform grids) give the
    single-call numbers, and most of them run on a smaller grid."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnPair
    jobs, smaller = [], 0
    for seed in range(40, 64):
        a8, b8, ox, oy, radius = _disc_case(seed)
        jobs.append(dict(a=a8, b=b8, ox=ox, oy=oy, radius=radius,
                         legal=aln.legal(aln.RGN_MIN, 8, 8, 0)))
        P = AlnPair()
        P.a, P.b = aln.image(a8), aln.image(b8)
        P.ox, P.oy, P.radius = ox, oy, radius
        nx, ny, nseg, tr = aln.corr_patches_grid(P)
        h, w = a8.shape
        if tr:
            w, h = h, w
        smaller += nx * ny < aln.lib().aln_fft_size(w, w) * aln.lib().aln_fft_size(h, h)
    assert smaller >= len(jobs) // 2
    got = ctx.corr_patches_batch(jobs)
    for j, g in zip(jobs, got):
        single = ctx.corr_patches(j["a"], j["b"], j["ox"], j["oy"], j["radius"], j["legal"])
        assert g == single


@pytest.fixture(scope="module")
def ctx_pow2():
    """A context with power-of-two transform grids only."""
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    c.set_split_grids(False)
    yield c
    c.close()


def _grid_of(job):
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnPair
    P = AlnPair()
    P.a, P.b = aln.image(job["a"]), aln.image(job["b"])
    P.ox, P.oy, P.radius = job["ox"], job["oy"], job["radius"]
    return aln.corr_patches_grid(P)


SPLIT_NX = (160, 192, 320, 384, 640, 768, 1280, 1536, 2560, 3072)


@pytest.mark.parametrize("nx", SPLIT_NX)
def test_split_row_lengths_match_power_of_two(ctx, ctx_pow2, nx):
    """Rows of 3 * 2^k and 5 * 2^k points: a uint8 pair that needs exactly nx
    row points (width nx - 24, disc radius 24) is planned onto that split
    length and gives the power-of-two plan's numbers -- the same peak (the
    true offset), r within 1e-4, the sub-pixel offsets within 0.01 px."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    rad, m = 24, 16
    w = nx - rad
    h = w + 16                     # taller than wide: rows stay the x axis
    rng = np.random.default_rng(nx)
    tx, ty = (int(v) for v in rng.integers(-12, 13, 2))
    f = synth.field_np(nx, h + 2 * m, w + 2 * m)
    a = synth.to_u8(f[m:m + h, m:m + w] + rng.normal(0.0, 8.0, (h, w)))
    b = synth.to_u8(f[m + ty:m + ty + h, m + tx:m + tx + w] + rng.normal(0.0, 8.0, (h, w)))
    job = dict(a=a, b=b, ox=0, oy=0, radius=rad, legal=aln.legal(aln.RGN_MIN, 32, 32, 0))
    gx, _, _, tr = _grid_of(job)
    assert (gx, tr) == (nx, 0), (gx, tr)
    g = ctx.corr_patches_batch([job])[0]
    ref = ctx_pow2.corr_patches_batch([job])[0]
    assert g["status"] == ref["status"] == aln.ALN_OK
    assert (g["peak_x"], g["peak_y"]) == (ref["peak_x"], ref["peak_y"]) == (-tx, -ty), (g, ref)
    assert abs(g["r"] - ref["r"]) <= R_TOL, (g, ref)
    assert abs(g["dx"] - ref["dx"]) <= PX_TOL and abs(g["dy"] - ref["dy"]) <= PX_TOL, (g, ref)


@pytest.mark.parametrize("W", [170, 250, 300])
def test_split_montage_strips_against_oracle(ctx, orc, W):
    """Montage strips whose rows need W + 64 points: 256 (a power of two),
    320 (5 * 64) and 384 (3 * 128) -- held to the oracle's bar, alone and in
    one batch with the other widths."""
    import oracle
    from alignment_projects_gb300 import synth
    lg_o = oracle.legal(oracle.RGN_SECTION, 1500, 1500, 30000)
    ps = [synth.montage_pair(900 + W + k, wmin=w, wmax=w)
          for k, w in enumerate((W, 170, 250, 300))]
    jobs = [dict(a=p.a, b=p.b, ox=p.ox, oy=p.oy, radius=p.radius, legal=aln_legal(lg_o))
            for p in ps]
    want_nx = {170: 256, 250: 320, 300: 384}[W]
    assert _grid_of(jobs[0])[0] == want_nx
    batch = ctx.corr_patches_batch(jobs)
    g = ctx.corr_patches(jobs[0]["a"], jobs[0]["b"], 0, 0, 64, jobs[0]["legal"])
    assert g == batch[0]
    assert_parity(g, _oracle_pair(orc, ps[0], lg_o), f"split strip W={W}")
    if not ps[0].decoy:
        assert (g["peak_x"], g["peak_y"]) == ps[0].truth


@pytest.mark.parametrize("ns", [-1, 0, 256, 512, 1024, 2048])
def test_segmented_columns(ctx, orc, ns):
    """CorrPatches with the column axis cut into segments of every forced
    length, by the cost model, and not at all: each form matches the oracle
    on montage strips (disc radius 64) and on small disc cases."""
    import oracle
    from alignment_projects_gb300 import synth
    jobs, refs = [], []
    for seed in (11, 12):
        p = synth.montage_pair(seed)
        lg_o = oracle.legal(oracle.RGN_SECTION, 1500, 1500, 30000)
        jobs.append(dict(a=p.a, b=p.b, ox=p.ox, oy=p.oy, radius=p.radius, legal=aln_legal(lg_o)))
        refs.append(_oracle_pair(orc, p, lg_o))
    for seed in range(40, 48):
        a8, b8, ox, oy, radius = _disc_case(seed)
        lg_o = oracle.legal(oracle.RGN_MIN, 8, 8, 0)
        if seed % 2:   # FP64 rasters: the FP64 r formula on segmented columns
            a8 = a8.astype(np.float64) / 7.0 + 0.25
            b8 = b8.astype(np.float64) / 7.0 - 0.5
        jobs.append(dict(a=a8, b=b8, ox=ox, oy=oy, radius=radius, legal=aln_legal(lg_o)))
        A, VA = oracle.image_to_points(a8)
        B, VB = oracle.image_to_points(b8)
        refs.append(orc.corr_patches(A, VA, B, VB, ox, oy, radius, lg_o))
    ctx.set_segmenting(ns)
    try:
        got = ctx.corr_patches_batch(jobs)
    finally:
        ctx.set_segmenting(0)
    for k, (g, o) in enumerate(zip(got, refs)):
        assert_parity(g, o, f"segments {ns} job {k}")


def test_batch_equals_single(ctx):
    """A mixed-size batch gives exactly the per-pair results."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    pairs = []
    for s in range(6):
        p = synth.uneven_pair(100 + s, smax=300)
        pairs.append(dict(a=p.a, b=p.b, ox=p.ox, oy=p.oy, radius=p.radius,
                          legal=aln.legal(aln.RGN_MIN, 8, 8, 0)))
    for s in range(3):
        p = synth.plain_pair(200 + s, n=100, margin=10)
        pairs.append(dict(a=p.a, b=p.b, legal=aln.legal(aln.RGN_MIN, 16, 16, 0)))
    batch = ctx.corr_patches_batch(pairs)
    for p, bres in zip(pairs, batch):
        single = ctx.corr_patches(p["a"], p["b"], p.get("ox", 0), p.get("oy", 0),
                                  p.get("radius", 4096), p["legal"])
        assert bres == single


def test_device_resident_inputs(ctx):
    import torch
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    p = synth.plain_pair(5, n=200, margin=20)
    lg = aln.legal(aln.RGN_MIN, 32, 32, 0)
    host = ctx.corr_patches(p.a, p.b, 0, 0, 4096, lg)
    da = torch.from_numpy(p.a).cuda()
    db = torch.from_numpy(p.b).cuda()
    dev = ctx.corr_patches(da, db, 0, 0, 4096, lg)
    assert host == dev


def test_strided_and_table_legality(ctx, orc):
    """Row stride > width, and a tabulated LegalRgn callback."""
    import oracle
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    p = synth.plain_pair(9, n=120, margin=12)
    big = np.zeros((120, 160), np.uint8)
    big[:, :120] = p.a
    a_view = big[:, :120]  # stride 160
    tw, th = 120, 120
    t = np.zeros((th, tw), np.uint8)
    ys, xs = np.mgrid[1:th + 1, 1:tw + 1]
    t[(xs * ys > 4000) & ((xs + ys) % 3 != 0)] = 1
    g = ctx.corr_patches(a_view, p.b, 0, 0, 4096, aln.legal(table=t))
    lo = oracle.Legal(oracle.RGN_TABLE, 0, 0, 0, t.ctypes.data, tw, th, 0, 0)
    A, VA = oracle.image_to_points(p.a)
    B, VB = oracle.image_to_points(p.b)
    o = orc.corr_patches(A, VA, B, VB, 0, 0, 4096, lo)
    assert_parity(g, o, "table")


def test_no_legal_lag(ctx):
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    p = synth.plain_pair(4, n=64, margin=8)
    g = ctx.corr_patches(p.a, p.b, 0, 0, 4096, aln.legal(aln.RGN_EXACT, 999, 999, 0))
    assert g["status"] == aln.ALN_NO_PEAK and g["r"] == 0.0
    # disc entirely outside the lag window
    g = ctx.corr_patches(p.a, p.b, 5000, 5000, 3)
    assert g["status"] == aln.ALN_NO_PEAK


def test_bad_arguments_raise(ctx):
    import alignment_projects_gb300 as aln
    a = np.zeros((0, 5), np.uint8)
    with pytest.raises(aln.AlnError):
        ctx.corr_patches(a, a)
    big = np.zeros((5000, 8), np.uint8)
    with pytest.raises(aln.AlnError):
        ctx.corr_patches(big, big)   # FFT size 16384 > 8192


def test_spectrum_cache_same_numbers(ctx):
    """Jobs sharing image b under one key (the reference's fft2 cache) give
    exactly the results of uncached calls: the first job of a key fills the
    entry, the rest (same batch and later batches) read it."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    rng = np.random.default_rng(7)
    b = synth.plain_pair(300, n=160, margin=12).b
    pairs = []
    for s in range(6):
        a = synth.plain_pair(310 + s, n=150, margin=10).a
        pairs.append(dict(a=a, b=b, ox=int(rng.integers(-5, 6)), oy=int(rng.integers(-5, 6)),
                          radius=40, legal=aln.legal(aln.RGN_MIN, 16, 16, 0)))
    # a wide pair (solved transposed) and a different-size pair under the same key
    w = synth.montage_pair(21)
    pairs.append(dict(a=w.a, b=w.b, ox=w.ox, oy=w.oy, radius=w.radius,
                      legal=aln.legal(aln.RGN_SECTION, 1500, 1500, 30000)))
    # keyed jobs take one column transform per column: compare with the
    # unsegmented uncached form
    ctx.set_segmenting(-1)
    try:
        plain = ctx.corr_patches_batch(pairs)
    finally:
        ctx.set_segmenting(0)
    ctx.profile_reset()
    keyed = [dict(p, b_key=(99 if k < 6 else 100)) for k, p in enumerate(pairs)]
    first = ctx.corr_patches_batch(keyed)
    c1 = ctx.counters()
    again = ctx.corr_patches_batch(keyed)
    c2 = ctx.counters()
    assert first == plain and again == plain
    assert c1["spec_fills"] == 2 and c1["spec_hits"] == 5
    assert c2["spec_fills"] == 2 and c2["spec_hits"] == 12


def test_spectrum_cache_images_and_off(ctx):
    """CorrImages jobs with a keyed b, and the cache switched off and on."""
    import alignment_projects_gb300 as aln
    rng = np.random.default_rng(3)
    b = rng.standard_normal((90, 110))
    jobs = [dict(kind=aln.CORR_S if k % 2 else aln.CORR_R, a=rng.standard_normal((80, 70)),
                 b=b, legal=aln.legal(aln.RGN_MIN, 0, 0, 400, aln.CNT_GT, 400))
            for k in range(5)]
    plain = ctx.corr_images_batch(jobs)
    keyed = [dict(j, b_key=7) for j in jobs]
    assert ctx.corr_images_batch(keyed) == plain
    ctx.set_spectrum_cache(0)
    assert ctx.counters()["spec_bytes"] == 0
    assert ctx.corr_images_batch(keyed) == plain
    ctx.set_spectrum_cache(1 << 30)
    assert ctx.corr_images_batch(keyed) == plain


@pytest.mark.parametrize("dt,w,h", [(np.uint8, 16, 20), (np.uint16, 16, 24), (np.uint8, 9, 12),
                                    (np.uint16, 40, 16), (np.uint8, 5, 70)])
def test_tiny_integer_patches(ctx, orc, dt, w, h):
    """Narrow integer patches (FFT widths 16..32): the row pass's staged
    16-byte loads land in every team's own, 16-byte aligned region."""
    import oracle
    import alignment_projects_gb300 as aln
    rng = np.random.default_rng(w * 100 + h)
    top = 255 if dt == np.uint8 else 4095
    m = min(4, w - 1, h - 1)   # overlaps of at least m x m (two pixels are always r = 1)
    pairs = []
    for k in range(24):   # several pairs: many teams per CTA
        a = rng.integers(0, top + 1, (h, w)).astype(dt)
        b = np.roll(a, (1, 2), axis=(0, 1)).copy()
        pairs.append(dict(a=a, b=b, legal=aln.legal(aln.RGN_MIN, m, m, 0)))
    got = ctx.corr_patches_batch(pairs)
    for p, g in zip(pairs, got):
        A, VA = oracle.image_to_points(p["a"])
        B, VB = oracle.image_to_points(p["b"])
        o = orc.corr_patches(A, VA, B, VB, 0, 0, 4096, oracle.legal(oracle.RGN_MIN, m, m, 0))
        assert_parity(g, o, f"{dt.__name__} {w}x{h}")
