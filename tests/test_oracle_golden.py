"""The C restatement (oracle/aln_oracle.c) against the reference's own outputs.

tests/golden/*.npz were produced by tests/golden/make_golden.py, which runs the
reference's unmodified correlation sources.  The restatement must reproduce
them to the last bits (FP64 with the same operation order); a tolerance of
1e-12 covers libm differences between hosts.
"""
import numpy as np
import pytest

from conftest import legal_from, load_golden

TOL = 1e-12


def close(a, b, tol=TOL):
    return abs(float(a) - float(b)) <= tol * max(1.0, abs(float(b)))


@pytest.mark.parametrize("case", sorted(load_golden("corr_patches")))
def test_corr_patches_golden(orc, case):
    d = load_golden("corr_patches")[case]
    lg = legal_from(d["legal"])
    o = orc.corr_patches(d["pa"], d["va"], d["pb"], d["vb"], int(d["ox"]), int(d["oy"]),
                         int(d["radius"]), lg)
    assert close(o["r"], d["r"]), (o["r"], float(d["r"]))
    if o["status"] == 1:
        # no legal lag: the reference returns 0.0 and leaves dx, dy untouched
        assert float(d["r"]) == 0.0
    else:
        assert close(o["dx"], d["dx"]) and close(o["dy"], d["dy"]), (o, d["dx"], d["dy"])


def test_kat_testnormcorr_values():
    """Retired_Proj/4_TestNormCorr: exact copy at lag (-4, +2) gives r = 1."""
    d = load_golden("corr_patches")["kat_testnormcorr"]
    assert float(d["r"]) == 1.0
    assert round(float(d["dx"])) == -4 and float(d["dy"]) == 2.0


@pytest.mark.parametrize("case", sorted(load_golden("corr_images")))
def test_corr_images_golden(orc, case):
    d = load_golden("corr_images")[case]
    lg = legal_from(d["legal"])
    disc = [int(v) for v in d["disc"]]
    o = orc.corr_images(int(d["kind"]), d["pa"], d["va"], d["pb"], d["vb"], lg,
                        float(d["mincor"]), float(d["nbmaxht"]), *disc)
    assert close(o["r"], d["r"]), (o["r"], float(d["r"]))
    assert close(o["dx"], d["dx"]) and close(o["dy"], d["dy"])


@pytest.mark.parametrize("case", ["fft_8x16", "fft_64x32", "fft_32x128"])
def test_fft_golden(orc, case):
    d = load_golden("fft")[case]
    F = orc.fft_2d(d["x"])
    assert np.abs(F - d["F"]).max() <= 1e-12 * np.abs(d["F"]).max()
    x = d["x"]
    G = orc.ift_2d(F * np.conj(orc.fft_2d(np.roll(x, (2, 3), (0, 1)))), x.shape[1])
    assert np.abs(G - d["G"]).max() <= 1e-12 * np.abs(d["G"]).max()


def test_kat_time_fft(orc):
    """Retired_Proj/4_Time_FFT: a copy shifted by index 2N+3 is recovered."""
    d = load_golden("fft")["kat_time_fft"]
    N = d["in1"].shape[0]
    G = orc.ift_2d(orc.fft_2d(d["in1"]) * np.conj(orc.fft_2d(d["in2"])), N)
    assert int(np.argmax(G)) == int(d["argmax"])
    x, y = divmod(int(d["argmax"]), N)
    x = x - N if x > N // 2 else x
    y = y - N if y > N // 2 else y
    assert (x, y) == (-2, -3)


@pytest.mark.parametrize("case", ["conv_37x50", "conv_64x64"])
def test_convolve_golden(orc, case):
    d = load_golden("convolve")[case]
    out = orc.convolve(d["src"], d["K"])
    assert np.abs(out - d["dst"]).max() <= 1e-12


@pytest.mark.parametrize("case", ["p2i_f0", "p2i_f1"])
def test_patch_to_image_golden(orc, case):
    d = load_golden("patch_to_image")[case]
    o = orc.corr_patch_to_image(d["pa"], d["va"], d["img2"], 0, 0, 4096,
                                bool(int(d["bfilter"])))
    assert close(o["r"], d["r"]) and close(o["dx"], d["dx"]) and close(o["dy"], d["dy"])


@pytest.mark.parametrize("case", sorted(load_golden("thm_scan")))
def test_thm_scan_golden(orc, case):
    d = load_golden("thm_scan")[case]
    disc = tuple(int(v) for v in d["disc"])
    o = orc.thm_search(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]),
                       rthresh=float(d["rthresh"]), pretweak=int(d["pretweak"]),
                       disc=disc, mode=int(d["mode"]), ang0=float(d["ang0"]),
                       hfang=float(d["hfang"]), step=float(d["step"]))
    for k in ("A", "X", "Y", "R"):
        assert close(o[k], d[k]), (k, o[k], float(d[k]))
    assert o["err"] == int(d["err"])


@pytest.mark.parametrize("case", sorted(load_golden("thm_finish")))
def test_thm_finish_golden(orc, case):
    """PostTweaks / FinishAtFullRes (CThmScan.cpp:796-842) from a prior best."""
    d = load_golden("thm_finish")[case]
    o = orc.thm_finish(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]), int(d["mode"]),
                       d["prior"], tptwk=d["tptwk"])
    for k in ("A", "X", "Y", "R"):
        assert close(o[k], d[k]), (k, o[k], float(d[k]))
    assert np.abs(np.array(o["tptwk"]) - d["tptwk_out"]).max() <= 1e-12


@pytest.mark.parametrize("case", sorted(load_golden("thm_scan_f")))
def test_thm_scan_f_golden(orc, case):
    """The sweep with useCorrR off (RFromAngle through CorrImagesF)."""
    d = load_golden("thm_scan_f")[case]
    o = orc.thm_search(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]), usecorrr=0,
                       mode=int(d["mode"]), ang0=float(d["ang0"]), hfang=float(d["hfang"]),
                       step=float(d["step"]))
    for k in ("A", "X", "Y", "R"):
        assert close(o[k], d[k]), (k, o[k], float(d[k]))
    assert o["err"] == int(d["err"])


def test_decimate_golden(orc):
    d = load_golden("decimate")["dec8"]
    xy, v = orc.decimate_normalize(d["pa"], d["va"], int(d["w"]), int(d["h"]),
                                   int(d["lbin"]))
    assert np.array_equal(xy, d["xy"])
    assert np.abs(v - d["v"]).max() <= 1e-12


@pytest.mark.parametrize("lbin,masked", [(8, False), (8, True), (5, True), (16, False)])
def test_decimate_against_reference_build(lbin, masked):
    """DecimateVector + Normalize: the restatement against the reference's
    own build on raster-order point lists, incl. lbin 16 (full bins wrap the
    reference's uint8 counter to 0 and are dropped) -- bitwise."""
    import oracle
    if not oracle.ref_available():
        try:
            oracle.build_ref()
        except Exception:
            pass
    if not oracle.ref_available():
        pytest.skip("the reference's own build exists only where its sources are mounted")
    orc, ref = oracle.Oracle(), oracle.Ref()
    rng = np.random.default_rng(lbin + 100 * masked)
    h, w = 133, 171
    img = rng.integers(0, 256, (h, w)).astype(np.float64)
    keep = np.ones((h, w), bool)
    if masked:
        yy, xx = np.mgrid[0:h, 0:w]
        keep = ((xx - 80) ** 2 + (yy - 60) ** 2) < 70 ** 2
    ys, xs = np.nonzero(keep)
    pts = np.stack([xs, ys], 1).astype(np.float64)
    vals = img[ys, xs]
    xo, vo = orc.decimate_normalize(pts, vals, w, h, lbin)
    xr, vr = ref.decimate_normalize(pts, vals, w, h, lbin)
    assert np.array_equal(xo, xr)
    assert np.array_equal(vo, vr)
    if lbin == 16:   # a full 16 x 16 bin is dropped
        assert len(xr) < (-(-w // 16)) * (-(-h // 16))


@pytest.mark.parametrize("case", sorted(load_golden("mesh")))
def test_mesh_optimizer_golden(orc, case):
    """GradDescStep, CorrVectors and ImproveControlPts: the restatement is the
    reference's bit for bit (same sums in the same order)."""
    d = load_golden("mesh")[case]
    bnew, drdc = orc.grad_desc_step(d["ac0"], d["am_idx"], d["am_w"], d["av"], d["bimg"])
    assert np.array_equal(bnew, d["bnew0"])
    assert np.array_equal(drdc, d["drdc0"])
    cv, nnz = orc.corr_vectors(d["av"], bnew)
    assert cv == float(d["corr0"]) and nnz == int(d["nnz0"])
    r, ac, it = orc.improve_control_pts(d["ac0"], d["am_idx"], d["am_w"], d["av"], d["bimg"],
                                        float(d["ini"]), float(d["fin"]))
    assert r == float(d["corr"])
    assert np.array_equal(ac, d["ac"])
