"""The C++ drop-in (libaln_corr_shim.so) exports the reference's
Correlation.h symbols under exactly the reference's mangled names, so its
callers relink unchanged.  Checked against the reference's own build
(oracle/_ref, compiled from its sources by oracle/ref/Makefile) and by linking
one of the reference's own caller programs against the shim.  No GPU needed:
nothing here runs a correlation."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

EXPECTED = {
    "FFTSize": "_Z7FFTSizeii",
    "FFTSizeSQR": "_Z10FFTSizeSQRiiii",
    "FFT_2D": "_Z6FFT_2DRSt6vectorISt7complexIdESaIS1_EERKS_IdSaIdEEiibP8_IO_FILE",
    "IFT_2D": "_Z6IFT_2DRSt6vectorIdSaIdEERKS_ISt7complexIdESaIS4_EEiiP8_IO_FILE",
    "ParabPeakFFT": "_Z12ParabPeakFFTRdS_iPKdii",
    "Convolve": "_Z8ConvolveRSt6vectorIdSaIdEERKS1_iiPKdiibbRS_ISt7complexIdESaIS8_EEP8_IO_FILE",
    "CorrPatches": "_Z11CorrPatchesP8_IO_FILEiRdS1_RKSt6vectorI5PointSaIS3_EERKS2_IdSaIdEES7_SB_"
                   "iiiPFbiiPvESC_SE_SC_RS2_ISt7complexIdESaISG_EE",
    "CorrPatchToImage": "_Z16CorrPatchToImageRdS_RKSt6vectorI5PointSaIS1_EERKS0_IdSaIdEES9_iiib",
    "CorrImagesF": "_Z11CorrImagesFP8_IO_FILEiRdS1_RKSt6vectorI5PointSaIS3_EERKS2_IdSaIdEES7_SB_"
                   "PFbiiPvESC_SE_SC_ddiiiiRS2_ISt7complexIdESaISG_EE",
    "CorrImagesR": "_Z11CorrImagesRP8_IO_FILEiRdS1_RKSt6vectorI5PointSaIS3_EERKS2_IdSaIdEES7_SB_"
                   "PFbiiPvESC_SE_SC_ddiiiiRS2_ISt7complexIdESaISG_EE",
    "CorrImagesS": "_Z11CorrImagesSP8_IO_FILEiRdS1_RKSt6vectorI5PointSaIS3_EERKS2_IdSaIdEES7_SB_"
                   "PFbiiPvESC_SE_SC_ddiiiiRS2_ISt7complexIdESaISG_EE",
    "GradDescStep": "_Z12GradDescStepRSt6vectorIdSaIdEERS_I5PointSaIS3_EERKS5_RKS_IS1_SaIS1_EERKS1_SE_ii",
    "CorrVectors": "_Z11CorrVectorsP8_IO_FILERKSt6vectorIdSaIdEES5_Pi",
    "ImproveControlPts": "_Z17ImproveControlPtsRSt6vectorI5PointSaIS0_EERKS_IS_IdSaIdEESaIS5_EERKS5_SB_iiP8_IO_FILEPKcdd",
}


# class CThmScan (0_GEN/CThmScan.h:57-223): every public member function and
# the exported BigEnough, as the reference's CThmScan.o defines them
EXPECTED_THM = [
    "_Z9BigEnoughiiPv",
    "_ZN8CThmScanC1Ev", "_ZN8CThmScanC2Ev",
    "_ZN8CThmScan10InitializeEP8_IO_FILER6CorRec",
    "_ZN8CThmScan9PretweaksEddR6ThmRec",
    "_ZN8CThmScan10RFromAngleER6CorRecdR6ThmReci",
    "_ZN8CThmScan9DebugAngsEiiiidddR6ThmRec",
    "_ZN8CThmScan13AngleScanMaxRER6CorRecdddbR6ThmRec",
    "_ZN8CThmScan16AngleScanConstXYER6CorRecdddR6ThmRec",
    "_ZN8CThmScan12AngleScanSelER6CorRecdddbR6ThmRec",
    "_ZN8CThmScan19AngleScanWithTweaksER6CorRecdddR6ThmRec",
    "_ZN8CThmScan8PeakHuntER6CorRecdR6ThmRec",
    "_ZN8CThmScan14UsePriorAnglesER6CorReciddR6ThmRec",
    "_ZN8CThmScan15DenovoBestAngleER6CorRecdddR6ThmRecb",
    "_ZN8CThmScan10PostTweaksER6CorRecR6ThmRec",
    "_ZN8CThmScan15FinishAtFullResER6CorRecR6ThmRec",
]


def _exports(path):
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True,
                         check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


@pytest.fixture(scope="module")
def shim():
    from alignment_projects_gb300 import build as b
    return b.build_shim()


def test_shim_exports_reference_signatures(shim):
    ex = _exports(shim)
    for name, mangled in EXPECTED.items():
        assert mangled in ex, name
    for mangled in EXPECTED_THM:
        assert mangled in ex, mangled
    # nothing else at namespace scope: the shim adds no stray symbols
    assert {s for s in ex if s.startswith("_Z") and "St" not in s[:4]} <= \
        set(EXPECTED.values()) | set(EXPECTED_THM)


def test_same_names_as_the_reference_build(shim):
    import oracle
    if not oracle.ref_available():
        try:
            oracle.build_ref()
        except Exception:
            pass
    if not oracle.ref_available():
        pytest.skip("the reference's own build exists only where its sources are mounted")
    ref = _exports(oracle.REF_SO)
    for name, mangled in EXPECTED.items():
        assert mangled in ref, name
    for mangled in EXPECTED_THM:
        assert mangled in ref, mangled


def test_reference_caller_links_against_shim(shim):
    """The reference's own CorrPatches test program (Retired_Proj/4_TestNormCorr),
    compiled from its sources where they lie, links against the shim in place
    of Correlation.o."""
    import oracle
    src = os.path.join(oracle.reference_tree(), "Retired_Proj", "4_TestNormCorr",
                       "testnormcorr.cpp")
    timer = os.path.join(os.path.dirname(oracle.REF_SO), "Timer.o")
    if not (os.path.exists(src) and oracle.ref_available() and os.path.exists(timer)):
        pytest.skip("the reference's sources are not mounted here")
    gen = os.path.join(oracle.reference_tree(), "0_GEN")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "testnormcorr")
        subprocess.check_call(["g++", "-O1", "-w", "-DTIXML_USE_STL", "-I" + gen,
                               "-I" + os.path.join(oracle.reference_tree(), "0_UTL"),
                               "-I" + os.path.join(ROOT, "oracle", "ref"),
                               "-o", exe, src, timer, "-L" + os.path.dirname(shim),
                               "-laln_corr_shim", "-laln_corr", "-lpthread",
                               "-Wl,-rpath," + os.path.dirname(shim)])
        assert os.path.exists(exe)


def _reference_tree():
    import oracle
    if not (os.path.isdir(os.path.join(oracle.reference_tree(), "0_GEN")) and
            oracle.ref_available()):
        pytest.skip("the reference's sources are not mounted here")
    return oracle.reference_tree()


def test_thmscan_layout_matches_reference(tmp_path):
    """class CThmScan, ThmRec and CorRec have the reference's sizes and member
    offsets (callers built from the reference's header allocate the object
    and run its inline setters; the shim's member functions read it)."""
    tree = _reference_tree()
    src = os.path.join(ROOT, "tests", "cpp", "thmscan_layout.cpp")
    outs = []
    for ref in (False, True):
        exe = os.path.join(str(tmp_path), "layout%d" % ref)
        cmd = ["g++", "-std=c++17", "-w", "-o", exe, src]
        cmd += (["-DALN_REFERENCE_HEADERS", "-DTIXML_USE_STL",
                 "-I" + os.path.join(tree, "0_GEN"), "-I" + os.path.join(tree, "0_UTL")]
                if ref else ["-I" + os.path.join(ROOT, "alignment_projects_gb300", "shim")])
        subprocess.check_call(cmd)
        outs.append(subprocess.run([exe], capture_output=True, text=True, check=True).stdout)
    assert outs[0] == outs[1], (outs[0], outs[1])


def test_reference_thmscan_caller_links_against_shim(tmp_path):
    """A CThmScan caller compiled from the reference's own headers (the call
    sequences of ApproximateMatch / CThmUtil) links against the shim in
    place of CThmScan.o and Correlation.o."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from shim_util import build_thm_check
    exe = build_thm_check(str(tmp_path), reference_headers=_reference_tree())
    assert os.path.exists(exe)


def test_thmscan_rejects_fractional_a_points(tmp_path):
    """The CThmScan drop-in bins thumbnail A on integer pixels; a ThmRec whose
    A points are fractional is refused on the host (logged, R = 0) before any
    GPU call, so this runs here without a GPU."""
    import sys
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from shim_util import build_thm_check, thm_case, parse_thm_lines
    exe = build_thm_check(str(tmp_path))
    rng = np.random.default_rng(0)
    pa = rng.random((50, 2)) * 20.0          # fractional
    pb = np.stack(np.meshgrid(np.arange(20.0), np.arange(20.0)), -1).reshape(-1, 2)
    cases = os.path.join(str(tmp_path), "frac.bin")
    open(cases, "wb").write(thm_case(1, pa, rng.random(50), pb, rng.random(len(pb)), 10,
                                     ang0=1.5))
    log = os.path.join(str(tmp_path), "frac.log")
    out = subprocess.run([exe, cases, log], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    g = parse_thm_lines(out.stdout)[0]
    assert (g["A"], g["R"], g["X"], g["Y"]) == (1.5, 0.0, 0.0, 0.0)
    assert "integer pixels" in open(log).read()
