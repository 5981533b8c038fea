"""GB300-native tile matching for the Aligner EM pipeline.

FFT normalised cross-correlation (CorrPatches, CorrImagesF/R/S,
CorrPatchToImage, FFT_2D/IFT_2D) and the CThmScan angle sweep, as CUDA
kernels for sm_103a behind a C ABI (include/aln_corr.h).  This package is the
Python host side of that ABI.
"""
from .native import (  # noqa: F401
    AlnError,
    Context,
    Server,
    REQ_PATCHES,
    REQ_IMAGES,
    REQ_SWEEP,
    legal,
    image,
    lib,
    lib_path,
    parab_peak_fft,
    ALN_OK,
    ALN_NO_PEAK,
    U8,
    U16,
    F32,
    F64,
    RGN_NONE,
    RGN_MIN,
    RGN_SECTION,
    RGN_EXACT,
    RGN_TABLE,
    CNT_NONE,
    CNT_GT,
    CORR_F,
    CORR_R,
    CORR_S,
    THM_DENOVO,
    THM_RFROMANGLE,
    THM_PRIOR,
    THM_SCAN_HUNT,
    THM_SCAN_MAXR,
    THM_POSTTWEAKS,
    THM_FULLRES,
    thumbs_from_points,
)
