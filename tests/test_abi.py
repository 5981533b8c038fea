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
