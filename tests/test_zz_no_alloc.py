"""The allocation-free CorrPatches entry point (aln_corr_patches_noalloc).

It exists for callers that cannot allocate device memory -- code inside a
caller-managed pool or arena, or a plugin whose host forbids cudaMalloc while
it runs.  It must give what aln_corr_patches gives, call after call, while
using only the library's fixed device scratch array.

This file is collected last on purpose, so a run that stops at the first
failure has already run every other test.  It passes alone in a fresh process
and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

R_TOL = 1e-4
PX_TOL = 0.01


def _entry():
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnImage, AlnLegal, AlnResult
    L = aln.lib()
    f = L.aln_corr_patches_noalloc
    f.argtypes = [C.POINTER(AlnImage), C.POINTER(AlnImage), C.c_int, C.c_int, C.c_int,
                  C.POINTER(AlnLegal), C.c_void_p, C.POINTER(AlnResult)]
    f.restype = C.c_int
    return L, f


def _cases():
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    p1 = synth.plain_pair(31, n=256, margin=24)
    p2 = synth.montage_pair(41, wmax=256)
    return [
        (p1.a, p1.b, 0, 0, 4096, aln.legal(aln.RGN_MIN, 32, 32, 0)),
        (p2.a, p2.b, p2.ox, p2.oy, p2.radius, aln.legal(aln.RGN_SECTION, 1500, 1500, 30000)),
    ]


def test_noalloc_matches_corr_patches_on_consecutive_calls():
    import torch
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnResult
    torch.cuda.set_device(0)
    L, noalloc = _entry()
    ctx = aln.Context(0)
    cases = [(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), ox, oy, rad, lg)
             for a, b, ox, oy, rad, lg in _cases()]
    # results of the existing (allocating) entry point
    refs = [ctx.corr_patches(a, b, ox, oy, rad, lg) for a, b, ox, oy, rad, lg in cases]
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    # two different pairs back to back, then the first again: each call
    # reuses the scratch array the previous call left behind
    for k in (0, 1, 0):
        a, b, ox, oy, rad, lg = cases[k]
        ia, ib = aln.image(a), aln.image(b)
        res = AlnResult()
        rc = noalloc(C.byref(ia), C.byref(ib), ox, oy, rad, C.byref(lg), None, C.byref(res))
        assert rc == aln.ALN_OK, L.aln_last_error(None).decode()
        g, ref = res.as_dict(), refs[k]
        assert g["status"] == ref["status"] == aln.ALN_OK
        assert (g["peak_x"], g["peak_y"]) == (ref["peak_x"], ref["peak_y"])
        assert abs(g["r"] - ref["r"]) <= R_TOL
        assert abs(g["dx"] - ref["dx"]) <= PX_TOL and abs(g["dy"] - ref["dy"]) <= PX_TOL
        assert (g["nx"], g["ny"]) == (ref["nx"], ref["ny"])
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device memory changed during allocation-free calls"
    ctx.close()


def test_noalloc_rejects_pairs_beyond_the_scratch():
    import torch
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnResult
    L, noalloc = _entry()
    big = torch.zeros((1024, 1024), dtype=torch.uint8, device="cuda")
    ia, ib = aln.image(big), aln.image(big)
    res = AlnResult()
    rc = noalloc(C.byref(ia), C.byref(ib), 0, 0, 4096, None, None, C.byref(res))
    from alignment_projects_gb300.native import ALN_ERR_UNSUPPORTED
    assert rc == ALN_ERR_UNSUPPORTED
    msg = L.aln_last_error(None).decode()
    assert "scratch" in msg and "aln_corr_patches" in msg, msg


def test_noalloc_rejects_host_inputs():
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnResult
    L, noalloc = _entry()
    a = np.zeros((16, 16), np.uint8)
    ia, ib = aln.image(a), aln.image(a)
    res = AlnResult()
    assert noalloc(C.byref(ia), C.byref(ib), 0, 0, 10, None, None, C.byref(res)) == -1
