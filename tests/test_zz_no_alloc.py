"""The allocation-free CorrPatches entry point (aln_corr_patches_noalloc).

It exists for callers that cannot allocate device memory -- code inside a
caller-managed pool or arena, or a plugin whose host forbids cudaMalloc while
it runs.  It must give what aln_corr_patches gives, call after call, while
using only the library's fixed device scratch array, for every pixel type,
for tabulated legality (the table is copied into the scratch array) and up
to the sizes its header promises (a 512 x 512 pair over its whole lag
window, a 256 x 2048 montage strip pair with a disc).  Each case is also
held to the FP64 oracle's bar: the integer peak where the oracle's top-two
margin exceeds 1e-3, r within 1e-4, dx and dy within 0.01 px.

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
MARGIN = 1e-3


def _entry():
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnImage, AlnLegal, AlnResult
    L = aln.lib()
    f = L.aln_corr_patches_noalloc
    f.argtypes = [C.POINTER(AlnImage), C.POINTER(AlnImage), C.c_int, C.c_int, C.c_int,
                  C.POINTER(AlnLegal), C.c_void_p, C.POINTER(AlnResult)]
    f.restype = C.c_int
    return L, f


def _dev_image(arr):
    """A device copy of a host raster (any pixel type) and its aln_image."""
    import torch
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnImage
    a = np.ascontiguousarray(arr)
    dt = {np.uint8: aln.U8, np.uint16: aln.U16, np.float32: aln.F32,
          np.float64: aln.F64}[a.dtype.type]
    raw = torch.from_numpy(a.view(np.uint8).reshape(a.shape[0], -1).copy()).cuda()
    im = AlnImage(raw.data_ptr(), dt, a.shape[1], a.shape[0], a.shape[1], 0, 0, 1)
    im._keep = raw
    return im


def _table(n):
    ys, xs = np.mgrid[1:n + 1, 1:n + 1]
    t = np.zeros((n, n), np.uint8)
    t[(xs * ys > n * n // 4) & ((xs + ys) % 3 != 0)] = 1
    return t


def _case(name):
    """(a, b, ox, oy, radius, legal kind, legal args) of one named case."""
    import oracle
    from alignment_projects_gb300 import synth
    if name == "u8":
        p = synth.plain_pair(31, n=256, margin=24)
        return p.a, p.b, 0, 0, 4096, (oracle.RGN_MIN, 32, 32, 0)
    if name == "u16":
        p = synth.uneven_pair(23, smin=120, smax=240)
        return p.a, p.b, p.ox, p.oy, p.radius, (oracle.RGN_MIN, 8, 8, 0)
    if name in ("f32", "f64"):
        p = synth.plain_pair(33, n=200, margin=20)
        dt = np.float32 if name == "f32" else np.float64
        rng = np.random.default_rng(5)
        a = (p.a * 0.37 + rng.random(p.a.shape)).astype(dt)
        b = (p.b * 0.37 + rng.random(p.b.shape)).astype(dt)
        return a, b, 0, 0, 4096, (oracle.RGN_MIN, 24, 24, 0)
    if name == "table":
        p = synth.plain_pair(9, n=120, margin=12)
        return p.a, p.b, 0, 0, 4096, ("table", _table(120))
    if name == "full512":   # the header's first size example
        p = synth.plain_pair(35, n=512, margin=64)
        return p.a, p.b, 0, 0, 4096, (oracle.RGN_MIN, 32, 32, 0)
    if name == "strip256":  # the header's second size example
        p = synth.montage_pair(41, wmin=256, wmax=256)
        return p.a, p.b, p.ox, p.oy, p.radius, (oracle.RGN_SECTION, 1500, 1500, 30000)
    raise KeyError(name)


CASES = ["u8", "u16", "f32", "f64", "table", "full512", "strip256"]


def _legals(lg):
    import oracle
    import alignment_projects_gb300 as aln
    if lg[0] == "table":
        t = lg[1]
        return (aln.legal(table=t),
                oracle.Legal(oracle.RGN_TABLE, 0, 0, 0, t.ctypes.data, t.shape[1], t.shape[0],
                             0, 0))
    return aln.legal(*lg), oracle.legal(*lg)


@pytest.fixture(scope="module")
def prepared():
    """Per case: device images, legality, the allocating entry point's
    result and the oracle's."""
    import torch
    import oracle
    import alignment_projects_gb300 as aln
    torch.cuda.set_device(0)
    orc = oracle.Oracle()
    ctx = aln.Context(0)
    out = {}
    for name in CASES:
        a, b, ox, oy, rad, lg = _case(name)
        lg_a, lg_o = _legals(lg)
        ref = ctx.corr_patches(a, b, ox, oy, rad, lg_a)
        A, VA = oracle.image_to_points(a)
        B, VB = oracle.image_to_points(b)
        o = orc.corr_patches(A, VA, B, VB, ox, oy, rad, lg_o)
        out[name] = dict(ia=_dev_image(a), ib=_dev_image(b), ox=ox, oy=oy, rad=rad, lg=lg_a,
                         lg_keep=lg, ref=ref, orc=o)
    ctx.close()
    torch.cuda.synchronize()
    return out


def _call(noalloc, c):
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnResult
    res = AlnResult()
    rc = noalloc(C.byref(c["ia"]), C.byref(c["ib"]), c["ox"], c["oy"], c["rad"],
                 C.byref(c["lg"]), None, C.byref(res))
    assert rc == aln.ALN_OK, aln.lib().aln_last_error(None).decode()
    return res.as_dict()


def _check(g, c, msg):
    import alignment_projects_gb300 as aln
    ref, o = c["ref"], c["orc"]
    # against the allocating entry point
    assert g["status"] == ref["status"] == aln.ALN_OK, (msg, g, ref)
    assert (g["nx"], g["ny"]) == (ref["nx"], ref["ny"]), msg
    assert abs(g["r"] - ref["r"]) <= R_TOL, (msg, g, ref)
    # against the FP64 oracle
    assert o["status"] == 0
    assert abs(g["r"] - o["r"]) <= R_TOL, (msg, g["r"], o["r"])
    if o["r"] - o["second"] > MARGIN:
        assert (g["peak_x"], g["peak_y"]) == (ref["peak_x"], ref["peak_y"]), (msg, g, ref)
        assert (g["peak_x"], g["peak_y"]) == (o["bigx"], o["bigy"]), (msg, g, o)
        for want in (ref, o):
            assert abs(g["dx"] - want["dx"]) <= PX_TOL, (msg, g, want)
            assert abs(g["dy"] - want["dy"]) <= PX_TOL, (msg, g, want)


@pytest.mark.parametrize("name", CASES)
def test_noalloc_matches_corr_patches_and_oracle(prepared, name):
    """Two calls in a row on the same pair give the same numbers (the second
    starts from the scratch the first left behind), and both meet the bar."""
    _, noalloc = _entry()
    c = prepared[name]
    g1 = _call(noalloc, c)
    g2 = _call(noalloc, c)
    for k in ("status", "peak_x", "peak_y", "r", "dx", "dy"):
        assert g1[k] == g2[k], (name, k, g1, g2)
    _check(g1, c, name)


def test_noalloc_consecutive_different_pairs_allocate_nothing(prepared):
    """Every case back to back, then the first again: each call reuses the
    scratch array the previous (different) call left behind, and the
    device's free memory does not move."""
    import torch
    _, noalloc = _entry()
    _call(noalloc, prepared[CASES[0]])   # the one-time set-up happens here at the latest
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for name in CASES + [CASES[0]]:
        _check(_call(noalloc, prepared[name]), prepared[name], name)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, "device memory changed during allocation-free calls"


def test_noalloc_rejects_pairs_beyond_the_scratch():
    import torch
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnResult, ALN_ERR_UNSUPPORTED
    L, noalloc = _entry()
    big = torch.zeros((1024, 1024), dtype=torch.uint8, device="cuda")
    ia, ib = aln.image(big), aln.image(big)
    res = AlnResult()
    rc = noalloc(C.byref(ia), C.byref(ib), 0, 0, 4096, None, None, C.byref(res))
    assert rc == ALN_ERR_UNSUPPORTED
    msg = L.aln_last_error(None).decode()
    assert "scratch" in msg and "aln_corr_patches" in msg, msg


def test_noalloc_rejects_host_inputs():
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300.native import AlnResult, ALN_ERR_ARG
    L, noalloc = _entry()
    a = np.zeros((16, 16), np.uint8)
    ia, ib = aln.image(a), aln.image(a)
    res = AlnResult()
    assert noalloc(C.byref(ia), C.byref(ib), 0, 0, 10, None, None, C.byref(res)) == ALN_ERR_ARG
    # a host pointer flagged as device memory is caught by the pointer check
    ia.on_device = ib.on_device = 1
    assert noalloc(C.byref(ia), C.byref(ib), 0, 0, 10, None, None, C.byref(res)) == ALN_ERR_ARG
    assert "device" in L.aln_last_error(None).decode()
