"""CPU oracle for the tile-matching hot path -- TEST INFRASTRUCTURE ONLY.

Two checkers live here:

* ``Oracle``: ctypes bindings to ``aln_oracle.c``, the project's FP64 C
  restatement of the reference algorithm (CorrPatches, CorrImagesF/R/S,
  CorrPatchToImage, Convolve, the CThmScan sweep).  It builds anywhere gcc
  exists, including the GPU host, and is the CPU baseline ("port").
* ``Ref``: ctypes bindings to ``_ref/libalnref.so``, the reference's own
  unmodified sources compiled by ``ref/Makefile`` with a project FP64 FFT in
  place of FFTW.  It only exists where the reference tree is mounted; it pins
  the restatement and generates tests/golden/.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
use this package, and only as the checker.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libaln_oracle.so")
REF_SO = os.path.join(REF_DIR, "libalnref.so")
TREE_RECORD = os.path.join(REF_DIR, "tree.txt")


def reference_tree() -> str:
    """The reference source tree the reference build uses: $ALN_REFERENCE_TREE,
    else the tree build_ref() last compiled from (recorded beside its
    outputs), else "" (not available)."""
    t = os.environ.get("ALN_REFERENCE_TREE", "")
    if t:
        return t
    try:
        with open(TREE_RECORD) as f:
            return f.read().strip()
    except OSError:
        return ""

RGN_NONE, RGN_MIN, RGN_SECTION, RGN_EXACT, RGN_TABLE = 0, 1, 2, 3, 4
CNT_NONE, CNT_GT = 0, 1


class Legal(C.Structure):
    """Mirror of ``aln_legal`` (include/aln_corr.h)."""

    _fields_ = [
        ("rgn_kind", C.c_int),
        ("rgn_a", C.c_int),
        ("rgn_b", C.c_int),
        ("rgn_area", C.c_longlong),
        ("table", C.c_void_p),
        ("table_w", C.c_int),
        ("table_h", C.c_int),
        ("cnt_kind", C.c_int),
        ("cnt_n", C.c_longlong),
    ]


def legal(rgn=RGN_NONE, a=0, b=0, area=0, cnt=CNT_NONE, n=0) -> Legal:
    return Legal(rgn, a, b, area, None, 0, 0, cnt, n)


class CorrOut(C.Structure):
    _fields_ = [
        ("r", C.c_double),
        ("dx", C.c_double),
        ("dy", C.c_double),
        ("status", C.c_int),
        ("bigx", C.c_int),
        ("bigy", C.c_int),
        ("nx", C.c_int),
        ("ny", C.c_int),
        ("second", C.c_double),
        ("w1", C.c_int),
        ("h1", C.c_int),
        ("w2", C.c_int),
        ("h2", C.c_int),
        ("b1l", C.c_int),
        ("b1b", C.c_int),
        ("b2l", C.c_int),
        ("b2b", C.c_int),
        ("rslt", C.c_void_p),
        ("Rimg", C.c_void_p),
        ("Simg", C.c_void_p),
        ("Aimg", C.c_void_p),
        ("s_mean", C.c_double),
        ("s_sd", C.c_double),
        ("rx", C.c_int),
        ("ry", C.c_int),
    ]


class ThmParams(C.Structure):
    _fields_ = [
        ("rthresh", C.c_double),
        ("nbmaxht", C.c_double),
        ("constxy", C.c_int),
        ("pretweak", C.c_int),
        ("usecorrr", C.c_int),
        ("Ox", C.c_int),
        ("Oy", C.c_int),
        ("Rx", C.c_int),
        ("Ry", C.c_int),
        ("tdfm", C.c_double * 6),
    ]


class ThmRec(C.Structure):
    _fields_ = [("A", C.c_double), ("X", C.c_double), ("Y", C.c_double),
                ("R", C.c_double), ("T", C.c_double * 6), ("pm", C.c_double)]


class ThmMargins(C.Structure):
    """orc_thm_margins: the decision margins of one search (aln_oracle.h)."""
    _fields_ = [("eps", C.c_double), ("eps_px", C.c_double), ("mR", C.c_double),
                ("mpx", C.c_double), ("tolA", C.c_double), ("mpk", C.c_double),
                ("ndec", C.c_int),
                ("nties", C.c_int), ("thr_tie", C.c_int)]


# tie thresholds of the sweep parity bar: a decision whose relative score
# margin exceeds SWEEP_EPS (and whose rounded offsets sit farther than
# SWEEP_EPS_PX from a rounding boundary) is far above the FP32 correlator's
# error (measured |dR|/R ~1e-7), so the GPU must take it the same way
SWEEP_EPS = 1e-5
SWEEP_EPS_PX = 1e-4


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _pts(p):
    p = np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 2)
    return p


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc, seconds)."""
    srcs = [os.path.join(HERE, "aln_oracle.c"), os.path.join(HERE, "fft64.c")]
    hdrs = [os.path.join(HERE, "aln_oracle.h"), os.path.join(HERE, "fft64.h"),
            os.path.join(HERE, "..", "include", "aln_corr.h")]
    if not force and os.path.exists(ORACLE_SO):
        t = os.path.getmtime(ORACLE_SO)
        if all(os.path.getmtime(s) <= t for s in srcs + hdrs):
            return ORACLE_SO
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = ORACLE_SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                           "-o", tmp] + srcs + ["-lm", "-lpthread"])
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(tree: str | None = None) -> str | None:
    """Compile the reference's own sources from `tree` (default:
    reference_tree()); None when no tree is given or it is not mounted."""
    tree = tree or reference_tree()
    if not tree or not os.path.isdir(os.path.join(tree, "0_GEN")):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), "-j8",
                           "REF=" + tree], stdout=subprocess.DEVNULL)
    with open(TREE_RECORD, "w") as f:
        f.write(os.path.abspath(tree) + "\n")
    return REF_SO


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def image_to_points(img: np.ndarray, x0: int = 0, y0: int = 0, keep_zeros=True):
    """Dense raster -> (points, values) as the reference's callers pass tiles:
    every pixel of the box is a point (zero-valued pixels paint nothing but
    still define the bounding box)."""
    h, w = img.shape
    ys, xs = np.mgrid[0:h, 0:w]
    pts = np.stack([xs.ravel() + x0, ys.ravel() + y0], axis=1).astype(np.float64)
    vals = img.astype(np.float64).ravel()
    if not keep_zeros:
        m = vals != 0
        pts, vals = pts[m], vals[m]
    return pts, vals


class _Lib:
    def __init__(self, path):
        self.lib = C.CDLL(path)


def mesh_arrays(am_idx, am_w, ac):
    """Compressed multiplier rows (nm x k indices, -1 unused, and weights)
    and control points (nc x 2) as contiguous arrays."""
    idx = np.ascontiguousarray(am_idx, np.int32)
    wts = np.ascontiguousarray(am_w, np.float64)
    assert idx.shape == wts.shape and idx.ndim == 2
    return idx, wts, np.ascontiguousarray(ac, np.float64).reshape(-1, 2).copy()


class _Mesh:
    """GradDescStep / CorrVectors / ImproveControlPts
    (0_GEN/Correlation.cpp:1403-1721) through the prefix's entry points."""

    _pfx = ""

    def _mesh_types(self):
        for fn in ("corr_vectors", "improve_control_pts"):
            getattr(self.lib, self._pfx + fn).restype = C.c_double

    def grad_desc_step(self, ac, am_idx, am_w, av, bimg):
        idx, wts, ac = mesh_arrays(am_idx, am_w, ac)
        av = np.ascontiguousarray(av, np.float64)
        bimg = np.ascontiguousarray(bimg, np.float64)
        nm, k = idx.shape
        bnew = np.zeros(nm)
        d = np.zeros((len(ac), 2))
        getattr(self.lib, self._pfx + "grad_desc_step")(
            _p(bnew), _p(d), _p(ac), len(ac), _p(idx), _p(wts), k, nm, _p(av), _p(bimg),
            bimg.shape[1], bimg.shape[0])
        return bnew, d

    def corr_vectors(self, a, b):
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        nnz = C.c_int(0)
        r = getattr(self.lib, self._pfx + "corr_vectors")(_p(a), _p(b), len(a), C.byref(nnz))
        return r, nnz.value

    def improve_control_pts(self, ac, am_idx, am_w, av, bimg, ini_thresh, fin_thresh):
        """Returns (corr, optimised control points[, evaluations])."""
        idx, wts, ac = mesh_arrays(am_idx, am_w, ac)
        av = np.ascontiguousarray(av, np.float64)
        bimg = np.ascontiguousarray(bimg, np.float64)
        nm, k = idx.shape
        args = [_p(ac), len(ac), _p(idx), _p(wts), k, nm, _p(av), _p(bimg), bimg.shape[1],
                bimg.shape[0], C.c_double(ini_thresh), C.c_double(fin_thresh)]
        if self._pfx == "orc_":
            it = C.c_int(0)
            r = self.lib.orc_improve_control_pts(*args, C.byref(it))
            return r, ac, it.value
        return self.lib.ref_improve_control_pts(*args), ac


class Oracle(_Lib, _Mesh):
    """The FP64 C restatement (aln_oracle.c)."""

    _pfx = "orc_"

    def __init__(self, path: str | None = None):
        super().__init__(path or build())
        L = self.lib
        for fn in ("orc_corr_patches", "orc_corr_images", "orc_corr_patch_to_image"):
            getattr(L, fn).restype = C.c_double
        L.orc_normalize.restype = C.c_double
        L.orc_linefit_r.restype = C.c_double
        self._mesh_types()

    def corr_patches(self, p1, v1, p2, v2, ox=0, oy=0, radius=4096, lg=None,
                     want_rslt=False):
        p1, p2 = _pts(p1), _pts(p2)
        v1 = np.ascontiguousarray(v1, np.float64)
        v2 = np.ascontiguousarray(v2, np.float64)
        out = CorrOut()
        buf = None
        if want_rslt:
            # sizes are known only after the bbox: compute them here
            from math import floor, ceil
            w1 = int(ceil(p1[:, 0].max())) - int(floor(p1[:, 0].min())) + 1
            h1 = int(ceil(p1[:, 1].max())) - int(floor(p1[:, 1].min())) + 1
            w2 = int(ceil(p2[:, 0].max())) - int(floor(p2[:, 0].min())) + 1
            h2 = int(ceil(p2[:, 1].max())) - int(floor(p2[:, 1].min())) + 1
            nx = self.lib.orc_fft_size(w1, w2)
            ny = self.lib.orc_fft_size(h1, h2)
            buf = np.zeros((ny, nx), np.float64)
            out.rslt = buf.ctypes.data
        self.lib.orc_corr_patches(_p(p1), _p(v1), len(v1), _p(p2), _p(v2), len(v2),
                                  ox, oy, radius, C.byref(lg) if lg else None,
                                  C.byref(out))
        res = {k: getattr(out, k) for k in ("r", "dx", "dy", "status", "bigx", "bigy",
                                             "nx", "ny", "second", "w1", "h1", "w2",
                                             "h2", "b1l", "b1b", "b2l", "b2b")}
        if buf is not None:
            res["rslt"] = buf
        return res

    def corr_images(self, kind, p1, v1, p2, v2, lg=None, mincor=0.0, nbmaxht=0.75,
                    ox=0, oy=0, rx=-1, ry=-1, want_images=False):
        p1, p2 = _pts(p1), _pts(p2)
        v1 = np.ascontiguousarray(v1, np.float64)
        v2 = np.ascontiguousarray(v2, np.float64)
        out = CorrOut()
        bufs = {}
        if want_images:
            from math import floor, ceil
            w1 = int(ceil(p1[:, 0].max())) - int(floor(p1[:, 0].min())) + 1
            h1 = int(ceil(p1[:, 1].max())) - int(floor(p1[:, 1].min())) + 1
            w2 = int(ceil(p2[:, 0].max())) - int(floor(p2[:, 0].min())) + 1
            h2 = int(ceil(p2[:, 1].max())) - int(floor(p2[:, 1].min())) + 1
            shape = (h1 + h2 - 1, w1 + w2 - 1)
            bufs["R"] = np.zeros(shape, np.float64)
            bufs["S"] = np.zeros(shape, np.float64)
            bufs["A"] = np.zeros(shape, np.uint8)
            out.Rimg = bufs["R"].ctypes.data
            out.Simg = bufs["S"].ctypes.data
            out.Aimg = bufs["A"].ctypes.data
        self.lib.orc_corr_images(kind, _p(p1), _p(v1), len(v1), _p(p2), _p(v2), len(v2),
                                 C.byref(lg) if lg else None, C.c_double(mincor),
                                 C.c_double(nbmaxht), ox, oy, rx, ry, C.byref(out))
        res = {k: getattr(out, k) for k in ("r", "dx", "dy", "status", "bigx", "bigy",
                                             "nx", "ny", "second", "s_mean", "s_sd",
                                             "rx", "ry", "w1", "h1", "w2", "h2",
                                             "b1l", "b1b", "b2l", "b2b")}
        res.update(bufs)
        return res

    def corr_patch_to_image(self, p1, v1, img2, ox=0, oy=0, radius=4096, bfilter=False):
        p1 = _pts(p1)
        v1 = np.ascontiguousarray(v1, np.float64)
        i2 = np.ascontiguousarray(img2, np.float64).ravel()
        out = CorrOut()
        self.lib.orc_corr_patch_to_image(_p(p1), _p(v1), len(v1), _p(i2), len(i2),
                                         ox, oy, radius, int(bfilter), C.byref(out))
        return {k: getattr(out, k) for k in ("r", "dx", "dy", "status", "bigx", "bigy")}

    def fft_2d(self, img):
        """Unnormalised r2c of img[ny][nx] -> [ny][nx/2+1] complex128."""
        from ctypes import CDLL  # noqa: F401
        img = np.ascontiguousarray(img, np.float64)
        ny, nx = img.shape
        out = np.zeros((ny, nx // 2 + 1), np.complex128)
        if self.lib.fft64_r2c_2d(ny, nx, _p(img), _p(out)) != 0:
            raise ValueError("size")
        return out

    def ift_2d(self, spec, nx):
        spec = np.ascontiguousarray(spec, np.complex128)
        ny = spec.shape[0]
        out = np.zeros((ny, nx), np.float64)
        if self.lib.fft64_c2r_2d(ny, nx, _p(spec), _p(out)) != 0:
            raise ValueError("size")
        return out

    def convolve(self, src, K, sym=True, prenorm=True):
        src = np.ascontiguousarray(src, np.float64)
        K = np.ascontiguousarray(K, np.float64)
        hs, ws = src.shape
        hk, wk = K.shape
        dst = np.zeros_like(src)
        self.lib.orc_convolve(_p(dst), _p(src), ws, hs, _p(K), wk, hk, int(sym),
                              int(prenorm))
        return dst

    def image_from_points(self, pts, vals, xmin, ymin, w, h):
        """ImageFromValuesAndPoints + DistributePixel (h x w FP64 raster)."""
        xy = _pts(pts)
        v = np.ascontiguousarray(vals, np.float64)
        img = np.zeros((h, w), np.float64)
        self.lib.orc_image_from_points(_p(img), w, h, _p(v), _p(xy), len(v), xmin, ymin)
        return img

    def decimate_normalize(self, pts, vals, w, h, lbin, normalize=True):
        xy = _pts(pts).copy()
        v = np.ascontiguousarray(vals, np.float64).copy()
        k = self.lib.orc_decimate(_p(xy), _p(v), len(v), w, h, lbin)
        xy, v = xy[:k].copy(), v[:k].copy()
        if normalize:
            self.lib.orc_normalize(_p(v), len(v))
        return xy, v

    def thm_search(self, pa, va, pb, vb, req_area, olap1d=0, rthresh=0.3,
                   nbmaxht=0.75, pretweak=0, constxy=1, usecorrr=1, disc=(0, 0, -1, -1),
                   mode=0, ang0=0.0, hfang=10.0, step=0.5, tdfm=None):
        pa, pb = _pts(pa), _pts(pb)
        va = np.ascontiguousarray(va, np.float64)
        vb = np.ascontiguousarray(vb, np.float64)
        P = ThmParams()
        P.rthresh, P.nbmaxht = rthresh, nbmaxht
        P.constxy, P.pretweak, P.usecorrr = constxy, pretweak, usecorrr
        P.Ox, P.Oy, P.Rx, P.Ry = disc
        t = tdfm if tdfm is not None else (1, 0, 0, 0, 1, 0)
        for i in range(6):
            P.tdfm[i] = t[i]
        best = ThmRec()
        ncalls = C.c_int(0)
        M = ThmMargins()
        M.eps, M.eps_px = SWEEP_EPS, SWEEP_EPS_PX
        err = self.lib.orc_thm_search_m(_p(pa), _p(va), len(va), _p(pb), _p(vb), len(vb),
                                        C.c_long(req_area), olap1d, C.byref(P), mode,
                                        C.c_double(ang0), C.c_double(hfang),
                                        C.c_double(step), C.byref(best), C.byref(ncalls),
                                        C.byref(M))
        return {"A": best.A, "X": best.X, "Y": best.Y, "R": best.R, "err": err,
                "ncalls": ncalls.value,
                "margins": {"mR": M.mR, "mpx": M.mpx, "tolA": M.tolA, "mpk": M.mpk,
                            "ndec": M.ndec,
                            "nties": M.nties, "thr_tie": bool(M.thr_tie)}}

    def thm_finish(self, pa, va, pb, vb, req_area, mode, prior, tptwk=None, olap1d=0,
                   rthresh=0.3, nbmaxht=0.75, pretweak=0, constxy=1, tdfm=None):
        """PostTweaks (mode 5) / FinishAtFullRes (mode 6) from prior (A, X, Y, R)."""
        pa, pb = _pts(pa), _pts(pb)
        va = np.ascontiguousarray(va, np.float64)
        vb = np.ascontiguousarray(vb, np.float64)
        P = ThmParams()
        P.rthresh, P.nbmaxht = rthresh, nbmaxht
        P.constxy, P.pretweak, P.usecorrr = constxy, pretweak, 1
        P.Ox, P.Oy, P.Rx, P.Ry = 0, 0, -1, -1
        t = tdfm if tdfm is not None else (1, 0, 0, 0, 1, 0)
        for i in range(6):
            P.tdfm[i] = t[i]
        pr = np.ascontiguousarray(prior, np.float64)
        tw = None if tptwk is None else np.ascontiguousarray(tptwk, np.float64)
        tout = np.zeros(6, np.float64)
        best = ThmRec()
        ncalls = C.c_int(0)
        err = self.lib.orc_thm_finish(_p(pa), _p(va), len(va), _p(pb), _p(vb), len(vb),
                                      C.c_long(req_area), olap1d, C.byref(P), mode, _p(pr),
                                      _p(tw) if tw is not None else None, C.byref(best),
                                      _p(tout), C.byref(ncalls))
        return {"A": best.A, "X": best.X, "Y": best.Y, "R": best.R, "err": err,
                "ncalls": ncalls.value, "tptwk": tout.tolist()}


APPROX_STATUS = {0: "ok", 1: "crop", 2: "thumbs", 3: "sweep", 4: "limxy"}


def approx_defaults(**kw):
    """ApproximateMatch settings (1_DMesh/ApproximateMatch.cpp:120-154 with
    matchparams-style values) as a dict the Ref and the library take."""
    d = dict(xyconf=0.75, olap1d=0, olap2d=40000, thmdec=4, mode_prior=0, ang0=0.0,
             hfangdn=10.0, hfangpr=1.0, rthresh=0.3, nbmaxht=0.75, pretweak=0, tweaks=0,
             limxy=0)
    d.update(kw)
    return d


class Ref(_Lib, _Mesh):
    """The reference's own code (compiled from its sources; x86 host only)."""

    _pfx = "ref_"

    def __init__(self, path: str | None = None):
        super().__init__(path or REF_SO)
        L = self.lib
        for fn in ("ref_corr_patches", "ref_corr_images", "ref_corr_patch_to_image"):
            getattr(L, fn).restype = C.c_double
        self._mesh_types()

    def pixpair_condition(self, tile, order=2, r1=0, r2=0, max1dpix=0):
        """PixPair::Load's conditioning of a uint8 tile through the
        reference's functions (refwrap's ref_pixpair_condition)."""
        t = np.ascontiguousarray(tile, np.uint8)
        h, w = t.shape
        ws, hs, scl = w, h, 1
        while max1dpix > 0 and (ws > max1dpix or hs > max1dpix):
            ws, hs, scl = ws // 2, hs // 2, scl * 2
        vfy = np.zeros((hs, ws))
        aln = np.zeros((hs, ws))
        self.lib.ref_pixpair_condition(_p(t), w, h, order, r1, r2, ws, hs, scl, _p(vfy), _p(aln))
        return vfy, aln, scl

    def approx_match(self, a, b, tab, **params):
        """The reference's ApproximateMatch sequence on two whole tiles
        (refwrap's ref_approx_match).  Returns a dict with status, A, X, Y,
        R, T, err, sweep (A, X, Y, R), crop (aO, bO, w, h)."""
        p = approx_defaults(**params)
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        out = np.zeros(21)
        st = self.lib.ref_approx_match(
            _p(a), _p(b), a.shape[1], a.shape[0], C.c_double(tab[0]), C.c_double(tab[1]),
            C.c_double(p["xyconf"]), p["olap1d"], C.c_long(p["olap2d"]), p["thmdec"],
            p["mode_prior"], C.c_double(p["ang0"]), C.c_double(p["hfangdn"]),
            C.c_double(p["hfangpr"]), C.c_double(p["rthresh"]), C.c_double(p["nbmaxht"]),
            p["pretweak"], p["tweaks"], p["limxy"], _p(out))
        return {"status": st, "A": out[0], "X": out[1], "Y": out[2], "R": out[3],
                "T": out[4:10].tolist(), "err": int(out[10]), "sweep": out[11:15].tolist(),
                "crop": [int(v) for v in out[15:21]]}

    def corr_patches(self, p1, v1, p2, v2, ox=0, oy=0, radius=4096, lg=None):
        p1, p2 = _pts(p1), _pts(p2)
        v1 = np.ascontiguousarray(v1, np.float64)
        v2 = np.ascontiguousarray(v2, np.float64)
        dx, dy = C.c_double(0), C.c_double(0)
        r = self.lib.ref_corr_patches(len(v1), _p(p1), _p(v1), len(v2), _p(p2), _p(v2),
                                      ox, oy, radius, C.byref(lg) if lg else None,
                                      C.byref(dx), C.byref(dy))
        return {"r": r, "dx": dx.value, "dy": dy.value}

    def corr_images(self, kind, p1, v1, p2, v2, lg=None, mincor=0.0, nbmaxht=0.75,
                    ox=0, oy=0, rx=-1, ry=-1):
        p1, p2 = _pts(p1), _pts(p2)
        v1 = np.ascontiguousarray(v1, np.float64)
        v2 = np.ascontiguousarray(v2, np.float64)
        dx, dy = C.c_double(0), C.c_double(0)
        r = self.lib.ref_corr_images(kind, len(v1), _p(p1), _p(v1), len(v2), _p(p2),
                                     _p(v2), C.byref(lg) if lg else None,
                                     C.c_double(mincor), C.c_double(nbmaxht), ox, oy,
                                     rx, ry, C.byref(dx), C.byref(dy))
        return {"r": r, "dx": dx.value, "dy": dy.value}

    def corr_patch_to_image(self, p1, v1, img2, ox=0, oy=0, radius=4096, bfilter=False):
        p1 = _pts(p1)
        v1 = np.ascontiguousarray(v1, np.float64)
        i2 = np.ascontiguousarray(img2, np.float64).ravel()
        dx, dy = C.c_double(0), C.c_double(0)
        r = self.lib.ref_corr_patch_to_image(len(v1), _p(p1), _p(v1), len(i2), _p(i2),
                                             ox, oy, radius, int(bfilter), C.byref(dx),
                                             C.byref(dy))
        return {"r": r, "dx": dx.value, "dy": dy.value}

    def fft_2d(self, img):
        img = np.ascontiguousarray(img, np.float64)
        ny, nx = img.shape
        out = np.zeros((ny, nx // 2 + 1), np.complex128)
        self.lib.ref_fft_2d(_p(img), nx, ny, _p(out))
        return out

    def ift_2d(self, spec, nx):
        spec = np.ascontiguousarray(spec, np.complex128)
        ny = spec.shape[0]
        out = np.zeros((ny, nx), np.float64)
        self.lib.ref_ift_2d(_p(spec), nx, ny, _p(out))
        return out

    def convolve(self, src, K, sym=True, prenorm=True):
        src = np.ascontiguousarray(src, np.float64)
        K = np.ascontiguousarray(K, np.float64)
        hs, ws = src.shape
        hk, wk = K.shape
        dst = np.zeros_like(src)
        self.lib.ref_convolve(_p(dst), _p(src), ws, hs, _p(K), wk, hk, int(sym),
                              int(prenorm))
        return dst

    def decimate_normalize(self, pts, vals, w, h, lbin, normalize=True):
        xy = _pts(pts).copy()
        v = np.ascontiguousarray(vals, np.float64).copy()
        k = self.lib.ref_decimate_normalize(len(v), _p(xy), _p(v), w, h, lbin,
                                            int(normalize))
        return xy[:k].copy(), v[:k].copy()

    def thm_search(self, pa, va, pb, vb, req_area, olap1d=0, rthresh=0.3,
                   nbmaxht=0.75, pretweak=0, constxy=1, usecorrr=1, disc=(0, 0, -1, -1),
                   mode=0, ang0=0.0, hfang=10.0, step=0.5, tdfm=None, logpath=None):
        pa, pb = _pts(pa), _pts(pb)
        va = np.ascontiguousarray(va, np.float64)
        vb = np.ascontiguousarray(vb, np.float64)
        out = np.zeros(4, np.float64)
        td = None
        if tdfm is not None:
            td = np.ascontiguousarray(tdfm, np.float64)
        err = self.lib.ref_thm_search(
            len(va), _p(pa), _p(va), len(vb), _p(pb), _p(vb), C.c_long(req_area),
            olap1d, C.c_double(rthresh), C.c_double(nbmaxht), pretweak, constxy,
            usecorrr, disc[0], disc[1], disc[2], disc[3], mode, C.c_double(ang0),
            C.c_double(hfang), C.c_double(step), _p(td) if td is not None else None,
            _p(out), logpath.encode() if logpath else None)
        return {"A": out[0], "X": out[1], "Y": out[2], "R": out[3], "err": err}

    def thm_finish(self, pa, va, pb, vb, req_area, mode, prior, tptwk=None, olap1d=0,
                   rthresh=0.3, nbmaxht=0.75, pretweak=0, constxy=1, tdfm=None):
        pa, pb = _pts(pa), _pts(pb)
        va = np.ascontiguousarray(va, np.float64)
        vb = np.ascontiguousarray(vb, np.float64)
        pr = np.ascontiguousarray(prior, np.float64)
        tw = None if tptwk is None else np.ascontiguousarray(tptwk, np.float64)
        td = None if tdfm is None else np.ascontiguousarray(tdfm, np.float64)
        out = np.zeros(10, np.float64)
        err = self.lib.ref_thm_finish(
            len(va), _p(pa), _p(va), len(vb), _p(pb), _p(vb), C.c_long(req_area), olap1d,
            C.c_double(rthresh), C.c_double(nbmaxht), pretweak, constxy, 1, mode, _p(pr),
            _p(tw) if tw is not None else None, _p(td) if td is not None else None, _p(out))
        return {"A": out[0], "X": out[1], "Y": out[2], "R": out[3], "err": err,
                "tptwk": out[4:10].tolist()}
