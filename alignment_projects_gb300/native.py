"""ctypes bindings of the C ABI (include/aln_corr.h) of libaln_corr.so.

The library is the product: every call here goes to the CUDA kernels.  There
is no CPU fallback -- if the shared library is missing or no GPU is present,
loading or creating a context raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

ALN_OK, ALN_NO_PEAK = 0, 1
ALN_ERR_ARG, ALN_ERR_CUDA, ALN_ERR_NOMEM, ALN_ERR_UNSUPPORTED = -1, -2, -3, -4
ALN_ERR_TIMEOUT, ALN_ERR_REFUSED, ALN_ERR_CANCELLED = -5, -6, -7
U8, U16, F32, F64 = 0, 1, 2, 3
RGN_NONE, RGN_MIN, RGN_SECTION, RGN_EXACT, RGN_TABLE = 0, 1, 2, 3, 4
CNT_NONE, CNT_GT = 0, 1

_DTYPES = {np.dtype(np.uint8): U8, np.dtype(np.uint16): U16,
           np.dtype(np.float32): F32, np.dtype(np.float64): F64}
_TORCH_DTYPES = {"torch.uint8": U8, "torch.uint16": U16, "torch.float32": F32,
                 "torch.float64": F64}


class AlnImage(C.Structure):
    _fields_ = [("data", C.c_void_p), ("dtype", C.c_int), ("w", C.c_int), ("h", C.c_int),
                ("stride", C.c_int), ("x0", C.c_int), ("y0", C.c_int),
                ("on_device", C.c_int)]


class AlnLegal(C.Structure):
    _fields_ = [("rgn_kind", C.c_int), ("rgn_a", C.c_int), ("rgn_b", C.c_int),
                ("rgn_area", C.c_longlong), ("table", C.c_void_p), ("table_w", C.c_int),
                ("table_h", C.c_int), ("cnt_kind", C.c_int), ("cnt_n", C.c_longlong)]


class AlnResult(C.Structure):
    _fields_ = [("r", C.c_double), ("dx", C.c_double), ("dy", C.c_double),
                ("status", C.c_int), ("peak_x", C.c_int), ("peak_y", C.c_int),
                ("nx", C.c_int), ("ny", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AlnImageJob(C.Structure):
    _fields_ = [("a", AlnImage), ("b", AlnImage), ("kind", C.c_int), ("legal", AlnLegal),
                ("mincor", C.c_double), ("nbmaxht", C.c_double), ("ox", C.c_int),
                ("oy", C.c_int), ("rx", C.c_int), ("ry", C.c_int), ("b_key", C.c_ulonglong)]


CORR_F, CORR_R, CORR_S = 0, 1, 2
THM_DENOVO, THM_RFROMANGLE, THM_PRIOR, THM_SCAN_HUNT, THM_SCAN_MAXR = 0, 1, 2, 3, 4
THM_POSTTWEAKS, THM_FULLRES = 5, 6


class AlnThumbs(C.Structure):
    _fields_ = [("a", C.c_void_p), ("a_mask", C.c_void_p), ("a_w", C.c_int), ("a_h", C.c_int),
                ("a_stride", C.c_int), ("a_x0", C.c_int), ("a_y0", C.c_int), ("b", AlnImage),
                ("req_area", C.c_longlong), ("olap1d", C.c_int), ("b_key", C.c_ulonglong)]


DISC_OF_ANGLE = C.CFUNCTYPE(None, C.c_void_p, C.c_double, C.POINTER(C.c_int),
                            C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int))


class AlnThmParams(C.Structure):
    _fields_ = [("rthresh", C.c_double), ("nbmaxht", C.c_double), ("constxy", C.c_int),
                ("pretweak", C.c_int), ("usecorrr", C.c_int), ("ox", C.c_int), ("oy", C.c_int),
                ("rx", C.c_int), ("ry", C.c_int), ("tdfm", C.c_double * 6),
                ("disc_of_angle", DISC_OF_ANGLE), ("disc_user", C.c_void_p)]


class AlnThmResult(C.Structure):
    _fields_ = [("A", C.c_double), ("X", C.c_double), ("Y", C.c_double), ("R", C.c_double),
                ("T", C.c_double * 6), ("err", C.c_int), ("ncalls", C.c_int)]


class AlnTilePair(C.Structure):
    _fields_ = [("a", AlnImage), ("b", AlnImage), ("tabx", C.c_double), ("taby", C.c_double)]


class AlnApproxParams(C.Structure):
    _fields_ = [("xyconf", C.c_double), ("olap1d", C.c_int), ("olap2d", C.c_longlong),
                ("thmdec", C.c_int), ("mode_prior", C.c_int), ("ang0", C.c_double),
                ("hfangdn", C.c_double), ("hfangpr", C.c_double), ("rthresh", C.c_double),
                ("nbmaxht", C.c_double), ("pretweak", C.c_int), ("tweaks", C.c_int),
                ("limxy", C.c_int)]


class AlnApproxResult(C.Structure):
    _fields_ = [("status", C.c_int), ("err", C.c_int), ("A", C.c_double), ("X", C.c_double),
                ("Y", C.c_double), ("R", C.c_double), ("T", C.c_double * 6),
                ("sweep", C.c_double * 4), ("crop", C.c_int * 4), ("crop_w", C.c_int),
                ("crop_h", C.c_int)]


class AlnThmPair(C.Structure):
    _fields_ = [("atl", C.c_int), ("acr", C.c_int), ("btl", C.c_int), ("bcr", C.c_int),
                ("err", C.c_int), ("A", C.c_double), ("R", C.c_double), ("T", C.c_double * 6)]


def thmpair_write(dir_, alr, blr, recs):
    """Append ThmPair entries (dicts atl, acr, btl, bcr, err, A, R, T) to
    <dir>/ThmPair_<alr>^<blr>.txt (0_GEN/PipeFiles.cpp's format)."""
    n = len(recs)
    arr = (AlnThmPair * n)()
    for k, r in enumerate(recs):
        arr[k] = AlnThmPair(r["atl"], r["acr"], r["btl"], r["bcr"], r.get("err", 0), r["A"],
                            r["R"], (C.c_double * 6)(*r["T"]))
    rc = lib().aln_thmpair_write(dir_.encode(), alr, blr, n, arr)
    if rc < 0:
        raise AlnError(rc, lib().aln_last_error(None).decode())


def thmpair_read(dir_, alr, blr) -> list:
    """The table's entries as dicts (ReadAllThmPair)."""
    L = lib()
    n = L.aln_thmpair_read(dir_.encode(), alr, blr, 0, None)
    if n < 0:
        raise AlnError(n, L.aln_last_error(None).decode())
    arr = (AlnThmPair * max(n, 1))()
    L.aln_thmpair_read(dir_.encode(), alr, blr, n, arr)
    return [{"atl": r.atl, "acr": r.acr, "btl": r.btl, "bcr": r.bcr, "err": r.err, "A": r.A,
             "R": r.R, "T": list(r.T)} for r in arr[:n]]


class AlnMeshJob(C.Structure):
    _fields_ = [("nc", C.c_int), ("ac", C.c_void_p), ("nm", C.c_int), ("k", C.c_int),
                ("am_idx", C.c_void_p), ("am_w", C.c_void_p), ("av", C.c_void_p),
                ("bimg", C.c_void_p), ("w", C.c_int), ("h", C.c_int),
                ("ini_thresh", C.c_double), ("fin_thresh", C.c_double), ("on_device", C.c_int)]


class AlnMeshResult(C.Structure):
    _fields_ = [("status", C.c_int), ("corr", C.c_double), ("corr0", C.c_double),
                ("evals", C.c_int)]


def mesh_job(ac, am_idx, am_w, av, bimg, ini_thresh=0.0, fin_thresh=0.0):
    """An aln_mesh_job over host arrays (kept alive on the struct): ac nc x 2,
    am_idx / am_w nm x k (indices ascending per row, -1 unused), av nm,
    bimg h x w.  ac is copied; the optimised points land in job._ac."""
    acs = np.ascontiguousarray(ac, np.float64).reshape(-1, 2).copy()
    idx = np.ascontiguousarray(am_idx, np.int32)
    wts = np.ascontiguousarray(am_w, np.float64)
    avs = np.ascontiguousarray(av, np.float64)
    bim = np.ascontiguousarray(bimg, np.float64)
    assert idx.shape == wts.shape and idx.ndim == 2 and len(avs) == idx.shape[0]
    J = AlnMeshJob(len(acs), acs.ctypes.data, idx.shape[0], idx.shape[1], idx.ctypes.data,
                   wts.ctypes.data, avs.ctypes.data, bim.ctypes.data, bim.shape[1], bim.shape[0],
                   ini_thresh, fin_thresh, 0)
    J._ac = acs
    J._keep = (idx, wts, avs, bim)
    return J


def thumbs_from_points(pa, va, pb, vb, req_area, olap1d=0):
    """Point lists with integer coordinates (a ThmRec) -> AlnThumbs.  A
    becomes a grid with a presence mask; B a raster over its bounding box."""
    pa = np.asarray(pa, np.float64).reshape(-1, 2)
    pb = np.asarray(pb, np.float64).reshape(-1, 2)
    assert np.all(pa == np.round(pa)) and np.all(pb == np.round(pb))
    ax, ay = pa[:, 0].astype(np.int64), pa[:, 1].astype(np.int64)
    ax0, ay0 = int(ax.min()), int(ay.min())
    aw, ah = int(ax.max()) - ax0 + 1, int(ay.max()) - ay0 + 1
    agrid = np.zeros((ah, aw), np.float64)
    amask = np.zeros((ah, aw), np.uint8)
    agrid[ay - ay0, ax - ax0] = np.asarray(va, np.float64)
    amask[ay - ay0, ax - ax0] = 1
    bx, by = pb[:, 0].astype(np.int64), pb[:, 1].astype(np.int64)
    bx0, by0 = int(bx.min()), int(by.min())
    bw, bh = int(bx.max()) - bx0 + 1, int(by.max()) - by0 + 1
    braster = np.zeros((bh, bw), np.float64)
    np.add.at(braster, (by - by0, bx - bx0), np.asarray(vb, np.float64))
    T = AlnThumbs()
    T.a = agrid.ctypes.data
    T.a_mask = None if amask.all() else amask.ctypes.data
    T.a_w, T.a_h, T.a_stride, T.a_x0, T.a_y0 = aw, ah, aw, ax0, ay0
    T.b = image(braster, bx0, by0)
    T.req_area, T.olap1d = req_area, olap1d
    T._keep = (agrid, amask, braster)
    return T


class AlnPair(C.Structure):
    _fields_ = [("a", AlnImage), ("b", AlnImage), ("ox", C.c_int), ("oy", C.c_int),
                ("radius", C.c_int), ("legal", AlnLegal), ("b_key", C.c_ulonglong)]


class AlnServerParams(C.Structure):
    _fields_ = [("device", C.c_int), ("workers", C.c_int), ("mem_budget", C.c_size_t),
                ("max_batch", C.c_int), ("cache_bytes", C.c_size_t)]


REQ_PATCHES, REQ_IMAGES, REQ_SWEEP = 0, 1, 2


class AlnRequest(C.Structure):
    _fields_ = [("kind", C.c_int), ("pair", AlnPair), ("job", AlnImageJob),
                ("thumbs", AlnThumbs), ("thm", AlnThmParams), ("thm_mode", C.c_int),
                ("ang0", C.c_double), ("hfang", C.c_double), ("step", C.c_double)]


class AlnReply(C.Structure):
    _fields_ = [("status", C.c_int), ("corr", AlnResult), ("sweep", AlnThmResult),
                ("queue_ms", C.c_double), ("total_ms", C.c_double), ("batch_size", C.c_int)]


_lib = None


def lib():
    """Load libaln_corr.so (building it first when sources are newer)."""
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        L.aln_ctx_create.argtypes = [C.c_int, C.POINTER(C.c_void_p)]
        L.aln_ctx_destroy.argtypes = [C.c_void_p]
        L.aln_last_error.restype = C.c_char_p
        L.aln_last_error.argtypes = [C.c_void_p]
        L.aln_corr_patches.argtypes = [C.c_void_p, C.POINTER(AlnImage), C.POINTER(AlnImage),
                                       C.c_int, C.c_int, C.c_int, C.POINTER(AlnLegal),
                                       C.POINTER(AlnResult)]
        L.aln_corr_patches_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnPair),
                                             C.POINTER(AlnResult)]
        L.aln_corr_images.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnImage),
                                      C.POINTER(AlnImage), C.POINTER(AlnLegal), C.c_double,
                                      C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.POINTER(AlnResult)]
        L.aln_corr_images_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnImageJob),
                                            C.POINTER(AlnResult)]
        L.aln_thm_search_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnThumbs),
                                           C.POINTER(AlnThmParams), C.c_int, C.c_double,
                                           C.c_double, C.c_double, C.POINTER(AlnThmResult)]
        L.aln_thm_finish_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnThumbs),
                                           C.POINTER(AlnThmParams), C.c_int,
                                           C.POINTER(AlnThmResult), C.c_void_p,
                                           C.POINTER(AlnThmResult), C.c_void_p]
        L.aln_corr_patch_to_image.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                              C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                              C.c_int, C.POINTER(AlnResult)]
        L.aln_fft_2d.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.aln_convolve.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                   C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
        L.aln_ift_2d.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        L.aln_ctx_set_profiling.argtypes = [C.c_void_p, C.c_int]
        L.aln_ctx_profile_reset.argtypes = [C.c_void_p]
        L.aln_ctx_profile.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_char_p),
                                      C.POINTER(C.c_longlong), C.POINTER(C.c_double)]
        L.aln_ctx_counter.argtypes = [C.c_void_p, C.c_int]
        L.aln_ctx_counter.restype = C.c_longlong
        L.aln_ctx_set_workspace_limit.argtypes = [C.c_void_p, C.c_size_t]
        L.aln_ctx_set_spectrum_cache.argtypes = [C.c_void_p, C.c_size_t]
        L.aln_parab_peak_fft.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                         C.c_void_p, C.c_int, C.c_int]
        L.aln_thm_call_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnThumbs),
                                         C.POINTER(AlnThmParams), C.c_int, C.c_void_p,
                                         C.POINTER(AlnThmResult), C.c_void_p, C.c_void_p]
        L.aln_decimate_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnImage),
                                         C.POINTER(C.c_void_p), C.c_int, C.c_int,
                                         C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                         C.c_void_p]
        L.aln_corr_patches_grid.argtypes = [C.POINTER(AlnPair), C.POINTER(C.c_int),
                                            C.POINTER(C.c_int), C.POINTER(C.c_int),
                                            C.POINTER(C.c_int)]
        L.aln_ctx_set_segmenting.argtypes = [C.c_void_p, C.c_int]
        L.aln_ctx_set_tuning.argtypes = [C.c_void_p, C.c_int]
        L.aln_ctx_set_split_grids.argtypes = [C.c_void_p, C.c_int]
        L.aln_approx_match_batch.argtypes = [C.c_void_p, C.c_int, C.POINTER(AlnTilePair),
                                             C.POINTER(AlnApproxParams),
                                             C.POINTER(AlnApproxResult)]
        L.aln_points_image.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                       C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(AlnImage), C.c_void_p]
        L.aln_thmpair_write.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(AlnThmPair)]
        L.aln_thmpair_read.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int,
                                       C.POINTER(AlnThmPair)]
        L.aln_pixpair_dims.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.POINTER(C.c_int)]
        L.aln_pixpair_condition.argtypes = [C.c_void_p, C.POINTER(AlnImage), C.c_int, C.c_int,
                                            C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.aln_improve_control_pts_batch.argtypes = [C.c_void_p, C.c_int,
                                                    C.POINTER(AlnMeshJob),
                                                    C.POINTER(AlnMeshResult)]
        L.aln_grad_desc_step.argtypes = [C.c_void_p, C.POINTER(AlnMeshJob), C.c_void_p,
                                         C.c_void_p, C.POINTER(C.c_double)]
        L.aln_corr_vectors.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.aln_server_create.argtypes = [C.POINTER(AlnServerParams), C.POINTER(C.c_void_p)]
        L.aln_server_destroy.argtypes = [C.c_void_p]
        L.aln_server_submit.argtypes = [C.c_void_p, C.POINTER(AlnRequest),
                                        C.POINTER(C.c_ulonglong)]
        L.aln_server_wait.argtypes = [C.c_void_p, C.c_ulonglong, C.c_int, C.POINTER(AlnReply)]
        L.aln_server_collect.argtypes = [C.c_void_p, C.c_int, C.c_int,
                                         C.POINTER(C.c_ulonglong), C.POINTER(AlnReply)]
        L.aln_server_counter.argtypes = [C.c_void_p, C.c_int]
        L.aln_server_counter.restype = C.c_longlong
        L.aln_server_last_error.argtypes = [C.c_void_p]
        L.aln_server_last_error.restype = C.c_char_p
        _lib = L
    return _lib


def lib_path() -> str:
    return _build.LIB


class AlnError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"aln error {code}: {msg}")
        self.code = code


def legal(rgn=RGN_NONE, a=0, b=0, area=0, cnt=CNT_NONE, n=0, table=None) -> AlnLegal:
    """Typed LegalRgn / LegalCnt (see aln_legal in include/aln_corr.h)."""
    L = AlnLegal(rgn, a, b, area, None, 0, 0, cnt, n)
    if table is not None:
        t = np.ascontiguousarray(table, dtype=np.uint8)
        L.rgn_kind = RGN_TABLE
        L.table = t.ctypes.data
        L.table_h, L.table_w = t.shape
        L._keep = t  # keep the buffer alive with the struct
    return L


def image(arr, x0: int = 0, y0: int = 0) -> AlnImage:
    """Describe a 2D raster (numpy array on the host, or a CUDA torch tensor)."""
    if hasattr(arr, "data_ptr"):  # torch tensor
        assert arr.dim() == 2 and arr.stride(1) == 1
        dt = _TORCH_DTYPES[str(arr.dtype)]
        im = AlnImage(arr.data_ptr(), dt, arr.shape[1], arr.shape[0], arr.stride(0), x0, y0,
                      1 if arr.is_cuda else 0)
        im._keep = arr
        return im
    a = np.asarray(arr)
    if a.dtype not in _DTYPES:
        a = a.astype(np.float64)
    if a.strides[1] != a.itemsize:
        a = np.ascontiguousarray(a)
    im = AlnImage(a.ctypes.data, _DTYPES[a.dtype], a.shape[1], a.shape[0],
                  a.strides[0] // a.itemsize, x0, y0, 0)
    im._keep = a
    return im


class Context:
    """One aln_ctx: a CUDA stream plus workspaces on one device."""

    def __init__(self, device: int = 0):
        self._L = lib()
        h = C.c_void_p()
        rc = self._L.aln_ctx_create(device, C.byref(h))
        if rc != ALN_OK:
            raise AlnError(rc, self._L.aln_last_error(None).decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self._L.aln_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc < 0:
            raise AlnError(rc, self._L.aln_last_error(self.h).decode())
        return rc

    # -- tracing ----------------------------------------------------------
    def set_profiling(self, on: bool):
        self._L.aln_ctx_set_profiling(self.h, int(on))

    def profile_reset(self):
        self._L.aln_ctx_profile_reset(self.h)

    def profile(self) -> dict:
        """{kernel: (launches, total_ms)} since the last reset."""
        cap = 64
        names = (C.c_char_p * cap)()
        launches = (C.c_longlong * cap)()
        ms = (C.c_double * cap)()
        n = self._L.aln_ctx_profile(self.h, cap, names, launches, ms)
        return {names[i].decode(): (launches[i], ms[i]) for i in range(min(n, cap))}

    def counters(self) -> dict:
        return {"launches": self._L.aln_ctx_counter(self.h, 0),
                "h2d_bytes": self._L.aln_ctx_counter(self.h, 1),
                "d2h_bytes": self._L.aln_ctx_counter(self.h, 2),
                "spec_hits": self._L.aln_ctx_counter(self.h, 3),
                "spec_fills": self._L.aln_ctx_counter(self.h, 4),
                "spec_bytes": self._L.aln_ctx_counter(self.h, 5),
                "chunks": self._L.aln_ctx_counter(self.h, 6),
                "h2d_copies": self._L.aln_ctx_counter(self.h, 7),
                "tune_classes": self._L.aln_ctx_counter(self.h, 8),
                "spec_evictions": self._L.aln_ctx_counter(self.h, 9),
                "host_plan_us": self._L.aln_ctx_counter(self.h, 10),
                "host_prep_us": self._L.aln_ctx_counter(self.h, 11)}

    def set_segmenting(self, ns: int):
        """CorrPatches column segments: 0 the class's measured plan (or the
        cost model with tuning off), -1 off, or a forced segment transform
        length (power of two, 64..2048)."""
        self._check(self._L.aln_ctx_set_segmenting(self.h, ns))

    def set_tuning(self, on: bool):
        """Measured column plans per pair class (the autotuner) or the fixed
        cost model."""
        self._check(self._L.aln_ctx_set_tuning(self.h, int(bool(on))))

    def set_split_grids(self, on: bool):
        """CorrPatches rows of 3 * 2^k and 5 * 2^k points where shorter than
        the power of two (default on), or powers of two only."""
        self._check(self._L.aln_ctx_set_split_grids(self.h, int(bool(on))))

    def set_spectrum_cache(self, nbytes: int):
        self._check(self._L.aln_ctx_set_spectrum_cache(self.h, nbytes))

    def set_workspace_limit(self, nbytes: int):
        self._check(self._L.aln_ctx_set_workspace_limit(self.h, nbytes))

    # -- Convolve (Correlation.h) -------------------------------------------
    def convolve(self, src, K, sym=True, prenorm=True) -> np.ndarray:
        src = np.ascontiguousarray(src, np.float64)
        K = np.ascontiguousarray(K, np.float64)
        dst = np.zeros_like(src)
        hs, ws = src.shape
        hk, wk = K.shape
        self._check(self._L.aln_convolve(self.h, src.ctypes.data, ws, hs, K.ctypes.data, wk,
                                         hk, int(sym), int(prenorm), dst.ctypes.data))
        return dst

    # -- FFT support (Correlation.h FFT_2D / IFT_2D) -----------------------
    def fft_2d(self, x):
        x = np.ascontiguousarray(x, np.float64)
        ny, nx = x.shape
        out = np.zeros((ny, nx // 2 + 1), np.complex128)
        self._check(self._L.aln_fft_2d(self.h, x.ctypes.data, nx, ny, out.ctypes.data))
        return out

    def ift_2d(self, spec, nfast):
        spec = np.ascontiguousarray(spec, np.complex128)
        ny = spec.shape[0]
        out = np.zeros((ny, nfast), np.float64)
        self._check(self._L.aln_ift_2d(self.h, spec.ctypes.data, nfast, ny, out.ctypes.data))
        return out

    # -- CorrPatches ----------------------------------------------------------
    def corr_patches(self, a, b, ox=0, oy=0, radius=4096, lg=None, a_origin=(0, 0),
                     b_origin=(0, 0)) -> dict:
        ia = image(a, *a_origin)
        ib = image(b, *b_origin)
        res = AlnResult()
        self._check(self._L.aln_corr_patches(self.h, C.byref(ia), C.byref(ib), ox, oy, radius,
                                             C.byref(lg) if lg is not None else None,
                                             C.byref(res)))
        return res.as_dict()

    # -- CorrPatchToImage -----------------------------------------------------
    def corr_patch_to_image(self, pts, vals, img2, ox=0, oy=0, radius=4096,
                            bfilter=False) -> dict:
        xy = np.ascontiguousarray(pts, np.float64).reshape(-1, 2)
        v = np.ascontiguousarray(vals, np.float64)
        i2 = np.ascontiguousarray(img2, np.float64)
        res = AlnResult()
        self._check(self._L.aln_corr_patch_to_image(self.h, xy.ctypes.data, v.ctypes.data,
                                                    len(v), i2.ctypes.data, i2.size, ox, oy,
                                                    radius, int(bfilter), C.byref(res)))
        return res.as_dict()

    # -- CorrImagesR / CorrImagesS ------------------------------------------
    def corr_images(self, kind, a, b, lg=None, mincor=0.0, nbmaxht=0.75, ox=0, oy=0, rx=-1,
                    ry=-1, a_origin=(0, 0), b_origin=(0, 0)) -> dict:
        ia = image(a, *a_origin)
        ib = image(b, *b_origin)
        res = AlnResult()
        self._check(self._L.aln_corr_images(self.h, kind, C.byref(ia), C.byref(ib),
                                            C.byref(lg) if lg is not None else None,
                                            mincor, nbmaxht, ox, oy, rx, ry, C.byref(res)))
        return res.as_dict()

    def corr_images_batch(self, jobs) -> list:
        """jobs: dicts with kind, a, b, [legal, mincor, nbmaxht, ox, oy, rx, ry,
        a_origin, b_origin, b_key]."""
        jobs = list(jobs)
        arr = (AlnImageJob * len(jobs))()
        keep = []
        for k, j in enumerate(jobs):
            ia = image(j["a"], *j.get("a_origin", (0, 0)))
            ib = image(j["b"], *j.get("b_origin", (0, 0)))
            keep += [ia, ib]
            arr[k].a, arr[k].b, arr[k].kind = ia, ib, j["kind"]
            if j.get("legal") is not None:
                keep.append(j["legal"])
                arr[k].legal = j["legal"]
            arr[k].mincor = j.get("mincor", 0.0)
            arr[k].nbmaxht = j.get("nbmaxht", 0.75)
            arr[k].ox, arr[k].oy = j.get("ox", 0), j.get("oy", 0)
            arr[k].rx, arr[k].ry = j.get("rx", -1), j.get("ry", -1)
            arr[k].b_key = j.get("b_key", 0)
        out = (AlnResult * len(jobs))()
        self._check(self._L.aln_corr_images_batch(self.h, len(jobs), arr, out))
        return [o.as_dict() for o in out]

    # -- CThmScan sweep -------------------------------------------------------
    def thm_search_batch(self, thumbs, rthresh=0.3, nbmaxht=0.75, pretweak=0, constxy=1,
                         usecorrr=1, disc=(0, 0, -1, -1), mode=THM_DENOVO, ang0=0.0,
                         hfang=10.0, step=0.5, tdfm=None) -> list:
        thumbs = list(thumbs)
        arr = (AlnThumbs * len(thumbs))()
        for k, t in enumerate(thumbs):
            arr[k] = t
        P = AlnThmParams()
        P.rthresh, P.nbmaxht = rthresh, nbmaxht
        P.constxy, P.pretweak, P.usecorrr = constxy, pretweak, usecorrr
        P.ox, P.oy, P.rx, P.ry = disc
        for i, v in enumerate(tdfm if tdfm is not None else (1, 0, 0, 0, 1, 0)):
            P.tdfm[i] = v
        out = (AlnThmResult * len(thumbs))()
        self._check(self._L.aln_thm_search_batch(self.h, len(thumbs), arr, C.byref(P), mode,
                                                 ang0, hfang, step, out))
        return [{"A": o.A, "X": o.X, "Y": o.Y, "R": o.R, "err": o.err, "ncalls": o.ncalls,
                 "T": list(o.T)} for o in out]

    def thm_finish_batch(self, thumbs, mode, priors, tptwk=None, **params) -> list:
        """PostTweaks (THM_POSTTWEAKS) / FinishAtFullRes (THM_FULLRES) per pair
        from priors (dicts with A, X, Y, R) and pretweak transforms (6 each)."""
        thumbs = list(thumbs)
        n = len(thumbs)
        arr = (AlnThumbs * n)()
        pri = (AlnThmResult * n)()
        for k, (t, p) in enumerate(zip(thumbs, priors)):
            arr[k] = t
            pri[k].A, pri[k].X, pri[k].Y, pri[k].R = p["A"], p["X"], p["Y"], p["R"]
        tw = None
        if tptwk is not None:
            tw = np.ascontiguousarray(tptwk, np.float64).reshape(n, 6)
        tout = np.zeros((n, 6), np.float64)
        P = _thm_params(**params)
        out = (AlnThmResult * n)()
        self._check(self._L.aln_thm_finish_batch(
            self.h, n, arr, C.byref(P), mode, pri,
            tw.ctypes.data if tw is not None else None, out, tout.ctypes.data))
        return [{"A": o.A, "X": o.X, "Y": o.Y, "R": o.R, "err": o.err, "ncalls": o.ncalls,
                 "T": list(o.T), "tptwk": tout[k].tolist()} for k, o in enumerate(out)]

    def approx_match_batch(self, pairs, **params) -> list:
        """ApproximateMatch for [(a, b, (tabx, taby))] tile pairs (numpy arrays
        or CUDA tensors of equal size and type); params as
        aln_approx_params (defaults: 1_DMesh/ApproximateMatch.cpp's with
        XYCONF 0.75, OLAP2D 40000, THMDEC 4, a denovo sweep of +-10 deg)."""
        d = dict(xyconf=0.75, olap1d=0, olap2d=40000, thmdec=4, mode_prior=0, ang0=0.0,
                 hfangdn=10.0, hfangpr=1.0, rthresh=0.3, nbmaxht=0.75, pretweak=0, tweaks=0,
                 limxy=0)
        d.update(params)
        P = AlnApproxParams(**d)
        n = len(pairs)
        arr = (AlnTilePair * n)()
        keep = []
        for k, (a, b, tab) in enumerate(pairs):
            ia, ib = image(a), image(b)
            keep += [ia, ib]
            arr[k].a, arr[k].b = ia, ib
            arr[k].tabx, arr[k].taby = tab
        res = (AlnApproxResult * n)()
        self._check(self._L.aln_approx_match_batch(self.h, n, arr, C.byref(P), res))
        return [{"status": r.status, "err": r.err, "A": r.A, "X": r.X, "Y": r.Y, "R": r.R,
                 "T": list(r.T), "sweep": list(r.sweep),
                 "crop": list(r.crop) + [r.crop_w, r.crop_h]} for r in res]

    def points_image(self, xy, v, xmin, ymin, w, h, slot=0):
        """ImageFromValuesAndPoints / DistributePixel on the device: returns
        (h x w FP64 raster copy, the aln_image of the device raster)."""
        xy = np.ascontiguousarray(xy, np.float64).reshape(-1, 2)
        v = np.ascontiguousarray(v, np.float64)
        out = np.zeros((h, w), np.float64)
        im = AlnImage()
        self._check(self._L.aln_points_image(self.h, slot, len(v), xy.ctypes.data,
                                             v.ctypes.data, xmin, ymin, w, h, C.byref(im),
                                             out.ctypes.data))
        return out, im

    def pixpair_condition(self, tile, order=2, r1=0, r2=0, max1dpix=0):
        """PixPair::Load's conditioning of one tile: (vfy, aln, scl) -- the
        flattened image and the matcher's image at the working size."""
        ws, hs, scl = C.c_int(), C.c_int(), C.c_int()
        h, w = tile.shape
        if self._L.aln_pixpair_dims(w, h, max1dpix, C.byref(ws), C.byref(hs),
                                    C.byref(scl)) != ALN_OK:
            raise AlnError(ALN_ERR_ARG, "tile size not a multiple of the scale")
        vfy = np.zeros((hs.value, ws.value), np.float64)
        aln_ = np.zeros((hs.value, ws.value), np.float64)
        im = image(tile)
        self._check(self._L.aln_pixpair_condition(self.h, C.byref(im), order, r1, r2, max1dpix,
                                                  vfy.ctypes.data, aln_.ctypes.data))
        return vfy, aln_, scl.value

    def improve_control_pts_batch(self, jobs) -> list:
        """ImproveControlPts for a list of mesh_job()s at once.  Returns per
        job dict(corr, corr0, evals, ac) (ac: the optimised nc x 2 points)."""
        jobs = list(jobs)
        n = len(jobs)
        arr = (AlnMeshJob * n)()
        for k, J in enumerate(jobs):
            arr[k] = J
        res = (AlnMeshResult * n)()
        self._check(self._L.aln_improve_control_pts_batch(self.h, n, arr, res))
        return [{"corr": r.corr, "corr0": r.corr0, "evals": r.evals, "ac": J._ac.copy()}
                for r, J in zip(res, jobs)]

    def grad_desc_step(self, job):
        """GradDescStep at job's control points: (bnew normalised, dRdc nc x
        2, CorrVectors(av, bnew))."""
        bnew = np.zeros(job.nm, np.float64)
        d = np.zeros((job.nc, 2), np.float64)
        c = C.c_double(0.0)
        self._check(self._L.aln_grad_desc_step(self.h, C.byref(job), bnew.ctypes.data,
                                               d.ctypes.data, C.byref(c)))
        return bnew, d, c.value

    def corr_vectors(self, a, b):
        """CorrVectors(a, b): (correlation, count of products >= 1e-8)."""
        a = np.ascontiguousarray(a, np.float64)
        b = np.ascontiguousarray(b, np.float64)
        out, nnz = C.c_double(0.0), C.c_int(0)
        self._check(self._L.aln_corr_vectors(self.h, a.ctypes.data, b.ctypes.data, len(a),
                                             C.byref(out), C.byref(nnz)))
        return out.value, nnz.value

    def decimate(self, images, lbin, masks=None, normalize=True) -> list:
        """MakeThumbs' DecimateVector + Normalize of 2-D arrays (point lists
        in raster order; masks: per image None or a 0/1 array of the same
        shape).  Returns [(vals[oh, ow] FP64, present[oh, ow] uint8, sd)]."""
        images = [np.ascontiguousarray(a) for a in images]
        n = len(images)
        ims = (AlnImage * n)()
        mk = (C.c_void_p * n)()
        keep = []
        for k, a in enumerate(images):
            ims[k] = image(a)
            m = None if masks is None else masks[k]
            if m is not None:
                m = np.ascontiguousarray(m, np.uint8)
                keep.append(m)
                mk[k] = m.ctypes.data
        outs = []
        ov = (C.c_void_p * n)()
        om = (C.c_void_p * n)()
        for k, a in enumerate(images):
            oh, ow = -(-a.shape[0] // lbin), -(-a.shape[1] // lbin)
            v = np.empty((oh, ow), np.float64)
            m = np.empty((oh, ow), np.uint8)
            outs.append((v, m))
            ov[k], om[k] = v.ctypes.data, m.ctypes.data
        sd = np.zeros(n, np.float64)
        self._check(self._L.aln_decimate_batch(self.h, n, ims, mk, lbin, int(normalize), ov, om,
                                               sd.ctypes.data))
        return [(v, m, float(sd[k])) for k, (v, m) in enumerate(outs)]

    def thm_call_batch(self, thumbs, op, args, best=None, tptwk=None, **params) -> list:
        """One CThmScan member-function call per pair (THMOP_*; args: 4 per
        pair, see aln_thm_call_batch), from the object state best (dicts
        with A, X, Y, R[, T, err]) and tptwk (6 per pair)."""
        thumbs = list(thumbs)
        n = len(thumbs)
        arr = (AlnThumbs * n)()
        res = (AlnThmResult * n)()
        for k, t in enumerate(thumbs):
            arr[k] = t
            b = best[k] if best is not None else {}
            res[k].A, res[k].X = b.get("A", -999.0), b.get("X", -999.0)
            res[k].Y, res[k].R = b.get("Y", -999.0), b.get("R", -999.0)
            for i, v in enumerate(b.get("T", (1, 0, 0, 0, 1, 0))):
                res[k].T[i] = v
            res[k].err = b.get("err", 0)
        a = np.zeros((n, 4), np.float64)
        a[:] = np.asarray(args, np.float64).reshape(-1, 4)
        tw = np.tile(np.array([1, 0, 0, 0, 1, 0], np.float64), (n, 1))
        if tptwk is not None:
            tw[:] = np.asarray(tptwk, np.float64).reshape(n, 6)
        ret = np.zeros(n, np.float64)
        P = _thm_params(**params)
        self._check(self._L.aln_thm_call_batch(self.h, n, arr, C.byref(P), op, a.ctypes.data,
                                               res, tw.ctypes.data, ret.ctypes.data))
        return [{"A": o.A, "X": o.X, "Y": o.Y, "R": o.R, "err": o.err, "ncalls": o.ncalls,
                 "T": list(o.T), "tptwk": tw[k].tolist(), "ret": float(ret[k])}
                for k, o in enumerate(res)]

    def corr_patches_batch(self, pairs) -> list:
        """pairs: iterable of dicts with a, b, [ox, oy, radius, legal, a_origin, b_origin,
        b_key (spectrum-cache key of b, 0 = none)]."""
        pairs = list(pairs)
        arr = (AlnPair * len(pairs))()
        keep = []
        for k, p in enumerate(pairs):
            ia = image(p["a"], *p.get("a_origin", (0, 0)))
            ib = image(p["b"], *p.get("b_origin", (0, 0)))
            keep += [ia, ib]
            arr[k].a = ia
            arr[k].b = ib
            arr[k].ox = p.get("ox", 0)
            arr[k].oy = p.get("oy", 0)
            arr[k].radius = p.get("radius", 4096)
            lg = p.get("legal")
            if lg is not None:
                keep.append(lg)
                arr[k].legal = lg
            arr[k].b_key = p.get("b_key", 0)
        out = (AlnResult * len(pairs))()
        self._check(self._L.aln_corr_patches_batch(self.h, len(pairs), arr, out))
        return [o.as_dict() for o in out]


def corr_patches_grid(pair: AlnPair):
    """(nx, ny, nseg, transposed) of the transform grid CorrPatches uses for
    one pair, in the frame the pair is solved in (nseg > 0: the column axis
    in nseg segments of ny points); (0, 0, 0, t) for an empty window."""
    nx, ny, ns, tr = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    rc = lib().aln_corr_patches_grid(C.byref(pair), C.byref(nx), C.byref(ny), C.byref(ns),
                                     C.byref(tr))
    if rc < 0:
        raise AlnError(rc, "aln_corr_patches_grid")
    return nx.value, ny.value, ns.value, tr.value


def parab_peak_fft(xpk, ypk, d, I):
    I = np.ascontiguousarray(I, np.float64)
    x, y = C.c_double(xpk), C.c_double(ypk)
    lib().aln_parab_peak_fft(C.byref(x), C.byref(y), d, I.ctypes.data, I.shape[1], I.shape[0])
    return x.value, y.value


def _thm_params(rthresh=0.3, nbmaxht=0.75, pretweak=0, constxy=1, usecorrr=1,
                disc=(0, 0, -1, -1), tdfm=None, disc_of_angle=None) -> AlnThmParams:
    """disc_of_angle: None, or a Python function deg -> (ox, oy, rx, ry)
    (CThmScan's newAngProc); the returned params keep its C callback alive."""
    P = AlnThmParams()
    P.rthresh, P.nbmaxht = rthresh, nbmaxht
    P.constxy, P.pretweak, P.usecorrr = constxy, pretweak, usecorrr
    P.ox, P.oy, P.rx, P.ry = disc
    for i, v in enumerate(tdfm if tdfm is not None else (1, 0, 0, 0, 1, 0)):
        P.tdfm[i] = v
    if disc_of_angle is not None:
        def tramp(user, deg, ox, oy, rx, ry):
            ox[0], oy[0], rx[0], ry[0] = (int(v) for v in disc_of_angle(deg))
        P._cb = DISC_OF_ANGLE(tramp)
        P.disc_of_angle = P._cb
    return P


# CThmScan member functions for aln_thm_call_batch
(THMOP_RFROMANGLE, THMOP_SCAN_MAXR, THMOP_SCAN_CONSTXY, THMOP_SCAN_SEL, THMOP_SCAN_TWEAKS,
 THMOP_PEAKHUNT, THMOP_PRIOR, THMOP_DENOVO, THMOP_PRETWEAKS, THMOP_POSTTWEAKS,
 THMOP_FULLRES) = range(11)


def _reply_dict(rep: AlnReply, kind: int) -> dict:
    d = {"status": rep.status, "queue_ms": rep.queue_ms, "total_ms": rep.total_ms,
         "batch_size": rep.batch_size}
    if kind == REQ_SWEEP:
        o = rep.sweep
        d.update({"A": o.A, "X": o.X, "Y": o.Y, "R": o.R, "err": o.err, "ncalls": o.ncalls,
                  "T": list(o.T)})
    else:
        d.update(rep.corr.as_dict())
        d["status"] = rep.status if rep.status < 0 else rep.corr.status
    return d


class Server:
    """Continuous-batching request server (aln_server_* in include/aln_corr.h).

    submit_* queue one request and return its ticket; wait(ticket) or
    collect() hand the replies over.  Inputs stay referenced here until their
    reply has been handed over."""

    def __init__(self, device: int = 0, workers: int = 2, mem_budget: int = 0,
                 max_batch: int = 0, cache_bytes: int = 0):
        self._L = lib()
        P = AlnServerParams(device, workers, mem_budget, max_batch, cache_bytes)
        h = C.c_void_p()
        rc = self._L.aln_server_create(C.byref(P), C.byref(h))
        if rc != ALN_OK:
            raise AlnError(rc, self._L.aln_last_error(None).decode())
        self.h = h
        self._keep = {}

    def close(self):
        if getattr(self, "h", None):
            self._L.aln_server_destroy(self.h)
            self.h = None
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _submit(self, req: AlnRequest, keep) -> int:
        t = C.c_ulonglong()
        rc = self._L.aln_server_submit(self.h, C.byref(req), C.byref(t))
        if rc < 0:
            raise AlnError(rc, "submit refused")
        self._keep[t.value] = (req.kind, keep)
        return t.value

    def submit_patches(self, a, b, ox=0, oy=0, radius=4096, lg=None, b_key=0,
                       a_origin=(0, 0), b_origin=(0, 0)) -> int:
        req = AlnRequest()
        req.kind = REQ_PATCHES
        ia, ib = image(a, *a_origin), image(b, *b_origin)
        req.pair.a, req.pair.b = ia, ib
        req.pair.ox, req.pair.oy, req.pair.radius = ox, oy, radius
        if lg is not None:
            req.pair.legal = lg
        req.pair.b_key = b_key
        return self._submit(req, (ia, ib, lg))

    def submit_images(self, kind, a, b, lg=None, mincor=0.0, ox=0, oy=0, rx=-1, ry=-1,
                      b_key=0, a_origin=(0, 0), b_origin=(0, 0)) -> int:
        req = AlnRequest()
        req.kind = REQ_IMAGES
        ia, ib = image(a, *a_origin), image(b, *b_origin)
        j = req.job
        j.a, j.b, j.kind = ia, ib, kind
        if lg is not None:
            j.legal = lg
        j.mincor, j.nbmaxht = mincor, 0.75
        j.ox, j.oy, j.rx, j.ry = ox, oy, rx, ry
        j.b_key = b_key
        return self._submit(req, (ia, ib, lg))

    def submit_sweep(self, thumbs: AlnThumbs, mode=0, ang0=0.0, hfang=10.0, step=0.5,
                     **params) -> int:
        req = AlnRequest()
        req.kind = REQ_SWEEP
        req.thumbs = thumbs
        req.thm = _thm_params(**params)
        req.thm_mode, req.ang0, req.hfang, req.step = mode, ang0, hfang, step
        return self._submit(req, (thumbs,))

    def wait(self, ticket: int, timeout_ms: int = -1) -> dict:
        rep = AlnReply()
        rc = self._L.aln_server_wait(self.h, ticket, timeout_ms, C.byref(rep))
        if rc < 0:
            raise AlnError(rc, "wait")
        kind, _ = self._keep.pop(ticket)
        return _reply_dict(rep, kind)

    def collect(self, cap: int = 4096, timeout_ms: int = 100) -> list:
        """Up to cap finished replies as (ticket, reply dict)."""
        tk = (C.c_ulonglong * cap)()
        reps = (AlnReply * cap)()
        n = self._L.aln_server_collect(self.h, cap, timeout_ms, tk, reps)
        if n < 0:
            raise AlnError(n, "collect")
        out = []
        for i in range(n):
            kind, _ = self._keep.pop(tk[i])
            out.append((tk[i], _reply_dict(reps[i], kind)))
        return out

    def counters(self) -> dict:
        c = self._L.aln_server_counter
        return {"submitted": c(self.h, 0), "finished": c(self.h, 1), "batches": c(self.h, 2),
                "waiting": c(self.h, 3), "spec_hits": c(self.h, 4), "spec_fills": c(self.h, 5),
                "spec_evictions": c(self.h, 6), "spec_bytes": c(self.h, 7)}
