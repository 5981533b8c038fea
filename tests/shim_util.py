"""Helpers for the C++ drop-in tests: case files for tests/cpp/shim_check.cpp."""
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_check(out_dir):
    from alignment_projects_gb300 import build as b
    shim = b.build_shim()
    exe = os.path.join(out_dir, "shim_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-o", exe,
                           os.path.join(HERE, "cpp", "shim_check.cpp"),
                           "-I" + os.path.join(ROOT, "alignment_projects_gb300", "shim"),
                           "-L" + os.path.dirname(shim), "-laln_corr_shim", "-laln_corr",
                           "-Wl,-rpath," + os.path.dirname(shim)])
    return exe


def case(kind, p1, v1, p2, v2, ox=0, oy=0, radius=4096, rx=-1, ry=-1, rgn_min=0,
         rgn_area=0, cnt_n=-1, mincor=0.0, reuse=0):
    def cloud(p, v):
        p = np.ascontiguousarray(p, np.float64).reshape(-1, 2)
        v = np.ascontiguousarray(v, np.float64)
        return struct.pack("<i", len(v)) + p.tobytes() + v.tobytes()
    return (struct.pack("<i", kind) + cloud(p1, v1) + cloud(p2, v2)
            + struct.pack("<iiiiiiqqdi", ox, oy, radius, rx, ry, rgn_min, rgn_area, cnt_n,
                          mincor, reuse))


def build_thm_check(out_dir, reference_headers=None):
    """tests/cpp/thmscan_check.cpp against the shim: compiled with the
    shim's header, or with the reference's own headers (reference_headers =
    its source tree) plus the reference objects the program's TAffine and
    Point uses need."""
    from alignment_projects_gb300 import build as b
    shim = b.build_shim()
    exe = os.path.join(out_dir, "thmscan_check" + ("_ref" if reference_headers else ""))
    cmd = ["g++", "-std=c++17", "-O2", "-w", "-o", exe,
           os.path.join(HERE, "cpp", "thmscan_check.cpp")]
    if reference_headers:
        import oracle
        objs = os.path.dirname(oracle.REF_SO)
        cmd += ["-DALN_REFERENCE_HEADERS", "-DTIXML_USE_STL",
                "-I" + os.path.join(reference_headers, "0_GEN"),
                "-I" + os.path.join(reference_headers, "0_UTL"),
                "-I" + os.path.join(ROOT, "oracle", "ref"),
                os.path.join(objs, "TAffine.o"), os.path.join(objs, "CPoint.o")]
    else:
        cmd += ["-I" + os.path.join(ROOT, "alignment_projects_gb300", "shim")]
    cmd += ["-L" + os.path.dirname(shim), "-laln_corr_shim", "-laln_corr", "-lpthread",
            "-Wl,-rpath," + os.path.dirname(shim)]
    subprocess.check_call(cmd)
    return exe


def thm_case(mode, pa, va, pb, vb, req, olap1d=0, rthresh=0.3, nbmaxht=0.75, pretweak=0,
             constxy=1, usecorrr=1, disc=(0, 0, -1, -1), ang0=0.0, hfang=10.0, step=0.5,
             prior=(0.0, 0.0, 0.0, 0.0), tptwk=(1.0, 0.0, 0.0, 0.0, 1.0, 0.0)):
    def cloud(p, v):
        p = np.ascontiguousarray(p, np.float64).reshape(-1, 2)
        v = np.ascontiguousarray(v, np.float64)
        return struct.pack("<i", len(v)) + p.tobytes() + v.tobytes()
    return (struct.pack("<i", mode) + cloud(pa, va) + cloud(pb, vb)
            + struct.pack("<qiddiiiiiiiddd", req, olap1d, rthresh, nbmaxht, pretweak, constxy,
                          usecorrr, *[int(v) for v in disc], ang0, hfang, step)
            + struct.pack("<4d", *prior) + struct.pack("<6d", *tptwk))


def parse_thm_lines(text):
    out = []
    for ln in text.strip().splitlines():
        f = ln.split()
        out.append(dict(A=float(f[0]), X=float(f[1]), Y=float(f[2]), R=float(f[3]),
                        err=int(f[4]), ret=float(f[5]), tptwk=[float(v) for v in f[6:12]]))
    return out
