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
