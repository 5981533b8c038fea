"""Compile the GB300 library (libaln_corr.so) in-tree with nvcc for sm_103a."""
from __future__ import annotations

import hashlib
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libaln_corr.so")

SOURCES = ["aln_corr.cu"]
HEADERS = ["aln_fft.cuh", "aln_fft_reg.cuh", "aln_corr_kernels.cuh", "aln_pipeline.cuh",
           "aln_sweep.cuh", "aln_server.cuh", "aln_mesh.cuh", "aln_approx.cuh",
           "aln_tune.cuh", "aln_points.cuh",
           "aln_thmpair.cuh", "aln_ingest.cuh", "aln_row_layout.cuh"]
NVCC_FLAGS = [
    "-gencode", "arch=compute_103a,code=sm_103a",
    "-O3", "-lineinfo", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.isabs(c) and os.path.exists(c) or not os.path.isabs(c)):
            return c
    return "nvcc"


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


SHIM_SRCS = [os.path.join(PKG, "shim", s)
             for s in ("aln_correlation_shim.cpp", "aln_thmscan_shim.cpp")]
SHIM_HDRS = [os.path.join(PKG, "shim", h)
             for h in ("aln_correlation.hpp", "aln_thmscan.hpp", "aln_shim_util.hpp")]
SHIM_LIB = os.path.join(LIBDIR, "libaln_corr_shim.so")


def build_shim(force: bool = False, verbose: bool = False) -> str:
    """The C++ drop-in for the Correlation.h entry points and class CThmScan (g++), linked
    against libaln_corr.so in the same directory."""
    lib = build(force=force, verbose=verbose)
    deps = SHIM_SRCS + SHIM_HDRS + [os.path.join(ROOT, "include", "aln_corr.h"), lib]
    if not force and not _stale(SHIM_LIB, deps):
        return SHIM_LIB
    tmp = SHIM_LIB + ".tmp%d" % os.getpid()
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off",
           "-shared", "-o", tmp] + SHIM_SRCS + ["-L" + LIBDIR, "-laln_corr",
           "-Wl,-rpath,$ORIGIN"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(tmp, SHIM_LIB)
    return SHIM_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, h) for h in HEADERS] + [
        os.path.join(ROOT, "include", "aln_corr.h"), os.path.abspath(__file__)]
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    # the build id names the autotuner's choice file: a new build measures anew
    h = hashlib.sha1()
    for d in deps:
        with open(d, "rb") as f:
            h.update(f.read())
    cmd = ([_nvcc()] + NVCC_FLAGS + ['-DALN_BUILD_ID="%s"' % h.hexdigest()[:12],
                                     "-shared", "-o", tmp] + srcs + ["-lcudart", "-ldl"])
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
    print(build_shim(verbose=True))
