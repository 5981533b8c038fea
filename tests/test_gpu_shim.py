"""The C++ drop-in on the GPU: a C++ program calls CorrPatches / CorrImagesR /
CorrImagesS / FFT_2D / IFT_2D through the reference's signatures
(alignment_projects_gb300/shim/aln_correlation.hpp); results match the
reference's golden outputs (r within 1e-4, offsets within 0.01 px where the
peak is clear) and the fft2 cache vector gives the same numbers."""
import os
import subprocess

import numpy as np
import pytest

from conftest import load_golden
from shim_util import build_check, case

pytestmark = pytest.mark.gpu

MARGIN = 1e-3


def _legal_args(lg):
    kind, a, b, area, ck, cn = (int(v) for v in lg)
    assert kind in (0, 1)
    return dict(rgn_min=max(a, 1) if kind == 1 else 0, rgn_area=area if kind == 1 else 0,
                cnt_n=cn if ck == 1 else -1)


def test_cpp_callers_through_shim(tmp_path, orc):
    import oracle
    exe = build_check(str(tmp_path))
    gp = load_golden("corr_patches")
    gi = load_golden("corr_images")
    blob, expect = b"", []
    for k in ("kat_testnormcorr", "plain96_s1", "plain96_s2", "ragged_none", "ragged_disc",
              "ragged_cnt", "u16_holes"):
        d = gp[k]
        la = _legal_args(d["legal"])
        blob += case(0, d["pa"], d["va"], d["pb"], d["vb"], int(d["ox"]), int(d["oy"]),
                     int(d["radius"]), **la)
        o = orc.corr_patches(d["pa"], d["va"], d["pb"], d["vb"], int(d["ox"]), int(d["oy"]),
                             int(d["radius"]), oracle.legal(*[int(v) for v in d["legal"]]))
        expect.append((k, float(d["r"]), float(d["dx"]), float(d["dy"]),
                       o["r"] - o["second"] > MARGIN, 1e-4))
    # the same image b again through the same fft2 vector (cache path)
    d = gp["plain96_s1"]
    la = _legal_args(d["legal"])
    blob += case(0, d["pa"], d["va"], d["pb"], d["vb"], int(d["ox"]), int(d["oy"]),
                 int(d["radius"]), reuse=1, **la)
    expect.append(("plain96_s1 cached", float(d["r"]), float(d["dx"]), float(d["dy"]), True,
                   1e-4))
    for k in ("img_s0_k1_d0_m0", "img_s0_k1_d1_m1", "img_s0_k2_d0_m0", "img_s0_k2_d1_m0",
              "img_s1_k2_d1_m1", "img_s0_k0_d0_m0", "img_s1_k0_d1_m1"):
        d = gi[k]
        kind = int(d["kind"])
        disc = [int(v) for v in d["disc"]]
        la = _legal_args(d["legal"])
        blob += case(kind if kind else 3, d["pa"], d["va"], d["pb"], d["vb"], disc[0], disc[1],
                     4096, disc[2], disc[3], mincor=float(d["mincor"]), **la)
        o = orc.corr_images(kind, d["pa"], d["va"], d["pb"], d["vb"],
                            oracle.legal(*[int(v) for v in d["legal"]]), float(d["mincor"]),
                            0.75, *disc)
        tol = 1e-4 if kind == 1 else 1e-4 * max(1.0, abs(float(d["r"])))
        expect.append((k, float(d["r"]), float(d["dx"]), float(d["dy"]),
                       o["r"] - o["second"] > MARGIN, tol))
    cases = os.path.join(str(tmp_path), "cases.bin")
    open(cases, "wb").write(blob)
    out = subprocess.run([exe, cases], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert len(lines) == len(expect) + 1
    for (name, r, dx, dy, clear, tol), ln in zip(expect, lines):
        gr, gdx, gdy = (float(v) for v in ln.split())
        assert abs(gr - r) <= tol, (name, gr, r)
        if clear:
            assert abs(gdx - dx) <= 0.01 and abs(gdy - dy) <= 0.01, (name, gdx, gdy, dx, dy)
    f = lines[-1].split()
    assert f[0] == "fft" and int(f[1]) == 4 * 5 and float(f[2]) < 1e-4 and int(f[3]) == 1024


def _thm_compare(g, ref, msg):
    assert g["err"] == int(ref["err"]), (msg, g, ref)
    A, R = float(ref["A"]), float(ref["R"])
    assert abs(g["A"] - A) <= 0.05, (msg, g, ref)
    assert abs(g["R"] - R) <= 1e-3 * max(1.0, abs(R)), (msg, g, ref)
    if abs(g["A"] - A) < 1e-9:
        assert abs(g["X"] - float(ref["X"])) <= 0.01 and \
            abs(g["Y"] - float(ref["Y"])) <= 0.01, (msg, g, ref)


def test_cpp_thmscan_through_shim(tmp_path):
    """class CThmScan through the C++ drop-in: a C++ program makes the
    reference's call sequences (DenovoBestAngle, RFromAngle, UsePriorAngles,
    AngleScanSel with MaxR, PostTweaks, FinishAtFullRes) on the golden
    thumbnail pairs; results match the reference's golden outputs with the
    sweep's bar (tests/test_gpu_sweep.py)."""
    from shim_util import build_thm_check, thm_case, parse_thm_lines
    exe = build_thm_check(str(tmp_path))
    blob, expect = b"", []
    gs = load_golden("thm_scan")
    for k in sorted(gs):
        d = gs[k]
        blob += thm_case(int(d["mode"]), d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]),
                         rthresh=float(d["rthresh"]), pretweak=int(d["pretweak"]),
                         disc=tuple(int(v) for v in d["disc"]), ang0=float(d["ang0"]),
                         hfang=float(d["hfang"]), step=float(d["step"]))
        expect.append((k, d, None))
    gf = load_golden("thm_finish")
    for k in sorted(gf):
        d = gf[k]
        blob += thm_case(int(d["mode"]), d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]),
                         prior=tuple(float(v) for v in d["prior"]),
                         tptwk=tuple(float(v) for v in d["tptwk"]))
        expect.append((k, dict(A=d["A"], X=d["X"], Y=d["Y"], R=d["R"], err=0),
                       d["tptwk_out"]))
    cases = os.path.join(str(tmp_path), "thm_cases.bin")
    open(cases, "wb").write(blob)
    out = subprocess.run([exe, cases], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    got = parse_thm_lines(out.stdout)
    assert len(got) == len(expect)
    for (name, ref, tw), g in zip(expect, got):
        _thm_compare(g, ref, name)
        if tw is not None and abs(g["A"] - float(ref["A"])) < 1e-9:
            assert np.abs(np.array(g["tptwk"]) - tw).max() <= 1e-6, (name, g, tw)


def test_cpp_thmscan_callbacks_and_table(tmp_path):
    """SetNewAngProc through the drop-in (a C++ callback giving a fixed disc
    for every angle equals SetDisc with that disc), and DebugAngs' angle
    table (one line per angle; the row at the centre angle equals
    RFromAngle there)."""
    from shim_util import build_thm_check, thm_case, parse_thm_lines
    exe = build_thm_check(str(tmp_path))
    d = load_golden("thm_scan")["thm_s0_denovo"]
    common = dict(pa=d["pa"], va=d["va"], pb=d["pb"], vb=d["vb"], req=int(d["req"]))
    disc = (0, 5, 12, 12)
    blob = (thm_case(0, common["pa"], common["va"], common["pb"], common["vb"], common["req"],
                     disc=disc)
            + thm_case(8, common["pa"], common["va"], common["pb"], common["vb"],
                       common["req"], disc=disc)
            + thm_case(9, common["pa"], common["va"], common["pb"], common["vb"],
                       common["req"], ang0=-2.0, hfang=1.0, step=0.5))
    cases = os.path.join(str(tmp_path), "cb_cases.bin")
    open(cases, "wb").write(blob)
    out = subprocess.run([exe, cases], capture_output=True, text=True, timeout=600,
                         cwd=str(tmp_path))
    assert out.returncode == 0, out.stderr
    fixed, cb, table = parse_thm_lines(out.stdout)
    assert cb["ret"] == fixed["ret"] + 10.0   # the callback was called
    for k in ("A", "X", "Y", "R", "err"):
        assert cb[k] == fixed[k], (k, cb, fixed)
    rows = open(os.path.join(str(tmp_path), "angs_1.2^3.4.log")).read().split("\n")
    assert rows[0].split() == ["Deg", "R", "X", "Y"]
    vals = [[float(v) for v in r.split()] for r in rows[1:] if r.strip()]
    assert [round(v[0], 3) for v in vals] == [-3.0, -2.5, -2.0, -1.5, -1.0]
    mid = vals[2]
    assert abs(mid[1] - table["R"]) <= 1e-4 and abs(mid[2] - table["X"]) <= 1e-3 and \
        abs(mid[3] - table["Y"]) <= 1e-3


def test_cpp_mesh_optimizer_through_shim(tmp_path):
    """GradDescStep / CorrVectors / ImproveControlPts called with the
    reference's dense multiplier rows through the C++ drop-in: the reference's
    golden numbers (the GPU sums in blocks: 1e-9 on correlations, 1e-6 px)."""
    import struct
    from alignment_projects_gb300 import build as b
    shim = b.build_shim()
    exe = os.path.join(str(tmp_path), "mesh_check")
    here = os.path.dirname(os.path.abspath(__file__))
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-o", exe,
                           os.path.join(here, "cpp", "mesh_check.cpp"),
                           "-I" + os.path.join(here, "..", "alignment_projects_gb300", "shim"),
                           "-L" + os.path.dirname(shim), "-laln_corr_shim", "-laln_corr",
                           "-Wl,-rpath," + os.path.dirname(shim)])
    cases = load_golden("mesh")
    names = sorted(cases)
    blob = b""
    for n in names:
        d = cases[n]
        nc, nm = len(d["ac0"]), len(d["av"])
        h, w = d["bimg"].shape
        dense = np.zeros((nm, nc))
        rows = np.repeat(np.arange(nm), d["am_idx"].shape[1])
        idx = d["am_idx"].ravel()
        keep = idx >= 0
        dense[rows[keep], idx[keep]] = d["am_w"].ravel()[keep]
        blob += struct.pack("<4i2d", nc, nm, w, h, float(d["ini"]), float(d["fin"]))
        blob += np.ascontiguousarray(d["ac0"], np.float64).tobytes() + dense.tobytes()
        blob += np.ascontiguousarray(d["av"]).tobytes() + np.ascontiguousarray(d["bimg"]).tobytes()
    path = os.path.join(str(tmp_path), "mesh.bin")
    with open(path, "wb") as f:
        f.write(blob)
    out = subprocess.run([exe, path], check=True, capture_output=True, text=True).stdout
    lines = out.strip().splitlines()
    assert len(lines) == len(names)
    for n, ln in zip(names, lines):
        d = cases[n]
        v = [float(x) for x in ln.split()]
        assert abs(v[0] - float(d["corr0"])) <= 1e-9, n
        assert abs(v[1] - float(d["corr"])) <= 1e-9, n
        assert np.abs(np.array(v[2:]).reshape(-1, 2) - d["ac"]).max() <= 1e-6, n
