"""Generate golden fixtures by running the reference's own code.

Run here (where the reference tree is mounted):
    make -C oracle/ref && python tests/golden/make_golden.py

Every fixture stores its inputs and the outputs of the reference's unmodified
functions (oracle/_ref/libalnref.so, built from the reference sources with a
project FP64 FFT behind the FFTW entry points).  The fixtures are committed;
tests compare the C restatement (oracle/aln_oracle.c) and the GPU library
against them on machines where the reference tree does not exist.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from alignment_projects_gb300 import synth  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def legal_tuple(lg):
    return np.array([lg.rgn_kind, lg.rgn_a, lg.rgn_b, lg.rgn_area, lg.cnt_kind, lg.cnt_n],
                    np.int64)


def corr_patches_cases(ref):
    cases = []
    # 1. testnormcorr known-answer test (Retired_Proj/4_TestNormCorr/testnormcorr.cpp:20-63)
    pb = np.array([(0, 3), (2, 3), (3, 2), (3, 3), (3, 4), (4, 3), (5, 4)], float)
    vb = np.array([1, 2, 1, 3, 1, 2, 1], float)
    pa = np.array([(7, 2), (8, 2), (9, 2), (7, 1), (8, 1)], float)
    va = np.array([1, 0, 1, 3, 2], float)
    cases.append(("kat_testnormcorr", pa, va, pb, vb, 0, 0, 4096, O.legal(O.RGN_MIN, 2, 2, 0)))
    # 2. plain uint8 pairs (small version of the 512^2 workload)
    for seed in (1, 2, 3):
        p = synth.plain_pair(seed, n=96, margin=12)
        A, VA = O.image_to_points(p.a)
        B, VB = O.image_to_points(p.b)
        cases.append((f"plain96_s{seed}", A, VA, B, VB, 0, 0, 4096, O.legal(O.RGN_MIN, 32, 32, 0)))
    # 3. disc and legality kinds, ragged sizes, offsets in the point coordinates
    p = synth.plain_pair(7, n=80, margin=10)
    A, VA = O.image_to_points(p.a[:70, :50], 13, -4)
    B, VB = O.image_to_points(p.b[:60, :77], -2, 9)
    for name, ox, oy, rad, lg in [
        ("ragged_none", 0, 0, 4096, O.legal()),
        ("ragged_disc", 15, -13, 9, O.legal(O.RGN_MIN, 10, 10, 0)),
        ("ragged_section", 0, 0, 4096, O.legal(O.RGN_SECTION, 40, 45, 1500)),
        ("ragged_exact", 0, 0, 4096, O.legal(O.RGN_EXACT, 21, 21, 0)),
        ("ragged_cnt", 0, 0, 4096, O.legal(O.RGN_MIN, 5, 5, 0, O.CNT_GT, 800)),
        ("ragged_nolegal", 0, 0, 4096, O.legal(O.RGN_EXACT, 999, 999, 0)),
    ]:
        cases.append((name, A, VA, B, VB, ox, oy, rad, lg))
    # 4. point clouds with holes (zero-valued and missing pixels) and uint16 values
    p = synth.uneven_pair(11)
    A, VA = O.image_to_points(p.a, keep_zeros=True)
    B, VB = O.image_to_points(p.b, keep_zeros=True)
    keep = np.random.default_rng(3).random(len(VA)) > 0.1
    cases.append(("u16_holes", A[keep], VA[keep], B, VB, 0, 0, p.radius,
                  O.legal(O.RGN_MIN, 8, 8, 0)))
    # 5. montage-style strip (small)
    p = synth.montage_pair(5, long_side=256, wmin=40, wmax=60, jitter=10)
    A, VA = O.image_to_points(p.a)
    B, VB = O.image_to_points(p.b)
    cases.append(("strip256", A, VA, B, VB, 0, 0, 16, O.legal(O.RGN_SECTION, 200, 200, 3000)))
    out = {}
    for name, pa, va, pb, vb, ox, oy, rad, lg in cases:
        res = ref.corr_patches(pa, va, pb, vb, ox, oy, rad, lg)
        out[name] = dict(pa=pa, va=va, pb=pb, vb=vb, ox=ox, oy=oy, radius=rad,
                         legal=legal_tuple(lg), r=res["r"], dx=res["dx"], dy=res["dy"])
    return out


def corr_images_cases(ref):
    out = {}
    for seed in (0, 1):
        ta, tb, th, t = synth.thumb_pair(seed, tile=512, dec=8)
        A, VA = O.image_to_points(ta)
        B, VB = O.image_to_points(tb)
        VA = (VA - VA.mean()) / VA.std(ddof=1)
        VB = (VB - VB.mean()) / VB.std(ddof=1)
        ang = np.deg2rad(-th + 0.25)
        R = np.array([[np.cos(ang), -np.sin(ang)], [np.sin(ang), np.cos(ang)]])
        Ar = A @ R.T
        lg = O.legal(O.RGN_MIN, 0, 0, 100, O.CNT_GT, 100)
        out[f"in_s{seed}"] = dict(pa=Ar, va=VA, pb=B, vb=VB)
        for kind in (0, 1, 2):
            for di, disc in enumerate([(0, 0, -1, -1), (2, -3, 20, 14)]):
                for mincor in (0.0, 0.1):
                    res = ref.corr_images(kind, Ar, VA, B, VB, lg, mincor, 0.75, *disc)
                    out[f"img_s{seed}_k{kind}_d{di}_m{int(mincor*10)}"] = dict(
                        kind=kind, ref_in=f"in_s{seed}", legal=legal_tuple(lg),
                        mincor=mincor, nbmaxht=0.75, disc=np.array(disc), r=res["r"],
                        dx=res["dx"], dy=res["dy"])
    return out


def fft_cases(ref):
    rng = np.random.default_rng(17)
    out = {}
    for (ny, nx) in [(8, 16), (64, 32), (32, 128)]:
        x = rng.standard_normal((ny, nx))
        F = ref.fft_2d(x)
        G = ref.ift_2d(F * np.conj(ref.fft_2d(np.roll(x, (2, 3), (0, 1)))), nx)
        out[f"fft_{ny}x{nx}"] = dict(x=x, F=F, G=G)
    # time_fft KAT (Retired_Proj/4_Time_FFT/time_fft.cpp:14-67): shifted copy
    N = 64
    in1 = rng.random(N * N)
    in2 = np.zeros(N * N)
    in2[(np.arange(N * N) + 2 * N + 3) % (N * N)] = in1
    F1 = ref.fft_2d(in1.reshape(N, N))
    F2 = ref.fft_2d(in2.reshape(N, N))
    G = ref.ift_2d(F1 * np.conj(F2), N)
    out["kat_time_fft"] = dict(in1=in1.reshape(N, N), in2=in2.reshape(N, N), G=G,
                               argmax=int(np.argmax(G)))
    return out


def convolve_cases(ref):
    rng = np.random.default_rng(23)
    K = np.array([[-1, -1, -1], [-1, 9, -1], [-1, -1, -1]], float)
    out = {}
    for (h, w) in [(37, 50), (64, 64)]:
        src = rng.standard_normal((h, w))
        out[f"conv_{h}x{w}"] = dict(src=src, K=K, dst=ref.convolve(src, K))
    return out


def patch_to_image_cases(ref):
    p = synth.plain_pair(3, n=100, margin=10)
    A, VA = O.image_to_points(p.a)
    VA = (VA - VA.mean()) / VA.std() / 40
    img2 = np.zeros((256, 256))
    img2[:100, :100] = (p.b - p.b.mean()) / p.b.std() / 40
    out = {}
    for bf in (0, 1):
        res = ref.corr_patch_to_image(A, VA, img2, 0, 0, 4096, bool(bf))
        out[f"p2i_f{bf}"] = dict(pa=A, va=VA, img2=img2, bfilter=bf, r=res["r"],
                                 dx=res["dx"], dy=res["dy"])
    return out


def thm_cases(ref):
    out = {}
    for seed in (0, 2):
        ta, tb, th, t = synth.thumb_pair(seed, tile=768, dec=8)
        A, VA = O.image_to_points(ta)
        B, VB = O.image_to_points(tb)
        A, VA = ref.decimate_normalize(A, VA, 96, 96, 1)
        B, VB = ref.decimate_normalize(B, VB, 96, 96, 1)
        req = 3125 // 16
        out[f"in_s{seed}"] = dict(pa=A, va=VA, pb=B, vb=VB)
        for name, mode, kw in [("denovo", 0, {}), ("prior", 2, dict(hfang=1.0)),
                               ("maxr", 4, dict(hfang=3.0)),
                               ("tweak", 0, dict(pretweak=1, rthresh=5.0)),
                               ("disc", 1, dict(disc=(3, 2, 10, 10), ang0=-th))]:
            res = ref.thm_search(A, VA, B, VB, req, mode=mode, **kw)
            args = dict(hfang=10.0, step=0.5, ang0=0.0, rthresh=0.3, pretweak=0,
                        disc=(0, 0, -1, -1))
            args.update(kw)
            out[f"thm_s{seed}_{name}"] = dict(
                ref_in=f"in_s{seed}", req=req, mode=mode, ang0=args["ang0"],
                hfang=args["hfang"], step=args["step"], rthresh=args["rthresh"],
                pretweak=args["pretweak"], disc=np.array(args["disc"]),
                A=res["A"], X=res["X"], Y=res["Y"], R=res["R"], err=res["err"])
    return out


def thm_finish_cases(ref):
    """PostTweaks from the de-novo result (identity and a skewed prior
    pretweak), FinishAtFullRes on the full-resolution tile (scale 4)."""
    out = {}
    for seed in (0, 2):
        ta, tb, th, t = synth.thumb_pair(seed, tile=768, dec=8)
        A, VA = O.image_to_points(ta)
        B, VB = O.image_to_points(tb)
        A, VA = ref.decimate_normalize(A, VA, 96, 96, 1)
        B, VB = ref.decimate_normalize(B, VB, 96, 96, 1)
        req = 3125 // 16
        best = ref.thm_search(A, VA, B, VB, req, mode=0)
        prior = np.array([best["A"], best["X"], best["Y"], best["R"]])
        out[f"in_s{seed}"] = dict(pa=A, va=VA, pb=B, vb=VB)
        for name, tw in (("id", None), ("skew", [1.0, 0.02, 0.0, 0.0, 0.99, 0.0])):
            res = ref.thm_finish(A, VA, B, VB, req, 5, prior, tptwk=tw)
            out[f"post_s{seed}_{name}"] = dict(
                ref_in=f"in_s{seed}", req=req, mode=5, prior=prior,
                tptwk=np.array(tw if tw is not None else [1, 0, 0, 0, 1, 0], np.float64),
                A=res["A"], X=res["X"], Y=res["Y"], R=res["R"], tptwk_out=res["tptwk"])
    ta, tb, th, t = synth.thumb_pair(7, tile=128, dec=4)
    fa, fb, _, _ = synth.thumb_pair(7, tile=128, dec=1)
    A, VA = O.image_to_points(ta)
    B, VB = O.image_to_points(tb)
    A, VA = ref.decimate_normalize(A, VA, 32, 32, 1)
    B, VB = ref.decimate_normalize(B, VB, 32, 32, 1)
    best = ref.thm_search(A, VA, B, VB, 100, mode=0)
    A1, V1 = O.image_to_points(fa)
    B1, W1 = O.image_to_points(fb)
    A1, V1 = ref.decimate_normalize(A1, V1, 128, 128, 1)
    B1, W1 = ref.decimate_normalize(B1, W1, 128, 128, 1)
    prior = np.array([best["A"], best["X"] * 4, best["Y"] * 4, best["R"]])
    res = ref.thm_finish(A1, V1, B1, W1, 1600, 6, prior)
    out["full_s7"] = dict(pa=A1.astype(np.int32), va=V1, pb=B1.astype(np.int32), vb=W1,
                          req=1600, mode=6, prior=prior,
                          tptwk=np.array([1, 0, 0, 0, 1, 0], np.float64),
                          A=res["A"], X=res["X"], Y=res["Y"], R=res["R"],
                          tptwk_out=res["tptwk"])
    return out


def thm_f_cases(ref):
    """The sweep with useCorrR off: RFromAngle through CorrImagesF."""
    out = {}
    ta, tb, th, t = synth.thumb_pair(3, tile=512, dec=8)
    A, VA = O.image_to_points(ta)
    B, VB = O.image_to_points(tb)
    A, VA = ref.decimate_normalize(A, VA, 64, 64, 1)
    B, VB = ref.decimate_normalize(B, VB, 64, 64, 1)
    req = 3125 // 64
    out["in_s3"] = dict(pa=A, va=VA, pb=B, vb=VB)
    for name, mode, kw in [("denovo", 0, {}), ("maxr", 4, dict(hfang=3.0))]:
        res = ref.thm_search(A, VA, B, VB, req, mode=mode, usecorrr=0, **kw)
        out[f"thmf_s3_{name}"] = dict(
            ref_in="in_s3", req=req, mode=mode, ang0=0.0, hfang=kw.get("hfang", 10.0),
            step=0.5, rthresh=0.3, pretweak=0, disc=np.array((0, 0, -1, -1)),
            A=res["A"], X=res["X"], Y=res["Y"], R=res["R"], err=res["err"])
    return out


def decimate_cases(ref):
    ta, tb, th, t = synth.thumb_pair(4, tile=512, dec=2)
    A, VA = O.image_to_points(ta.astype(np.float64))
    keep = np.random.default_rng(9).random(len(VA)) > 0.05
    A, VA = A[keep], VA[keep]
    xy, v = ref.decimate_normalize(A, VA, 256, 256, 8)
    return {"dec8": dict(pa=A, va=VA, w=256, h=256, lbin=8, xy=xy, v=v)}


def mesh_cases(ref):
    """GradDescStep / ImproveControlPts (0_GEN/Correlation.cpp:1403-1721):
    triangle and bilinear multipliers, several lattices, and the early exits
    (initial correlation below iniThresh; finThresh < 0 skips the search)."""
    out = {}
    specs = [("tri22", 1, "tri", (2, 2), 0.2, 0.5), ("quad21", 2, "quad", (2, 1), 0.2, 0.5),
             ("tri33", 3, "tri", (3, 3), 0.2, 0.5), ("quad33", 4, "quad", (3, 3), 0.2, 0.5),
             ("lowini", 5, "tri", (2, 2), 0.999, 0.5), ("skip", 6, "quad", (2, 2), 0.2, -1.0)]
    for name, seed, kind, cells, ini, fin in specs:
        c = synth.mesh_case(seed, box=(72, 60), cells=cells, kind=kind, field=140)
        bnew, d = ref.grad_desc_step(c["ac"], c["am_idx"], c["am_w"], c["av"], c["bimg"])
        cv, nnz = ref.corr_vectors(c["av"], bnew)
        r, ac = ref.improve_control_pts(c["ac"], c["am_idx"], c["am_w"], c["av"], c["bimg"],
                                        ini, fin)
        out["mesh_" + name] = dict(ac0=c["ac"], am_idx=c["am_idx"], am_w=c["am_w"], av=c["av"],
                                   bimg=c["bimg"], ini=ini, fin=fin, bnew0=bnew, drdc0=d,
                                   corr0=cv, nnz0=nnz, corr=r, ac=ac)
    return out


def approx_cases(ref):
    """ApproximateMatch's chain (1_DMesh/ApproximateMatch.cpp:115-194) through
    the reference's own functions: crop, thumbnails, denovo and prior
    sweeps, PostTweaks, FinishAtFullRes, the coordinate change, and the
    early exits (crop too small, LIMXY)."""
    out = {}
    specs = [("denovo", 1, {}, None), ("tweaks", 2, dict(tweaks=1), None),
             ("prior", 3, dict(mode_prior=1, hfangpr=2.0), "theta"),
             ("whole", 4, dict(xyconf=0.0, olap2d=20000), None),
             ("nocrop", 5, dict(olap2d=200000), None), ("limxy", 6, dict(limxy=1), None)]
    for name, seed, kw, ang in specs:
        c = synth.approx_tile_pair(seed, tile=384, shift=(70.0, 24.0))
        if ang:
            kw = dict(kw, ang0=round(-c["theta"] * 2) / 2)   # a prior near the truth
        prm = O.approx_defaults(olap2d=kw.pop("olap2d", 20000), **kw)
        r = ref.approx_match(c["a"], c["b"], c["tab"], **prm)
        out["approx_" + name] = dict(a=c["a"], b=c["b"], tab=np.array(c["tab"]),
                                     truth=np.array(c["truth"]),
                                     params=np.array([prm[k] for k in APPROX_KEYS], np.float64),
                                     status=r["status"], A=r["A"], X=r["X"], Y=r["Y"], R=r["R"],
                                     T=np.array(r["T"]), err=r["err"], sweep=np.array(r["sweep"]),
                                     crop=np.array(r["crop"]))
    return out


APPROX_KEYS = ("xyconf", "olap1d", "olap2d", "thmdec", "mode_prior", "ang0", "hfangdn",
               "hfangpr", "rthresh", "nbmaxht", "pretweak", "tweaks", "limxy")


def pixpair_cases(ref):
    """PixPair::Load's tile conditioning (0_GEN/CPixPair.cpp:209-494):
    Legendre flattening of orders 0-6, the DoG band-pass, downsampling."""
    out = {}
    for name, seed, order, r1, r2, mx, shape in [("o2", 1, 2, 0, 0, 0, (160, 224)),
                                                 ("o2dog", 2, 2, 3, 6, 0, (160, 224)),
                                                 ("o0down", 3, 0, 0, 0, 100, (192, 256)),
                                                 ("o6dogdown", 4, 6, 2, 4, 64, (192, 256))]:
        f = synth.field_np(seed * 17 + 3, *shape)
        yy, xx = np.mgrid[0:shape[0], 0:shape[1]]
        f = f + 25.0 * (xx / shape[1]) - 15.0 * (yy / shape[0]) ** 2   # a shading to flatten
        t = synth.to_u8(f)
        vfy, aln, scl = ref.pixpair_condition(t, order, r1, r2, mx)
        out["pixpair_" + name] = dict(tile=t, order=order, r1=r1, r2=r2, max1dpix=mx, scl=scl,
                                      vfy=vfy, aln=aln)
    return out


def save(name, d):
    flat = {}
    for case, fields in d.items():
        for k, v in fields.items():
            flat[f"{case}::{k}"] = np.asarray(v)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **flat)
    print(name, len(d), "cases")


def main():
    # the reference source tree: argv[1], else $ALN_REFERENCE_TREE / the tree
    # of the last reference build
    tree = sys.argv[1] if len(sys.argv) > 1 else None
    if O.build_ref(tree) is None:
        sys.exit("usage: make_golden.py <reference source tree>")
    ref = O.Ref()
    save("corr_patches", corr_patches_cases(ref))
    save("corr_images", corr_images_cases(ref))
    save("fft", fft_cases(ref))
    save("convolve", convolve_cases(ref))
    save("patch_to_image", patch_to_image_cases(ref))
    save("thm_scan", thm_cases(ref))
    save("thm_finish", thm_finish_cases(ref))
    save("thm_scan_f", thm_f_cases(ref))
    save("decimate", decimate_cases(ref))
    save("mesh", mesh_cases(ref))
    save("approx", approx_cases(ref))
    save("pixpair", pixpair_cases(ref))


if __name__ == "__main__":
    main()
