"""GPU parity of the CThmScan sweep (0_GEN/CThmScan.cpp) against the
reference's golden sweep results and the oracle, through the C ABI.

The sweep is a discrete search: every comparison of two angles' S scores
steers it.  Where two compared scores differ by less than the FP32 error of
the correlator (~1e-6 relative) the GPU may take the other branch; the bar
is therefore: the same error code, the angle within 0.05 deg (the fine-scan
step is 0.025 deg), the score within 1e-3 relative, and -- when the angle
is the same -- the offsets within 0.01 px.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    yield c
    c.close()


def compare(g, ref, msg):
    assert g["err"] == int(ref["err"]), (msg, g, ref)
    A, R = float(ref["A"]), float(ref["R"])
    assert abs(g["A"] - A) <= 0.05, (msg, g, ref)
    assert abs(g["R"] - R) <= 1e-3 * max(1.0, abs(R)), (msg, g, ref)
    if abs(g["A"] - A) < 1e-9:
        assert abs(g["X"] - float(ref["X"])) <= 0.01 and abs(g["Y"] - float(ref["Y"])) <= 0.01, \
            (msg, g, ref)


@pytest.mark.parametrize("case", sorted(load_golden("thm_scan")))
def test_sweep_golden(ctx, case):
    import alignment_projects_gb300 as aln
    d = load_golden("thm_scan")[case]
    T = aln.thumbs_from_points(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]))
    disc = tuple(int(v) for v in d["disc"])
    g = ctx.thm_search_batch([T], rthresh=float(d["rthresh"]), pretweak=int(d["pretweak"]),
                             disc=disc, mode=int(d["mode"]), ang0=float(d["ang0"]),
                             hfang=float(d["hfang"]), step=float(d["step"]))[0]
    compare(g, d, case)


def test_sweep_batch_of_pairs_matches_oracle(ctx, orc):
    """Several thumbnail pairs in one call, against the oracle pair by pair."""
    import oracle
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    thumbs, refs = [], []
    for seed in range(4):
        ta, tb, th, t = synth.thumb_pair(40 + seed, tile=768, dec=8)
        A, VA = oracle.image_to_points(ta)
        B, VB = oracle.image_to_points(tb)
        A, VA = orc.decimate_normalize(A, VA, 96, 96, 1)
        B, VB = orc.decimate_normalize(B, VB, 96, 96, 1)
        thumbs.append(aln.thumbs_from_points(A, VA, B, VB, 195))
        refs.append(orc.thm_search(A, VA, B, VB, 195, mode=0))
    got = ctx.thm_search_batch(thumbs, mode=aln.THM_DENOVO)
    for k, (g, r) in enumerate(zip(got, refs)):
        compare(g, r, f"pair {k}")


@pytest.mark.parametrize("case", sorted(load_golden("thm_finish")))
def test_finish_golden(ctx, case):
    """PostTweaks / FinishAtFullRes from the reference's prior, against its
    golden results (the same bar as the sweep)."""
    import alignment_projects_gb300 as aln
    d = load_golden("thm_finish")[case]
    T = aln.thumbs_from_points(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]))
    prior = dict(zip("AXYR", (float(v) for v in d["prior"])))
    g = ctx.thm_finish_batch([T], int(d["mode"]), [prior], tptwk=[d["tptwk"]])[0]
    ref = dict(A=d["A"], X=d["X"], Y=d["Y"], R=d["R"], err=0)
    compare(g, ref, case)
    if abs(g["A"] - float(d["A"])) < 1e-9:
        assert np.abs(np.array(g["tptwk"]) - d["tptwk_out"]).max() <= 1e-6, (g, d["tptwk_out"])


@pytest.mark.parametrize("case", sorted(load_golden("thm_scan_f")))
def test_sweep_f_golden(ctx, case):
    """useCorrR off: every correlator call is CorrImagesF."""
    import alignment_projects_gb300 as aln
    d = load_golden("thm_scan_f")[case]
    T = aln.thumbs_from_points(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]))
    g = ctx.thm_search_batch([T], usecorrr=0, mode=int(d["mode"]), ang0=float(d["ang0"]),
                             hfang=float(d["hfang"]), step=float(d["step"]))[0]
    compare(g, d, case)
