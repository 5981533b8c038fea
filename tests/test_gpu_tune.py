"""The autotuner (aln_tune.cuh): measured column plans per CorrPatches pair
class, recorded per GPU and build, and held fixed once made."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pairs(seeds, smin, smax):
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    jobs, ps = [], []
    for s in seeds:
        p = synth.uneven_pair(s, smin=smin, smax=smax)
        ps.append(p)
        jobs.append(dict(a=p.a, b=p.b, ox=p.ox, oy=p.oy, radius=p.radius,
                         legal=aln.legal(aln.RGN_MIN, 8, 8, 0)))
    return jobs, ps


def _tune_file():
    import glob
    import alignment_projects_gb300 as aln
    d = os.environ.get("ALN_TUNE_DIR") or os.path.join(os.path.dirname(aln.lib_path()), "tune")
    files = glob.glob(os.path.join(d, "*.txt"))
    return files


def test_tuned_plans_meet_the_bar_and_stay_fixed(orc):
    """A batch of uneven uint16 pairs with tuning on: classes get measured
    (or were already), the choice file records them, every pair meets the
    oracle bar, a second context reuses the choices without timing, gives
    the same numbers bit for bit, and one pair alone gives its batch numbers."""
    import oracle
    import alignment_projects_gb300 as aln
    jobs, ps = _pairs(range(500, 512), 300, 900)
    c1 = aln.Context(0)
    c1.set_tuning(True)
    g1 = c1.corr_patches_batch(jobs)
    n1 = c1.counters()["tune_classes"]
    c1.close()
    assert _tune_file(), "no choice file written"
    lines = sum(len(open(f).read().splitlines()) for f in _tune_file())
    assert lines >= n1
    c2 = aln.Context(0)
    g2 = c2.corr_patches_batch(jobs)
    assert c2.counters()["tune_classes"] == 0   # every class already measured
    assert g1 == g2
    alone = c2.corr_patches(jobs[3]["a"], jobs[3]["b"], jobs[3]["ox"], jobs[3]["oy"],
                            jobs[3]["radius"], jobs[3]["legal"])
    assert alone == g1[3]
    c2.close()
    lo = oracle.legal(oracle.RGN_MIN, 8, 8, 0)
    for p, g in zip(ps, g1):
        A, VA = oracle.image_to_points(p.a)
        B, VB = oracle.image_to_points(p.b)
        o = orc.corr_patches(A, VA, B, VB, p.ox, p.oy, p.radius, lo)
        assert abs(g["r"] - o["r"]) <= 1e-4
        if o["r"] - o["second"] > 1e-3:
            assert (g["peak_x"], g["peak_y"]) == (o["bigx"], o["bigy"])
            assert abs(g["dx"] - o["dx"]) <= 0.01 and abs(g["dy"] - o["dy"]) <= 0.01


def test_fixed_and_tuned_plans_agree():
    """Tuning off (the fixed cost model) and on: the same peaks, r within
    the FP32 bar."""
    import alignment_projects_gb300 as aln
    jobs, _ = _pairs(range(520, 528), 200, 1000)
    c = aln.Context(0)
    c.set_tuning(False)
    fixed = c.corr_patches_batch(jobs)
    c.set_tuning(True)
    tuned = c.corr_patches_batch(jobs)
    c.close()
    for f, t in zip(fixed, tuned):
        assert (f["peak_x"], f["peak_y"]) == (t["peak_x"], t["peak_y"])
        assert abs(f["r"] - t["r"]) <= 1e-4


def test_parallel_planning_equals_single_pairs():
    """A batch large enough to plan on host threads (640 pairs, above the
    512-pair threshold) gives each pair the numbers it gets alone, bit for
    bit; classes the autotuner had not measured are planned again on the
    calling thread after the parallel pass (measuring runs GPU batches)."""
    import alignment_projects_gb300 as aln
    jobs, _ = _pairs(range(2000, 2640), 64, 400)
    c = aln.Context(0)
    c.set_tuning(True)
    got = c.corr_patches_batch(jobs)
    for k in range(0, len(jobs), 37):
        j = jobs[k]
        alone = c.corr_patches(j["a"], j["b"], j["ox"], j["oy"], j["radius"], j["legal"])
        assert alone == got[k], (k, alone, got[k])
    c.close()
