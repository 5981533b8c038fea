"""PixPair::Load's tile conditioning on the GPU (aln_pixpair_condition:
LegPolyFlatten, Normalize, the DoG band-pass, downsampling; 0_GEN/
CPixPair.cpp:209-494) against the reference's own functions
(tests/golden/pixpair.npz).  The per-pixel arithmetic is the reference's;
sums over all pixels run in blocks, and the DoG convolution uses FP32
transforms, so: 1e-9 without DoG, 1e-4 (of the unit sd) with it."""
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


@pytest.mark.parametrize("case", sorted(load_golden("pixpair")))
def test_conditioning_golden(ctx, case):
    d = load_golden("pixpair")[case]
    vfy, aln_, scl = ctx.pixpair_condition(d["tile"], int(d["order"]), int(d["r1"]),
                                           int(d["r2"]), int(d["max1dpix"]))
    assert scl == int(d["scl"])
    assert np.abs(vfy - d["vfy"]).max() <= 1e-9
    tol = 1e-4 if int(d["r2"]) > 0 else 1e-9
    assert np.abs(aln_ - d["aln"]).max() <= tol, np.abs(aln_ - d["aln"]).max()


def test_conditioning_repeats_and_rejects_bad_sizes(ctx):
    import alignment_projects_gb300 as aln
    d = load_golden("pixpair")["pixpair_o2"]
    a = ctx.pixpair_condition(d["tile"], 2)
    b = ctx.pixpair_condition(d["tile"], 2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    with pytest.raises(aln.AlnError):
        ctx.pixpair_condition(d["tile"][:99, :150], 2, max1dpix=64)   # 99 not a multiple of 2
