"""GPU parity of the mesh optimizer (GradDescStep, CorrVectors and
ImproveControlPts, 0_GEN/Correlation.cpp:1403-1721) against the reference's
golden results and the oracle, through the C ABI.

Per-point arithmetic is the reference's, in its order; the sums over the
points run in a fixed blocked order on the GPU instead of one sequential
loop, so the numbers agree to FP64 rounding of those sums: bnew and dRdc
within 1e-9 relative, correlations within 1e-9, optimised control points
within 1e-6 px (the step rule takes the same branches), and the same number
of gradient evaluations.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

CORR_TOL = 1e-9
PT_TOL = 1e-6


@pytest.fixture(scope="module")
def ctx():
    import alignment_projects_gb300 as aln
    c = aln.Context(0)
    yield c
    c.close()


def _job(d, ac=None):
    import alignment_projects_gb300 as aln
    return aln.mesh_job(d["ac0"] if ac is None else ac, d["am_idx"], d["am_w"], d["av"],
                        d["bimg"], float(d["ini"]), float(d["fin"]))


@pytest.mark.parametrize("case", sorted(load_golden("mesh")))
def test_grad_desc_step_golden(ctx, case):
    d = load_golden("mesh")[case]
    bnew, drdc, corr = ctx.grad_desc_step(_job(d))
    assert np.abs(bnew - d["bnew0"]).max() <= 1e-9 * max(1.0, np.abs(d["bnew0"]).max())
    assert np.abs(drdc - d["drdc0"]).max() <= 1e-9 * max(1.0, np.abs(d["drdc0"]).max())
    assert abs(corr - float(d["corr0"])) <= CORR_TOL
    # CorrVectors on the reference's own bnew: the same products, summed in blocks
    cv, nnz = ctx.corr_vectors(d["av"], d["bnew0"])
    assert abs(cv - float(d["corr0"])) <= CORR_TOL and nnz == int(d["nnz0"])


@pytest.mark.parametrize("case", sorted(load_golden("mesh")))
def test_improve_control_pts_golden(ctx, orc, case):
    d = load_golden("mesh")[case]
    g = ctx.improve_control_pts_batch([_job(d)])[0]
    assert abs(g["corr"] - float(d["corr"])) <= CORR_TOL, (g["corr"], float(d["corr"]))
    assert np.abs(g["ac"] - d["ac"]).max() <= PT_TOL, (g["ac"], d["ac"])
    r, ac, it = orc.improve_control_pts(d["ac0"], d["am_idx"], d["am_w"], d["av"], d["bimg"],
                                        float(d["ini"]), float(d["fin"]))
    assert g["evals"] == it


def test_batch_equals_single_and_repeats(ctx):
    """Every golden mesh in one call gives each job the numbers it gets
    alone, bit for bit, and a second run repeats them."""
    cases = load_golden("mesh")
    names = sorted(cases)
    alone = [ctx.improve_control_pts_batch([_job(cases[n])])[0] for n in names]
    both = ctx.improve_control_pts_batch([_job(cases[n]) for n in names])
    again = ctx.improve_control_pts_batch([_job(cases[n]) for n in names])
    for a, b, c in zip(alone, both, again):
        assert a["corr"] == b["corr"] == c["corr"]
        assert np.array_equal(a["ac"], b["ac"]) and np.array_equal(b["ac"], c["ac"])
        assert a["evals"] == b["evals"] == c["evals"]


@pytest.mark.parametrize("seed,kind,cells", [(11, "tri", (4, 4)), (12, "quad", (6, 3))])
def test_large_region_matches_oracle(ctx, orc, seed, kind, cells):
    """A 400 x 320 region (128k points, many blocks per job) and finer
    lattices, against the oracle."""
    from alignment_projects_gb300 import synth
    import alignment_projects_gb300 as aln
    c = synth.mesh_case(seed, box=(400, 320), cells=cells, kind=kind, field=480)
    r, ac, it = orc.improve_control_pts(c["ac"], c["am_idx"], c["am_w"], c["av"], c["bimg"],
                                        0.2, 0.5)
    g = ctx.improve_control_pts_batch([aln.mesh_job(c["ac"], c["am_idx"], c["am_w"], c["av"],
                                                    c["bimg"], 0.2, 0.5)])[0]
    assert abs(g["corr"] - r) <= CORR_TOL
    assert np.abs(g["ac"] - ac).max() <= PT_TOL
    assert g["evals"] == it
    # the optimiser moves the lattice toward the synthetic warp
    assert np.abs(g["ac"] - c["truth"]).max() < np.abs(c["ac"] - c["truth"]).max()


def test_bad_jobs_raise(ctx):
    import alignment_projects_gb300 as aln
    d = load_golden("mesh")["mesh_tri22"]
    J = _job(d)
    J.nc = 0
    with pytest.raises(aln.AlnError):
        ctx.improve_control_pts_batch([J])
