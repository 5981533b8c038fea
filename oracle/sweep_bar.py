"""TEST INFRASTRUCTURE (the checker): the parity bar of the CThmScan angle
sweep (0_GEN/CThmScan.cpp) against the oracle, and its per-config error
table.

The sweep is a discrete search: every comparison of two scores (the ConstXY
ranking, the LineFit tests and the roundings they see, MaxR's maximum,
PeakHunt's bracket tests, the rthresh tests) steers it.  The oracle notes
each decision with its margin (oracle.SWEEP_EPS relative on scores,
oracle.SWEEP_EPS_PX on rounded offsets -- far above the FP32 correlator's
error).  The bar:

* no decision below the thresholds: the GPU lands on the identical angle
  (|dA| <= 1e-9 deg), with the same err code, R within 1e-4 relative and
  X, Y within 0.01 px;
* otherwise the angle may move by at most the oracle's tolA (the bracket
  PeakHunt held when it met its first tie; unbounded only after a tied
  ranking, rounding or threshold), and the err code may differ only after a
  tied rthresh test; at the identical angle the same R / X / Y bar holds
  unless the answer's own correlator peak was a tie.

Every pair lands in exactly one bucket of `SweepStats`, which is what the
bench prints per config.
"""
from __future__ import annotations

A_EXACT = 1e-9
R_TOL = 1e-4
PX_TOL = 0.01


def check(g: dict, o: dict, msg: str = "") -> dict:
    """Assert the bar for GPU result g against oracle result o (with its
    "margins"); returns the pair's error record."""
    m = o["margins"]
    from oracle import SWEEP_EPS
    if not m["thr_tie"]:
        assert g["err"] == o["err"], (msg, "err", g, o)
    dA = abs(g["A"] - o["A"])
    tied = m["nties"] > 0
    assert dA <= m["tolA"] + A_EXACT, (msg, "angle outside the tie bound", dA, m, g, o)
    rscale = max(1.0, abs(o["R"]))
    dR = abs(g["R"] - o["R"]) / rscale
    dxy = max(abs(g["X"] - o["X"]), abs(g["Y"] - o["Y"]))
    pk_tie = m["mpk"] < SWEEP_EPS
    if dA <= A_EXACT:
        assert dR <= R_TOL, (msg, "R", g, o)
        if not pk_tie:
            assert dxy <= PX_TOL, (msg, "X/Y", g, o)
    else:
        # a tied bracket test sent PeakHunt the other way inside its bracket:
        # both answers sit at the peak of R(angle), a whisker apart
        assert dR <= 10 * R_TOL, (msg, "R after a tied branch", g, o)
    return {"exact": dA <= A_EXACT, "tied": tied, "dA": dA, "dR": dR,
            "dxy": dxy if dA <= A_EXACT else None, "tolA": m["tolA"]}


class SweepStats:
    """Per-config error table: pairs, decisions with no tie (must be exact),
    exact angles, max |dA|, max relative |dR|, max |dX|,|dY| at the same
    angle."""

    def __init__(self):
        self.rows = []

    def add(self, rec: dict):
        self.rows.append(rec)

    def table(self) -> dict:
        r = self.rows
        return {
            "pairs": len(r),
            "untied": sum(1 for x in r if not x["tied"]),
            "untied_exact": sum(1 for x in r if not x["tied"] and x["exact"]),
            "angle_exact": sum(1 for x in r if x["exact"]),
            "max_abs_dA_deg": max((x["dA"] for x in r), default=0.0),
            "max_tolA_deg": max((x["tolA"] for x in r if x["tolA"] < 1e29), default=0.0),
            "max_rel_dR": max((x["dR"] for x in r), default=0.0),
            "max_abs_dxy_same_angle": max((x["dxy"] for x in r if x["dxy"] is not None),
                                          default=0.0),
        }
