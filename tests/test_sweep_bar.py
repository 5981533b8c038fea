"""The sweep parity bar itself (oracle/sweep_bar.py), on the CPU: the
oracle's decision margins on the reference's golden sweeps, and mistakes
planted in a copy of the oracle's answer that the bar must catch."""
import copy

import pytest

from conftest import load_golden
from oracle.sweep_bar import SweepStats, check


def _search(orc, d):
    return orc.thm_search(d["pa"], d["va"], d["pb"], d["vb"], int(d["req"]),
                          rthresh=float(d["rthresh"]), pretweak=int(d["pretweak"]),
                          disc=tuple(int(v) for v in d["disc"]), mode=int(d["mode"]),
                          ang0=float(d["ang0"]), hfang=float(d["hfang"]),
                          step=float(d["step"]))


@pytest.fixture(scope="module")
def golden_runs(orc):
    return {c: _search(orc, d) for c, d in sorted(load_golden("thm_scan").items())}


def test_margins_on_golden_sweeps(golden_runs):
    for case, o in golden_runs.items():
        m = o["margins"]
        assert m["ndec"] > 0, case
        assert 0.0 <= m["mR"] and 0.0 <= m["tolA"], case
        if "maxr" in case or "disc" in case:
            # one maximum over a handful of well separated scores
            assert m["nties"] == 0 and m["tolA"] == 0.0, (case, m)
        if case.endswith("denovo"):
            # only PeakHunt's last bracket tests are ties: the answer can
            # move inside the bracket (half-width 0.0375 deg) and no farther
            assert 0.0 < m["tolA"] <= 2 * 0.5 * 0.05 * 1.5, (case, m)


def test_bar_accepts_the_oracle_itself(golden_runs):
    st = SweepStats()
    for case, o in golden_runs.items():
        st.add(check(dict(o), o, case))
    t = st.table()
    assert t["pairs"] == len(golden_runs) and t["angle_exact"] == t["pairs"]
    assert t["max_abs_dA_deg"] == 0.0 and t["max_rel_dR"] == 0.0


def test_bar_catches_planted_mistakes(golden_runs):
    caught = 0
    for case, o in golden_runs.items():
        m = o["margins"]
        # one fine-scan step (0.025 deg) off: a wrong branch beyond any tie
        if m["tolA"] < 0.025:
            bad = dict(o, A=o["A"] + 0.025)
            with pytest.raises(AssertionError):
                check(bad, o, case)
            caught += 1
        # a wrong err code where no rthresh test was a tie
        if not m["thr_tie"]:
            with pytest.raises(AssertionError):
                check(dict(o, err=o["err"] ^ 1), o, case)
        # the right angle with a sub-pixel offset 0.05 px off
        if m["mpk"] >= 1e-5:
            with pytest.raises(AssertionError):
                check(dict(o, X=o["X"] + 0.05), o, case)
        # the right angle with R 1e-3 off
        with pytest.raises(AssertionError):
            check(dict(o, R=o["R"] + 1e-3 * max(1.0, abs(o["R"]))), o, case)
    assert caught == len(golden_runs)


def test_bar_allows_a_move_inside_the_tie_bound(golden_runs):
    o = copy.deepcopy(golden_runs["thm_s0_denovo"])
    tol = o["margins"]["tolA"]
    assert tol > 0
    g = dict(o, A=o["A"] + 0.5 * tol, X=o["X"] + 0.03)
    rec = check(g, o, "inside")
    assert not rec["exact"] and rec["dxy"] is None
