"""The continuous-batching server (aln_server_*): every reply equals the
result of the same request run alone, whatever batch it landed in; requests
submitted while batches run are admitted into later batches; spectrum keys
are reused across requests; waits are bounded."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMING = ("queue_ms", "total_ms", "batch_size")


def strip(d):
    return {k: v for k, v in d.items() if k not in TIMING}


def _thumbs(seed):
    import oracle
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    ta, tb, th, t = synth.thumb_pair(seed, tile=512, dec=8)
    A, VA = oracle.image_to_points(ta)
    B, VB = oracle.image_to_points(tb)
    VA = (VA - VA.mean()) / VA.std(ddof=1)
    VB = (VB - VB.mean()) / VB.std(ddof=1)
    return aln.thumbs_from_points(A, VA, B, VB, 200)


def _requests():
    """A mix: montage strips, uneven uint16 patches, CorrImages R/S, sweeps."""
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    reqs = []
    for s in range(6):
        p = synth.montage_pair(40 + s)
        reqs.append(("p", dict(a=p.a, b=p.b, ox=p.ox, oy=p.oy, radius=p.radius,
                               lg=aln.legal(aln.RGN_SECTION, 1500, 1500, 30000))))
    for s in range(8):
        p = synth.uneven_pair(60 + s, smax=300)
        reqs.append(("p", dict(a=p.a, b=p.b, ox=p.ox, oy=p.oy, radius=p.radius,
                               lg=aln.legal(aln.RGN_MIN, 8, 8, 0))))
    rng = np.random.default_rng(5)
    for s in range(4):
        reqs.append(("i", dict(kind=aln.CORR_S if s % 2 else aln.CORR_R,
                               a=rng.standard_normal((60, 70)), b=rng.standard_normal((80, 64)),
                               lg=aln.legal(aln.RGN_MIN, 0, 0, 300, aln.CNT_GT, 300))))
    for s in range(2):
        reqs.append(("s", dict(thumbs=_thumbs(70 + s))))
    return reqs


def _submit(srv, kind, kw):
    if kind == "p":
        return srv.submit_patches(**kw)
    if kind == "i":
        return srv.submit_images(**kw)
    return srv.submit_sweep(kw["thumbs"], mode=0)


@pytest.fixture(scope="module")
def reqs():
    return _requests()


def test_alone_equals_mixed(reqs):
    import alignment_projects_gb300 as aln
    srv = aln.Server(0, workers=2)
    try:
        alone = []
        for kind, kw in reqs:   # one at a time: each runs in a batch of one
            r = srv.wait(_submit(srv, kind, kw))
            assert r["batch_size"] == 1
            alone.append(r)
        # the same requests, twice over, from two submitting threads at once
        order = list(range(len(reqs))) * 2
        tickets = {}

        def feed(idx):
            for i in idx:
                tickets[_submit(srv, *reqs[i])] = i

        th = [threading.Thread(target=feed, args=(order[k::2],)) for k in range(2)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        got = {}
        while len(got) < len(order):
            for tk, rep in srv.collect(timeout_ms=1000):
                got[tk] = rep
        assert max(r["batch_size"] for r in got.values()) > 1
        for tk, rep in got.items():
            i = tickets[tk]
            assert strip(rep) == strip(alone[i]), (i, rep, alone[i])
            assert rep["status"] >= 0
        c = srv.counters()
        assert c["submitted"] == c["finished"] == len(reqs) + len(order)
        assert c["waiting"] == 0
    finally:
        srv.close()


def test_max_batch_and_spectrum_keys():
    import alignment_projects_gb300 as aln
    from alignment_projects_gb300 import synth
    srv = aln.Server(0, workers=1, max_batch=4)
    try:
        b = synth.plain_pair(400, n=120, margin=8).b
        lg = aln.legal(aln.RGN_MIN, 16, 16, 0)
        a_s = [synth.plain_pair(401 + s, n=110, margin=6).a for s in range(10)]
        plain = [srv.wait(srv.submit_patches(a, b, lg=lg, radius=30)) for a in a_s]
        tks = [srv.submit_patches(a, b, lg=lg, radius=30, b_key=1234) for a in a_s]
        keyed = [srv.wait(t) for t in tks]
        assert all(r["batch_size"] <= 4 for r in keyed)
        # keyed jobs take one column transform per column, an unkeyed one may
        # be segmented: the same peaks, values within FP32 rounding
        for k, p in zip(keyed, plain):
            assert (k["peak_x"], k["peak_y"], k["status"]) == (p["peak_x"], p["peak_y"],
                                                               p["status"])
            assert abs(k["r"] - p["r"]) <= 1e-6
            assert abs(k["dx"] - p["dx"]) <= 1e-4 and abs(k["dy"] - p["dy"]) <= 1e-4
        assert srv.counters()["spec_hits"] >= 8
    finally:
        srv.close()


def test_bounded_wait_and_bad_ticket():
    import alignment_projects_gb300 as aln
    srv = aln.Server(0, workers=1)
    try:
        t = srv.submit_sweep(_thumbs(90), mode=0)
        with pytest.raises(aln.AlnError) as e:
            srv.wait(t, timeout_ms=0)
        assert e.value.code == aln.native.ALN_ERR_TIMEOUT
        r = srv.wait(t)
        assert r["status"] == 0 and r["ncalls"] > 100
        with pytest.raises(aln.AlnError):
            srv.wait(t)                       # handed over already
        with pytest.raises(aln.AlnError):
            srv.wait(987654321, timeout_ms=0)  # never issued
    finally:
        srv.close()
