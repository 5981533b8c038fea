"""The ThmPair table (0_GEN/PipeFiles.h:146-152, PipeFiles.cpp:1129-1360):
the library writes the reference's header and line format and reads its
entries back (host file I/O, no GPU)."""
import os


def _recs():
    return [dict(atl=3, acr=0, btl=7, bcr=1, err=0, A=-2.264270019531, R=4.824218604,
                 T=[0.9992, -0.0395, -70.1335, 0.0395, 0.9992, -23.8165]),
            dict(atl=4, acr=0, btl=8, bcr=0, err=1, A=0.5, R=0.21,
                 T=[1.0, 0.0, 12.5, 0.0, 1.0, -3.25]),
            dict(atl=-1, acr=0, btl=9, bcr=0, err=0, A=0.0, R=0.0, T=[1, 0, 0, 0, 1, 0])]


def test_write_then_read(tmp_path):
    import alignment_projects_gb300 as aln
    d = str(tmp_path)
    aln.thmpair_write(d, 12, 13, _recs()[:2])
    aln.thmpair_write(d, 12, 13, _recs()[2:])   # a negative tile id is skipped
    text = open(os.path.join(d, "ThmPair_12^13.txt")).read().splitlines()
    assert text[0] == "Atl\tAcr\tBtl\tBcr\tErr\tDeg\tR\tT0\tT1\tX\tT3\tT4\tY"
    assert len(text) == 3
    r = _recs()[0]
    want = "%d\t%d\t%d\t%d\t%d\t%f\t%f\t%f\t%f\t%f\t%f\t%f\t%f" % (
        r["atl"], r["acr"], r["btl"], r["bcr"], r["err"], r["A"], r["R"], *r["T"])
    assert text[1] == want
    back = aln.thmpair_read(d, 12, 13)
    assert len(back) == 2
    for b, r in zip(back, _recs()[:2]):
        assert (b["atl"], b["acr"], b["btl"], b["bcr"], b["err"]) == \
               (r["atl"], r["acr"], r["btl"], r["bcr"], r["err"])
        assert abs(b["A"] - r["A"]) <= 5e-7 and abs(b["R"] - r["R"]) <= 5e-7
        assert max(abs(x - y) for x, y in zip(b["T"], r["T"])) <= 5e-7


def test_missing_table_raises(tmp_path):
    import pytest
    import alignment_projects_gb300 as aln
    with pytest.raises(aln.AlnError):
        aln.thmpair_read(str(tmp_path), 1, 2)
