// Drives class CThmScan through the C++ drop-in (libaln_corr_shim.so) with
// the reference's call sequences (the ones ApproximateMatch and CThmUtil
// make).  Compiled against the shim's header (aln_thmscan.hpp), or, with
// -DALN_REFERENCE_HEADERS, against the reference's own 0_GEN/CThmScan.h to
// show that a caller built from the reference's headers links against the
// shim.  Reads cases from a binary file, writes one line per case:
//   A X Y R err ret t0 t1 t2 t3 t4 t5       (t: the object's Tptwk after)
//
// case record (little-endian): int32 mode, int32 na, double[2na] A points,
// double[na] A values, int32 nb, double[2nb], double[nb], int64 reqArea,
// int32 olap1D, double rthresh, nbmaxht, int32 pretweak, constxy, usecorrr,
// Ox, Oy, Rx, Ry, double ang0, hfang, step, double prior[4] (A X Y R),
// double tptwk[6]
// modes: 0 DenovoBestAngle, 1 RFromAngle, 2 UsePriorAngles,
// 3 AngleScanSel + PeakHunt, 4 AngleScanMaxR (favorCenter), 5 PostTweaks,
// 6 FinishAtFullRes, 7 Pretweaks then RFromAngle, 8 DenovoBestAngle with
// SetNewAngProc giving the case's disc for every angle (and SetDisc off),
// 9 DebugAngs(1, 2, 3, 4, ang0, hfang, step) (writes angs_1.2^3.4.log in
// the working directory; the line reports RFromAngle at ang0)
#ifdef ALN_REFERENCE_HEADERS
#include "CThmScan.h"
#else
#include "aln_thmscan.hpp"
#endif

#include <cstdint>
#include <cstdio>
#include <vector>

static int g_disc[4];
static int g_disc_calls = 0;

static void disc_proc(int &Ox, int &Oy, int &Rx, int &Ry, double deg)
{
    (void)deg;
    Ox = g_disc[0];
    Oy = g_disc[1];
    Rx = g_disc[2];
    Ry = g_disc[3];
    ++g_disc_calls;
}

template <typename T>
static bool rd(FILE *f, T &v)
{
    return fread(&v, sizeof v, 1, f) == 1;
}

static bool rd_cloud(FILE *f, std::vector<Point> &p, std::vector<double> &v)
{
    int32_t n;
    if (!rd(f, n))
        return false;
    p.resize(n);
    v.resize(n);
    for (int i = 0; i < n; ++i)
        if (!rd(f, p[i].x) || !rd(f, p[i].y))
            return false;
    for (int i = 0; i < n; ++i)
        if (!rd(f, v[i]))
            return false;
    return true;
}

int main(int argc, char **argv)
{
    if (argc < 2)
        return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f)
        return 2;
    FILE *flog = fopen(argc > 2 ? argv[2] : "/dev/null", "w");
    for (;;) {
        int32_t mode;
        if (!rd(f, mode))
            break;
        ThmRec thm;
        if (!rd_cloud(f, thm.ap, thm.av) || !rd_cloud(f, thm.bp, thm.bv))
            return 3;
        int64_t req;
        int32_t olap1d, pretweak, constxy, usecorrr, Ox, Oy, Rx, Ry;
        double rthresh, nbmaxht, ang0, hfang, step, prior[4], tp[6];
        rd(f, req);
        rd(f, olap1d);
        rd(f, rthresh);
        rd(f, nbmaxht);
        rd(f, pretweak);
        rd(f, constxy);
        rd(f, usecorrr);
        rd(f, Ox);
        rd(f, Oy);
        rd(f, Rx);
        rd(f, Ry);
        rd(f, ang0);
        rd(f, hfang);
        rd(f, step);
        for (double &v : prior)
            rd(f, v);
        for (double &v : tp)
            if (!rd(f, v))
                return 3;
        thm.ftc.clear();
        thm.reqArea = (long)req;
        thm.olap1D = olap1d;
        thm.scl = 1;

        CThmScan S;
        CorRec best;
        S.Initialize(flog, best);
        S.SetRThresh(rthresh);
        S.SetNbMaxHt(nbmaxht);
        S.SetSweepConstXY(constxy);
        S.SetSweepPretweak(pretweak);
        S.SetUseCorrR(usecorrr);
        S.SetDisc(Ox, Oy, Rx, Ry);
        TAffine T;
        for (int i = 0; i < 6; ++i)
            T.t[i] = tp[i];
        S.SetTptwk(T);
        double ret = 0.0;
        switch (mode) {
        case 0:
            ret = S.DenovoBestAngle(best, ang0, hfang, step, thm, true);
            break;
        case 1:
            S.RFromAngle(best, ang0, thm);
            break;
        case 2:
            ret = S.UsePriorAngles(best, 1, ang0, hfang, thm);
            break;
        case 3:
            S.AngleScanSel(best, ang0, hfang, step, false, thm);
            ret = S.PeakHunt(best, step * 0.05 * 1.5, thm);
            break;
        case 4:
            S.SetSweepConstXY(0);
            ret = S.AngleScanSel(best, ang0, hfang, step, true, thm);
            break;
        case 5:
        case 6:
            best.A = prior[0];
            best.X = prior[1];
            best.Y = prior[2];
            best.R = prior[3];
            if (mode == 5)
                S.PostTweaks(best, thm);
            else
                S.FinishAtFullRes(best, thm);
            break;
        case 7:
            ret = S.Pretweaks(0.0, ang0, thm);
            S.RFromAngle(best, ang0, thm);
            break;
        case 8:
            g_disc[0] = Ox;
            g_disc[1] = Oy;
            g_disc[2] = Rx;
            g_disc[3] = Ry;
            g_disc_calls = 0;
            S.SetDisc(0, 0, -1, -1);
            S.SetNewAngProc(disc_proc);
            ret = S.DenovoBestAngle(best, ang0, hfang, step, thm, true);
            ret += 10.0 * (g_disc_calls > 0);
            break;
        case 9:
            S.DebugAngs(1, 2, 3, 4, ang0, hfang, step, thm);
            S.RFromAngle(best, ang0, thm);
            break;
        default:
            return 4;
        }
        TAffine Tout;
        S.GetTptwk(Tout);
        printf("%.17g %.17g %.17g %.17g %d %.17g", best.A, best.X, best.Y, best.R, S.GetErr(),
               ret);
        for (int i = 0; i < 6; ++i)
            printf(" %.17g", Tout.t[i]);
        printf("\n");
    }
    fclose(f);
    fclose(flog);
    return 0;
}
