// aln_thmscan_shim.cpp -- libaln_corr_shim.so: class CThmScan of
// aln_thmscan.hpp over the C ABI of libaln_corr.so (GPU).
//
// Each public member function is one aln_thm_call_batch call: the sweep's
// angles (a scan, each bracket step of the peak hunt, the pretweak sweeps)
// run as GPU batches instead of one correlator call after another.  The
// object's state goes in and comes back: the CorRec the member function
// takes by reference, err, the pretweak transform Tptwk, and the disc and
// useCorrR that PostTweaks / FinishAtFullRes set.  On the host the shim only
// converts ThmRec: A's points (integer thumbnail pixels) to a value grid
// with a presence mask, B's points to a raster over their bounding box, the
// ftc vector to a spectrum-cache key.  There is no CPU fallback: a GPU
// failure is logged to flog and the call returns as the reference does
// when nothing correlates (R 0, false).
#include "aln_thmscan.hpp"

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/aln_corr.h"
#include "aln_shim_util.hpp"

namespace {

// the reference's ME (0_GEN/CThmScan.cpp:17): BigEnough reads its olap1D
CThmScan *g_me = nullptr;

// ThmRec -> aln_thumbs.  A: the bounding grid of the (integer) points, each
// present point's value (coincident points add, as their splats would), a
// mask of present points.  B: the points' raster over their bounding box.
struct ThumbsBuf {
    aln_thumbs t;
    std::vector<double> a, b;
    std::vector<unsigned char> mask;
};

bool thumbs_of(ThmRec &thm, ThumbsBuf &T, FILE *flog)
{
    memset(&T.t, 0, sizeof T.t);
    if (thm.ap.empty() || thm.bp.empty() || thm.av.size() != thm.ap.size() ||
        thm.bv.size() != thm.bp.size()) {
        fprintf(flog, "CThmScan (GPU): empty or mismatched thumbnail point lists\n");
        return false;
    }
    const aln_shim::IBoxD A = aln_shim::bbox(thm.ap);
    const int aw = A.R - A.L + 1, ah = A.T - A.B + 1;
    T.a.assign((size_t)aw * ah, 0.0);
    T.mask.assign((size_t)aw * ah, 0);
    for (size_t k = 0; k < thm.ap.size(); ++k) {
        const double x = thm.ap[k].x, y = thm.ap[k].y;
        if (x != floor(x) || y != floor(y)) {
            fprintf(flog, "CThmScan (GPU): thumbnail A points must lie on integer pixels\n");
            return false;
        }
        const size_t i = (size_t)((int)x - A.L) + (size_t)aw * (size_t)((int)y - A.B);
        T.a[i] += thm.av[k];
        T.mask[i] = 1;
    }
    const aln_shim::IBoxD B = aln_shim::bbox(thm.bp);
    T.b = aln_shim::raster(thm.bp, thm.bv, B);
    T.t.a = T.a.data();
    T.t.a_mask = T.mask.data();
    T.t.a_w = aw;
    T.t.a_h = ah;
    T.t.a_stride = aw;
    T.t.a_x0 = A.L;
    T.t.a_y0 = A.B;
    T.t.b = aln_shim::image_of(T.b, B);
    T.t.req_area = thm.reqArea;
    T.t.olap1d = thm.olap1D;
    // ftc: B's spectrum stays cached while the record keeps its key
    const int bw = B.R - B.L + 1, bh = B.T - B.B + 1;
    T.t.b_key = aln_shim::key_of(thm.ftc, (size_t)bw * bh + 1);
    return true;
}

void disc_tramp(void *user, double deg, int *ox, int *oy, int *rx, int *ry)
{
    (*(T_NewAngProc *)user)(*ox, *oy, *rx, *ry, deg);
}

}   // namespace

bool CThmScan::gpu_call(int op, CorRec &best, ThmRec &thm, double a0, double a1, double a2,
                        double a3, double *ret)
{
    g_me = this;
    olap1D = thm.olap1D;
    *ret = 0.0;
    ThumbsBuf T;
    if (!thumbs_of(thm, T, flog))
        return false;
    aln_thm_params P;
    memset(&P, 0, sizeof P);
    P.rthresh = rthresh;
    P.nbmaxht = nbmaxht;
    P.constxy = swpConstXY;
    P.pretweak = swpPretweak;
    P.usecorrr = useCorrR;
    P.ox = Ox;
    P.oy = Oy;
    P.rx = Rx;
    P.ry = Ry;
    memcpy(P.tdfm, Tdfm.t, sizeof P.tdfm);
    if (newAngProc) {
        P.disc_of_angle = disc_tramp;
        P.disc_user = &newAngProc;
    }
    aln_thm_result r;
    memset(&r, 0, sizeof r);
    r.A = best.A;
    r.X = best.X;
    r.Y = best.Y;
    r.R = best.R;
    memcpy(r.T, best.T.t, sizeof r.T);
    r.err = err;
    double tp[6], args[4] = {a0, a1, a2, a3};
    memcpy(tp, Tptwk.t, sizeof tp);
    aln_ctx *c = aln_shim::ctx();
    if (!c) {
        fprintf(flog, "CThmScan (GPU): no CUDA context\n");
        return false;
    }
    if (aln_thm_call_batch(c, 1, &T.t, &P, op, args, &r, tp, ret) < 0) {
        fprintf(flog, "CThmScan (GPU): %s\n", aln_last_error(c));
        *ret = 0.0;
        return false;
    }
    best.A = r.A;
    best.X = r.X;
    best.Y = r.Y;
    best.R = r.R;
    memcpy(best.T.t, r.T, sizeof r.T);
    err = r.err;
    memcpy(Tptwk.t, tp, sizeof tp);
    return true;
}

bool BigEnough(int sx, int sy, void *a)
{
    return sx >= g_me->olap1D && sy >= g_me->olap1D && (long)sx * sy > (long)a;
}

// Defaults of 0_GEN/CThmScan.cpp:161-178.
CThmScan::CThmScan()
{
    g_me = this;
    TCD.nthr = 1;
    TCD.thm = nullptr;
    newAngProc = nullptr;
    flog = stdout;
    rthresh = 0.30;
    nbmaxht = 0.75;
    err = errOK;
    swpConstXY = 1;
    swpPretweak = 1;
    swpNThreads = 1;
    useCorrR = 0;
    Ox = Oy = 0;
    Rx = Ry = -1;
    olap1D = 0;
}

void CThmScan::Initialize(FILE *flog, CorRec &best)
{
    SetFlog(flog);
    fprintf(flog, "\n---- Thumbnail matching ----\n");
    best.X = best.Y = best.A = best.R = -999.0;
}

bool CThmScan::Pretweaks(double bestR, double deg, ThmRec &thm)
{
    CorRec none;
    double ret;
    gpu_call(ALN_THMOP_PRETWEAKS, none, thm, bestR, deg, 0.0, 0.0, &ret);
    fprintf(flog, "Pretweaks (GPU): changed=%d, Tptwk [%g %g %g; %g %g %g]\n", ret != 0.0,
            Tptwk.t[0], Tptwk.t[1], Tptwk.t[2], Tptwk.t[3], Tptwk.t[4], Tptwk.t[5]);
    return ret != 0.0;
}

// iaux selects a pretweak sweep record of the reference's internal tables;
// callers outside CThmScan pass the default (-1), which is all this serves.
void CThmScan::RFromAngle(CorRec &C, double deg, ThmRec &thm, int iaux)
{
    (void)iaux;
    double ret;
    if (!gpu_call(ALN_THMOP_RFROMANGLE, C, thm, deg, 0.0, 0.0, 0.0, &ret)) {
        C.A = deg;
        C.R = C.X = C.Y = 0.0;
    }
}

// The angle table of 0_GEN/CThmScan.cpp:372-403 (file angs_<a>^<b>.log),
// every angle in one GPU batch.
void CThmScan::DebugAngs(int alyr, int atil, int blyr, int btil, double center, double hlfwid,
                         double step, ThmRec &thm)
{
    char file[256];
    snprintf(file, sizeof file, "angs_%d.%d^%d.%d.log", alyr, atil, blyr, btil);
    FILE *f = fopen(file, "w");
    if (!f)
        return;
    fprintf(f, "Deg\tR\tX\tY\n");
    std::vector<double> angs;
    for (double a = center - hlfwid; a <= center + hlfwid; a += step)
        angs.push_back(a);
    g_me = this;
    olap1D = thm.olap1D;
    ThumbsBuf T;
    aln_ctx *c = aln_shim::ctx();
    if (!angs.empty() && c && thumbs_of(thm, T, flog)) {
        aln_thm_params P;
        memset(&P, 0, sizeof P);
        P.rthresh = rthresh;
        P.nbmaxht = nbmaxht;
        P.constxy = swpConstXY;
        P.pretweak = swpPretweak;
        P.usecorrr = useCorrR;
        P.ox = Ox;
        P.oy = Oy;
        P.rx = Rx;
        P.ry = Ry;
        memcpy(P.tdfm, Tdfm.t, sizeof P.tdfm);
        if (newAngProc) {
            P.disc_of_angle = disc_tramp;
            P.disc_user = &newAngProc;
        }
        const size_t n = angs.size();
        std::vector<aln_thumbs> th(n, T.t);
        std::vector<aln_thm_result> r(n);
        std::vector<double> args(4 * n, 0.0), tp(6 * n);
        for (size_t k = 0; k < n; ++k) {
            memset(&r[k], 0, sizeof r[k]);
            args[4 * k] = angs[k];
            memcpy(&tp[6 * k], Tptwk.t, sizeof Tptwk.t);
        }
        if (aln_thm_call_batch(c, (int)n, th.data(), &P, ALN_THMOP_RFROMANGLE, args.data(),
                               r.data(), tp.data(), nullptr) < 0)
            fprintf(flog, "CThmScan (GPU): %s\n", aln_last_error(c));
        else
            for (size_t k = 0; k < n; ++k)
                fprintf(f, "%.3f\t%.4f\t%.3f\t%.3f\n", r[k].A, r[k].R, r[k].X, r[k].Y);
    }
    fclose(f);
}

double CThmScan::AngleScanMaxR(CorRec &best, double center, double hlfwid, double step,
                               bool favorCenter, ThmRec &thm)
{
    double ret;
    gpu_call(ALN_THMOP_SCAN_MAXR, best, thm, center, hlfwid, step, favorCenter ? 1.0 : 0.0,
             &ret);
    return ret;
}

double CThmScan::AngleScanConstXY(CorRec &best, double center, double hlfwid, double step,
                                  ThmRec &thm)
{
    double ret;
    gpu_call(ALN_THMOP_SCAN_CONSTXY, best, thm, center, hlfwid, step, 0.0, &ret);
    return ret;
}

double CThmScan::AngleScanSel(CorRec &best, double center, double hlfwid, double step,
                              bool favorCenter, ThmRec &thm)
{
    double ret;
    gpu_call(ALN_THMOP_SCAN_SEL, best, thm, center, hlfwid, step, favorCenter ? 1.0 : 0.0,
             &ret);
    return ret;
}

double CThmScan::AngleScanWithTweaks(CorRec &best, double center, double hlfwid, double step,
                                     ThmRec &thm)
{
    double ret;
    gpu_call(ALN_THMOP_SCAN_TWEAKS, best, thm, center, hlfwid, step, 0.0, &ret);
    return ret;
}

double CThmScan::PeakHunt(CorRec &best, double hlfwid, ThmRec &thm)
{
    double ret;
    gpu_call(ALN_THMOP_PEAKHUNT, best, thm, 0.0, hlfwid, 0.0, 0.0, &ret);
    fprintf(flog, "PeakHunt (GPU): R=%.3f, A=%.3f, X=%.3f, Y=%.3f\n", best.R, best.A, best.X,
            best.Y);
    return ret;
}

bool CThmScan::UsePriorAngles(CorRec &best, int nprior, double ang0, double hfangpr,
                              ThmRec &thm)
{
    fprintf(flog, "Approx: Using prior angles n=%d, med=%f\n", nprior, ang0);
    double ret;
    const bool ok = gpu_call(ALN_THMOP_PRIOR, best, thm, ang0, hfangpr, 0.0, 0.0, &ret);
    if (!ok || ret == 0.0) {
        fprintf(flog, "FAIL: Approx: Prior angles R=%g below thresh=%g\n", best.R, rthresh);
        err = errLowRPrior;
        return false;
    }
    return true;
}

bool CThmScan::DenovoBestAngle(CorRec &best, double ang0, double hfangdn, double step,
                               ThmRec &thm, bool failmsg)
{
    double ret;
    const bool ok = gpu_call(ALN_THMOP_DENOVO, best, thm, ang0, hfangdn, step, 0.0, &ret);
    if (!ok || ret == 0.0) {
        if (failmsg)
            fprintf(flog, "FAIL: Approx: Denovo R=%g below thresh=%g\n", best.R, rthresh);
        err = errLowRDenov;
        return false;
    }
    return true;
}

void CThmScan::PostTweaks(CorRec &best, ThmRec &thm)
{
    const int ox = (int)best.X, oy = (int)best.Y;
    double ret;
    gpu_call(ALN_THMOP_POSTTWEAKS, best, thm, 0.0, 0.0, 0.0, 0.0, &ret);
    SetUseCorrR(true);
    SetDisc(ox, oy, 40, 40);
}

void CThmScan::FinishAtFullRes(CorRec &best, ThmRec &thm)
{
    const int ox = (int)best.X, oy = (int)best.Y;
    fprintf(flog, "Approx: LowRes  R=%.3f, X=%.3f, Y=%.3f\n", best.R, best.X, best.Y);
    double ret;
    gpu_call(ALN_THMOP_FULLRES, best, thm, 0.0, 0.0, 0.0, 0.0, &ret);
    SetUseCorrR(true);
    SetDisc(ox, oy, 80, 80);
    fprintf(flog, "Approx: FullRes (GPU) R=%.3f, X=%.3f, Y=%.3f\n", best.R, best.X, best.Y);
}
