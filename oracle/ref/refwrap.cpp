/*
 * refwrap.cpp -- extern "C" entry points into the reference's own,
 * unmodified correlation code (compiled from its sources by
 * oracle/ref/Makefile into oracle/_ref/libalnref.so).
 *
 * TEST INFRASTRUCTURE ONLY: used to pin the C restatement (oracle/aln_oracle.c)
 * and to generate the golden fixtures under tests/golden/.  The product never
 * links it.  Only the reference's public functions are called:
 *   CorrPatches       0_GEN/Correlation.cpp:901-1170
 *   CorrPatchToImage  0_GEN/Correlation.cpp:1186-1355
 *   CorrImagesF/R/S   0_GEN/Correlation.cpp:3066-3290
 *   FFT_2D / IFT_2D   0_GEN/Correlation_fft_fftw.cpp:36-92
 *   Convolve          0_GEN/Correlation.cpp:371-457
 *   CThmScan          0_GEN/CThmScan.cpp (configured as 1_DMesh/ApproximateMatch.cpp:147-154)
 *   DecimateVector / Normalize  0_GEN/Maths.cpp:1315-1364, 192-212
 */
#include "Correlation.h"
#include "CThmScan.h"
#include "Maths.h"
#include "TAffine.h"

#include "../../include/aln_corr.h"

#include <stdio.h>
#include <string.h>

#include <vector>
using namespace std;

static FILE *quiet_log()
{
    static FILE *f = fopen("/dev/null", "w");
    return f;
}

static void to_points(vector<Point> &p, vector<double> &v, int n,
                      const double *xy, const double *val)
{
    p.resize(n);
    v.resize(n);
    for (int i = 0; i < n; ++i) {
        p[i] = Point(xy[2 * i], xy[2 * i + 1]);
        v[i] = val[i];
    }
}

/* The typed legality descriptor evaluated as an EvalType callback. */
static bool rgn_cb(int sx, int sy, void *a)
{
    const aln_legal *L = (const aln_legal *)a;
    switch (L->rgn_kind) {
    case ALN_RGN_MIN:
        return sx >= L->rgn_a && sy >= L->rgn_b && (long long)sx * sy > L->rgn_area;
    case ALN_RGN_SECTION:
        return (long long)sx * sy > L->rgn_area && (sx >= L->rgn_a || sy > L->rgn_b);
    case ALN_RGN_EXACT:
        return sx == L->rgn_a && sy == L->rgn_b;
    case ALN_RGN_TABLE:
        if (sx < 1 || sy < 1 || sx > L->table_w || sy > L->table_h)
            return false;
        return L->table[(size_t)(sy - 1) * L->table_w + (sx - 1)] != 0;
    default:
        return true;
    }
}

static bool cnt_cb(int c1, int c2, void *a)
{
    const aln_legal *L = (const aln_legal *)a;
    return c1 > L->cnt_n && c2 > L->cnt_n;
}

extern "C" {

double ref_corr_patches(int n1, const double *xy1, const double *v1,
                        int n2, const double *xy2, const double *v2,
                        int Ox, int Oy, int radius, const aln_legal *L,
                        double *dx, double *dy)
{
    vector<Point> p1, p2;
    vector<double> a1, a2;
    vector<CD> ftc;
    to_points(p1, a1, n1, xy1, v1);
    to_points(p2, a2, n2, xy2, v2);
    EvalType lr = (L && L->rgn_kind != ALN_RGN_NONE) ? rgn_cb : NULL;
    EvalType lc = (L && L->cnt_kind == ALN_CNT_GT) ? cnt_cb : NULL;
    return CorrPatches(quiet_log(), false, *dx, *dy, p1, a1, p2, a2, Ox, Oy,
                       radius, lr, (void *)L, lc, (void *)L, ftc);
}

/* kind: 0 = CorrImagesF, 1 = CorrImagesR, 2 = CorrImagesS */
double ref_corr_images(int kind, int n1, const double *xy1, const double *v1,
                       int n2, const double *xy2, const double *v2,
                       const aln_legal *L, double mincor, double nbmaxht,
                       int Ox, int Oy, int Rx, int Ry, double *dx, double *dy)
{
    vector<Point> p1, p2;
    vector<double> a1, a2;
    vector<CD> ftc;
    to_points(p1, a1, n1, xy1, v1);
    to_points(p2, a2, n2, xy2, v2);
    EvalType lr = (L && L->rgn_kind != ALN_RGN_NONE) ? rgn_cb : NULL;
    EvalType lc = (L && L->cnt_kind == ALN_CNT_GT) ? cnt_cb : NULL;
    double (*fn)(FILE *, int, double &, double &, const vector<Point> &,
                 const vector<double> &, const vector<Point> &,
                 const vector<double> &, EvalType, void *, EvalType, void *,
                 double, double, int, int, int, int, vector<CD> &) =
        kind == 0 ? CorrImagesF : kind == 1 ? CorrImagesR : CorrImagesS;
    return fn(quiet_log(), false, *dx, *dy, p1, a1, p2, a2, lr, (void *)L, lc,
              (void *)L, mincor, nbmaxht, Ox, Oy, Rx, Ry, ftc);
}

double ref_corr_patch_to_image(int n1, const double *xy1, const double *v1,
                               int n2sq, const double *i2, int Ox, int Oy,
                               int radius, int bFilter, double *dx, double *dy)
{
    vector<Point> p1;
    vector<double> a1;
    to_points(p1, a1, n1, xy1, v1);
    vector<double> im2(i2, i2 + n2sq);
    /* CorrPatchToImage prints its report on stdout */
    fflush(stdout);
    return CorrPatchToImage(*dx, *dy, p1, a1, im2, Ox, Oy, radius, bFilter != 0);
}

int ref_fft_2d(const double *in, int nfast, int nslow, double *out)
{
    vector<double> vin(in, in + (size_t)nfast * nslow);
    vector<CD> vout;
    int M = FFT_2D(vout, vin, nfast, nslow, false, quiet_log());
    memcpy(out, &vout[0], sizeof(CD) * (size_t)M);
    return M;
}

int ref_ift_2d(const double *in, int nfast, int nslow, double *out)
{
    size_t M = (size_t)nslow * (nfast / 2 + 1);
    vector<CD> vin((const CD *)in, (const CD *)in + M);
    vector<double> vout;
    IFT_2D(vout, vin, nfast, nslow, quiet_log());
    memcpy(out, &vout[0], sizeof(double) * vout.size());
    return 0;
}

void ref_convolve(double *dst, const double *src, int ws, int hs,
                  const double *K, int wk, int hk, int sym, int prenorm)
{
    vector<double> s(src, src + (size_t)ws * hs), d;
    vector<CD> kfft;
    Convolve(d, s, ws, hs, K, wk, hk, sym != 0, prenorm != 0, kfft, quiet_log());
    memcpy(dst, &d[0], sizeof(double) * d.size());
}

void ref_parab_peak_fft(double *xpk, double *ypk, int d, const double *I,
                        int nx, int ny)
{
    ParabPeakFFT(*xpk, *ypk, d, I, nx, ny);
}

/* DecimateVector + Normalize as 1_DMesh/CThmUtil.cpp:470-523 applies them.
 * Points are replaced in place; returns the new count. */
int ref_decimate_normalize(int n, double *xy, double *v, int w, int h, int lbin,
                           int normalize)
{
    vector<Point> p;
    vector<double> a;
    to_points(p, a, n, xy, v);
    DecimateVector(p, a, w, h, lbin);
    if (normalize)
        Normalize(a);
    int k = (int)p.size();
    for (int i = 0; i < k; ++i) {
        xy[2 * i] = p[i].x;
        xy[2 * i + 1] = p[i].y;
        v[i] = a[i];
    }
    return k;
}

/*
 * One CThmScan search configured as ApproximateMatch does
 * (1_DMesh/ApproximateMatch.cpp:147-154), on thumbnails already built.
 * mode: 0 = DenovoBestAngle(ang0, hfang, step), 1 = RFromAngle(ang0) with the
 * disc, 2 = UsePriorAngles(ang0, hfang), 3 = AngleScanSel(ang0, hfang, step)
 * then PeakHunt(step*0.05*1.5) (no thresholds), 4 = AngleScanMaxR.
 * out[0..3] = A, X, Y, R of the best record; returns GetErr() (or 0/1 for
 * the success flag in modes 0 and 2 as err).
 */
int ref_thm_search(int na, const double *xya, const double *va,
                   int nb, const double *xyb, const double *vb,
                   long reqArea, int olap1D, double rthresh, double nbmaxht,
                   int pretweak, int constxy, int usecorrr,
                   int Ox, int Oy, int Rx, int Ry,
                   int mode, double ang0, double hfang, double step,
                   const double *tdfm6, double *out, const char *logpath)
{
    FILE *flog = logpath ? fopen(logpath, "w") : quiet_log();
    ThmRec thm;
    to_points(thm.ap, thm.av, na, xya, va);
    to_points(thm.bp, thm.bv, nb, xyb, vb);
    thm.ftc.clear();
    thm.reqArea = reqArea;
    thm.olap1D = olap1D;
    thm.scl = 1;

    CThmScan S;
    CorRec best;
    S.Initialize(flog, best);
    if (tdfm6)
        S.SetTdfm(TAffine(tdfm6));
    S.SetRThresh(rthresh);
    S.SetNbMaxHt(nbmaxht);
    S.SetSweepConstXY(constxy);
    S.SetSweepPretweak(pretweak);
    S.SetUseCorrR(usecorrr);
    S.SetDisc(Ox, Oy, Rx, Ry);

    int ok = 1;
    switch (mode) {
    case 0:
        ok = S.DenovoBestAngle(best, ang0, hfang, step, thm, true);
        break;
    case 1:
        S.RFromAngle(best, ang0, thm);
        break;
    case 2:
        ok = S.UsePriorAngles(best, 1, ang0, hfang, thm);
        break;
    case 3:
        S.AngleScanSel(best, ang0, hfang, step, false, thm);
        S.PeakHunt(best, step * 0.05 * 1.5, thm);
        break;
    case 4:
        S.SetSweepConstXY(0);
        S.AngleScanSel(best, ang0, hfang, step, true, thm);
        break;
    }
    out[0] = best.A;
    out[1] = best.X;
    out[2] = best.Y;
    out[3] = best.R;
    if (logpath)
        fclose(flog);
    (void)ok;
    return S.GetErr();
}

/*
 * CThmScan's finishing stages from a prior best record and pretweak
 * transform: mode 5 = PostTweaks(best, thm) (0_GEN/CThmScan.cpp:796-802),
 * 6 = FinishAtFullRes(best, thm) (:810-842), thm being the full-resolution
 * record there.  prior[0..3] = A, X, Y, R; out[0..3] = A, X, Y, R after,
 * out[4..9] = the pretweak transform after.
 */
int ref_thm_finish(int na, const double *xya, const double *va,
                   int nb, const double *xyb, const double *vb,
                   long reqArea, int olap1D, double rthresh, double nbmaxht,
                   int pretweak, int constxy, int usecorrr, int mode,
                   const double *prior, const double *tptwk6, const double *tdfm6,
                   double *out)
{
    FILE *flog = quiet_log();
    ThmRec thm;
    to_points(thm.ap, thm.av, na, xya, va);
    to_points(thm.bp, thm.bv, nb, xyb, vb);
    thm.ftc.clear();
    thm.reqArea = reqArea;
    thm.olap1D = olap1D;
    thm.scl = 1;

    CThmScan S;
    CorRec best;
    S.Initialize(flog, best);
    if (tdfm6)
        S.SetTdfm(TAffine(tdfm6));
    if (tptwk6)
        S.SetTptwk(TAffine(tptwk6));
    S.SetRThresh(rthresh);
    S.SetNbMaxHt(nbmaxht);
    S.SetSweepConstXY(constxy);
    S.SetSweepPretweak(pretweak);
    S.SetUseCorrR(usecorrr);
    best.A = prior[0];
    best.X = prior[1];
    best.Y = prior[2];
    best.R = prior[3];
    if (mode == 5)
        S.PostTweaks(best, thm);
    else
        S.FinishAtFullRes(best, thm);
    out[0] = best.A;
    out[1] = best.X;
    out[2] = best.Y;
    out[3] = best.R;
    TAffine T;
    S.GetTptwk(T);
    for (int i = 0; i < 6; ++i)
        out[4 + i] = T.t[i];
    return S.GetErr();
}

} /* extern "C" */
