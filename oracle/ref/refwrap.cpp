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
 *   GradDescStep / CorrVectors / ImproveControlPts  0_GEN/Correlation.cpp:1403-1721
 *   BoxesFromShifts / BBoxFromPoints  0_GEN/Geometry.cpp:78-176
 *   LegPolyFlatten / Normalize  0_GEN/Maths.cpp:1006-1085, 192-212
 * ref_approx_match chains them as 1_DMesh/ApproximateMatch.cpp does; the
 * few lines of 1_DMesh/CThmUtil.cpp it needs (that file is not compiled
 * here) are restated beside it.
 */
#include "Correlation.h"
#include "CThmScan.h"
#include "Maths.h"
#include "TAffine.h"
#include "Geometry.h"
#include <math.h>

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


/* The reference's dense multiplier rows from the compressed form
 * (row i: slots am_idx[i*k + s] / am_w[i*k + s], index -1 unused). */
static void dense_am(vector<vector<double> > &am, int nm, int nc, int k,
                     const int *am_idx, const double *am_w)
{
    am.assign(nm, vector<double>(nc, 0.0));
    for (int i = 0; i < nm; ++i)
        for (int s = 0; s < k; ++s)
            if (am_idx[(size_t)i * k + s] >= 0)
                am[i][am_idx[(size_t)i * k + s]] = am_w[(size_t)i * k + s];
}

void ref_grad_desc_step(double *bnew, double *dRdc, const double *ac, int nc,
                        const int *am_idx, const double *am_w, int k, int nm,
                        const double *av, const double *bimg, int w, int h)
{
    vector<vector<double> > am;
    dense_am(am, nm, nc, k, am_idx, am_w);
    vector<Point> c(nc), d;
    for (int j = 0; j < nc; ++j)
        c[j] = Point(ac[2 * j], ac[2 * j + 1]);
    vector<double> a(av, av + nm), b(bimg, bimg + (size_t)w * h), bn;
    GradDescStep(bn, d, c, am, a, b, w, h);
    for (int i = 0; i < nm; ++i)
        bnew[i] = bn[i];
    for (int j = 0; j < nc; ++j) {
        dRdc[2 * j] = d[j].x;
        dRdc[2 * j + 1] = d[j].y;
    }
}

double ref_corr_vectors(const double *a, const double *b, int n, int *nnz)
{
    vector<double> va(a, a + n), vb(b, b + n);
    return CorrVectors(quiet_log(), va, vb, nnz);
}

double ref_improve_control_pts(double *ac, int nc, const int *am_idx, const double *am_w,
                               int k, int nm, const double *av, const double *bimg, int w,
                               int h, double ini_thresh, double fin_thresh)
{
    vector<vector<double> > am;
    dense_am(am, nm, nc, k, am_idx, am_w);
    vector<Point> c(nc);
    for (int j = 0; j < nc; ++j)
        c[j] = Point(ac[2 * j], ac[2 * j + 1]);
    vector<double> a(av, av + nm), b(bimg, bimg + (size_t)w * h);
    double r = ImproveControlPts(c, am, a, b, w, h, quiet_log(), "golden", ini_thresh,
                                 fin_thresh);
    for (int j = 0; j < nc; ++j) {
        ac[2 * j] = c[j].x;
        ac[2 * j + 1] = c[j].y;
    }
    return r;
}


/* CThmUtil's SubI (1_DMesh/CThmUtil.h): points relative to their bbox. */
struct SubIRec {
    vector<double> v;
    vector<Point> p;
    Point O;
    int w, h;
};

/* SubI_ThesePoints, 1_DMesh/CThmUtil.cpp:163-189 (values of a w-wide raster) */
static void subi_these(SubIRec &S, const double *v, int w, const vector<Point> &p)
{
    IBox B;
    BBoxFromPoints(B, p);
    S.v.resize(p.size());
    S.p.resize(p.size());
    for (size_t i = 0; i < p.size(); ++i) {
        S.v[i] = v[int(p[i].x) + w * int(p[i].y)];
        S.p[i].x = p[i].x - B.L;
        S.p[i].y = p[i].y - B.B;
    }
    S.O = Point(B.L, B.B);
    S.w = B.R - B.L + 1;
    S.h = B.T - B.B + 1;
}

/* MakeThumbs, 1_DMesh/CThmUtil.cpp:470-523 */
static bool make_thumbs(ThmRec &thm, const SubIRec &a, const SubIRec &b, int dec, long olap2d,
                        int olap1d)
{
    thm.av = a.v;
    thm.bv = b.v;
    thm.ap = a.p;
    thm.bp = b.p;
    thm.ftc.clear();
    thm.reqArea = olap2d;
    thm.olap1D = olap1d;
    thm.scl = dec;
    if (dec > 1) {
        DecimateVector(thm.ap, thm.av, a.w, a.h, dec);
        DecimateVector(thm.bp, thm.bv, b.w, b.h, dec);
        thm.reqArea /= dec * dec;
        thm.olap1D /= dec;
    }
    if ((long)thm.ap.size() < thm.reqArea)
        return false;
    if (!Normalize(thm.av) || !Normalize(thm.bv))
        return false;
    return true;
}

/*
 * ApproximateMatch (1_DMesh/ApproximateMatch.cpp:115-194) for one pair of
 * w x h tiles whose connected regions are the whole tiles, px.scl = 1,
 * Tdfm = identity, MODE 'C' (mode_prior = 1: UsePriorAngles from ang0 with
 * HFANGPR) or a denovo sweep (mode_prior = 0: DenovoBestAngle(ang0, HFANGDN,
 * 0.5)); Tab = the translation (tabx, taby) of a into b.  Crop with XYCONF
 * (CThmUtil.cpp:385-426), MakeThumbs(THMDEC), the sweep, Finish
 * (CThmUtil.cpp:889-971: PostTweaks when TWEAKS, X, Y scaled back,
 * MakeThumbs(1), FinishAtFullRes, IsectToImageCoords, Check_LIMXY).
 * Returns 0 ok, 1 crop too small, 2 thumbnails too small or flat, 3 sweep
 * failed, 4 LIMXY rejection.  out[0..3] A, X, Y, R; out[4..9] T;
 * out[10] err; out[11..14] the sweep's A, X, Y, R; out[15..18] the crop
 * origins aO, bO; out[19..20] the crop size.
 */
int ref_approx_match(const double *a, const double *b, int w, int h, double tabx,
                     double taby, double xyconf, int olap1d, long olap2d, int thmdec,
                     int mode_prior, double ang0, double hfangdn, double hfangpr,
                     double rthresh, double nbmaxht, int pretweak, int tweaks, int limxy,
                     double *out)
{
    FILE *flog = quiet_log();
    for (int i = 0; i < 21; ++i)
        out[i] = 0.0;
    vector<Point> all;
    all.reserve((size_t)w * h);
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x)
            all.push_back(Point(x, y));
    SubIRec oa, ob;
    bool whole = xyconf == 0.0;
    IBox Ba, Bb;
    if (!whole) {
        const int dx = int(xyconf * tabx), dy = int(xyconf * taby);
        BoxesFromShifts(Ba, Bb, w, h, w, h, dx, dy);
        const int ow = Ba.R - Ba.L + 1, oh = Ba.T - Ba.B + 1;
        const int min1d = olap1d > 8 ? olap1d : 8;
        whole = ow < min1d || oh < min1d;
    }
    if (whole) {
        subi_these(oa, a, w, all);
        subi_these(ob, b, w, all);
    } else {
        const IBox *Bx[2] = {&Ba, &Bb};
        SubIRec *S[2] = {&oa, &ob};
        const double *V[2] = {a, b};
        for (int q = 0; q < 2; ++q) {
            vector<Point> sel;
            for (const Point &P : all)
                if (P.x >= Bx[q]->L && P.x <= Bx[q]->R && P.y >= Bx[q]->B && P.y <= Bx[q]->T)
                    sel.push_back(P);
            if ((long)sel.size() <= olap2d)
                return 1;
            subi_these(*S[q], V[q], w, sel);
        }
    }
    out[15] = oa.O.x;
    out[16] = oa.O.y;
    out[17] = ob.O.x;
    out[18] = ob.O.y;
    out[19] = oa.w;
    out[20] = oa.h;
    ThmRec thm;
    if (!make_thumbs(thm, oa, ob, thmdec, olap2d, olap1d))
        return 2;
    CThmScan S;
    CorRec best;
    S.Initialize(flog, best);
    S.SetTdfm(TAffine());
    S.SetRThresh(rthresh);
    S.SetNbMaxHt(nbmaxht);
    S.SetSweepConstXY(true);
    S.SetSweepPretweak(pretweak);
    S.SetUseCorrR(true);
    S.SetDisc(0, 0, -1, -1);
    const bool ok = mode_prior ? S.UsePriorAngles(best, 1, ang0, hfangpr, thm)
                               : S.DenovoBestAngle(best, ang0, hfangdn, 0.5, thm, true);
    out[11] = best.A;
    out[12] = best.X;
    out[13] = best.Y;
    out[14] = best.R;
    out[10] = S.GetErr();
    if (!ok)
        return 3;
    if (tweaks)
        S.PostTweaks(best, thm);
    best.X *= thm.scl;
    best.Y *= thm.scl;
    if (!make_thumbs(thm, oa, ob, 1, olap2d, olap1d))
        return 2;
    S.FinishAtFullRes(best, thm);
    // IsectToImageCoords, CThmUtil.cpp:657-668
    Point aO = oa.O;
    best.T.Apply_R_Part(aO);
    best.X += ob.O.x - aO.x;
    best.Y += ob.O.y - aO.y;
    best.T.SetXY(best.X, best.Y);
    out[0] = best.A;
    out[1] = best.X;
    out[2] = best.Y;
    out[3] = best.R;
    for (int i = 0; i < 6; ++i)
        out[4 + i] = best.T.t[i];
    out[10] = S.GetErr();
    // Check_LIMXY, CThmUtil.cpp:817-845
    TAffine Tab(1.0, 0.0, tabx, 0.0, 1.0, taby), I;
    I.InverseOf(Tab);
    I = I * best.T;
    const double err = sqrt(I.t[2] * I.t[2] + I.t[5] * I.t[5]);
    if (limxy && err > limxy)
        return 4;
    return 0;
}


/*
 * PixPair::Load's conditioning of one uint8 tile (0_GEN/CPixPair.cpp:
 * 209-494): the reference's LegPolyFlatten, Convolve and Normalize; its
 * static MakeDoGKernel (:38-83) and the PixPair::Downsample member (:90-110)
 * restated here (CPixPair.cpp is not compiled).  vfy / aln: ws x hs outputs
 * (the caller sizes them with the same halving rule).  Returns 0.
 */
int ref_pixpair_condition(const unsigned char *ras, int w, int h, int order, int r1, int r2,
                          int ws, int hs, int scl, double *vfy, double *aln)
{
    vector<double> avf, flt;
    LegPolyFlatten(avf, ras, w, h, order);
    const vector<double> *al = &avf;
    if (r2 > 0) {
        const int d = 3 * r2, D = 2 * d + 1;
        double s1 = 0.0, s2 = 0.0;
        for (int y = -d; y <= d; ++y)
            for (int x = -d; x <= d; ++x) {
                double R = x * x + y * y;
                s1 += exp(-(R / (2 * r1 * r1)));
                s2 += exp(-(R / (2 * r2 * r2)));
            }
        vector<double> DoG(D * D);
        for (int y = -d; y <= d; ++y)
            for (int x = -d; x <= d; ++x) {
                double R = x * x + y * y;
                double v1 = exp(-(R / (2 * r1 * r1)));
                double v2 = exp(-(R / (2 * r2 * r2)));
                DoG[x + d + D * (y + d)] = v1 / s1 - v2 / s2;
            }
        vector<CD> kfft;
        Convolve(flt, avf, w, h, &DoG[0], D, D, true, true, kfft, quiet_log());
        Normalize(flt);
        al = &flt;
    }
    const int n = scl * scl;
    const vector<double> *src[2] = {&avf, al};
    double *dst[2] = {vfy, aln};
    for (int q = 0; q < 2; ++q)
        for (int iy = 0; iy < hs; ++iy)
            for (int ix = 0; ix < ws; ++ix) {
                double sum = 0.0;
                for (int dy = 0; dy < scl; ++dy)
                    for (int dx = 0; dx < scl; ++dx)
                        sum += (*src[q])[ix * scl + dx + w * (iy * scl + dy)];
                dst[q][ix + ws * iy] = sum / n;
            }
    return 0;
}

} /* extern "C" */
