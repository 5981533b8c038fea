// aln_correlation_shim.cpp -- libaln_corr_shim.so: the Correlation.h entry
// points of aln_correlation.hpp over the C ABI of libaln_corr.so (GPU).
//
// What the shim does on the host is the boundary's format work only: point
// lists become bounding-box rasters (BBoxFromPoints, 0_GEN/Geometry.cpp:
// 78-106; integer points are placed, fractional clouds go to the device's
// DistributePixel splat, aln_points_image), EvalType callbacks become typed
// legality descriptors,
// the reference's fft2 / ftc cache vectors become spectrum-cache keys.  Every
// correlation runs on the GPU; there is no CPU fallback: if the GPU library
// fails, the call logs the error to flog and returns 0.0, the reference's
// "no result" value.
#include "aln_correlation.hpp"

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <vector>

#include "../../include/aln_corr.h"
#include "aln_shim_util.hpp"

namespace {

using aln_shim::ctx;
using aln_shim::IBoxD;
using aln_shim::bbox;
using aln_shim::raster;
using aln_shim::image_of_points;
using aln_shim::image_of;
using aln_shim::key_of;

// LegalRgn -> a table over every overlap size the pair can have; LegalCnt
// -> the count threshold n of "c1 > n && c2 > n" (EnoughPoints,
// 0_GEN/CThmScan.cpp:39-42), found by bisection and checked; any other
// LegalCnt shape is refused.
bool legal_of(EvalType rgn, void *arglr, EvalType cnt, void *arglc, int w1, int h1, int w2,
              int h2, aln_legal &lg, std::vector<unsigned char> &tab, FILE *flog)
{
    memset(&lg, 0, sizeof lg);
    if (rgn) {
        const int tw = w1 < w2 ? w1 : w2, th = h1 < h2 ? h1 : h2;
        tab.assign((size_t)tw * th, 0);
        for (int sy = 1; sy <= th; ++sy)
            for (int sx = 1; sx <= tw; ++sx)
                tab[(size_t)(sy - 1) * tw + (sx - 1)] = rgn(sx, sy, arglr) ? 1 : 0;
        lg.rgn_kind = ALN_RGN_TABLE;
        lg.table = tab.data();
        lg.table_w = tw;
        lg.table_h = th;
    }
    if (cnt) {
        const long long cmax = (long long)w1 * h1 + (long long)w2 * h2 + 1;
        if (!cnt((int)cmax, (int)cmax, arglc)) {
            lg.cnt_kind = ALN_CNT_GT;   // never legal
            lg.cnt_n = cmax;
            return true;
        }
        long long lo = -1, hi = cmax;   // cnt(c, c) false at lo, true at hi
        if (cnt(0, 0, arglc))
            hi = 0;
        while (hi - lo > 1) {
            const long long m = (lo + hi) / 2;
            (cnt((int)m, (int)m, arglc) ? hi : lo) = m;
        }
        const long long n = hi - 1;
        const bool ok = (n < 0 || !cnt((int)n, (int)cmax, arglc)) &&
                        (n < 0 || !cnt((int)cmax, (int)n, arglc)) &&
                        cnt((int)hi, (int)cmax, arglc) && cnt((int)cmax, (int)hi, arglc);
        if (!ok) {
            fprintf(flog, "GPU correlation: LegalCnt is not of the form c1 > n && c2 > n\n");
            return false;
        }
        lg.cnt_kind = ALN_CNT_GT;
        lg.cnt_n = n;
    }
    return true;
}

}   // namespace

int FFTSize(int n1, int n2) { return aln_fft_size(n1, n2); }

int FFTSizeSQR(int w1, int h1, int w2, int h2) { return aln_fft_size_sqr(w1, h1, w2, h2); }

int FFT_2D(std::vector<CD> &out, const std::vector<double> &in, int Nfast, int Nslow,
           bool cached, FILE *flog)
{
    const int M = Nslow * (Nfast / 2 + 1);
    if (cached && (int)out.size() == M)
        return M;
    out.resize(M);
    const int rc = aln_fft_2d(ctx(), in.data(), Nfast, Nslow, (double *)out.data());
    if (rc < 0)
        fprintf(flog, "FFT_2D: %s\n", aln_last_error(ctx()));
    return M;
}

void IFT_2D(std::vector<double> &out, const std::vector<CD> &in, int Nfast, int Nslow,
            FILE *flog)
{
    out.resize((size_t)Nfast * Nslow);
    if (aln_ift_2d(ctx(), (const double *)in.data(), Nfast, Nslow, out.data()) < 0)
        fprintf(flog, "IFT_2D: %s\n", aln_last_error(ctx()));
}

void Convolve(std::vector<double> &dst, const std::vector<double> &src, int ws, int hs,
              const double *K, int wk, int hk, bool kIsSymmetric, bool preNormK,
              std::vector<CD> &kfft, FILE *flog)
{
    const int Nx = aln_fft_size(ws, wk / (1 + kIsSymmetric)),
              Ny = aln_fft_size(hs, hk / (1 + kIsSymmetric));
    std::vector<double> out((size_t)ws * hs);   // dst may be src
    if (aln_convolve(ctx(), src.data(), ws, hs, K, wk, hk, kIsSymmetric ? 1 : 0,
                     preNormK ? 1 : 0, out.data()) < 0) {
        fprintf(flog, "Convolve (GPU): %s\n", aln_last_error(ctx()));
        return;
    }
    dst.swap(out);
    kfft.resize((size_t)Ny * (Nx / 2 + 1));
}

void ParabPeakFFT(double &xpk, double &ypk, int d, const double *I, int nx, int ny)
{
    aln_parab_peak_fft(&xpk, &ypk, d, I, nx, ny);
}

double CorrPatches(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2, int Ox,
                   int Oy, int radius, EvalType LegalRgn, void *arglr, EvalType LegalCnt,
                   void *arglc, std::vector<CD> &fft2)
{
    if (ip1.empty() || ip2.empty())
        return 0.0;
    const IBoxD B1 = bbox(ip1), B2 = bbox(ip2);
    std::vector<double> r1, r2;
    aln_pair P;
    memset(&P, 0, sizeof P);
    if (!image_of_points(ip1, iv1, B1, 0, r1, P.a) || !image_of_points(ip2, iv2, B2, 1, r2, P.b)) {
        fprintf(flog, "CorrPatches (GPU): %s\n", aln_last_error(ctx()));
        return 0.0;
    }
    P.ox = Ox;
    P.oy = Oy;
    P.radius = radius;
    std::vector<unsigned char> tab;
    if (!legal_of(LegalRgn, arglr, LegalCnt, arglc, P.a.w, P.a.h, P.b.w, P.b.h, P.legal, tab,
                  flog))
        return 0.0;
    const int Nx = aln_fft_size(P.a.w, P.b.w), Ny = aln_fft_size(P.a.h, P.b.h);
    P.b_key = key_of(fft2, (size_t)Ny * (Nx / 2 + 1));
    aln_result res;
    if (aln_corr_patches_batch(ctx(), 1, &P, &res) < 0) {
        fprintf(flog, "CorrPatches (GPU): %s\n", aln_last_error(ctx()));
        return 0.0;
    }
    if (res.status != ALN_OK) {
        if (verbose)
            fprintf(flog, "NormCorr: No legal subregions at all...\n");
        return 0.0;
    }
    if (verbose)
        fprintf(flog, "NormCorr: Maximum correlation of %f at [%d,%d].\n", res.r, res.peak_x,
                res.peak_y);
    dx = res.dx;
    dy = res.dy;
    return res.r;
}

double CorrPatchToImage(double &dx, double &dy, const std::vector<Point> &ip1,
                        const std::vector<double> &iv1, const std::vector<double> &i2, int Ox,
                        int Oy, int radius, bool bFilter)
{
    aln_result res;
    const int rc = aln_corr_patch_to_image(ctx(), (const double *)ip1.data(), iv1.data(),
                                           (int)ip1.size(), i2.data(), (int)i2.size(), Ox, Oy,
                                           radius, bFilter ? 1 : 0, &res);
    if (rc < 0 || res.status != ALN_OK)
        return 0.0;
    dx = res.dx;
    dy = res.dy;
    return res.r;
}

namespace {

double corr_images(int kind, FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2,
                   EvalType LegalRgn, void *arglr, EvalType LegalCnt, void *arglc,
                   double mincor, double nbmaxht, int Ox, int Oy, int Rx, int Ry,
                   std::vector<CD> &fft2)
{
    if (ip1.empty() || ip2.empty())
        return 0.0;
    const IBoxD B1 = bbox(ip1), B2 = bbox(ip2);
    std::vector<double> r1, r2;
    aln_image_job J;
    memset(&J, 0, sizeof J);
    if (!image_of_points(ip1, iv1, B1, 0, r1, J.a) || !image_of_points(ip2, iv2, B2, 1, r2, J.b)) {
        fprintf(flog, "CorrImages (GPU): %s\n", aln_last_error(ctx()));
        return 0.0;
    }
    J.kind = kind;
    J.mincor = mincor;
    J.nbmaxht = nbmaxht;
    J.ox = Ox;
    J.oy = Oy;
    J.rx = Rx;
    J.ry = Ry;
    std::vector<unsigned char> tab;
    if (!legal_of(LegalRgn, arglr, LegalCnt, arglc, J.a.w, J.a.h, J.b.w, J.b.h, J.legal, tab,
                  flog))
        return 0.0;
    const int Nx = aln_fft_size(J.a.w, J.b.w), Ny = aln_fft_size(J.a.h, J.b.h);
    J.b_key = key_of(fft2, (size_t)Ny * (Nx / 2 + 1));
    aln_result res;
    if (aln_corr_images_batch(ctx(), 1, &J, &res) < 0) {
        fprintf(flog, "CorrImages (GPU): %s\n", aln_last_error(ctx()));
        return 0.0;
    }
    if (res.status != ALN_OK)
        return 0.0;
    if (verbose)
        fprintf(flog, "CorrImages: peak %f at [%d,%d].\n", res.r, res.peak_x, res.peak_y);
    dx = res.dx;
    dy = res.dy;
    return res.r;
}

}   // namespace

double CorrImagesF(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2,
                   EvalType LegalRgn, void *arglr, EvalType LegalCnt, void *arglc,
                   double mincor, double nbmaxht, int Ox, int Oy, int Rx, int Ry,
                   std::vector<CD> &fft2)
{
    return corr_images(ALN_CORR_F, flog, verbose, dx, dy, ip1, iv1, ip2, iv2, LegalRgn, arglr,
                       LegalCnt, arglc, mincor, nbmaxht, Ox, Oy, Rx, Ry, fft2);
}

double CorrImagesR(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2,
                   EvalType LegalRgn, void *arglr, EvalType LegalCnt, void *arglc,
                   double mincor, double nbmaxht, int Ox, int Oy, int Rx, int Ry,
                   std::vector<CD> &fft2)
{
    return corr_images(ALN_CORR_R, flog, verbose, dx, dy, ip1, iv1, ip2, iv2, LegalRgn, arglr,
                       LegalCnt, arglc, mincor, nbmaxht, Ox, Oy, Rx, Ry, fft2);
}

double CorrImagesS(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2,
                   EvalType LegalRgn, void *arglr, EvalType LegalCnt, void *arglc,
                   double mincor, double nbmaxht, int Ox, int Oy, int Rx, int Ry,
                   std::vector<CD> &fft2)
{
    return corr_images(ALN_CORR_S, flog, verbose, dx, dy, ip1, iv1, ip2, iv2, LegalRgn, arglr,
                       LegalCnt, arglc, mincor, nbmaxht, Ox, Oy, Rx, Ry, fft2);
}

// ---------------------------------------------------------------------------
// mesh optimizer: the dense multiplier rows compressed to their nonzero
// entries (ascending control point), then the GPU's aln_improve_control_pts
// ---------------------------------------------------------------------------

namespace {

struct MeshArgs {
    std::vector<double> ac;
    std::vector<int> idx;
    std::vector<double> wts;
    aln_mesh_job job;
};

bool mesh_args(MeshArgs &M, const std::vector<Point> &ac,
               const std::vector<std::vector<double> > &am, const std::vector<double> &av,
               const std::vector<double> &bimg, int w, int h, FILE *flog)
{
    const int nc = (int)ac.size(), nm = (int)am.size();
    int k = 1;
    for (const auto &row : am) {
        int c = 0;
        for (double v : row)
            c += v != 0.0;
        if (c > k)
            k = c;
    }
    if (nc > ALN_MESH_MAX_NC || k > ALN_MESH_MAX_K || (int)av.size() != nm) {
        fprintf(flog, "GPU mesh: %d control points / %d multipliers per point unsupported\n",
                nc, k);
        return false;
    }
    M.ac.resize(2 * (size_t)nc);
    for (int j = 0; j < nc; ++j) {
        M.ac[2 * j] = ac[j].x;
        M.ac[2 * j + 1] = ac[j].y;
    }
    M.idx.assign((size_t)nm * k, -1);
    M.wts.assign((size_t)nm * k, 0.0);
    for (int i = 0; i < nm; ++i) {
        int s = 0;
        for (int j = 0; j < (int)am[i].size() && j < nc; ++j)
            if (am[i][j] != 0.0) {
                M.idx[(size_t)i * k + s] = j;
                M.wts[(size_t)i * k + s] = am[i][j];
                ++s;
            }
    }
    memset(&M.job, 0, sizeof M.job);
    M.job.nc = nc;
    M.job.ac = M.ac.data();
    M.job.nm = nm;
    M.job.k = k;
    M.job.am_idx = M.idx.data();
    M.job.am_w = M.wts.data();
    M.job.av = av.data();
    M.job.bimg = bimg.data();
    M.job.w = w;
    M.job.h = h;
    return true;
}

}   // namespace

void GradDescStep(std::vector<double> &bnew, std::vector<Point> &dRdc,
                  const std::vector<Point> &ac, const std::vector<std::vector<double> > &am,
                  const std::vector<double> &av, const std::vector<double> &bimg, int w, int h)
{
    MeshArgs M;
    const int nc = (int)ac.size();
    bnew.assign(am.size(), 0.0);
    dRdc.assign(nc, Point(0.0, 0.0));
    if (!mesh_args(M, ac, am, av, bimg, w, h, stderr))
        return;
    std::vector<double> d(2 * (size_t)nc);
    if (aln_grad_desc_step(ctx(), &M.job, bnew.data(), d.data(), nullptr) < 0) {
        fprintf(stderr, "GPU mesh: %s\n", aln_last_error(ctx()));
        return;
    }
    for (int j = 0; j < nc; ++j)
        dRdc[j] = Point(d[2 * j], d[2 * j + 1]);
}

double CorrVectors(FILE *flog, const std::vector<double> &a, const std::vector<double> &b,
                   int *nnz)
{
    if (!flog)
        flog = stdout;
    if (a.size() != b.size()) {
        fprintf(flog, "CorrVectors: Sizes differ! %d %ld\n", (int)a.size(), (long)b.size());
        return 0.0;   // the reference exits here; the library never does
    }
    double r = 0.0;
    if (aln_corr_vectors(ctx(), a.data(), b.data(), (int)a.size(), &r, nnz) < 0) {
        fprintf(flog, "GPU CorrVectors: %s\n", aln_last_error(ctx()));
        return 0.0;
    }
    return r;
}

double ImproveControlPts(std::vector<Point> &ac, const std::vector<std::vector<double> > &am,
                         const std::vector<double> &av, const std::vector<double> &bimg, int w,
                         int h, FILE *flog, const char *describe, double iniThresh,
                         double finThresh)
{
    MeshArgs M;
    if (!mesh_args(M, ac, am, av, bimg, w, h, flog))
        return 0.0;
    M.job.ini_thresh = iniThresh;
    M.job.fin_thresh = finThresh;
    aln_mesh_result r;
    if (aln_improve_control_pts_batch(ctx(), 1, &M.job, &r) < 0) {
        fprintf(flog, "GPU mesh: %s\n", aln_last_error(ctx()));
        return 0.0;
    }
    // the reference's report lines (Correlation.cpp:1631-1720)
    fprintf(flog, "STAT: ImproveCpt: Initial %s correlation %f (%ld pixels).\n", describe,
            r.corr0, (long)av.size());
    if (r.corr0 < iniThresh) {
        fprintf(flog, "FAIL: ImproveCpt: Correlation %f less than %f at start.\n", r.corr0,
                iniThresh);
        return 0.0;
    }
    if (finThresh < 0) {
        fprintf(flog, "STAT: ImproveCpt: Skipping optimizer; final corr %f\n", r.corr);
        return r.corr;
    }
    for (size_t j = 0; j < ac.size(); ++j)
        ac[j] = Point(M.ac[2 * j], M.ac[2 * j + 1]);
    fprintf(flog, "STAT: ImproveCpt: Final %s correlation %f, (threshold %f).\n", describe,
            r.corr, finThresh);
    return r.corr;
}
