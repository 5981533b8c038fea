/*
 * aln_oracle.h -- CPU FP64 restatement of Aligner's correlation hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker: tests/, the smoke test and
 * the CPU-baseline leg of bench.py may call it; the product library never
 * links it.  Each function restates the reference algorithm it names
 * (file:line in the reference tree) in plain C with FP64 arithmetic and the
 * project FFT (fft64.c) in place of FFTW.  Its outputs are pinned against
 * the reference's own code (oracle/_ref, built from the reference sources)
 * by tests/golden/.
 *
 * Point clouds are passed as xy[2*i], xy[2*i+1] plus values v[i].
 */
#pragma once

#include "../include/aln_corr.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- helpers -------------------------------------------------------- */

int orc_ceil_pow2(int n);                       /* Maths.cpp:97-105 */
int orc_fft_size(int n1, int n2);               /* Correlation.cpp:344-347 */
int orc_fft_size_sqr(int w1, int h1, int w2, int h2); /* Correlation.cpp:355-359 */

/* BBoxFromPoints (IBox), Geometry.cpp:78-106: box[0..3] = L, R, B, T */
void orc_bbox(const double *xy, int n, int box[4]);

/* ImageFromValuesAndPoints + DistributePixel, Geometry.cpp:661-685,
 * Maths.h:236-276.  I is w*h doubles, zeroed here. */
void orc_image_from_points(double *I, int w, int h, const double *v,
                           const double *xy, int n, int xmin, int ymin);

/* Stats (sample std), Maths.cpp:111-141; Normalize, Maths.cpp:192-212 */
void orc_stats(const double *v, int n, double *avg, double *sd);
double orc_normalize(double *v, int n);

/* DecimateVector, Maths.cpp:1315-1364: returns the new point count. */
int orc_decimate(double *xy, double *v, int n, int w, int h, int lbin);

/* LineFit (lincor only), Maths.cpp:457-507 */
double orc_linefit_r(const double *x, const double *y, int n);

/* ParabPeakFFT, Correlation.cpp:482-517 */
void orc_parab_peak_fft(double *xpk, double *ypk, int d, const double *I,
                        int nx, int ny);

/* Legality of one overlap (the typed EvalType callbacks) */
int orc_legal_rgn(const aln_legal *L, int olw, int olh);
int orc_legal_cnt(const aln_legal *L, int c1, int c2);

/* ---- correlators ---------------------------------------------------- */

typedef struct orc_corr_out {
    double r, dx, dy;
    int status;          /* 0 ok, 1 no legal lag / too small */
    int bigx, bigy;      /* integer lag of the peak */
    int nx, ny;          /* FFT size */
    double second;       /* best value among legal lags other than the peak
                            (-1e30 if none): the top-two margin is r-second */
    int w1, h1, w2, h2;  /* bbox sizes */
    int b1l, b1b, b2l, b2b;
    /* optional rasters (caller-owned, may be NULL):
       CorrPatches: rslt, nx*ny doubles, the reference's final rslt array
       CorrImages:  wR*hR doubles for R and S, wR*hR bytes for A */
    double *rslt;
    double *Rimg, *Simg;
    unsigned char *Aimg;
    double s_mean, s_sd;  /* CorrImagesS: Stats(S) */
    int rx, ry;           /* CorrImages: peak in R-image coordinates */
} orc_corr_out;

/* CorrPatches, Correlation.cpp:901-1170 */
double orc_corr_patches(const double *xy1, const double *v1, int n1,
                        const double *xy2, const double *v2, int n2,
                        int Ox, int Oy, int radius, const aln_legal *L,
                        orc_corr_out *out);

/* CorrImagesF/R/S, Correlation.cpp:3066-3290 (kind 0 F, 1 R, 2 S) */
double orc_corr_images(int kind, const double *xy1, const double *v1, int n1,
                       const double *xy2, const double *v2, int n2,
                       const aln_legal *L, double mincor, double nbmaxht,
                       int Ox, int Oy, int Rx, int Ry, orc_corr_out *out);

/* CorrPatchToImage, Correlation.cpp:1186-1355 (no stdout report) */
double orc_corr_patch_to_image(const double *xy1, const double *v1, int n1,
                               const double *i2, int n2sq, int Ox, int Oy,
                               int radius, int bFilter, orc_corr_out *out);

/* Convolve, Correlation.cpp:371-457 (kfft not cached) */
void orc_convolve(double *dst, const double *src, int ws, int hs,
                  const double *K, int wk, int hk, int sym, int prenorm);

/* ---- CThmScan ------------------------------------------------------- */

/* Search parameters, the CThmScan setters (CThmScan.h:115-157). */
typedef struct orc_thm_params {
    double rthresh, nbmaxht;
    int constxy, pretweak, usecorrr;
    int Ox, Oy, Rx, Ry;
    double tdfm[6];       /* TAffine Tdfm (linear part used) */
} orc_thm_params;

typedef struct orc_thm_rec {
    double A, X, Y, R;
    double T[6];
    double pm;            /* checker field (not in the reference's ThmRec): the
                             correlator call's own top-two score margin,
                             relative to max(1, |score|); 1e30 if no peak */
} orc_thm_rec;

/* Decision margins of one search (checker instrumentation; the reference
 * has no counterpart).  Every comparison that steers the search -- the
 * ConstXY ranking prefix down to the accepted angle, the LineFit |r| >= 0.7
 * tests, the X/Y roundings those fits see, the correlator peaks whose X, Y
 * are used, MaxR's maximum, PeakHunt's bracket tests, the Pretweaks tests
 * and the rthresh tests -- is noted with its margin.  A GPU search whose
 * own arithmetic differs from the oracle's by less than `eps` (relative, on
 * scores) and `eps_px` (on the rounded offsets) takes every decision whose
 * margin exceeds those the same way, so it must land on the identical
 * angle when nties == 0.  Otherwise the angle may move by at most tolA
 * (1e30: unbounded -- a flipped ranking or threshold can send the search
 * anywhere), and the err code may differ iff thr_tie. */
typedef struct orc_thm_margins {
    double eps, eps_px;   /* inputs: tie thresholds */
    double mR;            /* smallest relative score margin noted */
    double mpx;           /* smallest distance (px) of a rounded X/Y from .5 */
    double tolA;          /* angle bound if every tie flipped (0 if none) */
    double mpk;           /* the answer's own correlator top-two margin */
    int ndec, nties;      /* decisions noted, decisions below the thresholds */
    int thr_tie;          /* an rthresh test was a tie: err may differ */
} orc_thm_margins;

/* mode: 0 DenovoBestAngle(ang0, hfang, step), 1 RFromAngle(ang0),
 * 2 UsePriorAngles(ang0, hfang), 3 AngleScanSel(ConstXY/MaxR by params,
 * favorCenter=false) then PeakHunt(step*0.05*1.5), 4 AngleScanMaxR(favorCenter).
 * Mirrors refwrap's ref_thm_search.  Returns the CThmScan err code. */
int orc_thm_search(const double *xya, const double *va, int na,
                   const double *xyb, const double *vb, int nb,
                   long reqArea, int olap1D, const orc_thm_params *P,
                   int mode, double ang0, double hfang, double step,
                   orc_thm_rec *best, int *ncalls);

/* orc_thm_search with the decision margins of the run (M may be NULL;
 * M->eps and M->eps_px are read, the rest written). */
int orc_thm_search_m(const double *xya, const double *va, int na,
                     const double *xyb, const double *vb, int nb,
                     long reqArea, int olap1D, const orc_thm_params *P,
                     int mode, double ang0, double hfang, double step,
                     orc_thm_rec *best, int *ncalls, orc_thm_margins *M);

/* PostTweaks (mode 5) / FinishAtFullRes (mode 6) from a prior best
 * (A, X, Y, R) and pretweak transform (NULL: identity).  Mirrors refwrap's
 * ref_thm_finish; tptwk_out (may be NULL) receives the transform after. */
int orc_thm_finish(const double *xya, const double *va, int na,
                   const double *xyb, const double *vb, int nb,
                   long reqArea, int olap1D, const orc_thm_params *P, int mode,
                   const double *prior, const double *tptwk6, orc_thm_rec *best,
                   double *tptwk_out, int *ncalls);

/* ---- mesh optimizer ------------------------------------------------- */

/* The control-point multipliers am (nm rows of nc, mostly zero in the
 * reference's dense form) are passed compressed: row i's k slots
 * am_idx[i*k + s] / am_w[i*k + s] hold its nonzero multipliers in increasing
 * control-point order, unused slots have index -1.  Skipping the zero terms
 * leaves every sum of the reference's dense loops unchanged, so the results
 * are the reference's bit for bit. */

/* GradDescStep, 0_GEN/Correlation.cpp:1403-1478 (with NormalizeNonZeros,
 * Maths.cpp:247-268): bnew[nm], dRdc[2*nc] = (x, y) per control point. */
void orc_grad_desc_step(double *bnew, double *dRdc, const double *ac, int nc,
                        const int *am_idx, const double *am_w, int k, int nm,
                        const double *av, const double *bimg, int w, int h);

/* CorrVectors, 0_GEN/Correlation.cpp:1490-1530 (nnz may be NULL) */
double orc_corr_vectors(const double *a, const double *b, int n, int *nnz);

/* ImproveControlPts, 0_GEN/Correlation.cpp:1605-1721: ac[2*nc] in/out;
 * returns the correlation; *iters = GradDescStep evaluations after the
 * first (may be NULL). */
double orc_improve_control_pts(double *ac, int nc, const int *am_idx, const double *am_w,
                               int k, int nm, const double *av, const double *bimg,
                               int w, int h, double ini_thresh, double fin_thresh,
                               int *iters);

#ifdef __cplusplus
}
#endif
