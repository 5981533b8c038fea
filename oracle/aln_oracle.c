/*
 * aln_oracle.c -- CPU FP64 restatement of Aligner's correlation hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see aln_oracle.h).  Every function restates the
 * reference routine cited beside it; arithmetic is FP64 with the reference's
 * operation order where rounding could matter (integral images, angle lists,
 * rotation), and the FFT is the project's FP64 fft64.c.  Build with
 * -ffp-contract=off so x86 and Arm hosts produce identical bits.
 */
#define _GNU_SOURCE
#include "aln_oracle.h"
#include "fft64.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358 /* GenDefs.h:16 (truncated, as the reference uses it) */

static inline int imax(int a, int b) { return a > b ? a : b; }
static inline int imin(int a, int b) { return a < b ? a : b; }

/* ------------------------------------------------------------------ */
/* helpers                                                             */
/* ------------------------------------------------------------------ */

int orc_ceil_pow2(int n)
{
    int p = 1;
    while (p < n)
        p *= 2;
    return p;
}

int orc_fft_size(int n1, int n2) { return orc_ceil_pow2(n1 + n2 - 1); }

int orc_fft_size_sqr(int w1, int h1, int w2, int h2)
{
    return orc_ceil_pow2(imax(w1 + w2, h1 + h2) - 1);
}

void orc_bbox(const double *xy, int n, int box[4])
{
    if (n <= 0) {
        box[0] = box[1] = box[2] = box[3] = 0;
        return;
    }
    double xlo = xy[0], xhi = xy[0], ylo = xy[1], yhi = xy[1];
    for (int i = 1; i < n; ++i) {
        double t = xy[2 * i];
        if (t < xlo)
            xlo = t;
        else if (t > xhi)
            xhi = t;
        t = xy[2 * i + 1];
        if (t < ylo)
            ylo = t;
        else if (t > yhi)
            yhi = t;
    }
    box[0] = (int)floor(xlo);
    box[1] = (int)ceil(xhi);
    box[2] = (int)floor(ylo);
    box[3] = (int)ceil(yhi);
}

/* bilinear forward splat of one value (Maths.h:236-276) */
static void splat(double x, double y, double val, double *I, int w, int h)
{
    int ix = (int)floor(x), iy = (int)floor(y);
    long i = ix + (long)w * iy;
    double alpha = x - ix, beta = y - iy;

    if (ix >= 0 && ix < w) {
        if (iy >= 0 && iy < h)
            I[i] += (1.0 - alpha) * (1.0 - beta) * val;
        if (iy + 1 >= 0 && iy + 1 < h)
            I[i + w] += (1.0 - alpha) * beta * val;
    }
    if (ix + 1 >= 0 && ix + 1 < w) {
        if (iy >= 0 && iy < h)
            I[i + 1] += alpha * (1.0 - beta) * val;
        if (iy + 1 >= 0 && iy + 1 < h)
            I[i + 1 + w] += alpha * beta * val;
    }
}

void orc_image_from_points(double *I, int w, int h, const double *v,
                           const double *xy, int n, int xmin, int ymin)
{
    memset(I, 0, sizeof(double) * (size_t)w * h);
    for (int i = 0; i < n; ++i)
        splat(xy[2 * i] - xmin, xy[2 * i + 1] - ymin, v[i], I, w, h);
}

void orc_stats(const double *v, int n, double *avg, double *sd)
{
    double sum = 0.0, sum2 = 0.0;
    for (int i = 0; i < n; ++i) {
        sum += v[i];
        sum2 += v[i] * v[i];
    }
    *avg = sum;
    *sd = 0.0;
    if (n > 1) {
        *avg /= n;
        *sd = sqrt(fmax(sum2 - n * *avg * *avg, 0.0) / (n - 1.0));
    }
}

double orc_normalize(double *v, int n)
{
    double avg, sd;
    orc_stats(v, n, &avg, &sd);
    for (int i = 0; i < n; ++i)
        v[i] = (v[i] - avg) / sd;
    return sd;
}

int orc_decimate(double *xy, double *v, int n, int w, int h, int lbin)
{
    w = (w + lbin - 1) / lbin;
    h = (h + lbin - 1) / lbin;
    int nr = w * h;
    double *vr = (double *)calloc((size_t)nr, sizeof(double));
    unsigned char *cr = (unsigned char *)calloc((size_t)nr, 1);
    for (int ip = 0; ip < n; ++ip) {
        int x = (int)xy[2 * ip] / lbin, y = (int)xy[2 * ip + 1] / lbin;
        int ir = x + w * y;
        vr[ir] += v[ip];
        ++cr[ir];   /* uint8 counter, as the reference's vector<uint8> */
    }
    int k = 0;
    for (int ir = 0; ir < nr; ++ir) {
        int cnt = cr[ir];
        if (cnt) {
            int y = ir / w, x = ir - w * y;
            v[k] = vr[ir] / cnt;
            xy[2 * k] = x;
            xy[2 * k + 1] = y;
            ++k;
        }
    }
    free(vr);
    free(cr);
    return k;
}

double orc_linefit_r(const double *x, const double *y, int n)
{
    double cnt = 0, sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
    for (int i = 0; i < n; ++i) {
        double X = x[i], Y = y[i];
        sx += X;
        sy += Y;
        sxx += X * X;
        syy += Y * Y;
        sxy += X * Y;
        ++cnt;
    }
    double r = cnt * sxy - sx * sy;
    double vx = cnt * sxx - sx * sx;
    double vy = cnt * syy - sy * sy;
    return r / sqrt(vx * vy);
}

static inline double lk(const double *I, int nx, int ny, int x, int y)
{
    if (x < 0)
        x += nx;
    if (y < 0)
        y += ny;
    return I[x + (long)nx * y];
}

void orc_parab_peak_fft(double *xpk, double *ypk, int d, const double *I,
                        int nx, int ny)
{
    int ix = (int)*xpk, iy = (int)*ypk;
    double z1 = lk(I, nx, ny, ix, iy), z0, z2;

    if (ix - d >= 0 && ix + d < nx && (z0 = lk(I, nx, ny, ix - d, iy)) != 0.0 &&
        (z2 = lk(I, nx, ny, ix + d, iy)) != 0.0) {
        z0 = d * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * d)
            *xpk += z0;
    }
    if (iy - d >= 0 && iy + d < ny && (z0 = lk(I, nx, ny, ix, iy - d)) != 0.0 &&
        (z2 = lk(I, nx, ny, ix, iy + d)) != 0.0) {
        z0 = d * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * d)
            *ypk += z0;
    }
}

/* ParabPeak, Correlation.cpp:2975-3010 (neighbours must be > 0) */
static void parab_peak(double *xpk, double *ypk, int d, const double *I, int w, int h)
{
    int ix = (int)*xpk, iy = (int)*ypk;
    double z1 = I[ix + (long)w * iy], z0, z2;
    if (ix - d >= 0 && ix + d < w && (z0 = I[ix - d + (long)w * iy]) > 0.0 &&
        (z2 = I[ix + d + (long)w * iy]) > 0.0) {
        z0 = d * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * d)
            *xpk += z0;
    }
    if (iy - d >= 0 && iy + d < h && (z0 = I[ix + (long)w * (iy - d)]) > 0.0 &&
        (z2 = I[ix + (long)w * (iy + d)]) > 0.0) {
        z0 = d * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * d)
            *ypk += z0;
    }
}

int orc_legal_rgn(const aln_legal *L, int sx, int sy)
{
    if (!L)
        return 1;
    switch (L->rgn_kind) {
    case ALN_RGN_MIN:
        return sx >= L->rgn_a && sy >= L->rgn_b && (long long)sx * sy > L->rgn_area;
    case ALN_RGN_SECTION:
        return (long long)sx * sy > L->rgn_area && (sx >= L->rgn_a || sy > L->rgn_b);
    case ALN_RGN_EXACT:
        return sx == L->rgn_a && sy == L->rgn_b;
    case ALN_RGN_TABLE:
        if (sx < 1 || sy < 1 || sx > L->table_w || sy > L->table_h)
            return 0;
        return L->table[(size_t)(sy - 1) * L->table_w + (sx - 1)] != 0;
    default:
        return 1;
    }
}

int orc_legal_cnt(const aln_legal *L, int c1, int c2)
{
    if (!L || L->cnt_kind != ALN_CNT_GT)
        return 1;
    return c1 > L->cnt_n && c2 > L->cnt_n;
}

/* ------------------------------------------------------------------ */
/* integral images and overlap boxes                                   */
/* ------------------------------------------------------------------ */

typedef struct {
    int L, R, B, T;
} ibox;

/* IntegrateImage, Correlation.cpp:49-105 (same recursion, same rounding) */
static void integrate(double *S, double *S2, int *nz, int wS, int hS,
                      const double *I, int wI)
{
    double t;
    S[0] = (t = I[0]);
    S2[0] = t * t;
    nz[0] = (t != 0.0);
    for (int x = 1; x < wS; ++x) {
        S[x] = S[x - 1] + (t = I[x]);
        S2[x] = S2[x - 1] + t * t;
        nz[x] = nz[x - 1] + (t != 0.0);
    }
    for (int y = 1; y < hS; ++y) {
        long j = (long)wS * y, k = (long)wI * y;
        S[j] = S[j - wS] + (t = I[k]);
        S2[j] = S2[j - wS] + t * t;
        nz[j] = nz[j - wS] + (t != 0.0);
    }
    for (int y = 1; y < hS; ++y) {
        long i = (long)wS * y, k = (long)wI * y;
        for (int x = 1; x < wS; ++x) {
            long j = i + x, m = k + x;
            S[j] = S[j - 1] + S[j - wS] - S[j - wS - 1] + (t = I[m]);
            S2[j] = S2[j - 1] + S2[j - wS] - S2[j - wS - 1] + t * t;
            nz[j] = nz[j - 1] + nz[j - wS] - nz[j - wS - 1] + (t != 0.0);
        }
    }
}

/* IntegralTable, Correlation.cpp:112-150 */
static double table_d(const double *t, int wS, ibox B)
{
    double r = t[B.R + (long)wS * B.T];
    if (B.L > 0)
        r -= t[B.L - 1 + (long)wS * B.T];
    if (B.B > 0)
        r -= t[B.R + (long)wS * (B.B - 1)];
    if (B.L > 0 && B.B > 0)
        r += t[(B.L - 1) + (long)wS * (B.B - 1)];
    return r;
}

static int table_i(const int *t, int wS, ibox B)
{
    int r = t[B.R + (long)wS * B.T];
    if (B.L > 0)
        r -= t[B.L - 1 + (long)wS * B.T];
    if (B.B > 0)
        r -= t[B.R + (long)wS * (B.B - 1)];
    if (B.L > 0 && B.B > 0)
        r += t[(B.L - 1) + (long)wS * (B.B - 1)];
    return r;
}

/* BoxesFromShifts, Geometry.cpp:150-176 */
static void boxes_from_shifts(ibox *B1, ibox *B2, int w1, int h1, int w2, int h2,
                              int x, int y)
{
    B2->L = imax(0, x);
    B2->R = imin(w2 - 1, x + w1 - 1);
    B2->B = imax(0, y);
    B2->T = imin(h2 - 1, y + h1 - 1);
    B2->R = imax(B2->R, B2->L);
    B2->T = imax(B2->T, B2->B);
    B1->L = B2->L - x;
    B1->R = B2->R - x;
    B1->B = B2->B - y;
    B1->T = B2->T - y;
}

/* Sums over both images for one lag (CLinCorr / RCalc state). */
typedef struct {
    double *s1, *q1, *s2, *q2;
    int *n1, *n2;
    int w1, h1, w2, h2, Nx, Nxy;
} lagcalc;

static void lag_init(lagcalc *c, const double *I1, int w1, int h1,
                     const double *I2, int w2, int h2, int Nx, int Ny)
{
    c->w1 = w1;
    c->h1 = h1;
    c->w2 = w2;
    c->h2 = h2;
    c->Nx = Nx;
    c->Nxy = Nx * Ny;
    size_t a = (size_t)w1 * h1, b = (size_t)w2 * h2;
    c->s1 = (double *)malloc(sizeof(double) * a);
    c->q1 = (double *)malloc(sizeof(double) * a);
    c->n1 = (int *)malloc(sizeof(int) * a);
    c->s2 = (double *)malloc(sizeof(double) * b);
    c->q2 = (double *)malloc(sizeof(double) * b);
    c->n2 = (int *)malloc(sizeof(int) * b);
    integrate(c->s1, c->q1, c->n1, w1, h1, I1, Nx);
    integrate(c->s2, c->q2, c->n2, w2, h2, I2, Nx);
}

static void lag_free(lagcalc *c)
{
    free(c->s1);
    free(c->q1);
    free(c->n1);
    free(c->s2);
    free(c->q2);
    free(c->n2);
}

/* legality of lag (x, y); sets the boxes and counts */
static int lag_valid(const lagcalc *c, const aln_legal *L, int x, int y,
                     ibox *O1, ibox *O2, int *olw, int *olh, int check_cnt_always)
{
    boxes_from_shifts(O1, O2, c->w1, c->h1, c->w2, c->h2, x, y);
    *olw = O1->R - O1->L + 1;
    *olh = O1->T - O1->B + 1;
    int ok = 1;
    int has_rgn = L && L->rgn_kind != ALN_RGN_NONE;
    int has_cnt = L && L->cnt_kind == ALN_CNT_GT;
    if (has_rgn && !orc_legal_rgn(L, *olw, *olh)) {
        ok = 0;
        if (!check_cnt_always)
            return 0;
    }
    if (has_cnt) {
        int c1 = table_i(c->n1, c->w1, *O1), c2 = table_i(c->n2, c->w2, *O2);
        if (!orc_legal_cnt(L, c1, c2))
            ok = 0;
    }
    return ok;
}

/* CLinCorr::GetCorr / RCalc::CalcR core: Pearson r from the sums */
static double lag_r(const lagcalc *c, ibox O1, ibox O2, int olw, int olh,
                    double rslt, int *odd)
{
    double n = olw * olh;
    double a1 = table_d(c->s1, c->w1, O1), a2 = table_d(c->q1, c->w1, O1);
    double b1 = table_d(c->s2, c->w2, O2), b2 = table_d(c->q2, c->w2, O2);
    double num = n * rslt / c->Nxy - a1 * b1;
    double d1 = n * a2 - a1 * a1;
    double d2 = n * b2 - b1 * b1;
    double d = d1 * d2;
    double r = (d < n * n * 1.0E-9 ? 0.0 : num / sqrt(d));
    if (odd)
        *odd = fabs(r) > 1.0001;
    return r;
}

/* fft2 * conj(fft1) into fft1 (Correlation.cpp:977-985) */
static void cross_spectrum(double *f1, const double *f2, size_t M)
{
    for (size_t i = 0; i < M; ++i) {
        double a = f2[2 * i], b = f2[2 * i + 1];
        double c = f1[2 * i], d = -f1[2 * i + 1];
        f1[2 * i] = a * c - b * d;
        f1[2 * i + 1] = a * d + b * c;
    }
}

/* ------------------------------------------------------------------ */
/* CorrPatches, Correlation.cpp:901-1170                               */
/* ------------------------------------------------------------------ */

double orc_corr_patches(const double *xy1, const double *v1, int n1,
                        const double *xy2, const double *v2, int n2,
                        int Ox, int Oy, int radius, const aln_legal *L,
                        orc_corr_out *out)
{
    orc_corr_out dummy;
    if (!out) {
        memset(&dummy, 0, sizeof dummy);
        out = &dummy;
    }
    out->status = 0;
    out->second = -1e30;
    if (n1 <= 0 || n2 <= 0) {
        out->status = -1;
        out->r = out->dx = out->dy = 0.0;
        return 0.0;
    }
    int B1[4], B2[4];
    orc_bbox(xy1, n1, B1);
    orc_bbox(xy2, n2, B2);
    int w1 = B1[1] - B1[0] + 1, h1 = B1[3] - B1[2] + 1;
    int w2 = B2[1] - B2[0] + 1, h2 = B2[3] - B2[2] + 1;
    int Nx = orc_fft_size(w1, w2), Ny = orc_fft_size(h1, h2);
    size_t M = (size_t)Ny * (Nx / 2 + 1), NN = (size_t)Nx * Ny;
    out->nx = Nx;
    out->ny = Ny;
    out->w1 = w1;
    out->h1 = h1;
    out->w2 = w2;
    out->h2 = h2;
    out->b1l = B1[0];
    out->b1b = B1[2];
    out->b2l = B2[0];
    out->b2b = B2[2];

    double *i1 = (double *)malloc(sizeof(double) * NN);
    double *i2 = (double *)malloc(sizeof(double) * NN);
    orc_image_from_points(i1, Nx, Ny, v1, xy1, n1, B1[0], B1[2]);
    orc_image_from_points(i2, Nx, Ny, v2, xy2, n2, B2[0], B2[2]);

    double *f1 = (double *)malloc(sizeof(double) * 2 * M);
    double *f2 = (double *)malloc(sizeof(double) * 2 * M);
    fft64_r2c_2d(Ny, Nx, i2, f2);
    fft64_r2c_2d(Ny, Nx, i1, f1);
    cross_spectrum(f1, f2, M);
    double *rslt = out->rslt ? out->rslt : (double *)malloc(sizeof(double) * NN);
    fft64_c2r_2d(Ny, Nx, f1, rslt);
    free(f1);
    free(f2);

    lagcalc lc;
    lag_init(&lc, i1, w1, h1, i2, w2, h2, Nx, Ny);

    double biggest = -1.0E30, second = -1.0E30;
    int bigx = -1, bigy = -1;
    int nnegx = w1 - 1, nnegy = h1 - 1, nposx = w2, nposy = h2;
    int rsqr = radius * radius;

    for (int iy = 0; iy < Ny; ++iy) {
        int y = iy;
        if (y >= Ny - nnegy)
            y -= Ny;
        else if (y >= nposy) {
            memset(&rslt[(size_t)Nx * iy], 0, sizeof(double) * Nx);
            continue;
        }
        int dy = y - Oy;
        for (int ix = 0; ix < Nx; ++ix) {
            int x = ix;
            size_t i = ix + (size_t)Nx * iy;
            if (x >= Nx - nnegx)
                x -= Nx;
            else if (x >= nposx) {
                rslt[i] = 0.0;
                continue;
            }
            int dx = x - Ox;
            if (dx * dx + dy * dy > rsqr) {
                rslt[i] = 0.0;
                continue;
            }
            ibox O1, O2;
            int olw, olh;
            if (!lag_valid(&lc, L, x, y, &O1, &O2, &olw, &olh, 0)) {
                rslt[i] = 0.0;
                continue;
            }
            int odd = 0;
            double r = lag_r(&lc, O1, O2, olw, olh, rslt[i], &odd);
            if (odd && out->status == 0)
                out->status = -2; /* the reference would exit(44) here */
            rslt[i] = r;
            if (r > biggest) {
                if (biggest > second)
                    second = biggest;
                biggest = r;
                bigx = x;
                bigy = y;
            } else if (r > second)
                second = r;
        }
    }
    lag_free(&lc);
    free(i1);
    free(i2);

    out->second = second;
    if (biggest < -2.0) {
        if (!out->rslt)
            free(rslt);
        out->status = 1;
        out->r = 0.0;
        out->dx = out->dy = 0.0;
        out->bigx = out->bigy = 0;
        return 0.0;
    }
    double dx = bigx, dy = bigy;
    orc_parab_peak_fft(&dx, &dy, 1, rslt, Nx, Ny);
    dx += B2[0] - B1[0];
    dy += B2[2] - B1[2];
    if (!out->rslt)
        free(rslt);
    out->r = biggest;
    out->dx = dx;
    out->dy = dy;
    out->bigx = bigx;
    out->bigy = bigy;
    return biggest;
}

/* ------------------------------------------------------------------ */
/* Convolve, Correlation.cpp:371-457                                   */
/* ------------------------------------------------------------------ */

void orc_convolve(double *dst, const double *src, int ws, int hs,
                  const double *K, int wk, int hk, int sym, int prenorm)
{
    int Nk = wk * hk;
    int Nx = orc_fft_size(ws, wk / (1 + (sym != 0)));
    int Ny = orc_fft_size(hs, hk / (1 + (sym != 0)));
    size_t Nxy = (size_t)Nx * Ny, M = (size_t)Ny * (Nx / 2 + 1);
    double *KK = (double *)calloc(Nxy, sizeof(double));
    double nrm = 1.0;
    if (prenorm) {
        nrm = 0.0;
        for (int i = 0; i < Nk; ++i)
            nrm += K[i];
        if (!nrm)
            nrm = 1.0;
    }
    int w2 = wk / 2, h2 = hk / 2;
    for (int i = -h2; i <= h2; ++i) {
        int y = (i >= 0 ? i : Ny + i);
        for (int j = -w2; j <= w2; ++j) {
            int x = (j >= 0 ? j : Nx + j);
            KK[x + (size_t)Nx * y] = K[j + w2 + wk * (i + h2)] / nrm;
        }
    }
    double *kf = (double *)malloc(sizeof(double) * 2 * M);
    fft64_r2c_2d(Ny, Nx, KK, kf);

    double *SS = (double *)calloc(Nxy, sizeof(double));
    for (int y = 0; y < hs; ++y)
        memcpy(SS + (size_t)Nx * y, src + (size_t)ws * y, sizeof(double) * ws);
    double *sf = (double *)malloc(sizeof(double) * 2 * M);
    fft64_r2c_2d(Ny, Nx, SS, sf);
    for (size_t i = 0; i < M; ++i) {
        double a = sf[2 * i], b = sf[2 * i + 1], c = kf[2 * i], d = kf[2 * i + 1];
        sf[2 * i] = a * c - b * d;
        sf[2 * i + 1] = a * d + b * c;
    }
    fft64_c2r_2d(Ny, Nx, sf, SS);
    for (int y = 0; y < hs; ++y)
        for (int x = 0; x < ws; ++x)
            dst[x + (size_t)ws * y] = SS[x + (size_t)Nx * y] / (double)Nxy;
    free(KK);
    free(kf);
    free(SS);
    free(sf);
}

/* ------------------------------------------------------------------ */
/* CCorImg and CorrImagesF/R/S, Correlation.cpp:1851-3290              */
/* ------------------------------------------------------------------ */

typedef struct {
    int B1[4], B2[4];
    int w1, h1, w2, h2, nnegx, nposx, nnegy, nposy, cx, cy, wR, hR, nR;
} ccor;

/* CCorImg::SetDims, Correlation.cpp:1949-2005 */
static int ccor_setdims(ccor *c, const double *xy1, int n1, const double *xy2, int n2)
{
    orc_bbox(xy1, n1, c->B1);
    orc_bbox(xy2, n2, c->B2);
    c->w1 = c->B1[1] - c->B1[0] + 1;
    c->h1 = c->B1[3] - c->B1[2] + 1;
    c->w2 = c->B2[1] - c->B2[0] + 1;
    c->h2 = c->B2[3] - c->B2[2] + 1;
    c->nnegx = c->w1 - 1;
    c->nposx = c->w2;
    c->nnegy = c->h1 - 1;
    c->nposy = c->h2;
    c->cx = c->nnegx;
    c->cy = c->nnegy;
    c->wR = c->nnegx + c->nposx;
    c->hR = c->nnegy + c->nposy;
    c->nR = c->wR * c->hR;
    const int mindelta = 11 / 2 + 1;
    return !(c->nnegx < mindelta || c->nposx < mindelta || c->nnegy < mindelta ||
             c->nposy < mindelta);
}

/* CCorImg::MaskA, Correlation.cpp:2011-2054 */
static void ccor_mask(const ccor *c, unsigned char *A, int Ox, int Oy, int Rx, int Ry)
{
    if (Rx <= 0 || Ry <= 0)
        return;
    Ox += c->B1[0] - c->B2[0] + c->cx;
    Oy += c->B1[2] - c->B2[2] + c->cy;
    int xmin = Ox - Rx, xmax = Ox + Rx, ymin = Oy - Ry, ymax = Oy + Ry;
    double rx2 = Rx * Rx, asq = rx2 / ((double)Ry * Ry);
    for (int i = 0; i < c->nR; ++i) {
        int y = i / c->wR;
        if (y < ymin || y > ymax) {
            A[i] = 0;
            continue;
        }
        int x = i - c->wR * y;
        if (x < xmin || x > xmax) {
            A[i] = 0;
            continue;
        }
        x -= Ox;
        y -= Oy;
        if (x * x + asq * y * y > rx2)
            A[i] = 0;
    }
}

/* MakeRandA / MakeSandRandA, Correlation.cpp:2060-2380.
 * want_r / want_s select which of R and S to build. */
static void ccor_make(const ccor *c, double *R, double *S, unsigned char *A,
                      const double *xy1, const double *v1, int n1,
                      const double *xy2, const double *v2, int n2,
                      const aln_legal *L, int Ox, int Oy, int Rx, int Ry)
{
    int Nx = orc_fft_size(c->w1, c->w2), Ny = orc_fft_size(c->h1, c->h2);
    size_t M = (size_t)Ny * (Nx / 2 + 1), NN = (size_t)Nx * Ny;
    double *i1 = (double *)malloc(sizeof(double) * NN);
    double *i2 = (double *)malloc(sizeof(double) * NN);
    orc_image_from_points(i1, Nx, Ny, v1, xy1, n1, c->B1[0], c->B1[2]);
    orc_image_from_points(i2, Nx, Ny, v2, xy2, n2, c->B2[0], c->B2[2]);
    double *f1 = (double *)malloc(sizeof(double) * 2 * M);
    double *f2 = (double *)malloc(sizeof(double) * 2 * M);
    fft64_r2c_2d(Ny, Nx, i2, f2);
    fft64_r2c_2d(Ny, Nx, i1, f1);
    cross_spectrum(f1, f2, M);
    double *rslt = (double *)malloc(sizeof(double) * NN);
    fft64_c2r_2d(Ny, Nx, f1, rslt);

    lagcalc lc;
    lag_init(&lc, i1, c->w1, c->h1, i2, c->w2, c->h2, Nx, Ny);
    for (int y = -c->nnegy; y < c->nposy; ++y) {
        size_t iy = (size_t)Nx * (y >= 0 ? y : Ny + y);
        for (int x = -c->nnegx; x < c->nposx; ++x) {
            size_t ix = (x >= 0 ? x : Nx + x);
            int ir = c->cx + x + c->wR * (c->cy + y);
            ibox O1, O2;
            int olw, olh;
            A[ir] = (unsigned char)lag_valid(&lc, L, x, y, &O1, &O2, &olw, &olh, 1);
            double r = lag_r(&lc, O1, O2, olw, olh, rslt[ix + iy], NULL);
            R[ir] = (r > -1.0 && r < 1.0 ? r : 0.0);
        }
    }
    ccor_mask(c, A, Ox, Oy, Rx, Ry);

    if (S) {
        for (size_t i = 0; i < M; ++i) {
            double re = f1[2 * i], im = f1[2 * i + 1];
            double mag = hypot(re, im);
            if (mag > 1e-10) {
                double s = sqrt(mag);
                f1[2 * i] = re / s;
                f1[2 * i + 1] = im / s;
            }
        }
        fft64_c2r_2d(Ny, Nx, f1, rslt);
        for (int y = -c->nnegy; y < c->nposy; ++y) {
            size_t iy = (size_t)Nx * (y >= 0 ? y : Ny + y);
            for (int x = -c->nnegx; x < c->nposx; ++x) {
                size_t ix = (x >= 0 ? x : Nx + x);
                int ir = c->cx + x + c->wR * (c->cy + y);
                S[ir] = rslt[ix + iy] / lc.Nxy;
            }
        }
    }
    lag_free(&lc);
    free(i1);
    free(i2);
    free(f1);
    free(f2);
    free(rslt);
}

/* CCorImg::MakeF, Correlation.cpp:2412-2492 */
static void ccor_make_f(const ccor *c, double *F, unsigned char *A, const double *R)
{
    static const double K[9] = {-1, -1, -1, -1, 9, -1, -1, -1, -1};
    int grd = 3 / 2, wR = c->wR, hR = c->hR, nR = c->nR;
    orc_convolve(F, R, wR, hR, K, 3, 3, 1, 1);
    if (grd < 2)
        grd = 2;
    int nz = grd * wR;
    memset(A, 0, (size_t)nz);
    memset(A + nR - nz, 0, (size_t)nz);
    for (int i = 0; i < nz; ++i) {
        F[i] = 0.0;
        F[nR - nz + i] = 0.0;
    }
    for (int y = grd; y < hR - grd; ++y)
        for (int x = 0; x < grd; ++x) {
            int i = x + wR * y;
            A[i] = 0;
            F[i] = 0.0;
            i = wR - 1 - x + wR * y;
            A[i] = 0;
            F[i] = 0.0;
        }
    double vmax = 1e-7;
    for (int i = 0; i < nR; ++i)
        if (F[i] > vmax)
            vmax = F[i];
    for (int i = 0; i < nR; ++i)
        F[i] = (F[i] > 0.0) ? F[i] / vmax : 0.0;
}

/*
 * OrderF, Correlation.cpp:2509-2569.  The reference std::sorts candidate
 * indices by decreasing value (an unstable sort); this restatement breaks
 * exact ties by increasing index, which coincides with the reference
 * whenever candidate values are distinct.
 */
static int cmp_desc(const void *a, const void *b, void *key)
{
    int i = *(const int *)a, j = *(const int *)b;
    double x = ((const double *)key)[i], y = ((const double *)key)[j];
    if (x > y)
        return -1;
    if (x < y)
        return 1;
    return (i > j) - (i < j);
}

static int ccor_order(const ccor *c, int *order, const double *F,
                      const unsigned char *A, const double *R, double mincor)
{
    int n = 0;
    for (int i = 0; i < c->nR; ++i)
        if (A[i] && (mincor <= 0.0 || R[i] > mincor))
            order[n++] = i;
    qsort_r(order, (size_t)n, sizeof(int), cmp_desc, (void *)F);
    return n;
}

/* FPeak, Correlation.cpp:2580-2767 */
static int ccor_fpeak(const ccor *c, int *prx, int *pry, const int *order, int nO,
                      const double *F, const double *R, double nbmaxht)
{
    int wR = c->wR, hR = c->hR;
    unsigned char *mask = (unsigned char *)calloc((size_t)c->nR, 1);
    int found = 0;
    for (int i = 0; i < nO && !found; ++i) {
        int ri = 0x7FFFFFFF, k = order[i], ro, rm;
        if (mask[k])
            continue;
        double fpk = F[k], tol = nbmaxht * fpk;
        int ry = k / wR, rx = k - wR * ry;
        int y, x, hit;

        hit = 0;
        for (y = ry - 1; y >= 0; --y)
            if (F[rx + wR * y] <= 0.5 * fpk) {
                ri = imin(ri, ry - y);
                hit = 1;
                break;
            }
        if (!hit)
            continue;
        hit = 0;
        for (y = ry + 1; y < hR; ++y)
            if (F[rx + wR * y] <= 0.5 * fpk) {
                ri = imin(ri, y - ry);
                hit = 1;
                break;
            }
        if (!hit)
            continue;
        hit = 0;
        for (x = rx - 1; x >= 0; --x)
            if (F[x + wR * ry] <= 0.5 * fpk) {
                ri = imin(ri, rx - x);
                hit = 1;
                break;
            }
        if (!hit)
            continue;
        hit = 0;
        for (x = rx + 1; x < wR; ++x)
            if (F[x + wR * ry] <= 0.5 * fpk) {
                ri = imin(ri, x - rx);
                hit = 1;
                break;
            }
        if (!hit)
            continue;

        if (ri <= 1 && R[k] < 0.1)
            continue;
        ro = 3 * ri;
        if (ry - ro < 0 || ry + ro >= hR || rx - ro < 0 || rx + ro >= wR)
            continue;
        if ((rm = ri / 3) < 1)
            rm = 1;
        for (y = ry - rm; y <= ry + rm; ++y)
            for (x = rx - rm; x <= rx + rm; ++x)
                mask[x + wR * y] = 1;
        int bad = 0;
        for (y = ry - ro; y <= ry + ro && !bad; ++y)
            for (x = rx - ro; x <= rx + ro; ++x) {
                if (y >= ry - ri && y <= ry + ri && x >= rx - ri && x <= rx + ri)
                    continue;
                if (F[x + wR * y] > tol) {
                    bad = 1;
                    break;
                }
            }
        if (!bad) {
            *prx = rx;
            *pry = ry;
            found = 1;
        }
    }
    free(mask);
    return found;
}

/* ReturnR, Correlation.cpp:3016-3043 */
static double ccor_return_r(const ccor *c, double *dx, double *dy, int rx, int ry,
                            const double *Rreport, const double *Rtweak)
{
    double bigR = Rreport[rx + c->wR * ry];
    *dx = rx;
    *dy = ry;
    parab_peak(dx, dy, 1, Rtweak, c->wR, c->hR);
    *dx += c->B2[0] - c->B1[0] - c->cx;
    *dy += c->B2[2] - c->B1[2] - c->cy;
    return bigR;
}

double orc_corr_images(int kind, const double *xy1, const double *v1, int n1,
                       const double *xy2, const double *v2, int n2,
                       const aln_legal *L, double mincor, double nbmaxht,
                       int Ox, int Oy, int Rx, int Ry, orc_corr_out *out)
{
    orc_corr_out dummy;
    if (!out) {
        memset(&dummy, 0, sizeof dummy);
        out = &dummy;
    }
    out->status = 0;
    out->second = -1e30;
    out->r = out->dx = out->dy = 0.0;
    if (n1 <= 0 || n2 <= 0) {
        out->status = -1;
        return 0.0;
    }
    ccor c;
    if (!ccor_setdims(&c, xy1, n1, xy2, n2)) {
        out->status = 1;
        return 0.0;
    }
    out->w1 = c.w1;
    out->h1 = c.h1;
    out->w2 = c.w2;
    out->h2 = c.h2;
    out->nx = orc_fft_size(c.w1, c.w2);
    out->ny = orc_fft_size(c.h1, c.h2);
    out->b1l = c.B1[0];
    out->b1b = c.B1[2];
    out->b2l = c.B2[0];
    out->b2b = c.B2[2];
    size_t nR = (size_t)c.nR;
    double *R = out->Rimg ? out->Rimg : (double *)malloc(sizeof(double) * nR);
    double *S = NULL;
    unsigned char *A = out->Aimg ? out->Aimg : (unsigned char *)malloc(nR);
    if (kind == 2)
        S = out->Simg ? out->Simg : (double *)malloc(sizeof(double) * nR);
    ccor_make(&c, R, S, A, xy1, v1, n1, xy2, v2, n2, L, Ox, Oy, Rx, Ry);

    int *order = (int *)malloc(sizeof(int) * (nR ? nR : 1));
    int rx = 0, ry = 0, ok = 0;
    double r = 0.0, dx = 0.0, dy = 0.0;
    if (kind == 0) {
        double *F = (double *)malloc(sizeof(double) * nR);
        ccor_make_f(&c, F, A, R);
        int nO = ccor_order(&c, order, F, A, R, mincor);
        ok = nO > 0 && ccor_fpeak(&c, &rx, &ry, order, nO, F, R, nbmaxht);
        if (ok)
            r = ccor_return_r(&c, &dx, &dy, rx, ry, R, R);
        free(F);
    } else {
        const double *key = (kind == 1) ? R : S;
        int nO = ccor_order(&c, order, key, A, R, mincor);
        ok = nO > 0;
        if (ok) {
            rx = order[0] % c.wR;
            ry = order[0] / c.wR;
            out->second = (nO > 1) ? key[order[1]] : -1e30;
            r = ccor_return_r(&c, &dx, &dy, rx, ry, key, key);
            if (kind == 2) {
                double mn, sd;
                orc_stats(S, c.nR, &mn, &sd);
                out->s_mean = mn;
                out->s_sd = sd;
                out->second = 10.0 * (out->second - mn) / (sd * sqrt((double)nR));
                r = 10.0 * (r - mn) / (sd * sqrt((double)nR));
            }
        }
    }
    free(order);
    if (!out->Rimg)
        free(R);
    if (!out->Aimg)
        free(A);
    if (S && !out->Simg)
        free(S);
    if (!ok) {
        out->status = 1;
        return 0.0;
    }
    out->r = r;
    out->dx = dx;
    out->dy = dy;
    out->rx = rx;
    out->ry = ry;
    out->bigx = rx - c.cx;
    out->bigy = ry - c.cy;
    return r;
}

/* ------------------------------------------------------------------ */
/* CorrPatchToImage, Correlation.cpp:1186-1355                         */
/* ------------------------------------------------------------------ */

double orc_corr_patch_to_image(const double *xy1, const double *v1, int n1,
                               const double *i2, int Nsqr, int Ox, int Oy,
                               int radius, int bFilter, orc_corr_out *out)
{
    orc_corr_out dummy;
    if (!out) {
        memset(&dummy, 0, sizeof dummy);
        out = &dummy;
    }
    int N = (int)sqrt((double)Nsqr);
    double norm = (double)n1 * Nsqr;
    int B1[4];
    orc_bbox(xy1, n1, B1);
    int w1 = B1[1] - B1[0] + 1, h1 = B1[3] - B1[2] + 1;
    int w2 = 0, h2 = 0;
    for (int i = 0; i < Nsqr; ++i)
        if (i2[i] != 0.0) {
            int y = i / N, x = i - N * y;
            if (y > h2)
                h2 = y;
            if (x > w2)
                w2 = x;
        }
    ++w2;
    ++h2;
    double *im1 = (double *)calloc((size_t)Nsqr, sizeof(double));
    for (int i = 0; i < n1; ++i) {
        int x = (int)xy1[2 * i], y = (int)xy1[2 * i + 1];
        im1[x + (size_t)N * y] = v1[i];
    }
    size_t M = (size_t)N * (N / 2 + 1);
    double *f1 = (double *)malloc(sizeof(double) * 2 * M);
    double *f2 = (double *)malloc(sizeof(double) * 2 * M);
    fft64_r2c_2d(N, N, i2, f2);
    fft64_r2c_2d(N, N, im1, f1);
    int yrow = N / 2 + 1;
    for (size_t i = 0; i < M; ++i) {
        double a = f2[2 * i], b = f2[2 * i + 1];
        double c = f1[2 * i], d = -f1[2 * i + 1];
        double re = a * c - b * d, im = a * d + b * c;
        if (bFilter) {
            int x = (int)(i / yrow), y = (int)(i - (size_t)yrow * x);
            if (x >= N / 2)
                x -= N;
            double rad2 = ((double)x * x + (double)y * y) / 10000.0;
            double filt = rad2 > 10.0 ? 0.0 : exp(-rad2);
            re = re * filt;
            im = im * filt;
        }
        f1[2 * i] = re;
        f1[2 * i + 1] = im;
    }
    double *rslt = (double *)malloc(sizeof(double) * (size_t)Nsqr);
    fft64_c2r_2d(N, N, f1, rslt);
    double biggest = -1.0E30;
    int bigx = -1, bigy = -1, rsqr = radius * radius;
    for (int i = 0; i < Nsqr; ++i) {
        int y = i / N, x = i - N * y;
        if (y > N - h1)
            y -= N;
        else if (y >= h2)
            continue;
        if (x > N - w1)
            x -= N;
        else if (x >= w2)
            continue;
        int dx = x - Ox, dy = y - Oy;
        if (dx * dx + dy * dy > rsqr)
            continue;
        if (rslt[i] > biggest) {
            biggest = rslt[i];
            bigx = x;
            bigy = y;
        }
    }
    biggest /= norm;
    out->status = biggest > 1.0001 ? -2 : 0;
    double dx = bigx, dy = bigy;
    orc_parab_peak_fft(&dx, &dy, 1, rslt, N, N);
    out->r = biggest;
    out->dx = dx;
    out->dy = dy;
    out->bigx = bigx;
    out->bigy = bigy;
    out->nx = out->ny = N;
    free(im1);
    free(f1);
    free(f2);
    free(rslt);
    return biggest;
}

/* ------------------------------------------------------------------ */
/* CThmScan, 0_GEN/CThmScan.cpp                                        */
/* ------------------------------------------------------------------ */

typedef struct {
    const double *xya, *va, *xyb, *vb;
    int na, nb;
    long reqArea;
    int olap1D;
    orc_thm_params P;
    double Tptwk[6];
    /* pretweak sweep records (TCD.vT) */
    int nT;
    int Tsel[64];
    double Ta[64];
    double *pts;   /* scratch for rotated points */
    int ncalls;
    orc_thm_margins *M;   /* decision margins (checker instrumentation), or NULL */
} thm_state;

#define ORC_UNBOUNDED 1e30

/* ---- decision margins (checker instrumentation, no reference counterpart) */

static void note_tie(thm_state *s, double tol)
{
    s->M->nties++;
    if (tol > s->M->tolA)
        s->M->tolA = tol;
}

/* a comparison of two scores x, y; tol = how far the answer's angle can move
 * if it goes the other way */
static void note_r(thm_state *s, double x, double y, double tol)
{
    if (!s->M)
        return;
    s->M->ndec++;
    if (x == 0.0 && y == 0.0)   /* two calls without a legal lag: exact on any host */
        return;
    double m = fabs(x - y) / fmax(1.0, fmax(fabs(x), fabs(y)));
    if (m < s->M->mR)
        s->M->mR = m;
    if (m < s->M->eps)
        note_tie(s, tol);
}

/* two records' scores; calls with the same transform are the same
   computation on any host (bit for bit), so their exact tie is not one */
static void note_rec(thm_state *s, const orc_thm_rec *a, const orc_thm_rec *b, double tol)
{
    if (!s->M)
        return;
    if (memcmp(a->T, b->T, sizeof a->T) == 0) {
        s->M->ndec++;
        return;
    }
    note_r(s, a->R, b->R, tol);
}

/* an rthresh test of score x; tol as note_r */
static void note_thr(thm_state *s, double x, double thr, double tol)
{
    if (!s->M)
        return;
    double m = fabs(x - thr) / fmax(1.0, fabs(x));
    s->M->ndec++;
    if (m < s->M->mR)
        s->M->mR = m;
    if (m < s->M->eps) {
        s->M->thr_tie = 1;
        note_tie(s, tol);
    }
}

/* the correlator peak of record C is used (its X, Y steer or are the answer) */
static void note_pk(thm_state *s, const orc_thm_rec *C, double tol)
{
    if (!s->M)
        return;
    s->M->ndec++;
    if (C->pm < s->M->mR)
        s->M->mR = C->pm;
    if (C->pm < s->M->eps)
        note_tie(s, tol);
}

/* x is rounded half away from zero (the ConstXY line fits) */
static void note_round(thm_state *s, double x)
{
    if (!s->M)
        return;
    double a = fabs(x);
    double m = fabs(a - floor(a) - 0.5);
    s->M->ndec++;
    if (m < s->M->mpx)
        s->M->mpx = m;
    if (m < s->M->eps_px)
        note_tie(s, ORC_UNBOUNDED);
}

static void aff_one(double t[6])
{
    t[0] = 1; t[1] = 0; t[2] = 0;
    t[3] = 0; t[4] = 1; t[5] = 0;
}

/* TAffine::operator*, TAffine.cpp:220-232 */
static void aff_mul(double r[6], const double L[6], const double R[6])
{
    double t[6];
    t[0] = L[0] * R[0] + L[1] * R[3];
    t[1] = L[0] * R[1] + L[1] * R[4];
    t[2] = L[0] * R[2] + L[1] * R[5] + L[2];
    t[3] = L[3] * R[0] + L[4] * R[3];
    t[4] = L[3] * R[1] + L[4] * R[4];
    t[5] = L[3] * R[2] + L[4] * R[5] + L[5];
    memcpy(r, t, sizeof t);
}

/* TAffine::NUSelect and the NUSet* transforms, TAffine.cpp:60-135 */
static void aff_nu(double t[6], int sel, double a)
{
    aff_one(t);
    switch (sel) {
    case 1: t[0] = a; break;                   /* XScl */
    case 2: t[4] = a; break;                   /* YScl */
    case 3: t[1] = a; break;                   /* XSkw */
    case 4: t[3] = a; break;                   /* YSkw */
    case 5: {                                  /* Rot */
        double c = cos(a), s = sin(a);
        t[0] = c; t[1] = -s; t[3] = s; t[4] = c;
        break;
    }
    default: t[0] = a; t[4] = a; break;        /* Scl */
    }
}

/* RFromAngle, CThmScan.cpp:329-366 */
static void thm_rfromangle(thm_state *s, orc_thm_rec *C, double deg, int iaux)
{
    double R[6], T[6], D[6];
    C->A = deg;
    aff_nu(R, 5, deg * ORC_PI / 180.0);
    memcpy(T, s->Tptwk, sizeof T);
    if (iaux >= 0 && iaux < s->nT) {
        double M[6];
        aff_nu(M, s->Tsel[iaux], s->Ta[iaux]);
        aff_mul(T, M, s->Tptwk);
    }
    aff_mul(D, s->P.tdfm, T);
    aff_mul(C->T, R, D);
    for (int i = 0; i < s->na; ++i) {
        double x = s->xya[2 * i], y = s->xya[2 * i + 1];
        s->pts[2 * i] = x * C->T[0] + y * C->T[1];
        s->pts[2 * i + 1] = x * C->T[3] + y * C->T[4];
    }
    aln_legal L;
    memset(&L, 0, sizeof L);
    L.rgn_kind = ALN_RGN_MIN;
    L.rgn_a = L.rgn_b = s->olap1D;
    L.rgn_area = s->reqArea;
    L.cnt_kind = ALN_CNT_GT;
    L.cnt_n = s->reqArea;
    orc_corr_out o;
    memset(&o, 0, sizeof o);
    C->R = orc_corr_images(s->P.usecorrr ? 2 : 0, s->pts, s->va, s->na, s->xyb, s->vb,
                           s->nb, &L, 0.0, s->P.nbmaxht, s->P.Ox, s->P.Oy, s->P.Rx,
                           s->P.Ry, &o);
    C->X = o.dx;
    C->Y = o.dy;
    /* the call's own top-two margin (CorrImagesS/R: best vs runner-up key;
       CorrImagesF picks by FPeak's rules, its margin is not a score gap) */
    C->pm = (o.status == 0 && o.second > -1e29)
                ? fabs(C->R - o.second) / fmax(1.0, fabs(C->R)) : ORC_UNBOUNDED;
    s->ncalls++;
}

static int round_ref(double x) { return x >= 0.0 ? (int)(x + 0.5) : (int)(x - 0.5); }

/* std::sort by decreasing R (CSort_vC_Dec, CThmScan.cpp:502-511); ties by index */
static int cmp_vc(const void *a, const void *b, void *vc)
{
    int i = *(const int *)a, j = *(const int *)b;
    double x = ((const orc_thm_rec *)vc)[i].R, y = ((const orc_thm_rec *)vc)[j].R;
    if (x > y)
        return -1;
    if (x < y)
        return 1;
    return (i > j) - (i < j);
}

#define MAXANG 4096

/* AngleScanConstXY, CThmScan.cpp:514-621 */
static double thm_scan_constxy(thm_state *s, orc_thm_rec *best, double center,
                               double hlfwid, double step)
{
    orc_thm_rec *vC = (orc_thm_rec *)malloc(sizeof(orc_thm_rec) * MAXANG);
    int *order = (int *)malloc(sizeof(int) * MAXANG);
    best->X = best->Y = best->A = best->R = 0.0;
    best->pm = ORC_UNBOUNDED;
    int nC = 0;
    for (double a = center - hlfwid; a <= center + hlfwid && nC < MAXANG; a += step)
        vC[nC++].A = a;
    for (int ic = 0; ic < nC; ++ic)
        thm_rfromangle(s, &vC[ic], vC[ic].A, ic);
    for (int i = 0; i < nC; ++i)
        order[i] = i;
    qsort_r(order, (size_t)nC, sizeof(int), cmp_vc, vC);
    const double rthresh = 0.7;
    const int m = 3, M = 2 * m + 1;
    for (int i = 0; i < nC; ++i) {
        int ic = order[i];
        /* the ranking decides which candidate is examined next */
        if (i + 1 < nC)
            note_r(s, vC[ic].R, vC[order[i + 1]].R, ORC_UNBOUNDED);
        if (ic < m || nC - 1 - ic < m)
            continue;
        double A[7], X[7], Y[7];
        int n = 0;
        for (int j = ic - m; j <= ic + m; ++j) {
            A[n] = vC[j].A;
            X[n] = round_ref(vC[j].X);
            Y[n] = round_ref(vC[j].Y);
            note_pk(s, &vC[j], ORC_UNBOUNDED);
            note_round(s, vC[j].X);
            note_round(s, vC[j].Y);
            ++n;
        }
        double lc = orc_linefit_r(A, X, M);
        if (isfinite(lc))
            note_r(s, fabs(lc), rthresh, ORC_UNBOUNDED);
        if (isfinite(lc) && fabs(lc) < rthresh)
            continue;
        lc = orc_linefit_r(A, Y, M);
        if (isfinite(lc))
            note_r(s, fabs(lc), rthresh, ORC_UNBOUNDED);
        if (isfinite(lc) && fabs(lc) < rthresh)
            continue;
        *best = vC[ic];
        break;
    }
    free(vC);
    free(order);
    return best->R;
}

/* AngleScanMaxR, CThmScan.cpp:431-493 */
static double thm_scan_maxr(thm_state *s, orc_thm_rec *best, double center,
                            double hlfwid, double step, int favorCenter)
{
    orc_thm_rec *vC = (orc_thm_rec *)malloc(sizeof(orc_thm_rec) * MAXANG);
    int nC = 0;
    vC[nC++].A = center;
    if (favorCenter) {
        double cwide = 2.0 * step, cstep = step / 3.0;
        for (double a = center - cwide; a <= center + cwide && nC < MAXANG; a += cstep)
            vC[nC++].A = a;
        if (hlfwid >= 180) {
            double opc = center + 180;
            for (double a = opc - cwide; a <= opc + cwide && nC < MAXANG; a += cstep)
                vC[nC++].A = a;
        }
    }
    for (double a = center - hlfwid; a <= center + hlfwid && nC < MAXANG; a += step)
        vC[nC++].A = a;
    for (int ic = 0; ic < nC; ++ic)
        thm_rfromangle(s, &vC[ic], vC[ic].A, ic);
    *best = vC[0];
    for (int ic = 1; ic < nC; ++ic)
        if (vC[ic].R > best->R)
            *best = vC[ic];
    /* the maximum against every other candidate (the first maximum wins) */
    for (int ic = 0; ic < nC; ++ic)
        if (vC[ic].A != best->A || vC[ic].R != best->R)
            note_rec(s, best, &vC[ic], fabs(vC[ic].A - best->A));
    free(vC);
    return best->R;
}

static double thm_scan_sel(thm_state *s, orc_thm_rec *best, double center,
                           double hlfwid, double step, int favorCenter)
{
    if (s->P.constxy)
        return thm_scan_constxy(s, best, center, hlfwid, step);
    return thm_scan_maxr(s, best, center, hlfwid, step, favorCenter);
}

/* NewXFromParabola, CThmScan.cpp:48-61 */
static double new_x_parab(double x1, double d, double y0, double y1, double y2)
{
    double D = d * (y0 - y2) / (2 * (y0 + y2 - y1 - y1));
    if (fabs(D) <= 2 * d)
        x1 += D;
    return x1;
}

/* PTWInterp, CThmScan.cpp:119-155 (uses sweep record 0) */
static double thm_ptw_interp(thm_state *s, double *ynew, int sel, double x1, double y1,
                             double d, double deg)
{
    orc_thm_rec C;
    s->Tsel[0] = sel;
    s->Ta[0] = x1 - d;
    thm_rfromangle(s, &C, deg, 0);
    double y0 = C.R;
    s->Ta[0] = x1 + d;
    thm_rfromangle(s, &C, deg, 0);
    double y2 = C.R;
    double xnew = new_x_parab(x1, d, y0, y1, y2);
    s->Ta[0] = xnew;
    thm_rfromangle(s, &C, deg, 0);
    *ynew = C.R;
    if (xnew != x1)   /* else the same call as y1's */
        note_r(s, *ynew, y1, ORC_UNBOUNDED);
    if (*ynew < y1) {
        xnew = x1;
        *ynew = y1;
    }
    return xnew;
}

/* Pretweaks, CThmScan.cpp:205-323 */
static int thm_pretweaks(thm_state *s, double bestR, double deg, const double *bestT)
{
    int vused[5] = {0, 0, 0, 0, 0}, anychange = 0;
    const double astep = 0.02;
    const int nstep = 5;
    orc_thm_rec vC[64];
    for (int itype = 0; itype < 5; ++itype) {
        s->nT = 0;
        for (int sel = 0; sel < 5; ++sel) {
            if (vused[sel])
                continue;
            double abase = (sel >= 0 && sel <= 2) ? 1.0 : 0.0;
            for (int j = -nstep; j <= nstep; ++j) {
                vC[s->nT].A = deg;
                s->Tsel[s->nT] = sel;
                s->Ta[s->nT] = abase + j * astep;
                s->nT++;
            }
        }
        int nc = s->nT;
        for (int ic = 0; ic < nc; ++ic)
            thm_rfromangle(s, &vC[ic], vC[ic].A, ic);
        double rbest = 0;
        int ibest = -1;
        for (int ic = 0; ic < nc; ++ic)
            if (vC[ic].R > rbest) {
                rbest = vC[ic].R;
                ibest = ic;
            }
        for (int ic = 0; ic < nc; ++ic)
            if (ic != ibest) {
                if (ibest >= 0)
                    note_rec(s, &vC[ic], &vC[ibest], ORC_UNBOUNDED);
                else
                    note_r(s, vC[ic].R, 0.0, ORC_UNBOUNDED);
            }
        if (ibest == -1)
            break;
        int bsel = s->Tsel[ibest];
        double ba = s->Ta[ibest];
        const double ba0 = ba;
        ba = thm_ptw_interp(s, &rbest, bsel, ba, rbest, astep, deg);
        /* the untweaked transform scores exactly bestR on any host */
        if (!(ba == ba0 && bestT && memcmp(vC[ibest].T, bestT, 6 * sizeof(double)) == 0))
            note_r(s, rbest, bestR, ORC_UNBOUNDED);
        if (rbest > bestR) {
            double M[6];
            aff_nu(M, bsel, ba);
            aff_mul(s->Tptwk, M, s->Tptwk);
            vused[bsel] = 1;
            bestR = rbest;
            anychange = 1;
        } else
            break;
    }
    s->nT = 0;
    return anychange;
}

static double thm_scan_tweaks(thm_state *s, orc_thm_rec *best, double center,
                              double hlfwid, double step)
{
    double r0 = thm_scan_sel(s, best, center, hlfwid, step, 1);
    if (s->P.pretweak)
        note_thr(s, r0, s->P.rthresh, ORC_UNBOUNDED);
    if (r0 < s->P.rthresh) {
        if (s->P.pretweak) {
            if (thm_pretweaks(s, best->R, (best->R > 0.0 ? best->A : center),
                              best->R > 0.0 ? best->T : NULL))
                thm_scan_sel(s, best, center, hlfwid, step, 1);
        }
    }
    return best->R;
}

/* PeakHunt, CThmScan.cpp:676-728 */
static double thm_peak_hunt(thm_state *s, orc_thm_rec *best, double hlfwid)
{
    orc_thm_rec C, B0 = *best;
    double L = best->A - hlfwid, R = best->A + hlfwid, M;
    thm_rfromangle(s, best, M = (L + R) / 2.0, -1);
    while (R - L > 0.0001) {
        double a;
        thm_rfromangle(s, &C, a = (L + M) / 2.0, -1);
        /* either branch keeps the answer inside [L, R] */
        note_r(s, C.R, best->R, R - L);
        if (C.R >= best->R) {
            R = M;
            *best = C;
            M = a;
        } else
            L = a;
        thm_rfromangle(s, &C, a = (M + R) / 2.0, -1);
        note_r(s, C.R, best->R, R - L);
        if (C.R >= best->R) {
            L = M;
            *best = C;
            M = a;
        } else
            R = a;
    }
    note_r(s, B0.R, best->R, fabs(B0.A - best->A));
    if (B0.R > best->R)
        *best = B0;
    return best->R;
}

int orc_thm_search(const double *xya, const double *va, int na,
                   const double *xyb, const double *vb, int nb,
                   long reqArea, int olap1D, const orc_thm_params *P,
                   int mode, double ang0, double hfang, double step,
                   orc_thm_rec *best, int *ncalls)
{
    return orc_thm_search_m(xya, va, na, xyb, vb, nb, reqArea, olap1D, P, mode, ang0, hfang,
                            step, best, ncalls, NULL);
}

int orc_thm_search_m(const double *xya, const double *va, int na,
                     const double *xyb, const double *vb, int nb,
                     long reqArea, int olap1D, const orc_thm_params *P,
                     int mode, double ang0, double hfang, double step,
                     orc_thm_rec *best, int *ncalls, orc_thm_margins *M)
{
    thm_state s;
    memset(&s, 0, sizeof s);
    s.M = M;
    if (M) {
        M->mR = M->mpx = M->mpk = ORC_UNBOUNDED;
        M->tolA = 0.0;
        M->ndec = M->nties = M->thr_tie = 0;
    }
    s.xya = xya;
    s.va = va;
    s.na = na;
    s.xyb = xyb;
    s.vb = vb;
    s.nb = nb;
    s.reqArea = reqArea;
    s.olap1D = olap1D;
    s.P = *P;
    aff_one(s.Tptwk);
    s.pts = (double *)malloc(sizeof(double) * 2 * (size_t)(na > 0 ? na : 1));
    int err = 0;
    best->X = best->Y = best->A = best->R = -999.0;   /* CThmScan::Initialize */
    best->pm = ORC_UNBOUNDED;
    switch (mode) {
    case 0: {
        /* the short-circuit chain of DenovoBestAngle; a tie on one of the
           first two tests changes which stages run */
        double r = thm_scan_tweaks(&s, best, ang0, hfang, step);
        note_thr(&s, r, P->rthresh, ORC_UNBOUNDED);
        if (r < P->rthresh) {
            err = 1; /* errLowRDenov */
            break;
        }
        r = thm_scan_sel(&s, best, best->A, step * 2.0, step * 0.05, 0);
        note_thr(&s, r, P->rthresh, ORC_UNBOUNDED);
        if (r < P->rthresh) {
            err = 1;
            break;
        }
        r = thm_peak_hunt(&s, best, step * 0.05 * 1.5);
        note_thr(&s, r, P->rthresh, 0.0);
        if (r < P->rthresh)
            err = 1;
        break;
    }
    case 1:
        thm_rfromangle(&s, best, ang0, -1);
        break;
    case 2: {
        double r = thm_scan_tweaks(&s, best, ang0, hfang, 0.1);
        note_thr(&s, r, P->rthresh, ORC_UNBOUNDED);
        if (r < P->rthresh) {
            err = 2; /* errLowRPrior */
            break;
        }
        r = thm_peak_hunt(&s, best, 0.1 * 1.5);
        note_thr(&s, r, P->rthresh, 0.0);
        if (r < P->rthresh)
            err = 2;
        break;
    }
    case 3:
        thm_scan_sel(&s, best, ang0, hfang, step, 0);
        thm_peak_hunt(&s, best, step * 0.05 * 1.5);
        break;
    case 4:
        s.P.constxy = 0;
        thm_scan_sel(&s, best, ang0, hfang, step, 1);
        break;
    }
    /* the answer's own correlator peak: its X, Y are reported */
    if (best->R > -999.0) {
        note_pk(&s, best, ORC_UNBOUNDED);
        if (M)
            M->mpk = best->pm;
    }
    free(s.pts);
    if (ncalls)
        *ncalls = s.ncalls;
    return err;
}

/* PostTweaks (mode 5, CThmScan.cpp:796-802) and FinishAtFullRes (mode 6,
 * :810-842) from a prior best record (prior[0..3] = A, X, Y, R) and pretweak
 * transform; mirrors refwrap's ref_thm_finish. */
int orc_thm_finish(const double *xya, const double *va, int na,
                   const double *xyb, const double *vb, int nb,
                   long reqArea, int olap1D, const orc_thm_params *P, int mode,
                   const double *prior, const double *tptwk6, orc_thm_rec *best,
                   double *tptwk_out, int *ncalls)
{
    thm_state s;
    memset(&s, 0, sizeof s);
    s.xya = xya;
    s.va = va;
    s.na = na;
    s.xyb = xyb;
    s.vb = vb;
    s.nb = nb;
    s.reqArea = reqArea;
    s.olap1D = olap1D;
    s.P = *P;
    if (tptwk6)
        memcpy(s.Tptwk, tptwk6, sizeof s.Tptwk);
    else
        aff_one(s.Tptwk);
    s.pts = (double *)malloc(sizeof(double) * 2 * (size_t)(na > 0 ? na : 1));
    memset(best, 0, sizeof *best);
    best->A = prior[0];
    best->X = prior[1];
    best->Y = prior[2];
    best->R = prior[3];
    s.P.usecorrr = 1;                       /* SetUseCorrR(true) */
    s.P.Ox = (int)best->X;                  /* SetDisc((int)X, (int)Y, r, r) */
    s.P.Oy = (int)best->Y;
    if (mode == 5) {
        s.P.Rx = s.P.Ry = 40;
        thm_pretweaks(&s, best->R, best->A, NULL);
        thm_rfromangle(&s, best, best->A, -1);
    } else {
        orc_thm_rec b0 = *best;
        s.P.Rx = s.P.Ry = 80;
        thm_rfromangle(&s, best, best->A, -1);
        if (fabs(best->X - b0.X) <= 20 && fabs(best->Y - b0.Y) <= 20)
            best->R = b0.R;
        else
            *best = b0;
    }
    if (tptwk_out)
        memcpy(tptwk_out, s.Tptwk, sizeof s.Tptwk);
    free(s.pts);
    if (ncalls)
        *ncalls = s.ncalls;
    return 0;
}

/* ------------------------------------------------------------------ */
/* Mesh optimizer, 0_GEN/Correlation.cpp:1403-1721                     */
/* ------------------------------------------------------------------ */

/* NormalizeNonZeros with MeanStd::Stats (sample sd), Maths.cpp:111-124,247-268 */
static void normalize_nonzeros(double *v, int n)
{
    double sum = 0.0, sum2 = 0.0, avg, sd = 0.0;
    int m = 0;
    for (int i = 0; i < n; ++i)
        if (v[i]) {
            sum += v[i];
            sum2 += v[i] * v[i];
            ++m;
        }
    avg = sum;
    if (m > 1) {
        avg /= m;
        sd = sqrt(fmax(sum2 - m * avg * avg, 0.0) / (m - 1.0));
    }
    for (int i = 0; i < n; ++i)
        if (v[i])
            v[i] = (v[i] - avg) / sd;
}

void orc_grad_desc_step(double *bnew, double *dRdc, const double *ac, int nc,
                        const int *am_idx, const double *am_w, int k, int nm,
                        const double *av, const double *bimg, int w, int h)
{
    for (int j = 0; j < 2 * nc; ++j)
        dRdc[j] = 0.0;
    for (int i = 0; i < nm; ++i) {
        const int *ix = am_idx + (size_t)i * k;
        const double *aw = am_w + (size_t)i * k;
        double x = 0.0, y = 0.0;
        for (int s = 0; s < k; ++s)
            if (ix[s] >= 0) {
                x += aw[s] * ac[2 * ix[s]];
                y += aw[s] * ac[2 * ix[s] + 1];
            }
        if (x < 0.0 || x >= w - 1 || y < 0.0 || y >= h - 1) {
            bnew[i] = 0.0;
            continue;
        }
        int xl = (int)x, xr = xl + 1, yl = (int)y, yu = yl + 1;
        double alpha = x - xl, beta = y - yl;
        double ll = bimg[(size_t)w * yl + xl];
        double ul = bimg[(size_t)w * yu + xl];
        double ur = bimg[(size_t)w * yu + xr];
        double lr = bimg[(size_t)w * yl + xr];
        double t = lr - ll, u = ul - ll, v = ll - lr - ul + ur;
        bnew[i] = ll + alpha * t + beta * u + alpha * beta * v;
        double dbdx = t + beta * v, dbdy = u + alpha * v;
        dbdx *= av[i];
        dbdy *= av[i];
        for (int s = 0; s < k; ++s)
            if (ix[s] >= 0) {
                dRdc[2 * ix[s]] += aw[s] * dbdx;
                dRdc[2 * ix[s] + 1] += aw[s] * dbdy;
            }
    }
    normalize_nonzeros(bnew, nm);
}

double orc_corr_vectors(const double *a, const double *b, int n, int *nnz)
{
    double sum2 = 0.0;
    int nz = 0, N = n;
    for (int i = 0; i < n; ++i) {
        double prod = a[i] * b[i];
        sum2 += prod;
        if (fabs(prod) < 1.0E-8)
            ++nz;
    }
    if (!isfinite(sum2)) {
        nz = N;
        sum2 = 0.0;
    }
    N -= nz;
    if (nnz)
        *nnz = N;
    return N ? sum2 / N : 0.0;
}

double orc_improve_control_pts(double *ac, int nc, const int *am_idx, const double *am_w,
                               int k, int nm, const double *av, const double *bimg,
                               int w, int h, double ini_thresh, double fin_thresh,
                               int *iters)
{
    double *bnew = (double *)malloc(sizeof(double) * (size_t)(nm > 0 ? nm : 1));
    double *dRdc = (double *)malloc(sizeof(double) * 2 * (size_t)nc);
    double *dnew = (double *)malloc(sizeof(double) * 2 * (size_t)nc);
    double *anew = (double *)malloc(sizeof(double) * 2 * (size_t)nc);
    int inarow = 0, it = 0;
    orc_grad_desc_step(bnew, dRdc, ac, nc, am_idx, am_w, k, nm, av, bimg, w, h);
    double corr = orc_corr_vectors(av, bnew, nm, NULL), corr_last = corr;
    if (corr < ini_thresh)
        corr = 0.0;
    else if (fin_thresh >= 0) {
        for (double step = 10.0; step > 0.05;) {
            double S = 0.0;
            for (int i = 0; i < nc; ++i)
                S += dRdc[2 * i] * dRdc[2 * i] + dRdc[2 * i + 1] * dRdc[2 * i + 1];
            if (!S)
                break;   /* all derivatives zero */
            S = step / sqrt(S);
            for (int i = 0; i < nc; ++i) {
                anew[2 * i] = ac[2 * i] + S * dRdc[2 * i];
                anew[2 * i + 1] = ac[2 * i + 1] + S * dRdc[2 * i + 1];
            }
            orc_grad_desc_step(bnew, dnew, anew, nc, am_idx, am_w, k, nm, av, bimg, w, h);
            double c_new = orc_corr_vectors(av, bnew, nm, NULL);
            ++it;
            if (c_new > corr) {
                memcpy(ac, anew, sizeof(double) * 2 * (size_t)nc);
                memcpy(dRdc, dnew, sizeof(double) * 2 * (size_t)nc);
                corr_last = corr;
                corr = c_new;
            } else
                step /= 2.0;
            if (step <= 2.0 && corr - corr_last < 0.0001) {
                if (++inarow >= 3)
                    break;
            } else
                inarow = 0;
        }
    }
    free(bnew);
    free(dRdc);
    free(dnew);
    free(anew);
    if (iters)
        *iters = it;
    return corr;
}
