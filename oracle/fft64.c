/*
 * fft64.c -- double-precision FFTs for the CPU oracle (test infrastructure).
 *
 * An iterative radix-2 Cooley-Tukey transform with per-size twiddle tables,
 * a half-length complex trick for real rows, and blocked column passes.
 * Written for this project from the textbook algorithm; it implements the
 * FFTW contract described in fft64.h.
 */
#include "fft64.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define MAXLOG 24

static pthread_mutex_t tw_lock = PTHREAD_MUTEX_INITIALIZER;
static double *tw_tab[MAXLOG + 1];   /* tw_tab[k]: n = 2^k, n/2 complex e^{-2 pi i j/n} */
static int *br_tab[MAXLOG + 1];      /* bit-reversal permutation for n = 2^k */

static int ilog2_exact(int n)
{
    if (n < 1)
        return -1;
    int k = 0;
    while ((1 << k) < n)
        ++k;
    return ((1 << k) == n && k <= MAXLOG) ? k : -1;
}

static void ensure_tables(int k)
{
    pthread_mutex_lock(&tw_lock);
    if (!tw_tab[k]) {
        int n = 1 << k;
        double *t = (double *)malloc(sizeof(double) * (size_t)(n > 1 ? n : 2));
        for (int j = 0; j < n / 2; ++j) {
            double a = -2.0 * M_PI * (double)j / (double)n;
            t[2 * j] = cos(a);
            t[2 * j + 1] = sin(a);
        }
        int *b = (int *)malloc(sizeof(int) * (size_t)n);
        for (int j = 0; j < n; ++j) {
            int r = 0;
            for (int q = 0; q < k; ++q)
                if (j & (1 << q))
                    r |= 1 << (k - 1 - q);
            b[j] = r;
        }
        br_tab[k] = b;
        /* publish the twiddles last: readers test tw_tab[k] */
        __atomic_store_n(&tw_tab[k], t, __ATOMIC_RELEASE);
    }
    pthread_mutex_unlock(&tw_lock);
}

static void c2c_pow2(int k, double *d, int sign)
{
    int n = 1 << k;
    if (n == 1)
        return;
    if (!__atomic_load_n(&tw_tab[k], __ATOMIC_ACQUIRE))
        ensure_tables(k);
    const double *tw = tw_tab[k];
    const int *br = br_tab[k];

    for (int i = 0; i < n; ++i) {
        int j = br[i];
        if (j > i) {
            double tr = d[2 * i], ti = d[2 * i + 1];
            d[2 * i] = d[2 * j];
            d[2 * i + 1] = d[2 * j + 1];
            d[2 * j] = tr;
            d[2 * j + 1] = ti;
        }
    }
    for (int len = 2; len <= n; len <<= 1) {
        int half = len >> 1, step = n / len;
        for (int s = 0; s < n; s += len) {
            for (int j = 0; j < half; ++j) {
                /* forward (sign -1) uses e^{-i..}; inverse conjugates */
                double wr = tw[2 * j * step];
                double wi = (sign > 0) ? -tw[2 * j * step + 1] : tw[2 * j * step + 1];
                double *a = d + 2 * (s + j);
                double *b = d + 2 * (s + j + half);
                double br_ = b[0] * wr - b[1] * wi;
                double bi_ = b[0] * wi + b[1] * wr;
                b[0] = a[0] - br_;
                b[1] = a[1] - bi_;
                a[0] += br_;
                a[1] += bi_;
            }
        }
    }
}

int fft64_c2c_1d(int n, double *data, int sign)
{
    int k = ilog2_exact(n);
    if (k < 0)
        return -1;
    c2c_pow2(k, data, sign);
    return 0;
}

/* e^{-2 pi i j / n} for the real-row post-processing, from the table of n. */
static inline void twid(int kn, int j, double *c, double *s)
{
    const double *tw = tw_tab[kn];
    int n = 1 << kn;
    j &= n - 1;
    if (j < n / 2) {
        *c = tw[2 * j];
        *s = tw[2 * j + 1];
    } else {
        *c = -tw[2 * (j - n / 2)];
        *s = -tw[2 * (j - n / 2) + 1];
    }
}

/* real row of length n (even, power of two) -> n/2+1 complex bins */
static void r2c_row(int kn, const double *x, double *X, double *z)
{
    int n = 1 << kn, h = n >> 1;
    for (int i = 0; i < h; ++i) {
        z[2 * i] = x[2 * i];
        z[2 * i + 1] = x[2 * i + 1];
    }
    c2c_pow2(kn - 1, z, -1);
    for (int k = 0; k <= h; ++k) {
        int k1 = (k == h) ? 0 : k;
        int k2 = (h - k) % h;
        double zr = z[2 * k1], zi = z[2 * k1 + 1];
        double cr = z[2 * k2], ci = -z[2 * k2 + 1];   /* conj(Z[h-k]) */
        double er = 0.5 * (zr + cr), ei = 0.5 * (zi + ci);
        /* O = (Z - conj) / (2i) */
        double dr = 0.5 * (zr - cr), di = 0.5 * (zi - ci);
        double or_ = di, oi = -dr;
        double c, s;
        twid(kn, k, &c, &s);
        X[2 * k] = er + (or_ * c - oi * s);
        X[2 * k + 1] = ei + (or_ * s + oi * c);
    }
}

/* n/2+1 complex bins -> real row of length n, unnormalised inverse */
static void c2r_row(int kn, const double *X, double *x, double *z)
{
    int n = 1 << kn, h = n >> 1;
    for (int k = 0; k < h; ++k) {
        double ar = X[2 * k], ai = X[2 * k + 1];
        double br = X[2 * (h - k)], bi = -X[2 * (h - k) + 1]; /* conj(X[h-k]) */
        if (k == 0) {
            /* halfcomplex rows carry no imaginary part at 0 and n/2 */
            ai = 0.0;
            bi = 0.0;
        }
        double er = ar + br, ei = ai + bi;
        double dr = ar - br, di = ai - bi;
        double c, s;
        twid(kn, k, &c, &s);
        /* O = W^{-k} * d, W^{-k} = (c, -s) */
        double or_ = dr * c + di * s;
        double oi = di * c - dr * s;
        /* Z = E + i O */
        z[2 * k] = er - oi;
        z[2 * k + 1] = ei + or_;
    }
    c2c_pow2(kn - 1, z, +1);
    for (int i = 0; i < h; ++i) {
        x[2 * i] = z[2 * i];
        x[2 * i + 1] = z[2 * i + 1];
    }
}

#define CB 8

int fft64_r2c_2d(int n0, int n1, const double *in, double *out)
{
    int k0 = ilog2_exact(n0), k1 = ilog2_exact(n1);
    if (k0 < 0 || k1 < 1)
        return -1;
    ensure_tables(k1);
    ensure_tables(k1 - 1);
    ensure_tables(k0);
    int m = n1 / 2 + 1;
    double *z = (double *)malloc(sizeof(double) * (size_t)n1);
    for (int r = 0; r < n0; ++r)
        r2c_row(k1, in + (size_t)r * n1, out + (size_t)r * 2 * m, z);
    free(z);
    double *col = (double *)malloc(sizeof(double) * 2 * (size_t)n0 * CB);
    for (int c0 = 0; c0 < m; c0 += CB) {
        int nb = (m - c0 < CB) ? m - c0 : CB;
        for (int r = 0; r < n0; ++r)
            for (int b = 0; b < nb; ++b) {
                col[2 * ((size_t)b * n0 + r)] = out[2 * ((size_t)r * m + c0 + b)];
                col[2 * ((size_t)b * n0 + r) + 1] = out[2 * ((size_t)r * m + c0 + b) + 1];
            }
        for (int b = 0; b < nb; ++b)
            c2c_pow2(k0, col + 2 * (size_t)b * n0, -1);
        for (int r = 0; r < n0; ++r)
            for (int b = 0; b < nb; ++b) {
                out[2 * ((size_t)r * m + c0 + b)] = col[2 * ((size_t)b * n0 + r)];
                out[2 * ((size_t)r * m + c0 + b) + 1] = col[2 * ((size_t)b * n0 + r) + 1];
            }
    }
    free(col);
    return 0;
}

int fft64_c2r_2d(int n0, int n1, const double *in, double *out)
{
    int k0 = ilog2_exact(n0), k1 = ilog2_exact(n1);
    if (k0 < 0 || k1 < 1)
        return -1;
    ensure_tables(k1);
    ensure_tables(k1 - 1);
    ensure_tables(k0);
    int m = n1 / 2 + 1;
    double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)n0 * m);
    double *col = (double *)malloc(sizeof(double) * 2 * (size_t)n0 * CB);
    for (int c0 = 0; c0 < m; c0 += CB) {
        int nb = (m - c0 < CB) ? m - c0 : CB;
        for (int r = 0; r < n0; ++r)
            for (int b = 0; b < nb; ++b) {
                col[2 * ((size_t)b * n0 + r)] = in[2 * ((size_t)r * m + c0 + b)];
                col[2 * ((size_t)b * n0 + r) + 1] = in[2 * ((size_t)r * m + c0 + b) + 1];
            }
        for (int b = 0; b < nb; ++b)
            c2c_pow2(k0, col + 2 * (size_t)b * n0, +1);
        for (int r = 0; r < n0; ++r)
            for (int b = 0; b < nb; ++b) {
                tmp[2 * ((size_t)r * m + c0 + b)] = col[2 * ((size_t)b * n0 + r)];
                tmp[2 * ((size_t)r * m + c0 + b) + 1] = col[2 * ((size_t)b * n0 + r) + 1];
            }
    }
    free(col);
    double *z = (double *)malloc(sizeof(double) * (size_t)n1);
    for (int r = 0; r < n0; ++r)
        c2r_row(k1, tmp + (size_t)r * 2 * m, out + (size_t)r * n1, z);
    free(z);
    free(tmp);
    return 0;
}
