/*
 * fftw_shim.c -- the four FFTW 3.x entry points the reference calls
 * (0_GEN/Correlation_fft_fftw.cpp:22-26,85-89), implemented over the
 * project's FP64 FFT (oracle/fft64.c).  Test infrastructure only: it lets the
 * reference's unmodified correlation code be compiled and run as the oracle.
 *
 * Plans carry their pointers, as FFTW plans do; FFTW_ESTIMATE is ignored.
 */
#include "fftw3.h"
#include "../fft64.h"

#include <stdio.h>
#include <stdlib.h>

struct fftw_plan_s {
    int kind;           /* 0 r2c, 1 c2r */
    int n0, n1;
    double *rin, *rout;
    double *cin, *cout;
};

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out,
                               unsigned flags)
{
    (void)flags;
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->kind = 0;
    p->n0 = n0;
    p->n1 = n1;
    p->rin = in;
    p->cout = (double *)out;
    return p;
}

fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out,
                               unsigned flags)
{
    (void)flags;
    fftw_plan p = (fftw_plan)calloc(1, sizeof(*p));
    p->kind = 1;
    p->n0 = n0;
    p->n1 = n1;
    p->cin = (double *)in;
    p->rout = out;
    return p;
}

void fftw_execute(const fftw_plan p)
{
    int rc = (p->kind == 0) ? fft64_r2c_2d(p->n0, p->n1, p->rin, p->cout)
                            : fft64_c2r_2d(p->n0, p->n1, p->cin, p->rout);
    if (rc) {
        fprintf(stderr, "fftw_shim: unsupported size %d x %d\n", p->n0, p->n1);
        abort();
    }
}

void fftw_destroy_plan(fftw_plan p)
{
    free(p);
}
