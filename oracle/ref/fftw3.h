/*
 * Minimal stand-in for <fftw3.h> used only to compile the reference's own
 * 0_GEN/Correlation_fft_fftw.cpp for the CPU oracle (test infrastructure).
 *
 * It declares just the four FFTW 3.x entry points that file calls
 * (0_GEN/Correlation_fft_fftw.cpp:22-26,85-89) with FFTW's public
 * signatures; fftw_shim.c implements them on top of oracle/fft64.c.
 * FFTW itself is not installed in this environment.
 */
#pragma once

typedef double fftw_complex[2];
typedef struct fftw_plan_s *fftw_plan;

#define FFTW_ESTIMATE (1U << 6)

#ifdef __cplusplus
extern "C" {
#endif

fftw_plan fftw_plan_dft_r2c_2d(int n0, int n1, double *in, fftw_complex *out,
                               unsigned flags);
fftw_plan fftw_plan_dft_c2r_2d(int n0, int n1, fftw_complex *in, double *out,
                               unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);

#ifdef __cplusplus
}
#endif
