/*
 * fft64 -- double-precision 2D real FFTs for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker's FFT: it stands in for
 * FFTW 3.x (which the reference links, 0_GEN/Correlation_fft_fftw.cpp:10-92)
 * because neither FFTW nor MKL is installed here.  Nothing in the product
 * library links or calls it.
 *
 * Contract (the FFTW contract the reference relies on):
 *   - real input in[n0][n1] row-major (n0 = Nslow, n1 = Nfast),
 *   - r2c output out[n0][n1/2+1] complex, interleaved (re, im), sign -1,
 *   - c2r is the unnormalised inverse (result is n0*n1 times the data),
 *     columns first, then rows; the imaginary parts of the kx = 0 and
 *     kx = n1/2 bins are ignored by the row pass, as FFTW's halfcomplex
 *     row transforms do.
 *   - sizes are powers of two (the reference only ever asks for CeilPow2
 *     sizes, 0_GEN/Correlation.cpp:344-359).
 */
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

/* Returns 0 on success, -1 on a size that is not a power of two >= 2. */
int fft64_r2c_2d(int n0, int n1, const double *in, double *out_cplx);
int fft64_c2r_2d(int n0, int n1, const double *in_cplx, double *out);

/* 1D complex, in place, unnormalised.  sign = -1 forward, +1 inverse. */
int fft64_c2c_1d(int n, double *data_cplx, int sign);

#ifdef __cplusplus
}
#endif
