// aln_fft.cuh -- FP32 FFT building blocks for sm_103a (shared-memory Stockham).
//
// A CTA runs G transforms of length L (a power of two) at once.  Data live
// in shared memory as float2; each pass reads one buffer and writes the
// other (Stockham autosort: no bit reversal), so a transform of length
// 2^k takes ceil(k/2) passes of radix 4 (plus one radix-2 pass when k is
// odd).  All threads of the CTA share the butterflies of all G transforms.
//
// Twiddles come from a device table tw[N + m] = exp(-2 pi i m / N) for every
// power of two N <= ALN_MAX_N, built on the host in double precision.
//
// Conventions are FFTW's (the reference's FFT_2D / IFT_2D,
// 0_GEN/Correlation_fft_fftw.cpp:10-92): forward sign -1, both directions
// unnormalised, real rows of length N become N/2+1 complex bins, and the
// inverse real pass ignores the imaginary parts of bins 0 and N/2.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#define ALN_MAX_LOG 13
#define ALN_MAX_N (1 << ALN_MAX_LOG)

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b)
{
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// exp(DIR * 2 pi i m / N), DIR = -1 forward, +1 inverse
template <int DIR>
__device__ __forceinline__ float2 twiddle(const float2 *__restrict__ tw, int N, int m)
{
    float2 w = __ldg(&tw[N + (m & (N - 1))]);
    return DIR < 0 ? w : make_float2(w.x, -w.y);
}

// One radix-4 Stockham pass over G transforms of length L (L >= 4).
// Ns = current sub-transform size (1, 4, 16, ...).
template <int DIR>
__device__ __forceinline__ void pass_r4(const float2 *src, float2 *dst, int G, int L,
                                        int logL, int Ns, int logNs,
                                        const float2 *__restrict__ tw)
{
    const int nb = L >> 2;
    const int logNb = logL - 2;
    const int total = G << logNb;
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        const int g = b >> logNb;
        const int j = b & (nb - 1);
        const float2 *s = src + (g << logL);
        float2 *d = dst + (g << logL);
        const int k = j & (Ns - 1);
        float2 a0 = s[j], a1 = s[j + nb], a2 = s[j + 2 * nb], a3 = s[j + 3 * nb];
        if (Ns > 1) {
            const int step = k << (logL - logNs - 2);
            a1 = cmul(a1, twiddle<DIR>(tw, L, step));
            a2 = cmul(a2, twiddle<DIR>(tw, L, 2 * step));
            a3 = cmul(a3, twiddle<DIR>(tw, L, 3 * step));
        }
        const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
        const float2 t2 = cadd(a1, a3), t3 = csub(a1, a3);
        // DIR * i * t3
        const float2 it3 = DIR < 0 ? make_float2(t3.y, -t3.x) : make_float2(-t3.y, t3.x);
        const int base = ((j - k) << 2) + k;
        d[base] = cadd(t0, t2);
        d[base + Ns] = cadd(t1, it3);
        d[base + 2 * Ns] = csub(t0, t2);
        d[base + 3 * Ns] = csub(t1, it3);
    }
}

template <int DIR>
__device__ __forceinline__ void pass_r2(const float2 *src, float2 *dst, int G, int L,
                                        int logL, int Ns, int logNs,
                                        const float2 *__restrict__ tw)
{
    const int nb = L >> 1;
    const int logNb = logL - 1;
    const int total = G << logNb;
    for (int b = threadIdx.x; b < total; b += blockDim.x) {
        const int g = b >> logNb;
        const int j = b & (nb - 1);
        const float2 *s = src + (g << logL);
        float2 *d = dst + (g << logL);
        const int k = j & (Ns - 1);
        float2 a0 = s[j], a1 = s[j + nb];
        if (Ns > 1)
            a1 = cmul(a1, twiddle<DIR>(tw, L, k << (logL - logNs - 1)));
        const int base = ((j - k) << 1) + k;
        d[base] = cadd(a0, a1);
        d[base + Ns] = csub(a0, a1);
    }
}

// Full transform of G sequences of length 2^logL held in buf0; buf1 is
// scratch of the same size.  Returns the buffer holding the result.  The
// caller must __syncthreads() before (data loaded) -- this routine syncs
// after every pass, so the result is visible on return.
template <int DIR>
__device__ float2 *fft_smem(float2 *buf0, float2 *buf1, int G, int logL,
                            const float2 *__restrict__ tw)
{
    const int L = 1 << logL;
    float2 *src = buf0, *dst = buf1;
    int logNs = 0;
    while (logNs + 2 <= logL) {
        pass_r4<DIR>(src, dst, G, L, logL, 1 << logNs, logNs, tw);
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
        logNs += 2;
    }
    if (logNs < logL) {
        pass_r2<DIR>(src, dst, G, L, logL, 1 << logNs, logNs, tw);
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// Real-row post-processing: Z = FFT_L(x[2n] + i x[2n+1]) (L = N/2) ->
// X[k], k = 0..L, of the length-N real transform.  twN = table base for N.
__device__ __forceinline__ float2 r2c_bin(const float2 *Z, int L, int logL, int k,
                                          const float2 *__restrict__ tw)
{
    const float2 a = Z[k & (L - 1)];
    const float2 b = cconj(Z[(L - k) & (L - 1)]);
    const float2 e = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y));
    const float2 dd = make_float2(0.5f * (a.x - b.x), 0.5f * (a.y - b.y));
    const float2 o = make_float2(dd.y, -dd.x);   // -i * dd
    const float2 w = twiddle<-1>(tw, 2 * L, k);
    return cadd(e, cmul(o, w));
}

// Real-row pre-processing for the inverse: X[0..L] (Hermitian half of a
// length-N real sequence) -> Z[k], k = 0..L-1, such that the unnormalised
// inverse FFT_L of Z gives N * (x[2n] + i x[2n+1]) / N ... i.e. exactly
// (x[2n], x[2n+1]) of the unnormalised length-N inverse.
__device__ __forceinline__ float2 c2r_pre(const float2 *X, int L, int k,
                                          const float2 *__restrict__ tw)
{
    float2 a = X[k];
    float2 b = cconj(X[L - k]);
    if (k == 0) {
        a.y = 0.f;
        b.y = 0.f;
    }
    const float2 e = cadd(a, b);
    const float2 dd = csub(a, b);
    const float2 o = cmul(dd, twiddle<+1>(tw, 2 * L, k));   // W^{-k} * dd
    return make_float2(e.x - o.y, e.y + o.x);                // e + i o
}
