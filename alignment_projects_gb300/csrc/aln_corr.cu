// aln_corr.cu -- GB300 (sm_103a) FFT normalised cross-correlation: host
// planning and orchestration of CorrPatches (0_GEN/Correlation.cpp:901-1170),
// CorrImagesF/R/S, CorrPatchToImage, the FFT_2D / IFT_2D / Convolve drop-ins
// and the C ABI of include/aln_corr.h.
//
// The batched pipeline (aln_pipeline.cuh) runs each chunk of jobs sharing a
// transform grid: k_transpose (wide jobs), k3_sat + k_mean + k2_sat2w
// (summed-area-table rows the lag window needs, mean shifts), k2_rowfft
// (row spectra T[kx][y]), k2_corrcol or k2_corrseg (column transforms,
// spectral product, inverse; the window's lag rows -> Q), k2_lagrow /
// k2_lagimg / k2_lagp2i (inverse rows, r or S per lag, legality, row argmax),
// k_final* (argmax, ParabPeakFFT / ParabPeak, S score).  The CThmScan sweep
// (aln_sweep.cuh) and the request server (aln_server.cuh) drive it.
//
// The kernels defined in this file are the shared-memory FFT path: FFT_2D /
// IFT_2D / Convolve, the allocation-free entry point, and CorrPatches grids
// outside the register FFT's range:
//   k_colsum    column prefix sums of v, v^2, (v != 0) -> summed-area-table
//               rows the lag window needs; column totals
//   k_mean      mean of each image -> shift mu (integer for integer pixels)
//   k_rowscan   x-prefix of the needed rows -> summed-area-table rows
//   k_rowfft    per image row: (v - mu) zero-padded to Nx, real FFT,
//               written transposed T[kx][y]
//   k_colfft    image b: column FFTs -> spectrum X2[kx][ky]
//   k_corrcol   image a: column FFTs, X2 * conj(X1), inverse column FFTs,
//               only the lag rows of the window -> Q[kx][j]
//   k_lagrow    per lag row: inverse real FFT, Pearson r per lag, legality,
//               disc, row argmax
//   k_final     argmax over rows (ties: smallest storage index, as the
//               reference's row-major scan with strict '>'), ParabPeakFFT
//
// Pearson r is shift-invariant: with C' the cross sum of the mean-shifted
// images, num = n*C' - (S1 - n mu1)(S2 - n mu2) equals the reference's
// n*C - S1*S2, and d1, d2 use the unshifted sums exactly as the reference
// (CLinCorr::GetCorr, 0_GEN/Correlation.cpp:705-757).  The shift keeps the
// FP32 FFT error proportional to the signal, not to the mean.
#include "aln_fft.cuh"
#include "aln_corr_kernels.cuh"
#include "../../include/aln_corr.h"

#include <cuda_runtime.h>
#include <ctype.h>
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>
#include <sys/stat.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <set>
#include <atomic>
#include <chrono>
#include <mutex>
#include <thread>
#include <string>
#include <tuple>
#include <vector>

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------

__device__ __forceinline__ double load_px(const void *p, int dt, long long idx)
{
    switch (dt) {
    case ALN_U8: return (double)((const uint8_t *)p)[idx];
    case ALN_U16: return (double)((const uint16_t *)p)[idx];
    case ALN_F32: return (double)((const float *)p)[idx];
    default: return ((const double *)p)[idx];
    }
}

__device__ __forceinline__ int sat_slot(const PairDev &p, int i, int y)
{
    const int len0 = p.need_hi[i][0] - p.need_lo[i][0] + 1;
    return (y <= p.need_hi[i][0]) ? y - p.need_lo[i][0] : len0 + y - p.need_lo[i][1];
}

__device__ __forceinline__ bool row_needed(const PairDev &p, int i, int y)
{
    return (y >= p.need_lo[i][0] && y <= p.need_hi[i][0]) ||
           (y >= p.need_lo[i][1] && y <= p.need_hi[i][1]);
}

__device__ __forceinline__ int nslots(const PairDev &p, int i)
{
    int n = 0;
    for (int k = 0; k < 2; ++k)
        if (p.need_hi[i][k] >= p.need_lo[i][k])
            n += p.need_hi[i][k] - p.need_lo[i][k] + 1;
    return n;
}

// IntegralTable, 0_GEN/Correlation.cpp:112-150, on slot-indexed SAT rows
__device__ __forceinline__ double sat_box(const double *t, const PairDev &p, int i,
                                          int L, int R, int B, int T)
{
    const int w = p.w[i];
    double r = t[(long long)sat_slot(p, i, T) * w + R];
    if (L > 0)
        r -= t[(long long)sat_slot(p, i, T) * w + L - 1];
    if (B > 0)
        r -= t[(long long)sat_slot(p, i, B - 1) * w + R];
    if (L > 0 && B > 0)
        r += t[(long long)sat_slot(p, i, B - 1) * w + L - 1];
    return r;
}

// exact integer box sum; equals the reference's FP64 IntegralTable result
// whenever the sums are below 2^53 (always, for 8/16-bit pixels)
__device__ __forceinline__ long long sat_box_i64(const long long *t, const PairDev &p, int i,
                                                 int L, int R, int B, int T)
{
    const int w = p.w[i];
    long long r = t[(long long)sat_slot(p, i, T) * w + R];
    if (L > 0)
        r -= t[(long long)sat_slot(p, i, T) * w + L - 1];
    if (B > 0)
        r -= t[(long long)sat_slot(p, i, B - 1) * w + R];
    if (L > 0 && B > 0)
        r += t[(long long)sat_slot(p, i, B - 1) * w + L - 1];
    return r;
}

__device__ __forceinline__ int sat_box_n(const int *t, const PairDev &p, int i, int L,
                                         int R, int B, int T)
{
    const int w = p.w[i];
    int r = t[(long long)sat_slot(p, i, T) * w + R];
    if (L > 0)
        r -= t[(long long)sat_slot(p, i, T) * w + L - 1];
    if (B > 0)
        r -= t[(long long)sat_slot(p, i, B - 1) * w + R];
    if (L > 0 && B > 0)
        r += t[(long long)sat_slot(p, i, B - 1) * w + L - 1];
    return r;
}

__device__ __forceinline__ bool rgn_ok(const PairDev &p, int sx, int sy)
{
    switch (p.rgn_kind) {
    case ALN_RGN_MIN:
        return sx >= p.rgn_a && sy >= p.rgn_b && (long long)sx * sy > p.rgn_area;
    case ALN_RGN_SECTION:
        return (long long)sx * sy > p.rgn_area && (sx >= p.rgn_a || sy > p.rgn_b);
    case ALN_RGN_EXACT:
        return sx == p.rgn_a && sy == p.rgn_b;
    case ALN_RGN_TABLE:
        if (sx < 1 || sy < 1 || sx > p.table_w || sy > p.table_h)
            return false;
        return p.table[(long long)(sy - 1) * p.table_w + (sx - 1)] != 0;
    default:
        return true;
    }
}

// Pearson r of lag (x, y) given the shifted cross sum cs = C'/(Nx*Ny).
// Returns false (and r = 0) for an illegal lag, as CLinCorr::CheckSize /
// CheckDensity / GetCorr do (0_GEN/Correlation.cpp:658-757).
// num / sqrt(d1 * d2) without an FP64 divide or square root: FP32
// reciprocal square roots of the factors, one Newton step in FP64 on their
// product (relative error ~1e-14).  Factors outside the FP32 range take the
// plain formula.
__device__ __forceinline__ double div_sqrt2(double num, double d1, double d2)
{
    const double d = d1 * d2;
    if (!(d1 > 1e-30 && d1 < 1e30 && d2 > 1e-30 && d2 < 1e30))
        return num / sqrt(d);
    double y = (double)(rsqrtf((float)d1) * rsqrtf((float)d2));
    y = y * (1.5 - 0.5 * d * y * y);
    return num * y;
}

// CLinCorr::GetCorr's terms for integer pixels (0_GEN/Correlation.cpp:
// 705-757).  The normalisation terms n*Q - S^2 >= 0 are exact in unsigned
// 64-bit arithmetic (valid while n*Q < 2^64: always for 8-bit pixels, for
// 16-bit ones while n < 2^20), and the shifted sums S - n mu are exact
// integers; the rest is FP32 -- the cross sum cs comes from the FP32 FFT, so
// FP32 here adds an error of the same order (~1e-7 in r), and this GPU's
// FP64 pipe is narrow (FP64 arithmetic bounded the lag kernel).  The
// flat-overlap guard d1 d2 < n^2 1e-9 is evaluated in FP32 too.
__device__ __forceinline__ double r_int(const PairDev &p, long long n, float cs, long long s1,
                                        long long q1, long long s2, long long q2)
{
    typedef unsigned long long u64;
    const u64 un = (u64)n;
    const u64 d1 = un * (u64)q1 - (u64)s1 * (u64)s1, d2 = un * (u64)q2 - (u64)s2 * (u64)s2;
    const float f1 = __ull2float_rn(d1), f2 = __ull2float_rn(d2), fn = __ll2float_rn(n);
    if (f1 * f2 < fn * fn * 1.0e-9f)
        return 0.0;
    const long long m1 = (long long)p.mu[0], m2 = (long long)p.mu[1];
    const float num = fmaf(fn, cs, -(__ll2float_rn(s1 - n * m1) * __ll2float_rn(s2 - n * m2)));
    return (double)(num * (rsqrtf(f1) * rsqrtf(f2)));
}

// the overlap sizes for which r_int is exact on this pair's pixel types
__device__ __forceinline__ bool r_int_ok(const PairDev &p, long long n)
{
    if ((p.sat_int & 3) != 3)
        return false;
    const bool u8 = p.dt[0] == ALN_U8 && p.dt[1] == ALN_U8;
    return u8 || n < (1ll << 20);
}

// cs: the cross sum at this lag (the inverse transform's value over Nx Ny)
__device__ __forceinline__ bool lag_r(const PairDev &p, int x, int y, float cs, double &r)
{
    const int w1 = p.w[0], h1 = p.h[0], w2 = p.w[1], h2 = p.h[1];
    // BoxesFromShifts, 0_GEN/Geometry.cpp:150-176
    int L2 = max(0, x), R2 = min(w2 - 1, x + w1 - 1);
    int B2 = max(0, y), T2 = min(h2 - 1, y + h1 - 1);
    R2 = max(R2, L2);
    T2 = max(T2, B2);
    const int L1 = L2 - x, R1 = R2 - x, B1 = B2 - y, T1 = T2 - y;
    const int olw = R1 - L1 + 1, olh = T1 - B1 + 1;
    r = 0.0;
    // a transposed job evaluates LegalRgn on the caller's (untransposed) box
    if (p.rgn_kind != ALN_RGN_NONE &&
        !(p.transposed ? rgn_ok(p, olh, olw) : rgn_ok(p, olw, olh)))
        return false;
    if (p.cnt_kind == ALN_CNT_GT) {
        const int c1 = sat_box_n(p.satN[0], p, 0, L1, R1, B1, T1);
        const int c2 = sat_box_n(p.satN[1], p, 1, L2, R2, B2, T2);
        if (!(c1 > p.cnt_n && c2 > p.cnt_n))
            return false;
    }
    if (r_int_ok(p, (long long)olw * olh)) {
        r = r_int(p, (long long)olw * olh, cs,
                 sat_box_i64((const long long *)p.satS[0], p, 0, L1, R1, B1, T1),
                 sat_box_i64((const long long *)p.satQ[0], p, 0, L1, R1, B1, T1),
                 sat_box_i64((const long long *)p.satS[1], p, 1, L2, R2, B2, T2),
                 sat_box_i64((const long long *)p.satQ[1], p, 1, L2, R2, B2, T2));
        return true;
    }
    const double n = (double)(olw * olh);
    double s1, q1, s2, q2;
    if (p.sat_int & 1) {
        s1 = (double)sat_box_i64((const long long *)p.satS[0], p, 0, L1, R1, B1, T1);
        q1 = (double)sat_box_i64((const long long *)p.satQ[0], p, 0, L1, R1, B1, T1);
    } else {
        s1 = sat_box(p.satS[0], p, 0, L1, R1, B1, T1);
        q1 = sat_box(p.satQ[0], p, 0, L1, R1, B1, T1);
    }
    if (p.sat_int & 2) {
        s2 = (double)sat_box_i64((const long long *)p.satS[1], p, 1, L2, R2, B2, T2);
        q2 = (double)sat_box_i64((const long long *)p.satQ[1], p, 1, L2, R2, B2, T2);
    } else {
        s2 = sat_box(p.satS[1], p, 1, L2, R2, B2, T2);
        q2 = sat_box(p.satQ[1], p, 1, L2, R2, B2, T2);
    }
    const double num = n * (double)cs - (s1 - n * p.mu[0]) * (s2 - n * p.mu[1]);
    const double d1 = n * q1 - s1 * s1;
    const double d2 = n * q2 - s2 * s2;
    const double d = d1 * d2;
    r = (d < n * n * 1.0E-9) ? 0.0 : div_sqrt2(num, d1, d2);
    return true;
}

// RCalc::Valid + RCalc::CalcR (0_GEN/Correlation.cpp:1790-1845): legality
// of lag (x, y) and, when want_r, its Pearson r clamped to (-1, 1) (0 outside).
__device__ __forceinline__ bool lag_eval(const PairDev &p, int x, int y, double cs, bool want_r,
                                         double &r)
{
    const int w1 = p.w[0], h1 = p.h[0], w2 = p.w[1], h2 = p.h[1];
    int L2 = max(0, x), R2 = min(w2 - 1, x + w1 - 1);
    int B2 = max(0, y), T2 = min(h2 - 1, y + h1 - 1);
    R2 = max(R2, L2);
    T2 = max(T2, B2);
    const int L1 = L2 - x, R1 = R2 - x, B1 = B2 - y, T1 = T2 - y;
    const int olw = R1 - L1 + 1, olh = T1 - B1 + 1;
    bool ok = true;
    if (p.rgn_kind != ALN_RGN_NONE && !rgn_ok(p, olw, olh))
        ok = false;
    if (ok && p.cnt_kind == ALN_CNT_GT) {
        const int c1 = sat_box_n(p.satN[0], p, 0, L1, R1, B1, T1);
        const int c2 = sat_box_n(p.satN[1], p, 1, L2, R2, B2, T2);
        if (!(c1 > p.cnt_n && c2 > p.cnt_n))
            ok = false;
    }
    r = 0.0;
    if (want_r) {
        const double n = (double)(olw * olh);
        double s1, q1, s2, q2;
        if (p.sat_int & 1) {
            s1 = (double)sat_box_i64((const long long *)p.satS[0], p, 0, L1, R1, B1, T1);
            q1 = (double)sat_box_i64((const long long *)p.satQ[0], p, 0, L1, R1, B1, T1);
        } else {
            s1 = sat_box(p.satS[0], p, 0, L1, R1, B1, T1);
            q1 = sat_box(p.satQ[0], p, 0, L1, R1, B1, T1);
        }
        if (p.sat_int & 2) {
            s2 = (double)sat_box_i64((const long long *)p.satS[1], p, 1, L2, R2, B2, T2);
            q2 = (double)sat_box_i64((const long long *)p.satQ[1], p, 1, L2, R2, B2, T2);
        } else {
            s2 = sat_box(p.satS[1], p, 1, L2, R2, B2, T2);
            q2 = sat_box(p.satQ[1], p, 1, L2, R2, B2, T2);
        }
        const double num = n * cs - (s1 - n * p.mu[0]) * (s2 - n * p.mu[1]);
        const double d1 = n * q1 - s1 * s1;
        const double d2 = n * q2 - s2 * s2;
        const double d = d1 * d2;
        const double v = (d < n * n * 1.0E-9) ? 0.0 : div_sqrt2(num, d1, d2);
        r = (v > -1.0 && v < 1.0) ? v : 0.0;
    }
    return ok;
}

// CCorImg::MaskA, 0_GEN/Correlation.cpp:2011-2054, on R-image indices
__device__ __forceinline__ bool oval_ok(const PairDev &p, int ix, int iy)
{
    if (!p.oval_on)
        return true;
    if (iy < p.ocy - p.ory || iy > p.ocy + p.ory)
        return false;
    if (ix < p.ocx - p.orx || ix > p.ocx + p.orx)
        return false;
    const int x = ix - p.ocx, y = iy - p.ocy;
    return !((double)(x * x) + p.oasq * y * y > p.orx2);
}

__device__ __forceinline__ int isqrt_ll(long long v)
{
    if (v < 0)
        return -1;
    long long s = (long long)sqrt((double)v);
    while (s * s > v)
        --s;
    while ((s + 1) * (s + 1) <= v)
        ++s;
    return (int)s;
}

// ---------------------------------------------------------------------------
// summed-area tables and mean shift
// ---------------------------------------------------------------------------

// grid (ceil(maxw/128), 2, npairs), block 128: one thread per column walks
// down the rows (IntegrateImage's sums, 0_GEN/Correlation.cpp:49-105).
__global__ void k_colsum(PairDev *pairs)
{
    PairDev &p = pairs[blockIdx.z];
    const int i = blockIdx.y;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int w = p.w[i], h = p.h[i], dt = p.dt[i];
    if (c >= w || p.status != 0)
        return;
    const void *img = p.img[i];
    const long long st = p.stride[i];
    double *S = p.satS[i], *Q = p.satQ[i];
    int *N = p.satN[i];
    if (dt == ALN_U8 || dt == ALN_U16) {
        long long s = 0, q = 0;
        int nz = 0;
        for (int y = 0; y < h; ++y) {
            const long long v = dt == ALN_U8 ? ((const uint8_t *)img)[y * st + c]
                                             : ((const uint16_t *)img)[y * st + c];
            s += v;
            q += v * v;
            nz += (v != 0);
            if (row_needed(p, i, y)) {
                const long long o = (long long)sat_slot(p, i, y) * w + c;
                S[o] = (double)s;
                Q[o] = (double)q;
                N[o] = nz;
            }
        }
        p.colsum[i][c] = (double)s;
    } else {
        double s = 0.0, q = 0.0;
        int nz = 0;
        for (int y = 0; y < h; ++y) {
            const double v = load_px(img, dt, y * st + c);
            s += v;
            q += v * v;
            nz += (v != 0.0);
            if (row_needed(p, i, y)) {
                const long long o = (long long)sat_slot(p, i, y) * w + c;
                S[o] = s;
                Q[o] = q;
                N[o] = nz;
            }
        }
        p.colsum[i][c] = s;
    }
}

// grid (2, npairs), block 256: deterministic total -> mean shift
__global__ void k_mean(PairDev *pairs)
{
    PairDev &p = pairs[blockIdx.y];
    const int i = blockIdx.x;
    if (p.status != 0)
        return;
    if (p.sat_nonly) {   // no value sums: CorrImagesS correlates unshifted images
        if (threadIdx.x == 0)
            p.mu[i] = 0.0;
        return;
    }
    __shared__ double part[256];
    double s = 0.0;
    for (int c = threadIdx.x; c < p.w[i]; c += blockDim.x)
        s += p.colsum[i][c];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int k = 128; k > 0; k >>= 1) {
        if (threadIdx.x < k)
            part[threadIdx.x] += part[threadIdx.x + k];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double mean = part[0] / ((double)p.w[i] * p.h[i]);
        double mu = (p.dt[i] == ALN_U8 || p.dt[i] == ALN_U16) ? floor(mean + 0.5) : mean;
        if (p.dt[i] == ALN_F32)
            mu = (double)(float)mu;   // exactly representable in the FP32 row pass
        p.mu[i] = p.no_shift ? 0.0 : mu;
    }
}

// grid (maxslots, 2, npairs), block 256: inclusive x-prefix of one needed row
__global__ void k_rowscan(PairDev *pairs)
{
    PairDev &p = pairs[blockIdx.z];
    const int i = blockIdx.y;
    const int slot = blockIdx.x;
    if (p.status != 0 || slot >= nslots(p, i))
        return;
    const int w = p.w[i];
    double *S = p.satS[i] + (long long)slot * w;
    double *Q = p.satQ[i] + (long long)slot * w;
    int *N = p.satN[i] + (long long)slot * w;
    const int per = (w + blockDim.x - 1) / blockDim.x;
    const int c0 = threadIdx.x * per, c1 = min(w, c0 + per);
    double s = 0.0, q = 0.0;
    int n = 0;
    for (int c = c0; c < c1; ++c) {
        s += S[c];
        q += Q[c];
        n += N[c];
    }
    __shared__ double ss[256], sq[256];
    __shared__ int sn[256];
    ss[threadIdx.x] = s;
    sq[threadIdx.x] = q;
    sn[threadIdx.x] = n;
    __syncthreads();
    if (threadIdx.x == 0) {
        double as = 0.0, aq = 0.0;
        int an = 0;
        for (int t = 0; t < (int)blockDim.x; ++t) {
            const double ts = ss[t], tq = sq[t];
            const int tn = sn[t];
            ss[t] = as;
            sq[t] = aq;
            sn[t] = an;
            as += ts;
            aq += tq;
            an += tn;
        }
    }
    __syncthreads();
    s = ss[threadIdx.x];
    q = sq[threadIdx.x];
    n = sn[threadIdx.x];
    for (int c = c0; c < c1; ++c) {
        s += S[c];
        q += Q[c];
        n += N[c];
        S[c] = s;
        Q[c] = q;
        N[c] = n;
    }
}

// ---------------------------------------------------------------------------
// forward row pass: (v - mu), zero pad, real FFT, transposed store
// ---------------------------------------------------------------------------

// grid (ceil(maxh/RB), 2, npairs), block 256, smem 2*RB*(L+1) float2
__global__ void k_rowfft(PairDev *pairs, const float2 *__restrict__ tw, int RB, int only_img)
{
    extern __shared__ float2 smem[];
    PairDev &p = pairs[blockIdx.z];
    const int i = only_img >= 0 ? only_img : blockIdx.y;
    if (p.status != 0)
        return;
    const int h = p.h[i], w = p.w[i], dt = p.dt[i];
    const int y0 = blockIdx.x * RB;
    if (y0 >= h)
        return;
    const int logL = p.logNx - 1, L = 1 << logL, pitch = L + 1;
    float2 *b0 = smem, *b1 = smem + RB * pitch;
    const void *img = p.img[i];
    const long long st = p.stride[i];
    const double mu = p.mu[i];
    for (int e = threadIdx.x; e < RB * L; e += blockDim.x) {
        const int r = e >> logL, n = e & (L - 1);
        const int y = y0 + r;
        float2 z = make_float2(0.f, 0.f);
        if (y < h) {
            const int xa = 2 * n, xb = 2 * n + 1;
            if (xa < w)
                z.x = (float)(load_px(img, dt, y * st + xa) - mu);
            if (xb < w)
                z.y = (float)(load_px(img, dt, y * st + xb) - mu);
        }
        b0[r * pitch + n] = z;
    }
    __syncthreads();
    // G transforms with row pitch L+1: run the passes on a padded layout by
    // viewing each row as its own transform (pitch folded into the index).
    float2 *src = b0, *dst = b1;
    int logNs = 0;
    for (; logNs + 2 <= logL; logNs += 2) {
        const int nb = L >> 2, Ns = 1 << logNs;
        for (int b = threadIdx.x; b < RB * nb; b += blockDim.x) {
            const int g = b / nb, j = b - g * nb, k = j & (Ns - 1);
            const float2 *s = src + g * pitch;
            float2 *d = dst + g * pitch;
            float2 a0 = s[j], a1 = s[j + nb], a2 = s[j + 2 * nb], a3 = s[j + 3 * nb];
            if (Ns > 1) {
                const int step = k << (logL - logNs - 2);
                a1 = cmul(a1, twiddle<-1>(tw, L, step));
                a2 = cmul(a2, twiddle<-1>(tw, L, 2 * step));
                a3 = cmul(a3, twiddle<-1>(tw, L, 3 * step));
            }
            const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = csub(a1, a3);
            const float2 it3 = make_float2(t3.y, -t3.x);
            const int base = ((j - k) << 2) + k;
            d[base] = cadd(t0, t2);
            d[base + Ns] = cadd(t1, it3);
            d[base + 2 * Ns] = csub(t0, t2);
            d[base + 3 * Ns] = csub(t1, it3);
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    if (logNs < logL) {
        const int nb = L >> 1, Ns = 1 << logNs;
        for (int b = threadIdx.x; b < RB * nb; b += blockDim.x) {
            const int g = b / nb, j = b - g * nb, k = j & (Ns - 1);
            const float2 *s = src + g * pitch;
            float2 *d = dst + g * pitch;
            float2 a0 = s[j], a1 = s[j + nb];
            if (Ns > 1)
                a1 = cmul(a1, twiddle<-1>(tw, L, k << (logL - logNs - 1)));
            const int base = ((j - k) << 1) + k;
            d[base] = cadd(a0, a1);
            d[base + Ns] = csub(a0, a1);
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    // post-process and store transposed: T[kx][y]
    float2 *T = p.T[i];
    const int Ts = p.Ts[i];
    const int rows = min(RB, h - y0);
    for (int e = threadIdx.x; e < (L + 1) * RB; e += blockDim.x) {
        const int kx = e / RB, r = e - kx * RB;
        if (r < rows)
            T[(long long)kx * Ts + y0 + r] = r2c_bin(src + r * pitch, L, logL, kx, tw);
    }
}

// ---------------------------------------------------------------------------
// column passes
// ---------------------------------------------------------------------------

template <int DIR>
__device__ float2 *fft_cols(float2 *b0, float2 *b1, int G, int logL, int pitch,
                            const float2 *__restrict__ tw)
{
    const int L = 1 << logL;
    float2 *src = b0, *dst = b1;
    int logNs = 0;
    for (; logNs + 2 <= logL; logNs += 2) {
        const int nb = L >> 2, Ns = 1 << logNs;
        for (int b = threadIdx.x; b < G * nb; b += blockDim.x) {
            const int g = b / nb, j = b - g * nb, k = j & (Ns - 1);
            const float2 *s = src + g * pitch;
            float2 *d = dst + g * pitch;
            float2 a0 = s[j], a1 = s[j + nb], a2 = s[j + 2 * nb], a3 = s[j + 3 * nb];
            if (Ns > 1) {
                const int step = k << (logL - logNs - 2);
                a1 = cmul(a1, twiddle<DIR>(tw, L, step));
                a2 = cmul(a2, twiddle<DIR>(tw, L, 2 * step));
                a3 = cmul(a3, twiddle<DIR>(tw, L, 3 * step));
            }
            const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3), t3 = csub(a1, a3);
            const float2 it3 = DIR < 0 ? make_float2(t3.y, -t3.x) : make_float2(-t3.y, t3.x);
            const int base = ((j - k) << 2) + k;
            d[base] = cadd(t0, t2);
            d[base + Ns] = cadd(t1, it3);
            d[base + 2 * Ns] = csub(t0, t2);
            d[base + 3 * Ns] = csub(t1, it3);
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    if (logNs < logL) {
        const int nb = L >> 1, Ns = 1 << logNs;
        for (int b = threadIdx.x; b < G * nb; b += blockDim.x) {
            const int g = b / nb, j = b - g * nb, k = j & (Ns - 1);
            const float2 *s = src + g * pitch;
            float2 *d = dst + g * pitch;
            float2 a0 = s[j], a1 = s[j + nb];
            if (Ns > 1)
                a1 = cmul(a1, twiddle<DIR>(tw, L, k << (logL - logNs - 1)));
            const int base = ((j - k) << 1) + k;
            d[base] = cadd(a0, a1);
            d[base + Ns] = csub(a0, a1);
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// grid (ceil((Nx/2+1)/CG), npairs), block 256, smem 2*CG*(Ny+1) float2
// Forward column FFTs of image 1 (b): X2[kx][ky].
__global__ void k_colfft(PairDev *pairs, const float2 *__restrict__ tw, int CG)
{
    extern __shared__ float2 smem[];
    PairDev &p = pairs[blockIdx.y];
    if (p.status != 0)
        return;
    const int L = 1 << (p.logNx - 1);
    const int Ny = p.Ny, logNy = p.logNy, pitch = Ny + 1;
    const int kx0 = blockIdx.x * CG;
    if (kx0 > L)
        return;
    const int G = min(CG, L + 1 - kx0);
    float2 *b0 = smem, *b1 = smem + CG * pitch;
    const float2 *T = p.T[1];
    const int Ts = p.Ts[1], h = p.h[1];
    for (int e = threadIdx.x; e < G * Ny; e += blockDim.x) {
        const int g = e >> logNy, y = e & (Ny - 1);
        b0[g * pitch + y] = (y < h) ? T[(long long)(kx0 + g) * Ts + y] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *res = fft_cols<-1>(b0, b1, G, logNy, pitch, tw);
    for (int e = threadIdx.x; e < G * Ny; e += blockDim.x) {
        const int g = e >> logNy, y = e & (Ny - 1);
        p.X2[(long long)(kx0 + g) * Ny + y] = res[g * pitch + y];
    }
}

// grid (ceil((Nx/2+1)/CG), npairs): image 0 (a) column FFTs, cross spectrum
// X2 * conj(X1) (0_GEN/Correlation.cpp:977-985), inverse column FFTs, store
// the window's lag rows Q[kx][j].
__global__ void k_corrcol(PairDev *pairs, const float2 *__restrict__ tw, int CG)
{
    extern __shared__ float2 smem[];
    PairDev &p = pairs[blockIdx.y];
    if (p.status != 0)
        return;
    const int L = 1 << (p.logNx - 1);
    const int Ny = p.Ny, logNy = p.logNy, pitch = Ny + 1;
    const int kx0 = blockIdx.x * CG;
    if (kx0 > L)
        return;
    const int G = min(CG, L + 1 - kx0);
    float2 *b0 = smem, *b1 = smem + CG * pitch;
    const float2 *T = p.T[0];
    const int Ts = p.Ts[0], h = p.h[0];
    for (int e = threadIdx.x; e < G * Ny; e += blockDim.x) {
        const int g = e >> logNy, y = e & (Ny - 1);
        b0[g * pitch + y] = (y < h) ? T[(long long)(kx0 + g) * Ts + y] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *res = fft_cols<-1>(b0, b1, G, logNy, pitch, tw);
    float2 *oth = (res == b0) ? b1 : b0;
    for (int e = threadIdx.x; e < G * Ny; e += blockDim.x) {
        const int g = e >> logNy, y = e & (Ny - 1);
        const float2 x2 = p.X2[(long long)(kx0 + g) * Ny + y];
        res[g * pitch + y] = cmulc(x2, res[g * pitch + y]);
    }
    __syncthreads();
    float2 *fin = fft_cols<+1>(res, oth, G, logNy, pitch, tw);
    const int Wy = p.yhi - p.ylo + 1;
    for (int e = threadIdx.x; e < G * Wy; e += blockDim.x) {
        const int g = e / Wy, j = e - g * Wy;
        const int y = p.ylo + j;
        const int ys = y < 0 ? y + Ny : y;
        p.Q[(long long)(kx0 + g) * Wy + j] = fin[g * pitch + ys];
    }
}

// ---------------------------------------------------------------------------
// lag rows: inverse real FFT, normalisation, legality, disc, row argmax
// ---------------------------------------------------------------------------

__device__ __forceinline__ void best_merge(double &r, long long &k, double r2, long long k2)
{
    if (r2 > r || (r2 == r && k2 < k)) {
        r = r2;
        k = k2;
    }
}

// grid (ceil(maxWy/RBL), npairs), block 256, smem 2*RBL*(L+1) float2
__global__ void k_lagrow(PairDev *pairs, const float2 *__restrict__ tw, int RBL)
{
    extern __shared__ float2 smem[];
    __shared__ double red_r[32];
    __shared__ long long red_k[32];
    PairDev &p = pairs[blockIdx.y];
    if (p.status != 0)
        return;
    const int Wy = p.yhi - p.ylo + 1, Wx = p.xhi - p.xlo + 1;
    const int j0 = blockIdx.x * RBL;
    if (j0 >= Wy)
        return;
    const int logL = p.logNx - 1, L = 1 << logL, pitch = L + 1;
    const int Nx = p.Nx, Ny = p.Ny;
    float2 *bX = smem + RBL * pitch;   // spectrum rows (L+1 bins)
    float2 *bZ = smem;                 // pre-processed rows
    const int rows = min(RBL, Wy - j0);
    for (int e = threadIdx.x; e < (L + 1) * RBL; e += blockDim.x) {
        const int kx = e / RBL, r = e - kx * RBL;
        bX[r * pitch + kx] = (r < rows) ? p.Q[(long long)kx * Wy + j0 + r] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < RBL * L; e += blockDim.x) {
        const int r = e >> logL, k = e & (L - 1);
        bZ[r * pitch + k] = c2r_pre(bX + r * pitch, L, k, tw);
    }
    __syncthreads();
    float2 *res = fft_cols<+1>(bZ, bX, RBL, logL, pitch, tw);
    const float inv = 1.0f / ((float)Nx * (float)Ny);   // a power of two: exact
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r = 0; r < rows; ++r) {
        const int j = j0 + r, y = p.ylo + j;
        const long long dy = y - p.oy;
        const int xr = isqrt_ll(p.rsqr - dy * dy);
        const int xa = xr < 0 ? 1 : max(p.xlo, p.ox - xr);
        const int xb = xr < 0 ? 0 : min(p.xhi, p.ox + xr);
        const int ys = y < 0 ? y + Ny : y;
        double br = -1.0e30;
        long long bk = 0x7fffffffffffffffLL;
        const float *row = (const float *)(res + r * pitch);
        for (int x = p.xlo + threadIdx.x; x <= p.xhi; x += blockDim.x) {
            double rv = 0.0;
            if (x >= xa && x <= xb) {
                const int xs = x < 0 ? x + Nx : x;
                if (lag_r(p, x, y, row[xs] * inv, rv))
                    best_merge(br, bk, rv, (long long)ys * Nx + xs);
            }
            p.rr[(long long)j * Wx + (x - p.xlo)] = rv;
        }
        for (int o = 16; o > 0; o >>= 1) {
            const double r2 = __shfl_down_sync(0xffffffff, br, o);
            const long long k2 = __shfl_down_sync(0xffffffff, bk, o);
            best_merge(br, bk, r2, k2);
        }
        if (lane == 0) {
            red_r[wid] = br;
            red_k[wid] = bk;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            for (int q = 1; q < nw; ++q)
                best_merge(br, bk, red_r[q], red_k[q]);
            p.rb[j].r = br;
            p.rb[j].key = bk;
        }
        __syncthreads();
    }
}

// value at FFT storage index (xs, ys) after the reference's lag loop:
// r for a legal lag in the disc, 0 otherwise (dead zone, outside the disc,
// illegal) -- the rslt array ParabPeakFFT reads.
__device__ double stored_value(const PairDev &p, int xs, int ys)
{
    const int nnegx = p.w[0] - 1, nposx = p.w[1];
    const int nnegy = p.h[0] - 1, nposy = p.h[1];
    int x, y;
    if (xs >= p.rnx - nnegx)
        x = xs - p.rnx;
    else if (xs < nposx)
        x = xs;
    else
        return 0.0;
    if (ys >= p.rny - nnegy)
        y = ys - p.rny;
    else if (ys < nposy)
        y = ys;
    else
        return 0.0;
    if (x < p.xlo || x > p.xhi || y < p.ylo || y > p.yhi)
        return 0.0;
    const int Wx = p.xhi - p.xlo + 1;
    return p.rr[(long long)(y - p.ylo) * Wx + (x - p.xlo)];
}

// grid (npairs), block 256
__global__ void k_final(PairDev *pairs, ResultDev *res, int nreal_x_is_one, int nreal_y_is_one)
{
    __shared__ double red_r[32];
    __shared__ long long red_k[32];
    PairDev &p = pairs[blockIdx.x];
    if (p.status != 0)
        return;
    const int Wy = p.yhi - p.ylo + 1;
    double br = -1.0e30;
    long long bk = 0x7fffffffffffffffLL;
    for (int j = threadIdx.x; j < Wy; j += blockDim.x)
        best_merge(br, bk, p.rb[j].r, p.rb[j].key);
    for (int o = 16; o > 0; o >>= 1) {
        const double r2 = __shfl_down_sync(0xffffffff, br, o);
        const long long k2 = __shfl_down_sync(0xffffffff, bk, o);
        best_merge(br, bk, r2, k2);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        red_r[wid] = br;
        red_k[wid] = bk;
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q)
        best_merge(br, bk, red_r[q], red_k[q]);
    ResultDev &o = res[blockIdx.x];
    if (br < -2.0) {
        p.status = ALN_NO_PEAK;
        p.r = p.dx = p.dy = 0.0;
        p.px = p.py = 0;
        o.r = o.dx = o.dy = 0.0;
        o.status = ALN_NO_PEAK;
        o.px = o.py = 0;
        return;
    }
    const int Nx = p.Nx, Ny = p.Ny;
    const int ys0 = (int)(bk / Nx), xs0 = (int)(bk - (long long)ys0 * Nx);
    // storage index -> lag: the window's non-negative lags are stored at
    // themselves (<= xhi, yhi), the negative ones above them (x + Nx > xhi
    // because the grid is wider than the window)
    const int bigx = xs0 > p.xhi ? xs0 - Nx : xs0;
    const int bigy = ys0 > p.yhi ? ys0 - Ny : ys0;
    // ParabPeakFFT, 0_GEN/Correlation.cpp:482-517, d = 1, on the reference's
    // FFT-sized raster (nx, ny and the storage indices xs, ys are the
    // reference's, which may be larger than the transform grid).
    const int xs = bigx < 0 ? bigx + p.rnx : bigx, ys = bigy < 0 ? bigy + p.rny : bigy;
    const int nx = nreal_x_is_one ? 1 : p.rnx, ny = nreal_y_is_one ? 1 : p.rny;
    double xpk = bigx, ypk = bigy;
    const int ix = bigx, iy = bigy;
    const double z1 = br;
    double z0, z2;
    if (ix - 1 >= 0 && ix + 1 < nx && (z0 = stored_value(p, ix - 1, ys)) != 0.0 &&
        (z2 = stored_value(p, ix + 1, ys)) != 0.0) {
        z0 = 1 * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * 1)
            xpk += z0;
    }
    if (iy - 1 >= 0 && iy + 1 < ny && (z0 = stored_value(p, xs, iy - 1)) != 0.0 &&
        (z2 = stored_value(p, xs, iy + 1)) != 0.0) {
        z0 = 1 * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * 1)
            ypk += z0;
    }
    p.r = br;
    p.dx = xpk + (p.x0[1] - p.x0[0]);
    p.dy = ypk + (p.y0[1] - p.y0[0]);
    p.px = bigx;
    p.py = bigy;
    p.status = ALN_OK;
    if (p.transposed) {   // back to the caller's frame
        const double t = p.dx;
        p.dx = p.dy;
        p.dy = t;
        p.px = bigy;
        p.py = bigx;
    }
    o.r = p.r;
    o.dx = p.dx;
    o.dy = p.dy;
    o.status = ALN_OK;
    o.px = p.px;
    o.py = p.py;
}

// ---------------------------------------------------------------------------
// FFT_2D / IFT_2D drop-ins (FFTW layout, FP64 on the host side)
// ---------------------------------------------------------------------------

// X2[kx][ky] (float2) -> out[ky][kx] (double complex), FFTW r2c layout
__global__ void k_spec_to_fftw(const float2 *X, int L1, int Ny, double *out)
{
    const long long n = (long long)L1 * Ny;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int ky = (int)(e / L1), kx = (int)(e - (long long)ky * L1);
        const float2 v = X[(long long)kx * Ny + ky];
        out[2 * e] = v.x;
        out[2 * e + 1] = v.y;
    }
}

// in[ky][kx] (double complex) -> S[kx][ky] (float2)
__global__ void k_fftw_to_spec(const double *in, int L1, int Ny, float2 *S)
{
    const long long n = (long long)L1 * Ny;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int kx = (int)(e / Ny), ky = (int)(e - (long long)kx * Ny);
        S[e] = make_float2((float)in[2 * ((long long)ky * L1 + kx)],
                           (float)in[2 * ((long long)ky * L1 + kx) + 1]);
    }
}

// inverse column FFTs of S[kx][ky] (all rows) -> Q[kx][y] (in place allowed)
__global__ void k_icolfft(const float2 *S, float2 *Qo, int L1, int logNy,
                          const float2 *__restrict__ tw, int CG)
{
    extern __shared__ float2 smem[];
    const int Ny = 1 << logNy, pitch = Ny + 1;
    const int kx0 = blockIdx.x * CG;
    if (kx0 >= L1)
        return;
    const int G = min(CG, L1 - kx0);
    float2 *b0 = smem, *b1 = smem + CG * pitch;
    for (int e = threadIdx.x; e < G * Ny; e += blockDim.x) {
        const int g = e >> logNy, y = e & (Ny - 1);
        b0[g * pitch + y] = S[(long long)(kx0 + g) * Ny + y];
    }
    __syncthreads();
    float2 *res = fft_cols<+1>(b0, b1, G, logNy, pitch, tw);
    for (int e = threadIdx.x; e < G * Ny; e += blockDim.x) {
        const int g = e >> logNy, y = e & (Ny - 1);
        Qo[(long long)(kx0 + g) * Ny + y] = res[g * pitch + y];
    }
}

// inverse real rows of Q[kx][y] -> out[y][x] (double, unnormalised)
__global__ void k_irowfft(const float2 *Q, int logNx, int Ny, double *out,
                          const float2 *__restrict__ tw, int RBL)
{
    extern __shared__ float2 smem[];
    const int logL = logNx - 1, L = 1 << logL, pitch = L + 1;
    const int y0 = blockIdx.x * RBL;
    if (y0 >= Ny)
        return;
    const int rows = min(RBL, Ny - y0);
    float2 *bX = smem + RBL * pitch, *bZ = smem;
    for (int e = threadIdx.x; e < (L + 1) * RBL; e += blockDim.x) {
        const int kx = e / RBL, r = e - kx * RBL;
        bX[r * pitch + kx] = (r < rows) ? Q[(long long)kx * Ny + y0 + r] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < RBL * L; e += blockDim.x) {
        const int r = e >> logL, k = e & (L - 1);
        bZ[r * pitch + k] = c2r_pre(bX + r * pitch, L, k, tw);
    }
    __syncthreads();
    float2 *res = fft_cols<+1>(bZ, bX, RBL, logL, pitch, tw);
    const int Nx = 2 * L;
    for (int e = threadIdx.x; e < rows * Nx; e += blockDim.x) {
        const int r = e / Nx, x = e - r * Nx;
        const float *row = (const float *)(res + r * pitch);
        out[(long long)(y0 + r) * Nx + x] = (double)row[x];
    }
}

#include "aln_pipeline.cuh"

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct ProfRec {
    const char *name;
    cudaEvent_t a, b;
};

// One cached spectrum of an image b (the reference's fft2 / ftc cache
// argument): X2 in the layout k2_corrcol reads, for one FFT size and frame.
struct SpecEntry {
    float2 *X2;
    size_t bytes;
    unsigned long long tick;   // last chunk that used it
};
// (namespace, key, Nx, Ny, transposed, no_shift, radix); namespace 0: the
// caller's keys, 1: keys the library makes (the sweep's thumbnails).
// no_shift: the spectrum is of b itself (CorrImagesS) rather than of b minus
// its mean; radix: the column FFT's per-thread radix (its rounding).
typedef std::tuple<int, unsigned long long, int, int, int, int, int> SpecKey;

struct aln_ctx {
    int device;
    cudaStream_t stream;
    float2 *tw;
    char *ws;
    size_t ws_cap;
    PairDev *dpairs;          // the current chunk's entries of the batch job table
    ResultDev *dres;
    PairDev *dpairs_base;
    PairDev *htab;            // pinned host job tables, one per parity
    ResultDev *dres_base;
    size_t dpairs_cap;        // jobs the batch tables hold
    cudaStream_t cstream;     // host-to-device staging copies
    cudaEvent_t ev_copy[2];               // a window's staging is copied
    cudaEvent_t ev_wdone[2];              // a window's kernels are done (staging free)
    ResultDev *hres;          // pinned result buffer
    size_t hres_cap;
    size_t ws_budget;
    long long h2d_bytes, d2h_bytes;
    char err[512];
    // tracing: launch count always; CUDA-event times per launch when on
    long long launches;
    int prof_on;
    std::vector<ProfRec> prof;            // pending records
    std::vector<cudaEvent_t> ev_pool;
    std::map<std::string, std::pair<long long, double>> prof_acc;  // name -> (launches, ms)
    std::vector<std::string> prof_names;  // stable storage for returned names
    // spectrum cache (device-resident X2 per keyed image b)
    std::map<SpecKey, SpecEntry> spec;
    std::set<std::pair<unsigned long long, SpecKey>> spec_lru;   // (tick, key) of every entry
    std::multimap<size_t, float2 *> spec_free;   // evicted buffers by size
    size_t spec_bytes, spec_cap;                 // all buffers held / limit
    unsigned long long spec_tick;
    long long spec_hits, spec_fills, spec_evictions;
    long long host_plan_us, host_prep_us;        // batch host time: planning, chunk preparation
    int *dsel;                                   // cache-fill job lists (whole batch)
    int *hsel;                                   // their page-locked host copy
    size_t dsel_cap;
    int *dsel_cur;                               // the current chunk's list
    unsigned long long sweep_serial;             // key namespace of each sweep call
    long long chunks;                            // chunks run since the last reset
    long long h2d_copies;                        // staging transfers issued
    int seg_ns;                                  // CorrPatches column segments:
                                                 // 0 cost model, -1 off, > 0 forced length
    int sms;                                     // SM count (0: not queried yet)
    char *pts_buf[2];                            // aln_points_image rasters, per slot
    size_t pts_cap[2];
    int tune_on;                                 // measured segment choices (aln_tune.cuh)
    int split_on;                                // CorrPatches rows of 3 * 2^k, 5 * 2^k points
    int tuning;                                  // inside a timing run
    int tune_defer;                              // parallel planning: unknown classes wait
    long long tune_classes;                      // classes this context measured
};

static cudaEvent_t ev_get(aln_ctx *c)
{
    if (!c->ev_pool.empty()) {
        cudaEvent_t e = c->ev_pool.back();
        c->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

static void prof_begin(aln_ctx *c, const char *name)
{
    c->launches++;
    if (!c->prof_on)
        return;
    ProfRec r;
    r.name = name;
    r.a = ev_get(c);
    r.b = ev_get(c);
    cudaEventRecord(r.a, c->stream);
    c->prof.push_back(r);
}

static void prof_end(aln_ctx *c)
{
    if (c->prof_on && !c->prof.empty())
        cudaEventRecord(c->prof.back().b, c->stream);
}

// the same for work on the copy stream (host-to-device staging)
static void prof_begin_copy(aln_ctx *c, const char *name)
{
    if (!c->prof_on)
        return;
    ProfRec r;
    r.name = name;
    r.a = ev_get(c);
    r.b = ev_get(c);
    cudaEventRecord(r.a, c->cstream);
    c->prof.push_back(r);
}

static void prof_end_copy(aln_ctx *c)
{
    if (c->prof_on && !c->prof.empty())
        cudaEventRecord(c->prof.back().b, c->cstream);
}

// fold finished records into the per-kernel totals (stream must be idle)
static void prof_collect(aln_ctx *c)
{
    for (auto &r : c->prof) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, r.a, r.b);
        auto &acc = c->prof_acc[r.name];
        acc.first += 1;
        acc.second += ms;
        c->ev_pool.push_back(r.a);
        c->ev_pool.push_back(r.b);
    }
    c->prof.clear();
}

#define LAUNCH(c, name, kern, grid, block, smem, ...)                               \
    do {                                                                             \
        prof_begin(c, name);                                                         \
        kern<<<grid, block, smem, (c)->stream>>>(__VA_ARGS__);                       \
        prof_end(c);                                                                 \
    } while (0)

// errors of calls made without a context (aln_ctx_create, the planning
// query, the allocation-free entry point): one message per host thread
static thread_local char g_create_err[512];

// (a context's message under a lock: batch planning runs on several host
// threads)
static std::mutex g_err_lock;
static int set_err(aln_ctx *c, int code, const char *fmt, ...)
{
    char *buf = c ? c->err : g_create_err;
    va_list ap;
    va_start(ap, fmt);
    if (c) {
        std::lock_guard<std::mutex> g(g_err_lock);
        vsnprintf(buf, 512, fmt, ap);
    } else {
        vsnprintf(buf, 512, fmt, ap);
    }
    va_end(ap);
    return code;
}

#define CK(call)                                                                     \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess)                                                       \
            return set_err(ctx, ALN_ERR_CUDA, "%s: %s (%s:%d)", #call,               \
                           cudaGetErrorString(e_), __FILE__, __LINE__);              \
    } while (0)

static const int kSmemMax = 200 * 1024;

// Raise a kernel's dynamic shared-memory limit once per (device, kernel),
// not before every launch: the attribute call is a driver round trip.
static std::mutex g_attr_lock;
static std::map<std::pair<int, const void *>, int> g_attr_set;

static void smem_attr(int device, const void *fn, size_t bytes)
{
    std::lock_guard<std::mutex> lk(g_attr_lock);
    int &cur = g_attr_set[std::make_pair(device, fn)];
    if ((int)bytes > cur) {
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        cur = (int)bytes;
    }
}

static int configure_kernels()
{
    const void *ks[] = {(const void *)k_rowfft, (const void *)k_colfft,
                        (const void *)k_corrcol, (const void *)k_lagrow,
                        (const void *)k_icolfft, (const void *)k_irowfft};
    for (const void *k : ks) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmemMax);
        if (e != cudaSuccess)
            return (int)e;
    }
    return 0;
}

extern "C" int aln_ctx_create(int device, aln_ctx **out)
{
    *out = nullptr;
    aln_ctx *ctx = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess)
        return set_err(nullptr, ALN_ERR_CUDA, "cudaSetDevice(%d): %s", device,
                       cudaGetErrorString(e));
    ctx = new aln_ctx();
    ctx->device = device;
    ctx->stream = nullptr;
    ctx->tw = nullptr;
    ctx->ws = nullptr;
    ctx->ws_cap = 0;
    ctx->dpairs = nullptr;
    ctx->dres = nullptr;
    ctx->dpairs_base = nullptr;
    ctx->htab = nullptr;
    ctx->dres_base = nullptr;
    ctx->dpairs_cap = 0;
    ctx->cstream = nullptr;
    ctx->hres = nullptr;
    ctx->hres_cap = 0;
    ctx->h2d_bytes = ctx->d2h_bytes = 0;
    ctx->err[0] = 0;
    ctx->launches = 0;
    ctx->prof_on = 0;
    ctx->ws_budget = (size_t)4 << 30;
    ctx->spec_bytes = 0;
    ctx->spec_cap = (size_t)8 << 30;
    ctx->spec_tick = 0;
    ctx->spec_hits = ctx->spec_fills = ctx->spec_evictions = 0;
    ctx->host_plan_us = ctx->host_prep_us = 0;
    ctx->dsel = nullptr;
    ctx->hsel = nullptr;
    ctx->dsel_cap = 0;
    ctx->dsel_cur = nullptr;
    ctx->sweep_serial = 0;
    ctx->chunks = 0;
    ctx->h2d_copies = 0;
    ctx->seg_ns = 0;
    ctx->sms = 0;
    {
        const char *t = getenv("ALN_TUNE");
        ctx->tune_on = !(t && t[0] == '0');
    }
    ctx->split_on = 1;
    ctx->tuning = 0;
    ctx->tune_defer = 0;
    ctx->tune_classes = 0;
    ctx->pts_buf[0] = ctx->pts_buf[1] = nullptr;
    ctx->pts_cap[0] = ctx->pts_cap[1] = 0;
    // the copy stream at the device's highest priority: its staging blocks
    // are scheduled ahead of the compute kernels' waiting blocks
    int prio_lo = 0, prio_hi = 0;
    cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&ctx->cstream, cudaStreamNonBlocking, prio_hi)) !=
            cudaSuccess) {
        set_err(nullptr, ALN_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
        delete ctx;
        return ALN_ERR_CUDA;
    }
    for (int q = 0; q < 2; ++q)
        if ((e = cudaEventCreateWithFlags(&ctx->ev_copy[q], cudaEventDisableTiming)) !=
                cudaSuccess ||
            (e = cudaEventCreateWithFlags(&ctx->ev_wdone[q], cudaEventDisableTiming)) !=
                cudaSuccess) {
            set_err(nullptr, ALN_ERR_CUDA, "events: %s", cudaGetErrorString(e));
            delete ctx;
            return ALN_ERR_CUDA;
        }
    if (int ke = configure_kernels()) {
        set_err(nullptr, ALN_ERR_CUDA, "kernel attributes: %s",
                cudaGetErrorString((cudaError_t)ke));
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return ALN_ERR_CUDA;
    }
    // twiddle tables tw[base + N + m] = exp(-2 pi i m / N): every power of
    // two N <= ALN_MAX_N (base 0), then N = 3 * 2^k and N = 5 * 2^k
    // (tw_base(N), aln_fft_reg.cuh)
    std::vector<float2> h(TW_TOTAL, make_float2(0.f, 0.f));
    h[0] = make_float2(1.f, 0.f);
    for (int n1 : {1, 3, 5})
        for (int N = n1; N <= ALN_MAX_N; N <<= 1)
            for (int m = 0; m < N; ++m) {
                const double a = -2.0 * M_PI * (double)m / (double)N;
                h[tw_base(N) + N + m] = make_float2((float)cos(a), (float)sin(a));
            }
    if ((e = cudaMalloc(&ctx->tw, sizeof(float2) * h.size())) != cudaSuccess ||
        (e = cudaMemcpy(ctx->tw, h.data(), sizeof(float2) * h.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess) {
        set_err(nullptr, ALN_ERR_CUDA, "twiddles: %s", cudaGetErrorString(e));
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return ALN_ERR_CUDA;
    }
    *out = ctx;
    return ALN_OK;
}

extern "C" void aln_ctx_destroy(aln_ctx *ctx)
{
    if (!ctx)
        return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->tw);
    cudaFree(ctx->ws);
    cudaStreamSynchronize(ctx->cstream);
    cudaFree(ctx->dpairs_base);
    cudaFree(ctx->dres_base);
    if (ctx->htab)
        cudaFreeHost(ctx->htab);
    for (auto &e : ctx->spec)
        cudaFree(e.second.X2);
    for (auto &f : ctx->spec_free)
        cudaFree(f.second);
    cudaFree(ctx->dsel);
    if (ctx->hsel)
        cudaFreeHost(ctx->hsel);
    for (int q = 0; q < 2; ++q)
        if (ctx->pts_buf[q])
            cudaFree(ctx->pts_buf[q]);
    if (ctx->hres)
        cudaFreeHost(ctx->hres);
    for (int q = 0; q < 2; ++q) {
        cudaEventDestroy(ctx->ev_copy[q]);
        cudaEventDestroy(ctx->ev_wdone[q]);
    }
    cudaStreamDestroy(ctx->cstream);
    prof_collect(ctx);
    for (cudaEvent_t e : ctx->ev_pool)
        cudaEventDestroy(e);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
}

extern "C" const char *aln_last_error(const aln_ctx *ctx)
{
    return ctx ? ctx->err : g_create_err;
}

static int ceil_pow2(int n)
{
    int p = 1;
    while (p < n)
        p *= 2;
    return p;
}

extern "C" int aln_fft_size(int n1, int n2) { return ceil_pow2(n1 + n2 - 1); }

// CorrPatches row half-lengths L = 3 * 2^k and 5 * 2^k (grids Nx = 2L of
// 160-3072 points) the row kernels are built for, ascending
#define ALN_CASES_LMIX(X) X(80) X(96) X(160) X(192) X(320) X(384) X(640) X(768) X(1280) X(1536)

// The CorrPatches grid length for `need` points: the smallest power of two
// >= need, or with split lengths on the smallest 2L >= need of
// ALN_CASES_LMIX when that is shorter.  The FFT's work per row and the
// number of column transforms both scale with the length, and the row
// transform's cost per point barely depends on the split (a radix-3 or
// radix-5 step in registers), so the shortest grid is the fastest.
static int patches_len(int need, bool split)
{
    int best = std::max(2, ceil_pow2(need));
    if (split) {
#define X(v) if (2 * (v) >= need && 2 * (v) < best) best = 2 * (v); else
        ALN_CASES_LMIX(X) {}
#undef X
    }
    return best;
}

extern "C" int aln_fft_size_sqr(int w1, int h1, int w2, int h2)
{
    return ceil_pow2(std::max(w1 + w2, h1 + h2) - 1);
}

static int ilog2(int n)
{
    int k = 0;
    while ((1 << k) < n)
        ++k;
    return k;
}

static size_t dtype_size(int dt)
{
    switch (dt) {
    case ALN_U8: return 1;
    case ALN_U16: return 2;
    case ALN_F32: return 4;
    case ALN_F64: return 8;
    default: return 0;
    }
}

static int ensure_ws(aln_ctx *ctx, size_t bytes)
{
    if (bytes <= ctx->ws_cap)
        return ALN_OK;
    if (ctx->ws) {
        CK(cudaStreamSynchronize(ctx->cstream));
        CK(cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->ws);
        ctx->ws = nullptr;
        ctx->ws_cap = 0;
    }
    size_t cap = bytes + bytes / 4;
    cudaError_t e = cudaMalloc(&ctx->ws, cap);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_err(ctx, ALN_ERR_NOMEM, "workspace of %zu bytes: %s", cap,
                       cudaGetErrorString(e));
    }
    ctx->ws_cap = cap;
    return ALN_OK;
}

static int ensure_pairs(aln_ctx *ctx, size_t n)
{
    ctx->dpairs = ctx->dpairs_base;
    ctx->dres = ctx->dres_base;
    if (n <= ctx->dpairs_cap)
        return ALN_OK;
    if (ctx->dpairs_base) {
        CK(cudaStreamSynchronize(ctx->stream));
        cudaFree(ctx->dpairs_base);
        cudaFree(ctx->dres_base);
        cudaFreeHost(ctx->htab);
        ctx->htab = nullptr;
        ctx->dpairs = ctx->dpairs_base = nullptr;
        ctx->dres = ctx->dres_base = nullptr;
        ctx->dpairs_cap = 0;
    }
    size_t cap = std::max<size_t>(n + n / 4, 64);
    CK(cudaMalloc(&ctx->dpairs_base, cap * sizeof(PairDev)));
    CK(cudaHostAlloc((void **)&ctx->htab, cap * sizeof(PairDev), cudaHostAllocDefault));
    CK(cudaMalloc(&ctx->dres_base, cap * sizeof(ResultDev)));
    ctx->dpairs = ctx->dpairs_base;
    ctx->dres = ctx->dres_base;
    ctx->dpairs_cap = cap;
    return ALN_OK;
}

static inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// CorrImagesF/R/S parameters of a job (0_GEN/Correlation.h:159-220).
struct ImgSpec {
    int kind;   // 0 CorrPatches (no spec), 1 R, 2 S, 3 CorrPatchToImage, 4 F
    double mincor, nbmaxht;
    int ox, oy, rx, ry;
    // CorrPatchToImage
    int p2i_w1, p2i_h1, p2i_w2, p2i_h2, p2i_filter;
    double p2i_norm;
};

// Host-side plan of one pair: sizes, window, needed SAT rows, workspace.
struct PairPlan {
    PairDev d;
    int orig_nx, orig_ny;        // the reference's FFT size (caller's frame)
    int frame_nx1, frame_ny1;    // the solving frame's FFT size is 1 on that axis
    int transposed;
    size_t ws_bytes;
    size_t in_bytes[2];          // staging of host inputs (caller's layout)
    size_t tr_bytes[2];          // transposed copies
    const aln_pair *src;
    int index;
    int key_ns;                  // spectrum-cache key of image b (0: none)
    unsigned long long key;
    char *staged[2];             // device staging of host inputs (set per window)
    int tune_deferred;           // planned while its autotuner class was unknown
};

// Cache entry bookkeeping: the map and the (tick, key) LRU index together.
static void spec_touch(aln_ctx *ctx, std::map<SpecKey, SpecEntry>::iterator it)
{
    ctx->spec_lru.erase(std::make_pair(it->second.tick, it->first));
    it->second.tick = ctx->spec_tick;
    ctx->spec_lru.insert(std::make_pair(it->second.tick, it->first));
}
static void spec_insert(aln_ctx *ctx, const SpecKey &K, const SpecEntry &e)
{
    ctx->spec[K] = e;
    ctx->spec_lru.insert(std::make_pair(e.tick, K));
}
static std::map<SpecKey, SpecEntry>::iterator
spec_erase(aln_ctx *ctx, std::map<SpecKey, SpecEntry>::iterator it)
{
    ctx->spec_lru.erase(std::make_pair(it->second.tick, it->first));
    return ctx->spec.erase(it);
}

// Whether `bytes` more of device memory leave the workspace budget plus
// 2 GiB free (the cache grows into free HBM, never into what the batches
// need next).
static bool spec_room(aln_ctx *ctx, size_t bytes)
{
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return fr >= bytes + ctx->ws_budget + ((size_t)2 << 30);
}

// A device buffer for a new cache entry of `bytes`, evicting entries not used
// by the current chunk (least recently used first) while the cache is at its
// cap or the device is short of free memory.  Buffers are reused on the
// context's stream, so a kernel still reading an evicted entry finishes
// before the buffer is filled again.  Returns NULL when nothing fits.
static float2 *spec_alloc(aln_ctx *ctx, size_t bytes)
{
    auto f = ctx->spec_free.find(bytes);
    if (f != ctx->spec_free.end()) {
        float2 *b = f->second;
        ctx->spec_free.erase(f);
        return b;
    }
    while (ctx->spec_bytes + bytes > ctx->spec_cap || !spec_room(ctx, bytes)) {
        if (!ctx->spec_free.empty()) {
            auto g = std::prev(ctx->spec_free.end());
            cudaFree(g->second);   // waits for the device: rare
            ctx->spec_bytes -= g->first;
            ctx->spec_free.erase(g);
            continue;
        }
        if (ctx->spec_lru.empty() || ctx->spec_lru.begin()->first >= ctx->spec_tick)
            return nullptr;   // every entry is in use by the current chunk
        auto lru = ctx->spec.find(ctx->spec_lru.begin()->second);
        float2 *b = lru->second.X2;
        const size_t lb = lru->second.bytes;
        spec_erase(ctx, lru);
        ctx->spec_evictions++;
        if (lb == bytes)
            return b;
        ctx->spec_free.insert(std::make_pair(lb, b));
    }
    float2 *b = nullptr;
    if (cudaMalloc(&b, bytes) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    ctx->spec_bytes += bytes;
    return b;
}

// Drops every entry of namespace ns with key in [k0, k1] (buffers kept for reuse).
static void spec_drop(aln_ctx *ctx, int ns, unsigned long long k0, unsigned long long k1)
{
    for (auto it = ctx->spec.begin(); it != ctx->spec.end();) {
        if (std::get<0>(it->first) == ns && std::get<1>(it->first) >= k0 &&
            std::get<1>(it->first) <= k1) {
            ctx->spec_free.insert(std::make_pair(it->second.bytes, it->second.X2));
            it = spec_erase(ctx, it);
        } else {
            ++it;
        }
    }
}

static void need_rows(const PairDev &d, int img, int lo[2], int hi[2])
{
    // rows T and B-1 (when B > 0) of the overlap box for every lag row
    int tmin = 1 << 30, tmax = -1, bmin = 1 << 30, bmax = -1;
    const int h1 = d.h[0], h2 = d.h[1];
    for (int y = d.ylo; y <= d.yhi; ++y) {
        int B2 = std::max(0, y), T2 = std::min(h2 - 1, y + h1 - 1);
        T2 = std::max(T2, B2);
        const int B = img == 0 ? B2 - y : B2;
        const int T = img == 0 ? T2 - y : T2;
        tmin = std::min(tmin, T);
        tmax = std::max(tmax, T);
        if (B > 0) {
            bmin = std::min(bmin, B - 1);
            bmax = std::max(bmax, B - 1);
        }
    }
    int a0 = tmin, a1 = tmax, c0 = bmin, c1 = bmax;
    if (c1 < c0) {
        lo[0] = a0;
        hi[0] = a1;
        lo[1] = 1;
        hi[1] = 0;
        return;
    }
    if (c0 < a0) {
        std::swap(a0, c0);
        std::swap(a1, c1);
    }
    if (c0 <= a1 + 1) {
        lo[0] = a0;
        hi[0] = std::max(a1, c1);
        lo[1] = 1;
        hi[1] = 0;
    } else {
        lo[0] = a0;
        hi[0] = a1;
        lo[1] = c0;
        hi[1] = c1;
    }
}

#include "aln_tune.cuh"

// allow_split: the caller runs the register pipeline (batch path), whose row
// kernels take the split lengths of ALN_CASES_LMIX; the allocation-free
// entry point's kernels take powers of two only.
static int plan_pair(aln_ctx *ctx, const aln_pair &P, PairPlan &pl, bool allow_transpose = false,
                     const ImgSpec *spec = nullptr, bool allow_segment = false,
                     bool allow_split = false)
{
    if (spec)
        allow_transpose = false;   // the R image keeps the caller's orientation
    PairDev &d = pl.d;
    memset(&d, 0, sizeof d);
    const aln_image *im[2] = {&P.a, &P.b};
    for (int i = 0; i < 2; ++i) {
        if (!im[i]->data || im[i]->w < 1 || im[i]->h < 1 || im[i]->stride < im[i]->w ||
            !dtype_size(im[i]->dtype))
            return set_err(ctx, ALN_ERR_ARG, "image %d: bad data/size/stride/dtype", i);
        d.img[i] = im[i]->data;
        d.dt[i] = im[i]->dtype;
        d.stride[i] = im[i]->stride;
        d.w[i] = im[i]->w;
        d.h[i] = im[i]->h;
        d.x0[i] = im[i]->x0;
        d.y0[i] = im[i]->y0;
    }
    pl.orig_nx = ceil_pow2(d.w[0] + d.w[1] - 1);
    pl.orig_ny = ceil_pow2(d.h[0] + d.h[1] - 1);
    d.ox = P.ox;
    d.oy = P.oy;
    // Wide pairs are solved transposed: their summed-area rows are then short
    // (and the FFT shapes match the tall pairs').  r, the disc and the
    // sub-pixel rules are symmetric in x and y; legality is evaluated on the
    // caller's box orientation.
    pl.transposed = allow_transpose && (d.w[0] + d.w[1]) > (d.h[0] + d.h[1]);
    if (pl.transposed) {
        d.transposed = 1;
        for (int i = 0; i < 2; ++i) {
            d.src_img[i] = d.img[i];
            d.src_stride[i] = d.stride[i];
            std::swap(d.w[i], d.h[i]);
            std::swap(d.x0[i], d.y0[i]);
        }
        std::swap(d.ox, d.oy);
    }
    const int fnx = ceil_pow2(d.w[0] + d.w[1] - 1), fny = ceil_pow2(d.h[0] + d.h[1] - 1);
    pl.frame_nx1 = fnx == 1;
    pl.frame_ny1 = fny == 1;
    d.Nx = std::max(2, fnx);
    d.Ny = std::max(2, fny);
    if (d.Nx > ALN_MAX_N || d.Ny > ALN_MAX_N)
        return set_err(ctx, ALN_ERR_UNSUPPORTED, "FFT size %dx%d exceeds %d", d.Nx, d.Ny,
                       ALN_MAX_N);
    d.logNx = ilog2(d.Nx);
    d.logNy = ilog2(d.Ny);
    d.rnx = d.Nx;
    d.rny = d.Ny;
    const int P_ox = d.ox, P_oy = d.oy;
    const long long rad = P.radius < 0 ? -(long long)P.radius : P.radius;
    d.rsqr = rad * rad;
    const int R = (int)std::min<long long>(rad, 1 << 20);
    d.xlo = std::max(-(d.w[0] - 1), P_ox - R);
    d.xhi = std::min(d.w[1] - 1, P_ox + R);
    d.ylo = std::max(-(d.h[0] - 1), P_oy - R);
    d.yhi = std::min(d.h[1] - 1, P_oy + R);
    d.rgn_kind = P.legal.rgn_kind;
    d.rgn_a = P.legal.rgn_a;
    d.rgn_b = P.legal.rgn_b;
    d.rgn_area = P.legal.rgn_area;
    d.table_w = P.legal.table_w;
    d.table_h = P.legal.table_h;
    d.cnt_kind = P.legal.cnt_kind;
    d.cnt_n = P.legal.cnt_n;
    if (d.rgn_kind == ALN_RGN_TABLE &&
        (!P.legal.table || d.table_w < 1 || d.table_h < 1))
        return set_err(ctx, ALN_ERR_ARG, "legality table missing");
    if (d.rgn_kind < 0 || d.rgn_kind > ALN_RGN_TABLE)
        return set_err(ctx, ALN_ERR_ARG, "bad rgn_kind %d", d.rgn_kind);
    if (spec && spec->kind == 3) {
        // CorrPatchToImage: both images are the N x N frame; every storage
        // row/column of the inverse is kept; no summed-area tables
        d.mode = JOB_P2I;
        d.no_shift = 1;
        d.Nx = d.w[0];   // circular correlation on the N x N frame itself
        d.Ny = d.h[0];
        d.logNx = ilog2(d.Nx);
        d.logNy = ilog2(d.Ny);
        pl.orig_nx = d.Nx;
        pl.orig_ny = d.Ny;
        pl.frame_nx1 = pl.frame_ny1 = 0;
        d.p2i_filter = spec->p2i_filter;
        d.p2i_w1 = spec->p2i_w1;
        d.p2i_h1 = spec->p2i_h1;
        d.p2i_w2 = spec->p2i_w2;
        d.p2i_h2 = spec->p2i_h2;
        d.p2i_norm = spec->p2i_norm;
        d.ox = spec->ox;
        d.oy = spec->oy;
        d.rsqr = (long long)spec->rx * spec->rx;   // rx carries the radius
        d.xlo = 0;
        d.xhi = d.Nx - 1;
        d.ylo = 0;
        d.yhi = d.Ny - 1;
        for (int i = 0; i < 2; ++i) {
            d.need_lo[i][0] = d.need_lo[i][1] = 1;
            d.need_hi[i][0] = d.need_hi[i][1] = 0;
        }
    } else if (spec) {
        // CCorImg::SetDims "too small" rule, 0_GEN/Correlation.cpp:1991-2000
        const int mindelta = 11 / 2 + 1;
        if (d.w[0] - 1 < mindelta || d.w[1] < mindelta || d.h[0] - 1 < mindelta ||
            d.h[1] < mindelta) {
            d.status = ALN_NO_PEAK;
            pl.ws_bytes = 0;
            pl.in_bytes[0] = pl.in_bytes[1] = 0;
            return ALN_OK;
        }
        d.mode = spec->kind == 2 ? JOB_IMAGES_S : spec->kind == 4 ? JOB_IMAGES_F : JOB_IMAGES_R;
        d.want_s = spec->kind == 2;
        d.want_r = spec->kind == 1 || spec->kind == 4 || (spec->kind == 2 && spec->mincor > 0.0);
        d.nbmaxht = spec->nbmaxht;
        d.no_shift = d.want_s;
        // S key alone: no value sums, only counts; FP32 keys in the lag scan
        d.sat_nonly = d.mode == JOB_IMAGES_S && !d.want_r;
        d.s_float = d.sat_nonly;
        d.mincor = spec->mincor;
        d.cx = d.w[0] - 1;
        d.cy = d.h[0] - 1;
        d.wR = d.w[0] + d.w[1] - 1;
        d.hR = d.h[0] + d.h[1] - 1;
        if (spec->rx > 0 && spec->ry > 0) {
            d.oval_on = 1;
            d.ocx = spec->ox + d.x0[0] - d.x0[1] + d.cx;
            d.ocy = spec->oy + d.y0[0] - d.y0[1] + d.cy;
            d.orx = spec->rx;
            d.ory = spec->ry;
            d.orx2 = (double)(spec->rx * spec->rx);
            d.oasq = d.orx2 / ((double)spec->ry * spec->ry);
        }
    }
    if (d.xlo > d.xhi || d.ylo > d.yhi) {
        d.status = ALN_NO_PEAK;   // empty search region
        pl.ws_bytes = 0;
        pl.in_bytes[0] = pl.in_bytes[1] = 0;
        return ALN_OK;
    }
    if (d.mode == JOB_PATCHES) {
        // CorrPatches reads the correlation at the disc's lags only, so the
        // transform grid only has to keep those lags free of wrap-around: the
        // circular correlation at lag x holds the linear one at x + m Nx for
        // every m, whose support is [-(w0-1), w1-1]; Nx > max(w1-1-xlo,
        // xhi+w0-1) leaves m = 0 alone for every x in [xlo, xhi].  The grid
        // also holds both images unfolded (Nx >= w0, w1).  The plain product
        // makes the values at those lags the same sums as on the reference's
        // grid (the whitened S product of CorrImagesS is not grid-invariant).
        // The row axis may take a split length (3 * 2^k or 5 * 2^k points,
        // patches_len); columns stay powers of two (segments or one
        // transform).  The sums at the disc's lags are the same on any
        // alias-free grid.
        const int ny = std::max(2, ceil_pow2(std::max(
                                       std::max(d.h[0], d.h[1]),
                                       std::max(d.h[1] - 1 - d.ylo, d.yhi + d.h[0] - 1) + 1)));
        d.Ny = std::min(d.Ny, ny);
        // (columns of >= 8 points: the register pipeline's range)
        const bool split = allow_split && (ctx ? ctx->split_on != 0 : true) && d.Ny >= 8;
        const int nx = patches_len(std::max(std::max(d.w[0], d.w[1]),
                                            std::max(d.w[1] - 1 - d.xlo, d.xhi + d.w[0] - 1) + 1),
                                   split);
        d.Nx = std::min(d.Nx, nx);
        d.logNx = odd_part(d.Nx) == 1 ? ilog2(d.Nx) : 0;   // the split lengths have none
        d.logNy = ilog2(d.Ny);
        // Segmented columns (k2_corrseg) where they take fewer FFT
        // point-passes: 2 nseg + 1 transforms of NS points against 3 of Ny
        // (cost per transform ~ N (log2 N + 4), loads and exchanges
        // included); a segment of NS points serves NS - Wy + 1 rows of a.
        const int pol = ctx ? ctx->seg_ns : 0;
        if (allow_segment && pol >= 0 && d.Nx / 2 >= 8 && d.Nx / 2 <= 4096) {
            const int Wy = d.yhi - d.ylo + 1;
            auto cost = [](int n, int transforms) {
                return (double)transforms * n * (ilog2(n) + 4);
            };
            double best = 0.85 * cost(d.Ny, 3);
            int bns = 0, bseg = 0;
            std::vector<int> valid;   // segment lengths this pair can take
            auto nseg_of = [&](int ns) { return (d.h[0] + (ns - Wy + 1) - 1) / (ns - Wy + 1); };
            for (int ns = 64; ns <= 2048 && ns < d.Ny; ns *= 2) {
                if (pol > 0 && ns != pol)
                    continue;
                const int B = ns - Wy + 1;
                // the lag kernels key a negative lag row y by y + NS (its
                // storage row): that must stay >= 0 for the window's rows
                if (B < 1 || ns <= -d.ylo)
                    continue;
                const int nseg = nseg_of(ns);
                if (nseg > 64)
                    continue;
                valid.push_back(ns);
                const double c = cost(ns, 2 * nseg + 1);
                if (pol > 0 || c < best) {
                    best = c;
                    bns = ns;
                    bseg = nseg;
                }
            }
            // the measured choice of the pair's class (aln_tune.cuh): the
            // candidates are the cost model's pick, then one transform per
            // column, then the other valid lengths
            if (pol == 0 && !valid.empty()) {
                std::vector<int> cand{bns};
                if (bns)
                    cand.push_back(0);
                for (int ns : valid)
                    if (ns != bns)
                        cand.push_back(ns);
                int t = -1;
                if (ctx && ctx->tune_on && !ctx->tuning)
                    t = tuned_segment(ctx, P, d, Wy, cand);
                else if (!ctx)
                    t = recorded_segment(d, Wy);
                if (t == -2) {   // class not measured yet; planned again after
                    pl.tune_deferred = 1;
                    t = -1;
                }
                if (t == 0) {
                    bns = 0;
                } else if (t > 0 && std::find(valid.begin(), valid.end(), t) != valid.end()) {
                    bns = t;
                    bseg = nseg_of(t);
                }
            }
            if (bns) {
                d.Ny = bns;
                d.logNy = ilog2(bns);
                d.nseg = bseg;
                d.seg_len = (d.h[0] + bseg - 1) / bseg;
            }
        }
    }
    if (d.mode != JOB_P2I && !(d.sat_nonly && d.cnt_kind != ALN_CNT_GT))
        for (int i = 0; i < 2; ++i)
            need_rows(d, i, d.need_lo[i], d.need_hi[i]);
    else if (d.mode != JOB_P2I)
        for (int i = 0; i < 2; ++i) {   // no table is read
            d.need_lo[i][0] = d.need_lo[i][1] = 1;
            d.need_hi[i][0] = d.need_hi[i][1] = 0;
        }
    const int L1 = d.Nx / 2 + 1;
    const int Wy = d.yhi - d.ylo + 1, Wx = d.xhi - d.xlo + 1;
    size_t b = 0;
    for (int i = 0; i < 2; ++i) {
        pl.in_bytes[i] = im[i]->on_device ? 0 : al256((size_t)d.w[i] * d.h[i] * dtype_size(d.dt[i]));
        b += pl.in_bytes[i];
        pl.tr_bytes[i] = pl.transposed
                             ? al256((size_t)((d.w[i] + 15) & ~15) * d.h[i] * dtype_size(d.dt[i]))
                             : 0;
        b += pl.tr_bytes[i];
        d.Ts[i] = (d.h[i] + 3) & ~3;
        b += al256((size_t)L1 * d.Ts[i] * sizeof(float2));
        int ns = 0;
        for (int k = 0; k < 2; ++k)
            if (d.need_hi[i][k] >= d.need_lo[i][k])
                ns += d.need_hi[i][k] - d.need_lo[i][k] + 1;
        b += 2 * al256((size_t)ns * d.w[i] * sizeof(double)) + al256((size_t)ns * d.w[i] * sizeof(int));
        b += al256((size_t)d.w[i] * sizeof(double));
        b += 2 * al256((size_t)SAT_WARPS * d.w[i] * sizeof(double)) +
             al256((size_t)SAT_WARPS * d.w[i] * sizeof(int));
    }
    b += al256((size_t)L1 * d.Ny * sizeof(float2));
    b += al256((size_t)L1 * Wy * sizeof(float2));
    b += al256((size_t)Wx * Wy * sizeof(double));
    b += al256((size_t)Wy * sizeof(RowBest));
    if (d.rgn_kind == ALN_RGN_TABLE)
        b += al256((size_t)d.table_w * d.table_h);
    if (d.want_r && d.want_s)
        b += al256((size_t)L1 * Wy * sizeof(float2));
    if (d.mode == JOB_IMAGES_S && d.want_r)
        b += al256((size_t)Wx * Wy * sizeof(double));
    if (d.mode == JOB_IMAGES_F)
        b += al256((size_t)Wx * Wy * sizeof(double)) + al256((size_t)Wx * Wy);
    pl.ws_bytes = b;
    return ALN_OK;
}

extern "C" int aln_corr_patches_grid(const aln_pair *P, int *nx, int *ny, int *nseg,
                                     int *transposed)
{
    if (!P || !nx || !ny || !nseg || !transposed)
        return ALN_ERR_ARG;
    PairPlan pl;
    if (int rc = plan_pair(nullptr, *P, pl, true, nullptr, P->b_key == 0, true))
        return rc;
    const bool empty = pl.d.status == ALN_NO_PEAK;
    *nx = empty ? 0 : pl.d.Nx;
    *ny = empty ? 0 : pl.d.Ny;
    *nseg = empty ? 0 : pl.d.nseg;
    *transposed = pl.transposed ? 1 : 0;
    return empty ? ALN_NO_PEAK : ALN_OK;
}

// carve a pair's workspace starting at base; returns bytes used.  Host
// inputs already staged by their window keep that staging.
static size_t carve(PairPlan &pl, char *base, const aln_pair &P)
{
    PairDev &d = pl.d;
    char *p = base;
    const int L1 = d.Nx / 2 + 1;
    const int Wy = d.yhi - d.ylo + 1, Wx = d.xhi - d.xlo + 1;
    for (int i = 0; i < 2; ++i) {
        if (pl.in_bytes[i]) {
            // staging of a host input, in the caller's layout: the window's
            // staging buffer when set, else the pair's own workspace
            char *q = pl.staged[i];
            if (!q) {
                q = p;
                p += pl.in_bytes[i];
            }
            if (pl.transposed) {
                d.src_img[i] = q;
                d.src_stride[i] = d.h[i];   // caller's width
            } else {
                d.img[i] = q;
                d.stride[i] = d.w[i];
            }
        }
        if (pl.tr_bytes[i]) {
            d.img[i] = p;
            d.stride[i] = (d.w[i] + 15) & ~15;
            p += pl.tr_bytes[i];
        }
        d.T[i] = (float2 *)p;
        p += al256((size_t)L1 * d.Ts[i] * sizeof(float2));
        int ns = 0;
        for (int k = 0; k < 2; ++k)
            if (d.need_hi[i][k] >= d.need_lo[i][k])
                ns += d.need_hi[i][k] - d.need_lo[i][k] + 1;
        d.satS[i] = (double *)p;
        p += al256((size_t)ns * d.w[i] * sizeof(double));
        d.satQ[i] = (double *)p;
        p += al256((size_t)ns * d.w[i] * sizeof(double));
        d.satN[i] = (int *)p;
        p += al256((size_t)ns * d.w[i] * sizeof(int));
        d.colsum[i] = (double *)p;
        p += al256((size_t)d.w[i] * sizeof(double));
        d.segS[i] = (double *)p;
        p += al256((size_t)SAT_WARPS * d.w[i] * sizeof(double));
        d.segQ[i] = (double *)p;
        p += al256((size_t)SAT_WARPS * d.w[i] * sizeof(double));
        d.segN[i] = (int *)p;
        p += al256((size_t)SAT_WARPS * d.w[i] * sizeof(int));
    }
    d.X2 = (float2 *)p;
    p += al256((size_t)L1 * d.Ny * sizeof(float2));
    d.Q = (float2 *)p;
    p += al256((size_t)L1 * Wy * sizeof(float2));
    d.rr = (double *)p;
    p += al256((size_t)Wx * Wy * sizeof(double));
    d.rb = (RowBest *)p;
    p += al256((size_t)Wy * sizeof(RowBest));
    if (d.rgn_kind == ALN_RGN_TABLE) {
        d.table = (const unsigned char *)p;
        p += al256((size_t)d.table_w * d.table_h);
    }
    if (d.want_r && d.want_s) {
        d.Q2 = (float2 *)p;
        p += al256((size_t)L1 * Wy * sizeof(float2));
    }
    if (d.mode == JOB_IMAGES_S && d.want_r) {
        d.rr2 = (double *)p;
        p += al256((size_t)Wx * Wy * sizeof(double));
    }
    if (d.mode == JOB_IMAGES_F) {
        d.fimg = (double *)p;
        p += al256((size_t)Wx * Wy * sizeof(double));
        d.fst = (unsigned char *)p;
        p += al256((size_t)Wx * Wy);
    }
    (void)P;
    return (size_t)(p - base);
}

static int rows_per_cta(int L) { return std::max(1, std::min(16, 4096 / L)); }
static int cols_per_cta(int Ny) { return std::max(1, std::min(16, 4096 / Ny)); }

template <int LL>
static void launch_rowfft2(aln_ctx *ctx, int n, int maxh)
{
    constexpr int T = rowfft_T<LL>();
    const int thr = rowfft_threads(T), G = thr / T;
    const size_t sm = ((size_t)G * rowfft_pitch<LL>() + 16) * sizeof(float2);
    smem_attr(ctx->device, (const void *)k2_rowfft<LL>, sm);
    LAUNCH(ctx, "k2_rowfft", k2_rowfft<LL>, dim3((maxh + G - 1) / G, 2, n), thr, sm,
           ctx->dpairs, ctx->tw, -1, (const int *)nullptr);
}

// spectrum-cache fills: b's rows and columns of the selected jobs -> X2
template <int LL>
static void launch_fill_rows(aln_ctx *ctx, int nsel, int maxh)
{
    constexpr int T = rowfft_T<LL>();
    const int thr = rowfft_threads(T), G = thr / T;
    const size_t sm = ((size_t)G * rowfft_pitch<LL>() + 16) * sizeof(float2);
    smem_attr(ctx->device, (const void *)k2_rowfft<LL>, sm);
    LAUNCH(ctx, "k2_rowfft", k2_rowfft<LL>, dim3((maxh + G - 1) / G, 1, nsel), thr, sm,
           ctx->dpairs, ctx->tw, 1, (const int *)ctx->dsel_cur);
}

template <int NY, int RAD>
static void launch_fill_cols_rad(aln_ctx *ctx, int nsel, int L)
{
    constexpr int T = NY / RAD;
    const int thr = std::max(256, T), G = thr / T;
    const size_t sm = (size_t)G * RegFFT<NY, -1, RAD>::SMEM * sizeof(float2);   // k2_colspec's FF
    smem_attr(ctx->device, (const void *)k2_colspec<NY, RAD>, sm);
    LAUNCH(ctx, "k2_colspec", (k2_colspec<NY, RAD>), dim3((L + 1 + G - 1) / G, nsel), thr, sm,
           ctx->dpairs, ctx->tw, (const int *)ctx->dsel_cur);
}

// the cache entry is computed with the radix of the column kernel that reads it
template <int NY>
static void launch_fill_cols(aln_ctx *ctx, int nsel, int L, int var)
{
    if (var == 1)
        launch_fill_cols_rad<NY, corrcol_radix<NY, 1>()>(ctx, nsel, L);
    else
        launch_fill_cols_rad<NY, corrcol_radix<NY, 0>()>(ctx, nsel, L);
}

#define ALN_CASES_SEG(X) X(64) X(128) X(256) X(512) X(1024) X(2048)

static int corrcol_radix_of(int Ny, int var)
{
    (void)var;   // every form uses fft_radix (corrcol_radix)
    return fft_radix(Ny);
}

template <int NY, int VAR>
static void launch_corrcol_var(aln_ctx *ctx, int n, int L, int cached)
{
    constexpr int T = NY / corrcol_radix<NY, VAR>();
    constexpr int thr = corrcol_threads<NY, VAR>(), G = thr / T;
    // per team: k2_corrcol's exchange buffer (FF::SMEM) and b's spectrum (NY)
    const size_t sm =
        (size_t)G * (RegFFT<NY, -1, corrcol_radix<NY, VAR>()>::SMEM + NY) * sizeof(float2);
    void (*kern)(PairDev *, const float2 *, int) = k2_corrcol<NY, VAR>;
    smem_attr(ctx->device, (const void *)kern, sm);
    LAUNCH(ctx, "k2_corrcol", kern, dim3((L + 1 + G - 1) / G, n), thr, sm, ctx->dpairs, ctx->tw,
           cached);
}

template <int NY>
static void launch_corrcol2(aln_ctx *ctx, int n, int L, int cached, int var)
{
    if (var == 1)
        launch_corrcol_var<NY, 1>(ctx, n, L, cached);
    else if (var == 2)
        launch_corrcol_var<NY, 2>(ctx, n, L, cached);
    else
        launch_corrcol_var<NY, 0>(ctx, n, L, cached);
}

// A team runs its column's segments one after another, so a call with few
// columns (a single pair, say) gets fewer teams per CTA to spread them over
// more SMs: the largest G (teams per CTA) that still gives 2 CTAs per SM,
// down to 1.  Each column's arithmetic is the same whatever G is.
template <int NS>
static void launch_corrseg(aln_ctx *ctx, int n, int L)
{
    constexpr int T = NS / corrseg_radix<NS>(), GMAX = 256 / T;
    if (!ctx->sms) {
        cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device);
        ctx->sms = std::max(ctx->sms, 1);
    }
    int G = GMAX;
    while (G > 1 && (long long)((L + 1 + G - 1) / G) * n < 2LL * ctx->sms)
        G /= 2;
    // float2 per team: k2_corrseg's exchange buffer (FF::SMEM), then the parked
    // spectrum and accumulator when they are not held in registers
    constexpr int per_team =
        RegFFT<NS, -1, corrseg_radix<NS>()>::SMEM + (corrseg_regs<NS>() ? 0 : 2 * NS);
    const size_t sm = (size_t)G * per_team * sizeof(float2);
    smem_attr(ctx->device, (const void *)k2_corrseg<NS>, (size_t)GMAX * per_team * sizeof(float2));
    LAUNCH(ctx, "k2_corrseg", k2_corrseg<NS>, dim3((L + 1 + G - 1) / G, n), G * T, sm,
           ctx->dpairs, ctx->tw);
}

template <int LL>
static void launch_lagrow2(aln_ctx *ctx, int n, int maxWy)
{
    constexpr int T = FFTOf<LL, +1>::T;
    constexpr int thr = lagrow_threads(T), G = thr / T;
    const size_t sm = (size_t)G * lag_pitch<LL>() * sizeof(float2);
    smem_attr(ctx->device, (const void *)k2_lagrow<LL>, sm);
    LAUNCH(ctx, "k2_lagrow", k2_lagrow<LL>, dim3((maxWy + G - 1) / G, n), thr, sm,
           ctx->dpairs, ctx->tw);
}

template <int LL>
static void launch_lagp2i(aln_ctx *ctx, int n, int maxWy)
{
    constexpr int T = RegFFT<LL, +1>::T;
    const int thr = std::max(256, T), G = thr / T;
    const size_t sm = (size_t)G * lag_pitch<LL>() * sizeof(float2);
    smem_attr(ctx->device, (const void *)k2_lagp2i<LL>, sm);
    LAUNCH(ctx, "k2_lagp2i", k2_lagp2i<LL>, dim3((maxWy + G - 1) / G, n), thr, sm, ctx->dpairs,
           ctx->tw);
}

template <int LL>
static void launch_lagimg2(aln_ctx *ctx, int n, int maxWy, bool both, bool sonly)
{
    constexpr int T = RegFFT<LL, +1>::T;
    const int thr = std::max(256, T), G = thr / T;
    const size_t sm = (size_t)G * lag_pitch<LL>() * (both ? 2 : 1) * sizeof(float2);
    void (*kern)(PairDev *, const float2 *) = sonly ? k2_lagimg<LL, true> : k2_lagimg<LL, false>;
    smem_attr(ctx->device, (const void *)kern, sm);
    LAUNCH(ctx, "k2_lagimg", kern, dim3((maxWy + G - 1) / G, n), thr, sm, ctx->dpairs, ctx->tw);
}

#define ALN_CASES_L(X) X(8) X(16) X(32) X(64) X(128) X(256) X(512) X(1024) X(2048) X(4096)
#define ALN_CASES_NY(X) ALN_CASES_L(X) X(8192)

// register-FFT pipeline for one chunk: rows (both images), fused columns,
// lag rows.  L = Nx/2 in [16, 4096], Ny in [16, 8192].
static int launch_fft_pipeline(aln_ctx *ctx, int L, int Ny, int n, int maxh, int maxWy,
                               int mode = JOB_PATCHES, bool both = false, bool sonly = false,
                               bool seg = false)
{
    switch (L) {
#define X(v) case v: launch_rowfft2<v>(ctx, n, maxh); break;
        ALN_CASES_L(X)
        ALN_CASES_LMIX(X)
#undef X
    default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "row length %d", L);
    }
    if (seg) {
        switch (Ny) {
#define X(v) case v: launch_corrseg<v>(ctx, n, L); break;
            ALN_CASES_SEG(X)
#undef X
        default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "segment length %d", Ny);
        }
    } else switch (Ny) {
#define X(v) case v: launch_corrcol2<v>(ctx, n, L, 0, mode == JOB_PATCHES ? 1 : sonly ? 2 : 0); break;
        ALN_CASES_NY(X)
#undef X
    default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "column length %d", Ny);
    }
    if (mode == JOB_PATCHES) {
        switch (L) {
#define X(v) case v: launch_lagrow2<v>(ctx, n, maxWy); break;
            ALN_CASES_L(X)
            ALN_CASES_LMIX(X)
#undef X
        default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "row length %d", L);
        }
    } else if (mode == JOB_P2I) {
        switch (L) {
#define X(v) case v: launch_lagp2i<v>(ctx, n, maxWy); break;
            ALN_CASES_L(X)
#undef X
        default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "row length %d", L);
        }
    } else {
        switch (L) {
#define X(v) case v: launch_lagimg2<v>(ctx, n, maxWy, both, sonly); break;
            ALN_CASES_L(X)
#undef X
        default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "row length %d", L);
        }
    }
    return ALN_OK;
}

// One chunk of jobs sharing (Nx, Ny, kind): the sizes its launches need and
// where its jobs sit in the batch's job table.
struct ChunkLaunch {
    int off, n;                        // jobs [off, off + n) of the batch table
    int maxw, maxh, maxslots, maxWy;
    int sw, sh;                        // largest caller-frame image of transposed jobs
    int t8;                            // every transposed job is uint8 (128-byte tiles)
    int Nx, Ny, mode, both, sonly, frame_nx1, frame_ny1;
    int seg;                           // CorrPatches with segmented columns
    int fill_off, nfill, fill_maxh;    // spectrum-cache fills: sel[fill_off ...]
};

// Host side of a chunk: carve each job's workspace (the chunk's work buffer
// is reused by every chunk, in stream order), resolve spectrum-cache keys,
// write the job table entries hd[0..n).
static void prep_chunk(aln_ctx *ctx, std::vector<PairPlan *> &chunk, int off, char *work_base,
                       PairDev *hd, std::vector<int> &fills, ChunkLaunch &cl)
{
    const int n = (int)chunk.size();
    cl.off = off;
    cl.n = n;
    cl.maxw = cl.maxh = cl.maxslots = cl.maxWy = 1;
    cl.sw = cl.sh = 0;
    cl.t8 = 1;
    cl.Nx = chunk[0]->d.Nx;
    cl.Ny = chunk[0]->d.Ny;
    cl.fill_off = (int)fills.size();
    cl.fill_maxh = 1;
    char *work = work_base;
    const bool reg_path = cl.Nx / 2 >= 8 && cl.Nx / 2 <= 4096 && cl.Ny >= 8 && cl.Ny <= 8192;
    ++ctx->spec_tick;
    for (int k = 0; k < n; ++k) {
        PairPlan &pl = *chunk[k];
        work += carve(pl, work, *pl.src);
        pl.d.b_cached = 0;
        if (pl.key && reg_path && pl.d.mode != JOB_P2I && ctx->spec_cap > 0) {
            const SpecKey K(pl.key_ns, pl.key, pl.d.Nx, pl.d.Ny, pl.d.transposed,
                            pl.d.no_shift,
                            corrcol_radix_of(pl.d.Ny, pl.d.mode == JOB_PATCHES ? 1 : 0));
            auto it = ctx->spec.find(K);
            if (it != ctx->spec.end()) {
                spec_touch(ctx, it);
                pl.d.b_cached = 1;
                pl.d.X2 = it->second.X2;
                ctx->spec_hits++;
            } else {
                const size_t bytes = al256((size_t)(pl.d.Nx / 2 + 1) * pl.d.Ny * sizeof(float2));
                if (float2 *buf = spec_alloc(ctx, bytes)) {
                    spec_insert(ctx, K, SpecEntry{buf, bytes, ctx->spec_tick});
                    pl.d.b_cached = 1;
                    pl.d.X2 = buf;
                    fills.push_back(k);
                    cl.fill_maxh = std::max(cl.fill_maxh, pl.d.h[1]);
                    ctx->spec_fills++;
                }
            }
        }
        for (int i = 0; i < 2; ++i) {
            cl.maxw = std::max(cl.maxw, pl.d.w[i]);
            cl.maxh = std::max(cl.maxh, pl.d.h[i]);
            int ns = 0;
            for (int q = 0; q < 2; ++q)
                if (pl.d.need_hi[i][q] >= pl.d.need_lo[i][q])
                    ns += pl.d.need_hi[i][q] - pl.d.need_lo[i][q] + 1;
            cl.maxslots = std::max(cl.maxslots, ns);
            if (pl.d.transposed) {
                cl.sw = std::max(cl.sw, pl.d.h[i]);
                cl.sh = std::max(cl.sh, pl.d.w[i]);
                cl.t8 &= pl.d.dt[i] == ALN_U8;
            }
        }
        cl.maxWy = std::max(cl.maxWy, pl.d.yhi - pl.d.ylo + 1);
        pl.d.sat_int = (pl.d.dt[0] == ALN_U8 || pl.d.dt[0] == ALN_U16 ? 1 : 0) |
                       (pl.d.dt[1] == ALN_U8 || pl.d.dt[1] == ALN_U16 ? 2 : 0);
        hd[k] = pl.d;
    }
    cl.nfill = (int)fills.size() - cl.fill_off;
    cl.mode = hd[0].mode;
    cl.both = hd[0].want_r && hd[0].want_s;
    cl.sonly = hd[0].s_float != 0;
    cl.frame_nx1 = chunk[0]->frame_nx1;
    cl.frame_ny1 = chunk[0]->frame_ny1;
    cl.seg = hd[0].nseg > 0;
}

// The chunk's kernels on the compute stream (its job table, fill list and
// staged inputs are already on the device, in stream order).
static int launch_chunk(aln_ctx *ctx, std::vector<PairPlan *> &chunk, const ChunkLaunch &cl)
{
    const int n = cl.n, Nx = cl.Nx, Ny = cl.Ny, L = Nx / 2;
    ctx->chunks++;
    ctx->dpairs = ctx->dpairs_base + cl.off;
    ctx->dres = ctx->dres_base + cl.off;
    ctx->dsel_cur = ctx->dsel + cl.fill_off;
    cudaStream_t st = ctx->stream;
    for (int k = 0; k < n; ++k)   // tabulated legality (pageable source: staged at the call)
        if (chunk[k]->d.rgn_kind == ALN_RGN_TABLE)
            CK(cudaMemcpyAsync((void *)chunk[k]->d.table, chunk[k]->src->legal.table,
                               (size_t)chunk[k]->d.table_w * chunk[k]->d.table_h,
                               cudaMemcpyHostToDevice, st));
    if (cl.sw > 0)
        LAUNCH(ctx, "k_transpose", k_transpose,
               dim3(cl.t8 ? (cl.sw + 128 * TR_TILES - 1) / (128 * TR_TILES)
                          : (cl.sw + 32 * TR_TILES - 1) / (32 * TR_TILES),
                    (cl.sh + 31) / 32, 2 * n),
               dim3(32, 8), 0, ctx->dpairs);
    const int mode = cl.mode;
    if (mode != JOB_P2I) {
        LAUNCH(ctx, "k3_sat", k3_sat, dim3((cl.maxw + 31) / 32, 2 * n), dim3(32, SAT_WARPS), 0,
               ctx->dpairs);
        LAUNCH(ctx, "k_mean", k_mean, dim3(2, n), 256, 0, ctx->dpairs);
        if (cl.sonly)
            LAUNCH(ctx, "k2_sat2w", k2_sat2w<true>, dim3((cl.maxslots + 7) / 8, 2, n), 256, 0,
                   ctx->dpairs);
        else
            LAUNCH(ctx, "k2_sat2w", k2_sat2w<false>, dim3((cl.maxslots + 7) / 8, 2, n), 256,
                   0, ctx->dpairs);
    }
    if (cl.nfill > 0) {
        switch (L) {
#define X(v) case v: launch_fill_rows<v>(ctx, cl.nfill, cl.fill_maxh); break;
            ALN_CASES_L(X)
            ALN_CASES_LMIX(X)
#undef X
        default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "row length %d", L);
        }
        switch (Ny) {
#define X(v) case v: launch_fill_cols<v>(ctx, cl.nfill, L, mode == JOB_PATCHES ? 1 : 0); break;
            ALN_CASES_NY(X)
#undef X
        default: return set_err(ctx, ALN_ERR_UNSUPPORTED, "column length %d", Ny);
        }
    }
    if (L >= 8 && L <= 4096 && Ny >= 8 && Ny <= 8192) {
        if (int rc = launch_fft_pipeline(ctx, L, Ny, n, cl.maxh, cl.maxWy, mode, cl.both != 0,
                                         cl.sonly != 0, cl.seg != 0))
            return rc;
    } else if (mode != JOB_PATCHES) {
        return set_err(ctx, ALN_ERR_UNSUPPORTED, "CorrImages FFT size %d x %d", Nx, Ny);
    } else {
        {
            const int RB = rows_per_cta(L);
            const size_t sm = 2 * (size_t)RB * (L + 1) * sizeof(float2);
            LAUNCH(ctx, "k_rowfft", k_rowfft, dim3((cl.maxh + RB - 1) / RB, 2, n), 256, sm,
                   ctx->dpairs, ctx->tw, RB, -1);
        }
        {
            const int CG = cols_per_cta(Ny);
            const size_t sm = 2 * (size_t)CG * (Ny + 1) * sizeof(float2);
            const int gx = (L + 1 + CG - 1) / CG;
            LAUNCH(ctx, "k_colfft", k_colfft, dim3(gx, n), 256, sm, ctx->dpairs, ctx->tw, CG);
            LAUNCH(ctx, "k_corrcol", k_corrcol, dim3(gx, n), 256, sm, ctx->dpairs, ctx->tw, CG);
        }
        {
            const int RBL = std::max(1, std::min(8, 4096 / std::max(1, L)));
            const size_t sm = 2 * (size_t)RBL * (L + 1) * sizeof(float2);
            LAUNCH(ctx, "k_lagrow", k_lagrow, dim3((cl.maxWy + RBL - 1) / RBL, n), 256, sm,
                   ctx->dpairs, ctx->tw, RBL);
        }
    }
    if (mode == JOB_PATCHES)
        LAUNCH(ctx, "k_final", k_final, n, 256, 0, ctx->dpairs, ctx->dres, cl.frame_nx1,
               cl.frame_ny1);
    else if (mode == JOB_P2I)
        LAUNCH(ctx, "k_final_p2i", k_final_p2i, n, 256, 0, ctx->dpairs, ctx->dres);
    else if (mode == JOB_IMAGES_F) {
        int mw = 1, mh = 1;
        for (auto *pl : chunk) {
            mw = std::max(mw, pl->d.wR);
            mh = std::max(mh, pl->d.hR);
        }
        LAUNCH(ctx, "k_makef", k_makef, dim3((mw + 31) / 32, (mh + 7) / 8, n), dim3(32, 8), 0,
               ctx->dpairs);
        LAUNCH(ctx, "k_fpeak", k_fpeak, n, FPK_THREADS, 0, ctx->dpairs, ctx->dres);
    } else
        LAUNCH(ctx, "k_final_img", k_final_img, n, 256, 0, ctx->dpairs, ctx->dres);
    CK(cudaGetLastError());
    return ALN_OK;
}

static void fill_result(const PairPlan &pl, aln_result *o)
{
    o->status = pl.d.status == ALN_OK ? ALN_OK : ALN_NO_PEAK;
    o->r = o->status == ALN_OK ? pl.d.r : 0.0;
    o->dx = o->status == ALN_OK ? pl.d.dx : 0.0;
    o->dy = o->status == ALN_OK ? pl.d.dy : 0.0;
    o->peak_x = pl.d.px;
    o->peak_y = pl.d.py;
    o->nx = pl.orig_nx;
    o->ny = pl.orig_ny;
}

static int ensure_hres(aln_ctx *ctx, size_t n)
{
    if (n <= ctx->hres_cap)
        return ALN_OK;
    if (ctx->hres)
        cudaFreeHost(ctx->hres);
    ctx->hres = nullptr;
    ctx->hres_cap = 0;
    const size_t cap = std::max<size_t>(n, 4096);
    CK(cudaHostAlloc((void **)&ctx->hres, cap * sizeof(ResultDev), cudaHostAllocDefault));
    ctx->hres_cap = cap;
    return ALN_OK;
}

// Copies a window's host inputs into staging buffer `base` on the copy
// stream (after the kernels that last read this buffer), packed in window
// order, adjacent host images with one transfer; records ev_copy[wp].
// Staging addresses of a window's host inputs: packed in window order
// (aligned to the element size only), so adjacent host images stay adjacent.
static void assign_staging(std::vector<PairPlan *> &win, char *base)
{
    char *cur = base;
    for (PairPlan *pl : win) {
        const aln_image *im[2] = {&pl->src->a, &pl->src->b};
        for (int i = 0; i < 2; ++i) {
            pl->staged[i] = nullptr;
            if (!pl->in_bytes[i])
                continue;
            const size_t es = dtype_size(im[i]->dtype);
            cur = (char *)(((uintptr_t)cur + es - 1) & ~(uintptr_t)(es - 1));
            pl->staged[i] = cur;
            cur += (size_t)im[i]->w * im[i]->h * es;
        }
    }
}

// Host-to-device staging by the SMs: page-locked host memory is mapped into
// the device's address space, so a grid of 16-byte loads and stores moves
// it.  On GB300 this ran at the host link's 208 GB/s where copy-engine
// transfers of the same page-locked buffers inside this library's batches
// ran at 70 GB/s; its few small blocks run beside the compute kernels.
// Both addresses need not be aligned alike: then bytes, else a byte head,
// 16-byte body and byte tail.
#define H2D_UNROLL 4
__global__ void __launch_bounds__(256) k_h2d_stage(char *__restrict__ dst,
                                                   const char *__restrict__ src, size_t n)
{
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if ((((uintptr_t)dst ^ (uintptr_t)src) & 15) != 0) {
        for (size_t i = t0; i < n; i += stride)
            dst[i] = src[i];
        return;
    }
    const size_t mis = (16 - ((uintptr_t)src & 15)) & 15;
    const size_t head = mis < n ? mis : n;
    for (size_t i = t0; i < head; i += stride)
        dst[i] = src[i];
    const size_t nv = (n - head) / 16;
    const uint4 *__restrict__ s4 = (const uint4 *)(src + head);
    uint4 *__restrict__ d4 = (uint4 *)(dst + head);
    // H2D_UNROLL loads in flight per thread before their stores: few blocks
    // keep the host link busy, leaving the SMs' issue slots to the kernels
    // that run beside the staging
    size_t i = t0;
    for (; i + (H2D_UNROLL - 1) * stride < nv; i += H2D_UNROLL * stride) {
        uint4 v[H2D_UNROLL];
#pragma unroll
        for (int u = 0; u < H2D_UNROLL; ++u)
            v[u] = s4[i + u * stride];
#pragma unroll
        for (int u = 0; u < H2D_UNROLL; ++u)
            d4[i + u * stride] = v[u];
    }
    for (; i < nv; i += stride)
        d4[i] = s4[i];
    for (size_t j = head + nv * 16 + t0; j < n; j += stride)
        dst[j] = src[j];
}

static int stage_window(aln_ctx *ctx, std::vector<PairPlan *> &win, int wp)
{
    CK(cudaStreamWaitEvent(ctx->cstream, ctx->ev_wdone[wp], 0));
    prof_begin_copy(ctx, "h2d_staging");
    const char *run_src = nullptr, *run_end = nullptr;
    char *run_dst = nullptr;
    auto flush = [&]() -> int {
        if (!run_src || run_end <= run_src) {
            run_src = run_end = nullptr;
            return ALN_OK;
        }
        const size_t b = (size_t)(run_end - run_src);
        // page-locked runs by the SMs (k_h2d_stage), pageable ones by the
        // copy engine (it stages them through its own pinned buffers)
        // (the run's first and last bytes both page-locked and mapped at the
        // same offset: one allocation, or contiguous ones mapped alike)
        cudaPointerAttributes at, at2;
        const bool locked = cudaPointerGetAttributes(&at, run_src) == cudaSuccess &&
                            at.type == cudaMemoryTypeHost && at.devicePointer &&
                            cudaPointerGetAttributes(&at2, run_end - 1) == cudaSuccess &&
                            at2.type == cudaMemoryTypeHost &&
                            (const char *)at2.devicePointer - (const char *)at.devicePointer ==
                                (ptrdiff_t)(b - 1);
        cudaGetLastError();
        if (locked) {
            if (!ctx->sms) {
                cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, ctx->device);
                ctx->sms = std::max(ctx->sms, 1);
            }
            // the run through its device alias (the same address under UVA)
            k_h2d_stage<<<std::max(1, ctx->sms / 4), 256, 0, ctx->cstream>>>(
                run_dst, (const char *)at.devicePointer, b);
            CK(cudaGetLastError());
            ctx->launches++;
        } else {
            CK(cudaMemcpyAsync(run_dst, run_src, b, cudaMemcpyHostToDevice, ctx->cstream));
        }
        ctx->h2d_bytes += (long long)b;
        ctx->h2d_copies++;
        run_src = run_end = nullptr;
        run_dst = nullptr;
        return ALN_OK;
    };
    for (PairPlan *pl : win) {
        const aln_image *im[2] = {&pl->src->a, &pl->src->b};
        for (int i = 0; i < 2; ++i) {
            if (!pl->in_bytes[i])
                continue;
            const size_t es = dtype_size(im[i]->dtype);
            char *dst = pl->staged[i];
            const size_t bytes = (size_t)im[i]->w * im[i]->h * es;
            const char *src = (const char *)im[i]->data;
            if (im[i]->stride == im[i]->w) {
                if (run_src && src == run_end && dst == run_dst + (run_end - run_src)) {
                    run_end += bytes;
                } else {
                    if (int rc = flush())
                        return rc;
                    run_src = src;
                    run_end = src + bytes;
                    run_dst = dst;
                }
            } else {
                if (int rc = flush())
                    return rc;
                CK(cudaMemcpy2DAsync(dst, (size_t)im[i]->w * es, im[i]->data,
                                     (size_t)im[i]->stride * es, (size_t)im[i]->w * es, im[i]->h,
                                     cudaMemcpyHostToDevice, ctx->cstream));
                ctx->h2d_bytes += (long long)bytes;
            }
        }
    }
    if (int rc = flush())
        return rc;
    prof_end_copy(ctx);
    CK(cudaEventRecord(ctx->ev_copy[wp], ctx->cstream));
    return ALN_OK;
}

// Runs CorrPatches (specs == NULL) or CorrImages jobs in chunks of equal FFT
// size and job kind through the two-stage pipeline.
// spectrum key of a job's image b: namespace (0 caller, 1 library) and key
struct JobKey {
    int ns;
    unsigned long long key;
};

// Host threads for planning a batch of n pairs: one per 256 pairs, at most
// 16 and the machine's hardware threads; 1 below 512 pairs.
static int plan_threads(int n)
{
    if (n < 512)
        return 1;
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    return std::max(1, std::min({16, hw, n / 256}));
}

static int batch_impl(aln_ctx *ctx, int npairs, const aln_pair *pairs, const ImgSpec *specs,
                      aln_result *out, const JobKey *keys = nullptr)
{
    if (!ctx || npairs < 0 || (npairs && (!pairs || !out)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "bad arguments") : ALN_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    const auto t_plan0 = std::chrono::steady_clock::now();
    std::vector<PairPlan> plans(npairs);
    auto plan_one = [&](int k) {
        plans[k].src = &pairs[k];
        plans[k].index = k;
        plans[k].key_ns = keys ? keys[k].ns : 0;
        plans[k].key = keys ? keys[k].key : pairs[k].b_key;
        plans[k].tune_deferred = 0;
        const ImgSpec *sp = (specs && specs[k].kind != 0) ? &specs[k] : nullptr;
        return plan_pair(ctx, pairs[k], plans[k], sp == nullptr, sp,
                         sp == nullptr && plans[k].key == 0, sp == nullptr);
    };
    // Plans are independent per pair, and a large batch's planning (a few
    // microseconds per pair, while the device waits) runs on host threads.
    // A pair of an autotuner class not measured yet is planned again on this
    // thread afterwards: measuring runs timing batches on this context.
    const int nthr = plan_threads(npairs);
    if (nthr > 1) {
        ctx->tune_defer = 1;
        std::atomic<int> next(0), first_err(0);
        auto work = [&]() {
            for (;;) {
                const int k0 = next.fetch_add(64);
                if (k0 >= npairs || first_err.load(std::memory_order_relaxed))
                    return;
                for (int k = k0; k < std::min(npairs, k0 + 64); ++k)
                    if (int rc = plan_one(k)) {
                        int z = 0;
                        first_err.compare_exchange_strong(z, rc);
                        return;
                    }
            }
        };
        std::vector<std::thread> pool;
        for (int q = 1; q < nthr; ++q)
            pool.emplace_back(work);
        work();
        for (auto &th : pool)
            th.join();
        ctx->tune_defer = 0;
        if (int rc = first_err.load())
            return rc;
        for (int k = 0; k < npairs; ++k)
            if (plans[k].tune_deferred)
                if (int rc = plan_one(k))
                    return rc;
    } else {
        for (int k = 0; k < npairs; ++k)
            if (int rc = plan_one(k))
                return rc;
    }
    if (!ctx->tuning)
        ctx->host_plan_us += std::chrono::duration_cast<std::chrono::microseconds>(
                                 std::chrono::steady_clock::now() - t_plan0)
                                 .count();
    // Windows: runs of consecutive jobs (submission order) whose host inputs
    // fit one staging buffer.  A window's host images are copied on the copy
    // stream -- adjacent host images with one transfer, by the SMs when they
    // are page-locked -- while the previous window computes.  Inside a
    // window, jobs are grouped by FFT size and job kind (submission order
    // kept) and split into chunks bounded by the workspace budget.
    // Device-resident inputs need no staging: then the whole batch is one
    // window.  Host batches of at least 512 MB are cut into about four
    // windows (at least 128 MB each), so only the first window's copy is not
    // hidden behind computation: at the host link's ~210 GB/s a window's
    // copy takes half the time of its kernels for the montage strips.  (Eight
    // and sixteen windows measured slower end to end on the montage batch:
    // 96.9k and 85.9k pairs/s against 98.8k with four.)
    size_t host_bytes = 0;
    for (const auto &pl : plans)
        if (pl.d.status == 0)
            host_bytes += pl.in_bytes[0] + pl.in_bytes[1];
    const size_t win_cap = host_bytes >= ((size_t)512 << 20)
                               ? std::max((size_t)128 << 20, (host_bytes + 3) / 4)
                               : std::max((size_t)64 << 20, ctx->ws_budget * 4);
    std::vector<std::vector<PairPlan *>> windows(1);
    {
        size_t sb = 0;
        for (auto &pl : plans) {
            if (pl.d.status != 0)
                continue;
            const size_t st = pl.in_bytes[0] + pl.in_bytes[1] + 16;
            if (!windows.back().empty() && st > 16 && sb + st > win_cap) {
                windows.emplace_back();
                sb = 0;
            }
            windows.back().push_back(&pl);
            sb += st;
        }
    }
    std::vector<std::vector<std::vector<PairPlan *>>> wchunks(windows.size());
    size_t max_stage = 0, max_work = 0, max_n = 1;
    for (size_t w = 0; w < windows.size(); ++w) {
        std::map<std::tuple<int, int, int, int, int, int, int, int, int>,
                 std::vector<PairPlan *>>
            groups;
        size_t sb = 0;
        for (PairPlan *pl : windows[w]) {
            // transposed jobs apart: their chunks alone launch the transpose
            groups[std::make_tuple(pl->d.Nx, pl->d.Ny, pl->frame_nx1, pl->frame_ny1, pl->d.mode,
                                   pl->d.want_r, pl->d.want_s, pl->d.nseg > 0,
                                   pl->transposed ? 1 : 0)]
                .push_back(pl);
            sb += pl->in_bytes[0] + pl->in_bytes[1] + 16;
        }
        max_stage = std::max(max_stage, sb);
        for (auto &g : groups) {
            std::vector<PairPlan *> chunk;
            size_t wb = 0;
            for (PairPlan *pl : g.second) {
                const size_t wk = pl->ws_bytes - pl->in_bytes[0] - pl->in_bytes[1];
                if (!chunk.empty() && (wb + wk > ctx->ws_budget || chunk.size() >= 4096)) {
                    max_work = std::max(max_work, wb);
                    max_n = std::max(max_n, chunk.size());
                    wchunks[w].push_back(chunk);
                    chunk.clear();
                    wb = 0;
                }
                chunk.push_back(pl);
                wb += wk;
            }
            if (!chunk.empty()) {
                max_work = std::max(max_work, wb);
                max_n = std::max(max_n, chunk.size());
                wchunks[w].push_back(chunk);
            }
        }
    }
    max_stage = al256(max_stage);
    max_work = al256(max_work);
    (void)max_n;
    // one staging buffer per window parity; a single window needs one
    const size_t nstage = windows.size() > 1 ? 2 : 1;
    if (int rc = ensure_ws(ctx, nstage * max_stage + max_work))
        return rc;
    if (int rc = ensure_pairs(ctx, (size_t)std::max(npairs, 1)))
        return rc;
    if (int rc = ensure_hres(ctx, (size_t)std::max(npairs, 1)))
        return rc;
    // Staging addresses of every window first; then each chunk's host side
    // (workspaces, cache keys, its job-table slice) just before its launch,
    // so the host prepares chunk c + 1 while the device runs chunk c.  The
    // fill list holds at most one entry per job: sized for the whole batch.
    for (size_t w = 0; w < windows.size(); ++w)
        assign_staging(windows[w], ctx->ws + (w & 1) * max_stage);
    cudaStream_t st = ctx->stream;
    if ((size_t)npairs > ctx->dsel_cap) {
        CK(cudaStreamSynchronize(st));
        cudaFree(ctx->dsel);
        if (ctx->hsel)
            cudaFreeHost(ctx->hsel);
        ctx->dsel = nullptr;
        ctx->hsel = nullptr;
        ctx->dsel_cap = 0;
        const size_t cap = std::max<size_t>((size_t)npairs, 4096);
        CK(cudaMalloc(&ctx->dsel, cap * sizeof(int)));
        CK(cudaHostAlloc((void **)&ctx->hsel, cap * sizeof(int), cudaHostAllocDefault));
        ctx->dsel_cap = cap;
    }
    std::vector<std::vector<PairPlan *> *> order;
    std::vector<ChunkLaunch> cls;
    std::vector<int> fills;
    int off = 0;
    long long prep_us = 0;
    // two-stage pipeline: window w+1's copies are queued before window w's
    // kernels, on the copy stream; the kernels wait for their window only
    for (size_t w = 0; w <= windows.size(); ++w) {
        if (w < windows.size()) {
            if (int rc = stage_window(ctx, windows[w], (int)(w & 1))) {
                cudaStreamSynchronize(ctx->cstream);
                cudaStreamSynchronize(st);
                return rc;
            }
        }
        if (w == 0)
            continue;
        const size_t cw = w - 1;   // the window computed now
        const int wp = (int)(cw & 1);
        CK(cudaStreamWaitEvent(st, ctx->ev_copy[wp], 0));
        for (auto &chunk : wchunks[cw]) {
            const auto t0 = std::chrono::steady_clock::now();
            ChunkLaunch cl;
            prep_chunk(ctx, chunk, off, ctx->ws + nstage * max_stage, ctx->htab + off, fills,
                       cl);
            prep_us += std::chrono::duration_cast<std::chrono::microseconds>(
                           std::chrono::steady_clock::now() - t0)
                           .count();
            CK(cudaMemcpyAsync(ctx->dpairs_base + off, ctx->htab + off,
                               (size_t)cl.n * sizeof(PairDev), cudaMemcpyHostToDevice, st));
            if (cl.nfill) {   // through page-locked memory: no stream sync on the host
                memcpy(ctx->hsel + cl.fill_off, fills.data() + cl.fill_off,
                       (size_t)cl.nfill * sizeof(int));
                CK(cudaMemcpyAsync(ctx->dsel + cl.fill_off, ctx->hsel + cl.fill_off,
                                   (size_t)cl.nfill * sizeof(int), cudaMemcpyHostToDevice, st));
            }
            cls.push_back(cl);
            order.push_back(&chunk);
            off += cl.n;
            if (int rc = launch_chunk(ctx, chunk, cl)) {
                cudaStreamSynchronize(ctx->cstream);
                cudaStreamSynchronize(st);
                return rc;
            }
        }
        CK(cudaEventRecord(ctx->ev_wdone[wp], st));
    }
    if (!ctx->tuning)
        ctx->host_prep_us += prep_us;
    if (off > 0) {
        CK(cudaMemcpyAsync(ctx->hres, ctx->dres_base, (size_t)off * sizeof(ResultDev),
                           cudaMemcpyDeviceToHost, st));
        ctx->d2h_bytes += (long long)off * sizeof(ResultDev);
    }
    CK(cudaStreamSynchronize(st));
    prof_collect(ctx);
    for (size_t c = 0; c < order.size(); ++c)
        for (int k = 0; k < cls[c].n; ++k) {
            const ResultDev &r = ctx->hres[cls[c].off + k];
            PairDev &d = (*order[c])[k]->d;
            d.r = r.r;
            d.dx = r.dx;
            d.dy = r.dy;
            d.status = r.status;
            d.px = r.px;
            d.py = r.py;
        }
    for (int k = 0; k < npairs; ++k)
        fill_result(plans[k], &out[k]);
    return ALN_OK;
}

extern "C" int aln_corr_patches_batch(aln_ctx *ctx, int npairs, const aln_pair *pairs,
                                      aln_result *out)
{
    return batch_impl(ctx, npairs, pairs, nullptr, out);
}

extern "C" int aln_corr_images_batch(aln_ctx *ctx, int njobs, const aln_image_job *jobs,
                                     aln_result *out)
{
    if (!ctx || njobs < 0 || (njobs && (!jobs || !out)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "bad arguments") : ALN_ERR_ARG;
    std::vector<aln_pair> pairs(njobs);
    std::vector<ImgSpec> specs(njobs);
    for (int k = 0; k < njobs; ++k) {
        const aln_image_job &J = jobs[k];
        if (J.kind != ALN_CORR_R && J.kind != ALN_CORR_S && J.kind != ALN_CORR_F)
            return set_err(ctx, ALN_ERR_ARG, "CorrImages kind %d", J.kind);
        memset(&pairs[k], 0, sizeof(aln_pair));
        pairs[k].a = J.a;
        pairs[k].b = J.b;
        pairs[k].radius = 1 << 20;   // the whole R image; MaskA's oval is separate
        pairs[k].legal = J.legal;
        pairs[k].b_key = J.b_key;
        specs[k].kind = J.kind == ALN_CORR_S ? 2 : J.kind == ALN_CORR_F ? 4 : 1;
        specs[k].mincor = J.mincor;
        specs[k].nbmaxht = J.nbmaxht;
        specs[k].ox = J.ox;
        specs[k].oy = J.oy;
        specs[k].rx = J.rx;
        specs[k].ry = J.ry;
    }
    return batch_impl(ctx, njobs, pairs.data(), specs.data(), out);
}

extern "C" int aln_corr_patch_to_image(aln_ctx *ctx, const double *xy1, const double *v1,
                                       int n1, const double *i2, int n2sq, int ox, int oy,
                                       int radius, int bfilter, aln_result *out)
{
    if (!ctx || !xy1 || !v1 || !i2 || !out || n1 < 1 || n2sq < 1)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "patch_to_image: bad arguments") : ALN_ERR_ARG;
    const int N = (int)sqrt((double)n2sq);
    if (N < 16 || (N & (N - 1)) || N > ALN_MAX_N)
        return set_err(ctx, ALN_ERR_UNSUPPORTED,
                       "patch_to_image: image side %d (powers of two 16..%d)", N, ALN_MAX_N);
    // BBoxFromPoints of the patch (0_GEN/Geometry.cpp:78-106)
    double xlo = xy1[0], xhi = xy1[0], ylo = xy1[1], yhi = xy1[1];
    for (int i = 1; i < n1; ++i) {
        const double x = xy1[2 * i], y = xy1[2 * i + 1];
        if (x < xlo)
            xlo = x;
        else if (x > xhi)
            xhi = x;
        if (y < ylo)
            ylo = y;
        else if (y > yhi)
            yhi = y;
    }
    // the caller-embedded image's nonzero extent, and the patch image (points
    // truncated to pixels, later points overwrite: Correlation.cpp:1222-1249)
    int w2 = 0, h2 = 0;
    for (int i = 0; i < N * N; ++i)
        if (i2[i] != 0.0) {
            const int y = i / N, x = i - N * y;
            if (y > h2)
                h2 = y;
            if (x > w2)
                w2 = x;
        }
    std::vector<double> im1((size_t)N * N, 0.0);
    for (int i = 0; i < n1; ++i) {
        const int x = (int)xy1[2 * i], y = (int)xy1[2 * i + 1];
        if (x < 0 || y < 0 || x >= N || y >= N)
            return set_err(ctx, ALN_ERR_ARG, "patch_to_image: point %d outside the image", i);
        im1[x + (size_t)N * y] = v1[i];
    }
    aln_pair P;
    memset(&P, 0, sizeof P);
    P.a.data = im1.data();
    P.b.data = i2;
    P.a.dtype = P.b.dtype = ALN_F64;
    P.a.w = P.a.h = P.a.stride = N;
    P.b.w = P.b.h = P.b.stride = N;
    P.radius = 1 << 20;
    ImgSpec sp;
    memset(&sp, 0, sizeof sp);
    sp.kind = 3;
    sp.ox = ox;
    sp.oy = oy;
    sp.rx = radius;
    sp.p2i_w1 = (int)ceil(xhi) - (int)floor(xlo) + 1;
    sp.p2i_h1 = (int)ceil(yhi) - (int)floor(ylo) + 1;
    sp.p2i_w2 = w2 + 1;
    sp.p2i_h2 = h2 + 1;
    sp.p2i_filter = bfilter != 0;
    sp.p2i_norm = (double)n1 * ((double)N * N);
    return batch_impl(ctx, 1, &P, &sp, out);
}

extern "C" int aln_corr_images(aln_ctx *ctx, int kind, const aln_image *a, const aln_image *b,
                               const aln_legal *legal, double mincor, double nbmaxht, int ox,
                               int oy, int rx, int ry, aln_result *out)
{
    if (!ctx || !a || !b || !out)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "null argument") : ALN_ERR_ARG;
    aln_image_job J;
    memset(&J, 0, sizeof J);
    J.a = *a;
    J.b = *b;
    J.kind = kind;
    if (legal)
        J.legal = *legal;
    J.mincor = mincor;
    J.nbmaxht = nbmaxht;
    J.ox = ox;
    J.oy = oy;
    J.rx = rx;
    J.ry = ry;
    return aln_corr_images_batch(ctx, 1, &J, out);
}

extern "C" int aln_corr_patches(aln_ctx *ctx, const aln_image *a, const aln_image *b, int ox,
                                int oy, int radius, const aln_legal *legal, aln_result *out)
{
    if (!ctx || !a || !b || !out)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "null argument") : ALN_ERR_ARG;
    aln_pair P;
    memset(&P, 0, sizeof P);
    P.a = *a;
    P.b = *b;
    P.ox = ox;
    P.oy = oy;
    P.radius = radius;
    if (legal)
        P.legal = *legal;
    return aln_corr_patches_batch(ctx, 1, &P, out);
}

extern "C" void aln_parab_peak_fft(double *xpk, double *ypk, int d, const double *I, int nx,
                                   int ny)
{
    // ParabPeakFFT, 0_GEN/Correlation.cpp:482-517 (host arithmetic, O(1))
    auto lk = [&](int x, int y) {
        if (x < 0)
            x += nx;
        if (y < 0)
            y += ny;
        return I[x + (long long)nx * y];
    };
    const int ix = (int)*xpk, iy = (int)*ypk;
    const double z1 = lk(ix, iy);
    double z0, z2;
    if (ix - d >= 0 && ix + d < nx && (z0 = lk(ix - d, iy)) != 0.0 &&
        (z2 = lk(ix + d, iy)) != 0.0) {
        z0 = d * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * d)
            *xpk += z0;
    }
    if (iy - d >= 0 && iy + d < ny && (z0 = lk(ix, iy - d)) != 0.0 &&
        (z2 = lk(ix, iy + d)) != 0.0) {
        z0 = d * (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8 * d)
            *ypk += z0;
    }
}

extern "C" int aln_fft_2d(aln_ctx *ctx, const double *in, int nfast, int nslow, double *out)
{
    if (!ctx || !in || !out || nfast < 2 || nslow < 1 || (nfast & (nfast - 1)) ||
        (nslow & (nslow - 1)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "fft_2d: sizes must be powers of two, nfast >= 2")
                   : ALN_ERR_ARG;
    if (nfast > ALN_MAX_N || nslow > ALN_MAX_N)
        return set_err(ctx, ALN_ERR_UNSUPPORTED, "fft_2d: size above %d", ALN_MAX_N);
    CK(cudaSetDevice(ctx->device));
    const int L1 = nfast / 2 + 1;
    const size_t M = (size_t)L1 * nslow;
    const size_t inb = al256((size_t)nfast * nslow * 8), Tb = al256(M * 8), Xb = al256(M * 8),
                 ob = al256(M * 16);
    if (int rc = ensure_ws(ctx, inb + Tb + Xb + ob))
        return rc;
    if (int rc = ensure_pairs(ctx, 1))
        return rc;
    char *p = ctx->ws;
    PairDev d;
    memset(&d, 0, sizeof d);
    d.img[1] = p;
    d.dt[1] = ALN_F64;
    d.stride[1] = nfast;
    d.w[1] = nfast;
    d.h[1] = nslow;
    d.Nx = nfast;
    d.Ny = std::max(1, nslow);
    d.logNx = ilog2(nfast);
    d.logNy = ilog2(nslow);
    d.T[1] = (float2 *)(p + inb);
    d.Ts[1] = nslow;
    d.X2 = (float2 *)(p + inb + Tb);
    d.mu[1] = 0.0;
    double *dout = (double *)(p + inb + Tb + Xb);
    CK(cudaMemcpyAsync(p, in, (size_t)nfast * nslow * 8, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemcpyAsync(ctx->dpairs, &d, sizeof d, cudaMemcpyHostToDevice, ctx->stream));
    const int L = nfast / 2;
    const int RB = rows_per_cta(L);
    LAUNCH(ctx, "k_rowfft", k_rowfft, dim3((nslow + RB - 1) / RB, 1, 1), 256,
           2 * (size_t)RB * (L + 1) * sizeof(float2), ctx->dpairs, ctx->tw, RB, 1);
    const int CG = cols_per_cta(nslow);
    LAUNCH(ctx, "k_colfft", k_colfft, dim3((L1 + CG - 1) / CG, 1), 256,
           2 * (size_t)CG * (nslow + 1) * sizeof(float2), ctx->dpairs, ctx->tw, CG);
    LAUNCH(ctx, "k_spec_to_fftw", k_spec_to_fftw, (unsigned)std::min<size_t>(4096, (M + 255) / 256),
           256, 0, d.X2, L1, nslow, dout);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout, M * 16, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    return (int)M;
}

extern "C" int aln_ift_2d(aln_ctx *ctx, const double *in, int nfast, int nslow, double *out)
{
    if (!ctx || !in || !out || nfast < 2 || nslow < 1 || (nfast & (nfast - 1)) ||
        (nslow & (nslow - 1)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "ift_2d: sizes must be powers of two, nfast >= 2")
                   : ALN_ERR_ARG;
    if (nfast > ALN_MAX_N || nslow > ALN_MAX_N)
        return set_err(ctx, ALN_ERR_UNSUPPORTED, "ift_2d: size above %d", ALN_MAX_N);
    CK(cudaSetDevice(ctx->device));
    const int L1 = nfast / 2 + 1;
    const size_t M = (size_t)L1 * nslow;
    const size_t inb = al256(M * 16), Sb = al256(M * 8), Qb = al256(M * 8),
                 ob = al256((size_t)nfast * nslow * 8);
    if (int rc = ensure_ws(ctx, inb + Sb + Qb + ob))
        return rc;
    char *p = ctx->ws;
    double *din = (double *)p;
    float2 *S = (float2 *)(p + inb);
    float2 *Q = (float2 *)(p + inb + Sb);
    double *dout = (double *)(p + inb + Sb + Qb);
    CK(cudaMemcpyAsync(din, in, M * 16, cudaMemcpyHostToDevice, ctx->stream));
    LAUNCH(ctx, "k_fftw_to_spec", k_fftw_to_spec, (unsigned)std::min<size_t>(4096, (M + 255) / 256),
           256, 0, din, L1, nslow, S);
    const int CG = cols_per_cta(nslow);
    LAUNCH(ctx, "k_icolfft", k_icolfft, (L1 + CG - 1) / CG, 256,
           2 * (size_t)CG * (nslow + 1) * sizeof(float2), S, Q, L1, ilog2(nslow), ctx->tw, CG);
    const int L = nfast / 2;
    const int RBL = std::max(1, std::min(8, 4096 / L));
    LAUNCH(ctx, "k_irowfft", k_irowfft, (nslow + RBL - 1) / RBL, 256,
           2 * (size_t)RBL * (L + 1) * sizeof(float2), Q, ilog2(nfast), nslow, dout, ctx->tw, RBL);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(out, dout, (size_t)nfast * nslow * 8, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    prof_collect(ctx);
    return ALN_OK;
}

// Convolve's kernel frame: zeros, K / nrm at the wrapped offsets
// (0_GEN/Correlation.cpp:395-420), one thread per frame pixel.
__global__ void k_conv_frame(double *KK, int Nx, int Ny, const double *K, int wk, int hk,
                             double nrm)
{
    const long long n = (long long)Nx * Ny;
    const int w2 = wk / 2, h2 = hk / 2;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(e % Nx), y = (int)(e / Nx);
        const int j = x <= w2 ? x : x - Nx, i = y <= h2 ? y : y - Ny;   // offsets -w2..w2
        double v = 0.0;
        if (j >= -w2 && j <= w2 && i >= -h2 && i <= h2)
            v = K[(j + w2) + wk * (i + h2)] / nrm;
        KK[e] = v;
    }
}

// S = X * Y (spectra in the [kx][ky] layout)
__global__ void k_spec_mul(const float2 *X, const float2 *Y, float2 *S, long long n)
{
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        S[e] = cmul(X[e], Y[e]);
}

// dst[x + ws*y] = out[x + Nx*y] / (Nx*Ny) for the source's extent
__global__ void k_crop_scale(const double *out, int Nx, int Ny, double *dst, int ws, int hs)
{
    const long long n = (long long)ws * hs;
    const double s = 1.0 / ((double)Nx * Ny);
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(e % ws), y = (int)(e / ws);
        dst[e] = out[(long long)y * Nx + x] * s;
    }
}

extern "C" int aln_convolve(aln_ctx *ctx, const double *src, int ws, int hs, const double *K,
                            int wk, int hk, int sym, int prenorm, double *dst)
{
    if (!ctx || !src || !K || !dst || ws < 1 || hs < 1 || wk < 1 || hk < 1)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "convolve: bad arguments") : ALN_ERR_ARG;
    const int Nx = aln_fft_size(ws, wk / (1 + (sym ? 1 : 0)));
    const int Ny = aln_fft_size(hs, hk / (1 + (sym ? 1 : 0)));
    if (Nx < 2 || Nx > ALN_MAX_N || Ny > ALN_MAX_N)
        return set_err(ctx, ALN_ERR_UNSUPPORTED, "convolve: frame %d x %d", Nx, Ny);
    CK(cudaSetDevice(ctx->device));
    double nrm = 1.0;
    if (prenorm) {   // the kernel's sum, as the reference forms it
        nrm = 0.0;
        for (int i = 0; i < wk * hk; ++i)
            nrm += K[i];
        if (!nrm)
            nrm = 1.0;
    }
    const int L1 = Nx / 2 + 1;
    const size_t M = (size_t)L1 * Ny, NN = (size_t)Nx * Ny;
    const size_t sb = al256((size_t)ws * hs * 8), kb = al256((size_t)wk * hk * 8),
                 fb = al256(NN * 8), Tb = al256(M * 8);
    if (int rc = ensure_ws(ctx, sb + kb + fb + 2 * Tb + 3 * Tb + fb + sb))
        return rc;
    if (int rc = ensure_pairs(ctx, 2))
        return rc;
    char *p = ctx->ws;
    double *dsrc = (double *)p;                 p += sb;
    double *dK = (double *)p;                   p += kb;
    double *KK = (double *)p;                   p += fb;
    float2 *T0 = (float2 *)p;                   p += Tb;
    float2 *T1 = (float2 *)p;                   p += Tb;
    float2 *X0 = (float2 *)p;                   p += Tb;
    float2 *X1 = (float2 *)p;                   p += Tb;
    float2 *S = (float2 *)p;                    p += Tb;
    double *dout = (double *)p;                 p += fb;
    double *ddst = (double *)p;
    cudaStream_t st = ctx->stream;
    CK(cudaMemcpyAsync(dsrc, src, (size_t)ws * hs * 8, cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dK, K, (size_t)wk * hk * 8, cudaMemcpyHostToDevice, st));
    const unsigned gs = (unsigned)std::min<size_t>(4096, (NN + 255) / 256);
    LAUNCH(ctx, "k_conv_frame", k_conv_frame, gs, 256, 0, KK, Nx, Ny, dK, wk, hk, nrm);
    // forward transforms of the source (zero-padded) and the kernel frame
    PairDev d[2];
    memset(d, 0, sizeof d);
    const void *imgs[2] = {dsrc, KK};
    const int ww[2] = {ws, Nx}, hh[2] = {hs, Ny};
    float2 *Ts[2] = {T0, T1}, *Xs[2] = {X0, X1};
    for (int k = 0; k < 2; ++k) {
        d[k].img[1] = imgs[k];
        d[k].dt[1] = ALN_F64;
        d[k].stride[1] = ww[k];
        d[k].w[1] = ww[k];
        d[k].h[1] = hh[k];
        d[k].Nx = Nx;
        d[k].Ny = Ny;
        d[k].logNx = ilog2(Nx);
        d[k].logNy = ilog2(Ny);
        d[k].T[1] = Ts[k];
        d[k].Ts[1] = Ny;
        d[k].X2 = Xs[k];
    }
    CK(cudaMemcpyAsync(ctx->dpairs, d, sizeof d, cudaMemcpyHostToDevice, st));
    const int L = Nx / 2;
    const int RB = rows_per_cta(L);
    LAUNCH(ctx, "k_rowfft", k_rowfft, dim3((Ny + RB - 1) / RB, 1, 2), 256,
           2 * (size_t)RB * (L + 1) * sizeof(float2), ctx->dpairs, ctx->tw, RB, 1);
    const int CG = cols_per_cta(Ny);
    LAUNCH(ctx, "k_colfft", k_colfft, dim3((L1 + CG - 1) / CG, 2), 256,
           2 * (size_t)CG * (Ny + 1) * sizeof(float2), ctx->dpairs, ctx->tw, CG);
    const unsigned gm = (unsigned)std::min<size_t>(4096, (M + 255) / 256);
    LAUNCH(ctx, "k_spec_mul", k_spec_mul, gm, 256, 0, X0, X1, S, (long long)M);
    // inverse, crop, 1 / (Nx Ny)
    float2 *Q = T0;   // free again
    LAUNCH(ctx, "k_icolfft", k_icolfft, (L1 + CG - 1) / CG, 256,
           2 * (size_t)CG * (Ny + 1) * sizeof(float2), S, Q, L1, ilog2(Ny), ctx->tw, CG);
    const int RBL = std::max(1, std::min(8, 4096 / L));
    LAUNCH(ctx, "k_irowfft", k_irowfft, (Ny + RBL - 1) / RBL, 256,
           2 * (size_t)RBL * (L + 1) * sizeof(float2), Q, ilog2(Nx), Ny, dout, ctx->tw, RBL);
    LAUNCH(ctx, "k_crop_scale", k_crop_scale,
           (unsigned)std::min<size_t>(4096, ((size_t)ws * hs + 255) / 256), 256, 0, dout, Nx, Ny,
           ddst, ws, hs);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dst, ddst, (size_t)ws * hs * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    prof_collect(ctx);
    return ALN_OK;
}

// ---------------------------------------------------------------------------
// tracing (no reference counterpart: the reference logs wall-clock Timer
// lines, 0_GEN/Timer.cpp:25-52)
// ---------------------------------------------------------------------------

extern "C" int aln_ctx_set_profiling(aln_ctx *ctx, int on)
{
    if (!ctx)
        return ALN_ERR_ARG;
    ctx->prof_on = on ? 1 : 0;
    return ALN_OK;
}

extern "C" void aln_ctx_profile_reset(aln_ctx *ctx)
{
    if (!ctx)
        return;
    cudaStreamSynchronize(ctx->stream);
    prof_collect(ctx);
    ctx->prof_acc.clear();
    ctx->launches = 0;
    ctx->h2d_bytes = ctx->d2h_bytes = 0;
    ctx->spec_hits = ctx->spec_fills = ctx->spec_evictions = 0;
    ctx->host_plan_us = ctx->host_prep_us = 0;
    ctx->chunks = 0;
    ctx->h2d_copies = 0;
}

extern "C" int aln_ctx_profile(aln_ctx *ctx, int cap, const char **names,
                               long long *launches, double *ms)
{
    if (!ctx)
        return ALN_ERR_ARG;
    cudaStreamSynchronize(ctx->stream);
    prof_collect(ctx);
    ctx->prof_names.clear();
    for (auto &kv : ctx->prof_acc)
        ctx->prof_names.push_back(kv.first);
    int k = 0;
    for (auto &kv : ctx->prof_acc) {
        if (k >= cap)
            break;
        if (names)
            names[k] = ctx->prof_names[k].c_str();
        if (launches)
            launches[k] = kv.second.first;
        if (ms)
            ms[k] = kv.second.second;
        ++k;
    }
    return (int)ctx->prof_acc.size();
}

extern "C" long long aln_ctx_counter(aln_ctx *ctx, int which)
{
    if (!ctx)
        return -1;
    switch (which) {
    case 0: return ctx->launches;
    case 1: return ctx->h2d_bytes;
    case 2: return ctx->d2h_bytes;
    case 3: return ctx->spec_hits;
    case 4: return ctx->spec_fills;
    case 5: return (long long)ctx->spec_bytes;
    case 6: return ctx->chunks;
    case 7: return ctx->h2d_copies;
    case 8: return ctx->tune_classes;
    case 9: return ctx->spec_evictions;
    case 10: return ctx->host_plan_us;
    case 11: return ctx->host_prep_us;
    default: return -1;
    }
}

extern "C" int aln_ctx_set_segmenting(aln_ctx *ctx, int ns)
{
    if (!ctx || ns < -1 || (ns > 0 && (ns < 64 || ns > 2048 || (ns & (ns - 1)))))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "segment length %d", ns) : ALN_ERR_ARG;
    ctx->seg_ns = ns;
    return ALN_OK;
}

extern "C" int aln_ctx_set_tuning(aln_ctx *ctx, int on)
{
    if (!ctx)
        return ALN_ERR_ARG;
    ctx->tune_on = on ? 1 : 0;
    return ALN_OK;
}

extern "C" int aln_ctx_set_split_grids(aln_ctx *ctx, int on)
{
    if (!ctx)
        return ALN_ERR_ARG;
    ctx->split_on = on ? 1 : 0;
    return ALN_OK;
}

extern "C" int aln_ctx_set_spectrum_cache(aln_ctx *ctx, size_t bytes)
{
    if (!ctx)
        return ALN_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->spec_cap = bytes;
    ++ctx->spec_tick;   // nothing is in use now: every entry may go
    while (ctx->spec_bytes > bytes) {
        if (!ctx->spec_free.empty()) {
            auto g = std::prev(ctx->spec_free.end());
            cudaFree(g->second);
            ctx->spec_bytes -= g->first;
            ctx->spec_free.erase(g);
            continue;
        }
        if (ctx->spec_lru.empty())
            break;
        auto lru = ctx->spec.find(ctx->spec_lru.begin()->second);
        ctx->spec_free.insert(std::make_pair(lru->second.bytes, lru->second.X2));
        spec_erase(ctx, lru);
    }
    return ALN_OK;
}

extern "C" int aln_ctx_set_workspace_limit(aln_ctx *ctx, size_t bytes)
{
    if (!ctx || bytes < ((size_t)16 << 20))
        return ALN_ERR_ARG;
    ctx->ws_budget = bytes;
    return ALN_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free CorrPatches.  No reference counterpart.
//
// For callers that must not allocate device memory: code running inside a
// memory pool or arena they do not control, plugins of hosts that forbid
// cudaMalloc after start-up, or code whose allocations would stall a busy
// device.  The work space lives in one file-scope device array of
// ALN_NOALLOC_SCRATCH_BYTES, which every GPU that loads this library holds
// until the process exits.  Nothing here calls cudaMalloc, cudaFree or any
// allocating routine, and no host heap memory is used either.
// ---------------------------------------------------------------------------

#define ALN_NOALLOC_SCRATCH_BYTES ((size_t)ALN_NOALLOC_SCRATCH_MIB << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[ALN_NOALLOC_SCRATCH_BYTES];

// the twiddle table sits at the start of the scratch and survives calls
static const size_t kNoAllocTwBytes = (2 * ALN_MAX_N * sizeof(float2) + 255) & ~(size_t)255;

__global__ void k_fill_twiddles(float2 *tw)
{
    const int total = 2 * ALN_MAX_N;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        if (e == 0) {
            tw[0] = make_float2(1.f, 0.f);
            continue;
        }
        int N = 1;
        while (2 * N <= e)
            N <<= 1;
        const int m = e - N;
        double s, c;
        sincospi(-2.0 * (double)m / (double)N, &s, &c);
        tw[e] = make_float2((float)c, (float)s);
    }
}

static std::mutex g_noalloc_lock;
static char *g_noalloc_base[64];   // scratch device address per device, set once

// One-time set-up on the current device: look up the scratch address, allow
// the large shared-memory configurations, fill the twiddle table.
static int noalloc_setup(int dev, cudaStream_t st, char **base)
{
    std::lock_guard<std::mutex> g(g_noalloc_lock);
    if (g_noalloc_base[dev]) {
        *base = g_noalloc_base[dev];
        return ALN_OK;
    }
    char *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
    if (e != cudaSuccess)
        return set_err(nullptr, ALN_ERR_CUDA, "scratch address: %s", cudaGetErrorString(e));
    if (int ke = configure_kernels())
        return set_err(nullptr, ALN_ERR_CUDA, "kernel attributes: %s",
                       cudaGetErrorString((cudaError_t)ke));
    k_fill_twiddles<<<64, 256, 0, st>>>((float2 *)p);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return set_err(nullptr, ALN_ERR_CUDA, "twiddle set-up: %s", cudaGetErrorString(e));
    g_noalloc_base[dev] = p;
    *base = p;
    return ALN_OK;
}

extern "C" int aln_corr_patches_noalloc(const aln_image *a, const aln_image *b, int ox, int oy,
                                        int radius, const aln_legal *legal, void *stream,
                                        aln_result *out)
{
    aln_ctx *ctx = nullptr;   // errors go to aln_last_error(NULL)
    if (!a || !b || !out)
        return set_err(nullptr, ALN_ERR_ARG, "noalloc: null argument");
    if (!a->on_device || !b->on_device)
        return set_err(nullptr, ALN_ERR_ARG, "noalloc: images must be device pointers");
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64)
        return set_err(nullptr, ALN_ERR_ARG, "noalloc: device %d out of range", dev);
    // both images must live on the current device: a pointer into another
    // GPU's memory would be read over the peer link without any error
    for (const aln_image *im : {a, b}) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, im->data) != cudaSuccess) {
            cudaGetLastError();
            return set_err(nullptr, ALN_ERR_ARG, "noalloc: image pointer is not device memory");
        }
        if ((at.type != cudaMemoryTypeDevice && at.type != cudaMemoryTypeManaged) ||
            at.device != dev)
            return set_err(nullptr, ALN_ERR_ARG,
                           "noalloc: image memory is on device %d, the current device is %d",
                           at.device, dev);
    }
    cudaStream_t st = (cudaStream_t)stream;
    char *base = nullptr;
    if (int rc = noalloc_setup(dev, st, &base))
        return rc;

    aln_pair P;
    memset(&P, 0, sizeof P);
    P.a = *a;
    P.b = *b;
    P.ox = ox;
    P.oy = oy;
    P.radius = radius;
    if (legal)
        P.legal = *legal;
    PairPlan pl;
    memset(&pl, 0, sizeof pl);
    pl.src = &P;
    if (int rc = plan_pair(nullptr, P, pl))
        return rc;
    memset(out, 0, sizeof *out);
    out->nx = pl.orig_nx;
    out->ny = pl.orig_ny;
    if (pl.d.status != 0) {   // empty search region
        out->status = ALN_NO_PEAK;
        return ALN_OK;
    }
    const size_t head = kNoAllocTwBytes + al256(sizeof(PairDev)) + al256(sizeof(ResultDev));
    if (head + pl.ws_bytes > ALN_NOALLOC_SCRATCH_BYTES)
        return set_err(nullptr, ALN_ERR_UNSUPPORTED,
                       "noalloc: this pair needs %zu bytes of scratch; the allocation-free entry "
                       "point has %zu (use aln_corr_patches)",
                       head + pl.ws_bytes, (size_t)ALN_NOALLOC_SCRATCH_BYTES);
    float2 *tw = (float2 *)base;
    PairDev *dpair = (PairDev *)(base + kNoAllocTwBytes);
    ResultDev *dres = (ResultDev *)(base + kNoAllocTwBytes + al256(sizeof(PairDev)));
    carve(pl, base + head, P);
    PairDev &d = pl.d;
    if (d.rgn_kind == ALN_RGN_TABLE)
        CK(cudaMemcpyAsync((void *)d.table, P.legal.table, (size_t)d.table_w * d.table_h,
                           cudaMemcpyHostToDevice, st));
    CK(cudaMemcpyAsync(dpair, &d, sizeof(PairDev), cudaMemcpyHostToDevice, st));
    const int Nx = d.Nx, Ny = d.Ny, L = Nx / 2;
    int maxslots = 1;
    for (int i = 0; i < 2; ++i) {
        int ns = 0;
        for (int q = 0; q < 2; ++q)
            if (d.need_hi[i][q] >= d.need_lo[i][q])
                ns += d.need_hi[i][q] - d.need_lo[i][q] + 1;
        maxslots = std::max(maxslots, ns);
    }
    const int maxw = std::max(d.w[0], d.w[1]), maxh = std::max(d.h[0], d.h[1]);
    const int Wy = d.yhi - d.ylo + 1;
    k_colsum<<<dim3((maxw + 127) / 128, 2, 1), 128, 0, st>>>(dpair);
    k_mean<<<dim3(2, 1), 256, 0, st>>>(dpair);
    k_rowscan<<<dim3(maxslots, 2, 1), 256, 0, st>>>(dpair);
    {
        const int RB = rows_per_cta(L);
        const size_t sm = 2 * (size_t)RB * (L + 1) * sizeof(float2);
        k_rowfft<<<dim3((maxh + RB - 1) / RB, 2, 1), 256, sm, st>>>(dpair, tw, RB, -1);
    }
    {
        const int CG = cols_per_cta(Ny);
        const size_t sm = 2 * (size_t)CG * (Ny + 1) * sizeof(float2);
        const int gx = (L + 1 + CG - 1) / CG;
        k_colfft<<<dim3(gx, 1), 256, sm, st>>>(dpair, tw, CG);
        k_corrcol<<<dim3(gx, 1), 256, sm, st>>>(dpair, tw, CG);
    }
    {
        const int RBL = std::max(1, std::min(8, 4096 / std::max(1, L)));
        const size_t sm = 2 * (size_t)RBL * (L + 1) * sizeof(float2);
        k_lagrow<<<dim3((Wy + RBL - 1) / RBL, 1), 256, sm, st>>>(dpair, tw, RBL);
    }
    k_final<<<1, 256, 0, st>>>(dpair, dres, pl.orig_nx == 1, pl.orig_ny == 1);
    CK(cudaGetLastError());
    ResultDev hr;
    CK(cudaMemcpyAsync(&hr, dres, sizeof hr, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    out->status = hr.status == ALN_OK ? ALN_OK : ALN_NO_PEAK;
    out->r = out->status == ALN_OK ? hr.r : 0.0;
    out->dx = out->status == ALN_OK ? hr.dx : 0.0;
    out->dy = out->status == ALN_OK ? hr.dy : 0.0;
    out->peak_x = hr.px;
    out->peak_y = hr.py;
    return ALN_OK;
}

#include "aln_sweep.cuh"
#include "aln_ingest.cuh"
#include "aln_thmpair.cuh"
#include "aln_points.cuh"
#include "aln_approx.cuh"
#include "aln_mesh.cuh"
#include "aln_server.cuh"
