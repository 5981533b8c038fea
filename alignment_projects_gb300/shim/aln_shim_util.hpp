// aln_shim_util.hpp -- host helpers shared by the C++ drop-ins
// (aln_correlation_shim.cpp, aln_thmscan_shim.cpp): the per-thread GPU
// context, point lists -> bounding-box rasters (BBoxFromPoints,
// 0_GEN/Geometry.cpp:78-106; integer points placed on the host, fractional
// clouds splatted on the device by aln_points_image) and the fft2 / ftc
// cache vectors -> spectrum-cache keys.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <complex>
#include <vector>

#include "../../include/aln_corr.h"

namespace aln_shim {

typedef std::complex<double> CDv;

// one context per host thread (the reference serialises its FFTs under a
// mutex; here each thread has its own stream and workspace)
inline aln_ctx *ctx()
{
    static thread_local aln_ctx *c = nullptr;
    if (!c && aln_ctx_create(0, &c) != ALN_OK)
        c = nullptr;
    return c;
}

struct IBoxD {
    int L, R, B, T;
};

template <class P>
inline IBoxD bbox(const std::vector<P> &p)
{
    double xlo = p[0].x, xhi = p[0].x, ylo = p[0].y, yhi = p[0].y;
    for (size_t i = 1; i < p.size(); ++i) {
        const double x = p[i].x, y = p[i].y;
        if (x < xlo)
            xlo = x;
        else if (x > xhi)
            xhi = x;
        if (y < ylo)
            ylo = y;
        else if (y > yhi)
            yhi = y;
    }
    return IBoxD{(int)floor(xlo), (int)ceil(xhi), (int)floor(ylo), (int)ceil(yhi)};
}

// The points' raster over their bounding box: bilinear weights of each
// point's value on the four pixels around it, bounds-checked (integer
// points land on one pixel with weight 1).
template <class P>
inline std::vector<double> raster(const std::vector<P> &p, const std::vector<double> &v,
                           const IBoxD &B)
{
    const int w = B.R - B.L + 1, h = B.T - B.B + 1;
    std::vector<double> I((size_t)w * h, 0.0);
    for (size_t k = 0; k < p.size(); ++k) {
        const double x = p[k].x - B.L, y = p[k].y - B.B;
        int ix = (int)floor(x), iy = (int)floor(y);
        const double a = x - ix, b = y - iy, val = v[k];
        for (int dxp = 0; dxp < 2; ++dxp) {
            const int X = ix + dxp;
            if (X < 0 || X >= w)
                continue;
            const double wx = dxp ? a : 1.0 - a;
            for (int dyp = 0; dyp < 2; ++dyp) {
                const int Y = iy + dyp;
                if (Y < 0 || Y >= h)
                    continue;
                I[(size_t)X + (size_t)w * Y] += wx * (dyp ? b : 1.0 - b) * val;
            }
        }
    }
    return I;
}

inline aln_image image_of(const std::vector<double> &I, const IBoxD &B)
{
    aln_image im;
    im.data = I.data();
    im.dtype = ALN_F64;
    im.w = B.R - B.L + 1;
    im.h = B.T - B.B + 1;
    im.stride = im.w;
    im.x0 = B.L;
    im.y0 = B.B;
    im.on_device = 0;
    return im;
}

// A point list's raster as an aln_image.  Integer points are placed on the
// host (each value lands on its own pixel; that is a copy, duplicates add);
// a cloud with fractional points is splatted on the device with
// DistributePixel's bilinear weights (aln_points_image, context slot
// `slot`, valid until the next call with that slot).
template <class P>
inline bool image_of_points(const std::vector<P> &p, const std::vector<double> &v,
                            const IBoxD &B, int slot, std::vector<double> &host, aln_image &im)
{
    bool integral = true;
    for (const P &q : p)
        if (q.x != floor(q.x) || q.y != floor(q.y)) {
            integral = false;
            break;
        }
    if (integral) {
        host = raster(p, v, B);
        im = image_of(host, B);
        return true;
    }
    std::vector<double> xy(2 * p.size());
    for (size_t k = 0; k < p.size(); ++k) {
        xy[2 * k] = p[k].x;
        xy[2 * k + 1] = p[k].y;
    }
    return aln_points_image(ctx(), slot, (int)p.size(), xy.data(), v.data(), B.L, B.B,
                            B.R - B.L + 1, B.T - B.B + 1, &im, nullptr) == ALN_OK;
}

// fft2 / ftc: the reference reuses image 2's spectrum while the vector keeps
// the FFT's size.  The vector's contents are the shim's own: its first
// element carries the spectrum-cache key of the image it was filled for.
inline std::atomic<unsigned long long> g_key{1};

inline unsigned long long key_of(std::vector<CDv> &fft2, size_t M)
{
    unsigned long long k = 0;
    if (fft2.size() == M && M > 0) {
        const double re = fft2[0].real();
        memcpy(&k, &re, sizeof k);
        return k;
    }
    k = (g_key++ << 1) | 1;   // never 0 (0 means "no key")
    fft2.assign(M, CDv(0.0, 0.0));
    double re;
    memcpy(&re, &k, sizeof re);
    if (M)
        fft2[0] = CDv(re, 0.0);
    return k;
}

}   // namespace aln_shim
