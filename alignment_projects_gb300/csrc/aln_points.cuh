// aln_points.cuh -- point clouds to rasters on the device: the reference's
// ImageFromValuesAndPoints with DistributePixel's bilinear weights
// (0_GEN/Geometry.cpp:661-685, 0_GEN/Maths.h:236-276).  Included by
// aln_corr.cu.
//
// The weights and their products are the reference's, in FP64.  The sums
// per pixel are taken in 64-bit fixed point with atomic adds -- exact and
// independent of the order the points land in, so a cloud gives the same
// raster bit for bit on every run -- at a scale of 2^-k with k as large as
// the cloud's largest |value| allows (4 |v|max 2^k < 2^62): integer values
// on integer points come out exact, other sums within 2^-k of the FP64 sum.
#pragma once

__global__ void k_pts_absmax(const double *v, int n, unsigned long long *mx)
{
    unsigned long long m = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = max(m, (unsigned long long)__double_as_longlong(fabs(v[i])));
    for (int o = 16; o > 0; o >>= 1)
        m = max(m, __shfl_xor_sync(0xffffffff, m, o));
    if ((threadIdx.x & 31) == 0)
        atomicMax(mx, m);
}

__device__ __forceinline__ void pts_add(unsigned long long *acc, long long i, double q)
{
    atomicAdd(acc + i, (unsigned long long)__double2ll_rn(q));
}

// DistributePixel, Maths.h:236-276, at fixed-point scale 2^k (exact scaling)
__global__ void k_pts_splat(const double *xy, const double *v, int n, int xmin, int ymin,
                            int w, int h, const unsigned long long *mx, unsigned long long *acc)
{
    const double vmax = __longlong_as_double((long long)*mx);
    int e = 0;
    frexp(4.0 * vmax + 1.0, &e);   // 4 |v|max + 1 < 2^e
    const int k = min(60, 62 - e);
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const double x = __dsub_rn(xy[2 * p], (double)xmin);
        const double y = __dsub_rn(xy[2 * p + 1], (double)ymin);
        const int ix = (int)floor(x), iy = (int)floor(y);
        const double alpha = __dsub_rn(x, (double)ix), beta = __dsub_rn(y, (double)iy);
        const double val = ldexp(v[p], k);
        const long long i = ix + (long long)w * iy;
        if (ix >= 0 && ix < w) {
            if (iy >= 0 && iy < h)
                pts_add(acc, i, __dmul_rn(__dmul_rn(__dsub_rn(1.0, alpha),
                                                    __dsub_rn(1.0, beta)), val));
            if (iy + 1 >= 0 && iy + 1 < h)
                pts_add(acc, i + w, __dmul_rn(__dmul_rn(__dsub_rn(1.0, alpha), beta), val));
        }
        if (ix + 1 >= 0 && ix + 1 < w) {
            if (iy >= 0 && iy < h)
                pts_add(acc, i + 1, __dmul_rn(__dmul_rn(alpha, __dsub_rn(1.0, beta)), val));
            if (iy + 1 >= 0 && iy + 1 < h)
                pts_add(acc, i + 1 + w, __dmul_rn(__dmul_rn(alpha, beta), val));
        }
    }
}

__global__ void k_pts_finish(const unsigned long long *acc, long long npix,
                             const unsigned long long *mx, double *out)
{
    const double vmax = __longlong_as_double((long long)*mx);
    int e = 0;
    frexp(4.0 * vmax + 1.0, &e);
    const int k = min(60, 62 - e);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < npix;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = ldexp((double)(long long)acc[i], -k);
}

extern "C" int aln_points_image(aln_ctx *ctx, int slot, int n, const double *xy,
                                const double *v, int xmin, int ymin, int w, int h,
                                aln_image *out, double *host_copy)
{
    if (!ctx || slot < 0 || slot > 1 || n < 0 || (n && (!xy || !v)) || w < 1 || h < 1 || !out)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "points_image: bad arguments") : ALN_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    const size_t npix = (size_t)w * h;
    const size_t need = al256(npix * sizeof(double)) + al256(npix * 8) +
                        al256(std::max(n, 1) * 3 * sizeof(double)) + 256;
    if (need > ctx->pts_cap[slot]) {
        CK(cudaStreamSynchronize(ctx->stream));
        if (ctx->pts_buf[slot])
            cudaFree(ctx->pts_buf[slot]);
        ctx->pts_buf[slot] = nullptr;
        ctx->pts_cap[slot] = 0;
        if (cudaMalloc(&ctx->pts_buf[slot], need) != cudaSuccess) {
            cudaGetLastError();
            return set_err(ctx, ALN_ERR_NOMEM, "points_image: %zu bytes", need);
        }
        ctx->pts_cap[slot] = need;
    }
    char *p = ctx->pts_buf[slot];
    double *img = (double *)p;
    p += al256(npix * sizeof(double));
    unsigned long long *acc = (unsigned long long *)p;
    p += al256(npix * 8);
    double *dxy = (double *)p;
    double *dv = dxy + 2 * (size_t)n;
    p += al256(std::max(n, 1) * 3 * sizeof(double));
    unsigned long long *mx = (unsigned long long *)p;
    cudaStream_t st = ctx->stream;
    CK(cudaMemsetAsync(acc, 0, npix * 8, st));
    CK(cudaMemsetAsync(mx, 0, 8, st));
    if (n) {
        CK(cudaMemcpyAsync(dxy, xy, 2 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(dv, v, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
        ctx->h2d_bytes += 3 * (long long)n * sizeof(double);
        const int blk = (int)std::min<long long>(4096, (n + 255) / 256);
        LAUNCH(ctx, "k_pts_absmax", k_pts_absmax, blk, 256, 0, dv, n, mx);
        LAUNCH(ctx, "k_pts_splat", k_pts_splat, blk, 256, 0, dxy, dv, n, xmin, ymin, w, h, mx,
               acc);
        ctx->launches += 2;
    }
    LAUNCH(ctx, "k_pts_finish", k_pts_finish,
           (int)std::min<long long>(4096, ((long long)npix + 255) / 256), 256, 0, acc,
           (long long)npix, mx, img);
    ctx->launches++;
    CK(cudaGetLastError());
    out->data = img;
    out->dtype = ALN_F64;
    out->w = w;
    out->h = h;
    out->stride = w;
    out->x0 = xmin;
    out->y0 = ymin;
    out->on_device = 1;
    if (host_copy) {
        CK(cudaMemcpyAsync(host_copy, img, npix * sizeof(double), cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        ctx->d2h_bytes += (long long)(npix * sizeof(double));
    }
    return ALN_OK;
}
