// aln_ingest.cuh -- tile conditioning of PixPair::Load (0_GEN/CPixPair.cpp:
// 209-494) on the GPU: LegPolyFlatten (0_GEN/Maths.cpp:962-1085: remove the
// tile's projections on low-order Legendre products, then Normalize), the
// optional DoG band-pass (MakeDoGKernel, CPixPair.cpp:38-83, applied with
// Convolve and re-normalised) and the 2^k box downsampling to MAX1DPIX
// (PixPair::Downsample, CPixPair.cpp:90-110).  Included by aln_corr.cu.
//
// Per-pixel arithmetic follows the reference's operation order with
// explicit round-to-nearest FP64 steps; the sums over all pixels (the
// projection coefficients, mean and sd) run in a fixed blocked order, so a
// tile's numbers repeat exactly and differ from the reference's sequential
// sums by FP64 rounding only.  The DoG convolution is aln_convolve's (FP32
// transforms).
#pragma once

#define ING_THREADS 256
#define ING_BLOCKS 512

// LegPolyCreate (Maths.cpp:962-997) for orders 0..min(order, 6) at n
// samples: P[o * n + s]; orders above 6 stay 0, as there.
__global__ void k_leg_polys(double *P, int order, int n)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
        const double nn = n, n_1 = nn - 1.0;
        const double x = __ddiv_rn(__dsub_rn(__dmul_rn(2.0, (double)s), n_1), nn);
        auto pw = [&](double c, int k) {   // ((c * x) * x) ... k times, left to right
            double r = c;
            for (int q = 0; q < k; ++q)
                r = __dmul_rn(r, x);
            return r;
        };
        for (int o = 0; o <= order; ++o) {
            double v = 0.0;
            switch (o) {
            case 0: v = 1.0; break;
            case 1: v = x; break;
            case 2: v = __dsub_rn(pw(1.5, 2), 0.5); break;
            case 3: v = __dsub_rn(pw(2.5, 3), __dmul_rn(1.5, x)); break;
            case 4:
                v = __dmul_rn(0.125, __dadd_rn(__dsub_rn(pw(35.0, 4), pw(30.0, 2)), 3.0));
                break;
            case 5:
                v = __dmul_rn(0.125,
                              __dadd_rn(__dsub_rn(pw(63.0, 5), pw(70.0, 3)), __dmul_rn(15.0, x)));
                break;
            case 6:
                v = __dmul_rn(0.0625, __dsub_rn(__dadd_rn(__dsub_rn(pw(231.0, 6), pw(315.0, 4)),
                                                          pw(105.0, 2)),
                                                5.0));
                break;
            default: v = 0.0; break;
            }
            P[(long long)o * n + s] = v;
        }
    }
}

__global__ void k_ing_load(const void *src, int dt, long long stride, int w, int h, double *v)
{
    const long long n = (long long)w * h;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long y = i / w, x = i - y * w;
        v[i] = dt == ALN_U8 ? (double)((const uint8_t *)src)[y * stride + x]
                            : (double)((const uint16_t *)src)[y * stride + x];
    }
}

// block partial sums over a contiguous pixel range, in a fixed order
template <typename F>
__device__ __forceinline__ void ing_block_sums(long long n, F term, double *out2)
{
    __shared__ double sh[2][ING_THREADS / 32];
    const long long per = (n + gridDim.x - 1) / gridDim.x;
    const long long b0 = (long long)blockIdx.x * per, b1 = min(n, b0 + per);
    double a = 0.0, b = 0.0;
    for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        double ta, tb;
        term(i, ta, tb);
        a = __dadd_rn(a, ta);
        b = __dadd_rn(b, tb);
    }
    for (int o = 16; o > 0; o >>= 1) {
        a = __dadd_rn(a, __shfl_xor_sync(0xffffffff, a, o));
        b = __dadd_rn(b, __shfl_xor_sync(0xffffffff, b, o));
    }
    if ((threadIdx.x & 31) == 0) {
        sh[0][threadIdx.x >> 5] = a;
        sh[1][threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int q = 0; q < ING_THREADS / 32; ++q) {
            sa = __dadd_rn(sa, sh[0][q]);
            sb = __dadd_rn(sb, sh[1][q]);
        }
        out2[2 * blockIdx.x] = sa;
        out2[2 * blockIdx.x + 1] = sb;
    }
}

// sum F v and F F for F = XP[x] YP[y] (LegPolyFlatten's coefficient sums)
__global__ void __launch_bounds__(ING_THREADS)
k_leg_proj(const double *v, int w, int h, const double *XP, const double *YP, double *part)
{
    ing_block_sums((long long)w * h, [&](long long i, double &ta, double &tb) {
        const long long y = i / w, x = i - y * w;
        const double F = __dmul_rn(XP[x], YP[y]);
        ta = __dmul_rn(F, v[i]);
        tb = __dmul_rn(F, F);
    }, part);
}

// coef = (sum F v) / (sum F F) from the block partials, then v -= coef F
__global__ void k_leg_sub(double *v, int w, int h, const double *XP, const double *YP,
                          const double *part, int nblk)
{
    double c = 0.0, nr = 0.0;
    for (int b = 0; b < nblk; ++b) {
        c = __dadd_rn(c, part[2 * b]);
        nr = __dadd_rn(nr, part[2 * b + 1]);
    }
    const double coef = __ddiv_rn(c, nr);
    const long long n = (long long)w * h;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const long long y = i / w, x = i - y * w;
        v[i] = __dsub_rn(v[i], __dmul_rn(__dmul_rn(coef, XP[x]), YP[y]));
    }
}

__global__ void __launch_bounds__(ING_THREADS) k_ing_stats(const double *v, long long n,
                                                           double *part)
{
    ing_block_sums(n, [&](long long i, double &ta, double &tb) {
        ta = v[i];
        tb = __dmul_rn(v[i], v[i]);
    }, part);
}

// Normalize (Maths.cpp:192-212 with Stats' sample sd, :111-141)
__global__ void k_ing_normalize(double *v, long long n, const double *part, int nblk)
{
    double s = 0.0, s2 = 0.0;
    for (int b = 0; b < nblk; ++b) {
        s = __dadd_rn(s, part[2 * b]);
        s2 = __dadd_rn(s2, part[2 * b + 1]);
    }
    double avg = s, sd = 0.0;
    if (n > 1) {
        avg = __ddiv_rn(avg, (double)n);
        sd = __dsqrt_rn(__ddiv_rn(fmax(__dsub_rn(s2, __dmul_rn(__dmul_rn((double)n, avg), avg)),
                                       0.0),
                                  __dsub_rn((double)n, 1.0)));
    }
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        v[i] = __ddiv_rn(__dsub_rn(v[i], avg), sd);
}

// PixPair::Downsample: box means of scl x scl blocks, dy then dx
__global__ void k_ing_down(const double *src, int wf, double *dst, int ws, int hs, int scl)
{
    const long long n = (long long)ws * hs;
    const double nn = (double)(scl * scl);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const int iy = (int)(i / ws), ix = (int)(i - (long long)iy * ws);
        double sum = 0.0;
        for (int dy = 0; dy < scl; ++dy)
            for (int dx = 0; dx < scl; ++dx)
                sum = __dadd_rn(sum, src[(long long)ix * scl + dx + (long long)wf * (iy * scl + dy)]);
        dst[i] = __ddiv_rn(sum, nn);
    }
}

// MakeDoGKernel (CPixPair.cpp:38-83): one block sums the two Gaussians in
// the reference's order (one thread walks them), then fills the kernel
__global__ void k_dog_kernel(double *K, int r1, int r2)
{
    __shared__ double sums[2];
    const int d = 3 * r2, D = 2 * d + 1;
    const double a1 = (double)(2 * r1 * r1), a2 = (double)(2 * r2 * r2);
    if (threadIdx.x == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int y = -d; y <= d; ++y)
            for (int x = -d; x <= d; ++x) {
                const double R = (double)(x * x + y * y);
                s1 = __dadd_rn(s1, exp(-__ddiv_rn(R, a1)));
                s2 = __dadd_rn(s2, exp(-__ddiv_rn(R, a2)));
            }
        sums[0] = s1;
        sums[1] = s2;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < D * D; i += blockDim.x) {
        const int y = i / D - d, x = i % D - d;
        const double R = (double)(x * x + y * y);
        K[i] = __dsub_rn(__ddiv_rn(exp(-__ddiv_rn(R, a1)), sums[0]),
                         __ddiv_rn(exp(-__ddiv_rn(R, a2)), sums[1]));
    }
}

extern "C" int aln_pixpair_dims(int w, int h, int max1dpix, int *ws, int *hs, int *scl)
{
    if (w < 1 || h < 1 || !ws || !hs || !scl)
        return ALN_ERR_ARG;
    int a = w, b = h, s = 1;
    if (max1dpix > 0)
        while (a > max1dpix || b > max1dpix) {   // CPixPair.cpp:430-435
            a /= 2;
            b /= 2;
            s *= 2;
        }
    *ws = a;
    *hs = b;
    *scl = s;
    return (a * s == w && b * s == h) ? ALN_OK : ALN_NO_PEAK;
}

extern "C" int aln_pixpair_condition(aln_ctx *ctx, const aln_image *tile, int order, int r1,
                                     int r2, int max1dpix, double *vfy, double *aln)
{
    if (!ctx || !tile || !tile->data || !aln || tile->w < 2 || tile->h < 2 ||
        tile->stride < tile->w || tile->dtype != ALN_U8 ||
        order < 0 || (r2 > 0 && (r1 < 1 || r2 < r1)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "pixpair: bad arguments") : ALN_ERR_ARG;
    int ws, hs, scl;
    if (aln_pixpair_dims(tile->w, tile->h, max1dpix, &ws, &hs, &scl) != ALN_OK)
        return set_err(ctx, ALN_ERR_ARG, "pixpair: %d x %d not a multiple of the scale",
                       tile->w, tile->h);
    CK(cudaSetDevice(ctx->device));
    const int w = tile->w, h = tile->h;
    const long long n = (long long)w * h;
    const int dk = r2 > 0 ? 2 * 3 * r2 + 1 : 1;
    const size_t es = dtype_size(tile->dtype);
    const size_t need = al256(n * 8) * 2 + al256((size_t)(order + 1) * (w + h) * 8) +
                        al256(ING_BLOCKS * 2 * 8) + al256((size_t)dk * dk * 8) +
                        al256((size_t)ws * hs * 8) * 2 +
                        (tile->on_device ? 0 : al256((size_t)tile->stride * h * es));
    if (int rc = ensure_ws(ctx, need))
        return rc;
    char *p = ctx->ws;
    double *v = (double *)p;       p += al256(n * 8);
    double *flt = (double *)p;     p += al256(n * 8);
    double *XP = (double *)p;
    double *YP = XP + (size_t)(order + 1) * w;
    p += al256((size_t)(order + 1) * (w + h) * 8);
    double *part = (double *)p;    p += al256(ING_BLOCKS * 2 * 8);
    double *K = (double *)p;       p += al256((size_t)dk * dk * 8);
    double *dvfy = (double *)p;    p += al256((size_t)ws * hs * 8);
    double *daln = (double *)p;    p += al256((size_t)ws * hs * 8);
    cudaStream_t st = ctx->stream;
    const void *src = tile->data;
    if (!tile->on_device) {
        CK(cudaMemcpyAsync(p, tile->data, (size_t)tile->stride * h * es, cudaMemcpyHostToDevice,
                           st));
        ctx->h2d_bytes += (long long)tile->stride * h * es;
        src = p;
    }
    const int gb = (int)std::min<long long>(4096, (n + 255) / 256);
    LAUNCH(ctx, "k_ing_load", k_ing_load, gb, 256, 0, src, tile->dtype, (long long)tile->stride,
           w, h, v);
    // LegPolyFlatten: remove the (xo, yo) projections in the reference's order
    if (order > 0) {
        LAUNCH(ctx, "k_leg_polys", k_leg_polys, (w + 255) / 256, 256, 0, XP, order, w);
        LAUNCH(ctx, "k_leg_polys", k_leg_polys, (h + 255) / 256, 256, 0, YP, order, h);
        for (int xo = 0; xo <= order; ++xo)
            for (int yo = 0; yo <= order; ++yo) {
                if (xo + yo == 0)
                    continue;
                const double *xp = XP + (size_t)xo * w, *yp = YP + (size_t)yo * h;
                LAUNCH(ctx, "k_leg_proj", k_leg_proj, ING_BLOCKS, ING_THREADS, 0, v, w, h, xp, yp,
                       part);
                LAUNCH(ctx, "k_leg_sub", k_leg_sub, gb, 256, 0, v, w, h, xp, yp, part,
                       ING_BLOCKS);
            }
    }
    LAUNCH(ctx, "k_ing_stats", k_ing_stats, ING_BLOCKS, ING_THREADS, 0, v, n, part);
    LAUNCH(ctx, "k_ing_normalize", k_ing_normalize, gb, 256, 0, v, n, part, ING_BLOCKS);
    const double *full_aln = v;
    if (r2 > 0) {
        // the DoG band-pass: the kernel, Convolve (sym, prenorm), Normalize
        LAUNCH(ctx, "k_dog_kernel", k_dog_kernel, 1, 256, 0, K, r1, r2);
        std::vector<double> hv((size_t)n), hf((size_t)n), hk((size_t)dk * dk);
        CK(cudaMemcpyAsync(hv.data(), v, n * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(hk.data(), K, hk.size() * 8, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        // aln_convolve takes host buffers and its own workspace (the same
        // ctx->ws): keep this call's device results safe on the host
        if (int rc = aln_convolve(ctx, hv.data(), w, h, hk.data(), dk, dk, 1, 1, hf.data()))
            return rc;
        if (int rc = ensure_ws(ctx, need))
            return rc;
        p = ctx->ws;
        v = (double *)p;     p += al256(n * 8);
        flt = (double *)p;   p += al256(n * 8);
        p += al256((size_t)(order + 1) * (w + h) * 8);
        part = (double *)p;  p += al256(ING_BLOCKS * 2 * 8);
        p += al256((size_t)dk * dk * 8);
        dvfy = (double *)p;  p += al256((size_t)ws * hs * 8);
        daln = (double *)p;
        CK(cudaMemcpyAsync(v, hv.data(), n * 8, cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(flt, hf.data(), n * 8, cudaMemcpyHostToDevice, st));
        LAUNCH(ctx, "k_ing_stats", k_ing_stats, ING_BLOCKS, ING_THREADS, 0, flt, n, part);
        LAUNCH(ctx, "k_ing_normalize", k_ing_normalize, gb, 256, 0, flt, n, part, ING_BLOCKS);
        full_aln = flt;
    }
    const int gd = (int)std::min<long long>(4096, ((long long)ws * hs + 255) / 256);
    if (scl > 1) {
        LAUNCH(ctx, "k_ing_down", k_ing_down, gd, 256, 0, v, w, dvfy, ws, hs, scl);
        LAUNCH(ctx, "k_ing_down", k_ing_down, gd, 256, 0, full_aln, w, daln, ws, hs, scl);
    } else {
        dvfy = v;
        daln = const_cast<double *>(full_aln);
    }
    CK(cudaGetLastError());
    if (vfy)
        CK(cudaMemcpyAsync(vfy, dvfy, (size_t)ws * hs * 8, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(aln, daln, (size_t)ws * hs * 8, cudaMemcpyDeviceToHost, st));
    ctx->d2h_bytes += (long long)ws * hs * 8 * (vfy ? 2 : 1);
    CK(cudaStreamSynchronize(st));
    prof_collect(ctx);
    return ALN_OK;
}
