// aln_pipeline.cuh -- the batched CorrPatches kernels built on the
// register-resident FFT (aln_fft_reg.cuh).  Included by aln_corr.cu, after
// the device helpers (load_px, sat slots, lag_r, best_merge).
//
//   k3_sat    per 32-column band: warp-local column prefix sums of v, v^2,
//             (v != 0) at the needed rows, per-warp offsets; column totals
//             (k_mean turns them into mu)
//   k2_sat2w  per needed row: add the warp offset, x-prefix -> SAT row
//   k2_rowfft<L>   rows: (v - mu), zero pad, real FFT of length 2L, [kx][y]
//   k2_corrcol<Ny> per column kx: FFT of b's column (or the cached spectrum),
//             FFT of a's column, X2 * conj(X1), inverse FFT, the window's
//             lag rows -> Q[kx][j].  Nothing else leaves the SM.
//   k2_corrseg<NS> the same with the column cut into segments of a's rows
//             (CorrPatches): per segment two NS-point FFTs and the product,
//             summed per column, one inverse
//   k2_lagrow<L>   per lag row: inverse real FFT, r per lag, row argmax
//   k2_lagimg / k2_lagp2i, k_final_img / k_makef / k_fpeak / k_final_p2i:
//             the CorrImages and CorrPatchToImage ends of the pipeline
#pragma once

#include "aln_fft_reg.cuh"
#include "aln_row_layout.cuh"

__device__ __forceinline__ bool int_pixels(int dt) { return dt == ALN_U8 || dt == ALN_U16; }

// s + e += x with the rounding error of the sum kept in e (Knuth's TwoSum;
// explicit round-to-nearest operations, so nothing is contracted or reordered)
__device__ __forceinline__ void two_sum_acc(float &s, float &e, float x)
{
    const float t = __fadd_rn(s, x);
    const float bp = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(x, bp));
    e = __fadd_rn(e, err);
    s = t;
}

// Column prefix sums of v, v^2 and (v != 0) at the rows the lag window needs
// (IntegrateImage's sums, 0_GEN/Correlation.cpp:49-105, restricted to the
// rows IntegralTable will read).  The count table is written for every job
// (zeros without a count rule): skipping its stores changed this walk's
// code and made it 1.7x slower on the montage strips.  grid (ceil(w/32),
// 2*npairs), block (32, SAT_WARPS): each CTA owns 32 columns of one image;
// warp ty owns the rows of segment ty (sat_seg_start) and walks them once, storing its
// local column prefix at the needed rows.  The warps' exclusive offsets per
// column go to segoff[ty][c]; k2_sat2w adds them.  Exact int64 for 8/16-bit
// pixels, FP64 otherwise.  Also writes the column totals (mean shift).
#define SAT_WARPS 16

// Row segments of the column walk, balanced by work: a row costs 1, a row
// the lag window needs (stored) costs 1 + sat_need_cost, and segment g holds
// the rows whose cost position falls in [g, g + 1) * total / SAT_WARPS.  The
// needed rows sit at both ends of the image, so for uint8 pixels equal row
// counts left the first and last warps of a CTA twice as long as the rest,
// which waited at the CTA barrier (stall "barrier" 8.0 per issue on the
// montage strips; weight 2: k3_sat 4.19 -> 3.83 ms per step).  Wider pixels
// sum in 64 bits, so a stored row costs relatively less: weight 2 made the
// uint16 uneven batch's k3_sat 20 % slower, and they keep equal row counts.
// k3_sat and k2_sat2w compute the same map.  A segment spans at most
// 3 h / 16 rows (cost <= 3 h).
__device__ __forceinline__ int sat_need_cost(const PairDev &p, int i)
{
    return p.dt[i] == ALN_U8 ? 2 : 0;
}

__device__ __forceinline__ int sat_cost(const PairDev &p, int i, int y)
{
    const int k = sat_need_cost(p, i);
    int c = y;
    const int lo0 = p.need_lo[i][0], hi0 = p.need_hi[i][0];
    const int lo1 = p.need_lo[i][1], hi1 = p.need_hi[i][1];
    if (hi0 >= lo0)
        c += k * min(max(y - lo0, 0), hi0 - lo0 + 1);
    if (hi1 >= lo1)
        c += k * min(max(y - lo1, 0), hi1 - lo1 + 1);
    return c;
}

// segment of row y (0 <= y < h)
__device__ __forceinline__ int sat_seg_of(const PairDev &p, int i, int y)
{
    const long long total = sat_cost(p, i, p.h[i]);
    return (int)((long long)sat_cost(p, i, y) * SAT_WARPS / max(total, 1LL));
}

// first row of segment g (g = SAT_WARPS: h): the least y with
// cost(y) * SAT_WARPS >= g * total.  need_rows() makes the two needed
// intervals disjoint and ordered (or the second empty), so cost is linear
// with slope 1 before, between and after them and 1 + k inside them, and
// the least y with cost(y) >= C follows piece by piece.  (A binary search
// here -- some 14 dependent steps per warp -- cost the uneven batch's small
// images a fifth of their walk.)
__device__ __forceinline__ int sat_seg_start(const PairDev &p, int i, int g)
{
    const int h = p.h[i], k = sat_need_cost(p, i);
    const long long total = sat_cost(p, i, h);
    const int C = (int)(((long long)g * total + SAT_WARPS - 1) / SAT_WARPS);
    int y;
    if (k == 0) {
        y = C;
    } else {
        const int lo0 = p.need_lo[i][0], lo1 = p.need_lo[i][1];
        const int len0 = max(0, p.need_hi[i][0] - lo0 + 1);
        const int len1 = max(0, p.need_hi[i][1] - lo1 + 1);
        const int k1 = k + 1;
        if (len0 == 0 || C <= lo0)
            y = C;   // (len0 == 0: no needed row at all)
        else if (C <= lo0 + k1 * len0)
            y = lo0 + (C - lo0 + k) / k1;
        else if (len1 == 0 || C <= lo1 + k * len0)
            y = C - k * len0;
        else if (C <= lo1 + k * len0 + k1 * len1)
            y = lo1 + (C - lo1 - k * len0 + k) / k1;
        else
            y = C - k * (len0 + len1);
    }
    return min(max(y, 0), h);
}

// Accumulator of a warp's segment-local sums: 32-bit for uint8 pixels (a
// segment is at most 1536 rows -- h <= 8192 -- so the sums of v and v^2 stay
// below 2^27), the table type otherwise.
template <typename TA, typename PIX>
struct SatAcc {
    typedef TA type;
};
template <>
struct SatAcc<long long, uint8_t> {
    typedef unsigned type;
};

template <typename TA, typename PIX, bool SQ = true>
__device__ __forceinline__ void sat_cols(const PairDev &p, int i, TA *shS, TA *shQ, int *shN)
{
    typedef typename SatAcc<TA, PIX>::type AC;
    const int w = p.w[i];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int c = blockIdx.x * 32 + tx;
    const bool cok = c < w;
    const int y0 = sat_seg_start(p, i, ty), y1 = sat_seg_start(p, i, ty + 1);
    const PIX *img = (const PIX *)p.img[i];
    const long long st = p.stride[i];
    const int lo0 = p.need_lo[i][0], hi0 = p.need_hi[i][0];
    const int lo1 = p.need_lo[i][1], hi1 = p.need_hi[i][1];
    const int len0 = hi0 - lo0 + 1;
    const bool want_n = p.cnt_kind == ALN_CNT_GT;
    TA *__restrict__ S = (TA *)p.satS[i];
    TA *__restrict__ Q = (TA *)p.satQ[i];
    int *__restrict__ N = p.satN[i];
    AC s = 0, q = 0;
    int n = 0;
    if (cok) {
        const PIX *__restrict__ col = img + c;
        // walk [y0, y1) as store-free runs (loads batch freely) separated by
        // the needed rows, where the running prefix is stored
        int y = y0;
        while (y < y1) {
            int stop = y1;   // next needed row at or after y
            if (hi0 >= lo0 && hi0 >= y)
                stop = min(stop, max(lo0, y));
            if (hi1 >= lo1 && hi1 >= y)
                stop = min(stop, max(lo1, y));
#pragma unroll 8
            for (; y < stop; ++y) {
                const AC v = (AC)__ldg(&col[y * st]);
                if (SQ) {
                    s += v;
                    q += v * v;
                }
                if (want_n)
                    n += (v != 0);
            }
            if (y >= y1)
                break;
            // needed run: rows y .. end of its interval (within the warp's rows)
            const bool first = y >= lo0 && y <= hi0;
            const int rend = min(y1 - 1, first ? hi0 : hi1);
            const long long base = first ? (long long)(y - lo0) : (long long)(len0 + y - lo1);
            for (long long o = base * w + c; y <= rend; ++y, o += w) {
                const AC v = (AC)__ldg(&col[y * st]);
                if (SQ) {
                    s += v;
                    q += v * v;
                    S[o] = (TA)s;
                    Q[o] = (TA)q;
                }
                if (want_n)
                    n += (v != 0);
                N[o] = n;
            }
        }
    }
    shS[ty * 32 + tx] = (TA)s;
    shQ[ty * 32 + tx] = (TA)q;
    shN[ty * 32 + tx] = n;
    __syncthreads();
    if (!cok)
        return;
    TA os = 0, oq = 0;
    int on = 0;
    for (int g = 0; g < ty; ++g) {
        os += shS[g * 32 + tx];
        oq += shQ[g * 32 + tx];
        on += shN[g * 32 + tx];
    }
    if (SQ) {
        ((TA *)p.segS[i])[ty * w + c] = os;
        ((TA *)p.segQ[i])[ty * w + c] = oq;
        if (ty == SAT_WARPS - 1)
            p.colsum[i][c] = (double)(os + (TA)s);
    }
    p.segN[i][ty * w + c] = on;
}

__global__ void k3_sat(PairDev *pairs)
{
    __shared__ long long shS[32 * SAT_WARPS], shQ[32 * SAT_WARPS];
    __shared__ int shN[32 * SAT_WARPS];
    const PairDev &p = pairs[blockIdx.y >> 1];
    const int i = blockIdx.y & 1;
    if (p.status != 0 || blockIdx.x * 32 >= p.w[i])
        return;
    if (p.sat_nonly) {   // counts only (CorrImagesS without a mincor)
        if (p.cnt_kind != ALN_CNT_GT)
            return;
        switch (p.dt[i]) {
        case ALN_U8: sat_cols<long long, uint8_t, false>(p, i, shS, shQ, shN); break;
        case ALN_U16: sat_cols<long long, uint16_t, false>(p, i, shS, shQ, shN); break;
        case ALN_F32: sat_cols<double, float, false>(p, i, (double *)shS, (double *)shQ, shN); break;
        default: sat_cols<double, double, false>(p, i, (double *)shS, (double *)shQ, shN); break;
        }
        return;
    }
    switch (p.dt[i]) {
    case ALN_U8:
        sat_cols<long long, uint8_t>(p, i, shS, shQ, shN);
        break;
    case ALN_U16:
        sat_cols<long long, uint16_t>(p, i, shS, shQ, shN);
        break;
    case ALN_F32:
        sat_cols<double, float>(p, i, (double *)shS, (double *)shQ, shN);
        break;
    default:
        sat_cols<double, double>(p, i, (double *)shS, (double *)shQ, shN);
        break;
    }
}

// ---------------------------------------------------------------------------
// transposed copies of wide images (jobs solved in the transposed frame)
// ---------------------------------------------------------------------------

__device__ __forceinline__ unsigned long long load_bits(const char *p, int es, long long idx)
{
    switch (es) {
    case 1: return ((const uint8_t *)p)[idx];
    case 2: return ((const uint16_t *)p)[idx];
    case 4: return ((const uint32_t *)p)[idx];
    default: return ((const unsigned long long *)p)[idx];
    }
}

__device__ __forceinline__ void store_bits(char *p, int es, long long idx, unsigned long long v)
{
    switch (es) {
    case 1: ((uint8_t *)p)[idx] = (uint8_t)v; break;
    case 2: ((uint16_t *)p)[idx] = (uint16_t)v; break;
    case 4: ((uint32_t *)p)[idx] = (uint32_t)v; break;
    default: ((unsigned long long *)p)[idx] = v; break;
    }
}

// grid (ceil(max caller w / (32 TR_TILES)), ceil(max caller h / 32),
// 2*npairs), block (32, 8): frame pixel (xf, yf) = caller pixel (yf, xf).
// uint8 images use 32 x 128 tiles (blockIdx.x then counts 128 TR_TILES
// columns; a launch whose transposed images are all uint8 has grid x =
// ceil(max caller w / (128 TR_TILES))).  Each CTA moves TR_TILES tiles side
// by side: a 4 KB tile per CTA left the montage strips' transposes bound by
// block scheduling (hundreds of thousands of CTAs per step).
#define TR_TILES 4
__global__ void k_transpose(PairDev *pairs)
{
    __shared__ unsigned long long tile[32][33];
    PairDev &p = pairs[blockIdx.z >> 1];
    const int i = blockIdx.z & 1;
    if (p.status != 0 || !p.transposed)
        return;
    const int sw = p.h[i], sh = p.w[i];   // caller's width and height
    const int y0 = blockIdx.y * 32;
    if (y0 >= sh)
        return;
    const int es = p.dt[i] == ALN_U8 ? 1 : p.dt[i] == ALN_U16 ? 2 : p.dt[i] == ALN_F32 ? 4 : 8;
    const char *src = (const char *)p.src_img[i];
    const long long sst = p.src_stride[i];
    if (es == 1) {
        // uint8: 32 x 128 tiles
        unsigned char(*t8)[132] = (unsigned char(*)[132])tile;
        unsigned char *dst = (unsigned char *)p.img[i];
        const long long dstr = p.stride[i];
        const int tid = threadIdx.y * 32 + threadIdx.x;
        // 4-byte loads where the caller's rows allow them (4-byte aligned
        // base and stride, the whole word inside the row)
        const bool vec = (((uintptr_t)src | (uintptr_t)sst) & 3) == 0;
        for (int kt = 0; kt < TR_TILES; ++kt) {
            const int xb0 = (blockIdx.x * TR_TILES + kt) * 128;
            if (xb0 >= sw)
                break;   // uniform over the CTA
            if (kt > 0)
                __syncthreads();   // the previous tile's reads are done
            for (int rr = threadIdx.y; rr < 32; rr += 8) {
                const int yy = y0 + rr;
                const int xq = xb0 + 4 * threadIdx.x;
                if (vec && yy < sh && xq + 3 < sw) {
                    *(unsigned int *)&t8[rr][4 * threadIdx.x] =
                        *(const unsigned int *)(src + yy * sst + xq);
                    continue;
                }
                for (int m = 0; m < 4; ++m) {
                    const int x = xq + m;
                    t8[rr][4 * threadIdx.x + m] =
                        (yy < sh && x < sw) ? (unsigned char)src[yy * sst + x] : 0;
                }
            }
            __syncthreads();
            for (int e = tid; e < 128 * 8; e += 256) {
                const int j = e >> 3, wq = e & 7;
                const int xs = xb0 + j, ys = y0 + 4 * wq;
                if (xs >= sw || ys >= sh)
                    continue;
                if (ys + 3 < sh && (dstr & 3) == 0) {
                    const unsigned int word = (unsigned int)t8[4 * wq][j] |
                                              ((unsigned int)t8[4 * wq + 1][j] << 8) |
                                              ((unsigned int)t8[4 * wq + 2][j] << 16) |
                                              ((unsigned int)t8[4 * wq + 3][j] << 24);
                    *(unsigned int *)(dst + xs * dstr + ys) = word;
                } else {
                    for (int m = 0; m < 4 && ys + m < sh; ++m)
                        dst[xs * dstr + ys + m] = t8[4 * wq + m][j];
                }
            }
        }
        return;
    }
    char *dst = (char *)p.img[i];
    const long long dstr = p.stride[i];
    for (int kt = 0; kt < TR_TILES; ++kt) {
        const int x0 = (blockIdx.x * TR_TILES + kt) * 32;
        if (x0 >= sw)
            break;   // uniform over the CTA
        if (kt > 0)
            __syncthreads();
        for (int yy = threadIdx.y; yy < 32; yy += 8) {
            const int y = y0 + yy, x = x0 + threadIdx.x;
            if (y < sh && x < sw)
                tile[yy][threadIdx.x] = load_bits(src, es, y * sst + x);
        }
        __syncthreads();
        for (int xx = threadIdx.y; xx < 32; xx += 8) {
            const int x = x0 + xx, y = y0 + threadIdx.x;
            if (x < sw && y < sh)
                store_bits(dst, es, x * dstr + y, tile[threadIdx.x][xx]);
        }
    }
}

// The row pass of the summed-area tables: per needed row, add the warp
// segment offsets of k3_sat and take the x-prefix.  One warp per row (no
// block-wide synchronisation, so a CTA carries eight rows and small images
// do not pay one CTA per row); the warp walks the row 32 columns at a time,
// lane l on column c0 + l: coalesced loads and stores, an inclusive shuffle
// scan per 32 columns and a carry between them.  (On the uneven uint16 batch
// this took 16 ms per 20000 pairs where a CTA-per-row scan on the rows wider
// than 512 columns took 29 ms.)

template <typename TA>
__device__ __forceinline__ TA warp_incl_scan(TA v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const TA u = __shfl_up_sync(0xffffffff, v, o);
        if (lane >= o)
            v += u;
    }
    return v;
}

template <typename TA, bool SQ>
__device__ __forceinline__ void sat2_row_any(const PairDev &p, int i, int slot, int y, TA *S,
                                             TA *Q, int lane)
{
    const int w = p.w[i];
    const int seg = sat_seg_of(p, i, y);
    const TA *__restrict__ oS = (const TA *)p.segS[i] + (long long)seg * w;
    const TA *__restrict__ oQ = (const TA *)p.segQ[i] + (long long)seg * w;
    const int *__restrict__ oN = p.segN[i] + (long long)seg * w;
    TA *__restrict__ rS = S + (long long)slot * w;
    TA *__restrict__ rQ = Q + (long long)slot * w;
    int *__restrict__ rN = p.satN[i] + (long long)slot * w;
    // the count table only where a count rule reads it (uniform per job)
    const bool want_n = p.cnt_kind == ALN_CNT_GT;
    TA cs = 0, cq = 0;
    int cn = 0;
    for (int c0 = 0; c0 < w; c0 += 32) {
        const int c = c0 + lane;
        const bool ok = c < w;
        TA vs = 0, vq = 0;
        int vn = 0;
        if (ok) {
            if (SQ) {
                vs = rS[c] + oS[c];
                vq = rQ[c] + oQ[c];
            }
            if (want_n)
                vn = rN[c] + oN[c];
        }
        if (SQ) {
            vs = warp_incl_scan(vs, lane) + cs;
            vq = warp_incl_scan(vq, lane) + cq;
        }
        if (want_n)
            vn = warp_incl_scan(vn, lane) + cn;
        if (ok) {
            if (SQ) {
                rS[c] = vs;
                rQ[c] = vq;
            }
            if (want_n)
                rN[c] = vn;
        }
        if (SQ) {
            cs = __shfl_sync(0xffffffff, vs, 31);
            cq = __shfl_sync(0xffffffff, vq, 31);
        }
        if (want_n)
            cn = __shfl_sync(0xffffffff, vn, 31);
    }
}

// Counts-only form (CorrImagesS without a mincor): K rounds of 32 columns
// per pass, their loads issued together (one memory latency per pass), then
// scanned in registers in column order.  (Measured on the thumbnail sweep:
// 52 ms per 1024-pair step against 132 ms one round at a time; the same
// batching of the int64 S and Q tables needed 91 registers and ran slower.)
__device__ __forceinline__ void sat2_row_counts(const PairDev &p, int i, int slot, int y,
                                                int lane)
{
    constexpr int K = 8;
    const int w = p.w[i];
    const int seg = sat_seg_of(p, i, y);
    const int *__restrict__ oN = p.segN[i] + (long long)seg * w;
    int *__restrict__ rN = p.satN[i] + (long long)slot * w;
    int cn = 0;
    for (int cb = 0; cb < w; cb += 32 * K) {
        int vn[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int c = cb + 32 * k + lane;
            vn[k] = c < w ? rN[c] + oN[c] : 0;
        }
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if (cb + 32 * k >= w)
                break;   // uniform over the warp
            vn[k] = warp_incl_scan(vn[k], lane) + cn;
            cn = __shfl_sync(0xffffffff, vn[k], 31);
            const int c = cb + 32 * k + lane;
            if (c < w)
                rN[c] = vn[k];
        }
    }
}

// grid (ceil(maxslots / 8), 2, npairs), block 256: warp k takes slot 8*bx + k.
// NONLY: the form launched for chunks of counts-only jobs (its registers are
// not sized for the int64 tables).
template <bool NONLY>
__global__ void k2_sat2w(PairDev *pairs)
{
    const PairDev &p = pairs[blockIdx.z];
    const int i = blockIdx.y;
    const int slot = blockIdx.x * 8 + (threadIdx.x >> 5);
    if (p.status != 0 || slot >= nslots(p, i))
        return;
    const int len0 = p.need_hi[i][0] - p.need_lo[i][0] + 1;
    const int y = slot < len0 ? p.need_lo[i][0] + slot : p.need_lo[i][1] + slot - len0;
    const int lane = threadIdx.x & 31;
    if (NONLY) {
        if (p.sat_nonly)
            sat2_row_counts(p, i, slot, y, lane);
        else
            sat2_row_any<long long, false>(p, i, slot, y, (long long *)p.satS[i],
                                           (long long *)p.satQ[i], lane);
    } else if (p.sat_nonly)
        sat2_row_any<long long, false>(p, i, slot, y, (long long *)p.satS[i],
                                       (long long *)p.satQ[i], lane);
    else if (int_pixels(p.dt[i]))
        sat2_row_any<long long, true>(p, i, slot, y, (long long *)p.satS[i],
                                      (long long *)p.satQ[i], lane);
    else
        sat2_row_any<double, true>(p, i, slot, y, p.satS[i], p.satQ[i], lane);
}

// ---------------------------------------------------------------------------
// forward rows
// ---------------------------------------------------------------------------

// launch shape and shared-memory layout: aln_row_layout.cuh

// Each team of T threads (rowfft_T<L>()) transforms one row.  G =
// blockDim.x / T rows per CTA.
template <int L>
__global__ void __launch_bounds__(rowfft_threads(rowfft_T<L>()), rowfft_minb<L>())
k2_rowfft(PairDev *pairs, const float2 *__restrict__ tw, int only_img, const int *sel)
{
    using F = RowFFT<L>;
    constexpr int V = F::V, T = F::T;
    constexpr int G = rowfft_threads(T) / T;
    extern __shared__ float2 smem[];
    // sel: the jobs of this launch are pairs[sel[z]] (spectrum-cache fills)
    PairDev &p = pairs[sel ? sel[blockIdx.z] : blockIdx.z];
    const int i = only_img >= 0 ? only_img : blockIdx.y;
    if (p.status != 0 || (i == 1 && p.b_cached && !sel))
        return;
    const int team = threadIdx.x / T, t = threadIdx.x - team * T;
    const int h = p.h[i], w = p.w[i], dt = p.dt[i];
    const int y0 = blockIdx.x * G;
    if (y0 >= h)
        return;
    const int y = y0 + team;
    float2 *sm = smem + rowfft_base<L>(team);
    const void *img = p.img[i];
    const long long st = p.stride[i];
    float2 v[V];
    if (dt == ALN_U8 || dt == ALN_U16) {
        // integer pixels, integer shift: exact before the conversion.  The
        // row is staged in shared memory with 16-byte loads from its
        // 16-byte-aligned start (an aligned 16-byte block that holds a byte
        // of the row never leaves the row's allocation page).
        const int es = dt == ALN_U8 ? 1 : 2;
        const int mu = (int)p.mu[i];
        // the region's first 16-byte boundary (at most 8 bytes in): the row's
        // <= 4L + 30 staged bytes end inside the region (rowfft_pitch)
        unsigned char *sb = (unsigned char *)(((uintptr_t)sm + 15) & ~(uintptr_t)15);
        int off = 0;
        if (y < h) {
            const unsigned char *base = (const unsigned char *)img + (long long)y * st * es;
            const uintptr_t a0 = (uintptr_t)base & ~(uintptr_t)15;
            off = (int)((uintptr_t)base - a0);
            const int nvec = (off + w * es + 15) >> 4;
            const uint4 *src = (const uint4 *)a0;
            for (int k = t; k < nvec; k += T)
                ((uint4 *)sb)[k] = src[k];
        }
        team_sync<T>(team);   // each team reads back its own row only
        const unsigned char *rb8 = sb + off;
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const int n = F::in_idx(t, q);
            float2 z = make_float2(0.f, 0.f);
            if (y < h) {
                const int xa = 2 * n, xb = 2 * n + 1;
                if (xa < w)
                    z.x = (float)((es == 1 ? (int)rb8[xa] : (int)((const uint16_t *)rb8)[xa]) - mu);
                if (xb < w)
                    z.y = (float)((es == 1 ? (int)rb8[xb] : (int)((const uint16_t *)rb8)[xb]) - mu);
            }
            v[q] = z;
        }
    } else {
        const double mu = p.mu[i];
#pragma unroll
        for (int q = 0; q < V; ++q) {
            const int n = F::in_idx(t, q);
            float2 z = make_float2(0.f, 0.f);
            if (y < h) {
                const int xa = 2 * n, xb = 2 * n + 1;
                if (xa < w)
                    z.x = (float)(load_px(img, dt, y * st + xa) - mu);
                if (xb < w)
                    z.y = (float)(load_px(img, dt, y * st + xb) - mu);
            }
            v[q] = z;
        }
    }
    F::run_team(v, sm, t, tw, team);
    // split the half-length transform into the N/2+1 bins of the real row
    __syncthreads();
#pragma unroll
    for (int q = 0; q < V; ++q)
        sm[F::out_idx(t, q)] = v[q];
    __syncthreads();
    // bins for (kx, row) with row fastest: coalesced [kx][y] stores.  Bin kx
    // needs Z[kx] and conj(Z[L - kx]) (indices mod L), bin L - kx the same
    // two values swapped: one item makes both (kx = 0..L/2; L is even).  The
    // CTA has G * T threads, so thread x always takes row x % G and bins
    // kx = x / G + m T: its row's region and store pointers are set once.
    constexpr int THR = G * T;
    const int rr = threadIdx.x % G;
    if (rr >= min(G, h - y0))
        return;
    const float2 *Z = smem + rowfft_base<L>(rr);
    const long long Ts = p.Ts[i];
    const int kx0 = threadIdx.x / G;
    float2 *lo = p.T[i] + y0 + rr + kx0 * Ts;          // bin kx
    float2 *hi = p.T[i] + y0 + rr + (L - kx0) * Ts;    // bin L - kx
    const float2 *twk = tw + tw_base(2 * L) + 2 * L;   // exp(-2 pi i k / 2L) at twk[k]
    for (int kx = kx0; kx <= L / 2; kx += THR / G, lo += (THR / G) * Ts, hi -= (THR / G) * Ts) {
        const float2 A = Z[kx];
        const float2 B = Z[kx == 0 ? 0 : L - kx];
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int k = hh ? L - kx : kx;
            if (hh && k == kx)
                break;   // kx = L/2: one bin
            const float2 a = hh ? B : A;
            const float2 b = cconj(hh ? A : B);
            const float2 ev = make_float2(0.5f * (a.x + b.x), 0.5f * (a.y + b.y));
            const float2 dd = make_float2(0.5f * (a.x - b.x), 0.5f * (a.y - b.y));
            const float2 o = make_float2(dd.y, -dd.x);
            const float2 wv = __ldg(&twk[k]);
            *(hh ? hi : lo) = cadd(ev, cmul(o, wv));
        }
    }
}

// ---------------------------------------------------------------------------
// columns: forward b and a, product, inverse, window rows
// ---------------------------------------------------------------------------

// VAR: 1 = CorrPatches chunks (plain inverse only, no low-pass, no
// whitening), 2 = CorrImagesS without a mincor (whitened inverse only),
// 0 = any job; the specialised forms are compiled without the other jobs'
// branches.
// Per-thread radix of the column FFTs, per kernel form.  (Measured on the
// montage batch: 8 points per thread at 4096 -- twice the threads per
// column -- ran 45% slower than 16, so every form uses fft_radix.)
template <int NY, int VAR>
__host__ __device__ constexpr int corrcol_radix()
{
    return fft_radix(NY);
}

template <int NY, int VAR>
__host__ __device__ constexpr int corrcol_threads()
{
    return NY / corrcol_radix<NY, VAR>() >= 256 ? NY / corrcol_radix<NY, VAR>() : 256;
}

// Occupancy: the CorrPatches form keeps 2 CTAs per SM; the S-only form runs
// 3 (80 registers, small spills, faster).
template <int NY, int VAR>
__global__ void __launch_bounds__(corrcol_threads<NY, VAR>(),
                                  (NY >= 8192 || corrcol_threads<NY, VAR>() > 256) ? 1
                                                                                 : (VAR == 2 ? 3 : 2))
k2_corrcol(PairDev *pairs, const float2 *__restrict__ tw, int use_cached_b)
{
    constexpr bool PLAIN = VAR == 1, SONLY = VAR == 2;
    using FF = RegFFT<NY, -1, corrcol_radix<NY, VAR>()>;
    using FI = RegFFT<NY, +1, corrcol_radix<NY, VAR>()>;
    static_assert(FI::SMEM <= FF::SMEM, "the inverse runs in the forward transform's buffer");
    constexpr int R = FF::R, T = FF::T;
    extern __shared__ float2 smem[];
    PairDev &p = pairs[blockIdx.y];
    if (p.status != 0)
        return;
    const int L1 = (p.Nx >> 1) + 1;
    const int G = blockDim.x / T;
    const int team = threadIdx.x / T, t = threadIdx.x - team * T;
    const int kx = blockIdx.x * G + team;
    const bool live = kx < L1;
    if (blockIdx.x * G >= L1)
        return;
    float2 *sm = smem + team * FF::SMEM;
    float2 *sb = smem + G * FF::SMEM + team * NY;   // b's spectrum, this team's own slots
    const int kxc = live ? kx : L1 - 1;   // idle teams compute a copy, store nothing
    float2 va[R];
    {
        float2 vb[R];
        if (use_cached_b || p.b_cached) {
#pragma unroll
            for (int r = 0; r < R; ++r)
                vb[r] = p.X2[(long long)kxc * NY + t + r * T];
        } else {
            const float2 *Tb = p.T[1] + (long long)kxc * p.Ts[1];
            const int hb = p.h[1];
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int y = t + r * T;
                vb[r] = y < hb ? Tb[y] : make_float2(0.f, 0.f);
            }
            FF::run_team(vb, sm, t, tw, team);
        }
#pragma unroll
        for (int r = 0; r < R; ++r)
            sb[r * T + t] = vb[r];
    }
    {
        const float2 *Ta = p.T[0] + (long long)kxc * p.Ts[0];
        const int ha = p.h[0];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int y = t + r * T;
            va[r] = y < ha ? Ta[y] : make_float2(0.f, 0.f);
        }
    }
    FF::run_team(va, sm, t, tw, team);
#pragma unroll
    for (int r = 0; r < R; ++r)
        va[r] = cmulc(sb[r * T + t], va[r]);   // X2 * conj(X1)
    const bool is_p2i = VAR == 0 && p.mode == JOB_P2I;
    if (is_p2i && p.p2i_filter) {
        // CorrPatchToImage's low-pass (0_GEN/Correlation.cpp:1255-1283): the
        // reference names the row index "x" (wrapped) and the column "y"
#pragma unroll
        for (int r = 0; r < R; ++r) {
            int x = t + r * T;
            if (x >= NY / 2)
                x -= NY;
            const double rad2 = ((double)x * x + (double)kxc * kxc) / 10000.0;
            const float filt = rad2 > 10.0 ? 0.f : (float)exp(-rad2);
            va[r] = make_float2(va[r].x * filt, va[r].y * filt);
        }
    }
    // CorrPatches / CorrImagesR need the plain inverse; CorrImagesS the inverse
    // of the whitened product P / sqrt(|P|) (0_GEN/Correlation.cpp:2311-2317)
    const bool want_r = PLAIN || (!SONLY && (p.mode == JOB_PATCHES || is_p2i || p.want_r));
    const bool want_s = SONLY || (!PLAIN && p.want_s != 0);
    if (want_r && want_s) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            sb[r * T + t] = va[r];
    }
    const int Wy = p.yhi - p.ylo + 1;
    const int nnegy = p.h[0] - 1;
    if (want_r) {
        FI::run_team(va, sm, t, tw, team);
        if (live && is_p2i) {   // every storage row, in storage order
            float2 *Q = p.Q + (long long)kx * NY;
#pragma unroll
            for (int r = 0; r < R; ++r)
                Q[t + r * T] = va[r];
        } else if (live) {
            float2 *Q = p.Q + (long long)kx * Wy;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ys = t + r * T;
                const int y = ys >= NY - nnegy ? ys - NY : ys;
                if (y >= p.ylo && y <= p.yhi)
                    Q[y - p.ylo] = va[r];
            }
        }
    }
    if (want_s) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
            float2 v = want_r ? sb[r * T + t] : va[r];
            const float m = hypotf(v.x, v.y);
            if (m > 1e-10f) {
                const float q = 1.0f / sqrtf(m);
                v = make_float2(v.x * q, v.y * q);
            }
            va[r] = v;
        }
        FI::run_team(va, sm, t, tw, team);
        if (live) {
            float2 *Q = (want_r ? p.Q2 : p.Q) + (long long)kx * Wy;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const int ys = t + r * T;
                const int y = ys >= NY - nnegy ? ys - NY : ys;
                if (y >= p.ylo && y <= p.yhi)
                    Q[y - p.ylo] = va[r];
            }
        }
    }
}

// CorrPatches columns with the long axis cut into segments.  Only the Wy lag
// rows [ylo, yhi] are read, so for column kx
//   C[ylo + e] = sum_y conj(A[y]) B[y + ylo + e],   e in [0, Wy),
// splits over segments of a's rows, y = s*seg_len + j (j < seg_len): segment
// s pairs a's rows [s*seg_len, +seg_len) with b's rows [s*seg_len + ylo,
// +seg_len + Wy - 1), and NS >= seg_len + Wy - 1 makes its circular
// correlation on NS points the linear one at e in [0, Wy).  The segments'
// spectral products are summed (one accumulator per column) and inverted
// once: 2 nseg + 1 transforms of NS points instead of 3 of Ny.  Each thread
// keeps its accumulator and parked a-spectrum points to itself, in
// registers or its own shared-memory slots (corrseg_regs; no exchange).
// Output: Q[kx][e], as k2_corrcol; the column transform length the lag
// kernel normalises by is NS (p.Ny).
// Per-thread radix of the segment transforms.  Measured on the montage
// strips (6 segments of 512 points, accumulator then in shared memory):
// radix 8 at 3 CTAs per SM ran 25% faster than radix 16 at 2 (spills, low
// occupancy); at 1024 and 2048 points radix 16 stays ahead.
template <int NS>
__host__ __device__ constexpr int corrseg_radix()
{
    return NS == 512 ? 8 : fft_radix(NS);
}

// Where a thread keeps its parked a-spectrum points and the column's
// accumulated product: registers at radix <= 8 (each thread owns the same R
// points throughout; a third fewer shared-memory wavefronts than parking
// them in shared memory, 2 CTAs per SM at 128 registers instead of 3 at 80:
// k2_corrseg<512> 10.18 -> 9.84 ms per montage step), shared memory at
// radix 16 (32 more points per thread spilled 260-280 bytes).
template <int NS>
__host__ __device__ constexpr bool corrseg_regs()
{
    return corrseg_radix<NS>() <= 8;
}

template <int NS>
__global__ void __launch_bounds__(256, 2)
k2_corrseg(PairDev *pairs, const float2 *__restrict__ tw)
{
    using FF = RegFFT<NS, -1, corrseg_radix<NS>()>;
    using FI = RegFFT<NS, +1, corrseg_radix<NS>()>;
    static_assert(FI::SMEM <= FF::SMEM, "the inverse runs in the forward transform's buffer");
    constexpr int R = FF::R, T = FF::T;
    extern __shared__ float2 smem[];
    const PairDev &p = pairs[blockIdx.y];
    if (p.status != 0)
        return;
    const int L1 = (p.Nx >> 1) + 1;
    const int G = blockDim.x / T;
    const int team = threadIdx.x / T, t = threadIdx.x - team * T;
    const int kx = blockIdx.x * G + team;
    if (blockIdx.x * G >= L1)
        return;
    const bool live = kx < L1;
    const int kxc = live ? kx : L1 - 1;   // idle teams compute a copy, store nothing
    float2 *sm = smem + team * FF::SMEM;
    constexpr bool REGS = corrseg_regs<NS>();
    float2 parkr[REGS ? R : 1], accr[REGS ? R : 1];
    float2 *park = REGS ? nullptr : smem + G * FF::SMEM + team * (2 * NS);
    float2 *acc = REGS ? nullptr : park + NS;
    const float2 *Ta = p.T[0] + (long long)kxc * p.Ts[0];
    const float2 *Tb = p.T[1] + (long long)kxc * p.Ts[1];
    const int ha = p.h[0], hb = p.h[1];
    const int B = p.seg_len, nseg = p.nseg, ylo = p.ylo;
    const int Wy = p.yhi - p.ylo + 1;
    const int lb = B + Wy - 1;
    for (int s = 0; s < nseg; ++s) {
        const int y0 = s * B;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int j = t + r * T, y = y0 + j;
            v[r] = (j < B && y < ha) ? Ta[y] : make_float2(0.f, 0.f);
        }
        FF::run_team(v, sm, t, tw, team);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if constexpr (REGS)
                parkr[r] = v[r];
            else
                park[r * T + t] = v[r];
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int j = t + r * T, y = y0 + ylo + j;
            v[r] = (j < lb && y >= 0 && y < hb) ? Tb[y] : make_float2(0.f, 0.f);
        }
        FF::run_team(v, sm, t, tw, team);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            if constexpr (REGS) {
                const float2 q = cmulc(v[r], parkr[r]);   // X2 * conj(X1)
                accr[r] = s == 0 ? q : cadd(accr[r], q);
            } else {
                const float2 q = cmulc(v[r], park[r * T + t]);
                acc[r * T + t] = s == 0 ? q : cadd(acc[r * T + t], q);
            }
        }
    }
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        if constexpr (REGS)
            v[r] = accr[r];
        else
            v[r] = acc[r * T + t];
    }
    FI::run_team(v, sm, t, tw, team);
    if (live) {
        float2 *Q = p.Q + (long long)kx * Wy;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int e = t + r * T;
            if (e < Wy)
                Q[e] = v[r];
        }
    }
}

// Spectrum of image b alone into X2 (a cache entry): per column kx, the
// column FFT of b's row-pass output, stored as k2_corrcol reads a cached
// spectrum.  The same RegFFT code as the fused path, so the cached and the
// recomputed spectra are the same numbers.  grid (ceil((L+1)/G), nsel): the
// jobs are pairs[sel[y]].
// RAD: the per-thread radix of the column kernel that reads the entry (the
// same FFT code, so the cached and the recomputed spectra are the same
// numbers).
template <int NY, int RAD>
__global__ void __launch_bounds__(NY / RAD >= 256 ? NY / RAD : 256)
k2_colspec(PairDev *pairs, const float2 *__restrict__ tw, const int *sel)
{
    using FF = RegFFT<NY, -1, RAD>;
    constexpr int R = FF::R, T = FF::T;
    extern __shared__ float2 smem[];
    PairDev &p = pairs[sel[blockIdx.y]];
    if (p.status != 0)
        return;
    const int L1 = (p.Nx >> 1) + 1;
    const int G = blockDim.x / T;
    const int team = threadIdx.x / T, t = threadIdx.x - team * T;
    const int kx = blockIdx.x * G + team;
    if (blockIdx.x * G >= L1)
        return;
    float2 *sm = smem + team * FF::SMEM;
    const int kxc = kx < L1 ? kx : L1 - 1;
    const float2 *Tb = p.T[1] + (long long)kxc * p.Ts[1];
    const int hb = p.h[1];
    float2 vb[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int y = t + r * T;
        vb[r] = y < hb ? Tb[y] : make_float2(0.f, 0.f);
    }
    FF::run(vb, sm, t, tw);
    if (kx < L1) {
#pragma unroll
        for (int r = 0; r < R; ++r)
            p.X2[(long long)kx * NY + t + r * T] = vb[r];
    }
}

// ---------------------------------------------------------------------------
// lag rows
// ---------------------------------------------------------------------------
// The job's descriptor in shared memory: the lag scans read many of its
// fields inside loops that also store through its pointers; from global
// memory each read would be a fresh L1 round trip (the compiler cannot keep
// them across the stores).  All threads of the CTA must call this.
__device__ __forceinline__ const PairDev &stage_job(const PairDev *pairs, int j, PairDev &sp)
{
    const int *src = (const int *)(pairs + j);
    int *dst = (int *)&sp;
    for (int i = threadIdx.x; i < (int)(sizeof(PairDev) / sizeof(int)); i += blockDim.x)
        dst[i] = src[i];
    __syncthreads();
    return sp;
}


// The L+1 spectrum bins of the CTA's G lag rows j0 .. j0+G-1 (Q is [kx][j],
// stride Wy; rows past Wy repeat the last one) into the teams' shared rows
// (team g at base + g * stride), loaded by the whole CTA so that a warp's
// loads cover whole 8-row segments of Q (G consecutive j per kx); four loads
// per thread are in flight before their stores.
// G: rows per CTA (blockDim.x / T).  The copies are asynchronous
// (cp.async, 8 bytes each, global -> shared without registers), so every
// element a thread moves is in flight at once; the loads through registers
// this replaces kept four per thread in flight, and the lag kernels waited on
// them (long-scoreboard stalls, k2_lagimg 33 % warps active).  The caller's
// __syncthreads after the call publishes the rows to the CTA.
__device__ __forceinline__ void cp_async8(void *dst_shared, const void *src_global)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst_shared);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src_global) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

template <int L, int T, int G = (T >= 256 ? T : 256) / T>
__device__ __forceinline__ void load_lag_rows(float2 *base, int stride,
                                              const float2 *__restrict__ Q, int Wy, int j0)
{
    constexpr int TOT = (L + 1) * G;
    for (int e = threadIdx.x; e < TOT; e += blockDim.x) {
        const int kx = e / G, g = e - kx * G;
        cp_async8(&base[g * stride + padi(kx)], &Q[(long long)kx * Wy + min(j0 + g, Wy - 1)]);
    }
    cp_async_wait_all();
}

// Threads per CTA of k2_lagrow: eight lag rows per CTA for teams smaller
// than a warp (the split lengths' 8-thread teams would otherwise take 32 rows
// per CTA, and a 129-row disc window 160 team-rows), at least one whole warp
// (the row reduction shuffles over full warps), 256 threads for larger teams.
__host__ __device__ constexpr int lagrow_threads(int T)
{
    return T < 32 ? (8 * T < 32 ? 32 : 8 * T) : (T >= 256 ? T : 256);
}

template <int L>
__global__ void __launch_bounds__(lagrow_threads(FFTOf<L, +1>::T))
k2_lagrow(PairDev *pairs, const float2 *__restrict__ tw)
{
    using F = FFTOf<L, +1>;   // RegFFT, or MixFFT for L = 3 * 2^k, 5 * 2^k
    static_assert(F::SMEM <= lag_pitch<L>(), "the exchange buffer fits the team's row region");
    constexpr int V = F::V, T = F::T;
    constexpr int PITCH = lag_pitch<L>();   // holds L+1 bins, then 2L reals
    extern __shared__ float2 smem[];
    __shared__ double red_r[32];
    __shared__ long long red_k[32];
    __shared__ PairDev sp;
    const PairDev &p = stage_job(pairs, blockIdx.y, sp);
    if (p.status != 0)
        return;
    const int Wy = p.yhi - p.ylo + 1, Wx = p.xhi - p.xlo + 1;
    const int G = blockDim.x / T;
    const int team = threadIdx.x / T, t = threadIdx.x - team * T;
    const int j0 = blockIdx.x * G;
    if (j0 >= Wy)
        return;
    const int j = j0 + team;
    const bool live = j < Wy;
    float2 *sm = smem + team * PITCH;
    const int Nx = p.Nx, Ny = p.Ny;
    // spectrum bins of the CTA's lag rows
    load_lag_rows<L, T, lagrow_threads(T) / T>(smem, PITCH, p.Q, Wy, j0);
    __syncthreads();
    float2 v[V];
#pragma unroll
    for (int q = 0; q < V; ++q) {
        const int k = F::in_idx(t, q);
        float2 a = sm[padi(k)];
        float2 b = cconj(sm[padi(L - k)]);
        if (k == 0) {
            a.y = 0.f;
            b.y = 0.f;
        }
        const float2 e = cadd(a, b);
        const float2 dd = csub(a, b);
        const float2 wv = twn<2 * L, +1>(tw, k);   // W^{-k}
        const float2 o = cmul(dd, wv);
        v[q] = make_float2(e.x - o.y, e.y + o.x);
    }
    // the teams' rows are their own from here on: team barriers only
    F::run_team(v, sm, t, tw, team);
    __syncthreads();
    float *C = (float *)sm;   // 2L reals, unpadded
#pragma unroll
    for (int q = 0; q < V; ++q) {
        const int n = F::out_idx(t, q);
        C[2 * n] = v[q].x;
        C[2 * n + 1] = v[q].y;
    }
    __syncthreads();
    // 1 / (Nx Ny): exact for power-of-two grids; on the split lengths one
    // more FP32 rounding, below the transform's own error
    const float invf = 1.0f / ((float)Nx * (float)Ny);
    double br = -1.0e30;
    long long bk = 0x7fffffffffffffffLL;
    if (live) {
        const int y = p.ylo + j;
        const long long dy = y - p.oy;
        const int xr = isqrt_ll(p.rsqr - dy * dy);
        const int xa = xr < 0 ? 1 : max(p.xlo, p.ox - xr);
        const int xb = xr < 0 ? 0 : min(p.xhi, p.ox + xr);
        const int ys = y < 0 ? y + Ny : y;
        for (int x = p.xlo + t; x <= p.xhi; x += T) {
            double rv = 0.0;
            if (x >= xa && x <= xb) {
                const int xs = x < 0 ? x + Nx : x;
                if (lag_r(p, x, y, C[xs] * invf, rv))
                    best_merge(br, bk, rv, (long long)ys * Nx + xs);
            }
            p.rr[(long long)j * Wx + (x - p.xlo)] = rv;
        }
    }
    // team reduction
    for (int o = 16; o > 0; o >>= 1) {
        const double r2 = __shfl_down_sync(0xffffffff, br, o);
        const long long k2 = __shfl_down_sync(0xffffffff, bk, o);
        if ((threadIdx.x & 31) + o < 32 && ((threadIdx.x & 31) + o) / T == (threadIdx.x & 31) / T)
            best_merge(br, bk, r2, k2);
    }
    if (T <= 32) {
        if (live && t == 0) {
            p.rb[j].r = br;
            p.rb[j].key = bk;
        }
        return;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        red_r[wid] = br;
        red_k[wid] = bk;
    }
    __syncthreads();
    if (live && t == 0) {
        const int w0 = team * (T / 32);
        for (int q = 1; q < T / 32; ++q)
            best_merge(br, bk, red_r[w0 + q], red_k[w0 + q]);
        p.rb[j].r = br;
        p.rb[j].key = bk;
    }
}

// ---------------------------------------------------------------------------
// CorrImagesR/S lag images (CCorImg::MakeRandA / MakeSandRandA + OrderF +
// SimpleMax, 0_GEN/Correlation.cpp:2060-2380,2509-2569,2939-2948)
// ---------------------------------------------------------------------------

// Per lag row: inverse real FFT of the S rows (whitened product) and/or the
// R rows (plain product), S and R per lag, A = legality & oval (& R > mincor),
// the row's best candidate (key S or R; ties -> smallest R-image index) and
// the row's S sums.
// SONLY: chunks of S-key jobs without a mincor (the sweep's correlator):
// one inverse per row and the FP32-key scan only, compiled without the rest.
template <int L, bool SONLY>
__global__ void __launch_bounds__(256, SONLY ? 3 : 2) k2_lagimg(PairDev *pairs, const float2 *__restrict__ tw)
{
    using F = RegFFT<L, +1>;
    static_assert(F::SMEM <= lag_pitch<L>(), "the exchange buffer fits the team's row region");
    constexpr int R = F::R, T = F::T;
    constexpr int PITCH = lag_pitch<L>();
    extern __shared__ float2 smem[];
    __shared__ double red_r[32], red_s[32], red_s2[32];
    __shared__ long long red_k[32];
    __shared__ PairDev sp;
    const PairDev &p = stage_job(pairs, blockIdx.y, sp);
    if (p.status != 0)
        return;
    const int Wy = p.yhi - p.ylo + 1, Wx = p.xhi - p.xlo + 1;
    const int G = blockDim.x / T;
    const int team = threadIdx.x / T, t = threadIdx.x - team * T;
    const int j0 = blockIdx.x * G;
    if (j0 >= Wy)
        return;
    const int j = j0 + team;
    const bool live = j < Wy;
    const bool want_r = !SONLY && p.want_r != 0, want_s = SONLY || p.want_s != 0;
    const bool both = want_r && want_s;
    float2 *sm = smem + team * PITCH * (both ? 2 : 1);
    const int Nx = p.Nx, Ny = p.Ny;
    const float *CS = nullptr, *CR = nullptr;
#pragma unroll 1
    for (int pass = 0; pass < 2; ++pass) {
        const bool doS = pass == 0;
        if ((doS && !want_s) || (!doS && !want_r))
            continue;
        const float2 *Qs = doS ? (both ? p.Q2 : p.Q) : p.Q;
        float2 *reg = sm + ((both && !doS) ? PITCH : 0);
        __syncthreads();
        load_lag_rows<L, T>(smem + ((both && !doS) ? PITCH : 0), PITCH * (both ? 2 : 1), Qs,
                            Wy, j0);
        __syncthreads();
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int k = t + r * T;
            float2 a = reg[padi(k)];
            float2 b = cconj(reg[padi(L - k)]);
            if (k == 0) {
                a.y = 0.f;
                b.y = 0.f;
            }
            const float2 e = cadd(a, b);
            const float2 dd = csub(a, b);
            float2 wv = __ldg(&tw[2 * L + k]);
            wv.y = -wv.y;
            const float2 o = cmul(dd, wv);
            v[r] = make_float2(e.x - o.y, e.y + o.x);
        }
        F::run_team(v, reg, t, tw, team);   // the team's own row
        __syncthreads();
        float *C = (float *)reg;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int n = t + r * T;
            C[2 * n] = v[r].x;
            C[2 * n + 1] = v[r].y;
        }
        if (doS)
            CS = C;
        else
            CR = C;
    }
    __syncthreads();
    const double inv = 1.0 / ((double)Nx * (double)Ny);
    double br = -1.0e30, ss = 0.0, ss2 = 0.0;
    long long bk = 0x7fffffffffffffffLL;
    if (live && (SONLY || p.s_float)) {
        // S key alone: S = c / (Nx Ny) is strictly increasing in the FP32
        // inverse value c, so the scan compares c itself (same argmax, same
        // ties); the S statistics are compensated FP32 sums of c and c^2.
        const int y = p.ylo + j, iy = y + p.cy;
        float fs = 0.f, fe = 0.f, fq = 0.f, fqe = 0.f, bc = 0.f;
        float *rf = (float *)p.rr + (long long)j * Wx - p.xlo;
        for (int x = p.xlo + t; x <= p.xhi; x += T) {
            const float c = CS[x < 0 ? x + Nx : x];
            two_sum_acc(fs, fe, c);
            const float c2 = __fmul_rn(c, c);
            two_sum_acc(fq, fqe, c2);
            fqe = __fadd_rn(fqe, __fmaf_rn(c, c, -c2));
            rf[x] = c;
            // legality only for a lag that would become this thread's best
            // (its lags come in increasing key order: a tie never wins)
            if (bk == 0x7fffffffffffffffLL || c > bc) {
                double rv;
                const int ix = x + p.cx;
                if (lag_eval(p, x, y, 0.0, false, rv) && oval_ok(p, ix, iy)) {
                    bc = c;
                    bk = (long long)iy * p.wR + ix;
                }
            }
        }
        if (bk != 0x7fffffffffffffffLL)
            br = (double)bc;
        ss = (double)fs + (double)fe;
        ss2 = (double)fq + (double)fqe;
    } else if (!SONLY && live) {
        const int y = p.ylo + j, iy = y + p.cy;
        const bool keyS = p.mode == JOB_IMAGES_S;
        for (int x = p.xlo + t; x <= p.xhi; x += T) {
            const int xs = x < 0 ? x + Nx : x;
            double S = 0.0, rv = 0.0;
            if (want_s) {
                S = (double)CS[xs] * inv;
                ss += S;
                ss2 += S * S;
            }
            const bool legal = lag_eval(p, x, y, want_r ? (double)CR[xs] * inv : 0.0, want_r, rv);
            const double key = keyS ? S : rv;
            const long long o = (long long)j * Wx + (x - p.xlo);
            p.rr[o] = key;
            if (keyS && want_r)
                p.rr2[o] = rv;
            const int ix = x + p.cx;
            const bool cand = legal && oval_ok(p, ix, iy) && (p.mincor <= 0.0 || rv > p.mincor);
            if (p.mode == JOB_IMAGES_F)   // OrderF's candidates (A, R > mincor)
                p.fst[o] = cand ? 4 : 0;
            if (cand)
                best_merge(br, bk, key, (long long)iy * p.wR + ix);
        }
    }
    const int lane = threadIdx.x & 31;
    for (int o = 16; o > 0; o >>= 1) {
        const double r2 = __shfl_down_sync(0xffffffff, br, o);
        const long long k2 = __shfl_down_sync(0xffffffff, bk, o);
        const double a2 = __shfl_down_sync(0xffffffff, ss, o);
        const double b2 = __shfl_down_sync(0xffffffff, ss2, o);
        if (lane + o < 32 && (lane + o) / T == lane / T) {
            best_merge(br, bk, r2, k2);
            ss += a2;
            ss2 += b2;
        }
    }
    if (T <= 32) {
        if (live && t == 0) {
            p.rb[j].r = br;
            p.rb[j].key = bk;
            p.rb[j].ssum = ss;
            p.rb[j].ssum2 = ss2;
        }
        return;
    }
    const int wid = threadIdx.x >> 5;
    if (lane == 0) {
        red_r[wid] = br;
        red_k[wid] = bk;
        red_s[wid] = ss;
        red_s2[wid] = ss2;
    }
    __syncthreads();
    if (live && t == 0) {
        const int w0 = team * (T / 32);
        for (int q = 1; q < T / 32; ++q) {
            best_merge(br, bk, red_r[w0 + q], red_k[w0 + q]);
            ss += red_s[w0 + q];
            ss2 += red_s2[w0 + q];
        }
        p.rb[j].r = br;
        p.rb[j].key = bk;
        p.rb[j].ssum = ss;
        p.rb[j].ssum2 = ss2;
    }
}

// ParabPeak on the key image at R-image pixel (rx, ry) (neighbours must be
// > 0, 0_GEN/Correlation.cpp:2975-3010), ReturnR's offsets (:3016-3043); the
// S score 10 (S - mean) / (sd sqrt(nR)) with the sample sd for CorrImagesS
// (:3285-3289).  Writes the job's result.
__device__ void img_result(PairDev &p, int rx, int ry, double ss, double ss2, ResultDev &o)
{
    const int wR = p.wR, hR = p.hR;
    // the key image (the window is the whole R image); FP32 c when s_float:
    // ParabPeak's ratios and the S score are the same in c units
    const double *Id = p.rr;
    const float *If = (const float *)p.rr;
    const bool fl = p.s_float != 0;
    auto I = [&](long long k) -> double { return fl ? (double)If[k] : Id[k]; };
    double xpk = rx, ypk = ry;
    const double z1 = I(rx + (long long)wR * ry);
    double z0, z2;
    if (rx - 1 >= 0 && rx + 1 < wR && (z0 = I(rx - 1 + (long long)wR * ry)) > 0.0 &&
        (z2 = I(rx + 1 + (long long)wR * ry)) > 0.0) {
        z0 = (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8)
            xpk += z0;
    }
    if (ry - 1 >= 0 && ry + 1 < hR && (z0 = I(rx + (long long)wR * (ry - 1))) > 0.0 &&
        (z2 = I(rx + (long long)wR * (ry + 1))) > 0.0) {
        z0 = (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
        if (fabs(z0) <= 8)
            ypk += z0;
    }
    double r = z1;
    if (p.mode == JOB_IMAGES_S) {
        const double n = (double)wR * hR;
        const double mn = ss / n;
        const double sd = sqrt(fmax(ss2 - n * mn * mn, 0.0) / (n - 1.0));
        r = 10.0 * (z1 - mn) / (sd * sqrt(n));
    }
    p.r = r;
    p.dx = xpk + (p.x0[1] - p.x0[0]) - p.cx;
    p.dy = ypk + (p.y0[1] - p.y0[0]) - p.cy;
    p.px = rx - p.cx;
    p.py = ry - p.cy;
    p.status = ALN_OK;
    o.r = p.r;
    o.dx = p.dx;
    o.dy = p.dy;
    o.status = ALN_OK;
    o.px = p.px;
    o.py = p.py;
}

// grid (npairs), block 256: argmax over rows, ParabPeak on the key image
// (neighbours must be > 0, 0_GEN/Correlation.cpp:2975-3010), ReturnR's
// offsets (:3016-3043); CorrImagesS returns 10 (S - mean) / (sd sqrt(nR))
// with the sample sd over the whole S image (:3285-3289).
__global__ void k_final_img(PairDev *pairs, ResultDev *res)
{
    __shared__ double red_r[32], red_s[32], red_s2[32];
    __shared__ long long red_k[32];
    PairDev &p = pairs[blockIdx.x];
    if (p.status != 0)
        return;
    const int Wy = p.yhi - p.ylo + 1;
    double br = -1.0e30, ss = 0.0, ss2 = 0.0;
    long long bk = 0x7fffffffffffffffLL;
    for (int j = threadIdx.x; j < Wy; j += blockDim.x) {
        best_merge(br, bk, p.rb[j].r, p.rb[j].key);
        ss += p.rb[j].ssum;
        ss2 += p.rb[j].ssum2;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double r2 = __shfl_down_sync(0xffffffff, br, o);
        const long long k2 = __shfl_down_sync(0xffffffff, bk, o);
        const double a2 = __shfl_down_sync(0xffffffff, ss, o);
        const double b2 = __shfl_down_sync(0xffffffff, ss2, o);
        best_merge(br, bk, r2, k2);
        ss += a2;
        ss2 += b2;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        red_r[wid] = br;
        red_k[wid] = bk;
        red_s[wid] = ss;
        red_s2[wid] = ss2;
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    for (int q = 1; q < (int)(blockDim.x >> 5); ++q) {
        best_merge(br, bk, red_r[q], red_k[q]);
        ss += red_s[q];
        ss2 += red_s2[q];
    }
    ResultDev &o = res[blockIdx.x];
    if (bk == 0x7fffffffffffffffLL) {   // no candidate lag
        p.status = ALN_NO_PEAK;
        o.r = o.dx = o.dy = 0.0;
        o.status = ALN_NO_PEAK;
        o.px = o.py = 0;
        return;
    }
    const int ry = (int)(bk / p.wR), rx = (int)(bk - (long long)ry * p.wR);
    img_result(p, rx, ry, ss, ss2, o);
}

// ---------------------------------------------------------------------------
// CorrImagesF (0_GEN/Correlation.cpp:3066-3122): F = the R image filtered by
// the 3 x 3 kernel {-1 x 8, 9} (MakeF, :2412-2492), the best isolated F peak
// (FPeak, :2580-2767), ParabPeak and ReturnR on R there
// ---------------------------------------------------------------------------

// grid (ceil(wR/32), ceil(hR/8), njobs), block (32, 8).  MakeF convolves R
// over a frame of CeilPow2(wR) x CeilPow2(hR) and then clears a guard band of
// 2 pixels (F and the candidate flags); inside the band every tap lies in R,
// so the filter is the plain 3 x 3 stencil.  F keeps its positive part; the
// reference's division by the maximum is left out: every FPeak test compares
// F values with multiples of a peak's F, so a common positive scale changes
// no decision.
__global__ void k_makef(PairDev *pairs)
{
    PairDev &p = pairs[blockIdx.z];
    if (p.status != 0 || p.mode != JOB_IMAGES_F)
        return;
    const int wR = p.wR, hR = p.hR;
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= wR || y >= hR)
        return;
    const long long k = (long long)y * wR + x;
    const int grd = 2;
    if (x < grd || x >= wR - grd || y < grd || y >= hR - grd) {
        p.fimg[k] = 0.0;
        p.fst[k] = 0;
        return;
    }
    const double *R = p.rr;
    double f = 9.0 * R[k];
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx)
            if (dx || dy)
                f -= R[k + (long long)dy * wR + dx];
    p.fimg[k] = f > 0.0 ? f : 0.0;
}

// FPeak, one CTA of 1024 threads per job.  Candidates in OrderF's order (F
// descending; equal F: smaller index first) are taken one at a time: each
// thread keeps the best live candidate of its own pixels (k = t mod 1024)
// and rescans only when that one is visited or masked; a block argmax
// picks the next.  The candidate's tests run on the whole block: the four
// scans for the half-height radius ri (one warp each, 32 pixels per
// ballot), the guard-band bounds, the core mask, and the ring between ri and
// 3 ri for a neighbour above nbmaxht x peak.  The first candidate that passes
// is the peak.
#define FPK_THREADS 1024

__device__ __forceinline__ bool fpk_better(double a, long long ia, double b, long long ib)
{
    return a > b || (a == b && ia < ib);
}

__global__ void __launch_bounds__(FPK_THREADS) k_fpeak(PairDev *pairs, ResultDev *res)
{
    __shared__ double s_v[32];
    __shared__ long long s_i[32];
    __shared__ int s_dist[4];
    __shared__ long long s_pick;
    PairDev &p = pairs[blockIdx.x];
    if (p.status != 0 || p.mode != JOB_IMAGES_F)
        return;
    ResultDev &o = res[blockIdx.x];
    const int wR = p.wR, hR = p.hR;
    const long long nR = (long long)wR * hR;
    const double *F = p.fimg;
    unsigned char *st = p.fst;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    double lv = -1.0;
    long long li = -1;   // this thread's best live candidate (-1: rescan)
    for (;;) {
        if (li >= 0 && (st[li] & 3))
            li = -1;
        if (li < 0) {
            lv = -1.0;
            for (long long k = tid; k < nR; k += FPK_THREADS)
                if ((st[k] & 7) == 4 && (li < 0 || fpk_better(F[k], k, lv, li))) {
                    lv = F[k];
                    li = k;
                }
        }
        // block argmax (value desc, index asc); li < 0 never wins
        double bv = li >= 0 ? lv : -2.0;
        long long bi = li >= 0 ? li : 0x7fffffffffffffffLL;
        for (int off = 16; off > 0; off >>= 1) {
            const double v2 = __shfl_down_sync(0xffffffff, bv, off);
            const long long i2 = __shfl_down_sync(0xffffffff, bi, off);
            if (fpk_better(v2, i2, bv, bi)) {
                bv = v2;
                bi = i2;
            }
        }
        if (lane == 0) {
            s_v[wid] = bv;
            s_i[wid] = bi;
        }
        __syncthreads();
        if (tid == 0) {
            for (int w = 1; w < FPK_THREADS / 32; ++w)
                if (fpk_better(s_v[w], s_i[w], bv, bi)) {
                    bv = s_v[w];
                    bi = s_i[w];
                }
            s_pick = bv > -1.5 ? bi : -1;
        }
        __syncthreads();
        const long long k = s_pick;
        if (k < 0)
            break;   // every candidate tried
        const double fpk = F[k], half = 0.5 * fpk, tol = p.nbmaxht * fpk;
        const int ry = (int)(k / wR), rx = (int)(k - (long long)ry * wR);
        // ri: first pixel at or below half height up, down, left, right
        if (wid < 4) {
            const int dx = wid == 2 ? -1 : (wid == 3 ? 1 : 0);
            const int dy = wid == 0 ? -1 : (wid == 1 ? 1 : 0);
            const int lim = wid == 0 ? ry : wid == 1 ? hR - 1 - ry : wid == 2 ? rx : wR - 1 - rx;
            int found = -1;
            for (int d0 = 1; d0 <= lim && found < 0; d0 += 32) {
                const int d = d0 + lane;
                bool hit = false;
                if (d <= lim)
                    hit = F[(long long)(ry + dy * d) * wR + (rx + dx * d)] <= half;
                const unsigned b = __ballot_sync(0xffffffff, hit);
                if (b)
                    found = d0 + __ffs(b) - 1;
            }
            if (lane == 0)
                s_dist[wid] = found;
        }
        __syncthreads();
        if (tid == 0) {
            int ri = 1 << 30, ok = 1;
            for (int w = 0; w < 4; ++w) {
                if (s_dist[w] < 0)
                    ok = 0;   // Ri_edge
                else
                    ri = min(ri, s_dist[w]);
            }
            if (ok && ri <= 1 && p.rr[k] < 0.1)
                ok = 0;   // Micropk
            const int ro = 3 * ri;
            if (ok && (ry - ro < 0 || ry + ro >= hR || rx - ro < 0 || rx + ro >= wR))
                ok = 0;   // Ro_edge
            st[k] |= 2;   // visited
            s_dist[0] = ok ? ri : -1;
        }
        __syncthreads();
        const int ri = s_dist[0];
        if (ri >= 0) {
            const int ro = 3 * ri, rm = max(1, ri / 3);
            // mask the core peak region
            const int mw = 2 * rm + 1;
            for (int e = tid; e < mw * mw; e += FPK_THREADS) {
                const int yy = ry - rm + e / mw, xx = rx - rm + e % mw;
                st[(long long)yy * wR + xx] |= 1;
            }
            // any pixel above tol in the ring between ri and ro
            const int ow = 2 * ro + 1;
            const long long tot = (long long)ow * ow;
            int hi = 0;
            for (long long e = tid; e < tot && !hi; e += FPK_THREADS) {
                const int yy = ry - ro + (int)(e / ow), xx = rx - ro + (int)(e % ow);
                if (yy >= ry - ri && yy <= ry + ri && xx >= rx - ri && xx <= rx + ri)
                    continue;
                hi = F[(long long)yy * wR + xx] > tol;
            }
            hi = __syncthreads_or(hi);
            if (!hi) {
                if (tid == 0)
                    img_result(p, rx, ry, 0.0, 0.0, o);
                return;
            }
        }
        __syncthreads();
    }
    if (tid == 0) {   // All peaks rejected / no candidates
        p.status = ALN_NO_PEAK;
        o.r = o.dx = o.dy = 0.0;
        o.status = ALN_NO_PEAK;
        o.px = o.py = 0;
    }
}

// ---------------------------------------------------------------------------
// CorrPatchToImage (0_GEN/Correlation.cpp:1186-1355): raw correlation over an
// N x N frame, its own lag zones, ParabPeakFFT on the raw inverse
// ---------------------------------------------------------------------------

// Per storage row: inverse real FFT -> raw values (kept for the neighbour
// look-ups), the row's best lag by the reference's zone rules:
// y > N - h1 negative, else y >= h2 dead (likewise x), disc on (x, y).
template <int L>
__global__ void k2_lagp2i(PairDev *pairs, const float2 *__restrict__ tw)
{
    using F = RegFFT<L, +1>;
    static_assert(F::SMEM <= lag_pitch<L>(), "the exchange buffer fits the team's row region");
    constexpr int R = F::R, T = F::T;
    constexpr int PITCH = lag_pitch<L>();
    extern __shared__ float2 smem[];
    __shared__ double red_r[32];
    __shared__ long long red_k[32];
    PairDev &p = pairs[blockIdx.y];
    if (p.status != 0)
        return;
    const int N = p.Nx, Wy = p.Ny;
    const int G = blockDim.x / T;
    const int team = threadIdx.x / T, t = threadIdx.x - team * T;
    const int j0 = blockIdx.x * G;
    if (j0 >= Wy)
        return;
    const int j = j0 + team;
    const bool live = j < Wy;
    float2 *sm = smem + team * PITCH;
    load_lag_rows<L, T>(smem, PITCH, p.Q, Wy, j0);
    __syncthreads();
    float2 v[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int k = t + r * T;
        float2 a = sm[padi(k)];
        float2 b = cconj(sm[padi(L - k)]);
        if (k == 0) {
            a.y = 0.f;
            b.y = 0.f;
        }
        const float2 e = cadd(a, b);
        const float2 dd = csub(a, b);
        float2 wv = __ldg(&tw[2 * L + k]);
        wv.y = -wv.y;
        const float2 o = cmul(dd, wv);
        v[r] = make_float2(e.x - o.y, e.y + o.x);
    }
    F::run_team(v, sm, t, tw, team);   // the team's own row
    double br = -1.0e30;
    long long bk = 0x7fffffffffffffffLL;
    if (live) {
        // storage row j; its lag row by the reference's rule
        int y = j;
        bool ydead = false;
        if (y > N - p.p2i_h1)
            y -= N;
        else if (y >= p.p2i_h2)
            ydead = true;
        const long long dy = y - p.oy;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const int n = t + r * T;
            for (int h = 0; h < 2; ++h) {
                const int xs = 2 * n + h;
                const double val = h ? (double)v[r].y : (double)v[r].x;
                p.rr[(long long)j * N + xs] = val;
                if (ydead)
                    continue;
                int x = xs;
                if (x > N - p.p2i_w1)
                    x -= N;
                else if (x >= p.p2i_w2)
                    continue;
                const long long dx = x - p.ox;
                if (dx * dx + dy * dy > p.rsqr)
                    continue;
                best_merge(br, bk, val, (long long)j * N + xs);
            }
        }
    }
    const int lane = threadIdx.x & 31;
    for (int o = 16; o > 0; o >>= 1) {
        const double r2 = __shfl_down_sync(0xffffffff, br, o);
        const long long k2 = __shfl_down_sync(0xffffffff, bk, o);
        if (lane + o < 32 && (lane + o) / T == lane / T)
            best_merge(br, bk, r2, k2);
    }
    if (T <= 32) {
        if (live && t == 0) {
            p.rb[j].r = br;
            p.rb[j].key = bk;
        }
        return;
    }
    const int wid = threadIdx.x >> 5;
    if (lane == 0) {
        red_r[wid] = br;
        red_k[wid] = bk;
    }
    __syncthreads();
    if (live && t == 0) {
        const int w0 = team * (T / 32);
        for (int q = 1; q < T / 32; ++q)
            best_merge(br, bk, red_r[w0 + q], red_k[w0 + q]);
        p.rb[j].r = br;
        p.rb[j].key = bk;
    }
}

__global__ void k_final_p2i(PairDev *pairs, ResultDev *res)
{
    __shared__ double red_r[32];
    __shared__ long long red_k[32];
    PairDev &p = pairs[blockIdx.x];
    if (p.status != 0)
        return;
    const int N = p.Nx;
    double br = -1.0e30;
    long long bk = 0x7fffffffffffffffLL;
    for (int j = threadIdx.x; j < N; j += blockDim.x)
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
    int bigx = -1, bigy = -1;
    double biggest = -1.0E30;
    if (br > -1.0e30) {
        const int ys = (int)(bk / N), xs = (int)(bk - (long long)ys * N);
        bigy = ys > N - p.p2i_h1 ? ys - N : ys;
        bigx = xs > N - p.p2i_w1 ? xs - N : xs;
        biggest = br;
    }
    biggest /= p.p2i_norm;
    // ParabPeakFFT, d = 1, LkFFT on the raw inverse (0_GEN/Correlation.cpp:268-298,482-517)
    const double *I = p.rr;
    auto lk = [&](int x, int y) {
        if (x < 0)
            x += N;
        if (y < 0)
            y += N;
        return I[x + (long long)N * y];
    };
    double xpk = bigx, ypk = bigy;
    const int ix = bigx, iy = bigy;
    if (ix > -N && iy > -N) {
        const double z1 = lk(ix, iy);
        double z0, z2;
        if (ix - 1 >= 0 && ix + 1 < N && (z0 = lk(ix - 1, iy)) != 0.0 &&
            (z2 = lk(ix + 1, iy)) != 0.0) {
            z0 = (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
            if (fabs(z0) <= 8)
                xpk += z0;
        }
        if (iy - 1 >= 0 && iy + 1 < N && (z0 = lk(ix, iy - 1)) != 0.0 &&
            (z2 = lk(ix, iy + 1)) != 0.0) {
            z0 = (z0 - z2) / (2 * (z0 + z2 - z1 - z1));
            if (fabs(z0) <= 8)
                ypk += z0;
        }
    }
    p.r = biggest;
    p.dx = xpk;
    p.dy = ypk;
    p.px = bigx;
    p.py = bigy;
    // the reference exits (44) on a normalised peak above 1.0001
    p.status = biggest > 1.0001 ? ALN_NO_PEAK : ALN_OK;
    o.r = p.r;
    o.dx = p.dx;
    o.dy = p.dy;
    o.status = p.status;
    o.px = bigx;
    o.py = bigy;
}
