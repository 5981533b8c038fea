// aln_corr_kernels.cuh -- device-side data layout shared by the correlation
// kernels (aln_corr.cu) and the host orchestration.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

// Best legal lag of one lag row (written by the lag kernel).
struct RowBest {
    double r;        // best r in the row, -1e30 if no legal lag
    long long key;   // tie-break index of that lag (smallest wins)
    double ssum, ssum2;   // CorrImagesS: sums of S and S^2 over the row
};

// job kinds
enum { JOB_PATCHES = 0, JOB_IMAGES_R = 1, JOB_IMAGES_S = 2, JOB_P2I = 3, JOB_IMAGES_F = 4 };

// Compact per-pair result copied back to the host.
struct ResultDev {
    double r, dx, dy;
    int status, px, py, pad;
};

// One correlation job as the kernels see it.  Lives in device memory; the
// kernels write the mean shifts and the result back into it.
struct PairDev {
    // inputs: image 0 = patch 1 (a), image 1 = patch 2 (b)
    const void *img[2];
    int dt[2];          // enum aln_dtype
    int stride[2];      // elements per row
    int w[2], h[2];     // bounding boxes
    int x0[2], y0[2];   // bounding-box origins B.L, B.B
    int Nx, Ny, logNx, logNy;
    // the reference's FFT raster (CeilPow2(w1+w2-1) x CeilPow2(h1+h2-1) in
    // the solved frame): ParabPeakFFT reads its neighbours by that raster's
    // storage rules, whatever grid the job is transformed on
    int rnx, rny;
    // 1: the job is solved on transposed images (x <-> y); img/w/h/x0/y0,
    // the window and the disc are in the transposed frame, src_* describe
    // the caller's untransposed rasters for k_transpose
    int transposed;
    const void *src_img[2];
    int src_stride[2];
    // search region: lag window (inclusive) and disc
    int ox, oy;
    long long rsqr;
    int xlo, xhi, ylo, yhi;
    // legality (typed EvalType)
    int rgn_kind, rgn_a, rgn_b;
    long long rgn_area;
    const unsigned char *table;
    int table_w, table_h;
    int cnt_kind;
    long long cnt_n;
    // summed-area-table rows needed by the lag window, per image: [lo, hi] x 2
    int need_lo[2][2], need_hi[2][2];
    int sat_rows[2];    // last row the column walk must reach (max needed / h-1)
    // workspace
    float2 *T[2];       // row-pass output [kx][y], stride Ts[i]
    int Ts[2];
    float2 *X2;         // spectrum of image 1 (b): [kx][ky], stride Ny
    int nseg, seg_len;  // CorrPatches: the column axis cut into nseg segments
                        // of seg_len rows of a, each transformed on Ny points
                        // (k2_corrseg); 0 = one transform of the whole column
    int b_cached;       // 1: X2 holds b's spectrum already (a cache entry);
                        // the row pass skips b and the column pass reads X2
    float2 *Q;          // column-inverse output [kx][j], j = y - ylo, stride Wy
    double *satS[2], *satQ[2];   // summed-area tables of v and v^2, [y][x] stride w
    int *satN[2];                // summed-area table of (v != 0)
    int sat_int;                 // bit i: image i's S, Q tables hold int64
    int sat_nonly;               // 1: only the count table N is needed (S key alone)
    int s_float;                 // S key alone: rr holds the FP32 correlation c,
                                 // RowBest r/ssum/ssum2 are in c units (S = c / NxNy)
    double *segS[2], *segQ[2];   // per column-walk segment: exclusive column offsets
    int *segN[2];
    double *colsum[2];           // per-column totals (mean shift)
    double *rr;                  // r over the lag window [j][x - xlo] (the key image)
    RowBest *rb;                 // per lag row
    double mu[2];                // mean shift applied before the FFT
    // CorrImagesR/S (0_GEN/Correlation.cpp:1851-3290)
    int mode;                    // JOB_*
    int want_r, want_s;          // which inverse transforms the job needs
    int no_shift;                // S is not shift-invariant: mu = 0
    double mincor;               // candidates need R > mincor when > 0
    double nbmaxht;              // CorrImagesF: neighbour height limit (x peak)
    double *fimg;                // CorrImagesF: the F image [iy][ix] (wR x hR)
    unsigned char *fst;          // CorrImagesF: per R pixel, bit 2 candidate,
                                 // bit 1 visited, bit 0 masked (FPeak)
    int oval_on, ocx, ocy, orx, ory;   // MaskA oval in R-image indices
    double oasq, orx2;
    int cx, cy, wR, hR;          // R image: lag (x, y) at index (x + cx) + wR (y + cy)
    float2 *Q2;                  // whitened inverse rows when both R and S are needed
    double *rr2;                 // R image when the key is S and mincor > 0
    // CorrPatchToImage (0_GEN/Correlation.cpp:1186-1355)
    int p2i_filter;              // Gaussian low-pass of the cross spectrum
    int p2i_w1, p2i_h1, p2i_w2, p2i_h2;   // patch bbox size, image nonzero extent
    double p2i_norm;             // np1 * N^2
    // result
    double r, dx, dy;
    int status, px, py;
};
