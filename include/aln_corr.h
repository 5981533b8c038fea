/*
 * aln_corr.h -- C ABI of the GB300 tile-matching library (libaln_corr.so).
 *
 * This is the drop-in boundary for Aligner's FFT normalised
 * cross-correlation (0_GEN/Correlation.h) and the CThmScan angle sweep
 * (0_GEN/CThmScan.h).  Every entry point below names the reference
 * interface it replaces.  Plain C types only: pointers, sizes, status codes.
 *
 * Conventions shared with the reference:
 *   - rasters are row-major, element (x, y) at data[x + stride*y];
 *   - a raster is the bounding box of a point cloud (0_GEN/Geometry.cpp:78-106):
 *     (x0, y0) are the box's integer left/bottom (B.L, B.B), w/h its size;
 *     pixels without a point hold 0;
 *   - a lag (dx, dy) shifts image 1 into image 2's frame
 *     (0_GEN/Geometry.cpp:142-176);
 *   - FFT sizes are CeilPow2(n1 + n2 - 1) per axis
 *     (0_GEN/Correlation.cpp:344-347).
 *
 * Errors: the library never exits the process.  Hard errors are negative
 * status codes with a message from aln_last_error(); a search that finds no
 * legal lag returns ALN_NO_PEAK with r = dx = dy = 0, which is what the
 * reference returns in that case (0_GEN/Correlation.cpp:1074-1087,3098-3119).
 *
 * Threading: each aln_ctx owns a CUDA stream and its workspaces; use one
 * context per host thread.  Contexts are independent.
 */
#pragma once

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes --------------------------------------------------- */

enum aln_status {
    ALN_OK = 0,
    ALN_NO_PEAK = 1,            /* soft result: no legal lag / too small */
    ALN_ERR_ARG = -1,           /* bad argument (size, dtype, pointer) */
    ALN_ERR_CUDA = -2,          /* CUDA runtime error (message has details) */
    ALN_ERR_NOMEM = -3,         /* device allocation failed */
    ALN_ERR_UNSUPPORTED = -4,   /* size outside the compiled FFT plans */
    ALN_ERR_TIMEOUT = -5,       /* deadline passed / bounded wait gave up */
    ALN_ERR_REFUSED = -6,       /* admission refused (server full) */
    ALN_ERR_CANCELLED = -7      /* request cancelled */
};

enum aln_dtype { ALN_U8 = 0, ALN_U16 = 1, ALN_F32 = 2, ALN_F64 = 3 };

/* ---- inputs --------------------------------------------------------- */

typedef struct aln_image {
    const void *data;   /* host pointer, or device pointer if on_device */
    int dtype;          /* enum aln_dtype */
    int w, h;           /* bounding-box size in pixels */
    int stride;         /* elements between rows (>= w) */
    int x0, y0;         /* bounding-box origin B.L, B.B (integer) */
    int on_device;      /* 1 if data lives on the context's device */
} aln_image;

/*
 * Legality tests applied to every lag, the typed form of the reference's
 * EvalType callbacks (0_GEN/Correlation.h:91):
 *   LegalRgn(olw, olh): the overlap box size;
 *   LegalCnt(c1, c2):   non-zero pixel counts of image 1 / image 2 inside it.
 *
 * rgn_kind:
 *   ALN_RGN_NONE     always legal (LegalRgn == NULL)
 *   ALN_RGN_MIN      olw >= a && olh >= b && olw*olh > area
 *                    (CThmScan BigEnough, 0_GEN/CThmScan.cpp:28-33;
 *                     testnormcorr SomeArea with a=b=2, area=0)
 *   ALN_RGN_SECTION  olw*olh > area && (olw >= a || olh > b)
 *                    (1_DMesh/InSectionOverlap.cpp:41-47)
 *   ALN_RGN_EXACT    olw == a && olh == b (1_Mosaic_current/mos.cpp:1270-1274)
 *   ALN_RGN_TABLE    table[(olh-1)*table_w + (olw-1)] != 0, for any other
 *                    callback tabulated by the caller over
 *                    olw in [1, table_w], olh in [1, table_h]
 * cnt_kind:
 *   ALN_CNT_NONE     no count test (LegalCnt == NULL, or always true)
 *   ALN_CNT_GT       c1 > n && c2 > n (CThmScan EnoughPoints, 0_GEN/CThmScan.cpp:39-42)
 */
enum { ALN_RGN_NONE = 0, ALN_RGN_MIN = 1, ALN_RGN_SECTION = 2,
       ALN_RGN_EXACT = 3, ALN_RGN_TABLE = 4 };
enum { ALN_CNT_NONE = 0, ALN_CNT_GT = 1 };

typedef struct aln_legal {
    int rgn_kind;
    int rgn_a, rgn_b;
    long long rgn_area;
    const unsigned char *table;   /* host pointer (ALN_RGN_TABLE only) */
    int table_w, table_h;
    int cnt_kind;
    long long cnt_n;
} aln_legal;

/* ---- outputs -------------------------------------------------------- */

typedef struct aln_result {
    double r;           /* correlation (CorrPatches/R/F) or S score (S) */
    double dx, dy;      /* sub-pixel displacement placing image 1 into image 2 */
    int status;         /* ALN_OK or ALN_NO_PEAK */
    int peak_x, peak_y; /* integer lag of the peak (before bbox offsets) */
    int nx, ny;         /* FFT size used */
} aln_result;

typedef struct aln_ctx aln_ctx;

/* ---- context -------------------------------------------------------- */

/* Create a context on CUDA device `device`.  No reference counterpart
 * (the reference's state is the static mutex_fft, 0_GEN/Correlation.cpp:26-27). */
int aln_ctx_create(int device, aln_ctx **out);
void aln_ctx_destroy(aln_ctx *ctx);
/* Message of the last hard error on this context (or, when ctx is NULL, of
 * the calling thread's last failed call made without a context:
 * aln_ctx_create, aln_corr_patches_grid, aln_corr_patches_noalloc). */
const char *aln_last_error(const aln_ctx *ctx);

/* Upper bound on the device workspace one batch chunk may use (default
 * 4 GiB); larger batches are split into chunks.  No reference counterpart. */
int aln_ctx_set_workspace_limit(aln_ctx *ctx, size_t bytes);

/* ---- tracing: no reference counterpart (the reference logs wall-clock
 * "Timer:" lines, 0_GEN/Timer.cpp:25-52) ------------------------------ */

/* When on, every kernel launch is bracketed by CUDA events on the context's
 * stream; aln_ctx_profile() reports launches and summed device time per
 * kernel name since the last reset. */
int aln_ctx_set_profiling(aln_ctx *ctx, int on);
void aln_ctx_profile_reset(aln_ctx *ctx);
/* Fills up to cap entries; returns the number of kernel names recorded.
 * Name pointers stay valid until the next call on this context. */
int aln_ctx_profile(aln_ctx *ctx, int cap, const char **names, long long *launches,
                    double *ms);
/* which: 0 = kernel launches, 1 = host-to-device bytes, 2 = device-to-host
 * bytes, 3 = spectrum-cache hits, 4 = spectrum-cache fills (counted since
 * the last aln_ctx_profile_reset), 5 = device bytes the cache holds,
 * 6 = batch chunks run, 7 = host-to-device staging transfers issued (both
 * since the last reset), 8 = pair classes this context timed for the
 * autotuner, 9 = spectrum-cache entries evicted, 10 = host microseconds
 * spent planning batches, 11 = host microseconds preparing their chunks
 * (9-11 since the last reset). */
long long aln_ctx_counter(aln_ctx *ctx, int which);

/* Autotuner (no reference counterpart; replaces the reference's fixed
 * transform-size rule, 0_GEN/Correlation.cpp:333-359, for CorrPatches'
 * column plan): with tuning on (the default; environment ALN_TUNE=0 turns
 * it off for new contexts), the first CorrPatches pair of a new class --
 * (Nx/2, Ny, window height and a's height rounded up to powers of two, a's
 * pixel size) -- times every valid column plan (one Ny-point transform per
 * column, or segments of each valid length NS) on synthetic device pairs of
 * its geometry with CUDA events.  A plan that beats the cost model's pick by
 * more than 10 % becomes the class's plan; otherwise the class is marked
 * "cost model" and each of its pairs keeps its own cost-model plan.
 * Choices are kept per process and in <library dir>/tune/<GPU name>-<build
 * id>.txt (or $ALN_TUNE_DIR), which later processes read; an entry never
 * changes once made, so a pair's numbers do not depend on its batch.  Off:
 * the fixed cost model N (log2 N + 4) per transform. */
int aln_ctx_set_tuning(aln_ctx *ctx, int on);

/* CorrPatches transform rows of 3 * 2^k and 5 * 2^k points (on by
 * default).  Replaces the reference's power-of-two size rule (FFTSize,
 * 0_GEN/Correlation.cpp:333-359) on the row axis of the batched path: a
 * pair's grid is the shortest alias-free length for its disc among powers
 * of two and 2L for L in {80, 96, 160, 192, 320, 384, 640, 768, 1280,
 * 1536}.  The correlation sums at the disc's lags are the same on every
 * alias-free grid, so r, the peak and the sub-pixel offsets agree with the
 * power-of-two plan within FP32 rounding.  Off: powers of two only.
 * CorrImages jobs always keep the reference's power-of-two grids (the
 * whitened S product depends on the grid). */
int aln_ctx_set_split_grids(aln_ctx *ctx, int on);

/* Spectrum cache: the device-resident form of the reference's fft2 / ftc
 * cache arguments (CorrPatches' `vector<CD> &fft2`, 0_GEN/Correlation.cpp:
 * 901-915, 965-985; CorrImages' `ftc`, :3144-3290).  A job whose b_key is
 * non-zero names image b: the first job with that key (for its FFT size and
 * frame) stores b's spectrum in device memory, later jobs read it instead of
 * transforming b again.  Equal keys must mean equal images b (the caller's
 * promise, as in the reference, which reuses fft2 whenever its size
 * matches).  Results are the same numbers with or without the cache (a
 * keyed CorrPatches job always takes one column transform per column, so
 * the uncached job equal to it bit for bit is the unsegmented one,
 * aln_ctx_set_segmenting(ctx, -1); a segmented uncached job agrees within
 * FP32 rounding).
 * `bytes` bounds the device memory the cache holds (default 8 GiB; 0 turns
 * it off and releases it; SIZE_MAX: bounded by free device memory alone).
 * The cache also never grows into the last (workspace limit + 2 GiB) of
 * free device memory.  Least recently used entries are evicted first
 * (entries the running chunk reads are kept). */
int aln_ctx_set_spectrum_cache(aln_ctx *ctx, size_t bytes);

/* CorrPatches column segmenting for this context: 0 = the cost model
 * (default), -1 = never (one column transform per column), or a forced
 * segment transform length (a power of two, 64..2048; used where valid for
 * the pair's window).  Results agree within FP32 rounding either way. */
int aln_ctx_set_segmenting(aln_ctx *ctx, int ns);

/* ---- FFT support: 0_GEN/Correlation.h:14-31 ------------------------- */

/* FFTSize, 0_GEN/Correlation.cpp:344-347 */
int aln_fft_size(int n1, int n2);
/* FFTSizeSQR, 0_GEN/Correlation.cpp:355-359 */
int aln_fft_size_sqr(int w1, int h1, int w2, int h2);

/* FFT_2D, 0_GEN/Correlation_fft_fftw.cpp:36-56: unnormalised forward r2c of
 * in[Nslow][Nfast] (host, FP64) into out[Nslow][Nfast/2+1] complex
 * interleaved (host, FP64), computed on the GPU in FP32.  Returns
 * M = Nslow*(Nfast/2+1) or a negative status. */
int aln_fft_2d(aln_ctx *ctx, const double *in, int nfast, int nslow, double *out);

/* IFT_2D, 0_GEN/Correlation_fft_fftw.cpp:65-92: unnormalised c2r inverse.
 * Returns 0 or a negative status. */
int aln_ift_2d(aln_ctx *ctx, const double *in, int nfast, int nslow, double *out);

/* Convolve, 0_GEN/Correlation.cpp:371-457: dst (ws x hs, host FP64) = src
 * convolved with K (wk x hk) over the circular frame FFTSize(ws, wk/(1+sym))
 * x FFTSize(hs, hk/(1+sym)), K divided by its sum when prenorm (a zero sum
 * leaves it), the result divided by the frame size, as the reference.  FP32
 * transforms on the GPU.  The reference's kfft cache is not needed: the
 * kernel's transform is recomputed on the device. */
int aln_convolve(aln_ctx *ctx, const double *src, int ws, int hs, const double *K, int wk,
                 int hk, int sym, int prenorm, double *dst);

/* ParabPeakFFT, 0_GEN/Correlation.cpp:482-517 (host arithmetic, O(1)). */
void aln_parab_peak_fft(double *xpk, double *ypk, int d, const double *I,
                        int nx, int ny);

/* ---- correlation ---------------------------------------------------- */

/* CorrPatches, 0_GEN/Correlation.cpp:901-1170: Pearson-r correlation over
 * all lags inside the disc (Ox, Oy, radius), legal per `legal`, peak with
 * parabolic refinement; out->r, dx, dy as the reference returns them.
 * One pair per call (the plain per-pair path). */
int aln_corr_patches(aln_ctx *ctx, const aln_image *a, const aln_image *b,
                     int ox, int oy, int radius, const aln_legal *legal,
                     aln_result *out);

/* One CorrPatches job of a batch. */
typedef struct aln_pair {
    aln_image a, b;
    int ox, oy, radius;
    aln_legal legal;
    unsigned long long b_key;   /* != 0: image b's spectrum cache key (fft2) */
} aln_pair;

/* Many CorrPatches calls in one submission (pairs of any mix of sizes).
 * Pairs are grouped by FFT size and run by batched kernels; results are
 * identical to calling aln_corr_patches on each pair. */
int aln_corr_patches_batch(aln_ctx *ctx, int npairs, const aln_pair *pairs,
                           aln_result *out);

/* The transform grid CorrPatches uses for one pair (no reference
 * counterpart; a planning query).  The correlation at the disc's lags is
 * computed on the smallest power-of-two grid that holds both images and
 * keeps every lag of the disc window free of wrap-around, never larger than
 * the reference's FFTSize grid.  When it takes fewer FFT passes, the column
 * (long) axis is cut into *nseg segments of image a's rows, each correlated
 * on ny points (ny >= segment rows + window rows - 1) and summed in the
 * spectral domain; *nseg = 0 means one column transform of ny points.  A
 * pair with a spectrum-cache key (b_key) is never segmented.  nx, ny are in
 * the frame the pair is solved in: *transposed = 1 when a wide pair is
 * solved with x and y exchanged (as the batch entry points do).  The choice
 * depends on the pair alone (not on the batch it comes in: a pair gives the
 * same numbers alone and in any batch); aln_ctx_set_segmenting overrides it
 * per context.  Returns 0, ALN_NO_PEAK when the window is empty
 * (nx = ny = 0), or a negative status. */
int aln_corr_patches_grid(const aln_pair *pair, int *nx, int *ny, int *nseg, int *transposed);

/* CorrPatchToImage, 0_GEN/Correlation.cpp:1186-1355: the patch's points
 * (xy1[2i], xy1[2i+1], truncated to pixels) against a caller-embedded
 * square image i2 (N x N, N = sqrt(n2sq), a power of two 16..8192), raw
 * correlation / (n1 N^2), optional low-pass (bfilter), ParabPeakFFT on the
 * raw correlation.  out->dx, dy are the refined peak (no box offsets, as the
 * reference).  A normalised peak above 1.0001 (where the reference exits)
 * returns ALN_NO_PEAK. */
int aln_corr_patch_to_image(aln_ctx *ctx, const double *xy1, const double *v1, int n1,
                            const double *i2, int n2sq, int ox, int oy, int radius,
                            int bfilter, aln_result *out);

/* ---- CorrImagesF/R/S: 0_GEN/Correlation.h:159-220 ------------------ */

enum { ALN_CORR_F = 0, ALN_CORR_R = 1, ALN_CORR_S = 2 };

/* One CorrImages call: the R (and S) image over every lag, A = legality &
 * the oval MaskA (Rx, Ry > 0: semi-axes around (Ox, Oy), as
 * 0_GEN/Correlation.cpp:2011-2054), candidates A (and R > mincor when
 * mincor > 0), peak by maximal R (kind R) or maximal S, the FFT-whitened
 * correlation (kind S), ParabPeak refinement.  out->r is R at the peak
 * (kind R) or 10 (S - mean(S)) / (sd(S) sqrt(wR hR)) (kind S).  Images
 * smaller than the reference's SetDims limit give ALN_NO_PEAK.  Kind F
 * (CorrImagesF, 0_GEN/Correlation.cpp:3066-3122) filters R by the 3 x 3
 * kernel {-1 x 8, 9} and takes the highest well-isolated F peak (half-height
 * radius ri, no pixel above nbmaxht x peak between ri and 3 ri), reporting R
 * there; nbmaxht is used by kind F only. */
typedef struct aln_image_job {
    aln_image a, b;
    int kind;           /* ALN_CORR_F, ALN_CORR_R or ALN_CORR_S */
    aln_legal legal;
    double mincor, nbmaxht;
    int ox, oy, rx, ry;
    unsigned long long b_key;   /* != 0: image b's spectrum cache key (ftc) */
} aln_image_job;

/* CorrImagesF / R / S, 0_GEN/Correlation.cpp:3066-3122, 3144-3199, 3222-3290 */
int aln_corr_images(aln_ctx *ctx, int kind, const aln_image *a, const aln_image *b,
                    const aln_legal *legal, double mincor, double nbmaxht, int ox, int oy,
                    int rx, int ry, aln_result *out);
/* Many CorrImages calls in one submission (any mix of sizes). */
int aln_corr_images_batch(aln_ctx *ctx, int njobs, const aln_image_job *jobs,
                          aln_result *out);

/* ---- CThmScan angle sweep: 0_GEN/CThmScan.h:57-223 ------------------ */

/* Thumbnails of one pair, the ThmRec of 0_GEN/CThmScan.h:27-34.
 * A: values on an integer grid, point (x + a_x0, y + a_y0) holds
 *    a[x + a_stride*y] (present unless a_mask[...] == 0); the sweep rotates
 *    these points about the origin.
 * B: FP64 raster over the bounding box of B's points (ALN_F64, holes 0). */
typedef struct aln_thumbs {
    const double *a;
    const unsigned char *a_mask;   /* NULL: every grid point present */
    int a_w, a_h, a_stride, a_x0, a_y0;
    aln_image b;
    long long req_area;            /* ThmRec reqArea */
    int olap1d;                    /* ThmRec olap1D */
    unsigned long long b_key;      /* != 0: B's spectrum-cache key (ThmRec ftc),
                                      kept across calls; 0: cached for this call only */
} aln_thumbs;

/* CThmScan settings (its setters, 0_GEN/CThmScan.h:115-157). */
typedef struct aln_thm_params {
    double rthresh, nbmaxht;
    int constxy, pretweak, usecorrr;   /* usecorrr: CorrImagesS (1) or CorrImagesF (0) */
    int ox, oy, rx, ry;                /* SetDisc */
    double tdfm[6];                    /* SetTdfm (TAffine t[0..5]) */
    /* SetNewAngProc (T_NewAngProc, CThmScan.h:46-51): when set, called on
     * the host for every correlator call's angle (deg) to give its disc,
     * in place of ox, oy, rx, ry (NULL: the fixed disc) */
    void (*disc_of_angle)(void *user, double deg, int *ox, int *oy, int *rx, int *ry);
    void *disc_user;
} aln_thm_params;

/* CorRec (0_GEN/CThmScan.h:36-44) plus the search's err and call count. */
typedef struct aln_thm_result {
    double A, X, Y, R;
    double T[6];
    int err;       /* errOK 0, errLowRDenov 1, errLowRPrior 2 */
    int ncalls;    /* correlator calls made for this pair */
} aln_thm_result;

enum {
    ALN_THM_DENOVO = 0,      /* DenovoBestAngle(ang0, hfang, step), CThmScan.cpp:764-790 */
    ALN_THM_RFROMANGLE = 1,  /* RFromAngle(ang0), CThmScan.cpp:329-366 */
    ALN_THM_PRIOR = 2,       /* UsePriorAngles(ang0, hfang), CThmScan.cpp:734-758 */
    ALN_THM_SCAN_HUNT = 3,   /* AngleScanSel(ang0, hfang, step, false) + PeakHunt(step*0.075) */
    ALN_THM_SCAN_MAXR = 4,   /* AngleScanMaxR(ang0, hfang, step, favorCenter), :431-493 */
    ALN_THM_POSTTWEAKS = 5,  /* PostTweaks(best), CThmScan.cpp:796-802 (aln_thm_finish_batch) */
    ALN_THM_FULLRES = 6      /* FinishAtFullRes(best), CThmScan.cpp:810-842 (aln_thm_finish_batch) */
};

/* Runs one CThmScan search per pair, all pairs together: every correlator
 * call of a stage (scan, fine scan, each bracket step) over all pairs is one
 * GPU batch.  Results equal the reference's search on each pair. */
int aln_thm_search_batch(aln_ctx *ctx, int npairs, const aln_thumbs *thumbs,
                         const aln_thm_params *params, int mode, double ang0,
                         double hfang, double step, aln_thm_result *out);

/* CThmScan's finishing stages for many pairs (mode ALN_THM_POSTTWEAKS or
 * ALN_THM_FULLRES), each pair from prior[k] (its best record: A, X, Y, R)
 * and the sweep object's pretweak transform prior_tptwk[6k..6k+5] (TAffine
 * t[0..5]; NULL: identity).  For FinishAtFullRes the thumbs are the
 * full-resolution records and prior X, Y are already scaled to them (as
 * 1_DMesh/CThmUtil.cpp:941-949 does).  out_tptwk (may be NULL) receives the
 * pretweak transform after the call (6 per pair). */
int aln_thm_finish_batch(aln_ctx *ctx, int npairs, const aln_thumbs *thumbs,
                         const aln_thm_params *params, int mode, const aln_thm_result *prior,
                         const double *prior_tptwk, aln_thm_result *out, double *out_tptwk);

/* One CThmScan member-function call per pair (0_GEN/CThmScan.cpp:205-842),
 * from and to the object's state: best[k] is the CorRec the member function
 * takes by reference (A, X, Y, R, T in and out; err is the object's err,
 * set only where the member function sets it; ncalls counts this call's
 * correlator calls) and tptwk[6k..6k+5] the object's pretweak transform
 * (TAffine t[0..5], in and out; NULL: identity, not returned).  All pairs
 * run together: each stage's correlator calls over all pairs are one GPU
 * batch.  op and args[4k..4k+3] = (a0, a1, a2, a3) of pair k:
 *   ALN_THMOP_RFROMANGLE    RFromAngle(best, deg = a0)
 *   ALN_THMOP_SCAN_MAXR     AngleScanMaxR(best, center = a0, hlfwid = a1, step = a2,
 *                           favorCenter = a3 != 0)
 *   ALN_THMOP_SCAN_CONSTXY  AngleScanConstXY(best, a0, a1, a2)
 *   ALN_THMOP_SCAN_SEL      AngleScanSel(best, a0, a1, a2, a3 != 0)
 *   ALN_THMOP_SCAN_TWEAKS   AngleScanWithTweaks(best, a0, a1, a2)
 *   ALN_THMOP_PEAKHUNT      PeakHunt(best, hlfwid = a1)
 *   ALN_THMOP_PRIOR         UsePriorAngles(best, ang0 = a0, hfangpr = a1)
 *   ALN_THMOP_DENOVO        DenovoBestAngle(best, ang0 = a0, hfangdn = a1, step = a2)
 *   ALN_THMOP_PRETWEAKS     Pretweaks(bestR = a0, deg = a1) (best untouched)
 *   ALN_THMOP_POSTTWEAKS    PostTweaks(best)
 *   ALN_THMOP_FULLRES       FinishAtFullRes(best)
 * a1..a3 must be equal for every pair of a scan or hunt call.  ret[k]
 * (may be NULL) receives the member function's return value: R for the
 * scans and PeakHunt, 1 / 0 for the bool ones, 0 for the void ones.
 * PostTweaks and FinishAtFullRes also set the object's useCorrR and disc
 * (SetDisc((int)X, (int)Y, 40 or 80, ...)): the caller applies those to its
 * settings for later calls. */
enum {
    ALN_THMOP_RFROMANGLE = 0,
    ALN_THMOP_SCAN_MAXR = 1,
    ALN_THMOP_SCAN_CONSTXY = 2,
    ALN_THMOP_SCAN_SEL = 3,
    ALN_THMOP_SCAN_TWEAKS = 4,
    ALN_THMOP_PEAKHUNT = 5,
    ALN_THMOP_PRIOR = 6,
    ALN_THMOP_DENOVO = 7,
    ALN_THMOP_PRETWEAKS = 8,
    ALN_THMOP_POSTTWEAKS = 9,
    ALN_THMOP_FULLRES = 10
};
int aln_thm_call_batch(aln_ctx *ctx, int npairs, const aln_thumbs *thumbs,
                       const aln_thm_params *params, int op, const double *args,
                       aln_thm_result *best, double *tptwk, double *ret);

/* MakeThumbs' binning and normalisation (1_DMesh/CThmUtil.cpp:470-523):
 * DecimateVector (0_GEN/Maths.cpp:1315-1364) then, when normalize != 0,
 * Normalize (Maths.cpp:192-212), for n overlap rasters at once.  Image k
 * (any dtype, host or device memory) holds the point list in raster order:
 * the pixels with mask[k][x + stride*y] != 0 (mask NULL or mask[k] NULL:
 * every pixel), its bounding-box corner at (0, 0).  Output k (host or
 * device memory): the ceil(w/lbin) x ceil(h/lbin) grid of bin averages
 * out_vals[k] (FP64, [y][x]) and its presence mask out_mask[k] (1 where the
 * bin's point count -- a uint8 counter, so taken mod 256 as the reference's
 * -- is non-zero; absent bins hold 0), normalised to mean 0 and sample sd 1
 * over the present bins; out_sd[k] (may be NULL) receives that sd (0 with
 * fewer than two bins).  The numbers are the reference's bit for bit (the
 * same sums in the same order).  The present bins are the decimated point
 * list: an aln_thumbs A grid with a_mask = out_mask, or a B raster.  At most
 * 65535 images per call. */
int aln_decimate_batch(aln_ctx *ctx, int n, const aln_image *in,
                       const unsigned char *const *mask, int lbin, int normalize,
                       double *const *out_vals, unsigned char *const *out_mask, double *out_sd);

/* ImageFromValuesAndPoints with DistributePixel (0_GEN/Geometry.cpp:661-685,
 * 0_GEN/Maths.h:236-276) on the device: n points xy[2i], xy[2i+1] with
 * values v[i] (host) painted into a w x h raster whose corner is (xmin,
 * ymin), bilinear weights for fractional points, duplicates adding.  The
 * raster stays in the context's device memory (slot 0 or 1, reused by the
 * next call with that slot) and *out describes it (FP64, on_device = 1,
 * x0 = xmin, y0 = ymin), ready for the correlators; host_copy (may be NULL)
 * receives a copy (w x h doubles).  Per-pixel sums are exact 64-bit fixed
 * point at the finest scale the largest |v| allows, so the raster does not
 * depend on the order the points land in. */
int aln_points_image(aln_ctx *ctx, int slot, int n, const double *xy, const double *v,
                     int xmin, int ymin, int w, int h, aln_image *out, double *host_copy);

/* ---- ApproximateMatch ---------------------------------------------------
 * 1_DMesh/ApproximateMatch.cpp:115-194 for many tile pairs: CThmUtil's Crop
 * (1_DMesh/CThmUtil.cpp:385-426: the overlap boxes BoxesFromShifts gives for
 * XYCONF * Tab's translation, or the whole tiles), MakeThumbs (:470-523),
 * the sweep (:607-633) of a CThmScan set up as ApproximateMatch.cpp:147-154
 * does, and Finish (:889-971: PostTweaks, FinishAtFullRes,
 * IsectToImageCoords, the LIMXY test).  The tiles' connected regions are the
 * whole tiles, px.scl = 1 and Tdfm = identity. */
typedef struct aln_tile_pair {
    aln_image a, b;          /* two tiles of equal size and pixel type */
    double tabx, taby;       /* Tab: the translation of a into b's frame (px) */
} aln_tile_pair;

typedef struct aln_approx_params {
    double xyconf;           /* XYCONF: crop to the overlap Tab predicts (0: whole tiles) */
    int olap1d;              /* OLAP1D */
    long long olap2d;        /* OLAP2D */
    int thmdec;              /* THMDEC (1..255) */
    int mode_prior;          /* 1: UsePriorAngles(ang0, hfangpr) (MODE 'C');
                                0: DenovoBestAngle(ang0, hfangdn, 0.5) */
    double ang0, hfangdn, hfangpr;
    double rthresh, nbmaxht; /* RTRSH, NBMXHT */
    int pretweak, tweaks;    /* PRETWEAK (sweep), TWEAKS (PostTweaks) */
    int limxy;               /* LIMXY (0: no test) */
} aln_approx_params;

typedef struct aln_approx_result {
    int status;              /* 0 a guess; 1 crop too small; 2 thumbnails too small
                                or flat; 3 the sweep failed (err); 4 LIMXY reject */
    int err;                 /* CThmScan err */
    double A, X, Y, R;       /* the final record, X / Y in tile coordinates */
    double T[6];             /* the guess (TAffine t[0..5]) */
    double sweep[4];         /* A, X, Y, R after the sweep (thumbnail units) */
    int crop[4];             /* crop origins: a's (x, y), b's (x, y) */
    int crop_w, crop_h;
} aln_approx_result;

int aln_approx_match_batch(aln_ctx *ctx, int n, const aln_tile_pair *pairs,
                           const aln_approx_params *params, aln_approx_result *out);

/* ---- tile conditioning (PixPair::Load, 0_GEN/CPixPair.cpp:209-494) ------
 * aln_pixpair_dims: the working size PixPair::Load downsamples a w x h tile
 * to (halving while a side exceeds max1dpix; max1dpix <= 0: no
 * downsampling); ALN_NO_PEAK when w, h are not multiples of the scale (the
 * reference's "Dimensions not multiple of scale" failure).
 * aln_pixpair_condition: one uint8 tile (Raster8FromAny's) through LegPolyFlatten of
 * the given order (0_GEN/Maths.cpp:1006-1085) and Normalize, then, when
 * r2 > 0, the DoG band-pass of radii r1 < r2 (MakeDoGKernel + Convolve +
 * Normalize), then the box downsampling.  vfy (may be NULL) receives the
 * flattened image at the working size (PixPair's avs_vfy), aln the image the
 * matcher correlates (avs_aln: DoG'd when r2 > 0); both ws x hs doubles on
 * the host. */
int aln_pixpair_dims(int w, int h, int max1dpix, int *ws, int *hs, int *scl);
int aln_pixpair_condition(aln_ctx *ctx, const aln_image *tile, int order, int r1, int r2,
                          int max1dpix, double *vfy, double *aln);

/* ThmPair table entry (0_GEN/PipeFiles.h:146-152): a tile pair's match. */
typedef struct aln_thmpair {
    int atl, acr, btl, bcr;  /* tile ids and connected-region ids of a and b */
    int err;                 /* CThmScan err */
    double A, R;             /* angle (deg) and correlation */
    double T[6];             /* the a -> b transform (TAffine t[0..5]) */
} aln_thmpair;

/* Appends n entries to <dir>/ThmPair_<alr>^<blr>.txt (dir NULL or "": the
 * working directory), writing WriteThmPairHdr's header line first when the
 * table is new, each entry in WriteThmPair's format
 * (0_GEN/PipeFiles.cpp:1282-1360); entries with a negative tile id are
 * skipped, as there.  Appends from several processes are serialised with a
 * file lock. */
int aln_thmpair_write(const char *dir, int alr, int blr, int n, const aln_thmpair *recs);

/* Reads the table's entries (ReadAllThmPair, 0_GEN/PipeFiles.cpp:1216-1280):
 * returns how many there are (entries beyond cap are counted, not stored),
 * or a negative status. */
int aln_thmpair_read(const char *dir, int alr, int blr, int cap, aln_thmpair *out);

/* ---- mesh optimizer ---------------------------------------------------
 * GradDescStep, CorrVectors and ImproveControlPts of 0_GEN/Correlation.cpp
 * (declared Correlation.h:127-152), which 1_DMesh/ImproveMesh.cpp:503 and
 * 1_DMesh/InSectionOverlap.cpp:303 call after the FFT match to deform a
 * triangle (or box) mesh of control points for the best correlation.
 *
 * The reference's multipliers am are nm dense rows of nc doubles, all zero
 * but the three or four of the point's triangle or box.  Here each row is
 * compressed to k slots: am_idx[i*k + s] the control point (ascending
 * within the row, -1 for an unused slot) and am_w[i*k + s] its multiplier.
 * Dropping the zero terms leaves every per-point sum as the reference
 * computes it; the sums over points run in a fixed blocked order on the GPU,
 * so the results equal the reference's to FP64 rounding of those sums. */
#define ALN_MESH_MAX_NC 128   /* control points per job */
#define ALN_MESH_MAX_K 16     /* multiplier slots per point */

typedef struct aln_mesh_job {
    int nc;                   /* control points, 1..ALN_MESH_MAX_NC */
    double *ac;               /* nc x 2 (x, y) in B's frame, host: start in,
                                 optimised points out (ImproveControlPts' ac) */
    int nm, k;                /* points of region A; slots per point */
    const int *am_idx;        /* nm x k */
    const double *am_w;       /* nm x k */
    const double *av;         /* nm values of A, normalised (mean 0, sd 1) */
    const double *bimg;       /* w x h raster of B, row-major (w >= 2, h >= 2) */
    int w, h;
    double ini_thresh, fin_thresh;   /* ImproveControlPts' iniThresh, finThresh */
    int on_device;            /* 1: am_idx, am_w, av and bimg are device
                                 pointers on the context's device */
} aln_mesh_job;

typedef struct aln_mesh_result {
    int status;               /* ALN_OK */
    double corr;              /* ImproveControlPts' return value: the final
                                 correlation, 0 when the start was below
                                 ini_thresh, the start when fin_thresh < 0 */
    double corr0;             /* the starting correlation */
    int evals;                /* gradient evaluations after the first */
} aln_mesh_result;

/* ImproveControlPts (0_GEN/Correlation.cpp:1605-1721) for n meshes at once:
 * the gradient evaluations of all live jobs share each launch; every job
 * keeps the reference's step rule (10 px halving to 0.05, three small
 * improvements in a row end it).  jobs[i].ac is updated in place. */
int aln_improve_control_pts_batch(aln_ctx *ctx, int n, const aln_mesh_job *jobs,
                                  aln_mesh_result *out);

/* GradDescStep (0_GEN/Correlation.cpp:1403-1478) at job->ac: bnew (nm,
 * NormalizeNonZeros applied) and dRdc (nc x 2) into host buffers; either
 * may be NULL.  *corr (may be NULL) receives CorrVectors(av, bnew). */
int aln_grad_desc_step(aln_ctx *ctx, const aln_mesh_job *job, double *bnew, double *drdc,
                       double *corr);

/* CorrVectors (0_GEN/Correlation.cpp:1490-1530) of two host vectors of n
 * doubles: *out the correlation, *nnz (may be NULL) the count of products
 * not below 1e-8 in magnitude. */
int aln_corr_vectors(aln_ctx *ctx, const double *a, const double *b, int n, double *out,
                     int *nnz);

/* ---- allocation-free CorrPatches: no counterpart in the reference ---- */

/* Size of the device scratch array behind aln_corr_patches_noalloc. */
#define ALN_NOALLOC_SCRATCH_MIB 32

/*
 * CorrPatches for callers that cannot allocate device memory -- e.g. code
 * running inside a caller-managed memory pool or arena, or a plugin whose
 * host forbids cudaMalloc/cudaFree once it is running (allocation there would
 * synchronise the device or fragment the pool).  It computes what
 * aln_corr_patches computes, but allocates nothing: no cudaMalloc, no
 * cudaFree, no allocating library routine, no host heap.
 *
 * Work space comes from one file-scope device array of
 * ALN_NOALLOC_SCRATCH_MIB MiB that every GPU loading this library keeps until
 * the process exits.  A pair whose FFT work space does not fit is rejected
 * with ALN_ERR_UNSUPPORTED (message from aln_last_error(NULL)); 32 MiB holds,
 * for example, one 512 x 512 pair searched over its whole lag window, or a
 * montage strip pair up to 256 x 2048 with a disc.
 *
 * Inputs: a and b must be device pointers on the calling thread's current
 * device (on_device = 1; memory of another device is rejected with
 * ALN_ERR_ARG).  Output: *out in host memory.  The call runs on `stream` (a
 * cudaStream_t, NULL for the default stream) and is synchronous: it returns
 * after the result is copied back.
 *
 * Its kernels are the library's general-size FFT kernels on the caller's
 * frame (wide pairs are not transposed), so it agrees with aln_corr_patches
 * to FP32 rounding, not bit for bit: the same integer peak wherever the
 * top-two margin of r exceeds 1e-3, r within 1e-4, dx and dy within 0.01 px.
 *
 * The first call on each device performs a one-time set-up there (looks up
 * the scratch array's device address, fills the FFT twiddle table in it,
 * enables the large shared-memory kernel configurations).  Every call
 * synchronises its stream and copies through host memory, so no call, the
 * first or any later one, may be made while a stream of the device is being
 * captured into a CUDA graph.  All calls on a device share the one
 * scratch array and leave their data in it: calls that overlap on the GPU
 * (several host threads, or several streams) race and must be serialised by
 * the caller.  Every buffer is fully written before it is read, so no
 * clearing between calls is needed.
 */
int aln_corr_patches_noalloc(const aln_image *a, const aln_image *b, int ox, int oy,
                             int radius, const aln_legal *legal, void *stream,
                             aln_result *out);

/* ---- serving: continuous batching of pair-match requests -------------
 * No reference counterpart (the reference calls the correlator once per
 * pair from its worker threads, 0_GEN/CThmScan.cpp:67-107,
 * 1_DMesh/InSectionOverlap.cpp:190).
 *
 * A server owns `workers` host threads, each with its own context (CUDA
 * streams and workspace) on one device.  Requests wait in one FIFO queue.
 * Whenever a worker is free it takes every waiting request it can admit --
 * up to max_batch requests whose planned device workspace fits its share of
 * mem_budget -- and runs them as one batch; requests that arrive meanwhile
 * form the next batch, and the workers' batches run on the device at the
 * same time.  Sweep requests (ALN_REQ_SWEEP) are batched with each other.
 * A request's result does not depend on the batch it ran in: every job of a
 * batch is computed by the same kernels on its own data.
 *
 * The caller keeps every buffer a request points to alive and unchanged
 * until its reply has been read.  Image b of a request may carry a spectrum
 * key (aln_pair.b_key, aln_image_job.b_key): each worker keeps such spectra
 * resident (cache_bytes per worker) for reuse by later requests. */
typedef struct aln_server aln_server;

typedef struct aln_server_params {
    int device;
    int workers;          /* batches in flight on the device (0: 2) */
    size_t mem_budget;    /* device bytes for request workspaces, all workers
                             together (0: half of the free device memory, at most 16 GiB) */
    int max_batch;        /* requests per batch (0: 4096) */
    size_t cache_bytes;   /* spectrum cache per worker (0: 2 GiB; SIZE_MAX: bounded
                             by free device memory, aln_ctx_set_spectrum_cache) */
} aln_server_params;

enum { ALN_REQ_PATCHES = 0, ALN_REQ_IMAGES = 1, ALN_REQ_SWEEP = 2 };

typedef struct aln_request {
    int kind;                 /* ALN_REQ_* */
    aln_pair pair;            /* ALN_REQ_PATCHES: CorrPatches */
    aln_image_job job;        /* ALN_REQ_IMAGES: CorrImagesR/S */
    aln_thumbs thumbs;        /* ALN_REQ_SWEEP: one CThmScan search ... */
    aln_thm_params thm;       /* ... with these settings */
    int thm_mode;             /* ALN_THM_* */
    double ang0, hfang, step;
} aln_request;

typedef struct aln_reply {
    int status;               /* ALN_OK, or the request's negative error */
    aln_result corr;          /* ALN_REQ_PATCHES / ALN_REQ_IMAGES */
    aln_thm_result sweep;     /* ALN_REQ_SWEEP */
    double queue_ms;          /* submission -> its batch started */
    double total_ms;          /* submission -> result ready */
    int batch_size;           /* requests in that batch */
} aln_reply;

int aln_server_create(const aln_server_params *params, aln_server **out);
/* Stops the workers after their current batch; requests still waiting are
 * answered ALN_ERR_CANCELLED. */
void aln_server_destroy(aln_server *s);
/* Queue one request; *ticket identifies its reply.  ALN_ERR_REFUSED once
 * the server is stopping. */
int aln_server_submit(aln_server *s, const aln_request *req, unsigned long long *ticket);
/* Wait up to timeout_ms (< 0: no limit) for the reply of `ticket`; the reply
 * is handed over once (a second wait returns ALN_ERR_ARG).  ALN_ERR_TIMEOUT
 * if it is not ready in time. */
int aln_server_wait(aln_server *s, unsigned long long ticket, int timeout_ms, aln_reply *out);
/* Hand over up to `cap` finished replies (any tickets), waiting up to
 * timeout_ms for the first; returns how many. */
int aln_server_collect(aln_server *s, int cap, int timeout_ms, unsigned long long *tickets,
                       aln_reply *out);
/* which: 0 requests submitted, 1 finished, 2 batches run, 3 waiting now,
 * 4 spectrum-cache hits, 5 fills, 6 evictions, 7 device bytes the caches
 * hold (4-7 summed over the workers). */
long long aln_server_counter(aln_server *s, int which);
const char *aln_server_last_error(aln_server *s);

#ifdef __cplusplus
}
#endif
