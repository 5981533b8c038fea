// aln_mesh.cuh -- the mesh optimizer on the GPU: GradDescStep, CorrVectors
// and ImproveControlPts (0_GEN/Correlation.cpp:1403-1721), for many
// region-to-region meshes per call.  Included by aln_corr.cu.
//
// Each iteration of ImproveControlPts is one gradient evaluation of every
// live job:
//   k_mesh_prep    per job: the candidate control points ac + S dRdc
//                  (S = step / |dRdc|), or ac itself for the first evaluation
//   k_mesh_eval    per point: its position from the control points, B
//                  bilinear there (bnew), the gradient terms av * dB/dx;
//                  per block: dRdc over its points and the sums of the
//                  nonzero bnew (NormalizeNonZeros), written as partials
//   k_mesh_stats   per job: the partials summed in block order: dRdc, mean
//                  and sample sd of the nonzero bnew
//   k_mesh_corr    per point: the normalised bnew times av (CorrVectors),
//                  partial sums and small-product counts per block
//   k_mesh_decide  per job: the correlation; accept the candidate or halve
//                  the step; the convergence test; done flags
// Every sum runs in a fixed order (per warp in point order, then warps,
// then blocks), so a job's numbers do not depend on the batch or the run.
// They differ from the reference's single sequential loop by FP64 rounding
// of the sums only: per-point arithmetic uses explicit round-to-nearest
// operations in the reference's order (no contraction).
#pragma once

#define MESH_THREADS 256
#define MESH_WARPS (MESH_THREADS / 32)
#define MESH_CPL ((ALN_MESH_MAX_NC + 31) / 32)   // control points per lane

struct MeshDev {
    // inputs (device)
    const int *idx;
    const double *wts;
    const double *av;
    const double *bimg;
    double *bnew;
    double *part;         // [nblk][2 nc + 3]: dRdc partials, sum b, sum b^2, n
    double *part2;        // [nblk][2]: sum of products, small-product count
    int nc, nm, k, w, h, nblk;
    double ini, fin;
    // state
    double ac[2 * ALN_MESH_MAX_NC], acn[2 * ALN_MESH_MAX_NC];
    double drdc[2 * ALN_MESH_MAX_NC], drdcn[2 * ALN_MESH_MAX_NC];
    double corr, corr_last, corr0, step, avg, sd;
    int inarow, phase, done, evals, status;
};

// exact FP64 steps in the reference's order (nvcc would otherwise contract)
__device__ __forceinline__ double mmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double madd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double msub(double a, double b) { return __dsub_rn(a, b); }

// Candidate control points of each live job.  ImproveControlPts, Correlation.cpp:1660-1683.
__global__ void k_mesh_prep(MeshDev *jobs, int n)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    MeshDev &m = jobs[j];
    if (m.done)
        return;
    if (m.phase == 0) {
        for (int c = 0; c < 2 * m.nc; ++c)
            m.acn[c] = m.ac[c];
        return;
    }
    double S = 0.0;
    for (int c = 0; c < m.nc; ++c)
        S = madd(S, madd(mmul(m.drdc[2 * c], m.drdc[2 * c]),
                         mmul(m.drdc[2 * c + 1], m.drdc[2 * c + 1])));
    if (!S) {   // all derivatives zero
        m.done = 1;
        return;
    }
    S = __ddiv_rn(m.step, __dsqrt_rn(S));
    for (int c = 0; c < 2 * m.nc; ++c)
        m.acn[c] = madd(m.ac[c], mmul(S, m.drdc[c]));
}

// GradDescStep's per-point loop, Correlation.cpp:1423-1475.  grid (nblk,
// njobs): block b of a job owns points [b * per, (b + 1) * per); inside it,
// warp q owns a contiguous sub-range and walks it 32 points at a time.
__global__ void __launch_bounds__(MESH_THREADS) k_mesh_eval(MeshDev *jobs)
{
    __shared__ double sacn[2 * ALN_MESH_MAX_NC];
    __shared__ double swarp[MESH_WARPS][2 * ALN_MESH_MAX_NC];
    __shared__ double sstat[MESH_WARPS][3];
    MeshDev &m = jobs[blockIdx.y];
    if (m.done || (int)blockIdx.x >= m.nblk)
        return;
    const int nc = m.nc, k = m.k, w = m.w, h = m.h;
    for (int c = threadIdx.x; c < 2 * nc; c += blockDim.x)
        sacn[c] = m.acn[c];
    __syncthreads();
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    const long long per = ((long long)m.nm + m.nblk - 1) / m.nblk;
    const long long b0 = (long long)blockIdx.x * per;
    const long long b1 = min((long long)m.nm, b0 + per);
    const long long wper = (b1 - b0 + MESH_WARPS - 1) / MESH_WARPS;
    const long long w0 = min(b1, b0 + wq * wper), w1 = min(b1, w0 + wper);
    double accx[MESH_CPL], accy[MESH_CPL];
#pragma unroll
    for (int q = 0; q < MESH_CPL; ++q)
        accx[q] = accy[q] = 0.0;
    double ssum = 0.0, ssq = 0.0, scnt = 0.0;
    for (long long g = w0; g < w1; g += 32) {
        const long long i = g + lane;
        const bool ok = i < w1;
        double gx = 0.0, gy = 0.0;
        if (ok) {
            const int *ix = m.idx + i * k;
            const double *aw = m.wts + i * k;
            double x = 0.0, y = 0.0;
            for (int s = 0; s < k; ++s) {
                const int c = ix[s];
                if (c >= 0) {
                    x = madd(x, mmul(aw[s], sacn[2 * c]));
                    y = madd(y, mmul(aw[s], sacn[2 * c + 1]));
                }
            }
            double b = 0.0;
            if (!(x < 0.0 || x >= w - 1 || y < 0.0 || y >= h - 1)) {
                const int xl = (int)x, xr = xl + 1, yl = (int)y, yu = yl + 1;
                const double alpha = msub(x, (double)xl), beta = msub(y, (double)yl);
                const double ll = m.bimg[(long long)w * yl + xl];
                const double ul = m.bimg[(long long)w * yu + xl];
                const double ur = m.bimg[(long long)w * yu + xr];
                const double lr = m.bimg[(long long)w * yl + xr];
                const double t = msub(lr, ll), u = msub(ul, ll);
                const double v = madd(msub(msub(ll, lr), ul), ur);
                b = madd(madd(madd(ll, mmul(alpha, t)), mmul(beta, u)),
                         mmul(mmul(alpha, beta), v));
                const double a = m.av[i];
                gx = mmul(madd(t, mmul(beta, v)), a);
                gy = mmul(madd(u, mmul(alpha, v)), a);
            }
            m.bnew[i] = b;
            if (b != 0.0) {
                ssum = madd(ssum, b);
                ssq = madd(ssq, mmul(b, b));
                scnt += 1.0;
            }
        }
        // dRdc: the warp's points in order, lane l holding control points
        // l, l + 32, ...; each point's slots broadcast from its lane
        const int np = (int)min((long long)32, w1 - g);
        for (int p = 0; p < np; ++p) {
            const double px = __shfl_sync(0xffffffff, gx, p);
            const double py = __shfl_sync(0xffffffff, gy, p);
            if (px == 0.0 && py == 0.0)
                continue;   // outside B: no term (the reference skips the point)
            const long long ip = g + p;
            for (int s = 0; s < k; ++s) {
                const int c = m.idx[ip * k + s];
                if (c < 0 || (c & 31) != lane)
                    continue;
                const double a = m.wts[ip * k + s];
                const int q = c >> 5;
#pragma unroll
                for (int qq = 0; qq < MESH_CPL; ++qq)
                    if (qq == q) {
                        accx[qq] = madd(accx[qq], mmul(a, px));
                        accy[qq] = madd(accy[qq], mmul(a, py));
                    }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < MESH_CPL; ++q) {
        const int c = q * 32 + lane;
        if (c < nc) {
            swarp[wq][2 * c] = accx[q];
            swarp[wq][2 * c + 1] = accy[q];
        }
    }
    // the warp's nonzero-bnew sums: a fixed xor tree
    for (int o = 16; o > 0; o >>= 1) {
        ssum = madd(ssum, __shfl_xor_sync(0xffffffff, ssum, o));
        ssq = madd(ssq, __shfl_xor_sync(0xffffffff, ssq, o));
        scnt += __shfl_xor_sync(0xffffffff, scnt, o);
    }
    if (lane == 0) {
        sstat[wq][0] = ssum;
        sstat[wq][1] = ssq;
        sstat[wq][2] = scnt;
    }
    __syncthreads();
    double *out = m.part + (long long)blockIdx.x * (2 * nc + 3);
    for (int c = threadIdx.x; c < 2 * nc + 3; c += blockDim.x) {
        double s = 0.0;
        for (int q = 0; q < MESH_WARPS; ++q)
            s = madd(s, c < 2 * nc ? swarp[q][c] : sstat[q][c - 2 * nc]);
        out[c] = s;
    }
}

// The block partials summed in block order: dRdc of the candidate, the
// mean and sample sd of its nonzero bnew (MeanStd::Stats, Maths.cpp:111-124).
__global__ void k_mesh_stats(MeshDev *jobs)
{
    MeshDev &m = jobs[blockIdx.x];
    if (m.done)
        return;
    const int nc = m.nc, stride = 2 * nc + 3;
    for (int c = threadIdx.x; c < stride; c += blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < m.nblk; ++b)
            s = madd(s, m.part[(long long)b * stride + c]);
        if (c < 2 * nc)
            m.drdcn[c] = s;
        else
            m.part[c] = s;   // block 0's slots take the totals (read below)
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const double sum = m.part[2 * nc], sum2 = m.part[2 * nc + 1];
        const double n = m.part[2 * nc + 2];
        double avg = sum, sd = 0.0;
        if (n > 1.0) {
            avg = __ddiv_rn(avg, n);
            sd = __dsqrt_rn(__ddiv_rn(fmax(msub(sum2, mmul(mmul(n, avg), avg)), 0.0),
                                      msub(n, 1.0)));
        }
        m.avg = avg;
        m.sd = sd;
    }
}

// CorrVectors(av, NormalizeNonZeros(bnew)), Correlation.cpp:1490-1530.
__global__ void __launch_bounds__(MESH_THREADS) k_mesh_corr(MeshDev *jobs)
{
    __shared__ double sred[MESH_WARPS][2];
    MeshDev &m = jobs[blockIdx.y];
    if (m.done || (int)blockIdx.x >= m.nblk)
        return;
    const long long per = ((long long)m.nm + m.nblk - 1) / m.nblk;
    const long long b0 = (long long)blockIdx.x * per;
    const long long b1 = min((long long)m.nm, b0 + per);
    const double avg = m.avg, sd = m.sd;
    double s = 0.0, nz = 0.0;
    for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        double b = m.bnew[i];
        if (b != 0.0)
            b = __ddiv_rn(msub(b, avg), sd);
        const double prod = mmul(m.av[i], b);
        s = madd(s, prod);
        if (fabs(prod) < 1.0E-8)
            nz += 1.0;
    }
    for (int o = 16; o > 0; o >>= 1) {
        s = madd(s, __shfl_xor_sync(0xffffffff, s, o));
        nz += __shfl_xor_sync(0xffffffff, nz, o);
    }
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    if (lane == 0) {
        sred[wq][0] = s;
        sred[wq][1] = nz;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, c = 0.0;
        for (int q = 0; q < MESH_WARPS; ++q) {
            a = madd(a, sred[q][0]);
            c += sred[q][1];
        }
        m.part2[2 * blockIdx.x] = a;
        m.part2[2 * blockIdx.x + 1] = c;
    }
}

// The correlation of the candidate and ImproveControlPts' decisions,
// Correlation.cpp:1628-1715.
__global__ void k_mesh_decide(MeshDev *jobs, int n)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n)
        return;
    MeshDev &m = jobs[j];
    if (m.done)
        return;
    double sum2 = 0.0, nz = 0.0;
    for (int b = 0; b < m.nblk; ++b) {
        sum2 = madd(sum2, m.part2[2 * b]);
        nz += m.part2[2 * b + 1];
    }
    double N = (double)m.nm;
    if (!isfinite(sum2)) {
        nz = N;
        sum2 = 0.0;
    }
    N -= nz;
    const double c_new = N > 0.0 ? __ddiv_rn(sum2, N) : 0.0;
    if (m.phase == 0) {
        m.corr = m.corr_last = m.corr0 = c_new;
        for (int c = 0; c < 2 * m.nc; ++c)
            m.drdc[c] = m.drdcn[c];
        m.phase = 1;
        m.step = 10.0;
        m.inarow = 0;
        if (c_new < m.ini) {
            m.corr = 0.0;
            m.done = 1;
        } else if (m.fin < 0)
            m.done = 1;
        return;
    }
    m.evals++;
    if (c_new > m.corr) {
        for (int c = 0; c < 2 * m.nc; ++c) {
            m.ac[c] = m.acn[c];
            m.drdc[c] = m.drdcn[c];
        }
        m.corr_last = m.corr;
        m.corr = c_new;
    } else
        m.step = __ddiv_rn(m.step, 2.0);
    if (m.step <= 2.0 && msub(m.corr, m.corr_last) < 0.0001) {
        if (++m.inarow >= 3)
            m.done = 1;
    } else
        m.inarow = 0;
    if (!(m.step > 0.05))
        m.done = 1;
}

// bnew of each job with NormalizeNonZeros applied (aln_grad_desc_step's output)
__global__ void k_mesh_normalize(MeshDev *jobs)
{
    MeshDev &m = jobs[blockIdx.y];
    const double avg = m.avg, sd = m.sd;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < m.nm;
         i += (long long)gridDim.x * blockDim.x)
        if (m.bnew[i] != 0.0)
            m.bnew[i] = __ddiv_rn(msub(m.bnew[i], avg), sd);
}

__global__ void k_mesh_live(const MeshDev *jobs, int n, int *live)
{
    __shared__ int s;
    if (threadIdx.x == 0)
        s = 0;
    __syncthreads();
    int c = 0;
    for (int j = threadIdx.x; j < n; j += blockDim.x)
        c += jobs[j].done ? 0 : 1;
    atomicAdd(&s, c);
    __syncthreads();
    if (threadIdx.x == 0)
        *live = s;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// blocks per job: at least 4096 points per block (warps walk >= 512 each)
static int mesh_nblk(int nm) { return std::max(1, std::min(2048, (nm + 4095) / 4096)); }

// The whole ImproveControlPts loop for jobs[0..n) (n <= 65535).  initial_only:
// one evaluation at ac (GradDescStep), bnew left normalised on the device
// for the caller (*dbnew).
static int mesh_run(aln_ctx *ctx, int n, const aln_mesh_job *jobs, aln_mesh_result *out,
                    bool initial_only, std::vector<MeshDev> &hm, char **dev_base)
{
    if (!ctx || n < 0 || n > 65535 || (n && (!jobs || (!out && !initial_only))))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "mesh: bad arguments") : ALN_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    size_t bytes = al256((size_t)n * sizeof(MeshDev));
    int maxblk = 1;
    for (int j = 0; j < n; ++j) {
        const aln_mesh_job &J = jobs[j];
        if (J.nc < 1 || J.nc > ALN_MESH_MAX_NC || J.k < 1 || J.k > ALN_MESH_MAX_K ||
            J.nm < 0 || J.w < 2 || J.h < 2 || !J.ac ||
            (J.nm > 0 && (!J.am_idx || !J.am_w || !J.av)) || !J.bimg)
            return set_err(ctx, ALN_ERR_ARG, "mesh job %d: bad sizes or pointers", j);
        const size_t nm = (size_t)J.nm;
        if (!J.on_device)
            bytes += al256(nm * J.k * sizeof(int)) + al256(nm * J.k * sizeof(double)) +
                     al256(nm * sizeof(double)) + al256((size_t)J.w * J.h * sizeof(double));
        const int nb = mesh_nblk(J.nm);
        maxblk = std::max(maxblk, nb);
        bytes += al256(std::max<size_t>(nm, 1) * sizeof(double)) +
                 al256((size_t)nb * (2 * J.nc + 3) * sizeof(double)) +
                 al256((size_t)nb * 2 * sizeof(double));
    }
    bytes += 256;   // the live counter
    if (int rc = ensure_ws(ctx, bytes))
        return rc;
    char *p = ctx->ws;
    MeshDev *dm = (MeshDev *)p;
    p += al256((size_t)n * sizeof(MeshDev));
    cudaStream_t st = ctx->stream;
    hm.assign(n, MeshDev());
    for (int j = 0; j < n; ++j) {
        const aln_mesh_job &J = jobs[j];
        MeshDev &m = hm[j];
        memset(&m, 0, sizeof m);
        const size_t nm = (size_t)J.nm;
        auto put = [&](const void *src, size_t b) -> void * {
            void *d = p;
            p += al256(b);
            if (b)
                cudaMemcpyAsync(d, src, b, cudaMemcpyHostToDevice, st);
            ctx->h2d_bytes += (long long)b;
            return d;
        };
        if (J.on_device) {
            m.idx = J.am_idx;
            m.wts = J.am_w;
            m.av = J.av;
            m.bimg = J.bimg;
        } else {
            m.idx = (const int *)put(J.am_idx, nm * J.k * sizeof(int));
            m.wts = (const double *)put(J.am_w, nm * J.k * sizeof(double));
            m.av = (const double *)put(J.av, nm * sizeof(double));
            m.bimg = (const double *)put(J.bimg, (size_t)J.w * J.h * sizeof(double));
        }
        m.nblk = mesh_nblk(J.nm);
        m.bnew = (double *)p;
        p += al256(std::max<size_t>(nm, 1) * sizeof(double));
        m.part = (double *)p;
        p += al256((size_t)m.nblk * (2 * J.nc + 3) * sizeof(double));
        m.part2 = (double *)p;
        p += al256((size_t)m.nblk * 2 * sizeof(double));
        m.nc = J.nc;
        m.nm = J.nm;
        m.k = J.k;
        m.w = J.w;
        m.h = J.h;
        m.ini = initial_only ? -1e300 : J.ini_thresh;
        m.fin = initial_only ? -1.0 : J.fin_thresh;
        for (int c = 0; c < 2 * J.nc; ++c)
            m.ac[c] = J.ac[c];
    }
    int *dlive = (int *)p;
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dm, hm.data(), (size_t)n * sizeof(MeshDev), cudaMemcpyHostToDevice, st));
    int *hlive = nullptr;
    CK(cudaMallocHost((void **)&hlive, sizeof(int)));
    const int jb = (n + 127) / 128;
    int rc = ALN_OK;
    // an iteration cap far above the reference's step rule allows in practice
    // (each evaluation halves the step or raises the correlation, which is
    // bounded by 1)
    const int kMaxIter = 1 << 20;
    for (int it = 0; n > 0 && it < kMaxIter; ++it) {
        LAUNCH(ctx, "k_mesh_prep", k_mesh_prep, jb, 128, 0, dm, n);
        LAUNCH(ctx, "k_mesh_eval", k_mesh_eval, dim3(maxblk, n), MESH_THREADS, 0, dm);
        LAUNCH(ctx, "k_mesh_stats", k_mesh_stats, n, 256, 0, dm);
        LAUNCH(ctx, "k_mesh_corr", k_mesh_corr, dim3(maxblk, n), MESH_THREADS, 0, dm);
        LAUNCH(ctx, "k_mesh_decide", k_mesh_decide, jb, 128, 0, dm, n);
        ctx->launches += 5;
        if (initial_only)
            break;
        if ((it & 3) == 3 || it == 0) {
            k_mesh_live<<<1, 256, 0, st>>>(dm, n, dlive);
            ctx->launches++;
            cudaMemcpyAsync(hlive, dlive, sizeof(int), cudaMemcpyDeviceToHost, st);
            if (cudaStreamSynchronize(st) != cudaSuccess)
                break;
            if (*hlive == 0)
                break;
            if (it + 1 >= kMaxIter)
                rc = set_err(ctx, ALN_ERR_TIMEOUT, "mesh: iteration cap reached");
        }
    }
    if (initial_only && n > 0) {
        LAUNCH(ctx, "k_mesh_normalize", k_mesh_normalize, dim3(std::min(maxblk * 16, 4096), n),
               256, 0, dm);
        ctx->launches++;
    }
    cudaFreeHost(hlive);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(hm.data(), dm, (size_t)n * sizeof(MeshDev), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    prof_collect(ctx);
    if (!initial_only)
        for (int j = 0; j < n; ++j) {
            const MeshDev &m = hm[j];
            out[j].status = ALN_OK;
            out[j].corr = m.corr;
            out[j].corr0 = m.corr0;
            out[j].evals = m.evals;
            for (int c = 0; c < 2 * m.nc; ++c)
                jobs[j].ac[c] = m.ac[c];
        }
    if (dev_base)
        *dev_base = (char *)dm;
    return rc;
}

extern "C" int aln_improve_control_pts_batch(aln_ctx *ctx, int n, const aln_mesh_job *jobs,
                                             aln_mesh_result *out)
{
    std::vector<MeshDev> hm;
    for (int j0 = 0; j0 < n; j0 += 65535) {
        const int m = std::min(65535, n - j0);
        if (int rc = mesh_run(ctx, m, jobs + j0, out + j0, false, hm, nullptr))
            return rc;
    }
    return n >= 0 ? ALN_OK : (ctx ? set_err(ctx, ALN_ERR_ARG, "mesh: n < 0") : ALN_ERR_ARG);
}

extern "C" int aln_grad_desc_step(aln_ctx *ctx, const aln_mesh_job *job, double *bnew,
                                  double *drdc, double *corr)
{
    if (!ctx || !job)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "grad_desc_step: null job") : ALN_ERR_ARG;
    std::vector<MeshDev> hm;
    if (int rc = mesh_run(ctx, 1, job, nullptr, true, hm, nullptr))
        return rc;
    const MeshDev &m = hm[0];
    if (bnew && m.nm > 0)
        CK(cudaMemcpy(bnew, m.bnew, (size_t)m.nm * sizeof(double), cudaMemcpyDeviceToHost));
    if (drdc)
        for (int c = 0; c < 2 * m.nc; ++c)
            drdc[c] = m.drdc[c];
    if (corr)
        *corr = m.corr0;
    return ALN_OK;
}

// CorrVectors through the optimizer's own reduction: k_mesh_corr over b with
// mean 0 and sd 1 leaves every b as it is ((b - 0) / 1 is b exactly).
extern "C" int aln_corr_vectors(aln_ctx *ctx, const double *a, const double *b, int n,
                                double *out, int *nnz)
{
    if (!ctx || n < 0 || (n && (!a || !b)) || !out)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "corr_vectors: bad arguments") : ALN_ERR_ARG;
    CK(cudaSetDevice(ctx->device));
    const int nb = mesh_nblk(n);
    const size_t bytes = al256(sizeof(MeshDev)) + 2 * al256(std::max(n, 1) * sizeof(double)) +
                         al256((size_t)nb * 2 * sizeof(double));
    if (int rc = ensure_ws(ctx, bytes))
        return rc;
    char *p = ctx->ws;
    MeshDev *dm = (MeshDev *)p;
    p += al256(sizeof(MeshDev));
    double *da = (double *)p;
    p += al256(std::max(n, 1) * sizeof(double));
    double *db = (double *)p;
    p += al256(std::max(n, 1) * sizeof(double));
    MeshDev h;
    memset(&h, 0, sizeof h);
    h.av = da;
    h.bnew = db;
    h.nm = n;
    h.nblk = nb;
    h.part2 = (double *)p;
    h.avg = 0.0;
    h.sd = 1.0;
    h.phase = 1;   // k_mesh_corr only reads avg / sd / bnew / av
    cudaStream_t st = ctx->stream;
    if (n) {
        CK(cudaMemcpyAsync(da, a, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
        CK(cudaMemcpyAsync(db, b, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, st));
    }
    CK(cudaMemcpyAsync(dm, &h, sizeof h, cudaMemcpyHostToDevice, st));
    LAUNCH(ctx, "k_mesh_corr", k_mesh_corr, dim3(nb, 1), MESH_THREADS, 0, dm);
    std::vector<double> part((size_t)nb * 2);
    CK(cudaMemcpyAsync(part.data(), h.part2, part.size() * sizeof(double),
                       cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    prof_collect(ctx);
    // the block partials in block order (k_mesh_decide's sum)
    double sum2 = 0.0, nz = 0.0;
    for (int q = 0; q < nb; ++q) {
        sum2 += part[2 * q];
        nz += part[2 * q + 1];
    }
    double N = (double)n;
    if (!std::isfinite(sum2)) {
        nz = N;
        sum2 = 0.0;
    }
    N -= nz;
    *out = N > 0.0 ? sum2 / N : 0.0;
    if (nnz)
        *nnz = (int)N;
    return ALN_OK;
}
