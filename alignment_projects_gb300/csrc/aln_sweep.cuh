// aln_sweep.cuh -- the CThmScan rotation sweep (0_GEN/CThmScan.cpp) on the
// GPU, included at the end of aln_corr.cu.
//
// Every correlator call of the sweep (RFromAngle -> CorrImagesS,
// CThmScan.cpp:329-366) becomes a job: the thumbnail-A grid points are
// rotated by C.T = R(deg*PI/180) * (Tdfm * Tptwk) (FP64, the reference's
// operation order, PI truncated as GenDefs.h:16), splatted bilinearly into
// the bounding box of the rotated points (k_splat), and correlated with
// thumbnail B by the CorrImagesS pipeline.  A host controller runs the
// sweep logic for many pairs at once: each stage (coarse scan, fine scan,
// one bracket step of PeakHunt, one Pretweaks round) is one GPU batch over
// all pairs still in that stage.
#pragma once

#define ALN_PI_REF 3.14159265358   // GenDefs.h:16, truncated as the reference uses it

// One rotate-and-splat job: rotated A points -> FP32 raster [h1][w1].
struct SplatJob {
    double t0, t1, t3, t4;   // linear part of C.T
    long long T0, T1, T3, T4;   // the same in 2^-40 fixed point
    float i00, i01, i10, i11;   // inverse of the linear part
    float eu, ev;            // half-extents of the preimage of a 2 x 2 pixel square
    int L, B, w1, h1;        // bounding box of the rotated points
    float *out;
    const float *a;          // A values on the grid, a[x + stride*y] (FP32 copy)
    const unsigned char *mask;   // presence (NULL: all present)
    int aw, ah, astride, ax0, ay0;
};

#define SPLAT_FX 40   // fractional bits of the fixed-point coordinates

__global__ void k_f64_to_f32(const double *__restrict__ src, float *__restrict__ dst, size_t n)
{
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}

// grid (ceil(maxw/32), ceil(maxh/32), njobs), block 256: each thread gathers
// four output pixels of a 32 x 32 tile.  A point p = (px, py) lands at
// x = t0 px + t1 py - L, y = t3 px + t4 py - B and adds its value to the
// pixels around it with the bilinear weights of DistributePixel
// (0_GEN/Maths.h:236-276): pixel X receives the weight 1 - |x - X| when
// |x - X| < 1 (that is 1 - alpha at floor(x), alpha at floor(x) + 1), and
// the same in y.  Per pixel the candidate points are the grid points of the
// preimage of the square (X +- 1, Y +- 1); the test itself runs in 2^-40
// fixed point (exact integer arithmetic, 64-bit), the weights and the sum in
// FP32 in a fixed order, so the same transform always gives the same raster
// bit for bit, as the sweep's tie rules need.
__global__ void __launch_bounds__(256) k_splat(const SplatJob *jobs)
{
    const SplatJob &J = jobs[blockIdx.z];
    const int tx0 = blockIdx.x * 32, ty0 = blockIdx.y * 32;
    if (tx0 >= J.w1 || ty0 >= J.h1)
        return;
    const long long ONE = 1ll << SPLAT_FX;
    const int X = tx0 + (threadIdx.x & 31);
    const int gx_lo = J.ax0, gx_hi = J.ax0 + J.aw - 1;
    const int gy_lo = J.ay0, gy_hi = J.ay0 + J.ah - 1;
    for (int k = 0; k < 4; ++k) {
        const int Y = ty0 + (threadIdx.x >> 5) + 8 * k;
        if (X >= J.w1 || Y >= J.h1)
            continue;
        const int Xa = X + J.L, Ya = Y + J.B;   // rotated-frame coordinates
        const float uc = J.i00 * (float)Xa + J.i01 * (float)Ya;
        const float vc = J.i10 * (float)Xa + J.i11 * (float)Ya;
        const int u0 = max(gx_lo, (int)ceilf(uc - J.eu)), u1 = min(gx_hi, (int)floorf(uc + J.eu));
        const int v0 = max(gy_lo, (int)ceilf(vc - J.ev)), v1 = min(gy_hi, (int)floorf(vc + J.ev));
        const long long Xf = (long long)Xa << SPLAT_FX, Yf = (long long)Ya << SPLAT_FX;
        float acc = 0.0f;
        // (dx, dy) = fixed-point offset of point (u, v) from the pixel,
        // stepped exactly: +T0/+T3 per u, +T1/+T4 per v
        long long rx = (long long)u0 * J.T0 + (long long)v0 * J.T1 - Xf;
        long long ry = (long long)u0 * J.T3 + (long long)v0 * J.T4 - Yf;
        for (int v = v0; v <= v1; ++v, rx += J.T1, ry += J.T4) {
            const long long row = (long long)J.astride * (v - J.ay0) - J.ax0;
            long long dx = rx, dy = ry;
            for (int u = u0; u <= u1; ++u, dx += J.T0, dy += J.T3) {
                if (dx <= -ONE || dx >= ONE || dy <= -ONE || dy >= ONE)
                    continue;
                if (J.mask && !J.mask[row + u])
                    continue;
                // 1 - |d| from its top 24 fractional bits: an exact 32-bit
                // integer to FP32 conversion (64-bit ones use the FP64 pipe)
                const float wx = (float)(int)((ONE - (dx < 0 ? -dx : dx)) >> (SPLAT_FX - 24)) *
                                 5.9604644775390625e-8f;
                const float wy = (float)(int)((ONE - (dy < 0 ? -dy : dy)) >> (SPLAT_FX - 24)) *
                                 5.9604644775390625e-8f;
                acc += wx * wy * __ldg(&J.a[row + u]);
            }
        }
        J.out[(long long)Y * J.w1 + X] = acc;
    }
}

// ---------------------------------------------------------------------------
// host: affine algebra of TAffine (TAffine.cpp:60-135,220-232)
// ---------------------------------------------------------------------------

static void aff_one(double t[6])
{
    t[0] = 1; t[1] = 0; t[2] = 0;
    t[3] = 0; t[4] = 1; t[5] = 0;
}

static void aff_mul(double r[6], const double L[6], const double R[6])
{
    double t[6];
    t[0] = L[0] * R[0] + L[1] * R[3];
    t[1] = L[0] * R[1] + L[1] * R[4];
    t[2] = L[0] * R[2] + L[1] * R[5] + L[2];
    t[3] = L[3] * R[0] + L[4] * R[3];
    t[4] = L[3] * R[1] + L[4] * R[4];
    t[5] = L[3] * R[2] + L[4] * R[5] + L[5];
    memcpy(r, t, sizeof t);
}

// NUSelect: 0 Scl, 1 XScl, 2 YScl, 3 XSkw, 4 YSkw, 5 Rot
static void aff_nu(double t[6], int sel, double a)
{
    aff_one(t);
    switch (sel) {
    case 1: t[0] = a; break;
    case 2: t[4] = a; break;
    case 3: t[1] = a; break;
    case 4: t[3] = a; break;
    case 5: {
        const double c = cos(a), s = sin(a);
        t[0] = c; t[1] = -s; t[3] = s; t[4] = c;
        break;
    }
    default: t[0] = a; t[4] = a; break;
    }
}

// ---------------------------------------------------------------------------
// host: one pair's sweep state
// ---------------------------------------------------------------------------

struct ThmRec {
    double A, X, Y, R;
    double T[6];
};

struct ThmPair {
    const aln_thumbs *in;
    std::vector<std::pair<long long, long long>> hull;   // convex hull of A's points
    double Tptwk[6];
    const double *dev_a;            // device copies
    const float *dev_af;            // A's values in FP32 (what the splat reads)
    const unsigned char *dev_mask;
    aln_image dev_b;
    // pretweak sweep records (TCD.vT)
    std::vector<int> Tsel;
    std::vector<double> Ta;
    int ncalls;
    int err;
    ThmRec best;
    int own_disc;                   // SetDisc of this pair (finishing stages)
    int dox, doy, drx, dry;
};

struct Eval {
    int pair;
    double deg;
    int iaux;    // pretweak record, -1: none
    ThmRec *out;
};

static double cross3(const std::pair<long long, long long> &o, const std::pair<long long, long long> &a,
                     const std::pair<long long, long long> &b)
{
    return (double)(a.first - o.first) * (double)(b.second - o.second) -
           (double)(a.second - o.second) * (double)(b.first - o.first);
}

// Monotone-chain hull of the present A grid points (absolute coordinates).
static void make_hull(ThmPair &tp)
{
    const aln_thumbs &T = *tp.in;
    std::vector<std::pair<long long, long long>> pts;
    for (int y = 0; y < T.a_h; ++y) {
        int xl = -1, xr = -1;   // extreme present points of the row suffice
        for (int x = 0; x < T.a_w; ++x)
            if (!T.a_mask || T.a_mask[x + (size_t)T.a_stride * y]) {
                if (xl < 0)
                    xl = x;
                xr = x;
            }
        if (xl >= 0) {
            pts.push_back({xl + T.a_x0, y + T.a_y0});
            if (xr != xl)
                pts.push_back({xr + T.a_x0, y + T.a_y0});
        }
    }
    std::sort(pts.begin(), pts.end());
    pts.erase(std::unique(pts.begin(), pts.end()), pts.end());
    if (pts.size() < 3) {
        tp.hull = pts;
        return;
    }
    std::vector<std::pair<long long, long long>> h(2 * pts.size());
    size_t k = 0;
    for (size_t i = 0; i < pts.size(); ++i) {
        while (k >= 2 && cross3(h[k - 2], h[k - 1], pts[i]) <= 0)
            --k;
        h[k++] = pts[i];
    }
    for (size_t i = pts.size() - 1, t = k + 1; i > 0; --i) {
        while (k >= t && cross3(h[k - 2], h[k - 1], pts[i - 1]) <= 0)
            --k;
        h[k++] = pts[i - 1];
    }
    h.resize(k - 1);
    tp.hull = h;
}

struct SweepCtx {
    aln_ctx *ctx;
    std::vector<ThmPair> pairs;
    aln_thm_params P;
    char *arena = nullptr;   // splat rasters
    size_t arena_cap = 0;
    SplatJob *djobs = nullptr;
    size_t djobs_cap = 0;
    unsigned long long key_base = 0;   // thumbnail B of pair k without a caller key:
                                       // library key key_base + k + 1
};

// RFromAngle (CThmScan.cpp:329-366) for a list of evaluations: one GPU batch.
static int eval_batch(SweepCtx &S, std::vector<Eval> &ev)
{
    aln_ctx *ctx = S.ctx;
    const size_t CH = 8192;
    for (size_t c0 = 0; c0 < ev.size(); c0 += CH) {
        const size_t n = std::min(CH, ev.size() - c0);
        std::vector<SplatJob> jobs(n);
        std::vector<aln_pair> pairs(n);
        std::vector<ImgSpec> specs(n);
        std::vector<JobKey> keys(n);   // B's spectrum is reused across angles (and calls)
        size_t bytes = 0;
        for (size_t k = 0; k < n; ++k) {
            Eval &E = ev[c0 + k];
            ThmPair &tp = S.pairs[E.pair];
            ThmRec &C = *E.out;
            double R[6], T[6], D[6];
            C.A = E.deg;
            aff_nu(R, 5, E.deg * ALN_PI_REF / 180.0);
            memcpy(T, tp.Tptwk, sizeof T);
            if (E.iaux >= 0 && E.iaux < (int)tp.Tsel.size()) {
                double M[6];
                aff_nu(M, tp.Tsel[E.iaux], tp.Ta[E.iaux]);
                aff_mul(T, M, tp.Tptwk);
            }
            aff_mul(D, S.P.tdfm, T);
            aff_mul(C.T, R, D);
            SplatJob &J = jobs[k];
            J.t0 = C.T[0];
            J.t1 = C.T[1];
            J.t3 = C.T[3];
            J.t4 = C.T[4];
            const double fx = (double)(1ll << SPLAT_FX);
            J.T0 = llrint(J.t0 * fx);
            J.T1 = llrint(J.t1 * fx);
            J.T3 = llrint(J.t3 * fx);
            J.T4 = llrint(J.t4 * fx);
            {
                const double det = J.t0 * J.t4 - J.t1 * J.t3;
                const double m00 = J.t4 / det, m01 = -J.t1 / det;
                const double m10 = -J.t3 / det, m11 = J.t0 / det;
                J.i00 = (float)m00;
                J.i01 = (float)m01;
                J.i10 = (float)m10;
                J.i11 = (float)m11;
                // half-extents plus a margin for the FP32 centre (the exact
                // test decides)
                J.eu = (float)(fabs(m00) + fabs(m01)) + 1e-2f;
                J.ev = (float)(fabs(m10) + fabs(m11)) + 1e-2f;
            }
            double xlo = 1e300, xhi = -1e300, ylo = 1e300, yhi = -1e300;
            for (auto &h : tp.hull) {
                const double px = (double)h.first, py = (double)h.second;
                const double x = px * J.t0 + py * J.t1, y = px * J.t3 + py * J.t4;
                xlo = std::min(xlo, x);
                xhi = std::max(xhi, x);
                ylo = std::min(ylo, y);
                yhi = std::max(yhi, y);
            }
            J.L = (int)floor(xlo);
            J.B = (int)floor(ylo);
            J.w1 = (int)ceil(xhi) - J.L + 1;
            J.h1 = (int)ceil(yhi) - J.B + 1;
            J.a = tp.dev_af;
            J.mask = tp.dev_mask;
            J.aw = tp.in->a_w;
            J.ah = tp.in->a_h;
            J.astride = tp.in->a_stride;
            J.ax0 = tp.in->a_x0;
            J.ay0 = tp.in->a_y0;
            bytes += al256((size_t)J.w1 * J.h1 * sizeof(float));
        }
        if (bytes > S.arena_cap) {
            CK(cudaStreamSynchronize(ctx->stream));
            cudaFree(S.arena);
            S.arena = nullptr;
            S.arena_cap = 0;
            cudaError_t e = cudaMalloc(&S.arena, bytes + bytes / 4);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return set_err(ctx, ALN_ERR_NOMEM, "sweep arena: %s", cudaGetErrorString(e));
            }
            S.arena_cap = bytes + bytes / 4;
        }
        if (n > S.djobs_cap) {
            CK(cudaStreamSynchronize(ctx->stream));
            cudaFree(S.djobs);
            CK(cudaMalloc(&S.djobs, n * sizeof(SplatJob)));
            S.djobs_cap = n;
        }
        char *p = S.arena;
        int mw = 1, mh = 1;
        for (size_t k = 0; k < n; ++k) {
            SplatJob &J = jobs[k];
            J.out = (float *)p;
            p += al256((size_t)J.w1 * J.h1 * sizeof(float));
            mw = std::max(mw, J.w1);
            mh = std::max(mh, J.h1);
            const Eval &E = ev[c0 + k];
            const ThmPair &tp = S.pairs[E.pair];
            aln_pair &Pp = pairs[k];
            memset(&Pp, 0, sizeof Pp);
            Pp.a.data = J.out;
            Pp.a.dtype = ALN_F32;
            Pp.a.w = J.w1;
            Pp.a.h = J.h1;
            Pp.a.stride = J.w1;
            Pp.a.x0 = J.L;
            Pp.a.y0 = J.B;
            Pp.a.on_device = 1;
            Pp.b = tp.dev_b;
            Pp.radius = 1 << 20;
            // BigEnough / EnoughPoints (CThmScan.cpp:28-42) with thm.reqArea
            Pp.legal.rgn_kind = ALN_RGN_MIN;
            Pp.legal.rgn_a = Pp.legal.rgn_b = tp.in->olap1d;
            Pp.legal.rgn_area = tp.in->req_area;
            Pp.legal.cnt_kind = ALN_CNT_GT;
            Pp.legal.cnt_n = tp.in->req_area;
            if (tp.in->b_key)
                keys[k] = JobKey{0, tp.in->b_key};
            else
                keys[k] = JobKey{1, S.key_base + (unsigned long long)E.pair + 1};
            // RFromAngle: CorrImagesS, or CorrImagesF when useCorrR is off
            // (CThmScan.cpp:355-365)
            specs[k].kind = S.P.usecorrr ? 2 : 4;
            specs[k].nbmaxht = S.P.nbmaxht;
            specs[k].mincor = 0.0;
            specs[k].ox = tp.own_disc ? tp.dox : S.P.ox;
            specs[k].oy = tp.own_disc ? tp.doy : S.P.oy;
            specs[k].rx = tp.own_disc ? tp.drx : S.P.rx;
            specs[k].ry = tp.own_disc ? tp.dry : S.P.ry;
            if (S.P.disc_of_angle)   // newAngProc wins over SetDisc (CThmScan.cpp:350-356)
                S.P.disc_of_angle(S.P.disc_user, E.deg, &specs[k].ox, &specs[k].oy,
                                  &specs[k].rx, &specs[k].ry);
        }
        CK(cudaMemcpyAsync(S.djobs, jobs.data(), n * sizeof(SplatJob), cudaMemcpyHostToDevice,
                           ctx->stream));
        LAUNCH(ctx, "k_splat", k_splat, dim3((mw + 31) / 32, (mh + 31) / 32, (unsigned)n), 256, 0,
               S.djobs);
        CK(cudaGetLastError());
        std::vector<aln_result> res(n);
        if (int rc = batch_impl(ctx, (int)n, pairs.data(), specs.data(), res.data(),
                                keys.data()))
            return rc;
        for (size_t k = 0; k < n; ++k) {
            ThmRec &C = *ev[c0 + k].out;
            C.R = res[k].status == ALN_OK ? res[k].r : 0.0;
            C.X = res[k].status == ALN_OK ? res[k].dx : 0.0;
            C.Y = res[k].status == ALN_OK ? res[k].dy : 0.0;
            S.pairs[ev[c0 + k].pair].ncalls++;
        }
    }
    return ALN_OK;
}

static int round_ref(double x) { return x >= 0.0 ? (int)(x + 0.5) : (int)(x - 0.5); }

// LineFit lincor (Maths.cpp:457-507)
static double linefit_r(const double *x, const double *y, int n)
{
    double cnt = 0, sx = 0, sy = 0, sxx = 0, syy = 0, sxy = 0;
    for (int i = 0; i < n; ++i) {
        const double X = x[i], Y = y[i];
        sx += X;
        sy += Y;
        sxx += X * X;
        syy += Y * Y;
        sxy += X * Y;
        ++cnt;
    }
    const double r = cnt * sxy - sx * sy;
    const double vx = cnt * sxx - sx * sx;
    const double vy = cnt * syy - sy * sy;
    return r / sqrt(vx * vy);
}

// AngleScanSel (CThmScan.cpp:627-641) over a set of pairs: ConstXY
// (:514-621) or MaxR (:431-493).
static int scan_sel(SweepCtx &S, const std::vector<int> &ids, const std::vector<double> &center,
                    double hlfwid, double step, bool favorCenter, bool constxy)
{
    std::vector<std::vector<ThmRec>> vC(ids.size());
    std::vector<Eval> ev;
    for (size_t q = 0; q < ids.size(); ++q) {
        std::vector<double> angs;
        const double c = center[q];
        if (constxy) {
            for (double a = c - hlfwid; a <= c + hlfwid; a += step)
                angs.push_back(a);
        } else {
            angs.push_back(c);
            if (favorCenter) {
                const double cwide = 2.0 * step, cstep = step / 3.0;
                for (double a = c - cwide; a <= c + cwide; a += cstep)
                    angs.push_back(a);
                if (hlfwid >= 180) {
                    const double opc = c + 180;
                    for (double a = opc - cwide; a <= opc + cwide; a += cstep)
                        angs.push_back(a);
                }
            }
            for (double a = c - hlfwid; a <= c + hlfwid; a += step)
                angs.push_back(a);
        }
        vC[q].resize(angs.size());
        for (size_t k = 0; k < angs.size(); ++k)
            ev.push_back(Eval{ids[q], angs[k], -1, &vC[q][k]});
    }
    if (int rc = eval_batch(S, ev))
        return rc;
    for (size_t q = 0; q < ids.size(); ++q) {
        ThmRec &best = S.pairs[ids[q]].best;
        std::vector<ThmRec> &C = vC[q];
        const int nC = (int)C.size();
        if (!constxy) {
            best = C[0];
            for (int ic = 1; ic < nC; ++ic)
                if (C[ic].R > best.R)
                    best = C[ic];
            continue;
        }
        best.X = best.Y = best.A = best.R = 0.0;
        std::vector<int> order(nC);
        for (int i = 0; i < nC; ++i)
            order[i] = i;
        std::stable_sort(order.begin(), order.end(),
                         [&](int a, int b) { return C[a].R > C[b].R; });
        const double rthresh = 0.7;
        const int m = 3, M = 2 * m + 1;
        for (int i = 0; i < nC; ++i) {
            const int ic = order[i];
            if (ic < m || nC - 1 - ic < m)
                continue;
            double A[7], X[7], Y[7];
            int n = 0;
            for (int j = ic - m; j <= ic + m; ++j) {
                A[n] = C[j].A;
                X[n] = round_ref(C[j].X);
                Y[n] = round_ref(C[j].Y);
                ++n;
            }
            double lc = linefit_r(A, X, M);
            if (std::isfinite(lc) && fabs(lc) < rthresh)
                continue;
            lc = linefit_r(A, Y, M);
            if (std::isfinite(lc) && fabs(lc) < rthresh)
                continue;
            best = C[ic];
            break;
        }
    }
    return ALN_OK;
}

// PeakHunt (CThmScan.cpp:676-728): bracket bisection, all pairs in lockstep
// rounds (each pair stops on its own when its bracket is below 1e-4).
static int peak_hunt(SweepCtx &S, const std::vector<int> &ids, double hlfwid)
{
    const size_t n = ids.size();
    std::vector<ThmRec> B0(n), C(n);
    std::vector<double> L(n), R(n), M(n), a(n);
    std::vector<char> on(n, 1);
    std::vector<Eval> ev;
    for (size_t q = 0; q < n; ++q) {
        ThmRec &best = S.pairs[ids[q]].best;
        B0[q] = best;
        L[q] = best.A - hlfwid;
        R[q] = best.A + hlfwid;
        M[q] = (L[q] + R[q]) / 2.0;
        ev.push_back(Eval{ids[q], M[q], -1, &best});
    }
    if (int rc = eval_batch(S, ev))
        return rc;
    for (;;) {
        ev.clear();
        for (size_t q = 0; q < n; ++q) {
            on[q] = R[q] - L[q] > 0.0001;
            if (on[q]) {
                a[q] = (L[q] + M[q]) / 2.0;
                ev.push_back(Eval{ids[q], a[q], -1, &C[q]});
            }
        }
        if (ev.empty())
            break;
        if (int rc = eval_batch(S, ev))
            return rc;
        ev.clear();
        for (size_t q = 0; q < n; ++q) {
            if (!on[q])
                continue;
            ThmRec &best = S.pairs[ids[q]].best;
            if (C[q].R >= best.R) {
                R[q] = M[q];
                best = C[q];
                M[q] = a[q];
            } else
                L[q] = a[q];
            a[q] = (M[q] + R[q]) / 2.0;
            ev.push_back(Eval{ids[q], a[q], -1, &C[q]});
        }
        if (int rc = eval_batch(S, ev))
            return rc;
        for (size_t q = 0; q < n; ++q) {
            if (!on[q])
                continue;
            ThmRec &best = S.pairs[ids[q]].best;
            if (C[q].R >= best.R) {
                L[q] = M[q];
                best = C[q];
                M[q] = a[q];
            } else
                R[q] = a[q];
        }
    }
    for (size_t q = 0; q < n; ++q)
        if (B0[q].R > S.pairs[ids[q]].best.R)
            S.pairs[ids[q]].best = B0[q];
    return ALN_OK;
}

// Pretweaks (CThmScan.cpp:205-323) for one pair; returns whether Tptwk changed.
static int pretweaks(SweepCtx &S, int id, double bestR, double deg, bool *changed)
{
    ThmPair &tp = S.pairs[id];
    int vused[5] = {0, 0, 0, 0, 0};
    const double astep = 0.02;
    const int nstep = 5;
    *changed = false;
    for (int itype = 0; itype < 5; ++itype) {
        tp.Tsel.clear();
        tp.Ta.clear();
        for (int sel = 0; sel < 5; ++sel) {
            if (vused[sel])
                continue;
            const double abase = (sel >= 0 && sel <= 2) ? 1.0 : 0.0;
            for (int j = -nstep; j <= nstep; ++j) {
                tp.Tsel.push_back(sel);
                tp.Ta.push_back(abase + j * astep);
            }
        }
        const int nc = (int)tp.Tsel.size();
        std::vector<ThmRec> vC(nc);
        std::vector<Eval> ev;
        for (int ic = 0; ic < nc; ++ic)
            ev.push_back(Eval{id, deg, ic, &vC[ic]});
        if (int rc = eval_batch(S, ev))
            return rc;
        double rbest = 0;
        int ibest = -1;
        for (int ic = 0; ic < nc; ++ic)
            if (vC[ic].R > rbest) {
                rbest = vC[ic].R;
                ibest = ic;
            }
        if (ibest == -1)
            break;
        const int bsel = tp.Tsel[ibest];
        double x1 = tp.Ta[ibest];
        // PTWInterp (CThmScan.cpp:119-155) on record 0
        const double y1 = rbest, d = astep;
        ThmRec C;
        std::vector<Eval> one(1, Eval{id, deg, 0, &C});
        tp.Tsel[0] = bsel;
        tp.Ta[0] = x1 - d;
        if (int rc = eval_batch(S, one))
            return rc;
        const double y0 = C.R;
        tp.Ta[0] = x1 + d;
        if (int rc = eval_batch(S, one))
            return rc;
        const double y2 = C.R;
        double xnew = x1;
        {
            const double D = d * (y0 - y2) / (2 * (y0 + y2 - y1 - y1));
            if (fabs(D) <= 2 * d)
                xnew = x1 + D;
        }
        tp.Ta[0] = xnew;
        if (int rc = eval_batch(S, one))
            return rc;
        double ynew = C.R;
        if (ynew < y1) {
            xnew = x1;
            ynew = y1;
        }
        rbest = ynew;
        if (rbest > bestR) {
            double M[6];
            aff_nu(M, bsel, xnew);
            aff_mul(tp.Tptwk, M, tp.Tptwk);
            vused[bsel] = 1;
            bestR = rbest;
            *changed = true;
        } else
            break;
    }
    tp.Tsel.clear();
    tp.Ta.clear();
    return ALN_OK;
}

// AngleScanWithTweaks (CThmScan.cpp:647-668)
static int scan_with_tweaks(SweepCtx &S, const std::vector<int> &ids,
                            const std::vector<double> &center, double hlfwid, double step)
{
    if (int rc = scan_sel(S, ids, center, hlfwid, step, true, S.P.constxy != 0))
        return rc;
    if (!S.P.pretweak)
        return ALN_OK;
    std::vector<int> redo;
    std::vector<double> rc_center;
    for (size_t q = 0; q < ids.size(); ++q) {
        ThmRec &best = S.pairs[ids[q]].best;
        if (best.R < S.P.rthresh) {
            bool changed = false;
            if (int rc = pretweaks(S, ids[q], best.R, best.R > 0.0 ? best.A : center[q], &changed))
                return rc;
            if (changed) {
                redo.push_back(ids[q]);
                rc_center.push_back(center[q]);
            }
        }
    }
    if (!redo.empty())
        return scan_sel(S, redo, rc_center, hlfwid, step, true, S.P.constxy != 0);
    return ALN_OK;
}

// Device copies of the thumbnails, hulls and the initial sweep state
// (CThmScan::Initialize) for every pair; *dbuf receives the allocation.
static int sweep_setup(aln_ctx *ctx, SweepCtx &S, int npairs, const aln_thumbs *thumbs,
                       const aln_thm_params *params, char **dbuf_out)
{
    *dbuf_out = nullptr;
    CK(cudaSetDevice(ctx->device));
    S.ctx = ctx;
    S.P = *params;
    S.pairs.resize(npairs);
    S.key_base = (++ctx->sweep_serial) << 32;
    // device copies of the thumbnails
    size_t bytes = 0;
    for (int k = 0; k < npairs; ++k) {
        const aln_thumbs &T = thumbs[k];
        if (!T.a || T.a_w < 1 || T.a_h < 1 || T.a_stride < T.a_w || !T.b.data ||
            T.b.dtype != ALN_F64 || T.b.w < 1 || T.b.h < 1 || T.b.stride < T.b.w)
            return set_err(ctx, ALN_ERR_ARG, "thumbnail pair %d: bad grid/raster", k);
        bytes += al256((size_t)T.a_stride * T.a_h * 8) + al256((size_t)T.a_stride * T.a_h * 4) +
                 al256((size_t)T.a_stride * T.a_h) + al256((size_t)T.b.stride * T.b.h * 8);
    }
    char *dbuf = nullptr;
    if (bytes) {
        cudaError_t e = cudaMalloc(&dbuf, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_err(ctx, ALN_ERR_NOMEM, "thumbnails: %s", cudaGetErrorString(e));
        }
    }
    char *p = dbuf;
    int rc = ALN_OK;
    for (int k = 0; k < npairs && rc == ALN_OK; ++k) {
        const aln_thumbs &T = thumbs[k];
        ThmPair &tp = S.pairs[k];
        tp.in = &T;
        tp.ncalls = 0;
        tp.err = 0;
        aff_one(tp.Tptwk);
        const size_t ab = (size_t)T.a_stride * T.a_h * 8;
        tp.dev_a = (const double *)p;
        if (cudaMemcpyAsync(p, T.a, ab, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
            rc = set_err(ctx, ALN_ERR_CUDA, "thumbnail copy");
        p += al256(ab);
        // the splat multiplies in FP32: convert once here instead of per
        // gathered point (FP64 conversions run on the narrow FP64 pipe)
        tp.dev_af = (const float *)p;
        {
            const size_t na = (size_t)T.a_stride * T.a_h;
            LAUNCH(ctx, "k_f64_to_f32", k_f64_to_f32,
                   (unsigned)std::min<size_t>((na + 255) / 256, 1024), 256, 0, tp.dev_a,
                   (float *)p, na);
            p += al256(na * 4);
        }
        tp.dev_mask = nullptr;
        if (T.a_mask) {
            tp.dev_mask = (const unsigned char *)p;
            if (cudaMemcpyAsync(p, T.a_mask, (size_t)T.a_stride * T.a_h, cudaMemcpyHostToDevice,
                                ctx->stream) != cudaSuccess)
                rc = set_err(ctx, ALN_ERR_CUDA, "mask copy");
        }
        p += al256((size_t)T.a_stride * T.a_h);
        const size_t bb = (size_t)T.b.stride * T.b.h * 8;
        tp.dev_b = T.b;
        tp.dev_b.data = p;
        tp.dev_b.on_device = 1;
        if (cudaMemcpyAsync(p, T.b.data, bb, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess)
            rc = set_err(ctx, ALN_ERR_CUDA, "thumbnail copy");
        p += al256(bb);
        ctx->h2d_bytes += (long long)(ab + bb + (T.a_mask ? (size_t)T.a_stride * T.a_h : 0));
        make_hull(tp);
        if (tp.hull.empty())
            rc = set_err(ctx, ALN_ERR_ARG, "thumbnail pair %d: no A points", k);
        tp.best.X = tp.best.Y = tp.best.A = tp.best.R = -999.0;   // CThmScan::Initialize
        tp.own_disc = 0;
    }
    *dbuf_out = dbuf;
    return rc;
}

extern "C" int aln_thm_search_batch(aln_ctx *ctx, int npairs, const aln_thumbs *thumbs,
                                    const aln_thm_params *params, int mode, double ang0,
                                    double hfang, double step, aln_thm_result *out)
{
    if (!ctx || npairs < 0 || (npairs && (!thumbs || !params || !out)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "bad arguments") : ALN_ERR_ARG;
    SweepCtx S;
    char *dbuf = nullptr;
    int rc = sweep_setup(ctx, S, npairs, thumbs, params, &dbuf);
    std::vector<int> all(npairs);
    for (int k = 0; k < npairs; ++k)
        all[k] = k;
    std::vector<double> c0(npairs, ang0);
    auto failing = [&](const std::vector<int> &ids) {
        std::vector<int> keep;
        for (int id : ids)
            if (S.pairs[id].best.R < S.P.rthresh)
                S.pairs[id].err = (mode == ALN_THM_PRIOR) ? 2 : 1;
            else
                keep.push_back(id);
        return keep;
    };
    if (rc == ALN_OK) {
        switch (mode) {
        case ALN_THM_DENOVO: {
            // DenovoBestAngle (CThmScan.cpp:764-790)
            rc = scan_with_tweaks(S, all, c0, hfang, step);
            std::vector<int> ids = failing(all);
            if (rc == ALN_OK && !ids.empty()) {
                std::vector<double> cen;
                for (int id : ids)
                    cen.push_back(S.pairs[id].best.A);
                rc = scan_sel(S, ids, cen, step * 2.0, step * 0.05, false, S.P.constxy != 0);
            }
            ids = failing(ids);
            if (rc == ALN_OK && !ids.empty())
                rc = peak_hunt(S, ids, step * 0.05 * 1.5);
            failing(ids);
            break;
        }
        case ALN_THM_RFROMANGLE: {
            std::vector<Eval> ev;
            for (int k = 0; k < npairs; ++k)
                ev.push_back(Eval{k, ang0, -1, &S.pairs[k].best});
            rc = eval_batch(S, ev);
            break;
        }
        case ALN_THM_PRIOR: {
            // UsePriorAngles (CThmScan.cpp:734-758)
            rc = scan_with_tweaks(S, all, c0, hfang, 0.1);
            std::vector<int> ids = failing(all);
            if (rc == ALN_OK && !ids.empty())
                rc = peak_hunt(S, ids, 0.1 * 1.5);
            failing(ids);
            break;
        }
        case ALN_THM_SCAN_HUNT:
            rc = scan_sel(S, all, c0, hfang, step, false, S.P.constxy != 0);
            if (rc == ALN_OK)
                rc = peak_hunt(S, all, step * 0.05 * 1.5);
            break;
        case ALN_THM_SCAN_MAXR:
            rc = scan_sel(S, all, c0, hfang, step, true, false);
            break;
        default:
            rc = set_err(ctx, ALN_ERR_ARG, "bad sweep mode %d", mode);
        }
    }
    cudaStreamSynchronize(ctx->stream);
    spec_drop(ctx, 1, S.key_base, S.key_base + (unsigned long long)npairs + 1);
    cudaFree(S.arena);
    cudaFree(S.djobs);
    cudaFree(dbuf);
    if (rc != ALN_OK)
        return rc;
    for (int k = 0; k < npairs; ++k) {
        const ThmPair &tp = S.pairs[k];
        out[k].A = tp.best.A;
        out[k].X = tp.best.X;
        out[k].Y = tp.best.Y;
        out[k].R = tp.best.R;
        memcpy(out[k].T, tp.best.T, sizeof out[k].T);
        out[k].err = tp.err;
        out[k].ncalls = tp.ncalls;
    }
    return ALN_OK;
}

// CThmScan::PostTweaks (CThmScan.cpp:796-802) and FinishAtFullRes
// (:810-842) for many pairs, each from its prior best record and pretweak
// transform (the CThmScan object's state).  Both set useCorrR and a disc of
// radius 40 / 80 around the prior (X, Y) (truncated to int, as SetDisc gets
// them).  PostTweaks runs Pretweaks(prior R, prior A), then RFromAngle at
// the prior angle; FinishAtFullRes runs RFromAngle at the prior angle on
// the full-resolution thumbnails and keeps the result only when X and Y
// moved by at most 20 (then with the prior R).
extern "C" int aln_thm_finish_batch(aln_ctx *ctx, int npairs, const aln_thumbs *thumbs,
                                    const aln_thm_params *params, int mode,
                                    const aln_thm_result *prior, const double *prior_tptwk,
                                    aln_thm_result *out, double *out_tptwk)
{
    if (!ctx || npairs < 0 || (npairs && (!thumbs || !params || !prior || !out)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "bad arguments") : ALN_ERR_ARG;
    if (mode != ALN_THM_POSTTWEAKS && mode != ALN_THM_FULLRES)
        return set_err(ctx, ALN_ERR_ARG, "bad finishing mode %d", mode);
    aln_thm_params P = *params;
    P.usecorrr = 1;   // SetUseCorrR(true)
    SweepCtx S;
    char *dbuf = nullptr;
    int rc = sweep_setup(ctx, S, npairs, thumbs, &P, &dbuf);
    std::vector<ThmRec> b0(npairs);
    for (int k = 0; k < npairs && rc == ALN_OK; ++k) {
        ThmPair &tp = S.pairs[k];
        tp.best.A = prior[k].A;
        tp.best.X = prior[k].X;
        tp.best.Y = prior[k].Y;
        tp.best.R = prior[k].R;
        memcpy(tp.best.T, prior[k].T, sizeof tp.best.T);
        if (prior_tptwk)
            memcpy(tp.Tptwk, prior_tptwk + 6 * (size_t)k, sizeof tp.Tptwk);
        tp.own_disc = 1;
        tp.dox = (int)tp.best.X;
        tp.doy = (int)tp.best.Y;
        tp.drx = tp.dry = mode == ALN_THM_POSTTWEAKS ? 40 : 80;
        b0[k] = tp.best;
    }
    if (rc == ALN_OK && mode == ALN_THM_POSTTWEAKS)
        for (int k = 0; k < npairs && rc == ALN_OK; ++k) {
            bool changed = false;
            rc = pretweaks(S, k, S.pairs[k].best.R, S.pairs[k].best.A, &changed);
        }
    if (rc == ALN_OK) {
        std::vector<Eval> ev;
        for (int k = 0; k < npairs; ++k)
            ev.push_back(Eval{k, S.pairs[k].best.A, -1, &S.pairs[k].best});
        rc = eval_batch(S, ev);
    }
    if (rc == ALN_OK && mode == ALN_THM_FULLRES)
        for (int k = 0; k < npairs; ++k) {
            ThmRec &b = S.pairs[k].best;
            if (fabs(b.X - b0[k].X) <= 20 && fabs(b.Y - b0[k].Y) <= 20)
                b.R = b0[k].R;
            else
                b = b0[k];
        }
    cudaStreamSynchronize(ctx->stream);
    spec_drop(ctx, 1, S.key_base, S.key_base + (unsigned long long)npairs + 1);
    cudaFree(S.arena);
    cudaFree(S.djobs);
    cudaFree(dbuf);
    if (rc != ALN_OK)
        return rc;
    for (int k = 0; k < npairs; ++k) {
        const ThmPair &tp = S.pairs[k];
        out[k].A = tp.best.A;
        out[k].X = tp.best.X;
        out[k].Y = tp.best.Y;
        out[k].R = tp.best.R;
        memcpy(out[k].T, tp.best.T, sizeof out[k].T);
        out[k].err = 0;
        out[k].ncalls = tp.ncalls;
        if (out_tptwk)
            memcpy(out_tptwk + 6 * (size_t)k, tp.Tptwk, sizeof tp.Tptwk);
    }
    return ALN_OK;
}

// One CThmScan member-function call per pair from the caller's object
// state (best record, err, pretweak transform); see aln_thm_call_batch in
// the header for the ops and their arguments.
extern "C" int aln_thm_call_batch(aln_ctx *ctx, int npairs, const aln_thumbs *thumbs,
                                  const aln_thm_params *params, int op, const double *args,
                                  aln_thm_result *best, double *tptwk, double *ret)
{
    if (!ctx || npairs < 0 || (npairs && (!thumbs || !params || !args || !best)))
        return ctx ? set_err(ctx, ALN_ERR_ARG, "bad arguments") : ALN_ERR_ARG;
    if (op < ALN_THMOP_RFROMANGLE || op > ALN_THMOP_FULLRES)
        return set_err(ctx, ALN_ERR_ARG, "bad CThmScan op %d", op);
    const bool shared = op >= ALN_THMOP_SCAN_MAXR && op <= ALN_THMOP_DENOVO;
    for (int k = 1; shared && k < npairs; ++k)
        for (int j = 1; j < 4; ++j)
            if (args[4 * k + j] != args[j])
                return set_err(ctx, ALN_ERR_ARG, "op %d: a1..a3 differ between pairs", op);
    aln_thm_params P = *params;
    if (op == ALN_THMOP_POSTTWEAKS || op == ALN_THMOP_FULLRES)
        P.usecorrr = 1;   // SetUseCorrR(true)
    SweepCtx S;
    char *dbuf = nullptr;
    int rc = sweep_setup(ctx, S, npairs, thumbs, &P, &dbuf);
    std::vector<int> all(npairs);
    std::vector<double> a0(npairs), rv(npairs, 0.0);
    std::vector<ThmRec> b0(npairs);
    for (int k = 0; k < npairs && rc == ALN_OK; ++k) {
        ThmPair &tp = S.pairs[k];
        all[k] = k;
        a0[k] = args[4 * k];
        tp.best.A = best[k].A;
        tp.best.X = best[k].X;
        tp.best.Y = best[k].Y;
        tp.best.R = best[k].R;
        memcpy(tp.best.T, best[k].T, sizeof tp.best.T);
        tp.err = best[k].err;
        if (tptwk)
            memcpy(tp.Tptwk, tptwk + 6 * (size_t)k, sizeof tp.Tptwk);
        if (op == ALN_THMOP_POSTTWEAKS || op == ALN_THMOP_FULLRES) {
            tp.own_disc = 1;   // SetDisc((int)best.X, (int)best.Y, r, r)
            tp.dox = (int)tp.best.X;
            tp.doy = (int)tp.best.Y;
            tp.drx = tp.dry = op == ALN_THMOP_POSTTWEAKS ? 40 : 80;
        }
        b0[k] = tp.best;
    }
    const double a1 = npairs ? args[1] : 0.0, a2 = npairs ? args[2] : 0.0,
                 a3 = npairs ? args[3] : 0.0;
    auto rvals = [&](const std::vector<int> &ids) {
        for (int id : ids)
            rv[id] = S.pairs[id].best.R;
    };
    // ids still passing a stage of a `||` chain (the rest fail with err)
    auto passing = [&](const std::vector<int> &ids, int err) {
        std::vector<int> keep;
        for (int id : ids)
            if (S.pairs[id].best.R < S.P.rthresh) {
                S.pairs[id].err = err;
                rv[id] = 0.0;
            } else {
                keep.push_back(id);
                rv[id] = 1.0;
            }
        return keep;
    };
    if (rc == ALN_OK && npairs) {
        switch (op) {
        case ALN_THMOP_RFROMANGLE: {
            std::vector<Eval> ev;
            for (int k = 0; k < npairs; ++k)
                ev.push_back(Eval{k, a0[k], -1, &S.pairs[k].best});
            rc = eval_batch(S, ev);
            break;
        }
        case ALN_THMOP_SCAN_MAXR:
            rc = scan_sel(S, all, a0, a1, a2, a3 != 0.0, false);
            rvals(all);
            break;
        case ALN_THMOP_SCAN_CONSTXY:
            rc = scan_sel(S, all, a0, a1, a2, false, true);
            rvals(all);
            break;
        case ALN_THMOP_SCAN_SEL:
            rc = scan_sel(S, all, a0, a1, a2, a3 != 0.0, S.P.constxy != 0);
            rvals(all);
            break;
        case ALN_THMOP_SCAN_TWEAKS:
            rc = scan_with_tweaks(S, all, a0, a1, a2);
            rvals(all);
            break;
        case ALN_THMOP_PEAKHUNT:
            rc = peak_hunt(S, all, a1);
            rvals(all);
            break;
        case ALN_THMOP_PRIOR: {
            // UsePriorAngles (CThmScan.cpp:734-758)
            rc = scan_with_tweaks(S, all, a0, a1, 0.1);
            std::vector<int> ids = passing(all, 2);
            if (rc == ALN_OK && !ids.empty())
                rc = peak_hunt(S, ids, 0.1 * 1.5);
            passing(ids, 2);
            break;
        }
        case ALN_THMOP_DENOVO: {
            // DenovoBestAngle (CThmScan.cpp:764-790)
            rc = scan_with_tweaks(S, all, a0, a1, a2);
            std::vector<int> ids = passing(all, 1);
            if (rc == ALN_OK && !ids.empty()) {
                std::vector<double> cen;
                for (int id : ids)
                    cen.push_back(S.pairs[id].best.A);
                rc = scan_sel(S, ids, cen, a2 * 2.0, a2 * 0.05, false, S.P.constxy != 0);
            }
            ids = passing(ids, 1);
            if (rc == ALN_OK && !ids.empty())
                rc = peak_hunt(S, ids, a2 * 0.05 * 1.5);
            passing(ids, 1);
            break;
        }
        case ALN_THMOP_PRETWEAKS:
            for (int k = 0; k < npairs && rc == ALN_OK; ++k) {
                bool changed = false;
                rc = pretweaks(S, k, a0[k], args[4 * k + 1], &changed);
                rv[k] = changed ? 1.0 : 0.0;
            }
            break;
        case ALN_THMOP_POSTTWEAKS:
        case ALN_THMOP_FULLRES: {
            if (op == ALN_THMOP_POSTTWEAKS)
                for (int k = 0; k < npairs && rc == ALN_OK; ++k) {
                    bool changed = false;
                    rc = pretweaks(S, k, S.pairs[k].best.R, S.pairs[k].best.A, &changed);
                }
            std::vector<Eval> ev;
            for (int k = 0; k < npairs; ++k)
                ev.push_back(Eval{k, S.pairs[k].best.A, -1, &S.pairs[k].best});
            if (rc == ALN_OK)
                rc = eval_batch(S, ev);
            if (rc == ALN_OK && op == ALN_THMOP_FULLRES)
                for (int k = 0; k < npairs; ++k) {
                    ThmRec &b = S.pairs[k].best;
                    if (fabs(b.X - b0[k].X) <= 20 && fabs(b.Y - b0[k].Y) <= 20)
                        b.R = b0[k].R;
                    else
                        b = b0[k];
                }
            break;
        }
        }
    }
    cudaStreamSynchronize(ctx->stream);
    spec_drop(ctx, 1, S.key_base, S.key_base + (unsigned long long)npairs + 1);
    cudaFree(S.arena);
    cudaFree(S.djobs);
    cudaFree(dbuf);
    if (rc != ALN_OK)
        return rc;
    for (int k = 0; k < npairs; ++k) {
        const ThmPair &tp = S.pairs[k];
        best[k].A = tp.best.A;
        best[k].X = tp.best.X;
        best[k].Y = tp.best.Y;
        best[k].R = tp.best.R;
        memcpy(best[k].T, tp.best.T, sizeof best[k].T);
        best[k].err = tp.err;
        best[k].ncalls = tp.ncalls;
        if (tptwk)
            memcpy(tptwk + 6 * (size_t)k, tp.Tptwk, sizeof tp.Tptwk);
        if (ret)
            ret[k] = rv[k];
    }
    return ALN_OK;
}

// ---------------------------------------------------------------------------
// MakeThumbs' binning and normalisation (1_DMesh/CThmUtil.cpp:470-523):
// DecimateVector (0_GEN/Maths.cpp:1315-1364) and Normalize (:192-212)
// ---------------------------------------------------------------------------

struct DecJob {
    const void *img;            // device copy of the raster (caller's dtype)
    const unsigned char *mask;  // device copy of the point mask, or null
    int dt, w, h, stride;
    int ow, oh;                 // bin grid
    double *vals;               // device: bin values [oh][ow]
    unsigned char *pres;        // device: bin present
    double sd;
};

// grid (ceil(max ow / 32), ceil(max oh / 8), n), block (32, 8): one thread
// per bin sums its points in the point list's (raster) order, as the
// reference's accumulation visits them; the count is the reference's uint8
// counter (mod 256).
__global__ void k_decimate(DecJob *jobs, int lbin)
{
    DecJob &J = jobs[blockIdx.z];
    const int bx = blockIdx.x * 32 + threadIdx.x, by = blockIdx.y * 8 + threadIdx.y;
    if (bx >= J.ow || by >= J.oh)
        return;
    double s = 0.0;
    int cnt = 0;
    const int x0 = bx * lbin, y0 = by * lbin;
    const int x1 = min(J.w, x0 + lbin), y1 = min(J.h, y0 + lbin);
    for (int y = y0; y < y1; ++y)
        for (int x = x0; x < x1; ++x) {
            const long long k = (long long)y * J.stride + x;
            if (J.mask && !J.mask[k])
                continue;
            s = __dadd_rn(s, load_px(J.img, J.dt, k));
            ++cnt;
        }
    cnt &= 255;
    const long long o = (long long)by * J.ow + bx;
    J.vals[o] = cnt ? __ddiv_rn(s, (double)cnt) : 0.0;
    J.pres[o] = cnt != 0;
}

// Stats (Maths.cpp:132-141, MeanStd) over the present bins in raster order,
// one thread per image in the reference's operation order (no contraction),
// then (v - avg) / sd for every present bin.  grid n, block 256.
__global__ void k_normalize(DecJob *jobs)
{
    __shared__ double sh_avg, sh_sd;
    DecJob &J = jobs[blockIdx.x];
    const long long nb = (long long)J.ow * J.oh;
    if (threadIdx.x == 0) {
        double sum = 0.0, sum2 = 0.0;
        int n = 0;
        for (long long k = 0; k < nb; ++k)
            if (J.pres[k]) {
                const double v = J.vals[k];
                sum = __dadd_rn(sum, v);
                sum2 = __dadd_rn(sum2, __dmul_rn(v, v));
                ++n;
            }
        double avg = sum, sd = 0.0;
        if (n > 1) {
            avg = __ddiv_rn(avg, (double)n);
            const double t = __dsub_rn(sum2, __dmul_rn(__dmul_rn((double)n, avg), avg));
            sd = __dsqrt_rn(__ddiv_rn(fmax(t, 0.0), __dsub_rn((double)n, 1.0)));
        }
        sh_avg = avg;
        sh_sd = sd;
        J.sd = sd;
    }
    __syncthreads();
    for (long long k = threadIdx.x; k < nb; k += blockDim.x)
        if (J.pres[k])
            J.vals[k] = __ddiv_rn(__dsub_rn(J.vals[k], sh_avg), sh_sd);
}

extern "C" int aln_decimate_batch(aln_ctx *ctx, int n, const aln_image *in,
                                  const unsigned char *const *mask, int lbin, int normalize,
                                  double *const *out_vals, unsigned char *const *out_mask,
                                  double *out_sd)
{
    if (!ctx || n < 0 || (n && (!in || !out_vals || !out_mask)) || lbin < 1)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "bad arguments") : ALN_ERR_ARG;
    if (!n)
        return ALN_OK;
    if (n > 65535)   // one grid z index per image
        return set_err(ctx, ALN_ERR_ARG, "at most 65535 images per call (%d)", n);
    CK(cudaSetDevice(ctx->device));
    std::vector<DecJob> jobs(n);
    size_t bytes = 0;
    int mw = 1, mh = 1;
    for (int k = 0; k < n; ++k) {
        const aln_image &I = in[k];
        if (!I.data || I.w < 1 || I.h < 1 || I.stride < I.w || !dtype_size(I.dtype))
            return set_err(ctx, ALN_ERR_ARG, "image %d: bad data/size/stride/dtype", k);
        DecJob &J = jobs[k];
        J.dt = I.dtype;
        J.w = I.w;
        J.h = I.h;
        J.stride = I.stride;
        J.ow = (I.w + lbin - 1) / lbin;
        J.oh = (I.h + lbin - 1) / lbin;
        mw = std::max(mw, J.ow);
        mh = std::max(mh, J.oh);
        const size_t ib = (size_t)I.stride * I.h;
        bytes += al256(ib * dtype_size(I.dtype)) + (mask && mask[k] ? al256(ib) : 0) +
                 al256((size_t)J.ow * J.oh * 9);
    }
    char *buf = nullptr;
    {
        cudaError_t e = cudaMalloc(&buf, bytes + al256((size_t)n * sizeof(DecJob)));
        if (e != cudaSuccess) {
            cudaGetLastError();
            return set_err(ctx, ALN_ERR_NOMEM, "decimation buffers: %s", cudaGetErrorString(e));
        }
    }
    cudaStream_t st = ctx->stream;
    char *p = buf;
    int rc = ALN_OK;
    for (int k = 0; k < n && rc == ALN_OK; ++k) {
        const aln_image &I = in[k];
        DecJob &J = jobs[k];
        const size_t ib = (size_t)I.stride * I.h;
        // host or device sources alike (unified addressing)
        if (cudaMemcpyAsync(p, I.data, ib * dtype_size(I.dtype), cudaMemcpyDefault, st) !=
            cudaSuccess)
            rc = set_err(ctx, ALN_ERR_CUDA, "image %d copy", k);
        J.img = p;
        p += al256(ib * dtype_size(I.dtype));
        J.mask = nullptr;
        if (mask && mask[k]) {
            if (cudaMemcpyAsync(p, mask[k], ib, cudaMemcpyDefault, st) != cudaSuccess)
                rc = set_err(ctx, ALN_ERR_CUDA, "mask %d copy", k);
            J.mask = (const unsigned char *)p;
            p += al256(ib);
        }
        J.vals = (double *)p;
        J.pres = (unsigned char *)(p + (size_t)J.ow * J.oh * 8);
        p += al256((size_t)J.ow * J.oh * 9);
        J.sd = 0.0;
    }
    DecJob *dj = (DecJob *)p;
    if (rc == ALN_OK &&
        cudaMemcpyAsync(dj, jobs.data(), (size_t)n * sizeof(DecJob), cudaMemcpyHostToDevice,
                        st) != cudaSuccess)
        rc = set_err(ctx, ALN_ERR_CUDA, "job table copy");
    if (rc == ALN_OK) {
        LAUNCH(ctx, "k_decimate", k_decimate, dim3((mw + 31) / 32, (mh + 7) / 8, n), dim3(32, 8),
               0, dj, lbin);
        if (normalize)
            LAUNCH(ctx, "k_normalize", k_normalize, n, 256, 0, dj);
        for (int k = 0; k < n && rc == ALN_OK; ++k) {
            const size_t nb = (size_t)jobs[k].ow * jobs[k].oh;
            if (cudaMemcpyAsync(out_vals[k], jobs[k].vals, nb * 8, cudaMemcpyDefault, st) !=
                    cudaSuccess ||
                cudaMemcpyAsync(out_mask[k], jobs[k].pres, nb, cudaMemcpyDefault, st) !=
                    cudaSuccess)
                rc = set_err(ctx, ALN_ERR_CUDA, "result %d copy", k);
        }
        if (rc == ALN_OK && cudaMemcpyAsync(jobs.data(), dj, (size_t)n * sizeof(DecJob),
                                            cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = set_err(ctx, ALN_ERR_CUDA, "job table read-back");
    }
    cudaStreamSynchronize(ctx->stream);
    cudaFree(buf);
    if (rc != ALN_OK)
        return rc;
    CK(cudaGetLastError());
    if (out_sd)
        for (int k = 0; k < n; ++k)
            out_sd[k] = jobs[k].sd;
    return ALN_OK;
}
