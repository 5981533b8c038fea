// aln_approx.cuh -- ApproximateMatch on the GPU for many tile pairs
// (1_DMesh/ApproximateMatch.cpp:115-194 with CThmUtil's Crop, MakeThumbs,
// Sweep and Finish, 1_DMesh/CThmUtil.cpp:385-971).  Included by aln_corr.cu
// after aln_sweep.cuh.
//
// The stages run batched over the pairs: the overlap crop is a strided view
// of each tile (no copy), MakeThumbs is one aln_decimate_batch over all crops,
// the sweep one aln_thm_call_batch, PostTweaks and FinishAtFullRes one
// batch each.  The host does the integer box arithmetic and, at the end,
// IsectToImageCoords and the LIMXY test (a few flops per pair).
#pragma once

namespace {

// BoxesFromShifts, 0_GEN/Geometry.cpp:150-176
struct IBoxI {
    int L, R, B, T;
};
void boxes_from_shifts(IBoxI &B1, IBoxI &B2, int w1, int h1, int w2, int h2, int x, int y)
{
    B2.L = std::max(0, x);
    B2.R = std::min(w2 - 1, x + w1 - 1);
    B2.B = std::max(0, y);
    B2.T = std::min(h2 - 1, y + h1 - 1);
    B2.R = std::max(B2.R, B2.L);
    B2.T = std::max(B2.T, B2.B);
    B1.L = B2.L - x;
    B1.R = B2.R - x;
    B1.B = B2.B - y;
    B1.T = B2.T - y;
}

// A decimated (or full-resolution) thumbnail on the host: grid values,
// presence mask, and the aln_thumbs view of a pair of them.
struct Thumb {
    std::vector<double> v;
    std::vector<unsigned char> m;
    int w = 0, h = 0;
    double sd = 0.0;
    long long present = 0;
};

// aln_thumbs of a pair: A as its grid with the mask over the present bins'
// bounding box, B as a raster over its bounding box (absent bins 0), both
// with their corner offsets (the reference's point lists are relative to
// the crop's corner, absent bins simply missing)
bool thumbs_of(const Thumb &a, const Thumb &b, std::vector<double> &bras, aln_thumbs &T)
{
    auto bbox = [](const Thumb &t, int &x0, int &y0, int &x1, int &y1) {
        x0 = t.w;
        y0 = t.h;
        x1 = -1;
        y1 = -1;
        for (int y = 0; y < t.h; ++y)
            for (int x = 0; x < t.w; ++x)
                if (t.m[(size_t)y * t.w + x]) {
                    x0 = std::min(x0, x);
                    x1 = std::max(x1, x);
                    y0 = std::min(y0, y);
                    y1 = std::max(y1, y);
                }
        return x1 >= 0;
    };
    int ax0, ay0, ax1, ay1, bx0, by0, bx1, by1;
    if (!bbox(a, ax0, ay0, ax1, ay1) || !bbox(b, bx0, by0, bx1, by1))
        return false;
    memset(&T, 0, sizeof T);
    T.a = a.v.data() + (size_t)ay0 * a.w + ax0;
    T.a_mask = a.m.data() + (size_t)ay0 * a.w + ax0;
    T.a_w = ax1 - ax0 + 1;
    T.a_h = ay1 - ay0 + 1;
    T.a_stride = a.w;
    T.a_x0 = ax0;
    T.a_y0 = ay0;
    const int bw = bx1 - bx0 + 1, bh = by1 - by0 + 1;
    bras.assign((size_t)bw * bh, 0.0);
    for (int y = 0; y < bh; ++y)
        for (int x = 0; x < bw; ++x) {
            const size_t s = (size_t)(y + by0) * b.w + (x + bx0);
            if (b.m[s])
                bras[(size_t)y * bw + x] = b.v[s];
        }
    T.b.data = bras.data();
    T.b.dtype = ALN_F64;
    T.b.w = bw;
    T.b.h = bh;
    T.b.stride = bw;
    T.b.x0 = bx0;
    T.b.y0 = by0;
    T.b.on_device = 0;
    return true;
}

}   // namespace

extern "C" int aln_approx_match_batch(aln_ctx *ctx, int n, const aln_tile_pair *pairs,
                                      const aln_approx_params *P, aln_approx_result *out)
{
    if (!ctx || n < 0 || (n && (!pairs || !P || !out)) || n > 32767)
        return ctx ? set_err(ctx, ALN_ERR_ARG, "approx_match: bad arguments") : ALN_ERR_ARG;
    if (P && (P->thmdec < 1 || P->thmdec > 255))
        return set_err(ctx, ALN_ERR_ARG, "approx_match: thmdec %d", P ? P->thmdec : 0);
    // ---- Crop (CThmUtil.cpp:385-426): views of the overlap boxes ----------
    std::vector<aln_image> crop(2 * (size_t)n);
    std::vector<int> live;
    for (int k = 0; k < n; ++k) {
        aln_approx_result &o = out[k];
        memset(&o, 0, sizeof o);
        const aln_image &A = pairs[k].a, &B = pairs[k].b;
        if (!A.data || !B.data || A.w != B.w || A.h != B.h || A.w < 1 || A.h < 1 ||
            A.stride < A.w || B.stride < B.w || A.dtype != B.dtype || !dtype_size(A.dtype))
            return set_err(ctx, ALN_ERR_ARG, "approx_match pair %d: tiles must match", k);
        const int w = A.w, h = A.h;
        const size_t es = dtype_size(A.dtype);
        bool whole = P->xyconf == 0.0;
        IBoxI Ba{0, w - 1, 0, h - 1}, Bb{0, w - 1, 0, h - 1};
        if (!whole) {
            // GetOlapBoxes (CThmUtil.cpp:355-377) with px.scl = 1
            const int dx = (int)(P->xyconf * pairs[k].tabx);
            const int dy = (int)(P->xyconf * pairs[k].taby);
            boxes_from_shifts(Ba, Bb, w, h, w, h, dx, dy);
            const int min1d = std::max(P->olap1d, 8);
            if (Ba.R - Ba.L + 1 < min1d || Ba.T - Ba.B + 1 < min1d) {
                whole = true;   // "1D overlap too small": the whole tiles
                Ba = IBoxI{0, w - 1, 0, h - 1};
                Bb = Ba;
            } else if ((long long)(Ba.R - Ba.L + 1) * (Ba.T - Ba.B + 1) <= P->olap2d) {
                o.status = 1;   // SubI_ThisBox: small intersection
                continue;
            }
        }
        const IBoxI *bx[2] = {&Ba, &Bb};
        const aln_image *im[2] = {&A, &B};
        for (int i = 0; i < 2; ++i) {
            aln_image v = *im[i];
            v.data = (const char *)im[i]->data +
                     ((size_t)bx[i]->B * im[i]->stride + bx[i]->L) * es;
            v.w = bx[i]->R - bx[i]->L + 1;
            v.h = bx[i]->T - bx[i]->B + 1;
            v.x0 = v.y0 = 0;
            crop[2 * live.size() + i] = v;
        }
        o.crop[0] = Ba.L;
        o.crop[1] = Ba.B;
        o.crop[2] = Bb.L;
        o.crop[3] = Bb.B;
        o.crop_w = Ba.R - Ba.L + 1;
        o.crop_h = Ba.T - Ba.B + 1;
        live.push_back(k);
    }
    const int m = (int)live.size();
    if (m == 0)
        return ALN_OK;
    // ---- MakeThumbs (CThmUtil.cpp:470-523) at THMDEC and at 1 --------------
    auto make_thumbs = [&](int dec, std::vector<Thumb> &th) -> int {
        th.assign(2 * (size_t)m, Thumb());
        std::vector<double *> ov(2 * (size_t)m);
        std::vector<unsigned char *> om(2 * (size_t)m);
        std::vector<double> sd(2 * (size_t)m);
        for (int q = 0; q < 2 * m; ++q) {
            th[q].w = (crop[q].w + dec - 1) / dec;
            th[q].h = (crop[q].h + dec - 1) / dec;
            th[q].v.resize((size_t)th[q].w * th[q].h);
            th[q].m.resize((size_t)th[q].w * th[q].h);
            ov[q] = th[q].v.data();
            om[q] = th[q].m.data();
        }
        if (int rc = aln_decimate_batch(ctx, 2 * m, crop.data(), nullptr, dec, 1, ov.data(),
                                        om.data(), sd.data()))
            return rc;
        for (int q = 0; q < 2 * m; ++q) {
            th[q].sd = sd[q];
            long long c = 0;
            for (unsigned char b : th[q].m)
                c += b != 0;
            th[q].present = c;
        }
        return ALN_OK;
    };
    const int dec = P->thmdec;
    const long long req_thumb = P->olap2d / ((long long)dec * dec);
    std::vector<Thumb> thm;
    if (int rc = make_thumbs(dec, thm))
        return rc;
    std::vector<int> act;                 // pairs with usable thumbnails
    std::vector<aln_thumbs> T;
    std::vector<std::vector<double>> bras(m);
    for (int q = 0; q < m; ++q) {
        aln_approx_result &o = out[live[q]];
        const Thumb &a = thm[2 * q], &b = thm[2 * q + 1];
        aln_thumbs t;
        if (a.present < req_thumb || !(a.sd > 0.0) || !(b.sd > 0.0) ||
            !thumbs_of(a, b, bras[q], t)) {
            o.status = 2;
            continue;
        }
        t.req_area = req_thumb;
        t.olap1d = P->olap1d / dec;
        t.b_key = 0;
        T.push_back(t);
        act.push_back(q);
    }
    const int na = (int)act.size();
    if (na == 0)
        return ALN_OK;
    // ---- Sweep (CThmUtil.cpp:607-633) as ApproximateMatch configures it ---
    aln_thm_params prm;
    memset(&prm, 0, sizeof prm);
    prm.rthresh = P->rthresh;
    prm.nbmaxht = P->nbmaxht;
    prm.constxy = 1;
    prm.pretweak = P->pretweak;
    prm.usecorrr = 1;
    prm.ox = prm.oy = 0;
    prm.rx = prm.ry = -1;
    prm.tdfm[0] = prm.tdfm[4] = 1.0;
    std::vector<aln_thm_result> best(na);
    std::vector<double> tw(6 * (size_t)na), ret(na), args(4 * (size_t)na);
    for (int q = 0; q < na; ++q) {
        memset(&best[q], 0, sizeof best[q]);
        best[q].A = best[q].X = best[q].Y = best[q].R = -999.0;   // CThmScan::Initialize
        const double id[6] = {1, 0, 0, 0, 1, 0};
        memcpy(&tw[6 * q], id, sizeof id);
        args[4 * q] = P->ang0;
        args[4 * q + 1] = P->mode_prior ? P->hfangpr : P->hfangdn;
        args[4 * q + 2] = 0.5;
        args[4 * q + 3] = 0.0;
    }
    if (int rc = aln_thm_call_batch(ctx, na, T.data(), &prm,
                                    P->mode_prior ? ALN_THMOP_PRIOR : ALN_THMOP_DENOVO,
                                    args.data(), best.data(), tw.data(), ret.data()))
        return rc;
    std::vector<int> fin;   // pairs whose sweep succeeded
    for (int q = 0; q < na; ++q) {
        aln_approx_result &o = out[live[act[q]]];
        o.sweep[0] = best[q].A;
        o.sweep[1] = best[q].X;
        o.sweep[2] = best[q].Y;
        o.sweep[3] = best[q].R;
        o.err = best[q].err;
        if (ret[q] == 0.0)
            o.status = 3;
        else
            fin.push_back(q);
    }
    const int nf = (int)fin.size();
    if (nf == 0)
        return ALN_OK;
    // ---- Finish (CThmUtil.cpp:889-971) ------------------------------------
    std::vector<aln_thumbs> Tf(nf);
    std::vector<aln_thm_result> bf(nf);
    std::vector<double> twf(6 * (size_t)nf), zargs(4 * (size_t)nf, 0.0);
    for (int i = 0; i < nf; ++i) {
        Tf[i] = T[fin[i]];
        bf[i] = best[fin[i]];
        memcpy(&twf[6 * i], &tw[6 * fin[i]], 6 * sizeof(double));
    }
    if (P->tweaks)
        if (int rc = aln_thm_call_batch(ctx, nf, Tf.data(), &prm, ALN_THMOP_POSTTWEAKS,
                                        zargs.data(), bf.data(), twf.data(), nullptr))
            return rc;
    for (int i = 0; i < nf; ++i) {   // undo the thumbnail scale
        bf[i].X *= dec;
        bf[i].Y *= dec;
    }
    std::vector<Thumb> full;
    if (dec > 1) {
        if (int rc = make_thumbs(1, full))
            return rc;
    } else
        full = thm;
    std::vector<std::vector<double>> brf(nf);
    std::vector<int> ok(nf, 1);
    for (int i = 0; i < nf; ++i) {
        const int q = act[fin[i]];
        const Thumb &a = full[2 * q], &b = full[2 * q + 1];
        if (a.present < P->olap2d || !(a.sd > 0.0) || !(b.sd > 0.0) ||
            !thumbs_of(a, b, brf[i], Tf[i])) {
            ok[i] = 0;
            out[live[q]].status = 2;
            // a stand-in the call can run on; its result is not used
            Tf[i] = T[fin[i]];
        }
        Tf[i].req_area = P->olap2d;
        Tf[i].olap1d = P->olap1d;
        Tf[i].b_key = 0;
    }
    if (int rc = aln_thm_call_batch(ctx, nf, Tf.data(), &prm, ALN_THMOP_FULLRES, zargs.data(),
                                    bf.data(), twf.data(), nullptr))
        return rc;
    for (int i = 0; i < nf; ++i) {
        if (!ok[i])
            continue;
        aln_approx_result &o = out[live[act[fin[i]]]];
        aln_thm_result &b = bf[i];
        // IsectToImageCoords (CThmUtil.cpp:657-668): aO through T's linear part
        const double ax = o.crop[0], ay = o.crop[1];
        const double rx = b.T[0] * ax + b.T[1] * ay, ry = b.T[3] * ax + b.T[4] * ay;
        b.X += o.crop[2] - rx;
        b.Y += o.crop[3] - ry;
        b.T[2] = b.X;
        b.T[5] = b.Y;
        o.A = b.A;
        o.X = b.X;
        o.Y = b.Y;
        o.R = b.R;
        memcpy(o.T, b.T, sizeof o.T);
        o.err = b.err;
        // Check_LIMXY (CThmUtil.cpp:817-845): Tab^-1 * T's translation; Tab is
        // the pure translation (tabx, taby)
        const double ex = b.T[2] - pairs[live[act[fin[i]]]].tabx;
        const double ey = b.T[5] - pairs[live[act[fin[i]]]].taby;
        const double e = sqrt(ex * ex + ey * ey);
        o.status = (P->limxy && e > P->limxy) ? 4 : 0;
    }
    return ALN_OK;
}
