// Drives libaln_corr_shim.so through the reference's C++ signatures
// (aln_correlation.hpp).  Reads cases from a binary file, writes one result
// line per case:  r dx dy
//
// case record (little-endian): int32 kind, int32 n1, double[2*n1] points,
// double[n1] values, int32 n2, double[2*n2], double[n2], int32 Ox, Oy,
// radius, Rx, Ry, int32 rgn_min (0: no LegalRgn, else olw, olh >= it and
// area > rgn_area), int64 rgn_area, int64 cnt_n (-1: no LegalCnt), double
// mincor, int32 reuse (1: use the previous case's fft2 vector)
// kind 0 = CorrPatches, 1 = CorrImagesR, 2 = CorrImagesS, 3 = CorrImagesF
#include "aln_correlation.hpp"

#include <cstdint>
#include <cstdio>
#include <vector>

struct RgnArg {
    int mn;
    long long area;
};

static bool rgn_cb(int sx, int sy, void *a)
{
    const RgnArg *r = (const RgnArg *)a;
    return sx >= r->mn && sy >= r->mn && (long long)sx * sy > r->area;
}

static bool cnt_cb(int c1, int c2, void *a)
{
    const long long n = *(const long long *)a;
    return c1 > n && c2 > n;
}

template <typename T>
static bool rd(FILE *f, T &v)
{
    return fread(&v, sizeof v, 1, f) == 1;
}

static bool rd_cloud(FILE *f, std::vector<Point> &p, std::vector<double> &v)
{
    int32_t n;
    if (!rd(f, n))
        return false;
    p.resize(n);
    v.resize(n);
    for (int i = 0; i < n; ++i)
        if (!rd(f, p[i].x) || !rd(f, p[i].y))
            return false;
    for (int i = 0; i < n; ++i)
        if (!rd(f, v[i]))
            return false;
    return true;
}

int main(int argc, char **argv)
{
    if (argc < 2)
        return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f)
        return 2;
    std::vector<CD> fft2;
    int32_t kind;
    while (rd(f, kind)) {
        std::vector<Point> p1, p2;
        std::vector<double> v1, v2;
        int32_t Ox, Oy, rad, Rx, Ry, rmin, reuse;
        int64_t rarea, cn;
        double mincor;
        if (!rd_cloud(f, p1, v1) || !rd_cloud(f, p2, v2) || !rd(f, Ox) || !rd(f, Oy) ||
            !rd(f, rad) || !rd(f, Rx) || !rd(f, Ry) || !rd(f, rmin) || !rd(f, rarea) ||
            !rd(f, cn) || !rd(f, mincor) || !rd(f, reuse))
            return 3;
        if (!reuse)
            fft2.clear();
        RgnArg ra = {rmin, rarea};
        long long cnv = cn;
        EvalType lr = rmin > 0 ? rgn_cb : nullptr;
        EvalType lc = cn >= 0 ? cnt_cb : nullptr;
        double dx = 0.0, dy = 0.0, r = 0.0;
        if (kind == 0)
            r = CorrPatches(stderr, 0, dx, dy, p1, v1, p2, v2, Ox, Oy, rad, lr, &ra, lc, &cnv,
                            fft2);
        else if (kind == 3)
            r = CorrImagesF(stderr, 0, dx, dy, p1, v1, p2, v2, lr, &ra, lc, &cnv, mincor, 0.75,
                            Ox, Oy, Rx, Ry, fft2);
        else if (kind == 1)
            r = CorrImagesR(stderr, 0, dx, dy, p1, v1, p2, v2, lr, &ra, lc, &cnv, mincor, 0.75,
                            Ox, Oy, Rx, Ry, fft2);
        else
            r = CorrImagesS(stderr, 0, dx, dy, p1, v1, p2, v2, lr, &ra, lc, &cnv, mincor, 0.75,
                            Ox, Oy, Rx, Ry, fft2);
        printf("%.17g %.17g %.17g\n", r, dx, dy);
    }
    // FFT_2D / IFT_2D round trip on an 8 x 4 ramp: IFT(FFT(x)) = N x
    std::vector<double> in(32), back;
    for (int i = 0; i < 32; ++i)
        in[i] = i * 0.5 - 3.0;
    std::vector<CD> spec;
    const int M = FFT_2D(spec, in, 8, 4, false);
    IFT_2D(back, spec, 8, 4);
    double err = 0.0;
    for (int i = 0; i < 32; ++i) {
        const double d = back[i] / 32.0 - in[i];
        err = d > err ? d : (-d > err ? -d : err);
    }
    printf("fft %d %.3g %d\n", M, err, FFTSize(300, 257));
    return 0;
}
