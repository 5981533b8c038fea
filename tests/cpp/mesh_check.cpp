// A reference-style caller of the mesh optimizer (0_GEN/Correlation.h:127-152)
// linked against the C++ drop-in: reads cases from argv[1] (per case: nc, nm,
// w, h as int32; iniThresh, finThresh; ac[2 nc]; am dense nm x nc; av[nm];
// bimg[w h] as doubles), calls GradDescStep + CorrVectors at the start, then
// ImproveControlPts, and prints per case: corr0 corr ac...
#include <cstdio>
#include <vector>

#include "aln_correlation.hpp"

int main(int argc, char **argv)
{
    FILE *f = fopen(argv[1], "rb");
    FILE *lg = fopen("/dev/null", "w");
    if (!f || !lg)
        return 2;
    int hdr[4];
    while (fread(hdr, sizeof(int), 4, f) == 4) {
        const int nc = hdr[0], nm = hdr[1], w = hdr[2], h = hdr[3];
        double th[2];
        if (fread(th, sizeof(double), 2, f) != 2)
            return 3;
        std::vector<double> acd(2 * (size_t)nc), avd(nm), bimg((size_t)w * h);
        std::vector<std::vector<double> > am(nm, std::vector<double>(nc));
        if (fread(acd.data(), sizeof(double), acd.size(), f) != acd.size())
            return 3;
        for (int i = 0; i < nm; ++i)
            if (fread(am[i].data(), sizeof(double), nc, f) != (size_t)nc)
                return 3;
        if (fread(avd.data(), sizeof(double), nm, f) != (size_t)nm ||
            fread(bimg.data(), sizeof(double), bimg.size(), f) != bimg.size())
            return 3;
        std::vector<Point> ac(nc);
        for (int j = 0; j < nc; ++j)
            ac[j] = Point(acd[2 * j], acd[2 * j + 1]);
        std::vector<double> bnew;
        std::vector<Point> dRdc;
        GradDescStep(bnew, dRdc, ac, am, avd, bimg, w, h);
        const double c0 = CorrVectors(lg, avd, bnew);
        const double c = ImproveControlPts(ac, am, avd, bimg, w, h, lg, "check", th[0], th[1]);
        printf("%.17g %.17g", c0, c);
        for (int j = 0; j < nc; ++j)
            printf(" %.17g %.17g", ac[j].x, ac[j].y);
        printf("\n");
    }
    return 0;
}
