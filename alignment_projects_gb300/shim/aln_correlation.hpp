// aln_correlation.hpp -- the Correlation.h entry points (0_GEN/Correlation.h)
// that libaln_corr_shim.so serves on the GPU, declared with the reference's
// exact C++ signatures so that its callers link against the shim unchanged.
//
// The types are the reference's: Point is a pair of doubles (x, y)
// (0_GEN/CPoint.h), CD is std::complex<double> (0_GEN/GenDefs.h), EvalType
// is the legality callback of 0_GEN/Correlation.h.  A translation unit that
// includes the reference's own headers must not include this one (it would
// see Point twice); the reference's Correlation.h declares the same
// functions.
#pragma once

#include <complex>
#include <cstdio>
#include <vector>

class Point {
public:
    double x, y;

public:
    Point() : x(0.0), y(0.0) {}
    Point(double x, double y) : x(x), y(y) {}
};

typedef std::complex<double> CD;
typedef bool (*EvalType)(int sx, int sy, void *v);

// FFTSize, FFTSizeSQR (0_GEN/Correlation.cpp:344-359)
int FFTSize(int n1, int n2);
int FFTSizeSQR(int w1, int h1, int w2, int h2);

// FFT_2D / IFT_2D (0_GEN/Correlation_fft_fftw.cpp:10-92): FFTW's r2c / c2r
// contract, computed on the GPU in FP32.  FFT_2D with cached = true returns
// at once when out already holds Nslow * (Nfast/2+1) values.
int FFT_2D(std::vector<CD> &out, const std::vector<double> &in, int Nfast, int Nslow,
           bool cached, FILE *flog = stderr);
void IFT_2D(std::vector<double> &out, const std::vector<CD> &in, int Nfast, int Nslow,
            FILE *flog = stderr);

// Convolve (0_GEN/Correlation.cpp:371-457); kfft keeps the reference's size
// contract (its contents are not used: the GPU recomputes the kernel's
// transform)
void Convolve(std::vector<double> &dst, const std::vector<double> &src, int ws, int hs,
              const double *K, int wk, int hk, bool kIsSymmetric, bool preNormK,
              std::vector<CD> &kfft, FILE *flog);

// ParabPeakFFT (0_GEN/Correlation.cpp:482-517)
void ParabPeakFFT(double &xpk, double &ypk, int d, const double *I, int nx, int ny);

// CorrPatches (0_GEN/Correlation.cpp:901-1170)
double CorrPatches(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2, int Ox,
                   int Oy, int radius, EvalType LegalRgn, void *arglr, EvalType LegalCnt,
                   void *arglc, std::vector<CD> &fft2);

// CorrPatchToImage (0_GEN/Correlation.cpp:1186-1355)
double CorrPatchToImage(double &dx, double &dy, const std::vector<Point> &ip1,
                        const std::vector<double> &iv1, const std::vector<double> &i2, int Ox,
                        int Oy, int radius, bool bFilter);

// GradDescStep / CorrVectors / ImproveControlPts (0_GEN/Correlation.cpp:1403-1721)
void GradDescStep(std::vector<double> &bnew, std::vector<Point> &dRdc,
                  const std::vector<Point> &ac, const std::vector<std::vector<double> > &am,
                  const std::vector<double> &av, const std::vector<double> &bimg, int w, int h);
double CorrVectors(FILE *flog, const std::vector<double> &a, const std::vector<double> &b,
                   int *nnz = NULL);
double ImproveControlPts(std::vector<Point> &ac, const std::vector<std::vector<double> > &am,
                         const std::vector<double> &av, const std::vector<double> &bimg, int w,
                         int h, FILE *flog, const char *describe, double iniThresh,
                         double finThresh);

// CorrImagesF / CorrImagesR / CorrImagesS (0_GEN/Correlation.cpp:3066-3290)
double CorrImagesF(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2,
                   EvalType LegalRgn, void *arglr, EvalType LegalCnt, void *arglc,
                   double mincor, double nbmaxht, int Ox, int Oy, int Rx, int Ry,
                   std::vector<CD> &fft2);
double CorrImagesR(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2,
                   EvalType LegalRgn, void *arglr, EvalType LegalCnt, void *arglc,
                   double mincor, double nbmaxht, int Ox, int Oy, int Rx, int Ry,
                   std::vector<CD> &fft2);
double CorrImagesS(FILE *flog, int verbose, double &dx, double &dy,
                   const std::vector<Point> &ip1, const std::vector<double> &iv1,
                   const std::vector<Point> &ip2, const std::vector<double> &iv2,
                   EvalType LegalRgn, void *arglr, EvalType LegalCnt, void *arglc,
                   double mincor, double nbmaxht, int Ox, int Oy, int Rx, int Ry,
                   std::vector<CD> &fft2);
