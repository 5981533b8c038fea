// aln_thmscan.hpp -- class CThmScan (0_GEN/CThmScan.h:57-223) as
// libaln_corr_shim.so serves it on the GPU: the same class, member order and
// member function signatures as the reference, so that callers compiled
// against the reference's header (ApproximateMatch, CThmUtil, scapeops,
// cross_thisblock, Thumbs) link against the shim unchanged -- their inline
// setters write these members at these offsets.
//
// The types are the reference's: TAffine is six doubles t[0..5]
// (0_GEN/TAffine.h), CorRec a TAffine and four doubles, ThmRec the thumbnail
// record (0_GEN/CThmScan.h:27-34).  Only the data layout of TAffine is
// declared here (the shim never calls its member functions).  A translation
// unit that includes the reference's own headers must not include this one.
#pragma once

#include <cstdio>
#include <vector>

#include "aln_correlation.hpp"

// CThmScan error codes (0_GEN/CThmScan.h:13-17)
enum thmerrs { errOK = 0, errLowRDenov = 1, errLowRPrior = 2 };

class TAffine {
public:
    double t[6];

public:
    TAffine()
    {
        t[0] = 1.0; t[1] = 0.0; t[2] = 0.0;
        t[3] = 0.0; t[4] = 1.0; t[5] = 0.0;
    }
    TAffine(const TAffine &rhs)   // user-provided, as the reference's
    {
        for (int i = 0; i < 6; ++i)
            t[i] = rhs.t[i];
    }
    TAffine &operator=(const TAffine &rhs) = default;
};

typedef struct {
    std::vector<double> av, bv;
    std::vector<Point> ap, bp;
    std::vector<CD> ftc;   // B's spectrum cache (the shim keeps a key in it)
    long reqArea;
    int olap1D, scl;
} ThmRec;

class CorRec {
public:
    TAffine T;
    double X, Y, A, R;

public:
    CorRec() {}
    CorRec(double A) : A(A) {}
};

typedef void (*T_NewAngProc)(int &Ox, int &Oy, int &Rx, int &Ry, double deg);

class CThmScan {
    friend void *_TCDGet(void *icstart);
    friend bool BigEnough(int sx, int sy, void *a);

private:
    class PTWRec {
    public:
        double a;
        int sel;

    public:
        PTWRec(int sel, double a) : a(a), sel(sel) {}
    };
    class ThrCorDat {
    public:
        int nthr;

    public:
        ThmRec *thm;
        std::vector<CorRec> vC;
        std::vector<PTWRec> vT;
    };

private:
    ThrCorDat TCD;
    T_NewAngProc newAngProc;
    FILE *flog;
    TAffine Tdfm, Tptwk;
    double rthresh, nbmaxht;
    int err, swpConstXY, swpPretweak, swpNThreads, useCorrR, Ox, Oy, Rx, Ry, olap1D;

private:
    // one member-function call on the GPU (aln_thm_call_batch, one pair);
    // the shim's own, not exported
    __attribute__((visibility("hidden"))) bool gpu_call(int op, CorRec &best, ThmRec &thm,
                                                        double a0, double a1, double a2,
                                                        double a3, double *ret);

public:
    CThmScan();
    void Initialize(FILE *flog, CorRec &best);
    void SetFlog(FILE *flog) { this->flog = flog; }
    void SetTdfm(const TAffine &Tdfm) { this->Tdfm = Tdfm; }
    void SetRThresh(double rthresh) { this->rthresh = rthresh; }
    void SetNbMaxHt(double nbmaxht) { this->nbmaxht = nbmaxht; }
    void SetSweepConstXY(int swpConstXY) { this->swpConstXY = swpConstXY; }
    void SetSweepPretweak(int swpPretweak) { this->swpPretweak = swpPretweak; }
    void SetSweepNThreads(int swpNThreads) { this->swpNThreads = swpNThreads; }
    void SetUseCorrR(int useCorrR) { this->useCorrR = useCorrR; }
    void SetDisc(int Ox, int Oy, int Rx, int Ry)
    {
        this->Ox = Ox;
        this->Oy = Oy;
        this->Rx = Rx;
        this->Ry = Ry;
    }
    void SetNewAngProc(T_NewAngProc proc) { newAngProc = proc; }
    void GetTptwk(TAffine &Tptwk) { Tptwk = this->Tptwk; }
    void SetTptwk(const TAffine &Tptwk) { this->Tptwk = Tptwk; }
    int GetErr() { return err; }
    bool Pretweaks(double bestR, double deg, ThmRec &thm);
    void RFromAngle(CorRec &C, double deg, ThmRec &thm, int iaux = -1);
    void DebugAngs(int alyr, int atil, int blyr, int btil, double center, double hlfwid,
                   double step, ThmRec &thm);
    double AngleScanMaxR(CorRec &best, double center, double hlfwid, double step,
                         bool favorCenter, ThmRec &thm);
    double AngleScanConstXY(CorRec &best, double center, double hlfwid, double step,
                            ThmRec &thm);
    double AngleScanSel(CorRec &best, double center, double hlfwid, double step,
                        bool favorCenter, ThmRec &thm);
    double AngleScanWithTweaks(CorRec &best, double center, double hlfwid, double step,
                               ThmRec &thm);
    double PeakHunt(CorRec &best, double hlfwid, ThmRec &thm);
    bool UsePriorAngles(CorRec &best, int nprior, double ang0, double hfangpr, ThmRec &thm);
    bool DenovoBestAngle(CorRec &best, double ang0, double hfangdn, double step, ThmRec &thm,
                         bool failmsg);
    void PostTweaks(CorRec &best, ThmRec &thm);
    void FinishAtFullRes(CorRec &best, ThmRec &thm);
};

// LegalRgn of the sweep's correlator (0_GEN/CThmScan.cpp:28-33): reads the
// olap1D of the most recently used CThmScan, as the reference's does.
bool BigEnough(int sx, int sy, void *a);
