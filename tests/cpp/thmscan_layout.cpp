// Prints the data layout of class CThmScan and its record types, compiled
// against the shim's header (aln_thmscan.hpp) or, with
// -DALN_REFERENCE_HEADERS, against the reference's 0_GEN/CThmScan.h: the two
// outputs must be equal, since callers built from the reference's header
// run the shim's member functions on objects they lay out themselves.
// (private is opened only to name the members in offsetof; the standard
// headers come first so that they are not affected.)
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#define private public
#ifdef ALN_REFERENCE_HEADERS
#include "CThmScan.h"
#else
#include "aln_thmscan.hpp"
#endif
#undef private

#include <cstddef>
#include <cstdio>

#define OFF(C, m) printf(#C "." #m " %zu\n", offsetof(C, m))

int main()
{
    printf("sizeof CThmScan %zu ThmRec %zu CorRec %zu TAffine %zu\n", sizeof(CThmScan),
           sizeof(ThmRec), sizeof(CorRec), sizeof(TAffine));
    OFF(CThmScan, TCD);
    OFF(CThmScan, newAngProc);
    OFF(CThmScan, flog);
    OFF(CThmScan, Tdfm);
    OFF(CThmScan, Tptwk);
    OFF(CThmScan, rthresh);
    OFF(CThmScan, nbmaxht);
    OFF(CThmScan, err);
    OFF(CThmScan, swpConstXY);
    OFF(CThmScan, swpPretweak);
    OFF(CThmScan, swpNThreads);
    OFF(CThmScan, useCorrR);
    OFF(CThmScan, Ox);
    OFF(CThmScan, Oy);
    OFF(CThmScan, Rx);
    OFF(CThmScan, Ry);
    OFF(CThmScan, olap1D);
    OFF(ThmRec, av);
    OFF(ThmRec, bv);
    OFF(ThmRec, ap);
    OFF(ThmRec, bp);
    OFF(ThmRec, ftc);
    OFF(ThmRec, reqArea);
    OFF(ThmRec, olap1D);
    OFF(ThmRec, scl);
    OFF(CorRec, T);
    OFF(CorRec, X);
    OFF(CorRec, Y);
    OFF(CorRec, A);
    OFF(CorRec, R);
    return 0;
}
