/*
 * stubs.cpp -- the six debug/disk symbols the reference's correlation
 * sources reference but that live in libraries not built here (ImageIO,
 * Disk, File, Memory).  They are only reached under -dbgcor or from
 * unrelated code, so they do nothing.  Test infrastructure only.
 * Signatures follow 0_GEN/ImageIO.h:52,87,94, Disk.h:44, File.h:72,
 * Memory.h:13.
 */
#include <stdio.h>
#include <vector>
using namespace std;

void Raster8ToTif8(const char *, const unsigned char *, int, int, FILE *) {}
void RasterDblToTifFlt(const char *, const double *, int, int, FILE *) {}
void CorrThmToTif8(const char *, const vector<double> &, int, int, int, FILE *) {}
bool DskExists(const char *) { return false; }
FILE *FileOpenOrDie(const char *name, const char *rw, FILE *)
{
    return fopen(name, rw);
}
void VMStats(FILE *) {}
