// aln_thmpair.cuh -- the pipeline's ThmPair_<za>^<zb>.txt table
// (0_GEN/PipeFiles.h:146-152, PipeFiles.cpp:1129-1360): one line per tile
// pair match, tab separated, the reference's printf formats, the header
// line of WriteThmPairHdr.  Host file I/O around the GPU matcher, so the
// matcher's results feed the pipeline's later stages.  Included by
// aln_corr.cu.
#pragma once

#include <fcntl.h>
#include <sys/file.h>
#include <unistd.h>

static std::string thmpair_path(const char *dir, int alr, int blr)
{
    char name[64];
    snprintf(name, sizeof name, "ThmPair_%d^%d.txt", alr, blr);
    return (dir && dir[0]) ? std::string(dir) + "/" + name : std::string(name);
}

extern "C" int aln_thmpair_write(const char *dir, int alr, int blr, int n,
                                 const aln_thmpair *recs)
{
    if (n < 0 || (n && !recs))
        return set_err(nullptr, ALN_ERR_ARG, "thmpair_write: bad arguments");
    const std::string path = thmpair_path(dir, alr, blr);
    // one writer at a time per table (the reference's CMutex "tpr_za_zb")
    const int fd = open(path.c_str(), O_WRONLY | O_CREAT | O_APPEND, 0664);
    if (fd < 0)
        return set_err(nullptr, ALN_ERR_ARG, "thmpair_write: cannot open %s", path.c_str());
    flock(fd, LOCK_EX);
    FILE *f = fdopen(fd, "a");
    if (!f) {
        close(fd);
        return set_err(nullptr, ALN_ERR_ARG, "thmpair_write: cannot open %s", path.c_str());
    }
    if (lseek(fd, 0, SEEK_END) == 0)   // a new table: the header first
        fprintf(f, "Atl\tAcr\tBtl\tBcr\tErr\tDeg\tR\tT0\tT1\tX\tT3\tT4\tY\n");
    for (int k = 0; k < n; ++k) {
        const aln_thmpair &t = recs[k];
        if (t.atl < 0 || t.btl < 0)   // WriteThmPair bypasses invalid tile ids
            continue;
        fprintf(f, "%d\t%d\t%d\t%d\t%d\t%f\t%f\t%f\t%f\t%f\t%f\t%f\t%f\n", t.atl, t.acr, t.btl,
                t.bcr, t.err, t.A, t.R, t.T[0], t.T[1], t.T[2], t.T[3], t.T[4], t.T[5]);
    }
    fflush(f);
    flock(fd, LOCK_UN);
    fclose(f);
    return ALN_OK;
}

extern "C" int aln_thmpair_read(const char *dir, int alr, int blr, int cap, aln_thmpair *out)
{
    if (cap < 0 || (cap && !out))
        return set_err(nullptr, ALN_ERR_ARG, "thmpair_read: bad arguments");
    const std::string path = thmpair_path(dir, alr, blr);
    FILE *f = fopen(path.c_str(), "r");
    if (!f)
        return set_err(nullptr, ALN_ERR_ARG, "thmpair_read: cannot open %s", path.c_str());
    char line[1024];
    int n = 0;
    bool header = true;
    while (fgets(line, sizeof line, f)) {
        if (header) {   // ReadAllThmPair skips the first line
            header = false;
            continue;
        }
        aln_thmpair t;
        if (sscanf(line, "%d\t%d\t%d\t%d\t%d\t%lf\t%lf\t%lf\t%lf\t%lf\t%lf\t%lf\t%lf", &t.atl,
                   &t.acr, &t.btl, &t.bcr, &t.err, &t.A, &t.R, &t.T[0], &t.T[1], &t.T[2],
                   &t.T[3], &t.T[4], &t.T[5]) != 13)
            continue;
        if (n < cap)
            out[n] = t;
        ++n;
    }
    fclose(f);
    return n;
}
