// aln_tune.cuh -- measured plan choices for CorrPatches' columns (the
// autotuner).  Included by aln_corr.cu before plan_pair.
//
// A CorrPatches pair can take its column correlation in one transform of
// the grid's Ny points per column, or cut a's rows into segments and make
// 2 nseg + 1 transforms of NS points (k2_corrseg).  Which is fastest, and
// at which NS, depends on the kernels as they run on this GPU (occupancy,
// register FFT radix, shared-memory passes, how many columns a batch
// brings), not on a formula.  So the first time a pair of a new class
// appears, the tuner times every valid choice on synthetic device pairs of
// that exact geometry (CUDA events around whole batches of them) and
// records in a file named for the GPU and the library build (which later
// processes read back) either the fastest choice, when it beats the cost
// model's pick by more than 10 %, or "cost model" (-1).  With "cost model"
// every pair of the class keeps its own cost-model plan: the class spans a
// range of heights, and the representative's pick is not the others'.
//
// Class: (Nx / 2, the unsegmented Ny, the window height Wy rounded up to a
// power of two, a's height rounded up to a power of two, a's pixel size).
// A pair's plan is a function of the pair and the class's entry, and an
// entry never changes once made, so a pair gets the same numbers alone, in
// any batch and in later calls.  Choices invalid for a particular pair of a
// class (a segment too short for its window) fall back to the cost model.
#pragma once

#include <dlfcn.h>

#include <fstream>

#ifndef ALN_BUILD_ID
#define ALN_BUILD_ID "dev"
#endif

struct JobKey;
static int batch_impl(aln_ctx *ctx, int npairs, const aln_pair *pairs, const ImgSpec *specs,
                      aln_result *out, const JobKey *keys);

struct TuneKey {
    int dev, L, nyf, wyb, h0b, es;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(dev, L, nyf, wyb, h0b, es) <
               std::tie(o.dev, o.L, o.nyf, o.wyb, o.h0b, o.es);
    }
};

static std::mutex g_tune_lock;
static std::map<TuneKey, int> g_tune;           // -> -1 cost model, 0 unsegmented, NS > 0
static bool g_tune_loaded[64];
static std::string g_tune_path[64];

static int tune_pow2(int n)
{
    int p = 1;
    while (p < n)
        p <<= 1;
    return p;
}

// <dir of this library>/tune/<gpu name>-<build id>.txt, or $ALN_TUNE_DIR/...
static std::string tune_file(int dev)
{
    std::string dir;
    if (const char *e = getenv("ALN_TUNE_DIR"))
        dir = e;
    else {
        Dl_info info;
        if (dladdr((void *)&tune_pow2, &info) && info.dli_fname) {
            dir = info.dli_fname;
            const size_t s = dir.rfind('/');
            dir = (s == std::string::npos ? std::string(".") : dir.substr(0, s)) + "/tune";
        } else
            dir = "tune";
    }
    cudaDeviceProp prop;
    std::string name = cudaGetDeviceProperties(&prop, dev) == cudaSuccess ? prop.name : "gpu";
    for (char &c : name)
        if (!isalnum((unsigned char)c))
            c = '_';
    mkdir(dir.c_str(), 0775);
    return dir + "/" + name + "-" + ALN_BUILD_ID + ".txt";
}

// one line per class: "L nyf wyb h0b es ns  ms(choice) ..." (g_tune_lock held)
static void tune_load(int dev)
{
    if (g_tune_loaded[dev])
        return;
    g_tune_loaded[dev] = true;
    g_tune_path[dev] = tune_file(dev);
    std::ifstream f(g_tune_path[dev]);
    std::string line;
    while (std::getline(f, line)) {
        TuneKey k{dev, 0, 0, 0, 0, 0};
        int ns = -1;
        if (sscanf(line.c_str(), "%d %d %d %d %d %d", &k.L, &k.nyf, &k.wyb, &k.h0b, &k.es,
                   &ns) == 6 &&
            ns >= -1)
            g_tune[k] = ns;
    }
}

// Synthetic device images for a class's timing runs: the pair's sizes and
// pixel types, filled with a fixed pseudo-random pattern (the kernels'
// time does not depend on the values).
static int tune_images(aln_ctx *ctx, const aln_pair &P, void **buf, aln_pair &S)
{
    const aln_image *im[2] = {&P.a, &P.b};
    size_t off[2], total = 0;
    for (int i = 0; i < 2; ++i) {
        off[i] = total;
        total += al256((size_t)im[i]->w * im[i]->h * dtype_size(im[i]->dtype));
    }
    std::vector<unsigned char> h(total);
    unsigned x = 12345u;
    for (size_t i = 0; i < total; ++i) {
        x = x * 1664525u + 1013904223u;
        h[i] = (unsigned char)(x >> 24);
    }
    // float pixels: a pattern of small values (the random bytes would include
    // non-numbers), written over the byte pattern
    for (int i = 0; i < 2; ++i) {
        const size_t n = (size_t)im[i]->w * im[i]->h;
        if (im[i]->dtype == ALN_F32)
            for (size_t q = 0; q < n; ++q)
                ((float *)(h.data() + off[i]))[q] = (float)h[off[i] + q % 4096 * 4] * 0.25f;
        else if (im[i]->dtype == ALN_F64)
            for (size_t q = 0; q < n; ++q)
                ((double *)(h.data() + off[i]))[q] = (double)h[off[i] + q % 4096 * 8] * 0.25;
    }
    CK(cudaMalloc(buf, total));
    CK(cudaMemcpy(*buf, h.data(), total, cudaMemcpyHostToDevice));
    S = P;
    S.b_key = 0;
    aln_image *sm[2] = {&S.a, &S.b};
    for (int i = 0; i < 2; ++i) {
        sm[i]->data = (char *)*buf + off[i];
        sm[i]->stride = sm[i]->w;
        sm[i]->on_device = 1;
    }
    return ALN_OK;
}

// The class's measured choice for a pair planned as d (caller-frame pair P),
// whose valid segment lengths are cand (the cost model's pick first, 0 =
// unsegmented).  Returns the choice, or -1 for the cost model's plan (the
// class entry says so, or the class cannot be measured), or -2 for a class
// not measured yet while the context plans on several threads.
static int tuned_segment(aln_ctx *ctx, const aln_pair &P, const PairDev &d, int Wy,
                         const std::vector<int> &cand)
{
    const int dev = ctx->device;
    if (dev < 0 || dev >= 64 || cand.size() < 2)
        return -1;
    const TuneKey key{dev, d.Nx / 2, d.Ny, tune_pow2(Wy), tune_pow2(d.h[0]),
                      (int)dtype_size(d.dt[0])};
    // Entries never change once made, so each planning thread keeps the
    // ones it has seen and takes the lock only for a class new to it (with
    // 16 threads planning, one lock per pair cost the uneven batch 3 %).
    static thread_local std::map<TuneKey, int> seen;
    auto sit = seen.find(key);
    if (sit != seen.end())
        return sit->second;
    std::lock_guard<std::mutex> g(g_tune_lock);
    tune_load(dev);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
        seen[key] = it->second;
        return it->second;
    }
    if (ctx->tune_defer)
        return -2;   // parallel planning: the caller plans this pair again
    // time each choice on a batch of copies of a synthetic pair like P
    void *buf = nullptr;
    aln_pair S;
    if (tune_images(ctx, P, &buf, S) != ALN_OK) {
        cudaGetLastError();
        return -1;
    }
    const long long work = (long long)d.Nx * d.Ny;
    const int M = (int)std::max(4LL, std::min(512LL, (4LL << 20) / std::max(1LL, work)));
    std::vector<aln_pair> pairs(M, S);
    std::vector<aln_result> out(M);
    // keep the caller's counters and profile free of the timing runs
    const int prof = ctx->prof_on, pol = ctx->seg_ns;
    const long long launches = ctx->launches, h2d = ctx->h2d_bytes, d2h = ctx->d2h_bytes,
                    chunks = ctx->chunks, copies = ctx->h2d_copies;
    ctx->prof_on = 0;
    ctx->tuning = 1;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<float> ms(cand.size(), 1e30f);
    for (size_t c = 0; c < cand.size(); ++c) {
        ctx->seg_ns = cand[c] == 0 ? -1 : cand[c];
        bool ok = batch_impl(ctx, M, pairs.data(), nullptr, out.data(), nullptr) == ALN_OK;
        for (int rep = 0; rep < 2 && ok; ++rep) {
            cudaEventRecord(e0, ctx->stream);
            ok = batch_impl(ctx, M, pairs.data(), nullptr, out.data(), nullptr) == ALN_OK;
            cudaEventRecord(e1, ctx->stream);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            if (ok)
                ms[c] = std::min(ms[c], t);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->seg_ns = pol;
    ctx->tuning = 0;
    ctx->prof_on = prof;
    ctx->launches = launches;
    ctx->h2d_bytes = h2d;
    ctx->d2h_bytes = d2h;
    ctx->chunks = chunks;
    ctx->h2d_copies = copies;
    cudaFree(buf);
    cudaGetLastError();
    ctx->tune_classes++;
    // the fastest, where it beats the cost model's pick by > 10 % (a class
    // that leaves the common plan splits the batch's chunks); else the cost
    // model, pair by pair
    size_t best = 0;
    for (size_t c = 1; c < cand.size(); ++c)
        if (ms[c] < ms[best])
            best = c;
    if (ms[best] >= 1e29f)
        return -1;
    const int choice = ms[best] > 0.90f * ms[0] ? -1 : cand[best];
    g_tune[key] = choice;
    seen[key] = choice;
    if (FILE *f = fopen(g_tune_path[dev].c_str(), "a")) {
        fprintf(f, "%d %d %d %d %d %d ", key.L, key.nyf, key.wyb, key.h0b, key.es, choice);
        for (size_t c = 0; c < cand.size(); ++c)
            fprintf(f, " %d:%.4f", cand[c], ms[c]);
        fprintf(f, "\n");
        fclose(f);
    }
    return choice;
}

// The class's recorded choice, without measuring (planning queries without
// a context); -1 when the class has none yet.
static int recorded_segment(const PairDev &d, int Wy)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return -1;
    }
    const TuneKey key{dev, d.Nx / 2, d.Ny, tune_pow2(Wy), tune_pow2(d.h[0]),
                      (int)dtype_size(d.dt[0])};
    std::lock_guard<std::mutex> g(g_tune_lock);
    tune_load(dev);
    auto it = g_tune.find(key);
    return it == g_tune.end() ? -1 : it->second;
}
