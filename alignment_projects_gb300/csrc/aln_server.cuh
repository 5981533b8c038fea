// aln_server.cuh -- continuous batching of pair-match requests (the
// aln_server_* entry points), included at the end of aln_corr.cu.
//
// Requests wait in one FIFO queue.  Each worker thread owns a context (its
// own CUDA streams, workspace and spectrum cache); whenever it is free it
// takes every waiting request of one class (correlations, or sweeps) that it
// can admit -- at most max_batch, planned workspace within its share of the
// memory budget -- and runs them as one batch through the batched pipeline.
// Requests that arrive while batches are on the device wait for the next
// free worker, so the device always has the newest work queued behind the
// running batches, and the workers' batches overlap on the device.
#pragma once

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>
#include <unordered_set>

struct SrvReq {
    unsigned long long ticket;
    aln_request req;
    size_t bytes;        // planned device workspace (admission)
    double t_submit;     // ms, steady clock
};

struct aln_server {
    aln_server_params P;
    size_t worker_budget;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<SrvReq> q;
    std::unordered_map<unsigned long long, aln_reply> done;
    std::unordered_set<unsigned long long> outstanding;   // submitted, not handed over
    std::vector<std::thread> th;
    std::vector<aln_ctx *> ctxs;
    bool stop;
    unsigned long long next_ticket;
    long long n_sub, n_fin, n_batches;
    char err[512];
};

static double srv_now_ms()
{
    return std::chrono::duration<double, std::milli>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// CorrImages job -> (pair, spec), as aln_corr_images_batch builds them
static void srv_image_job(const aln_image_job &J, aln_pair &P, ImgSpec &S)
{
    memset(&P, 0, sizeof P);
    memset(&S, 0, sizeof S);
    P.a = J.a;
    P.b = J.b;
    P.radius = 1 << 20;
    P.legal = J.legal;
    P.b_key = J.b_key;
    S.kind = J.kind == ALN_CORR_S ? 2 : J.kind == ALN_CORR_F ? 4 : 1;
    S.mincor = J.mincor;
    S.nbmaxht = J.nbmaxht;
    S.ox = J.ox;
    S.oy = J.oy;
    S.rx = J.rx;
    S.ry = J.ry;
}

// Planned device workspace of one request (0 if it does not plan: the
// worker reports the error).  A sweep is charged a fixed share.
static size_t srv_bytes(const aln_request &r)
{
    static thread_local aln_ctx scratch;   // plan_pair only writes its error text
    PairPlan pl;
    if (r.kind == ALN_REQ_PATCHES) {
        if (plan_pair(&scratch, r.pair, pl, true, nullptr) != ALN_OK)
            return 0;
        return pl.ws_bytes;
    }
    if (r.kind == ALN_REQ_IMAGES) {
        aln_pair P;
        ImgSpec S;
        srv_image_job(r.job, P, S);
        if (plan_pair(&scratch, P, pl, false, &S) != ALN_OK)
            return 0;
        return pl.ws_bytes;
    }
    return (size_t)16 << 20;
}

static bool srv_is_sweep(const SrvReq &r) { return r.req.kind == ALN_REQ_SWEEP; }

// sweeps run together only with identical settings (one aln_thm_search_batch)
static bool srv_same_sweep(const aln_request &a, const aln_request &b)
{
    return memcmp(&a.thm, &b.thm, sizeof a.thm) == 0 && a.thm_mode == b.thm_mode &&
           a.ang0 == b.ang0 && a.hfang == b.hfang && a.step == b.step;
}

static void srv_run(aln_server *S, aln_ctx *ctx, std::vector<SrvReq> &batch,
                    std::vector<aln_reply> &rep)
{
    const int n = (int)batch.size();
    rep.assign(n, aln_reply());
    for (auto &r : rep)
        memset(&r, 0, sizeof r);
    if (srv_is_sweep(batch[0])) {
        std::vector<aln_thumbs> th(n);
        for (int k = 0; k < n; ++k)
            th[k] = batch[k].req.thumbs;
        std::vector<aln_thm_result> out(n);
        const aln_request &R0 = batch[0].req;
        const int rc = aln_thm_search_batch(ctx, n, th.data(), &R0.thm, R0.thm_mode, R0.ang0,
                                            R0.hfang, R0.step, out.data());
        for (int k = 0; k < n; ++k) {
            rep[k].status = rc < 0 ? rc : ALN_OK;
            if (rc >= 0)
                rep[k].sweep = out[k];
        }
        return;
    }
    std::vector<aln_pair> pairs(n);
    std::vector<ImgSpec> specs(n);
    for (int k = 0; k < n; ++k) {
        const aln_request &r = batch[k].req;
        if (r.kind == ALN_REQ_PATCHES) {
            pairs[k] = r.pair;
            memset(&specs[k], 0, sizeof specs[k]);   // kind 0: CorrPatches
        } else {
            srv_image_job(r.job, pairs[k], specs[k]);
        }
    }
    std::vector<aln_result> out(n);
    const int rc = batch_impl(ctx, n, pairs.data(), specs.data(), out.data());
    for (int k = 0; k < n; ++k) {
        rep[k].status = rc < 0 ? rc : ALN_OK;
        if (rc >= 0)
            rep[k].corr = out[k];
    }
    (void)S;
}

static void srv_worker(aln_server *S, int w)
{
    aln_ctx *ctx = S->ctxs[w];
    cudaSetDevice(S->P.device);
    std::vector<SrvReq> batch;
    std::vector<aln_reply> rep;
    for (;;) {
        batch.clear();
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->q.empty(); });
            if (S->stop)
                return;
            // admit: the head's class (sweeps: also its settings), FIFO
            // within it, up to max_batch requests and the worker's
            // workspace share (at least one request)
            const bool sweep = srv_is_sweep(S->q.front());
            const aln_request head = S->q.front().req;
            size_t bytes = 0;
            for (auto it = S->q.begin(); it != S->q.end() && (int)batch.size() < S->P.max_batch;) {
                if (srv_is_sweep(*it) != sweep || (sweep && !srv_same_sweep(it->req, head))) {
                    ++it;   // another class: keeps its place in the queue
                    continue;
                }
                if (!batch.empty() && bytes + it->bytes > S->worker_budget)
                    break;
                bytes += it->bytes;
                batch.push_back(*it);
                it = S->q.erase(it);
            }
        }
        const double t0 = srv_now_ms();
        srv_run(S, ctx, batch, rep);
        const double t1 = srv_now_ms();
        {
            std::lock_guard<std::mutex> lk(S->mu);
            for (size_t k = 0; k < batch.size(); ++k) {
                aln_reply &r = rep[k];
                r.queue_ms = t0 - batch[k].t_submit;
                r.total_ms = t1 - batch[k].t_submit;
                r.batch_size = (int)batch.size();
                S->done[batch[k].ticket] = r;
            }
            S->n_fin += (long long)batch.size();
            S->n_batches++;
            if (rep.size() && rep[0].status < 0)
                snprintf(S->err, sizeof S->err, "%s", aln_last_error(ctx));
        }
        S->cv_done.notify_all();
    }
}

extern "C" int aln_server_create(const aln_server_params *params, aln_server **out)
{
    if (!params || !out)
        return ALN_ERR_ARG;
    *out = nullptr;
    aln_server *S = new aln_server();
    S->P = *params;
    S->stop = false;
    S->next_ticket = 1;
    S->n_sub = S->n_fin = S->n_batches = 0;
    S->err[0] = 0;
    if (S->P.workers <= 0)
        S->P.workers = 2;
    if (S->P.max_batch <= 0)
        S->P.max_batch = 4096;
    if (S->P.cache_bytes == 0)
        S->P.cache_bytes = (size_t)2 << 30;
    if (cudaSetDevice(S->P.device) != cudaSuccess) {
        set_err(nullptr, ALN_ERR_CUDA, "server: device %d", S->P.device);
        delete S;
        return ALN_ERR_CUDA;
    }
    if (S->P.mem_budget == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        S->P.mem_budget = std::min(fr / 2, (size_t)16 << 30);
    }
    S->worker_budget = std::max((size_t)64 << 20, S->P.mem_budget / S->P.workers);
    for (int w = 0; w < S->P.workers; ++w) {
        aln_ctx *c = nullptr;
        const int rc = aln_ctx_create(S->P.device, &c);
        if (rc != ALN_OK) {
            for (aln_ctx *x : S->ctxs)
                aln_ctx_destroy(x);
            delete S;
            return rc;
        }
        // the batch pipeline splits a batch into chunks of half the share
        // (two staging buffers + work space stay within it)
        aln_ctx_set_workspace_limit(c, std::max((size_t)16 << 20, S->worker_budget / 2));
        aln_ctx_set_spectrum_cache(c, S->P.cache_bytes);
        S->ctxs.push_back(c);
    }
    for (int w = 0; w < S->P.workers; ++w)
        S->th.emplace_back(srv_worker, S, w);
    *out = S;
    return ALN_OK;
}

extern "C" void aln_server_destroy(aln_server *S)
{
    if (!S)
        return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        for (auto &r : S->q) {
            aln_reply c;
            memset(&c, 0, sizeof c);
            c.status = ALN_ERR_CANCELLED;
            S->done[r.ticket] = c;
        }
        S->q.clear();
    }
    S->cv_work.notify_all();
    S->cv_done.notify_all();
    for (auto &t : S->th)
        t.join();
    for (aln_ctx *c : S->ctxs)
        aln_ctx_destroy(c);
    delete S;
}

extern "C" int aln_server_submit(aln_server *S, const aln_request *req, unsigned long long *ticket)
{
    if (!S || !req || !ticket || req->kind < ALN_REQ_PATCHES || req->kind > ALN_REQ_SWEEP)
        return ALN_ERR_ARG;
    SrvReq r;
    r.req = *req;
    r.bytes = srv_bytes(*req);
    r.t_submit = srv_now_ms();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop)
            return ALN_ERR_REFUSED;
        r.ticket = S->next_ticket++;
        S->outstanding.insert(r.ticket);
        S->q.push_back(r);
        S->n_sub++;
    }
    S->cv_work.notify_one();
    *ticket = r.ticket;
    return ALN_OK;
}

extern "C" int aln_server_wait(aln_server *S, unsigned long long ticket, int timeout_ms,
                               aln_reply *out)
{
    if (!S || !out)
        return ALN_ERR_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    if (!S->outstanding.count(ticket))
        return ALN_ERR_ARG;
    auto ready = [&] { return S->done.count(ticket) != 0; };
    if (timeout_ms < 0)
        S->cv_done.wait(lk, ready);
    else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
        return ALN_ERR_TIMEOUT;
    *out = S->done[ticket];
    S->done.erase(ticket);
    S->outstanding.erase(ticket);
    return ALN_OK;
}

extern "C" int aln_server_collect(aln_server *S, int cap, int timeout_ms,
                                  unsigned long long *tickets, aln_reply *out)
{
    if (!S || cap < 0 || (cap && (!tickets || !out)))
        return ALN_ERR_ARG;
    std::unique_lock<std::mutex> lk(S->mu);
    auto ready = [&] { return !S->done.empty(); };
    if (timeout_ms < 0)
        S->cv_done.wait(lk, ready);
    else
        S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
    int k = 0;
    for (auto it = S->done.begin(); it != S->done.end() && k < cap;) {
        tickets[k] = it->first;
        out[k] = it->second;
        S->outstanding.erase(it->first);
        it = S->done.erase(it);
        ++k;
    }
    return k;
}

extern "C" long long aln_server_counter(aln_server *S, int which)
{
    if (!S)
        return -1;
    std::lock_guard<std::mutex> lk(S->mu);
    switch (which) {
    case 0: return S->n_sub;
    case 1: return S->n_fin;
    case 2: return S->n_batches;
    case 3: return (long long)S->q.size();
    case 4:
    case 5:
    case 6:
    case 7: {
        long long h = 0;
        for (aln_ctx *c : S->ctxs)
            h += which == 4 ? c->spec_hits : which == 5 ? c->spec_fills
                 : which == 6 ? c->spec_evictions : (long long)c->spec_bytes;
        return h;
    }
    default: return -1;
    }
}

extern "C" const char *aln_server_last_error(aln_server *S)
{
    return S ? S->err : "";
}
