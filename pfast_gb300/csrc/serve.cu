// serve.cu -- the request server: continuous batching of traveltime and gradient
// requests on one GPU (declared in include/pfast_gb300.h).
//
// Structure: `slots` worker threads, each owning a pfast_ctx (its own stream and device
// buffers, allocated stream-ordered so that one slot growing or freeing memory never
// synchronises the device).  Models and surveys live on the device under user IDs with
// reference counts; unused ones are evicted least recently used first when new data needs
// room.  Admission (serve_policy.h) runs under one mutex: a worker that becomes idle, a
// new submission or a finished request lets every idle worker try to start the next
// admissible request.  A request runs through the same survey pipelines as a direct call
// (pfast_survey3d_eval / _forward, engine2d), with max_batch set to the batch the policy
// granted, so its result does not depend on what else runs.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "engine.h"
#include "serve_policy.h"

using namespace pfast;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Model {
    int dim = 3, nr = 0, nc = 0, nz = 1;
    double dx = 0, dy = 0, dz = 0;
    double* d_vp = nullptr;
    double* d_wr = nullptr;
    size_t bytes = 0;
    int refs = 0;
    bool dropped = false;
    unsigned long long last_use = 0;
};

struct Survey {
    int dim = 3, nr = 0, nc = 0, nz = 1, numofr = 0, nrec = 0;
    pfast_survey3d* sv3 = nullptr;
    pfast_survey2d* sv2 = nullptr;
    size_t bytes = 0;
    int refs = 0;
    bool dropped = false;
    unsigned long long last_use = 0;
};

struct Job {
    long long ticket = 0;
    pfast_request req{};
    std::shared_ptr<Model> model;
    std::shared_ptr<Survey> survey;
    serve::Need need;
    int batch = 0;
    size_t bytes = 0;
    bool done = false;
    pfast_status status = PFAST_OK;
    std::string message;
    Clock::time_point t_submit, t_start, t_done;
};

void free_model(Model& m) {
    if (m.d_vp) cudaFree(m.d_vp);
    if (m.d_wr) cudaFree(m.d_wr);
    m.d_vp = m.d_wr = nullptr;
}

void free_survey(Survey& s) {
    if (s.sv3) pfast_survey3d_destroy(s.sv3);
    if (s.sv2) pfast_survey2d_destroy(s.sv2);
    s.sv3 = nullptr;
    s.sv2 = nullptr;
}

}  // namespace

struct pfast_server {
    pfast_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::unique_ptr<serve::Policy> policy;
    std::vector<pfast_ctx*> ctxs;
    std::vector<std::thread> workers;
    pfast_ctx* admin = nullptr;   // context for registration copies
    std::map<long long, std::shared_ptr<Model>> models;
    std::map<long long, std::shared_ptr<Survey>> surveys;
    std::map<long long, std::shared_ptr<Job>> jobs;
    long long next_ticket = 1;
    unsigned long long clock = 0;
    bool stopping = false;
    long long submitted = 0, completed = 0, failed = 0;
    size_t peak = 0;
};

namespace {

// Bytes a request needs: batch-independent part and per source solved at once (the buffers
// of the survey pipelines, with margin).
void request_need(const Model& m, const Survey& s, int kind, serve::Need& n) {
    const size_t N = (size_t)m.nz * m.nr * m.nc;
    if (m.dim == 3) {
        // lock words of either tile shape (4x8x32, 8x4x32): at most one tile per 4x4x32 nodes
        const size_t flags = (size_t)((m.nz + 3) / 4) * ((m.nr + 3) / 4) * ((m.nc + TJ - 1) / TJ) * 16;
        n.fixed = N * 20 + N * 8 + (size_t)s.nrec * 8 + (1u << 20);   // slowness (s, s32, s^2), output
        n.per_src = (kind == PFAST_REQ_GRADIENT ? N * 44 : N * 24) + flags + N / 8;
        n.nsrc = s.sv3->nsrc;
    } else {
        const size_t R = (size_t)s.numofr;
        n.fixed = N * 20 + N * 24 + (size_t)s.nrec * (R + 1) * 8 + (1u << 20);
        n.per_src = N * 8 * (1 + 2 * R + 3) + N * 16 * (1 + R) + N * 8;
        n.nsrc = s.sv2->nsrc;
    }
    n.nsrc = std::max(1, n.nsrc);
}

// Make room for `bytes` of resident data: evict unused models and surveys, least recently
// used first.  Caller holds the lock.
bool reserve_resident(pfast_server* srv, size_t bytes) {
    while (!srv->policy->reserve(bytes)) {
        unsigned long long best = ~0ull;
        int which = -1;
        long long id = 0;
        for (auto& kv : srv->models)
            if (kv.second->refs == 0 && kv.second->last_use < best) { best = kv.second->last_use; which = 0; id = kv.first; }
        for (auto& kv : srv->surveys)
            if (kv.second->refs == 0 && kv.second->last_use < best) { best = kv.second->last_use; which = 1; id = kv.first; }
        if (which < 0) return false;
        if (which == 0) {
            auto m = srv->models[id];
            srv->models.erase(id);
            free_model(*m);
            srv->policy->release(m->bytes);
        } else {
            auto s = srv->surveys[id];
            srv->surveys.erase(id);
            free_survey(*s);
            srv->policy->release(s->bytes);
        }
    }
    srv->peak = std::max(srv->peak, srv->policy->used());
    return true;
}

pfast_status run_job(pfast_ctx* ctx, Job& j) {
    const Model& m = *j.model;
    const Survey& s = *j.survey;
    pfast_options o = j.req.opt;
    o.max_batch = j.batch;
    const size_t N = (size_t)m.nz * m.nr * m.nc;
    cudaStream_t st = ctx->stream;
    if (m.dim == 3) {
        if (j.req.kind == PFAST_REQ_GRADIENT) {
            PFAST_TRY(ctx->out_a.ensure(sizeof(double) * N));
            double E = 0.0;
            PFAST_TRY(pfast_survey3d_eval(ctx, s.sv3, m.d_vp, &o, ctx->out_a.as<double>(), &E, nullptr));
            PFAST_CUDA_TRY(cudaMemcpyAsync(j.req.out, ctx->out_a.p, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
            if (j.req.out_misfit) *j.req.out_misfit = E;
        } else {
            PFAST_TRY(ctx->out_a.ensure(sizeof(double) * std::max(s.nrec, 1)));
            PFAST_TRY(pfast_survey3d_forward(ctx, s.sv3, m.d_vp, &o, ctx->out_a.as<double>(), nullptr));
            if (s.nrec > 0)
                PFAST_CUDA_TRY(cudaMemcpyAsync(j.req.out, ctx->out_a.p, sizeof(double) * s.nrec, cudaMemcpyDeviceToHost, st));
        }
    } else {
        if (j.req.kind == PFAST_REQ_GRADIENT) {
            if (!m.d_wr) { set_last_error("2D gradient request: model %s has no WR field", "(id)"); return PFAST_ERR_INVALID; }
            PFAST_TRY(ctx->out_a.ensure(sizeof(double) * N));
            PFAST_TRY(ctx->out_b.ensure(sizeof(double) * N));
            PFAST_TRY(ctx->out_c.ensure(sizeof(double) * N));
            double et = 0.0, er = 0.0;
            PFAST_TRY(eval2d_impl(ctx, s.sv2, m.d_vp, m.d_wr, &o, ctx->out_a.as<double>(), ctx->out_b.as<double>(),
                                  ctx->out_c.as<double>(), &et, &er, nullptr));
            PFAST_CUDA_TRY(cudaMemcpyAsync(j.req.out, ctx->out_c.p, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
            if (j.req.out_misfit) *j.req.out_misfit = er + et;
        } else {
            const size_t n = (size_t)std::max(s.nrec, 1) * (s.numofr + 1);
            PFAST_TRY(ctx->out_a.ensure(sizeof(double) * n));
            PFAST_TRY(forward2d_impl(ctx, s.sv2, m.d_vp, &o, ctx->out_a.as<double>(), nullptr, nullptr, nullptr, nullptr));
            if (s.nrec > 0)
                PFAST_CUDA_TRY(cudaMemcpyAsync(j.req.out, ctx->out_a.p, sizeof(double) * s.nrec * (s.numofr + 1),
                                               cudaMemcpyDeviceToHost, st));
        }
    }
    PFAST_CUDA_TRY(cudaStreamSynchronize(st));
    return PFAST_OK;
}

void worker_main(pfast_server* srv, int slot) {
    pfast_ctx* ctx = srv->ctxs[slot];
    cudaSetDevice(ctx->device);
    std::unique_lock<std::mutex> lk(srv->mu);
    for (;;) {
        std::shared_ptr<Job> job;
        serve::Decision d;
        srv->cv_work.wait(lk, [&] {
            if (srv->stopping && srv->policy->waiting() == 0) return true;
            d = srv->policy->next();
            return d.ticket >= 0;
        });
        if (d.ticket < 0) return;   // stopping, nothing left
        job = srv->jobs[d.ticket];
        job->batch = d.batch;
        job->bytes = d.bytes;
        job->t_start = Clock::now();
        srv->peak = std::max(srv->peak, srv->policy->used());
        lk.unlock();
        pfast_status st = run_job(ctx, *job);
        std::string msg = st != PFAST_OK ? std::string(pfast_last_error()) : std::string();
        ctx_release_buffers(ctx);   // stream-ordered: the memory returns to the pool
        cudaStreamSynchronize(ctx->stream);
        lk.lock();
        job->t_done = Clock::now();
        job->status = st;
        job->message = msg;
        job->done = true;
        srv->policy->finish(job->bytes);
        srv->completed += 1;
        if (st != PFAST_OK) srv->failed += 1;
        job->model->refs -= 1;
        job->survey->refs -= 1;
        job->model->last_use = ++srv->clock;
        job->survey->last_use = srv->clock;
        // dropped entries go once unused
        for (auto it = srv->models.begin(); it != srv->models.end();) {
            if (it->second->dropped && it->second->refs == 0) {
                free_model(*it->second);
                srv->policy->release(it->second->bytes);
                it = srv->models.erase(it);
            } else {
                ++it;
            }
        }
        for (auto it = srv->surveys.begin(); it != srv->surveys.end();) {
            if (it->second->dropped && it->second->refs == 0) {
                free_survey(*it->second);
                srv->policy->release(it->second->bytes);
                it = srv->surveys.erase(it);
            } else {
                ++it;
            }
        }
        job->model.reset();
        job->survey.reset();
        srv->cv_done.notify_all();
        srv->cv_work.notify_all();
    }
}

}  // namespace

extern "C" {

pfast_status pfast_server_create(const pfast_server_config* cfg, pfast_server** out) {
    if (!cfg || !out) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    *out = nullptr;
    if (cfg->slots < 1 || cfg->slots > 64 || !(cfg->hbm_budget_bytes > 0)) {
        set_last_error("server: slots must be in [1, 64] and the HBM budget positive");
        return PFAST_ERR_INVALID;
    }
    auto* srv = new pfast_server();
    srv->cfg = *cfg;
    srv->policy.reset(new serve::Policy((size_t)cfg->hbm_budget_bytes, cfg->slots,
                                        cfg->max_bypass > 0 ? cfg->max_bypass : 8));
    pfast_status s = pfast_ctx_create(cfg->device, &srv->admin);
    for (int k = 0; s == PFAST_OK && k < cfg->slots; ++k) {
        pfast_ctx* c = nullptr;
        s = pfast_ctx_create(cfg->device, &c);
        if (s == PFAST_OK) {
            ctx_stream_ordered(c);
            srv->ctxs.push_back(c);
        }
    }
    if (s != PFAST_OK) {
        for (pfast_ctx* c : srv->ctxs) pfast_ctx_destroy(c);
        if (srv->admin) pfast_ctx_destroy(srv->admin);
        delete srv;
        return s;
    }
    for (int k = 0; k < cfg->slots; ++k) srv->workers.emplace_back(worker_main, srv, k);
    *out = srv;
    return PFAST_OK;
}

pfast_status pfast_server_destroy(pfast_server* srv) {
    if (!srv) return PFAST_OK;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        srv->stopping = true;
    }
    srv->cv_work.notify_all();
    for (auto& t : srv->workers) t.join();
    for (auto& kv : srv->models) free_model(*kv.second);
    for (auto& kv : srv->surveys) free_survey(*kv.second);
    for (pfast_ctx* c : srv->ctxs) pfast_ctx_destroy(c);
    if (srv->admin) pfast_ctx_destroy(srv->admin);
    delete srv;
    return PFAST_OK;
}

pfast_status pfast_server_put_model(pfast_server* srv, long long model_id, int dim, int nrows, int ncols, int nz,
                                    double dx, double dy, double dz, const double* vp, const double* WR) {
    if (!srv || !vp) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    if ((dim != 2 && dim != 3) || nrows < 1 || ncols < 1 || nz < 1 || (dim == 2 && nz != 1)) {
        set_last_error("put_model: bad dimensions");
        return PFAST_ERR_INVALID;
    }
    auto m = std::make_shared<Model>();
    m->dim = dim; m->nr = nrows; m->nc = ncols; m->nz = nz; m->dx = dx; m->dy = dy; m->dz = dz;
    const size_t N = (size_t)nz * nrows * ncols;
    m->bytes = N * 8 * (WR ? 2 : 1);
    {
        std::lock_guard<std::mutex> g(srv->mu);
        auto it = srv->models.find(model_id);
        if (it != srv->models.end()) {
            if (it->second->refs > 0) { set_last_error("put_model: model %lld is in use", model_id); return PFAST_ERR_INVALID; }
            free_model(*it->second);
            srv->policy->release(it->second->bytes);
            srv->models.erase(it);
        }
        if (!reserve_resident(srv, m->bytes)) {
            set_last_error("put_model: %zu bytes do not fit the HBM budget", m->bytes);
            return PFAST_ERR_NOMEM;
        }
    }
    PFAST_CUDA_TRY(cudaSetDevice(srv->cfg.device));
    cudaError_t e = cudaMalloc(&m->d_vp, N * 8);
    if (e == cudaSuccess && WR) e = cudaMalloc(&m->d_wr, N * 8);
    if (e == cudaSuccess) e = cudaMemcpy(m->d_vp, vp, N * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && WR) e = cudaMemcpy(m->d_wr, WR, N * 8, cudaMemcpyHostToDevice);
    std::lock_guard<std::mutex> g(srv->mu);
    if (e != cudaSuccess) {
        free_model(*m);
        srv->policy->release(m->bytes);
        return cuda_fail(e, "put_model", __FILE__, __LINE__);
    }
    m->last_use = ++srv->clock;
    srv->models[model_id] = m;
    srv->cv_work.notify_all();
    return PFAST_OK;
}

static pfast_status put_survey(pfast_server* srv, long long survey_id, std::shared_ptr<Survey> s) {
    std::lock_guard<std::mutex> g(srv->mu);
    auto it = srv->surveys.find(survey_id);
    if (it != srv->surveys.end()) {
        if (it->second->refs > 0) {
            free_survey(*s);
            set_last_error("put_survey: survey %lld is in use", survey_id);
            return PFAST_ERR_INVALID;
        }
        free_survey(*it->second);
        srv->policy->release(it->second->bytes);
        srv->surveys.erase(it);
    }
    if (!reserve_resident(srv, s->bytes)) {
        free_survey(*s);
        set_last_error("put_survey: %zu bytes do not fit the HBM budget", s->bytes);
        return PFAST_ERR_NOMEM;
    }
    s->last_use = ++srv->clock;
    srv->surveys[survey_id] = s;
    srv->cv_work.notify_all();
    return PFAST_OK;
}

pfast_status pfast_server_put_survey3d(pfast_server* srv, long long survey_id, int nrows, int ncols, int nz, double dx,
                                       double dy, double dz, int nsrc, const int* src, const int* srnum,
                                       const int* rec, const double* nxyz, const double* T_obs) {
    if (!srv) { set_last_error("null server"); return PFAST_ERR_INVALID; }
    auto s = std::make_shared<Survey>();
    PFAST_TRY(pfast_survey3d_create(srv->admin, nrows, ncols, nz, dx, dy, dz, nsrc, src, srnum, rec, nxyz, T_obs,
                                    &s->sv3));
    PFAST_CUDA_TRY(cudaStreamSynchronize(srv->admin->stream));
    s->dim = 3; s->nr = nrows; s->nc = ncols; s->nz = nz; s->nrec = s->sv3->nrec;
    s->bytes = (size_t)s->nrec * 48 + (size_t)nsrc * 40 + (size_t)nz * nrows * ((ncols + 31) / 32) * 4;
    return put_survey(srv, survey_id, s);
}

pfast_status pfast_server_put_survey2d(pfast_server* srv, long long survey_id, int nrows, int ncols, double dx,
                                       double dz, int nsrc, const int* src, const int* srnum, int nrec,
                                       const int* rec, const double* nxy, const double* TT_obs, int NumofR,
                                       const double* TR_obs, const double* Z) {
    if (!srv) { set_last_error("null server"); return PFAST_ERR_INVALID; }
    auto s = std::make_shared<Survey>();
    PFAST_TRY(pfast_survey2d_create(srv->admin, nrows, ncols, dx, dz, nsrc, src, srnum, nrec, rec, nxy, TT_obs,
                                    NumofR, TR_obs, Z, &s->sv2));
    PFAST_CUDA_TRY(cudaStreamSynchronize(srv->admin->stream));
    s->dim = 2; s->nr = nrows; s->nc = ncols; s->nz = 1; s->nrec = nrec; s->numofr = NumofR;
    s->bytes = (size_t)nrec * (40 + 9 * (size_t)NumofR) + (size_t)nsrc * 24 + (size_t)NumofR * ncols * 32;
    return put_survey(srv, survey_id, s);
}

pfast_status pfast_server_drop(pfast_server* srv, int what, long long id) {
    if (!srv) { set_last_error("null server"); return PFAST_ERR_INVALID; }
    std::lock_guard<std::mutex> g(srv->mu);
    if (what == 0) {
        auto it = srv->models.find(id);
        if (it == srv->models.end()) { set_last_error("drop: no model %lld", id); return PFAST_ERR_INVALID; }
        if (it->second->refs == 0) {
            free_model(*it->second);
            srv->policy->release(it->second->bytes);
            srv->models.erase(it);
        } else {
            it->second->dropped = true;
        }
    } else {
        auto it = srv->surveys.find(id);
        if (it == srv->surveys.end()) { set_last_error("drop: no survey %lld", id); return PFAST_ERR_INVALID; }
        if (it->second->refs == 0) {
            free_survey(*it->second);
            srv->policy->release(it->second->bytes);
            srv->surveys.erase(it);
        } else {
            it->second->dropped = true;
        }
    }
    return PFAST_OK;
}

pfast_status pfast_server_submit(pfast_server* srv, const pfast_request* req, long long* ticket) {
    if (!srv || !req || !ticket || !req->out) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    if (req->kind != PFAST_REQ_FORWARD && req->kind != PFAST_REQ_GRADIENT) {
        set_last_error("submit: unknown request kind %d", req->kind);
        return PFAST_ERR_INVALID;
    }
    if (req->opt.precision != PFAST_PLAIN_FP64 && req->opt.precision != PFAST_MIXED) {
        set_last_error("submit: unknown precision %d", req->opt.precision);
        return PFAST_ERR_INVALID;
    }
    std::lock_guard<std::mutex> g(srv->mu);
    if (srv->stopping) { set_last_error("submit: server is stopping"); return PFAST_ERR_INVALID; }
    auto mi = srv->models.find(req->model_id);
    auto si = srv->surveys.find(req->survey_id);
    if (mi == srv->models.end() || mi->second->dropped) { set_last_error("submit: no model %lld", req->model_id); return PFAST_ERR_INVALID; }
    if (si == srv->surveys.end() || si->second->dropped) { set_last_error("submit: no survey %lld", req->survey_id); return PFAST_ERR_INVALID; }
    const Model& m = *mi->second;
    const Survey& s = *si->second;
    if (m.dim != s.dim || m.nr != s.nr || m.nc != s.nc || m.nz != s.nz) {
        set_last_error("submit: model %lld and survey %lld have different grids", req->model_id, req->survey_id);
        return PFAST_ERR_INVALID;
    }
    if (req->kind == PFAST_REQ_GRADIENT && ((m.dim == 3 && !s.sv3->has_picks) || (m.dim == 2 && !s.sv2->has_picks))) {
        set_last_error("submit: survey %lld has no picks", req->survey_id);
        return PFAST_ERR_INVALID;
    }
    if (req->kind == PFAST_REQ_GRADIENT && m.dim == 2 && !m.d_wr) {
        set_last_error("submit: 2D gradient needs a model with WR");
        return PFAST_ERR_INVALID;
    }
    auto j = std::make_shared<Job>();
    j->ticket = srv->next_ticket++;
    j->req = *req;
    j->model = mi->second;
    j->survey = si->second;
    request_need(m, s, req->kind, j->need);
    j->need.ticket = j->ticket;
    if (!srv->policy->feasible(j->need)) {
        set_last_error("submit: one source of this request needs %zu bytes, more than the HBM budget",
                       j->need.fixed + j->need.per_src);
        return PFAST_ERR_NOMEM;
    }
    j->model->refs += 1;
    j->survey->refs += 1;
    j->t_submit = Clock::now();
    srv->jobs[j->ticket] = j;
    srv->policy->enqueue(j->need);
    srv->submitted += 1;
    *ticket = j->ticket;
    srv->cv_work.notify_all();
    return PFAST_OK;
}

pfast_status pfast_server_wait(pfast_server* srv, long long ticket, pfast_request_result* res) {
    if (!srv) { set_last_error("null server"); return PFAST_ERR_INVALID; }
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->jobs.find(ticket);
    if (it == srv->jobs.end()) { set_last_error("wait: unknown ticket %lld", ticket); return PFAST_ERR_INVALID; }
    auto j = it->second;
    srv->cv_done.wait(lk, [&] { return j->done; });
    srv->jobs.erase(ticket);
    if (res) {
        res->status = j->status;
        res->batch = j->batch;
        res->queue_ms = ms_between(j->t_submit, j->t_start);
        res->run_ms = ms_between(j->t_start, j->t_done);
        res->total_ms = ms_between(j->t_submit, j->t_done);
    }
    if (j->status != PFAST_OK) set_last_error("%s", j->message.c_str());
    return j->status;
}

pfast_status pfast_server_stats_get(pfast_server* srv, pfast_server_stats* st) {
    if (!srv || !st) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    std::lock_guard<std::mutex> g(srv->mu);
    st->submitted = srv->submitted;
    st->completed = srv->completed;
    st->failed = srv->failed;
    st->running = srv->policy->running();
    st->waiting = (int)srv->policy->waiting();
    st->resident_models = (int)srv->models.size();
    st->resident_surveys = (int)srv->surveys.size();
    st->used_bytes = (double)srv->policy->used();
    st->peak_bytes = (double)srv->peak;
    st->budget_bytes = (double)srv->policy->budget();
    return PFAST_OK;
}

}  // extern "C"
