// engine.cu -- runtime of pfast_gb300: context, device buffers, 3D surveys, the
// outer-iteration driver, the 3D pipelines and the C ABI.
//
// The per-source loops of the reference drivers (src/T_PFAST3D.cpp:387-399,
// 672-686) become batches of sources on one GPU.  The plain solves keep the
// reference's outer-iteration semantics: an iteration = snapshot + 2^d ordered
// sweeps, repeated while some node moved by more than 1e-9 and fewer than MAXSwp
// iterations ran (src/T_pfsm3d.h:152, src/T_padjoint3d.h:135).  The mixed phases
// repeat while some processing of the iteration moved a node by more than their
// tolerance.  Converged sources retire from the batch; the others keep sweeping.

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <algorithm>
#include <thread>

#include "engine.h"
#include "tune_policy.h"

namespace pfast {

// ------------------------------------------------------------------ errors
static thread_local char g_err[512] = "";

void set_last_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

pfast_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    set_last_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    return e == cudaErrorMemoryAllocation ? PFAST_ERR_NOMEM : PFAST_ERR_CUDA;
}


// ------------------------------------------------------------------ buffers
pfast_status DevBuf::ensure(size_t bytes) {
    if (bytes <= cap) return PFAST_OK;
    if (p && !astream) cudaDeviceSynchronize();   // queued kernels may still use the old allocation
    release();
    size_t want = std::max<size_t>(bytes, 256);
    cudaError_t e = astream ? cudaMallocAsync(&p, want, astream) : cudaMalloc(&p, want);
    if (e != cudaSuccess) {
        p = nullptr;
        cap = 0;
        cudaGetLastError();
        set_last_error("cudaMalloc(%zu bytes) failed: %s", want, cudaGetErrorString(e));
        return PFAST_ERR_NOMEM;
    }
    cap = want;
    return PFAST_OK;
}

void DevBuf::release() {
    if (p) {
        if (astream) cudaFreeAsync(p, astream);
        else cudaFree(p);
    }
    p = nullptr;
    cap = 0;
}

pfast_status HostBuf::ensure(size_t bytes) {
    if (bytes <= cap) return PFAST_OK;
    if (p) {   // an async copy may still read or write the old buffer
        if (sstream) cudaStreamSynchronize(sstream);
        else cudaDeviceSynchronize();
    }
    release();
    size_t want = std::max<size_t>(bytes, 4096);
    PFAST_CUDA_TRY(cudaMallocHost(&p, want));
    cap = want;
    return PFAST_OK;
}

void HostBuf::release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
}

std::vector<DevBuf*> ctx_buffers(pfast_ctx* ctx) {
    return {&ctx->s64,  &ctx->s32,  &ctx->sq64,     &ctx->T32,    &ctx->tflags,    &ctx->T64,   &ctx->L64,
            &ctx->scratch, &ctx->mask, &ctx->act,  &ctx->changed, &ctx->ee,     &ctx->need,    &ctx->misc,
            &ctx->grad_tmp, &ctx->vp_tmp, &ctx->picks_tmp, &ctx->f2a, &ctx->f2b, &ctx->f2c, &ctx->work,
            &ctx->queue, &ctx->out_a, &ctx->out_b, &ctx->out_c, &ctx->dyn, &ctx->multi, &ctx->multi_meta, &ctx->sv_src, &ctx->sv_rec, &ctx->sv_nxyz,
            &ctx->sv_tobs, &ctx->sv_last};
}

void ctx_release_buffers(pfast_ctx* ctx) {
    for (DevBuf* b : ctx_buffers(ctx)) b->release();
}

void ctx_stream_ordered(pfast_ctx* ctx) {
    for (DevBuf* b : ctx_buffers(ctx)) b->astream = ctx->own_stream;
    for (HostBuf* b : {&ctx->h_act, &ctx->h_changed, &ctx->h_ee, &ctx->h_need, &ctx->h_work, &ctx->h_dyn})
        b->sstream = ctx->own_stream;
}

void add_elapsed(cudaEvent_t a, cudaEvent_t b, double* acc) {
    float ms = 0.f;
    if (cudaEventSynchronize(b) == cudaSuccess && cudaEventElapsedTime(&ms, a, b) == cudaSuccess && acc) *acc += ms;
}

pfast_status ctx_diag3(pfast_ctx* ctx, int nz, int nr, int nc, int shape, DiagTable3** out) {
    auto key = std::make_tuple(nz, nr, nc, shape);
    auto it = ctx->diag3.find(key);
    if (it == ctx->diag3.end()) {
        DiagTable3 t;
        PFAST_TRY(build_diag_table3(nz, nr, nc, shape, t));
        it = ctx->diag3.emplace(key, t).first;
    }
    *out = &it->second;
    return PFAST_OK;
}

pfast_status ctx_diag2(pfast_ctx* ctx, int nr, int nc, DiagTable2** out) {
    auto key = std::make_pair(nr, nc);
    auto it = ctx->diag2.find(key);
    if (it == ctx->diag2.end()) {
        DiagTable2 t;
        PFAST_TRY(build_diag_table2(nr, nc, t));
        it = ctx->diag2.emplace(key, t).first;
    }
    *out = &it->second;
    return PFAST_OK;
}

// ------------------------------------------------------------------ sweep driver
namespace {

// FP32 bulk phases stop once no node moves by more than ~8 ulps (relative);
// FP64 phases use the reference's absolute 1e-9.

Spacing3 make_spacing(double dx, double dy, double dz) {
    Spacing3 s;
    std::memset(&s, 0, sizeof(s));
    const double d[3] = {dx, dy, dz};
    for (int a = 0; a < 3; ++a) {
        s.d[a] = d[a];
        s.d2[a] = d[a] * d[a];
        s.inv2[a] = 1.0 / d[a] / d[a];
    }
    const double W = s.inv2[0] + s.inv2[1] + s.inv2[2];
    for (int a = 0; a < 3; ++a) {
        s.df[a] = (float)d[a];
        s.wf[a] = (float)s.inv2[a];
        s.rpf[a] = (float)(1.0 / (W - s.inv2[a]));
    }
    s.rWf = (float)(1.0 / W);
    s.iso = (dx == dy && dy == dz) ? 1 : 0;
    return s;
}

// Run outer iterations of `kind` over the active batch instances until each one
// converges or reaches maxiter.  iters[b] receives the iteration count of instance b.
// Autotuner, per (device, sweep kind, grid, active instances): the phase times of each
// (schedule, tile shape) candidate, measured by pfast_survey3d_autotune, which runs the same
// evaluation once with each; the choice itself is tune_policy.h.
static std::mutex g_tune_mu;
static std::map<std::tuple<int, int, int, int, int, int>, TuneEntry> g_tune;

static int tuned_candidate(const std::tuple<int, int, int, int, int, int>& key, unsigned allowed, int sms) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune.find(key);
    return tune_pick(it != g_tune.end() ? &it->second : nullptr, allowed, std::get<5>(key), sms);
}

static void tune_record(const std::tuple<int, int, int, int, int, int>& key, int which, double ms) {
    if (!(ms > 0.0)) return;
    std::lock_guard<std::mutex> g(g_tune_mu);
    TuneEntry& e = g_tune[key];
    e.ms[which] += ms;
    e.n[which] += 1;
}

// One outer iteration of a per-diagonal phase as a CUDA graph: the diff reset, the 8 x ndiag
// sweep launches and the per-instance reduction, captured once per (kind, launch arguments,
// active count) and replayed every iteration -- one launch instead of 8 x ndiag + 1.  The
// launches read the iteration and the current active count from ctx->dyn (a.dyn), written
// before each replay; blocks of instances that retired since the capture exit at once.
static pfast_status iteration_graph(pfast_ctx* ctx, const Sweep3Args& a, int kind, const DiagTable3& dt, int nb,
                                    int nact, cudaStream_t st, cudaGraphExec_t* out) {
    Sweep3Args k = a;
    k.dir = 0;
    k.iter = 0;
    const int extra[4] = {kind, nact, nb, dt.ndiag};
    std::vector<unsigned char> key(sizeof(k) + sizeof(extra));
    std::memcpy(key.data(), &k, sizeof(k));
    std::memcpy(key.data() + sizeof(k), extra, sizeof(extra));
    for (auto& g : ctx->iter_graphs)
        if (g.first == key) { *out = g.second; return PFAST_OK; }
    *out = nullptr;
    bool seen = false;
    for (auto& k2 : ctx->graph_seen) seen = seen || k2 == key;
    if (!seen) {   // first occurrence: launch one by one this time
        if (ctx->graph_seen.size() >= 64) ctx->graph_seen.erase(ctx->graph_seen.begin());
        ctx->graph_seen.push_back(key);
        return PFAST_OK;
    }
    cudaGraph_t graph = nullptr;
    PFAST_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    pfast_status r = PFAST_OK;
    cudaError_t e = cudaMemsetAsync(k.diff, 0, sizeof(int) * (size_t)k.ntiles * nb, st);
    for (int dir = 0; dir < 8 && !r && e == cudaSuccess; ++dir) {
        k.dir = dir;
        for (int d = 0; d < dt.ndiag && !r; ++d) r = launch_sweep3(kind, k, dt.h_off[d], dt.h_off[d + 1] - dt.h_off[d], nact, st);
    }
    if (!r && e == cudaSuccess) e = cudaMemsetAsync(k.changed, 0, sizeof(int) * nb, st);
    if (!r && e == cudaSuccess)
        r = launch_reduce_diff(k.diff, k.dirty, kind == kFwdPolish64 || kind == kAdjPolish64, 8, 0xff, k.ntiles, k.act,
                               nact, k.changed, st, k.dyn);
    const cudaError_t ec = cudaStreamEndCapture(st, &graph);
    if (r || e != cudaSuccess || ec != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        if (r) return r;
        return cuda_fail(e != cudaSuccess ? e : ec, "iteration graph capture", __FILE__, __LINE__);
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
    if (ctx->iter_graphs.size() >= 16) {   // bounded cache: drop the oldest
        cudaGraphExecDestroy(ctx->iter_graphs.front().second);
        ctx->iter_graphs.erase(ctx->iter_graphs.begin());
    }
    ctx->iter_graphs.emplace_back(std::move(key), exec);
    *out = exec;
    return PFAST_OK;
}

// Whether the tiles of a phase can move in 16-byte vectors: every grid row of the field (and of
// the staged auxiliary field: the forward's slowness, the FP32 adjoint's traveltime) starts on a
// 16-byte boundary.
int rows_aligned_impl(const Sweep3Args& a, int kind) {
    const int esz = (kind == kFwdFast32 || kind == kAdjFast32) ? 4 : 8;
    if (a.nc % (16 / esz) != 0 || reinterpret_cast<uintptr_t>(a.field) % 16 != 0) return 0;
    if (kind != kAdjPlain64 && kind != kAdjPolish64 && reinterpret_cast<uintptr_t>(a.aux) % 16 != 0) return 0;
    return 1;
}

pfast_status run_sweeps3(pfast_ctx* ctx, Sweep3Args a, int kind, int nb, std::vector<int>& active, int maxiter,
                         int* iters, long long nodes_per_sweep, long long* node_updates, int* not_conv,
                         double* ms_acc) {
    // Three schedules.  Per-diagonal launches spread every tile of every active instance over
    // all SMs (one warp per tile) and suit surveys with few instances; the dataflow kernel
    // (one block solves one instance, its sweep orders overlapping as their tile dependencies
    // allow, no host round trip per iteration) suits runs with about one instance per SM or
    // more; the hybrid runs the first, dense outer iteration per diagonal and the sparse rest
    // in the dataflow kernel.  Two tile shapes, 4x8x32 and 8x4x32 nodes in sweep-order axes.
    // Automatic: the autotuner above.  Grids whose tiles do not fit the dataflow kernel's
    // shared memory use the per-diagonal launches.
    int dev = 0, sms = 1;
    PFAST_CUDA_TRY(cudaGetDevice(&dev));
    PFAST_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const auto tkey = std::make_tuple(dev, kind, a.nz, a.nr, a.nc, (int)active.size());
    int dwarps[kTileShapes] = {}, dblocks[kTileShapes] = {};
    bool fits[kTileShapes] = {};
    for (int shape = 0; shape < kTileShapes; ++shape) {
        if (ctx->tile_shape != PFAST_TILE_AUTO && ctx->tile_shape - 1 != shape) continue;
        DiagTable3* t = nullptr;
        PFAST_TRY(ctx_diag3(ctx, a.nz, a.nr, a.nc, shape, &t));
        const int ntl = t->nbk * t->nbi * t->nbj;
        if (!active.empty()) PFAST_TRY(dataflow_shape(kind, shape, ntl, (int)active.size(), &dwarps[shape], &dblocks[shape]));
        fits[shape] = dwarps[shape] > 0;
    }
    const unsigned allowed = tune_allowed(ctx->schedule, ctx->tile_shape, fits);
    const int cand = tuned_candidate(tkey, allowed, sms);
    ctx->candidates = (ctx->candidates & ~(15 << 4 * kind)) | (cand + 1) << 4 * kind;
    const bool persistent = cand >> 1 == 1, hybrid = cand >> 1 == 2;
    a.shape = cand & 1;
    DiagTable3* dtp = nullptr;
    PFAST_TRY(ctx_diag3(ctx, a.nz, a.nr, a.nc, a.shape, &dtp));
    const DiagTable3& dt = *dtp;
    a.vec_rows = rows_aligned_impl(a, kind);
    PFAST_TRY(ctx->act.ensure(sizeof(int) * nb));
    PFAST_TRY(ctx->changed.ensure(sizeof(int) * nb));
    PFAST_TRY(ctx->h_act.ensure(sizeof(int) * nb));
    PFAST_TRY(ctx->h_changed.ensure(sizeof(int) * nb));
    int* h_act = ctx->h_act.as<int>();
    int* h_chg = ctx->h_changed.as<int>();
    a.act = ctx->act.as<int>();
    a.changed = ctx->changed.as<int>();
    a.diag_off = dt.d_off;
    a.diag_tiles = dt.d_tiles;
    a.nbk = dt.nbk;
    a.nbi = dt.nbi;
    a.nbj = dt.nbj;
    // tile-locking flags: every tile starts unlocked, with no snapshot yet
    const long long ntiles = (long long)dt.nbk * dt.nbi * dt.nbj;
    PFAST_TRY(ctx->tflags.ensure(sizeof(int) * 3 * ntiles * nb));
    a.ntiles = (int)ntiles;
    a.dirty = ctx->tflags.as<int>();
    a.stamp = a.dirty + ntiles * nb;
    a.diff = a.stamp + ntiles * nb;
    cudaStream_t st = ctx->stream;
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[0], st));
    PFAST_CUDA_TRY(cudaMemsetAsync(a.dirty, 0xff, sizeof(int) * ntiles * nb, st));
    PFAST_TRY(ctx->work.ensure(sizeof(unsigned long long) * nb));
    PFAST_TRY(ctx->h_work.ensure(sizeof(unsigned long long) * nb));
    a.work = ctx->work.as<unsigned long long>();
    PFAST_CUDA_TRY(cudaMemsetAsync(a.work, 0, sizeof(unsigned long long) * nb, st));
    PFAST_CUDA_TRY(cudaMemsetAsync(a.stamp, 0xff, sizeof(int) * ntiles * nb, st));
    const bool seeded = kind != kFwdPolish64;   // the forward polish starts from a reached field
    const bool polish = kind == kFwdPolish64 || kind == kAdjPolish64;
    if ((seeded || polish) && !active.empty()) {
        const int nact0 = (int)active.size();
        std::memcpy(h_act, active.data(), sizeof(int) * nact0);
        PFAST_CUDA_TRY(cudaMemcpyAsync(const_cast<int*>(a.act), h_act, sizeof(int) * nact0, cudaMemcpyHostToDevice, st));
        // only tiles with something to propagate start due
        if (seeded) PFAST_LAUNCH(ctx, launch_seed_tiles3(kind, a, nact0, st));
        // initial selected orders per tile, so the first polish sweep skips unselected tiles
        if (polish) PFAST_LAUNCH(ctx, launch_polish_orders3(kind, a, nb, nact0, st));
    }
    // The dataflow kernel on the active instances from outer iteration base on (iteration
    // counts, stamps and the cap are absolute).
    auto dataflow_solve = [&](int base) -> pfast_status {
        const int nact = (int)active.size();
        // Heaviest instances first, by the executed work of the same sweep kind's last phase
        // (else of the previous phase): the last round of blocks then holds the lightest ones,
        // which shortens the launch's tail.  Each block solves its instance alone, so the order
        // changes no bit.
        std::vector<int> order(active);
        const std::vector<unsigned long long>& w =
            (int)ctx->inst_work_kind[kind].size() == nb ? ctx->inst_work_kind[kind] : ctx->inst_work;
        if ((int)w.size() == nb)
            std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return w[x] > w[y]; });
        std::memcpy(h_act, order.data(), sizeof(int) * nact);
        PFAST_CUDA_TRY(cudaMemcpyAsync(const_cast<int*>(a.act), h_act, sizeof(int) * nact, cudaMemcpyHostToDevice, st));
        PFAST_TRY(ctx->queue.ensure(2 * sizeof(int)));
        PFAST_CUDA_TRY(cudaMemsetAsync(ctx->queue.p, 0, 2 * sizeof(int), st));
        Sweep3Args b = a;
        b.iter = base;
        b.dyn = nullptr;
        PFAST_TRY(launch_sweep3_dataflow(kind, b, nact, maxiter, ctx->queue.as<int>(), a.changed, dwarps[a.shape],
                                         dblocks[a.shape], st));
        ++ctx->launches;
        PFAST_TRY(ctx->h_dyn.ensure(2 * sizeof(int)));
        int* hq = ctx->h_dyn.as<int>();
        PFAST_CUDA_TRY(cudaMemcpyAsync(hq, ctx->queue.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
        PFAST_CUDA_TRY(cudaMemcpyAsync(h_chg, a.changed, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
        PFAST_CUDA_TRY(cudaStreamSynchronize(st));
        if (hq[1]) {
            set_last_error("dataflow sweep: a block made no progress for two seconds (internal error)");
            return PFAST_ERR_CUDA;
        }
        std::vector<int> still;
        for (int id : active) {
            iters[id] = h_chg[id] & 0xffff;
            if (h_chg[id] >> 30) still.push_back(id);
        }
        active.swap(still);
        return PFAST_OK;
    };
    if (persistent && maxiter > 0) PFAST_TRY(dataflow_solve(0));
    int it = 0;
    cudaGraphExec_t exec = nullptr;
    if (ctx->graphs && !persistent && maxiter > 0 && !active.empty()) {
        // captured with the first iteration's active count; later iterations only retire instances
        PFAST_TRY(ctx->dyn.ensure(2 * sizeof(int)));
        PFAST_TRY(ctx->h_dyn.ensure(2 * sizeof(int)));
        a.dyn = ctx->dyn.as<int>();
        PFAST_TRY(iteration_graph(ctx, a, kind, dt, nb, (int)active.size(), st, &exec));
        if (!exec) a.dyn = nullptr;   // launched one by one
    }
    const int diag_iters = hybrid ? std::min(maxiter, 1) : maxiter;   // hybrid: the first iteration
    while (!persistent && !active.empty() && it < diag_iters) {
        const int nact = (int)active.size();
        std::memcpy(h_act, active.data(), sizeof(int) * nact);
        PFAST_CUDA_TRY(cudaMemcpyAsync(const_cast<int*>(a.act), h_act, sizeof(int) * nact, cudaMemcpyHostToDevice, st));
        if (exec) {
            int* hd = ctx->h_dyn.as<int>();
            hd[0] = it;
            hd[1] = nact;
            PFAST_CUDA_TRY(cudaMemcpyAsync(ctx->dyn.p, hd, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
            PFAST_CUDA_TRY(cudaGraphLaunch(exec, st));
            ctx->launches += 8LL * dt.ndiag + 1;
        } else {
            PFAST_CUDA_TRY(cudaMemsetAsync(a.diff, 0, sizeof(int) * ntiles * nb, st));
            a.iter = it;
            for (int dir = 0; dir < 8; ++dir) {
                a.dir = dir;
                for (int d = 0; d < dt.ndiag; ++d) {
                    PFAST_LAUNCH(ctx, launch_sweep3(kind, a, dt.h_off[d], dt.h_off[d + 1] - dt.h_off[d], nact, st));
                }
            }
            PFAST_CUDA_TRY(cudaMemsetAsync(a.changed, 0, sizeof(int) * nb, st));
            PFAST_LAUNCH(ctx, launch_reduce_diff(a.diff, a.dirty, kind == kFwdPolish64 || kind == kAdjPolish64, 8, 0xff,
                                                 a.ntiles, a.act, nact, a.changed, st));
        }
        cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) return cuda_fail(le, "sweep launch", __FILE__, __LINE__);
        PFAST_CUDA_TRY(cudaMemcpyAsync(h_chg, a.changed, sizeof(int) * nb, cudaMemcpyDeviceToHost, st));
        PFAST_CUDA_TRY(cudaStreamSynchronize(st));
        ++it;
        std::vector<int> still;
        still.reserve(nact);
        for (int id : active) {
            iters[id] = it;
            if (!(h_chg[id] & 1)) continue;   // converged: no node moved by more than the tolerance
            // Moved, but no tile is due in any order: every tile is a fixed point of its update
            // (tile locking), so the next outer iteration would change nothing and pass the
            // convergence test.  It is counted without being launched.
            if (!(h_chg[id] & 2) && it < maxiter) { iters[id] = it + 1; continue; }
            still.push_back(id);
        }
        active.swap(still);
    }
    if (hybrid && !active.empty() && it < maxiter) PFAST_TRY(dataflow_solve(it));
    if (not_conv) *not_conv += (int)active.size();
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[1], st));
    unsigned long long* hw = ctx->h_work.as<unsigned long long>();
    PFAST_CUDA_TRY(cudaMemcpyAsync(hw, a.work, sizeof(unsigned long long) * nb, cudaMemcpyDeviceToHost, st));
    PFAST_CUDA_TRY(cudaStreamSynchronize(st));
    long long upd = 0;
    for (int b = 0; b < nb; ++b) upd += (long long)hw[b];
    if (node_updates) *node_updates += upd;
    ctx->inst_work.assign(hw, hw + nb);
    ctx->inst_work_kind[kind].assign(hw, hw + nb);
    double ms = 0.0;
    add_elapsed(ctx->ev[0], ctx->ev[1], &ms);
    if (ms_acc) *ms_acc += ms;
    if (ctx->tuning) tune_record(tkey, cand, ms);
    return PFAST_OK;
}

Sweep3Args base_args_impl(const pfast_survey3d* sv) {
    Sweep3Args a;
    std::memset(&a, 0, sizeof(a));
    a.nz = sv->nz;
    a.nr = sv->nr;
    a.nc = sv->nc;
    a.sp = make_spacing(sv->dx, sv->dy, sv->dz);
    a.wpr = (sv->nc + 31) / 32;
    a.polish_floor = kPolishFloor;
    a.src_r2 = 0;
    return a;
}

}  // namespace

pfast_status prepare_slowness(pfast_ctx* ctx, const double* vp, long long N, bool mixed, double sq_scale) {
    PFAST_TRY(ctx->s64.ensure(sizeof(double) * N));
    if (mixed) {
        PFAST_TRY(ctx->s32.ensure(sizeof(float) * N));
        PFAST_TRY(ctx->sq64.ensure(sizeof(double) * N));
    }
    PFAST_TRY(ctx->need.ensure(sizeof(int) * 4));
    PFAST_CUDA_TRY(cudaMemsetAsync(ctx->need.p, 0, sizeof(int), ctx->stream));
    PFAST_LAUNCH(ctx, launch_slowness(vp, ctx->s64.as<double>(), mixed ? ctx->s32.as<float>() : nullptr,
                                      mixed ? ctx->sq64.as<double>() : nullptr, sq_scale, ctx->need.as<int>(), N,
                                      ctx->stream));
    int bad = 0;
    PFAST_CUDA_TRY(cudaMemcpyAsync(&bad, ctx->need.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PFAST_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (bad) {
        set_last_error("the velocity model holds a value that is not a positive finite number");
        return PFAST_ERR_INVALID;
    }
    return PFAST_OK;
}

pfast_status forward3d_batch(pfast_ctx* ctx, const pfast_survey3d* sv, int b0, int nb, int precision, int maxswp,
                             pfast_stats* st) {
    const long long N = (long long)sv->nz * sv->nr * sv->nc;
    cudaStream_t s = ctx->stream;
    PFAST_TRY(ctx->T64.ensure(sizeof(double) * N * nb));
    PFAST_TRY(ctx->scratch.ensure(sizeof(double) * N * nb));
    std::vector<int> iters(nb, 0), active(nb);
    Sweep3Args a = base_args_impl(sv);
    a.fstride = N;
    a.src_kij = sv->d_src_kij + 3 * b0;
    a.src_r2 = ctx->near_radius * ctx->near_radius;
    const long long* src_lin = sv->d_src_lin + b0;
    int dummy_nc = 0;
    int* nc_ptr = st ? &st->not_converged : &dummy_nc;
    long long* nu = st ? &st->fwd_node_updates : nullptr;
    if (precision == PFAST_PLAIN_FP64) {
        PFAST_LAUNCH(ctx, launch_init_fwd3(ctx->T64.p, 0, N, N, src_lin, nb, s));
        if (ctx->near_radius > 0)
            PFAST_LAUNCH(ctx, launch_near_source3(ctx->T64.p, 0, N, a.src_kij, ctx->s64.as<double>(), sv->nz, sv->nr,
                                                  sv->nc, a.sp, ctx->near_radius, nb, s));
        for (int b = 0; b < nb; ++b) active[b] = b;
        a.field = ctx->T64.p;
        a.snap = ctx->scratch.p;
        a.aux = ctx->s64.p;
        a.tol_abs = kConvTol;
        a.tol_rel = 0.0;
        long long before = nu ? *nu : 0;
        PFAST_TRY(run_sweeps3(ctx, a, kFwdPlain64, nb, active, maxswp, iters.data(), N, nu, nc_ptr,
                              st ? &st->ms_fwd64 : nullptr));
        if (st) {
            st->fwd64_node_updates += *nu - before;
            for (int v : iters) st->fwd_iters_max = std::max(st->fwd_iters_max, v);
        }
    } else {
        float* T32 = ctx->scratch.as<float>();
        PFAST_LAUNCH(ctx, launch_init_fwd3(T32, 1, N, N, src_lin, nb, s));
        if (ctx->near_radius > 0)
            PFAST_LAUNCH(ctx, launch_near_source3(T32, 1, N, a.src_kij, ctx->s64.as<double>(), sv->nz, sv->nr, sv->nc,
                                                  a.sp, ctx->near_radius, nb, s));
        for (int b = 0; b < nb; ++b) active[b] = b;
        a.field = T32;
        a.snap = nullptr;   // the FP32 bulk kinds keep no snapshot
        a.aux = ctx->s32.p;
        a.tol_abs_f = 0.0f;
        a.tol_rel_f = (float)kTol32Rel;
        PFAST_TRY(run_sweeps3(ctx, a, kFwdFast32, nb, active, maxswp, iters.data(), N, nu, nc_ptr,
                              st ? &st->ms_fwd32 : nullptr));
        if (st) for (int v : iters) st->fwd32_iters_max = std::max(st->fwd32_iters_max, v);
        PFAST_LAUNCH(ctx, launch_widen(T32, ctx->T64.as<double>(), N, N, N, nb, s));
        if (ctx->near_radius > 0)   // the fixed region keeps its FP64 values in the polish
            PFAST_LAUNCH(ctx, launch_near_source3(ctx->T64.p, 0, N, a.src_kij, ctx->s64.as<double>(), sv->nz, sv->nr,
                                                  sv->nc, a.sp, ctx->near_radius, nb, s));
        std::fill(iters.begin(), iters.end(), 0);
        active.resize(nb);
        for (int b = 0; b < nb; ++b) active[b] = b;
        a.field = ctx->T64.p;
        a.snap = nullptr;   // the polish kinds keep no snapshot
        a.aux = ctx->sq64.p;
        a.slow64 = ctx->s64.as<double>();
        a.polish_floor = ctx->polish_floor;
        a.tol_abs = kConvTol;
        a.tol_rel = 0.0;
        long long before = nu ? *nu : 0;
        PFAST_TRY(run_sweeps3(ctx, a, kFwdPolish64, nb, active, maxswp, iters.data(), N, nu, nc_ptr,
                              st ? &st->ms_fwd64 : nullptr));
        if (st) {
            st->fwd64_node_updates += *nu - before;
            for (int v : iters) st->fwd_iters_max = std::max(st->fwd_iters_max, v);
        }
    }
    return PFAST_OK;
}

pfast_status adjoint3d_batch(pfast_ctx* ctx, const pfast_survey3d* sv, int b0, int nb, int precision, int maxswp,
                             double* ee_out, pfast_stats* st) {
    const long long N = (long long)sv->nz * sv->nr * sv->nc;
    const int wpr = (sv->nc + 31) / 32;
    const long long mwords = (long long)sv->nz * sv->nr * wpr;
    cudaStream_t s = ctx->stream;
    PFAST_TRY(ctx->L64.ensure(sizeof(double) * N * nb));
    PFAST_TRY(ctx->scratch.ensure(sizeof(double) * N * nb));
    PFAST_TRY(ctx->mask.ensure(sizeof(unsigned) * mwords * nb));
    PFAST_TRY(ctx->ee.ensure(sizeof(double) * nb));
    PFAST_TRY(ctx->need.ensure(sizeof(int) * nb));
    PFAST_TRY(ctx->h_ee.ensure(sizeof(double) * nb));
    PFAST_TRY(ctx->h_need.ensure(sizeof(int) * nb));
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
    PFAST_CUDA_TRY(cudaMemsetAsync(ctx->L64.p, 0, sizeof(double) * N * nb, s));
    PFAST_CUDA_TRY(cudaMemsetAsync(ctx->mask.p, 0, sizeof(unsigned) * mwords * nb, s));
    Bc3Args bc;
    bc.T = ctx->T64.as<double>();
    bc.L = ctx->L64.as<double>();
    bc.fstride = N;
    bc.mask = ctx->mask.as<unsigned>();
    bc.mask_stride = mwords;
    bc.wpr = wpr;
    bc.rec = sv->d_rec;
    bc.nxyz = sv->d_nxyz;
    bc.tobs = sv->d_tobs;
    bc.last = sv->d_last;
    bc.ch0 = sv->d_ch0 + b0;
    bc.srnum = sv->d_srnum + b0;
    bc.src_kij = sv->d_src_kij + 3 * b0;
    bc.EE = ctx->ee.as<double>();
    bc.need = ctx->need.as<int>();
    bc.nz = sv->nz;
    bc.nr = sv->nr;
    bc.nc = sv->nc;
    bc.dx = sv->dx;
    bc.dy = sv->dy;
    bc.dz = sv->dz;
    PFAST_LAUNCH(ctx, launch_bc3(bc, nb, s));
    PFAST_CUDA_TRY(cudaMemcpyAsync(ctx->h_ee.p, ctx->ee.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, s));
    PFAST_CUDA_TRY(cudaMemcpyAsync(ctx->h_need.p, ctx->need.p, sizeof(int) * nb, cudaMemcpyDeviceToHost, s));
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    add_elapsed(ctx->ev[2], ctx->ev[3], st ? &st->ms_other : nullptr);
    std::memcpy(ee_out, ctx->h_ee.p, sizeof(double) * nb);
    std::vector<int> active, iters(nb, 0);
    for (int b = 0; b < nb; ++b)
        if (ctx->h_need.as<int>()[b]) active.push_back(b);
    const long long interior =
        (long long)std::max(0, sv->nz - 2) * std::max(0, sv->nr - 2) * std::max(0, sv->nc - 2);
    Sweep3Args a = base_args_impl(sv);
    a.fstride = N;
    a.mask = ctx->mask.as<unsigned>();
    a.mask_stride = mwords;
    a.aux = ctx->T64.p;
    int dummy_nc = 0;
    int* nc_ptr = st ? &st->not_converged : &dummy_nc;
    long long* nu = st ? &st->adj_node_updates : nullptr;
    if (precision == PFAST_PLAIN_FP64) {
        a.field = ctx->L64.p;
        a.snap = ctx->scratch.p;
        a.tol_abs = kConvTol;
        a.tol_rel = 0.0;
        long long before = nu ? *nu : 0;
        PFAST_TRY(run_sweeps3(ctx, a, kAdjPlain64, nb, active, maxswp, iters.data(), interior, nu, nc_ptr,
                              st ? &st->ms_adj64 : nullptr));
        if (st) {
            st->adj64_node_updates += *nu - before;
            for (int v : iters) st->adj_iters_max = std::max(st->adj_iters_max, v);
        }
    } else {
        std::vector<int> active64 = active;
        float* L32 = ctx->scratch.as<float>();
        PFAST_TRY(ctx->T32.ensure(sizeof(float) * N * nb));
        PFAST_LAUNCH(ctx, launch_narrow(ctx->L64.as<double>(), L32, N, N, N, nb, s));
        PFAST_LAUNCH(ctx, launch_narrow(ctx->T64.as<double>(), ctx->T32.as<float>(), N, N, N, nb, s));
        a.field = L32;
        a.snap = nullptr;   // the FP32 bulk kinds keep no snapshot
        a.aux = ctx->T32.p;
        a.tol_abs_f = (float)kTol32AbsAdj;
        a.tol_rel_f = (float)kTol32Rel;
        PFAST_TRY(run_sweeps3(ctx, a, kAdjFast32, nb, active, maxswp, iters.data(), interior, nu, nc_ptr,
                              st ? &st->ms_adj32 : nullptr));
        if (st) for (int v : iters) st->adj32_iters_max = std::max(st->adj32_iters_max, v);
        PFAST_LAUNCH(ctx, launch_widen_lambda(L32, ctx->L64.as<double>(), ctx->mask.as<unsigned>(), N, N, mwords, sv->nz,
                                      sv->nr, sv->nc, wpr, nb, s));
        std::fill(iters.begin(), iters.end(), 0);
        a.field = ctx->L64.p;
        a.snap = nullptr;   // the polish kinds keep no snapshot
        a.aux = ctx->T64.p;
        a.polish_floor = ctx->polish_floor;
        a.tol_abs = kConvTol;
        a.tol_rel = 0.0;
        long long before = nu ? *nu : 0;
        PFAST_TRY(run_sweeps3(ctx, a, kAdjPolish64, nb, active64, maxswp, iters.data(), interior, nu, nc_ptr,
                              st ? &st->ms_adj64 : nullptr));
        if (st) {
            st->adj64_node_updates += *nu - before;
            for (int v : iters) st->adj_iters_max = std::max(st->adj_iters_max, v);
        }
    }
    return PFAST_OK;
}

namespace {

bool valid_options_impl(const pfast_options* opt) {
    if (!opt) return true;
    if (opt->precision != PFAST_PLAIN_FP64 && opt->precision != PFAST_MIXED) {
        set_last_error("unknown precision %d", opt->precision);
        return false;
    }
    if (opt->maxswp < 0 || opt->max_batch < 0) {
        set_last_error("negative maxswp / max_batch");
        return false;
    }
    if (!(opt->polish_floor >= 0.0 && opt->polish_floor < 1e-9)) {
        set_last_error("polish_floor must be in [0, 1e-9)");
        return false;
    }
    if (opt->schedule < PFAST_SCHEDULE_AUTO || opt->schedule > PFAST_SCHEDULE_HYBRID) {
        set_last_error("unknown schedule %d", opt->schedule);
        return false;
    }
    if (opt->near_source_radius < 0 || opt->near_source_radius > 64) {
        set_last_error("near_source_radius must be in [0, 64]");
        return false;
    }
    if (opt->tile_shape < PFAST_TILE_AUTO || opt->tile_shape > PFAST_TILE_8x4x32) {
        set_last_error("unknown tile_shape %d", opt->tile_shape);
        return false;
    }
    return true;
}

pfast_options resolve_impl(const pfast_options* opt, int default_maxswp) {
    pfast_options o;
    o.precision = PFAST_PLAIN_FP64;
    o.maxswp = default_maxswp;
    o.max_batch = 0;
    o.polish_floor = 0.0;
    o.schedule = PFAST_SCHEDULE_AUTO;
    o.near_source_radius = 0;
    o.tile_shape = PFAST_TILE_AUTO;
    if (opt) o = *opt;
    return o;
}

// Sources per batch: the caller's cap, else what fits in 85% of free device memory.
int pick_batch(int nsrc, int max_batch, size_t bytes_per_src) {
    int b = nsrc;
    if (max_batch > 0) b = std::min(b, max_batch);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && bytes_per_src > 0) {
        size_t fit = (size_t)(0.85 * (double)fr) / bytes_per_src;
        b = (int)std::min<size_t>((size_t)b, std::max<size_t>(1, fit));
    }
    return std::max(1, std::min(b, 65535));
}

void stats_begin_impl(pfast_stats* st) {
    if (st) std::memset(st, 0, sizeof(*st));
}

}  // namespace

Sweep3Args survey_sweep_args(const pfast_survey3d* sv) { return base_args_impl(sv); }
int rows_aligned(const Sweep3Args& a, int kind) { return rows_aligned_impl(a, kind); }
bool valid_options(const pfast_options* opt) { return valid_options_impl(opt); }
pfast_options resolve_options(const pfast_options* opt, int default_maxswp) { return resolve_impl(opt, default_maxswp); }
void stats_begin(pfast_stats* st) { stats_begin_impl(st); }

}  // namespace pfast

using namespace pfast;

// ====================================================================== C ABI
extern "C" {

const char* pfast_version(void) { return "pfast_gb300 0.1 (sm_103a)"; }

const char* pfast_status_string(pfast_status s) {
    switch (s) {
        case PFAST_OK: return "ok";
        case PFAST_ERR_INVALID: return "invalid argument";
        case PFAST_ERR_CUDA: return "CUDA error";
        case PFAST_ERR_NOMEM: return "out of device memory";
        case PFAST_ERR_NO_DEVICE: return "no CUDA device";
        case PFAST_ERR_NO_REFLECTION_POINT: return "no node above a reflector";
        case PFAST_ERR_NEGATIVE_TIME: return "negative reflected traveltime";
        case PFAST_ERR_OVER_CORRECTED: return "over corrected: the model update is too large";
        case PFAST_ERR_LINE_SEARCH: return "line search: cubic interpolation has no minimiser";
    }
    return "unknown status";
}

const char* pfast_last_error(void) { return g_err; }

void pfast_default_options(pfast_options* opt) {
    if (!opt) return;
    opt->precision = PFAST_PLAIN_FP64;
    opt->maxswp = 100;
    opt->max_batch = 0;
    opt->polish_floor = 0.0;
    opt->schedule = PFAST_SCHEDULE_AUTO;
    opt->near_source_radius = 0;
    opt->tile_shape = PFAST_TILE_AUTO;
}

pfast_status pfast_ctx_create(int device, pfast_ctx** out) {
    if (!out) { set_last_error("null output pointer"); return PFAST_ERR_INVALID; }
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        set_last_error("no CUDA device visible");
        return PFAST_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) { set_last_error("device %d out of range (%d devices)", device, n); return PFAST_ERR_INVALID; }
    PFAST_CUDA_TRY(cudaSetDevice(device));
    pfast_ctx* c = new pfast_ctx();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaStreamCreate", __FILE__, __LINE__); }
    c->stream = c->own_stream;
    for (auto& ev : c->ev) {
        e = cudaEventCreate(&ev);
        if (e != cudaSuccess) { delete c; return cuda_fail(e, "cudaEventCreate", __FILE__, __LINE__); }
    }
    *out = c;
    return PFAST_OK;
}

pfast_status pfast_ctx_destroy(pfast_ctx* ctx) {
    if (!ctx) return PFAST_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    pfast::ctx_release_buffers(ctx);
    for (HostBuf* b : {&ctx->h_act, &ctx->h_changed, &ctx->h_ee, &ctx->h_need, &ctx->h_work, &ctx->h_dyn}) b->release();
    for (auto& g : ctx->iter_graphs) cudaGraphExecDestroy(g.second);
    for (auto& kv : ctx->diag3) free_diag_table3(kv.second);
    for (auto& kv : ctx->diag2) free_diag_table2(kv.second);
    for (auto& ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return PFAST_OK;
}

pfast_status pfast_ctx_set_stream(pfast_ctx* ctx, void* stream) {
    if (!ctx) { set_last_error("null context"); return PFAST_ERR_INVALID; }
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return PFAST_OK;
}

pfast_status pfast_ctx_set_graphs(pfast_ctx* ctx, int enabled) {
    if (!ctx) { set_last_error("null context"); return PFAST_ERR_INVALID; }
    ctx->graphs = enabled != 0;
    return PFAST_OK;
}

pfast_status pfast_ctx_synchronize(pfast_ctx* ctx) {
    if (!ctx) { set_last_error("null context"); return PFAST_ERR_INVALID; }
    PFAST_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    return PFAST_OK;
}

// ------------------------------------------------------------------ 3D surveys
// scratch: the device arrays are the context's reused buffers (the one-call host entries, which
// destroy the survey before they return), copied on the context's stream; otherwise the survey
// owns them.
static pfast_status survey3d_create_impl(pfast_ctx* ctx, int nrows, int ncols, int nz, double dx, double dy, double dz,
                                         int nsrc, const int* src, const int* srnum, const int* rec,
                                         const double* nxyz, const double* T_obs, bool scratch,
                                         pfast_survey3d** out) {
    if (!ctx || !out) { set_last_error("null context or output"); return PFAST_ERR_INVALID; }
    *out = nullptr;
    if (nrows < 2 || ncols < 2 || nz < 2) {
        set_last_error("3D grid %dx%dx%d: every dimension must be >= 2", nrows, ncols, nz);
        return PFAST_ERR_INVALID;
    }
    if (!(dx > 0 && dy > 0 && dz > 0)) { set_last_error("grid spacings must be positive"); return PFAST_ERR_INVALID; }
    if (nsrc < 0 || (nsrc > 0 && (!src || !srnum))) { set_last_error("bad source arrays"); return PFAST_ERR_INVALID; }
    long long nrec = 0;
    for (int s = 0; s < nsrc; ++s) {
        if (srnum[s] < 0) { set_last_error("srnum[%d] < 0", s); return PFAST_ERR_INVALID; }
        nrec += srnum[s];
        const int i = src[3 * s], j = src[3 * s + 1], k = src[3 * s + 2];
        if (i < 0 || i >= nrows || j < 0 || j >= ncols || k < 0 || k >= nz) {
            set_last_error("source %d at (%d,%d,%d) outside the %dx%dx%d grid", s, i, j, k, nrows, ncols, nz);
            return PFAST_ERR_INVALID;
        }
    }
    if (nrec > 0x7fffffffLL) { set_last_error("too many receiver rows"); return PFAST_ERR_INVALID; }
    if (nrec > 0 && !rec) { set_last_error("null receiver array"); return PFAST_ERR_INVALID; }
    for (long long r = 0; r < nrec; ++r) {
        const int i = rec[3 * r], j = rec[3 * r + 1], k = rec[3 * r + 2];
        if (i < 0 || i >= nrows || j < 0 || j >= ncols || k < 0 || k >= nz) {
            set_last_error("receiver row %lld at (%d,%d,%d) outside the grid", r, i, j, k);
            return PFAST_ERR_INVALID;
        }
    }
    PFAST_CUDA_TRY(cudaSetDevice(ctx->device));
    pfast_survey3d* sv = new pfast_survey3d();
    sv->ctx = ctx;
    sv->nz = nz; sv->nr = nrows; sv->nc = ncols;
    sv->dx = dx; sv->dy = dy; sv->dz = dz;
    sv->nsrc = nsrc;
    sv->nrec = (int)nrec;
    sv->h_src.assign(src, src + 3 * (size_t)nsrc);
    sv->h_srnum.assign(srnum, srnum + nsrc);
    sv->h_ch0.assign(nsrc + 1, 0);
    for (int s = 0; s < nsrc; ++s) sv->h_ch0[s + 1] = sv->h_ch0[s] + srnum[s];
    std::vector<int> kij(3 * (size_t)std::max(nsrc, 1));
    std::vector<long long> lin(std::max(nsrc, 1));
    for (int s = 0; s < nsrc; ++s) {
        kij[3 * s] = src[3 * s + 2];
        kij[3 * s + 1] = src[3 * s];
        kij[3 * s + 2] = src[3 * s + 1];
        lin[s] = (long long)src[3 * s + 2] * nrows * ncols + (long long)src[3 * s] * ncols + src[3 * s + 1];
    }
    // last picked row at each node, per source (the reference's later rows overwrite earlier ones)
    sv->has_picks = nxyz && T_obs;
    std::vector<unsigned char> last(std::max<long long>(nrec, 1), 0);
    if (sv->has_picks) {
        // sources are independent (each marks its own rows): split them over host threads
        auto mark_range = [&](int s0, int s1) {
            std::vector<long long> keys;
            std::vector<size_t> used;
            for (int s = s0; s < s1; ++s)
                mark_last_rows(
                    sv->h_ch0[s], sv->h_ch0[s + 1],
                    [&](int r) { return (long long)rec[3 * r + 2] * nrows * ncols + (long long)rec[3 * r] * ncols + rec[3 * r + 1]; },
                    [&](int r) { return T_obs[r] < 100; }, [&](int r) { last[r] = 1; }, keys, used);
        };
        const int nth = (int)std::min<long long>(std::max(1u, std::min(16u, std::thread::hardware_concurrency())),
                                                 std::max<long long>(1, nrec / 65536));
        if (nth <= 1 || nsrc < 2) {
            mark_range(0, nsrc);
        } else {
            std::vector<std::thread> th;
            for (int t = 0; t < nth; ++t) {
                const int s0 = (int)((long long)nsrc * t / nth), s1 = (int)((long long)nsrc * (t + 1) / nth);
                if (s1 > s0) th.emplace_back(mark_range, s0, s1);
            }
            for (auto& x : th) x.join();
        }
    }
    pfast_status stt = PFAST_OK;
    if (scratch) {
        // the source tables in one buffer (16-byte aligned pieces), the rest in their own
        sv->borrowed = true;
        auto al = [](size_t b) { return (b + 15) / 16 * 16; };
        const size_t b_kij = al(sizeof(int) * 3 * nsrc), b_lin = al(sizeof(long long) * nsrc);
        const size_t b_ch0 = al(sizeof(int) * (nsrc + 1)), b_srn = al(sizeof(int) * nsrc);
        stt = ctx->sv_src.ensure(std::max<size_t>(b_kij + b_lin + b_ch0 + b_srn, 16));
        if (!stt) stt = ctx->sv_rec.ensure(std::max<size_t>(sizeof(int) * 3 * nrec, 16));
        if (!stt) stt = ctx->sv_nxyz.ensure(std::max<size_t>(sv->has_picks ? sizeof(double) * 3 * nrec : 0, 16));
        if (!stt) stt = ctx->sv_tobs.ensure(std::max<size_t>(sv->has_picks ? sizeof(double) * nrec : 0, 16));
        if (!stt) stt = ctx->sv_last.ensure(std::max<size_t>(nrec, 16));
        if (stt) { delete sv; return stt; }
        unsigned char* base = ctx->sv_src.as<unsigned char>();
        sv->d_src_kij = reinterpret_cast<int*>(base);
        sv->d_src_lin = reinterpret_cast<long long*>(base + b_kij);
        sv->d_ch0 = reinterpret_cast<int*>(base + b_kij + b_lin);
        sv->d_srnum = reinterpret_cast<int*>(base + b_kij + b_lin + b_ch0);
        sv->d_rec = ctx->sv_rec.as<int>();
        sv->d_nxyz = ctx->sv_nxyz.as<double>();
        sv->d_tobs = ctx->sv_tobs.as<double>();
        sv->d_last = ctx->sv_last.as<unsigned char>();
        auto cp = [&](void* dst, const void* h, size_t bytes) -> pfast_status {
            if (bytes) PFAST_CUDA_TRY(cudaMemcpyAsync(dst, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
            return PFAST_OK;
        };
        if (!stt) stt = cp(sv->d_src_kij, kij.data(), sizeof(int) * 3 * nsrc);
        if (!stt) stt = cp(sv->d_src_lin, lin.data(), sizeof(long long) * nsrc);
        if (!stt) stt = cp(sv->d_ch0, sv->h_ch0.data(), sizeof(int) * (nsrc + 1));
        if (!stt) stt = cp(sv->d_srnum, srnum, sizeof(int) * nsrc);
        if (!stt) stt = cp(sv->d_rec, rec, sizeof(int) * 3 * nrec);
        if (!stt && sv->has_picks) stt = cp(sv->d_nxyz, nxyz, sizeof(double) * 3 * nrec);
        if (!stt && sv->has_picks) stt = cp(sv->d_tobs, T_obs, sizeof(double) * nrec);
        if (!stt) stt = cp(sv->d_last, last.data(), sizeof(unsigned char) * nrec);
        // the host tables above are freed when this function returns
        if (!stt) {
            const cudaError_t e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) stt = cuda_fail(e, "survey upload", __FILE__, __LINE__);
        }
        if (stt) { delete sv; return stt; }
        *out = sv;
        return PFAST_OK;
    }
    auto up = [&](void** dst, const void* h, size_t bytes) -> pfast_status {
        PFAST_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(bytes, 16)));
        if (bytes) PFAST_CUDA_TRY(cudaMemcpy(*dst, h, bytes, cudaMemcpyHostToDevice));
        return PFAST_OK;
    };
    if (!stt) stt = up((void**)&sv->d_src_kij, kij.data(), sizeof(int) * 3 * nsrc);
    if (!stt) stt = up((void**)&sv->d_src_lin, lin.data(), sizeof(long long) * nsrc);
    if (!stt) stt = up((void**)&sv->d_ch0, sv->h_ch0.data(), sizeof(int) * (nsrc + 1));
    if (!stt) stt = up((void**)&sv->d_srnum, srnum, sizeof(int) * nsrc);
    if (!stt) stt = up((void**)&sv->d_rec, rec, sizeof(int) * 3 * nrec);
    if (!stt) stt = up((void**)&sv->d_nxyz, sv->has_picks ? nxyz : nullptr, sv->has_picks ? sizeof(double) * 3 * nrec : 0);
    if (!stt) stt = up((void**)&sv->d_tobs, sv->has_picks ? T_obs : nullptr, sv->has_picks ? sizeof(double) * nrec : 0);
    if (!stt) stt = up((void**)&sv->d_last, last.data(), sizeof(unsigned char) * nrec);
    if (stt) { pfast_survey3d_destroy(sv); return stt; }
    *out = sv;
    return PFAST_OK;
}

pfast_status pfast_survey3d_create(pfast_ctx* ctx, int nrows, int ncols, int nz, double dx, double dy, double dz,
                                   int nsrc, const int* src, const int* srnum, const int* rec, const double* nxyz,
                                   const double* T_obs, pfast_survey3d** out) {
    return survey3d_create_impl(ctx, nrows, ncols, nz, dx, dy, dz, nsrc, src, srnum, rec, nxyz, T_obs, false, out);
}



pfast_status pfast_survey3d_destroy(pfast_survey3d* sv) {
    if (!sv) return PFAST_OK;
    if (sv->borrowed) { delete sv; return PFAST_OK; }   // the context's buffers
    for (void* p : {(void*)sv->d_src_kij, (void*)sv->d_src_lin, (void*)sv->d_ch0, (void*)sv->d_srnum, (void*)sv->d_rec,
                    (void*)sv->d_nxyz, (void*)sv->d_tobs, (void*)sv->d_last})
        if (p) cudaFree(p);
    delete sv;
    return PFAST_OK;
}

static pfast_status survey3d_run(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp, const pfast_options* opt,
                                 double* grad, double* misfit, double* picks, pfast_stats* stats) {
    if (!ctx || !sv || !vp) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    if (!valid_options_impl(opt)) return PFAST_ERR_INVALID;
    const bool want_grad = grad != nullptr;
    if (want_grad && !sv->has_picks) { set_last_error("survey has no picks: gradient unavailable"); return PFAST_ERR_INVALID; }
    pfast_options o = resolve_impl(opt, 100);
    ctx->polish_floor = o.polish_floor > 0.0 ? (float)o.polish_floor : kPolishFloor;
    ctx->schedule = o.schedule;
    ctx->tile_shape = o.tile_shape;
    ctx->near_radius = o.near_source_radius;
    stats_begin_impl(stats);
    ctx->candidates = 0;
    PFAST_CUDA_TRY(cudaSetDevice(ctx->device));
    const long long N = (long long)sv->nz * sv->nr * sv->nc;
    cudaStream_t s = ctx->stream;
    cudaEvent_t t0 = ctx->ev[6], t1 = ctx->ev[7];
    PFAST_CUDA_TRY(cudaEventRecord(t0, s));
    const long long launches0 = ctx->launches;
    // the 3D forward polish on an isotropic grid works with (s h)^2 (its residual divided by 1/h^2)
    const double hsq = (sv->dx == sv->dy && sv->dy == sv->dz) ? sv->dx * sv->dx : 1.0;
    PFAST_TRY(prepare_slowness(ctx, vp, N, o.precision == PFAST_MIXED, hsq));
    if (want_grad) PFAST_CUDA_TRY(cudaMemsetAsync(grad, 0, sizeof(double) * N, s));
    const size_t per_src = (size_t)N * (want_grad ? 24 : 16) + (size_t)sv->nz * sv->nr * ((sv->nc + 31) / 32) * 4;
    const int B = pick_batch(std::max(sv->nsrc, 1), o.max_batch, per_src);
    double E = 0.0;
    std::vector<double> ee(B);
    for (int b0 = 0; b0 < sv->nsrc; b0 += B) {
        const int nb = std::min(B, sv->nsrc - b0);
        if (stats) ++stats->batches;
        PFAST_TRY(forward3d_batch(ctx, sv, b0, nb, o.precision, o.maxswp, stats));
        if (want_grad) {
            PFAST_TRY(adjoint3d_batch(ctx, sv, b0, nb, o.precision, o.maxswp, ee.data(), stats));
            for (int b = 0; b < nb; ++b) E += ee[b];   // loc_E += EE in source order
            PFAST_LAUNCH(ctx, launch_accumulate(grad, ctx->L64.as<double>(), N, vp, N, nb, o.precision == PFAST_PLAIN_FP64, s));
        }
        if (picks) PFAST_LAUNCH(ctx, launch_gather3(ctx->T64.as<double>(), N, sv->d_rec, sv->d_ch0 + b0, sv->d_srnum + b0, nb,
                                            sv->nz, sv->nr, sv->nc, picks, s));
    }
    if (want_grad && o.precision != PFAST_PLAIN_FP64) PFAST_LAUNCH(ctx, launch_finish_gradient(grad, vp, N, s));
    PFAST_CUDA_TRY(cudaEventRecord(t1, s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    if (stats) {
        add_elapsed(t0, t1, &stats->ms_total);
        stats->launches = ctx->launches - launches0;
        stats->candidates = ctx->candidates;
    }
    if (misfit) *misfit = E;
    return PFAST_OK;
}

pfast_status pfast_survey3d_eval(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp, const pfast_options* opt,
                                 double* grad, double* misfit, pfast_stats* stats) {
    if (!grad) { set_last_error("null gradient"); return PFAST_ERR_INVALID; }
    return survey3d_run(ctx, sv, vp, opt, grad, misfit, nullptr, stats);
}

pfast_status pfast_survey3d_forward(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp, const pfast_options* opt,
                                    double* picks, pfast_stats* stats) {
    if (!picks) { set_last_error("null picks"); return PFAST_ERR_INVALID; }
    return survey3d_run(ctx, sv, vp, opt, nullptr, nullptr, picks, stats);
}

pfast_status pfast_survey3d_autotune(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp, const pfast_options* opt,
                                     pfast_stats* stats) {
    if (!ctx || !sv || !vp) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    if (!valid_options_impl(opt)) return PFAST_ERR_INVALID;
    const long long N = (long long)sv->nz * sv->nr * sv->nc;
    PFAST_TRY(ctx->out_a.ensure(sizeof(double) * std::max<long long>(N, sv->nrec)));
    pfast_options o = resolve_impl(opt, 100);
    ctx->tuning = true;
    pfast_status r = PFAST_OK;
    for (int c = 0; c < PFAST_TUNE_CANDIDATES && r == PFAST_OK; ++c) {
        o.schedule = PFAST_SCHEDULE_DIAGONAL + c / 2;
        o.tile_shape = PFAST_TILE_4x8x32 + (c & 1);
        pfast_stats* sc = stats ? stats + c : nullptr;
        double E = 0.0;
        r = sv->has_picks ? survey3d_run(ctx, sv, vp, &o, ctx->out_a.as<double>(), &E, nullptr, sc)
                          : survey3d_run(ctx, sv, vp, &o, nullptr, nullptr, ctx->out_a.as<double>(), sc);
    }
    ctx->tuning = false;
    return r;
}

pfast_status pfast_eval3d(pfast_ctx* ctx, const double* vp, int nrows, int ncols, int nz, double dx, double dy, double dz,
                          int nsrc, const int* src, const int* srnum, const int* rec, const double* nxyz,
                          const double* T_obs, const pfast_options* opt, double* grad, double* misfit,
                          pfast_stats* stats) {
    if (!ctx || !vp || !grad || !nxyz || !T_obs) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    pfast_survey3d* sv = nullptr;
    PFAST_TRY(survey3d_create_impl(ctx, nrows, ncols, nz, dx, dy, dz, nsrc, src, srnum, rec, nxyz, T_obs, true, &sv));
    const long long N = (long long)nrows * ncols * nz;
    pfast_status r = ctx->vp_tmp.ensure(sizeof(double) * N);
    if (!r) r = ctx->grad_tmp.ensure(sizeof(double) * N);
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(ctx->vp_tmp.p, vp, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync(vp)", __FILE__, __LINE__);
    }
    if (!r) r = survey3d_run(ctx, sv, ctx->vp_tmp.as<double>(), opt, ctx->grad_tmp.as<double>(), misfit, nullptr, stats);
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(grad, ctx->grad_tmp.p, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync(grad)", __FILE__, __LINE__);
    }
    pfast_survey3d_destroy(sv);
    return r;
}

pfast_status pfast_forward3d(pfast_ctx* ctx, const double* vp, int nrows, int ncols, int nz, double dx, double dy,
                             double dz, int nsrc, const int* src, const int* srnum, const int* rec,
                             const pfast_options* opt, double* picks, pfast_stats* stats) {
    if (!ctx || !vp || !picks) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    pfast_survey3d* sv = nullptr;
    PFAST_TRY(survey3d_create_impl(ctx, nrows, ncols, nz, dx, dy, dz, nsrc, src, srnum, rec, nullptr, nullptr, true, &sv));
    const long long N = (long long)nrows * ncols * nz;
    pfast_status r = ctx->vp_tmp.ensure(sizeof(double) * N);
    if (!r) r = ctx->picks_tmp.ensure(sizeof(double) * std::max(sv->nrec, 1));
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(ctx->vp_tmp.p, vp, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync(vp)", __FILE__, __LINE__);
    }
    if (!r) r = survey3d_run(ctx, sv, ctx->vp_tmp.as<double>(), opt, nullptr, nullptr, ctx->picks_tmp.as<double>(), stats);
    if (!r && sv->nrec > 0) {
        cudaError_t e = cudaMemcpyAsync(picks, ctx->picks_tmp.p, sizeof(double) * sv->nrec, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "cudaMemcpyAsync(picks)", __FILE__, __LINE__);
    }
    pfast_survey3d_destroy(sv);
    return r;
}

// ------------------------------------------------------------------ reference-signature shims
static std::mutex g_default_mu;
static pfast_ctx* g_default[64] = {};

static pfast_status default_ctx(pfast_ctx** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_last_error("no CUDA device");
        return PFAST_ERR_NO_DEVICE;
    }
    if (dev < 0 || dev >= 64) { set_last_error("device id %d unsupported", dev); return PFAST_ERR_INVALID; }
    std::lock_guard<std::mutex> lk(g_default_mu);
    if (!g_default[dev]) PFAST_TRY(pfast_ctx_create(dev, &g_default[dev]));
    *out = g_default[dev];
    return PFAST_OK;
}

}  // extern "C"
pfast_status pfast::default_context(pfast_ctx** out) { return default_ctx(out); }
extern "C" {

pfast_status pfast_fsm3d(double* vp, double* U, int* src, int srcid, int MAXSwp, double dx, double dy, double dz,
                         int nrows, int ncols, int nz, int pe) {
    (void)pe;
    if (!vp || !U || !src || srcid < 0) { set_last_error("null argument or negative srcid"); return PFAST_ERR_INVALID; }
    pfast_ctx* ctx = nullptr;
    PFAST_TRY(default_ctx(&ctx));
    int zero = 0;
    pfast_survey3d* sv = nullptr;
    PFAST_TRY(pfast_survey3d_create(ctx, nrows, ncols, nz, dx, dy, dz, 1, src + 3 * srcid, &zero, nullptr, nullptr,
                                    nullptr, &sv));
    const long long N = (long long)nrows * ncols * nz;
    pfast_status r = ctx->vp_tmp.ensure(sizeof(double) * N);
    cudaStream_t s = ctx->stream;
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(ctx->vp_tmp.p, vp, sizeof(double) * N, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) r = cuda_fail(e, "copy vp", __FILE__, __LINE__);
    }
    if (!r) r = prepare_slowness(ctx, ctx->vp_tmp.as<double>(), N, false);
    ctx->schedule = PFAST_SCHEDULE_AUTO;
    ctx->near_radius = 0;
    if (!r) r = forward3d_batch(ctx, sv, 0, 1, PFAST_PLAIN_FP64, MAXSwp, nullptr);
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(U, ctx->T64.p, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = cuda_fail(e, "copy U", __FILE__, __LINE__);
    }
    pfast_survey3d_destroy(sv);
    return r;
}

pfast_status pfast_adjoint_fsm3d(double* U, double* T, double* T_obs, int* rec, double* nxyz, int* src, int* srnum,
                                 int srcid, int MAXSwp, double dx, double dy, double dz, int nrows, int ncols, int nz,
                                 int pe, double* EE) {
    (void)pe;
    if (!U || !T || !T_obs || !rec || !nxyz || !src || !srnum || srcid < 0) {
        set_last_error("null argument or negative srcid");
        return PFAST_ERR_INVALID;
    }
    pfast_ctx* ctx = nullptr;
    PFAST_TRY(default_ctx(&ctx));
    long long ch0 = 0;
    for (int s = 0; s < srcid; ++s) ch0 += srnum[s];
    pfast_survey3d* sv = nullptr;
    PFAST_TRY(pfast_survey3d_create(ctx, nrows, ncols, nz, dx, dy, dz, 1, src + 3 * srcid, srnum + srcid,
                                    rec + 3 * ch0, nxyz + 3 * ch0, T_obs + ch0, &sv));
    const long long N = (long long)nrows * ncols * nz;
    cudaStream_t s = ctx->stream;
    pfast_status r = ctx->T64.ensure(sizeof(double) * N);
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(ctx->T64.p, T, sizeof(double) * N, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) r = cuda_fail(e, "copy T", __FILE__, __LINE__);
    }
    double ee = 0.0;
    ctx->schedule = PFAST_SCHEDULE_AUTO;
    if (!r) r = adjoint3d_batch(ctx, sv, 0, 1, PFAST_PLAIN_FP64, MAXSwp, &ee, nullptr);
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(U, ctx->L64.p, sizeof(double) * N, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = cuda_fail(e, "copy lambda", __FILE__, __LINE__);
    }
    if (!r && EE) *EE = ee;
    pfast_survey3d_destroy(sv);
    return r;
}

}  // extern "C"
