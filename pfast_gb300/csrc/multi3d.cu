// multi3d.cu -- one misfit + gradient evaluation of many independent 3D models at once.
//
// The reference evaluates one model per run: its driver loops over the sources of a rank
// (src/T_PFAST3D.cpp:387-399), each a forward solve, a receiver boundary condition and an
// adjoint solve, and sums the gradient.  Here every sweep phase of every (model, source)
// instance of a set of models runs as ONE dataflow launch (kernels3d.cu): blocks take
// instances from a queue ordered largest grid first, each solves its instance to convergence
// and retires it, whatever the grid it belongs to.  The small per-model steps between phases
// (initial field, precision changes, receiver boundary condition, gradient sum) are launched
// per model.  Each model goes through exactly the operations of its own evaluation
// (forward3d_batch / adjoint3d_batch in engine.cu), so its gradient, misfit and iteration
// counts are bit-identical to evaluating it alone.

#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "engine.h"

namespace pfast {
namespace {

constexpr size_t kAlign = 256;
inline size_t up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct Model {
    const pfast_survey3d* sv = nullptr;
    const double* vp = nullptr;
    double* grad = nullptr;
    long long N = 0, mwords = 0;
    int ns = 0, ntiles = 0;
    // device work arrays (carved from ctx->multi)
    double *s64 = nullptr, *sq64 = nullptr, *T64 = nullptr, *L64 = nullptr, *scr = nullptr, *ee = nullptr;
    float *s32 = nullptr, *T32 = nullptr;
    unsigned* mask = nullptr;
    int *tflags = nullptr, *act = nullptr, *changed = nullptr, *need = nullptr, *bad = nullptr;
    unsigned long long* work = nullptr;
    // host
    std::vector<int> active, iters;
    double misfit = 0.0;
};

// Bytes of a model's work arrays (each rounded up to kAlign).
size_t model_bytes(const pfast_survey3d* sv, bool mixed) {
    const long long N = (long long)sv->nz * sv->nr * sv->nc, ns = std::max(sv->nsrc, 1);
    const long long mwords = (long long)sv->nz * sv->nr * ((sv->nc + 31) / 32);
    const long long nt = (long long)((sv->nz + TK - 1) / TK) * ((sv->nr + TI - 1) / TI) * ((sv->nc + TJ - 1) / TJ);
    size_t b = up(8 * N) + 3 * up(8 * N * ns) + up(4 * mwords * ns) + up(12 * nt * ns) + 3 * up(4 * ns) +
               up(8 * ns) + up(8 * ns) + up(4);
    if (mixed) b += up(4 * N) + up(8 * N) + up(4 * N * ns);
    return b;
}

void carve(Model& m, unsigned char*& p, bool mixed) {
    const long long N = m.N, ns = std::max(m.ns, 1);
    auto take = [&](size_t bytes) { unsigned char* q = p; p += up(bytes); return q; };
    m.s64 = (double*)take(8 * N);
    m.T64 = (double*)take(8 * N * ns);
    m.L64 = (double*)take(8 * N * ns);
    m.scr = (double*)take(8 * N * ns);
    m.mask = (unsigned*)take(4 * m.mwords * ns);
    m.tflags = (int*)take(12 * (size_t)m.ntiles * ns);
    m.act = (int*)take(4 * ns);
    m.changed = (int*)take(4 * ns);
    m.need = (int*)take(4 * ns);
    m.ee = (double*)take(8 * ns);
    m.work = (unsigned long long*)take(8 * ns);
    m.bad = (int*)take(4);
    if (mixed) {
        m.s32 = (float*)take(4 * N);
        m.sq64 = (double*)take(8 * N);
        m.T32 = (float*)take(4 * N * ns);
    }
}

// One sweep phase of `kind` over the active instances of every model: per model the lock words
// (all due, then the starting-field seed or the polish order pre-pass, exactly as run_sweeps3),
// then one dataflow launch over all (model, instance) items, largest grid first.  args[m] holds
// the model's phase arguments; iters of each model's active instances are filled in.
pfast_status multi_phase(pfast_ctx* ctx, std::vector<Model>& ms, std::vector<Sweep3Args>& args, int kind, int maxiter,
                         long long* updates, long long* updates_sub, int* iters_max, int* not_conv, double* ms_acc) {
    cudaStream_t st = ctx->stream;
    const int nm = (int)ms.size();
    std::vector<int2> items;
    int max_ntiles = 0;
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[0], st));
    for (int m = 0; m < nm; ++m) {
        Model& M = ms[m];
        Sweep3Args& a = args[m];
        const int ns = std::max(M.ns, 1);
        a.act = M.act;
        a.changed = M.changed;
        a.nbk = (M.sv->nz + TK - 1) / TK;
        a.nbi = (M.sv->nr + TI - 1) / TI;
        a.nbj = (M.sv->nc + TJ - 1) / TJ;
        a.ntiles = M.ntiles;
        a.dirty = M.tflags;
        a.stamp = a.dirty + (long long)M.ntiles * ns;
        a.diff = a.stamp + (long long)M.ntiles * ns;
        a.work = M.work;
        a.vec_rows = rows_aligned(a, kind);
        const int nact = (int)M.active.size();
        PFAST_CUDA_TRY(cudaMemsetAsync(a.dirty, 0xff, sizeof(int) * (size_t)M.ntiles * ns, st));
        PFAST_CUDA_TRY(cudaMemsetAsync(a.work, 0, sizeof(unsigned long long) * ns, st));
        PFAST_CUDA_TRY(cudaMemsetAsync(a.stamp, 0xff, sizeof(int) * (size_t)M.ntiles * ns, st));
        if (nact == 0) continue;
        PFAST_CUDA_TRY(cudaMemcpyAsync(M.act, M.active.data(), sizeof(int) * nact, cudaMemcpyHostToDevice, st));
        if (kind != kFwdPolish64) PFAST_LAUNCH(ctx, launch_seed_tiles3(kind, a, nact, st));
        if (kind == kFwdPolish64 || kind == kAdjPolish64) PFAST_LAUNCH(ctx, launch_polish_orders3(kind, a, ns, nact, st));
        for (int b : M.active) items.push_back(make_int2(m, b));
        max_ntiles = std::max(max_ntiles, M.ntiles);
    }
    // largest grids first, so that the last instances to finish are small ones
    std::stable_sort(items.begin(), items.end(),
                     [&](const int2& x, const int2& y) { return ms[x.x].N > ms[y.x].N; });
    const int nitems = (int)items.size();
    if (nitems > 0 && maxiter > 0) {
        const size_t tab = up(sizeof(Sweep3Args) * nm);
        PFAST_TRY(ctx->multi_meta.ensure(tab + sizeof(int2) * nitems));
        Sweep3Args* d_args = ctx->multi_meta.as<Sweep3Args>();
        int2* d_items = reinterpret_cast<int2*>(ctx->multi_meta.as<unsigned char>() + tab);
        // pageable copies: the host arrays may be reused right after the call returns
        PFAST_CUDA_TRY(cudaMemcpyAsync(d_args, args.data(), sizeof(Sweep3Args) * nm, cudaMemcpyHostToDevice, st));
        PFAST_CUDA_TRY(cudaMemcpyAsync(d_items, items.data(), sizeof(int2) * nitems, cudaMemcpyHostToDevice, st));
        int warps = 0, blocks = 0;
        PFAST_TRY(dataflow_shape(kind, 0, max_ntiles, nitems, &warps, &blocks, true));
        if (warps <= 0) {
            set_last_error("multi-model evaluation: a grid of %d tiles does not fit the dataflow kernel", max_ntiles);
            return PFAST_ERR_INVALID;
        }
        PFAST_TRY(ctx->queue.ensure(2 * sizeof(int)));
        PFAST_CUDA_TRY(cudaMemsetAsync(ctx->queue.p, 0, 2 * sizeof(int), st));
        PFAST_LAUNCH(ctx, launch_sweep3_dataflow_multi(kind, 0, d_args, d_items, nitems, max_ntiles, maxiter,
                                                       ctx->queue.as<int>(), warps, blocks, st));
    }
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[1], st));
    // results: stall flag, per-instance iterations, executed updates
    PFAST_TRY(ctx->h_dyn.ensure(2 * sizeof(int)));
    int* hq = ctx->h_dyn.as<int>();
    hq[1] = 0;
    if (nitems > 0 && maxiter > 0)
        PFAST_CUDA_TRY(cudaMemcpyAsync(hq, ctx->queue.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    std::vector<std::vector<int>> res(nm);
    std::vector<std::vector<unsigned long long>> wk(nm);
    for (int m = 0; m < nm; ++m) {
        const int ns = std::max(ms[m].ns, 1);
        res[m].assign(ns, 0);
        wk[m].assign(ns, 0);
        if (!ms[m].active.empty())
            PFAST_CUDA_TRY(cudaMemcpyAsync(res[m].data(), ms[m].changed, sizeof(int) * ns, cudaMemcpyDeviceToHost, st));
        PFAST_CUDA_TRY(cudaMemcpyAsync(wk[m].data(), ms[m].work, sizeof(unsigned long long) * ns, cudaMemcpyDeviceToHost, st));
    }
    PFAST_CUDA_TRY(cudaStreamSynchronize(st));
    if (hq[1]) {
        set_last_error("dataflow sweep: a block made no progress for two seconds (internal error)");
        return PFAST_ERR_CUDA;
    }
    for (int m = 0; m < nm; ++m) {
        Model& M = ms[m];
        std::vector<int> still;
        for (int b : M.active) {
            M.iters[b] = res[m][b] & 0xffff;
            if (iters_max) *iters_max = std::max(*iters_max, M.iters[b]);
            if ((res[m][b] >> 30) & 1) still.push_back(b);
        }
        if (not_conv) *not_conv += (int)still.size();
        long long u = 0;
        for (unsigned long long v : wk[m]) u += (long long)v;
        if (updates) *updates += u;
        if (updates_sub) *updates_sub += u;
    }
    double t = 0.0;
    add_elapsed(ctx->ev[0], ctx->ev[1], &t);
    if (ms_acc) *ms_acc += t;
    return PFAST_OK;
}

// The evaluation of one group of models that fits in device memory at once.
pfast_status eval_group(pfast_ctx* ctx, std::vector<Model>& ms, const pfast_options& o, pfast_stats* stats) {
    cudaStream_t st = ctx->stream;
    const bool mixed = o.precision == PFAST_MIXED;
    const int nm = (int)ms.size();
    size_t bytes = 0;
    for (Model& M : ms) bytes += model_bytes(M.sv, mixed);
    PFAST_TRY(ctx->multi.ensure(bytes));
    unsigned char* p = ctx->multi.as<unsigned char>();
    for (Model& M : ms) carve(M, p, mixed);
    pfast_stats dummy;
    std::memset(&dummy, 0, sizeof(dummy));
    pfast_stats* S = stats ? stats : &dummy;
    // ---- slowness of every model; reject a model with a velocity that is not positive
    for (Model& M : ms) {
        const double hsq = (M.sv->dx == M.sv->dy && M.sv->dy == M.sv->dz) ? M.sv->dx * M.sv->dx : 1.0;
        PFAST_CUDA_TRY(cudaMemsetAsync(M.bad, 0, sizeof(int), st));
        PFAST_LAUNCH(ctx, launch_slowness(M.vp, M.s64, mixed ? M.s32 : nullptr, mixed ? M.sq64 : nullptr, hsq, M.bad,
                                          M.N, st));
        PFAST_CUDA_TRY(cudaMemsetAsync(M.grad, 0, sizeof(double) * M.N, st));
    }
    std::vector<int> bad(nm, 0);
    for (int m = 0; m < nm; ++m)
        PFAST_CUDA_TRY(cudaMemcpyAsync(&bad[m], ms[m].bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    PFAST_CUDA_TRY(cudaStreamSynchronize(st));
    for (int m = 0; m < nm; ++m)
        if (bad[m]) {
            set_last_error("model %d holds a velocity that is not a positive finite number", m);
            return PFAST_ERR_INVALID;
        }
    std::vector<Sweep3Args> args(nm);
    auto base = [&](int m) {
        Sweep3Args a = survey_sweep_args(ms[m].sv);
        a.fstride = ms[m].N;
        return a;
    };
    auto all_active = [&]() {
        for (Model& M : ms) {
            M.active.resize(M.ns);
            std::iota(M.active.begin(), M.active.end(), 0);
            M.iters.assign(std::max(M.ns, 1), 0);
        }
    };
    const int r2 = o.near_source_radius * o.near_source_radius;
    // ---- forward (forward3d_batch)
    all_active();
    for (int m = 0; m < nm; ++m) {
        Model& M = ms[m];
        Sweep3Args& a = args[m];
        a = base(m);
        a.src_kij = M.sv->d_src_kij;
        a.src_r2 = r2;
        void* f0 = mixed ? (void*)M.scr : (void*)M.T64;
        PFAST_LAUNCH(ctx, launch_init_fwd3(f0, mixed ? 1 : 0, M.N, M.N, M.sv->d_src_lin, M.ns, st));
        if (o.near_source_radius > 0)
            PFAST_LAUNCH(ctx, launch_near_source3(f0, mixed ? 1 : 0, M.N, a.src_kij, M.s64, M.sv->nz, M.sv->nr,
                                                  M.sv->nc, a.sp, o.near_source_radius, M.ns, st));
        if (mixed) {
            a.field = M.scr;
            a.snap = nullptr;
            a.aux = M.s32;
            a.tol_abs_f = 0.0f;
            a.tol_rel_f = (float)kTol32Rel;
        } else {
            a.field = M.T64;
            a.snap = M.scr;
            a.aux = M.s64;
            a.tol_abs = kConvTol;
            a.tol_rel = 0.0;
        }
    }
    if (mixed) {
        PFAST_TRY(multi_phase(ctx, ms, args, kFwdFast32, o.maxswp, &S->fwd_node_updates, nullptr, &S->fwd32_iters_max,
                              &S->not_converged, &S->ms_fwd32));
        all_active();
        for (int m = 0; m < nm; ++m) {
            Model& M = ms[m];
            Sweep3Args& a = args[m];
            PFAST_LAUNCH(ctx, launch_widen(reinterpret_cast<float*>(M.scr), M.T64, M.N, M.N, M.N, M.ns, st));
            if (o.near_source_radius > 0)
                PFAST_LAUNCH(ctx, launch_near_source3(M.T64, 0, M.N, a.src_kij, M.s64, M.sv->nz, M.sv->nr, M.sv->nc,
                                                      a.sp, o.near_source_radius, M.ns, st));
            a.field = M.T64;
            a.snap = nullptr;
            a.aux = M.sq64;
            a.slow64 = M.s64;
            a.polish_floor = ctx->polish_floor;
            a.tol_abs = kConvTol;
            a.tol_rel = 0.0;
        }
    }
    PFAST_TRY(multi_phase(ctx, ms, args, mixed ? kFwdPolish64 : kFwdPlain64, o.maxswp, &S->fwd_node_updates,
                          &S->fwd64_node_updates, &S->fwd_iters_max, &S->not_converged, &S->ms_fwd64));
    // ---- receiver boundary condition and misfit (adjoint3d_batch)
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[2], st));
    std::vector<std::vector<double>> ee(nm);
    std::vector<std::vector<int>> need(nm);
    for (int m = 0; m < nm; ++m) {
        Model& M = ms[m];
        const int wpr = (M.sv->nc + 31) / 32;
        PFAST_CUDA_TRY(cudaMemsetAsync(M.L64, 0, sizeof(double) * M.N * M.ns, st));
        PFAST_CUDA_TRY(cudaMemsetAsync(M.mask, 0, sizeof(unsigned) * M.mwords * M.ns, st));
        Bc3Args bc;
        bc.T = M.T64;
        bc.L = M.L64;
        bc.fstride = M.N;
        bc.mask = M.mask;
        bc.mask_stride = M.mwords;
        bc.wpr = wpr;
        bc.rec = M.sv->d_rec;
        bc.nxyz = M.sv->d_nxyz;
        bc.tobs = M.sv->d_tobs;
        bc.last = M.sv->d_last;
        bc.ch0 = M.sv->d_ch0;
        bc.srnum = M.sv->d_srnum;
        bc.src_kij = M.sv->d_src_kij;
        bc.EE = M.ee;
        bc.need = M.need;
        bc.nz = M.sv->nz;
        bc.nr = M.sv->nr;
        bc.nc = M.sv->nc;
        bc.dx = M.sv->dx;
        bc.dy = M.sv->dy;
        bc.dz = M.sv->dz;
        PFAST_LAUNCH(ctx, launch_bc3(bc, M.ns, st));
        ee[m].assign(M.ns, 0.0);
        need[m].assign(M.ns, 0);
        PFAST_CUDA_TRY(cudaMemcpyAsync(ee[m].data(), M.ee, sizeof(double) * M.ns, cudaMemcpyDeviceToHost, st));
        PFAST_CUDA_TRY(cudaMemcpyAsync(need[m].data(), M.need, sizeof(int) * M.ns, cudaMemcpyDeviceToHost, st));
    }
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[3], st));
    PFAST_CUDA_TRY(cudaStreamSynchronize(st));
    add_elapsed(ctx->ev[2], ctx->ev[3], &S->ms_other);
    std::vector<std::vector<int>> active64(nm);
    for (int m = 0; m < nm; ++m) {
        Model& M = ms[m];
        M.misfit = 0.0;
        for (int b = 0; b < M.ns; ++b) M.misfit += ee[m][b];   // loc_E += EE in source order
        M.active.clear();
        for (int b = 0; b < M.ns; ++b)
            if (need[m][b]) M.active.push_back(b);
        M.iters.assign(std::max(M.ns, 1), 0);
        active64[m] = M.active;
        Sweep3Args& a = args[m];
        a = base(m);
        a.mask = M.mask;
        a.mask_stride = M.mwords;
        if (mixed) {
            PFAST_LAUNCH(ctx, launch_narrow(M.L64, reinterpret_cast<float*>(M.scr), M.N, M.N, M.N, M.ns, st));
            PFAST_LAUNCH(ctx, launch_narrow(M.T64, M.T32, M.N, M.N, M.N, M.ns, st));
            a.field = M.scr;
            a.snap = nullptr;
            a.aux = M.T32;
            a.tol_abs_f = (float)kTol32AbsAdj;
            a.tol_rel_f = (float)kTol32Rel;
        } else {
            a.field = M.L64;
            a.snap = M.scr;
            a.aux = M.T64;
            a.tol_abs = kConvTol;
            a.tol_rel = 0.0;
        }
    }
    if (mixed) {
        PFAST_TRY(multi_phase(ctx, ms, args, kAdjFast32, o.maxswp, &S->adj_node_updates, nullptr, &S->adj32_iters_max,
                              &S->not_converged, &S->ms_adj32));
        for (int m = 0; m < nm; ++m) {
            Model& M = ms[m];
            Sweep3Args& a = args[m];
            PFAST_LAUNCH(ctx, launch_widen_lambda(reinterpret_cast<float*>(M.scr), M.L64, M.mask, M.N, M.N, M.mwords,
                                                  M.sv->nz, M.sv->nr, M.sv->nc, (M.sv->nc + 31) / 32, M.ns, st));
            M.active = active64[m];
            M.iters.assign(std::max(M.ns, 1), 0);
            a.field = M.L64;
            a.snap = nullptr;
            a.aux = M.T64;
            a.polish_floor = ctx->polish_floor;
            a.tol_abs = kConvTol;
            a.tol_rel = 0.0;
        }
    }
    PFAST_TRY(multi_phase(ctx, ms, args, mixed ? kAdjPolish64 : kAdjPlain64, o.maxswp, &S->adj_node_updates,
                          &S->adj64_node_updates, &S->adj_iters_max, &S->not_converged, &S->ms_adj64));
    // ---- gradient: g -= lambda / v^3 in source order (mixed: lambda summed, one division)
    for (Model& M : ms) {
        PFAST_LAUNCH(ctx, launch_accumulate(M.grad, M.L64, M.N, M.vp, M.N, M.ns, !mixed, st));
        if (mixed) PFAST_LAUNCH(ctx, launch_finish_gradient(M.grad, M.vp, M.N, st));
    }
    if (stats) ++stats->batches;
    return PFAST_OK;
}

}  // namespace
}  // namespace pfast

using namespace pfast;

extern "C" pfast_status pfast_surveys3d_eval(pfast_ctx* ctx, int n, pfast_survey3d* const* surveys,
                                             const double* const* vp, double* const* grad, double* misfit,
                                             const pfast_options* opt, pfast_stats* stats) {
    if (!ctx || n < 0 || (n > 0 && (!surveys || !vp || !grad || !misfit))) {
        set_last_error("null argument");
        return PFAST_ERR_INVALID;
    }
    if (!valid_options(opt)) return PFAST_ERR_INVALID;
    const pfast_options o = resolve_options(opt, 100);
    for (int m = 0; m < n; ++m) {
        const pfast_survey3d* sv = surveys[m];
        if (!sv || !vp[m] || !grad[m]) { set_last_error("model %d: null survey, model or gradient", m); return PFAST_ERR_INVALID; }
        if (sv->ctx != ctx) { set_last_error("model %d: survey of another context", m); return PFAST_ERR_INVALID; }
        if (!sv->has_picks) { set_last_error("model %d: survey has no picks: gradient unavailable", m); return PFAST_ERR_INVALID; }
        const long long nt = (long long)((sv->nz + TK - 1) / TK) * ((sv->nr + TI - 1) / TI) * ((sv->nc + TJ - 1) / TJ);
        if (nt > kDataflowMaxTiles) {
            set_last_error("model %d: %lld tiles exceed the %d of a multi-model evaluation (evaluate it alone)", m, nt,
                           kDataflowMaxTiles);
            return PFAST_ERR_INVALID;
        }
    }
    stats_begin(stats);
    PFAST_CUDA_TRY(cudaSetDevice(ctx->device));
    ctx->polish_floor = o.polish_floor > 0.0 ? (float)o.polish_floor : kPolishFloor;
    ctx->near_radius = o.near_source_radius;
    cudaEvent_t t0 = ctx->ev[6], t1 = ctx->ev[7];
    PFAST_CUDA_TRY(cudaEventRecord(t0, ctx->stream));
    const long long launches0 = ctx->launches;
    const bool mixed = o.precision == PFAST_MIXED;
    // a survey without sources has a zero gradient and misfit
    std::vector<int> idx;
    for (int m = 0; m < n; ++m) {
        if (surveys[m]->nsrc > 0) { idx.push_back(m); continue; }
        PFAST_CUDA_TRY(cudaMemsetAsync(grad[m], 0, sizeof(double) * surveys[m]->nz * surveys[m]->nr * surveys[m]->nc,
                                       ctx->stream));
        misfit[m] = 0.0;
    }
    // groups of consecutive models whose work arrays fit in 85% of the free device memory (all
    // models at once when they fit); a model's results do not depend on its group
    const int nn = (int)idx.size();
    int m0 = 0;
    while (m0 < nn) {
        size_t fr = 0, tot = 0;
        PFAST_CUDA_TRY(cudaMemGetInfo(&fr, &tot));
        const size_t budget = (size_t)(0.85 * (double)(fr + ctx->multi.cap));
        size_t used = 0;
        int m1 = m0;
        while (m1 < nn) {
            const size_t b = model_bytes(surveys[idx[m1]], mixed) + 16 * kAlign;
            if (m1 > m0 && used + b > budget) break;
            used += b;
            ++m1;
        }
        std::vector<Model> ms(m1 - m0);
        for (int m = m0; m < m1; ++m) {
            Model& M = ms[m - m0];
            M.sv = surveys[idx[m]];
            M.vp = vp[idx[m]];
            M.grad = grad[idx[m]];
            M.N = (long long)M.sv->nz * M.sv->nr * M.sv->nc;
            M.mwords = (long long)M.sv->nz * M.sv->nr * ((M.sv->nc + 31) / 32);
            M.ns = M.sv->nsrc;
            M.ntiles = ((M.sv->nz + TK - 1) / TK) * ((M.sv->nr + TI - 1) / TI) * ((M.sv->nc + TJ - 1) / TJ);
        }
        PFAST_TRY(eval_group(ctx, ms, o, stats));
        for (int m = m0; m < m1; ++m) misfit[idx[m]] = ms[m - m0].misfit;
        m0 = m1;
    }
    PFAST_CUDA_TRY(cudaEventRecord(t1, ctx->stream));
    PFAST_CUDA_TRY(cudaStreamSynchronize(ctx->stream));
    if (stats) {
        add_elapsed(t0, t1, &stats->ms_total);
        stats->launches = ctx->launches - launches0;
    }
    return PFAST_OK;
}
