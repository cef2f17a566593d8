// engine2d.cu -- 2D surveys and pipelines: RT_fsm2d with Huygens reflection
// (src/RT_pfsm2d.h:116-380), the transmission / reflection adjoints
// (src/RT_padjoint2d.h:288-473) and the joint-gradient accumulation
// (src/RT_PFAST2D.cpp:420-457), batched over sources on one GPU.
//
// Device field layout per batch source b: slots [TT, TTd_0..TTd_{R-1},
// TTu_0..TTu_{R-1}], each nrows*ncols doubles, at (b*(1+2R) + slot)*N.

#include <cstring>
#include <algorithm>
#include <vector>

#include "engine.h"

namespace pfast {

#define PFAST_TRY2(expr)                  \
    do {                                  \
        pfast_status s__ = (expr);        \
        if (s__ != PFAST_OK) return s__;  \
    } while (0)

namespace {

constexpr double kTol32Rel2 = 1.0 / (1 << 20);
constexpr double kTol32AbsAdj2 = 1e-6;

// Per-instance device tables of one 2D phase.
struct InstTables {
    std::vector<long long> off, aux_off, mask_off, off32;
    std::vector<int> lim, src, srcnode, ir, gsrc;
};

// Upload a phase's instance tables into ctx->misc; returns device pointers.
struct InstDev {
    long long *off = nullptr, *aux_off = nullptr, *mask_off = nullptr, *off32 = nullptr;
    int *lim = nullptr, *src = nullptr, *srcnode = nullptr, *ir = nullptr, *gsrc = nullptr;
};

pfast_status upload_inst(pfast_ctx* ctx, DevBuf& buf, const InstTables& t, InstDev& d) {
    const size_t n = t.off.size();
    const std::vector<long long> z64(n, 0);
    const std::vector<int> z32(n, -1);
    const std::vector<long long>* v64[4] = {&t.off, &t.aux_off, &t.mask_off, &t.off32};
    const std::vector<int>* v32[5] = {&t.lim, &t.src, &t.srcnode, &t.ir, &t.gsrc};
    const size_t bytes = n * (4 * sizeof(long long) + 5 * sizeof(int)) + 9 * 8;
    PFAST_TRY2(buf.ensure(bytes));
    std::vector<unsigned char> h(bytes, 0);
    size_t at[9], o = 0;
    for (int k = 0; k < 4; ++k) {
        const std::vector<long long>& v = v64[k]->empty() ? z64 : *v64[k];
        at[k] = o;
        std::memcpy(h.data() + o, v.data(), n * sizeof(long long));
        o += n * sizeof(long long);
    }
    for (int k = 0; k < 5; ++k) {
        const std::vector<int>& v = v32[k]->empty() ? z32 : *v32[k];
        at[4 + k] = o;
        std::memcpy(h.data() + o, v.data(), n * sizeof(int));
        o += (n * sizeof(int) + 7) & ~size_t(7);
    }
    PFAST_CUDA_TRY(cudaMemcpyAsync(buf.p, h.data(), o, cudaMemcpyHostToDevice, ctx->stream));
    PFAST_CUDA_TRY(cudaStreamSynchronize(ctx->stream));   // h is a local staging vector
    unsigned char* base = buf.as<unsigned char>();
    d.off = (long long*)(base + at[0]);
    d.aux_off = (long long*)(base + at[1]);
    d.mask_off = (long long*)(base + at[2]);
    d.off32 = (long long*)(base + at[3]);
    d.lim = (int*)(base + at[4]);
    d.src = (int*)(base + at[5]);
    d.srcnode = (int*)(base + at[6]);
    d.ir = (int*)(base + at[7]);
    d.gsrc = (int*)(base + at[8]);
    return PFAST_OK;
}

// One outer iteration of a 2D phase as a replayed CUDA graph (see the 3D sweeps): the diff
// reset, the 4 x ndiag launches and the per-instance reduction, captured once per (kind,
// arguments, active count); the launches read the iteration and the active count from a.dyn.
static pfast_status iteration_graph2(pfast_ctx* ctx, const Sweep2Args& a, int kind, const DiagTable2& dt, int ninst,
                                     int nact, cudaStream_t st, cudaGraphExec_t* out) {
    Sweep2Args k = a;
    k.dir = 0;
    k.iter = 0;
    const int extra[5] = {2, kind, nact, ninst, dt.ndiag};
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
    cudaError_t e = cudaMemsetAsync(k.diff, 0, sizeof(int) * (size_t)k.ntiles * ninst, st);
    for (int dir = 0; dir < 4 && !r && e == cudaSuccess; ++dir) {
        k.dir = dir;
        for (int d = 0; d < dt.ndiag && !r; ++d) r = launch_sweep2(kind, k, d, dt.h_off[d + 1] - dt.h_off[d], nact, st);
    }
    if (!r && e == cudaSuccess) e = cudaMemsetAsync(k.changed, 0, sizeof(int) * ninst, st);
    if (!r && e == cudaSuccess)
        r = launch_reduce_diff(k.diff, k.dirty, kind == kFwdPolish64 || kind == kAdjPolish64, 4, 0xf, k.ntiles, k.act,
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

// Outer iterations of a 2D phase; caps[q] = iteration cap of instance q.
pfast_status run_sweeps2(pfast_ctx* ctx, Sweep2Args a, int kind, const DiagTable2& dt, int ninst,
                         std::vector<int>& active, const std::vector<int>& caps, int* iters, long long nodes,
                         long long* node_updates, int* not_conv, double* ms_acc) {
    PFAST_TRY2(ctx->act.ensure(sizeof(int) * ninst));
    PFAST_TRY2(ctx->changed.ensure(sizeof(int) * ninst));
    PFAST_TRY2(ctx->h_act.ensure(sizeof(int) * ninst));
    PFAST_TRY2(ctx->h_changed.ensure(sizeof(int) * ninst));
    int* h_act = ctx->h_act.as<int>();
    int* h_chg = ctx->h_changed.as<int>();
    a.act = ctx->act.as<int>();
    a.changed = ctx->changed.as<int>();
    a.diag_off = dt.d_off;
    a.diag_tiles = dt.d_tiles;
    a.nbi = dt.nbi;
    a.nbj = dt.nbj;
    cudaStream_t st = ctx->stream;
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[4], st));
    // instances whose cap is already used up run no iteration
    {
        std::vector<int> keep;
        for (int q : active)
            if (caps[q] > 0) keep.push_back(q);
        active.swap(keep);
    }
    // tile-locking flags (see the 3D sweeps): every tile unlocked, no snapshot yet
    const long long ntiles = (long long)dt.nbi * dt.nbj;
    PFAST_TRY2(ctx->tflags.ensure(sizeof(int) * 3 * ntiles * ninst));
    a.ntiles = (int)ntiles;
    a.dirty = ctx->tflags.as<int>();
    a.stamp = a.dirty + ntiles * ninst;
    a.diff = a.stamp + ntiles * ninst;
    PFAST_CUDA_TRY(cudaMemsetAsync(a.dirty, 0xff, sizeof(int) * ntiles * ninst, st));
    PFAST_CUDA_TRY(cudaMemsetAsync(a.stamp, 0xff, sizeof(int) * ntiles * ninst, st));
    if (kind != kFwdPolish64 && !active.empty()) {
        // only tiles with something to propagate start due
        const int nact0 = (int)active.size();
        std::memcpy(h_act, active.data(), sizeof(int) * nact0);
        PFAST_CUDA_TRY(cudaMemcpyAsync(const_cast<int*>(a.act), h_act, sizeof(int) * nact0, cudaMemcpyHostToDevice, st));
        PFAST_LAUNCH(ctx, launch_seed_tiles2(kind, a, nact0, st));
    }
    PFAST_TRY2(ctx->work.ensure(sizeof(unsigned long long) * ninst));
    PFAST_TRY2(ctx->h_work.ensure(sizeof(unsigned long long) * ninst));
    a.work = ctx->work.as<unsigned long long>();
    PFAST_CUDA_TRY(cudaMemsetAsync(a.work, 0, sizeof(unsigned long long) * ninst, st));
    int it = 0;
    cudaGraphExec_t exec = nullptr;
    if (ctx->graphs && !active.empty()) {
        // captured with the first iteration's active count; later iterations only retire instances
        PFAST_TRY2(ctx->dyn.ensure(2 * sizeof(int)));
        PFAST_TRY2(ctx->h_dyn.ensure(2 * sizeof(int)));
        a.dyn = ctx->dyn.as<int>();
        PFAST_TRY2(iteration_graph2(ctx, a, kind, dt, ninst, (int)active.size(), st, &exec));
        if (!exec) a.dyn = nullptr;   // launched one by one
    }
    while (!active.empty()) {
        const int nact = (int)active.size();
        std::memcpy(h_act, active.data(), sizeof(int) * nact);
        PFAST_CUDA_TRY(cudaMemcpyAsync(const_cast<int*>(a.act), h_act, sizeof(int) * nact, cudaMemcpyHostToDevice, st));
        if (exec) {
            int* hd = ctx->h_dyn.as<int>();
            hd[0] = it;
            hd[1] = nact;
            PFAST_CUDA_TRY(cudaMemcpyAsync(ctx->dyn.p, hd, 2 * sizeof(int), cudaMemcpyHostToDevice, st));
            PFAST_CUDA_TRY(cudaGraphLaunch(exec, st));
            ctx->launches += 4LL * dt.ndiag + 1;
        } else {
            PFAST_CUDA_TRY(cudaMemsetAsync(a.diff, 0, sizeof(int) * ntiles * ninst, st));
            a.iter = it;
            for (int dir = 0; dir < 4; ++dir) {
                a.dir = dir;
                for (int d = 0; d < dt.ndiag; ++d) {
                    PFAST_LAUNCH(ctx, launch_sweep2(kind, a, d, dt.h_off[d + 1] - dt.h_off[d], nact, st));
                }
            }
            PFAST_CUDA_TRY(cudaMemsetAsync(a.changed, 0, sizeof(int) * ninst, st));
            PFAST_LAUNCH(ctx, launch_reduce_diff(a.diff, a.dirty, kind == kFwdPolish64 || kind == kAdjPolish64, 4, 0xf,
                                                 a.ntiles, a.act, nact, a.changed, st));
        }
        cudaError_t le = cudaGetLastError();
        if (le != cudaSuccess) return cuda_fail(le, "sweep2 launch", __FILE__, __LINE__);
        PFAST_CUDA_TRY(cudaMemcpyAsync(h_chg, a.changed, sizeof(int) * ninst, cudaMemcpyDeviceToHost, st));
        PFAST_CUDA_TRY(cudaStreamSynchronize(st));
        ++it;
        std::vector<int> still;
        for (int q : active) {
            iters[q] = it;
            if (h_chg[q] & 1) {
                if (it < caps[q]) {
                    // moved, but every tile locked: the next iteration would change nothing and
                    // pass the convergence test; it is counted without being launched
                    if (!(h_chg[q] & 2)) iters[q] = it + 1;
                    else still.push_back(q);
                } else if (not_conv) {
                    ++*not_conv;
                }
            }
        }
        active.swap(still);
    }
    if (node_updates) {
        unsigned long long* hw = ctx->h_work.as<unsigned long long>();
        PFAST_CUDA_TRY(cudaMemcpyAsync(hw, a.work, sizeof(unsigned long long) * ninst, cudaMemcpyDeviceToHost, st));
        PFAST_CUDA_TRY(cudaStreamSynchronize(st));
        for (int q = 0; q < ninst; ++q) *node_updates += (long long)hw[q];
    }
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[5], st));
    add_elapsed(ctx->ev[4], ctx->ev[5], ms_acc);
    return PFAST_OK;
}

Sweep2Args base2(const pfast_survey2d* sv) {
    Sweep2Args a;
    std::memset(&a, 0, sizeof(a));
    a.nr = sv->nr;
    a.nc = sv->nc;
    a.dx = sv->dx;
    a.dz = sv->dz;
    a.inv2x = 1.0 / sv->dx / sv->dx;
    a.inv2z = 1.0 / sv->dz / sv->dz;
    a.dxf = (float)sv->dx;
    a.dzf = (float)sv->dz;
    a.wxf = (float)a.inv2x;
    a.wzf = (float)a.inv2z;
    a.rsumf = (float)(1.0 / (a.inv2x + a.inv2z));
    a.polish_floor = kPolishFloor;
    a.wpr = (sv->nc + 31) / 32;
    return a;
}

// One FSM phase over instance table t (fields at `fields` + t.off).  Plain: FP64 in
// place.  Mixed: FP32 bulk in scratch (instance q at q*N), widen, FP64 polish.
// `init` = initialise the fields to the point-source state first.
pfast_status fwd_phase2(pfast_ctx* ctx, pfast_survey2d* sv, double* fields, const InstTables& t, bool init,
                        int precision, int maxswp, const double* s64, const float* s32, pfast_stats* st) {
    const int ninst = (int)t.off.size();
    if (ninst == 0) return PFAST_OK;
    const long long N = (long long)sv->nr * sv->nc;
    DiagTable2* dt = nullptr;
    PFAST_TRY2(ctx_diag2(ctx, sv->nr, sv->nc, &dt));
    InstTables tt = t;
    tt.off32.resize(ninst);
    for (int q = 0; q < ninst; ++q) tt.off32[q] = (long long)q * N;
    InstDev d;
    PFAST_TRY2(upload_inst(ctx, ctx->misc, tt, d));
    PFAST_TRY2(ctx->scratch.ensure(sizeof(double) * N * ninst));
    cudaStream_t s = ctx->stream;
    Sweep2Args a = base2(sv);
    a.inst_lim = d.lim;
    a.inst_src = d.src;
    a.rowlim = sv->d_k2vec;
    a.src_r2 = ctx->near_radius * ctx->near_radius;
    // opt-in near-source start of the point-source instances (FP32 or FP64 fields)
    auto near = [&](void* base, int is_fp32, const long long* off) -> pfast_status {
        if (!init || ctx->near_radius <= 0) return PFAST_OK;
        PFAST_LAUNCH(ctx, launch_near_source2(base, is_fp32, off, d.src, d.lim, sv->d_k2vec, s64, sv->nr, sv->nc,
                                              sv->dx, sv->dz, ctx->near_radius, ninst, s));
        return PFAST_OK;
    };
    std::vector<int> active(ninst), iters(ninst, 0), caps(ninst, maxswp);
    for (int q = 0; q < ninst; ++q) active[q] = q;
    int dummy = 0;
    int* ncv = st ? &st->not_converged : &dummy;
    long long* nu = st ? &st->fwd_node_updates : nullptr;
    if (precision == PFAST_PLAIN_FP64) {
        if (init) PFAST_LAUNCH(ctx, launch_init2(fields, 0, d.off, d.srcnode, N, ninst, s));
        PFAST_TRY2(near(fields, 0, d.off));
        a.field = fields;
        a.inst_off = d.off;
        a.aux = s64;
        a.snap = ctx->scratch.p;
        a.tol_abs = kConvTol;
        long long before = nu ? *nu : 0;
        PFAST_TRY2(run_sweeps2(ctx, a, kFwdPlain64, *dt, ninst, active, caps, iters.data(), N, nu, ncv,
                               st ? &st->ms_fwd64 : nullptr));
        if (st) {
            st->fwd64_node_updates += *nu - before;
            for (int v : iters) st->fwd_iters_max = std::max(st->fwd_iters_max, v);
        }
    } else {
        float* f32 = ctx->scratch.as<float>();
        float* snap32 = f32 + N * ninst;
        if (init) PFAST_LAUNCH(ctx, launch_init2(f32, 1, d.off32, d.srcnode, N, ninst, s));
        else PFAST_LAUNCH(ctx, launch_narrow_inst(fields, f32, d.off, d.off32, N, ninst, s));
        PFAST_TRY2(near(f32, 1, d.off32));
        a.field = f32;
        a.inst_off = d.off32;
        a.aux = s32;
        a.snap = snap32;
        a.tol_rel = kTol32Rel2;
        PFAST_TRY2(run_sweeps2(ctx, a, kFwdFast32, *dt, ninst, active, caps, iters.data(), N, nu, ncv,
                               st ? &st->ms_fwd32 : nullptr));
        if (st) for (int v : iters) st->fwd32_iters_max = std::max(st->fwd32_iters_max, v);
        PFAST_LAUNCH(ctx, launch_widen_inst(f32, fields, d.off32, d.off, N, ninst, s));
        PFAST_TRY2(near(fields, 0, d.off));   // the fixed region keeps its FP64 values in the polish
        active.resize(ninst);
        for (int q = 0; q < ninst; ++q) { active[q] = q; iters[q] = 0; }
        a.field = fields;
        a.inst_off = d.off;
        a.aux = s64;
        a.snap = ctx->scratch.p;
        a.tol_abs = kConvTol;
        a.tol_rel = 0.0;
        long long before = nu ? *nu : 0;
        PFAST_TRY2(run_sweeps2(ctx, a, kFwdPolish64, *dt, ninst, active, caps, iters.data(), N, nu, ncv,
                               st ? &st->ms_fwd64 : nullptr));
        if (st) {
            st->fwd64_node_updates += *nu - before;
            for (int v : iters) st->fwd_iters_max = std::max(st->fwd_iters_max, v);
        }
    }
    return PFAST_OK;
}

// Forward for batch sources [b0, b0+nb) into ctx->f2a.
pfast_status forward2d_batch(pfast_ctx* ctx, pfast_survey2d* sv, int b0, int nb, int precision, int maxswp,
                             const double* s64, const float* s32, pfast_stats* st) {
    const int R = sv->numofr;
    const long long N = (long long)sv->nr * sv->nc;
    const int slots = 1 + 2 * R;
    PFAST_TRY2(ctx->f2a.ensure(sizeof(double) * N * slots * nb));
    double* F = ctx->f2a.as<double>();
    cudaStream_t s = ctx->stream;
    // phase A: transmission + down-going solves
    InstTables A;
    for (int b = 0; b < nb; ++b) {
        const int g = b0 + b;
        const int si = sv->h_src[2 * g], sj = sv->h_src[2 * g + 1];
        const int packed = (si << 16) | sj;
        const int node = si * sv->nc + sj;
        for (int slot = 0; slot <= R; ++slot) {
            A.off.push_back(((long long)b * slots + slot) * N);
            A.lim.push_back(slot == 0 ? -1 : slot - 1);   // rowlim rows 0..R-1: below-reflector limits
            A.src.push_back(packed);
            A.srcnode.push_back(node);
        }
    }
    PFAST_TRY2(fwd_phase2(ctx, sv, F, A, true, precision, maxswp, s64, s32, st));
    if (R == 0) return PFAST_OK;
    // phase B: TTu <- TTd, reflection points, INF above them
    InstTables B;
    for (int b = 0; b < nb; ++b)
        for (int ir = 0; ir < R; ++ir) {
            B.off.push_back(((long long)b * slots + 1 + R + ir) * N);
            B.aux_off.push_back(((long long)b * slots + 1 + ir) * N);
            B.ir.push_back(ir);
        }
    InstDev bd;
    PFAST_TRY2(upload_inst(ctx, ctx->misc, B, bd));
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
    const int nB = (int)B.off.size();
    PFAST_LAUNCH(ctx, launch_copy_inst(F, F, 0, bd.aux_off, bd.off, N, nB, s));
    PFAST_TRY2(ctx->need.ensure(sizeof(int)));
    PFAST_CUDA_TRY(cudaMemsetAsync(ctx->need.p, 0, sizeof(int), s));
    Reflect2Args ra;
    ra.U = F;
    ra.inst_off = bd.off;
    ra.inst_ir = bd.ir;
    ra.k2 = sv->d_k2vec + 2 * (long long)R * sv->nc;
    ra.qxcase = sv->d_k2vec + 3 * (long long)R * sv->nc;
    ra.k2vec = sv->d_k2vec + (long long)R * sv->nc;
    ra.Z = sv->d_Z;
    ra.nr = sv->nr;
    ra.nc = sv->nc;
    ra.dx = sv->dx;
    ra.dz = sv->dz;
    ra.err = ctx->need.as<int>();
    PFAST_LAUNCH(ctx, launch_reflect2(ra, nB, s));
    int herr = 0;
    PFAST_CUDA_TRY(cudaMemcpyAsync(&herr, ctx->need.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    add_elapsed(ctx->ev[2], ctx->ev[3], st ? &st->ms_other : nullptr);
    if (herr) {
        set_last_error("negative reflected traveltime at a reflection point");
        return PFAST_ERR_NEGATIVE_TIME;
    }
    // phase C: up-going solves above the reflection points (no source exclusion)
    InstTables C;
    for (int b = 0; b < nb; ++b)
        for (int ir = 0; ir < R; ++ir) {
            C.off.push_back(((long long)b * slots + 1 + R + ir) * N);
            C.lim.push_back(R + ir);   // rowlim rows R..2R-1: k2vec
            C.src.push_back(-1);
            C.srcnode.push_back(-1);
        }
    PFAST_TRY2(fwd_phase2(ctx, sv, F, C, false, precision, maxswp, s64, s32, st));
    return PFAST_OK;
}

// Adjoint phase over instances (lambda fields in `L` at t.off, T at F + t.aux_off,
// masks at ctx->mask + t.mask_off); BC + sweeps.  ee[q] accumulates the misfit.
pfast_status adj_phase2(pfast_ctx* ctx, pfast_survey2d* sv, double* L, const double* F, const InstTables& t,
                        int precision, const std::vector<int>& caps, std::vector<int>& iters_out, double* d_ee,
                        pfast_stats* st) {
    const int ninst = (int)t.off.size();
    if (ninst == 0) return PFAST_OK;
    const long long N = (long long)sv->nr * sv->nc;
    DiagTable2* dt = nullptr;
    PFAST_TRY2(ctx_diag2(ctx, sv->nr, sv->nc, &dt));
    InstTables tt = t;
    tt.off32.resize(ninst);
    for (int q = 0; q < ninst; ++q) tt.off32[q] = (long long)q * N;
    InstDev d;
    PFAST_TRY2(upload_inst(ctx, ctx->misc, tt, d));
    PFAST_TRY2(ctx->scratch.ensure(sizeof(double) * N * ninst));
    PFAST_TRY2(ctx->need.ensure(sizeof(int) * ninst));
    PFAST_TRY2(ctx->h_need.ensure(sizeof(int) * ninst));
    cudaStream_t s = ctx->stream;
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[2], s));
    Bc2Args bc;
    bc.T = F;
    bc.t_off = d.aux_off;
    bc.L = L;
    bc.l_off = d.off;
    bc.mask = ctx->mask.as<unsigned>();
    bc.mask_off = d.mask_off;
    bc.wpr = (sv->nc + 31) / 32;
    bc.inst_src = d.gsrc;
    bc.inst_ir = d.ir;
    bc.rec = sv->d_rec;
    bc.nxy = sv->d_nxy;
    bc.ttobs = sv->d_ttobs;
    bc.trobs = sv->d_trobs;
    bc.last_t = sv->d_last_t;
    bc.last_r = sv->d_last_r;
    bc.ch0 = sv->d_ch0;
    bc.srnum = sv->d_srnum;
    bc.src_ij = sv->d_src_ij;
    bc.numofr = sv->numofr;
    bc.EE = d_ee;
    bc.need = ctx->need.as<int>();
    bc.nr = sv->nr;
    bc.nc = sv->nc;
    bc.dx = sv->dx;
    bc.dz = sv->dz;
    PFAST_LAUNCH(ctx, launch_bc2(bc, ninst, s));
    PFAST_CUDA_TRY(cudaMemcpyAsync(ctx->h_need.p, ctx->need.p, sizeof(int) * ninst, cudaMemcpyDeviceToHost, s));
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[3], s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    add_elapsed(ctx->ev[2], ctx->ev[3], st ? &st->ms_other : nullptr);
    std::vector<int> active;
    for (int q = 0; q < ninst; ++q)
        if (ctx->h_need.as<int>()[q]) active.push_back(q);
    iters_out.assign(ninst, 0);
    Sweep2Args a = base2(sv);
    a.aux = F;
    a.aux_off = d.aux_off;
    a.mask = ctx->mask.as<unsigned>();
    a.mask_off = d.mask_off;
    std::vector<int> inst_lim(ninst, -1);
    a.inst_lim = d.lim;   // all -1 (unused by the adjoint)
    a.inst_src = d.src;
    const long long interior = (long long)std::max(0, sv->nr - 2) * std::max(0, sv->nc - 2);
    int dummy = 0;
    int* ncv = st ? &st->not_converged : &dummy;
    long long* nu = st ? &st->adj_node_updates : nullptr;
    if (precision == PFAST_PLAIN_FP64) {
        a.field = L;
        a.inst_off = d.off;
        a.snap = ctx->scratch.p;
        a.tol_abs = kConvTol;
        long long before = nu ? *nu : 0;
        PFAST_TRY2(run_sweeps2(ctx, a, kAdjPlain64, *dt, ninst, active, caps, iters_out.data(), interior, nu, ncv,
                               st ? &st->ms_adj64 : nullptr));
        if (st) {
            st->adj64_node_updates += *nu - before;
            for (int v : iters_out) st->adj_iters_max = std::max(st->adj_iters_max, v);
        }
    } else {
        std::vector<int> active64 = active;
        std::vector<int> it32(ninst, 0);
        float* f32 = ctx->scratch.as<float>();
        float* snap32 = f32 + N * ninst;
        PFAST_LAUNCH(ctx, launch_narrow_inst(L, f32, d.off, d.off32, N, ninst, s));
        a.field = f32;
        a.inst_off = d.off32;
        a.snap = snap32;
        a.tol_abs = kTol32AbsAdj2;
        a.tol_rel = kTol32Rel2;
        PFAST_TRY2(run_sweeps2(ctx, a, kAdjFast32, *dt, ninst, active, caps, it32.data(), interior, nu, ncv,
                               st ? &st->ms_adj32 : nullptr));
        if (st) for (int v : it32) st->adj32_iters_max = std::max(st->adj32_iters_max, v);
        PFAST_LAUNCH(ctx, launch_widen_lambda_inst(f32, L, d.off32, d.off, ctx->mask.as<unsigned>(), d.mask_off, sv->nr,
                                            sv->nc, (sv->nc + 31) / 32, ninst, s));
        a.field = L;
        a.inst_off = d.off;
        a.snap = ctx->scratch.p;
        a.tol_abs = kConvTol;
        a.tol_rel = 0.0;
        long long before = nu ? *nu : 0;
        PFAST_TRY2(run_sweeps2(ctx, a, kAdjPolish64, *dt, ninst, active64, caps, iters_out.data(), interior, nu, ncv,
                               st ? &st->ms_adj64 : nullptr));
        if (st) {
            st->adj64_node_updates += *nu - before;
            for (int v : iters_out) st->adj_iters_max = std::max(st->adj_iters_max, v);
        }
    }
    return PFAST_OK;
}

// Adjoints of batch sources [b0, b0+nb) from the fields in ctx->f2a: per source the
// transmission lambda (f2b slot 2b) and the summed reflection lambda (slot 2b+1).
// eeT/eeR receive the per-source misfits.
pfast_status adjoint2d_batch(pfast_ctx* ctx, pfast_survey2d* sv, int b0, int nb, int precision, int maxswp,
                             double* eeT, double* eeR, pfast_stats* st, bool do_t = true, bool do_r = true) {
    const int R = sv->numofr;
    const long long N = (long long)sv->nr * sv->nc;
    const int slots = 1 + 2 * R;
    const int wpr = (sv->nc + 31) / 32;
    const long long mwords = (long long)sv->nr * wpr;
    cudaStream_t s = ctx->stream;
    double* F = ctx->f2a.as<double>();
    PFAST_TRY2(ctx->f2b.ensure(sizeof(double) * N * 2 * nb));      // lamT, UR per source
    PFAST_TRY2(ctx->f2c.ensure(sizeof(double) * N * nb));          // lambda of the current reflector
    PFAST_TRY2(ctx->mask.ensure(sizeof(unsigned) * mwords * 2 * nb));
    PFAST_TRY2(ctx->ee.ensure(sizeof(double) * 2 * nb));
    PFAST_TRY2(ctx->h_ee.ensure(sizeof(double) * 2 * nb));
    double* LB = ctx->f2b.as<double>();
    double* LC = ctx->f2c.as<double>();
    PFAST_CUDA_TRY(cudaMemsetAsync(LB, 0, sizeof(double) * N * 2 * nb, s));
    PFAST_CUDA_TRY(cudaMemsetAsync(ctx->mask.p, 0, sizeof(unsigned) * mwords * 2 * nb, s));
    PFAST_CUDA_TRY(cudaMemsetAsync(ctx->ee.p, 0, sizeof(double) * 2 * nb, s));
    double* d_eeT = ctx->ee.as<double>();
    double* d_eeR = d_eeT + nb;
    // transmission adjoint, one instance per source
    InstTables T;
    for (int b = 0; b < nb; ++b) {
        T.off.push_back((long long)(2 * b) * N);
        T.aux_off.push_back(((long long)b * slots) * N);
        T.mask_off.push_back((long long)(2 * b) * mwords);
        T.gsrc.push_back(b0 + b);
        T.ir.push_back(-1);
    }
    std::vector<int> caps(nb, maxswp), iters;
    if (do_t) PFAST_TRY2(adj_phase2(ctx, sv, LB, F, T, precision, caps, iters, d_eeT, st));
    // reflection adjoints, reflector by reflector; the iteration counter and the
    // receiver mask carry over between reflectors (src/RT_padjoint2d.h:385-466)
    std::vector<int> count(nb, 0);
    for (int ir = 0; do_r && ir < R; ++ir) {
        PFAST_CUDA_TRY(cudaMemsetAsync(LC, 0, sizeof(double) * N * nb, s));
        InstTables Rt;
        for (int b = 0; b < nb; ++b) {
            Rt.off.push_back((long long)b * N);
            Rt.aux_off.push_back(((long long)b * slots + 1 + R + ir) * N);
            Rt.mask_off.push_back((long long)(2 * b + 1) * mwords);
            Rt.gsrc.push_back(b0 + b);
            Rt.ir.push_back(ir);
            caps[b] = std::max(0, maxswp - count[b]);
        }
        // bc2 adds into d_eeR[b] (one running misfit sum over the reflectors of a source)
        PFAST_TRY2(adj_phase2(ctx, sv, LC, F, Rt, precision, caps, iters, d_eeR, st));
        for (int b = 0; b < nb; ++b) count[b] += iters[b] + 1;
        std::vector<long long> dof(nb), sof(nb);
        for (int b = 0; b < nb; ++b) { dof[b] = (long long)(2 * b + 1) * N; sof[b] = (long long)b * N; }
        InstTables add;
        add.off = dof;
        add.aux_off = sof;
        InstDev ad;
        PFAST_TRY2(upload_inst(ctx, ctx->misc, add, ad));
        PFAST_LAUNCH(ctx, launch_addto2(LB, ad.off, LC, ad.aux_off, N, nb, s));
    }
    PFAST_CUDA_TRY(cudaMemcpyAsync(ctx->h_ee.p, ctx->ee.p, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    std::memcpy(eeT, ctx->h_ee.as<double>(), sizeof(double) * nb);
    std::memcpy(eeR, ctx->h_ee.as<double>() + nb, sizeof(double) * nb);
    return PFAST_OK;
}

int pick_batch2(int nsrc, int max_batch, size_t per_src) {
    int b = nsrc;
    if (max_batch > 0) b = std::min(b, max_batch);
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) == cudaSuccess && per_src > 0) {
        size_t fit = (size_t)(0.8 * (double)fr) / per_src;
        b = (int)std::min<size_t>((size_t)b, std::max<size_t>(1, fit));
    }
    return std::max(1, std::min(b, 16384));
}

}  // namespace

pfast_status forward2d_impl(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const pfast_options* opt,
                            double* Tr, double* TTd_host, double* TTu_host, double* TT_host, pfast_stats* st) {
    pfast_options o;
    o.precision = PFAST_PLAIN_FP64;
    o.maxswp = 500;
    o.max_batch = 0;
    o.polish_floor = 0.0;
    o.schedule = PFAST_SCHEDULE_AUTO;
    o.near_source_radius = 0;
    o.tile_shape = PFAST_TILE_AUTO;
    if (opt) o = *opt;
    if (o.near_source_radius < 0 || o.near_source_radius > 64) {
        set_last_error("near_source_radius must be in [0, 64]");
        return PFAST_ERR_INVALID;
    }
    ctx->near_radius = o.near_source_radius;
    if (st) std::memset(st, 0, sizeof(*st));
    if (sv->geom_status) {
        set_last_error(sv->geom_status == PFAST_ERR_INVALID ? "survey has no reflector geometry"
                                                              : "no node above a reflector (reflector geometry)");
        return sv->geom_status;
    }
    PFAST_CUDA_TRY(cudaSetDevice(ctx->device));
    const int R = sv->numofr;
    const long long N = (long long)sv->nr * sv->nc;
    cudaStream_t s = ctx->stream;
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[6], s));
    const long long l0 = ctx->launches;
    PFAST_TRY2(prepare_slowness(ctx, vp, N, true));
    const size_t per_src = (size_t)N * 8 * (1 + 2 * R) + (size_t)N * 16 * (1 + R);
    const int B = pick_batch2(std::max(sv->nsrc, 1), (TTd_host || TT_host) ? 1 : o.max_batch, per_src);
    for (int b0 = 0; b0 < sv->nsrc; b0 += B) {
        const int nb = std::min(B, sv->nsrc - b0);
        if (st) ++st->batches;
        PFAST_TRY2(forward2d_batch(ctx, sv, b0, nb, o.precision, o.maxswp, ctx->s64.as<double>(), ctx->s32.as<float>(), st));
        if (Tr) {
            std::vector<long long> sfo(nb);
            for (int b = 0; b < nb; ++b) sfo[b] = (long long)b * (1 + 2 * R) * N;
            InstTables t;
            t.off = sfo;
            InstDev d;
            PFAST_TRY2(upload_inst(ctx, ctx->misc, t, d));
            PFAST_LAUNCH(ctx, launch_gather2(ctx->f2a.as<double>(), d.off, R, N, sv->d_rec, sv->d_ch0, sv->d_srnum, nb, b0,
                                      sv->nc, Tr, s));
        }
        if (TT_host) {   // single-source shim path (B == 1)
            const double* F = ctx->f2a.as<double>();
            PFAST_CUDA_TRY(cudaMemcpyAsync(TT_host, F, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
            if (R > 0) {
                PFAST_CUDA_TRY(cudaMemcpyAsync(TTd_host, F + N, sizeof(double) * N * R, cudaMemcpyDeviceToHost, s));
                PFAST_CUDA_TRY(cudaMemcpyAsync(TTu_host, F + N * (1 + R), sizeof(double) * N * R, cudaMemcpyDeviceToHost, s));
            }
        }
    }
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[7], s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    if (st) {
        add_elapsed(ctx->ev[6], ctx->ev[7], &st->ms_total);
        st->launches = ctx->launches - l0;
    }
    return PFAST_OK;
}

pfast_status eval2d_impl(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const double* WR,
                         const pfast_options* opt, double* gT, double* gR, double* gRT, double* Et, double* Er,
                         pfast_stats* st) {
    pfast_options o;
    o.precision = PFAST_PLAIN_FP64;
    o.maxswp = 500;
    o.max_batch = 0;
    o.polish_floor = 0.0;
    o.schedule = PFAST_SCHEDULE_AUTO;
    o.near_source_radius = 0;
    o.tile_shape = PFAST_TILE_AUTO;
    if (opt) o = *opt;
    if (o.near_source_radius < 0 || o.near_source_radius > 64) {
        set_last_error("near_source_radius must be in [0, 64]");
        return PFAST_ERR_INVALID;
    }
    ctx->near_radius = o.near_source_radius;
    if (st) std::memset(st, 0, sizeof(*st));
    if (!sv->has_picks) { set_last_error("survey has no picks: gradient unavailable"); return PFAST_ERR_INVALID; }
    if (sv->geom_status) { set_last_error("no node above a reflector (reflector geometry)"); return sv->geom_status; }
    PFAST_CUDA_TRY(cudaSetDevice(ctx->device));
    const int R = sv->numofr;
    const long long N = (long long)sv->nr * sv->nc;
    cudaStream_t s = ctx->stream;
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[6], s));
    const long long l0 = ctx->launches;
    PFAST_TRY2(prepare_slowness(ctx, vp, N, true));
    PFAST_CUDA_TRY(cudaMemsetAsync(gT, 0, sizeof(double) * N, s));
    PFAST_CUDA_TRY(cudaMemsetAsync(gR, 0, sizeof(double) * N, s));
    const size_t per_src = (size_t)N * 8 * (1 + 2 * R + 3) + (size_t)N * 16 * (1 + R);
    const int B = pick_batch2(std::max(sv->nsrc, 1), o.max_batch, per_src);
    double et = 0.0, er = 0.0;
    std::vector<double> eeT(B), eeR(B);
    for (int b0 = 0; b0 < sv->nsrc; b0 += B) {
        const int nb = std::min(B, sv->nsrc - b0);
        if (st) ++st->batches;
        PFAST_TRY2(forward2d_batch(ctx, sv, b0, nb, o.precision, o.maxswp, ctx->s64.as<double>(), ctx->s32.as<float>(), st));
        PFAST_TRY2(adjoint2d_batch(ctx, sv, b0, nb, o.precision, o.maxswp, eeT.data(), eeR.data(), st));
        for (int b = 0; b < nb; ++b) { et += eeT[b]; er += eeR[b]; }
        // gradients in source order: instance list (lamT_b, UR_b), b = 0..nb-1
        InstTables acc;
        std::vector<int> slot;
        for (int b = 0; b < nb; ++b) {
            acc.off.push_back((long long)(2 * b) * N);
            slot.push_back(0);
            acc.off.push_back((long long)(2 * b + 1) * N);
            slot.push_back(1);
        }
        acc.lim = slot;
        InstDev d;
        PFAST_TRY2(upload_inst(ctx, ctx->misc, acc, d));
        PFAST_LAUNCH(ctx, launch_accumulate2(gT, gR, ctx->f2b.as<double>(), d.off, d.lim, vp, N, 2 * nb, s));
    }
    PFAST_LAUNCH(ctx, launch_blend2(gT, gR, WR, gRT, N, s));
    PFAST_CUDA_TRY(cudaEventRecord(ctx->ev[7], s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    if (st) {
        add_elapsed(ctx->ev[6], ctx->ev[7], &st->ms_total);
        st->launches = ctx->launches - l0;
    }
    if (Et) *Et = et;
    if (Er) *Er = er;
    return PFAST_OK;
}

}  // namespace pfast

using namespace pfast;

namespace {

// Reflector geometry, evaluated on the host with the reference's comparisons
// (src/RT_pfsm2d.h:174, 195-281): per reflector ir and column j
//   lim_down[ir][j] = largest row i with (i+1)*dz <= Z, -1 if none
//   k2vec[ir][j]    = reflection row (nrows-1 when the reflector is below the model)
//   k2[ir][j]       = reflection row, or -1 where no reinitialisation happens
//   qxcase[ir][j]   = x-difference used at the reflection point
// Returns PFAST_ERR_NO_REFLECTION_POINT where the reference exits.
int reflector_tables(int nr, int nc, double dz, int R, const double* Z, std::vector<int>& tab) {
    tab.assign((size_t)4 * R * nc, -1);
    int* lim = tab.data();
    int* k2vec = lim + (size_t)R * nc;
    int* k2t = lim + 2 * (size_t)R * nc;
    int* qxc = lim + 3 * (size_t)R * nc;
    for (int ir = 0; ir < R; ++ir) {
        const double* Zr = Z + (size_t)ir * nc * 3;
        for (int j = 0; j < nc; ++j) {
            int m = -1;
            for (int i = 0; i < nr; ++i)
                if ((i + 1) * dz <= Zr[j * 3 + 0]) m = i;
            lim[(size_t)ir * nc + j] = m;
        }
        for (int jj = 0; jj < nc; ++jj) {
            const bool left = jj == 0, right = jj == nc - 1;
            const double zj = Zr[jj * 3];
            int k2 = -1;
            for (int kk = 0; kk < nr - 1; ++kk) {
                const bool here = (kk + 1) * dz + dz <= zj;
                bool side;
                if (left) side = kk * dz + dz <= Zr[(jj + 1) * 3];
                else if (right) side = kk * dz + dz <= Zr[(jj - 1) * 3];
                else side = kk * dz + dz <= Zr[(jj - 1) * 3] || kk * dz + dz <= Zr[(jj + 1) * 3];
                if (here && side && kk >= k2) k2 = kk;
            }
            const size_t at = (size_t)ir * nc + jj;
            if (zj <= nr * dz && k2 > 0) {
                k2vec[at] = k2;
                k2t[at] = k2;
                if (left) qxc[at] = 2;
                else if (right) qxc[at] = 1;
                else if (k2 * dz + dz <= Zr[(jj - 1) * 3] && k2 * dz + dz <= Zr[(jj + 1) * 3]) qxc[at] = 0;
                else if (k2 * dz + dz <= Zr[(jj - 1) * 3]) qxc[at] = 1;
                else qxc[at] = 2;
            } else if (zj > nr * dz) {
                k2vec[at] = nr - 1;
                k2t[at] = -1;
            } else {
                return PFAST_ERR_NO_REFLECTION_POINT;
            }
        }
    }
    return PFAST_OK;
}

}  // namespace

extern "C" {

pfast_status pfast_survey2d_create(pfast_ctx* ctx, int nrows, int ncols, double dx, double dz, int nsrc, const int* src,
                                   const int* srnum, int nrec, const int* rec, const double* nxy, const double* TT_obs,
                                   int NumofR, const double* TR_obs, const double* Z, pfast_survey2d** out) {
    if (!ctx || !out) { set_last_error("null context or output"); return PFAST_ERR_INVALID; }
    *out = nullptr;
    if (nrows < 2 || ncols < 2 || nrows > 65535 || ncols > 65535) {
        set_last_error("2D grid %dx%d: dimensions must be in [2, 65535]", nrows, ncols);
        return PFAST_ERR_INVALID;
    }
    if (!(dx > 0 && dz > 0)) { set_last_error("grid spacings must be positive"); return PFAST_ERR_INVALID; }
    if (NumofR < 0) { set_last_error("negative NumofR"); return PFAST_ERR_INVALID; }
    if (nsrc < 0 || (nsrc > 0 && (!src || !srnum))) { set_last_error("bad source arrays"); return PFAST_ERR_INVALID; }
    long long tot = 0;
    for (int s = 0; s < nsrc; ++s) {
        if (srnum[s] < 0) { set_last_error("srnum[%d] < 0", s); return PFAST_ERR_INVALID; }
        tot += srnum[s];
        if (src[2 * s] < 0 || src[2 * s] >= nrows || src[2 * s + 1] < 0 || src[2 * s + 1] >= ncols) {
            set_last_error("source %d at (%d,%d) outside the %dx%d grid", s, src[2 * s], src[2 * s + 1], nrows, ncols);
            return PFAST_ERR_INVALID;
        }
    }
    if (tot > nrec) { set_last_error("sum(srnum)=%lld exceeds nrec=%d", tot, nrec); return PFAST_ERR_INVALID; }
    if (nrec > 0 && !rec) { set_last_error("null receiver array"); return PFAST_ERR_INVALID; }
    for (int r = 0; r < nrec; ++r)
        if (rec[2 * r] < 0 || rec[2 * r] >= nrows || rec[2 * r + 1] < 0 || rec[2 * r + 1] >= ncols) {
            set_last_error("receiver row %d at (%d,%d) outside the grid", r, rec[2 * r], rec[2 * r + 1]);
            return PFAST_ERR_INVALID;
        }
    PFAST_CUDA_TRY(cudaSetDevice(ctx->device));
    pfast_survey2d* sv = new pfast_survey2d();
    sv->ctx = ctx;
    sv->nr = nrows;
    sv->nc = ncols;
    sv->dx = dx;
    sv->dz = dz;
    sv->nsrc = nsrc;
    sv->nrec = nrec;
    sv->numofr = NumofR;
    sv->h_src.assign(src, src + 2 * (size_t)nsrc);
    sv->h_srnum.assign(srnum, srnum + nsrc);
    sv->h_ch0.assign(nsrc + 1, 0);
    for (int s = 0; s < nsrc; ++s) sv->h_ch0[s + 1] = sv->h_ch0[s] + srnum[s];
    std::vector<int> tab;
    if (NumofR > 0 && Z) {
        sv->h_Z.assign(Z, Z + (size_t)NumofR * ncols * 3);
        sv->geom_status = reflector_tables(nrows, ncols, dz, NumofR, Z, tab);
    } else if (NumofR > 0) {
        sv->geom_status = PFAST_ERR_INVALID;   // adjoint-only survey: no reflector geometry for forward solves
    }
    if (tab.empty()) tab.assign(4, -1);
    // the sweeps read rowlim rows 0..2R-1 (down-going limits, then k2vec); reorder
    // [lim | k2vec | k2 | qx] already is that layout.
    sv->has_picks = nxy && TT_obs && (NumofR == 0 || TR_obs);
    std::vector<unsigned char> last_t(std::max(nrec, 1), 0), last_r(std::max<size_t>((size_t)nrec * NumofR, 1), 0);
    if (sv->has_picks) {
        std::vector<long long> keys;
        std::vector<size_t> used;
        auto node_of = [&](int r) { return (long long)rec[2 * r] * ncols + rec[2 * r + 1]; };
        for (int s = 0; s < nsrc; ++s) {
            mark_last_rows(sv->h_ch0[s], sv->h_ch0[s + 1], node_of, [&](int r) { return TT_obs[r] < 100; },
                           [&](int r) { last_t[r] = 1; }, keys, used);
            for (int ir = 0; ir < NumofR; ++ir)
                mark_last_rows(
                    sv->h_ch0[s], sv->h_ch0[s + 1], node_of, [&](int r) { return TR_obs[(size_t)r * NumofR + ir] != 0; },
                    [&](int r) { last_r[(size_t)r * NumofR + ir] = 1; }, keys, used);
        }
    }
    auto up = [&](void** dst, const void* h, size_t bytes) -> pfast_status {
        PFAST_CUDA_TRY(cudaMalloc(dst, std::max<size_t>(bytes, 16)));
        if (bytes && h) PFAST_CUDA_TRY(cudaMemcpy(*dst, h, bytes, cudaMemcpyHostToDevice));
        return PFAST_OK;
    };
    pfast_status r = PFAST_OK;
    if (!r) r = up((void**)&sv->d_src_ij, src, sizeof(int) * 2 * nsrc);
    if (!r) r = up((void**)&sv->d_ch0, sv->h_ch0.data(), sizeof(int) * (nsrc + 1));
    if (!r) r = up((void**)&sv->d_srnum, srnum, sizeof(int) * nsrc);
    if (!r) r = up((void**)&sv->d_rec, rec, sizeof(int) * 2 * (size_t)nrec);
    if (!r) r = up((void**)&sv->d_nxy, sv->has_picks ? nxy : nullptr, sv->has_picks ? sizeof(double) * 2 * nrec : 0);
    if (!r) r = up((void**)&sv->d_ttobs, sv->has_picks ? TT_obs : nullptr, sv->has_picks ? sizeof(double) * nrec : 0);
    if (!r) r = up((void**)&sv->d_trobs, (sv->has_picks && NumofR) ? TR_obs : nullptr,
                   (sv->has_picks && NumofR) ? sizeof(double) * nrec * NumofR : 0);
    if (!r) r = up((void**)&sv->d_last_t, last_t.data(), last_t.size());
    if (!r) r = up((void**)&sv->d_last_r, last_r.data(), last_r.size());
    if (!r) r = up((void**)&sv->d_Z, (NumofR && Z) ? Z : nullptr, (NumofR && Z) ? sizeof(double) * 3 * (size_t)NumofR * ncols : 0);
    if (!r) r = up((void**)&sv->d_k2vec, tab.data(), sizeof(int) * tab.size());
    if (r) { pfast_survey2d_destroy(sv); return r; }
    *out = sv;
    return PFAST_OK;
}

pfast_status pfast_survey2d_destroy(pfast_survey2d* sv) {
    if (!sv) return PFAST_OK;
    for (void* p : {(void*)sv->d_src_ij, (void*)sv->d_ch0, (void*)sv->d_srnum, (void*)sv->d_rec, (void*)sv->d_nxy,
                    (void*)sv->d_ttobs, (void*)sv->d_trobs, (void*)sv->d_last_t, (void*)sv->d_last_r, (void*)sv->d_Z,
                    (void*)sv->d_k2vec})
        if (p) cudaFree(p);
    delete sv;
    return PFAST_OK;
}

pfast_status pfast_survey2d_forward(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const pfast_options* opt,
                                    double* Tr, pfast_stats* stats) {
    if (!ctx || !sv || !vp || !Tr) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    return forward2d_impl(ctx, sv, vp, opt, Tr, nullptr, nullptr, nullptr, stats);
}

pfast_status pfast_survey2d_eval(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const double* WR,
                                 const pfast_options* opt, double* gT, double* gR, double* gRT, double* Et, double* Er,
                                 pfast_stats* stats) {
    if (!ctx || !sv || !vp || !WR || !gT || !gR || !gRT) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    return eval2d_impl(ctx, sv, vp, WR, opt, gT, gR, gRT, Et, Er, stats);
}

// ------------------------------------------------------------------ reference-signature shims


pfast_status pfast_RT_fsm2d(double* vp, double* U, double* TTd, double* TTu, double* Z, int* src, int* rec, int* srnum,
                            int srcid, int NumofR, int MAXSwp, double dx, double dz, int nrows, int ncols, int pe) {
    (void)rec; (void)srnum; (void)pe;
    if (!vp || !U || !src || srcid < 0 || (NumofR > 0 && (!TTd || !TTu || !Z))) {
        set_last_error("null argument or negative srcid");
        return PFAST_ERR_INVALID;
    }
    pfast_ctx* ctx = nullptr;
    PFAST_TRY2(default_context(&ctx));
    int zero = 0;
    pfast_survey2d* sv = nullptr;
    PFAST_TRY2(pfast_survey2d_create(ctx, nrows, ncols, dx, dz, 1, src + 2 * srcid, &zero, 0, nullptr, nullptr, nullptr,
                                     NumofR, nullptr, Z, &sv));
    const long long N = (long long)nrows * ncols;
    pfast_status r = ctx->vp_tmp.ensure(sizeof(double) * N);
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(ctx->vp_tmp.p, vp, sizeof(double) * N, cudaMemcpyHostToDevice, ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "copy vp", __FILE__, __LINE__);
    }
    pfast_options o;
    o.precision = PFAST_PLAIN_FP64;
    o.maxswp = MAXSwp;
    o.max_batch = 1;
    o.polish_floor = 0.0;
    o.schedule = PFAST_SCHEDULE_AUTO;
    o.near_source_radius = 0;
    o.tile_shape = PFAST_TILE_AUTO;
    if (!r) r = forward2d_impl(ctx, sv, ctx->vp_tmp.as<double>(), &o, nullptr, TTd, TTu, U, nullptr);
    pfast_survey2d_destroy(sv);
    return r;
}

// Shared body of the two 2D adjoint shims: one source, the given traveltime
// fields placed into the forward-field layout, then the batched adjoint.
static pfast_status adjoint2d_shim(bool trans, double* Lout, const double* T, const double* Tu, const double* obs,
                                   int* rec, double* nxy, int* src, int* srnum, int srcid, int NumofR, int MAXSwp,
                                   double dx, double dz, int nrows, int ncols, double* EE) {
    if (!Lout || !obs || !rec || !nxy || !src || !srnum || srcid < 0 || (trans && !T) || (!trans && NumofR > 0 && !Tu)) {
        set_last_error("null argument or negative srcid");
        return PFAST_ERR_INVALID;
    }
    pfast_ctx* ctx = nullptr;
    PFAST_TRY2(default_context(&ctx));
    long long ch0 = 0;
    for (int s = 0; s < srcid; ++s) ch0 += srnum[s];
    const int nrec = srnum[srcid];
    const int R = trans ? 0 : NumofR;
    std::vector<double> tt(std::max(nrec, 1), 100.0);   // no transmission picks for the reflection shim
    const double* ttobs = trans ? obs + ch0 : tt.data();
    const double* trobs = trans ? nullptr : obs + ch0 * NumofR;
    pfast_survey2d* sv = nullptr;
    PFAST_TRY2(pfast_survey2d_create(ctx, nrows, ncols, dx, dz, 1, src + 2 * srcid, srnum + srcid, nrec, rec + 2 * ch0,
                                     nxy + 2 * ch0, ttobs, R, trobs, nullptr, &sv));
    const long long N = (long long)nrows * ncols;
    cudaStream_t s = ctx->stream;
    pfast_status r = ctx->f2a.ensure(sizeof(double) * N * (1 + 2 * R));
    if (!r) {
        cudaError_t e = cudaSuccess;
        if (trans) e = cudaMemcpyAsync(ctx->f2a.p, T, sizeof(double) * N, cudaMemcpyHostToDevice, s);
        else if (R > 0)
            e = cudaMemcpyAsync(ctx->f2a.as<double>() + N * (1 + R), Tu, sizeof(double) * N * R, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) r = cuda_fail(e, "copy T", __FILE__, __LINE__);
    }
    double eeT = 0.0, eeR = 0.0;
    if (!r) r = adjoint2d_batch(ctx, sv, 0, 1, PFAST_PLAIN_FP64, MAXSwp, &eeT, &eeR, nullptr, trans, !trans);
    if (!r) {
        cudaError_t e = cudaMemcpyAsync(Lout, ctx->f2b.as<double>() + (trans ? 0 : N), sizeof(double) * N,
                                        cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = cuda_fail(e, "copy lambda", __FILE__, __LINE__);
    }
    if (!r && EE) *EE = trans ? eeT : eeR;
    pfast_survey2d_destroy(sv);
    return r;
}

pfast_status pfast_Tadjoint_fsm2d(double* U, double* T, double* T_obs, int* rec, double* nxyz, int* src, int* srnum,
                                  int srcid, int MAXSwp, double dx, double dz, int nrows, int ncols, int pe, double* EE) {
    (void)pe;
    return adjoint2d_shim(true, U, T, nullptr, T_obs, rec, nxyz, src, srnum, srcid, 0, MAXSwp, dx, dz, nrows, ncols, EE);
}

pfast_status pfast_Radjoint_fsm2d(double* UR, double* Td, double* Tu, double* TR_obs, int* rec, double* nxyz, int* src,
                                  int* srnum, int srcid, int NumofR, int MAXSwp, double dx, double dz, int nrows,
                                  int ncols, int pe, double* EE) {
    (void)pe;
    (void)Td;   // unused by the reference too
    return adjoint2d_shim(false, UR, nullptr, Tu, TR_obs, rec, nxyz, src, srnum, srcid, NumofR, MAXSwp, dx, dz, nrows,
                          ncols, EE);
}

}  // extern "C"

// ------------------------------------------------------------------ host-buffer forms
namespace {

struct HostDev2 {
    pfast_ctx* ctx;
    std::vector<void*> ptrs;
    ~HostDev2() {
        for (void* p : ptrs) cudaFree(p);
    }
    pfast_status up(double** d, const double* h, size_t n) {
        void* p = nullptr;
        PFAST_CUDA_TRY(cudaMalloc(&p, sizeof(double) * std::max<size_t>(n, 1)));
        ptrs.push_back(p);
        if (h) PFAST_CUDA_TRY(cudaMemcpyAsync(p, h, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        *d = static_cast<double*>(p);
        return PFAST_OK;
    }
};

pfast_status down(pfast_ctx* ctx, double* h, const double* d, size_t n) {
    PFAST_CUDA_TRY(cudaMemcpyAsync(h, d, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    return PFAST_OK;
}

}  // namespace

extern "C" {

pfast_status pfast_forward2d(pfast_ctx* ctx, const double* vp, int nrows, int ncols, double dx, double dz, int nsrc,
                             const int* src, const int* srnum, int nrec, const int* rec, int NumofR, const double* Z,
                             const pfast_options* opt, double* Tr, pfast_stats* stats) {
    if (!ctx || !vp || !Tr) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    pfast_survey2d* sv = nullptr;
    PFAST_TRY2(pfast_survey2d_create(ctx, nrows, ncols, dx, dz, nsrc, src, srnum, nrec, rec, nullptr, nullptr, NumofR,
                                     nullptr, Z, &sv));
    const size_t N = (size_t)nrows * ncols;
    HostDev2 hd{ctx, {}};
    double *d_vp = nullptr, *d_tr = nullptr;
    pfast_status r = hd.up(&d_vp, vp, N);
    if (!r) r = hd.up(&d_tr, nullptr, (size_t)std::max(nrec, 1) * (NumofR + 1));
    if (!r) r = pfast_survey2d_forward(ctx, sv, d_vp, opt, d_tr, stats);
    if (!r && nrec > 0) r = down(ctx, Tr, d_tr, (size_t)nrec * (NumofR + 1));
    if (!r) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "synchronize", __FILE__, __LINE__);
    }
    pfast_survey2d_destroy(sv);
    return r;
}

pfast_status pfast_eval2d(pfast_ctx* ctx, const double* vp, const double* WR, int nrows, int ncols, double dx,
                          double dz, int nsrc, const int* src, const int* srnum, int nrec, const int* rec,
                          const double* nxy, const double* TT_obs, int NumofR, const double* TR_obs, const double* Z,
                          const pfast_options* opt, double* gT, double* gR, double* gRT, double* Et, double* Er,
                          pfast_stats* stats) {
    if (!ctx || !vp || !WR || !gT || !gR || !gRT || !nxy || !TT_obs) {
        set_last_error("null argument");
        return PFAST_ERR_INVALID;
    }
    pfast_survey2d* sv = nullptr;
    PFAST_TRY2(pfast_survey2d_create(ctx, nrows, ncols, dx, dz, nsrc, src, srnum, nrec, rec, nxy, TT_obs, NumofR,
                                     TR_obs, Z, &sv));
    const size_t N = (size_t)nrows * ncols;
    HostDev2 hd{ctx, {}};
    double *d_vp = nullptr, *d_wr = nullptr, *d_gt = nullptr, *d_gr = nullptr, *d_grt = nullptr;
    pfast_status r = hd.up(&d_vp, vp, N);
    if (!r) r = hd.up(&d_wr, WR, N);
    if (!r) r = hd.up(&d_gt, nullptr, N);
    if (!r) r = hd.up(&d_gr, nullptr, N);
    if (!r) r = hd.up(&d_grt, nullptr, N);
    if (!r) r = pfast_survey2d_eval(ctx, sv, d_vp, d_wr, opt, d_gt, d_gr, d_grt, Et, Er, stats);
    if (!r) r = down(ctx, gT, d_gt, N);
    if (!r) r = down(ctx, gR, d_gr, N);
    if (!r) r = down(ctx, gRT, d_grt, N);
    if (!r) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) r = cuda_fail(e, "synchronize", __FILE__, __LINE__);
    }
    pfast_survey2d_destroy(sv);
    return r;
}

}  // extern "C"
