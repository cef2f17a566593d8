// engine.h -- host-side runtime of pfast_gb300 (internal): context, device
// buffers, surveys and the sweep driver.
#pragma once

#include <map>
#include <tuple>
#include <vector>
#include <string>

#include "kernels.h"
#include "kernels2d.h"

namespace pfast {

// Grow-only device buffer.  With `astream` set (contexts of the request server) the buffer
// is allocated and freed stream-ordered on that stream, so growing or releasing it never
// synchronises the device (other slots' work keeps running).
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaStream_t astream = nullptr;
    pfast_status ensure(size_t bytes);
    void release();
    template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

// Pinned host scratch for per-iteration flags and lists.  With `sstream` set, growing waits
// for that stream only (its context's copies) instead of the whole device.
struct HostBuf {
    void* p = nullptr;
    size_t cap = 0;
    cudaStream_t sstream = nullptr;
    pfast_status ensure(size_t bytes);
    void release();
    template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

struct PhaseTimer {
    cudaEvent_t a = nullptr, b = nullptr;
};

}  // namespace pfast

struct pfast_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // device work buffers (reused across calls)
    pfast::DevBuf s64, s32, sq64, T32, tflags, T64, L64, scratch, mask, act, changed, ee, need, misc, grad_tmp, vp_tmp, picks_tmp;
    pfast::DevBuf f2a, f2b, f2c;       // 2D field buffers
    pfast::HostBuf h_act, h_changed, h_ee, h_need, h_work;
    pfast::DevBuf work;                 // executed node updates per instance (sweep kernels)
    pfast::DevBuf queue;                // work counter of the persistent sweep kernel
    pfast::DevBuf out_a, out_b, out_c;  // request server: device outputs of a request
    pfast::DevBuf dyn;                  // replayed iteration graphs: outer iteration, active instances
    pfast::DevBuf multi;                // multi-model evaluations: the models' work arrays
    pfast::DevBuf multi_meta;           // multi-model evaluations: argument table and instance list
    // the one-call host entries' survey arrays (source tables, receiver rows, picks), reused
    pfast::DevBuf sv_src, sv_rec, sv_nxyz, sv_tobs, sv_last;
    pfast::HostBuf h_dyn;
    // One outer iteration of a per-diagonal phase as an instantiated CUDA graph, keyed by the
    // sweep kind, the launch arguments and the active-instance count it was captured with.
    std::vector<std::pair<std::vector<unsigned char>, cudaGraphExec_t>> iter_graphs;
    // executed node updates per batch instance of the latest 3D phase, and of the latest phase
    // of each sweep kind: the dataflow kernel takes the instances heaviest first by the same
    // kind's last figures (else the previous phase's), a longest-processing-time order
    std::vector<unsigned long long> inst_work;
    std::vector<unsigned long long> inst_work_kind[6];
    // keys seen once: a phase is captured the second time its key comes up, so one-off shapes
    // (uneven batches, a serving mix) do not pay for a graph they never replay
    std::vector<std::vector<unsigned char>> graph_seen;
    bool graphs = true;                 // replay per-diagonal outer iterations as CUDA graphs
    std::map<std::tuple<int, int, int, int>, pfast::DiagTable3> diag3;   // (nz, nr, nc, tile shape)
    std::map<std::pair<int, int>, pfast::DiagTable2> diag2;
    cudaEvent_t ev[8] = {};
    long long launches = 0;
    float polish_floor = pfast::kPolishFloor;   // of the current 3D evaluation (pfast_options)
    int schedule = PFAST_SCHEDULE_AUTO;         // of the current 3D evaluation (pfast_options)
    int tile_shape = PFAST_TILE_AUTO;           // of the current 3D evaluation (pfast_options)
    int candidates = 0;                         // per sweep kind: 1 + candidate of its last phase (pfast_stats)
    int near_radius = 0;                        // of the current 3D evaluation (pfast_options)
    bool tuning = false;                        // record phase times for the schedule autotuner
};

struct pfast_survey3d {
    pfast_ctx* ctx = nullptr;
    int nz = 0, nr = 0, nc = 0;
    double dx = 0, dy = 0, dz = 0;
    int nsrc = 0, nrec = 0;
    std::vector<int> h_src, h_srnum, h_ch0;
    int* d_src_kij = nullptr;        // per source (k, i, j)
    long long* d_src_lin = nullptr;  // per source linear node index
    int* d_ch0 = nullptr;
    int* d_srnum = nullptr;
    int* d_rec = nullptr;
    double* d_nxyz = nullptr;
    double* d_tobs = nullptr;
    unsigned char* d_last = nullptr;
    bool has_picks = false;
    bool borrowed = false;           // device arrays are the context's scratch (one-call entries)
};

struct pfast_survey2d {
    pfast_ctx* ctx = nullptr;
    int nr = 0, nc = 0;
    double dx = 0, dz = 0;
    int nsrc = 0, nrec = 0, numofr = 0;
    std::vector<int> h_src, h_srnum, h_ch0;
    std::vector<int> h_k2vec;         // [numofr][nc]: row of the last node above each reflector
    std::vector<double> h_Z;
    int* d_src_ij = nullptr;
    int* d_ch0 = nullptr;
    int* d_srnum = nullptr;
    int* d_rec = nullptr;
    double* d_nxy = nullptr;
    double* d_ttobs = nullptr;
    double* d_trobs = nullptr;
    unsigned char* d_last_t = nullptr;   // last transmission-picked row at its node
    unsigned char* d_last_r = nullptr;   // [nrec*numofr] last reflection-picked row at its node
    double* d_Z = nullptr;
    int* d_k2vec = nullptr;
    bool has_picks = false;
    int geom_status = 0;             // PFAST_ERR_NO_REFLECTION_POINT if a reflector has no node above it
};

// Launch a kernel through one of the launch_* helpers and count it in ctx->launches.
#define PFAST_LAUNCH(ctx, expr)                \
    do {                                        \
        pfast_status s__ = (expr);              \
        if (s__ != PFAST_OK) return s__;        \
        ++(ctx)->launches;                      \
    } while (0)

namespace pfast {

// Marks the last row of every node within one source's block of receiver rows [r0, r1):
// the reference's loops write the receivers in row order, so a node picked twice keeps its
// later row.  node_of(r) -> node index (>= 0), picked(r) -> whether row r is picked,
// mark(r) records the row.  A flat open-addressing table (keys, reused across blocks and
// cleared only where it was written) instead of one hash-set allocation per node.
template <class NodeOf, class Picked, class Mark>
void mark_last_rows(int r0, int r1, NodeOf node_of, Picked picked, Mark mark, std::vector<long long>& keys,
                    std::vector<size_t>& used) {
    int bits = 4;
    while ((1ll << bits) < 2ll * (r1 - r0)) ++bits;
    const size_t cap = (size_t)1 << bits;
    if (keys.size() < cap) keys.assign(cap, -1);
    used.clear();
    for (int r = r1 - 1; r >= r0; --r) {
        if (!picked(r)) continue;
        const long long node = node_of(r);
        size_t h = (size_t)(((unsigned long long)node * 0x9E3779B97F4A7C15ull) >> (64 - bits));
        while (keys[h] != -1 && keys[h] != node) h = (h + 1) & (cap - 1);
        if (keys[h] == -1) {
            keys[h] = node;
            used.push_back(h);
            mark(r);
        }
    }
    for (size_t h : used) keys[h] = -1;
}

pfast_status ctx_diag3(pfast_ctx* ctx, int nz, int nr, int nc, int shape, DiagTable3** out);
pfast_status ctx_diag2(pfast_ctx* ctx, int nr, int nc, DiagTable2** out);

// The process-wide context of the calling thread's current device (reference shims).
pfast_status default_context(pfast_ctx** out);

// Slowness arrays of a model (s64 always; s32 and s^2 * sq_scale for the mixed mode); rejects a
// model with a non-positive or non-finite velocity.
pfast_status prepare_slowness(pfast_ctx* ctx, const double* vp, long long N, bool mixed, double sq_scale = 1.0);

// Every device buffer of a context; release them all (stream-ordered for server contexts);
// make a context's buffers stream-ordered on its own stream (request server slots).
std::vector<DevBuf*> ctx_buffers(pfast_ctx* ctx);
void ctx_release_buffers(pfast_ctx* ctx);
void ctx_stream_ordered(pfast_ctx* ctx);

// Time between two recorded events, added to *acc (ms).
void add_elapsed(cudaEvent_t a, cudaEvent_t b, double* acc);

// Forward solve for sources [b0, b0+nb) of a 3D survey into ctx->T64 (FP64).
pfast_status forward3d_batch(pfast_ctx* ctx, const pfast_survey3d* sv, int b0, int nb, int precision, int maxswp,
                             pfast_stats* st);
// Adjoint for the same batch (T in ctx->T64): lambda into ctx->L64, EE per source into ee_out.
pfast_status adjoint3d_batch(pfast_ctx* ctx, const pfast_survey3d* sv, int b0, int nb, int precision, int maxswp,
                             double* ee_out, pfast_stats* st);

// FP32 bulk phases stop once no node moves by more than ~8 ulps (relative; the adjoint also
// 1e-6 absolute); FP64 phases use the reference's absolute 1e-9.
constexpr double kTol32Rel = 1.0 / (1 << 20);
constexpr double kTol32AbsAdj = 1e-6;
// Sweep arguments common to every phase of a survey's evaluation (grid, spacing, floor).
Sweep3Args survey_sweep_args(const pfast_survey3d* sv);
// Whether a phase's tiles can move in 16-byte vectors (Sweep3Args::vec_rows).
int rows_aligned(const Sweep3Args& a, int kind);
bool valid_options(const pfast_options* opt);
pfast_options resolve_options(const pfast_options* opt, int default_maxswp);
void stats_begin(pfast_stats* st);

// 2D pipelines (engine2d.cu).
pfast_status forward2d_impl(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const pfast_options* opt,
                            double* Tr, double* TTd_host, double* TTu_host, double* TT_host, pfast_stats* st);
pfast_status eval2d_impl(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const double* WR,
                         const pfast_options* opt, double* gT, double* gR, double* gRT, double* Et, double* Er,
                         pfast_stats* st);

}  // namespace pfast
