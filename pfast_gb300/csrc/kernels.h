// kernels.h -- host-side launchers of the pfast_gb300 CUDA kernels (internal).
#pragma once

#include <vector>
#include "common.cuh"

namespace pfast {

// ------------------------------------------------------------------ 3D sweeps
// Arguments of one tile-diagonal launch of a 3D sweep.  A "batch" holds
// `nbatch` instances (sources) whose fields lie at field + inst*fstride.
struct Sweep3Args {
    void* field;              // Real fields, per instance
    long long fstride;        // elements between instances (same for snap / aux / T)
    const void* aux;          // plain forward: slowness 1/vp (double); FP32 forward: slowness (float);
                              // polish forward: slowness squared, times h^2 on isotropic grids (double); adjoint: T per instance
                              // (double, or float for the FP32 adjoint)
    const double* slow64;     // polish forward: slowness (double), for the restart branch
    const unsigned* mask;     // adjoint: fixed-node bits, per instance, mask_stride words apart
    long long mask_stride;
    int wpr;                  // mask words per grid row
    const int* src_kij;       // forward: per-instance source node (k, i, j)
    int src_r2;               // forward: nodes with squared node distance <= src_r2 from the source are
                              // fixed (0: the source node only, the reference's point source)
    void* snap;               // per-instance snapshot of the iteration start (Real)
    int* changed;             // per-instance "an update exceeded the tolerance" flag
    const int* act;           // active instance ids; grid.y indexes it
    const int* diag_off;      // tile-diagonal table: tiles of diagonal d are
    const unsigned* diag_tiles;  //   diag_tiles[diag_off[d] .. diag_off[d+1])
    int nz, nr, nc;
    int nbk, nbi, nbj;
    Spacing3 sp;
    int dir;                  // sweep order 0..7: bit2 = s3>0 (z), bit1 = s1>0 (rows), bit0 = s2>0 (cols)
    int iter;                 // outer-iteration index (snapshot stamps)
    int ntiles;               // tiles per instance (nbk*nbi*nbj)
    int* dirty;               // per (instance, tile): sweep orders still to process (see sweep3d_kernel)
    int* stamp;               // per (instance, tile): iteration of the tile's snapshot
    int* diff;                // per (instance, tile): differs from its snapshot by > tol
    double tol_abs, tol_rel;  // change test: |new-old| > tol_abs + tol_rel*|new| (FP64 sweeps)
    float tol_abs_f, tol_rel_f;  // the same test for the FP32 sweeps, evaluated in FP32
    float polish_floor;       // polish sweeps: corrections at or below this are dropped (seconds;
                              // adjoint: relative to 1 + |lambda|)
    unsigned long long* work; // per instance: nodes of the tiles processed (executed node updates); may be null
    int shape;                // tile shape: 0 = 4x8x32, 1 = 8x4x32 (common.cuh: TileShape)
    int vec_rows;             // rows of the field (and of the FP32 adjoint's traveltime) start on 16-byte
                              // boundaries: nc a multiple of 16 / element size, 16-byte aligned fields;
                              // tiles then move in 16-byte vectors
    const int* dyn;           // per-diagonal launches of a replayed iteration graph: dyn[0] = outer
                              // iteration (instead of iter), dyn[1] = active instances (blocks with
                              // blockIdx.y >= dyn[1] exit); null: iter and the grid
};

// Tile-diagonal table for a grid: tiles (bk, bi, bj) in flipped coordinates with
// bk+bi+bj = d, packed bk | bi<<10 | bj<<20.
struct DiagTable3 {
    int shape = 0;
    int nbk = 0, nbi = 0, nbj = 0, ndiag = 0;
    std::vector<int> h_off;
    int* d_off = nullptr;
    unsigned* d_tiles = nullptr;
};

pfast_status build_diag_table3(int nz, int nr, int nc, int shape, DiagTable3& t);
void free_diag_table3(DiagTable3& t);

// changed[act[b]], b < nact: bit 0 = any diff over the tiles of instance act[b]; bit 1 = some
// tile still due in some order (lock words `dirty`: order bits order_mask, selected orders
// `shift` bits higher for the selective polish kinds).
pfast_status launch_reduce_diff(const int* diff, const int* dirty, bool selective, int shift, int order_mask,
                                int ntiles, const int* act, int nact, int* changed, cudaStream_t st,
                                const int* dyn = nullptr);
// Polish kinds: the tile's initially selected orders in bits 8-15 of its lock word (bits 0-7
// kept: all orders due, or as seeded), computed from a.field (forward) or a.aux (adjoint) for
// the active instances a.act[0..nact).
pfast_status launch_polish_orders3(int kind, const Sweep3Args& a, int nb, int nact, cudaStream_t st);
// Initial lock words from the starting field (a.field, active instances a.act[0..nact)): 0xff
// where the tile's halo box holds a reached traveltime / nonzero lambda, else 0.  Every kind but
// the forward polish (whose starting field is reached everywhere): no-op for that one.
pfast_status launch_seed_tiles3(int kind, const Sweep3Args& a, int nact, cudaStream_t st);
// One tile-diagonal launch over grid (tiles, nact): a.act must hold at least nact entries
// (every block reads a.act[blockIdx.y] before it tests whether its instance is still active).
pfast_status launch_sweep3(int kind, const Sweep3Args& a, int d0, int tiles, int nact, cudaStream_t st);
// Dataflow sweep kernel (one launch per phase): `blocks` blocks of `warps` warps take the
// nact instances of a.act from queue[0] (zeroed by the caller) and solve each to convergence
// (maxiter outer iterations at most); result[inst] = iterations | 1<<30 if not converged
// (| 1<<29 and queue[1] |= 1 if a block stalled: an internal error).  a.dirty, a.diff,
// a.stamp as for the per-diagonal launches; a.ntiles <= kDataflowMaxTiles.
pfast_status launch_sweep3_dataflow(int kind, const Sweep3Args& a, int nact, int maxiter, int* queue, int* result,
                                    int warps, int blocks, cudaStream_t st);
// The dataflow kernel over instances of several grids: item q is instance items[q].y of the grid
// whose arguments are models[items[q].x] (a device array; each model's result goes to its own
// `changed` array); max_ntiles: the largest grid's tile count (<= kDataflowMaxTiles); warps and
// blocks from dataflow_shape(kind, shape, max_ntiles, nitems, warps, blocks, true).
pfast_status launch_sweep3_dataflow_multi(int kind, int shape, const Sweep3Args* models, const int2* items, int nitems,
                                          int max_ntiles, int maxiter, int* queue, int warps, int blocks,
                                          cudaStream_t st);
// Warps per block (as many as shared memory holds) and resident blocks
// of the dataflow kernel; *warps = 0 when a grid of ntiles tiles does not fit.
pfast_status dataflow_shape(int kind, int shape, int ntiles, int nact, int* warps, int* blocks, bool multi = false);

// The sweep launchers of one tile shape (kernels3d_tiles.cuh; instantiated for Shape48 in
// kernels3d.cu and for Shape84 in kernels3d_s84.cu); the functions above dispatch to them.
template <class SH>
struct ShapeLaunchers {
    static pfast_status sweep(int kind, const Sweep3Args& a, int d0, int tiles, int nact, cudaStream_t st);
    static pfast_status dataflow(int kind, const Sweep3Args& a, int nact, int maxiter, int* queue, int* result,
                                 int warps, int blocks, cudaStream_t st);
    static pfast_status dataflow_multi(int kind, const Sweep3Args* models, const int2* items, int nitems,
                                       int max_ntiles, int maxiter, int* queue, int warps, int blocks, cudaStream_t st);
    static pfast_status dataflow_shape(int kind, int ntiles, int nact, bool multi, int* warps, int* blocks);
    static pfast_status seed(int kind, const Sweep3Args& a, int nact, cudaStream_t st);
    static pfast_status orders(int kind, const Sweep3Args& a, int nact, cudaStream_t st);
};
extern template struct ShapeLaunchers<Shape48>;
extern template struct ShapeLaunchers<Shape84>;

// Small 3D kernels.
// s64 = 1.0/vp, s32 = (float)s64 (if non-null), sq64 = s64*s64*sq_scale (if non-null); *bad is set
// when some vp is not a positive finite number.
pfast_status launch_slowness(const double* vp, double* s64, float* s32, double* sq64, double sq_scale, int* bad, long long n,
                             cudaStream_t st);
// Opt-in near-source start: nodes within `radius` nodes (Euclidean) of each instance's source get
// 0.5*(s_src + s_node)*distance.  field: FP32 (is_fp32) or FP64 fields, fstride apart.
pfast_status launch_near_source3(void* field, int is_fp32, long long fstride, const int* src_kij, const double* s64,
                                 int nz, int nr, int nc, const Spacing3& sp, int radius, int nb, cudaStream_t st);
pfast_status launch_init_fwd3(void* field, int is_fp32, long long fstride, long long n, const long long* src_lin,
                              int nbatch, cudaStream_t st);
pfast_status launch_widen(const float* src, double* dst, long long fstride32, long long fstride64, long long n,
                          int nbatch, cudaStream_t st);
// lam64 <- lam32 for non-fixed nodes (fixed nodes keep their FP64 boundary value).
pfast_status launch_widen_lambda(const float* l32, double* l64, const unsigned* mask, long long fstride32,
                                 long long fstride64, long long mask_stride, int nz, int nr, int nc, int wpr,
                                 int nbatch, cudaStream_t st);
pfast_status launch_narrow(const double* src, float* dst, long long fstride64, long long fstride32, long long n,
                           int nbatch, cudaStream_t st);

// Receiver boundary condition + misfit (src/T_padjoint3d.h:90-127) for a batch of
// sources.  rows of batch source b: [ch0[b], ch0[b]+srnum[b]); `last` marks the last
// picked row at its node (earlier rows at the same node are overwritten by it in the
// reference's sequential loop).
struct Bc3Args {
    const double* T; double* L; long long fstride;
    unsigned* mask; long long mask_stride; int wpr;
    const int* rec; const double* nxyz; const double* tobs; const unsigned char* last;
    const int* ch0; const int* srnum; const int* src_kij;   // per batch source
    double* EE; int* need;                                   // per batch source
    int nz, nr, nc; double dx, dy, dz;
};
pfast_status launch_bc3(const Bc3Args& a, int nbatch, cudaStream_t st);

// exact: grad[n] <- grad[n] - lam_b[n] / (v*v*v), b = 0..nbatch-1 in order (src/T_PFAST3D.cpp:393);
// otherwise grad[n] <- grad[n] + lam_b[n] in order (running sum, finished by launch_finish_gradient).
pfast_status launch_accumulate(double* grad, const double* lam, long long fstride, const double* vp, long long n,
                               int nbatch, bool exact, cudaStream_t st);
// g = -g / v^3: the mixed-precision path's single division after its running lambda sum.
pfast_status launch_finish_gradient(double* grad, const double* vp, long long n, cudaStream_t st);
// picks[row] = T_b[rec[row]] for rows of each batch source.
pfast_status launch_gather3(const double* T, long long fstride, const int* rec, const int* ch0, const int* srnum,
                            int nbatch, int nz, int nr, int nc, double* picks, cudaStream_t st);

}  // namespace pfast
