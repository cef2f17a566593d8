// kernels3d.cu -- 3D fast-sweeping Eikonal and adjoint-state kernels for sm_103a: the sweep
// kernels of tile shape 4x8x32 (kernels3d_tiles.cuh; shape 8x4x32 in kernels3d_s84.cu), the
// launch dispatch by tile shape, the tile-diagonal tables, and the small per-node kernels.

#include "kernels3d_tiles.cuh"

namespace pfast {

template struct ShapeLaunchers<Shape48>;

namespace {

// changed[act[b]] bit 0 = OR over the tiles of instance act[b] of diff; bit 1 = some tile
// is still due in some order (its lock word: the order bits `order_mask`; selective kinds
// hold the selected orders `shift` bits higher, and an order counts when due and selected).
__global__ void reduce_diff_kernel(const int* __restrict__ diff, const int* __restrict__ dirty, int selective,
                                   int shift, int order_mask, int ntiles, const int* __restrict__ act,
                                   int* __restrict__ changed, const int* __restrict__ dyn) {
    if (dyn && (int)blockIdx.x >= __ldcg(dyn + 1)) return;   // replayed graph: beyond the active count
    const int inst = act[blockIdx.x];
    const int* d = diff + (long long)inst * ntiles;
    const int* w = dirty + (long long)inst * ntiles;
    int any = 0, due = 0;
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) {
        any |= d[t];
        const int dm = w[t];
        due |= (selective ? (dm & (dm >> shift)) : dm) & order_mask;
    }
    any = __syncthreads_or(any);
    due = __syncthreads_or(due);
    if (threadIdx.x == 0) changed[inst] = (any ? 1 : 0) | (due ? 2 : 0);
}

}  // namespace

// ------------------------------------------------------------------ tables
pfast_status build_diag_table3(int nz, int nr, int nc, int shape, DiagTable3& t) {
    if (shape < 0 || shape >= kTileShapes) {
        set_last_error("unknown tile shape %d", shape);
        return PFAST_ERR_INVALID;
    }
    const int tk = shape_tk(shape), ti = shape_ti(shape);
    t.shape = shape;
    t.nbk = (nz + tk - 1) / tk;
    t.nbi = (nr + ti - 1) / ti;
    t.nbj = (nc + TJ - 1) / TJ;
    if (t.nbk > 1023 || t.nbi > 1023 || t.nbj > 1023) {
        set_last_error("grid %dx%dx%d too large for the tile table", nz, nr, nc);
        return PFAST_ERR_INVALID;
    }
    t.ndiag = t.nbk + t.nbi + t.nbj - 2;
    std::vector<unsigned> tiles;
    t.h_off.assign(t.ndiag + 1, 0);
    for (int dd = 0; dd < t.ndiag; ++dd) {
        t.h_off[dd] = (int)tiles.size();
        for (int bk = 0; bk < t.nbk; ++bk)
            for (int bi = 0; bi < t.nbi; ++bi) {
                const int bj = dd - bk - bi;
                if (bj >= 0 && bj < t.nbj) tiles.push_back((unsigned)bk | ((unsigned)bi << 10) | ((unsigned)bj << 20));
            }
    }
    t.h_off[t.ndiag] = (int)tiles.size();
    PFAST_CUDA_TRY(cudaMalloc(&t.d_off, sizeof(int) * t.h_off.size()));
    PFAST_CUDA_TRY(cudaMalloc(&t.d_tiles, sizeof(unsigned) * tiles.size()));
    PFAST_CUDA_TRY(cudaMemcpy(t.d_off, t.h_off.data(), sizeof(int) * t.h_off.size(), cudaMemcpyHostToDevice));
    PFAST_CUDA_TRY(cudaMemcpy(t.d_tiles, tiles.data(), sizeof(unsigned) * tiles.size(), cudaMemcpyHostToDevice));
    return PFAST_OK;
}

void free_diag_table3(DiagTable3& t) {
    if (t.d_off) cudaFree(t.d_off);
    if (t.d_tiles) cudaFree(t.d_tiles);
    t.d_off = nullptr;
    t.d_tiles = nullptr;
}

// ------------------------------------------------------------------ dispatch by tile shape
static bool known_shape(int shape) {
    if (shape >= 0 && shape < kTileShapes) return true;
    set_last_error("unknown tile shape %d", shape);
    return false;
}

pfast_status launch_sweep3(int kind, const Sweep3Args& a, int d0, int tiles, int nact, cudaStream_t st) {
    if (tiles <= 0 || nact <= 0) return PFAST_OK;
    if (!known_shape(a.shape)) return PFAST_ERR_INVALID;
    return a.shape ? ShapeLaunchers<Shape84>::sweep(kind, a, d0, tiles, nact, st)
                   : ShapeLaunchers<Shape48>::sweep(kind, a, d0, tiles, nact, st);
}

pfast_status launch_sweep3_dataflow(int kind, const Sweep3Args& a, int nact, int maxiter, int* queue, int* result,
                                    int warps, int blocks, cudaStream_t st) {
    if (nact <= 0 || maxiter <= 0) return PFAST_OK;
    if (warps < 1 || warps > 32 || blocks < 1 || a.ntiles > kDataflowMaxTiles) {
        set_last_error("dataflow sweep: bad shape (%d warps, %d blocks, %d tiles)", warps, blocks, a.ntiles);
        return PFAST_ERR_INVALID;
    }
    if (!known_shape(a.shape)) return PFAST_ERR_INVALID;
    return a.shape ? ShapeLaunchers<Shape84>::dataflow(kind, a, nact, maxiter, queue, result, warps, blocks, st)
                   : ShapeLaunchers<Shape48>::dataflow(kind, a, nact, maxiter, queue, result, warps, blocks, st);
}

pfast_status launch_sweep3_dataflow_multi(int kind, int shape, const Sweep3Args* models, const int2* items, int nitems,
                                          int max_ntiles, int maxiter, int* queue, int warps, int blocks,
                                          cudaStream_t st) {
    if (nitems <= 0 || maxiter <= 0) return PFAST_OK;
    if (warps < 1 || warps > 32 || blocks < 1 || max_ntiles > kDataflowMaxTiles) {
        set_last_error("dataflow sweep: bad shape (%d warps, %d blocks, %d tiles)", warps, blocks, max_ntiles);
        return PFAST_ERR_INVALID;
    }
    if (!known_shape(shape)) return PFAST_ERR_INVALID;
    return shape ? ShapeLaunchers<Shape84>::dataflow_multi(kind, models, items, nitems, max_ntiles, maxiter, queue, warps,
                                                           blocks, st)
                 : ShapeLaunchers<Shape48>::dataflow_multi(kind, models, items, nitems, max_ntiles, maxiter, queue, warps,
                                                           blocks, st);
}

pfast_status dataflow_shape(int kind, int shape, int ntiles, int nact, int* warps, int* blocks, bool multi) {
    if (!known_shape(shape)) return PFAST_ERR_INVALID;
    return shape ? ShapeLaunchers<Shape84>::dataflow_shape(kind, ntiles, nact, multi, warps, blocks)
                 : ShapeLaunchers<Shape48>::dataflow_shape(kind, ntiles, nact, multi, warps, blocks);
}

pfast_status launch_seed_tiles3(int kind, const Sweep3Args& a, int nact, cudaStream_t st) {
    if (!known_shape(a.shape)) return PFAST_ERR_INVALID;
    return a.shape ? ShapeLaunchers<Shape84>::seed(kind, a, nact, st) : ShapeLaunchers<Shape48>::seed(kind, a, nact, st);
}

pfast_status launch_polish_orders3(int kind, const Sweep3Args& a, int nb, int nact, cudaStream_t st) {
    (void)nb;
    if (!known_shape(a.shape)) return PFAST_ERR_INVALID;
    return a.shape ? ShapeLaunchers<Shape84>::orders(kind, a, nact, st)
                   : ShapeLaunchers<Shape48>::orders(kind, a, nact, st);
}

pfast_status launch_reduce_diff(const int* diff, const int* dirty, bool selective, int shift, int order_mask,
                                int ntiles, const int* act, int nact, int* changed, cudaStream_t st, const int* dyn) {
    if (nact <= 0) return PFAST_OK;
    reduce_diff_kernel<<<nact, 256, 0, st>>>(diff, dirty, selective ? 1 : 0, shift, order_mask, ntiles, act, changed,
                                             dyn);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "reduce_diff launch", __FILE__, __LINE__);
    return PFAST_OK;
}

// ------------------------------------------------------------------ small kernels
namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(long long n) {
    long long b = (n + kThreads - 1) / kThreads;
    return (unsigned)std::min<long long>(b, 152LL * 64);
}

__global__ void slowness_kernel(const double* __restrict__ vp, double* __restrict__ s64, float* __restrict__ s32,
                                double* __restrict__ sq64, int* __restrict__ bad, long long n, double sq_scale) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double v = vp[t];
        if (!(v > 0.0 && v < INFINITY)) *bad = 1;
        const double s = 1.0 / v;   // s = 1.0/vp, src/T_pfsm3d.h:75
        s64[t] = s;
        if (s32) s32[t] = (float)s;
        if (sq64) sq64[t] = (s * s) * sq_scale;
    }
}

template <typename Real>
__global__ void init_fwd_kernel(Real* __restrict__ f, long long fstride, long long n, const long long* __restrict__ src_lin) {
    const int b = blockIdx.y;
    Real* g = f + b * fstride;
    const long long sn = src_lin[b];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        g[t] = (t == sn) ? Real(0) : Real(kInf);   // point-source initialisation, src/T_pfsm3d.h:139-148
}

// Near-source start (opt-in): block y = instance, threads over the (2r+1)^3 cube.
template <typename Real>
__global__ void near_source_kernel(Real* __restrict__ f, long long fstride, const int* __restrict__ src_kij,
                                   const double* __restrict__ s64, int nz, int nr, int nc, double dx, double dy,
                                   double dz, int r) {
    const int b = blockIdx.y;
    const int sk = src_kij[3 * b], si = src_kij[3 * b + 1], sj = src_kij[3 * b + 2];
    const int w = 2 * r + 1;
    const long long plane = (long long)nr * nc;
    const double ss = s64[sk * plane + (long long)si * nc + sj];
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < w * w * w; t += gridDim.x * blockDim.x) {
        const int qk = t / (w * w) - r, qi = (t / w) % w - r, qj = t % w - r;
        const int k = sk + qk, i = si + qi, j = sj + qj;
        if (k < 0 || k >= nz || i < 0 || i >= nr || j < 0 || j >= nc) continue;
        if (qk * qk + qi * qi + qj * qj > r * r) continue;
        const long long node = k * plane + (long long)i * nc + j;
        const double ex = qj * dx, ey = qi * dy, ez = qk * dz;
        const double dist = sqrt(ex * ex + ey * ey + ez * ez);
        f[b * fstride + node] = Real(0.5 * (ss + s64[node]) * dist);
    }
}

__global__ void widen_kernel(const float* __restrict__ a, double* __restrict__ b, long long s32, long long s64, long long n) {
    const int k = blockIdx.y;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        b[k * s64 + t] = (double)a[k * s32 + t];
}

__global__ void narrow_kernel(const double* __restrict__ a, float* __restrict__ b, long long s64, long long s32, long long n) {
    const int k = blockIdx.y;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        b[k * s32 + t] = (float)a[k * s64 + t];
}

__global__ void widen_lambda_kernel(const float* __restrict__ a, double* __restrict__ b, const unsigned* __restrict__ mask,
                                    long long s32, long long s64, long long ms, int nz, int nr, int nc, int wpr) {
    const int k = blockIdx.y;
    const long long n = (long long)nz * nr * nc;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long row = t / nc;
        const int j = (int)(t - row * nc);
        const bool fixed = (mask[k * ms + row * wpr + (j >> 5)] >> (j & 31)) & 1u;
        if (!fixed) b[k * s64 + t] = (double)a[k * s32 + t];
    }
}

// One warp per source.  Lanes evaluate 32 consecutive receiver rows; the misfit is
// summed by lane 0 in row order (the reference's EE += ... sequence).
__global__ void bc3_kernel(const Bc3Args A) {
    const int b = blockIdx.x;
    const int lane = threadIdx.x;
    const double* T = A.T + b * A.fstride;
    double* L = A.L + b * A.fstride;
    unsigned* mask = A.mask + b * A.mask_stride;
    const long long plane = (long long)A.nr * A.nc;
    const int r0 = A.ch0[b], nrec = A.srnum[b];
    const int sk = A.src_kij[3 * b], si = A.src_kij[3 * b + 1], sj = A.src_kij[3 * b + 2];
    double E = 0.0;
    bool big = false;
    for (int base = 0; base < nrec; base += 32) {
        const int r = base + lane;
        double e = 0.0;
        if (r < nrec) {
            const int row = r0 + r;
            const double tob = A.tobs[row];
            if (tob < 100) {   // only picked first arrivals, src/T_padjoint3d.h:95
                const int i = A.rec[3 * row], j = A.rec[3 * row + 1], k = A.rec[3 * row + 2];
                const long long o = k * plane + (long long)i * A.nc + j;
                atomicOr(&mask[((long long)k * A.nr + i) * A.wpr + (j >> 5)], 1u << (j & 31));
                const double res = tob - T[o];
                e = res * res / 2.0;
                if (A.last[row] && !(i == si && j == sj && k == sk)) {
                    const double ny = A.nxyz[3 * row], nx = A.nxyz[3 * row + 1], nzz = A.nxyz[3 * row + 2];
                    const double Tz = (k + 1 >= A.nz) ? (T[o] - T[o - plane]) / A.dz : (T[o + plane] - T[o]) / A.dz;
                    const double Ty = (i + 1 >= A.nr) ? (T[o] - T[o - A.nc]) / A.dy : (T[o + A.nc] - T[o]) / A.dy;
                    const double Tx = (j + 1 >= A.nc) ? (T[o] - T[o - 1]) / A.dx : (T[o + 1] - T[o]) / A.dx;
                    double v = 0.0;
                    if (fabs(tob - T[o]) > 1e-9 && fabs(nx * Tx + ny * Ty + nzz * Tz) > 1e-6)
                        v = (tob - T[o]) / (nx * Tx + ny * Ty + nzz * Tz);
                    L[o] = v;
                    if (fabs(v) > kConvTol) big = true;
                }
            }
        }
        for (int l = 0; l < 32; ++l) {
            const double el = __shfl_sync(0xffffffffu, e, l);
            if (lane == 0) E += el;   // adding 0 for unpicked rows leaves E unchanged
        }
    }
    big = __any_sync(0xffffffffu, big);
    if (lane == 0) {
        A.EE[b] = E;
        A.need[b] = big ? 1 : 0;   // first isconv(p=0, U) test of src/T_padjoint3d.h:135
    }
}

// exact: g -= lambda_b / v^3 over the batch's sources, one division per source in source
// order, as the reference accumulates (src/T_PFAST3D.cpp:393).  Otherwise (the mixed-precision
// path: FP64 divisions are scarce on this part) g holds the running sum of lambda over the
// sources, added in source order, so the sum does not depend on how the sources are split into
// batches; finish_gradient_kernel divides once at the end.
__global__ void accumulate_kernel(double* __restrict__ g, const double* __restrict__ lam, long long fstride,
                                  const double* __restrict__ vp, long long n, int nb, int exact) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        double acc = g[t];
        if (exact) {
            const double v = vp[t];
            const double v3 = v * v * v;
            for (int b = 0; b < nb; ++b) acc = acc - lam[b * fstride + t] / v3;
        } else {
            for (int b = 0; b < nb; ++b) acc += __ldcs(lam + b * fstride + t);
        }
        g[t] = acc;
    }
}

// g = -(sum of lambda) / v^3 after the last batch of the mixed-precision path.
__global__ void finish_gradient_kernel(double* __restrict__ g, const double* __restrict__ vp, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double v = vp[t];
        g[t] = 0.0 - g[t] / (v * v * v);
    }
}

__global__ void gather3_kernel(const double* __restrict__ T, long long fstride, const int* __restrict__ rec,
                               const int* __restrict__ ch0, const int* __restrict__ srnum, int nz, int nr, int nc,
                               double* __restrict__ picks) {
    const int b = blockIdx.y;
    const long long plane = (long long)nr * nc;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < srnum[b]; r += gridDim.x * blockDim.x) {
        const int row = ch0[b] + r;
        const int i = rec[3 * row], j = rec[3 * row + 1], k = rec[3 * row + 2];
        picks[row] = T[b * fstride + k * plane + (long long)i * nc + j];
    }
}

}  // namespace

#define PFAST_LAUNCH_CHECK()                                                                   \
    do {                                                                                       \
        cudaError_t e__ = cudaGetLastError();                                                  \
        if (e__ != cudaSuccess) return cuda_fail(e__, "kernel launch", __FILE__, __LINE__);    \
    } while (0)

pfast_status launch_slowness(const double* vp, double* s64, float* s32, double* sq64, double sq_scale, int* bad, long long n,
                             cudaStream_t st) {
    slowness_kernel<<<grid_for(n), kThreads, 0, st>>>(vp, s64, s32, sq64, bad, n, sq_scale);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_near_source3(void* field, int is_fp32, long long fstride, const int* src_kij, const double* s64,
                                 int nz, int nr, int nc, const Spacing3& sp, int radius, int nb, cudaStream_t st) {
    if (radius <= 0 || nb <= 0) return PFAST_OK;
    const int w = 2 * radius + 1;
    dim3 grid((unsigned)((w * w * w + kThreads - 1) / kThreads), nb);
    if (is_fp32)
        near_source_kernel<float><<<grid, kThreads, 0, st>>>((float*)field, fstride, src_kij, s64, nz, nr, nc, sp.d[0],
                                                             sp.d[1], sp.d[2], radius);
    else
        near_source_kernel<double><<<grid, kThreads, 0, st>>>((double*)field, fstride, src_kij, s64, nz, nr, nc,
                                                              sp.d[0], sp.d[1], sp.d[2], radius);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "near_source launch", __FILE__, __LINE__);
    return PFAST_OK;
}

pfast_status launch_init_fwd3(void* field, int is_fp32, long long fstride, long long n, const long long* src_lin,
                              int nbatch, cudaStream_t st) {
    dim3 grid(std::max(1u, grid_for(n) / std::max(1, nbatch / 8 + 1)), nbatch);
    if (is_fp32) init_fwd_kernel<float><<<grid, kThreads, 0, st>>>((float*)field, fstride, n, src_lin);
    else init_fwd_kernel<double><<<grid, kThreads, 0, st>>>((double*)field, fstride, n, src_lin);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_widen(const float* a, double* b, long long s32, long long s64, long long n, int nbatch, cudaStream_t st) {
    dim3 grid(std::max(1u, grid_for(n) / std::max(1, nbatch / 8 + 1)), nbatch);
    widen_kernel<<<grid, kThreads, 0, st>>>(a, b, s32, s64, n);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_narrow(const double* a, float* b, long long s64, long long s32, long long n, int nbatch, cudaStream_t st) {
    dim3 grid(std::max(1u, grid_for(n) / std::max(1, nbatch / 8 + 1)), nbatch);
    narrow_kernel<<<grid, kThreads, 0, st>>>(a, b, s64, s32, n);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_widen_lambda(const float* l32, double* l64, const unsigned* mask, long long s32, long long s64,
                                 long long ms, int nz, int nr, int nc, int wpr, int nbatch, cudaStream_t st) {
    const long long n = (long long)nz * nr * nc;
    dim3 grid(std::max(1u, grid_for(n) / std::max(1, nbatch / 8 + 1)), nbatch);
    widen_lambda_kernel<<<grid, kThreads, 0, st>>>(l32, l64, mask, s32, s64, ms, nz, nr, nc, wpr);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_bc3(const Bc3Args& a, int nbatch, cudaStream_t st) {
    bc3_kernel<<<nbatch, 32, 0, st>>>(a);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_accumulate(double* grad, const double* lam, long long fstride, const double* vp, long long n,
                               int nbatch, bool exact, cudaStream_t st) {
    accumulate_kernel<<<grid_for(n), kThreads, 0, st>>>(grad, lam, fstride, vp, n, nbatch, exact ? 1 : 0);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_finish_gradient(double* grad, const double* vp, long long n, cudaStream_t st) {
    finish_gradient_kernel<<<grid_for(n), kThreads, 0, st>>>(grad, vp, n);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

pfast_status launch_gather3(const double* T, long long fstride, const int* rec, const int* ch0, const int* srnum,
                            int nbatch, int nz, int nr, int nc, double* picks, cudaStream_t st) {
    dim3 grid(16, nbatch);
    gather3_kernel<<<grid, kThreads, 0, st>>>(T, fstride, rec, ch0, srnum, nz, nr, nc, picks);
    PFAST_LAUNCH_CHECK();
    return PFAST_OK;
}

}  // namespace pfast
