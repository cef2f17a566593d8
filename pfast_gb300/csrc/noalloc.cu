// noalloc.cu -- pfast_fsm3d_noalloc: the single-source first-arrival solve for
// callers that cannot allocate device memory.
//
// Who needs it: a host program whose own pool allocator or memory budget owns every
// byte of the device and forbids libraries to call cudaMalloc (simulation frameworks
// and game engines commonly do this), or a latency-bound loop that must not meet the
// allocator's implicit synchronisation.  The caller owns the model and the output on
// the device; every byte of work memory this entry point needs comes from one
// file-scope static device array of fixed size, which each GPU that loads the library
// holds until the process exits.
//
// The array holds, for at most PFAST_NOALLOC_MAX_NODES grid nodes: the slowness
// field, the iteration-start snapshot, the tile-diagonal table, the per-tile
// locking flags and a few words.
// Its device address is taken with cudaGetSymbolAddress once per device, on the
// first call made on that device (with that device current), and cached for the
// life of the process; that first call should come before any stream capture, and
// the cached address is not valid after cudaDeviceReset (the module is loaded again,
// possibly elsewhere).  Every call shares the array and it keeps the last call's
// contents: this file writes or clears everything it reads before reading it, and
// calls that overlap on the GPU (on different streams or host threads) race on it.
//
// The call blocks the calling thread: it reads a velocity-check flag and, once per
// outer iteration, a convergence flag back to the host (synchronising `stream` each
// time), because the number of iterations depends on the field.
//
// The sweeps are the library's plain FP64 kernels (bit-identical to pfast_fsm3d).

#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "kernels.h"

namespace pfast {
namespace {

constexpr long long kMaxNodes = PFAST_NOALLOC_MAX_NODES;
constexpr int kMaxTiles = 16384;
constexpr int kMaxDiag = 3072;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }
constexpr size_t kOffSlow = 0;                                              // double[kMaxNodes]
constexpr size_t kOffSnap = align256(kOffSlow + 8 * (size_t)kMaxNodes);     // double[kMaxNodes]
constexpr size_t kOffTiles = align256(kOffSnap + 8 * (size_t)kMaxNodes);    // unsigned[kMaxTiles]
constexpr size_t kOffDiag = align256(kOffTiles + 4 * (size_t)kMaxTiles);    // int[kMaxDiag + 1]
constexpr size_t kOffFlags = align256(kOffDiag + 4 * (size_t)(kMaxDiag + 1));   // int[3*kMaxTiles]: dirty, stamp, diff
constexpr size_t kOffWords = align256(kOffFlags + 12 * (size_t)kMaxTiles);
// words: [0..1] source linear index (long long), [2..4] source (k,i,j), [5] active id,
//        [6] changed flag, [7] bad-velocity flag
constexpr size_t kScratchBytes = align256(kOffWords + 64);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
unsigned char* g_base[64] = {};   // device address of g_noalloc_scratch, per device

pfast_status scratch_base(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_base[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)", __FILE__, __LINE__);
        g_base[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_base[dev];
    return PFAST_OK;
}

}  // namespace
}  // namespace pfast

using namespace pfast;

extern "C" pfast_status pfast_fsm3d_noalloc(const double* vp, double* U, int src_row, int src_col, int src_z,
                                           int MAXSwp, double dx, double dy, double dz, int nrows, int ncols, int nz,
                                           void* stream) {
    if (!vp || !U) { set_last_error("null device pointer"); return PFAST_ERR_INVALID; }
    if (nrows < 2 || ncols < 2 || nz < 2) {
        set_last_error("grid %dx%dx%d: every dimension must be >= 2", nrows, ncols, nz);
        return PFAST_ERR_INVALID;
    }
    const long long N = (long long)nrows * ncols * nz;
    if (N > kMaxNodes) {
        set_last_error("grid of %lld nodes exceeds the no-allocation limit of %lld nodes (PFAST_NOALLOC_MAX_NODES)",
                       N, kMaxNodes);
        return PFAST_ERR_INVALID;
    }
    if (src_row < 0 || src_row >= nrows || src_col < 0 || src_col >= ncols || src_z < 0 || src_z >= nz) {
        set_last_error("source (%d,%d,%d) outside the grid", src_row, src_col, src_z);
        return PFAST_ERR_INVALID;
    }
    if (!(dx > 0 && dy > 0 && dz > 0) || MAXSwp < 0) {
        set_last_error("spacings must be positive and MAXSwp non-negative");
        return PFAST_ERR_INVALID;
    }
    // tile-diagonal table on the host (same packing as the allocating path)
    const int nbk = (nz + TK - 1) / TK, nbi = (nrows + TI - 1) / TI, nbj = (ncols + TJ - 1) / TJ;
    const int ndiag = nbk + nbi + nbj - 2;
    if (nbk > 1023 || nbi > 1023 || nbj > 1023 || ndiag > kMaxDiag || (long long)nbk * nbi * nbj > kMaxTiles) {
        set_last_error("grid %dx%dx%d needs more tiles than the no-allocation table holds (%d)", nrows, ncols, nz,
                       kMaxTiles);
        return PFAST_ERR_INVALID;
    }
    std::vector<unsigned> tiles;
    std::vector<int> off(ndiag + 1, 0);
    for (int d = 0; d < ndiag; ++d) {
        off[d] = (int)tiles.size();
        for (int bk = 0; bk < nbk; ++bk)
            for (int bi = 0; bi < nbi; ++bi) {
                const int bj = d - bk - bi;
                if (bj >= 0 && bj < nbj) tiles.push_back((unsigned)bk | ((unsigned)bi << 10) | ((unsigned)bj << 20));
            }
    }
    off[ndiag] = (int)tiles.size();

    int dev = 0;
    PFAST_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_last_error("device id %d unsupported", dev); return PFAST_ERR_INVALID; }
    unsigned char* base = nullptr;
    pfast_status st0 = scratch_base(dev, &base);
    if (st0 != PFAST_OK) return st0;
    cudaStream_t s = (cudaStream_t)stream;
    double* slow = reinterpret_cast<double*>(base + kOffSlow);
    double* snap = reinterpret_cast<double*>(base + kOffSnap);
    unsigned* d_tiles = reinterpret_cast<unsigned*>(base + kOffTiles);
    int* d_off = reinterpret_cast<int*>(base + kOffDiag);
    int* words = reinterpret_cast<int*>(base + kOffWords);
    long long* d_src_lin = reinterpret_cast<long long*>(words);
    int* d_src_kij = words + 2;
    int* d_act = words + 5;
    int* d_changed = words + 6;
    int* d_bad = words + 7;
    int* d_dirty = reinterpret_cast<int*>(base + kOffFlags);
    const int ntiles = nbk * nbi * nbj;

    int hw[8];
    const long long lin = (long long)src_z * nrows * ncols + (long long)src_row * ncols + src_col;
    std::memcpy(hw, &lin, sizeof(lin));
    hw[2] = src_z;
    hw[3] = src_row;
    hw[4] = src_col;
    hw[5] = 0;   // the single instance
    hw[6] = 0;
    hw[7] = 0;
    PFAST_CUDA_TRY(cudaMemcpyAsync(words, hw, sizeof(hw), cudaMemcpyHostToDevice, s));
    PFAST_CUDA_TRY(cudaMemcpyAsync(d_tiles, tiles.data(), sizeof(unsigned) * tiles.size(), cudaMemcpyHostToDevice, s));
    PFAST_CUDA_TRY(cudaMemcpyAsync(d_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice, s));

    pfast_status r = launch_slowness(vp, slow, nullptr, nullptr, 1.0, d_bad, N, s);
    if (r) return r;
    int bad = 0;
    PFAST_CUDA_TRY(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    if (bad) {
        set_last_error("the velocity model holds a value that is not a positive finite number");
        return PFAST_ERR_INVALID;
    }
    r = launch_init_fwd3(U, 0, N, N, d_src_lin, 1, s);
    if (r) return r;

    Sweep3Args a;
    std::memset(&a, 0, sizeof(a));
    a.field = U;
    a.fstride = N;
    a.aux = slow;
    a.src_kij = d_src_kij;
    a.snap = snap;
    a.changed = d_changed;
    a.act = d_act;
    a.diag_off = d_off;
    a.diag_tiles = d_tiles;
    a.nz = nz;
    a.nr = nrows;
    a.nc = ncols;
    a.nbk = nbk;
    a.nbi = nbi;
    a.nbj = nbj;
    const double dd[3] = {dx, dy, dz};
    for (int k = 0; k < 3; ++k) {
        a.sp.d[k] = dd[k];
        a.sp.d2[k] = dd[k] * dd[k];
        a.sp.inv2[k] = 1.0 / dd[k] / dd[k];
    }
    a.tol_abs = kConvTol;
    a.ntiles = ntiles;
    a.dirty = d_dirty;
    a.stamp = d_dirty + ntiles;
    a.diff = d_dirty + 2 * ntiles;
    PFAST_CUDA_TRY(cudaMemsetAsync(a.dirty, 0xff, sizeof(int) * ntiles, s));
    PFAST_CUDA_TRY(cudaMemsetAsync(a.stamp, 0xff, sizeof(int) * ntiles, s));
    // outer iterations of src/T_pfsm3d.h:152: snapshot + 8 sweeps while some node moved by > 1e-9
    for (int it = 0; it < MAXSwp; ++it) {
        PFAST_CUDA_TRY(cudaMemsetAsync(a.diff, 0, sizeof(int) * ntiles, s));
        a.iter = it;
        for (int dir = 0; dir < 8; ++dir) {
            a.dir = dir;
            for (int d = 0; d < ndiag; ++d) {
                r = launch_sweep3(kFwdPlain64, a, off[d], off[d + 1] - off[d], 1, s);
                if (r) return r;
            }
        }
        PFAST_CUDA_TRY(cudaMemsetAsync(d_changed, 0, sizeof(int), s));
        r = launch_reduce_diff(a.diff, a.dirty, false, 8, 0xff, ntiles, d_act, 1, d_changed, s);
        if (r) return r;
        int changed = 0;
        PFAST_CUDA_TRY(cudaMemcpyAsync(&changed, d_changed, sizeof(int), cudaMemcpyDeviceToHost, s));
        PFAST_CUDA_TRY(cudaStreamSynchronize(s));
        // converged, or moved with every tile locked (the next iteration would change nothing)
        if (!(changed & 1) || !(changed & 2)) break;
    }
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));   // the host table vectors are read by the copies above
    return PFAST_OK;
}
