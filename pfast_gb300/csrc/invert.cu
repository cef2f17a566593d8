// invert.cu -- the drivers' outer inversion loop with the model, gradients, search
// direction and L-BFGS pairs resident on the device.
//
// Reference: src/RT_PFAST2D.cpp:412-816 (2D) and src/T_PFAST3D.cpp:359-656 (3D), with
// regu2d / regu3d, magnitudeOf, gd2sk, beta_HS, beta_CGDESCENT, cubicInterp, updatevp
// and check_conv of src/RT_padjoint2d.h:475-646 and src/T_padjoint3d.h:174-342.
//
// Device work per iteration: one gradient evaluation of the survey (the sweep
// pipelines of engine.cu / engine2d.cu), a cuFFT Z2Z transform pair per
// regularisation, and a handful of streaming passes over N-vectors (inner products,
// axpy, the clamp of updatevp).  Every N-vector stays in HBM; the host holds only the
// scalars (misfits, step lengths, inner products), which it needs to take the
// line-search branches exactly as the reference does.
//
// Inner products: every thread of a fixed grid (kRedBlocks x 256) accumulates a
// grid-stride slice, blocks reduce in a fixed tree, and the host adds the block sums
// in block order -- the same result on every run.  The per-element expressions keep
// the reference's operand order (e.g. (alpha1*dk)*(-g1+g0) in gd2sk); the summation
// order differs from the reference's sequential loop, a rounding-level difference.
#include <cufft.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "engine.h"

using namespace pfast;

namespace {

constexpr int kRedBlocks = 608;   // 4 per SM on 152 SMs
constexpr int kRedThreads = 256;
constexpr int kEwThreads = 256;
constexpr double kPi = 3.141592653589793;   // PI, src/T_pfsm3d.h:25

enum RedOp : int {
    kDot = 0,     // a0 += x*y
    kNegDot,      // a0 += -x*y                          (dphi = sum -dk*Dj)
    kHS,          // a0 += x*(x-y), a1 += -z*(x-y)        (beta_HS: x = g1, y = g0, z = dk)
    kCGD1,        // a0 += z*(-x+y), a1 += (-x+y)^2       (beta_CGDESCENT, first pass)
    kCGD2,        // a0 += ((-x+y) - 2*z*s0/s1)*(-x)/s1   (second pass: s0 = ny, s1 = dTy)
    kPair,        // gd2sk: a0 += s0*z*(-x+y), a1 += (-x+y)^2, w0 = s0*z, w1 = -x+y
    kRhoDot,      // a0 += s0*x*y                         (two-loop: rho*sk*q, rho*yk*d)
    kMaxAbs,      // a0 = max |x|                         (magnitudeOf)
    kConv,        // a0 = max s0*s0*x*x/y/y               (check_conv: x = dk, y = vp)
};

__device__ __forceinline__ double vmax(double a, double b) { return (b >= a) ? b : a; }

__global__ void __launch_bounds__(kRedThreads) reduce_kernel(int op, const double* __restrict__ x,
                                                             const double* __restrict__ y,
                                                             const double* __restrict__ z, double s0, double s1,
                                                             long long n, double* __restrict__ part,
                                                             double* __restrict__ w0, double* __restrict__ w1) {
    double a0 = 0.0, a1 = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        switch (op) {
            case kDot: a0 += x[i] * y[i]; break;
            case kNegDot: a0 += -x[i] * y[i]; break;
            case kHS: {
                const double d = x[i] - y[i];
                a0 += x[i] * d;
                a1 += -z[i] * d;
            } break;
            case kCGD1: {
                const double t = -x[i] + y[i];
                a0 += z[i] * t;
                a1 += t * t;
            } break;
            case kCGD2: {
                const double t = -x[i] + y[i];
                a0 += (t - 2 * z[i] * s0 / s1) * (-x[i]) / s1;
            } break;
            case kPair: {
                const double t = -x[i] + y[i];
                a0 += s0 * z[i] * t;
                a1 += t * t;
                w0[i] = s0 * z[i];
                w1[i] = t;
            } break;
            case kRhoDot: a0 += s0 * x[i] * y[i]; break;
            case kMaxAbs: a0 = vmax(a0, fabs(x[i])); break;
            case kConv: a0 = vmax(a0, s0 * s0 * x[i] * x[i] / y[i] / y[i]); break;
        }
    }
    const bool mx = (op == kMaxAbs || op == kConv);
    for (int o = 16; o > 0; o >>= 1) {
        const double b0 = __shfl_down_sync(0xffffffffu, a0, o);
        const double b1 = __shfl_down_sync(0xffffffffu, a1, o);
        a0 = mx ? vmax(a0, b0) : a0 + b0;
        a1 += b1;
    }
    __shared__ double s[2][kRedThreads / 32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        s[0][w] = a0;
        s[1][w] = a1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double r0 = s[0][0], r1 = s[1][0];
        for (int k = 1; k < kRedThreads / 32; ++k) {
            r0 = mx ? vmax(r0, s[0][k]) : r0 + s[0][k];
            r1 += s[1][k];
        }
        part[2 * blockIdx.x] = r0;
        part[2 * blockIdx.x + 1] = r1;
    }
}

// out = a + s*b
__global__ void axpy_kernel(double* __restrict__ out, const double* __restrict__ a, double s,
                            const double* __restrict__ b, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] + s * b[i];
}

// out = a - s*b
__global__ void axmy_kernel(double* __restrict__ out, const double* __restrict__ a, double s,
                            const double* __restrict__ b, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = a[i] - s * b[i];
}

// out = s*x
__global__ void scale_kernel(double* __restrict__ out, double s, const double* __restrict__ x, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = s * x[i];
}

__global__ void to_complex_kernel(cufftDoubleComplex* __restrict__ c, const double* __restrict__ x, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) c[i] = make_cuDoubleComplex(x[i], 0.0);
}

// regu2d / regu3d spectral filter: F /= 1 + nux^2 kx[j]^2 + nuy^2 ky[i]^2 (+ nuz^2 kz[k]^2),
// terms added in that order (src/RT_padjoint2d.h:533-538, src/T_padjoint3d.h:232-239).
__global__ void regu_filter_kernel(cufftDoubleComplex* __restrict__ c, const double* __restrict__ kx,
                                   const double* __restrict__ ky, const double* __restrict__ kz, double nux,
                                   double nuy, double nuz, int nr, int nc, long long n, int three_d) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const int j = (int)(idx % nc);
    const long long r = idx / nc;
    const int i = (int)(r % nr);
    const int k = (int)(r / nr);
    double den = 1 + nux * nux * kx[j] * kx[j] + nuy * nuy * ky[i] * ky[i];
    if (three_d) den = den + nuz * nuz * kz[k] * kz[k];
    cufftDoubleComplex v = c[idx];
    v.x = v.x / den;
    v.y = v.y / den;
    c[idx] = v;
}

// real part of the unscaled inverse transform times 1/N; zero in water (vp == 330).
__global__ void regu_finish_kernel(double* __restrict__ out, const cufftDoubleComplex* __restrict__ c,
                                   const double* __restrict__ vp, double scale, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (fabs(vp[i] - 330) < 1e-9) ? 0.0 : c[i].x * scale;
}

// updatevp (src/RT_padjoint2d.h:497-505): vp += a*dk outside water, clamped to [minv, maxv].
__global__ void updatevp_kernel(double* __restrict__ vp, const double* __restrict__ dk, double a, double minv,
                                double maxv, long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = vp[i];
    if (fabs(v - 330) > 1e-9) {
        v = v + a * dk[i];
        if (v > maxv) v = maxv;
        if (v < minv) v = minv;
        vp[i] = v;
    }
}

inline unsigned ew_blocks(long long n) { return (unsigned)((n + kEwThreads - 1) / kEwThreads); }

// k of regu2d / regu3d (src/RT_padjoint2d.h:520-529): -kmax + ks*j, then entries j and n/2+j swapped.
std::vector<double> kvec(int n, double d) {
    const double kmax = kPi / d, ks = 2 * kPi / n / d;
    std::vector<double> k(n);
    for (int j = 0; j < n; ++j) k[j] = -kmax + ks * j;
    for (int j = 0; j < n / 2; ++j) std::swap(k[j], k[n / 2 + j]);
    return k;
}

pfast_status cufft_fail(cufftResult r, const char* what) {
    set_last_error("%s failed: cuFFT error %d", what, (int)r);
    return r == CUFFT_ALLOC_FAILED ? PFAST_ERR_NOMEM : PFAST_ERR_CUDA;
}

#define INV_TRY(expr)                          \
    do {                                       \
        pfast_status s__ = (expr);             \
        if (s__ != PFAST_OK) return s__;       \
    } while (0)

#define INV_LAUNCH(inv, call)                                                          \
    do {                                                                               \
        call;                                                                          \
        cudaError_t e__ = cudaGetLastError();                                          \
        if (e__ != cudaSuccess) return cuda_fail(e__, #call, __FILE__, __LINE__);      \
        ++(inv)->ctx->launches;                                                        \
    } while (0)

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

struct pfast_inversion {
    pfast_ctx* ctx = nullptr;
    int dim = 0;
    pfast_survey2d* sv2 = nullptr;
    pfast_survey3d* sv3 = nullptr;
    pfast_invert_options o{};
    int nz = 1, nr = 0, nc = 0;
    long long N = 0;
    // device N-vectors
    double *vp = nullptr, *WR = nullptr, *Djk1 = nullptr, *Djk0 = nullptr, *dk = nullptr, *q = nullptr,
           *Dj1 = nullptr, *locvp = nullptr;
    double *g_raw = nullptr;                 // this iteration's gradient, unregularised
    double *gT = nullptr, *gR = nullptr;     // 2D parts of the main evaluation
    double *gT_af = nullptr, *gR_af = nullptr;
    double *lsT = nullptr, *lsR = nullptr, *lsRT = nullptr;   // 2D line-search evaluation
    double *sk = nullptr, *yk = nullptr;     // [LM][N]
    double *kx = nullptr, *ky = nullptr, *kz = nullptr;
    cufftDoubleComplex* fbuf = nullptr;
    cufftHandle plan = 0;
    bool have_plan = false;
    double* part = nullptr;                  // device block sums
    double* h_part = nullptr;                // pinned host copy
    std::vector<void*> allocs;
    // host scalars of the loop
    std::vector<double> globalE, rho, ai;
    double alpha0 = 0.0, alpha1 = 5.0e3, c1 = 1.0e-4, c2 = 0.9;
    int iter = 0;
    bool converged = false;
    bool resume_pending = false;             // next step takes its gradient from g_raw (resume)
    pfast_invert_report last{};
};

namespace {

pfast_status dalloc(pfast_inversion* inv, double** p, long long count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(double) * (size_t)std::max<long long>(count, 1));
    if (e != cudaSuccess) {
        cudaGetLastError();
        set_last_error("cudaMalloc(%lld doubles) failed: %s", count, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? PFAST_ERR_NOMEM : PFAST_ERR_CUDA;
    }
    inv->allocs.push_back(q);
    *p = static_cast<double*>(q);
    return PFAST_OK;
}

pfast_status upload(pfast_inversion* inv, double* d, const double* h, size_t n) {
    PFAST_CUDA_TRY(cudaMemcpyAsync(d, h, sizeof(double) * n, cudaMemcpyHostToDevice, inv->ctx->stream));
    return PFAST_OK;
}

// r0, r1 = the two accumulators of `op` over n elements (see RedOp).
pfast_status reduce(pfast_inversion* inv, int op, const double* x, const double* y, const double* z, double s0,
                    double s1, double* r0, double* r1 = nullptr, double* w0 = nullptr, double* w1 = nullptr) {
    const long long n = inv->N;
    const int nb = (int)std::min<long long>(kRedBlocks, std::max<long long>(1, (n + kRedThreads - 1) / kRedThreads));
    cudaStream_t s = inv->ctx->stream;
    INV_LAUNCH(inv, (reduce_kernel<<<nb, kRedThreads, 0, s>>>(op, x, y, z, s0, s1, n, inv->part, w0, w1)));
    PFAST_CUDA_TRY(cudaMemcpyAsync(inv->h_part, inv->part, sizeof(double) * 2 * nb, cudaMemcpyDeviceToHost, s));
    PFAST_CUDA_TRY(cudaStreamSynchronize(s));
    const bool mx = (op == kMaxAbs || op == kConv);
    double a0 = inv->h_part[0], a1 = inv->h_part[1];
    for (int b = 1; b < nb; ++b) {
        const double v = inv->h_part[2 * b];
        a0 = mx ? ((v >= a0) ? v : a0) : a0 + v;
        a1 += inv->h_part[2 * b + 1];
    }
    if (r0) *r0 = a0;
    if (r1) *r1 = a1;
    return PFAST_OK;
}

pfast_status axpy(pfast_inversion* inv, double* out, const double* a, double s, const double* b) {
    INV_LAUNCH(inv, (axpy_kernel<<<ew_blocks(inv->N), kEwThreads, 0, inv->ctx->stream>>>(out, a, s, b, inv->N)));
    return PFAST_OK;
}

pfast_status axmy(pfast_inversion* inv, double* out, const double* a, double s, const double* b) {
    INV_LAUNCH(inv, (axmy_kernel<<<ew_blocks(inv->N), kEwThreads, 0, inv->ctx->stream>>>(out, a, s, b, inv->N)));
    return PFAST_OK;
}

pfast_status copy(pfast_inversion* inv, double* dst, const double* src) {
    PFAST_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * inv->N, cudaMemcpyDeviceToDevice, inv->ctx->stream));
    return PFAST_OK;
}

// regu2d / regu3d: out = regularised g, water mask of the CURRENT model (inv->vp).  out may alias g.
pfast_status regu(pfast_inversion* inv, double* out, const double* g) {
    const long long n = inv->N;
    cudaStream_t s = inv->ctx->stream;
    INV_LAUNCH(inv, (to_complex_kernel<<<ew_blocks(n), kEwThreads, 0, s>>>(inv->fbuf, g, n)));
    cufftResult r = cufftExecZ2Z(inv->plan, inv->fbuf, inv->fbuf, CUFFT_FORWARD);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2Z(forward)");
    ++inv->ctx->launches;
    if (inv->dim == 2) {
        // 2D: kx over columns with nux, the rows' term with nuz (src/RT_padjoint2d.h:533-534)
        INV_LAUNCH(inv, (regu_filter_kernel<<<ew_blocks(n), kEwThreads, 0, s>>>(
                            inv->fbuf, inv->kx, inv->ky, inv->kz, inv->o.nux, inv->o.nuz, 0.0, inv->nr, inv->nc, n, 0)));
    } else {
        INV_LAUNCH(inv, (regu_filter_kernel<<<ew_blocks(n), kEwThreads, 0, s>>>(
                            inv->fbuf, inv->kx, inv->ky, inv->kz, inv->o.nux, inv->o.nuy, inv->o.nuz, inv->nr, inv->nc,
                            n, 1)));
    }
    r = cufftExecZ2Z(inv->plan, inv->fbuf, inv->fbuf, CUFFT_INVERSE);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftExecZ2Z(inverse)");
    ++inv->ctx->launches;
    INV_LAUNCH(inv, (regu_finish_kernel<<<ew_blocks(n), kEwThreads, 0, s>>>(out, inv->fbuf, inv->vp,
                                                                             1.0 / (double)n, n)));
    return PFAST_OK;
}

// Gradient of the survey at `model`.  g_sel: the gradient the loop uses (per RTtag);
// E: joint misfit (global_E); phi: the misfit the line search compares (per RTtag).
pfast_status evaluate(pfast_inversion* inv, const double* model, bool main, double** g_sel, double* E, double* phi,
                      double* Et, double* Er, pfast_invert_report* rep) {
    const auto t0 = std::chrono::steady_clock::now();
    if (inv->dim == 2) {
        double et = 0.0, er = 0.0;
        double* T = main ? inv->gT : inv->lsT;
        double* R = main ? inv->gR : inv->lsR;
        double* RT = main ? inv->g_raw : inv->lsRT;
        INV_TRY(eval2d_impl(inv->ctx, inv->sv2, model, inv->WR, &inv->o.eval, T, R, RT, &et, &er, nullptr));
        const double e = er + et;    // loc_E = loc_Er + loc_Et (src/RT_PFAST2D.cpp:435)
        switch (inv->o.rttag) {
            case PFAST_RT_TRANSMISSION: *g_sel = T; *phi = et; break;
            case PFAST_RT_REFLECTION: *g_sel = R; *phi = er; break;
            default: *g_sel = RT; *phi = e; break;
        }
        *E = e;
        if (Et) *Et = et;
        if (Er) *Er = er;
    } else {
        double e = 0.0;
        double* G = main ? inv->g_raw : inv->Dj1;
        INV_TRY(pfast_survey3d_eval(inv->ctx, inv->sv3, model, &inv->o.eval, G, &e, nullptr));
        *g_sel = G;
        *E = e;
        *phi = e;
        if (Et) *Et = 0.0;
        if (Er) *Er = 0.0;
    }
    rep->evals += 1;
    rep->ms_eval += ms_since(t0);
    return PFAST_OK;
}

// cubicInterp (src/RT_padjoint2d.h:619-630); PFAST_ERR_LINE_SEARCH where the reference
// returns no value.
pfast_status cubic_interp(double alpha0, double alpha1, double phi0, double phi1, double dphi0, double dphi1,
                          double* out) {
    const double a = (-2. * (phi1 - phi0) + (dphi0 + dphi1) * (alpha1 - alpha0)) /
                     ((alpha1 - alpha0) * (alpha1 - alpha0) * (alpha1 - alpha0));
    const double b = (3. * (phi1 - phi0) - (2. * dphi0 + dphi1) * (alpha1 - alpha0)) /
                     ((alpha1 - alpha0) * (alpha1 - alpha0));
    const double c = dphi0;
    if (std::fabs(a) > 0 && (b * b - 3 * a * c) > 0) {
        *out = alpha0 + (-b + std::sqrt(b * b - 3 * a * c)) / (3. * a);
        return PFAST_OK;
    }
    if (a == 0 && std::fabs(b) > 0 && (b * b - 3 * a * c) < 0) {
        *out = -c / (2. * b);
        return PFAST_OK;
    }
    set_last_error("cubic interpolation has no minimiser for (alpha0, alpha1, phi0, phi1, dphi0, dphi1) = "
                   "(%g %g %g %g %g %g)", alpha0, alpha1, phi0, phi1, dphi0, dphi1);
    return PFAST_ERR_LINE_SEARCH;
}

// L-BFGS: gd2sk (src/RT_padjoint2d.h:590-604) and the two-loop recursion
// (src/RT_PFAST2D.cpp:520-546).  ai[i % LM] is used where the reference's first loop reads
// ai[i] (the same value while Iterk - 2 < LM; past that the reference reads beyond ai).
pfast_status lbfgs_direction(pfast_inversion* inv) {
    const int LM = inv->o.LM, it = inv->iter;
    const long long N = inv->N;
    const int slot = (it - 2) % LM;
    double dTy = 0.0, ny = 0.0;
    INV_TRY(reduce(inv, kPair, inv->Djk1, inv->Djk0, inv->dk, inv->alpha1, 0.0, &dTy, &ny, inv->sk + (size_t)slot * N,
                   inv->yk + (size_t)slot * N));
    const double gamma = dTy / ny;
    inv->rho[slot] = 1.0 / dTy;
    INV_TRY(copy(inv, inv->q, inv->Djk1));
    const int lo = (it - LM - 1 >= 0) ? it - LM - 1 : 0;
    for (int i = it - 2; i >= lo; --i) {
        const int m = i % LM;
        double a = 0.0;
        INV_TRY(reduce(inv, kRhoDot, inv->sk + (size_t)m * N, inv->q, nullptr, inv->rho[m], 0.0, &a));
        inv->ai[m] = a;
        INV_TRY(axmy(inv, inv->q, inv->q, a, inv->yk + (size_t)m * N));
    }
    INV_LAUNCH(inv, (scale_kernel<<<ew_blocks(N), kEwThreads, 0, inv->ctx->stream>>>(inv->dk, gamma, inv->q, N)));
    for (int i = lo; i <= it - 2; ++i) {
        const int m = i % LM;
        double tmp = 0.0;
        INV_TRY(reduce(inv, kRhoDot, inv->yk + (size_t)m * N, inv->dk, nullptr, inv->rho[m], 0.0, &tmp));
        INV_TRY(axpy(inv, inv->dk, inv->dk, inv->ai[m] - tmp, inv->sk + (size_t)m * N));
    }
    return PFAST_OK;
}

pfast_status step(pfast_inversion* inv, pfast_invert_report* rep) {
    const auto t_iter = std::chrono::steady_clock::now();
    std::memset(rep, 0, sizeof(*rep));
    inv->iter += 1;
    const int it = inv->iter;
    rep->iter = it;
    PFAST_CUDA_TRY(cudaSetDevice(inv->ctx->device));
    INV_TRY(copy(inv, inv->Djk0, inv->Djk1));
    if (inv->resume_pending) {
        // resumed iteration: the stored gradient, unregularised, and the stored misfit
        // (src/T_PFAST3D.cpp:366-385)
        inv->resume_pending = false;
        INV_TRY(copy(inv, inv->Djk1, inv->g_raw));
        rep->E = inv->globalE[it - 1];
    } else {
        // gradient at the current model
        double* g = nullptr;
        double E = 0.0, phi = 0.0, Et = 0.0, Er = 0.0;
        INV_TRY(evaluate(inv, inv->vp, true, &g, &E, &phi, &Et, &Er, rep));
        if (g != inv->g_raw) INV_TRY(copy(inv, inv->g_raw, g));
        inv->globalE.push_back(E);
        rep->E = E;
        rep->Et = Et;
        rep->Er = Er;
        INV_TRY(regu(inv, inv->Djk1, inv->g_raw));
        double mx = 0.0;
        if (inv->o.schemetag != PFAST_SCHEME_LBFGS || it == 1) {
            INV_TRY(reduce(inv, kMaxAbs, inv->Djk1, nullptr, nullptr, 0.0, 0.0, &mx));
            inv->alpha1 = 5e2 * (1. / mx);     // 5e2 * magnitudeOf(Djk1)
        }
        if (inv->dim == 2 && inv->o.keep_components) {
            INV_TRY(regu(inv, inv->gR_af, inv->gR));
            INV_TRY(regu(inv, inv->gT_af, inv->gT));
        }
    }
    // search direction (src/RT_PFAST2D.cpp:498-552)
    if (it == 1) {
        INV_TRY(copy(inv, inv->dk, inv->Djk1));
    } else {
        switch (inv->o.schemetag) {
            case PFAST_SCHEME_HS: {
                double ta = 0.0, tb = 0.0;
                INV_TRY(reduce(inv, kHS, inv->Djk1, inv->Djk0, inv->dk, 0.0, 0.0, &ta, &tb));
                INV_TRY(axpy(inv, inv->dk, inv->Djk1, ta / tb, inv->dk));
                inv->c1 = 1.0e-4;
                inv->c2 = 0.1;
            } break;
            case PFAST_SCHEME_CGDESCENT: {
                double dTy = 0.0, ny = 0.0, beta = 0.0;
                INV_TRY(reduce(inv, kCGD1, inv->Djk1, inv->Djk0, inv->dk, 0.0, 0.0, &dTy, &ny));
                INV_TRY(reduce(inv, kCGD2, inv->Djk1, inv->Djk0, inv->dk, ny, dTy, &beta));
                INV_TRY(axpy(inv, inv->dk, inv->Djk1, beta, inv->dk));
                inv->c1 = 1.0e-4;
                inv->c2 = 0.1;
            } break;
            default:
                INV_TRY(lbfgs_direction(inv));
                inv->alpha0 = 0.0;
                inv->alpha1 = 1.0;
                inv->c1 = 1.0e-4;
                inv->c2 = 0.9;
                break;
        }
    }
    rep->alpha_start = inv->alpha1;
    // line search (src/RT_PFAST2D.cpp:561-807)
    const auto t_ls = std::chrono::steady_clock::now();
    const int MAX = inv->o.max_linesearch;
    if (inv->o.lsrc == PFAST_LS_SECANT_EXACT) {
        int count = 0;
        inv->alpha0 = 0.0;
        double f0 = 0.0, f1 = 0.0;
        while (std::fabs(inv->alpha1 - inv->alpha0) / std::fabs(inv->alpha0) > 1e-2 && count++ < MAX) {
            INV_TRY(axpy(inv, inv->locvp, inv->vp, inv->alpha1, inv->dk));
            double* gl = nullptr;
            double e1, p1;
            INV_TRY(evaluate(inv, inv->locvp, false, &gl, &e1, &p1, nullptr, nullptr, rep));
            INV_TRY(regu(inv, inv->Dj1, gl));
            f0 = 0.0;
            INV_TRY(reduce(inv, kDot, inv->Dj1, inv->dk, nullptr, 0.0, 0.0, &f1));
            const double alphak = inv->alpha1 - (inv->alpha1 - inv->alpha0) * f1 / (f1 - f0);
            inv->alpha0 = inv->alpha1;
            inv->alpha1 = alphak;
            f0 = f1;
        }
        rep->count = count;
        rep->stopped = count > MAX;
    } else if (inv->o.lsrc == PFAST_LS_SECANT_WOLFE || inv->o.lsrc == PFAST_LS_CUBIC) {
        const double phi0 = inv->globalE[it - 1];
        double dphi0 = 0.0;
        INV_TRY(reduce(inv, kNegDot, inv->dk, inv->Djk1, nullptr, 0.0, 0.0, &dphi0));
        inv->alpha0 = 0.0;
        const bool loop = inv->o.lsrc == PFAST_LS_SECANT_WOLFE || inv->o.schemetag == PFAST_SCHEME_LBFGS;
        bool wolfe = false;
        int count = 0;
        auto trial = [&](double* phi1, double* dphi1) -> pfast_status {
            INV_TRY(axpy(inv, inv->locvp, inv->vp, inv->alpha1, inv->dk));
            double* gl = nullptr;
            double e1;
            INV_TRY(evaluate(inv, inv->locvp, false, &gl, &e1, phi1, nullptr, nullptr, rep));
            INV_TRY(regu(inv, inv->Dj1, gl));
            INV_TRY(reduce(inv, kNegDot, inv->dk, inv->Dj1, nullptr, 0.0, 0.0, dphi1));
            return PFAST_OK;
        };
        auto record = [&](double a1, double phi1, double dphi1) {
            if (rep->ntrials < PFAST_INV_MAX_TRIALS) {
                double* t = rep->trial[rep->ntrials++];
                t[0] = inv->alpha0; t[1] = a1; t[2] = phi0; t[3] = phi1; t[4] = dphi0; t[5] = dphi1;
            }
        };
        if (loop) {
            while (!wolfe && count++ < MAX) {
                double phi1 = 0.0, dphi1 = 0.0;
                INV_TRY(trial(&phi1, &dphi1));
                const double tried = inv->alpha1;
                if (phi1 <= phi0 + inv->c1 * inv->alpha1 * dphi0 && std::fabs(dphi1) <= -inv->c2 * dphi0) {
                    wolfe = true;
                } else if (inv->o.lsrc == PFAST_LS_SECANT_WOLFE) {
                    inv->alpha1 = inv->alpha1 - (inv->alpha1 - inv->alpha0) * dphi1 / (dphi1 - dphi0);
                } else {
                    double nx = 0.0;
                    INV_TRY(cubic_interp(inv->alpha0, inv->alpha1, phi0, phi1, dphi0, dphi1, &nx));
                    inv->alpha1 = nx;
                }
                // lsrc 2 prints the trial's alpha1, lsrc 3 prints it after the update
                record(inv->o.lsrc == PFAST_LS_SECANT_WOLFE ? tried : inv->alpha1, phi1, dphi1);
            }
            rep->stopped = count > MAX;
        } else {
            // 2D cubic line search without L-BFGS: one trial, then the interpolated step
            // (src/RT_PFAST2D.cpp:752-806)
            double phi1 = 0.0, dphi1 = 0.0;
            INV_TRY(trial(&phi1, &dphi1));
            double nx = 0.0;
            INV_TRY(cubic_interp(inv->alpha0, inv->alpha1, phi0, phi1, dphi0, dphi1, &nx));
            inv->alpha1 = nx;
            record(inv->alpha1, phi1, dphi1);
        }
        rep->count = count;
    } else if (inv->o.lsrc != PFAST_LS_NONE) {
        set_last_error("line search tag %d unknown", inv->o.lsrc);
        return PFAST_ERR_INVALID;
    }
    rep->ms_linesearch = ms_since(t_ls);
    rep->stepsize = inv->alpha1;
    // updatevp and check_conv (src/RT_padjoint2d.h:475-505)
    INV_LAUNCH(inv, (updatevp_kernel<<<ew_blocks(inv->N), kEwThreads, 0, inv->ctx->stream>>>(
                        inv->vp, inv->dk, inv->alpha1, inv->o.minv, inv->o.maxv, inv->N)));
    const double chgE = it >= 2 ? (inv->globalE[it - 2] - inv->globalE[it - 1]) / inv->globalE[it - 2] : 1;
    pfast_status result = PFAST_OK;
    if (chgE <= inv->o.conv_tol) {
        inv->converged = true;
    } else {
        double mn = 0.0;
        INV_TRY(reduce(inv, kConv, inv->dk, inv->vp, nullptr, inv->alpha1, 0.0, &mn));
        const double mynorm = std::sqrt(mn);
        if (mynorm / (double)inv->N >= 1) {
            set_last_error("Over corrected: sqrt(max (step*dk/vp)^2) / N = %g", mynorm / (double)inv->N);
            result = PFAST_ERR_OVER_CORRECTED;
        }
    }
    PFAST_CUDA_TRY(cudaStreamSynchronize(inv->ctx->stream));
    rep->converged = inv->converged ? 1 : 0;
    rep->ms_total = ms_since(t_iter);
    inv->last = *rep;
    return result;
}

pfast_status validate(const pfast_invert_options* o, int dim) {
    if (o->schemetag < 1 || o->schemetag > 3) {
        set_last_error("schemetag %d unknown (1 HS, 2 CG_DESCENT, 3 L-BFGS)", o->schemetag);
        return PFAST_ERR_INVALID;
    }
    if (o->lsrc < 0 || o->lsrc > 3) { set_last_error("lsrc %d unknown", o->lsrc); return PFAST_ERR_INVALID; }
    if (o->LM < 1) { set_last_error("LM must be >= 1"); return PFAST_ERR_INVALID; }
    if (o->max_linesearch < 1 || o->max_linesearch > PFAST_INV_MAX_TRIALS) {
        set_last_error("max_linesearch must be in [1, %d]", PFAST_INV_MAX_TRIALS);
        return PFAST_ERR_INVALID;
    }
    if (dim == 2 && (o->rttag < 1 || o->rttag > 3)) { set_last_error("RTtag %d unknown", o->rttag); return PFAST_ERR_INVALID; }
    if (o->eval.precision != PFAST_PLAIN_FP64 && o->eval.precision != PFAST_MIXED) {
        set_last_error("unknown precision %d", o->eval.precision);
        return PFAST_ERR_INVALID;
    }
    if (o->eval.maxswp < 1) { set_last_error("maxswp must be >= 1"); return PFAST_ERR_INVALID; }
    return PFAST_OK;
}

pfast_status setup(pfast_inversion* inv, const double* vp, const double* WR) {
    const long long N = inv->N;
    const int LM = inv->o.LM;
    PFAST_CUDA_TRY(cudaSetDevice(inv->ctx->device));
    for (double** p : {&inv->vp, &inv->Djk1, &inv->Djk0, &inv->dk, &inv->q, &inv->Dj1, &inv->locvp, &inv->g_raw})
        INV_TRY(dalloc(inv, p, N));
    if (inv->dim == 2) {
        for (double** p : {&inv->WR, &inv->gT, &inv->gR, &inv->lsT, &inv->lsR, &inv->lsRT}) INV_TRY(dalloc(inv, p, N));
        if (inv->o.keep_components) {
            INV_TRY(dalloc(inv, &inv->gT_af, N));
            INV_TRY(dalloc(inv, &inv->gR_af, N));
        }
    }
    INV_TRY(dalloc(inv, &inv->sk, N * LM));
    INV_TRY(dalloc(inv, &inv->yk, N * LM));
    INV_TRY(dalloc(inv, &inv->part, 2 * kRedBlocks));
    {
        void* f = nullptr;
        cudaError_t e = cudaMalloc(&f, sizeof(cufftDoubleComplex) * (size_t)N);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_last_error("cudaMalloc(FFT buffer) failed: %s", cudaGetErrorString(e));
            return PFAST_ERR_NOMEM;
        }
        inv->allocs.push_back(f);
        inv->fbuf = static_cast<cufftDoubleComplex*>(f);
    }
    PFAST_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&inv->h_part), sizeof(double) * 2 * kRedBlocks));
    // wavenumbers: columns (dx), rows (dy in 3D, dz in 2D), z (dz, 3D)
    std::vector<double> kx, ky, kz;
    if (inv->dim == 2) {
        kx = kvec(inv->nc, inv->sv2->dx);
        ky = kvec(inv->nr, inv->sv2->dz);
        kz = {0.0};
    } else {
        kx = kvec(inv->nc, inv->sv3->dx);
        ky = kvec(inv->nr, inv->sv3->dy);
        kz = kvec(inv->nz, inv->sv3->dz);
    }
    INV_TRY(dalloc(inv, &inv->kx, (long long)kx.size()));
    INV_TRY(dalloc(inv, &inv->ky, (long long)ky.size()));
    INV_TRY(dalloc(inv, &inv->kz, (long long)kz.size()));
    INV_TRY(upload(inv, inv->kx, kx.data(), kx.size()));
    INV_TRY(upload(inv, inv->ky, ky.data(), ky.size()));
    INV_TRY(upload(inv, inv->kz, kz.data(), kz.size()));
    cufftResult r = inv->dim == 2 ? cufftPlan2d(&inv->plan, inv->nr, inv->nc, CUFFT_Z2Z)
                                  : cufftPlan3d(&inv->plan, inv->nz, inv->nr, inv->nc, CUFFT_Z2Z);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftPlan");
    inv->have_plan = true;
    r = cufftSetStream(inv->plan, inv->ctx->stream);
    if (r != CUFFT_SUCCESS) return cufft_fail(r, "cufftSetStream");
    INV_TRY(upload(inv, inv->vp, vp, (size_t)N));
    if (WR) INV_TRY(upload(inv, inv->WR, WR, (size_t)N));
    PFAST_CUDA_TRY(cudaMemsetAsync(inv->Djk1, 0, sizeof(double) * N, inv->ctx->stream));
    PFAST_CUDA_TRY(cudaMemsetAsync(inv->dk, 0, sizeof(double) * N, inv->ctx->stream));
    PFAST_CUDA_TRY(cudaMemsetAsync(inv->sk, 0, sizeof(double) * N * LM, inv->ctx->stream));
    PFAST_CUDA_TRY(cudaMemsetAsync(inv->yk, 0, sizeof(double) * N * LM, inv->ctx->stream));
    PFAST_CUDA_TRY(cudaStreamSynchronize(inv->ctx->stream));
    inv->rho.assign(LM, 0.0);
    inv->ai.assign(LM, 0.0);
    return PFAST_OK;
}

void release(pfast_inversion* inv) {
    if (!inv) return;
    if (inv->ctx) {
        cudaSetDevice(inv->ctx->device);
        cudaStreamSynchronize(inv->ctx->stream);
    }
    if (inv->have_plan) cufftDestroy(inv->plan);
    for (void* p : inv->allocs) cudaFree(p);
    if (inv->h_part) cudaFreeHost(inv->h_part);
    delete inv;
}

const double* field_ptr(const pfast_inversion* inv, int field) {
    switch (field) {
        case PFAST_INV_VP: return inv->vp;
        case PFAST_INV_GRAD_RAW: return inv->g_raw;
        case PFAST_INV_GRAD: return inv->Djk1;
        case PFAST_INV_DIRECTION: return inv->dk;
        case PFAST_INV_GR_RAW: return inv->dim == 2 ? inv->gR : nullptr;
        case PFAST_INV_GR: return inv->gR_af;
        case PFAST_INV_GT_RAW: return inv->dim == 2 ? inv->gT : nullptr;
        case PFAST_INV_GT: return inv->gT_af;
    }
    return nullptr;
}

}  // namespace

extern "C" {

void pfast_invert_default_options(int dim, pfast_invert_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    pfast_default_options(&o->eval);
    o->eval.maxswp = dim == 2 ? 500 : 100;   // MAXSwp, src/RT_PFAST2D.cpp:75, src/T_PFAST3D.cpp:69
    o->schemetag = PFAST_SCHEME_LBFGS;
    o->lsrc = PFAST_LS_SECANT_WOLFE;
    o->LM = 5;
    o->max_linesearch = dim == 2 ? 5 : 2;    // MAXLineSch
    o->rttag = PFAST_RT_JOINT;
    // 2D: the driver's initial nux, nuy (src/RT_PFAST2D.cpp:79; its nuy weights the rows, here nuz);
    // 3D: the values of the shipped 3D example input (par/Field3D.inp)
    o->nux = dim == 2 ? 80.0 : 200.0;
    o->nuy = dim == 2 ? 0.0 : 200.0;
    o->nuz = dim == 2 ? 50.0 : 10.0;
    o->minv = dim == 2 ? 1600.0 : 1400.0;    // MINV / MAXV, src/RT_padjoint2d.h:13-21, src/T_padjoint3d.h:17-21
    o->maxv = dim == 2 ? 4500.0 : 8000.0;
    o->conv_tol = dim == 2 ? 1e-3 : 1e-2;    // check_conv thresholds
    o->keep_components = 0;
}

pfast_status pfast_inversion2d_create(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const double* WR,
                                      const pfast_invert_options* opt, pfast_inversion** out) {
    if (!ctx || !sv || !vp || !WR || !opt || !out) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    *out = nullptr;
    if (!sv->has_picks) { set_last_error("survey has no picks: gradient unavailable"); return PFAST_ERR_INVALID; }
    INV_TRY(validate(opt, 2));
    pfast_inversion* inv = new pfast_inversion();
    inv->ctx = ctx;
    inv->dim = 2;
    inv->sv2 = sv;
    inv->o = *opt;
    inv->nz = 1;
    inv->nr = sv->nr;
    inv->nc = sv->nc;
    inv->N = (long long)sv->nr * sv->nc;
    pfast_status s = setup(inv, vp, WR);
    if (s != PFAST_OK) {
        release(inv);
        return s;
    }
    *out = inv;
    return PFAST_OK;
}

pfast_status pfast_inversion3d_create(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp,
                                      const pfast_invert_options* opt, pfast_inversion** out) {
    if (!ctx || !sv || !vp || !opt || !out) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    *out = nullptr;
    if (!sv->has_picks) { set_last_error("survey has no picks: gradient unavailable"); return PFAST_ERR_INVALID; }
    INV_TRY(validate(opt, 3));
    pfast_inversion* inv = new pfast_inversion();
    inv->ctx = ctx;
    inv->dim = 3;
    inv->sv3 = sv;
    inv->o = *opt;
    inv->o.schemetag = PFAST_SCHEME_LBFGS;   // src/T_PFAST3D.cpp:428
    inv->o.keep_components = 0;
    inv->nz = sv->nz;
    inv->nr = sv->nr;
    inv->nc = sv->nc;
    inv->N = (long long)sv->nz * sv->nr * sv->nc;
    pfast_status s = setup(inv, vp, nullptr);
    if (s != PFAST_OK) {
        release(inv);
        return s;
    }
    *out = inv;
    return PFAST_OK;
}

pfast_status pfast_inversion_resume(pfast_inversion* inv, int k, const double* grad_prev, const double* grad_cur,
                                    const double* E_hist, int nE, double alpha1) {
    if (!inv || !grad_prev || !grad_cur || !E_hist) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    if (inv->iter != 0) { set_last_error("resume must come before the first step"); return PFAST_ERR_INVALID; }
    if (k < 1 || nE < k + 1) {
        set_last_error("resume after k = %d iterations needs k >= 1 and %d misfits (got %d)", k, k + 1, nE);
        return PFAST_ERR_INVALID;
    }
    PFAST_CUDA_TRY(cudaSetDevice(inv->ctx->device));
    INV_TRY(upload(inv, inv->Djk1, grad_prev, (size_t)inv->N));
    INV_TRY(upload(inv, inv->dk, grad_prev, (size_t)inv->N));
    INV_TRY(upload(inv, inv->g_raw, grad_cur, (size_t)inv->N));
    PFAST_CUDA_TRY(cudaStreamSynchronize(inv->ctx->stream));
    inv->globalE.assign(E_hist, E_hist + k + 1);   // later iterations overwrite what follows
    inv->alpha1 = alpha1;
    inv->iter = k;
    inv->resume_pending = true;
    return PFAST_OK;
}

pfast_status pfast_inversion_step(pfast_inversion* inv, pfast_invert_report* rep) {
    if (!inv || !rep) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    return step(inv, rep);
}

pfast_status pfast_inversion_field(pfast_inversion* inv, int field, const double** dev) {
    if (!inv || !dev) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    const double* p = field_ptr(inv, field);
    if (!p) { set_last_error("field %d not available for this inversion", field); return PFAST_ERR_INVALID; }
    *dev = p;
    return PFAST_OK;
}

pfast_status pfast_inversion_get(pfast_inversion* inv, int field, double* host) {
    if (!inv || !host) { set_last_error("null argument"); return PFAST_ERR_INVALID; }
    const double* p = field_ptr(inv, field);
    if (!p) { set_last_error("field %d not available for this inversion", field); return PFAST_ERR_INVALID; }
    PFAST_CUDA_TRY(cudaSetDevice(inv->ctx->device));
    PFAST_CUDA_TRY(cudaMemcpyAsync(host, p, sizeof(double) * inv->N, cudaMemcpyDeviceToHost, inv->ctx->stream));
    PFAST_CUDA_TRY(cudaStreamSynchronize(inv->ctx->stream));
    return PFAST_OK;
}

pfast_status pfast_inversion_destroy(pfast_inversion* inv) {
    release(inv);
    return PFAST_OK;
}

}  // extern "C"
