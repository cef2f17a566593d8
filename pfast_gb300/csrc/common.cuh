// common.cuh -- shared definitions of the pfast_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>

#include "../../include/pfast_gb300.h"

namespace pfast {

// The reference's "infinity" for unreached nodes (INF macro, src/T_pfsm3d.h:12-14).
constexpr double kInf = 9999999.0;
// isconv tolerance (src/T_pfsm3d.h:126, src/RT_pfsm2d.h:112).
constexpr double kConvTol = 1e-9;
// Default polish floor: FP64 polish corrections at or below this (seconds, or relative to
// 1 + |lambda| for the adjoint) are dropped, so converged regions reach a bitwise fixed
// point; an order of magnitude under the 1e-9 convergence tolerance.
constexpr float kPolishFloor = 1e-10f;

// ---------------------------------------------------------------- 3D tiles
// One warp sweeps one TK x TI x TJ tile.  Lane = (lk, li), TK*TI == 32; each lane
// walks its own j-pencil, starting one step after its upstream lanes, so the lanes
// of a step form one anti-diagonal hyperplane lk+li+lj = t of the tile.
constexpr int TK = 4, TI = 8, TJ = 32;
static_assert(TK * TI == 32, "one lane per (k,i) pencil");
// Halo box in shared memory: (TK+2) planes x (TI+2) rows x (TJ+2) columns.  The plane
// stride PS is padded so that the 32 lanes of a diagonal step hit distinct banks
// (address = lk*(PS-1) + li*(HJ-1) + t with HJ-1 = 33 = 1 mod 32 and PS-1 = 8 mod 32).
constexpr int HK = TK + 2, HI = TI + 2, HJ = TJ + 2, PS = 361;
static_assert(PS >= HI * HJ && (PS - 1) % 32 == 8 && (HJ - 1) % 32 == 1, "bank-conflict-free stride");
// Interior tile (the forward's staged slowness) layout, flipped like the box: [TK][SPS] with rows of SJ.
constexpr int SJ = TJ + 2, SPS = 297;
static_assert(SPS >= TI * SJ && (SPS - 1) % 32 == 8, "bank-conflict-free stride");
// Tile shapes.  One warp sweeps a TK x TI x TJ tile, lane = (kf, if) with TK*TI = 32, TJ = 32;
// the halo box's plane stride PS is the smallest >= HI*HJ with PS - 1 = TI (mod 32), so that the
// lanes of a wavefront step, at kf*(PS-1) + if*(HJ-1) + t, hit 32 distinct banks; the staged
// interior tile's plane stride SPS likewise.  Shape 0 is 4x8x32 (the constants above), shape 1
// 8x4x32: the same 1024 nodes and 42 wavefront steps, half as many tiles along z and twice as
// many along the rows.
template <int TK_, int TI_>
struct TileShape {
    static constexpr int TK = TK_, TI = TI_, TJ = 32;
    static constexpr int HK = TK + 2, HI = TI + 2, HJ = TJ + 2;
    static constexpr int PS = HI * HJ + ((TI + 1 - HI * HJ) % 32 + 32) % 32;
    static constexpr int SJ = TJ + 2;
    static constexpr int SPS = TI * SJ + ((TI + 1 - TI * SJ) % 32 + 32) % 32;
    static_assert(TK * TI == 32 && (PS - 1) % 32 == TI && (HJ - 1) % 32 == 1 && (SPS - 1) % 32 == TI,
                  "bank-conflict-free strides");
};
using Shape48 = TileShape<4, 8>;
using Shape84 = TileShape<8, 4>;
static_assert(Shape48::PS == PS && Shape48::SPS == SPS && Shape48::TK == TK && Shape48::TI == TI, "shape 0");
constexpr int kTileShapes = 2;
__host__ __device__ constexpr int shape_tk(int shape) { return shape ? Shape84::TK : Shape48::TK; }
__host__ __device__ constexpr int shape_ti(int shape) { return shape ? Shape84::TI : Shape48::TI; }
// Inside code templated on a shape SH: its constants under the usual names.
#define PFAST_TILE_SHAPE(SH)                                                                          \
    constexpr int TK = SH::TK, TI = SH::TI, TJ = SH::TJ, HK = SH::HK, HI = SH::HI, HJ = SH::HJ;       \
    constexpr int PS = SH::PS, SJ = SH::SJ, SPS = SH::SPS;                                           \
    (void)TK; (void)TI; (void)TJ; (void)HK; (void)HI; (void)HJ; (void)PS; (void)SJ; (void)SPS

// Warps (tiles) per CTA.
constexpr int kDataflowMaxTiles = 8192;   // tiles per instance the dataflow kernel keeps in shared memory
constexpr int kWarps3 = 1;   // one-warp CTAs: the finest shared-memory granularity, hence the most warps per SM

// ---------------------------------------------------------------- 2D tiles
// One warp sweeps one T2I x T2J tile; lane = row, pencil along j.
constexpr int T2I = 32, T2J = 64;
constexpr int H2I = T2I + 2, H2J = T2J + 2;
// Row stride: lane li at step t touches li*(R2-1) + t; R2-1 = 65 = 1 mod 32 puts the
// 32 lanes of a step on 32 distinct banks.
constexpr int R2 = 66 + 0;
static_assert(R2 >= H2J && (R2 - 1) % 32 == 1, "bank-conflict-free row stride");
constexpr int kWarps2 = 4;

// Spacing constants, axis 0 = x (columns j, dx), 1 = y (rows i, dy), 2 = z (k, dz).
// inv2[a] = (1.0/d)/d exactly as the reference forms 1.0/da/da (src/T_pfsm3d.h:115).
struct Spacing3 {
    double d[3];
    double d2[3];    // d*d
    double inv2[3];  // (1.0/d)/d
    // FP32 constants of the fast kernels, computed on the host so that no FP64
    // instruction runs in an FP32 kernel: w = 1/d^2, rp[a] = 1/(W - w[a]), rW = 1/W.
    float df[3], wf[3], rpf[3], rWf;
    int iso;         // dx == dy == dz
};

// Bit-pattern helpers.  For doubles >= +0 (including +inf) the IEEE bit patterns
// order like the values, so comparisons and minima of traveltimes can run on the
// integer pipe (FP64 issue slots are scarce on this part).
__device__ __forceinline__ long long dbits(double x) { return __double_as_longlong(x); }
// (x < y) ? x : y for x, y >= +0: the reference's MIN macro
__device__ __forceinline__ double min_nonneg(double x, double y) { return dbits(x) < dbits(y) ? x : y; }
// max(e, 0) and min(e, 0) by the sign bit
__device__ __forceinline__ double pos_sign(double e) { return __double2hiint(e) < 0 ? 0.0 : e; }
__device__ __forceinline__ double neg_sign(double e) { return __double2hiint(e) < 0 ? e : 0.0; }

// FP64 <-> FP32 conversions on the integer pipe, from the IEEE 754 binary64/binary32
// layouts (sign | exponent | fraction; biases 1023 and 127).  narrow_trunc keeps the top
// 23 fraction bits (truncation); magnitudes below 2^-126 give 0 and above 2^127 give
// +-FLT_MAX.  widen_exact is exact for normal floats and maps zero and subnormals to 0.
// They serve the polish updates, whose step sizes and derivative scales need FP32
// precision only.
__device__ __forceinline__ float narrow_trunc(double x) {
    const long long b = dbits(x);
    const unsigned hi = (unsigned)((unsigned long long)b >> 32), lo = (unsigned)b;
    const unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
    if (mag < (897u << 20)) return 0.0f;
    if (mag >= (1151u << 20)) return __uint_as_float(sign | 0x7f7fffffu);
    return __uint_as_float(sign | ((mag - (896u << 20)) << 3) | (lo >> 29));
}
// (float)(v - r) for doubles v, r >= 0 without an FP64 instruction: each is split on the
// integer pipe into h + l (h: its top 24 significant bits, l: the next 29 bits rounded down to
// an FP32 value), and (h_v - h_r) + (l_v - l_r) is formed in FP32.  The heads' difference is
// exact when v and r are within a factor 2 (Sterbenz), so the result has the difference's
// FP32 precision although v and r are large (the FP32 kernels' traveltime offsets).
__device__ __forceinline__ float2 split_hl(double x) {
    const unsigned long long b = (unsigned long long)dbits(x);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const unsigned mag = hi & 0x7fffffffu;
    if (mag < (897u << 20)) return make_float2(0.0f, 0.0f);   // below 2^-126: negligible here
    const float h = __uint_as_float(((mag - (896u << 20)) << 3) | (lo >> 29));
    const unsigned r = lo & 0x1fffffffu;
    if (r == 0u) return make_float2(h, 0.0f);
    const int n = __clz(r);   // r's leading one at bit 31 - n
    const int e = (int)(mag >> 20) - 1023 - 52 + (31 - n);
    if (e < -126) return make_float2(h, 0.0f);
    const unsigned frac = (unsigned)(((unsigned long long)r << (n + 1)) & 0xffffffffull) >> 9;
    return make_float2(h, __uint_as_float(((unsigned)(e + 127) << 23) | frac));
}
__device__ __forceinline__ float offset_f32(double v, double r) {
    const float2 a = split_hl(v), c = split_hl(r);
    return (a.x - c.x) + (a.y - c.y);
}

__device__ __forceinline__ double widen_exact(float f) {
    const unsigned u = __float_as_uint(f), mag = u & 0x7fffffffu;
    if (mag < 0x00800000u) return 0.0;
    return __hiloint2double((int)((u & 0x80000000u) | ((mag >> 3) + (896u << 20))), (int)(mag << 29));
}

// Which kernel flavour a sweep runs.
enum SweepKind : int {
    kFwdPlain64 = 0,   // reference arithmetic, FP64, U = min(U, q)
    kFwdFast32 = 1,    // FP32 bulk sweeps
    kFwdPolish64 = 2,  // FP64 polish from a near-converged field
    kAdjPlain64 = 3,   // reference arithmetic, FP64
    kAdjFast32 = 4,    // FP32 bulk adjoint sweeps
    kAdjPolish64 = 5,  // FP64 adjoint polish
};

}  // namespace pfast

// Return a failing pfast_status from the enclosing function.
#define PFAST_TRY(expr)                          \
    do {                                         \
        pfast_status s__ = (expr);               \
        if (s__ != PFAST_OK) return s__;         \
    } while (0)

#define PFAST_CUDA_TRY(expr)                                                        \
    do {                                                                            \
        cudaError_t e__ = (expr);                                                   \
        if (e__ != cudaSuccess) return ::pfast::cuda_fail(e__, #expr, __FILE__, __LINE__); \
    } while (0)

namespace pfast {
pfast_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);
void set_last_error(const char* fmt, ...);
}  // namespace pfast
