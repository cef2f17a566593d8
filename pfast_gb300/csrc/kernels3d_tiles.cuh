// kernels3d_tiles.cuh -- the 3D sweep kernels (per-diagonal and dataflow), their tile I/O and
// node updates, and their launchers, templated on the tile shape (common.cuh: TileShape).
// Included by kernels3d.cu (shape 4x8x32) and kernels3d_s84.cu (shape 8x4x32), which each
// instantiate ShapeLaunchers for their shape, so the two shapes compile in parallel.
//
// Sweep scheme.  The reference sweeps the grid lexicographically in 8 orders
// (src/T_pfsm3d.h:158-178, src/T_padjoint3d.h:139-161).  In sweep order
// (s3,s1,s2) a node sees its three upstream neighbours (k-s3, i-s1, j-s2) already
// updated in this sweep and its three downstream neighbours not yet updated.  Any
// visiting order with that property gives the same values, so this file visits
// tiles on anti-diagonal tile hyperplanes (one launch per tile-diagonal, tiles of a
// diagonal in parallel) and, inside a tile, nodes on anti-diagonal node hyperplanes
// (one warp step per hyperplane).  The result of every node is the reference's.
//
// Flavours: kFwdPlain64 / kAdjPlain64 evaluate the reference's expressions in the
// reference's order (the library is built with -fmad=false, so no FMA contraction):
// bit-identical results.  kFwdFast32 / kAdjFast32 are the FP32 bulk sweeps and run
// no FP64 instruction.  kFwdPolish64 / kAdjPolish64 are the FP64 polish sweeps in
// residual-correction form: the local residual is formed in FP64 and the correction
// step in FP32, so the fixed point is the FP64 one while FP64 issue slots (about 2
// lanes per clock per SM on this part) go only where the precision is needed.

#pragma once

#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>
#include <algorithm>
#include <type_traits>
#include "kernels.h"
#include "dataflow3.h"

namespace pfast {

namespace {


template <int KIND> struct Traits;
template <> struct Traits<kFwdPlain64>   { using Real = double; using Aux = double; static constexpr bool adj = false; };
template <> struct Traits<kFwdFast32>    { using Real = float;  using Aux = float;  static constexpr bool adj = false; };
template <> struct Traits<kFwdPolish64>  { using Real = double; using Aux = double; static constexpr bool adj = false; };
template <> struct Traits<kAdjPlain64>   { using Real = double; using Aux = double; static constexpr bool adj = true; };
template <> struct Traits<kAdjFast32>    { using Real = float;  using Aux = float;  static constexpr bool adj = true; };
template <> struct Traits<kAdjPolish64>  { using Real = double; using Aux = double; static constexpr bool adj = true; };

// Whether the adjoint's traveltime is read through register windows and warp shuffles
// (FP64 kinds, whose two FP64 boxes would halve the resident warps) or staged as a halo
// box like the field (FP32 bulk: a small box, and a coalesced load beats per-lane reads).
template <int KIND>
__host__ __device__ constexpr bool t_windows() {
    return Traits<KIND>::adj && sizeof(typename Traits<KIND>::Aux) == 8;
}

// Whether the field itself is kept in register windows instead of a shared-memory halo box
// (forward polish in the dataflow kernel, COHERENT).  A lane holds its pencil's new value at
// jf-1 and old values at jf .. jf+3 (loads issued three steps ahead); the upstream lanes' new
// values and the downstream lanes' old values come by warp shuffle, the face halo pencils from
// owner lanes, and each changed node is stored as it is updated.  The warp then needs no shared
// memory, so a dataflow block holds 24 (forward) or 16 (adjoint) warps instead of 11 boxes of
// 17 KB (3D gradient workload: forward polish 167 -> 151 ms, adjoint polish 155 -> 125 ms).
// The per-diagonal launches keep the box: with windows their forward polish ran slower
// (159 -> 179 ms).
template <int KIND, bool COHERENT>
__host__ __device__ constexpr bool u_windows() {
    return (KIND == kFwdPolish64 || KIND == kAdjPolish64) && COHERENT;
}

// Shared memory per warp: the field's halo box, plus the FP32 bulk adjoint's traveltime
// box.  The forward's slowness is read per node through L1 (each lane walks its own row,
// so a fetched line serves the next steps).
// FP32 forward: the tile's slowness is staged in shared memory beside the box (interior tile,
// flipped like the box), so that a wavefront step reads it there instead of issuing a global
// load per node: with most of the SM's shared memory holding tile boxes, the L1 is too small to
// keep the slowness lines of the resident tiles, and every such load went to L2 on the step's
// dependency chain (3D gradient workload: FP32 forward 139 -> 116 ms per evaluation).  The FP64
// kinds keep the per-node load: their staged tile (9.5 KB) would cost a third of the resident
// warps, which was slower (forward polish 159 -> 197 ms).
template <int KIND>
__host__ __device__ constexpr bool stage_slowness() {
    return KIND == kFwdFast32;
}

template <int KIND, class SH, bool COHERENT = false>
__host__ __device__ constexpr int warp_smem_bytes() {
    using T = Traits<KIND>;
    if (u_windows<KIND, COHERENT>()) return 16;   // no box
    return int(SH::HK * SH::PS * sizeof(typename T::Real) +
               (T::adj && !t_windows<KIND>() ? SH::HK * SH::PS * sizeof(typename T::Aux) : 0) +
               (stage_slowness<KIND>() ? SH::TK * SH::SPS * sizeof(typename T::Aux) : 0));
}



// ----------------------------------------------------------- node updates
// Reference Godunov update (src/T_pfsm3d.h:99-119).  a/b/c: neighbour minima along
// x/y/z; s: slowness 1.0/vp (precomputed, bit-identical to the reference's per-node
// division).  Expressions keep the reference's operand order; the ordering tests
// run on the bit patterns (same outcome for non-negative values).
__device__ __forceinline__ double eik3_plain(double a, double b, double c, double s, const Spacing3& sp) {
    double da = sp.d[0], db = sp.d[1], dc = sp.d[2];
    double ia = sp.inv2[0], ib = sp.inv2[1], ic = sp.inv2[2];
    double t;
    if (dbits(b) > dbits(a)) { t = a; a = b; b = t; t = da; da = db; db = t; t = ia; ia = ib; ib = t; }
    if (dbits(c) > dbits(a)) { t = a; a = c; c = t; t = da; da = dc; dc = t; t = ia; ia = ic; ic = t; }
    if (dbits(c) > dbits(b)) { t = b; b = c; c = t; t = db; db = dc; dc = t; t = ib; ib = ic; ic = t; }
    double q = dc * s + c;
    if (dbits(q) <= dbits(b)) return q;
    double A = dc * dc + db * db;
    double B = -2. * (b * dc * dc + c * db * db);
    double C = dc * dc * b * b + db * db * c * c - db * db * dc * dc * s * s;
    double D = B * B - 4. * A * C;
    q = (D >= 0) ? (-B + sqrt(D)) / 2. / A : kInf;
    if (dbits(q) <= dbits(a)) return q;
    A = ia + ib + ic;   // 1.0/da/da + 1.0/db/db + 1.0/dc/dc, each term precomputed as (1.0/d)/d
    B = -2.0 * (a / da / da + b / db / db + c / dc / dc);
    C = a * a / da / da + b * b / db / db + c * c / dc / dc - s * s;
    D = B * B - 4. * A * C;
    q = (D >= 0) ? (-B + sqrt(D)) / 2. / A : kInf;
    return q;
}

// FP32 Godunov solution in difference form relative to the smallest neighbour c
// (x = q - c), with FMA and host-precomputed reciprocals:
//   1 term:  x = dc*s
//   2 terms: x = (wb*B + sqrt((wb+wc) s^2 - wb wc B^2)) / (wb+wc),         B = b-c
//   3 terms: x = (wa*A + wb*B + sqrt(W s^2 - wa wb (A-B)^2 - wa wc A^2 - wb wc B^2)) / W,  A = a-c
__device__ __forceinline__ float eik3_fast(float a, float b, float c, float s, const Spacing3& K) {
    float da = K.df[0], db = K.df[1], dc = K.df[2];
    float wa = K.wf[0], wb = K.wf[1], wc = K.wf[2];
    float ra = K.rpf[0], rb = K.rpf[1], rc = K.rpf[2];
    float t;
    if (b > a) { t = a; a = b; b = t; t = da; da = db; db = t; t = wa; wa = wb; wb = t; t = ra; ra = rb; rb = t; }
    if (c > a) { t = a; a = c; c = t; t = da; da = dc; dc = t; t = wa; wa = wc; wc = t; t = ra; ra = rc; rc = t; }
    if (c > b) { t = b; b = c; c = t; t = db; db = dc; dc = t; t = wb; wb = wc; wc = t; t = rb; rb = rc; rc = t; }
    float q = fmaf(dc, s, c);
    if (q <= b) return q;
    const float s2 = s * s;
    const float B = b - c;
    const float wbB = wb * B;
    const float D = fmaf(wb + wc, s2, -wbB * wc * B);
    q = (D >= 0.f) ? c + (wbB + sqrtf(D)) * ra : (float)kInf;
    if (q <= a) return q;
    const float A = a - c;
    const float AB = A - B;
    const float W = wa + wb + wc;
    const float D3 = W * s2 - (wa * wb * AB * AB + wa * wc * A * A + wb * wc * B * B);
    return (D3 >= 0.f) ? c + (fmaf(wa, A, wbB) + sqrtf(D3)) * K.rWf : (float)kInf;
}

// Square root by the hardware approximation (PTX sqrt.approx.f32, a few ulps): the FP32 bulk
// result is only the starting point of the FP64 polish.
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// The same solution on an isotropic grid (one spacing h): unit weights, sh = s h, the three
// neighbour minima sorted by min/max (values >= 0 or +inf: no NaN arises), so
//   2 terms: x = (B + sqrt(2 sh^2 - B^2)) / 2
//   3 terms: x = (A + B + sqrt(3 sh^2 - (A-B)^2 - A^2 - B^2)) / 3.
// All three candidates are formed and the first admissible one selected, without branches: in a
// wavefront step the lanes' nodes fall into different cases, so a branching form runs the
// union of the paths with divergence bookkeeping anyway.  The selected value is the same
// expression as in the branching form, bit for bit (candidates from unreached neighbours may
// be inf or NaN; they are never selected).
__device__ __forceinline__ float eik3_fast_iso(float a, float b, float c, float sh) {
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    const float c0 = fminf(lo, c), mid = fmaxf(lo, c);
    const float b0 = fminf(hi, mid), a0 = fmaxf(hi, mid);
    const float q1 = c0 + sh;
    const float B = b0 - c0;
    const float D = fmaf(2.0f * sh, sh, -B * B);
    const float q2 = (D >= 0.f) ? fmaf(0.5f, B + sqrt_approx(D), c0) : (float)kInf;
    const float A = a0 - c0, AB = A - B;
    const float D3 = fmaf(3.0f * sh, sh, -fmaf(AB, AB, fmaf(A, A, B * B)));
    const float q3 = (D3 >= 0.f) ? fmaf(1.0f / 3.0f, (A + B) + sqrt_approx(D3), c0) : (float)kInf;
    return q1 <= b0 ? q1 : (q2 <= a0 ? q2 : q3);
}

// narrow_trunc for 0 <= x < 2^128 (traveltime differences): no sign, no overflow clamp.
__device__ __forceinline__ float narrow_pos(double x) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    return hi < (897u << 20) ? 0.0f : __uint_as_float(((hi - (896u << 20)) << 3) | (lo >> 29));
}

// FP64 polish Godunov update: one Newton step from the current value U0 on
//   f(q) = sum_m w_m max(q - a_m, 0)^2 - s^2,
// whose root is the Godunov value (the 1-, 2- and 3-term cases of
// src/T_pfsm3d.h:106-118 are the pieces of f).  f in FP64, the step f/f' in FP32.
// s2 = s^2 (precomputed); the rare restart branch (U0 at or below every
// neighbour) takes the 1-term value with the slowness itself.
// big: the step leaves a second-order remainder (about sum_active(w) step^2 / f') above the
// floor, so the node wants another Newton step in the same order.
__device__ __forceinline__ double eik3_newton(double U0, double a, double b, double c, double s2, const double* slow,
                                              long long node, const Spacing3& sp, float floor, bool& big,
                                              float& dstep) {
    // FP64 for what fixes the root (the differences and the residual f, 7 FP64 instructions
    // in the isotropic case); the derivative f' and the step in FP32.  Isotropic grids: s2 holds
    // (s h)^2 and f is the residual divided by 1/h^2 (same root, unit weights).
    const double px = pos_sign(U0 - a), py = pos_sign(U0 - b), pz = pos_sign(U0 - c);
    double f;
    float wx, wy, wz;
    if (sp.iso) {
        f = fma(px, px, fma(py, py, fma(pz, pz, -s2)));
        wx = wy = wz = 1.0f;
    } else {
        f = fma(sp.inv2[0] * px, px, fma(sp.inv2[1] * py, py, fma(sp.inv2[2] * pz, pz, -s2)));
        wx = sp.wf[0]; wy = sp.wf[1]; wz = sp.wf[2];
    }
    const float fx = narrow_pos(px), fy = narrow_pos(py), fz = narrow_pos(pz);
    const float fp = 2.0f * (wx * fx + wy * fy + wz * fz);
    if (!(fp > 0.0f)) {
        big = true;
        dstep = INFINITY;   // a restart: the change is not a Newton step
        const double s = __ldg(slow + node);
        return fmin(fma(sp.d[0], s, a), fmin(fma(sp.d[1], s, b), fma(sp.d[2], s, c)));
    }
    const float step = __fdividef(narrow_trunc(f), fp);
    const float sw = (dbits(px) > 0 ? wx : 0.0f) + (dbits(py) > 0 ? wy : 0.0f) +
                     (dbits(pz) > 0 ? wz : 0.0f);   // p >= 0: integer tests keep the FP64 pipe free
    big = sw * step * step > floor * fp;
    dstep = fabsf(step);   // the change of the node, to FP32 precision
    // corrections far below the 1e-9 convergence tolerance are dropped, so that a
    // converged region reaches a bitwise fixed point (and its tiles lock)
    return fabsf(step) <= floor ? U0 : U0 - widen_exact(step);
}

// Adjoint updates.  The reference's upwind formula (src/T_padjoint3d.h:51-66)
// collapses, with w = 1/d^2 of each neighbour's axis and e_m = T_m - T0, to
//   den = sum_m w_m max(-e_m, 0),   num = sum_m w_m max(e_m, 0) lambda_m,   lambda = num / den
// (POS(-(T_p-T0)/d)/d = w max(-e_p,0), -NEG(-(T0-T_m)/d)/d = w max(-e_m,0),
//  POS(-(T0-T_m)/d)/d = w max(e_m,0), -NEG(-(T_p-T0)/d)/d = w max(e_p,0)).

// Reference adjoint update (src/T_padjoint3d.h:42-71); operand order kept.
__device__ __forceinline__ double pos_ref(double x) { return (x + fabs(x)) / 2.0; }   // POS macro
__device__ __forceinline__ double neg_ref(double x) { return (x - fabs(x)) / 2.0; }   // NEG macro
__device__ __forceinline__ bool unreached64(double T0, double a, double b, double c, double d, double e, double f) {
    const long long inf = dbits(kInf);   // T >= INF, on the bit patterns (T >= 0)
    return dbits(T0) >= inf || dbits(a) >= inf || dbits(b) >= inf || dbits(c) >= inf || dbits(d) >= inf ||
           dbits(e) >= inf || dbits(f) >= inf;
}

__device__ __forceinline__ double adj3_plain(double T0, double Txp, double Txm, double Typ, double Tym,
                                             double Tzp, double Tzm, double Lxp, double Lxm, double Lyp,
                                             double Lym, double Lzp, double Lzm, const Spacing3& sp) {
    if (unreached64(T0, Txp, Txm, Typ, Tym, Tzp, Tzm)) return 0.0;
    const double dx = sp.d[0], dy = sp.d[1], dz = sp.d[2];
    const double gxp = -(Txp - T0) / dx, gxm = -(T0 - Txm) / dx;
    const double gyp = -(Typ - T0) / dy, gym = -(T0 - Tym) / dy;
    const double gzp = -(Tzp - T0) / dz, gzm = -(T0 - Tzm) / dz;
    const double a1 = pos_ref(gxp), a2 = neg_ref(gxm);
    const double b1 = pos_ref(gyp), b2 = neg_ref(gym);
    const double c1 = pos_ref(gzp), c2 = neg_ref(gzm);
    const double La1 = pos_ref(gxm) * Lxm, La2 = neg_ref(gxp) * Lxp;
    const double Lb1 = pos_ref(gym) * Lym, Lb2 = neg_ref(gyp) * Lyp;
    const double Lc1 = pos_ref(gzm) * Lzm, Lc2 = neg_ref(gzp) * Lzp;
    const double den = (a1 - a2) / dx + (b1 - b2) / dy + (c1 - c2) / dz;
    if (fabs(den) > 1e-9) return ((La1 - La2) / dx + (Lb1 - Lb2) / dy + (Lc1 - Lc2) / dz) / den;
    return 0.0;
}

// FP32 bulk adjoint update (T as FP32 values; unreached nodes hold INF).  A change of
// less than 2^-24 relative keeps the old value, so converged regions reach a bitwise fixed
// point (rounding alone would otherwise keep flipping last bits).  The two neighbours of an
// axis enter as a commutative pair (two products, one sum) and the axes in a fixed order, so
// the bits do not depend on which neighbour the sweep visits first: a node keeps one value
// in all eight sweep orders once its neighbours have settled.
__device__ __forceinline__ float adj3_bulk(float T0, float Ta, float Tb, float Tc, float Td, float Te, float Tf,
                                           float La, float Lb, float Lc, float Ld, float Le, float Lf, float L0,
                                           const Spacing3& sp) {
    // a traveltime at or above INF around the node: lambda 0 (selected at the end, without a
    // branch; the other terms may then be inf or NaN and are discarded)
    const float ti = (float)kInf;
    const bool unreached = fmaxf(fmaxf(fmaxf(T0, Ta), fmaxf(Tb, Tc)), fmaxf(fmaxf(Td, Te), Tf)) >= ti;
    // per axis: den = max(-e1, 0) + max(-e2, 0), num = max(e1, 0) L1 + max(e2, 0) L2
    auto pair = [&](float T1, float L1, float T2, float L2, float& d, float& n) {
        const float e1 = T1 - T0, e2 = T2 - T0;
        d = fmaxf(-e1, 0.f) + fmaxf(-e2, 0.f);
        const float p1 = fmaxf(e1, 0.f) * L1, p2 = fmaxf(e2, 0.f) * L2;
        n = p1 + p2;
    };
    float dx, nx, dy, ny, dz, nz;
    pair(Ta, La, Tb, Lb, dx, nx);   // x neighbours
    pair(Tc, Lc, Td, Ld, dy, ny);   // y
    pair(Te, Le, Tf, Lf, dz, nz);   // z
    float den, num, r;
    if (sp.iso) {   // one weight: it cancels in num / den
        den = (dx + dy) + dz;
        num = (nx + ny) + nz;
        r = (den * sp.wf[0] > 1e-9f) ? __fdividef(num, den) : 0.f;
    } else {
        const float wx = sp.wf[0], wy = sp.wf[1], wz = sp.wf[2];
        den = (wx * dx + wy * dy) + wz * dz;
        num = (wx * nx + wy * ny) + wz * nz;
        r = (fabsf(den) > 1e-9f) ? __fdividef(num, den) : 0.f;
    }
    return unreached ? 0.f : (fabsf(r - L0) <= 5.96e-8f * fabsf(L0) ? L0 : r);
}

// FP64 polish adjoint update in residual-correction form.  With mu_m = lambda_m where
// e_m > 0 and lambda0 where e_m < 0, the residual is
//   r = num - den*lambda0 = sum_m w_m e_m mu_m,
// formed in FP64 (the differences e_m are exact, Sterbenz); den = -sum_m w_m min(e_m, 0)
// only scales the step r/den and is formed in FP32, as is the step.  The fixed point is
// r = 0 in FP64.  13 FP64 instructions in the isotropic case.
__device__ __forceinline__ double adj3_polish(double T0, double Txp, double Txm, double Typ, double Tym, double Tzp,
                                              double Tzm, double Lxp, double Lxm, double Lyp, double Lym, double Lzp,
                                              double Lzm, double L0, const Spacing3& sp, float floor, bool& big,
                                              float& dstep) {
    dstep = INFINITY;   // the branches that reset lambda to 0
    if (unreached64(T0, Txp, Txm, Typ, Tym, Tzp, Tzm)) return 0.0;
    const double exp_ = Txp - T0, exm = Txm - T0, eyp = Typ - T0, eym = Tym - T0, ezp = Tzp - T0, ezm = Tzm - T0;
    auto mu = [&](double e, double L) { return __double2hiint(e) < 0 ? L0 : L; };
    auto nf = [](double e) {   // max(-e, 0), narrowed from the magnitude's bits (|e| < 2^128)
        const int hi = __double2hiint(e);
        const unsigned mag = (unsigned)hi & 0x7fffffffu, lo = (unsigned)__double2loint(e);
        return hi < 0 && mag >= (897u << 20) ? __uint_as_float(((mag - (896u << 20)) << 3) | (lo >> 29)) : 0.0f;
    };
    double r;
    float den;
    if (sp.iso) {
        r = fma(exp_, mu(exp_, Lxp), fma(exm, mu(exm, Lxm), fma(eyp, mu(eyp, Lyp),
            fma(eym, mu(eym, Lym), fma(ezp, mu(ezp, Lzp), ezm * mu(ezm, Lzm))))));
        den = ((nf(exp_) + nf(exm)) + (nf(eyp) + nf(eym))) + (nf(ezp) + nf(ezm));
        if (!(den * sp.wf[0] > 1e-9f)) return 0.0;
    } else {
        const double rx = fma(exp_, mu(exp_, Lxp), exm * mu(exm, Lxm));
        const double ry = fma(eyp, mu(eyp, Lyp), eym * mu(eym, Lym));
        const double rz = fma(ezp, mu(ezp, Lzp), ezm * mu(ezm, Lzm));
        r = fma(sp.inv2[0], rx, fma(sp.inv2[1], ry, sp.inv2[2] * rz));
        den = sp.wf[0] * (nf(exp_) + nf(exm)) + sp.wf[1] * (nf(eyp) + nf(eym)) + sp.wf[2] * (nf(ezp) + nf(ezm));
        if (!(den > 1e-9f)) return 0.0;
    }
    const float step = __fdividef(narrow_trunc(r), den);
    const float tol = floor * (1.0f + fabsf(narrow_trunc(L0)));
    big = fabsf(step) * 1.2e-7f > tol;   // the local equation is linear: only the FP32 step's error remains
    dstep = fabsf(step);
    return fabsf(step) <= tol ? L0 : L0 + widen_exact(step);
}

// ----------------------------------------------------------- tile I/O
// A tile's halo box is kept in shared memory in the coordinates of the current sweep order:
// each axis is reversed where the sweep descends, so that every order walks the box the same
// way.  Node (kf, if, jf) of the flipped tile lies at (kf+1)*PS + (if+1)*HJ + jf+1 and its
// flipped upstream neighbours at -PS, -HJ, -1; a wavefront step of lanes (kf, if) touches
// kf*(PS-1) + if*(HJ-1) + t, and with PS-1 = 8, HJ-1 = 1 (mod 32) the 32 lanes hit 32
// distinct banks in every order (in grid coordinates the descending orders meet 2-way
// conflicts).  Halo position z = 0..ek+1 around a tile of ek planes (grid plane k0-1+z) lies
// at flipped zf = z where the sweep ascends along z, else ek+1-z; likewise rows and columns.
//
// load_box: the halo box at origin (k0-1, i0-1, j0-1), one box row per warp instruction
// (lanes along the row, coalesced); out-of-grid entries get `fill`; the rows and columns
// beyond a partial tile's halo are neither loaded nor stored (never read).  Twelve rows are
// loaded before they are stored, to keep many loads in flight.
// COHERENT: the field, which the dataflow kernel itself writes (other warps of the block
// stored the neighbouring tiles): read through L2, not the read-only path.
template <typename T, bool COHERENT, class SH>
__device__ __forceinline__ void load_box(T* box, const T* __restrict__ g, int k0, int i0, int j0, int ek, int ei,
                                         int ej, bool pz, bool py, bool px, int nz, int nr, int nc, T fill, int lane) {
    PFAST_TILE_SHAPE(SH);
    constexpr int NROW = HK * HI;
    constexpr int RB = 12;
    static_assert(NROW % RB == 0 && HJ - 32 <= 32, "row batching");
    const long long plane = (long long)nr * nc;
    const int gj0 = j0 - 1 + lane, gj1 = j0 + 31 + lane;
    const bool s0 = lane <= ej + 1, s1 = lane < HJ - 32 && lane + 32 <= ej + 1;   // within the halo
    const bool c0 = s0 && (unsigned)gj0 < (unsigned)nc;
    const bool c1 = s1 && (unsigned)gj1 < (unsigned)nc;
    const int xf0 = px ? lane : ej + 1 - lane, xf1 = px ? lane + 32 : ej - 31 - lane;
#pragma unroll 1
    for (int rb = 0; rb < NROW; rb += RB) {
        T v0[RB], v1[RB];
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int r = rb + u, z = r / HI, y = r - z * HI;
            const int gk = k0 - 1 + z, gi = i0 - 1 + y;
            const bool rok = z <= ek + 1 && y <= ei + 1 && (unsigned)gk < (unsigned)nz && (unsigned)gi < (unsigned)nr;
            const T* row = g + gk * plane + (long long)gi * nc;
            if constexpr (COHERENT) {
                v0[u] = (rok && c0) ? __ldcg(row + gj0) : fill;
                v1[u] = (rok && c1) ? __ldcg(row + gj1) : fill;
            } else {
                v0[u] = (rok && c0) ? __ldg(row + gj0) : fill;
                v1[u] = (rok && c1) ? __ldg(row + gj1) : fill;
            }
        }
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const int r = rb + u, z = r / HI, y = r - z * HI;
            if (z > ek + 1 || y > ei + 1) continue;
            T* brow = box + (pz ? z : ek + 1 - z) * PS + (py ? y : ei + 1 - y) * HJ;
            if (s0) brow[xf0] = v0[u];
            if (s1) brow[xf1] = v1[u];
        }
    }
}

// Vector form of load_box, for grids whose rows start on 16-byte boundaries (ncols a multiple of
// V = 16 / sizeof(T) and a 16-byte aligned field): box rows are read as aligned V-element vectors
// from grid column j0 - V on, so the halo columns j0 - 1 and j0 + ej come with their vectors
// (a vector lies wholly inside or outside the grid).  The first MV = TJ / V vectors of each row
// (columns j0 - V .. j0 + TJ - V - 1) are read by 32 / MV rows of lanes at a time; the last two
// (columns j0 + TJ - V .. j0 + TJ + V - 1) by 16 rows of lane pairs.  A lane's columns, and so its
// flipped box positions, are fixed for the whole load.
template <typename T, bool COHERENT, class SH>
__device__ __forceinline__ void load_box_vec(T* box, const T* __restrict__ g, int k0, int i0, int j0, int ek, int ei,
                                             int ej, bool pz, bool py, bool px, int nz, int nr, int nc, T fill,
                                             int lane) {
    PFAST_TILE_SHAPE(SH);
    using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int V = 16 / sizeof(T);
    constexpr int MV = TJ / V;          // main vectors per row: 8 (FP32) or 16 (FP64)
    constexpr int RPI = 32 / MV;        // rows per main pass: 4 or 2
    constexpr int NROW = HK * HI;
    const long long plane = (long long)nr * nc;
#pragma unroll
    for (int part = 0; part < 2; ++part) {
        const int q = part == 0 ? lane % MV : MV + (lane & 1);   // the lane's vector in the row
        const int rsub = part == 0 ? lane / MV : lane >> 1;      // its row within a pass
        const int rstep = part == 0 ? RPI : 16;
        const int gx = j0 - V + q * V;                           // grid column of the vector's first element
        const bool vin = gx >= 0 && gx < nc;
        int xf[V];
        bool xs[V];
#pragma unroll
        for (int e = 0; e < V; ++e) {
            const int bx = gx + e - (j0 - 1);                    // halo-box column
            xs[e] = bx >= 0 && bx <= ej + 1;
            xf[e] = px ? bx : ej + 1 - bx;
        }
        constexpr int BATCH = 8;
#pragma unroll 1
        for (int r0 = 0; r0 < NROW; r0 += BATCH * rstep) {
            VT v[BATCH];
#pragma unroll
            for (int u = 0; u < BATCH; ++u) {
                const int r = r0 + u * rstep + rsub, z = r / HI, y = r - z * HI;
                const int gk = k0 - 1 + z, gi = i0 - 1 + y;
                const bool ok = vin && r < NROW && z <= ek + 1 && y <= ei + 1 && (unsigned)gk < (unsigned)nz &&
                                (unsigned)gi < (unsigned)nr;
                const VT* src = reinterpret_cast<const VT*>(g + gk * plane + (long long)gi * nc + gx);
                if (ok) v[u] = COHERENT ? __ldcg(src) : __ldg(src);
                else {
                    T* f = reinterpret_cast<T*>(&v[u]);
#pragma unroll
                    for (int e = 0; e < V; ++e) f[e] = fill;
                }
            }
#pragma unroll
            for (int u = 0; u < BATCH; ++u) {
                const int r = r0 + u * rstep + rsub, z = r / HI, y = r - z * HI;
                if (r >= NROW || z > ek + 1 || y > ei + 1) continue;
                T* brow = box + (pz ? z : ek + 1 - z) * PS + (py ? y : ei + 1 - y) * HJ;
                const T* f = reinterpret_cast<const T*>(&v[u]);
#pragma unroll
                for (int e = 0; e < V; ++e)
                    if (xs[e]) brow[xf[e]] = f[e];
            }
        }
    }
}

// Vector write-back of the tile's interior (same alignment condition; ej is then a multiple of
// V): lane (row of a pass, vector) gathers V flipped box entries and stores them at once.
template <typename T, class SH>
__device__ __forceinline__ void store_tile_vec(T* __restrict__ fld, const T* box, int k0, int i0, int j0, int ek,
                                               int ei, int ej, bool pz, bool py, bool px, int nr, int nc, int lane) {
    PFAST_TILE_SHAPE(SH);
    using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
    constexpr int V = 16 / sizeof(T);
    constexpr int MV = TJ / V, RPI = 32 / MV;
    const long long plane = (long long)nr * nc;
    const int q = lane % MV, rsub = lane / MV;
    const bool qok = q * V < ej;
#pragma unroll 4
    for (int r0 = 0; r0 < TK * TI; r0 += RPI) {
        const int r = r0 + rsub, rk = r / TI, ri = r - rk * TI;
        if (!qok || rk >= ek || ri >= ei) continue;
        const int base = ((pz ? rk : ek - 1 - rk) + 1) * PS + ((py ? ri : ei - 1 - ri) + 1) * HJ + 1;
        VT v;
        T* f = reinterpret_cast<T*>(&v);
#pragma unroll
        for (int e = 0; e < V; ++e) {
            const int rj = q * V + e;
            f[e] = box[base + (px ? rj : ej - 1 - rj)];
        }
        *reinterpret_cast<VT*>(fld + (k0 + rk) * plane + (long long)(i0 + ri) * nc + j0 + q * V) = v;
    }
}

// The tile's interior values of a node field (the forward's slowness) into the warp's interior
// tile, flipped like the box: node (kf, if, jf) at kf*SPS + if*SJ + jf, so that step t of lane
// (kf, if) reads kf*(SPS-1) + if*(SJ-1) + t (SPS-1 = 8, SJ-1 = 1 mod 32: 32 distinct banks).
// vec: 16-byte vector rows (same condition as load_box_vec), else one column per lane.
template <typename T, class SH>
__device__ __forceinline__ void load_interior(T* dst, const T* __restrict__ g, int k0, int i0, int j0, int ek, int ei,
                                              int ej, bool pz, bool py, bool px, int nr, int nc, bool vec, int lane) {
    PFAST_TILE_SHAPE(SH);
    const long long plane = (long long)nr * nc;
    if (vec) {
        using VT = typename std::conditional<sizeof(T) == 4, float4, double2>::type;
        constexpr int V = 16 / sizeof(T);
        constexpr int MV = TJ / V, RPI = 32 / MV;
        const int q = lane % MV, rsub = lane / MV;
        const bool qok = q * V < ej;
#pragma unroll 1
        for (int r0 = 0; r0 < TK * TI; r0 += 4 * RPI) {
            VT v[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int r = r0 + u * RPI + rsub, rk = r / TI, ri = r - rk * TI;
                if (qok && rk < ek && ri < ei)
                    v[u] = __ldg(reinterpret_cast<const VT*>(g + (k0 + rk) * plane + (long long)(i0 + ri) * nc + j0 + q * V));
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int r = r0 + u * RPI + rsub, rk = r / TI, ri = r - rk * TI;
                if (!(qok && rk < ek && ri < ei)) continue;
                T* row = dst + (pz ? rk : ek - 1 - rk) * SPS + (py ? ri : ei - 1 - ri) * SJ;
                const T* f = reinterpret_cast<const T*>(&v[u]);
#pragma unroll
                for (int e = 0; e < V; ++e) {
                    const int rj = q * V + e;
                    row[px ? rj : ej - 1 - rj] = f[e];
                }
            }
        }
    } else {
        const int jf = px ? lane : ej - 1 - lane;
#pragma unroll 1
        for (int m0 = 0; m0 < TK * TI; m0 += 8) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int rk = (m0 + u) / TI, ri = (m0 + u) % TI;
                if (rk < ek && ri < ei && lane < ej) v[u] = __ldg(g + (k0 + rk) * plane + (long long)(i0 + ri) * nc + j0 + lane);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int rk = (m0 + u) / TI, ri = (m0 + u) % TI;
                if (rk < ek && ri < ei && lane < ej)
                    dst[(pz ? rk : ek - 1 - rk) * SPS + (py ? ri : ei - 1 - ri) * SJ + jf] = v[u];
            }
        }
    }
}

// Index of tile node (rk, ri, rj) (tile coordinates, grid orientation) in the flipped box.
template <class SH>
__device__ __forceinline__ int box_index(int rk, int ri, int rj, int ek, int ei, int ej, bool pz, bool py, bool px) {
    return ((pz ? rk : ek - 1 - rk) + 1) * SH::PS + ((py ? ri : ei - 1 - ri) + 1) * SH::HJ + (px ? rj : ej - 1 - rj) + 1;
}

// r[o] = m[o ^ c] for the 8 order bits of m: an order mask of the flipped coordinates of sweep
// order dir, mapped to grid orders with c = ~dir & 7 (order o in grid terms ascends along an
// axis in flipped terms exactly where o and dir agree).
__device__ __forceinline__ unsigned xor_permute8(unsigned m, int c) {
    if (c & 1) m = ((m & 0x55u) << 1) | ((m & 0xaau) >> 1);
    if (c & 2) m = ((m & 0x33u) << 2) | ((m & 0xccu) >> 2);
    if (c & 4) m = ((m & 0x0fu) << 4) | ((m & 0xf0u) >> 4);
    return m;
}

// ----------------------------------------------------------- octant selection (polish)
// Sweep order o: bit 0 = columns ascending, bit 1 = rows ascending, bit 2 = z ascending.
// Order masks: bit o set for the orders with that axis ascending / descending.
constexpr unsigned kAscX = 0xaa, kDescX = 0x55, kAscY = 0xcc, kDescY = 0x33, kAscZ = 0xf0, kDescZ = 0x0f;

// Forward polish: the orders in which every active axis (U0 above its smaller neighbour)
// visits that smaller neighbour before the node, so the Newton step reads refreshed upwind
// values.  Arguments are bit patterns of values >= 0 (lo = index - 1, hi = index + 1).
__device__ __forceinline__ unsigned fwd_orders(long long u, long long xlo, long long xhi, long long ylo,
                                               long long yhi, long long zlo, long long zhi) {
    unsigned m = 0xff;
    if (u > (xlo < xhi ? xlo : xhi)) m &= xlo < xhi ? kAscX : (xhi < xlo ? kDescX : 0xffu);
    if (u > (ylo < yhi ? ylo : yhi)) m &= ylo < yhi ? kAscY : (yhi < ylo ? kDescY : 0xffu);
    if (u > (zlo < zhi ? zlo : zhi)) m &= zlo < zhi ? kAscZ : (zhi < zlo ? kDescZ : 0xffu);
    return m;
}

// One axis of fwd_orders together with the axis minimum the Newton step reads (the same value
// as min_nonneg), so that the two share their bit-pattern compares.
__device__ __forceinline__ unsigned fwd_axis(long long u, double lo, double hi, unsigned asc, unsigned desc,
                                             double& mn) {
    const long long bl = dbits(lo), bh = dbits(hi);
    const bool lt = bl < bh, gt = bh < bl;
    mn = lt ? lo : hi;
    return u > (lt ? bl : bh) ? (lt ? asc : (gt ? desc : 0xffu)) : 0xffu;
}

// Adjoint polish: lambda at a node depends on the neighbours with a larger traveltime.
// Where exactly one neighbour of an axis is larger, the orders that visit it first;
// where both are (or neither), any order.
__device__ __forceinline__ unsigned adj_orders(long long t, long long xlo, long long xhi, long long ylo,
                                               long long yhi, long long zlo, long long zhi) {
    unsigned m = 0xff;
    const bool a = xlo > t, b = xhi > t, c = ylo > t, d = yhi > t, e = zlo > t, f = zhi > t;
    if (a != b) m &= a ? kAscX : kDescX;
    if (c != d) m &= c ? kAscY : kDescY;
    if (e != f) m &= e ? kAscZ : kDescZ;
    return m;
}

// ----------------------------------------------------------- dependency-aware marking
// Ordered integer of a value >= 0 (its bit pattern), for FP32 and FP64 fields.
__device__ __forceinline__ long long obits(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ int obits(float x) { return __float_as_int(x); }

// ----------------------------------------------------------- the sweep kernel
// Tile locking: a tile whose processing changed no bit of its field, and none of
// whose face neighbours has changed a face node since, is a fixed point of the node
// update for that sweep order (each node's update returned its own value with the
// neighbour values it still has).  For the plain and FP32 updates the node update does
// not depend on the order, so one quiet processing locks the tile for all eight; the
// polish updates select nodes by sweep order (octant selection), so a tile locks for
// an order only once it has been quiet in that order.  Per (source, tile):
//   dirty[t]  bit o set: process the tile in sweep order o; set at the start (all tiles,
//             or for the FP32 bulk and the adjoint polish the tiles with something to
//             propagate), and for all eight orders by a face neighbour whose changed face
//             node the tile reads, or by the tile itself (see process_tile),
//   stamp[t]  outer iteration in which the tile last took its snapshot (plain kinds),
//   diff[t]   plain kinds: whether the tile differs from its snapshot by more than the
//             tolerance after its latest processing; mixed kinds: whether some processing
//             in this iteration moved a node by more than the tolerance (cleared each
//             iteration).
// The outer-iteration test (the reference's isconv for the plain kinds) is the OR of diff
// over the tiles of a source: a skipped tile has not moved.
// Tile (tk, ti, tj) and its index of the diagonal-table entry pk in sweep order dir (the
// table is in flipped coordinates).
__device__ __forceinline__ int tile_of(const Sweep3Args& A, unsigned pk, int dir, int& tk, int& ti, int& tj) {
    const int bkf = pk & 1023, bif = (pk >> 10) & 1023, bjf = pk >> 20;
    tk = (dir & 4) ? bkf : A.nbk - 1 - bkf;
    ti = (dir & 2) ? bif : A.nbi - 1 - bif;
    tj = (dir & 1) ? bjf : A.nbj - 1 - bjf;
    return (tk * A.nbi + ti) * A.nbj + tj;
}

// Whether a tile with lock word dm is processed in sweep order dir.  Polish kinds: bits 8-15
// hold the orders in which some node of the tile is selected (from the order pre-pass, then
// recorded at each processing).
template <int KIND>
__device__ __forceinline__ bool tile_due(int dm, int dir) {
    constexpr bool kSelective = (KIND == kFwdPolish64 || KIND == kAdjPolish64);
    const int omask = kSelective ? (dm >> 8) & 0xff : 0xff;
    return (dm & omask & (1 << dir)) != 0;
}

// One warp processes one tile (inst, tid) in sweep order dir, outer iteration iter; dmask is
// the tile's lock word as read by the caller, which has checked tile_due.  wsm: the warp's
// shared-memory slice.  COHERENT: the field may have been written by this same kernel launch
// (dataflow schedule), so it is read through L2 instead of the read-only path.
// The box is in the flipped coordinates of order dir (see load_box); the lanes (kf, if) walk
// their pencils jf = 0..ej-1 so that step t updates the flipped hyperplane kf+if+jf = t.
template <int KIND, bool COHERENT, class SH>
__device__ __forceinline__ void process_tile(const Sweep3Args& A, const int inst, const int tid, const int tk,
                                             const int ti, const int tj, const int dir, const int iter,
                                             const int dmask, unsigned char* wsm, const int lane) {
    PFAST_TILE_SHAPE(SH);
    using Real = typename Traits<KIND>::Real;
    using Aux = typename Traits<KIND>::Aux;
    using Bits = typename std::conditional<sizeof(Real) == 8, unsigned long long, unsigned>::type;
    constexpr bool ADJ = Traits<KIND>::adj;
    const bool pz = dir & 4, py = dir & 2, px = dir & 1;
    int* dirty = A.dirty + (long long)inst * A.ntiles;
    const int obit = 1 << dir;
    constexpr bool kSelective = (KIND == kFwdPolish64 || KIND == kAdjPolish64);
    // Convergence test of the FP32 bulk and polish kinds: a node that moved by more than the
    // tolerance in some processing of this outer iteration (the flag is ORed over the
    // iteration's processings; a polish change is its FP32 step, so the test needs no FP64
    // instruction).  The plain kinds compare with a snapshot taken at the tile's first
    // processing in the iteration, as the reference's isconv does.
    constexpr bool kSnap = KIND == kFwdPlain64 || KIND == kAdjPlain64;
    // The tile's lock word as lane 0 last wrote it.  Face neighbours are never processed at the
    // same time (per-diagonal: other launches; dataflow: the dependencies), so it is composed
    // here without reading it back.
    int dword = kSelective ? (dmask & ~obit) : 0;
    if (lane == 0) {
        dirty[tid] = dword;
        if (A.work) atomicAdd(A.work + inst, (unsigned long long)(min(TK, A.nz - tk * TK) * min(TI, A.nr - ti * TI) *
                                                                  min(TJ, A.nc - tj * TJ)));
    }

    const int k0 = tk * TK, i0 = ti * TI, j0 = tj * TJ;
    const int ek = min(TK, A.nz - k0), ei = min(TI, A.nr - i0), ej = min(TJ, A.nc - j0);
    const int nz = A.nz, nr = A.nr, nc = A.nc;
    const long long plane = (long long)nr * nc;

    Real* box = reinterpret_cast<Real*>(wsm);
    Aux* aux = reinterpret_cast<Aux*>(reinterpret_cast<unsigned char*>(box) + HK * PS * sizeof(Real));
    constexpr bool TWIN = t_windows<KIND>();
    constexpr bool UWIN = u_windows<KIND, COHERENT>();
    Real* fld = reinterpret_cast<Real*>(A.field) + inst * A.fstride;

    // ---- stage the field halo box (out-of-grid: +inf for the forward so that the
    // neighbour minimum reduces to the one-sided rule at faces; never read by the adjoint)
    const Real fill = ADJ ? Real(0) : Real(INFINITY);
    if constexpr (!UWIN) {
        if (A.vec_rows) load_box_vec<Real, COHERENT, SH>(box, fld, k0, i0, j0, ek, ei, ej, pz, py, px, nz, nr, nc, fill, lane);
        else load_box<Real, COHERENT, SH>(box, fld, k0, i0, j0, ek, ei, ej, pz, py, px, nz, nr, nc, fill, lane);
    }
    Aux* stile = reinterpret_cast<Aux*>(reinterpret_cast<unsigned char*>(box) + HK * PS * sizeof(Real));
    if constexpr (stage_slowness<KIND>())
        load_interior<Aux, SH>(stile, reinterpret_cast<const Aux*>(A.aux), k0, i0, j0, ek, ei, ej, pz, py, px, nr, nc,
                           A.vec_rows != 0, lane);

    // ---- auxiliary data
    unsigned fixed_bits = 0;   // adjoint: fixed nodes of this lane's pencil, bit jf (flipped position)
    const int lkf = lane / TI, lif = lane % TI;
    const bool lane_ok = lkf < ek && lif < ei;
    const int lk = pz ? lkf : ek - 1 - lkf;   // the lane's position in the tile, grid orientation
    const int li = py ? lif : ei - 1 - lif;
    if constexpr (ADJ) {
        if constexpr (!TWIN) {
            const Aux* tb = reinterpret_cast<const Aux*>(A.aux) + inst * A.fstride;
            if (A.vec_rows) load_box_vec<Aux, false, SH>(aux, tb, k0, i0, j0, ek, ei, ej, pz, py, px, nz, nr, nc, Aux(0), lane);
            else load_box<Aux, false, SH>(aux, tb, k0, i0, j0, ek, ei, ej, pz, py, px, nz, nr, nc, Aux(0), lane);
        }
        if (lane_ok) {
            const unsigned fb = A.mask[inst * A.mask_stride + ((long long)(k0 + lk) * nr + (i0 + li)) * A.wpr + (j0 >> 5)];
            fixed_bits = px ? fb : (__brev(fb) >> (32 - ej));
        }
    }

    // ---- snapshot at the tile's first processing in this outer iteration (its values are
    // still the iteration-start values then: only the tile itself writes them)
    Real* snp = kSnap ? reinterpret_cast<Real*>(A.snap) + inst * A.fstride : nullptr;
    if constexpr (kSnap) {
        int* stamp = A.stamp + (long long)inst * A.ntiles;
        if (__ldcg(stamp + tid) != iter) {
#pragma unroll 4
            for (int m = 0; m < 32; ++m) {
                const int rk = m / TI, ri = m % TI;
                if (rk < ek && ri < ei && lane < ej)
                    snp[(k0 + rk) * plane + (long long)(i0 + ri) * nc + j0 + lane] =
                        box[box_index<SH>(rk, ri, lane, ek, ei, ej, pz, py, px)];
            }
            if (lane == 0) stamp[tid] = iter;
        }
    }
    __syncwarp();

    // ---- wavefront over the tile's node hyperplanes
    const int gk = k0 + lk, gi = i0 + li;
    const int steps = ek + ei + ej - 2;
    const int toff = lane_ok ? lkf + lif : (1 << 20);   // flipped column of step t: t - toff
    const int cl = (lkf + 1) * PS + (lif + 1) * HJ + 1 - lkf - lif;   // box index of step t: cl + t
    const int sl = lkf * (SPS - 1) + lif * (SJ - 1);                   // staged slowness of step t: sl + t
    const int dj = px ? 1 : -1, gjA = j0 + (px ? 0 : ej - 1);      // grid column of jf: gjA + dj*jf
    int sk = -1, si = -1, sj = -1, qkqi = 0;
    bool near_src = false;   // forward: the tile meets the fixed region around the source
    if constexpr (!ADJ) {
        sk = A.src_kij[3 * inst]; si = A.src_kij[3 * inst + 1]; sj = A.src_kij[3 * inst + 2];
        const int ddk = max(0, max(k0 - sk, sk - (k0 + ek - 1))), ddi = max(0, max(i0 - si, si - (i0 + ei - 1)));
        const int ddj = max(0, max(j0 - sj, sj - (j0 + ej - 1)));
        near_src = ddk * ddk + ddi * ddi + ddj * ddj <= A.src_r2;
        qkqi = (gk - sk) * (gk - sk) + (gi - si) * (gi - si);
    }
    const bool row_interior = ADJ ? (gk >= 1 && gk <= nz - 2 && gi >= 1 && gi <= nr - 2) : true;
    unsigned sel = 0;   // polish: orders (flipped coordinates) in which some node of this lane's pencil is selected
    const long long rowbase = gk * plane + (long long)gi * nc;
    const Aux* srow = ADJ ? nullptr : reinterpret_cast<const Aux*>(A.aux) + rowbase;
    bool chg = false;   // this lane's pencil changed
    // Face marks in flipped terms (u: the upstream face of the sweep, d: the downstream one): a
    // changed face node that a node of the face neighbour depends on.  The plain kinds mark
    // every changed face node (their tile skipping must stay exact).  Elsewhere the dependency
    // is one-directional: a forward update reads only neighbours below the node's value (the
    // Godunov update and its Newton form exclude larger ones), and lambda at a node reads only
    // neighbours of larger traveltime.
    constexpr bool kPrune = KIND != kFwdPlain64 && KIND != kAdjPlain64;
    bool m_zu = false, m_zd = false, m_yu = false, m_yd = false, m_xu = false, m_xd = false;
    bool restep = false;   // polish: some update left a remainder above the floor (visit again in this order)
    // FP32 bulk: some changed node feeds an in-tile node that this pass visited before it
    // (so the tile is not yet a fixed point of the update)
    bool stale = false;
    bool moved = false;   // FP32 bulk, polish: some node of this lane moved by more than the tolerance
    const float tol_step = (float)A.tol_abs;

    // ---- adjoint traveltime windows (FP64 kinds).  Lane (kf, if) (flipped coordinates) is at flipped
    // position jf = t - kf - if in step t and keeps its pencil's traveltimes at jf-1, jf, jf+1
    // (tm, t0, tp), with loads issued three steps ahead (q1, q2).  Lane (kf-1, if) is one
    // position ahead, so its tm is the traveltime at (kf-1, if, jf); lane (kf+1, if) is one
    // behind and its tp is the one at (kf+1, if, jf); likewise along if.  The halo pencils
    // outside the tile are tracked by owner lanes at their consumer's position: lanes 0..TI-1
    // the flipped k-1 face, the next TI the k+1 face, then TK lanes each for the i-1 and i+1
    // faces (24 lanes in both tile shapes).
    const Aux* Tb = TWIN ? reinterpret_cast<const Aux*>(A.aux) + inst * A.fstride : nullptr;
    const Aux* trow = (TWIN && lane_ok) ? Tb + rowbase : nullptr;
    const Aux* hrow = nullptr;
    const Real* urow = (UWIN && lane_ok) ? fld + rowbase : nullptr;   // the field's windows (UWIN)
    const Real* uhrow = nullptr;
    int hpos = 0;
    if constexpr (TWIN || UWIN) {
        int lkh = 0, lih = 0;
        bool own = false;
        if (lane < TI) {
            own = lane < ei; lkh = pz ? -1 : ek; lih = py ? lane : ei - 1 - lane; hpos = lane;
        } else if (lane < 2 * TI) {
            const int x = lane - TI;
            own = x < ei; lkh = pz ? ek : -1; lih = py ? x : ei - 1 - x; hpos = ek - 1 + x;
        } else if (lane < 2 * TI + 2 * TK) {
            const int y = (lane - 2 * TI) % TK;
            const bool lo = lane < 2 * TI + TK;
            own = y < ek; lkh = pz ? y : ek - 1 - y;
            lih = lo ? (py ? -1 : ei) : (py ? ei : -1);
            hpos = lo ? y : y + ei - 1;
        }
        const int gkh = k0 + lkh, gih = i0 + lih;
        if (own && (unsigned)gkh < (unsigned)nz && (unsigned)gih < (unsigned)nr) {
            if constexpr (TWIN) hrow = Tb + gkh * plane + (long long)gih * nc;
            if constexpr (UWIN) uhrow = fld + gkh * plane + (long long)gih * nc;
        }
    }
    // traveltime of pencil row r at flipped position p, zero outside [plo, phi] or the grid
    auto tload = [&](const Aux* r, int p, int plo, int phi) -> Aux {
        const int g = j0 + (px ? p : ej - 1 - p);
        return (r != nullptr && p >= plo && p <= phi && (unsigned)g < (unsigned)nc) ? __ldg(r + g) : Aux(0);
    };
    const int jf0 = -lkf - lif;
    Aux tm = Aux(0), t0 = Aux(0), tp = Aux(0), q1 = Aux(0), q2 = Aux(0), h0 = Aux(0), hq1 = Aux(0), hq2 = Aux(0);
    if constexpr (TWIN) {
        tm = tload(trow, jf0 - 1, -1, ej); t0 = tload(trow, jf0, -1, ej); tp = tload(trow, jf0 + 1, -1, ej);
        q1 = tload(trow, jf0 + 2, -1, ej); q2 = tload(trow, jf0 + 3, -1, ej);
        h0 = tload(hrow, -hpos, 0, ej - 1); hq1 = tload(hrow, 1 - hpos, 0, ej - 1); hq2 = tload(hrow, 2 - hpos, 0, ej - 1);
    }
    // field of pencil row r at flipped position p: the fill outside [plo, phi] or the grid (UWIN)
    auto uload = [&](const Real* r, int p, int plo, int phi) -> Real {
        const int g = j0 + (px ? p : ej - 1 - p);
        if (r == nullptr || p < plo || p > phi || (unsigned)g >= (unsigned)nc) return fill;
        if constexpr (COHERENT) return __ldcg(r + g);
        else return __ldg(r + g);
    };
    // UWIN: um = new value at jf-1, u0 / up / uq1 / uq2 = old values at jf .. jf+3; uh*: the
    // owned halo pencil at the consumer's position and two ahead
    Real um = Real(0), u0 = Real(0), up = Real(0), uq1 = Real(0), uq2 = Real(0);
    Real uh0 = Real(0), uhq1 = Real(0), uhq2 = Real(0);
    if constexpr (UWIN) {
        um = uload(urow, jf0 - 1, -1, ej); u0 = uload(urow, jf0, -1, ej); up = uload(urow, jf0 + 1, -1, ej);
        uq1 = uload(urow, jf0 + 2, -1, ej); uq2 = uload(urow, jf0 + 3, -1, ej);
        uh0 = uload(uhrow, -hpos, 0, ej - 1); uhq1 = uload(uhrow, 1 - hpos, 0, ej - 1); uhq2 = uload(uhrow, 2 - hpos, 0, ej - 1);
    }

#pragma unroll 1
    for (int t = 0; t < steps; ++t) {
        const int ljf = t - toff;
        // adjoint: the traveltimes around this lane's node, flipped orientation (u: upstream)
        Aux Tzu = Aux(0), Tzd = Aux(0), Tyu = Aux(0), Tyd = Aux(0), Txu = Aux(0), Txd = Aux(0);
        if constexpr (TWIN) {
            const Aux a = __shfl_sync(0xffffffffu, tm, (lane - TI) & 31);
            const Aux b = __shfl_sync(0xffffffffu, tp, (lane + TI) & 31);
            const Aux c_ = __shfl_sync(0xffffffffu, tm, (lane - 1) & 31);
            const Aux d = __shfl_sync(0xffffffffu, tp, (lane + 1) & 31);
            const Aux hkl = __shfl_sync(0xffffffffu, h0, lif);
            const Aux hkh = __shfl_sync(0xffffffffu, h0, TI + lif);
            const Aux hil = __shfl_sync(0xffffffffu, h0, 2 * TI + lkf);
            const Aux hih = __shfl_sync(0xffffffffu, h0, 2 * TI + TK + lkf);
            Tzu = lkf == 0 ? hkl : a; Tzd = lkf == ek - 1 ? hkh : b;
            Tyu = lif == 0 ? hil : c_; Tyd = lif == ei - 1 ? hih : d;
            Txu = tm; Txd = tp;
        }
        // UWIN: the neighbours of this lane's node (flipped; u: upstream, new values; d:
        // downstream, old values): lane (kf-1, if) is one position ahead and holds the new value
        // at this jf as its um, lane (kf+1, if) one behind holds the old one as its up
        Real wzu = Real(0), wzd = Real(0), wyu = Real(0), wyd = Real(0);
        if constexpr (UWIN) {
            const Real a = __shfl_sync(0xffffffffu, um, (lane - TI) & 31);
            const Real b = __shfl_sync(0xffffffffu, up, (lane + TI) & 31);
            const Real c_ = __shfl_sync(0xffffffffu, um, (lane - 1) & 31);
            const Real d = __shfl_sync(0xffffffffu, up, (lane + 1) & 31);
            const Real hkl = __shfl_sync(0xffffffffu, uh0, lif);
            const Real hkh = __shfl_sync(0xffffffffu, uh0, TI + lif);
            const Real hil = __shfl_sync(0xffffffffu, uh0, 2 * TI + lkf);
            const Real hih = __shfl_sync(0xffffffffu, uh0, 2 * TI + TK + lkf);
            wzu = lkf == 0 ? hkl : a; wzd = lkf == ek - 1 ? hkh : b;
            wyu = lif == 0 ? hil : c_; wyd = lif == ei - 1 ? hih : d;
        }
        Real res = u0;   // UWIN: this lane's value at jf after the step
        if ((unsigned)ljf < (unsigned)ej) {
            const int c = cl + t;
            const Real xu = UWIN ? um : box[c - 1], xd = UWIN ? up : box[c + 1];
            const Real yu = UWIN ? wyu : box[c - HJ], yd = UWIN ? wyd : box[c + HJ];
            const Real zu = UWIN ? wzu : box[c - PS], zd = UWIN ? wzd : box[c + PS];
            const Real old = UWIN ? u0 : box[c];
            Real nv = old;
            float dstep = INFINITY;   // polish: the size of this node's change
            if constexpr (ADJ && !TWIN) {   // FP32 bulk: the traveltimes from the staged box
                t0 = aux[c]; Txu = aux[c - 1]; Txd = aux[c + 1]; Tyu = aux[c - HJ]; Tyd = aux[c + HJ];
                Tzu = aux[c - PS]; Tzd = aux[c + PS];
            }
            if constexpr (!ADJ) {
                const int gj = gjA + dj * ljf;
                bool free_node = true;   // the source node (and the opt-in fixed region) stays
                if (near_src) free_node = qkqi + (gj - sj) * (gj - sj) > A.src_r2;
                if (free_node) {
                    Aux s;
                    if constexpr (stage_slowness<KIND>()) s = stile[sl + t];
                    else s = __ldg(srow + gj);
                    // the neighbour minima are symmetric in the two neighbours of an axis
                    if constexpr (KIND == kFwdPlain64) {
                        nv = min_nonneg(old, eik3_plain(min_nonneg(xd, xu), min_nonneg(yd, yu), min_nonneg(zd, zu), s, A.sp));
                    } else if constexpr (KIND == kFwdFast32) {
                        // field values are >= +0 or +inf: fminf is the reference's MIN here
                        const float xa = fminf(xd, xu), yb = fminf(yd, yu), zc = fminf(zd, zu);
                        nv = fminf(old, A.sp.iso ? eik3_fast_iso(xa, yb, zc, s * A.sp.df[0]) : eik3_fast(xa, yb, zc, s, A.sp));
                    } else {   // polish: one Newton step of the local Godunov equation (aux holds s^2, (s h)^2 when isotropic)
                        // Octant selection: if an axis is active (U0 above its smaller neighbour) and
                        // that neighbour is the one this sweep visits after the node, the update would
                        // read a value the sweep has not refreshed; the node keeps its value and is
                        // updated by the sweep that visits its upwind neighbours first.  A Newton step
                        // is not monotone, so without this every sweep would move every node.
                        // Integer compares of the bit patterns (values >= 0), in flipped terms: this
                        // sweep is order 7 there (every axis ascending).
                        double mx, my, mz;
                        const long long bo_ = dbits(old);
                        const unsigned m = fwd_axis(bo_, xu, xd, kAscX, kDescX, mx) & fwd_axis(bo_, yu, yd, kAscY, kDescY, my) &
                                           fwd_axis(bo_, zu, zd, kAscZ, kDescZ, mz);
                        sel |= m;
                        if (m & 0x80u) {
                            bool big = false;
                            nv = eik3_newton(old, mx, my, mz, s, A.slow64, rowbase + gj, A.sp, A.polish_floor, big, dstep);
                            restep |= big;
                        }
                    }
                }
            } else {
                const int gj = gjA + dj * ljf;
                if (row_interior && gj >= 1 && gj <= nc - 2 && !((fixed_bits >> ljf) & 1u)) {
                    if constexpr (KIND == kAdjPlain64) {
                        // the reference's operand order, in grid orientation (m: index - 1, p: index + 1)
                        const Real Lxp = px ? xd : xu, Lxm = px ? xu : xd, Lyp = py ? yd : yu, Lym = py ? yu : yd;
                        const Real Lzp = pz ? zd : zu, Lzm = pz ? zu : zd;
                        const Aux Txp = px ? Txd : Txu, Txm = px ? Txu : Txd, Typ = py ? Tyd : Tyu, Tym = py ? Tyu : Tyd;
                        const Aux Tzp = pz ? Tzd : Tzu, Tzm = pz ? Tzu : Tzd;
                        nv = adj3_plain(t0, Txp, Txm, Typ, Tym, Tzp, Tzm, Lxp, Lxm, Lyp, Lym, Lzp, Lzm, A.sp);
                    } else if constexpr (KIND == kAdjFast32) {
                        // the update is symmetric in the two neighbours of an axis
                        nv = adj3_bulk(t0, Txd, Txu, Tyd, Tyu, Tzd, Tzu, xd, xu, yd, yu, zd, zu, old, A.sp);
                    } else {
                        // Octant selection (see the forward polish): lambda at a node depends on the
                        // neighbours with a larger traveltime.  Where on some axis only the neighbour
                        // visited after the node is larger, the node waits for its own sweep; where
                        // both are larger no sweep order has both fresh, and the node is updated.
                        const unsigned m = adj_orders(dbits(t0), dbits(Txu), dbits(Txd), dbits(Tyu), dbits(Tyd),
                                                      dbits(Tzu), dbits(Tzd));
                        sel |= m;
                        if (m & 0x80u) {
                            // the residual's FP64 sum in grid orientation (m: index - 1, p: index + 1),
                            // the same in every sweep order
                            const Real Lxp = px ? xd : xu, Lxm = px ? xu : xd, Lyp = py ? yd : yu, Lym = py ? yu : yd;
                            const Real Lzp = pz ? zd : zu, Lzm = pz ? zu : zd;
                            const Aux Txp = px ? Txd : Txu, Txm = px ? Txu : Txd, Typ = py ? Tyd : Tyu;
                            const Aux Tym = py ? Tyu : Tyd, Tzp = pz ? Tzd : Tzu, Tzm = pz ? Tzu : Tzd;
                            bool big = false;
                            nv = adj3_polish(t0, Txp, Txm, Typ, Tym, Tzp, Tzm, Lxp, Lxm, Lyp, Lym, Lzp, Lzm, old, A.sp,
                                             A.polish_floor, big, dstep);
                            restep |= big;
                        }
                    }
                }
            }
            Bits bo, bn;
            memcpy(&bo, &old, sizeof(Real));
            memcpy(&bn, &nv, sizeof(Real));
            res = nv;
            if (bo != bn) {
                if constexpr (UWIN) fld[rowbase + gjA + dj * ljf] = nv;
                else box[c] = nv;
                chg = true;
                if constexpr (kSelective) {
                    if (dstep > tol_step) moved = true;
                } else if constexpr (!kSnap) {
                    if (fabsf(old - nv) > A.tol_abs_f + A.tol_rel_f * fabsf(nv)) moved = true;
                }
                if constexpr (kPrune) {
                    // does the neighbour across a face (value vn, traveltime tn) depend on this node?
                    // The neighbour values were read before this step's stores, none of which
                    // touches them (they lie on the hyperplanes t - 1 and t + 1).
                    const auto lo = min(obits(old), obits(nv));
                    auto dep = [&](Real vn, Aux tn) {
                        if constexpr (ADJ) return obits(t0) > obits(tn);
                        else return lo < obits(vn);
                    };
                    if (lkf == 0 && dep(zu, Tzu)) m_zu = true;
                    if (lkf == ek - 1 && dep(zd, Tzd)) m_zd = true;
                    if (lif == 0 && dep(yu, Tyu)) m_yu = true;
                    if (lif == ei - 1 && dep(yd, Tyd)) m_yd = true;
                    if (ljf == 0 && dep(xu, Txu)) m_xu = true;
                    if (ljf == ej - 1 && dep(xd, Txd)) m_xd = true;
                    if constexpr (!kSelective) {
                        // the in-tile neighbours this pass visited before the node (flipped upstream)
                        if ((lkf > 0 && dep(zu, Tzu)) || (lif > 0 && dep(yu, Tyu)) || (ljf > 0 && dep(xu, Txu)))
                            stale = true;
                    }
                } else {
                    if (ljf == 0) m_xu = true;
                    if (ljf == ej - 1) m_xd = true;
                }
            }
        }
        if constexpr (TWIN) {   // slide the windows to step t + 1
            tm = t0; t0 = tp; tp = q1; q1 = q2; q2 = tload(trow, t + 4 - lkf - lif, -1, ej);
            h0 = hq1; hq1 = hq2; hq2 = tload(hrow, t + 3 - hpos, 0, ej - 1);
        }
        if constexpr (UWIN) {
            um = res; u0 = up; up = uq1; uq1 = uq2; uq2 = uload(urow, t + 4 - lkf - lif, -1, ej);
            uh0 = uhq1; uhq1 = uhq2; uhq2 = uload(uhrow, t + 3 - hpos, 0, ej - 1);
        }
        if constexpr (!UWIN) __syncwarp();
    }

    if constexpr (kSelective) {
        const unsigned tsel = xor_permute8(__reduce_or_sync(0xffffffffu, sel), ~dir & 7);
        dword = (dword & 0xff) | (int)(tsel << 8);
        if (lane == 0) dirty[tid] = dword;
    }

    // ---- nothing changed: the field and its snapshot comparison stand as they are
    if (!__any_sync(0xffffffffu, chg)) return;

    // ---- unlock this tile and every face neighbour that sees a changed face node (flipped
    // faces mapped back to grid faces)
    const bool klo = kPrune ? (pz ? m_zu : m_zd) : chg && lk == 0, khi = kPrune ? (pz ? m_zd : m_zu) : chg && lk == ek - 1;
    const bool ilo = kPrune ? (py ? m_yu : m_yd) : chg && li == 0, ihi = kPrune ? (py ? m_yd : m_yu) : chg && li == ei - 1;
    const unsigned f_klo = __ballot_sync(0xffffffffu, klo);
    const unsigned f_khi = __ballot_sync(0xffffffffu, khi);
    const unsigned f_ilo = __ballot_sync(0xffffffffu, ilo);
    const unsigned f_ihi = __ballot_sync(0xffffffffu, ihi);
    const unsigned f_jlo = __ballot_sync(0xffffffffu, px ? m_xu : m_xd);
    const unsigned f_jhi = __ballot_sync(0xffffffffu, px ? m_xd : m_xu);
    // Own re-marking.  A polish sweep in order o leaves every node that selects o consistent
    // with the values it reads (its active neighbours come before it in o), so after small
    // updates the tile is due again in o only when a neighbour or another order changes
    // something.  An FP32 bulk pass in which no changed node feeds an already visited node
    // leaves the tile a fixed point of the update: it stays locked until a neighbour marks it.
    // The plain kinds re-mark all orders (their tile skipping must stay exact).
    bool again = true;
    if constexpr (kSelective) again = __any_sync(0xffffffffu, restep);
    else if constexpr (kPrune) again = __any_sync(0xffffffffu, stale);
    if (lane == 0) {
        // neighbours keep their selection bits: OR in the eight order bits (two tiles of one
        // launch can share a face neighbour, hence atomic)
        const int sk_ = A.nbi * A.nbj;
        dirty[tid] = dword | (again ? 0xff : (kSelective ? (0xff & ~obit) : 0));
        if (f_klo && tk > 0) atomicOr(dirty + tid - sk_, 0xff);
        if (f_khi && tk < A.nbk - 1) atomicOr(dirty + tid + sk_, 0xff);
        if (f_ilo && ti > 0) atomicOr(dirty + tid - A.nbj, 0xff);
        if (f_ihi && ti < A.nbi - 1) atomicOr(dirty + tid + A.nbj, 0xff);
        if (f_jlo && tj > 0) atomicOr(dirty + tid - 1, 0xff);
        if (f_jhi && tj < A.nbj - 1) atomicOr(dirty + tid + 1, 0xff);
    }

    // ---- write back (UWIN: stored as updated); the FP64 kinds compare with the iteration-start
    // snapshot
    if constexpr (!kSnap) {
        if constexpr (UWIN) {
        } else if (A.vec_rows) {
            store_tile_vec<Real, SH>(fld, box, k0, i0, j0, ek, ei, ej, pz, py, px, nr, nc, lane);
        } else {
#pragma unroll 8
            for (int m = 0; m < 32; ++m) {
                const int rk = m / TI, ri = m % TI;
                if (rk < ek && ri < ei && lane < ej)
                    fld[(k0 + rk) * plane + (long long)(i0 + ri) * nc + j0 + lane] =
                        box[box_index<SH>(rk, ri, lane, ek, ei, ej, pz, py, px)];
            }
        }
        if (__any_sync(0xffffffffu, moved) && lane == 0) A.diff[(long long)inst * A.ntiles + tid] = 1;
    } else {
#pragma unroll 1
        for (int m0 = 0; m0 < 32; m0 += 8) {
            Real p[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int m = m0 + u, rk = m / TI, ri = m % TI;
                p[u] = Real(0);
                if (rk < ek && ri < ei && lane < ej) p[u] = __ldcg(snp + (k0 + rk) * plane + (long long)(i0 + ri) * nc + j0 + lane);
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int m = m0 + u, rk = m / TI, ri = m % TI;
                if (rk < ek && ri < ei && lane < ej) {
                    const Real v = box[box_index<SH>(rk, ri, lane, ek, ei, ej, pz, py, px)];
                    fld[(k0 + rk) * plane + (long long)(i0 + ri) * nc + j0 + lane] = v;
                    if (fabs(p[u] - v) > A.tol_abs) moved = true;   // isconv, src/T_pfsm3d.h:126
                }
            }
        }
        const bool any_moved = __any_sync(0xffffffffu, moved);
        if (lane == 0) A.diff[(long long)inst * A.ntiles + tid] = any_moved ? 1 : 0;
    }
}

// One launch per tile diagonal: block (x, y) = (tile of the diagonal, active instance).
template <int KIND, class SH>
// d0, ntd: the diagonal's first entry in diag_tiles and its tile count.
__global__ void __launch_bounds__(kWarps3 * 32) sweep3d_kernel(const Sweep3Args A, const int d0, const int ntd) {
    PFAST_TILE_SHAPE(SH);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile_idx = blockIdx.x * kWarps3 + warp;
    if (tile_idx >= ntd) return;
    // Three independent reads, issued before any is tested, so that a locked tile costs two
    // memory round trips (these, then its lock word): the iteration and active count of a
    // replayed iteration graph, the instance of this block row (act holds at least gridDim.y
    // entries) and the tile of this diagonal entry.
    int2 dyn = make_int2(A.iter, (int)gridDim.y);
    if (A.dyn) dyn = __ldcg(reinterpret_cast<const int2*>(A.dyn));
    const int inst = A.act[blockIdx.y];
    const unsigned pk = A.diag_tiles[d0 + tile_idx];
    if ((int)blockIdx.y >= dyn.y) return;   // a source retired since the graph was captured
    const int iter = dyn.x;
    int tk, ti, tj;
    const int tid = tile_of(A, pk, A.dir, tk, ti, tj);
    const int dm = __ldcg(A.dirty + (long long)inst * A.ntiles + tid);
    if (!tile_due<KIND>(dm, A.dir)) return;   // locked tile for this order (warp-uniform)
    __syncwarp();
    process_tile<KIND, false, SH>(A, inst, tid, tk, ti, tj, A.dir, iter, dm, smem_raw + warp * warp_smem_bytes<KIND, SH>(),
                              lane);
}

// ----------------------------------------------------------- dataflow schedule
// One launch per phase.  Each block takes instances (sources) from a queue and runs the
// whole solve of one instance: outer iterations of eight sweep orders until the instance's
// convergence test passes or maxiter iterations ran.  Within an outer iteration the items
// (sweep order o, tile x) form the dataflow graph of dataflow3.h: an item is ready once the
// items it reads from are done, so the sweeps of different orders overlap and no barrier
// separates tile diagonals or orders.  Per tile, two 4-bit counters in shared memory (one
// per order parity, four tiles per word) count the item's missing dependencies; a ring of
// ready items in shared memory feeds the block's warps.
//   A warp takes about its share of the ready items (1 to 32, one per lane) and reads their
//   lock words.  A tile that is not due in the item's order (tile locking) completes at once,
//   lane by lane; of the due items the warp processes one (process_tile) and returns the
//   others to the ring for idle warps.  Completing (o, x) re-arms x's counter of parity o for
//   order o + 2 and decrements its dependents' counters; those that reach zero join the ring.
//   The iteration ends when all 8 x ntiles items completed; the block then tests convergence
//   as the per-diagonal schedule's reduction does (any tile moved / any tile still due).
// Every tile processing sees exactly the neighbour values and lock words it sees in the
// per-diagonal schedule, so both schedules give the same bits.  All waits are on this block's
// own shared memory (no block waits for another) and are bounded: a block that sees no
// progress for two seconds sets *err, records the instance as not converged and exits.
// result[inst] = iterations | 1 << 30 when not converged.  A.iter is the first iteration's
// number: a solve continued from per-diagonal iterations counts on from them.
constexpr unsigned kSlotEmpty = 0xffffffffu;
// shared-memory copy of a model's arguments (multi-grid launches)
constexpr int kDfArgsBytes = (int)((sizeof(Sweep3Args) + 15) / 16 * 16);
static_assert(sizeof(Sweep3Args) % 8 == 0 && sizeof(Sweep3Args) % 4 == 0, "argument copy by words");

struct DataflowShared {
    unsigned head, tail;   // ring positions: next to take / next to fill
    int done;              // items completed in this outer iteration
    int abort;
    int item;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void df_push(unsigned* slots, unsigned qmask, DataflowShared* sh, unsigned e) {
    const unsigned p = atomicAdd(&sh->tail, 1u);
    unsigned* slot = slots + (p & qmask);
    // a slot still holds an earlier round's item only while that item's taker is about to
    // exchange it out (at most ntiles <= ring size items are outstanding): wait for it
    for (int spin = 0; atomicCAS(slot, kSlotEmpty, e) != kSlotEmpty; ++spin)
        if (spin > (1 << 22) || *(volatile int*)&sh->abort) { *(volatile int*)&sh->abort = 1; return; }
}

// One missing dependency of item (od, y) fewer; push it when it was the last.
__device__ __forceinline__ void df_notify(unsigned* cnt, unsigned* slots, unsigned qmask, DataflowShared* sh, int y,
                                          int od) {
    const unsigned shf = 8u * (unsigned)(y & 3) + 4u * (unsigned)(od & 1);
    const unsigned old = (atomicSub(cnt + (y >> 2), 1u << shf) >> shf) & 15u;
    if (old == 1u) df_push(slots, qmask, sh, ((unsigned)y << 3) | (unsigned)od);
    else if (old == 0u) *(volatile int*)&sh->abort = 1;   // more completions than dependencies: stop
}

// Completion of item (o, x): re-arm x's counter of parity o for order o + 2 (it is zero: it
// fired for (o, x), and no dependency of (o + 2, x) completes before (o, x) did), then notify
// the dependents (dataflow3.h: dependents()).
__device__ __forceinline__ void df_complete(const TileGrid3& g, unsigned* cnt, unsigned* slots, unsigned qmask,
                                            DataflowShared* sh, int o, int x) {
    if (o + 2 < 8)
        atomicAdd(cnt + (x >> 2), (unsigned)dep_count(g, o + 2, x) << (8u * (unsigned)(x & 3) + 4u * (unsigned)(o & 1)));
    __threadfence_block();
    if (o < 7) df_notify(cnt, slots, qmask, sh, x, o + 1);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const int y = tile_neighbour(g, x, a, s);
            if (y < 0) continue;
            if (side_upstream(o, a, 1 - s)) df_notify(cnt, slots, qmask, sh, y, o);
            if (o < 7 && !side_upstream(o + 1, a, 1 - s)) df_notify(cnt, slots, qmask, sh, y, o + 1);
        }
}

// The warps' part of one outer iteration of instance inst.
template <int KIND, class SH>
__device__ __forceinline__ void df_iteration(const Sweep3Args& A, const int inst, const int iter, const TileGrid3& g,
                                             unsigned* cnt, unsigned* slots, const unsigned qmask,
                                             DataflowShared* sh, unsigned char* wsm, const int lane, const int nw) {
    PFAST_TILE_SHAPE(SH);
    const int total = 8 * A.ntiles;
    const int* dirty = A.dirty + (long long)inst * A.ntiles;
    int last_done = -1;
    unsigned long long idle_since = 0;
    for (;;) {
        if (*(volatile int*)&sh->abort) return;   // a stalled block gives up (warp-uniform read)
        // ---- take up to 32 ready items, about this warp's share of the ring
        unsigned h = 0;
        int n = 0;
        if (lane == 0) {
            for (int tries = 0; tries < 32; ++tries) {
                const unsigned hh = *(volatile unsigned*)&sh->head, tt = *(volatile unsigned*)&sh->tail;
                const int avail = (int)(tt - hh);
                if (avail <= 0) break;
                const int want = min(32, max(1, avail / nw));
                if (atomicCAS(&sh->head, hh, hh + (unsigned)want) == hh) { h = hh; n = want; break; }
            }
        }
        n = __shfl_sync(0xffffffffu, n, 0);
        h = __shfl_sync(0xffffffffu, h, 0);
        if (n == 0) {
            const int d = *(volatile int*)&sh->done;
            if (d >= total || *(volatile int*)&sh->abort) return;
            if (lane == 0) {   // nothing ready while other warps work: wait, bounded
                const unsigned long long now = global_ns();
                if (d != last_done) { last_done = d; idle_since = now; }
                else if (now - idle_since > 2000000000ull) *(volatile int*)&sh->abort = 1;
            }
            __nanosleep(128);
            __syncwarp();
            continue;
        }
        unsigned e = kSlotEmpty;
        if (lane < n) {
            unsigned* slot = slots + ((h + (unsigned)lane) & qmask);
            // the item's producer reserved this position before we took it: it is being written
            for (int spin = 0; (e = atomicExch(slot, kSlotEmpty)) == kSlotEmpty; ++spin)
                if (spin > (1 << 22) || *(volatile int*)&sh->abort) { *(volatile int*)&sh->abort = 1; break; }
        }
        __threadfence_block();
        const bool have = e != kSlotEmpty;
        const int x = (int)(e >> 3), o = (int)(e & 7u);
        int dm = 0;
        bool due = false;
        if (have) {
            dm = __ldcg(dirty + x);
            due = tile_due<KIND>(dm, o);
        }
        const unsigned dmask = __ballot_sync(0xffffffffu, due);
        const int mine = dmask ? __ffs(dmask) - 1 : -1;
        int ncomp = 0;
        if (have && !due) {   // locked in this order: nothing to compute
            df_complete(g, cnt, slots, qmask, sh, o, x);
            ncomp = 1;
        }
        if (due && lane != mine) df_push(slots, qmask, sh, e);   // for an idle warp
        if (mine >= 0) {
            const int ex = __shfl_sync(0xffffffffu, x, mine), eo = __shfl_sync(0xffffffffu, o, mine);
            const int edm = __shfl_sync(0xffffffffu, dm, mine);
            const int tj = ex % g.nbj, ti = (ex / g.nbj) % g.nbi, tk = ex / (g.nbj * g.nbi);
            process_tile<KIND, true, SH>(A, inst, ex, tk, ti, tj, eo, iter, edm, wsm, lane);
            __threadfence_block();   // the tile's field and lock words before its dependents start
            __syncwarp();
            if (lane == 0) {
                df_complete(g, cnt, slots, qmask, sh, eo, ex);
                ++ncomp;
            }
        }
        const int c = __reduce_add_sync(0xffffffffu, ncomp);
        if (lane == 0 && c) atomicAdd(&sh->done, c);
    }
}

// Warps per block of the dataflow kernel, at most: what 227 KB of shared memory holds beside
// the counters and ring of an 8192-tile grid (24 at most), so that the register budget of a
// thread follows the block size.  The register-window kinds use no box: 24 warps for the
// forward polish (85 registers a thread; 20 warps measured 2 % slower), 16 for the adjoint
// polish, which also keeps the traveltime windows (128 registers; 20 warps measured 3 % slower).
template <int KIND, class SH>
__host__ __device__ constexpr int df_max_warps() {
    return u_windows<KIND, true>() ? (KIND == kAdjPolish64 ? 16 : 24)
           : (227 * 1024 - 256 - 40960) / warp_smem_bytes<KIND, SH, true>() < 24
               ? (227 * 1024 - 256 - 40960) / warp_smem_bytes<KIND, SH, true>()
               : 24;
}

// MULTI: instances of several grids in one launch.  Item q of the queue is models[items[q].x]'s
// instance items[q].y; the block copies that model's arguments into shared memory when it takes
// the item, and the result goes to the model's `changed` array.  Otherwise the instances are
// A.act[q] of the one grid in A and results go to result[].
template <int KIND, bool MULTI, class SH>
__global__ void __launch_bounds__(df_max_warps<KIND, SH>() * 32, 1) sweep3d_dataflow(const Sweep3Args A0,
                                                                      const Sweep3Args* __restrict__ models,
                                                                      const int2* __restrict__ items, const int nact,
                                                                      const int maxiter, int* __restrict__ queue,
                                                                      int* __restrict__ result, const int qcap) {
    PFAST_TILE_SHAPE(SH);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ DataflowShared sh;
    constexpr bool kSelective = (KIND == kFwdPolish64 || KIND == kAdjPolish64);
    const int nthr = blockDim.x, nw = nthr >> 5;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char* wsm = smem_raw + warp * warp_smem_bytes<KIND, SH, true>();
    // after the warps' boxes: (MULTI: the current model's arguments,) the counters, the ring
    unsigned char* dyn = smem_raw + nw * warp_smem_bytes<KIND, SH, true>();
    Sweep3Args& s_args = *reinterpret_cast<Sweep3Args*>(dyn);
    unsigned* cnt = reinterpret_cast<unsigned*>(dyn + (MULTI ? kDfArgsBytes : 0));
    const unsigned qmask = (unsigned)qcap - 1u;
    int cur_model = -1;
    for (;;) {
        if (threadIdx.x == 0) sh.item = atomicAdd(queue, 1);
        __syncthreads();
        const int item = sh.item;
        __syncthreads();
        if (item >= nact) return;   // block-uniform
        int inst;
        if constexpr (MULTI) {
            const int2 mi = items[item];
            if (mi.x != cur_model) {   // block-uniform
                const int* srcw = reinterpret_cast<const int*>(models + mi.x);
                int* dstw = reinterpret_cast<int*>(&s_args);
                for (int w = threadIdx.x; w < (int)(sizeof(Sweep3Args) / 4); w += nthr) dstw[w] = srcw[w];
                cur_model = mi.x;
                __syncthreads();
            }
            inst = mi.y;
        } else {
            inst = A0.act[item];
        }
        const Sweep3Args& A = MULTI ? s_args : A0;
        const int ntiles = A.ntiles, ncw = (ntiles + 3) >> 2;
        unsigned* slots = cnt + ncw;
        const TileGrid3 g{A.nbk, A.nbi, A.nbj};
        int* diff = A.diff + (long long)inst * ntiles;
        const int* dirty = A.dirty + (long long)inst * ntiles;
        int it = A.iter;   // the first outer iteration (a continuation starts past 0); maxiter is absolute
        bool moved = true, aborted = false;
        while (it < maxiter) {
            // counters of orders 0 and 1, an empty ring, cleared per-tile change flags
            for (int w = threadIdx.x; w < ncw; w += nthr) {
                unsigned v = 0;
                for (int b = 0; b < 4; ++b) {
                    const int x = 4 * w + b;
                    if (x < ntiles) v |= (unsigned)(dep_count(g, 0, x) | (dep_count(g, 1, x) << 4)) << (8 * b);
                }
                cnt[w] = v;
            }
            for (int q = threadIdx.x; q < qcap; q += nthr) slots[q] = kSlotEmpty;
            for (int t = threadIdx.x; t < ntiles; t += nthr) diff[t] = 0;
            if (threadIdx.x == 0) {
                sh.head = 0;
                sh.tail = 1;
                sh.done = 0;
                sh.abort = 0;
            }
            __syncthreads();
            if (threadIdx.x == 0) slots[0] = (unsigned)first_tile(g) << 3;   // (order 0, first tile)
            __syncthreads();
            df_iteration<KIND, SH>(A, inst, it, g, cnt, slots, qmask, &sh, wsm, lane, nw);
            __syncthreads();
            if (sh.abort) { aborted = true; break; }   // block-uniform
            // convergence: some tile moved in this iteration / some tile still due in some order
            int any = 0, due = 0;
            for (int t = threadIdx.x; t < ntiles; t += nthr) {
                any |= __ldcg(diff + t);
                const int dm = __ldcg(dirty + t);
                due |= (kSelective ? (dm & (dm >> 8)) : dm) & 0xff;
            }
            any = __syncthreads_or(any);
            due = __syncthreads_or(due);
            ++it;
            if (!any) { moved = false; break; }
            // moved, but every tile is a fixed point of its update: the next iteration would
            // change nothing and pass the test; it is counted without running
            if (!due && it < maxiter) { ++it; moved = false; break; }
        }
        if (threadIdx.x == 0) {
            int* res = MULTI ? A.changed : result;
            res[inst] = it | (moved ? (1 << 30) : 0) | (aborted ? (1 << 29) : 0);
        }
        if (aborted) {
            if (threadIdx.x == 0) atomicOr(queue + 1, 1);   // the host reports the stall
            return;                                        // block-uniform
        }
    }
}

// Polish pre-pass: lock word of every tile = all eight orders due | (orders in which some node
// of the tile is selected) << 8, the selection computed from the field the polish starts
// from (forward: the widened bulk traveltimes; adjoint: the fixed traveltimes), so that the
// first polish sweep skips the tiles none of whose nodes it selects.  One warp per tile
// (lane = column, looping over the tile's rows) writes the tile's lock word.
template <bool ADJ, class SH>
__global__ void tile_orders_kernel(const Sweep3Args A) {
    PFAST_TILE_SHAPE(SH);
    const int tid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (tid >= A.ntiles) return;   // whole warps
    const int inst = A.act[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int nz = A.nz, nr = A.nr, nc = A.nc;
    const long long plane = (long long)nr * nc;
    const double* f = reinterpret_cast<const double*>(ADJ ? A.aux : A.field) + inst * A.fstride;
    const int tj = tid % A.nbj, ti = (tid / A.nbj) % A.nbi, tk = tid / (A.nbj * A.nbi);
    const int k0 = tk * TK, i0 = ti * TI, j = tj * TJ + lane;
    int sk = 0, si = 0, sj = 0;
    if (!ADJ) { sk = A.src_kij[3 * inst]; si = A.src_kij[3 * inst + 1]; sj = A.src_kij[3 * inst + 2]; }
    const long long inf = dbits(INFINITY);
    unsigned m = 0;
#pragma unroll 4
    for (int r = 0; r < TK * TI; ++r) {   // 4 rows' loads in flight together
        const int k = k0 + r / TI, i = i0 + r % TI;
        if (k >= nz || i >= nr || j >= nc) continue;
        const long long t = k * plane + (long long)i * nc + j;
        const long long xl = j > 0 ? dbits(__ldg(f + t - 1)) : inf, xh = j < nc - 1 ? dbits(__ldg(f + t + 1)) : inf;
        const long long yl = i > 0 ? dbits(__ldg(f + t - nc)) : inf, yh = i < nr - 1 ? dbits(__ldg(f + t + nc)) : inf;
        const long long zl = k > 0 ? dbits(__ldg(f + t - plane)) : inf, zh = k < nz - 1 ? dbits(__ldg(f + t + plane)) : inf;
        if constexpr (ADJ) {
            const bool interior = k >= 1 && k <= nz - 2 && i >= 1 && i <= nr - 2 && j >= 1 && j <= nc - 2;
            const bool fixed = (A.mask[inst * A.mask_stride + ((long long)k * nr + i) * A.wpr + (j >> 5)] >> (j & 31)) & 1u;
            if (interior && !fixed) m |= adj_orders(dbits(__ldg(f + t)), xl, xh, yl, yh, zl, zh);
        } else {
            const int qk = k - sk, qi = i - si, qj = j - sj;
            if (qk * qk + qi * qi + qj * qj > A.src_r2) m |= fwd_orders(dbits(__ldg(f + t)), xl, xh, yl, yh, zl, zh);
        }
    }
    m = __reduce_or_sync(0xffffffffu, m);
    int* w = A.dirty + (long long)inst * A.ntiles + tid;
    if (lane == 0) *w = (*w & 0xff) | (int)(m << 8);
}

// Initial lock words from the field a phase starts from: a tile is due in every order
// (0xff) only if its halo box holds a value an update can propagate -- forward: a reached
// traveltime (below the reference's INF); adjoint: a nonzero lambda -- and locked (0)
// otherwise.  An update whose neighbours and own value are all unreached (all zero) returns
// the same value, so such a tile is a fixed point until a neighbour's change marks it.  That
// holds bit for bit for the reference's updates too: every forward candidate from unreached
// neighbours is at least INF, which the reference's MIN does not take over INF, and the
// adjoint's POS/NEG terms of zero lambdas are +0 or -0, whose difference is +0.  FLOORED (the
// adjoint polish): live only where some |lambda| exceeds a quarter of the polish floor -- an
// update is a weighted sum of its upwind neighbours with weights summing to about 1, so in a
// box of smaller values every correction stays within the floor and is dropped anyway.  One
// warp per tile, lane = column of the box rows.
template <typename Real, bool ADJ, bool FLOORED, class SH>
__global__ void seed_tiles_kernel(const Sweep3Args A) {
    PFAST_TILE_SHAPE(SH);
    const double thr = 0.25 * (double)A.polish_floor;   // FLOORED (adjoint polish): |lambda| above it
    const int tid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (tid >= A.ntiles) return;   // whole warps
    const int inst = A.act[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int nz = A.nz, nr = A.nr, nc = A.nc;
    const long long plane = (long long)nr * nc;
    const Real* f = reinterpret_cast<const Real*>(A.field) + inst * A.fstride;
    const int tj = tid % A.nbj, ti = (tid / A.nbj) % A.nbi, tk = tid / (A.nbj * A.nbi);
    const int k0 = tk * TK, i0 = ti * TI, j0 = tj * TJ;
    auto hit = [&](Real x) -> bool {
        if constexpr (FLOORED) return dbits(fabs(x)) > dbits(thr);
        else return ADJ ? (x != Real(0)) : (x < Real(kInf));
    };
    // the box's HK x HI rows of TJ + 2 columns (lanes: columns j0-1 .. j0+30, lanes 0-1 also
    // j0+31, j0+32), in batches of 12 rows whose loads are all in flight together
    constexpr int kRows = HK * HI, kBatch = 12;
    static_assert(kRows % kBatch == 0, "whole batches");
    const int ja = j0 - 1 + lane, jb = j0 + 31 + lane;
    const bool oka = (unsigned)ja < (unsigned)nc, okb = lane < 2 && (unsigned)jb < (unsigned)nc;
    bool live = false;
    const Real none = ADJ ? Real(0) : Real(kInf);   // a value that is not a hit
#pragma unroll 1
    for (int r0 = 0; r0 < kRows && !live; r0 += kBatch) {
        Real xa[kBatch], xb[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; ++u) {
            const int k = k0 - 1 + (r0 + u) / HI, i = i0 - 1 + (r0 + u) % HI;
            const bool in = (unsigned)k < (unsigned)nz && (unsigned)i < (unsigned)nr;
            const Real* row = f + k * plane + (long long)i * nc;
            xa[u] = in && oka ? __ldg(row + ja) : none;
            xb[u] = in && okb ? __ldg(row + jb) : none;
        }
        bool v = false;
#pragma unroll
        for (int u = 0; u < kBatch; ++u) v |= hit(xa[u]) || hit(xb[u]);
        live = __any_sync(0xffffffffu, v);
    }
    if (lane == 0) A.dirty[(long long)inst * A.ntiles + tid] = live ? 0xff : 0;
}



// Dataflow schedule: shared memory of a block = its warps' tile boxes + the dependency
// counters (one byte per tile) + the ring of ready items (a power of two >= ntiles words).
inline int dataflow_qcap(int ntiles) {
    int q = 1;
    while (q < ntiles) q <<= 1;
    return q;
}

inline size_t dataflow_extra_bytes(int ntiles, bool multi) {
    return (size_t)4 * ((ntiles + 3) / 4) + (size_t)4 * dataflow_qcap(ntiles) + (multi ? kDfArgsBytes : 0);
}

template <int KIND, class SH>
pfast_status launch_one(const Sweep3Args& a, int d0, int tiles, int nact, cudaStream_t st) {
    static bool attr_set = false;
    const size_t smem = (size_t)kWarps3 * warp_smem_bytes<KIND, SH>();
    if (!attr_set) {
        PFAST_CUDA_TRY(cudaFuncSetAttribute(sweep3d_kernel<KIND, SH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)smem));
        attr_set = true;
    }
    dim3 grid((tiles + kWarps3 - 1) / kWarps3, nact);
    sweep3d_kernel<KIND, SH><<<grid, kWarps3 * 32, smem, st>>>(a, d0, tiles);
    return PFAST_OK;
}

template <int KIND, class SH>
pfast_status dataflow_shape_k(int ntiles, int nact, bool multi, int* warps, int* blocks) {
    static std::map<std::tuple<int, int, int, bool>, std::pair<int, int>> cache;   // (device, ntiles, nact, multi)
    static std::mutex mu;
    int dev = 0, sms = 0, smem_max = 0;
    PFAST_CUDA_TRY(cudaGetDevice(&dev));
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(std::make_tuple(dev, ntiles, nact, multi));
        if (it != cache.end()) {
            *warps = it->second.first;
            *blocks = it->second.second;
            return PFAST_OK;
        }
    }
    PFAST_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PFAST_CUDA_TRY(cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const long long room = (long long)smem_max - 256 - (long long)dataflow_extra_bytes(ntiles, multi);
    const int w = (int)std::min<long long>(df_max_warps<KIND, SH>(), room / warp_smem_bytes<KIND, SH, true>());
    if (ntiles > kDataflowMaxTiles || w < 1) {
        *warps = 0;
        *blocks = 0;
        return PFAST_OK;
    }
    const size_t smem = (size_t)w * warp_smem_bytes<KIND, SH, true>() + dataflow_extra_bytes(ntiles, multi);
    auto fn = multi ? sweep3d_dataflow<KIND, true, SH> : sweep3d_dataflow<KIND, false, SH>;
    // the opt-in maximum (less the kernel's static shared memory), not this grid's size: a cached
    // shape of a larger grid launches later with more than a smaller grid's call would allow
    cudaFuncAttributes fa;
    PFAST_CUDA_TRY(cudaFuncGetAttributes(&fa, fn));
    PFAST_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        smem_max - (int)fa.sharedSizeBytes));
    int per_sm = 0;
    PFAST_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, w * 32, smem));
    *warps = w;
    *blocks = std::max(1, std::min(nact, std::max(1, per_sm) * sms));
    std::lock_guard<std::mutex> lk(mu);
    cache[std::make_tuple(dev, ntiles, nact, multi)] = {*warps, *blocks};
    return PFAST_OK;
}

template <int KIND, class SH>
pfast_status launch_dataflow_k(const Sweep3Args& a, int nact, int maxiter, int* queue, int* result, int warps,
                               int blocks, cudaStream_t st) {
    const size_t smem = (size_t)warps * warp_smem_bytes<KIND, SH, true>() + dataflow_extra_bytes(a.ntiles, false);
    sweep3d_dataflow<KIND, false, SH><<<blocks, warps * 32, smem, st>>>(a, nullptr, nullptr, nact, maxiter, queue,
                                                                        result, dataflow_qcap(a.ntiles));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "dataflow sweep launch", __FILE__, __LINE__);
    return PFAST_OK;
}

template <int KIND, class SH>
pfast_status launch_dataflow_multi_k(const Sweep3Args* models, const int2* items, int nitems, int max_ntiles,
                                     int maxiter, int* queue, int warps, int blocks, cudaStream_t st) {
    const size_t smem = (size_t)warps * warp_smem_bytes<KIND, SH, true>() + dataflow_extra_bytes(max_ntiles, true);
    Sweep3Args unused;
    std::memset(&unused, 0, sizeof(unused));
    sweep3d_dataflow<KIND, true, SH><<<blocks, warps * 32, smem, st>>>(unused, models, items, nitems, maxiter, queue,
                                                                       nullptr, dataflow_qcap(max_ntiles));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "dataflow sweep launch", __FILE__, __LINE__);
    return PFAST_OK;
}

}  // namespace

// Calls F<KIND>::run(args...) for the sweep kind given at run time.
#define PFAST_KIND_SWITCH(kind, CALL)                        \
    switch (kind) {                                          \
        case kFwdPlain64: { constexpr int K = kFwdPlain64; return CALL; }   \
        case kFwdFast32: { constexpr int K = kFwdFast32; return CALL; }     \
        case kFwdPolish64: { constexpr int K = kFwdPolish64; return CALL; } \
        case kAdjPlain64: { constexpr int K = kAdjPlain64; return CALL; }   \
        case kAdjFast32: { constexpr int K = kAdjFast32; return CALL; }     \
        case kAdjPolish64: { constexpr int K = kAdjPolish64; return CALL; } \
    }                                                        \
    set_last_error("unknown sweep kind %d", kind);           \
    return PFAST_ERR_INVALID

template <class SH>
pfast_status ShapeLaunchers<SH>::sweep(int kind, const Sweep3Args& a, int d0, int tiles, int nact, cudaStream_t st) {
    PFAST_KIND_SWITCH(kind, (launch_one<K, SH>(a, d0, tiles, nact, st)));
}

template <class SH>
pfast_status ShapeLaunchers<SH>::dataflow(int kind, const Sweep3Args& a, int nact, int maxiter, int* queue,
                                          int* result, int warps, int blocks, cudaStream_t st) {
    PFAST_KIND_SWITCH(kind, (launch_dataflow_k<K, SH>(a, nact, maxiter, queue, result, warps, blocks, st)));
}

template <class SH>
pfast_status ShapeLaunchers<SH>::dataflow_multi(int kind, const Sweep3Args* models, const int2* items, int nitems,
                                                int max_ntiles, int maxiter, int* queue, int warps, int blocks,
                                                cudaStream_t st) {
    PFAST_KIND_SWITCH(kind, (launch_dataflow_multi_k<K, SH>(models, items, nitems, max_ntiles, maxiter, queue, warps,
                                                             blocks, st)));
}

template <class SH>
pfast_status ShapeLaunchers<SH>::dataflow_shape(int kind, int ntiles, int nact, bool multi, int* warps, int* blocks) {
    PFAST_KIND_SWITCH(kind, (dataflow_shape_k<K, SH>(ntiles, nact, multi, warps, blocks)));
}

template <class SH>
pfast_status ShapeLaunchers<SH>::seed(int kind, const Sweep3Args& a, int nact, cudaStream_t st) {
    if (nact <= 0) return PFAST_OK;
    dim3 grid((unsigned)((a.ntiles + 7) / 8), nact);
    switch (kind) {
        case kFwdPlain64: seed_tiles_kernel<double, false, false, SH><<<grid, 256, 0, st>>>(a); break;
        case kAdjPlain64: seed_tiles_kernel<double, true, false, SH><<<grid, 256, 0, st>>>(a); break;
        case kFwdFast32: seed_tiles_kernel<float, false, false, SH><<<grid, 256, 0, st>>>(a); break;
        case kAdjFast32: seed_tiles_kernel<float, true, false, SH><<<grid, 256, 0, st>>>(a); break;
        case kAdjPolish64: seed_tiles_kernel<double, true, true, SH><<<grid, 256, 0, st>>>(a); break;
        default: return PFAST_OK;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "seed tiles launch", __FILE__, __LINE__);
    return PFAST_OK;
}

template <class SH>
pfast_status ShapeLaunchers<SH>::orders(int kind, const Sweep3Args& a, int nact, cudaStream_t st) {
    if (nact <= 0) return PFAST_OK;
    dim3 grid((unsigned)((a.ntiles + 7) / 8), nact);
    if (kind == kAdjPolish64) tile_orders_kernel<true, SH><<<grid, 256, 0, st>>>(a);
    else tile_orders_kernel<false, SH><<<grid, 256, 0, st>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "polish orders launch", __FILE__, __LINE__);
    return PFAST_OK;
}

}  // namespace pfast
