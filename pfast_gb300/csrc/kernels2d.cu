// kernels2d.cu -- 2D fast-sweeping Eikonal (with Huygens reflection) and adjoint
// kernels for sm_103a.
//
// Same scheme as the 3D kernels: the 4 sweep orders of the reference
// (src/RT_pfsm2d.h:168-181, src/RT_padjoint2d.h:351-369) are run as wavefronts of
// T2I x T2J tiles (one launch per tile anti-diagonal); inside a tile lane = row,
// and step t updates the node anti-diagonal li + lj = t.  Upstream neighbours are
// final and downstream ones untouched when a node is updated, exactly as in the
// reference's lexicographic loop, so the plain FP64 flavour is bit-identical.

#include <vector>
#include <algorithm>
#include "kernels2d.h"

namespace pfast {

namespace {

template <int KIND> struct Traits2;
template <> struct Traits2<kFwdPlain64>  { using Real = double; using Aux = double; static constexpr bool adj = false; };
template <> struct Traits2<kFwdFast32>   { using Real = float;  using Aux = float;  static constexpr bool adj = false; };
template <> struct Traits2<kFwdPolish64> { using Real = double; using Aux = double; static constexpr bool adj = false; };
template <> struct Traits2<kAdjPlain64>  { using Real = double; using Aux = double; static constexpr bool adj = true; };
template <> struct Traits2<kAdjFast32>   { using Real = float;  using Aux = float;  static constexpr bool adj = true; };
template <> struct Traits2<kAdjPolish64> { using Real = double; using Aux = double; static constexpr bool adj = true; };

// The FP64 adjoint kinds read the traveltime through register windows (no second FP64 box);
// the FP32 bulk adjoint stages it as a box of FP32 offsets.
template <int KIND>
__host__ __device__ constexpr bool t_windows2() {
    return Traits2<KIND>::adj && sizeof(typename Traits2<KIND>::Aux) == 8;
}

template <int KIND>
__host__ __device__ constexpr int warp_smem2() {
    using T = Traits2<KIND>;
    return int(H2I * R2 * sizeof(typename T::Real) +
               (T::adj && !t_windows2<KIND>() ? H2I * R2 * sizeof(typename T::Aux) : 0));
}

__device__ __forceinline__ double ref_min(double x, double y) { return (x < y) ? x : y; }
__device__ __forceinline__ float ref_min(float x, float y) { return (x < y) ? x : y; }

// Reference 2D Godunov update (src/RT_pfsm2d.h:89-102), operand order kept.
// a: x-neighbour minimum (spacing dx), b: z-neighbour minimum (dz).
__device__ __forceinline__ double eik2_plain(double a, double b, double s, double dx, double dz, double i2x,
                                             double i2z) {
    double da = dx, db = dz, ia = i2x, ib = i2z, t;
    if (b > a) { t = a; a = b; b = t; t = da; da = db; db = t; t = ia; ia = ib; ib = t; }
    double q = b + db * s;
    if (q <= a) return q;
    const double A = ia + ib;   // 1.0/da/da + 1.0/db/db with each term precomputed as (1.0/d)/d
    const double B = -2. * (a / da / da + b / db / db);
    const double C = a * a / da / da + b * b / db / db - s * s;
    const double D = B * B - 4 * A * C;
    return (D >= 0) ? (-B + sqrt(D)) / 2. / A : kInf;
}

// Same solution in difference form: x = q - b, with B = a - b >= 0:
//   1 term  x = db*s;  2 terms  x = (wa*B + sqrt((wa+wb) s^2 - wa wb B^2)) / (wa+wb)
template <typename R>
__device__ __forceinline__ R eik2_fast(R a, R b, R s, R dx, R dz, R wx, R wz, R rsum) {
    R da = dx, db = dz, wa = wx, wb = wz, t;
    if (b > a) { t = a; a = b; b = t; t = da; da = db; db = t; t = wa; wa = wb; wb = t; }
    R q = fma(db, s, b);
    if (q <= a) return q;
    const R B = a - b;
    const R waB = wa * B;
    const R D = fma(wa + wb, s * s, -waB * wb * B);
    return (D >= R(0)) ? b + (waB + sqrt(D)) * rsum : R(kInf);
}

__device__ __forceinline__ double pos_ref(double x) { return (x + fabs(x)) / 2.0; }
__device__ __forceinline__ double neg_ref(double x) { return (x - fabs(x)) / 2.0; }

// Reference 2D adjoint update (src/RT_padjoint2d.h:42-65).
__device__ __forceinline__ double adj2_plain(double T0, double Txp, double Txm, double Tzp, double Tzm, double Lxp,
                                             double Lxm, double Lzp, double Lzm, double dx, double dz) {
    if (Txp >= kInf || T0 >= kInf || Txm >= kInf || Tzp >= kInf || Tzm >= kInf) return 0.0;
    const double gxp = -(Txp - T0) / dx, gxm = -(T0 - Txm) / dx;
    const double gzp = -(Tzp - T0) / dz, gzm = -(T0 - Tzm) / dz;
    const double a1 = pos_ref(gxp), a2 = neg_ref(gxm);
    const double b1 = pos_ref(gzp), b2 = neg_ref(gzm);
    const double La1 = pos_ref(gxm) * Lxm, La2 = neg_ref(gxp) * Lxp;
    const double Lb1 = pos_ref(gzm) * Lzm, Lb2 = neg_ref(gzp) * Lzp;
    if (fabs((a1 - a2) / dx + (b1 - b2) / dz) > 1e-9)
        return ((La1 - La2) / dx + (Lb1 - Lb2) / dz) / ((a1 - a2) / dx + (b1 - b2) / dz);
    return 0.0;
}

// Fast adjoint forms (see kernels3d.cu): den = sum_m w_m max(-e_m, 0),
// num = sum_m w_m max(e_m, 0) lambda_m with e_m = T_m - T0.
template <typename R>
__device__ __forceinline__ void adj2_terms(R T0, R Txp, R Txm, R Tzp, R Tzm, R Lxp, R Lxm, R Lzp, R Lzm, R wx, R wz,
                                           R& num, R& den) {
    const R z = R(0);
    R e;
    e = Txp - T0; den = wx * fmax(-e, z); num = wx * fmax(e, z) * Lxp;
    e = Txm - T0; den = fma(wx, fmax(-e, z), den); num = fma(wx * fmax(e, z), Lxm, num);
    e = Tzp - T0; den = fma(wz, fmax(-e, z), den); num = fma(wz * fmax(e, z), Lzp, num);
    e = Tzm - T0; den = fma(wz, fmax(-e, z), den); num = fma(wz * fmax(e, z), Lzm, num);
}

__device__ __forceinline__ float adj2_bulk(float T0, float Txp, float Txm, float Tzp, float Tzm, float Lxp, float Lxm,
                                           float Lzp, float Lzm, float wx, float wz) {
    const float ti = INFINITY;
    if (Txp >= ti || T0 >= ti || Txm >= ti || Tzp >= ti || Tzm >= ti) return 0.f;
    float num, den;
    adj2_terms<float>(T0, Txp, Txm, Tzp, Tzm, Lxp, Lxm, Lzp, Lzm, wx, wz, num, den);
    return (fabsf(den) > 1e-9f) ? __fdividef(num, den) : 0.f;
}

// FP64 polish adjoint update in residual-correction form (see kernels3d.cu): with mu_m =
// lambda_m where e_m > 0 and lambda0 where e_m < 0, r = num - den*lambda0 = sum_m w_m e_m mu_m
// in FP64 (11 FP64 instructions); den only scales the step and is FP32.  big: the FP32 step
// leaves a remainder above the floor.
__device__ __forceinline__ double adj2_polish(double T0, double Txp, double Txm, double Tzp, double Tzm, double Lxp,
                                              double Lxm, double Lzp, double Lzm, double L0, double wx, double wz,
                                              float wxf, float wzf, float floor, bool& big, float& dstep) {
    dstep = INFINITY;   // the branches that reset lambda to 0
    const long long inf = dbits(kInf);   // T >= INF on the bit patterns (T >= 0)
    if (dbits(Txp) >= inf || dbits(T0) >= inf || dbits(Txm) >= inf || dbits(Tzp) >= inf || dbits(Tzm) >= inf)
        return 0.0;
    const double exp_ = Txp - T0, exm = Txm - T0, ezp = Tzp - T0, ezm = Tzm - T0;
    auto mu = [&](double e, double L) { return __double2hiint(e) < 0 ? L0 : L; };
    auto nf = [](double e) { return __double2hiint(e) < 0 ? -narrow_trunc(e) : 0.0f; };   // max(-e, 0)
    const double r = fma(wx, fma(exp_, mu(exp_, Lxp), exm * mu(exm, Lxm)),
                         wz * fma(ezp, mu(ezp, Lzp), ezm * mu(ezm, Lzm)));
    const float den = wxf * (nf(exp_) + nf(exm)) + wzf * (nf(ezp) + nf(ezm));
    if (!(den > 1e-9f)) return 0.0;
    const float step = __fdividef(narrow_trunc(r), den);
    const float tol = floor * (1.0f + fabsf(narrow_trunc(L0)));
    big = fabsf(step) * 1.2e-7f > tol;
    dstep = fabsf(step);
    // corrections far below the convergence tolerance are dropped (bitwise fixed point, tiles lock)
    return fabsf(step) <= tol ? L0 : L0 + widen_exact(step);
}

// FP64 polish Godunov update, one Newton step on f(q) = wx max(q-a,0)^2 + wz max(q-b,0)^2 - s^2
// (FP64 differences and residual, 8 FP64 instructions; FP32 derivative and step); a: x-neighbour
// minimum, b: z-neighbour minimum.  big: the step's second-order remainder exceeds the floor.
__device__ __forceinline__ double eik2_newton(double U0, double a, double b, double s, double dx, double dz, double wx,
                                              double wz, float wxf, float wzf, float floor, bool& big,
                                              float& dstep) {
    const double px = pos_sign(U0 - a), pz = pos_sign(U0 - b);
    const double f = fma(wx * px, px, fma(wz * pz, pz, -s * s));
    const float fp = 2.0f * (wxf * narrow_trunc(px) + wzf * narrow_trunc(pz));
    if (!(fp > 0.0f)) {
        big = true;
        dstep = INFINITY;   // a restart: the change is not a Newton step
        return fmin(fma(dx, s, a), fma(dz, s, b));
    }
    const float step = __fdividef(narrow_trunc(f), fp);
    const float sw = (dbits(px) > 0 ? wxf : 0.0f) + (dbits(pz) > 0 ? wzf : 0.0f);
    big = sw * step * step > floor * fp;
    dstep = fabsf(step);   // the change of the node, to FP32 precision
    return fabsf(step) <= floor ? U0 : U0 - widen_exact(step);   // bitwise fixed point once converged
}

// Ordered integer of a value >= 0 (its bit pattern), FP32 or FP64.
__device__ __forceinline__ long long obits2(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ long long obits2(float x) { return __float_as_int(x); }

// Bitwise equality of two field values (FP32 or FP64).
template <typename Real>
__device__ __forceinline__ bool bits_same(Real a, Real b) {
    if constexpr (sizeof(Real) == 8) return __double_as_longlong(a) == __double_as_longlong(b);
    else return __float_as_uint(a) == __float_as_uint(b);
}

// ----------------------------------------------------------- quadrant selection (2D polish)
// Sweep order o: bit 0 = columns ascending, bit 1 = rows ascending.  The 2D form of the 3D
// octant selection: a polish update runs only in the orders that visit the node's active
// upwind neighbours (forward) / its larger-traveltime neighbours (adjoint) first.
constexpr unsigned kAscX2 = 0xa, kDescX2 = 0x5, kAscZ2 = 0xc, kDescZ2 = 0x3;

__device__ __forceinline__ unsigned fwd_orders2(long long u, long long xlo, long long xhi, long long zlo,
                                                long long zhi) {
    unsigned m = 0xf;
    if (u > (xlo < xhi ? xlo : xhi)) m &= xlo < xhi ? kAscX2 : (xhi < xlo ? kDescX2 : 0xfu);
    if (u > (zlo < zhi ? zlo : zhi)) m &= zlo < zhi ? kAscZ2 : (zhi < zlo ? kDescZ2 : 0xfu);
    return m;
}

__device__ __forceinline__ unsigned adj_orders2(long long t, long long xlo, long long xhi, long long zlo,
                                                long long zhi) {
    unsigned m = 0xf;
    const bool a = xlo > t, b = xhi > t, c = zlo > t, e = zhi > t;
    if (a != b) m &= a ? kAscX2 : kDescX2;
    if (c != e) m &= c ? kAscZ2 : kDescZ2;
    return m;
}

template <typename Dst, typename Src, typename Conv>
__device__ __forceinline__ void load_box2(Dst* box, const Src* __restrict__ g, int i0, int j0, int nr, int nc,
                                          Dst fill, int lane, Conv conv) {
    constexpr int NE = H2I * H2J;
    constexpr int BATCH = 16;
#pragma unroll 1
    for (int base = 0; base < NE; base += 32 * BATCH) {
        Dst v[BATCH];
#pragma unroll
        for (int u = 0; u < BATCH; ++u) {
            const int e = base + u * 32 + lane;
            v[u] = fill;
            if (e < NE) {
                const int y = e / H2J, x = e - y * H2J;
                const int gi = i0 - 1 + y, gj = j0 - 1 + x;
                if ((unsigned)gi < (unsigned)nr && (unsigned)gj < (unsigned)nc) v[u] = conv(g[(long long)gi * nc + gj]);
            }
        }
#pragma unroll
        for (int u = 0; u < BATCH; ++u) {
            const int e = base + u * 32 + lane;
            if (e < NE) {
                const int y = e / H2J, x = e - y * H2J;
                box[y * R2 + x] = v[u];
            }
        }
    }
}

struct Ident2 {
    template <typename T> __device__ __forceinline__ T operator()(T v) const { return v; }
};

// Initial lock words from the field a phase starts from (as in the 3D sweeps): a tile is due
// in every order only if its halo box holds a reached traveltime (forward) or a nonzero lambda
// (adjoint); otherwise it is a fixed point of the update until a neighbour's change marks it.
// SEL (the adjoint polish): an idle tile keeps all four orders selected (bits 4-7), so that a
// neighbour's mark makes it due, and a tile counts as live only where some |lambda| exceeds a
// quarter of the polish floor (smaller values give corrections within the floor).  One warp per tile, lane = column of the box rows.
template <typename Real, bool ADJ, bool SEL>
__global__ void seed_tiles2_kernel(const Sweep2Args A) {
    const double thr = 0.25 * (double)A.polish_floor;   // SEL (adjoint polish): |lambda| above it
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (t >= A.ntiles) return;   // whole warps
    const int q = A.act[blockIdx.y];
    const int lane = threadIdx.x & 31;
    const int nr = A.nr, nc = A.nc;
    const Real* f = reinterpret_cast<const Real*>(A.field) + A.inst_off[q];
    const int i0 = (t / A.nbj) * T2I, j0 = (t % A.nbj) * T2J;
    bool live = false;
#pragma unroll 1
    for (int i = i0 - 1; i <= i0 + T2I && !live; ++i) {
        if ((unsigned)i >= (unsigned)nr) continue;
        bool v = false;
        for (int j = j0 - 1 + lane; j <= j0 + T2J; j += 32) {
            if ((unsigned)j >= (unsigned)nc) continue;
            const Real x = __ldg(f + (long long)i * nc + j);
            if constexpr (ADJ && SEL) v |= dbits(fabs(x)) > dbits(thr);
            else v |= ADJ ? (x != Real(0)) : (x < Real(kInf));
        }
        live = __any_sync(0xffffffffu, v);
    }
    if (lane == 0) A.dirty[(long long)q * A.ntiles + t] = live ? 0xff : (SEL ? 0xf0 : 0);
}

template <int KIND>
__global__ void __launch_bounds__(kWarps2 * 32) sweep2d_kernel(const Sweep2Args A, const int d) {
    using Real = typename Traits2<KIND>::Real;
    using Aux = typename Traits2<KIND>::Aux;
    constexpr bool ADJ = Traits2<KIND>::adj;
    extern __shared__ __align__(16) unsigned char smem_raw[];

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int d0 = A.diag_off[d];
    const int tile_idx = blockIdx.x * kWarps2 + warp;
    if (tile_idx >= A.diag_off[d + 1] - d0) return;
    int iter = A.iter;
    if (A.dyn) {   // replayed iteration graph
        if ((int)blockIdx.y >= __ldcg(A.dyn + 1)) return;
        iter = __ldcg(A.dyn);
    }
    const int q = A.act[blockIdx.y];

    const unsigned pk = A.diag_tiles[d0 + tile_idx];
    const bool py = A.dir & 2, px = A.dir & 1;
    const int bif = pk & 0xffff, bjf = pk >> 16;
    const int ti = py ? bif : A.nbi - 1 - bif;
    const int tj = px ? bjf : A.nbj - 1 - bjf;
    // tile locking, as in the 3D sweeps: bits 0-3 = orders still to process, bits 4-7 (polish)
    // = orders in which some node of the tile is selected
    constexpr bool kSelective = (KIND == kFwdPolish64 || KIND == kAdjPolish64);
    const int tid = ti * A.nbj + tj;
    int* dirty = A.dirty + (long long)q * A.ntiles;
    const int dm = __ldcg(dirty + tid);
    const int obit = 1 << A.dir;
    const int omask = kSelective ? (dm >> 4) & 0xf : 0xf;
    if (!(dm & omask & obit)) return;   // locked for this order (warp-uniform)
    __syncwarp();
    // Convergence test of the mixed kinds (FP32 bulk, polish): a node that moved by more than
    // the tolerance in some processing of this outer iteration, ORed over the iteration (a
    // polish change is its FP32 step).  The plain kinds compare with a snapshot taken at the
    // tile's first processing in the iteration, as the reference's isconv does.
    constexpr bool kSnap = KIND == kFwdPlain64 || KIND == kAdjPlain64;
    // the tile's lock word as lane 0 last wrote it (no other tile of this launch writes it)
    int dword = kSelective ? (dm & ~obit) : 0;
    if (lane == 0) {
        dirty[tid] = dword;
        if (A.work) atomicAdd(A.work + q, (unsigned long long)(min(T2I, A.nr - ti * T2I) * min(T2J, A.nc - tj * T2J)));
    }
    const int i0 = ti * T2I, j0 = tj * T2J;
    const int nr = A.nr, nc = A.nc;
    const int ei = min(T2I, nr - i0), ej = min(T2J, nc - j0);
    const long long n = (long long)nr * nc;

    Real* box = reinterpret_cast<Real*>(smem_raw + warp * warp_smem2<KIND>());
    Aux* tbox = reinterpret_cast<Aux*>(reinterpret_cast<unsigned char*>(box) + H2I * R2 * sizeof(Real));
    Real* fld = reinterpret_cast<Real*>(A.field) + A.inst_off[q];
    Real* snp = kSnap ? reinterpret_cast<Real*>(A.snap) + q * n : nullptr;

    const Real fill = ADJ ? Real(0) : Real(INFINITY);
    load_box2(box, fld, i0, j0, nr, nc, fill, lane, Ident2());

    const int lif = lane;
    const bool lane_ok = lif < ei;
    const int li = py ? lif : ei - 1 - lif;
    const int gi = i0 + li;
    unsigned fixed_lo = 0, fixed_hi = 0;
    if constexpr (ADJ) {
        const double* T = reinterpret_cast<const double*>(A.aux) + A.aux_off[q];
        if constexpr (!t_windows2<KIND>()) {
            // offsets from the tile corner's traveltime, formed without FP64 instructions
            const long long inf = dbits(kInf);
            double tr = T[(long long)i0 * nc + j0];
            if (dbits(tr) >= inf) tr = 0.0;
            load_box2(tbox, T, i0, j0, nr, nc, Aux(0), lane,
                      [tr, inf](double v) { return dbits(v) >= inf ? (Aux)INFINITY : (Aux)offset_f32(v, tr); });
        }
        if (lane_ok) {
            const unsigned* mrow = A.mask + A.mask_off[q] + (long long)gi * A.wpr + (j0 >> 5);
            fixed_lo = mrow[0];
            if ((j0 >> 5) + 1 < A.wpr) fixed_hi = mrow[1];
        }
    }

    // snapshot at the tile's first processing in this outer iteration (plain kinds)
    if constexpr (kSnap) {
        int* stamp = A.stamp + (long long)q * A.ntiles;
        if (__ldcg(stamp + tid) != iter) {
            for (int y = 0; y < ei; ++y)
                for (int x = lane; x < ej; x += 32) snp[(long long)(i0 + y) * nc + j0 + x] = box[(y + 1) * R2 + x + 1];
            if (lane == 0) stamp[tid] = iter;
        }
    }
    __syncwarp();
    bool moved = false;
    const float tabs_f = narrow_trunc(A.tol_abs), trel_f = narrow_trunc(A.tol_rel);   // FP32 kinds' test
    // the mixed kinds' test at a changed node (old -> nv; dstep: the polish step's size)
    auto note_move = [&](Real old, Real nv, float dstep) {
        if constexpr (kSelective) {
            if (dstep > tabs_f) moved = true;
        } else if constexpr (!kSnap) {
            if (fabsf(old - nv) > tabs_f + trel_f * fabsf(nv)) moved = true;
        }
    };

    int lim_row = -1, si = -1, sj = -1;
    if (A.inst_lim[q] >= 0) lim_row = A.inst_lim[q];
    if (A.inst_src[q] >= 0) { si = A.inst_src[q] >> 16; sj = A.inst_src[q] & 0xffff; }
    const int* rl = lim_row >= 0 ? A.rowlim + (long long)lim_row * nc : nullptr;
    const Aux* slow = reinterpret_cast<const Aux*>(A.aux);
    const bool row_interior = gi >= 1 && gi <= nr - 2;

    const float wx = A.wxf, wz = A.wzf, rsum = A.rsumf;
    const int cb = (li + 1) * R2 + 1;
    const int steps = ei + ej - 1;
    bool chg = false, chg_jlo = false, chg_jhi = false;
    unsigned sel = 0;
    // Face marks and own re-marking as in the 3D sweeps: the plain kinds mark every changed
    // face node; the others only where the neighbour's node depends on the changed one (forward:
    // a neighbour below the node's value; adjoint: a larger traveltime).
    constexpr bool kPrune = KIND != kFwdPlain64 && KIND != kAdjPlain64;
    bool m_ilo = false, m_ihi = false;
    bool restep = false;   // polish: a remainder above the floor (visit again in this order)
    bool stale = false;    // FP32 bulk: a changed node feeds an in-tile node visited before it

    // ---- adjoint traveltime of the FP64 kinds through register windows (as in the 3D sweeps):
    // lane lif (flipped row) is at flipped column jf = t - lif in step t and keeps its row's
    // traveltimes at jf-1, jf, jf+1 (loads issued three steps ahead); lane lif-1 is one column
    // ahead and lane lif+1 one behind, so their windows hold the rows above and below at jf;
    // lanes 0 and ei-1 read the halo rows outside the tile at their own position.
    constexpr bool TWIN2 = t_windows2<KIND>();
    const double* Tq = TWIN2 ? reinterpret_cast<const double*>(A.aux) + A.aux_off[q] : nullptr;
    const int glo = i0 + (py ? -1 : ei), ghi = i0 + (py ? ei : -1);   // rows of flipped rows -1 and ei
    const double* trow = (TWIN2 && lane_ok) ? Tq + (long long)gi * nc : nullptr;
    const double* hlrow = (TWIN2 && lif == 0 && (unsigned)glo < (unsigned)nr) ? Tq + (long long)glo * nc : nullptr;
    const double* hhrow =
        (TWIN2 && lif == ei - 1 && (unsigned)ghi < (unsigned)nr) ? Tq + (long long)ghi * nc : nullptr;
    auto tl = [&](const double* r, int p, int plo, int phi) -> double {
        const int g = j0 + (px ? p : ej - 1 - p);
        return (r != nullptr && p >= plo && p <= phi && (unsigned)g < (unsigned)nc) ? __ldg(r + g) : 0.0;
    };
    double tm = 0.0, t0w = 0.0, tp = 0.0, q1 = 0.0, q2 = 0.0;
    double hl0 = 0.0, hl1 = 0.0, hl2 = 0.0, hh0 = 0.0, hh1 = 0.0, hh2 = 0.0;
    if constexpr (TWIN2) {
        const int f0 = -lif;
        tm = tl(trow, f0 - 1, -1, ej); t0w = tl(trow, f0, -1, ej); tp = tl(trow, f0 + 1, -1, ej);
        q1 = tl(trow, f0 + 2, -1, ej); q2 = tl(trow, f0 + 3, -1, ej);
        hl0 = tl(hlrow, f0, 0, ej - 1); hl1 = tl(hlrow, f0 + 1, 0, ej - 1); hl2 = tl(hlrow, f0 + 2, 0, ej - 1);
        hh0 = tl(hhrow, f0, 0, ej - 1); hh1 = tl(hhrow, f0 + 1, 0, ej - 1); hh2 = tl(hhrow, f0 + 2, 0, ej - 1);
    }

#pragma unroll 1
    for (int t = 0; t < steps; ++t) {
        const int ljf = t - lif;
        // adjoint: the traveltimes around this lane's node, in grid orientation
        Aux T0 = Aux(0), Txm = Aux(0), Txp = Aux(0), Tzm = Aux(0), Tzp = Aux(0);
        if constexpr (TWIN2) {
            const double up = __shfl_sync(0xffffffffu, tm, (lane - 1) & 31);
            const double dn = __shfl_sync(0xffffffffu, tp, (lane + 1) & 31);
            const double fim = lif == 0 ? hl0 : up, fip = lif == ei - 1 ? hh0 : dn;
            T0 = t0w;
            Txm = px ? tm : tp; Txp = px ? tp : tm;
            Tzm = py ? fim : fip; Tzp = py ? fip : fim;
        }
        if (lane_ok && ljf >= 0 && ljf < ej) {
            const int lj = px ? ljf : ej - 1 - ljf;
            const int c = cb + lj;
            const int gj = j0 + lj;
            if constexpr (!ADJ) {
                // the source node (and the opt-in fixed region around it) keeps its value
                const bool upd = (rl == nullptr || gi <= __ldg(rl + gj)) &&
                                 (si < 0 || (gi - si) * (gi - si) + (gj - sj) * (gj - sj) > A.src_r2);
                if (upd) {
                    const Real old = box[c];
                    Real nv = old;
                    float dstep = INFINITY;   // polish: the size of this node's change
                    const Real bz = ref_min(box[c - R2], box[c + R2]);
                    const Real ax = ref_min(box[c + 1], box[c - 1]);
                    const Real s = __ldg(slow + (long long)gi * nc + gj);
                    if constexpr (KIND == kFwdPlain64) {
                        const double qv = eik2_plain(ax, bz, s, A.dx, A.dz, A.inv2x, A.inv2z);
                        nv = ref_min(old, qv);
                    } else if constexpr (KIND == kFwdFast32) {
                        const float qv = eik2_fast<float>(ax, bz, s, A.dxf, A.dzf, wx, wz, rsum);
                        nv = ref_min(old, qv);
                    } else {
                        const unsigned m = fwd_orders2(dbits(old), dbits(box[c - 1]), dbits(box[c + 1]),
                                                       dbits(box[c - R2]), dbits(box[c + R2]));
                        sel |= m;
                        if (m & obit) {
                            bool big = false;
                            nv = eik2_newton(old, ax, bz, s, A.dx, A.dz, A.inv2x, A.inv2z, A.wxf, A.wzf,
                                             A.polish_floor, big, dstep);
                            restep |= big;
                        }
                    }
                    if (!bits_same(old, nv)) {
                        box[c] = nv;
                        chg = true;
                        note_move(old, nv, dstep);
                        if constexpr (kPrune) {
                            auto dep = [&](int n) { return min(obits2(old), obits2(nv)) < obits2(box[n]); };
                            if (li == 0 && dep(c - R2)) m_ilo = true;
                            if (li == ei - 1 && dep(c + R2)) m_ihi = true;
                            if (lj == 0 && dep(c - 1)) chg_jlo = true;
                            if (lj == ej - 1 && dep(c + 1)) chg_jhi = true;
                            if constexpr (!kSelective) {
                                if (lif > 0 && dep(py ? c - R2 : c + R2)) stale = true;
                                if (ljf > 0 && dep(px ? c - 1 : c + 1)) stale = true;
                            }
                        } else {
                            if (lj == 0) chg_jlo = true;
                            if (lj == ej - 1) chg_jhi = true;
                        }
                    }
                }
            } else {
                const unsigned fb = lj < 32 ? (fixed_lo >> lj) : (fixed_hi >> (lj - 32));
                if (row_interior && gj >= 1 && gj <= nc - 2 && !(fb & 1u)) {
                    const Real old = box[c];
                    Real r = old;
                    float dstep = INFINITY;   // polish: the size of this node's change
                    if constexpr (!TWIN2) {   // FP32 bulk: from the staged offsets
                        T0 = tbox[c]; Txp = tbox[c + 1]; Txm = tbox[c - 1]; Tzp = tbox[c + R2]; Tzm = tbox[c - R2];
                    }
                    if constexpr (KIND == kAdjPlain64) {
                        r = adj2_plain(T0, Txp, Txm, Tzp, Tzm, box[c + 1], box[c - 1], box[c + R2], box[c - R2], A.dx,
                                       A.dz);
                    } else if constexpr (KIND == kAdjFast32) {
                        r = adj2_bulk(T0, Txp, Txm, Tzp, Tzm, box[c + 1], box[c - 1], box[c + R2], box[c - R2], wx, wz);
                    } else {
                        const unsigned m = adj_orders2(dbits(T0), dbits(Txm), dbits(Txp), dbits(Tzm), dbits(Tzp));
                        sel |= m;
                        if (m & obit) {
                            bool big = false;
                            r = adj2_polish(T0, Txp, Txm, Tzp, Tzm, box[c + 1], box[c - 1], box[c + R2], box[c - R2],
                                            old, A.inv2x, A.inv2z, A.wxf, A.wzf, A.polish_floor, big, dstep);
                            restep |= big;
                        }
                    }
                    if (!bits_same(old, r)) {
                        box[c] = r;
                        chg = true;
                        note_move(old, r, dstep);
                        if constexpr (kPrune) {
                            // lambda at the neighbour node reads this node if its traveltime is larger
                            // (FP32 bulk: offsets from the tile's corner, compared as values)
                            auto dep = [&](Aux tn) {
                                if constexpr (sizeof(Aux) == 8) return obits2(T0) > obits2(tn);
                                else return T0 > tn;
                            };
                            if (li == 0 && dep(Tzm)) m_ilo = true;
                            if (li == ei - 1 && dep(Tzp)) m_ihi = true;
                            if (lj == 0 && dep(Txm)) chg_jlo = true;
                            if (lj == ej - 1 && dep(Txp)) chg_jhi = true;
                            if constexpr (!kSelective) {
                                if (lif > 0 && dep(py ? Tzm : Tzp)) stale = true;
                                if (ljf > 0 && dep(px ? Txm : Txp)) stale = true;
                            }
                        } else {
                            if (lj == 0) chg_jlo = true;
                            if (lj == ej - 1) chg_jhi = true;
                        }
                    }
                }
            }
        }
        if constexpr (TWIN2) {   // slide the windows to step t + 1
            tm = t0w; t0w = tp; tp = q1; q1 = q2; q2 = tl(trow, t + 4 - lif, -1, ej);
            hl0 = hl1; hl1 = hl2; hl2 = tl(hlrow, t + 3 - lif, 0, ej - 1);
            hh0 = hh1; hh1 = hh2; hh2 = tl(hhrow, t + 3 - lif, 0, ej - 1);
        }
        __syncwarp();
    }

    if constexpr (kSelective) {
        const unsigned tsel = __reduce_or_sync(0xffffffffu, sel);
        dword = (dword & 0xf) | (int)(tsel << 4);
        if (lane == 0) dirty[tid] = dword;
    }
    // nothing changed: the field and its convergence flag stand as they are
    if (!__any_sync(0xffffffffu, chg)) return;
    // unlock this tile and the face neighbours that see a changed face node (lane = row)
    const unsigned f_ilo = __ballot_sync(0xffffffffu, kPrune ? m_ilo : chg && li == 0);
    const unsigned f_ihi = __ballot_sync(0xffffffffu, kPrune ? m_ihi : chg && li == ei - 1);
    const unsigned f_jlo = __ballot_sync(0xffffffffu, chg_jlo);
    const unsigned f_jhi = __ballot_sync(0xffffffffu, chg_jhi);
    // own re-marking (see the 3D sweeps): a polish tile stays locked in this order after
    // updates with remainders below the floor; an FP32 bulk tile none of whose changed nodes
    // feeds an already visited node is a fixed point until a neighbour marks it
    bool again = true;
    if constexpr (kSelective) again = __any_sync(0xffffffffu, restep);
    else if constexpr (kPrune) again = __any_sync(0xffffffffu, stale);
    if (lane == 0) {
        dirty[tid] = dword | (again ? 0xf : (kSelective ? (0xf & ~obit) : 0));
        if (f_ilo && ti > 0) atomicOr(dirty + tid - A.nbj, 0xf);
        if (f_ihi && ti < A.nbi - 1) atomicOr(dirty + tid + A.nbj, 0xf);
        if (f_jlo && tj > 0) atomicOr(dirty + tid - 1, 0xf);
        if (f_jhi && tj < A.nbj - 1) atomicOr(dirty + tid + 1, 0xf);
    }
    for (int y = 0; y < ei; ++y) {
        for (int x = lane; x < ej; x += 32) {
            const long long at = (long long)(i0 + y) * nc + j0 + x;
            const Real v = box[(y + 1) * R2 + x + 1];
            fld[at] = v;
            if constexpr (kSnap)
                if (fabs(__ldcg(snp + at) - v) > A.tol_abs + A.tol_rel * fabs(v)) moved = true;   // isconv
        }
    }
    const bool any_moved = __any_sync(0xffffffffu, moved);
    if constexpr (kSnap) {
        if (lane == 0) A.diff[(long long)q * A.ntiles + tid] = any_moved ? 1 : 0;
    } else {
        if (lane == 0 && any_moved) A.diff[(long long)q * A.ntiles + tid] = 1;
    }
}

template <int KIND>
pfast_status launch_one2(const Sweep2Args& a, int d, int tiles, int nact, cudaStream_t st) {
    static bool attr_set = false;
    const size_t smem = (size_t)kWarps2 * warp_smem2<KIND>();
    if (!attr_set) {
        PFAST_CUDA_TRY(cudaFuncSetAttribute(sweep2d_kernel<KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr_set = true;
    }
    dim3 grid((tiles + kWarps2 - 1) / kWarps2, nact);
    sweep2d_kernel<KIND><<<grid, kWarps2 * 32, smem, st>>>(a, d);
    return PFAST_OK;
}

constexpr int kThreads = 256;

__global__ void init2_kernel_d(double* base, const long long* off, const int* srcnode, long long n) {
    const int q = blockIdx.y;
    double* f = base + off[q];
    const int sn = srcnode[q];
    const long long s = sn >= 0 ? sn : -1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        f[t] = (t == s) ? 0.0 : kInf;
}
__global__ void init2_kernel_f(float* base, const long long* off, const int* srcnode, long long n) {
    const int q = blockIdx.y;
    float* f = base + off[q];
    const int sn = srcnode[q];
    const long long s = sn >= 0 ? sn : -1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        f[t] = (t == s) ? 0.0f : (float)kInf;
}

template <typename T>
__global__ void copy_inst_kernel(const T* a, T* b, const long long* oa, const long long* ob, long long n) {
    const int q = blockIdx.y;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        b[ob[q] + t] = a[oa[q] + t];
}

__global__ void widen_inst_kernel(const float* a, double* b, const long long* oa, const long long* ob, long long n) {
    const int q = blockIdx.y;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        b[ob[q] + t] = (double)a[oa[q] + t];
}

__global__ void narrow_inst_kernel(const double* a, float* b, const long long* oa, const long long* ob, long long n) {
    const int q = blockIdx.y;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        b[ob[q] + t] = (float)a[oa[q] + t];
}

__global__ void widen_lambda_inst_kernel(const float* a, double* b, const long long* oa, const long long* ob,
                                         const unsigned* mask, const long long* mo, int nr, int nc, int wpr) {
    const int q = blockIdx.y;
    const long long n = (long long)nr * nc;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const long long i = t / nc;
        const int j = (int)(t - i * nc);
        if (!((mask[mo[q] + i * wpr + (j >> 5)] >> (j & 31)) & 1u)) b[ob[q] + t] = (double)a[oa[q] + t];
    }
}

// One thread per (source, reflector) instance: the reflection points of one
// reflector, columns in the reference's order, then the INF reset above them.
__global__ void reflect2_kernel(const Reflect2Args A, int ninst) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= ninst) return;
    double* U = A.U + A.inst_off[q];
    const int ir = A.inst_ir[q];
    const int nc = A.nc, nr = A.nr;
    const double dx = A.dx, dz = A.dz;
    const int* k2r = A.k2 + (long long)ir * nc;
    const int* qxc = A.qxcase + (long long)ir * nc;
    const double* Zr = A.Z + (long long)ir * nc * 3;
    for (int step = 0; step < nc; ++step) {
        // interior columns 1..nc-2 first, then column 0, then column nc-1 (src/RT_pfsm2d.h:195,238,259)
        const int jj = step < nc - 2 ? step + 1 : (step == nc - 2 ? 0 : nc - 1);
        const int k2 = k2r[jj];
        if (k2 < 0) continue;   // reflector below the model at this column: no reflection point
        double qx;
        const int cs = qxc[jj];
        if (cs == 0) qx = (U[(long long)k2 * nc + jj + 1] - U[(long long)k2 * nc + jj - 1]) / 2.0 / dx;
        else if (cs == 1) qx = (U[(long long)k2 * nc + jj] - U[(long long)k2 * nc + jj - 1]) / dx;
        else qx = (U[(long long)k2 * nc + jj + 1] - U[(long long)k2 * nc + jj]) / dx;
        const double u0 = U[(long long)k2 * nc + jj];
        const double qz = (U[(long long)(k2 + 1) * nc + jj] - u0) / dz;
        const double dnx = Zr[jj * 3 + 2], dnz = Zr[jj * 3 + 1], zd = Zr[jj * 3 + 0];
        const double rz = qz - 2 * (qx * dnx + qz * dnz) * dnz;
        const double v = u0 + qz * (zd - k2 * dz - dz) + rz * ((k2 + 1) * dz + dz - zd);
        U[(long long)(k2 + 1) * nc + jj] = v;
        if (v < 0) *A.err = 1;
    }
    for (int j = 0; j < nc; ++j) {
        const int kv = A.k2vec[(long long)ir * nc + j];
        for (int i = 0; i <= kv && i < nr; ++i) U[(long long)i * nc + j] = kInf;
    }
}

// One warp per instance: receiver boundary condition and misfit, rows in order.
__global__ void bc2_kernel(const Bc2Args A) {
    const int q = blockIdx.x, lane = threadIdx.x;
    const int s = A.inst_src[q], ir = A.inst_ir[q];
    const double* T = A.T + A.t_off[q];
    double* L = A.L + A.l_off[q];
    unsigned* mask = A.mask + A.mask_off[q];
    const int nc = A.nc, nr = A.nr;
    const int r0 = A.ch0[s], nrec = A.srnum[s];
    const int si = A.src_ij[2 * s], sj = A.src_ij[2 * s + 1];
    const bool trans = ir < 0;
    const double Cr = 1.0;
    double E = A.EE[q];   // running misfit: the reflection adjoint keeps one sum over all reflectors
    bool big = false;
    for (int base = 0; base < nrec; base += 32) {
        const int r = base + lane;
        double e = 0.0;
        if (r < nrec) {
            const int row = r0 + r;
            const double tob = trans ? A.ttobs[row] : A.trobs[(long long)row * A.numofr + ir];
            const bool picked = trans ? (tob < 100) : (tob != 0);
            if (picked) {
                const int i = A.rec[2 * row], j = A.rec[2 * row + 1];
                const long long o = (long long)i * nc + j;
                atomicOr(&mask[(long long)i * A.wpr + (j >> 5)], 1u << (j & 31));
                e = Cr * (tob - T[o]) * (tob - T[o]) / 2.0;
                const bool last = trans ? A.last_t[row] : A.last_r[(long long)row * A.numofr + ir];
                if (last && !(trans && i == si && j == sj)) {
                    const double ny = A.nxy[2 * row], nx = A.nxy[2 * row + 1];
                    const double Tz = (i + 1 >= nr) ? (T[o] - T[o - nc]) / A.dz : (T[o + nc] - T[o]) / A.dz;
                    const double Tx = (j + 1 >= nc) ? (T[o] - T[o - 1]) / A.dx : (T[o + 1] - T[o]) / A.dx;
                    double v = 0.0;
                    if (fabs(tob - T[o]) > 1e-9 && fabs(nx * Tx + ny * Tz) > 1e-6) v = Cr * (tob - T[o]) / (nx * Tx + ny * Tz);
                    L[o] = v;
                    if (fabs(v) > kConvTol) big = true;
                }
            }
        }
        for (int l = 0; l < 32; ++l) {
            const double el = __shfl_sync(0xffffffffu, e, l);
            if (lane == 0) E += el;
        }
    }
    big = __any_sync(0xffffffffu, big);
    if (lane == 0) {
        A.EE[q] = E;
        A.need[q] = big ? 1 : 0;
    }
}

__global__ void accumulate2_kernel(double* gT, double* gR, const double* lam, const long long* lo, const int* gslot,
                                   const double* vp, long long n, int ninst) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const double v = vp[t];
        const double v3 = v * v * v;
        double aT = gT[t], aR = gR[t];
        for (int q = 0; q < ninst; ++q) {
            const double x = lam[lo[q] + t] / v3;
            if (gslot[q] == 0) aT = aT - x;
            else aR = aR - x;
        }
        gT[t] = aT;
        gR[t] = aR;
    }
}

__global__ void blend2_kernel(const double* gT, const double* gR, const double* WR, double* gRT, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        gRT[t] = gT[t] * (1. - WR[t]) + gR[t] * WR[t];   // src/RT_PFAST2D.cpp:434
}

__global__ void addto2_kernel(double* dst, const long long* dof, const double* src, const long long* sof, long long n) {
    const int q = blockIdx.y;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x)
        dst[dof[q] + t] = dst[dof[q] + t] + src[sof[q] + t];
}

__global__ void gather2_kernel(const double* fields, const long long* sfo, int numofr, long long n, const int* rec,
                               const int* ch0, const int* srnum, int b0, int nc, double* Tr) {
    const int b = blockIdx.y;
    const int s = b0 + b;
    for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < srnum[s]; r += gridDim.x * blockDim.x) {
        const int row = ch0[s] + r;
        const long long o = (long long)rec[2 * row] * nc + rec[2 * row + 1];
        const double* base = fields + sfo[b];
        Tr[(long long)row * (numofr + 1)] = base[o];
        for (int ir = 0; ir < numofr; ++ir) Tr[(long long)row * (numofr + 1) + 1 + ir] = base[(1 + numofr + ir) * n + o];
    }
}

inline unsigned grid_for(long long n, int ninst) {
    long long b = (n + kThreads - 1) / kThreads;
    long long cap = std::max(1LL, 152LL * 16 / std::max(1, ninst) + 1);
    return (unsigned)std::max(1LL, std::min(b, cap));
}

}  // namespace

#define PFAST_LAUNCH_CHECK2()                                                                 \
    do {                                                                                      \
        cudaError_t e__ = cudaGetLastError();                                                 \
        if (e__ != cudaSuccess) return cuda_fail(e__, "kernel launch", __FILE__, __LINE__);   \
    } while (0)

pfast_status build_diag_table2(int nr, int nc, DiagTable2& t) {
    t.nbi = (nr + T2I - 1) / T2I;
    t.nbj = (nc + T2J - 1) / T2J;
    if (t.nbi > 65535 || t.nbj > 65535) {
        set_last_error("2D grid %dx%d too large", nr, nc);
        return PFAST_ERR_INVALID;
    }
    t.ndiag = t.nbi + t.nbj - 1;
    std::vector<unsigned> tiles;
    t.h_off.assign(t.ndiag + 1, 0);
    for (int d = 0; d < t.ndiag; ++d) {
        t.h_off[d] = (int)tiles.size();
        for (int bi = 0; bi < t.nbi; ++bi) {
            const int bj = d - bi;
            if (bj >= 0 && bj < t.nbj) tiles.push_back((unsigned)bi | ((unsigned)bj << 16));
        }
    }
    t.h_off[t.ndiag] = (int)tiles.size();
    PFAST_CUDA_TRY(cudaMalloc(&t.d_off, sizeof(int) * t.h_off.size()));
    PFAST_CUDA_TRY(cudaMalloc(&t.d_tiles, sizeof(unsigned) * tiles.size()));
    PFAST_CUDA_TRY(cudaMemcpy(t.d_off, t.h_off.data(), sizeof(int) * t.h_off.size(), cudaMemcpyHostToDevice));
    PFAST_CUDA_TRY(cudaMemcpy(t.d_tiles, tiles.data(), sizeof(unsigned) * tiles.size(), cudaMemcpyHostToDevice));
    return PFAST_OK;
}

void free_diag_table2(DiagTable2& t) {
    if (t.d_off) cudaFree(t.d_off);
    if (t.d_tiles) cudaFree(t.d_tiles);
    t.d_off = nullptr;
    t.d_tiles = nullptr;
}

template <typename Real>
__global__ void near_source2_kernel(Real* __restrict__ base, const long long* __restrict__ off,
                                    const int* __restrict__ inst_src, const int* __restrict__ inst_lim,
                                    const int* __restrict__ rowlim, const double* __restrict__ s64, int nr, int nc,
                                    double dx, double dz, int r) {
    const int q = blockIdx.y;
    if (inst_src[q] < 0) return;
    const int si = inst_src[q] >> 16, sj = inst_src[q] & 0xffff;
    const int* rl = inst_lim[q] >= 0 ? rowlim + (long long)inst_lim[q] * nc : nullptr;
    const double ss = s64[(long long)si * nc + sj];
    const int w = 2 * r + 1;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < w * w; t += gridDim.x * blockDim.x) {
        const int qi = t / w - r, qj = t % w - r;
        const int i = si + qi, j = sj + qj;
        if (i < 0 || i >= nr || j < 0 || j >= nc || qi * qi + qj * qj > r * r) continue;
        if (rl != nullptr && i > rl[j]) continue;   // below the reflector: not part of this solve
        const long long node = (long long)i * nc + j;
        const double ez = qi * dz, ex = qj * dx;
        base[off[q] + node] = Real(0.5 * (ss + s64[node]) * sqrt(ez * ez + ex * ex));
    }
}

pfast_status launch_near_source2(void* base, int is_fp32, const long long* off, const int* inst_src,
                                 const int* inst_lim, const int* rowlim, const double* s64, int nr, int nc, double dx,
                                 double dz, int radius, int ninst, cudaStream_t st) {
    if (radius <= 0 || ninst <= 0) return PFAST_OK;
    const int w = 2 * radius + 1;
    dim3 grid((unsigned)std::max(1, (w * w + 255) / 256), ninst);
    if (is_fp32)
        near_source2_kernel<float><<<grid, 256, 0, st>>>((float*)base, off, inst_src, inst_lim, rowlim, s64, nr, nc, dx,
                                                         dz, radius);
    else
        near_source2_kernel<double><<<grid, 256, 0, st>>>((double*)base, off, inst_src, inst_lim, rowlim, s64, nr, nc,
                                                          dx, dz, radius);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "near_source2 launch", __FILE__, __LINE__);
    return PFAST_OK;
}

pfast_status launch_seed_tiles2(int kind, const Sweep2Args& a, int nact, cudaStream_t st) {
    if (nact <= 0) return PFAST_OK;
    dim3 grid((unsigned)((a.ntiles + 7) / 8), nact);
    switch (kind) {
        case kFwdPlain64: seed_tiles2_kernel<double, false, false><<<grid, 256, 0, st>>>(a); break;
        case kAdjPlain64: seed_tiles2_kernel<double, true, false><<<grid, 256, 0, st>>>(a); break;
        case kFwdFast32: seed_tiles2_kernel<float, false, false><<<grid, 256, 0, st>>>(a); break;
        case kAdjFast32: seed_tiles2_kernel<float, true, false><<<grid, 256, 0, st>>>(a); break;
        case kAdjPolish64: seed_tiles2_kernel<double, true, true><<<grid, 256, 0, st>>>(a); break;
        default: return PFAST_OK;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "seed tiles2 launch", __FILE__, __LINE__);
    return PFAST_OK;
}

pfast_status launch_sweep2(int kind, const Sweep2Args& a, int d, int tiles, int nact, cudaStream_t st) {
    if (tiles <= 0 || nact <= 0) return PFAST_OK;
    switch (kind) {
        case kFwdPlain64: return launch_one2<kFwdPlain64>(a, d, tiles, nact, st);
        case kFwdFast32: return launch_one2<kFwdFast32>(a, d, tiles, nact, st);
        case kFwdPolish64: return launch_one2<kFwdPolish64>(a, d, tiles, nact, st);
        case kAdjPlain64: return launch_one2<kAdjPlain64>(a, d, tiles, nact, st);
        case kAdjFast32: return launch_one2<kAdjFast32>(a, d, tiles, nact, st);
        case kAdjPolish64: return launch_one2<kAdjPolish64>(a, d, tiles, nact, st);
    }
    set_last_error("unknown sweep kind %d", kind);
    return PFAST_ERR_INVALID;
}

pfast_status launch_init2(void* base, int is_fp32, const long long* off, const int* srcnode, long long n, int ninst,
                          cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    dim3 grid(grid_for(n, ninst), ninst);
    if (is_fp32) init2_kernel_f<<<grid, kThreads, 0, st>>>((float*)base, off, srcnode, n);
    else init2_kernel_d<<<grid, kThreads, 0, st>>>((double*)base, off, srcnode, n);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_copy_inst(const void* src, void* dst, int is_fp32, const long long* os, const long long* od,
                              long long n, int ninst, cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    dim3 grid(grid_for(n, ninst), ninst);
    if (is_fp32) copy_inst_kernel<float><<<grid, kThreads, 0, st>>>((const float*)src, (float*)dst, os, od, n);
    else copy_inst_kernel<double><<<grid, kThreads, 0, st>>>((const double*)src, (double*)dst, os, od, n);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_widen_inst(const float* a, double* b, const long long* oa, const long long* ob, long long n,
                               int ninst, cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    dim3 grid(grid_for(n, ninst), ninst);
    widen_inst_kernel<<<grid, kThreads, 0, st>>>(a, b, oa, ob, n);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_narrow_inst(const double* a, float* b, const long long* oa, const long long* ob, long long n,
                                int ninst, cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    dim3 grid(grid_for(n, ninst), ninst);
    narrow_inst_kernel<<<grid, kThreads, 0, st>>>(a, b, oa, ob, n);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_widen_lambda_inst(const float* a, double* b, const long long* oa, const long long* ob,
                                      const unsigned* mask, const long long* mo, int nr, int nc, int wpr, int ninst,
                                      cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    dim3 grid(grid_for((long long)nr * nc, ninst), ninst);
    widen_lambda_inst_kernel<<<grid, kThreads, 0, st>>>(a, b, oa, ob, mask, mo, nr, nc, wpr);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_reflect2(const Reflect2Args& a, int ninst, cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    reflect2_kernel<<<(ninst + 63) / 64, 64, 0, st>>>(a, ninst);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_bc2(const Bc2Args& a, int ninst, cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    bc2_kernel<<<ninst, 32, 0, st>>>(a);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_accumulate2(double* gT, double* gR, const double* lam, const long long* lo, const int* gslot,
                                const double* vp, long long n, int ninst, cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    accumulate2_kernel<<<grid_for(n, 1), kThreads, 0, st>>>(gT, gR, lam, lo, gslot, vp, n, ninst);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_blend2(const double* gT, const double* gR, const double* WR, double* gRT, long long n,
                           cudaStream_t st) {
    blend2_kernel<<<grid_for(n, 1), kThreads, 0, st>>>(gT, gR, WR, gRT, n);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_addto2(double* dst, const long long* dof, const double* src, const long long* sof, long long n,
                           int ninst, cudaStream_t st) {
    if (ninst <= 0) return PFAST_OK;
    dim3 grid(grid_for(n, ninst), ninst);
    addto2_kernel<<<grid, kThreads, 0, st>>>(dst, dof, src, sof, n);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

pfast_status launch_gather2(const double* fields, const long long* sfo, int numofr, long long n, const int* rec,
                            const int* ch0, const int* srnum, int nbatch, int b0, int nc, double* Tr, cudaStream_t st) {
    if (nbatch <= 0) return PFAST_OK;
    dim3 grid(8, nbatch);
    gather2_kernel<<<grid, kThreads, 0, st>>>(fields, sfo, numofr, n, rec, ch0, srnum, b0, nc, Tr);
    PFAST_LAUNCH_CHECK2();
    return PFAST_OK;
}

}  // namespace pfast
