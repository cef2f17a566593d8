// pfast_oracle.cpp -- CPU restatement of PFAST's traveltime + adjoint-state path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library in
// pfast_gb300/: tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg
// (and `bench.py --impl reference`) are the only callers.  The product path never
// links or calls it.
//
// It restates, in plain scalar C++, the algorithms of the PFAST sources
//   src/T_pfsm3d.h      (eikslv3d, isconv, fsm3d)
//   src/T_padjoint3d.h  (adjoint_slv3d, adjoint_fsm3d)
//   src/RT_pfsm2d.h     (eikslv2d, isconv, RT_fsm2d)
//   src/RT_padjoint2d.h (adjoint_slv2d, Tadjoint_fsm2d / Radjoint_fsm2d, Cr=1 overloads)
//   src/T_PFAST3D.cpp / src/RT_PFAST2D.cpp (per-source accumulation, pick gather)
// Every floating-point expression keeps the reference's operation order, so with
// FMA contraction off (-ffp-contract=off) the results are bit-identical to the
// reference's.  Build: oracle/build_oracle.py.
//
// Layouts (as in the reference): 2D field U[i*ncols+j], i = row (depth, dz),
// j = column (x, dx).  3D field U[k*nrows*ncols + i*ncols + j], k = z (dz),
// i = row (y, dy), j = column (x, dx).  3D src / rec / nxyz rows hold 3 entries
// (DIM=3, src/T_pfsm3d.h:16-18); 2D rows hold 2 (DIM=2, src/RT_pfsm2d.h:16-18).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <thread>
#include <atomic>
#include <mutex>
#include <condition_variable>

namespace {

const double kInf = 9999999.0;   // INF macro, src/T_pfsm3d.h:12-14, src/RT_pfsm2d.h
const double kTol = 1e-9;        // isconv tolerance, src/T_pfsm3d.h:126

inline double dmin(double x, double y) { return (x < y) ? x : y; }   // MIN macro
inline double pos_part(double x) { return (x + std::fabs(x)) / 2.0; } // POS, T_padjoint3d.h:8-10
inline double neg_part(double x) { return (x - std::fabs(x)) / 2.0; } // NEG, T_padjoint3d.h:12-14

// any |p-U| > 1e-9  -> not converged.  src/T_pfsm3d.h:122-129, src/RT_pfsm2d.h:110-114
bool converged(const double* p, const double* U, int64_t n) {
    for (int64_t t = 0; t < n; ++t)
        if (std::fabs(p[t] - U[t]) > kTol) return false;
    return true;
}

// ---------------------------------------------------------------- 3D forward
struct Grid3 {
    int nr, nc, nz;   // rows (y), cols (x), depth (z)
    int64_t plane() const { return (int64_t)nr * nc; }
    int64_t at(int k, int i, int j) const { return (int64_t)k * nr * nc + (int64_t)i * nc + j; }
    int64_t size() const { return plane() * nz; }
};

// Godunov upwind update at one node.  Follows src/T_pfsm3d.h:73-120:
// neighbour minima per axis (one-sided at faces), ordering a>=b>=c with the
// matching spacings, then the 1-, 2- and 3-term solutions.
double godunov3d(const double* U, double s, const Grid3& g, int k, int i, int j,
                 double dx, double dy, double dz) {
    double a, b, c;
    if (j == 0) a = U[g.at(k, i, j + 1)];
    else if (j + 1 >= g.nc) a = U[g.at(k, i, j - 1)];
    else a = dmin(U[g.at(k, i, j + 1)], U[g.at(k, i, j - 1)]);
    if (i == 0) b = U[g.at(k, i + 1, j)];
    else if (i + 1 >= g.nr) b = U[g.at(k, i - 1, j)];
    else b = dmin(U[g.at(k, i - 1, j)], U[g.at(k, i + 1, j)]);
    if (k == 0) c = U[g.at(k + 1, i, j)];
    else if (k + 1 >= g.nz) c = U[g.at(k - 1, i, j)];
    else c = dmin(U[g.at(k - 1, i, j)], U[g.at(k + 1, i, j)]);

    double da = dx, db = dy, dc = dz, t;
    if (b > a) { t = a; a = b; b = t; t = da; da = db; db = t; }
    if (c > a) { t = a; a = c; c = t; t = da; da = dc; dc = t; }
    if (c > b) { t = b; b = c; c = t; t = db; db = dc; dc = t; }
    if (!(c <= b && b <= a)) return 0.0;   // only reachable with NaN input (T_pfsm3d.h:104)

    double q = dc * s + c;
    if (q <= b) return q;
    double A = dc * dc + db * db;
    double B = -2. * (b * dc * dc + c * db * db);
    double C = dc * dc * b * b + db * db * c * c - db * db * dc * dc * s * s;
    if ((B * B - 4. * A * C) >= 0) q = (-B + std::sqrt(B * B - 4. * A * C)) / 2. / A;
    else q = kInf;
    if (q <= a) return q;
    A = 1.0 / da / da + 1.0 / db / db + 1.0 / dc / dc;
    B = -2.0 * (a / da / da + b / db / db + c / dc / dc);
    C = a * a / da / da + b * b / db / db + c * c / dc / dc - s * s;
    if ((B * B - 4. * A * C) >= 0) q = (-B + std::sqrt(B * B - 4. * A * C)) / 2. / A;
    else q = kInf;
    return q;
}

// Point-source FSM, src/T_pfsm3d.h:131-185.  Returns the number of outer
// iterations run (each = snapshot + 8 ordered sweeps); MAXSwp of them at most.
int fsm3d_core(const double* vp, double* U, int si, int sj, int sk, int maxswp,
               double dx, double dy, double dz, const Grid3& g) {
    const int64_t n = g.size();
    std::vector<double> p(n, 0.0);
    for (int64_t t = 0; t < n; ++t) U[t] = kInf;
    U[g.at(sk, si, sj)] = 0.0;
    int count = 0, bodies = 0;
    while (!converged(p.data(), U, n) && count++ < maxswp) {
        ++bodies;
        std::memcpy(p.data(), U, sizeof(double) * n);
        for (int s3 = -1; s3 <= 1; s3 += 2)
        for (int s1 = -1; s1 <= 1; s1 += 2)
        for (int s2 = -1; s2 <= 1; s2 += 2)
        for (int k = (s3 < 0 ? g.nz - 1 : 0); s3 < 0 ? k >= 0 : k < g.nz; k += s3)
        for (int i = (s1 < 0 ? g.nr - 1 : 0); s1 < 0 ? i >= 0 : i < g.nr; i += s1)
        for (int j = (s2 < 0 ? g.nc - 1 : 0); s2 < 0 ? j >= 0 : j < g.nc; j += s2) {
            if (i == si && j == sj && k == sk) continue;
            const int64_t at = g.at(k, i, j);
            double s = 1.0 / vp[at];
            double q = godunov3d(U, s, g, k, i, j, dx, dy, dz);
            U[at] = dmin(U[at], q);
        }
    }
    return bodies;
}

// Adjoint local update, src/T_padjoint3d.h:42-71 (interior nodes only).
double adjoint_node3d(const double* L, const double* T, const Grid3& g, int k, int i, int j,
                      double dx, double dy, double dz) {
    const int64_t o = g.at(k, i, j);
    const int64_t xm = o - 1, xp = o + 1, ym = o - g.nc, yp = o + g.nc, zm = o - g.plane(), zp = o + g.plane();
    if (T[o] >= kInf || T[xp] >= kInf || T[xm] >= kInf || T[yp] >= kInf || T[ym] >= kInf ||
        T[zp] >= kInf || T[zm] >= kInf)
        return 0.0;
    double a1 = pos_part(-(T[xp] - T[o]) / dx);
    double a2 = neg_part(-(T[o] - T[xm]) / dx);
    double b1 = pos_part(-(T[yp] - T[o]) / dy);
    double b2 = neg_part(-(T[o] - T[ym]) / dy);
    double c1 = pos_part(-(T[zp] - T[o]) / dz);
    double c2 = neg_part(-(T[o] - T[zm]) / dz);
    double La1 = pos_part(-(T[o] - T[xm]) / dx) * L[xm];
    double La2 = neg_part(-(T[xp] - T[o]) / dx) * L[xp];
    double Lb1 = pos_part(-(T[o] - T[ym]) / dy) * L[ym];
    double Lb2 = neg_part(-(T[yp] - T[o]) / dy) * L[yp];
    double Lc1 = pos_part(-(T[o] - T[zm]) / dz) * L[zm];
    double Lc2 = neg_part(-(T[zp] - T[o]) / dz) * L[zp];
    double den = (a1 - a2) / dx + (b1 - b2) / dy + (c1 - c2) / dz;
    if (std::fabs(den) > 1e-9)
        return ((La1 - La2) / dx + (Lb1 - Lb2) / dy + (Lc1 - Lc2) / dz) / den;
    return 0.0;
}

// Receiver boundary condition, misfit and interior sweeps, src/T_padjoint3d.h:73-172.
double adjoint3d_core(double* L, const double* T, const double* Tobs, const int* rec,
                      const double* nxyz, int si, int sj, int sk, int ch0, int nrec,
                      int maxswp, double dx, double dy, double dz, const Grid3& g, int* iters) {
    const int64_t n = g.size();
    std::vector<double> p(n, 0.0);
    std::vector<unsigned char> fixed(n, 0);
    for (int64_t t = 0; t < n; ++t) L[t] = 0.0;
    double E = 0.0;
    for (int r = 0; r < nrec; ++r) {
        const int row = ch0 + r;
        const double tob = Tobs[row];
        if (!(tob < 100)) continue;                       // only picked first arrivals
        const int i = rec[row * 3 + 0], j = rec[row * 3 + 1], k = rec[row * 3 + 2];
        const int64_t o = g.at(k, i, j);
        fixed[o] = 1;
        E += (tob - T[o]) * (tob - T[o]) / 2.0;
        if (i == si && j == sj && k == sk) continue;      // receiver at the source: no BC
        const double ny = nxyz[row * 3 + 0], nx = nxyz[row * 3 + 1], nz = nxyz[row * 3 + 2];
        double Tz = (k + 1 >= g.nz) ? (T[o] - T[o - g.plane()]) / dz : (T[o + g.plane()] - T[o]) / dz;
        double Ty = (i + 1 >= g.nr) ? (T[o] - T[o - g.nc]) / dy : (T[o + g.nc] - T[o]) / dy;
        double Tx = (j + 1 >= g.nc) ? (T[o] - T[o - 1]) / dx : (T[o + 1] - T[o]) / dx;
        if (std::fabs(tob - T[o]) > 1e-9 && std::fabs(nx * Tx + ny * Ty + nz * Tz) > 1e-6)
            L[o] = (tob - T[o]) / (nx * Tx + ny * Ty + nz * Tz);
        else
            L[o] = 0.0;
    }
    int count = 0, bodies = 0;
    while (count++ < maxswp && !converged(p.data(), L, n)) {
        ++bodies;
        std::memcpy(p.data(), L, sizeof(double) * n);
        for (int s3 = -1; s3 <= 1; s3 += 2)
        for (int s1 = -1; s1 <= 1; s1 += 2)
        for (int s2 = -1; s2 <= 1; s2 += 2)
        for (int k = (s3 < 0 ? g.nz - 2 : 1); s3 < 0 ? k >= 1 : k < g.nz - 1; k += s3)
        for (int i = (s1 < 0 ? g.nr - 2 : 1); s1 < 0 ? i >= 1 : i < g.nr - 1; i += s1)
        for (int j = (s2 < 0 ? g.nc - 2 : 1); s2 < 0 ? j >= 1 : j < g.nc - 1; j += s2) {
            const int64_t o = g.at(k, i, j);
            if (fixed[o]) continue;
            L[o] = adjoint_node3d(L, T, g, k, i, j, dx, dy, dz);
        }
    }
    if (iters) *iters = bodies;
    return E;
}

// ---------------------------------------------------------------- 2D forward
struct Grid2 {
    int nr, nc;
    int64_t at(int i, int j) const { return (int64_t)i * nc + j; }
    int64_t size() const { return (int64_t)nr * nc; }
};

// Godunov 2D update, src/RT_pfsm2d.h:71-108.
double godunov2d(const double* U, double s, const Grid2& g, int i, int j, double dx, double dz) {
    double a, b;
    if (i == 0) b = U[g.at(i + 1, j)];
    else if (i + 1 >= g.nr) b = U[g.at(i - 1, j)];
    else b = dmin(U[g.at(i - 1, j)], U[g.at(i + 1, j)]);
    if (j == 0) a = U[g.at(i, j + 1)];
    else if (j + 1 >= g.nc) a = U[g.at(i, j - 1)];
    else a = dmin(U[g.at(i, j + 1)], U[g.at(i, j - 1)]);
    double da = dx, db = dz, t;
    if (b > a) { t = a; a = b; b = t; t = da; da = db; db = t; }
    double q = b + db * s;
    if (q <= a) return q;
    double A = 1.0 / da / da + 1.0 / db / db;
    double B = -2. * (a / da / da + b / db / db);
    double C = a * a / da / da + b * b / db / db - s * s;
    if ((B * B - 4. * A * C) >= 0) q = (-B + std::sqrt(B * B - 4 * A * C)) / 2. / A;
    else q = kInf;
    return q;
}

// Which nodes a 2D FSM solve may update.
enum Mask2 { kAllButSource = 0, kAboveReflector = 1, kAboveReflPoint = 2 };

// One 2D FSM solve to convergence over the masked node set (the three sweep
// loops of src/RT_pfsm2d.h:163-182, 300-317 and 346-365).  U holds the start field.
int fsm2d_solve(const double* vp, double* U, const Grid2& g, int si, int sj, Mask2 mask,
                const double* Zr /* reflector rows (ncols x 3) */, const int* k2vec,
                int maxswp, double dx, double dz) {
    const int64_t n = g.size();
    std::vector<double> p(n, 0.0);
    int count = 0, bodies = 0;
    while (!converged(p.data(), U, n) && count++ < maxswp) {
        ++bodies;
        std::memcpy(p.data(), U, sizeof(double) * n);
        for (int s1 = -1; s1 <= 1; s1 += 2)
        for (int s2 = -1; s2 <= 1; s2 += 2)
        for (int i = (s1 < 0 ? g.nr - 1 : 0); s1 < 0 ? i >= 0 : i < g.nr; i += s1)
        for (int j = (s2 < 0 ? g.nc - 1 : 0); s2 < 0 ? j >= 0 : j < g.nc; j += s2) {
            bool upd;
            if (mask == kAllButSource) upd = !(i == si && j == sj);
            else if (mask == kAboveReflector) upd = !(i == si && j == sj) && (i + 1) * dz <= Zr[j * 3 + 0];
            else upd = i <= k2vec[j];
            if (!upd) continue;
            const int64_t o = g.at(i, j);
            double q = godunov2d(U, 1.0 / vp[o], g, i, j, dx, dz);
            U[o] = dmin(U[o], q);
        }
    }
    return bodies;
}

// Mirror the down-going gradient about the reflector at one column and write the
// reflected time into the first row below the reflection point.  The three cases
// (interior column, left edge, right edge) follow src/RT_pfsm2d.h:195-281.
// Returns 0, or a negative status: -1 = no node above the reflector, -2 = negative time.
int reflect_column(double* U, const Grid2& g, const double* Zr, int jj, int* k2vec, double dx, double dz) {
    const int nc = g.nc, nr = g.nr;
    const double zj = Zr[jj * 3 + 0];
    const bool left = jj == 0, right = jj == nc - 1;
    int k2 = -1;
    for (int kk = 0; kk < nr - 1; ++kk) {
        bool here = (kk + 1) * dz + dz <= zj;
        bool side;
        if (left) side = kk * dz + dz <= Zr[(jj + 1) * 3];
        else if (right) side = kk * dz + dz <= Zr[(jj - 1) * 3];
        else side = kk * dz + dz <= Zr[(jj - 1) * 3] || kk * dz + dz <= Zr[(jj + 1) * 3];
        if (here && side && kk >= k2) k2 = kk;
    }
    if (zj <= nr * dz && k2 > 0) {
        double qx;
        if (left) qx = (U[g.at(k2, jj + 1)] - U[g.at(k2, jj)]) / dx;
        else if (right) qx = (U[g.at(k2, jj)] - U[g.at(k2, jj - 1)]) / dx;
        else if (k2 * dz + dz <= Zr[(jj - 1) * 3] && k2 * dz + dz <= Zr[(jj + 1) * 3])
            qx = (U[g.at(k2, jj + 1)] - U[g.at(k2, jj - 1)]) / 2.0 / dx;
        else if (k2 * dz + dz <= Zr[(jj - 1) * 3])
            qx = (U[g.at(k2, jj)] - U[g.at(k2, jj - 1)]) / dx;
        else
            qx = (U[g.at(k2, jj + 1)] - U[g.at(k2, jj)]) / dx;
        const double qz = (U[g.at(k2 + 1, jj)] - U[g.at(k2, jj)]) / dz;
        const double nxr = Zr[jj * 3 + 2], nzr = Zr[jj * 3 + 1];
        const double rz = qz - 2 * (qx * nxr + qz * nzr) * nzr;
        U[g.at(k2 + 1, jj)] = U[g.at(k2, jj)] + qz * (zj - k2 * dz - dz) + rz * ((k2 + 1) * dz + dz - zj);
        k2vec[jj] = k2;
        if (U[g.at(k2 + 1, jj)] < 0) return -2;
        return 0;
    }
    if (zj > nr * dz) { k2vec[jj] = nr - 1; return 0; }
    return -1;
}

} // namespace

extern "C" {

// ------------------------------------------------------------------ 3D API
// fsm3d (src/T_pfsm3d.h:131): vp[N] -> U[N].  src rows are (row, col, z).
int oracle_fsm3d(const double* vp, double* U, const int* src, int srcid, int maxswp,
                 double dx, double dy, double dz, int nrows, int ncols, int nz) {
    Grid3 g{nrows, ncols, nz};
    return fsm3d_core(vp, U, src[srcid * 3 + 0], src[srcid * 3 + 1], src[srcid * 3 + 2],
                      maxswp, dx, dy, dz, g);
}

// adjoint_fsm3d (src/T_padjoint3d.h:73): returns the misfit EE of this source.
double oracle_adjoint3d(double* L, const double* T, const double* Tobs, const int* rec,
                        const double* nxyz, const int* src, const int* srnum, int srcid, int maxswp,
                        double dx, double dy, double dz, int nrows, int ncols, int nz, int* iters) {
    Grid3 g{nrows, ncols, nz};
    int ch0 = 0;
    for (int s = 0; s < srcid; ++s) ch0 += srnum[s];
    return adjoint3d_core(L, T, Tobs, rec, nxyz, src[srcid * 3 + 0], src[srcid * 3 + 1],
                          src[srcid * 3 + 2], ch0, srnum[srcid], maxswp, dx, dy, dz, g, iters);
}

// One misfit + gradient evaluation over sources [s_begin, s_end) (the per-source
// loop of src/T_PFAST3D.cpp:387-399 with np=1): grad[n] starts at 0 and receives
// grad -= lambda_s / (v*v*v) in increasing source order; *misfit = sum of EE in
// source order.  nthreads workers solve sources concurrently; the accumulation
// still runs in source order, so the result does not depend on nthreads.
int oracle_eval3d(const double* vp, const int* src, const int* srnum, const int* rec,
                  const double* nxyz, const double* Tobs, int s_begin, int s_end, int maxswp,
                  double dx, double dy, double dz, int nrows, int ncols, int nz,
                  double* grad, double* misfit, int nthreads, int* fwd_iters, int* adj_iters) {
    Grid3 g{nrows, ncols, nz};
    const int64_t n = g.size();
    std::vector<int> ch0(s_end + 1, 0);
    for (int s = 0; s < s_end; ++s) ch0[s + 1] = ch0[s] + srnum[s];
    for (int64_t t = 0; t < n; ++t) grad[t] = 0.0;
    double E = 0.0;
    std::atomic<int> next{s_begin};
    int turn = s_begin;
    std::mutex mu;
    std::condition_variable cv;
    if (nthreads < 1) nthreads = 1;
    auto worker = [&]() {
        std::vector<double> T(n), L(n);
        for (;;) {
            int s = next.fetch_add(1);
            if (s >= s_end) return;
            int fi = fsm3d_core(vp, T.data(), src[s * 3], src[s * 3 + 1], src[s * 3 + 2], maxswp, dx, dy, dz, g);
            int ai = 0;
            double EE = adjoint3d_core(L.data(), T.data(), Tobs, rec, nxyz, src[s * 3], src[s * 3 + 1],
                                       src[s * 3 + 2], ch0[s], srnum[s], maxswp, dx, dy, dz, g, &ai);
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return turn == s; });
            for (int64_t t = 0; t < n; ++t) grad[t] = grad[t] - L[t] / (vp[t] * vp[t] * vp[t]);
            E += EE;
            if (fwd_iters) fwd_iters[s - s_begin] = fi;
            if (adj_iters) adj_iters[s - s_begin] = ai;
            ++turn;
            cv.notify_all();
        }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; ++w) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    *misfit = E;
    return 0;
}

// Forward picks, src/T_PFAST3D.cpp:672-686: picks[row] = T_s at rec[row] for the
// receiver rows of sources [s_begin, s_end) (rows numbered from ch0(s_begin)).
int oracle_forward3d(const double* vp, const int* src, const int* srnum, const int* rec,
                     int s_begin, int s_end, int maxswp, double dx, double dy, double dz,
                     int nrows, int ncols, int nz, double* picks, int nthreads) {
    Grid3 g{nrows, ncols, nz};
    const int64_t n = g.size();
    std::vector<int> ch0(s_end + 1, 0);
    for (int s = 0; s < s_end; ++s) ch0[s + 1] = ch0[s] + srnum[s];
    std::atomic<int> next{s_begin};
    if (nthreads < 1) nthreads = 1;
    auto worker = [&]() {
        std::vector<double> T(n);
        for (;;) {
            int s = next.fetch_add(1);
            if (s >= s_end) return;
            fsm3d_core(vp, T.data(), src[s * 3], src[s * 3 + 1], src[s * 3 + 2], maxswp, dx, dy, dz, g);
            for (int r = 0; r < srnum[s]; ++r) {
                const int row = ch0[s] + r;
                picks[row - ch0[s_begin]] = T[g.at(rec[row * 3 + 2], rec[row * 3 + 0], rec[row * 3 + 1])];
            }
        }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; ++w) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    return 0;
}

// ------------------------------------------------------------------ 2D API
// RT_fsm2d (src/RT_pfsm2d.h:116-380).  Z is the reflector table
// [NumofR*ncols][3] = (depth, n_z, n_x).  TTd/TTu are [NumofR][nrows*ncols].
// iters (optional) receives 2*NumofR+1 iteration counts: down_0, up_0, down_1, ...,
// transmission.  Returns 0, -1 (no node above a reflector) or -2 (negative
// reflected time), the two conditions on which the reference exits.
int oracle_rt_fsm2d(const double* vp, double* U, double* TTd, double* TTu, const double* Z,
                    const int* src, int srcid, int numofr, int maxswp, double dx, double dz,
                    int nrows, int ncols, int* iters) {
    Grid2 g{nrows, ncols};
    const int64_t n = g.size();
    const int si = src[srcid * 2 + 0], sj = src[srcid * 2 + 1];
    std::vector<int> k2vec(ncols, -1);
    for (int ir = 0; ir < numofr; ++ir) {
        const double* Zr = Z + (int64_t)ir * ncols * 3;
        for (int64_t t = 0; t < n; ++t) U[t] = kInf;
        U[g.at(si, sj)] = 0.0;
        int c = fsm2d_solve(vp, U, g, si, sj, kAboveReflector, Zr, nullptr, maxswp, dx, dz);
        if (iters) iters[2 * ir] = c;
        std::memcpy(TTd + ir * n, U, sizeof(double) * n);
        // reflection points: interior columns left to right, then the two edges
        for (int jj = 1; jj < ncols - 1; ++jj) {
            int st = reflect_column(U, g, Zr, jj, k2vec.data(), dx, dz);
            if (st) return st;
        }
        int st = reflect_column(U, g, Zr, 0, k2vec.data(), dx, dz);
        if (st) return st;
        st = reflect_column(U, g, Zr, ncols - 1, k2vec.data(), dx, dz);
        if (st) return st;
        for (int i = 0; i < nrows; ++i)
            for (int j = 0; j < ncols; ++j)
                if (i <= k2vec[j]) U[g.at(i, j)] = kInf;
        c = fsm2d_solve(vp, U, g, si, sj, kAboveReflPoint, Zr, k2vec.data(), maxswp, dx, dz);
        if (iters) iters[2 * ir + 1] = c;
        std::memcpy(TTu + ir * n, U, sizeof(double) * n);
    }
    for (int64_t t = 0; t < n; ++t) U[t] = kInf;
    U[g.at(si, sj)] = 0.0;
    int c = fsm2d_solve(vp, U, g, si, sj, kAllButSource, nullptr, nullptr, maxswp, dx, dz);
    if (iters) iters[2 * numofr] = c;
    return 0;
}

}  // extern "C"

namespace {

// Adjoint local update 2D, src/RT_padjoint2d.h:42-65 (interior nodes only).
double adjoint_node2d(const double* L, const double* T, const Grid2& g, int i, int j, double dx, double dz) {
    const int64_t o = g.at(i, j), xm = o - 1, xp = o + 1, zm = o - g.nc, zp = o + g.nc;
    if (T[xp] >= kInf || T[o] >= kInf || T[xm] >= kInf || T[zp] >= kInf || T[zm] >= kInf) return 0.0;
    double a1 = pos_part(-(T[xp] - T[o]) / dx);
    double a2 = neg_part(-(T[o] - T[xm]) / dx);
    double b1 = pos_part(-(T[zp] - T[o]) / dz);
    double b2 = neg_part(-(T[o] - T[zm]) / dz);
    double La1 = pos_part(-(T[o] - T[xm]) / dx) * L[xm];
    double La2 = neg_part(-(T[xp] - T[o]) / dx) * L[xp];
    double Lb1 = pos_part(-(T[o] - T[zm]) / dz) * L[zm];
    double Lb2 = neg_part(-(T[zp] - T[o]) / dz) * L[zp];
    if (std::fabs((a1 - a2) / dx + (b1 - b2) / dz) > 1e-9)
        return ((La1 - La2) / dx + (Lb1 - Lb2) / dz) / ((a1 - a2) / dx + (b1 - b2) / dz);
    return 0.0;
}

// Interior sweeps of the 2D adjoint (src/RT_padjoint2d.h:347-371 / 439-463).
// `count` is shared with the caller because Radjoint_fsm2d carries it across
// reflectors (src/RT_padjoint2d.h:385,439).
void adjoint2d_sweeps(double* L, const double* T, const unsigned char* fixed, const Grid2& g,
                      int maxswp, double dx, double dz, int& count, int* iters) {
    const int64_t n = g.size();
    std::vector<double> p(n, 0.0);
    int bodies = 0;
    while (count++ < maxswp && !converged(p.data(), L, n)) {
        ++bodies;
        std::memcpy(p.data(), L, sizeof(double) * n);
        for (int s1 = -1; s1 <= 1; s1 += 2)
        for (int s2 = -1; s2 <= 1; s2 += 2)
        for (int i = (s1 < 0 ? g.nr - 2 : 1); s1 < 0 ? i >= 1 : i < g.nr - 1; i += s1)
        for (int j = (s2 < 0 ? g.nc - 2 : 1); s2 < 0 ? j >= 1 : j < g.nc - 1; j += s2) {
            const int64_t o = g.at(i, j);
            if (fixed[o]) continue;
            L[o] = adjoint_node2d(L, T, g, i, j, dx, dz);
        }
    }
    if (iters) *iters = bodies;
}

// Receiver BC for one 2D field (the bodies of src/RT_padjoint2d.h:311-339 and 405-433).
// trans=true: transmission (pick if obs<100, no BC at the source node);
// trans=false: reflection (pick if obs!=0, BC everywhere).  The misfit terms are
// added to E in row order; the reflection adjoint keeps one running sum over all
// its reflectors (src/RT_padjoint2d.h:409).
void receiver_bc2d(double* L, const double* T, const double* obs, int obs_stride, int obs_off,
                   const int* rec, const double* nxy, int si, int sj, int ch0, int nrec,
                   const Grid2& g, double dx, double dz, unsigned char* fixed, bool trans, double& E) {
    const double Cr = 1.0;
    for (int r = 0; r < nrec; ++r) {
        const int row = ch0 + r;
        const double tob = obs[(int64_t)row * obs_stride + obs_off];
        if (trans ? !(tob < 100) : !(tob != 0)) continue;
        const int i = rec[row * 2 + 0], j = rec[row * 2 + 1];
        const int64_t o = g.at(i, j);
        fixed[o] = 1;
        E += Cr * (tob - T[o]) * (tob - T[o]) / 2.0;
        if (trans && i == si && j == sj) continue;
        const double ny = nxy[row * 2 + 0], nx = nxy[row * 2 + 1];
        double Tz = (i + 1 >= g.nr) ? (T[o] - T[o - g.nc]) / dz : (T[o + g.nc] - T[o]) / dz;
        double Tx = (j + 1 >= g.nc) ? (T[o] - T[o - 1]) / dx : (T[o + 1] - T[o]) / dx;
        if (std::fabs(tob - T[o]) > 1e-9 && std::fabs(nx * Tx + ny * Tz) > 1e-6)
            L[o] = Cr * (tob - T[o]) / (nx * Tx + ny * Tz);
        else
            L[o] = 0.0;
    }
}

} // namespace

extern "C" {

// Tadjoint_fsm2d, Cr=1 overload (src/RT_padjoint2d.h:288-380).
double oracle_tadjoint2d(double* L, const double* T, const double* Tobs, const int* rec,
                         const double* nxy, const int* src, const int* srnum, int srcid, int maxswp,
                         double dx, double dz, int nrows, int ncols, int* iters) {
    Grid2 g{nrows, ncols};
    const int64_t n = g.size();
    int ch0 = 0;
    for (int s = 0; s < srcid; ++s) ch0 += srnum[s];
    std::vector<unsigned char> fixed(n, 0);
    for (int64_t t = 0; t < n; ++t) L[t] = 0.0;
    double E = 0.0;
    receiver_bc2d(L, T, Tobs, 1, 0, rec, nxy, src[srcid * 2], src[srcid * 2 + 1], ch0, srnum[srcid], g, dx, dz,
                  fixed.data(), true, E);
    int count = 0;
    adjoint2d_sweeps(L, T, fixed.data(), g, maxswp, dx, dz, count, iters);
    return E;
}

// Radjoint_fsm2d, Cr=1 overload (src/RT_padjoint2d.h:382-473).  TRobs is
// [Nrec][NumofR]; Tu is [NumofR][N]; UR receives the sum over reflectors.  The
// receiver mask and the iteration counter carry over from one reflector to the
// next, as in the reference.
double oracle_radjoint2d(double* UR, const double* Tu, const double* TRobs, const int* rec,
                         const double* nxy, const int* src, const int* srnum, int srcid, int numofr,
                         int maxswp, double dx, double dz, int nrows, int ncols, int* iters) {
    Grid2 g{nrows, ncols};
    const int64_t n = g.size();
    int ch0 = 0;
    for (int s = 0; s < srcid; ++s) ch0 += srnum[s];
    std::vector<unsigned char> fixed(n, 0);
    std::vector<double> L(n);
    for (int64_t t = 0; t < n; ++t) UR[t] = 0;
    double E = 0.0;
    int count = 0;
    for (int ir = 0; ir < numofr; ++ir) {
        for (int64_t t = 0; t < n; ++t) L[t] = 0.0;
        const double* T = Tu + (int64_t)ir * n;
        receiver_bc2d(L.data(), T, TRobs, numofr, ir, rec, nxy, src[srcid * 2], src[srcid * 2 + 1], ch0,
                      srnum[srcid], g, dx, dz, fixed.data(), false, E);
        adjoint2d_sweeps(L.data(), T, fixed.data(), g, maxswp, dx, dz, count, iters ? iters + ir : nullptr);
        for (int64_t t = 0; t < n; ++t) UR[t] = UR[t] + L[t];
    }
    return E;
}

// 2D forward picks for sources [s_begin, s_end) (src/RT_PFAST2D.cpp:832-852):
// Tr[(row)*(NumofR+1)+0] = TT at the receiver, Tr[row*(NumofR+1)+1+ir] = TTu_ir.
// Rows are numbered from ch0(s_begin).  Returns the first nonzero RT_fsm2d status.
int oracle_forward2d(const double* vp, const double* Z, const int* src, const int* srnum, const int* rec,
                     int s_begin, int s_end, int numofr, int maxswp, double dx, double dz,
                     int nrows, int ncols, double* Tr, int nthreads) {
    Grid2 g{nrows, ncols};
    const int64_t n = g.size();
    std::vector<int> ch0(s_end + 1, 0);
    for (int s = 0; s < s_end; ++s) ch0[s + 1] = ch0[s] + srnum[s];
    std::atomic<int> next{s_begin};
    std::atomic<int> status{0};
    if (nthreads < 1) nthreads = 1;
    auto worker = [&]() {
        std::vector<double> U(n), TTd((size_t)n * (numofr > 0 ? numofr : 1)), TTu((size_t)n * (numofr > 0 ? numofr : 1));
        for (;;) {
            int s = next.fetch_add(1);
            if (s >= s_end) return;
            int st = oracle_rt_fsm2d(vp, U.data(), TTd.data(), TTu.data(), Z, src, s, numofr, maxswp, dx, dz,
                                     nrows, ncols, nullptr);
            if (st) { int z = 0; status.compare_exchange_strong(z, st); }
            for (int r = 0; r < srnum[s]; ++r) {
                const int row = ch0[s] + r, orow = row - ch0[s_begin];
                const int64_t o = g.at(rec[row * 2 + 0], rec[row * 2 + 1]);
                Tr[(int64_t)orow * (numofr + 1) + 0] = U[o];
                for (int ir = 0; ir < numofr; ++ir)
                    Tr[(int64_t)orow * (numofr + 1) + ir + 1] = TTu[ir * n + o];
            }
        }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; ++w) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    return status.load();
}

// 2D joint gradient for sources [s_begin, s_end) (src/RT_PFAST2D.cpp:420-436, np=1):
// gT -= lamT/v^3, gR -= lamR/v^3 in source order, gRT = gT*(1-WR) + gR*WR,
// Et / Er = misfit sums in source order.  Returns the first RT_fsm2d status.
int oracle_eval2d(const double* vp, const double* WR, const double* Z, const int* src, const int* srnum,
                  const int* rec, const double* nxy, const double* TTobs, const double* TRobs,
                  int s_begin, int s_end, int numofr, int maxswp, double dx, double dz, int nrows, int ncols,
                  double* gT, double* gR, double* gRT, double* Et, double* Er, int nthreads) {
    Grid2 g{nrows, ncols};
    const int64_t n = g.size();
    std::vector<int> ch0(s_end + 1, 0);
    for (int s = 0; s < s_end; ++s) ch0[s + 1] = ch0[s] + srnum[s];
    for (int64_t t = 0; t < n; ++t) { gT[t] = 0.0; gR[t] = 0.0; gRT[t] = 0.0; }
    double et = 0.0, er = 0.0;
    std::atomic<int> next{s_begin};
    std::atomic<int> status{0};
    int turn = s_begin;
    std::mutex mu;
    std::condition_variable cv;
    if (nthreads < 1) nthreads = 1;
    auto worker = [&]() {
        const size_t nr = numofr > 0 ? numofr : 1;
        std::vector<double> U(n), TTd(n * nr), TTu(n * nr), LT(n), LR(n);
        for (;;) {
            int s = next.fetch_add(1);
            if (s >= s_end) return;
            int st = oracle_rt_fsm2d(vp, U.data(), TTd.data(), TTu.data(), Z, src, s, numofr, maxswp, dx, dz,
                                     nrows, ncols, nullptr);
            if (st) { int z = 0; status.compare_exchange_strong(z, st); }
            double e1 = oracle_tadjoint2d(LT.data(), U.data(), TTobs, rec, nxy, src, srnum, s, maxswp, dx, dz,
                                          nrows, ncols, nullptr);
            double e2 = oracle_radjoint2d(LR.data(), TTu.data(), TRobs, rec, nxy, src, srnum, s, numofr, maxswp,
                                          dx, dz, nrows, ncols, nullptr);
            std::unique_lock<std::mutex> lk(mu);
            cv.wait(lk, [&] { return turn == s; });
            for (int64_t t = 0; t < n; ++t) gT[t] = gT[t] - LT[t] / (vp[t] * vp[t] * vp[t]);
            for (int64_t t = 0; t < n; ++t) gR[t] = gR[t] - LR[t] / (vp[t] * vp[t] * vp[t]);
            et += e1;
            er += e2;
            ++turn;
            cv.notify_all();
        }
    };
    std::vector<std::thread> pool;
    for (int w = 0; w < nthreads; ++w) pool.emplace_back(worker);
    for (auto& th : pool) th.join();
    for (int64_t t = 0; t < n; ++t) gRT[t] = gT[t] * (1. - WR[t]) + gR[t] * WR[t];
    *Et = et;
    *Er = er;
    return status.load();
}

}  // extern "C"
