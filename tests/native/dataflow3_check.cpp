// Checks the tile dataflow graph of the 3D sweeps (pfast_gb300/csrc/dataflow3.h) on the CPU,
// with the counter protocol of the dataflow sweep kernel: per tile two 4-bit counters, one per
// sweep-order parity; the items of order 0 start at dep_count(0, x), those of order 1 at
// dep_count(1, x); completing (o, x) first re-arms x's counter of parity o for order o + 2,
// then decrements the counters of its dependents, and an item whose counter reaches zero is
// ready.  Random schedules with up to W items in flight must:
//   - run every item of the outer iteration exactly once,
//   - start an item only after all of its dependencies (stated directly) completed,
//   - never run two face-neighbouring tiles at the same time,
//   - never decrement a counter below zero.
// Also checks that the dependents lists are exactly the inverse of the dependencies.
// Prints "ok <grid>" per grid, or "FAIL ..." and exits 1.
#include <cstdio>
#include <cstdlib>
#include <random>
#include <set>
#include <vector>

#include "dataflow3.h"

using pfast::TileGrid3;

static bool direct_dep(const TileGrid3& g, int o2, int y, int o, int x) {
    // is (o, x) a dependency of (o2, y)?
    if (x == y) return o2 > 0 && o == o2 - 1;
    for (int a = 0; a < 3; ++a)
        for (int s = 0; s < 2; ++s)
            if (pfast::tile_neighbour(g, y, a, s) == x) {
                if (pfast::side_upstream(o2, a, s)) return o == o2;
                return o2 > 0 && o == o2 - 1;
            }
    return false;
}

static int fail(const char* what, const TileGrid3& g, int o, int x) {
    std::printf("FAIL %s grid %dx%dx%d item (%d,%d)\n", what, g.nbk, g.nbi, g.nbj, o, x);
    return 1;
}

static int check_grid(const TileGrid3& g, unsigned seed, int width) {
    const int n = pfast::tile_count(g);
    // 1. dependents == inverse of dependencies
    std::vector<int> indeg(8 * n, 0);
    for (int o = 0; o < 8; ++o)
        for (int x = 0; x < n; ++x) {
            int t[16], od[16];
            const int m = pfast::dependents(g, o, x, t, od);
            if (m > 13) return fail("more than 13 dependents", g, o, x);
            for (int k = 0; k < m; ++k) {
                if (!direct_dep(g, od[k], t[k], o, x)) return fail("dependent without dependency", g, o, x);
                for (int k2 = 0; k2 < k; ++k2)
                    if (t[k2] == t[k] && od[k2] == od[k]) return fail("duplicate dependent", g, o, x);
                ++indeg[od[k] * n + t[k]];
            }
        }
    for (int o = 0; o < 8; ++o)
        for (int x = 0; x < n; ++x)
            if (indeg[o * n + x] != pfast::dep_count(g, o, x)) return fail("dep_count != in-degree", g, o, x);
    // 2. random schedules with the kernel's counter protocol
    std::mt19937 rng(seed);
    for (int rep = 0; rep < 20; ++rep) {
        std::vector<int> cnt(2 * n);
        for (int x = 0; x < n; ++x) {
            cnt[2 * x] = pfast::dep_count(g, 0, x);
            cnt[2 * x + 1] = pfast::dep_count(g, 1, x);
        }
        std::vector<int> ready, done(8 * n, 0);
        for (int x = 0; x < n; ++x)
            if (cnt[2 * x] == 0) ready.push_back(x);
        if (ready.size() != 1 || ready[0] != pfast::first_tile(g)) return fail("first tile", g, 0, ready.empty() ? -1 : ready[0]);
        ready[0] = pfast::first_tile(g);   // entries: x | o << 20
        std::vector<int> running;
        std::vector<int> busy(n, 0);
        int completed = 0;
        while (completed < 8 * n) {
            const bool can_start = !ready.empty() && (int)running.size() < width;
            const bool start = can_start && (running.empty() || rng() % 2);
            if (start) {
                const int k = rng() % ready.size();
                const int e = ready[k];
                ready[k] = ready.back();
                ready.pop_back();
                const int x = e & 0xfffff, o = e >> 20;
                for (int o2 = 0; o2 < 8; ++o2)
                    for (int y = 0; y < n; ++y)
                        if (direct_dep(g, o, x, o2, y) && !done[o2 * n + y]) return fail("started early", g, o, x);
                if (busy[x]) return fail("tile running twice", g, o, x);
                for (int a = 0; a < 3; ++a)
                    for (int s = 0; s < 2; ++s) {
                        const int y = pfast::tile_neighbour(g, x, a, s);
                        if (y >= 0 && busy[y]) return fail("face neighbours at the same time", g, o, x);
                    }
                busy[x] = 1;
                running.push_back(e);
            } else {
                if (running.empty()) return fail("stalled", g, -1, completed);
                const int k = rng() % running.size();
                const int e = running[k];
                running[k] = running.back();
                running.pop_back();
                const int x = e & 0xfffff, o = e >> 20;
                busy[x] = 0;
                if (done[o * n + x]) return fail("item ran twice", g, o, x);
                done[o * n + x] = 1;
                ++completed;
                if (o + 2 < 8) {   // re-arm for order o + 2 (the counter is zero: it fired for (o, x))
                    if (cnt[2 * x + (o & 1)] != 0) return fail("re-arm of a live counter", g, o, x);
                    cnt[2 * x + (o & 1)] = pfast::dep_count(g, o + 2, x);
                }
                int t[16], od[16];
                const int m = pfast::dependents(g, o, x, t, od);
                for (int q = 0; q < m; ++q) {
                    int& c = cnt[2 * t[q] + (od[q] & 1)];
                    if (c <= 0) return fail("counter below zero", g, od[q], t[q]);
                    if (--c == 0) ready.push_back(t[q] | (od[q] << 20));
                }
            }
        }
        if (!ready.empty() || !running.empty()) return fail("items left over", g, -1, (int)ready.size());
    }
    std::printf("ok %dx%dx%d\n", g.nbk, g.nbi, g.nbj);
    return 0;
}

int main() {
    const int grids[][3] = {{1, 1, 1}, {1, 1, 3}, {2, 1, 1}, {1, 4, 1}, {2, 2, 2}, {3, 4, 2}, {5, 2, 3}, {4, 4, 4}, {2, 7, 1}};
    unsigned seed = 12345;
    for (const auto& gd : grids)
        for (int width : {1, 3, 64})
            if (check_grid(TileGrid3{gd[0], gd[1], gd[2]}, seed++, width)) return 1;
    return 0;
}
