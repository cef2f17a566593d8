// dataflow3.h -- the 3D sweeps of one outer iteration as a dataflow graph of tile items
// (host and device code; the CPU check tests/native/dataflow3_check.cpp compiles it with g++).
//
// The reference runs an outer iteration as eight lexicographic sweeps, one after another
// (src/T_pfsm3d.h:158-178, src/T_padjoint3d.h:139-161).  A node update in sweep order o reads
// its three upstream neighbours' values of sweep o and its three downstream neighbours' values
// of sweep o-1.  With the grid cut into tiles, item (o, x) -- the processing of tile x in sweep
// order o -- therefore needs
//   (o-1, x)                                      (its own previous sweep; o > 0),
//   (o, n)   for each face neighbour n upstream of x in order o,
//   (o-1, n) for each face neighbour n downstream of x in order o (o > 0),
// and nothing else: every node of x then reads exactly the neighbour versions of the
// reference's sequential sweeps, and no two face neighbours are ever processed at the same
// time (each of any two neighbouring items depends on the other's earlier sweep or on the
// other itself).  Sweeps of different orders overlap wherever these dependencies allow, instead
// of waiting for the whole previous sweep, as a launch per sweep and tile diagonal does.
//
// Tiles: x = (tk * nbi + ti) * nbj + tj.  Order o: bit 2 set = z ascending, bit 1 = rows
// ascending, bit 0 = columns ascending (o = 0..7 is the reference's sweep sequence).
// Axis a: 0 = columns (tj), 1 = rows (ti), 2 = z (tk).  Side s of a tile along an axis:
// 0 = index - 1, 1 = index + 1.
#pragma once

#ifdef __CUDACC__
#define PFAST_HD __host__ __device__ __forceinline__
#else
#define PFAST_HD inline
#endif

namespace pfast {

struct TileGrid3 {
    int nbk, nbi, nbj;
};

PFAST_HD int tile_count(const TileGrid3& g) { return g.nbk * g.nbi * g.nbj; }

// The neighbour on side s of axis a, or -1 outside the tile grid.
PFAST_HD int tile_neighbour(const TileGrid3& g, int x, int a, int s) {
    const int tj = x % g.nbj, ti = (x / g.nbj) % g.nbi, tk = x / (g.nbj * g.nbi);
    const int d = s ? 1 : -1;
    if (a == 0) return (tj + d < 0 || tj + d >= g.nbj) ? -1 : x + d;
    if (a == 1) return (ti + d < 0 || ti + d >= g.nbi) ? -1 : x + d * g.nbj;
    return (tk + d < 0 || tk + d >= g.nbk) ? -1 : x + d * g.nbj * g.nbi;
}

// Whether, in sweep order o, the neighbour on side s of axis a is visited before the tile.
PFAST_HD bool side_upstream(int o, int a, int s) { return ((o >> a) & 1) ? s == 0 : s == 1; }

// Number of items (o, x) waits for.
PFAST_HD int dep_count(const TileGrid3& g, int o, int x) {
    int c = o > 0 ? 1 : 0;
    for (int a = 0; a < 3; ++a)
        for (int s = 0; s < 2; ++s)
            if (tile_neighbour(g, x, a, s) >= 0 && (side_upstream(o, a, s) || o > 0)) ++c;
    return c;
}

// The items that wait for (o, x), at most 13: tile[k], order[k] for k < the returned count.
//   (o+1, x)                                    for o < 7,
//   (o, n)   for each neighbour n that x is upstream of in order o,
//   (o+1, n) for each neighbour n that x is downstream of in order o+1 (o < 7).
// (x lies on side 1-s of its neighbour on side s.)
PFAST_HD int dependents(const TileGrid3& g, int o, int x, int* tile, int* order) {
    int n = 0;
    if (o < 7) { tile[n] = x; order[n] = o + 1; ++n; }
    for (int a = 0; a < 3; ++a)
        for (int s = 0; s < 2; ++s) {
            const int y = tile_neighbour(g, x, a, s);
            if (y < 0) continue;
            if (side_upstream(o, a, 1 - s)) { tile[n] = y; order[n] = o; ++n; }
            if (o < 7 && !side_upstream(o + 1, a, 1 - s)) { tile[n] = y; order[n] = o + 1; ++n; }
        }
    return n;
}

// The one item with no dependency: the first tile of sweep order 0 (all axes descending).
PFAST_HD int first_tile(const TileGrid3& g) { return tile_count(g) - 1; }

}  // namespace pfast
