// kernels2d.h -- host-side launchers of the 2D kernels (internal).
#pragma once

#include <vector>
#include "common.cuh"

namespace pfast {

// A 2D batch is a list of instances; instance q sweeps the field at
// base + inst_off[q], may update node (i, j) only if i <= rowlim[inst_lim[q]*nc + j]
// (inst_lim[q] < 0: no row limit) and never updates (inst_src[q] >> 16, inst_src[q] & 0xffff)
// when inst_src[q] >= 0.  These cover the three FSM solves of src/RT_pfsm2d.h:
// down-going (rows with (i+1)*dz <= reflector depth, not the source), up-going
// (rows up to the reflection point) and transmission (every node but the source).
struct Sweep2Args {
    void* field;                 // Real, instance fields at field + inst_off[q]
    const long long* inst_off;
    const int* inst_lim;
    const int* inst_src;
    const int* rowlim;           // [*][nc]
    const void* aux;             // forward: slowness (Real, shared); adjoint: T (double) at aux + aux_off[q]
    const long long* aux_off;
    const unsigned* mask;        // adjoint: fixed-node bits at mask + mask_off[q]
    const long long* mask_off;
    int wpr;
    void* snap;                  // per instance at snap + q*n (Real)
    int* changed;                // per instance
    const int* act;              // active instance ids (grid.y)
    const int* diag_off;
    const unsigned* diag_tiles;  // packed bi | bj<<16, flipped coordinates
    int nr, nc, nbi, nbj;
    double dx, dz;
    double inv2x, inv2z;         // (1.0/dx)/dx, (1.0/dz)/dz
    float dxf, dzf;              // FP32 copies of dx, dz (no FP64 instruction in the FP32 sweeps)
    float wxf, wzf, rsumf;       // FP32 inv2x, inv2z, 1/(inv2x + inv2z)
    float polish_floor;          // polish corrections at or below this are dropped
    int src_r2;                  // forward: nodes within squared node distance src_r2 of the source
                                 // are fixed (0: the source node alone, the reference's point source)
    int dir;                     // 0..3: bit1 = s1>0 (rows), bit0 = s2>0 (cols); reference order
    int iter;                    // outer iteration (snapshot stamps)
    int ntiles;                  // tiles per instance (nbi * nbj)
    int* dirty;                  // per (instance, tile): orders still due (bits 0-3), polish selection (4-7)
    int* stamp;                  // per (instance, tile): iteration of the tile's snapshot
    int* diff;                   // per (instance, tile): moved beyond the tolerance this iteration
    unsigned long long* work;    // per instance: nodes of the tiles processed; may be null
    double tol_abs, tol_rel;
    const int* dyn;              // replayed iteration graph: dyn[0] = outer iteration (instead of
                                 // iter), dyn[1] = active instances; null: iter and the grid
};

struct DiagTable2 {
    int nbi = 0, nbj = 0, ndiag = 0;
    std::vector<int> h_off;
    int* d_off = nullptr;
    unsigned* d_tiles = nullptr;
};

pfast_status build_diag_table2(int nr, int nc, DiagTable2& t);
void free_diag_table2(DiagTable2& t);
pfast_status launch_sweep2(int kind, const Sweep2Args& a, int d, int tiles, int nact, cudaStream_t st);
// Opt-in near-source start (not in the reference): in each instance q with a point source
// (inst_src[q] >= 0), the nodes within `radius` nodes (Euclidean) get the straight-ray time
// 0.5 (s_src + s_node) * distance; a down-going instance (inst_lim[q] >= 0) only above its
// reflector row limit.  Fields (FP32 if is_fp32) at base + off[q].
pfast_status launch_near_source2(void* base, int is_fp32, const long long* off, const int* inst_src,
                                 const int* inst_lim, const int* rowlim, const double* s64, int nr, int nc, double dx,
                                 double dz, int radius, int ninst, cudaStream_t st);
// Initial lock words from the starting field (active instances a.act[0..nact)): due where the
// tile's halo box holds a reached traveltime / nonzero lambda.  The forward polish: no-op.
pfast_status launch_seed_tiles2(int kind, const Sweep2Args& a, int nact, cudaStream_t st);

// Init: field(q) = 0 at inst_src node (or (si,sj) from src_ij for q), INF elsewhere.
pfast_status launch_init2(void* base, int is_fp32, const long long* inst_off, const int* inst_srcnode, long long n,
                          int ninst, cudaStream_t st);
pfast_status launch_copy_inst(const void* src, void* dst, int is_fp32, const long long* off_src, const long long* off_dst,
                              long long n, int ninst, cudaStream_t st);
pfast_status launch_widen_inst(const float* a, double* b, const long long* off32, const long long* off64, long long n,
                               int ninst, cudaStream_t st);
pfast_status launch_narrow_inst(const double* a, float* b, const long long* off64, const long long* off32, long long n,
                                int ninst, cudaStream_t st);
pfast_status launch_widen_lambda_inst(const float* a, double* b, const long long* off32, const long long* off64,
                                      const unsigned* mask, const long long* mask_off, int nr, int nc, int wpr,
                                      int ninst, cudaStream_t st);

// Reflection-point reinitialisation (src/RT_pfsm2d.h:195-295) on the up-going
// fields: per instance, columns in the reference's order (interior left to right,
// then the two edges); then every node at or above the reflection point is reset
// to INF.  k2[ir*nc + j] = reflection row (or -1 when the reflector lies below the
// model), qxcase[ir*nc + j] = 0 central / 1 backward / 2 forward x-difference.
struct Reflect2Args {
    double* U;
    const long long* inst_off;
    const int* inst_ir;
    const int* k2;
    const int* qxcase;
    const int* k2vec;
    const double* Z;   // [numofr*nc][3]
    int nr, nc;
    double dx, dz;
    int* err;          // set to 1 on a negative reflected time
};
pfast_status launch_reflect2(const Reflect2Args& a, int ninst, cudaStream_t st);

// Receiver boundary condition + misfit for 2D instances (transmission:
// src/RT_padjoint2d.h:311-339, reflection: 405-433).  Instance q belongs to batch
// source inst_b[q] and reflector inst_ir[q] (-1: transmission).
struct Bc2Args {
    const double* T; const long long* t_off;   // traveltime field per instance
    double* L; const long long* l_off;         // lambda field per instance (zeroed by the caller)
    unsigned* mask; const long long* mask_off;
    int wpr;
    const int* inst_src;                        // global source id per instance
    const int* inst_ir;
    const int* rec; const double* nxy;
    const double* ttobs; const double* trobs;   // [nrec], [nrec*numofr]
    const unsigned char* last_t; const unsigned char* last_r;
    const int* ch0; const int* srnum; const int* src_ij;   // indexed by global source id
    int numofr;
    double* EE; int* need;                      // per instance
    int nr, nc; double dx, dz;
};
pfast_status launch_bc2(const Bc2Args& a, int ninst, cudaStream_t st);

// g_b[n] <- g_b[n] - lam_q[n]/(v*v*v) for instances q in order; instance q adds into
// gradient slot gslot[q] (0 = transmission, 1 = reflection).
pfast_status launch_accumulate2(double* gT, double* gR, const double* lam, const long long* l_off, const int* gslot,
                                const double* vp, long long n, int ninst, cudaStream_t st);
// gRT = gT*(1-WR) + gR*WR
pfast_status launch_blend2(const double* gT, const double* gR, const double* WR, double* gRT, long long n,
                           cudaStream_t st);
// dst[n] += src_q[n] for instances q in order (sum of reflector adjoints, src/RT_padjoint2d.h:466).
pfast_status launch_addto2(double* dst, const long long* d_off, const double* src, const long long* s_off, long long n,
                           int ninst, cudaStream_t st);
// Picks: Tr[row*(numofr+1)+col] for the batch's sources.
pfast_status launch_gather2(const double* fields, const long long* src_field_off, int numofr, long long n,
                            const int* rec, const int* ch0, const int* srnum, int nbatch, int b0, int nc, double* Tr,
                            cudaStream_t st);

}  // namespace pfast
