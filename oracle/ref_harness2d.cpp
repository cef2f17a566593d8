// ref_harness2d.cpp -- exposes the UNMODIFIED reference 2D solvers (src/RT_pfsm2d.h,
// src/RT_padjoint2d.h, compiled where they lie) through extern "C" symbols, so the
// tests can check the oracle restatement against the reference itself.
// TEST INFRASTRUCTURE ONLY; built by oracle/build_ref.py into oracle/_ref/.
#include "RT_padjoint2d.h"

extern "C" {

// src/RT_pfsm2d.h:116
void ref_rt_fsm2d(double* vp, double* U, double* TTd, double* TTu, double* Z, int* src, int* rec,
                  int* srnum, int srcid, int numofr, int maxswp, double dx, double dz, int nrows,
                  int ncols) {
    RT_fsm2d(vp, U, TTd, TTu, Z, src, rec, srnum, srcid, numofr, maxswp, dx, dz, nrows, ncols, 0);
}

// src/RT_padjoint2d.h:288 (the Cr=1 overload the driver calls)
double ref_tadjoint2d(double* L, double* T, double* Tobs, int* rec, double* nxy, int* src,
                      int* srnum, int srcid, int maxswp, double dx, double dz, int nrows,
                      int ncols) {
    return Tadjoint_fsm2d(L, T, Tobs, rec, nxy, src, srnum, srcid, maxswp, dx, dz, nrows, ncols, 0);
}

// src/RT_padjoint2d.h:382
double ref_radjoint2d(double* UR, double* Td, double* Tu, double* TRobs, int* rec, double* nxy,
                      int* src, int* srnum, int srcid, int numofr, int maxswp, double dx,
                      double dz, int nrows, int ncols) {
    return Radjoint_fsm2d(UR, Td, Tu, TRobs, rec, nxy, src, srnum, srcid, numofr, maxswp, dx, dz,
                          nrows, ncols, 0);
}

}
