// ref_harness3d.cpp -- exposes the UNMODIFIED reference 3D solver (src/T_pfsm3d.h,
// src/T_padjoint3d.h, compiled where they lie) through extern "C" symbols, so the
// tests can check the oracle restatement against the reference itself.
// TEST INFRASTRUCTURE ONLY; built by oracle/build_ref.py into oracle/_ref/.
#include "T_padjoint3d.h"

extern "C" {

// src/T_pfsm3d.h:131
void ref_fsm3d(double* vp, double* U, int* src, int srcid, int maxswp, double dx, double dy,
               double dz, int nrows, int ncols, int nz) {
    fsm3d(vp, U, src, srcid, maxswp, dx, dy, dz, nrows, ncols, nz, 0);
}

// src/T_padjoint3d.h:73
double ref_adjoint3d(double* L, double* T, double* Tobs, int* rec, double* nxyz, int* src,
                     int* srnum, int srcid, int maxswp, double dx, double dy, double dz,
                     int nrows, int ncols, int nz) {
    return adjoint_fsm3d(L, T, Tobs, rec, nxyz, src, srnum, srcid, maxswp, dx, dy, dz, nrows,
                         ncols, nz, 0);
}

}
