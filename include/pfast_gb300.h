/*
 * pfast_gb300.h -- C ABI of the GB300 (sm_103a) implementation of PFAST's
 * traveltime-and-gradient hot path: the Godunov fast-sweeping Eikonal solver,
 * the Huygens reflection traveltime (2D) and the adjoint-state sweeps with
 * per-source gradient accumulation.
 *
 * Plain C types only: pointers, sizes, doubles.  Every call returns a status
 * code (PFAST_OK == 0); on failure pfast_last_error() holds a message.  No call
 * exits the process.
 *
 * Index conventions are the reference's:
 *   3D field  U[k*nrows*ncols + i*ncols + j]   k = z (dz), i = row (y, dy), j = col (x, dx)
 *   2D field  U[i*ncols + j]                   i = row (depth, dz), j = col (x, dx)
 *   3D src / rec / nxyz rows: 3 entries (row, col, z) / (n_y, n_x, n_z)
 *   2D src / rec / nxy rows:  2 entries (row, col) / (n_z, n_x)
 *   receiver rows of source s start at sum(srnum[0..s-1]).
 */
#ifndef PFAST_GB300_H
#define PFAST_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int pfast_status;

#define PFAST_OK 0
#define PFAST_ERR_INVALID 1              /* bad argument: size, index, null pointer */
#define PFAST_ERR_CUDA 2                 /* a CUDA runtime call failed */
#define PFAST_ERR_NOMEM 3                /* device memory exhausted */
#define PFAST_ERR_NO_DEVICE 4            /* no usable CUDA device */
#define PFAST_ERR_NO_REFLECTION_POINT 5  /* no node above a reflector (src/RT_pfsm2d.h:232,257,281) */
#define PFAST_ERR_NEGATIVE_TIME 6        /* reflected time < 0 (src/RT_pfsm2d.h:225-227,253,274) */
#define PFAST_ERR_OVER_CORRECTED 7       /* check_conv: sqrt(max (a*dk/vp)^2) / N >= 1 (src/RT_padjoint2d.h:489-490) */
#define PFAST_ERR_LINE_SEARCH 8          /* cubicInterp has no value for its arguments (src/RT_padjoint2d.h:619-630) */

/* Arithmetic of the sweeps. */
#define PFAST_PLAIN_FP64 0   /* reference arithmetic in FP64, bit-identical with FMA contraction off */
#define PFAST_MIXED 1        /* FP32 bulk sweeps, then FP64 polish sweeps until the FP64 test passes */

typedef struct pfast_ctx pfast_ctx;
typedef struct pfast_survey3d pfast_survey3d;
typedef struct pfast_survey2d pfast_survey2d;

typedef struct {
    int precision;   /* PFAST_PLAIN_FP64 or PFAST_MIXED */
    int maxswp;      /* MAXSwp: outer-iteration cap per solve (3D driver 100, 2D driver 500) */
    int max_batch;   /* sources per device batch; 0 = as many as fit */
    double polish_floor;  /* mixed mode (3D): FP64 polish corrections of at most this many seconds
                             (adjoint: times 1 + |lambda|) are dropped, so converged regions reach
                             a bitwise fixed point; 0 = the default, 1e-10.  Keep it well below the
                             1e-9 convergence tolerance. */
    int schedule;         /* 3D sweeps: 0 = automatic (per sweep kind, the fastest schedule and
                             tile shape measured by pfast_survey3d_autotune for this grid shape and
                             source count; untuned: persistent from 2 sources per SM), 1 = one launch
                             per tile diagonal (every tile of every source spread over all SMs), 2 =
                             persistent: one dataflow launch per phase, one block solves one source
                             with its sweep orders overlapping as the tile dependencies allow (grids
                             of at most 8192 tiles; larger grids use 1), 3 = hybrid: the first outer
                             iteration per tile diagonal, the rest in the dataflow kernel.  Same
                             results. */
    int near_source_radius;  /* 3D forward, opt-in (not in the reference): nodes within this many grid
                             nodes of the source (Euclidean, in nodes) start from the straight-ray
                             traveltime 0.5*(s_src + s_node)*distance and stay fixed, which removes most
                             of the first-order scheme's source error.  0 = off (the reference's
                             point-source start; results bit-identical to it). */
    int tile_shape;       /* 3D sweeps: nodes per tile (one warp updates one tile), in sweep-order
                             axes (z, rows, columns): 0 = automatic (as schedule 0; untuned 4x8x32),
                             1 = 4x8x32, 2 = 8x4x32.  Plain FP64 results are bit-identical for both
                             shapes; in the mixed mode the FP64 polish may stop at other bits within
                             its 1e-9 tolerance. */
} pfast_options;
#define PFAST_SCHEDULE_AUTO 0
#define PFAST_SCHEDULE_DIAGONAL 1
#define PFAST_SCHEDULE_PERSISTENT 2
#define PFAST_SCHEDULE_HYBRID 3
#define PFAST_TILE_AUTO 0
#define PFAST_TILE_4x8x32 1
#define PFAST_TILE_8x4x32 2
/* Candidates of the autotuner: (schedule, tile shape) pairs, index = 2*(schedule-1) + (shape-1). */
#define PFAST_TUNE_CANDIDATES 6

typedef struct {
    long long fwd_node_updates;   /* executed node updates, forward sweeps (all precisions) */
    long long adj_node_updates;   /* executed node updates, adjoint sweeps */
    long long fwd64_node_updates; /* of which FP64 */
    long long adj64_node_updates;
    int fwd_iters_max;            /* largest FP64 outer-iteration count over the solves */
    int adj_iters_max;
    int fwd32_iters_max;          /* largest FP32 outer-iteration count (mixed mode) */
    int adj32_iters_max;
    int not_converged;            /* solves that stopped at maxswp */
    int batches;                  /* device batches used */
    long long launches;           /* kernels launched */
    double ms_fwd32, ms_fwd64;    /* device time per phase, CUDA events on the context stream */
    double ms_adj32, ms_adj64;
    double ms_other;              /* initialisation, receiver conditions, gradient sums */
    double ms_total;
    int candidates;               /* 3D: per sweep kind k -- 0 plain forward, 1 FP32 forward, 2 polish
                                     forward, 3 plain adjoint, 4 FP32 adjoint, 5 polish adjoint -- bits
                                     4k..4k+3: 1 + the (schedule, tile shape) candidate (index as in
                                     pfast_survey3d_autotune) of its last phase; 0 = kind not run */
} pfast_stats;

/* ------------------------------------------------------------------ library */
const char* pfast_version(void);
const char* pfast_status_string(pfast_status s);
const char* pfast_last_error(void);          /* message of the last failure on this thread */
void pfast_default_options(pfast_options* opt);

pfast_status pfast_ctx_create(int device, pfast_ctx** out);
pfast_status pfast_ctx_destroy(pfast_ctx* ctx);
/* Run subsequent work on `stream` (a cudaStream_t); NULL restores the context's own stream. */
pfast_status pfast_ctx_set_stream(pfast_ctx* ctx, void* stream);
/* Per-diagonal sweeps (3D and 2D): replay each outer iteration as a captured CUDA graph
   (enabled = 1, the default) or launch its kernels one by one (0; results are the same). */
pfast_status pfast_ctx_set_graphs(pfast_ctx* ctx, int enabled);
pfast_status pfast_ctx_synchronize(pfast_ctx* ctx);

/* ---------------------------------------------- reference-signature entry points
 * Same argument order and meaning as the reference functions; host buffers; a
 * process-wide context on the current device.  `pe` is accepted and ignored
 * (rank id, used only in the reference's messages).  Output arrays are fully
 * overwritten, as in the reference.
 */
/* replaces fsm3d, src/T_pfsm3d.h:131 */
pfast_status pfast_fsm3d(double* vp, double* U, int* src, int srcid, int MAXSwp, double dx, double dy,
                         double dz, int nrows, int ncols, int nz, int pe);
/* replaces adjoint_fsm3d, src/T_padjoint3d.h:73 (the misfit EE is returned in *EE) */
pfast_status pfast_adjoint_fsm3d(double* U, double* T, double* T_obs, int* rec, double* nxyz, int* src,
                                 int* srnum, int srcid, int MAXSwp, double dx, double dy, double dz,
                                 int nrows, int ncols, int nz, int pe, double* EE);
/* replaces RT_fsm2d, src/RT_pfsm2d.h:116 (rec and srnum are unused there, as in the reference) */
pfast_status pfast_RT_fsm2d(double* vp, double* U, double* TTd, double* TTu, double* Z, int* src, int* rec,
                            int* srnum, int srcid, int NumofR, int MAXSwp, double dx, double dz, int nrows,
                            int ncols, int pe);
/* replaces Tadjoint_fsm2d (Cr = 1 overload), src/RT_padjoint2d.h:288 */
pfast_status pfast_Tadjoint_fsm2d(double* U, double* T, double* T_obs, int* rec, double* nxyz, int* src,
                                  int* srnum, int srcid, int MAXSwp, double dx, double dz, int nrows, int ncols,
                                  int pe, double* EE);
/* replaces Radjoint_fsm2d (Cr = 1 overload), src/RT_padjoint2d.h:382 */
pfast_status pfast_Radjoint_fsm2d(double* UR, double* Td, double* Tu, double* TR_obs, int* rec, double* nxyz,
                                  int* src, int* srnum, int srcid, int NumofR, int MAXSwp, double dx, double dz,
                                  int nrows, int ncols, int pe, double* EE);

/* ------------------------------------------------------------ batched surveys
 * A survey holds the acquisition geometry and picks on the device; evaluations
 * then take the model.  This is the per-source loop of the drivers
 * (src/T_PFAST3D.cpp:387-399, src/RT_PFAST2D.cpp:420-457) run as one batch on
 * one GPU: the gradient is summed in source order, so the result equals the
 * reference's single-process (np=1) result.
 */
/* 3D: src[nsrc*3], srnum[nsrc], rec[nrec*3], nxyz[nrec*3], T_obs[nrec]; host arrays, copied. */
pfast_status pfast_survey3d_create(pfast_ctx* ctx, int nrows, int ncols, int nz, double dx, double dy,
                                   double dz, int nsrc, const int* src, const int* srnum, const int* rec,
                                   const double* nxyz, const double* T_obs, pfast_survey3d** out);
pfast_status pfast_survey3d_destroy(pfast_survey3d* sv);
/* Misfit + gradient (T_PFAST3D.cpp:387-399).  vp, grad: DEVICE arrays [nz*nrows*ncols]. */
pfast_status pfast_survey3d_eval(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp, const pfast_options* opt,
                                 double* grad, double* misfit, pfast_stats* stats);
/* First-arrival picks (T_PFAST3D.cpp:672-686).  vp, picks: DEVICE arrays; picks[nrec]. */
pfast_status pfast_survey3d_forward(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp,
                                    const pfast_options* opt, double* picks, pfast_stats* stats);

/* Schedule and tile-shape autotuner: runs the survey's evaluation (gradient when it has picks,
 * else picks) once per candidate (schedule, tile shape) -- per-diagonal 4x8x32, per-diagonal
 * 8x4x32, persistent 4x8x32, persistent 8x4x32, hybrid 4x8x32, hybrid 8x4x32 -- on the DEVICE
 * model vp and records each
 * phase's time per (sweep kind, grid shape, source count); later calls with schedule and
 * tile_shape both automatic use, per phase, the fastest candidate.  stats: null, or an array of
 * PFAST_TUNE_CANDIDATES records in that order (a persistent candidate whose grid does not fit
 * the dataflow kernel runs per diagonal). */
pfast_status pfast_survey3d_autotune(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp, const pfast_options* opt,
                                     pfast_stats* stats);

/* Misfit + gradient of n independent (model, survey) pairs at once: the reference's per-model
 * evaluation (the source loop of src/T_PFAST3D.cpp:387-399, one model per run) for many models
 * of different grids.  Every sweep phase of all pairs runs as one dataflow launch over their
 * (model, source) instances, largest grid first, each instance retiring as it converges; the
 * steps between phases run per model.  Each pair's gradient, misfit and iteration counts equal
 * those of pfast_survey3d_eval on it alone (schedule and max_batch of opt are not used).
 * surveys[m] (of this context, with picks), vp[m] and grad[m] (DEVICE arrays of that grid's
 * size); misfit: HOST [n]; stats: summed over the pairs (optional).  Grids of at most 8192
 * tiles of 4x8x32 nodes; pairs are grouped to fit the device memory. */
pfast_status pfast_surveys3d_eval(pfast_ctx* ctx, int n, pfast_survey3d* const* surveys, const double* const* vp,
                                  double* const* grad, double* misfit, const pfast_options* opt, pfast_stats* stats);

/* One-call host-buffer forms (copies in and out inside the call). */
pfast_status pfast_eval3d(pfast_ctx* ctx, const double* vp, int nrows, int ncols, int nz, double dx, double dy,
                          double dz, int nsrc, const int* src, const int* srnum, const int* rec, const double* nxyz,
                          const double* T_obs, const pfast_options* opt, double* grad, double* misfit,
                          pfast_stats* stats);
pfast_status pfast_forward3d(pfast_ctx* ctx, const double* vp, int nrows, int ncols, int nz, double dx, double dy,
                             double dz, int nsrc, const int* src, const int* srnum, const int* rec,
                             const pfast_options* opt, double* picks, pfast_stats* stats);

/* 2D: src[nsrc*2], srnum[nsrc], rec[nrec*2], nxy[nrec*2], TT_obs[nrec], TR_obs[nrec*NumofR],
 * Z[NumofR*ncols*3] = (depth, n_z, n_x) per column.  nxy, TT_obs, TR_obs may be NULL for forward-only use. */
pfast_status pfast_survey2d_create(pfast_ctx* ctx, int nrows, int ncols, double dx, double dz, int nsrc,
                                   const int* src, const int* srnum, int nrec, const int* rec, const double* nxy,
                                   const double* TT_obs, int NumofR, const double* TR_obs, const double* Z,
                                   pfast_survey2d** out);
pfast_status pfast_survey2d_destroy(pfast_survey2d* sv);
/* Picks Tr[nrec*(NumofR+1)] (src/RT_PFAST2D.cpp:832-852).  vp, Tr: DEVICE arrays. */
pfast_status pfast_survey2d_forward(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp,
                                    const pfast_options* opt, double* Tr, pfast_stats* stats);
/* Joint gradient (src/RT_PFAST2D.cpp:420-457): gT, gR, gRT = gT*(1-WR)+gR*WR, and the
 * transmission / reflection misfits.  vp, WR, gT, gR, gRT: DEVICE arrays [nrows*ncols]. */
pfast_status pfast_survey2d_eval(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const double* WR,
                                 const pfast_options* opt, double* gT, double* gR, double* gRT, double* Et,
                                 double* Er, pfast_stats* stats);

/* One-call host-buffer forms of the 2D survey (copies in and out inside the call);
 * arguments as in pfast_survey2d_create.  Tr[nrec*(NumofR+1)] (src/RT_PFAST2D.cpp:832-852). */
pfast_status pfast_forward2d(pfast_ctx* ctx, const double* vp, int nrows, int ncols, double dx, double dz, int nsrc,
                             const int* src, const int* srnum, int nrec, const int* rec, int NumofR, const double* Z,
                             const pfast_options* opt, double* Tr, pfast_stats* stats);
/* Joint gradient with host buffers (src/RT_PFAST2D.cpp:420-457); WR, gT, gR, gRT: [nrows*ncols]. */
pfast_status pfast_eval2d(pfast_ctx* ctx, const double* vp, const double* WR, int nrows, int ncols, double dx,
                          double dz, int nsrc, const int* src, const int* srnum, int nrec, const int* rec,
                          const double* nxy, const double* TT_obs, int NumofR, const double* TR_obs, const double* Z,
                          const pfast_options* opt, double* gT, double* gR, double* gRT, double* Et, double* Er,
                          pfast_stats* stats);

/* ------------------------------------------------------------------ inversion loop
 * The drivers' outer loop (src/RT_PFAST2D.cpp:412-816, src/T_PFAST3D.cpp:359-656) with
 * every N-vector resident on the device: gradient of the survey, FFT low-pass
 * regularisation (regu2d / regu3d), search direction (L-BFGS two-loop recursion, HS or
 * CG_DESCENT), line search, updatevp and check_conv.  One pfast_inversion_step is one
 * "Iterating No. k" of the reference; the report carries what the reference prints.
 * Inner products are summed in a fixed order (identical results run to run); the FFT is
 * cuFFT's, so results agree with the reference to rounding, not bit for bit.
 */
typedef struct pfast_inversion pfast_inversion;

#define PFAST_SCHEME_HS 1          /* beta_HS, src/RT_padjoint2d.h:560-571 */
#define PFAST_SCHEME_CGDESCENT 2   /* beta_CGDESCENT, src/RT_padjoint2d.h:573-588 */
#define PFAST_SCHEME_LBFGS 3       /* gd2sk + two-loop recursion, src/RT_PFAST2D.cpp:520-546 */
#define PFAST_LS_NONE 0            /* lsrc 0: step alpha1 as is */
#define PFAST_LS_SECANT_EXACT 1    /* lsrc 1: secant on the directional derivative */
#define PFAST_LS_SECANT_WOLFE 2    /* lsrc 2: secant with the strong Wolfe test */
#define PFAST_LS_CUBIC 3           /* lsrc 3: cubic interpolation (strong Wolfe loop with L-BFGS) */
#define PFAST_RT_TRANSMISSION 1    /* RTtag (2D): gradient and line-search misfit of transmission only */
#define PFAST_RT_REFLECTION 2      /*              reflection only */
#define PFAST_RT_JOINT 3           /*              gT*(1-WR) + gR*WR and Et + Er */

typedef struct {
    pfast_options eval;   /* gradient evaluations (precision, MAXSwp, batch cap) */
    int schemetag;        /* PFAST_SCHEME_*; 3D runs L-BFGS whatever is asked (src/T_PFAST3D.cpp:428) */
    int lsrc;             /* PFAST_LS_* */
    int LM;               /* L-BFGS memory (drivers' command-line argument, default 5) */
    int max_linesearch;   /* MAXLineSch: trial models per line search (2D 5, 3D 2); at most 16 */
    int rttag;            /* PFAST_RT_* (2D) */
    double nux, nuy, nuz; /* regularisation lengths.  2D: nux (columns, dx) and nuz (rows, dz) are
                             the .inp's two values, which the 2D driver calls nux, nuy */
    double minv, maxv;    /* updatevp clamp, MINV / MAXV: 1600 / 4500 (2D), 1400 / 8000 (3D) */
    double conv_tol;      /* check_conv stops when (E[k-1]-E[k])/E[k-1] <= conv_tol: 1e-3 (2D), 1e-2 (3D) */
    int keep_components;  /* 2D: also regularise gR and gT each iteration (the driver writes them) */
} pfast_invert_options;

#define PFAST_INV_MAX_TRIALS 16
typedef struct {
    int iter;             /* Iterk, from 1 */
    double E, Et, Er;     /* misfits at the iteration's starting model: global_E (Et + Er in 2D) and parts */
    double alpha_start;   /* alpha1 entering the line search */
    int ntrials;          /* rows of trial[] filled (lsrc 2 and 3) */
    double trial[PFAST_INV_MAX_TRIALS][6];  /* (alpha0, alpha1, phi0, phi1, dphi0, dphi1) as printed */
    int count;            /* the line search's `count` after its loop */
    int stopped;          /* 1: count > MAXLineSch ("Line Search Stopped") */
    double stepsize;      /* alpha1 applied by updatevp */
    int converged;        /* check_conv returned true */
    int evals;            /* gradient evaluations made in this iteration */
    double ms_eval;       /* wall time of those evaluations */
    double ms_linesearch; /* wall time of the line search, its evaluations included */
    double ms_total;      /* wall time of the iteration */
} pfast_invert_report;

/* Fields readable after a step (pfast_inversion_get / _field). */
#define PFAST_INV_VP 0         /* current model (<p>_<k> after step k) */
#define PFAST_INV_GRAD_RAW 1   /* step's gradient before regularisation (<p>_bf_regu_RT<k>) */
#define PFAST_INV_GRAD 2       /* after regularisation (<p>_af_regu_RT<k>) */
#define PFAST_INV_DIRECTION 3  /* search direction dk */
#define PFAST_INV_GR_RAW 4     /* 2D with keep_components: reflection gradient, before / after */
#define PFAST_INV_GR 5
#define PFAST_INV_GT_RAW 6     /*                          transmission gradient, before / after */
#define PFAST_INV_GT 7

/* Defaults of the reference drivers for dim 2 (RT_PFAST2D) or 3 (T_PFAST3D). */
void pfast_invert_default_options(int dim, pfast_invert_options* opt);
/* vp [nrows*ncols] and WR [nrows*ncols] are HOST arrays (copied).  The survey must hold
 * picks and outlive the inversion. */
pfast_status pfast_inversion2d_create(pfast_ctx* ctx, pfast_survey2d* sv, const double* vp, const double* WR,
                                      const pfast_invert_options* opt, pfast_inversion** out);
/* vp [nz*nrows*ncols]: HOST array (copied). */
pfast_status pfast_inversion3d_create(pfast_ctx* ctx, pfast_survey3d* sv, const double* vp,
                                      const pfast_invert_options* opt, pfast_inversion** out);
/* Resume of T_PFAST3D (src/T_PFAST3D.cpp:346-385): `k` iterations are done and the run stopped
 * inside iteration k+1 after writing its gradient.  The next step skips its gradient evaluation
 * and uses grad_cur (<p>_bf_regu_<k+1>.vp, unregularised, used as is) as the gradient,
 * grad_prev (<p>_bf_regu_<k>.vp) as the previous gradient and search direction, E_hist[0..nE)
 * (global_E.tmp, nE >= k+1) as the misfit history and alpha1 (alpha1.tmp) as the last step.
 * The L-BFGS pair store starts empty.  The model is the one given at create (<p>.vp<k>).
 * HOST arrays [nz*nrows*ncols]. */
pfast_status pfast_inversion_resume(pfast_inversion* inv, int k, const double* grad_prev, const double* grad_cur,
                                    const double* E_hist, int nE, double alpha1);
/* One outer iteration.  Returns PFAST_ERR_OVER_CORRECTED after the model update when check_conv
 * aborts (the report and the updated model are still readable). */
pfast_status pfast_inversion_step(pfast_inversion* inv, pfast_invert_report* rep);
/* Copy a field (PFAST_INV_*) to a HOST array of the model's size. */
pfast_status pfast_inversion_get(pfast_inversion* inv, int field, double* host);
/* The DEVICE array of a field (valid until the next step or destroy). */
pfast_status pfast_inversion_field(pfast_inversion* inv, int field, const double** dev);
pfast_status pfast_inversion_destroy(pfast_inversion* inv);

/* ------------------------------------------------------------------ request server
 * No counterpart in the reference (its drivers run one survey per MPI job).  Continuous
 * batching on one GPU: traveltime (forward) and misfit-gradient requests of any grid size
 * arrive at any time; models and surveys stay resident on the device under an ID; a
 * request starts as soon as one of `slots` workers is free and its device memory fits the
 * HBM budget (resident data plus running requests), and running requests overlap on the
 * GPU, each on its own stream.  Admission is first come first served, except that a
 * younger request may overtake a waiting one that does not fit yet (at most `max_bypass`
 * times); a request's source batch is sized to its memory allowance.  Results do not
 * depend on what else runs: every request is computed exactly as it would be alone.
 */
typedef struct pfast_server pfast_server;

typedef struct {
    int device;
    int slots;                 /* requests running at once (workers), >= 1 */
    double hbm_budget_bytes;   /* device memory for resident models/surveys and running requests */
    int max_bypass;            /* overtakes of a waiting request before it blocks admission (8) */
} pfast_server_config;

#define PFAST_REQ_FORWARD 0    /* picks: 3D [nrec]; 2D [nrec*(NumofR+1)] (TT then each reflector) */
#define PFAST_REQ_GRADIENT 1   /* misfit and gradient [N]: 3D grad; 2D gRT = gT(1-WR) + gR WR */

typedef struct {
    int kind;                  /* PFAST_REQ_* */
    long long model_id;        /* registered with pfast_server_put_model */
    long long survey_id;       /* registered with pfast_server_put_survey3d / _2d (same grid) */
    pfast_options opt;         /* precision, maxswp, polish_floor, schedule; max_batch: the server's */
    double* out;               /* HOST output, written when the request completes */
    double* out_misfit;        /* gradient: HOST scalar, E (3D) or Et + Er (2D); may be NULL */
} pfast_request;

typedef struct {
    pfast_status status;       /* the request's own status */
    int batch;                 /* sources solved at once */
    double queue_ms;           /* submit -> start */
    double run_ms;             /* start -> done */
    double total_ms;           /* submit -> done */
} pfast_request_result;

typedef struct {
    long long submitted, completed, failed;
    int running, waiting;
    int resident_models, resident_surveys;
    double used_bytes, peak_bytes, budget_bytes;
} pfast_server_stats;

pfast_status pfast_server_create(const pfast_server_config* cfg, pfast_server** out);
/* Waits for every submitted request, then frees everything. */
pfast_status pfast_server_destroy(pfast_server* srv);
/* A velocity model (HOST array [nz*nrows*ncols], nz = 1 in 2D) kept on the device under
 * model_id; 2D gradient requests also need WR [nrows*ncols] (else NULL).  dim: 2 or 3.
 * Replacing an ID that requests still use fails (PFAST_ERR_INVALID). */
pfast_status pfast_server_put_model(pfast_server* srv, long long model_id, int dim, int nrows, int ncols, int nz,
                                    double dx, double dy, double dz, const double* vp, const double* WR);
/* Surveys, arguments as pfast_survey3d_create / pfast_survey2d_create (HOST arrays, copied). */
pfast_status pfast_server_put_survey3d(pfast_server* srv, long long survey_id, int nrows, int ncols, int nz, double dx,
                                       double dy, double dz, int nsrc, const int* src, const int* srnum,
                                       const int* rec, const double* nxyz, const double* T_obs);
pfast_status pfast_server_put_survey2d(pfast_server* srv, long long survey_id, int nrows, int ncols, double dx,
                                       double dz, int nsrc, const int* src, const int* srnum, int nrec,
                                       const int* rec, const double* nxy, const double* TT_obs, int NumofR,
                                       const double* TR_obs, const double* Z);
/* Forget a model (what = 0) or survey (what = 1); freed once no request uses it.  Unused
 * resident entries are also evicted, least recently used first, when new data needs room. */
pfast_status pfast_server_drop(pfast_server* srv, int what, long long id);
/* Queue a request; *ticket identifies it.  The output buffers must stay valid until wait. */
pfast_status pfast_server_submit(pfast_server* srv, const pfast_request* req, long long* ticket);
/* Block until the request is done; returns its status (message in pfast_last_error). */
pfast_status pfast_server_wait(pfast_server* srv, long long ticket, pfast_request_result* res);
pfast_status pfast_server_stats_get(pfast_server* srv, pfast_server_stats* st);

/* ------------------------------------------------------- no-allocation entry point
 * No counterpart in the reference.  The traveltime field of one point source --
 * the computation of pfast_fsm3d (plain FP64, bit-identical to it) -- for callers
 * that cannot allocate device memory: a host whose own pool allocator or memory
 * budget owns the device and forbids libraries to allocate, or a loop that must not
 * meet the allocator's synchronisation.  vp and U are DEVICE arrays
 * [nz*nrows*ncols] owned by the caller; `stream` is a cudaStream_t (NULL: the
 * default stream).  The call makes no cudaMalloc / cudaFree: its work memory is one
 * static device array sized for PFAST_NOALLOC_MAX_NODES grid nodes (about 16.1 MiB,
 * held by every GPU that loads the library until the process exits).  Larger grids
 * are rejected with PFAST_ERR_INVALID.  The first call on a device looks the array
 * up (cudaGetSymbolAddress) and caches its address; make that first call before any
 * stream capture, and do not reuse the library across cudaDeviceReset.  The call
 * blocks the calling thread: it synchronises `stream` after the velocity check and
 * once per outer iteration to read the convergence flag.  All calls share the
 * array: calls that overlap on the GPU race.
 */
#define PFAST_NOALLOC_MAX_NODES 1048576
pfast_status pfast_fsm3d_noalloc(const double* vp, double* U, int src_row, int src_col, int src_z, int MAXSwp,
                                 double dx, double dy, double dz, int nrows, int ncols, int nz, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PFAST_GB300_H */
