"""Python host side of pfast_gb300.

Two layers, both over the C ABI (include/pfast_gb300.h):

* Reference-signature functions with the reference's names, argument order and
  in-place outputs on numpy host arrays: fsm3d (src/T_pfsm3d.h:131),
  adjoint_fsm3d (src/T_padjoint3d.h:73), RT_fsm2d (src/RT_pfsm2d.h:116),
  Tadjoint_fsm2d (src/RT_padjoint2d.h:288), Radjoint_fsm2d
  (src/RT_padjoint2d.h:382).  Where the reference exits the process, these raise
  PfastError.  The adjoint functions return the misfit EE, as the reference does.
* Batched surveys (Survey3D / Survey2D): geometry and picks resident on the GPU,
  all sources of an evaluation in one call, device tensors in and out.
* Inversion: the drivers' outer loop (src/RT_PFAST2D.cpp:412-816,
  src/T_PFAST3D.cpp:359-656) over a survey, one call per "Iterating No. k".
"""
import ctypes as C

import numpy as np

from . import _capi
from ._capi import PFAST_MIXED, PFAST_PLAIN_FP64, PfastError, check, lib

__all__ = ["fsm3d", "adjoint_fsm3d", "RT_fsm2d", "Tadjoint_fsm2d", "Radjoint_fsm2d", "Context", "Survey3D",
           "Survey2D", "eval3d_many", "eval3d_host", "forward3d_host", "Inversion", "invert_options", "Server", "Ticket", "PfastError",
           "PFAST_PLAIN_FP64", "PFAST_MIXED"]


def _arr(a, dtype, name, writable=False):
    if not isinstance(a, np.ndarray) or a.dtype != dtype or not a.flags.c_contiguous:
        raise TypeError(f"{name}: expected a C-contiguous {np.dtype(dtype).name} numpy array")
    if writable and not a.flags.writeable:
        raise TypeError(f"{name}: array is read-only")
    return a.ctypes.data


# ------------------------------------------------------------ reference-signature layer
def fsm3d(vp, U, src, srcid, MAXSwp, dx, dy, dz, nrows, ncols, nz, pe=0):
    """First-arrival traveltime of source `srcid` into U (in place)."""
    n = nrows * ncols * nz
    if vp.size < n or U.size < n:
        raise ValueError("vp / U smaller than nrows*ncols*nz")
    check(lib().pfast_fsm3d(_arr(vp, np.float64, "vp"), _arr(U, np.float64, "U", True), _arr(src, np.int32, "src"),
                            srcid, MAXSwp, dx, dy, dz, nrows, ncols, nz, pe), "fsm3d")


def adjoint_fsm3d(U, T, T_obs, rec, nxyz, src, srnum, srcid, MAXSwp, dx, dy, dz, nrows, ncols, nz, pe=0):
    """Adjoint state of source `srcid` into U (in place); returns the misfit EE."""
    EE = C.c_double(0.0)
    check(lib().pfast_adjoint_fsm3d(_arr(U, np.float64, "U", True), _arr(T, np.float64, "T"),
                                    _arr(T_obs, np.float64, "T_obs"), _arr(rec, np.int32, "rec"),
                                    _arr(nxyz, np.float64, "nxyz"), _arr(src, np.int32, "src"),
                                    _arr(srnum, np.int32, "srnum"), srcid, MAXSwp, dx, dy, dz, nrows, ncols, nz, pe,
                                    C.addressof(EE)), "adjoint_fsm3d")
    return EE.value


def RT_fsm2d(vp, U, TTd, TTu, Z, src, rec, srnum, srcid, NumofR, MAXSwp, dx, dz, nrows, ncols, pe=0):
    """Transmission field into U and down/up-going reflection fields into TTd/TTu."""
    z = np.zeros(1, np.float64)
    zi = np.zeros(1, np.int32)
    check(lib().pfast_RT_fsm2d(_arr(vp, np.float64, "vp"), _arr(U, np.float64, "U", True),
                               _arr(TTd if NumofR else z, np.float64, "TTd", True),
                               _arr(TTu if NumofR else z, np.float64, "TTu", True),
                               _arr(Z if NumofR else z, np.float64, "Z"), _arr(src, np.int32, "src"),
                               _arr(rec if rec is not None else zi, np.int32, "rec"),
                               _arr(srnum if srnum is not None else zi, np.int32, "srnum"), srcid, NumofR, MAXSwp,
                               dx, dz, nrows, ncols, pe), "RT_fsm2d")


def Tadjoint_fsm2d(U, T, T_obs, rec, nxyz, src, srnum, srcid, MAXSwp, dx, dz, nrows, ncols, pe=0):
    EE = C.c_double(0.0)
    check(lib().pfast_Tadjoint_fsm2d(_arr(U, np.float64, "U", True), _arr(T, np.float64, "T"),
                                     _arr(T_obs, np.float64, "T_obs"), _arr(rec, np.int32, "rec"),
                                     _arr(nxyz, np.float64, "nxyz"), _arr(src, np.int32, "src"),
                                     _arr(srnum, np.int32, "srnum"), srcid, MAXSwp, dx, dz, nrows, ncols, pe,
                                     C.addressof(EE)), "Tadjoint_fsm2d")
    return EE.value


def Radjoint_fsm2d(UR, Td, Tu, TR_obs, rec, nxyz, src, srnum, srcid, NumofR, MAXSwp, dx, dz, nrows, ncols, pe=0):
    EE = C.c_double(0.0)
    check(lib().pfast_Radjoint_fsm2d(_arr(UR, np.float64, "UR", True), _arr(Td, np.float64, "Td"),
                                     _arr(Tu, np.float64, "Tu"), _arr(TR_obs, np.float64, "TR_obs"),
                                     _arr(rec, np.int32, "rec"), _arr(nxyz, np.float64, "nxyz"),
                                     _arr(src, np.int32, "src"), _arr(srnum, np.int32, "srnum"), srcid, NumofR,
                                     MAXSwp, dx, dz, nrows, ncols, pe, C.addressof(EE)), "Radjoint_fsm2d")
    return EE.value


# ------------------------------------------------------------ batched layer
def _opts(precision, maxswp, max_batch, polish_floor=0.0, schedule=0, near_source_radius=0, tile_shape=0):
    o = _capi.Options()
    o.precision = int(precision)
    o.maxswp = int(maxswp)
    o.max_batch = int(max_batch)
    o.polish_floor = float(polish_floor)
    o.schedule = int(schedule)
    o.near_source_radius = int(near_source_radius)
    o.tile_shape = int(tile_shape)
    return o


class Context:
    """A device context: one CUDA stream and the reusable device work buffers."""

    def __init__(self, device=0):
        self._h = C.c_void_p()
        check(lib().pfast_ctx_create(device, C.byref(self._h)), "ctx_create")
        self.device = device

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_handle):
        """Run on a cudaStream_t (an int handle, e.g. torch.cuda.current_stream().cuda_stream); None = own stream."""
        check(lib().pfast_ctx_set_stream(self._h, C.c_void_p(stream_handle) if stream_handle else None), "set_stream")

    def set_graphs(self, enabled):
        """Replay per-diagonal outer iterations (3D and 2D) as CUDA graphs (default) or launch one by one."""
        check(lib().pfast_ctx_set_graphs(self._h, 1 if enabled else 0), "set_graphs")

    def synchronize(self):
        check(lib().pfast_ctx_synchronize(self._h), "synchronize")

    def close(self):
        if self._h:
            lib().pfast_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _dev_ptr(t, name, dtype_name="float64", numel=None):
    if not getattr(t, "is_cuda", False):
        raise TypeError(f"{name}: expected a CUDA tensor")
    if str(t.dtype) != f"torch.{dtype_name}" or not t.is_contiguous():
        raise TypeError(f"{name}: expected a contiguous {dtype_name} CUDA tensor")
    if numel is not None and t.numel() < numel:
        raise ValueError(f"{name}: needs {numel} elements, has {t.numel()}")
    return t.data_ptr()


class Survey3D:
    """3D acquisition geometry + picks resident on the device.

    src: int32 [nsrc, 3] (row, col, z) node indices; srnum: int32 [nsrc];
    rec: int32 [sum(srnum), 3]; nxyz: float64 [sum(srnum), 3] (n_y, n_x, n_z);
    tobs: float64 [sum(srnum)] (rows with tobs >= 100 are not picked).
    """

    def __init__(self, ctx, nrows, ncols, nz, dx, dy, dz, src, srnum, rec, nxyz=None, tobs=None):
        self.ctx = ctx
        self.shape = (nz, nrows, ncols)
        self.nsrc = len(srnum)
        self.nrec = int(np.asarray(srnum).sum())
        src = np.ascontiguousarray(src, np.int32)
        srnum = np.ascontiguousarray(srnum, np.int32)
        rec = np.ascontiguousarray(rec, np.int32)
        self._keep = [src, srnum, rec]
        nx = tx = None
        if nxyz is not None:
            nx = np.ascontiguousarray(nxyz, np.float64)
            tx = np.ascontiguousarray(tobs, np.float64)
            self._keep += [nx, tx]
        self._h = C.c_void_p()
        check(lib().pfast_survey3d_create(ctx.handle, nrows, ncols, nz, dx, dy, dz, self.nsrc, src.ctypes.data,
                                          srnum.ctypes.data, rec.ctypes.data, nx.ctypes.data if nx is not None else None,
                                          tx.ctypes.data if tx is not None else None, C.byref(self._h)),
              "survey3d_create")

    def eval(self, vp, grad=None, precision=PFAST_PLAIN_FP64, maxswp=100, max_batch=0, polish_floor=0.0, schedule=0,
             near_source_radius=0, tile_shape=0):
        """Misfit + gradient for the device model vp (torch float64 [nz, nrows, ncols]).
        schedule / tile_shape: 0 automatic, else as pfast_options.  Returns (grad tensor,
        misfit, stats dict)."""
        import torch
        n = int(np.prod(self.shape))
        if grad is None:
            grad = torch.empty(self.shape, dtype=torch.float64, device=vp.device)
        E = C.c_double(0)
        st = _capi.Stats()
        o = _opts(precision, maxswp, max_batch, polish_floor, schedule, near_source_radius, tile_shape)
        check(lib().pfast_survey3d_eval(self.ctx.handle, self._h, _dev_ptr(vp, "vp", numel=n), C.byref(o),
                                        _dev_ptr(grad, "grad", numel=n), C.addressof(E), C.byref(st)), "survey3d_eval")
        return grad, E.value, st.as_dict()

    def autotune(self, vp, precision=PFAST_MIXED, maxswp=100):
        """Time every (schedule, tile shape) candidate on this survey and model
        (pfast_survey3d_autotune); later automatic evaluations of this grid and source count
        use, per sweep phase, the fastest one.  Returns {candidate name: stats}."""
        n = len(_capi.PFAST_TUNE_CANDIDATES)
        sts = (_capi.Stats * n)()
        o = _opts(precision, maxswp, 0)
        check(lib().pfast_survey3d_autotune(self.ctx.handle, self._h, _dev_ptr(vp, "vp", numel=int(np.prod(self.shape))),
                                            C.byref(o), sts), "survey3d_autotune")
        return {name: sts[c].as_dict() for c, name in enumerate(_capi.PFAST_TUNE_CANDIDATES)}

    def forward(self, vp, picks=None, precision=PFAST_PLAIN_FP64, maxswp=100, max_batch=0, polish_floor=0.0,
                schedule=0, near_source_radius=0, tile_shape=0):
        """First-arrival picks [sum(srnum)] for the device model vp.  Returns (picks, stats)."""
        import torch
        n = int(np.prod(self.shape))
        if picks is None:
            picks = torch.empty(max(self.nrec, 1), dtype=torch.float64, device=vp.device)
        st = _capi.Stats()
        o = _opts(precision, maxswp, max_batch, polish_floor, schedule, near_source_radius, tile_shape)
        check(lib().pfast_survey3d_forward(self.ctx.handle, self._h, _dev_ptr(vp, "vp", numel=n), C.byref(o),
                                           _dev_ptr(picks, "picks", numel=self.nrec), C.byref(st)), "survey3d_forward")
        return picks[:self.nrec], st.as_dict()

    def close(self):
        if self._h:
            lib().pfast_survey3d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Survey2D:
    """2D geometry, picks and reflectors resident on the device.

    src: int32 [nsrc, 2] (row, col); rec: int32 [nrec, 2]; nxy: float64 [nrec, 2] (n_z, n_x);
    tt_obs: float64 [nrec]; tr_obs: float64 [nrec, numofr]; Z: float64 [numofr*ncols, 3].
    """

    def __init__(self, ctx, nrows, ncols, dx, dz, src, srnum, rec, numofr=0, Z=None, nxy=None, tt_obs=None,
                 tr_obs=None):
        self.ctx = ctx
        self.shape = (nrows, ncols)
        self.numofr = numofr
        self.nsrc = len(srnum)
        src = np.ascontiguousarray(src, np.int32)
        srnum = np.ascontiguousarray(srnum, np.int32)
        rec = np.ascontiguousarray(rec, np.int32)
        self.nrec = int(rec.shape[0])
        arrs = [src, srnum, rec]
        ptr = lambda a: a.ctypes.data if a is not None else None
        Zc = np.ascontiguousarray(Z, np.float64) if (Z is not None and numofr) else None
        nx = np.ascontiguousarray(nxy, np.float64) if nxy is not None else None
        tt = np.ascontiguousarray(tt_obs, np.float64) if tt_obs is not None else None
        tr = np.ascontiguousarray(tr_obs, np.float64) if (tr_obs is not None and numofr) else None
        self._keep = arrs + [Zc, nx, tt, tr]
        self._h = C.c_void_p()
        check(lib().pfast_survey2d_create(ctx.handle, nrows, ncols, dx, dz, self.nsrc, ptr(src), ptr(srnum),
                                          self.nrec, ptr(rec), ptr(nx), ptr(tt), numofr, ptr(tr), ptr(Zc),
                                          C.byref(self._h)), "survey2d_create")

    def forward(self, vp, precision=PFAST_PLAIN_FP64, maxswp=500, max_batch=0, near_source_radius=0):
        """Picks Tr [nrec, numofr+1] (transmission, then each reflector).  Returns (Tr, stats).
        near_source_radius > 0: opt-in straight-ray start of the nodes within that many nodes of
        each source (not in the reference)."""
        import torch
        n = self.shape[0] * self.shape[1]
        Tr = torch.zeros((max(self.nrec, 1), self.numofr + 1), dtype=torch.float64, device=vp.device)
        st = _capi.Stats()
        o = _opts(precision, maxswp, max_batch, near_source_radius=near_source_radius)
        check(lib().pfast_survey2d_forward(self.ctx.handle, self._h, _dev_ptr(vp, "vp", numel=n), C.byref(o),
                                           Tr.data_ptr(), C.byref(st)), "survey2d_forward")
        return Tr[:self.nrec], st.as_dict()

    def eval(self, vp, WR, precision=PFAST_PLAIN_FP64, maxswp=500, max_batch=0, near_source_radius=0):
        """Joint gradient.  Returns dict(gT, gR, gRT, Et, Er, stats)."""
        import torch
        n = self.shape[0] * self.shape[1]
        gT, gR, gRT = (torch.empty(self.shape, dtype=torch.float64, device=vp.device) for _ in range(3))
        Et, Er = C.c_double(0), C.c_double(0)
        st = _capi.Stats()
        o = _opts(precision, maxswp, max_batch, near_source_radius=near_source_radius)
        check(lib().pfast_survey2d_eval(self.ctx.handle, self._h, _dev_ptr(vp, "vp", numel=n),
                                        _dev_ptr(WR, "WR", numel=n), C.byref(o), gT.data_ptr(), gR.data_ptr(),
                                        gRT.data_ptr(), C.addressof(Et), C.addressof(Er), C.byref(st)),
              "survey2d_eval")
        return dict(gT=gT, gR=gR, gRT=gRT, Et=Et.value, Er=Er.value, stats=st.as_dict())

    def close(self):
        if self._h:
            lib().pfast_survey2d_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def eval3d_many(ctx, surveys, vps, grads=None, precision=PFAST_PLAIN_FP64, maxswp=100, polish_floor=0.0,
                near_source_radius=0):
    """Misfit + gradient of many (Survey3D, device model) pairs at once (pfast_surveys3d_eval):
    every sweep phase of all pairs runs as one dataflow launch over their (model, source)
    instances.  Each pair's results equal Survey3D.eval on it alone.  Returns (list of gradient
    tensors, list of misfits, summed stats dict)."""
    import torch
    n = len(surveys)
    if len(vps) != n:
        raise ValueError("one model per survey")
    if grads is None:
        grads = [torch.empty(sv.shape, dtype=torch.float64, device=vp.device) for sv, vp in zip(surveys, vps)]
    hs = (C.c_void_p * max(n, 1))(*[sv._h.value for sv in surveys])
    vs = (C.c_void_p * max(n, 1))(*[_dev_ptr(vp, "vp", numel=int(np.prod(sv.shape))) for sv, vp in zip(surveys, vps)])
    gs = (C.c_void_p * max(n, 1))(*[_dev_ptr(g, "grad", numel=int(np.prod(sv.shape))) for sv, g in zip(surveys, grads)])
    E = np.zeros(max(n, 1))
    st = _capi.Stats()
    o = _opts(precision, maxswp, 0, polish_floor, 0, near_source_radius)
    check(lib().pfast_surveys3d_eval(ctx.handle, n, C.addressof(hs), C.addressof(vs), C.addressof(gs), E.ctypes.data,
                                     C.byref(o), C.byref(st)), "surveys3d_eval")
    return grads, [float(e) for e in E[:n]], st.as_dict()


def eval3d_host(ctx, vp, dx, dy, dz, src, srnum, rec, nxyz, tobs, precision=PFAST_PLAIN_FP64, maxswp=100,
                max_batch=0, grad=None, polish_floor=0.0):
    """One-call host-buffer evaluation (pfast_eval3d): copies in, evaluates, copies the gradient out.
    vp: float64 [nz, nrows, ncols] host array.  Returns (grad, misfit, stats)."""
    nz, nr, nc = vp.shape
    if grad is None:
        grad = np.empty_like(vp)
    src = np.ascontiguousarray(src, np.int32)
    srnum = np.ascontiguousarray(srnum, np.int32)
    rec = np.ascontiguousarray(rec, np.int32)
    nxyz = np.ascontiguousarray(nxyz, np.float64)
    tobs = np.ascontiguousarray(tobs, np.float64)
    E = C.c_double(0)
    st = _capi.Stats()
    o = _opts(precision, maxswp, max_batch, polish_floor)
    check(lib().pfast_eval3d(ctx.handle, _arr(vp, np.float64, "vp"), nr, nc, nz, dx, dy, dz, len(srnum),
                             src.ctypes.data, srnum.ctypes.data, rec.ctypes.data, nxyz.ctypes.data, tobs.ctypes.data,
                             C.byref(o), _arr(grad, np.float64, "grad", True), C.addressof(E), C.byref(st)), "eval3d")
    return grad, E.value, st.as_dict()


def forward3d_host(ctx, vp, dx, dy, dz, src, srnum, rec, precision=PFAST_PLAIN_FP64, maxswp=100, max_batch=0):
    nz, nr, nc = vp.shape
    src = np.ascontiguousarray(src, np.int32)
    srnum = np.ascontiguousarray(srnum, np.int32)
    rec = np.ascontiguousarray(rec, np.int32)
    picks = np.empty(max(int(srnum.sum()), 1))
    st = _capi.Stats()
    o = _opts(precision, maxswp, max_batch)
    check(lib().pfast_forward3d(ctx.handle, _arr(vp, np.float64, "vp"), nr, nc, nz, dx, dy, dz, len(srnum),
                                src.ctypes.data, srnum.ctypes.data, rec.ctypes.data, C.byref(o), picks.ctypes.data,
                                C.byref(st)), "forward3d")
    return picks[:int(srnum.sum())], st.as_dict()


# ------------------------------------------------------------ inversion loop
def invert_options(dim, **kw):
    """pfast_invert_options with the reference driver's defaults for `dim` (2 or 3), overridden by
    keywords: precision, maxswp, max_batch (gradient evaluations), schemetag, lsrc, LM,
    max_linesearch, rttag, nux, nuy, nuz, minv, maxv, conv_tol, keep_components."""
    o = _capi.InvertOptions()
    lib().pfast_invert_default_options(int(dim), C.byref(o))
    for k, v in kw.items():
        if k in ("precision", "maxswp", "max_batch"):
            setattr(o.eval, k, int(v))
        elif k in dict(_capi.InvertOptions._fields_):
            setattr(o, k, v)
        else:
            raise TypeError(f"unknown inversion option {k!r}")
    return o


class Inversion:
    """The outer inversion loop on the device (pfast_inversion*).

    Inversion(survey, vp, WR=None, **options): survey is a Survey2D (WR required, float64
    [nrows, ncols]) or a Survey3D; vp is the starting model as a float64 host array.  step()
    runs one iteration and returns the report the reference prints (misfits, the line-search
    rows (alpha0, alpha1, phi0, phi1, dphi0, dphi1), the step size, convergence).  step()
    raises PfastError with status PFAST_ERR_OVER_CORRECTED where the reference aborts with
    "Over corrected"; the updated model is still readable."""

    FIELDS = dict(vp=_capi.PFAST_INV_VP, grad_raw=_capi.PFAST_INV_GRAD_RAW, grad=_capi.PFAST_INV_GRAD,
                  direction=_capi.PFAST_INV_DIRECTION, gR_raw=_capi.PFAST_INV_GR_RAW, gR=_capi.PFAST_INV_GR,
                  gT_raw=_capi.PFAST_INV_GT_RAW, gT=_capi.PFAST_INV_GT)

    def __init__(self, survey, vp, WR=None, **options):
        self.survey = survey
        self.ctx = survey.ctx
        self.shape = tuple(survey.shape)
        dim = len(self.shape)
        self.options = invert_options(dim, **options)
        vp = np.ascontiguousarray(vp, np.float64).reshape(self.shape)
        self._h = C.c_void_p()
        if dim == 2:
            if WR is None:
                raise ValueError("a 2D inversion needs WR")
            wr = np.ascontiguousarray(np.broadcast_to(np.asarray(WR, np.float64), self.shape))
            check(lib().pfast_inversion2d_create(self.ctx.handle, survey._h, vp.ctypes.data, wr.ctypes.data,
                                                 C.byref(self.options), C.byref(self._h)), "inversion2d_create")
        else:
            check(lib().pfast_inversion3d_create(self.ctx.handle, survey._h, vp.ctypes.data, C.byref(self.options),
                                                 C.byref(self._h)), "inversion3d_create")
        self.history = []

    def resume(self, k, grad_prev, grad_cur, E_hist, alpha1):
        """T_PFAST3D's resume: k iterations done, the next step uses grad_cur (unregularised) and
        grad_prev, the misfit history E_hist and the last step length alpha1."""
        gp = np.ascontiguousarray(grad_prev, np.float64).reshape(self.shape)
        gc = np.ascontiguousarray(grad_cur, np.float64).reshape(self.shape)
        eh = np.ascontiguousarray(E_hist, np.float64)
        check(lib().pfast_inversion_resume(self._h, int(k), gp.ctypes.data, gc.ctypes.data, eh.ctypes.data, len(eh),
                                           float(alpha1)), "inversion_resume")
        self.history = [None] * int(k)

    def step(self):
        rep = _capi.InvertReport()
        st = lib().pfast_inversion_step(self._h, C.byref(rep))
        d = rep.as_dict()
        self.history.append(d)
        check(st, "inversion_step")
        return d

    def run(self, max_iter):
        """Iterate until check_conv stops the loop or max_iter iterations ran (MAXIter)."""
        out = []
        while len(self.history) < max_iter:
            d = self.step()
            out.append(d)
            if d["converged"]:
                break
        return out

    def get(self, field="vp"):
        a = np.empty(self.shape)
        check(lib().pfast_inversion_get(self._h, self.FIELDS[field], a.ctypes.data), "inversion_get")
        return a

    def close(self):
        if self._h:
            lib().pfast_inversion_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------ request server
class Server:
    """Continuous-batching request server (pfast_server_*): models and surveys resident on the
    device under IDs, forward and gradient requests of any size admitted against an HBM budget
    and run `slots` at a time on their own streams.

        srv = Server(device=0, slots=4, hbm_budget_gb=150)
        srv.put_model(1, vp3d, (dx, dy, dz))             # 3D: vp [nz, nrows, ncols]
        srv.put_survey3d(7, shape, spacing, src, srnum, rec, nxyz, tobs)
        t = srv.submit_gradient(1, 7)                     # returns a Ticket
        grad, misfit, info = t.result()
    """

    def __init__(self, device=0, slots=4, hbm_budget_gb=150.0, max_bypass=8):
        cfg = _capi.ServerConfig(device=device, slots=slots, hbm_budget_bytes=float(hbm_budget_gb) * 1e9,
                                 max_bypass=max_bypass)
        self._h = C.c_void_p()
        check(lib().pfast_server_create(C.byref(cfg), C.byref(self._h)), "server_create")
        self._shapes = {}     # model id -> (dim, shape); survey id -> (dim, nrec, numofr)
        self._surveys = {}

    def put_model(self, model_id, vp, spacing, WR=None):
        vp = np.ascontiguousarray(vp, np.float64)
        dim = vp.ndim
        if dim == 3:
            nz, nr, nc = vp.shape
            dx, dy, dz = spacing
        else:
            nr, nc = vp.shape
            nz = 1
            dx, dz = spacing
            dy = 0.0
        wr = None if WR is None else np.ascontiguousarray(np.broadcast_to(np.asarray(WR, np.float64), vp.shape))
        check(lib().pfast_server_put_model(self._h, int(model_id), dim, nr, nc, nz, dx, dy, dz, vp.ctypes.data,
                                           wr.ctypes.data if wr is not None else None), "server_put_model")
        self._shapes[int(model_id)] = (dim, vp.shape)

    def put_survey3d(self, survey_id, shape, spacing, src, srnum, rec, nxyz=None, tobs=None):
        nz, nr, nc = shape
        dx, dy, dz = spacing
        a = [np.ascontiguousarray(src, np.int32), np.ascontiguousarray(srnum, np.int32),
             np.ascontiguousarray(rec, np.int32)]
        nx = None if nxyz is None else np.ascontiguousarray(nxyz, np.float64)
        tx = None if tobs is None else np.ascontiguousarray(tobs, np.float64)
        check(lib().pfast_server_put_survey3d(self._h, int(survey_id), nr, nc, nz, dx, dy, dz, len(a[1]),
                                              a[0].ctypes.data, a[1].ctypes.data, a[2].ctypes.data,
                                              nx.ctypes.data if nx is not None else None,
                                              tx.ctypes.data if tx is not None else None), "server_put_survey3d")
        self._surveys[int(survey_id)] = (3, int(a[1].sum()), 0)

    def put_survey2d(self, survey_id, shape, spacing, src, srnum, rec, numofr=0, Z=None, nxy=None, tt_obs=None,
                     tr_obs=None):
        nr, nc = shape
        dx, dz = spacing
        src = np.ascontiguousarray(src, np.int32)
        srnum = np.ascontiguousarray(srnum, np.int32)
        rec = np.ascontiguousarray(rec, np.int32)
        ptr = lambda x: None if x is None else x.ctypes.data
        Zc = np.ascontiguousarray(Z, np.float64) if (Z is not None and numofr) else None
        nx = None if nxy is None else np.ascontiguousarray(nxy, np.float64)
        tt = None if tt_obs is None else np.ascontiguousarray(tt_obs, np.float64)
        tr = np.ascontiguousarray(tr_obs, np.float64) if (tr_obs is not None and numofr) else None
        check(lib().pfast_server_put_survey2d(self._h, int(survey_id), nr, nc, dx, dz, len(srnum), ptr(src), ptr(srnum),
                                              len(rec), ptr(rec), ptr(nx), ptr(tt), numofr, ptr(tr), ptr(Zc)),
              "server_put_survey2d")
        self._surveys[int(survey_id)] = (2, len(rec), numofr)

    def drop_model(self, model_id):
        check(lib().pfast_server_drop(self._h, 0, int(model_id)), "server_drop")

    def drop_survey(self, survey_id):
        check(lib().pfast_server_drop(self._h, 1, int(survey_id)), "server_drop")

    def _submit(self, kind, model_id, survey_id, precision, maxswp, polish_floor, out):
        dim, shape = self._shapes.get(int(model_id), (3, None))   # unknown IDs: the library rejects them
        req = _capi.Request(kind=kind, model_id=int(model_id), survey_id=int(survey_id))
        req.opt = _opts(precision, maxswp if maxswp else (100 if dim == 3 else 500), 0, polish_floor)
        misfit = np.zeros(1)
        req.out = out.ctypes.data
        req.out_misfit = misfit.ctypes.data
        t = C.c_longlong()
        check(lib().pfast_server_submit(self._h, C.byref(req), C.byref(t)), "server_submit")
        return Ticket(self, t.value, kind, out, misfit)

    def submit_forward(self, model_id, survey_id, precision=PFAST_MIXED, maxswp=0, polish_floor=0.0):
        dim, nrec, numofr = self._surveys.get(int(survey_id), (3, 1, 0))
        out = np.empty((max(nrec, 1), numofr + 1) if dim == 2 else max(nrec, 1))
        return self._submit(_capi.PFAST_REQ_FORWARD, model_id, survey_id, precision, maxswp, polish_floor, out)

    def submit_gradient(self, model_id, survey_id, precision=PFAST_MIXED, maxswp=0, polish_floor=0.0):
        out = np.empty(self._shapes.get(int(model_id), (3, (1,)))[1])
        return self._submit(_capi.PFAST_REQ_GRADIENT, model_id, survey_id, precision, maxswp, polish_floor, out)

    def stats(self):
        st = _capi.ServerStats()
        check(lib().pfast_server_stats_get(self._h, C.byref(st)), "server_stats")
        return st.as_dict()

    def close(self):
        if self._h:
            lib().pfast_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Ticket:
    """A submitted request; result() blocks until it is done and returns (output, misfit, info)."""

    def __init__(self, server, ticket, kind, out, misfit):
        self.server, self.ticket, self.kind, self._out, self._misfit = server, ticket, kind, out, misfit
        self._res = None

    def result(self):
        if self._res is None:
            r = _capi.RequestResult()
            st = lib().pfast_server_wait(self.server._h, self.ticket, C.byref(r))
            self._res = r.as_dict()
            check(st, "server request")
        return self._out, (float(self._misfit[0]) if self.kind == _capi.PFAST_REQ_GRADIENT else None), self._res
