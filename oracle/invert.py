"""CPU restatement of PFAST's inversion loop (TEST INFRASTRUCTURE ONLY): the checker
for the library's inversion entry points (pfast_inversion2d_create / 3d / _step).

Follows the outer loop of src/RT_PFAST2D.cpp:412-816 (2D) and src/T_PFAST3D.cpp:359-656
(3D) with the helpers of src/RT_padjoint2d.h:475-646 and src/T_padjoint3d.h:174-342:
the FFT low-pass regularisation regu2d / regu3d, magnitudeOf, the L-BFGS pair store
gd2sk and two-loop recursion, the HS / CG_DESCENT betas, the line searches (lsrc 1
secant "exact", 2 secant strong Wolfe, 3 cubic, 0 none), updatevp and check_conv.
Gradients come from oracle.port (np = 1 source order).  The FFT is numpy's (the
reference links the vendored fftn.c); the two agree to rounding, so this oracle
agrees with the reference to ~1e-12 relative, not bit for bit.

Pinned against the iteration traces the reference printed for its 2D example
(par/RT_SynMod2D_Inv_RT.out, _Trans.out, _Ref.out): residuals and line-search values
to the 6 digits printed.

Deliberate deviation: the first L-BFGS loop of the reference subtracts ai[i] * yk
where ai[i % LM] was just computed (src/RT_PFAST2D.cpp:529, src/T_PFAST3D.cpp:468);
the two agree while Iterk - 2 < LM, after that the reference reads past ai's end.
ai[i % LM] is used.
"""
import math

import numpy as np

from . import port

PI = 3.141592653589793   # PI macro, src/T_pfsm3d.h:25


class OverCorrected(RuntimeError):
    """check_conv's "Over corrected..abort..." (src/RT_padjoint2d.h:489-490)."""


def _kvec(n, d):
    """k of regu2d / regu3d (src/RT_padjoint2d.h:520-529): -kmax + ks*j, then entry j and
    entry n/2 + j swapped for j < n/2."""
    kmax, ks = PI / d, 2 * PI / n / d
    k = np.array([-kmax + ks * j for j in range(n)])
    h = n // 2
    a = k[:h].copy()
    k[:h] = k[h:2 * h]
    k[h:2 * h] = a
    return k


def regu(D, vp, nus, ds):
    """regu2d / regu3d (src/RT_padjoint2d.h:506-547, src/T_padjoint3d.h:208-260):
    D / (1 + nux^2 kx^2 + nuy^2 ky^2 [+ nuz^2 kz^2]) in the wavenumber domain, real part of
    the inverse transform, zero where vp == 330 (water).
    D, vp: (nrows, ncols) or (nz, nrows, ncols).  nus, ds: per axis, fastest (columns) first:
    2D (nux, nuz), (dx, dz); 3D (nux, nuy, nuz), (dx, dy, dz)."""
    F = np.fft.fftn(D)
    den = np.ones(D.shape)
    for a, (nu, d) in enumerate(zip(nus, ds)):       # the reference's term order: columns first
        ax = D.ndim - 1 - a
        k = _kvec(D.shape[ax], d)
        shape = [1] * D.ndim
        shape[ax] = -1
        den = den + ((nu * nu * k) * k).reshape(shape)
    F = F / den
    R = np.fft.ifftn(F).real
    return np.where(np.abs(vp - 330) < 1e-9, 0.0, R)


def magnitude_of(g):
    """magnitudeOf (src/RT_padjoint2d.h:631-637)."""
    return 1.0 / np.max(np.abs(g))


def cubic_interp(a0, a1, p0, p1, d0, d1):
    """cubicInterp (src/RT_padjoint2d.h:619-630).  Raises where the reference falls off the
    end of the function without a return value."""
    a = (-2. * (p1 - p0) + (d0 + d1) * (a1 - a0)) / ((a1 - a0) * (a1 - a0) * (a1 - a0))
    b = (3. * (p1 - p0) - (2. * d0 + d1) * (a1 - a0)) / ((a1 - a0) * (a1 - a0))
    c = d0
    if abs(a) > 0 and (b * b - 3 * a * c) > 0:
        return a0 + (-b + math.sqrt(b * b - 3 * a * c)) / (3. * a)
    if a == 0 and abs(b) > 0 and (b * b - 3 * a * c) < 0:
        return -c / (2. * b)
    raise RuntimeError("cubicInterp: no value for these arguments")


class Loop:
    """State and one outer iteration of the drivers' loop.  `grad(model)` returns
    (g, E, phi, Et, Er): the gradient the loop uses (per RTtag), the joint misfit stored in
    global_E, the misfit the line search compares (per RTtag), and the two parts (None in 3D).
    `regu(g)` regularises with the CURRENT model's water mask."""

    def __init__(self, vp, grad, nus, ds, dim, schemetag=3, lsrc=2, LM=5, max_linesearch=None,
                 minv=None, maxv=None, conv_tol=None):
        self.vp = np.array(vp, dtype=np.float64, copy=True)
        self.grad, self.nus, self.ds, self.dim = grad, nus, ds, dim
        self.schemetag, self.lsrc, self.LM = schemetag, lsrc, LM
        self.max_ls = max_linesearch or (5 if dim == 2 else 2)      # MAXLineSch
        self.minv = minv if minv is not None else (1600.0 if dim == 2 else 1400.0)   # MINV / MAXV
        self.maxv = maxv if maxv is not None else (4500.0 if dim == 2 else 8000.0)
        self.conv_tol = conv_tol if conv_tol is not None else (1e-3 if dim == 2 else 1e-2)
        n = self.vp.size
        self.Djk1 = np.zeros(n)
        self.dk = np.zeros(n)
        self.sk = np.zeros((LM, n))
        self.yk = np.zeros((LM, n))
        self.rho = np.zeros(LM)
        self.ai = np.zeros(LM)
        self.alpha0, self.alpha1 = 0.0, 5.0e3
        self.c1, self.c2 = 1.0e-4, 0.9
        self.globalE = []
        self.it = 0
        self.converged = False

    def _regu(self, g):
        return regu(g.reshape(self.vp.shape), self.vp, self.nus, self.ds).ravel()

    def _eval(self, model):
        g, E, phi, Et, Er = self.grad(model.reshape(self.vp.shape))
        return g.ravel(), E, phi, Et, Er

    def _lbfgs(self, Djk0):
        """gd2sk (src/RT_padjoint2d.h:590-604) and the two-loop recursion (src/RT_PFAST2D.cpp:520-546)."""
        LM, it, g1 = self.LM, self.it, self.Djk1
        y = -g1 + Djk0
        dTy = np.sum(self.alpha1 * self.dk * y)
        gamma = dTy / np.sum(y * y)
        slot = (it - 2) % LM
        self.rho[slot] = 1.0 / dTy
        self.sk[slot] = self.alpha1 * self.dk
        self.yk[slot] = y
        q = g1.copy()
        lo = it - LM - 1 if it - LM - 1 >= 0 else 0
        for i in range(it - 2, lo - 1, -1):
            m = i % LM
            self.ai[m] = np.sum(self.rho[m] * self.sk[m] * q)
            q = q - self.ai[m] * self.yk[m]
        d = gamma * q
        for i in range(lo, it - 1):
            m = i % LM
            tmp = np.sum(self.rho[m] * self.yk[m] * d)
            d = d + self.sk[m] * (self.ai[m] - tmp)
        return d

    def resume(self, k, grad_prev, grad_cur, E_hist, alpha1):
        """T_PFAST3D's resume (src/T_PFAST3D.cpp:346-385): k iterations done; the next step uses
        grad_cur unregularised as its gradient, grad_prev as the previous gradient and direction."""
        self.it = k
        self.Djk1 = np.array(grad_prev, dtype=np.float64).ravel()
        self.dk = self.Djk1.copy()
        self.globalE = list(E_hist[:k + 1])
        self.alpha1 = alpha1
        self._resume = np.array(grad_cur, dtype=np.float64).ravel()

    def step(self):
        """One "Iterating No. k".  Returns the record the reference prints."""
        self.it += 1
        it = self.it
        Djk0 = self.Djk1.copy()
        if getattr(self, "_resume", None) is not None:
            self.Djk1, self._resume = self._resume, None
            rec = dict(iter=it, E=self.globalE[it - 1], trials=[], count=0, stopped=False)
        else:
            g, E, _, Et, Er = self._eval(self.vp)
            self.globalE.append(E)
            rec = dict(iter=it, E=E, Et=Et, Er=Er, grad_raw=g.copy(), trials=[], count=0, stopped=False)
            self.Djk1 = self._regu(g)
            if self.schemetag == 3:
                if it == 1:
                    self.alpha1 = 5e2 * magnitude_of(self.Djk1)
            else:
                self.alpha1 = 5e2 * magnitude_of(self.Djk1)
        g1 = self.Djk1
        if it == 1:
            self.dk = g1.copy()
        elif self.schemetag == 1:         # beta_HS, src/RT_padjoint2d.h:560-571
            beta = np.sum(g1 * (g1 - Djk0)) / np.sum(-self.dk * (g1 - Djk0))
            self.dk = g1 + self.dk * beta
            self.c1, self.c2 = 1.0e-4, 0.1
        elif self.schemetag == 2:         # beta_CGDESCENT, src/RT_padjoint2d.h:573-588
            dTy = np.sum(self.dk * (-g1 + Djk0))
            ny = np.sum((-g1 + Djk0) * (-g1 + Djk0))
            beta = np.sum(((-g1 + Djk0) - 2 * self.dk * ny / dTy) * (-g1) / dTy)
            self.dk = g1 + self.dk * beta
            self.c1, self.c2 = 1.0e-4, 0.1
        elif self.schemetag == 3:
            self.dk = self._lbfgs(Djk0)
            self.alpha0, self.alpha1 = 0.0, 1.0
            self.c1, self.c2 = 1.0e-4, 0.9
        else:
            raise ValueError("Numerical Optimization Method Unknown")
        rec["alpha_start"] = self.alpha1
        vp, dk = self.vp.ravel(), self.dk
        if self.lsrc == 1:               # src/RT_PFAST2D.cpp:563-615
            count, self.alpha0 = 0, 0.0
            f0 = 0.0
            while True:
                a0, a1 = self.alpha0, self.alpha1
                with np.errstate(divide="ignore", invalid="ignore"):
                    go = abs(a1 - a0) / abs(a0) > 1e-2 if a0 != 0 else (a1 != a0)
                if not go:
                    break
                count += 1
                if count - 1 >= self.max_ls:
                    break
                g1t, _, _, _, _ = self._eval(vp + self.alpha1 * dk)
                Dj1 = self._regu(g1t)
                f0 = 0.0
                f1 = np.sum(Dj1 * dk)
                alphak = self.alpha1 - (self.alpha1 - self.alpha0) * f1 / (f1 - f0)
                self.alpha0, self.alpha1 = self.alpha1, alphak
                f0 = f1
            rec["count"] = count
            rec["stopped"] = count > self.max_ls
        elif self.lsrc in (2, 3):
            phi0 = self.globalE[it - 1]
            dphi0 = np.sum(-dk * self.Djk1)
            self.alpha0 = 0.0
            loop = self.lsrc == 2 or self.schemetag == 3 or self.dim == 3
            count = 0
            wolfe = False
            while True:
                if not loop and count == 1:
                    break
                if wolfe:
                    break
                count += 1
                if count - 1 >= self.max_ls:
                    break
                g1t, _, phi1, _, _ = self._eval(vp + self.alpha1 * dk)
                Dj1 = self._regu(g1t)
                dphi1 = np.sum(-dk * Dj1)
                a_tried = self.alpha1
                if not loop:         # one interpolation, no count kept (src/RT_PFAST2D.cpp:752-806)
                    self.alpha1 = cubic_interp(self.alpha0, self.alpha1, phi0, phi1, dphi0, dphi1)
                    rec["trials"].append((self.alpha0, self.alpha1, phi0, phi1, dphi0, dphi1))
                    count = 0
                    break
                if phi1 <= phi0 + self.c1 * self.alpha1 * dphi0 and abs(dphi1) <= -self.c2 * dphi0:
                    wolfe = True
                elif self.lsrc == 2:
                    self.alpha1 = self.alpha1 - (self.alpha1 - self.alpha0) * dphi1 / (dphi1 - dphi0)
                else:
                    self.alpha1 = cubic_interp(self.alpha0, self.alpha1, phi0, phi1, dphi0, dphi1)
                shown = a_tried if self.lsrc == 2 else self.alpha1   # lsrc 3 prints after the update
                rec["trials"].append((self.alpha0, shown, phi0, phi1, dphi0, dphi1))
            rec["count"] = count
            rec["stopped"] = bool(loop and count > self.max_ls)
        elif self.lsrc != 0:
            raise ValueError("Line search tag unknown")
        rec["stepsize"] = self.alpha1
        # updatevp, src/RT_padjoint2d.h:497-505
        free = np.abs(vp - 330) > 1e-9
        vnew = vp + self.alpha1 * dk
        vnew = np.where(vnew > self.maxv, self.maxv, vnew)
        vnew = np.where(vnew < self.minv, self.minv, vnew)
        self.vp = np.where(free, vnew, vp).reshape(self.vp.shape)
        # check_conv, src/RT_padjoint2d.h:475-495
        chgE = (self.globalE[it - 2] - self.globalE[it - 1]) / self.globalE[it - 2] if it >= 2 else 1.0
        if chgE <= self.conv_tol:
            self.converged = True
        else:
            v = self.vp.ravel()
            mynorm = math.sqrt(np.max(self.alpha1 * self.alpha1 * dk * dk / v / v))
            if mynorm / v.size >= 1:
                raise OverCorrected("Over corrected")
        rec["converged"] = self.converged
        return rec


def loop2d(vp, WR, Z, src, srnum, rec, nxy, TT, TR, numofr, dx, dz, nux, nuz, rttag=3, maxswp=500,
           nthreads=8, **kw):
    """The 2D loop of RT_PFAST2D (RTtag 3 joint, 1 transmission, 2 reflection)."""
    def grad(model):
        r = port.eval2d(model, WR, Z, src, srnum, rec, nxy, TT, TR, numofr, maxswp, dx, dz, nthreads=nthreads)
        E = r["Er"] + r["Et"]                                   # loc_E = loc_Er + loc_Et
        g, phi = {3: (r["gRT"], E), 1: (r["gT"], r["Et"]), 2: (r["gR"], r["Er"])}[rttag]
        return g, E, phi, r["Et"], r["Er"]
    return Loop(vp, grad, (nux, nuz), (dx, dz), 2, **kw)


def loop3d(vp, src, srnum, rec, nxyz, tobs, dx, dy, dz, nux, nuy, nuz, maxswp=100, nthreads=8, **kw):
    """The 3D loop of T_PFAST3D (schemetag forced to 3 after the first gradient, src/T_PFAST3D.cpp:428)."""
    def grad(model):
        g, E, _, _ = port.eval3d(model, src, srnum, rec, nxyz, tobs, maxswp, dx, dy, dz, nthreads=nthreads)
        return g, E, E, None, None
    kw.setdefault("schemetag", 3)
    return Loop(vp, grad, (nux, nuy, nuz), (dx, dy, dz), 3, **kw)
