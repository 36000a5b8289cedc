"""CPU restatement of one RAJZEL FATT stage, the checker of the GPU loop.

TEST INFRASTRUCTURE ONLY: imported by tests and never by the product.

Follows fatt.c:108-258 (iteration loop and stopping rule), descent.c,
LBFGS.c:36-165 (history pairs, gamma, rho, the two-loop recursion in slot
order), check_descent.c (history reset), wolfels.c:16-110 (weak-Wolfe step
search), calc_mat_change_wolfe.c:28-50 (model update with hard limits),
precond.c:12-58 with gauss_filt.c:14-141 (SPATFILTER 4) and the horizontal
taper of taper_grad.c:118-193, and util.c's maximum_m (signed maximum).

Two precisions.  precision="gpu" (the default) follows the GPU loop it
checks: dot products and recursion scalars in double, vectors float32 with
each update computed in double and rounded once.  precision="reference"
follows the reference operation by operation: float dot products summed in
x-outer order (dotp.c, dotp_matrix.c), float recursion scalars and model
updates (LBFGS.c, wolfels.c, calc_mat_change_wolfe.c), the misfit compared as
the float wolfels.c keeps it; tests pin that mode to the reference's own
compiled fatt().  The Gaussian filter here is the reference's direct 2-D
convolution, accumulated in double.  The gradient is the oracle's grad_obj
(the reference's own float arithmetic, pinned to it).
"""
from __future__ import annotations

import math

import numpy as np

from . import Params, grad_obj

F32, F64 = np.float32, np.float64


def _opt(o, name):
    return o[name] if isinstance(o, dict) else getattr(o, name)


def gauss_filt(g, filt_size_grad, filt_size_grad1):
    """gauss_filt.c:14-141: 2-D Gaussian with edge-replicated borders."""
    fs, fs1 = int(filt_size_grad), int(filt_size_grad1)
    if fs == 0 or fs1 == 0:
        return g.astype(F32, copy=True)
    if fs % 2 == 0:
        fs += 1 if fs > 0 else -1
    if fs1 % 2 == 0:
        fs1 += 1 if fs1 > 0 else -1
    hfx, hfy = abs(fs) // 2, abs(fs1) // 2
    sigx, sigy = F32(hfx // 2), F32(hfy // 2)  # integer division, as the reference
    sx, sy = F32(2.0) * sigx * sigx, F32(2.0) * sigy * sigy
    ii = np.arange(-hfx, hfx + 1)[None, :]
    jj = np.arange(-hfy, hfy + 1)[:, None]
    kern = np.exp(-(ii * ii) / F64(sx) - (jj * jj) / F64(sy))
    kern = kern / kern.sum()
    ny, nx = g.shape
    ext = np.pad(g.astype(F64), ((hfy, hfy), (hfx, hfx)), mode="edge")
    out = np.zeros((ny, nx), F64)
    for a in range(2 * hfy + 1):
        for b in range(2 * hfx + 1):
            out += kern[a, b] * ext[a:a + ny, b:b + nx]
    return out.astype(F32)


def taper_hor_coeff(ny, dh, gradt1, gradt2, expo):
    """taper_grad.c:118-172 (sws 2): per-row coefficients, rows 1-based."""
    tl, ifw = gradt2 - gradt1, gradt2 - gradt1 + 1
    win = np.ones(max(ifw, 1) + 1, F32)
    a = F32(3.0)
    for i in range(1, ifw + 1):
        if i <= tl:
            x = float(a * F32(i - tl)) / (tl / 2.0)
            win[i] = F32(math.exp(-(1.0 / 2.0) * x * x))
    coef = np.zeros(ny, F32)
    h = 1
    for j in range(1, ny + 1):
        tap = F32(0.0)
        if gradt1 <= j <= gradt2 and h <= ifw:
            tap = win[h]
        if j > gradt2:
            tap = F32(math.pow(float(F32(j) * F32(dh)), float(F32(expo))))
        coef[j - 1] = tap
        if j >= gradt1:
            h += 1
    return coef


def precond(g, o, dh):
    """precond.c:12-58 with SPATFILTER 4 and the horizontal taper."""
    out = g.astype(F32, copy=True)
    if _opt(o, "spatfilter") == 4:
        out = gauss_filt(out, _opt(o, "filt_size_grad"), _opt(o, "filt_size_grad1"))
    if _opt(o, "taper_hor"):
        coef = taper_hor_coeff(out.shape[0], dh, _opt(o, "gradt1"), _opt(o, "gradt2"), _opt(o, "exp_taper_grad_hor"))
        out = (out * coef[:, None]).astype(F32)
    return out


def _step(vp, h, step, lo, hi):
    """calc_mat_change_wolfe.c:28-50 (the step taken in double)."""
    v = (vp.astype(F64) + F64(F32(step)) * h.astype(F64)).astype(F32)
    bad = (v < F32(lo)) | (v > F32(hi)) | (v < F32(0.0))
    return np.where(bad, vp, v).astype(F32)


def _dot(a, b):
    return float(np.dot(a.astype(F64).ravel(), b.astype(F64).ravel()))


def _dot_ref(a, b):
    """dotp.c / dotp_matrix.c: float products summed one by one in a float,
    x outer (cells of one column after another)."""
    prod = (np.asarray(a, F32).T * np.asarray(b, F32).T).ravel()
    return F32(np.cumsum(prod, dtype=F32)[-1]) if prod.size else F32(0.0)


def _step_ref(vp, h, step, lo, hi):
    """calc_mat_change_wolfe.c:28-50 in float."""
    v = (vp + F32(step) * np.asarray(h, F32)).astype(F32)
    bad = (v < F32(lo)) | (v > F32(hi)) | (v < F32(0.0))
    return np.where(bad, vp, v).astype(F32)


def _axpby(alpha, x, beta, y):
    if beta == 0.0:
        return (alpha * x.astype(F64)).astype(F32)
    return (alpha * x.astype(F64) + beta * y.astype(F64)).astype(F32)


def fatt(p: Params, vp0, srcx, srcz, recx, recz, Tobs, o, precision="gpu", trace=None):
    """One FATT stage; returns (vp, misfit per iteration, iterations, gradient
    evaluations).  trace, a list, receives the misfit of every gradient
    evaluation in call order."""
    if precision == "reference":
        return _fatt_reference(p, vp0, srcx, srcz, recx, recz, Tobs, o, trace)
    m = int(_opt(o, "nlbfgs"))
    itermax, stepmax = int(_opt(o, "itermax")), int(_opt(o, "stepmax"))
    c1, c2, scalefac = F32(_opt(o, "c1")), F32(_opt(o, "c2")), F32(_opt(o, "scalefac"))
    lo, hi, pro, eps_scale = _opt(o, "vp_lo"), _opt(o, "vp_hi"), _opt(o, "pro"), F32(_opt(o, "eps_scale"))
    slot_order = _opt(o, "recursion") == 0
    vp = np.asarray(vp0, F32).copy()
    evals = 0

    def gradient(model):
        nonlocal evals
        S = (1.0 / model.astype(F64)).astype(F32)  # calc_S.c:21
        g, L2, _, _, _ = grad_obj(p, S, srcx, srcz, recx, recz, Tobs)
        evals += 1
        if trace is not None:
            trace.append(L2)
        return L2, precond(g, o, p.dh)

    Y = [np.zeros_like(vp) for _ in range(m)]
    Sv = [np.zeros_like(vp) for _ in range(m)]
    rho, alpha = [0.0] * m, [0.0] * m
    vp_old = grad_old = None
    hist = []
    it, ptr, done_iters = 1, 0, 0
    while it <= itermax:
        if it > 2 and m > 0:
            ptr = (ptr + 1) % m
        L2, grad = gradient(vp)
        # LBFGS.c
        if it == 1:
            H = _axpby(-1.0, grad, 0.0, None)
        else:
            Y[ptr] = (grad - grad_old).astype(F32)
            Sv[ptr] = (vp - vp_old).astype(F32)
            ys, yy = _dot(Y[ptr], Sv[ptr]), _dot(Y[ptr], Y[ptr])
            gamma = ys / yy if yy != 0.0 else 0.0
            for k in range(m):
                d = _dot(Y[k], Sv[k])
                rho[k] = 1.0 / d if d != 0.0 else 0.0
            order = [m - 1 - i for i in range(m)] if slot_order else [(ptr - i) % m for i in range(m)]
            q = _axpby(-1.0, grad, 0.0, None)
            for k in order:
                alpha[k] = rho[k] * _dot(Sv[k], q)
                q = _axpby(-alpha[k], Y[k], 1.0, q)
            r = _axpby(gamma, q, 0.0, None)
            for k in reversed(order):
                beta = rho[k] * _dot(Y[k], r)
                r = _axpby(alpha[k] - beta, Sv[k], 1.0, r)
            H = r
        vp_old, grad_old = vp.copy(), grad.copy()
        # check_descent.c
        den = _dot(grad, grad)
        pdesc = -_dot(H, grad) / den if den != 0.0 else 0.0
        if pdesc < 0.0:
            Y = [np.zeros_like(vp) for _ in range(m)]
            Sv = [np.zeros_like(vp) for _ in range(m)]
        if _opt(o, "spatfilter") == 4:
            H = gauss_filt(H, _opt(o, "filt_size_grad"), _opt(o, "filt_size_grad1"))
        # wolfels.c
        if it == 1:
            a = F32(eps_scale * F32(vp.max()) / F32(H.max()))
        else:
            a = F32(1.0)
        a = F32(a / scalefac)
        mu, nu = F32(0.0), F32(1e30)
        lsiter = 0
        g0s0 = _dot(grad, H)
        while True:
            a = F32((nu + mu) / scalefac) if nu < F32(1e30) else F32(scalefac * a)
            if lsiter >= stepmax:
                a = F32(0.0)
                break
            ft, gt = gradient(_step(vp, H, a, lo, hi))
            lsiter += 1
            gts0 = _dot(gt, H)
            if ft > L2 + float(c1 * a) * g0s0:
                nu = a
            elif gts0 < float(c2) * g0s0:
                mu = a
            else:
                break
        hist.append(L2)
        vp = _step(vp, H, a, lo, hi)
        done_iters = it
        diff = abs((hist[it - 3] - hist[it - 1]) / hist[it - 3]) if it > 2 else 1e20
        if diff <= pro or a < F32(1e-10):
            break
        it += 1
    return vp, np.array(hist), done_iters, evals


def _fatt_reference(p, vp0, srcx, srcz, recx, recz, Tobs, o, trace):
    """fatt.c:96-258 with GRAD_METHOD 2 and LINESEARCH 1 in the reference's
    own float arithmetic (LBFGS.c:36-165 in slot order, check_descent.c,
    wolfels.c:28-100, calc_mat_change_wolfe.c)."""
    m = int(_opt(o, "nlbfgs"))
    itermax, stepmax = int(_opt(o, "itermax")), int(_opt(o, "stepmax"))
    c1, c2, scalefac = F32(_opt(o, "c1")), F32(_opt(o, "c2")), F32(_opt(o, "scalefac"))
    lo, hi, pro, eps_scale = _opt(o, "vp_lo"), _opt(o, "vp_hi"), _opt(o, "pro"), F32(_opt(o, "eps_scale"))
    vp = np.asarray(vp0, F32).copy()
    evals = 0

    def gradient(model):
        nonlocal evals
        S = (1.0 / model.astype(F64)).astype(F32)  # calc_S.c:21
        g, L2, _, _, _ = grad_obj(p, S, srcx, srcz, recx, recz, Tobs)
        evals += 1
        if trace is not None:
            trace.append(L2)
        return L2, precond(g, o, p.dh)

    Y = [np.zeros_like(vp) for _ in range(m)]
    Sv = [np.zeros_like(vp) for _ in range(m)]
    rho, alpha = [F32(0.0)] * m, [F32(0.0)] * m
    vp_old = grad_old = None
    hist, steps = [], []
    it, ptr, done_iters = 1, 0, 0
    while it <= itermax:
        if it > 2 and m > 0:
            ptr = (ptr + 1) % m
        L2, grad = gradient(vp)
        gradm = (-grad).astype(F32)
        if it == 1:
            H = gradm.copy()
        else:
            Y[ptr] = (grad - grad_old).astype(F32)
            Sv[ptr] = (vp - vp_old).astype(F32)
            gamma = F32(_dot_ref(Y[ptr], Sv[ptr]) / _dot_ref(Y[ptr], Y[ptr]))
            for k in range(m):
                d = _dot_ref(Y[k], Sv[k])
                rho[k] = F32(1.0 / float(d)) if abs(float(d)) > 0.0 else F32(0.0)
            q = gradm.copy()
            for k in range(m - 1, -1, -1):
                alpha[k] = F32(rho[k] * _dot_ref(Sv[k], q))
                q = (q - alpha[k] * Y[k]).astype(F32)
            r = (gamma * q).astype(F32)
            for k in range(m):
                beta = F32(rho[k] * _dot_ref(Y[k], r))
                r = (r + Sv[k] * F32(alpha[k] - beta)).astype(F32)
            H = r
        vp_old, grad_old = vp.copy(), grad.copy()
        pdesc = F32(-_dot_ref(H, grad) / _dot_ref(grad, grad))
        if pdesc < 0.0:
            Y = [np.zeros_like(vp) for _ in range(m)]
            Sv = [np.zeros_like(vp) for _ in range(m)]
        if _opt(o, "spatfilter") == 4:
            H = gauss_filt(H, _opt(o, "filt_size_grad"), _opt(o, "filt_size_grad1"))
        a = F32(F32(eps_scale * F32(vp.max())) / F32(H.max())) if it == 1 else F32(1.0)
        a = F32(a / scalefac)
        mu, nu = F32(0.0), F32(1e30)
        lsiter = 0
        while True:
            a = F32(F32(nu + mu) / scalefac) if float(nu) < 1e30 else F32(scalefac * a)
            if lsiter >= stepmax:
                a = F32(0.0)
                break
            ft, gt = gradient(_step_ref(vp, H, a, lo, hi))
            ft = F32(ft)
            lsiter += 1
            g0s0, gts0 = _dot_ref(grad, H), _dot_ref(gt, H)
            if float(ft) > L2 + float(F32(F32(c1 * a) * g0s0)):
                nu = a
            elif gts0 < F32(c2 * g0s0):
                mu = a
            else:
                break
        hist.append(L2)
        steps.append(a)
        vp = _step_ref(vp, H, a, lo, hi)
        done_iters = it
        diff = abs((hist[it - 3] - hist[it - 1]) / hist[it - 3]) if it > 2 else 1e20
        if diff <= pro or a < 1e-10:
            break
        it += 1
    return vp, np.array(hist), done_iters, evals
