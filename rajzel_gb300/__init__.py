"""rajzel_gb300 -- GB300-native forward + adjoint Eikonal engine for RAJZEL.

Python mirror of the C ABI in ``include/rajzel_gb300.h`` (ctypes over the
in-tree ``librajzel_gb300.so``).  Names follow the reference's C entry points:

    ctx = Context(device=0)
    ctx.set_grid(nx, ny, dh, time, ttnorm, eps_adj)     # the reference globals
    ctx.set_velocity(vp)  or  ctx.set_slowness(S)       # calc_S.c
    ctx.set_receivers(recx, recz)                       # 1-based grid indices
    TT, Tmod, passes = ctx.eikonal(srcx, srcz)          # eikonal()
    lam, passes = ctx.eikonal_adj(TT, Tres)             # eikonal_adj()
    TT, Tmod, passes = ctx.forward(srcx[], srcz[])      # forward()
    grad, L2 = ctx.grad_obj(srcx[], srcz[], Tobs)       # grad_obj()

Fields are numpy float32 arrays shaped [ny][nx] (row-major, x fastest), the
memory order of the reference's NR matrices.  There is no CPU fallback: the
CUDA library must be built (``python -m rajzel_gb300.build``) and a CUDA
device present, or the calls raise.
"""
from __future__ import annotations

import collections
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "librajzel_gb300.so")

RZ_OK, RZ_EINVAL, RZ_ENOCONV, RZ_ECUDA, RZ_ENOMEM, RZ_ETIMEOUT, RZ_ESTATE, RZ_EUNSUPPORTED = range(8)
RZ_MODE_REFERENCE, RZ_MODE_FAST, RZ_MODE_FP64 = 0, 1, 2
RZ_DEVICE_PTRS = 1
RZ_GRADIENT_REFERENCE, RZ_GRADIENT_EXACT = 0, 1

class RajzelError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dh", C.c_float), ("time", C.c_float),
                ("ttnorm", C.c_float), ("eps_adj", C.c_float), ("max_passes", C.c_int)]


class ErrorReport(C.Structure):
    """rz_error: a float result's error against the FP64 oracle on the same inputs."""
    _fields_ = [("shots", C.c_int), ("tt_rel", C.c_double), ("tt_rel_l2", C.c_double), ("tmod_rel", C.c_double),
                ("grad_rel_l2", C.c_double),
                ("grad_rel_max", C.c_double), ("misfit_rel", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def load_library(path: str = LIB_PATH):
    """Load the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m rajzel_gb300.build`")
    lib = C.CDLL(path)
    vp = C.c_void_p
    lib.rz_abi_version.restype = C.c_int
    lib.rz_strerror.restype = C.c_char_p
    lib.rz_strerror.argtypes = [C.c_int]
    lib.rz_create.argtypes = [C.POINTER(vp), C.c_int]
    lib.rz_destroy.argtypes = [vp]
    lib.rz_destroy.restype = None
    lib.rz_last_error.argtypes = [vp]
    lib.rz_last_error.restype = C.c_char_p
    lib.rz_set_stream.argtypes = [vp, vp]
    lib.rz_set_mode.argtypes = [vp, C.c_int]
    lib.rz_set_grid.argtypes = [vp, C.POINTER(_Grid)]
    lib.rz_set_slowness.argtypes = [vp, vp, C.c_int]
    lib.rz_set_velocity.argtypes = [vp, vp, C.c_int]
    lib.rz_set_receivers.argtypes = [vp, C.c_int, vp, vp]
    lib.rz_forward.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, C.c_int]
    lib.rz_grad_obj.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, C.c_int]
    lib.rz_shot_info.argtypes = [vp, C.c_int, vp, vp, vp]
    lib.rz_shot_fields.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int]
    lib.rz_eikonal.argtypes = [vp, C.c_float, C.c_float, vp, vp, vp, C.c_int]
    lib.rz_shot_timeline.argtypes = [vp, C.c_int, vp]
    lib.rz_kernel_stats.argtypes = [vp, vp, vp, vp]
    lib.rz_eikonal_adj.argtypes = [vp, vp, vp, vp, vp, C.c_int]
    lib.rz_set_memory_cap.argtypes = [vp, C.c_size_t]
    lib.rz_shot_work.argtypes = [vp, C.c_int, vp, vp]
    lib.rz_set_graphs.argtypes = [vp, C.c_int]
    lib.rz_autotune.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp]
    lib.rz_grad_obj_multi.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp, C.c_int]
    lib.rz_fatt_defaults.argtypes = [vp]
    lib.rz_fatt.argtypes = [vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    lib.rz_misfit.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int]
    lib.rz_precond.argtypes = [vp, vp, vp, C.c_int]
    lib.rz_set_gradient.argtypes = [vp, C.c_int]
    lib.rz_backward.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int]
    lib.rz_status_code.argtypes = [C.c_int]
    lib.rz_status_code.restype = C.c_int
    lib.rz_batch_status.argtypes = [vp, vp]
    lib.rz_batch_status.restype = C.c_int
    lib.rz_tuned_shape.argtypes = [vp, C.c_int, vp, vp, vp]
    lib.rz_tuned_shape.restype = C.c_int
    lib.rz_set_refine.argtypes = [vp, C.c_int]
    lib.rz_set_refine.restype = C.c_int
    lib.rz_set_wait_test.argtypes = [vp, C.c_uint, C.c_int]
    lib.rz_set_wait_test.restype = C.c_int
    lib.rz_forward_f64.argtypes = [vp, C.c_int, vp, vp, vp, vp, C.c_int]
    lib.rz_grad_obj_f64.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp, C.c_int]
    lib.rz_set_error_check.argtypes = [vp, C.c_int]
    lib.rz_error_report.argtypes = [vp, vp]
    for name in ("rz_forward_f64", "rz_grad_obj_f64", "rz_set_error_check", "rz_error_report", "rz_set_memory_cap", "rz_shot_work", "rz_set_graphs", "rz_autotune", "rz_grad_obj_multi", "rz_fatt_defaults", "rz_fatt", "rz_precond", "rz_misfit", "rz_set_gradient", "rz_backward", "rz_create", "rz_set_stream", "rz_set_mode", "rz_set_grid", "rz_set_slowness", "rz_set_velocity",
                 "rz_set_receivers", "rz_forward", "rz_grad_obj", "rz_shot_info", "rz_shot_fields", "rz_eikonal",
                 "rz_eikonal_adj", "rz_shot_timeline", "rz_kernel_stats"):
        getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def grad_obj_multi(ctxs, srcx, srcz, Tobs):
    """rz_grad_obj_multi: one persistent launch over the shots of several
    contexts (one grid each); returns [(grad, L2)] per context."""
    n = len(ctxs)
    lib = ctxs[0].lib
    sx = [_f32(a) for a in srcx]
    sz = [_f32(a) for a in srcz]
    tob = [_f32(t).reshape(len(sx[i]), ctxs[i].ntr) if ctxs[i].ntr else np.zeros((len(sx[i]), 1), np.float32)
           for i, t in enumerate(Tobs)]
    grads = [np.empty((c.ny, c.nx), np.float32) for c in ctxs]
    P = C.c_void_p * n
    handles = P(*[c.h.value for c in ctxs])
    ns = (C.c_int * n)(*[len(a) for a in sx])
    L2 = (C.c_double * n)()
    st = lib.rz_grad_obj_multi(n, handles, ns, P(*[a.ctypes.data for a in sx]), P(*[a.ctypes.data for a in sz]),
                               P(*[a.ctypes.data for a in tob]), P(*[g.ctypes.data for g in grads]), L2, 0)
    ctxs[0]._check(st, "rz_grad_obj_multi")
    return [(grads[i], L2[i]) for i in range(n)]


class FattOpts(C.Structure):
    """rz_fatt_opts: the reference's FATT parameters (RAJZEL .inp / workflow names)."""
    _fields_ = [("itermax", C.c_int), ("nlbfgs", C.c_int), ("stepmax", C.c_int), ("eps_scale", C.c_float),
                ("c1", C.c_float), ("c2", C.c_float), ("scalefac", C.c_float), ("vp_lo", C.c_float),
                ("vp_hi", C.c_float), ("pro", C.c_float), ("spatfilter", C.c_int), ("filt_size_grad", C.c_int),
                ("filt_size_grad1", C.c_int), ("taper_hor", C.c_int), ("gradt1", C.c_int), ("gradt2", C.c_int),
                ("exp_taper_grad_hor", C.c_float), ("recursion", C.c_int)]


FattResult = collections.namedtuple("FattResult", "vp misfit iterations evaluations steps")


def fatt_opts(**kw):
    """rz_fatt_defaults() with keyword overrides (field names of rz_fatt_opts)."""
    o = FattOpts()
    load_library().rz_fatt_defaults(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One GPU engine instance (owns device buffers and a CUDA stream)."""

    def __init__(self, device: int = 0, mode: str = "reference"):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.rz_create(C.byref(h), int(device))
        if st != RZ_OK:
            raise RajzelError(st, f"rz_create(device={device}) failed: {self.lib.rz_strerror(st).decode()}")
        self.h = h
        self.nx = self.ny = 0
        self.ntr = 0
        self.set_mode(mode)

    # -- plumbing -----------------------------------------------------------
    def _check(self, st, what):
        if st != RZ_OK:
            msg = self.lib.rz_last_error(self.h).decode(errors="replace")
            raise RajzelError(st, f"{what}: {self.lib.rz_strerror(st).decode()}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.lib.rz_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_handle: int | None):
        self._check(self.lib.rz_set_stream(self.h, C.c_void_p(stream_handle or 0)), "rz_set_stream")

    def set_mode(self, mode):
        m = {"reference": RZ_MODE_REFERENCE, "fast": RZ_MODE_FAST, "fp64": RZ_MODE_FP64}.get(mode, mode)
        self._check(self.lib.rz_set_mode(self.h, int(m)), "rz_set_mode")
        self.mode = m

    # -- configuration (the reference's globals, model, receivers) ----------
    def set_grid(self, nx, ny, dh, time, ttnorm=1e-6, eps_adj=1e-9, max_passes=10000):
        g = _Grid(int(nx), int(ny), float(dh), float(time), float(ttnorm), float(eps_adj), int(max_passes))
        self._check(self.lib.rz_set_grid(self.h, C.byref(g)), "rz_set_grid")
        self.nx, self.ny = int(nx), int(ny)

    def set_slowness(self, S):
        S = _f32(S)
        assert S.size == self.nx * self.ny
        self._check(self.lib.rz_set_slowness(self.h, _ptr(S), 0), "rz_set_slowness")

    def set_velocity(self, vp):
        vp = _f32(vp)
        assert vp.size == self.nx * self.ny
        self._check(self.lib.rz_set_velocity(self.h, _ptr(vp), 0), "rz_set_velocity")

    def set_receivers(self, recx, recz):
        recx, recz = _i32(recx), _i32(recz)
        self._check(self.lib.rz_set_receivers(self.h, len(recx), _ptr(recx), _ptr(recz)), "rz_set_receivers")
        self.ntr = len(recx)

    def set_gradient(self, kind: str):
        """'reference' (Leung-Qian, the reference's gradient) or 'exact' (dJ/dVp of the discrete misfit)."""
        k = {"reference": RZ_GRADIENT_REFERENCE, "exact": RZ_GRADIENT_EXACT}[kind]
        self._check(self.lib.rz_set_gradient(self.h, k), "rz_set_gradient")

    def backward(self, srcx, srcz, dTmod):
        """sum over shots of (dTmod/dVp)^T dTmod: the vector-Jacobian product of the forward map."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        dTmod = _f32(dTmod).reshape(n, self.ntr) if self.ntr else np.zeros((n, 1), np.float32)
        grad = np.empty((self.ny, self.nx), np.float32)
        self._check(self.lib.rz_backward(self.h, n, _ptr(srcx), _ptr(srcz), _ptr(dTmod), _ptr(grad), 0),
                    "rz_backward")
        return grad

    def fatt(self, srcx, srcz, Tobs, vp, opts=None, **kw):
        """FATT stage (rz_fatt): returns FattResult(vp, misfit, iterations, evaluations, steps)."""
        o = opts if opts is not None else fatt_opts(**kw)
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        Tobs = _f32(Tobs).reshape(n, self.ntr) if self.ntr else np.zeros((n, 1), np.float32)
        model = _f32(vp).reshape(self.ny, self.nx).copy()
        mis = np.zeros(max(o.itermax, 1), np.float64)
        steps = np.zeros(max(o.itermax, 1), np.float32)
        it, ev = C.c_int(0), C.c_int(0)
        self._check(self.lib.rz_fatt(self.h, C.byref(o), n, _ptr(srcx), _ptr(srcz), _ptr(Tobs), _ptr(model),
                                     _ptr(mis), _ptr(steps), C.byref(it), C.byref(ev)), "rz_fatt")
        return FattResult(model, mis[: it.value], it.value, ev.value, steps[: it.value])

    def misfit(self, srcx, srcz, Tobs):
        """0.5 * sum (Tmod - Tobs)^2 over unmuted picks (rz_misfit: forward solves only)."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        Tobs = _f32(Tobs).reshape(n, self.ntr) if self.ntr else np.zeros((n, 1), np.float32)
        L2 = C.c_double(0.0)
        self._check(self.lib.rz_misfit(self.h, n, _ptr(srcx), _ptr(srcz), _ptr(Tobs), C.byref(L2), 0), "rz_misfit")
        return L2.value

    def precond(self, grad, opts=None, **kw):
        """precond() on one gradient (rz_precond): Gaussian filter and horizontal taper."""
        o = opts if opts is not None else fatt_opts(**kw)
        g = _f32(grad).reshape(self.ny, self.nx).copy()
        self._check(self.lib.rz_precond(self.h, C.byref(o), _ptr(g), 0), "rz_precond")
        return g

    def autotune(self, srcx, srcz, Tobs):
        """rz_autotune on this batch: {'warps': best, 'ms': time, 'candidates': {warps: ms}}."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        Tobs = _f32(Tobs).reshape(n, self.ntr) if self.ntr else np.zeros((n, 1), np.float32)
        grad = np.empty((self.ny, self.nx), np.float32)
        best, ms = C.c_int(0), C.c_double(0.0)
        cw, cm, nc = (C.c_int * 8)(), (C.c_double * 8)(), C.c_int(8)
        self._check(self.lib.rz_autotune(self.h, n, _ptr(srcx), _ptr(srcz), _ptr(Tobs), _ptr(grad), 0, C.byref(best),
                                         C.byref(ms), cw, cm, C.byref(nc)), "rz_autotune")
        w, cta, rows = C.c_int(0), C.c_int(0), C.c_int(0)
        self._check(self.lib.rz_tuned_shape(self.h, n, C.byref(w), C.byref(cta), C.byref(rows)), "rz_tuned_shape")
        return {"warps": best.value, "ms": ms.value, "candidates": {cw[i]: cm[i] for i in range(min(nc.value, 8))},
                "shape": {"sweeping_warps": w.value, "cta_warps": cta.value or "widest", "check_rows": rows.value}}

    def set_graphs(self, enable: bool):
        """Capture rz_grad_obj's device sequence as a CUDA graph and replay it (default on)."""
        self._check(self.lib.rz_set_graphs(self.h, int(bool(enable))), "rz_set_graphs")

    def set_memory_cap(self, nbytes: int):
        """Bytes of device memory the per-shot field slots may use (0 = automatic)."""
        self._check(self.lib.rz_set_memory_cap(self.h, int(nbytes)), "rz_set_memory_cap")

    # -- the hot path -------------------------------------------------------
    def eikonal(self, srcx, srcz):
        TT = np.empty((self.ny, self.nx), np.float32)
        Tmod = np.empty(max(self.ntr, 1), np.float32)
        p = C.c_int(0)
        self._check(self.lib.rz_eikonal(self.h, float(srcx), float(srcz), _ptr(TT), _ptr(Tmod), C.byref(p), 0),
                    "rz_eikonal")
        return TT, Tmod[: self.ntr], p.value

    def eikonal_adj(self, TT, Tres):
        TT = _f32(TT)
        Tres = _f32(Tres) if self.ntr else np.zeros(1, np.float32)
        lam = np.empty((self.ny, self.nx), np.float32)
        p = C.c_int(0)
        self._check(self.lib.rz_eikonal_adj(self.h, _ptr(TT), _ptr(Tres), _ptr(lam), C.byref(p), 0), "rz_eikonal_adj")
        return lam, p.value

    def forward(self, srcx, srcz, want_tt=True):
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        TT = np.empty((n, self.ny, self.nx), np.float32) if want_tt else None
        Tmod = np.empty((n, max(self.ntr, 1)), np.float32)
        passes = np.zeros(n, np.int32)
        self._check(self.lib.rz_forward(self.h, n, _ptr(srcx), _ptr(srcz), _ptr(TT), _ptr(Tmod), _ptr(passes), 0),
                    "rz_forward")
        return TT, Tmod[:, : self.ntr], passes

    def grad_obj(self, srcx, srcz, Tobs, out=None):
        """Misfit and stacked gradient (host buffers); `out`, if given, is a
        C-contiguous float32 [ny][nx] array that receives the gradient."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        Tobs = _f32(Tobs).reshape(n, self.ntr)
        if out is not None:
            if out.dtype != np.float32 or out.shape != (self.ny, self.nx) or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous float32 array of shape (ny, nx)")
            grad = out
        else:
            grad = np.empty((self.ny, self.nx), np.float32)
        L2 = C.c_double(0.0)
        self._check(self.lib.rz_grad_obj(self.h, n, _ptr(srcx), _ptr(srcz), _ptr(Tobs), _ptr(grad), C.byref(L2), 0),
                    "rz_grad_obj")
        return grad, L2.value

    def forward_device(self, srcx, srcz, tt_ptr: int = 0, tmod_ptr: int = 0):
        """Asynchronous forward on device buffers (RZ_DEVICE_PTRS): TT
        [n][ny][nx] and Tmod [n][ntr] float32, either may be 0."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        self._check(self.lib.rz_forward(self.h, len(srcx), _ptr(srcx), _ptr(srcz), C.c_void_p(tt_ptr or None),
                                        C.c_void_p(tmod_ptr or None), None, RZ_DEVICE_PTRS), "rz_forward(device)")

    def grad_obj_device(self, srcx, srcz, tobs_ptr: int, grad_ptr: int, l2_ptr: int):
        """Asynchronous variant on device buffers (RZ_DEVICE_PTRS): Tobs
        [n][ntr] float32, grad [ny][nx] float32, L2 one float64."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        self._check(self.lib.rz_grad_obj(self.h, len(srcx), _ptr(srcx), _ptr(srcz), C.c_void_p(tobs_ptr),
                                         C.c_void_p(grad_ptr), C.c_void_p(l2_ptr), RZ_DEVICE_PTRS),
                    "rz_grad_obj(device)")

    # -- the FP64 oracle and the error of float results ----------------------
    def forward_f64(self, srcx, srcz, want_tt=True):
        """FP64 oracle traveltimes [n][ny][nx] (or None) and picks [n][ntr], float64."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        TT = np.empty((n, self.ny, self.nx), np.float64) if want_tt else None
        Tmod = np.empty((n, max(self.ntr, 1)), np.float64)
        self._check(self.lib.rz_forward_f64(self.h, n, _ptr(srcx), _ptr(srcz), _ptr(TT), _ptr(Tmod), 0),
                    "rz_forward_f64")
        return TT, Tmod[:, : self.ntr]

    def grad_obj_f64(self, srcx, srcz, Tobs):
        """FP64 oracle gradient [ny][nx] (float64) and misfit of the context's gradient kind."""
        srcx, srcz = _f32(srcx), _f32(srcz)
        n = len(srcx)
        Tobs = _f32(Tobs).reshape(n, self.ntr)
        grad = np.empty((self.ny, self.nx), np.float64)
        L2 = C.c_double(0.0)
        self._check(self.lib.rz_grad_obj_f64(self.h, n, _ptr(srcx), _ptr(srcz), _ptr(Tobs), _ptr(grad),
                                             C.byref(L2), 0), "rz_grad_obj_f64")
        return grad, L2.value

    def set_error_check(self, enable: bool):
        """Later float calls also run the FP64 oracle and record their error (error_report)."""
        self._check(self.lib.rz_set_error_check(self.h, int(bool(enable))), "rz_set_error_check")

    def error_report(self):
        """Error of the last checked call against the FP64 oracle, as a dict (rz_error)."""
        e = ErrorReport()
        self._check(self.lib.rz_error_report(self.h, C.byref(e)), "rz_error_report")
        return e.as_dict()

    def set_refine(self, enable: bool):
        """Refine converged traveltimes to the FP64 fixpoint (rz_set_refine)."""
        self._check(self.lib.rz_set_refine(self.h, int(bool(enable))), "rz_set_refine")

    def set_wait_test(self, spin_limit: int = 0, withhold_handoff: bool = False):
        """Test hook of the timeout path (rz_set_wait_test)."""
        self._check(self.lib.rz_set_wait_test(self.h, int(spin_limit), int(bool(withhold_handoff))),
                    "rz_set_wait_test")

    def batch_status(self):
        """OR of the device status bits of every shot of the last batch (waits for the stream)."""
        b = C.c_int(0)
        self._check(self.lib.rz_batch_status(self.h, C.byref(b)), "rz_batch_status")
        return b.value

    def shot_info(self, shot):
        a, b, s = C.c_int(0), C.c_int(0), C.c_int(0)
        self._check(self.lib.rz_shot_info(self.h, int(shot), C.byref(a), C.byref(b), C.byref(s)), "rz_shot_info")
        return a.value, b.value, s.value

    def shot_work(self, shot):
        """(forward, adjoint) directional sweeps actually run for one shot of the last batch."""
        a, b = C.c_int(0), C.c_int(0)
        self._check(self.lib.rz_shot_work(self.h, int(shot), C.byref(a), C.byref(b)), "rz_shot_work")
        return a.value, b.value

    def kernel_stats(self):
        """(kernels launched so far, summed shot-kernel ms since the last call, shot-kernel calls)."""
        n, ms, calls = C.c_longlong(0), C.c_double(0), C.c_int(0)
        self._check(self.lib.rz_kernel_stats(self.h, C.byref(n), C.byref(ms), C.byref(calls)), "rz_kernel_stats")
        return n.value, ms.value, calls.value

    def shot_timeline(self, shot):
        """Device time stamps (ns) of one shot of the last batch (see rz_shot_timeline)."""
        out = np.zeros(8, np.uint64)
        self._check(self.lib.rz_shot_timeline(self.h, int(shot), _ptr(out)), "rz_shot_timeline")
        return out

    def shot_fields(self, shot):
        TT = np.empty((self.ny, self.nx), np.float32)
        lam = np.empty((self.ny, self.nx), np.float32)
        Tres = np.empty(max(self.ntr, 1), np.float32)
        self._check(self.lib.rz_shot_fields(self.h, int(shot), _ptr(TT), _ptr(lam), _ptr(Tres), 0), "rz_shot_fields")
        return TT, lam, Tres[: self.ntr]
