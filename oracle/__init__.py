"""CPU oracles for RAJZEL's forward + adjoint Eikonal path.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline / reference arm, always as the checker or the
timed CPU baseline, never by the ``rajzel_gb300`` product.

Two libraries sit behind this module:

* ``librz_oracle.so`` -- ``rz_oracle.c``, this repository's C restatement of
  the reference algorithm (float variant bit-identical to the reference, plus
  an all-double variant that serves as the FP64 oracle).  Built everywhere.
* ``_ref/libref.so`` -- the reference's own C sources compiled unmodified
  (see ``Makefile``), built only where those sources are present.  It pins the
  restatement: tests check the two agree bit for bit.

All fields are flat row-major ``[ny][nx]`` float32/float64 numpy arrays; source
positions are metres (``srcpos[1]``/``srcpos[2]`` of the reference); receiver
positions are the reference's 1-based grid indices (``recpos[1]``/``recpos[2]``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "librz_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")


def _makefile_refsrc() -> str:
    """The reference source directory the build recipe (oracle/Makefile, REFSRC) names."""
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REFSRC"):
                return line.split("=", 1)[1].strip()
    return ""


# where the reference's sources are read from: RAJZEL_REFERENCE_SRC, else the recipe's default
REF_SRC = os.environ.get("RAJZEL_REFERENCE_SRC") or _makefile_refsrc()

RZO_OK, RZO_EINVAL, RZO_ENOCONV = 0, 1, 2


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dh", C.c_float), ("time", C.c_float),
                ("ttnorm", C.c_float), ("eps_adj", C.c_float), ("max_passes", C.c_int)]


def build(ref: bool = True, quiet: bool = True) -> None:
    """Compile the restatement (always) and the reference library (when its
    sources exist).  Each make target is a no-op when up to date."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "port"], check=True, stdout=out)
    if ref and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-C", HERE, "ref", f"REFSRC={REF_SRC}"], check=True, stdout=out)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_port = None
_ref = None


def _load_port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_SO):
            build(ref=False)
        lib = C.CDLL(PORT_SO)
        G = C.POINTER(_Grid)
        lib.rzo_eikonal.argtypes = [G, _f32p, C.c_float, C.c_float, _f32p, C.POINTER(C.c_int)]
        lib.rzo_eikonal_f64.argtypes = [G, _f64p, C.c_double, C.c_double, _f64p, C.POINTER(C.c_int)]
        lib.rzo_calc_fa.argtypes = [G, _f32p, C.c_int, _i32p, _i32p, _f32p]
        lib.rzo_calc_fa.restype = None
        lib.rzo_calc_res.argtypes = [G, _f32p, _f32p, _f32p, _f32p, C.c_int, _i32p, _i32p]
        lib.rzo_calc_res.restype = C.c_double
        lib.rzo_eikonal_adj.argtypes = [G, _f32p, _f32p, C.c_int, _i32p, _i32p, _f32p, C.POINTER(C.c_int)]
        lib.rzo_eikonal_adj_f64.argtypes = [G, _f64p, _f64p, C.c_int, _i32p, _i32p, _f64p, C.POINTER(C.c_int)]
        lib.rzo_ass_grad.argtypes = [G, _f32p, _f32p, _f32p]
        lib.rzo_ass_grad.restype = None
        lib.rzo_cp_grad_frame.argtypes = [G, _f32p]
        lib.rzo_cp_grad_frame.restype = None
        lib.rzo_grad_obj.argtypes = [G, _f32p, C.c_int, _f32p, _f32p, C.c_int, _i32p, _i32p, _f32p, _f32p,
                                     C.POINTER(C.c_double), C.c_void_p, C.c_void_p, C.c_void_p]
        lib.rzo_grad_obj_f64.argtypes = [G, _f64p, C.c_int, _f64p, _f64p, C.c_int, _i32p, _i32p, _f64p, _f64p,
                                         C.POINTER(C.c_double)]
        lib.rzo_shot_partition.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        lib.rzo_grad_exact_f64.argtypes = [G, _f64p, C.c_int, _f64p, _f64p, C.c_int, _i32p, _i32p, _f64p, _f64p,
                                           C.POINTER(C.c_double)]
        lib.rzo_misfit_f64.argtypes = [G, _f64p, C.c_int, _f64p, _f64p, C.c_int, _i32p, _i32p, _f64p,
                                       C.POINTER(C.c_double)]
        lib.rzo_shot_partition.restype = None
        _port = lib
    return _port


def _load_ref():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError("reference oracle not built (its sources are absent here)")
        lib = C.CDLL(REF_SO)
        lib.ref_set_params.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float]
        lib.ref_set_params.restype = None
        lib.ref_eikonal.argtypes = [_f32p, C.c_float, C.c_float, C.c_int, _i32p, _i32p, _f32p, _f32p]
        lib.ref_eikonal_adj.argtypes = [_f32p, _f32p, C.c_int, _i32p, _i32p, _f32p]
        lib.ref_calc_FA_res.argtypes = [_f32p, _f32p, _f32p, _f32p, C.c_int, _i32p, _i32p]
        lib.ref_calc_FA_res.restype = C.c_double
        lib.ref_grad_obj.argtypes = [_f32p, C.c_int, _f32p, _f32p, C.c_int, _i32p, _i32p, _f32p, _f32p,
                                     C.c_void_p, C.c_void_p]
        lib.ref_grad_obj.restype = C.c_double
        lib.ref_ass_grad.argtypes = [_f32p, _f32p, _f32p]
        lib.ref_ass_grad.restype = None
        lib.ref_cp_grad_frame.argtypes = [_f32p]
        lib.ref_cp_grad_frame.restype = None
        lib.ref_counter.argtypes = [C.c_int]
        lib.ref_counter.restype = C.c_long
        lib.ref_precond.argtypes = [_f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_float]
        lib.ref_precond.restype = None
        lib.ref_fatt_stage.argtypes = [_f32p, C.c_int, _f32p, _f32p, C.c_int, _i32p, _i32p, _f32p, C.c_int,
                                       C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                       C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_float, _f64p, _f32p]
        lib.ref_fatt_stage.restype = C.c_int
        lib.ref_evals.argtypes = [_f64p, C.c_int]
        lib.ref_evals.restype = C.c_int
        _ref = lib
    return _ref


class Params:
    """The reference's process globals that the hot path reads."""

    def __init__(self, nx, ny, dh, time, ttnorm=1e-6, eps_adj=1e-9, max_passes=1000):
        self.nx, self.ny = int(nx), int(ny)
        self.dh, self.time = float(dh), float(time)
        self.ttnorm, self.eps_adj = float(ttnorm), float(eps_adj)
        self.max_passes = int(max_passes)

    def grid(self):
        return _Grid(self.nx, self.ny, self.dh, self.time, self.ttnorm, self.eps_adj, self.max_passes)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _check(st, what):
    if st != RZO_OK:
        raise RuntimeError(f"oracle {what} failed with status {st}")


# --------------------------------------------------------------------------
# restatement ("port")
# --------------------------------------------------------------------------

def eikonal(p: Params, S, srcx, srcz):
    """Forward field (float, reference arithmetic).  Returns (TT, passes)."""
    lib = _load_port()
    S = _f32(S).reshape(-1)
    TT = np.empty(p.nx * p.ny, np.float32)
    it = C.c_int(0)
    _check(lib.rzo_eikonal(C.byref(p.grid()), S, srcx, srcz, TT, C.byref(it)), "eikonal")
    return TT.reshape(p.ny, p.nx), it.value


def eikonal_f64(p: Params, S, srcx, srcz):
    lib = _load_port()
    S = _f64(S).reshape(-1)
    TT = np.empty(p.nx * p.ny, np.float64)
    it = C.c_int(0)
    _check(lib.rzo_eikonal_f64(C.byref(p.grid()), S, srcx, srcz, TT, C.byref(it)), "eikonal_f64")
    return TT.reshape(p.ny, p.nx), it.value


def calc_fa(p: Params, TT, recx, recz):
    lib = _load_port()
    recx, recz = _i32(recx), _i32(recz)
    out = np.empty(len(recx), np.float32)
    lib.rzo_calc_fa(C.byref(p.grid()), _f32(TT).reshape(-1), len(recx), recx, recz, out)
    return out


def calc_res(p: Params, TT, Tmod, Tobs, recx, recz, Tres=None):
    lib = _load_port()
    recx, recz = _i32(recx), _i32(recz)
    Tres = np.zeros(len(recx), np.float32) if Tres is None else _f32(Tres).copy()
    l2 = lib.rzo_calc_res(C.byref(p.grid()), _f32(TT).reshape(-1), _f32(Tmod), _f32(Tobs), Tres, len(recx),
                          recx, recz)
    return Tres, l2


def eikonal_adj(p: Params, TT, Tres, recx, recz):
    lib = _load_port()
    recx, recz = _i32(recx), _i32(recz)
    lam = np.empty(p.nx * p.ny, np.float32)
    it = C.c_int(0)
    _check(lib.rzo_eikonal_adj(C.byref(p.grid()), _f32(TT).reshape(-1), _f32(Tres), len(recx), recx, recz, lam,
                               C.byref(it)), "eikonal_adj")
    return lam.reshape(p.ny, p.nx), it.value


def eikonal_adj_f64(p: Params, TT, Tres, recx, recz):
    lib = _load_port()
    recx, recz = _i32(recx), _i32(recz)
    lam = np.empty(p.nx * p.ny, np.float64)
    it = C.c_int(0)
    _check(lib.rzo_eikonal_adj_f64(C.byref(p.grid()), _f64(TT).reshape(-1), _f64(Tres), len(recx), recx, recz,
                                   lam, C.byref(it)), "eikonal_adj_f64")
    return lam.reshape(p.ny, p.nx), it.value


def grad_obj(p: Params, S, srcx, srcz, recx, recz, Tobs, Tres0=None):
    """Misfit + stacked gradient over all shots on one rank.
    Returns (grad, L2, fwd_passes, adj_passes, Tres_final)."""
    lib = _load_port()
    srcx, srcz = _f32(srcx), _f32(srcz)
    recx, recz = _i32(recx), _i32(recz)
    ns, ntr = len(srcx), len(recx)
    Tobs = _f32(Tobs).reshape(-1)
    assert Tobs.size == ns * ntr
    grad = np.empty(p.nx * p.ny, np.float32)
    L2 = C.c_double(0)
    Tres = np.zeros(ntr, np.float32) if Tres0 is None else _f32(Tres0).copy()
    fp = np.zeros(ns, np.int32)
    ap = np.zeros(ns, np.int32)
    _check(lib.rzo_grad_obj(C.byref(p.grid()), _f32(S).reshape(-1), ns, srcx, srcz, ntr, recx, recz, Tobs, grad,
                            C.byref(L2), Tres.ctypes.data, fp.ctypes.data, ap.ctypes.data), "grad_obj")
    return grad.reshape(p.ny, p.nx), L2.value, fp, ap, Tres


def grad_obj_f64(p: Params, S, srcx, srcz, recx, recz, Tobs):
    lib = _load_port()
    recx, recz = _i32(recx), _i32(recz)
    ns, ntr = len(srcx), len(recx)
    grad = np.empty(p.nx * p.ny, np.float64)
    L2 = C.c_double(0)
    _check(lib.rzo_grad_obj_f64(C.byref(p.grid()), _f64(S).reshape(-1), ns, _f64(srcx), _f64(srcz), ntr, recx,
                                recz, _f64(Tobs).reshape(-1), grad, C.byref(L2)), "grad_obj_f64")
    return grad.reshape(p.ny, p.nx), L2.value


def grad_exact_f64(p: Params, S, srcx, srcz, recx, recz, Tobs):
    """Exact discrete adjoint gradient dJ/dVp (FP64), J = 0.5 sum (Tmod-Tobs)^2."""
    lib = _load_port()
    recx, recz = _i32(recx), _i32(recz)
    ns, ntr = len(srcx), len(recx)
    grad = np.empty(p.nx * p.ny, np.float64)
    L2 = C.c_double(0)
    _check(lib.rzo_grad_exact_f64(C.byref(p.grid()), _f64(S).reshape(-1), ns, _f64(srcx), _f64(srcz), ntr, recx,
                                  recz, _f64(Tobs).reshape(-1), grad, C.byref(L2)), "grad_exact_f64")
    return grad.reshape(p.ny, p.nx), L2.value


def misfit_f64(p: Params, S, srcx, srcz, recx, recz, Tobs):
    """J = 0.5 sum (Tmod-Tobs)^2 over unmuted picks, FP64 forward."""
    lib = _load_port()
    recx, recz = _i32(recx), _i32(recz)
    L2 = C.c_double(0)
    _check(lib.rzo_misfit_f64(C.byref(p.grid()), _f64(S).reshape(-1), len(srcx), _f64(srcx), _f64(srcz), len(recx),
                              recx, recz, _f64(Tobs).reshape(-1), C.byref(L2)), "misfit_f64")
    return L2.value


def ass_grad(p: Params, grad, S, lam):
    lib = _load_port()
    g = _f32(grad).reshape(-1).copy()
    lib.rzo_ass_grad(C.byref(p.grid()), g, _f32(S).reshape(-1), _f32(lam).reshape(-1))
    return g.reshape(p.ny, p.nx)


def cp_grad_frame(p: Params, A):
    """cp_grad_frame.c:18-49 on a copy of A [ny][nx]."""
    lib = _load_port()
    a = _f32(A).reshape(-1).copy()
    lib.rzo_cp_grad_frame(C.byref(p.grid()), a)
    return a.reshape(p.ny, p.nx)


def shot_partition(nshots, np_, myid):
    lib = _load_port()
    a, b = C.c_int(0), C.c_int(0)
    lib.rzo_shot_partition(nshots, np_, myid, C.byref(a), C.byref(b))
    return a.value, b.value


# --------------------------------------------------------------------------
# the reference's own compiled code ("ref")
# --------------------------------------------------------------------------

class Ref:
    """Calls into the unmodified reference sources (only where built)."""

    def __init__(self, p: Params):
        self.p = p
        self.lib = _load_ref()
        self.lib.ref_set_params(p.nx, p.ny, p.dh, p.time, p.ttnorm, p.eps_adj)

    def eikonal(self, S, srcx, srcz, recx=(), recz=()):
        recx, recz = _i32(recx), _i32(recz)
        TT = np.empty(self.p.nx * self.p.ny, np.float32)
        Tmod = np.empty(max(len(recx), 1), np.float32)
        it = self.lib.ref_eikonal(_f32(S).reshape(-1), srcx, srcz, len(recx), recx, recz, TT, Tmod)
        return TT.reshape(self.p.ny, self.p.nx), Tmod[: len(recx)], it

    def eikonal_adj(self, TT, Tres, recx, recz):
        recx, recz = _i32(recx), _i32(recz)
        lam = np.empty(self.p.nx * self.p.ny, np.float32)
        it = self.lib.ref_eikonal_adj(_f32(TT).reshape(-1), _f32(Tres), len(recx), recx, recz, lam)
        return lam.reshape(self.p.ny, self.p.nx), it

    def calc_res(self, TT, Tmod, Tobs, recx, recz, Tres=None):
        recx, recz = _i32(recx), _i32(recz)
        Tres = np.zeros(len(recx), np.float32) if Tres is None else _f32(Tres).copy()
        l2 = self.lib.ref_calc_FA_res(_f32(TT).reshape(-1), _f32(Tmod), _f32(Tobs), Tres, len(recx), recx, recz)
        return Tres, l2

    def grad_obj(self, S, srcx, srcz, recx, recz, Tobs):
        recx, recz = _i32(recx), _i32(recz)
        grad = np.empty(self.p.nx * self.p.ny, np.float32)
        Tres = np.zeros(len(recx), np.float32)
        L2 = self.lib.ref_grad_obj(_f32(S).reshape(-1), len(srcx), _f32(srcx), _f32(srcz), len(recx), recx, recz,
                                   _f32(Tobs).reshape(-1), grad, None, Tres.ctypes.data)
        return grad.reshape(self.p.ny, self.p.nx), L2, Tres

    def ass_grad(self, grad, S, lam):
        g = _f32(grad).reshape(-1).copy()
        self.lib.ref_ass_grad(g, _f32(S).reshape(-1), _f32(lam).reshape(-1))
        return g.reshape(self.p.ny, self.p.nx)

    def cp_grad_frame(self, A):
        a = _f32(A).reshape(-1).copy()
        self.lib.ref_cp_grad_frame(a)
        return a.reshape(self.p.ny, self.p.nx)

    def precond(self, grad, o):
        """precond() of the reference (precond.c:12-58): SPATFILTER 4 and the
        horizontal taper as the options (an rz_fatt_opts-like dict) select."""
        g = _f32(grad).reshape(-1).copy()
        self.lib.ref_precond(g, int(o["spatfilter"]), int(o["filt_size_grad"]), int(o["filt_size_grad1"]),
                             int(o["taper_hor"]), int(o["gradt1"]), int(o["gradt2"]), float(o["exp_taper_grad_hor"]))
        return g.reshape(self.p.ny, self.p.nx)

    def fatt(self, vp0, srcx, srcz, recx, recz, Tobs, o):
        """One FATT stage by the reference's own fatt() (l-BFGS + weak Wolfe).
        Returns (vp, misfit per iteration, accepted step per iteration, the
        misfit of every gradient evaluation in call order)."""
        recx, recz = _i32(recx), _i32(recz)
        vp = _f32(vp0).reshape(-1).copy()
        n_it = int(o["itermax"])
        mis = np.zeros(n_it, np.float64)
        steps = np.zeros(n_it, np.float32)
        it = self.lib.ref_fatt_stage(vp, len(srcx), _f32(srcx), _f32(srcz), len(recx), recx, recz,
                                     _f32(Tobs).reshape(-1), n_it, int(o["nlbfgs"]), int(o["stepmax"]),
                                     float(o["eps_scale"]), float(o["c1"]), float(o["c2"]), float(o["scalefac"]),
                                     float(o["vp_lo"]), float(o["vp_hi"]), float(o["pro"]), int(o["spatfilter"]),
                                     int(o["filt_size_grad"]), int(o["filt_size_grad1"]), int(o["taper_hor"]),
                                     int(o["gradt1"]), int(o["gradt2"]), float(o["exp_taper_grad_hor"]), mis, steps)
        ev = np.zeros(4096, np.float64)
        n = self.lib.ref_evals(ev, len(ev))
        return vp.reshape(self.p.ny, self.p.nx), mis[:it], steps[:it], ev[: min(n, len(ev))]
