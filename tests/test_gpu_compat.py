"""The reference-signature shim (eikonal(), eikonal_adj(), grad_obj() with the
reference's NR matrices and globals) against the oracle, through a tiny C
host program (tests/compat/harness.c) that plays the part of RAJZEL."""
import ctypes as C
import os
import subprocess
import tempfile

import numpy as np
import pytest

import oracle as O
from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def build_harness(mpi):
    """The harness with the shim compiled in; mpi: the shim's RZ_COMPAT_MPI
    branch against the single-rank MPI stand-in of oracle/stub."""
    from rajzel_gb300 import build as B
    B.build()
    O.build(ref=False)
    out = os.path.join(tempfile.mkdtemp(prefix="rzh"), "libharness_mpi.so" if mpi else "libharness.so")
    pkg = os.path.join(ROOT, "rajzel_gb300")
    extra = ["-DRZ_COMPAT_MPI", "-I", os.path.join(ROOT, "oracle", "stub")] if mpi else []
    # the shim is compiled into the harness and bound to it (-Bsymbolic): its err(),
    # writemod(), ... calls then reach the harness, as they reach the RAJZEL program
    # that links it, and not the C library's err() of the loading process
    subprocess.run(["gcc", "-O2", "-fPIC", "-shared", *extra, "-I", os.path.join(ROOT, "include"), "-o", out,
                    os.path.join(HERE, "compat", "harness.c"), os.path.join(pkg, "csrc", "rz_compat.c"),
                    "-Wl,-Bsymbolic", "-L", pkg, "-lrajzel_gb300", f"-Wl,-rpath,{pkg}", "-lm"], check=True)
    lib = C.CDLL(out, mode=C.RTLD_LOCAL)
    f32 = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    lib.h_set.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float]
    lib.h_eikonal.argtypes = [f32, C.c_float, C.c_float, C.c_int, i32, i32, f32, f32]
    lib.h_eikonal_adj.argtypes = [f32, f32, C.c_int, i32, i32, f32]
    lib.h_grad_obj.argtypes = [C.c_char_p, f32, C.c_int, f32, f32, C.c_int, i32, i32, f32, f32]
    lib.h_grad_obj.restype = C.c_double
    lib.h_forward.argtypes = [f32, C.c_int, f32, f32, C.c_int, i32, i32, f32, f32]
    lib.h_picks.argtypes = [C.c_int, C.c_int, f32]
    lib.h_picks.restype = C.c_int
    return lib


@pytest.fixture(scope="module")
def harness(gpu_lib):
    return build_harness(False)


@pytest.fixture(scope="module")
def harness_mpi(gpu_lib):
    return build_harness(True)


def test_shim_eikonal_and_adjoint(harness):
    w = synth.small_case(777, 130, 90, nshots=1)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    harness.h_set(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    TT = np.empty((w.ny, w.nx), np.float32)
    Tmod = np.empty(w.ntr, np.float32)
    harness.h_eikonal(S, w.srcx[0], w.srcz[0], w.ntr, w.recx, w.recz, TT, Tmod)
    to, _ = O.eikonal(p, S, w.srcx[0], w.srcz[0])
    assert np.array_equal(TT, to) and np.array_equal(Tmod, O.calc_fa(p, to, w.recx, w.recz))
    Tres, _ = O.calc_res(p, to, Tmod, Tmod * np.float32(1.01), w.recx, w.recz)
    lam = np.empty_like(TT)
    harness.h_eikonal_adj(to, Tres, w.ntr, w.recx, w.recz, lam)
    lo, _ = O.eikonal_adj(p, to, Tres, w.recx, w.recz)
    assert np.array_equal(lam, lo)


def test_shim_grad_obj_reads_pick_files(harness):
    w = synth.small_case(778, 110, 75, nshots=3)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    Tobs = np.stack([O.calc_fa(p, O.eikonal(p, S * np.float32(1.02), w.srcx[i], w.srcz[i])[0], w.recx, w.recz)
                     for i in range(3)])
    harness.h_set(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    grad = np.empty((w.ny, w.nx), np.float32)
    d = tempfile.mkdtemp(prefix="rzp")
    L2 = harness.h_grad_obj(os.path.join(d, "p").encode(), S, 3, w.srcx, w.srcz, w.ntr, w.recx, w.recz,
                            np.ascontiguousarray(Tobs), grad)
    go, L2o, _, _, _ = O.grad_obj(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert np.array_equal(grad, go) and L2 == L2o


def test_shim_grad_obj_mpi_branch_repairs_the_corner(harness_mpi):
    """With RZ_COMPAT_MPI the shim calls the reference's sum_grad_MPI, which
    leaves grad[NY][NX] unwritten (a NaN in the harness); the frame copy after
    it (grad_obj.c:68-70) must restore the reference's gradient."""
    w = synth.small_case(779, 96, 64, nshots=3)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    Tobs = np.stack([O.calc_fa(p, O.eikonal(p, S * np.float32(0.98), w.srcx[i], w.srcz[i])[0], w.recx, w.recz)
                     for i in range(3)])
    harness_mpi.h_set(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    grad = np.empty((w.ny, w.nx), np.float32)
    d = tempfile.mkdtemp(prefix="rzp")
    L2 = harness_mpi.h_grad_obj(os.path.join(d, "p").encode(), S, 3, w.srcx, w.srcz, w.ntr, w.recx, w.recz,
                                np.ascontiguousarray(Tobs), grad)
    go, L2o, _, _, _ = O.grad_obj(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert np.isfinite(grad).all() and np.array_equal(grad, go) and L2 == L2o


def test_shim_forward_batches_shots_and_writes_every_shots_picks(harness):
    """forward() runs the rank's shots in batched engine calls, writes each
    shot's picks through write_picks() in shot order and leaves the last
    shot's traveltimes and picks behind, as forward.c:19-24 over eikonal()."""
    w = synth.small_case(780, 120, 70, nshots=5)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    harness.h_set(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    TT = np.empty((w.ny, w.nx), np.float32)
    Tmod = np.empty(w.ntr, np.float32)
    harness.h_forward(S, 5, w.srcx, w.srcz, w.ntr, w.recx, w.recz, TT, Tmod)
    for s in range(5):
        to, _ = O.eikonal(p, S, w.srcx[s], w.srcz[s])
        got = np.empty(w.ntr, np.float32)
        calls = harness.h_picks(s + 1, w.ntr, got)
        assert calls == 5 and np.array_equal(got, O.calc_fa(p, to, w.recx, w.recz))
    assert np.array_equal(TT, to) and np.array_equal(Tmod, O.calc_fa(p, to, w.recx, w.recz))
