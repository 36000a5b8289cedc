"""GPU tests of the exact discrete adjoint (RZ_GRADIENT_EXACT, rz_backward).

The GPU gradient (FP32 sweeps) is compared with the FP64 exact-adjoint
oracle, and its projections on random slowness perturbations with central
finite differences of the FP64 misfit.  Tolerance: 1e-4 relative.
"""
import numpy as np
import pytest

import oracle as O
from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu
GRAD_TOL = 1e-4


@pytest.fixture(scope="module")
def R(gpu_lib):
    O.build(ref=False)
    return gpu_lib


def case(seed, nx, ny, nshots, muted=False):
    w = synth.small_case(seed, nx, ny, nshots=nshots)
    S32 = synth.slowness(w.vp_true)
    p64 = O.Params(w.nx, w.ny, w.dh, w.time, 1e-14, w.eps_adj)
    Tobs = np.empty((nshots, w.ntr), np.float32)
    for i in range(nshots):
        t, _ = O.eikonal_f64(p64, 1.0 / (w.vp_true.astype(np.float64) * 1.03), w.srcx[i], w.srcz[i])
        Tobs[i] = t[w.recz - 1, w.recx - 1]
    if muted:
        Tobs[:, ::7] = -1.0
    return w, S32, p64, Tobs


def gpu_ctx(R, w, S32, mode):
    ctx = R.Context(0, mode)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_slowness(S32)
    ctx.set_receivers(w.recx, w.recz)
    ctx.set_gradient("exact")
    return ctx


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("mode", ["fast", "reference"])
@pytest.mark.parametrize("nx,ny,muted", [(60, 45, False), (130, 70, True), (40, 150, False)])
def test_exact_gradient_matches_fp64_oracle(R, mode, nx, ny, muted):
    w, S32, p64, Tobs = case(nx + ny, nx, ny, 3, muted)
    ctx = gpu_ctx(R, w, S32, mode)
    g, L2 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    g64, L64 = O.grad_exact_f64(p64, S32.astype(np.float64), w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert rel_l2(g, g64) <= GRAD_TOL
    assert abs(L2 - L64) <= GRAD_TOL * abs(L64)


def test_exact_gradient_central_differences_20_perturbations(R):
    """<g, dS> against (J(S + e dS) - J(S - e dS)) / 2e for 20 random slowness
    perturbations dS, J the FP64 misfit; g is the GPU dJ/dVp converted to dJ/dS."""
    w, S32, p64, Tobs = case(9, 64, 48, 2)
    ctx = gpu_ctx(R, w, S32, "fast")
    g_vp, _ = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    S = S32.astype(np.float64)
    g_s = -np.asarray(g_vp, np.float64) / (S * S)  # dJ/dS = dJ/dVp * dVp/dS, Vp = 1/S
    rng = np.random.default_rng(20)
    worst = 0.0
    for _ in range(20):
        d = rng.standard_normal(S.shape) * S
        eps = 1e-6
        jp = O.misfit_f64(p64, S + eps * d, w.srcx, w.srcz, w.recx, w.recz, Tobs)
        jm = O.misfit_f64(p64, S - eps * d, w.srcx, w.srcz, w.recx, w.recz, Tobs)
        fd = (jp - jm) / (2 * eps)
        worst = max(worst, abs(fd - float((g_s * d).sum())) / abs(fd))
    assert worst <= GRAD_TOL, worst


def test_backward_equals_exact_grad_obj_and_ignores_chunking(R):
    """rz_backward with dTmod = Tmod - Tobs is the exact rz_grad_obj; a memory
    cap that splits the batch (forward fields recomputed per chunk) changes
    nothing."""
    w, S32, _, Tobs = case(3, 90, 60, 5)
    ctx = gpu_ctx(R, w, S32, "fast")
    g_exact, _ = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    _, Tmod, _ = ctx.forward(w.srcx, w.srcz, want_tt=False)
    g_bwd = ctx.backward(w.srcx, w.srcz, Tmod - Tobs)
    assert np.array_equal(g_bwd, g_exact)
    nxp = 32 * ((w.nx + 31) // 32)
    nst = (w.ny + 31) // 32
    skew = nst * (nxp + 64) * 32
    slot = 4 * (3 * w.ny * nxp + 6 * skew + 2 * nst * (nxp + 96))
    ctx.set_memory_cap(2 * slot)
    g_chunked = ctx.backward(w.srcx, w.srcz, Tmod - Tobs)
    assert np.allclose(g_chunked, g_exact, rtol=1e-6, atol=1e-6 * np.abs(g_exact).max())


def test_reference_gradient_unchanged_by_exact_switch(R):
    """Switching kinds back restores the reference's gradient bit for bit."""
    w, S32, _, Tobs = case(4, 50, 40, 2)
    ctx = gpu_ctx(R, w, S32, "reference")
    ctx.set_gradient("reference")
    g1, l1 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    ctx.set_gradient("exact")
    ctx.grad_obj(w.srcx, w.srcz, Tobs)
    ctx.set_gradient("reference")
    g2, l2 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    go, lo, _, _, _ = O.grad_obj(p, S32, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert np.array_equal(g1, go) and np.array_equal(g2, go) and l1 == lo == l2


def test_packed_weights_round_trip(R):
    """The linear sweeps read both weights of a cell from one float: the
    smaller magnitude, the x direction in the sign bit, the z direction and
    which magnitude is stored in the two lowest significand bits, 2.0 for a
    cell with no upwind neighbour.  Every case must come back with its
    directions, the smaller weight within 3 ulp (its two lowest bits are
    flags) and the larger as 1 minus it."""
    import ctypes as C
    import os
    lib = C.CDLL(os.path.join(os.path.dirname(R.__file__), "librz_selftest.so"))
    fp = C.POINTER(C.c_float)
    lib.rz_selftest_weights.argtypes = [fp, fp, C.c_long, fp, fp, fp]
    rng = np.random.default_rng(11)
    wa = rng.uniform(0.0, 1.0, 4000).astype(np.float32)
    wa[:6] = [0.0, 1.0, 0.5, 1e-7, 1 - 1e-7, 0.25]
    sx = np.where(rng.random(wa.size) < 0.5, -1.0, 1.0).astype(np.float32)
    sz = np.where(rng.random(wa.size) < 0.5, -1.0, 1.0).astype(np.float32)
    wx = sx * wa
    wz = (sz * (np.float32(1.0) - wa)).astype(np.float32)
    # the source and cells outside the grid: no upwind neighbour
    wx = np.concatenate([wx, np.zeros(2, np.float32)])
    wz = np.concatenate([wz, np.zeros(2, np.float32)])
    n = wx.size
    ox, oz, pk = (np.empty(n, np.float32) for _ in range(3))
    ptr = lambda a: a.ctypes.data_as(fp)  # noqa: E731
    assert lib.rz_selftest_weights(ptr(wx), ptr(wz), n, ptr(ox), ptr(oz), ptr(pk)) == 0
    assert np.all(pk[-2:] == 2.0) and np.all(ox[-2:] == 0) and np.all(oz[-2:] == 0)
    ax, az = np.abs(wx[:-2]), np.abs(wz[:-2])
    # directions (a zero weight may come back as -0 or +0)
    nzx, nzz = ax > 0, az > 0
    assert np.all(np.sign(ox[:-2][nzx]) == np.sign(wx[:-2][nzx]))
    assert np.all(np.sign(oz[:-2][nzz]) == np.sign(wz[:-2][nzz]))
    # the smaller weight within 3 ulp, the larger within an ulp of 1 minus it
    small = np.minimum(ax, az)
    got_small = np.where(ax <= az, np.abs(ox[:-2]), np.abs(oz[:-2]))
    got_small = np.where(ax == az, np.minimum(np.abs(ox[:-2]), np.abs(oz[:-2])), got_small)
    assert np.all(np.abs(got_small.astype(np.float64) - small) <= 3 * np.spacing(small).astype(np.float64) + 1e-45)
    assert np.all(np.abs(np.abs(ox[:-2]) + np.abs(oz[:-2]) - 1.0) <= 2 ** -23)
