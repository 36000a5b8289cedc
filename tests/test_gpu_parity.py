"""GPU parity tests: the CUDA path (through the C ABI) against the oracle.

Reference mode must reproduce the reference bit for bit (fields compared as
values: +0 and -0 count as equal).  Fast mode must stay within 1e-5 relative
of the FP64 oracle on traveltimes; on gradients it must be no further from the
FP64 oracle than twice the reference's own float arithmetic plus 1e-4
(relative L2), because the reference's float gradient itself sits ~1e-3 away.
"""
import ctypes as C
import glob
import hashlib
import math
import os

import numpy as np
import pytest

import oracle as O
from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TT_TOL = 1e-5
GRAD_TOL = 1e-4


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


@pytest.fixture(scope="module")
def R(gpu_lib):
    O.build(ref=False)
    return gpu_lib


def make_ctx(R, w, mode="reference", max_passes=500, ttnorm=None):
    ctx = R.Context(0, mode)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm if ttnorm is None else ttnorm, w.eps_adj, max_passes=max_passes)
    ctx.set_slowness(synth.slowness(w.vp_true))
    ctx.set_receivers(w.recx, w.recz)
    return ctx


def params(w):
    return O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)


# ---------------------------------------------------------------------------
# golden fixtures (made by the reference's own code)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "fwd_*.npz"))))
def test_forward_matches_golden(R, path):
    d = np.load(path)
    if str(d["kind"]) == "forward_digest":
        w = synth.fwd_500x174()
        ctx = make_ctx(R, w)
        TT, Tmod, passes = ctx.eikonal(w.srcx[0], w.srcz[0])
        assert digest(TT) == str(d["TT_sha256"])
        assert np.array_equal(Tmod, d["Tmod"]) and passes == int(d["passes"])
        return
    w = synth.Workload("g", int(d["nx"]), int(d["ny"]), float(d["dh"]), float(d["time"]), float(d["ttnorm"]),
                       float(d["eps_adj"]), d["vp"], d["vp"], d["srcx"], d["srcz"], d["recx"], d["recz"])
    ctx = make_ctx(R, w)
    TT, Tmod, passes = ctx.forward(w.srcx, w.srcz)
    for i in range(len(w.srcx)):
        assert digest(TT[i]) == str(d["TT_sha256"][i])
        assert np.array_equal(Tmod[i], d["Tmod"][i])
        assert passes[i] == d["passes"][i]


@pytest.mark.parametrize("path", [p for p in sorted(glob.glob(os.path.join(GOLDEN, "grad_*.npz"))) if "muted" not in p])
def test_gradient_matches_golden(R, path):
    d = np.load(path)
    w = synth.Workload("g", int(d["nx"]), int(d["ny"]), float(d["dh"]), float(d["time"]), float(d["ttnorm"]),
                       float(d["eps_adj"]), d["vp"], d["vp"], d["srcx"], d["srcz"], d["recx"], d["recz"])
    ctx = make_ctx(R, w)
    grad, L2 = ctx.grad_obj(w.srcx, w.srcz, d["Tobs"])
    assert np.array_equal(grad, d["grad"])
    assert L2 == float(d["L2"])
    TT, lam, Tres = ctx.shot_fields(0)
    assert np.array_equal(Tres, d["shot0_Tres"])
    assert np.array_equal(lam, d["shot0_lam"])
    assert ctx.shot_info(0)[1] == int(d["shot0_adj_passes"])


# ---------------------------------------------------------------------------
# reference mode against the oracle on varied shapes
# ---------------------------------------------------------------------------
# 70x512 fills 16 warps; 40x600 and 37x1100 are swept in 2 and 3 bands of strips
SHAPES = [(3, 3), (5, 40), (40, 30), (64, 64), (33, 97), (100, 77), (257, 130), (70, 512), (511, 33), (40, 600),
          (37, 1100)]


@pytest.mark.parametrize("nx,ny", SHAPES)
def test_forward_reference_mode_bit_exact(R, nx, ny):
    w = synth.small_case(nx * 1000 + ny, nx, ny, nshots=3)
    p = params(w)
    S = synth.slowness(w.vp_true)
    ctx = make_ctx(R, w)
    TT, Tmod, passes = ctx.forward(w.srcx, w.srcz)
    for i in range(3):
        to, po = O.eikonal(p, S, w.srcx[i], w.srcz[i])
        assert np.array_equal(TT[i], to), f"shot {i}: {int((TT[i] != to).sum())} cells differ"
        assert passes[i] == po
        assert np.array_equal(Tmod[i], O.calc_fa(p, to, w.recx, w.recz))


def test_forward_sources_on_borders_and_corners(R):
    nx, ny, dh = 70, 45, 10.0
    w = synth.small_case(7, nx, ny, dh=dh, nshots=1)
    xs = np.array([dh, nx * dh, dh, nx * dh, 35 * dh, dh, 35 * dh], np.float32)
    zs = np.array([dh, dh, ny * dh, ny * dh, dh, 20 * dh, ny * dh], np.float32)
    ctx = make_ctx(R, w)
    TT, _, passes = ctx.forward(xs, zs)
    p = params(w)
    S = synth.slowness(w.vp_true)
    for i in range(len(xs)):
        to, po = O.eikonal(p, S, xs[i], zs[i])
        assert np.array_equal(TT[i], to) and passes[i] == po


@pytest.mark.parametrize("nx,ny,dh", [(40, 30, 10.0), (100, 77, 12.5), (150, 130, 5.0), (90, 200, 20.0),
                                      (50, 700, 10.0)])
def test_gradient_reference_mode_bit_exact(R, nx, ny, dh):
    w = synth.small_case(nx + 7 * ny, nx, ny, dh=dh, nshots=4)
    p = params(w)
    S = synth.slowness(w.vp_true)
    rng = np.random.default_rng(nx)
    Tobs = np.empty((4, w.ntr), np.float32)
    for i in range(4):
        to, _ = O.eikonal(p, S * np.float32(0.97), w.srcx[i], w.srcz[i])
        Tobs[i] = O.calc_fa(p, to, w.recx, w.recz) * (1 + 0.01 * rng.standard_normal(w.ntr)).astype(np.float32)
    ctx = make_ctx(R, w)
    grad, L2 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    go, L2o, fp, ap, _ = O.grad_obj(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert np.array_equal(grad, go), f"{int((grad != go).sum())} gradient cells differ"
    assert L2 == L2o
    for i in range(4):
        assert ctx.shot_info(i)[:2] == (fp[i], ap[i])


def test_eikonal_adj_entry_point(R):
    w = synth.small_case(99, 80, 70, nshots=1)
    p = params(w)
    S = synth.slowness(w.vp_true)
    to, _ = O.eikonal(p, S, w.srcx[0], w.srcz[0])
    Tmod = O.calc_fa(p, to, w.recx, w.recz)
    Tres, _ = O.calc_res(p, to, Tmod, Tmod * np.float32(1.02), w.recx, w.recz)
    ctx = make_ctx(R, w)
    lam, passes = ctx.eikonal_adj(to, Tres)
    lo, po = O.eikonal_adj(p, to, Tres, w.recx, w.recz)
    assert np.array_equal(lam, lo) and passes == po


@pytest.mark.parametrize("scale", [1e-29, 1e-36])
def test_eikonal_adj_tiny_lambda(R, scale):
    """Residuals scaled by 1e-29 and 1e-36 make the numerators of sweep_adj.c's
    rhs/DH divisions tiny: below 2^-96, where Markstein's division by DH runs
    on the numerator scaled by 2^64, and (1e-36) so small that the quotient is
    subnormal, which takes IEEE division.  Lambda stays bit-exact with the
    reference algorithm."""
    w = synth.small_case(99, 80, 70, nshots=1)
    p = params(w)
    S = synth.slowness(w.vp_true)
    to, _ = O.eikonal(p, S, w.srcx[0], w.srcz[0])
    Tmod = O.calc_fa(p, to, w.recx, w.recz)
    Tres, _ = O.calc_res(p, to, Tmod, Tmod * np.float32(1.02), w.recx, w.recz)
    Tres = (Tres.astype(np.float64) * scale).astype(np.float32)
    assert np.all(Tres != 0)
    ctx = make_ctx(R, w)
    lam, passes = ctx.eikonal_adj(to, Tres)
    lo, po = O.eikonal_adj(p, to, Tres, w.recx, w.recz)
    assert np.array_equal(lam, lo) and passes == po
    nz = np.abs(lo[lo != 0])  # cells with lambda this small give numerators below 2^-96 / subnormal quotients
    assert np.any(nz < (1e-26 if scale == 1e-29 else 1.1754944e-38))


def _one_pass(p, fn, *args):
    """The oracle's field after one pass (max_passes 1 ends it with a
    no-convergence status, which is expected here)."""
    lib = O._load_port()
    q = O.Params(p.nx, p.ny, p.dh, p.time, p.ttnorm, p.eps_adj, 1)
    return fn(lib, q, *args)


def _norm1(new, old):
    """norm1.c's mean change: |new - old| in float, added in x-outer order to
    a float through double, divided by NX*NY in float."""
    d = np.abs(new.astype(np.float32) - old.astype(np.float32)).T.ravel()
    s = np.float32(0.0)
    for v in d:
        s = np.float32(np.float64(s) + np.float64(v))
    return np.float32(s / np.float32(d.size))


@pytest.mark.parametrize("phase", ["forward", "adjoint"])
def test_stopping_rule_at_its_boundary_after_the_first_pass(R, phase):
    """TTNORM equal to the first pass's mean change, and the next float above:
    the reference continues at the first and stops at the second.  The GPU's
    estimate cannot decide there, so it replays the exact sequential sum
    against the pass's start field, which the first pass does not copy (it is
    the initial field, rebuilt for the replay).  Fields and pass counts must
    equal the oracle's at both values."""
    w = synth.small_case(123, 80, 70, nshots=1)
    p = params(w)
    S = synth.slowness(w.vp_true)
    sx, sz = w.srcx[0], w.srcz[0]
    to, _ = O.eikonal(p, S, sx, sz)
    Tmod = O.calc_fa(p, to, w.recx, w.recz)
    Tres, _ = O.calc_res(p, to, Tmod, Tmod * np.float32(1.02), w.recx, w.recz)
    if phase == "forward":
        def fwd1(lib, q):
            TT = np.empty(p.nx * p.ny, np.float32)
            it = C.c_int(0)
            lib.rzo_eikonal(C.byref(q.grid()), O._f32(S).reshape(-1), sx, sz, TT, C.byref(it))
            return TT.reshape(p.ny, p.nx)
        start = np.full((p.ny, p.nx), np.float32(2.0 * np.float64(np.float32(w.time))), np.float32)
        start[int(np.floor(sz / w.dh + 0.5)) - 1, int(np.floor(sx / w.dh + 0.5)) - 1] = 0.0
        l1 = _norm1(_one_pass(p, fwd1), start)
    else:
        def adj1(lib, q):
            lam = np.empty(p.nx * p.ny, np.float32)
            it = C.c_int(0)
            rx, rz = O._i32(w.recx), O._i32(w.recz)
            lib.rzo_eikonal_adj(C.byref(q.grid()), O._f32(to).reshape(-1), O._f32(Tres), len(rx), rx, rz, lam,
                                C.byref(it))
            return lam.reshape(p.ny, p.nx)
        start = np.zeros((p.ny, p.nx), np.float32)
        start[1:-1, 1:-1] = np.float32(10.0 * np.float64(np.float32(w.time)))
        for i in range(len(w.recx)):
            h, k = int(w.recx[i]) - 1, int(w.recz[i]) - 1
            if 0 < h < p.nx - 1 and 0 < k < p.ny - 1:
                start[k, h] = Tres[i]
        l1 = _norm1(_one_pass(p, adj1), start)
    passes = []
    for tn in (l1, np.nextafter(l1, np.float32(np.inf))):
        q = O.Params(p.nx, p.ny, p.dh, p.time, float(tn), p.eps_adj)
        ctx = make_ctx(R, w, ttnorm=float(tn))
        if phase == "forward":
            got, _, pg = ctx.eikonal(sx, sz)
            want, pw = O.eikonal(q, S, sx, sz)
        else:
            got, pg = ctx.eikonal_adj(to, Tres)
            want, pw = O.eikonal_adj(q, to, Tres, w.recx, w.recz)
        assert np.array_equal(got, want) and pg == pw
        passes.append(pw)
    assert passes[0] > passes[1] == 1  # the boundary is exactly at l1


def test_batched_equals_single_shot(R):
    w = synth.small_case(5, 120, 90, nshots=5)
    ctx = make_ctx(R, w)
    TT, _, _ = ctx.forward(w.srcx, w.srcz)
    for i in range(5):
        t1, _, _ = ctx.eikonal(w.srcx[i], w.srcz[i])
        assert np.array_equal(TT[i], t1)


def _noisy_picks(p, w, S, n, seed):
    rng = np.random.default_rng(seed)
    Tobs = np.empty((n, w.ntr), np.float32)
    for i in range(n):
        to, _ = O.eikonal(p, S * np.float32(0.97), w.srcx[i], w.srcz[i])
        Tobs[i] = O.calc_fa(p, to, w.recx, w.recz) * (1 + 0.01 * rng.standard_normal(w.ntr)).astype(np.float32)
    return Tobs


@pytest.mark.parametrize("mode", ["reference", "fast"])
def test_memory_cap_chunks_do_not_change_results(R, mode):
    """A memory cap smaller than the batch's field slots makes the batch run
    in chunks (here 2+2+1 shots); every result must equal the unchunked run
    bit for bit, and in reference mode also the oracle."""
    w = synth.small_case(77, 90, 70, nshots=5)
    p = params(w)
    S = synth.slowness(w.vp_true)
    Tobs = _noisy_picks(p, w, S, 5, 11)
    ctx = make_ctx(R, w, mode=mode)
    g_all, l_all = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    TT_all, Tm_all, pf_all = ctx.forward(w.srcx, w.srcz)
    nxp = 32 * ((w.nx + 31) // 32)
    nst = (w.ny + 31) // 32
    slot = 4 * (3 * w.ny * nxp + 2 * nst * (32 * (nxp // 32) + 64) * 32 + 2 * nst * (nxp + 96))
    ctx.set_memory_cap(2 * slot + slot // 2)
    g_c, l_c = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    assert np.array_equal(g_c, g_all) and l_c == l_all
    TT_c, Tm_c, pf_c = ctx.forward(w.srcx, w.srcz)
    assert np.array_equal(TT_c, TT_all) and np.array_equal(Tm_c, Tm_all) and np.array_equal(pf_c, pf_all)
    # fields are kept for the last chunk only
    with pytest.raises(R.RajzelError):
        ctx.shot_fields(0)
    ctx.shot_fields(4)
    if mode == "reference":
        go, L2o, _, _, _ = O.grad_obj(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
        assert np.array_equal(g_c, go) and l_c == L2o


# ---------------------------------------------------------------------------
# fast mode against the FP64 oracle
# ---------------------------------------------------------------------------
def test_fast_mode_traveltimes_within_tolerance(R):
    w = synth.small_case(31, 200, 150, nshots=3)
    p = params(w)
    S = synth.slowness(w.vp_true)
    ctx = make_ctx(R, w, mode="fast")
    TT, _, _ = ctx.forward(w.srcx, w.srcz)
    for i in range(3):
        t64, _ = O.eikonal_f64(p, S.astype(np.float64), w.srcx[i], w.srcz[i])
        assert np.abs(TT[i] - t64).max() / np.abs(t64).max() <= TT_TOL


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def test_fast_mode_gradient_within_tolerance(R):
    """The receiver scaling Tres/(dT/dz) (calc_FA_res.c:52-69) differences
    neighbouring float traveltimes, so even the reference's own float
    arithmetic sits ~1e-3 from the FP64 oracle on gradients.  Fast mode must
    be no worse than that, plus GRAD_TOL."""
    w = synth.small_case(32, 160, 100, nshots=4)
    p = params(w)
    S = synth.slowness(w.vp_true)
    rng = np.random.default_rng(3)
    Tobs = np.empty((4, w.ntr), np.float32)
    for i in range(4):
        to, _ = O.eikonal(p, S * np.float32(0.97), w.srcx[i], w.srcz[i])
        Tobs[i] = O.calc_fa(p, to, w.recx, w.recz) * (1 + 0.01 * rng.standard_normal(w.ntr)).astype(np.float32)
    ctx = make_ctx(R, w, mode="fast")
    grad, L2 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    g64, L64 = O.grad_obj_f64(p, S.astype(np.float64), w.srcx.astype(np.float64), w.srcz.astype(np.float64),
                              w.recx, w.recz, Tobs.astype(np.float64))
    g32, L32, _, _, _ = O.grad_obj(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    err_ref = rel_l2(g32, g64)
    assert rel_l2(grad, g64) <= 2.0 * err_ref + GRAD_TOL
    assert abs(L2 - L64) / abs(L64) <= 2.0 * abs(L32 - L64) / abs(L64) + GRAD_TOL


# ---------------------------------------------------------------------------
# arithmetic self-test and error handling
# ---------------------------------------------------------------------------
def test_certified_godunov_branch_matches_double(R):
    lib = C.CDLL(os.path.join(os.path.dirname(R.__file__), "librz_selftest.so"))
    lib.rz_selftest_godunov.argtypes = [C.c_ulonglong, C.c_long, C.POINTER(C.c_ulonglong)]
    bad = C.c_ulonglong(1)
    assert lib.rz_selftest_godunov(12345, 20_000_000, C.byref(bad)) == 0
    assert bad.value == 0


@pytest.mark.parametrize("dh", [10.0, 5.0, 12.5, 20.0, 7.3])
def test_tiny_numerator_divisions_match_ieee(R, dh):
    """Divisions of numerators below 2^-96 (normal and subnormal, quotients
    down to the subnormal range): by DH (Markstein at 2^64 times the size) and
    by a general positive divisor, bit for bit against IEEE division on 2e7
    random draws each."""
    lib = C.CDLL(os.path.join(os.path.dirname(R.__file__), "librz_selftest.so"))
    lib.rz_selftest_div_tiny.argtypes = [C.c_ulonglong, C.c_long, C.c_float, C.POINTER(C.c_ulonglong)]
    bad = (C.c_ulonglong * 2)(1, 1)
    rc = lib.rz_selftest_div_tiny(99, 20_000_000, dh, bad)
    if rc == 4:
        pytest.skip(f"Markstein division not exact for DH={dh}; the engine uses IEEE division")
    assert rc == 0 and (bad[0], bad[1]) == (0, 0)


def _shot_sum(R, vals):
    lib = C.CDLL(os.path.join(os.path.dirname(R.__file__), "librz_selftest.so"))
    lib.rz_selftest_shot_sum.argtypes = [C.c_void_p, C.c_long, C.c_int, C.c_void_p]
    vals = np.ascontiguousarray(vals, dtype=np.float32)
    nshots, ncells = vals.shape
    out = np.full(ncells, np.nan)
    assert lib.rz_selftest_shot_sum(vals.ctypes.data, ncells, nshots, out.ctypes.data) == 0
    return out


def _exact_sums(vals):
    """Correctly rounded sums of the columns (math.fsum of the exact values)."""
    return np.array([math.fsum(col) for col in vals.astype(np.float64).T])


def test_stack_shot_sum_fixed_point(R):
    """The fast-mode stack sums a cell's shots in a 64-bit fixed-point word.
    With an exponent span of at most 31 within 128 shots nothing is dropped
    and the result is the correctly rounded exact sum; over any span and
    shot count the error stays within n 2^-53 max|x| plus one double
    rounding per 128-shot block and per block sum."""
    rng = np.random.default_rng(5)
    ncells = 3001  # not a multiple of the 256-thread block
    for n in (0, 1, 7, 100, 128):
        mag = (1.0 + rng.random((n, ncells))) * 2.0 ** rng.integers(-12, 13, (n, ncells))
        v = (np.where(rng.random((n, ncells)) < 0.5, -mag, mag) * (rng.random((n, ncells)) > 0.05))
        v = v.astype(np.float32)
        got = _shot_sum(R, v)
        assert np.array_equal(got, _exact_sums(v) if n else np.zeros(ncells))
    # subnormals only: exact
    v = (rng.integers(-2**20, 2**20, (50, ncells)) * 2.0**-149).astype(np.float32)
    assert np.array_equal(_shot_sum(R, v), _exact_sums(v))
    # exponents over +-100 (dropped low bits), several 128-shot blocks
    for n in (129, 300, 1000):
        mag = (1.0 + rng.random((n, ncells))) * 2.0 ** rng.integers(-100, 101, (n, ncells))
        v = np.where(rng.random((n, ncells)) < 0.5, -mag, mag).astype(np.float32)
        got = _shot_sum(R, v)
        a = np.abs(v.astype(np.float64))
        bound = 2.0**-53 * (n * a.max(axis=0) + 2 * (-(-n // 128)) * a.sum(axis=0))
        assert np.all(np.abs(got - _exact_sums(v)) <= bound)
    # cancellation inside one block, and non-finite values propagate as in double
    v = np.zeros((6, 6), np.float32)
    v[:3, 0] = [3.0e30, 1.0, -3.0e30]
    v[:2, 1] = [np.inf, 1.0]
    v[:2, 2] = [-np.inf, 2.0]
    v[:2, 3] = [np.inf, -np.inf]
    v[:3, 4] = [1.0, np.nan, 2.0]
    v[:, 5] = -0.0
    got = _shot_sum(R, v)
    # 1.0 is 101 binades below 3e30: dropped, as a double sum drops it
    assert got[0] == 0.0 and got[1] == np.inf and got[2] == -np.inf
    assert np.isnan(got[3]) and np.isnan(got[4]) and got[5] == 0.0


def test_invalid_model_is_rejected_with_its_cell(R):
    """The slowness is checked on the device (calc_S.c gives no error path):
    a zero, negative or NaN velocity, or an infinite slowness, is refused
    with the first bad cell, and the context works once a valid model is set."""
    w = synth.small_case(7, 40, 24, nshots=1)
    ctx = make_ctx(R, w)
    TT0, _, _ = ctx.eikonal(w.srcx[0], w.srcz[0])
    for bad_vp in (0.0, -1500.0, np.nan):
        vp = w.vp_true.copy()
        vp[5, 7] = bad_vp
        vp[9, 3] = bad_vp
        with pytest.raises(R.RajzelError) as e:
            ctx.set_velocity(vp)
        assert e.value.status == R.RZ_EINVAL and f"cell {5 * w.nx + 7} " in str(e.value)
    S = synth.slowness(w.vp_true)
    S[11, 2] = np.inf
    with pytest.raises(R.RajzelError) as e:
        ctx.set_slowness(S)
    assert e.value.status == R.RZ_EINVAL and f"cell {11 * w.nx + 2} " in str(e.value)
    ctx.set_velocity(w.vp_true)
    TT1, _, _ = ctx.eikonal(w.srcx[0], w.srcz[0])
    assert np.array_equal(TT0, TT1)


@pytest.mark.parametrize("mode", ["reference", "fast"])
def test_pinned_host_models_match_pageable(R, mode):
    """A velocity or slowness in pinned host memory (read by the device
    directly where it reaches host memory coherently) gives the results of
    the same model in pageable memory, and an invalid pinned model is refused
    with its first bad cell."""
    torch = pytest.importorskip("torch")
    w = synth.small_case(31, 90, 70, nshots=3)
    p = params(w)
    S = synth.slowness(w.vp_true)
    Tobs = _noisy_picks(p, w, S, 3, 5)
    ctx = make_ctx(R, w, mode=mode)
    ctx.set_velocity(w.vp_start)
    g0, l0 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    vp = torch.empty((w.ny, w.nx), dtype=torch.float32, pin_memory=True).numpy()
    vp[...] = w.vp_start
    ctx.set_velocity(vp)
    g1, l1 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    assert np.array_equal(g1, g0) and l1 == l0
    Sp = torch.empty((w.ny, w.nx), dtype=torch.float32, pin_memory=True).numpy()
    Sp[...] = synth.slowness(w.vp_start)
    ctx.set_slowness(Sp)
    g2, l2 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    ctx.set_slowness(synth.slowness(w.vp_start))
    g3, l3 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    assert np.array_equal(g2, g3) and l2 == l3
    # the gradient into a pinned buffer (written by the device where it
    # reaches host memory), the misfit and the status words alongside
    ctx.set_velocity(w.vp_start)
    gpin = torch.zeros((w.ny, w.nx), dtype=torch.float32, pin_memory=True).numpy()
    g4, l4 = ctx.grad_obj(w.srcx, w.srcz, Tobs, out=gpin)
    assert g4 is gpin and np.array_equal(gpin, g0) and l4 == l0
    ctx1 = make_ctx(R, w, mode=mode, max_passes=1)
    with pytest.raises(R.RajzelError) as e:
        ctx1.grad_obj(w.srcx, w.srcz, Tobs, out=gpin)
    assert e.value.status == R.RZ_ENOCONV
    vp[4, 6] = -1.0
    with pytest.raises(R.RajzelError) as e:
        ctx.set_velocity(vp)
    assert e.value.status == R.RZ_EINVAL and f"cell {4 * w.nx + 6} " in str(e.value)
    ctx.set_velocity(w.vp_start)
    assert np.array_equal(ctx.grad_obj(w.srcx, w.srcz, Tobs)[0], g0)


def test_errors_are_status_codes(R):
    w = synth.small_case(1, 30, 20, nshots=1)
    ctx = R.Context(0)
    with pytest.raises(R.RajzelError) as e:
        ctx.set_grid(30, 20, 10.0, 40.0, ttnorm=0.0)  # the reference would loop forever
    assert e.value.status == R.RZ_EINVAL
    ctx = make_ctx(R, w)
    with pytest.raises(R.RajzelError) as e:
        ctx.eikonal(-50.0, 10.0)  # source index 0 would be out of bounds in the reference
    assert e.value.status == R.RZ_EINVAL
    with pytest.raises(R.RajzelError) as e:
        ctx.set_receivers(np.array([31], np.int32), np.array([2], np.int32))
    assert e.value.status == R.RZ_EINVAL
    ctx2 = make_ctx(R, w, max_passes=1)
    with pytest.raises(R.RajzelError) as e:
        ctx2.eikonal(w.srcx[0], w.srcz[0])
    assert e.value.status == R.RZ_ENOCONV
    # the context stays usable after errors
    TT, _, _ = ctx.eikonal(w.srcx[0], w.srcz[0])
    assert np.isfinite(TT).all()


# ---------------------------------------------------------------------------
# full-size workload: size-independent properties
# ---------------------------------------------------------------------------
def test_full_size_gradient_properties(R):
    w = synth.grad_1700x350(nshots=8, ntr=850)
    ctx_t = make_ctx(R, w, mode="fast")
    _, Tobs, _ = ctx_t.forward(w.srcx, w.srcz, want_tt=False)
    results = {}
    for mode in ("reference", "fast"):
        ctx = R.Context(0, mode)
        ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
        ctx.set_velocity(w.vp_start)
        ctx.set_receivers(w.recx, w.recz)
        results[mode] = ctx.grad_obj(w.srcx, w.srcz, Tobs) + (ctx,)
    (gr, Lr, ctx_r), (gf, Lf, _) = results["reference"], results["fast"]
    assert np.isfinite(gr).all() and np.isfinite(gf).all()
    # two float evaluations of a gradient whose float error vs FP64 is ~1e-3
    assert rel_l2(gf, gr) <= 5e-3
    assert abs(Lf - Lr) / Lr <= 5e-3
    TT, lam, _ = ctx_r.shot_fields(0)
    hs, ks = synth.grid_index(w.srcx[0], w.dh) - 1, synth.grid_index(w.srcz[0], w.dh) - 1
    assert TT[ks, hs] == 0.0 and (TT >= 0).all() and TT.max() < 2 * w.time
    # reference mode at full size against the oracle for one shot
    p = params(w)
    S = synth.slowness(w.vp_start)
    to, _ = O.eikonal(p, S, w.srcx[0], w.srcz[0])
    assert np.array_equal(TT, to)


@pytest.mark.parametrize("mode", ["reference", "fast"])
def test_multi_grid_launch_equals_per_grid_calls(R, mode):
    """One persistent launch over three grids (one of them banded, one leaving
    warps of the CTA idle) gives every grid exactly its rz_grad_obj result."""
    shapes = [(120, 90, 5), (60, 600, 3), (200, 40, 7)]
    ctxs, ws, tobs, want = [], [], [], []
    for k, (nx, ny, ns) in enumerate(shapes):
        w = synth.small_case(300 + k, nx, ny, nshots=ns)
        p = params(w)
        S = synth.slowness(w.vp_true)
        Tobs = _noisy_picks(p, w, S, ns, 40 + k)
        ctx = make_ctx(R, w, mode=mode)
        want.append(ctx.grad_obj(w.srcx, w.srcz, Tobs) + ([ctx.shot_info(i)[:2] for i in range(ns)],))
        ctxs.append(ctx)
        ws.append(w)
        tobs.append(Tobs)
    got = R.grad_obj_multi(ctxs, [w.srcx for w in ws], [w.srcz for w in ws], tobs)
    for (g, l2), (gw, lw, passes), ctx, w in zip(got, want, ctxs, ws):
        assert np.array_equal(g, gw) and l2 == lw
        assert [ctx.shot_info(i)[:2] for i in range(w.nshots)] == passes


@pytest.mark.parametrize("mode", ["reference", "fast"])
def test_graph_replay_equals_direct_launches(R, mode):
    """rz_grad_obj replays one captured graph across calls with new sources,
    picks and models; every result equals the uncaptured path."""
    w = synth.small_case(91, 110, 80, nshots=4)
    p = params(w)
    S = synth.slowness(w.vp_true)
    direct = make_ctx(R, w, mode=mode)
    direct.set_graphs(False)
    graph = make_ctx(R, w, mode=mode)
    rng = np.random.default_rng(5)
    for call in range(3):
        sx = (w.srcx + rng.uniform(-30, 30, 4)).clip(10.0, (w.nx - 1) * w.dh).astype(np.float32)
        Tobs = _noisy_picks(p, w, S, 4, 60 + call)
        vp = (w.vp_true * np.float32(1.0 + 0.01 * call)).astype(np.float32)
        for ctx in (direct, graph):
            ctx.set_velocity(vp)
        g0, l0 = direct.grad_obj(sx, w.srcz, Tobs)
        g1, l1 = graph.grad_obj(sx, w.srcz, Tobs)
        assert np.array_equal(g0, g1) and l0 == l1
        assert [graph.shot_info(i) for i in range(4)] == [direct.shot_info(i) for i in range(4)]
        f0 = direct.shot_fields(3)
        f1 = graph.shot_fields(3)
        assert all(np.array_equal(a, b) for a, b in zip(f0, f1))
        # timings are read between replays, as bench.py does
        launches, ms, calls = graph.kernel_stats()
        assert calls == 1 and ms > 0


def test_autotuner_picks_a_width_that_changes_no_result(R):
    """rz_autotune times the launch shapes (band width x CTA width x check
    task height) on the batch itself; the chosen shape is used afterwards and
    gives the same result."""
    w = synth.small_case(17, 70, 700, nshots=3)  # 22 strips: 2, 3 or 4 bands
    p = params(w)
    S = synth.slowness(w.vp_true)
    Tobs = _noisy_picks(p, w, S, 3, 71)
    ctx = make_ctx(R, w)
    g0, l0 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    res = ctx.autotune(w.srcx, w.srcz, Tobs)
    assert set(res["candidates"]) == {11, 8, 6} and res["warps"] in res["candidates"]
    assert all(ms > 0 for ms in res["candidates"].values())
    shape = res["shape"]  # band width, CTA width and fixpoint-check task height
    assert shape["sweeping_warps"] == res["warps"] and shape["check_rows"] in (32, 64, 128)
    g1, l1 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    assert np.array_equal(g0, g1) and l0 == l1
    go, L2o, _, _, _ = O.grad_obj(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert np.array_equal(g1, go)


@pytest.mark.parametrize("kind,refine", [("exact", True), ("exact", False), ("reference", True)])
def test_multi_grid_launch_exact_refined_equals_per_grid_calls(R, kind, refine):
    """The exact gradient and refined traveltimes through one persistent launch
    over three grids (one banded) equal each grid's own rz_grad_obj, bit for
    bit: the tile-fed preparation, the packed weight streams and the
    refinement's linear sweeps do not depend on the launch they run in."""
    shapes = [(120, 90, 4), (60, 600, 3), (200, 40, 5)]
    ctxs, ws, tobs, want = [], [], [], []
    for k, (nx, ny, ns) in enumerate(shapes):
        w = synth.small_case(500 + k, nx, ny, nshots=ns)
        p = params(w)
        S = synth.slowness(w.vp_true)
        Tobs = _noisy_picks(p, w, S, ns, 60 + k)
        ctx = make_ctx(R, w, mode="fast")
        ctx.set_gradient(kind)
        ctx.set_refine(refine)
        want.append(ctx.grad_obj(w.srcx, w.srcz, Tobs))
        ctxs.append(ctx)
        ws.append(w)
        tobs.append(Tobs)
    got = R.grad_obj_multi(ctxs, [w.srcx for w in ws], [w.srcz for w in ws], tobs)
    for (g, l2), (gw, lw) in zip(got, want):
        assert np.array_equal(g, gw) and l2 == lw
