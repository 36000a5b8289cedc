"""GPU tests of the FP64 oracle (rz_forward_f64, rz_grad_obj_f64, RZ_MODE_FP64)
and of the error reports it attaches to float results (rz_set_error_check).

The GPU FP64 oracle is pinned to the CPU FP64 restatement (oracle/rz_oracle.c
*_f64, the reference's algorithm in double): traveltimes bit for bit, gradients
within 1e-12 (only the order of the misfit and stack sums differs), the exact
adjoint within 1e-10 (the CPU visits cells in arrival order, the GPU sweeps).

At the benchmark size (1700 x 350, paths of up to ~1800 cells) float32
traveltimes carry the rounding of every update along the path: the
reference's own float arithmetic sits 1.3-2.0e-5 (max-norm) and up to ~1.1e-5
(relative L2) from FP64 there.  Fast mode is gated at "no further from FP64
than the reference's own float arithmetic"; small grids meet 1e-5.
"""
import numpy as np
import pytest

import oracle as O
from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu
TT_TOL = 1e-5
GRAD_TOL = 1e-4


@pytest.fixture(scope="module")
def R(gpu_lib):
    O.build(ref=False)
    return gpu_lib


def ctx_for(R, w, mode, vp=None, ttnorm=None, kind="reference", refine=False):
    ctx = R.Context(0, mode)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm if ttnorm is None else ttnorm, w.eps_adj)
    ctx.set_velocity(w.vp_true if vp is None else vp)
    ctx.set_receivers(w.recx, w.recz)
    ctx.set_gradient(kind)
    ctx.set_refine(refine)
    return ctx


def picks(R, w, scale=0.97):
    """Observed picks from a perturbed model (float reference mode)."""
    ctx = ctx_for(R, w, "reference", vp=(w.vp_true * np.float32(scale)).astype(np.float32))
    _, Tobs, _ = ctx.forward(w.srcx, w.srcz, want_tt=False)
    return Tobs


def rel_l2(a, b):
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))


def tt_rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / np.abs(b).max())


@pytest.mark.parametrize("nx,ny", [(3, 3), (60, 45), (97, 70), (33, 130)])
def test_fp64_forward_equals_cpu_fp64_oracle(R, nx, ny):
    w = synth.small_case(nx * 7 + ny, nx, ny, nshots=3)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx = ctx_for(R, w, "reference")
    S = synth.slowness(w.vp_true).astype(np.float64)
    TT, Tmod = ctx.forward_f64(w.srcx, w.srcz)
    for i in range(w.nshots):
        t64, _ = O.eikonal_f64(p, S, w.srcx[i], w.srcz[i])
        assert np.array_equal(TT[i], t64)
        assert np.array_equal(Tmod[i], t64[w.recz - 1, w.recx - 1])


def test_fp64_leung_qian_gradient_equals_cpu_fp64_oracle(R):
    w = synth.small_case(77, 120, 80, nshots=4)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    Tobs = picks(R, w)
    ctx = ctx_for(R, w, "reference")
    g, L2 = ctx.grad_obj_f64(w.srcx, w.srcz, Tobs)
    S = synth.slowness(w.vp_true).astype(np.float64)
    g64, L64 = O.grad_obj_f64(p, S, w.srcx.astype(np.float64), w.srcz.astype(np.float64), w.recx, w.recz,
                              Tobs.astype(np.float64))
    assert rel_l2(g, g64) <= 1e-12
    assert abs(L2 - L64) <= 1e-12 * abs(L64)


@pytest.mark.parametrize("muted", [False, True])
def test_fp64_exact_gradient_equals_cpu_exact_oracle(R, muted):
    w = synth.small_case(78, 90, 64, nshots=3)
    p64 = O.Params(w.nx, w.ny, w.dh, w.time, 1e-14, w.eps_adj)
    Tobs = picks(R, w)
    if muted:
        Tobs[:, ::5] = -1.0
    ctx = ctx_for(R, w, "reference", ttnorm=1e-14, kind="exact")
    g, L2 = ctx.grad_obj_f64(w.srcx, w.srcz, Tobs)
    S = synth.slowness(w.vp_true).astype(np.float64)
    g64, L64 = O.grad_exact_f64(p64, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert rel_l2(g, g64) <= 1e-10
    assert abs(L2 - L64) <= 1e-12 * abs(L64)


def test_fp64_mode_runs_the_float_api_in_double(R):
    """RZ_MODE_FP64 behind rz_forward / rz_grad_obj / rz_misfit: the double
    results rounded to float."""
    w = synth.small_case(79, 70, 50, nshots=2)
    Tobs = picks(R, w)
    ctx = ctx_for(R, w, "fp64")
    TT, Tmod, passes = ctx.forward(w.srcx, w.srcz)
    TT64, Tmod64 = ctx.forward_f64(w.srcx, w.srcz)
    assert np.array_equal(TT, TT64.astype(np.float32)) and np.array_equal(Tmod, Tmod64.astype(np.float32))
    g, L2 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    g64, L64 = ctx.grad_obj_f64(w.srcx, w.srcz, Tobs)
    assert np.array_equal(g, g64.astype(np.float32)) and L2 == L64
    assert ctx.misfit(w.srcx, w.srcz, Tobs) == L64


@pytest.mark.parametrize("mode", ["reference", "fast"])
def test_error_report_matches_numpy(R, mode):
    """rz_error_report of a checked gradient call equals the same figures
    computed here from the returned fields and the FP64 oracle."""
    w = synth.small_case(80, 110, 75, nshots=3)
    Tobs = picks(R, w)
    ctx = ctx_for(R, w, mode)
    ctx.set_error_check(True)
    g, L2 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    rep = ctx.error_report()
    ref = ctx_for(R, w, "reference")
    g64, L64 = ref.grad_obj_f64(w.srcx, w.srcz, Tobs)
    TT64, Tmod64 = ref.forward_f64(w.srcx, w.srcz)
    assert rep["shots"] == w.nshots
    tt = max(tt_rel(ctx.shot_fields(i)[0], TT64[i]) for i in range(w.nshots))
    _, Tmod, _ = ctx.forward(w.srcx, w.srcz, want_tt=False)
    assert rep["tt_rel"] == pytest.approx(tt, rel=1e-9, abs=1e-300)
    assert rep["tmod_rel"] == pytest.approx(tt_rel(Tmod, Tmod64), rel=1e-9, abs=1e-300)
    assert rep["grad_rel_l2"] == pytest.approx(rel_l2(g, g64), rel=1e-6)
    assert rep["grad_rel_max"] == pytest.approx(tt_rel(g, g64), rel=1e-9)
    assert rep["misfit_rel"] == pytest.approx(abs(L2 - L64) / L64, rel=1e-6, abs=1e-15)
    if mode == "fast":
        assert rep["tt_rel"] <= TT_TOL


def test_full_size_fast_traveltimes_against_fp64(R):
    """1700 x 350, 8 of the benchmark's shots: fast-mode traveltimes against
    the GPU FP64 oracle (itself pinned to the CPU FP64 oracle on one shot) are
    no further from FP64 than the reference's own float arithmetic
    (reference mode, bit-exact with the reference) on the same shots."""
    w = synth.grad_1700x350(nshots=100, ntr=850)
    idx = np.arange(0, 100, 13)[:8]
    sx, sz = w.srcx[idx], w.srcz[idx]
    TT = {m: ctx_for(R, w, m, vp=w.vp_start).forward(sx, sz)[0] for m in ("fast", "reference")}
    TT64, _ = ctx_for(R, w, "fast", vp=w.vp_start).forward_f64(sx, sz)
    for i in range(len(idx)):
        e_fast, e_ref = tt_rel(TT["fast"][i], TT64[i]), tt_rel(TT["reference"][i], TT64[i])
        assert e_fast <= e_ref * (1 + 1e-3) + 1e-7, (i, e_fast, e_ref)
        assert e_fast <= 2.5e-5 and rel_l2(TT["fast"][i], TT64[i]) <= 1.5e-5
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    t64, _ = O.eikonal_f64(p, synth.slowness(w.vp_start).astype(np.float64), sx[0], sz[0])
    assert np.array_equal(TT64[0], t64)


def test_small_grid_fast_traveltimes_within_1e5_of_fp64(R):
    w = synth.small_case(31, 200, 150, nshots=3)
    ctx = ctx_for(R, w, "fast")
    TT, _, _ = ctx.forward(w.srcx, w.srcz)
    TT64, _ = ctx.forward_f64(w.srcx, w.srcz)
    assert max(tt_rel(TT[i], TT64[i]) for i in range(3)) <= TT_TOL


def test_full_size_error_check_gates(R):
    """The benchmark workload's 100 shots through rz_set_error_check: fast
    traveltimes no further from FP64 than the reference's own float
    arithmetic; Leung-Qian gradient no further than twice the reference's
    plus 1e-4."""
    w = synth.grad_1700x350(nshots=100, ntr=850)
    tobs_ctx = ctx_for(R, w, "fast")
    _, Tobs, _ = tobs_ctx.forward(w.srcx, w.srcz, want_tt=False)
    reps = {}
    for mode, kind in (("reference", "reference"), ("fast", "reference"), ("fast", "exact")):
        ctx = ctx_for(R, w, mode, vp=w.vp_start, kind=kind)
        ctx.set_error_check(True)
        ctx.grad_obj(w.srcx, w.srcz, Tobs)
        reps[mode, kind] = ctx.error_report()
    fast, ref, ex = reps["fast", "reference"], reps["reference", "reference"], reps["fast", "exact"]
    assert fast["shots"] == 100 and ref["shots"] == 100
    assert fast["tt_rel"] <= ref["tt_rel"] * (1 + 1e-3) + 1e-7 and ex["tt_rel"] == fast["tt_rel"]
    assert fast["grad_rel_l2"] <= 2 * ref["grad_rel_l2"] + GRAD_TOL
    # the exact gradient of the float misfit: its residuals carry the float
    # traveltimes' path error (misfit 5.6e-4 from FP64), ~3e-3 here
    assert ex["grad_rel_l2"] <= 5e-3


# ---------------------------------------------------------------------------
# traveltime refinement (rz_set_refine)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("mode", ["fast", "reference"])
def test_refined_traveltimes_reach_fp64(R, mode):
    """With refinement the float traveltimes are the FP64 fixpoint rounded to
    float: within 1e-7 of FP64 at the benchmark size (1700 x 350), where the
    unrefined float fields sit ~2e-5 away."""
    w = synth.grad_1700x350(nshots=100, ntr=850)
    idx = np.arange(0, 100, 13)[:8]
    sx, sz = w.srcx[idx], w.srcz[idx]
    ctx = ctx_for(R, w, mode, vp=w.vp_start, refine=True)
    TT, Tmod, _ = ctx.forward(sx, sz)
    TT64, Tmod64 = ctx.forward_f64(sx, sz)
    errs = [tt_rel(TT[i], TT64[i]) for i in range(len(idx))]
    assert max(errs) <= 1e-7, errs
    assert tt_rel(Tmod, Tmod64) <= 1e-7


def test_refined_exact_gradient_within_1e4_at_full_size(R):
    """The benchmark's 100 shots: the exact gradient of refined traveltimes is
    within 1e-4 (relative L2) of the FP64 oracle's exact gradient, and the
    misfit within 1e-6; the Leung-Qian gradient of refined traveltimes stays
    no further from FP64 than the unrefined one."""
    w = synth.grad_1700x350(nshots=100, ntr=850)
    _, Tobs, _ = ctx_for(R, w, "fast").forward(w.srcx, w.srcz, want_tt=False)
    reps = {}
    for kind, refine in (("exact", True), ("reference", True), ("reference", False)):
        ctx = ctx_for(R, w, "fast", vp=w.vp_start, kind=kind, refine=refine)
        ctx.set_error_check(True)
        ctx.grad_obj(w.srcx, w.srcz, Tobs)
        reps[kind, refine] = ctx.error_report()
    ex = reps["exact", True]
    assert ex["shots"] == 100 and ex["tt_rel"] <= 1e-7
    assert ex["grad_rel_l2"] <= GRAD_TOL and ex["misfit_rel"] <= 1e-5
    assert reps["reference", True]["grad_rel_l2"] <= reps["reference", False]["grad_rel_l2"]


@pytest.mark.parametrize("nx,ny", [(5, 4), (33, 31), (70, 600), (257, 40)])
def test_refined_paths_on_odd_and_banded_shapes(R, nx, ny):
    """Shapes that are not multiples of the 32-row strip or 32-column block,
    a 5 x 4 grid, and a 600-row grid swept in bands, on rough random models
    with interior sources: refined traveltimes are within 3e-7 of the FP64
    fixpoint, and the exact gradient of refined traveltimes within 1e-4 of
    the FP64 exact gradient (error report of the same call).  On these models
    the TTNORM-stopped iterate lies up to 1.7e-5 from the fixpoint (70 x 600),
    so the one linear solve starts where upwind choices still flip at
    near-ties; 3e-7 covers what that leaves (2.0e-7 measured)."""
    w = synth.small_case(700 + nx, nx, ny, nshots=3)
    Tobs = picks(R, w)
    ctx = ctx_for(R, w, "fast", kind="exact", refine=True)
    ctx.set_error_check(True)
    ctx.grad_obj(w.srcx, w.srcz, Tobs)
    rep = ctx.error_report()
    assert rep["shots"] == 3 and rep["tt_rel"] <= 3e-7, rep
    assert rep["grad_rel_l2"] <= GRAD_TOL, rep


def test_refined_error_check_compares_with_the_fixpoint(R):
    """The error check of a refined call runs the FP64 forward to the fixpoint
    of the discrete equations, that of an unrefined call stops at TTNORM as the
    reference does: on a rough 70 x 600 model the refined field is within 3e-7
    of the first, while the reference's float field (8-9 passes, as the
    TTNORM-stopped FP64 run; the fixpoint takes 19-22) is within 1.2e-6 of the
    second and 1.7e-5 from the first (the CPU oracles measure the same)."""
    w = synth.small_case(770, 70, 600, nshots=3)
    ctx = ctx_for(R, w, "fast", refine=True)
    ctx.set_error_check(True)
    TT1, _, _ = ctx.forward(w.srcx, w.srcz)
    assert ctx.error_report()["tt_rel"] <= 3e-7
    ctx0 = ctx_for(R, w, "reference")
    ctx0.set_error_check(True)
    TT0, _, _ = ctx0.forward(w.srcx, w.srcz)
    assert ctx0.error_report()["tt_rel"] <= 2e-6
    T64, _ = ctx_for(R, w, "fast", ttnorm=1e-30).forward_f64(w.srcx, w.srcz)
    assert tt_rel(TT1, T64) <= 3e-7
    assert tt_rel(TT0, T64) >= 1e-5


def test_refined_exact_gradient_central_differences_config2(R):
    """<g, dS> of the refined exact gradient against central differences of
    the FP64 misfit (GPU FP64 oracle) on 20 random slowness perturbations, 16
    of the benchmark's shots on 1700 x 350 with 850 receivers, as the relative
    L2 error of the 20 directional derivatives.  The realised perturbation is
    the difference of the two float models, so the float rounding of
    S +- eps dS does not enter."""
    w = synth.grad_1700x350(nshots=100, ntr=850)
    idx = np.linspace(0, 99, 16).round().astype(int)
    sx, sz = w.srcx[idx], w.srcz[idx]
    _, Tobs, _ = ctx_for(R, w, "fast").forward(sx, sz, want_tt=False)
    g_vp, _ = ctx_for(R, w, "fast", vp=w.vp_start, kind="exact", refine=True).grad_obj(sx, sz, Tobs)
    S = synth.slowness(w.vp_start)
    g_s = -np.asarray(g_vp, np.float64) / (S.astype(np.float64) ** 2)
    cm = R.Context(0, "fp64")
    cm.set_grid(w.nx, w.ny, w.dh, w.time, 1e-14, w.eps_adj)
    cm.set_receivers(w.recx, w.recz)
    rng = np.random.default_rng(20)
    fds, projs = [], []
    for _ in range(20):
        d = rng.standard_normal(S.shape) * S
        sp, sm = (S + 1e-6 * d).astype(np.float32), (S - 1e-6 * d).astype(np.float32)
        step = (sp.astype(np.float64) - sm.astype(np.float64)) / 2
        cm.set_slowness(sp)
        jp = cm.misfit(sx, sz, Tobs)
        cm.set_slowness(sm)
        jm = cm.misfit(sx, sz, Tobs)
        fds.append((jp - jm) / 2)
        projs.append(float((g_s * step).sum()))
    fds, projs = np.array(fds), np.array(projs)
    # over the 20 directions (a single random direction can be nearly
    # orthogonal to the gradient, which inflates its own relative error)
    assert np.linalg.norm(fds - projs) / np.linalg.norm(fds) <= GRAD_TOL


def test_exact_and_reference_gradients_agree_in_direction(R):
    """The reference's Leung-Qian gradient (ass_grad.c: lambda S^3, the
    adjoint of the continuous problem with the residuals scaled by dT/dz) and
    the exact dJ/dVp of the discrete misfit, on the benchmark workload's
    interior: the measured cosine and scale ratio, kept within bands."""
    w = synth.grad_1700x350(nshots=100, ntr=850)
    idx = np.linspace(0, 99, 16).round().astype(int)
    sx, sz = w.srcx[idx], w.srcz[idx]
    _, Tobs, _ = ctx_for(R, w, "fast").forward(sx, sz, want_tt=False)
    ge, _ = ctx_for(R, w, "fast", vp=w.vp_start, kind="exact", refine=True).grad_obj(sx, sz, Tobs)
    gr, _ = ctx_for(R, w, "reference", vp=w.vp_start).grad_obj(sx, sz, Tobs)
    a, b = ge[2:-2, 2:-2].astype(np.float64), gr[2:-2, 2:-2].astype(np.float64)
    cos = float((a * b).sum() / np.linalg.norm(a) / np.linalg.norm(b))
    scale = float(np.linalg.norm(b) / np.linalg.norm(a))
    assert 0.6 <= cos <= 0.8, cos
    assert 0.02 <= scale <= 0.08, scale
