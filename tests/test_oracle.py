"""CPU tests of the oracle: the C restatement against the reference's own
compiled code and against the committed golden fixtures."""
import ctypes as C
import glob
import hashlib
import os

import numpy as np
import pytest

from rajzel_gb300 import synth

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def _params(O, d):
    return O.Params(int(d["nx"]), int(d["ny"]), float(d["dh"]), float(d["time"]), float(d["ttnorm"]),
                    float(d["eps_adj"]))


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "fwd_*.npz"))))
def test_port_forward_matches_golden(oracle_mod, path):
    O = oracle_mod
    d = np.load(path)
    if str(d["kind"]) == "forward_digest":
        w = synth.fwd_500x174()
        p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
        TT, it = O.eikonal(p, synth.slowness(w.vp_true), w.srcx[0], w.srcz[0])
        assert digest(TT) == str(d["TT_sha256"])
        assert np.array_equal(O.calc_fa(p, TT, w.recx, w.recz), d["Tmod"])
        assert it == int(d["passes"])
        return
    p = _params(O, d)
    S = synth.slowness(d["vp"])
    for i in range(len(d["srcx"])):
        TT, it = O.eikonal(p, S, d["srcx"][i], d["srcz"][i])
        assert digest(TT) == str(d["TT_sha256"][i])
        if "TT" in d:
            assert np.array_equal(TT, d["TT"][i])
        assert np.array_equal(O.calc_fa(p, TT, d["recx"], d["recz"]), d["Tmod"][i])
        assert it == d["passes"][i]


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "grad_*.npz"))))
def test_port_gradient_matches_golden(oracle_mod, path):
    O = oracle_mod
    d = np.load(path)
    p = _params(O, d)
    S = synth.slowness(d["vp"])
    grad, L2, fp, ap, Tres_last = O.grad_obj(p, S, d["srcx"], d["srcz"], d["recx"], d["recz"], d["Tobs"])
    assert digest(grad) == str(d["grad_sha256"])
    assert L2 == float(d["L2"])
    assert np.array_equal(Tres_last, d["Tres_last"])
    TT, _ = O.eikonal(p, S, d["srcx"][0], d["srcz"][0])
    Tmod = O.calc_fa(p, TT, d["recx"], d["recz"])
    Tres, _ = O.calc_res(p, TT, Tmod, d["Tobs"][0], d["recx"], d["recz"])
    assert np.array_equal(Tres, d["shot0_Tres"])
    lam, it = O.eikonal_adj(p, TT, Tres, d["recx"], d["recz"])
    assert digest(lam) == str(d["shot0_lam_sha256"])
    assert it == int(d["shot0_adj_passes"])


def _random_case(rng):
    nx, ny = int(rng.integers(4, 70)), int(rng.integers(4, 50))
    dh = float(rng.choice([5.0, 10.0, 12.5, 20.0]))
    w = synth.small_case(int(rng.integers(1 << 30)), nx, ny, dh=dh, nshots=3)
    return w


@pytest.mark.parametrize("seed", range(6))
def test_port_equals_reference_random(oracle_mod, seed):
    """The restatement and the reference's compiled sources agree bit for bit."""
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference sources not present on this machine")
    rng = np.random.default_rng(100 + seed)
    w = _random_case(rng)
    ttnorm = float(rng.choice([1e-6, 1e-10]))
    p = O.Params(w.nx, w.ny, w.dh, w.time, ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    ref = O.Ref(p)
    for i in range(3):
        TTr, Tm, itr = ref.eikonal(S, w.srcx[i], w.srcz[i], w.recx, w.recz)
        TTp, itp = O.eikonal(p, S, w.srcx[i], w.srcz[i])
        assert np.array_equal(TTr, TTp) and itr == itp
        Tobs = (Tm * (1 + 0.02 * rng.standard_normal(w.ntr))).astype(np.float32)
        Tobs[rng.random(w.ntr) < 0.1] = -1.0
        Tr_r, _ = ref.calc_res(TTr, Tm, Tobs, w.recx, w.recz)
        Tr_p, _ = O.calc_res(p, TTp, Tm, Tobs, w.recx, w.recz)
        assert np.array_equal(Tr_r, Tr_p)
        Lr, itr = ref.eikonal_adj(TTr, Tr_r, w.recx, w.recz)
        Lp, itp = O.eikonal_adj(p, TTp, Tr_p, w.recx, w.recz)
        assert np.array_equal(Lr, Lp) and itr == itp
    Tobs = np.abs(rng.normal(1.0, 0.5, (3, w.ntr))).astype(np.float32)
    Tobs[rng.random(Tobs.shape) < 0.1] = -1.0  # muted picks: Tres carries over between shots
    gr, L2r, Tres_r = ref.grad_obj(S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    gp, L2p, _, _, Tres_p = O.grad_obj(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert np.array_equal(gr, gp) and L2r == L2p and np.array_equal(Tres_r, Tres_p)


def test_fp64_oracle_close_to_float(oracle_mod):
    O = oracle_mod
    w = synth.small_case(5, 60, 40, nshots=1)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    t32, _ = O.eikonal(p, S, w.srcx[0], w.srcz[0])
    t64, _ = O.eikonal_f64(p, S.astype(np.float64), w.srcx[0], w.srcz[0])
    assert np.abs(t32 - t64).max() / np.abs(t64).max() < 1e-5


def test_ttnorm_iterate_and_fixpoint_differ_on_rough_models(oracle_mod):
    """The FP64 oracle stopped by TTNORM (a mean change of 1e-6 s per pass) is
    not the fixpoint of the discrete equations on a rough random model with
    interior sources: on 70 x 600 it stops after 8-9 passes, 1.7e-5 (relative,
    max norm) from the fixpoint that 19-22 passes reach, because single cells
    still moving by ~1e-6 s vanish in the grid mean.  Refined traveltimes
    approximate the fixpoint, so their error check runs the FP64 forward to
    it."""
    O = oracle_mod
    w = synth.small_case(770, 70, 600, nshots=3)
    S = synth.slowness(w.vp_true).astype(np.float64)
    stop = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    fix = O.Params(w.nx, w.ny, w.dh, w.time, 1e-30, w.eps_adj)
    diffs, passes = [], []
    for i in range(3):
        ta, pa = O.eikonal_f64(stop, S, w.srcx[i], w.srcz[i])
        tb, pb = O.eikonal_f64(fix, S, w.srcx[i], w.srcz[i])
        diffs.append(np.abs(ta - tb).max() / np.abs(tb).max())
        passes.append((pa, pb))
    assert max(diffs) > 1e-5 and min(diffs) > 1e-6
    assert all(pb > 2 * pa for pa, pb in passes)


def test_pow_cube_pin(oracle_mod):
    """ass_grad.c:23 uses libm pow(S,3.0); it is faithful but not always the
    correctly rounded cube, which is why the reference-mode GPU stack takes
    the per-cell cube from the host C library.  The count is recorded."""
    O = oracle_mod
    lib = C.CDLL(O.PORT_SO)
    lib.rzo_pin_cube.argtypes = [C.c_float, C.c_float]
    lib.rzo_pin_cube.restype = C.c_long
    n = lib.rzo_pin_cube(1.0 / 5000.0, 1.0 / 4000.0)
    assert n >= 0


def test_shot_partition_matches_init_mpishot(oracle_mod):
    """init_MPIshot.c:19-30: contiguous blocks, the first nshots%NP ranks get one more."""
    O = oracle_mod
    for nshots, np_ in [(100, 8), (7, 3), (5, 5), (3, 4)]:
        spans = [O.shot_partition(nshots, np_, r) for r in range(np_)]
        assert spans[0][0] == 1 and spans[-1][1] == nshots + 1
        assert all(spans[i][1] == spans[i + 1][0] for i in range(np_ - 1))
        sizes = [b - a for a, b in spans]
        assert max(sizes) - min(sizes) <= 1 and sizes == sorted(sizes, reverse=True)


@pytest.mark.parametrize("nx,ny", [(5, 5), (5, 9), (6, 5), (7, 11), (20, 13), (64, 33)])
def test_frame_copy_is_the_cell_two_inside(oracle_mod, nx, ny):
    """cp_grad_frame.c:18-49 leaves in every cell the value of the cell
    nearest to it two cells inside the grid (for nx, ny >= 5), and a second
    application changes nothing: the rule by which the stack of a one-chunk
    batch writes the frame cells itself."""
    O = oracle_mod
    p = O.Params(nx, ny, 10.0, 20.0)
    rng = np.random.default_rng(nx * 100 + ny)
    A = np.zeros((ny, nx), np.float32)
    A[1:-1, 1:-1] = rng.standard_normal((ny - 2, nx - 2)).astype(np.float32)
    framed = O.cp_grad_frame(p, A)
    k, h = np.clip(np.arange(ny), 2, ny - 3), np.clip(np.arange(nx), 2, nx - 3)
    assert np.array_equal(framed, A[np.ix_(k, h)])
    assert np.array_equal(O.cp_grad_frame(p, framed), framed)
    if O.ref_available():
        assert np.array_equal(O.Ref(p).cp_grad_frame(A), framed)


def _fd_case(O, seed, nx, ny, nshots, muted=False):
    w = synth.small_case(seed, nx, ny, nshots=nshots)
    p = O.Params(w.nx, w.ny, w.dh, w.time, 1e-14, w.eps_adj)
    vp = w.vp_true.astype(np.float64)
    Tobs = np.empty((nshots, w.ntr))
    for i in range(nshots):
        t, _ = O.eikonal_f64(p, 1.0 / (vp * 1.03), w.srcx[i], w.srcz[i])
        Tobs[i] = t[w.recz - 1, w.recx - 1]
    if muted:
        Tobs[:, ::5] = -1.0
    return w, p, vp, Tobs


@pytest.mark.parametrize("muted", [False, True])
def test_exact_adjoint_oracle_matches_finite_differences(oracle_mod, muted):
    """The FP64 exact discrete adjoint (cells visited in order of decreasing
    traveltime) against central differences of the FP64 misfit along random
    slowness perturbations."""
    O = oracle_mod
    w, p, vp, Tobs = _fd_case(O, 5, 48, 36, 2, muted)
    S = 1.0 / vp
    g_vp, L2 = O.grad_exact_f64(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    assert L2 == pytest.approx(O.misfit_f64(p, S, w.srcx, w.srcz, w.recx, w.recz, Tobs), rel=1e-15)
    g_s = -g_vp * vp * vp  # dJ/dS = dJ/dVp * dVp/dS
    rng = np.random.default_rng(1)
    for _ in range(4):
        d = rng.standard_normal(S.shape) * S
        eps = 1e-6
        jp = O.misfit_f64(p, S + eps * d, w.srcx, w.srcz, w.recx, w.recz, Tobs)
        jm = O.misfit_f64(p, S - eps * d, w.srcx, w.srcz, w.recx, w.recz, Tobs)
        fd = (jp - jm) / (2 * eps)
        assert abs(fd - (g_s * d).sum()) <= 1e-6 * abs(fd)


# ---------------------------------------------------------------------------
# FATT and preconditioning: the restatement against the reference's own
# compiled fatt(), LBFGS.c, wolfels.c, check_descent.c, precond.c,
# gauss_filt.c and taper_grad.c
# ---------------------------------------------------------------------------
def _fatt_case(O, seed, nx, ny, ns, pert):
    """Picks from the true model; start = the true model with a smooth slow
    anomaly (the reference's l-BFGS makes progress on these)."""
    w = synth.small_case(seed, nx, ny, nshots=ns)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S_true = synth.slowness(w.vp_true)
    Tobs = np.stack([O.calc_fa(p, O.eikonal(p, S_true, w.srcx[i], w.srcz[i])[0], w.recx, w.recz) for i in range(ns)])
    yy, xx = np.mgrid[0:ny, 0:nx]
    bump = np.exp(-(((xx - nx / 2) / (nx / 5)) ** 2 + ((yy - ny / 2) / (ny / 5)) ** 2))
    vp0 = (w.vp_true * (1 - pert * bump)).astype(np.float32)
    return w, p, Tobs, vp0


FATT_OPTS = dict(itermax=6, nlbfgs=3, stepmax=8, eps_scale=0.01, c1=1e-4, c2=0.9, scalefac=2.0, vp_lo=1000.0,
                 vp_hi=6000.0, pro=0.0, spatfilter=0, filt_size_grad=0, filt_size_grad1=0, taper_hor=0, gradt1=1,
                 gradt2=1, exp_taper_grad_hor=0.0, recursion=0)


@pytest.mark.parametrize("seed,nx,ny,ns,pert,taper", [(56, 60, 40, 4, 0.08, 0), (57, 80, 50, 5, 0.1, 0),
                                                      (57, 80, 50, 5, 0.1, 1)])
def test_fatt_restatement_equals_reference_fatt(oracle_mod, seed, nx, ny, ns, pert, taper):
    """One FATT stage (l-BFGS in slot order, weak-Wolfe line search, model
    limits, the horizontal taper) by the restatement in the reference's own
    precision equals the reference's compiled fatt() bit for bit: the misfit
    of every gradient evaluation in call order and the final model."""
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference sources not present on this machine")
    from oracle import fatt as F
    w, p, Tobs, vp0 = _fatt_case(O, seed, nx, ny, ns, pert)
    o = dict(FATT_OPTS, taper_hor=taper, gradt1=3, gradt2=8, exp_taper_grad_hor=0.5)
    vr, mr, steps, evr = O.Ref(p).fatt(vp0, w.srcx, w.srcz, w.recx, w.recz, Tobs, o)
    trace = []
    vq, mq, it, ev = F.fatt(p, vp0, w.srcx, w.srcz, w.recx, w.recz, Tobs, o, precision="reference", trace=trace)
    assert len(mr) >= 3 and it == len(mr) and ev == len(evr)
    assert np.array_equal(np.array(trace), evr)  # exact misfits of every evaluation
    assert np.allclose(mq, mr, rtol=5e-7, atol=0)  # fatt.c's log prints %e (7 digits)
    assert np.array_equal(vq, vr)


@pytest.mark.parametrize("fs,fs1,taper", [(6, 4, 0), (7, 5, 1), (12, 9, 0), (0, 0, 1)])
def test_precond_restatement_matches_reference(oracle_mod, fs, fs1, taper):
    """precond() with SPATFILTER 4 (gauss_filt.c, even sizes rounded up) and
    the horizontal taper (taper_grad.c sws 2): the restatement's Gaussian
    accumulates in double, the reference's in float (1e-6 relative); the
    taper alone is bit-exact."""
    O = oracle_mod
    if not O.ref_available():
        pytest.skip("reference sources not present on this machine")
    from oracle import fatt as F
    w = synth.small_case(61, 70, 45, nshots=1)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    g = np.random.default_rng(fs + fs1).standard_normal((w.ny, w.nx)).astype(np.float32)
    o = dict(FATT_OPTS, spatfilter=4 if fs else 0, filt_size_grad=fs, filt_size_grad1=fs1, taper_hor=taper, gradt1=3,
             gradt2=8, exp_taper_grad_hor=1.0)
    a = O.Ref(p).precond(g, o)
    b = F.precond(g, o, p.dh)
    if fs == 0:
        assert np.array_equal(a, b)
    else:
        assert np.abs(a - b).max() <= 1e-6 * np.abs(a).max()
