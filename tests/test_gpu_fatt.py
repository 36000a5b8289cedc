"""GPU tests of the FATT loop (rz_fatt) and gradient preconditioning
(rz_precond) against the CPU restatement in oracle/fatt.py."""
import numpy as np
import pytest

import oracle as O
from oracle import fatt as OF
from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R(gpu_lib):
    O.build(ref=False)
    return gpu_lib


def make(R, w, mode):
    ctx = R.Context(0, mode)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_receivers(w.recx, w.recz)
    return ctx


@pytest.mark.parametrize("fs,fs1,taper", [(10, 6, False), (7, 12, True), (0, 5, True), (80, 40, False)])
def test_precond_matches_oracle(R, fs, fs1, taper):
    """Separable GPU Gaussian filter + taper against the reference's direct 2-D
    convolution (float accumulation on the GPU: 1e-5 relative)."""
    w = synth.small_case(3, 150, 90, nshots=1)
    ctx = make(R, w, "fast")
    rng = np.random.default_rng(fs + fs1)
    g = rng.standard_normal((w.ny, w.nx)).astype(np.float32)
    opts = dict(spatfilter=4, filt_size_grad=fs, filt_size_grad1=fs1, taper_hor=int(taper), gradt1=5, gradt2=14,
                exp_taper_grad_hor=0.5)
    got = ctx.precond(g, **opts)
    want = OF.precond(g, opts, w.dh)
    scale = np.abs(want).max()
    assert np.abs(got - want).max() <= 1e-5 * scale


def fatt_case(sub=8, nshots=8):
    """The FATT model at 1/sub resolution; picks from the true model, start = its depth average."""
    w = synth.fatt_small(sub=sub, nshots=nshots)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S_true = synth.slowness(w.vp_true)
    Tobs = np.empty((nshots, w.ntr), np.float32)
    for i in range(nshots):
        t, _ = O.eikonal(p, S_true, w.srcx[i], w.srcz[i])
        Tobs[i] = O.calc_fa(p, t, w.recx, w.recz)
    return w, p, Tobs, w.vp_start


@pytest.mark.parametrize("recursion", [0, 1])
def test_fatt_matches_oracle_loop(R, recursion):
    """Reference-mode gradients are bit-exact, so the GPU loop and the CPU
    restatement follow the same trajectory up to the summation order of
    their double dot products."""
    w, p, Tobs, start = fatt_case()
    opts = dict(itermax=5, nlbfgs=3, recursion=recursion, vp_lo=1000.0, vp_hi=6000.0)
    ctx = make(R, w, "reference")
    vp_g, mis_g, it_g, ev_g, _ = ctx.fatt(w.srcx, w.srcz, Tobs, start, **opts)
    full = R.fatt_opts(**opts)
    o = {f: getattr(full, f) for f, _ in R.FattOpts._fields_}
    vp_o, mis_o, it_o, ev_o = OF.fatt(p, start, w.srcx, w.srcz, w.recx, w.recz, Tobs, o)
    assert (it_g, ev_g) == (it_o, ev_o)
    np.testing.assert_allclose(mis_g, mis_o, rtol=1e-5)
    assert np.abs(vp_g - vp_o).max() <= 1e-4 * np.abs(vp_o).max()


def test_fatt_fast_mode_reduces_misfit_and_model_error(R):
    w, p, Tobs, start = fatt_case(sub=4, nshots=12)
    ctx = make(R, w, "fast")
    vp, mis, it, ev, _ = ctx.fatt(w.srcx, w.srcz, Tobs, start, itermax=8, nlbfgs=5, vp_lo=1000.0, vp_hi=6000.0,
                               recursion=1)
    assert it >= 3 and ev >= it
    assert mis[-1] < 0.5 * mis[0]
    err0 = np.linalg.norm(start - w.vp_true)
    err1 = np.linalg.norm(vp - w.vp_true)
    assert err1 < err0


def test_fatt_rejects_bad_options(R):
    w, p, Tobs, start = fatt_case(sub=16, nshots=1)
    ctx = make(R, w, "fast")
    with pytest.raises(R.RajzelError):
        ctx.fatt(w.srcx, w.srcz, Tobs, start, itermax=0)
    with pytest.raises(R.RajzelError):
        ctx.fatt(w.srcx, w.srcz, Tobs, start, recursion=7)
