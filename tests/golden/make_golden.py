"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference's own C sources (compiled unmodified into
oracle/_ref/libref.so by oracle/Makefile) on small seeded synthetic inputs and
stores inputs and outputs.  Large outputs are stored as SHA-256 digests of
their float32 bytes; bit-exact comparisons only need the digest.

    python tests/golden/make_golden.py      # needs the reference sources

The fixtures are committed; this script is how they were made.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from rajzel_gb300 import synth  # noqa: E402


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def case_forward(name, nx, ny, dh, seed, nsrc=3, store_full=True):
    w = synth.small_case(seed, nx, ny, dh=dh, nshots=nsrc)
    S = synth.slowness(w.vp_true)
    p = O.Params(nx, ny, dh, w.time, w.ttnorm, w.eps_adj)
    ref = O.Ref(p)
    out = dict(kind="forward", nx=nx, ny=ny, dh=dh, time=w.time, ttnorm=w.ttnorm, eps_adj=w.eps_adj, vp=w.vp_true,
               srcx=w.srcx, srcz=w.srcz, recx=w.recx, recz=w.recz)
    TTs, Tmods, passes = [], [], []
    for i in range(nsrc):
        TT, Tmod, it = ref.eikonal(S, w.srcx[i], w.srcz[i], w.recx, w.recz)
        TTs.append(TT)
        Tmods.append(Tmod)
        passes.append(it)
    if store_full:
        out["TT"] = np.stack(TTs)
    out["TT_sha256"] = np.array([digest(t) for t in TTs])
    out["Tmod"] = np.stack(Tmods)
    out["passes"] = np.array(passes, np.int32)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def case_gradient(name, nx, ny, dh, seed, nsrc=3, mute=0.0, store_full=True):
    w = synth.small_case(seed, nx, ny, dh=dh, nshots=nsrc)
    S = synth.slowness(w.vp_true)
    p = O.Params(nx, ny, dh, w.time, w.ttnorm, w.eps_adj)
    ref = O.Ref(p)
    rng = np.random.default_rng(seed + 1000)
    Tobs = np.empty((nsrc, w.ntr), np.float32)
    for i in range(nsrc):
        _, Tmod, _ = ref.eikonal(S * np.float32(1.03), w.srcx[i], w.srcz[i], w.recx, w.recz)
        Tobs[i] = Tmod * (1.0 + 0.01 * rng.standard_normal(w.ntr)).astype(np.float32)
    if mute > 0:
        Tobs[rng.random(Tobs.shape) < mute] = -1.0
    grad, L2, Tres_last = ref.grad_obj(S, w.srcx, w.srcz, w.recx, w.recz, Tobs)
    out = dict(kind="gradient", nx=nx, ny=ny, dh=dh, time=w.time, ttnorm=w.ttnorm, eps_adj=w.eps_adj, vp=w.vp_true,
               srcx=w.srcx, srcz=w.srcz, recx=w.recx, recz=w.recz, Tobs=Tobs, L2=np.float64(L2),
               grad_sha256=np.array(digest(grad)), Tres_last=Tres_last)
    if store_full:
        out["grad"] = grad
    # per-shot adjoint fields of the first shot (inputs from the reference's own forward)
    TT, Tmod, _ = ref.eikonal(S, w.srcx[0], w.srcz[0], w.recx, w.recz)
    Tres, _ = ref.calc_res(TT, Tmod, Tobs[0], w.recx, w.recz)
    lam, it = ref.eikonal_adj(TT, Tres, w.recx, w.recz)
    out.update(shot0_Tres=Tres, shot0_lam_sha256=np.array(digest(lam)), shot0_adj_passes=np.int32(it))
    if store_full:
        out["shot0_lam"] = lam
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)


def main():
    if not O.ref_available():
        O.build(ref=True)
    if not O.ref_available():
        sys.exit("reference sources not available: cannot regenerate fixtures")
    case_forward("fwd_45x33", 45, 33, 10.0, seed=11)
    case_forward("fwd_97x70", 97, 70, 12.5, seed=12)
    case_forward("fwd_3x3", 3, 3, 10.0, seed=13, nsrc=2)
    case_gradient("grad_40x30", 40, 30, 10.0, seed=21)
    case_gradient("grad_100x77", 100, 77, 10.0, seed=22)
    case_gradient("grad_64x64_muted", 64, 64, 20.0, seed=23, mute=0.15)
    # the 500 x 174 forward workload: digests only (87,000 cells)
    w = synth.fwd_500x174()
    S = synth.slowness(w.vp_true)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    TT, Tmod, it = O.Ref(p).eikonal(S, w.srcx[0], w.srcz[0], w.recx, w.recz)
    np.savez_compressed(os.path.join(HERE, "fwd_500x174.npz"), kind="forward_digest", TT_sha256=np.array(digest(TT)),
                        Tmod=Tmod, passes=np.int32(it), TT_row2=TT[1].copy(), TT_col250=TT[:, 249].copy())
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
