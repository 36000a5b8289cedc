"""GPU tests of the rajzel_gpu driver on RAJZEL parameter directories
(INVMAT 0: forward modelling, 2: grid search, 1: FATT stage)."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import rzio
from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu
NX, NY, DH = 96, 40, 10.0


@pytest.fixture(scope="module")
def driver(gpu_lib):
    from rajzel_gb300 import build as B
    O.build(ref=False)
    B.build()
    return B.DRIVER


def setup_dir(root, **inp):
    rzio.makedirs(root, "src", "rec", "model", "picks", "obs", "tt", "log", "grad")
    rng = np.random.default_rng(4)
    z = np.arange(NY)[:, None] * DH
    vp = (1600.0 + 2.5 * z + 40.0 * rng.standard_normal((NY, NX)) * 0.1).astype(np.float32)
    vp = np.repeat(vp[:, :1], NX, axis=1) + (30.0 * np.sin(np.arange(NX) / 9.0)).astype(np.float32)[None, :]
    vp = vp.astype(np.float32)
    srcx = np.array([105.0, 330.0, 610.0, 880.0], np.float32)
    srcz = np.full(4, 20.0, np.float32)
    recx = np.arange(1, NX - 1, 2) * DH
    recz = np.full(len(recx), 20.0)
    rzio.write_sources(os.path.join(root, "src/s.dat"), srcx, srcz)
    rzio.write_receivers(os.path.join(root, "rec/r.dat"), recx, recz)
    rzio.write_model(os.path.join(root, "model/true.vp"), vp)
    rzio.write_inp(os.path.join(root, "par.inp"), NX=NX, NY=NY, DH=DH, TIME=10.0, SOURCE_FILE="src/s.dat",
                   REC_FILE="rec/r.dat", **inp)
    irx = np.floor(recx / DH + 0.5).astype(np.int32)
    irz = np.floor(recz / DH + 0.5).astype(np.int32)
    return vp, srcx, srcz, irx, irz


def run(driver, root, *args):
    r = subprocess.run([driver, "par.inp", *args], cwd=root, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr + r.stdout
    return r.stdout


def params():
    return O.Params(NX, NY, DH, 10.0, 1e-6, 1e-9)


def test_forward_modelling_writes_reference_picks_and_fields(driver, tmp_path):
    root = str(tmp_path)
    vp, srcx, srcz, irx, irz = setup_dir(root, INVMAT=0, SEISMO=1, SNAP=1)
    run(driver, root)
    p = params()
    S = synth.slowness(vp)
    for s in range(4):
        tt, _ = O.eikonal(p, S, srcx[s], srcz[s])
        tmod = O.calc_fa(p, tt, irx, irz)
        got = rzio.read_picks(os.path.join(root, "picks/picks"), s + 1)
        want = np.array([float("%e" % v) for v in tmod], np.float32)
        assert np.array_equal(got, want)
        field = rzio.read_model(os.path.join(root, f"tt/snap_shot_{s + 1}.tt"), NX, NY)
        assert np.array_equal(field, tt)


def test_grid_search_misfits(driver, tmp_path):
    root = str(tmp_path)
    vp, srcx, srcz, irx, irz = setup_dir(root, INVMAT=2, VP0="1550.0, 1750.0, 100.0", GRAD0="2.0, 3.0, 0.5")
    p = params()
    S = synth.slowness(vp)
    tobs = []
    for s in range(4):
        tt, _ = O.eikonal(p, S, srcx[s], srcz[s])
        t = O.calc_fa(p, tt, irx, irz)
        rzio.write_picks(os.path.join(root, "obs/picks"), s + 1, t)
        tobs.append(rzio.read_picks(os.path.join(root, "obs/picks"), s + 1))
    run(driver, root)
    lines = open(os.path.join(root, "grid.dat")).read().splitlines()
    assert lines[0].split() == ["Objfcn", "vp0", "grad0"]
    rows = [list(map(float, ln.split())) for ln in lines[1:]]
    assert len(rows) == 4  # ceil(200/100) x ceil(1/0.5)
    for L2, vp0, grad0 in rows:
        j = np.arange(1, NY + 1, dtype=np.float32)
        col = np.float32(grad0) * ((j - 1) * np.float32(DH)) + np.float32(vp0)
        model = np.repeat(col[:, None], NX, axis=1).astype(np.float32)
        Sm = synth.slowness(model)
        want = 0.0
        for s in range(4):
            tt, _ = O.eikonal(p, Sm, srcx[s], srcz[s])
            r = O.calc_fa(p, tt, irx, irz).astype(np.float64) - tobs[s]
            want += float((r.astype(np.float32) ** 2).astype(np.float64).sum())
        assert L2 == pytest.approx(0.5 * want, rel=2e-6)


def test_fatt_stage_matches_library_call(driver, gpu_lib, tmp_path):
    root = str(tmp_path)
    vp, srcx, srcz, irx, irz = setup_dir(root, INVMAT=1, ITERMAX=3, NLBFGS=3, MFILE="model/start")
    p = params()
    S = synth.slowness(vp)
    for s in range(4):
        tt, _ = O.eikonal(p, S, srcx[s], srcz[s])
        rzio.write_picks(os.path.join(root, "obs/picks"), s + 1, O.calc_fa(p, tt, irx, irz))
    start = np.repeat(vp.mean(axis=1, keepdims=True), NX, axis=1).astype(np.float32)
    rzio.write_model(os.path.join(root, "model/start.vp"), start)
    with open(os.path.join(root, "wf.inp"), "w") as f:
        f.write("PRO\tSPATFILTER\tWD_DAMP\t\tWD_DAMP1\tFILT_SIZE_GRAD\tFILT_SIZE_GRAD1\n")
        f.write("0.0\t0\t\t1e-3\t\t1e-3\t\t0\t\t0\n")
    run(driver, root, "wf.inp")
    final = rzio.read_model(os.path.join(root, "model/inv_vp_stage_1.bin"), NX, NY)
    log = [ln.split() for ln in open(os.path.join(root, "misfit.dat")).read().splitlines()]
    assert 1 <= len(log) <= 3 and all(row[2] == "1" for row in log)
    # the same stage through the library
    ctx = gpu_lib.Context(0, "reference")
    ctx.set_grid(NX, NY, DH, 10.0, 1e-6, 1e-9)
    ctx.set_receivers(irx, irz)
    tobs = np.stack([rzio.read_picks(os.path.join(root, "obs/picks"), s + 1) for s in range(4)])
    res = ctx.fatt(srcx, srcz, tobs, start, itermax=3, nlbfgs=3, stepmax=10, eps_scale=0.01, c1=1e-4, c2=0.9,
                   scalefac=2.0, vp_lo=1000.0, vp_hi=6000.0, pro=0.0, recursion=0)
    assert np.array_equal(final, res.vp)
    assert len(log) == res.iterations
    assert float(log[-1][1]) == pytest.approx(res.misfit[-1], rel=1e-6)
