"""CPU tests of the RAJZEL file formats (include/rajzel_io.h)."""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
import rzio

# the reference tree's example parameter files, beside its sources (absent on the GPU machine)
REF_PAR = os.path.join(os.path.dirname(oracle.REF_SRC.rstrip("/")), "par")


@pytest.fixture(scope="module")
def L():
    return rzio.lib()


def test_par_file_positional(L, tmp_path):
    p = tmp_path / "a.inp"
    rzio.write_inp(p, INVMAT=2, NX=123, NY=45, DH=12.5, TIME=7.0, SOURCE_FILE="src/s.dat", REC_FILE="rec/r.dat",
                   REFREC="10.0 , -2.5", GRADT="4, 6, 100, 110", C1C2="2e-4, 0.85", VP0="1500.0, 2501.0, 1.0")
    P = rzio.Par()
    assert L.rz_read_par(str(p).encode(), C.byref(P)) == 0, L.rz_io_error()
    assert P.nlines == 63
    assert (P.INVMAT, P.NX, P.NY) == (2, 123, 45)
    assert P.DH == np.float32(12.5) and P.TIME == np.float32(7.0)
    assert P.SOURCE_FILE == b"src/s.dat" and P.REC_FILE == b"rec/r.dat"
    assert list(P.REFREC) == [10.0, -2.5]
    assert (P.GRADT1, P.GRADT2, P.GRADT3, P.GRADT4) == (4, 6, 100, 110)
    assert P.C1 == np.float32(2e-4) and P.C2 == np.float32(0.85)
    assert (P.VP0_1, P.VP0_2, P.DVP0) == (1500.0, 2501.0, 1.0)
    assert P.GRIDSEARCH_FILE == b"grid.dat" and P.NLBFGS == 5 and P.LINESEARCH == 1


@pytest.mark.skipif(not os.path.isdir(REF_PAR), reason="reference parameter files not present")
def test_reference_example_parameter_file(L):
    P = rzio.Par()
    assert L.rz_read_par(os.path.join(REF_PAR, "RAJZEL_marm_OBC.inp").encode(), C.byref(P)) == 0, L.rz_io_error()
    assert P.nlines == 63
    assert (P.INVMAT, P.NX, P.NY, P.DH, P.TIME) == (0, 500, 174, 20.0, 6.0)
    assert P.TTNORM == np.float32(1e-10) and P.EPS_ADJ == np.float32(1e-9)
    assert (P.GRADT1, P.GRADT2, P.GRADT3, P.GRADT4) == (22, 25, 490, 500)
    assert P.C1 == np.float32(1e-4) and P.C2 == np.float32(0.9)
    assert (P.GRAD_METHOD, P.NLBFGS, P.LINESEARCH, P.STEPMAX) == (2, 20, 2, 10)
    assert (P.VP0_1, P.VP0_2, P.DVP0) == (1500.0, 2501.0, 1.0)
    pro, sf, wd, wd1, f1, f2, n = C.c_float(), C.c_int(), C.c_float(), C.c_float(), C.c_int(), C.c_int(), C.c_int()
    assert L.rz_read_workflow(os.path.join(REF_PAR, "FATT_workflow_marmousi.inp").encode(), 1, C.byref(pro),
                              C.byref(sf), C.byref(wd), C.byref(wd1), C.byref(f1), C.byref(f2), C.byref(n)) == 0
    assert (pro.value, sf.value, f1.value, f2.value, n.value) == (0.0, 4, 80, 40, 1)


def test_sources_and_receivers(L, tmp_path):
    s = tmp_path / "s.dat"
    rzio.write_sources(s, [800.0, 880.0, 960.5], [460.0, 20.0, 40.0])
    n = C.c_int()
    assert L.rz_read_sources(str(s).encode(), C.byref(n), None, None, 0) == 0 and n.value == 3
    x, z = np.zeros(3, np.float32), np.zeros(3, np.float32)
    assert L.rz_read_sources(str(s).encode(), C.byref(n), x.ctypes.data_as(C.c_void_p), z.ctypes.data_as(C.c_void_p),
                             3) == 0
    assert np.array_equal(x, [800.0, 880.0, 960.5]) and np.array_equal(z, [460.0, 20.0, 40.0])
    bad = tmp_path / "bad.dat"
    bad.write_text("1\n1.0 2.0 3.0 4.0 5.0\n")
    assert L.rz_read_sources(str(bad).encode(), C.byref(n), x.ctypes.data_as(C.c_void_p),
                             z.ctypes.data_as(C.c_void_p), 3) != 0
    assert b"Missing parameter" in L.rz_io_error()

    r = tmp_path / "r.dat"
    rzio.write_receivers(r, [0.0, 10.0, 24.9, 25.1, 100.0], [20.0, 20.0, 40.0, 40.0, 35.0])
    ref = (C.c_float * 2)(0.0, 0.0)
    nt = C.c_int()
    assert L.rz_read_receivers(str(r).encode(), C.c_float(10.0), ref, C.byref(nt), None, None, 0) == 0
    assert nt.value == 4  # x index 0 is dropped
    rx, rz = np.zeros(4, np.int32), np.zeros(4, np.int32)
    assert L.rz_read_receivers(str(r).encode(), C.c_float(10.0), ref, C.byref(nt), rx.ctypes.data_as(C.c_void_p),
                               rz.ctypes.data_as(C.c_void_p), 4) == 0
    assert list(rx) == [1, 2, 3, 10] and list(rz) == [2, 4, 4, 4]  # iround((x + REFREC)/DH)


def test_model_and_picks_round_trip(L, tmp_path):
    nx, ny = 7, 5
    vp = (np.arange(nx * ny, dtype=np.float32).reshape(ny, nx) + 1500.0)
    f = tmp_path / "m.vp"
    assert L.rz_write_model(str(f).encode(), nx, ny, vp.ctypes.data_as(C.c_void_p)) == 0
    raw = np.fromfile(f, np.float32)
    assert np.array_equal(raw[:ny], vp[:, 0])  # x outer, depth inner
    back = np.zeros_like(vp)
    assert L.rz_read_model(str(f).encode(), nx, ny, back.ctypes.data_as(C.c_void_p)) == 0
    assert np.array_equal(back, vp)
    t = np.array([0.1234567, 1.5, 2.0e-3], np.float32)
    pre = str(tmp_path / "p").encode()
    assert L.rz_write_picks(pre, 3, 3, t.ctypes.data_as(C.c_void_p)) == 0
    assert open(tmp_path / "p_3.dat").read().splitlines()[0] == "1.234567e-01 "
    got = np.zeros(3, np.float32)
    assert L.rz_read_picks(pre, 3, 3, got.ctypes.data_as(C.c_void_p)) == 0
    assert np.allclose(got, t, rtol=1e-6)
