"""CPU tests of host-side logic: seeded workloads, grid indexing, the
reference-compatible parameter conventions."""
import numpy as np

from rajzel_gb300 import synth


def test_grid_index_is_iround():
    # iround(x/DH) = floor(x/DH + 0.5) on float32 division (fd.h:18, eikonal.c:31)
    assert synth.grid_index(np.float32(5000.0), 20.0) == 250
    assert synth.grid_index(np.float32(29.999), 20.0) == 1
    assert synth.grid_index(np.float32(30.0), 20.0) == 2


def test_workloads_are_seeded_and_shaped():
    a, b = synth.grad_1700x350(nshots=4, ntr=10), synth.grad_1700x350(nshots=4, ntr=10)
    assert a.vp_true.shape == (350, 1700) and np.array_equal(a.vp_true, b.vp_true)
    assert a.vp_true.min() >= 1500 * 0.85 and a.vp_true.max() <= 4500 * 1.15
    assert (a.recz == 2).all() and a.recx.min() >= 1 and a.recx.max() <= 1700
    c = synth.fwd_500x174()
    assert c.vp_true.shape == (174, 500) and c.srcx[0] == 5000.0 and c.srcz[0] == 40.0


def test_slowness_matches_calc_s():
    vp = np.array([1500.0, 2345.6, 4999.9], np.float32)
    S = synth.slowness(vp)
    assert np.array_equal(S, (1.0 / vp.astype(np.float64)).astype(np.float32))


def test_uneven_grids_split():
    sizes = [synth.uneven_grid(i, nshots=2, ntr=4) for i in range(3)]
    assert [(w.nx, w.ny) for w in sizes] == [(512, 256), (1024, 512), (2048, 768)]
