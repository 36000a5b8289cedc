"""GPU tests of the failure path: a bounded device wait that runs out.

The reference has no failure handling beyond err() -> MPI_Abort
(util.c:7-17).  Here every wait for another warp is bounded; when one runs
out the kernel records a status bit, the CTA's other waits return at once,
every tensor copy still lands, and the call returns RZ_ETIMEOUT.  The test
makes a wait run out without any fault: one warp withholds one hand-off
signal (a flag that nothing else sets) under a small poll budget.
"""
import numpy as np
import pytest
import torch

import oracle as O
from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def R(gpu_lib):
    O.build(ref=False)
    return gpu_lib


def make(R, w, mode):
    ctx = R.Context(0, mode)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_velocity(w.vp_true)
    ctx.set_receivers(w.recx, w.recz)
    return ctx


@pytest.mark.parametrize("mode,ny", [("fast", 96), ("reference", 96), ("fast", 700)])
def test_withheld_handoff_times_out_and_context_recovers(R, mode, ny):
    """3 strips (pipelined sweeps) and 22 strips (banded sweeps)."""
    w = synth.small_case(606 + ny, 150, ny, nshots=3)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    Tobs = np.stack([O.calc_fa(p, O.eikonal(p, S * np.float32(0.97), w.srcx[i], w.srcz[i])[0], w.recx, w.recz)
                     for i in range(w.nshots)])
    ctx = make(R, w, mode)
    g0, l0 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    ctx.set_wait_test(4096, True)
    with pytest.raises(R.RajzelError) as e:
        ctx.grad_obj(w.srcx, w.srcz, Tobs)
    assert e.value.status == R.RZ_ETIMEOUT
    assert all(ctx.shot_info(i)[2] & 2 for i in range(w.nshots))  # a wait for another warp gave up
    # the device-pointer path reports the same through rz_batch_status
    tob = torch.from_numpy(np.ascontiguousarray(Tobs)).cuda()
    g = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
    l2 = torch.empty(1, dtype=torch.float64, device="cuda")
    ctx.grad_obj_device(w.srcx, w.srcz, tob.data_ptr(), g.data_ptr(), l2.data_ptr())
    bits = ctx.batch_status()
    assert bits & 2 and R.load_library().rz_status_code(bits) == R.RZ_ETIMEOUT
    # normal operation again: the same result as before
    ctx.set_wait_test(0, False)
    g1, l1 = ctx.grad_obj(w.srcx, w.srcz, Tobs)
    assert np.array_equal(g0, g1) and l0 == l1 and ctx.batch_status() == 0
