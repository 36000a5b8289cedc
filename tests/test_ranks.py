"""CPU tests of the multi-rank host logic (rajzel_gb300/ranks.py): the
reference's shot split, and the FP64 sums over ranks run as two gloo ranks."""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

import oracle as O
from rajzel_gb300 import ranks, synth


def test_shot_range_is_init_mpishot_split():
    O.build(ref=False)
    for nshots in (0, 1, 5, 7, 100, 1024):
        for nranks in (1, 2, 3, 8, 13):
            spans = [ranks.shot_range(nshots, nranks, r) for r in range(nranks)]
            # contiguous, disjoint, complete
            assert spans[0][0] == 0 and spans[-1][1] == nshots
            assert all(spans[i][1] == spans[i + 1][0] for i in range(nranks - 1))
            # the reference's 1-based [NSHOT1, NSHOT2)
            for r, (a, b) in enumerate(spans):
                assert O.shot_partition(nshots, nranks, r) == (a + 1, b + 1)
    with pytest.raises(ValueError):
        ranks.shot_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = synth.small_case(21, 48, 30, nshots=5)
        p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
        S = synth.slowness(w.vp_true)
        Tobs = np.stack([O.calc_fa(p, O.eikonal(p, S * np.float32(0.98), w.srcx[i], w.srcz[i])[0], w.recx, w.recz)
                         for i in range(w.nshots)])
        a, b = ranks.shot_range(w.nshots, world, rank)
        g, l2 = O.grad_obj_f64(p, S.astype(np.float64), w.srcx[a:b].astype(np.float64),
                               w.srcz[a:b].astype(np.float64), w.recx, w.recz, Tobs[a:b].astype(np.float64))
        g_sum, l2_sum = ranks.allreduce_gradient(g, l2, dist)
        slowest = ranks.max_over_ranks(1.5 + rank, dist)
        if rank == 0:
            q.put((g_sum, l2_sum, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_sum_gradient_and_misfit():
    """Two ranks each take their init_MPIshot block of a 5-shot batch; the
    FP64 sums over the ranks equal the single-rank batch."""
    O.build(ref=False)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    try:
        g_sum, l2_sum, slowest = q.get(timeout=240)
    finally:
        for pr in procs:
            pr.join(timeout=60)
    assert all(pr.exitcode == 0 for pr in procs)
    w = synth.small_case(21, 48, 30, nshots=5)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    S = synth.slowness(w.vp_true)
    Tobs = np.stack([O.calc_fa(p, O.eikonal(p, S * np.float32(0.98), w.srcx[i], w.srcz[i])[0], w.recx, w.recz)
                     for i in range(w.nshots)])
    g, l2 = O.grad_obj_f64(p, S.astype(np.float64), w.srcx.astype(np.float64), w.srcz.astype(np.float64), w.recx,
                           w.recz, Tobs.astype(np.float64))
    scale = np.abs(g).max()
    assert scale > 0 and np.abs(g_sum - g).max() <= 1e-12 * scale
    assert l2_sum == pytest.approx(l2, rel=1e-12)
    assert slowest == 2.5
