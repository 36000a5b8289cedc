"""The allocation-free forward entry point (rz_eikonal_noalloc).

Callers that cannot allocate GPU memory (fixed pools or memory budgets, hosts
without an allocator) get the same traveltimes as rz_eikonal() from a static
device array.  This file sorts last so that a run stopping at the first
failure has run every other test first; it also passes alone in a fresh
process, where its first call performs the one-time set-up.
"""
import ctypes as C

import numpy as np
import pytest

from rajzel_gb300 import synth

pytestmark = pytest.mark.gpu


class _Grid(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("dh", C.c_float), ("time", C.c_float),
                ("ttnorm", C.c_float), ("eps_adj", C.c_float), ("max_passes", C.c_int)]


def test_noalloc_forward_matches_eikonal_on_two_calls(gpu_lib):
    import torch
    R = gpu_lib
    lib = R.load_library()
    f = lib.rz_eikonal_noalloc
    f.argtypes = [C.POINTER(_Grid), C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int

    w = synth.small_case(4242, 300, 170, nshots=2)  # six strips, ragged last block
    S = synth.slowness(w.vp_true)
    ctx = R.Context(0, "reference")
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_slowness(S)
    grid = _Grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj, 10000)

    S_d = torch.from_numpy(S).cuda()
    TT_d = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
    info_d = torch.full((2,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    for i in range(2):  # two calls in a row share the static array
        TT_ref, _, passes_ref = ctx.eikonal(w.srcx[i], w.srcz[i])
        st = f(C.byref(grid), S_d.data_ptr(), float(w.srcx[i]), float(w.srcz[i]), TT_d.data_ptr(),
               info_d.data_ptr(), None)
        assert st == R.RZ_OK
        torch.cuda.synchronize()
        info = info_d.cpu().numpy()
        assert np.array_equal(TT_d.cpu().numpy(), TT_ref)  # reference mode: bit-exact
        assert info[0] == passes_ref and info[1] == 0


def test_noalloc_rejects_oversized_and_bad_input(gpu_lib):
    lib = gpu_lib.load_library()
    f = lib.rz_eikonal_noalloc
    f.argtypes = [C.POINTER(_Grid), C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    big = _Grid(60000, 500, 10.0, 40.0, 1e-6, 1e-9, 100)  # needs ~120 Mi floats of working space
    assert f(C.byref(big), C.c_void_p(16), 100.0, 20.0, C.c_void_p(16), C.c_void_p(16), None) == gpu_lib.RZ_EUNSUPPORTED
    ok = _Grid(100, 50, 10.0, 40.0, 1e-6, 1e-9, 100)
    assert f(C.byref(ok), C.c_void_p(16), -500.0, 20.0, C.c_void_p(16), C.c_void_p(16), None) == gpu_lib.RZ_EINVAL


def test_noalloc_reports_invalid_slowness_and_no_convergence(gpu_lib):
    """An invalid slowness sets status bit 5 (RZ_EINVAL, no solve), a pass
    limit of 1 the forward no-convergence bit (RZ_ENOCONV); the next call
    with good input is exact again."""
    import torch
    R = gpu_lib
    lib = R.load_library()
    f = lib.rz_eikonal_noalloc
    f.argtypes = [C.POINTER(_Grid), C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    w = synth.small_case(4343, 90, 70, nshots=1)
    S = synth.slowness(w.vp_true)
    bad = S.copy()
    bad[33, 44] = 0.0
    grid1 = _Grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj, 1)
    grid = _Grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj, 10000)
    TT_d = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
    info_d = torch.zeros(2, dtype=torch.int32, device="cuda")
    for g, model, want in ((grid1, bad, R.RZ_EINVAL), (grid1, S, R.RZ_ENOCONV)):
        S_d = torch.from_numpy(model).cuda()
        assert f(C.byref(g), S_d.data_ptr(), float(w.srcx[0]), float(w.srcz[0]), TT_d.data_ptr(),
                 info_d.data_ptr(), None) == R.RZ_OK
        torch.cuda.synchronize()
        assert lib.rz_status_code(int(info_d.cpu()[1])) == want
    ctx = R.Context(0, "reference")
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_slowness(S)
    TT_ref, _, passes = ctx.eikonal(w.srcx[0], w.srcz[0])
    S_d = torch.from_numpy(S).cuda()
    assert f(C.byref(grid), S_d.data_ptr(), float(w.srcx[0]), float(w.srcz[0]), TT_d.data_ptr(),
             info_d.data_ptr(), None) == R.RZ_OK
    torch.cuda.synchronize()
    assert np.array_equal(TT_d.cpu().numpy(), TT_ref) and info_d.cpu().tolist() == [passes, 0]


def test_noalloc_calls_capture_into_cuda_graphs(gpu_lib):
    """After one warm call, two calls (two sources) are captured into two CUDA
    graphs on a side stream; replays in either order give rz_eikonal's
    traveltimes and pass counts bit for bit (the graphs share the static
    array and replay one after the other on one stream)."""
    import torch
    R = gpu_lib
    lib = R.load_library()
    f = lib.rz_eikonal_noalloc
    f.argtypes = [C.POINTER(_Grid), C.c_void_p, C.c_float, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int

    w = synth.small_case(4343, 200, 100, nshots=2)
    S = synth.slowness(w.vp_true)
    ctx = R.Context(0, "reference")
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_slowness(S)
    grid = _Grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj, 10000)
    S_d = torch.from_numpy(S).cuda()
    TT = [torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda") for _ in range(2)]
    info = [torch.zeros(2, dtype=torch.int32, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    assert f(C.byref(grid), S_d.data_ptr(), float(w.srcx[0]), float(w.srcz[0]), TT[0].data_ptr(),
             info[0].data_ptr(), None) == R.RZ_OK  # warm call: the one-time set-up
    torch.cuda.synchronize()

    side = torch.cuda.Stream()
    graphs = [torch.cuda.CUDAGraph() for _ in range(2)]
    for i in range(2):
        with torch.cuda.graph(graphs[i], stream=side):
            st = f(C.byref(grid), S_d.data_ptr(), float(w.srcx[i]), float(w.srcz[i]), TT[i].data_ptr(),
                   info[i].data_ptr(), C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert st == R.RZ_OK
    want = [ctx.eikonal(w.srcx[i], w.srcz[i]) for i in range(2)]
    for order in ((1, 0), (0, 1)):
        for i in range(2):
            TT[i].fill_(-1.0)
            info[i].fill_(-7)
        for i in order:
            graphs[i].replay()
        torch.cuda.synchronize()
        for i in range(2):
            TT_ref, _, passes_ref = want[i]
            assert np.array_equal(TT[i].cpu().numpy(), TT_ref)
            got = info[i].cpu().numpy()
            assert got[0] == passes_ref and got[1] == 0
