#!/usr/bin/env python
"""Benchmark: batched forward + adjoint Eikonal gradient (RAJZEL grad_obj).

Workload (one "step"): the gradient and misfit of 100 surface shots with 850
receivers on a 1700 x 350 grid at DH = 10 m (layered 1500-4500 m/s start
model; picks from the same model with 12 Gaussian anomalies), i.e. forward
Eikonal + residuals + adjoint Eikonal + gradient stack for every shot.  Seeded
synthetic model (no dataset involved).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--mode fast|reference]
    python bench.py --impl reference ...   # the reference algorithm on the host CPUs

Prints one JSON line.  `value` is shots/s with inputs resident in HBM
(device-timed with CUDA events on the launching stream); `e2e` is the same
metric through the public C ABI with host buffers (model and picks uploaded,
gradient and misfit read back every step).  With N GPUs every rank runs an
independent replica of the workload (shots are independent; the reference's
only exchange is a gradient sum).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "fwd+adjoint shots/s & point-updates/s, batched vs plain GPU, rel err<=1e-5"
WORKLOAD = "grad_1700x350: 100 shots x 850 receivers, 1700x350 grid, dh=10 m, fwd+residual+adjoint+stack"
ALG_BYTES_FWD = 12  # per forward point-update: slowness read, traveltime read + write
ALG_BYTES_ADJ = 16  # per adjoint point-update: traveltime, lambda read + write, receiver flag
CHECK_BYTES_FWD = 8  # per cell of a forward fixpoint check: traveltime, slowness read
CHECK_BYTES_ADJ = 9  # per interior cell of an adjoint fixpoint check: traveltime, lambda, receiver flag
ALG_BYTES_EXACT_ADJ = 20  # per exact-adjoint point-update: mu read + write, x and z weight, receiver term


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# host CPU: the reference algorithm on all host cores
# ---------------------------------------------------------------------------
def _workload(name, nshots):
    from rajzel_gb300 import synth
    if name == "grad_1700x350":
        return synth.grad_1700x350(nshots=nshots)
    if name == "fatt":
        return synth.fatt_2000x500(nshots=nshots)
    if name == "stress":
        return synth.stress_8192x2048(nshots=nshots)
    if name.startswith("uneven"):
        return synth.uneven_grid(int(name[-1]))
    raise KeyError(name)


def _cpu_worker(args):
    """One worker process = one MPI rank of the reference: grad_obj over its shots."""
    kind, shots, nshots_total, wname = args
    import numpy as np
    import oracle as O
    from rajzel_gb300 import synth
    w = _workload(wname, nshots_total)
    p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    Sobs = synth.slowness(w.vp_true)
    S = synth.slowness(w.vp_start)
    idx = np.asarray(shots, int)
    t0 = time.perf_counter()
    if kind == "reference":
        ref = O.Ref(p)
        Tobs = np.stack([ref.eikonal(Sobs, w.srcx[i], w.srcz[i], w.recx, w.recz)[1] for i in idx]) if len(idx) else None
        t0 = time.perf_counter()
        if len(idx):
            ref.grad_obj(S, w.srcx[idx], w.srcz[idx], w.recx, w.recz, Tobs)
    else:
        Tobs = np.stack([O.calc_fa(p, O.eikonal(p, Sobs, w.srcx[i], w.srcz[i])[0], w.recx, w.recz) for i in idx]) \
            if len(idx) else None
        t0 = time.perf_counter()
        if len(idx):
            O.grad_obj(p, S, w.srcx[idx], w.srcz[idx], w.recx, w.recz, Tobs)
    return time.perf_counter() - t0


def cpu_run(nshots_sample, cores, kind, wname="grad_1700x350", nshots_total=100, pool=None):
    """Time grad_obj over `nshots_sample` shots split across `cores` processes
    exactly as init_MPIshot splits shots over ranks; returns wall seconds
    (the slowest rank's grad_obj, as the reference's shot loop ends at its
    MPI_Allreduce).  A pool of `cores` spawned processes may be passed in
    and reused across calls."""
    import multiprocessing as mp
    import oracle as O
    O.build(ref=(kind == "reference"))
    spans = [O.shot_partition(nshots_sample, cores, r) for r in range(cores)]
    jobs = [(kind, list(range(a - 1, b - 1)), nshots_total, wname) for a, b in spans]
    if pool is not None:
        return max(pool.map(_cpu_worker, jobs))
    with mp.get_context("spawn").Pool(cores) as own:
        return max(own.map(_cpu_worker, jobs))


def cpu_kind():
    import oracle as O
    return "reference" if os.path.isdir(O.REF_SRC) else "port"


def run_reference_arm(args, rank):
    """`--impl reference`: the reference algorithm timed on the host cores."""
    if rank != 0:
        return
    import multiprocessing as mp
    from rajzel_gb300 import synth
    w = synth.grad_1700x350(nshots=100)
    cores = os.cpu_count() or 1
    kind = cpu_kind()
    sample = w.nshots  # the whole 100-shot batch per step, as the GPU arm's step
    with mp.get_context("spawn").Pool(cores) as pool:
        for _ in range(args.warmup):
            cpu_run(sample, cores, kind, pool=pool)
        secs = [cpu_run(sample, cores, kind, pool=pool) for _ in range(args.steps)]
    total = sum(secs)
    value = sample * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "shots/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "mode": "reference algorithm", "shots": sample, "receivers": w.ntr,
                   "grid": [w.nx, w.ny], "dh": w.dh, "ttnorm": w.ttnorm,
                   "parallelism": f"{cores} host processes, init_MPIshot split",
                   "l2": "per-shot working set ~12 MB per process; no flush"},
        "cpu_baseline": {"value": value, "unit": "shots/s", "cores": cores, "kind": kind,
                         "sample": f"all {sample} shots per step, one process per core, init_MPIshot split"},
        "e2e": {"value": value, "unit": "shots/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 100 ms."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            return

        def reader():
            for line in self.proc.stdout:
                self.rows.append((time.time(), [x.strip() for x in line.split(",")]))
        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = [r for t, r in self.rows if t0 - 0.15 <= t <= t1 + 0.15] or [r for _, r in self.rows[-3:]]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def read_traffic(nshots_run):
    """DRAM bytes per shot-kernel launch from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "shot_kernel_grad_1700x350.md")
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_shot:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) * nshots_run if m else None


def run_gpu_arm(args, rank, world, local_rank):
    import numpy as np
    import torch
    import rajzel_gb300 as R
    from rajzel_gb300 import build as B
    from rajzel_gb300 import synth

    B.build()
    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    w = synth.grad_1700x350(nshots=args.shots)
    stream = torch.cuda.Stream()  # a real stream handle: the events below time exactly the library's work
    torch.cuda.set_stream(stream)
    ctx = R.Context(local_rank, args.mode)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_receivers(w.recx, w.recz)
    ctx.set_velocity(w.vp_true)
    _, Tobs, _ = ctx.forward(w.srcx, w.srcz, want_tt=False)  # observed picks (not timed)
    ctx.set_velocity(w.vp_start)
    if args.profile_only:  # a profiler run may time another gradient path
        ctx.set_gradient(args.gradient)
        ctx.set_refine(args.refine)
    tobs_d = torch.from_numpy(np.ascontiguousarray(Tobs)).cuda()
    grad_d = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
    l2_d = torch.empty(1, dtype=torch.float64, device="cuda")

    def step():
        ctx.grad_obj_device(w.srcx, w.srcz, tobs_d.data_ptr(), grad_d.data_ptr(), l2_d.data_ptr())

    tuned = ctx.autotune(w.srcx, w.srcz, Tobs)  # band width for this batch (set-up, not timed)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    # passes and point-updates of one step (identical every step: same inputs)
    passes = np.array([ctx.shot_info(i)[:2] for i in range(w.nshots)])
    sweeps = np.array([ctx.shot_work(i) for i in range(w.nshots)])
    # point-updates actually performed (a pass proven by the fixpoint check to
    # change nothing is counted by the reference's rule but not swept)
    pu_fwd = int(sweeps[:, 0].sum()) * w.nx * w.ny
    pu_adj = int(sweeps[:, 1].sum()) * (w.nx - 2) * (w.ny - 2)
    checks = (passes - (sweeps + 3) // 4).sum(axis=0)  # successful fixpoint checks (forward, adjoint)
    launches0, _, _ = ctx.kernel_stats()  # also clears the per-launch timing list

    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t_wall0 = time.time()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.time()
    ms = e0.elapsed_time(e1)
    if dist:
        dist.barrier()
    time.sleep(0.15)
    clocks.stop()
    launches1, shot_ms, shot_calls = ctx.kernel_stats()
    # the device-pointer calls return before the device is done: read every
    # shot's status bits now (a timeout or non-convergence voids the line)
    bits = ctx.batch_status()
    if bits:
        raise SystemExit(f"device status bits 0x{bits:x} in the timed loop")
    if dist:
        from rajzel_gb300 import ranks
        ms = ranks.max_over_ranks(ms, dist, device=f"cuda:{local_rank}")
    value = world * w.nshots * args.steps / (ms / 1e3)
    kernel_ms = shot_ms / max(shot_calls, 1)
    alg_bytes = (pu_fwd * ALG_BYTES_FWD + pu_adj * ALG_BYTES_ADJ + int(checks[0]) * CHECK_BYTES_FWD * w.nx * w.ny
                 + int(checks[1]) * CHECK_BYTES_ADJ * (w.nx - 2) * (w.ny - 2))
    hbm_peak, peak_src = 6800.0, "fallback"
    try:
        hbm_peak, peak_src = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]), "measured"
    except Exception:
        pass
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    traffic = read_traffic(w.nshots)

    if args.profile_only:
        if rank == 0:
            print(json.dumps({"profile_only": True, "ms_per_step": ms / args.steps, "kernel_ms": kernel_ms}))
        return

    # the plain per-shot GPU path: the same kernels, one shot per launch
    nplain = min(8, w.nshots)
    t0 = time.perf_counter()
    for i in range(nplain):
        ctx.grad_obj_device(w.srcx[i:i + 1], w.srcz[i:i + 1], tobs_d[i].data_ptr(), grad_d.data_ptr(),
                            l2_d.data_ptr())
        torch.cuda.synchronize()
    plain_value = world * nplain / (time.perf_counter() - t0)

    # end to end through the public API with host buffers
    ctx2 = R.Context(local_rank, args.mode)
    ctx2.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx2.set_receivers(w.recx, w.recz)
    # the step's inputs (velocity, picks) and its gradient live in pinned host memory
    def pinned(shape):
        return torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()
    vp_host, tobs_host, g_host = pinned((w.ny, w.nx)), pinned(np.shape(Tobs)), pinned((w.ny, w.nx))
    vp_host[...] = w.vp_start
    tobs_host[...] = Tobs
    e2e_steps = max(3, args.steps // 2)
    for _ in range(2):
        ctx2.set_velocity(vp_host)
        ctx2.grad_obj(w.srcx, w.srcz, tobs_host, out=g_host)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx2.set_velocity(vp_host)
        g_host, L2 = ctx2.grad_obj(w.srcx, w.srcz, tobs_host, out=g_host)
    e2e_s = time.perf_counter() - t0
    e2e_value = world * w.nshots * e2e_steps / e2e_s
    h2d = vp_host.nbytes + tobs_host.nbytes + 2 * 4 * w.nshots
    d2h = g_host.nbytes + 8 + 4 * w.nshots

    # the other two arithmetic paths on the same batch, and every path's
    # error against the FP64 GPU oracle (all outside the timed region above)
    exact_line = time_mode(R, w, Tobs, stream, local_rank, "fast", "exact", args.steps, args.warmup, hbm_peak,
                           peak_src, refine=True)
    refined_line = time_mode(R, w, Tobs, stream, local_rank, "fast", "reference", args.steps, args.warmup,
                             hbm_peak, peak_src, refine=True)
    refmode_line = time_mode(R, w, Tobs, stream, local_rank, "reference", "reference",
                             max(3, args.steps // 4), args.warmup, hbm_peak, peak_src)
    errors = fp64_errors(R, w, Tobs, local_rank)

    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = w.nshots
    kind = cpu_kind()
    cpu_s = cpu_run(sample, cores, kind)
    clk = clocks.summary(t_wall0, t_wall1)
    line = {
        "metric": METRIC, "value": value, "unit": "shots/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 sweeps, f64 stack/misfit" if args.mode == "fast" else "f32/f64 reference-exact",
        "data": "synthetic (seeded layered model + Gaussian anomalies)",
        "config": {"workload": WORKLOAD, "mode": args.mode, "shots": w.nshots, "receivers": w.ntr,
                   "grid": [w.nx, w.ny], "dh": w.dh, "ttnorm": w.ttnorm,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU, one CTA per shot",
                   "l2": "per-shot working set ~1.2 GB > 126 MB L2; no flush"},
        "point_updates_per_s": world * (pu_fwd + pu_adj) * args.steps / (ms / 1e3),
        "point_updates_per_step": pu_fwd + pu_adj,
        "passes_fwd_adj": [int(passes[:, 0].sum()), int(passes[:, 1].sum())],
        "sweeps_fwd_adj": [int(sweeps[:, 0].sum()), int(sweeps[:, 1].sum())],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": peak_src,
                     "traffic": traffic,
                     "kernel": "rz::shot_kernel", "kernel_ms": kernel_ms,
                     "algorithmic_bytes_per_launch": alg_bytes},
        "cpu_baseline": {"value": sample / cpu_s, "unit": "shots/s", "cores": cores, "kind": kind,
                         "sample": f"grad_obj over all {sample} shots of the step, one process per core"},
        "e2e": {"value": e2e_value, "unit": "shots/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "plain_per_shot_gpu": {"value": plain_value, "unit": "shots/s",
                               "how": f"same kernels, one shot per launch, {nplain} shots, synchronised"},
        "batched_over_plain": value / plain_value,
        "gpu_launches": int(launches1 - launches0),
        "autotune": tuned, "cuda_graphs": True,
        "errors_vs_fp64": errors,
        "exact_gradient": exact_line,
        "refined_traveltimes": refined_line,
        "reference_mode": refmode_line,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def time_mode(R, w, Tobs, stream, dev, mode, kind, steps, warmup, hbm_peak, peak_src, refine=False):
    """shots/s of the gradient step in another arithmetic mode, gradient kind
    or with refined traveltimes (device buffers, CUDA events on the launching
    stream) and the shot kernel's byte-model roofline: fast mode with the
    exact discrete adjoint of refined traveltimes (the gradient that meets the
    1e-4 gate), the Leung-Qian gradient of refined traveltimes, or reference
    (bit-exact) mode.  The byte model counts the forward and adjoint sweeps
    and fixpoint checks; the refinement's linear sweeps are not counted."""
    import numpy as np
    import torch
    ctx = R.Context(dev, mode)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_receivers(w.recx, w.recz)
    ctx.set_velocity(w.vp_start)
    ctx.set_gradient(kind)
    ctx.set_refine(refine)
    tobs_d = torch.from_numpy(np.ascontiguousarray(Tobs)).cuda()
    grad_d = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
    l2_d = torch.empty(1, dtype=torch.float64, device="cuda")

    def step():
        ctx.grad_obj_device(w.srcx, w.srcz, tobs_d.data_ptr(), grad_d.data_ptr(), l2_d.data_ptr())

    for _ in range(max(warmup, 3)):
        step()
    torch.cuda.synchronize()
    ctx.kernel_stats()
    ms = _events_ms(step, stream, steps)
    _, shot_ms, calls = ctx.kernel_stats()
    bits = ctx.batch_status()
    if bits:
        raise SystemExit(f"{mode}/{kind}: device status bits 0x{bits:x}")
    sweeps = np.array([ctx.shot_work(i) for i in range(w.nshots)])
    passes = np.array([ctx.shot_info(i)[:2] for i in range(w.nshots)])
    checks = (passes - (sweeps + 3) // 4).sum(axis=0)  # passes proven by a fixpoint check, not swept
    adj_bytes = ALG_BYTES_EXACT_ADJ if kind == "exact" else ALG_BYTES_ADJ
    pu_fwd = int(sweeps[:, 0].sum()) * w.nx * w.ny
    pu_adj = int(sweeps[:, 1].sum()) * (w.nx * w.ny if kind == "exact" else (w.nx - 2) * (w.ny - 2))
    alg = (pu_fwd * ALG_BYTES_FWD + pu_adj * adj_bytes + int(checks[0]) * CHECK_BYTES_FWD * w.nx * w.ny
           + int(checks[1]) * CHECK_BYTES_ADJ * (w.nx - 2) * (w.ny - 2))
    kernel_ms = shot_ms / max(calls, 1)
    achieved = alg / (kernel_ms / 1e3) / 1e9
    return {"mode": mode, "gradient": kind, "refined": refine, "value": w.nshots / (ms / 1e3), "unit": "shots/s",
            "ms_per_step": ms,
            "steps": steps, "sweeps_fwd_adj": [int(sweeps[:, 0].sum()), int(sweeps[:, 1].sum())],
            "point_updates_per_s": (pu_fwd + pu_adj) / (ms / 1e3),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "peak_source": peak_src, "kernel_ms": kernel_ms,
                         "algorithmic_bytes_per_launch": alg}}


def fp64_errors(R, w, Tobs, dev):
    """Every path's error against the FP64 GPU oracle on the benchmark batch
    (rz_set_error_check: the oracle runs the same 100 shots in double):
    traveltimes (max-norm and relative L2, worst shot), picks, gradient
    (rel. L2) and misfit.  Float32 traveltimes carry the rounding of every
    update along paths of up to ~1800 cells: unrefined, the fast path sits
    exactly where the reference's own float arithmetic does (above 1e-5
    max-norm), so it is gated there; refined (rz_set_refine), traveltimes are
    gated at 1e-5.  Gradient gates: Leung-Qian no further from FP64 than
    twice the reference's own float arithmetic plus 1e-4 (its receiver
    scaling, calc_FA_res.c, differences neighbouring float traveltimes);
    exact gradient of refined traveltimes 1e-4."""
    out = {}
    for label, mode, kind, refine in (("fast", "fast", "reference", False),
                                      ("reference", "reference", "reference", False),
                                      ("exact_refined", "fast", "exact", True),
                                      ("fast_refined", "fast", "reference", True),
                                      ("exact_unrefined", "fast", "exact", False)):
        ctx = R.Context(dev, mode)
        ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
        ctx.set_receivers(w.recx, w.recz)
        ctx.set_velocity(w.vp_start)
        ctx.set_gradient(kind)
        ctx.set_refine(refine)
        ctx.set_error_check(True)
        ctx.grad_obj(w.srcx, w.srcz, Tobs)
        out[label] = ctx.error_report()
        ctx.close()
    ref = out["reference"]
    tt_gate = max(1e-5, ref["tt_rel"] * (1 + 1e-3) + 1e-7)
    lq_gate = 2 * ref["grad_rel_l2"] + 1e-4
    out["gates"] = {"fast_tt_rel": tt_gate, "refined_tt_rel": 1e-5, "fast_grad_rel_l2": lq_gate,
                    "exact_refined_grad_rel_l2": 1e-4}
    out["pass"] = bool(out["fast"]["tt_rel"] <= tt_gate and out["fast"]["grad_rel_l2"] <= lq_gate
                       and out["exact_refined"]["tt_rel"] <= 1e-5 and out["fast_refined"]["tt_rel"] <= 1e-5
                       and out["exact_refined"]["grad_rel_l2"] <= 1e-4)
    out["oracle"] = "FP64 GPU oracle (the reference's algorithm in double) on the same 100 shots"
    return out


# ---------------------------------------------------------------------------
# the other named workloads (one JSON line each; the default run is the one above)
# ---------------------------------------------------------------------------
def _events_ms(fn, stream, steps):
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def _context(R, w, mode, stream, vp):
    ctx = R.Context(torch_device_index(), mode)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_grid(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
    ctx.set_receivers(w.recx, w.recz)
    ctx.set_velocity(vp)
    return ctx


def torch_device_index():
    import torch
    return torch.cuda.current_device()


def run_workload(args, local_rank):
    """fwd_500x174: one forward solve (latency); uneven: 256 shots over three
    grids, forward + adjoint gradient; stress: 1024 shots on 8192 x 2048
    under a 120 GB cap on the field slots; fatt: 30 l-BFGS iterations, 200
    shots x 1000 receivers on 2000 x 500; phases: per-shot phase times of
    every gradient path on the benchmark batch."""
    import numpy as np
    import torch
    import rajzel_gb300 as R
    from rajzel_gb300 import build as B
    from rajzel_gb300 import synth
    B.build()
    torch.cuda.set_device(local_rank)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    out = {"workload": args.workload, "mode": args.mode, "data": "synthetic (seeded)"}
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    t_wall0 = time.time()
    if args.workload == "fwd_500x174":
        w = synth.fwd_500x174()
        ctx = _context(R, w, args.mode, stream, w.vp_true)
        tt = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
        step = lambda: ctx.forward_device(w.srcx, w.srcz, tt.data_ptr(), 0)  # noqa: E731
        for _ in range(max(args.warmup, 3)):
            step()
        ms = _events_ms(step, stream, args.steps)
        passes = ctx.shot_info(0)[0]
        import oracle as O
        O.build(ref=False)
        p = O.Params(w.nx, w.ny, w.dh, w.time, w.ttnorm, w.eps_adj)
        S = synth.slowness(w.vp_true)
        t0 = time.perf_counter()
        reps = 5
        for _ in range(reps):
            O.eikonal(p, S, w.srcx[0], w.srcz[0])
        cpu_ms = 1e3 * (time.perf_counter() - t0) / reps
        out.update({"metric": "forward solve latency", "value": ms, "unit": "ms", "higher_is_better": False,
                    "passes": passes, "point_updates_per_s": passes * 4 * w.nx * w.ny / (ms / 1e3),
                    "cpu_baseline": {"value": cpu_ms, "unit": "ms", "cores": 1, "kind": "port",
                                     "sample": "the same solve, one core (the reference solves a shot on one rank)"}})
    elif args.workload == "phases":
        # where a shot's time goes on each gradient path of the benchmark batch:
        # medians over the 100 shots of the shot kernel's device clock stamps
        # (rz_shot_timeline: 0 start, 7 refinement start, 1 forward done,
        # 2 residuals, 3 adjoint prepared, 4 adjoint done)
        w = synth.grad_1700x350(nshots=100)
        ctx = _context(R, w, "fast", stream, w.vp_true)
        _, Tobs, _ = ctx.forward(w.srcx, w.srcz, want_tt=False)
        tobs_d = torch.from_numpy(np.ascontiguousarray(Tobs)).cuda()
        paths = {}
        for mode, kind, refine in [("fast", "reference", False), ("reference", "reference", False),
                                   ("fast", "exact", False), ("fast", "reference", True), ("fast", "exact", True)]:
            c = _context(R, w, mode, stream, w.vp_start)
            c.set_gradient(kind)
            c.set_refine(refine)
            g = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
            l2 = torch.empty(1, dtype=torch.float64, device="cuda")
            step = lambda: c.grad_obj_device(w.srcx, w.srcz, tobs_d.data_ptr(), g.data_ptr(), l2.data_ptr())  # noqa
            for _ in range(max(args.warmup, 3)):
                step()
            ms = _events_ms(step, stream, args.steps)
            if c.batch_status():
                raise SystemExit(f"{mode}/{kind}: device status bits 0x{c.batch_status():x}")
            st = np.array([c.shot_timeline(i) for i in range(w.nshots)], dtype=np.float64)
            med = lambda a, b: float(np.median(st[:, b] - st[:, a]) / 1e3)  # noqa: E731
            sw = np.array([c.shot_work(i) for i in range(w.nshots)]).mean(axis=0)
            paths[f"{mode} arithmetic, {'exact' if kind == 'exact' else 'Leung-Qian'} gradient"
                  + (", refined traveltimes" if refine else "")] = {
                "ms_per_step": ms, "shots_per_s": w.nshots / (ms / 1e3),
                "us_per_shot": {"forward": med(0, 7 if refine else 1), "refinement": med(7, 1) if refine else 0.0,
                                "residuals": med(1, 2), "adjoint_preparation": med(2, 3), "adjoint": med(3, 4)},
                "sweeps_per_shot_fwd_adj": sw.tolist()}
        out.update({"metric": "per-shot phase times (median over the batch)", "paths": paths, "shots": w.nshots})
    elif args.workload == "uneven":
        grids = [synth.uneven_grid(i) for i in range(3)]
        ctxs, bufs, streams = [], [], []
        for w in grids:
            st = torch.cuda.Stream()
            ctx = _context(R, w, args.mode, st, w.vp_true)
            _, Tobs, _ = ctx.forward(w.srcx, w.srcz, want_tt=False)
            ctx.set_velocity(w.vp_start)
            bufs.append((torch.from_numpy(np.ascontiguousarray(Tobs)).cuda(),
                         torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda"),
                         torch.empty(1, dtype=torch.float64, device="cuda")))
            ctxs.append(ctx)
            streams.append(st)

        def launch(i):
            w, (to, g, l2) = grids[i], bufs[i]
            ctxs[i].grad_obj_device(w.srcx, w.srcz, to.data_ptr(), g.data_ptr(), l2.data_ptr())

        def concurrent():
            for i in range(3):
                launch(i)

        tobs_h = [b[0].cpu().numpy() for b in bufs]

        def multi():  # one persistent launch over the three grids
            R.grad_obj_multi(ctxs, [w.srcx for w in grids], [w.srcz for w in grids], tobs_h)

        for _ in range(max(args.warmup, 3)):
            concurrent()
            multi()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            concurrent()
        torch.cuda.synchronize()
        conc_ms = 1e3 * (time.perf_counter() - t0) / args.steps
        t0 = time.perf_counter()
        for _ in range(args.steps):
            multi()
        torch.cuda.synchronize()
        multi_ms = 1e3 * (time.perf_counter() - t0) / args.steps
        per_grid = []
        for i, w in enumerate(grids):
            ms_i = _events_ms(lambda: launch(i), streams[i], max(1, args.steps // 2))
            sw = np.array([ctxs[i].shot_work(s) for s in range(w.nshots)]).sum(axis=0)
            per_grid.append({"grid": [w.nx, w.ny], "shots": w.nshots, "ms": ms_i,
                             "sweeps_fwd_adj": [int(sw[0]), int(sw[1])],
                             "point_updates": int(sw[0]) * w.nx * w.ny + int(sw[1]) * (w.nx - 2) * (w.ny - 2)})
        nsh = sum(w.nshots for w in grids)
        pu = sum(g["point_updates"] for g in per_grid)
        cores = os.cpu_count() or 1
        kind = cpu_kind()
        cpu_s = 0.0
        for i, w in enumerate(grids):  # one shot per core of each grid, scaled to the grid's shots
            cpu_s += cpu_run(cores, cores, kind, f"uneven{i}", w.nshots) * w.nshots / cores
        out["cpu_baseline"] = {"value": nsh / cpu_s, "unit": "shots/s", "cores": cores, "kind": kind,
                               "sample": "grad_obj of one shot per core on each grid, scaled to 86/85/85 shots"}
        best = min(conc_ms, multi_ms)
        out.update({"metric": "fwd+adjoint shots/s", "value": nsh / (multi_ms / 1e3), "unit": "shots/s",
                    "higher_is_better": True, "ms_per_step": multi_ms, "shots": nsh,
                    "point_updates_per_s": pu / (multi_ms / 1e3), "per_grid": per_grid,
                    "how": "one persistent launch over the three grids (rz_grad_obj_multi), host buffers, "
                           "host-timed around a full sync",
                    "three_streams": {"ms_per_step": conc_ms, "shots_per_s": nsh / (conc_ms / 1e3),
                                      "how": "each grid's batch on its own stream, device buffers"},
                    "best_ms": best})
    elif args.workload == "stress":
        w = synth.stress_8192x2048(nshots=args.shots if args.shots != 100 else 1024)
        ctx = _context(R, w, args.mode, stream, w.vp_true)
        ctx.set_memory_cap(120 << 30)
        to = torch.empty((w.nshots, w.ntr), dtype=torch.float32, device="cuda")
        t0 = time.perf_counter()
        ctx.forward_device(w.srcx, w.srcz, 0, to.data_ptr())
        torch.cuda.synchronize()
        fwd_s = time.perf_counter() - t0
        ctx.set_velocity(w.vp_start)
        g = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
        l2 = torch.empty(1, dtype=torch.float64, device="cuda")
        step = lambda: ctx.grad_obj_device(w.srcx, w.srcz, to.data_ptr(), g.data_ptr(), l2.data_ptr())  # noqa
        ms = _events_ms(step, stream, max(1, args.steps))
        pf = sum(ctx.shot_info(s)[0] for s in range(w.nshots))
        pa = sum(ctx.shot_info(s)[1] for s in range(w.nshots))
        sw = np.array([ctx.shot_work(s) for s in range(w.nshots)]).sum(axis=0)
        pu = int(sw[0]) * w.nx * w.ny + int(sw[1]) * (w.nx - 2) * (w.ny - 2)  # sweeps actually run
        # the same batch with the exact gradient of refined traveltimes: larger
        # field slots, so more chunks under the same cap (one warm-up, one step)
        ctx.set_gradient("exact")
        ctx.set_refine(True)
        step()
        exact_ms = _events_ms(step, stream, 1)
        if ctx.batch_status():
            raise SystemExit(f"stress, exact gradient: device status bits 0x{ctx.batch_status():x}")
        out["exact_gradient_run"] = {"value": w.nshots / (exact_ms / 1e3), "unit": "shots/s", "ms_per_step": exact_ms,
                                     "refined": True}
        ctx.set_gradient("reference")
        ctx.set_refine(False)
        cores = os.cpu_count() or 1
        kind = cpu_kind()
        cpu_s = cpu_run(cores, cores, kind, "stress", w.nshots)
        out["cpu_baseline"] = {"value": cores / cpu_s, "unit": "shots/s", "cores": cores, "kind": kind,
                               "sample": "grad_obj of one shot per core (the first shots of the 1024)"}
        out.update({"metric": "fwd+adjoint shots/s", "value": w.nshots / (ms / 1e3), "unit": "shots/s",
                    "higher_is_better": True, "ms_per_step": ms, "shots": w.nshots,
                    "forward_only_s": fwd_s, "passes_fwd_adj": [pf, pa], "sweeps_fwd_adj": [int(sw[0]), int(sw[1])],
                    "point_updates_per_s": pu / (ms / 1e3), "memory_cap_bytes": 120 << 30,
                    "peak_allocated_note": "field slots sized to the cap, chunks of a multiple of the SM count"})
    elif args.workload == "fatt":
        w = synth.fatt_2000x500(nshots=args.shots if args.shots != 100 else 200)
        ctx = _context(R, w, args.mode, stream, w.vp_true)
        _, Tobs, _ = ctx.forward(w.srcx, w.srcz, want_tt=False)  # observed picks from the true model
        # the reference's example workflow: Gaussian-filtered gradients (SPATFILTER 4,
        # 80 x 40 points) and the horizontal taper of its parameter file
        opts = dict(itermax=30, nlbfgs=5, stepmax=10, vp_lo=1000.0, vp_hi=6000.0, recursion=1, spatfilter=4,
                    filt_size_grad=80, filt_size_grad1=40, taper_hor=1, gradt1=22, gradt2=25,
                    exp_taper_grad_hor=0.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vp, mis, it, ev, _ = ctx.fatt(w.srcx, w.srcz, Tobs, w.vp_start, **opts)
        secs = time.perf_counter() - t0
        err0 = float(np.linalg.norm(w.vp_start - w.vp_true) / np.linalg.norm(w.vp_true))
        err1 = float(np.linalg.norm(vp - w.vp_true) / np.linalg.norm(w.vp_true))
        # the same inversion in the reference's own float arithmetic, for the model difference
        ref = None
        if args.mode == "fast" and not args.no_ref_run:
            ctx_r = _context(R, w, "reference", stream, w.vp_true)
            t1 = time.perf_counter()
            vp_r, mis_r, it_r, ev_r, _ = ctx_r.fatt(w.srcx, w.srcz, Tobs, w.vp_start, **opts)
            ref = {"seconds": time.perf_counter() - t1, "iterations": it_r, "evaluations": ev_r,
                   "final_misfit": float(mis_r[-1]) if len(mis_r) else None,
                   "model_rel_diff_fast_vs_reference": float(np.linalg.norm(vp - vp_r) / np.linalg.norm(vp_r))}

        def rel(a, b):
            return float(np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b))

        # the same stage with the FP64 oracle computing every gradient (RZ_MODE_FP64):
        # the final model's error against that run
        fp64 = None
        if not args.no_ref_run:
            ctx64 = _context(R, w, "fp64", stream, w.vp_true)
            t1 = time.perf_counter()
            vp64, mis64, it64, ev64, _ = ctx64.fatt(w.srcx, w.srcz, Tobs, w.vp_start, **opts)
            fp64 = {"seconds": time.perf_counter() - t1, "iterations": it64, "evaluations": ev64,
                    "final_misfit": float(mis64[-1]) if len(mis64) else None,
                    "model_rel_error_true": rel(vp64, w.vp_true), "final_model_rel_diff_vs_fp64": rel(vp, vp64)}
        # the stage on the exact gradient of refined traveltimes (the gradient of the misfit
        # it minimises), with its own FP64 oracle run
        exact = None
        if args.mode == "fast" and not args.no_ref_run:
            ctx_e = _context(R, w, "fast", stream, w.vp_true)
            ctx_e.set_gradient("exact")
            ctx_e.set_refine(True)
            t1 = time.perf_counter()
            vp_e, mis_e, it_e, ev_e, _ = ctx_e.fatt(w.srcx, w.srcz, Tobs, w.vp_start, **opts)
            exact = {"seconds": time.perf_counter() - t1, "iterations": it_e, "evaluations": ev_e,
                     "misfit_first_last": [float(mis_e[0]), float(mis_e[-1])] if len(mis_e) else None,
                     "model_rel_error_start_final": [rel(w.vp_start, w.vp_true), rel(vp_e, w.vp_true)]}
            ctx_e64 = _context(R, w, "fp64", stream, w.vp_true)
            ctx_e64.set_gradient("exact")
            vp_e64, mis_e64, it_e64, ev_e64, _ = ctx_e64.fatt(w.srcx, w.srcz, Tobs, w.vp_start, **opts)
            exact["fp64_run"] = {"iterations": it_e64, "evaluations": ev_e64,
                                 "model_rel_error_true": rel(vp_e64, w.vp_true)}
            exact["final_model_rel_diff_vs_fp64"] = rel(vp_e, vp_e64)
        out.update({"metric": "FATT stage wall time", "value": secs, "unit": "s", "higher_is_better": False,
                    "iterations": it, "gradient_evaluations": ev, "shots": w.nshots, "receivers": w.ntr,
                    "ms_per_gradient": 1e3 * secs / max(ev, 1), "shots_per_s": w.nshots * ev / secs,
                    "misfit_first_last": [float(mis[0]), float(mis[-1])] if len(mis) else None,
                    "model_rel_error_start_final": [err0, err1], "options": opts, "reference_mode_run": ref,
                    "fp64_oracle_run": fp64, "exact_gradient_run": exact})
        cores = os.cpu_count() or 1
        kind = cpu_kind()
        cpu_s = cpu_run(cores, cores, kind, "fatt", w.nshots)
        per_eval = cpu_s * w.nshots / cores
        out["cpu_baseline"] = {"value": per_eval * ev, "unit": "s", "cores": cores, "kind": kind,
                               "sample": f"grad_obj of one shot per core, scaled to {w.nshots} shots x {ev} evaluations"}
    t_wall1 = time.time()
    time.sleep(0.15)
    clocks.stop()
    out["clocks"] = clocks.summary(t_wall0, t_wall1)
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["fast", "reference"], default="fast")
    ap.add_argument("--shots", type=int, default=100, help="shots per step (the workload has 100)")
    ap.add_argument("--workload", choices=["grad_1700x350", "fwd_500x174", "uneven", "stress", "fatt", "phases"],
                    default="grad_1700x350", help="the benchmark workload (default) or another named one")
    ap.add_argument("--no-ref-run", action="store_true", help="fatt: skip the reference-arithmetic comparison run")
    ap.add_argument("--profile-only", action="store_true",
                    help="only the device-timed loop (for profiler runs); no baselines, no JSON contract line")
    ap.add_argument("--gradient", choices=["reference", "exact"], default="reference",
                    help="with --profile-only: the gradient kind of the timed loop")
    ap.add_argument("--refine", action="store_true", help="with --profile-only: refined traveltimes")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
    elif args.workload != "grad_1700x350":
        run_workload(args, local_rank)
    else:
        run_gpu_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
