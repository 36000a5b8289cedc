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


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# host CPU: the reference algorithm on all host cores
# ---------------------------------------------------------------------------
def _cpu_worker(args):
    """One worker process = one MPI rank of the reference: grad_obj over its shots."""
    kind, shots, nshots_total, seed = args
    import numpy as np
    import oracle as O
    from rajzel_gb300 import synth
    w = synth.grad_1700x350(nshots=nshots_total)
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


def cpu_run(nshots_sample, cores, kind):
    """Time grad_obj over `nshots_sample` shots split across `cores` processes
    exactly as init_MPIshot splits shots over ranks; returns wall seconds."""
    import multiprocessing as mp
    import oracle as O
    O.build(ref=(kind == "reference"))
    spans = [O.shot_partition(nshots_sample, cores, r) for r in range(cores)]
    jobs = [(kind, list(range(a - 1, b - 1)), 100, 0) for a, b in spans]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        times = pool.map(_cpu_worker, jobs)
    return max(times)


def cpu_kind():
    import oracle as O
    return "reference" if os.path.isdir(O.REF_SRC) else "port"


def run_reference_arm(args, rank):
    """`--impl reference`: the reference algorithm timed on the host cores."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    kind = cpu_kind()
    sample = cores  # one shot per core per step
    for _ in range(args.warmup):
        cpu_run(sample, cores, kind)
    secs = [cpu_run(sample, cores, kind) for _ in range(args.steps)]
    total = sum(secs)
    value = sample * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "shots/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded)",
        "config": {"workload": WORKLOAD, "sample_shots_per_step": sample, "cores": cores},
        "cpu_baseline": {"value": value, "unit": "shots/s", "cores": cores, "kind": kind,
                         "sample": f"{sample} of the 100 shots per step, one process per core, init_MPIshot split"},
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
    tobs_d = torch.from_numpy(np.ascontiguousarray(Tobs)).cuda()
    grad_d = torch.empty((w.ny, w.nx), dtype=torch.float32, device="cuda")
    l2_d = torch.empty(1, dtype=torch.float64, device="cuda")

    def step():
        ctx.grad_obj_device(w.srcx, w.srcz, tobs_d.data_ptr(), grad_d.data_ptr(), l2_d.data_ptr())

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    # passes and point-updates of one step (identical every step: same inputs)
    passes = np.array([ctx.shot_info(i)[:2] for i in range(w.nshots)])
    pu_fwd = int(passes[:, 0].sum()) * 4 * w.nx * w.ny
    pu_adj = int(passes[:, 1].sum()) * 4 * (w.nx - 2) * (w.ny - 2)
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
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * w.nshots * args.steps / (ms / 1e3)
    kernel_ms = shot_ms / max(shot_calls, 1)
    alg_bytes = pu_fwd * ALG_BYTES_FWD + pu_adj * ALG_BYTES_ADJ
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
    vp_host = np.ascontiguousarray(w.vp_start)
    e2e_steps = max(3, args.steps // 2)
    for _ in range(2):
        ctx2.set_velocity(vp_host)
        ctx2.grad_obj(w.srcx, w.srcz, Tobs)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx2.set_velocity(vp_host)
        g_host, L2 = ctx2.grad_obj(w.srcx, w.srcz, Tobs)
    e2e_s = time.perf_counter() - t0
    e2e_value = world * w.nshots * e2e_steps / e2e_s
    h2d = vp_host.nbytes + Tobs.nbytes + 2 * 4 * w.nshots
    d2h = g_host.nbytes + 8 + 4 * w.nshots

    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = 2 * cores
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
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved / hbm_peak, "peak_source": peak_src,
                     "traffic": traffic,
                     "kernel": "rz::shot_kernel", "kernel_ms": kernel_ms,
                     "algorithmic_bytes_per_launch": alg_bytes},
        "cpu_baseline": {"value": sample / cpu_s, "unit": "shots/s", "cores": cores, "kind": kind,
                         "sample": f"grad_obj over {sample} of the 100 shots, one process per core"},
        "e2e": {"value": e2e_value, "unit": "shots/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "plain_per_shot_gpu": {"value": plain_value, "unit": "shots/s",
                               "how": f"same kernels, one shot per launch, {nplain} shots, synchronised"},
        "batched_over_plain": value / plain_value,
        "gpu_launches": int(launches1 - launches0),
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["fast", "reference"], default="fast")
    ap.add_argument("--shots", type=int, default=100, help="shots per step (the workload has 100)")
    ap.add_argument("--profile-only", action="store_true",
                    help="only the device-timed loop (for profiler runs); no baselines, no JSON contract line")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference_arm(args, rank)
    else:
        run_gpu_arm(args, rank, world, local_rank)


if __name__ == "__main__":
    main()
