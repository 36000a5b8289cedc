"""Seeded synthetic models and acquisition geometry for the benchmark shapes.

No public dataset is involved: every model is generated from a fixed seed
with the shapes, sizes and value ranges of the workloads below.  Positions
follow the reference's conventions: sources in metres (srcpos[1]/[2],
sources.c:68-69), receivers as 1-based grid indices iround(x/DH)
(receiver.c:55-56).

Workloads
  fwd_500x174   forward only, 500 x 174 at DH=20 m: linear 1500->4000 m/s
                depth gradient + 6 Gaussian anomalies (+-15%, sigma 200-600 m),
                source at (5000 m, 40 m), TTNORM 1e-6
  grad_1700x350 forward + adjoint gradient, 1700 x 350 at DH=10 m: layered
                1500-4500 m/s gradient (+12 Gaussian anomalies in the true
                model), 100 surface shots, 850 receivers at z=20 m
  uneven_3grids 256 shots over 512x256 / 1024x512 / 2048x768 at DH=10 m,
                smooth random velocity 1500-5000 m/s (Gaussian-filtered white
                noise, correlation length 300 m)
  fatt_2000x500 2000 x 500 at DH=12.5 m, 200 shots x 1000 receivers, layered
                model + 4500 m/s block + Gaussians; start = 1-D depth average
  stress_8192x2048  8192 x 2048 at DH=5 m, 1024 shots x 4096 receivers,
                water layer over a 1800->5000 m/s gradient + 4500 m/s polygon
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    nx: int
    ny: int
    dh: float
    time: float
    ttnorm: float
    eps_adj: float
    vp_true: np.ndarray
    vp_start: np.ndarray
    srcx: np.ndarray            # metres
    srcz: np.ndarray            # metres
    recx: np.ndarray            # 1-based grid index
    recz: np.ndarray            # 1-based grid index
    meta: dict = field(default_factory=dict)

    @property
    def nshots(self):
        return len(self.srcx)

    @property
    def ntr(self):
        return len(self.recx)


def grid_index(x_m, dh):
    """iround(x/DH) of fd.h:18 on float32 coordinates."""
    q = (np.asarray(x_m, np.float32) / np.float32(dh)).astype(np.float64)
    return np.floor(q + 0.5).astype(np.int32)


def _gaussians(rng, nx, ny, dh, count, amp, sig_lo, sig_hi):
    x = (np.arange(nx) * dh)[None, :]
    z = (np.arange(ny) * dh)[:, None]
    pert = np.zeros((ny, nx))
    for _ in range(count):
        cx, cz = rng.uniform(0, nx * dh), rng.uniform(0, ny * dh)
        sig = rng.uniform(sig_lo, sig_hi)
        a = rng.uniform(-amp, amp)
        pert += a * np.exp(-((x - cx) ** 2 + (z - cz) ** 2) / (2 * sig * sig))
    return pert


def _layered(rng, ny, dh, v0, v1, nlayers=6):
    z = np.arange(ny) * dh
    zmax = ny * dh
    base = v0 + (v1 - v0) * z / zmax
    bounds = np.sort(rng.uniform(0.1 * zmax, 0.95 * zmax, nlayers))
    steps = np.zeros(ny)
    for b in bounds:
        steps += rng.uniform(-120, 180) * (z >= b)
    return np.clip(base + steps, v0, v1)


def fwd_500x174(seed=1234):
    rng = np.random.default_rng(seed)
    nx, ny, dh = 500, 174, 20.0
    z = np.arange(ny) * dh
    v = 1500.0 + (4000.0 - 1500.0) * z / z[-1]
    v = np.repeat(v[:, None], nx, axis=1)
    v = v * (1.0 + _gaussians(rng, nx, ny, dh, 6, 0.15, 200.0, 600.0))
    vp = v.astype(np.float32)
    nrec = 250
    recx = (2 + 2 * np.arange(nrec)).astype(np.int32)
    recz = np.full(nrec, 2, np.int32)
    return Workload("fwd_500x174", nx, ny, dh, 10.0, 1e-6, 1e-9, vp, vp,
                    np.array([5000.0], np.float32), np.array([40.0], np.float32), recx, recz)


def grad_1700x350(seed=2024, nshots=100, ntr=850):
    rng = np.random.default_rng(seed)
    nx, ny, dh = 1700, 350, 10.0
    prof = _layered(rng, ny, dh, 1500.0, 4500.0)
    start = np.repeat(prof[:, None], nx, axis=1)
    true = start * (1.0 + _gaussians(rng, nx, ny, dh, 12, 0.12, 150.0, 500.0))
    # shots evenly spaced along the surface at z = 20 m (row 2, inside the adjoint frame)
    srcx = (dh * (2.0 + (nx - 4) * (np.arange(nshots) + 0.5) / nshots)).astype(np.float32)
    srcz = np.full(nshots, 20.0, np.float32)
    recx = grid_index(dh * (1.0 + np.linspace(1, nx - 2, ntr)), dh)
    recz = np.full(ntr, 2, np.int32)
    return Workload("grad_1700x350", nx, ny, dh, 20.0, 1e-6, 1e-9, true.astype(np.float32), start.astype(np.float32),
                    srcx, srcz, recx.astype(np.int32), recz)


def smooth_random(rng, nx, ny, dh, vmin, vmax, corr_m):
    from scipy.ndimage import gaussian_filter
    w = rng.standard_normal((ny, nx))
    f = gaussian_filter(w, sigma=corr_m / dh, mode="reflect")
    f = (f - f.min()) / max(f.max() - f.min(), 1e-12)
    return (vmin + (vmax - vmin) * f).astype(np.float32)


def uneven_grid(idx, seed=77, nshots=None, ntr=None):
    """One of the three grids of the uneven batch: 0 -> 512x256, 1 -> 1024x512, 2 -> 2048x768."""
    shapes = [(512, 256), (1024, 512), (2048, 768)]
    split = [86, 85, 85]
    nx, ny = shapes[idx]
    dh = 10.0
    rng = np.random.default_rng(seed + idx)
    vp = smooth_random(rng, nx, ny, dh, 1500.0, 5000.0, 300.0)
    ns = split[idx] if nshots is None else nshots
    srcx = rng.uniform(2 * dh, (nx - 2) * dh, ns).astype(np.float32)
    srcz = np.full(ns, 2 * dh, np.float32)
    nr = nx // 2 if ntr is None else ntr
    recx = grid_index(dh * (1.0 + np.linspace(1, nx - 2, nr)), dh)
    recz = np.full(nr, 2, np.int32)
    # picks from this model; gradients taken at a start model 3% slower
    return Workload(f"uneven_{nx}x{ny}", nx, ny, dh, 40.0, 1e-6, 1e-9, vp, (vp * np.float32(0.97)).astype(np.float32),
                    srcx, srcz, recx.astype(np.int32), recz)


def fatt_2000x500(seed=99, nshots=200, ntr=1000):
    rng = np.random.default_rng(seed)
    nx, ny, dh = 2000, 500, 12.5
    prof = _layered(rng, ny, dh, 1500.0, 4200.0)
    true = np.repeat(prof[:, None], nx, axis=1)
    bx0, bx1 = int(0.4 * nx), int(0.55 * nx)
    bz0, bz1 = int(0.35 * ny), int(0.5 * ny)
    true[bz0:bz1, bx0:bx1] = 4500.0
    true = true * (1.0 + _gaussians(rng, nx, ny, dh, 10, 0.08, 200.0, 600.0))
    start = np.repeat(true.mean(axis=1)[:, None], nx, axis=1)
    srcx = (dh * (2.0 + (nx - 4) * (np.arange(nshots) + 0.5) / nshots)).astype(np.float32)
    srcz = np.full(nshots, 2 * dh, np.float32)
    recx = grid_index(dh * (1.0 + np.linspace(1, nx - 2, ntr)), dh)
    recz = np.full(ntr, 2, np.int32)
    return Workload("fatt_2000x500", nx, ny, dh, 30.0, 1e-6, 1e-9, true.astype(np.float32),
                    start.astype(np.float32), srcx, srcz, recx.astype(np.int32), recz)


def fatt_small(sub=8, nshots=8, ntr=100, seed=99):
    """The FATT model sampled every `sub` cells (2000x500 / sub, dh*sub): a
    small case of the same structure for tests."""
    w = fatt_2000x500(seed=seed, nshots=1, ntr=10)
    vt = np.ascontiguousarray(w.vp_true[::sub, ::sub])
    vs = np.ascontiguousarray(w.vp_start[::sub, ::sub])
    ny, nx = vt.shape
    dh = w.dh * sub
    srcx = (dh * (2.0 + (nx - 4) * (np.arange(nshots) + 0.5) / nshots)).astype(np.float32)
    srcz = np.full(nshots, 2 * dh, np.float32)
    recx = grid_index(dh * (1.0 + np.linspace(1, nx - 2, ntr)), dh).astype(np.int32)
    recz = np.full(ntr, 2, np.int32)
    return Workload(f"fatt_{nx}x{ny}", nx, ny, dh, w.time, w.ttnorm, w.eps_adj, vt, vs, srcx, srcz, recx, recz)


def _polygon_mask(rng, nx, ny, dh, cx, cz, r_mean, nvert=9):
    """Cells inside a seeded random star-shaped polygon (even-odd ray casting)."""
    ang = np.sort(rng.uniform(0, 2 * np.pi, nvert))
    rad = r_mean * rng.uniform(0.55, 1.0, nvert)
    px, pz = cx + rad * np.cos(ang), cz + 0.6 * rad * np.sin(ang)
    X = (np.arange(nx) * dh)[None, :]
    Z = (np.arange(ny) * dh)[:, None]
    inside = np.zeros((ny, nx), bool)
    for i in range(nvert):
        x0, z0, x1, z1 = px[i], pz[i], px[(i + 1) % nvert], pz[(i + 1) % nvert]
        if z0 == z1:
            continue
        cross = ((z0 > Z) != (z1 > Z))
        xint = x0 + (Z - z0) * (x1 - x0) / (z1 - z0)
        inside ^= cross & (X < xint)
    return inside


def stress_8192x2048(seed=4096, nshots=1024, ntr=4096):
    """High-contrast stress case: 1500 m/s water layer over an 1800->5000 m/s
    gradient with an embedded 4500 m/s random-polygon block; dh = 5 m."""
    rng = np.random.default_rng(seed)
    nx, ny, dh = 8192, 2048, 5.0
    z = np.arange(ny) * dh
    water = 300.0
    v = np.where(z < water, 1500.0, 1800.0 + (5000.0 - 1800.0) * (z - water) / (z[-1] - water))
    vp = np.repeat(v[:, None], nx, axis=1).astype(np.float32)
    mask = _polygon_mask(rng, nx, ny, dh, 0.5 * nx * dh, 0.55 * ny * dh, 0.3 * ny * dh * 1.4)
    vp[mask] = 4500.0
    srcx = (dh * (2.0 + (nx - 4) * (np.arange(nshots) + 0.5) / nshots)).astype(np.float32)
    srcz = np.full(nshots, 2 * dh, np.float32)
    recx = grid_index(dh * (1.0 + np.linspace(1, nx - 2, ntr)), dh)
    recz = np.full(ntr, 2, np.int32)
    # start model: the block at 3500 m/s
    start = np.where(mask, np.float32(3500.0), vp).astype(np.float32)
    return Workload("stress_8192x2048", nx, ny, dh, 30.0, 1e-6, 1e-9, vp, start, srcx, srcz, recx.astype(np.int32),
                    recz)


def small_case(seed, nx, ny, dh=10.0, nshots=3, ntr=None, vmin=1500.0, vmax=4500.0):
    """Small seeded case for parity tests: smooth-ish random velocity."""
    rng = np.random.default_rng(seed)
    z = np.arange(ny)[:, None] / max(ny - 1, 1)
    base = vmin + (vmax - vmin) * 0.6 * z
    v = base + 0.4 * (vmax - vmin) * rng.random((ny, nx)) * 0.5
    v = np.clip(v, vmin, vmax).astype(np.float32)
    srcx = rng.uniform(1.0 * dh, (nx - 0.6) * dh, nshots).astype(np.float32)
    srcz = rng.uniform(1.0 * dh, (ny - 0.6) * dh, nshots).astype(np.float32)
    nr = max(1, nx // 2) if ntr is None else ntr
    recx = rng.integers(1, nx + 1, nr).astype(np.int32)
    recz = rng.integers(1, ny + 1, nr).astype(np.int32)
    return Workload(f"small_{nx}x{ny}", nx, ny, dh, 40.0, 1e-6, 1e-9, v, v, srcx, srcz, recx, recz)


def slowness(vp):
    """calc_S.c:21: S = 1.0/Vp evaluated in double, stored as float."""
    return (1.0 / np.asarray(vp, np.float64)).astype(np.float32)
