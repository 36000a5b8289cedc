// rz_fp64.cu -- the FP64 oracle on the GPU: the reference's forward and
// adjoint algorithm carried out entirely in double, and the exact discrete
// adjoint in double.  It attaches an error figure to the float results
// (rz_set_error_check / rz_error_report) and runs whole computations in FP64
// (RZ_MODE_FP64, rz_forward_f64, rz_grad_obj_f64).
//
// Arithmetic, operation by operation in double with no contraction:
//   forward point update  sweep.c:89-97 (both branches in double), sweep
//                         orders eikonal.c:50-53, stopping rule norm1.c:20-29
//                         (mean |change| >= TTNORM continues), start values
//                         zero_travel.c:22 and eikonal.c:35-36;
//   residuals             calc_FA_res.c:34-72 (a muted pick gives a zero
//                         residual, as rz_grad_obj defines it);
//   Leung-Qian adjoint    sweep_adj.c:33-68, orders eikonal_adj.c:43-46,
//                         start values init_travel_adj.c:44-57;
//   gradient              ass_grad.c:20-46 (lam*S^3 on the interior, summed in
//                         shot order) and cp_grad_frame.c:18-49;
//   exact adjoint         the adjoint of the Godunov update linearised at the
//                         converged FP64 traveltimes, mu = R + W^T mu, solved
//                         by the same four sweep orders until a pass changes
//                         no value; dJ/dVp = -S^2 sum mu * dG/dS.
//
// Decomposition: one CTA per shot walks the anti-diagonals of each
// directional sweep, one cell per thread, with a CTA barrier between
// diagonals.  Cells of one anti-diagonal are not neighbours; every update
// reads its upstream neighbours from the previous diagonal and its
// downstream ones not yet updated, which is exactly what the sequential
// Gauss-Seidel loop reads.  Speed is secondary here (the oracle runs beside
// the float path, not instead of it).
#include <algorithm>

#include "rz_device.cuh"
#include "rz_internal.h"

namespace rz {

namespace {

RZ_DEV double dadd(double a, double b) { return __dadd_rn(a, b); }
RZ_DEV double dsub(double a, double b) { return __dsub_rn(a, b); }
RZ_DEV double dmul(double a, double b) { return __dmul_rn(a, b); }
RZ_DEV double ddiv(double a, double b) { return __ddiv_rn(a, b); }

constexpr int kThreads = 512;

// sweep.c:89-97 in double: (a + b + sqrt(2 (s s)(dh dh) - d d)) / 2
RZ_DEV double godunov64(double a, double b, double s, double dh, double own) {
    const double d = dsub(a, b), sh = dmul(s, dh);
    double tt;
    if (fabs(d) >= sh) {
        tt = dadd(fmin(a, b), sh);
    } else {
        const double q = dsub(dmul(dmul(2.0, dmul(s, s)), dmul(dh, dh)), dmul(d, d));
        tt = dmul(dadd(dadd(a, b), __dsqrt_rn(q)), 0.5);
    }
    return fmin(own, tt);
}

RZ_DEV double block_sum64(double v, double *red) {
    const int l = threadIdx.x & 31, g = threadIdx.x >> 5, W = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (l == 0) red[g] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < W; ++i) t += red[i];
    __syncthreads();
    return t;
}

// mean |A - B| over the grid (norm1.c:20-29 in double)
RZ_DEV double mean_change64(const F64Params &P, const double *A, const double *B, double *red) {
    double part = 0.0;
    for (size_t c = threadIdx.x; c < P.fstride; c += blockDim.x) part += fabs(dsub(A[c], B[c]));
    return block_sum64(part, red) / ((double)P.nx * (double)P.ny);
}

RZ_DEV void copy64(const F64Params &P, const double *src, double *dst) {
    for (size_t c = threadIdx.x; c < P.fstride; c += blockDim.x) dst[c] = src[c];
    __syncthreads();
}

// one directional forward sweep over the whole grid (sweep.c:24-102)
template <int DX, int DY>
__device__ __noinline__ void sweep_fwd64(const F64Params &P, double *T) {
    const int nx = P.nx, ny = P.ny;
    for (int d = 0; d <= nx + ny - 2; ++d) {
        const int jlo = max(0, d - (nx - 1)), jhi = min(ny - 1, d);
        for (int j = jlo + (int)threadIdx.x; j <= jhi; j += blockDim.x) {
            const int i = d - j;
            const int h = DX > 0 ? i : nx - 1 - i, k = DY > 0 ? j : ny - 1 - j;
            const size_t c = (size_t)k * nx + h;
            const double own = T[c];
            const double w = h > 0 ? T[c - 1] : own, e = h < nx - 1 ? T[c + 1] : own;
            const double n = k > 0 ? T[c - nx] : own, s = k < ny - 1 ? T[c + nx] : own;
            T[c] = godunov64(fmin(w, e), fmin(n, s), (double)P.S[c], P.dh, own);
        }
        __syncthreads();
    }
}

// eikonal.c:31-57 in double; returns the passes run (status bits in *err).
// With P.fixpoint the loop ends at the first pass that changes no cell (the
// updates only ever lower a value, so it ends), the fixpoint of the discrete
// equations that a refined float field approximates.
RZ_DEV int forward64(const F64Params &P, int z, double *T, double *Told, double *red, int *err) {
    const int hs = P.src_h[z], ks = P.src_k[z];
    for (size_t c = threadIdx.x; c < P.fstride; c += blockDim.x) T[c] = 2.0 * P.time;
    __syncthreads();
    if (threadIdx.x == 0) T[(size_t)ks * P.nx + hs] = 0.0;
    __syncthreads();
    double l1 = 10.0 * P.time;
    int it = 0;
    while (P.fixpoint ? l1 > 0.0 : l1 >= P.ttnorm) {
        if (it >= P.max_passes) {
            *err |= ERR_NOCONV_FWD;
            break;
        }
        copy64(P, T, Told);
        sweep_fwd64<+1, +1>(P, T);
        sweep_fwd64<-1, +1>(P, T);
        sweep_fwd64<-1, -1>(P, T);
        sweep_fwd64<+1, -1>(P, T);
        l1 = mean_change64(P, T, Told, red);
        ++it;
    }
    return it;
}

// one directional Leung-Qian sweep over the interior (sweep_adj.c:25-75)
template <int DX, int DY>
__device__ __noinline__ void sweep_adj64(const F64Params &P, const double *T, double *L) {
    const int nx = P.nx, ny = P.ny, ni = nx - 2, nj = ny - 2;
    const double dh = P.dh;
    for (int d = 0; d <= ni + nj - 2; ++d) {
        const int jlo = max(0, d - (ni - 1)), jhi = min(nj - 1, d);
        for (int j = jlo + (int)threadIdx.x; j <= jhi; j += blockDim.x) {
            const int i = d - j;
            const int h = DX > 0 ? 1 + i : nx - 2 - i, k = DY > 0 ? 1 + j : ny - 2 - j;
            if (P.skip[(size_t)k * P.nxp + h]) continue;
            const size_t c = (size_t)k * nx + h;
            const double tc = T[c];
            const double ap = ddiv(-dsub(T[c + 1], tc), dh), am = ddiv(-dsub(tc, T[c - 1]), dh);
            const double bp = ddiv(-dsub(T[c + nx], tc), dh), bm = ddiv(-dsub(tc, T[c - nx]), dh);
            const double app = fmax(ap, 0.0), apm = fmin(ap, 0.0), amp = fmax(am, 0.0), amm = fmin(am, 0.0);
            const double bpp = fmax(bp, 0.0), bpm = fmin(bp, 0.0), bmp = fmax(bm, 0.0), bmm = fmin(bm, 0.0);
            const double lhs = dadd(ddiv(dsub(app, amm), dh), ddiv(dsub(bpp, bmm), dh));
            const double rhs = dadd(ddiv(dsub(dmul(amp, L[c - 1]), dmul(apm, L[c + 1])), dh),
                                    ddiv(dsub(dmul(bmp, L[c - nx]), dmul(bpm, L[c + nx])), dh));
            const double lt = lhs > P.eps_adj ? ddiv(rhs, lhs) : 0.0;
            L[c] = fmin(L[c], lt);
        }
        __syncthreads();
    }
}

// Signed linearisation weights of cell c on its upwind neighbours at the
// converged traveltimes (< 0: west / north neighbour, > 0: east / south),
// and dG/dS; zero at the source.
RZ_DEV void exact_coef64(const F64Params &P, const double *T, int h, int k, bool source, double *wx, double *wz,
                         double *gs) {
    *wx = 0.0, *wz = 0.0, *gs = 0.0;
    if (source) return;
    const int nx = P.nx, ny = P.ny;
    const size_t c = (size_t)k * nx + h;
    const double inf = 1e300;
    const double tw = h > 0 ? T[c - 1] : inf, te = h < nx - 1 ? T[c + 1] : inf;
    const double tn = k > 0 ? T[c - nx] : inf, ts = k < ny - 1 ? T[c + nx] : inf;
    const bool west = tw <= te, north = tn <= ts;
    const double a = west ? tw : te, b = north ? tn : ts;
    const double s = (double)P.S[c], sh = dmul(s, P.dh), d = dsub(a, b);
    if (fabs(d) >= sh) {
        if (a <= b) *wx = west ? -1.0 : 1.0;
        else *wz = north ? -1.0 : 1.0;
        *gs = P.dh;
        return;
    }
    const double r = __dsqrt_rn(dsub(dmul(dmul(2.0, sh), sh), dmul(d, d)));
    const double wa = ddiv(dsub(r, d), dmul(2.0, r)), wb = ddiv(dadd(r, d), dmul(2.0, r));
    *wx = west ? -wa : wa;
    *wz = north ? -wb : wb;
    *gs = ddiv(dmul(dmul(s, P.dh), P.dh), r);
}

// one directional sweep of the exact adjoint system mu = R + W^T mu; returns
// whether this thread changed a value
template <int DX, int DY>
__device__ __noinline__ bool sweep_exact64(const F64Params &P, const double *R, const double *WX, const double *WZ,
                                           double *M) {
    const int nx = P.nx, ny = P.ny;
    bool changed = false;
    for (int d = 0; d <= nx + ny - 2; ++d) {
        const int jlo = max(0, d - (nx - 1)), jhi = min(ny - 1, d);
        for (int j = jlo + (int)threadIdx.x; j <= jhi; j += blockDim.x) {
            const int i = d - j;
            const int h = DX > 0 ? i : nx - 1 - i, k = DY > 0 ? j : ny - 1 - j;
            const size_t c = (size_t)k * nx + h;
            double m = R[c];
            if (h > 0 && WX[c - 1] > 0.0) m = dadd(m, dmul(WX[c - 1], M[c - 1]));
            if (h < nx - 1 && WX[c + 1] < 0.0) m = dadd(m, dmul(-WX[c + 1], M[c + 1]));
            if (k > 0 && WZ[c - nx] > 0.0) m = dadd(m, dmul(WZ[c - nx], M[c - nx]));
            if (k < ny - 1 && WZ[c + nx] < 0.0) m = dadd(m, dmul(-WZ[c + nx], M[c + nx]));
            changed |= m != M[c];
            M[c] = m;
        }
        __syncthreads();
    }
    return changed;
}

}  // namespace

// One CTA per shot: forward to the stopping rule, picks and residuals, and
// (do_adjoint) the Leung-Qian adjoint field or the exact adjoint's mu.
__global__ void __launch_bounds__(kThreads) fp64_shot_kernel(const __grid_constant__ F64Params P) {
    __shared__ double red[kThreads / 32];
    const int z = blockIdx.x;
    if (z >= P.nshots) return;
    const int tid = threadIdx.x;
    double *T = P.T + (size_t)z * P.fstride;
    double *A = P.A + (size_t)z * P.fstride;  // forward snapshot, then adjoint snapshot or exact R
    double *L = P.L + (size_t)z * P.fstride;
    int err = 0;
    const int pf = forward64(P, z, T, A, red, &err);
    if (tid == 0) P.passes_fwd[z] = pf;

    // picks and residuals (calc_FA.c:15-18, calc_FA_res.c:34-72), misfit in receiver order
    if (tid == 0) {
        double l2 = 0.0;
        for (int r = 0; r < P.ntr; ++r) {
            const int h = P.rec_h[r], k = P.rec_k[r];
            const size_t c = (size_t)k * P.nx + h;
            const double tm = T[c];
            P.Tmod[(size_t)z * P.ntr + r] = tm;
            double tr = 0.0;
            if (P.do_residual) {
                const double tob = (double)P.Tobs[(size_t)z * P.ntr + r];
                if (P.cotangent) {
                    tr = tob;
                } else if (tob >= 0.0) {
                    const double res = dsub(tm, tob);
                    l2 = dadd(l2, dmul(res, res));
                    if (P.exact) {
                        tr = res;
                    } else {
                        const double gt = k <= P.ny - 2 ? ddiv(dsub(T[c + P.nx], tm), P.dh)
                                                        : ddiv(dsub(tm, T[c - P.nx]), P.dh);
                        tr = fabs(gt) > 0.0 ? ddiv(res, gt) : 0.0;
                    }
                }
                P.Tres[(size_t)z * P.ntr + r] = tr;
            }
        }
        if (P.do_residual) P.l2[z] = l2;
    }
    __syncthreads();

    if (!P.do_adjoint) {
        if (tid == 0) P.status[z] = err;
        return;
    }
    const int hs = P.src_h[z], ks = P.src_k[z];
    int pa = 0;
    if (!P.exact) {
        // init_travel_adj.c:44-57: frame 0, interior 10*TIME, receiver cells Tres (last receiver wins)
        for (size_t c = tid; c < P.fstride; c += blockDim.x) {
            const int k = (int)(c / P.nx), h = (int)(c - (size_t)k * P.nx);
            L[c] = (h > 0 && h < P.nx - 1 && k > 0 && k < P.ny - 1) ? 10.0 * P.time : 0.0;
        }
        __syncthreads();
        for (int i = tid; i < P.nrcell; i += blockDim.x)
            L[(size_t)P.rcell_k[i] * P.nx + P.rcell_h[i]] = P.Tres[(size_t)z * P.ntr + P.rcell_rec[i]];
        __syncthreads();
        double l1 = 10.0 * P.time;
        while (l1 >= P.ttnorm) {
            if (pa >= P.max_passes) {
                err |= ERR_NOCONV_ADJ;
                break;
            }
            copy64(P, L, A);
            sweep_adj64<+1, +1>(P, T, L);
            sweep_adj64<+1, -1>(P, T, L);
            sweep_adj64<-1, +1>(P, T, L);
            sweep_adj64<-1, -1>(P, T, L);
            l1 = mean_change64(P, L, A, red);
            ++pa;
        }
    } else {
        // weights at the converged traveltimes, R = dJ/dT at receiver cells
        // (each cell's receivers summed in receiver order), mu = 0
        double *WX = P.WX + (size_t)z * P.fstride, *WZ = P.WZ + (size_t)z * P.fstride;
        double *GS = P.GS + (size_t)z * P.fstride;
        for (size_t c = tid; c < P.fstride; c += blockDim.x) {
            const int k = (int)(c / P.nx), h = (int)(c - (size_t)k * P.nx);
            double wx, wz, gs;
            exact_coef64(P, T, h, k, h == hs && k == ks, &wx, &wz, &gs);
            WX[c] = wx, WZ[c] = wz, GS[c] = gs;
            A[c] = 0.0;
            L[c] = 0.0;
        }
        __syncthreads();
        for (int i = tid; i < P.nxcell; i += blockDim.x) {
            double sum = 0.0;
            for (int r = P.xcell_off[i]; r < P.xcell_off[i + 1]; ++r)
                sum = dadd(sum, P.Tres[(size_t)z * P.ntr + P.xcell_rec[r]]);
            A[(size_t)P.xcell_k[i] * P.nx + P.xcell_h[i]] = sum;
        }
        __syncthreads();
        for (;;) {
            if (pa >= P.max_passes) {
                err |= ERR_NOCONV_ADJ;
                break;
            }
            bool ch = sweep_exact64<+1, +1>(P, A, WX, WZ, L);
            ch |= sweep_exact64<+1, -1>(P, A, WX, WZ, L);
            ch |= sweep_exact64<-1, +1>(P, A, WX, WZ, L);
            ch |= sweep_exact64<-1, -1>(P, A, WX, WZ, L);
            ++pa;
            if (!__syncthreads_or(ch)) break;
        }
    }
    if (tid == 0) {
        P.passes_adj[z] = pa;
        P.status[z] = err;
    }
}

// Gradient of shots 0..nshots-1 of this launch added to grad64 in shot order:
// Leung-Qian lam*S^3 on the interior (ass_grad.c:23, ((lam s) s) s); exact
// sum mu * dG/dS, scaled by -S^2 in fp64_finish_kernel.  accumulate: continue
// the sums of earlier chunks.
__global__ void fp64_stack_kernel(const F64Params P, double *grad64, bool accumulate) {
    const long n = (long)P.fstride;
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        const int k = (int)(c / P.nx), h = (int)(c - (long)k * P.nx);
        double g = accumulate ? grad64[c] : 0.0;
        if (P.exact) {
            for (int z = 0; z < P.nshots; ++z)
                g = dadd(g, dmul(P.L[(size_t)z * P.fstride + c], P.GS[(size_t)z * P.fstride + c]));
        } else if (h > 0 && h < P.nx - 1 && k > 0 && k < P.ny - 1) {
            const double s = (double)P.S[c];
            for (int z = 0; z < P.nshots; ++z) g = dadd(g, dmul(dmul(dmul(P.L[(size_t)z * P.fstride + c], s), s), s));
        }
        grad64[c] = g;
    }
}

// exact: dJ/dVp = -S^2 dJ/dS per cell ((-s) s) g
__global__ void fp64_vp_scale_kernel(const float *S, long n, double *grad64) {
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        const double s = (double)S[c];
        grad64[c] = dmul(dmul(-s, s), grad64[c]);
    }
}

cudaError_t launch_fp64_shots(const F64Params &P, cudaStream_t st) {
    if (P.nshots < 1) return cudaSuccess;
    fp64_shot_kernel<<<P.nshots, kThreads, 0, st>>>(P);
    return cudaGetLastError();
}

cudaError_t launch_fp64_stack(const F64Params &P, double *grad64, bool accumulate, cudaStream_t st) {
    const long n = (long)P.fstride;
    const long blocks = std::min((n + 255) / 256, 152L * 8);
    fp64_stack_kernel<<<(unsigned)std::max(blocks, 1L), 256, 0, st>>>(P, grad64, accumulate);
    return cudaGetLastError();
}

cudaError_t launch_fp64_vp_scale(const float *S, long n, double *grad64, cudaStream_t st) {
    const long blocks = std::min((n + 255) / 256, 152L * 8);
    fp64_vp_scale_kernel<<<(unsigned)std::max(blocks, 1L), 256, 0, st>>>(S, n, grad64);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// errors of float results against the FP64 oracle
// ---------------------------------------------------------------------------
// non-negative doubles order like their bit patterns
RZ_DEV void atomic_max_pos(double *p, double v) {
    atomicMax(reinterpret_cast<unsigned long long *>(p), (unsigned long long)__double_as_longlong(v));
}

// acc[0] += sum (a - b)^2, acc[1] += sum b^2, acc[2] = max |a - b|, acc[3] = max |b|
// over n values; a float (pitch pa, rows of na values) or double, b double (pitch nb)
template <typename A>
__global__ void compare_kernel(const A *a, int pa, const double *b, int pb, int ncol, long nrow, size_t bstride_a,
                               size_t bstride_b, double *acc) {
    const size_t z = blockIdx.y;
    double s2 = 0.0, r2 = 0.0, dmax = 0.0, rmax = 0.0;
    const long n = (long)ncol * nrow;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const long r = i / ncol, c = i - r * ncol;
        const double x = (double)a[z * bstride_a + (size_t)r * pa + c], y = b[z * bstride_b + (size_t)r * pb + c];
        const double d = x - y;
        s2 += d * d, r2 += y * y;
        dmax = fmax(dmax, fabs(d)), rmax = fmax(rmax, fabs(y));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
        r2 += __shfl_xor_sync(0xffffffffu, r2, o);
        dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
        rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        double *q = acc + 4 * z;
        atomicAdd(q, s2);
        atomicAdd(q + 1, r2);
        atomic_max_pos(q + 2, dmax);
        atomic_max_pos(q + 3, rmax);
    }
}

cudaError_t launch_compare(const float *a, int pa, const double *b, int pb, int ncol, long nrow, int nbatch,
                           size_t bstride_a, size_t bstride_b, double *acc, cudaStream_t st) {
    const long n = (long)ncol * nrow;
    dim3 grid((unsigned)std::max(1L, std::min((n + 255) / 256, 152L * 2)), (unsigned)std::max(nbatch, 1));
    compare_kernel<float><<<grid, 256, 0, st>>>(a, pa, b, pb, ncol, nrow, bstride_a, bstride_b, acc);
    return cudaGetLastError();
}

__global__ void d2f_kernel(const double *src, float *dst, long n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        dst[i] = __double2float_rn(src[i]);
}

cudaError_t launch_d2f(const double *src, float *dst, long n, cudaStream_t st) {
    const long blocks = std::min((n + 255) / 256, 152L * 8);
    d2f_kernel<<<(unsigned)std::max(blocks, 1L), 256, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

}  // namespace rz
