// rz_fatt.cu -- the FATT inversion loop on the GPU engine: l-BFGS with a
// weak-Wolfe line search over rz_grad_obj, gradient preconditioning by a
// Gaussian filter and a horizontal taper.
//
// Follows the reference's loop step by step (fatt.c:108-258): gradient and
// misfit (grad_obj.c, with precond.c), steepest-descent direction
// (descent.c), l-BFGS direction (LBFGS.c:36-165), descent check
// (check_descent.c), Gaussian filter of the direction (fatt.c:177-184,
// gauss_filt.c), Wolfe line search (wolfels.c:16-110), model update with hard
// limits (calc_mat_change_wolfe.c), stopping rule (fatt.c:214-243).
//
// Precision: model, gradients and l-BFGS vectors are float vectors on the
// device; every dot product and every scalar of the two-loop recursion is
// double (the reference uses float, dotp.c); vector updates are computed in
// double and rounded once to float.  The recursion visits the history slots
// either in the reference's slot order (LBFGS.c:113-150: slot NLBFGS down to
// 1, then 1 up to NLBFGS, whatever their age) or newest-to-oldest and back
// (Nocedal & Wright, algorithm 7.4).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/rajzel_gb300.h"
#include "rz_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kPartials = 304;  // two blocks per SM for the reductions

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// partial[b] = sum of a*b over a grid-stride slice, in double
__global__ void dot_kernel(const float *a, const float *b, long n, double *partial) {
    __shared__ double red[kThreads / 32];
    double s = 0.0;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        s += (double)a[i] * (double)b[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < kThreads / 32; ++i) t += red[i];
        partial[blockIdx.x] = t;
    }
}

// partial[b] = max over a slice (maximum_m of util.c: signed maximum)
__global__ void max_kernel(const float *a, long n, float *partial) {
    __shared__ float red[kThreads / 32];
    float m = -INFINITY;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        m = fmaxf(m, a[i]);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = -INFINITY;
        for (int i = 0; i < kThreads / 32; ++i) t = fmaxf(t, red[i]);
        partial[blockIdx.x] = t;
    }
}

// y = RN32(alpha * x + beta * y), in double; beta == 0 does not read y
__global__ void axpby_kernel(long n, double alpha, const float *x, double beta, float *y) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        y[i] = (float)(beta == 0.0 ? alpha * (double)x[i] : alpha * (double)x[i] + beta * (double)y[i]);
}

// d = a - b
__global__ void sub_kernel(long n, const float *a, const float *b, float *d) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        d[i] = a[i] - b[i];
}

// calc_mat_change_wolfe.c:28-50: trial model with hard limits (step taken in double)
__global__ void model_step_kernel(long n, const float *vp, const float *h, float step, float lo, float hi,
                                  float *out) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float v0 = vp[i];
        float v = (float)((double)v0 + (double)step * (double)h[i]);
        if (v < lo) v = v0;
        if (v > hi) v = v0;
        if (v < 0.0f) v = v0;
        out[i] = v;
    }
}

// Gaussian filter (gauss_filt.c:56-127): the 2-D kernel exp(-ii^2/sx -
// jj^2/sy) / sum is the product of two normalised 1-D kernels, so it is
// applied as a row pass and a column pass, edges replicated.
__global__ void gauss_rows_kernel(const float *in, float *out, int nx, int ny, const float *w, int hf) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nx * ny) return;
    const int k = (int)(c / nx), h = (int)(c - (long)k * nx);
    const float *row = in + (size_t)k * nx;
    float s = 0.f;
    for (int i = -hf; i <= hf; ++i) s += row[min(max(h + i, 0), nx - 1)] * w[i + hf];
    out[c] = s;
}
__global__ void gauss_cols_kernel(const float *in, float *out, int nx, int ny, const float *w, int hf) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nx * ny) return;
    const int k = (int)(c / nx), h = (int)(c - (long)k * nx);
    float s = 0.f;
    for (int j = -hf; j <= hf; ++j) s += in[(size_t)min(max(k + j, 0), ny - 1) * nx + h] * w[j + hf];
    out[c] = s;
}

// multiply every row k by coef[k] (the horizontal taper of taper_grad.c:118-190)
__global__ void scale_rows_kernel(float *a, int nx, int ny, const float *coef) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nx * ny) return;
    a[c] *= coef[c / nx];
}

unsigned grid_for(long n) { return (unsigned)std::min<long>((n + kThreads - 1) / kThreads, 4L * kPartials); }

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct Fatt {
    rz_context *ctx;
    cudaStream_t st;
    int nx, ny;
    long n;
    rz_fatt_opts o;
    int nshots;
    const float *srcx, *srcz;
    // device vectors
    float *vp, *vp_old, *vnp1, *grad, *grad_old, *gt, *hgrad, *q, *r, *tmp, *ys;  // ys: [2 m][n]
    float *tobs, *wx, *wy, *taper;
    double *l2, *part;
    float *fpart;
    std::vector<double> rho, alpha;
    int evaluations = 0;
    int err = RZ_OK;
    char msg[256] = {0};

    float *y(int k) { return ys + (size_t)k * n; }
    float *s(int k) { return ys + (size_t)(o.nlbfgs + k) * n; }

    bool ck(cudaError_t e, const char *what) {
        if (e != cudaSuccess && err == RZ_OK) {
            err = e == cudaErrorMemoryAllocation ? RZ_ENOMEM : RZ_ECUDA;
            snprintf(msg, sizeof msg, "%s: %s", what, cudaGetErrorString(e));
        }
        return err == RZ_OK;
    }

    double dot(const float *a, const float *b) {
        dot_kernel<<<kPartials, kThreads, 0, st>>>(a, b, n, part);
        std::vector<double> h(kPartials);
        if (!ck(cudaGetLastError(), "dot") ||
            !ck(cudaMemcpyAsync(h.data(), part, sizeof(double) * kPartials, cudaMemcpyDeviceToHost, st), "dot") ||
            !ck(cudaStreamSynchronize(st), "dot"))
            return 0.0;
        double t = 0.0;
        for (double v : h) t += v;
        return t;
    }

    float maximum(const float *a) {
        max_kernel<<<kPartials, kThreads, 0, st>>>(a, n, fpart);
        std::vector<float> h(kPartials);
        if (!ck(cudaGetLastError(), "max") ||
            !ck(cudaMemcpyAsync(h.data(), fpart, sizeof(float) * kPartials, cudaMemcpyDeviceToHost, st), "max") ||
            !ck(cudaStreamSynchronize(st), "max"))
            return 0.f;
        return *std::max_element(h.begin(), h.end());
    }

    void axpby(double a, const float *x, double b, float *yv) {
        axpby_kernel<<<grid_for(n), kThreads, 0, st>>>(n, a, x, b, yv);
        ck(cudaGetLastError(), "axpby");
    }

    void copy(float *dst, const float *src) {
        ck(cudaMemcpyAsync(dst, src, sizeof(float) * n, cudaMemcpyDeviceToDevice, st), "copy");
    }

    void gauss(float *g) {
        if (o.spatfilter != 4 || !wx) return;
        gauss_rows_kernel<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(g, tmp, nx, ny, wx, o_hfx);
        gauss_cols_kernel<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(tmp, g, nx, ny, wy, o_hfy);
        ck(cudaGetLastError(), "gauss_filt");
    }

    // fatt.c:177-184: the search direction is filtered too
    void precondition_direction() { gauss(hgrad); }

    // precond.c:12-58 restricted to SPATFILTER 4 and the horizontal taper
    void precondition(float *g) {
        gauss(g);
        if (o.taper_hor && taper) {
            scale_rows_kernel<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, st>>>(g, nx, ny, taper);
            ck(cudaGetLastError(), "taper");
        }
    }
    int o_hfx = 0, o_hfy = 0;

    // misfit and preconditioned gradient at model m (grad_obj.c with precond.c)
    double grad_obj(const float *m, float *g) {
        if (err) return 0.0;
        int r = rz_set_velocity(ctx, m, RZ_DEVICE_PTRS);
        if (r == RZ_OK) r = rz_grad_obj(ctx, nshots, srcx, srcz, tobs, g, l2, RZ_DEVICE_PTRS);
        if (r != RZ_OK) {
            err = r;
            snprintf(msg, sizeof msg, "rz_grad_obj: %s", rz_last_error(ctx));
            return 0.0;
        }
        ++evaluations;
        precondition(g);
        double L2 = 0.0;
        ck(cudaMemcpyAsync(&L2, l2, sizeof(double), cudaMemcpyDeviceToHost, st), "misfit");
        ck(cudaStreamSynchronize(st), "misfit");
        return L2;
    }

    // LBFGS.c:36-165 with slot ptr (0-based) holding the newest pair
    void lbfgs(int iter, int ptr) {
        const int m = o.nlbfgs;
        if (iter == 1) {
            axpby(-1.0, grad, 0.0, hgrad);  // Hgrad = gradm = -grad (descent.c)
        } else {
            sub_kernel<<<grid_for(n), kThreads, 0, st>>>(n, grad, grad_old, y(ptr));
            sub_kernel<<<grid_for(n), kThreads, 0, st>>>(n, vp, vp_old, s(ptr));
            ck(cudaGetLastError(), "lbfgs pair");
            const double ys0 = dot(y(ptr), s(ptr)), yy = dot(y(ptr), y(ptr));
            const double gamma = yy != 0.0 ? ys0 / yy : 0.0;
            for (int k = 0; k < m; ++k) {
                const double d = dot(y(k), s(k));
                rho[k] = d != 0.0 ? 1.0 / d : 0.0;
            }
            // visiting order of the first loop: slot order m..1 (reference) or newest to oldest
            std::vector<int> order(m);
            for (int i = 0; i < m; ++i) order[i] = o.recursion == 0 ? m - 1 - i : ((ptr - i) % m + m) % m;
            axpby(-1.0, grad, 0.0, q);  // q = gradm
            for (int k : order) {
                alpha[k] = rho[k] * dot(s(k), q);
                axpby(-alpha[k], y(k), 1.0, q);
            }
            axpby(gamma, q, 0.0, r);
            for (int i = m - 1; i >= 0; --i) {
                const int k = order[i];
                const double beta = rho[k] * dot(y(k), r);
                axpby(alpha[k] - beta, s(k), 1.0, r);
            }
            copy(hgrad, r);
        }
        copy(vp_old, vp);
        copy(grad_old, grad);
    }

    // check_descent.c: a direction that is not a descent direction resets the history
    void check_descent() {
        const double nom = dot(hgrad, grad), den = dot(grad, grad);
        const double p = den != 0.0 ? -nom / den : 0.0;
        if (p < 0.0 && o.nlbfgs > 0)
            ck(cudaMemsetAsync(ys, 0, sizeof(float) * 2 * (size_t)o.nlbfgs * n, st), "reset history");
    }

    // wolfels.c:16-110
    float wolfe(int iter, double L2) {
        float alpha;
        if (iter == 1) {
            const float maxgrad = maximum(hgrad), maxvp = maximum(vp);
            alpha = o.eps_scale * maxvp / maxgrad;
        } else {
            alpha = 1.0f;
        }
        int lsiter = 0;
        bool done = false;
        float mu = 0.0f, nu = 1e30f;
        alpha = alpha / o.scalefac;
        const double g0s0 = dot(grad, hgrad);
        while (!done && !err) {
            if (nu < 1e30f) alpha = (nu + mu) / o.scalefac;
            else alpha = o.scalefac * alpha;
            if (lsiter >= o.stepmax) {
                alpha = 0.0f;
                break;
            }
            model_step_kernel<<<grid_for(n), kThreads, 0, st>>>(n, vp, hgrad, alpha, o.vp_lo, o.vp_hi, vnp1);
            ck(cudaGetLastError(), "model step");
            const double ft = grad_obj(vnp1, gt);
            ++lsiter;
            const double gts0 = dot(gt, hgrad);
            if (ft > L2 + o.c1 * alpha * g0s0) nu = alpha;
            else if (gts0 < o.c2 * g0s0) mu = alpha;
            else done = true;
        }
        return alpha;
    }
};

template <typename T>
bool dalloc(Fatt &F, T **p, size_t count) {
    return F.ck(cudaMalloc((void **)p, sizeof(T) * (count ? count : 1)), "cudaMalloc");
}

// Gaussian filter weights and horizontal taper coefficients (precond.c)
void setup_precond(Fatt &F, const rz_fatt_opts &o, int ny, float dh) {
    // Gaussian filter weights (gauss_filt.c:21-105): odd sizes, sigma = (size/2)/2
    // in integer arithmetic, weights normalised
    int fs = o.filt_size_grad, fs1 = o.filt_size_grad1;
    if (o.spatfilter == 4 && fs != 0 && fs1 != 0 && !F.err) {
        if (!(fs % 2)) fs += fs > 0 ? 1 : -1;
        if (!(fs1 % 2)) fs1 += fs1 > 0 ? 1 : -1;
        const int hfx = std::abs(fs) / 2, hfy = std::abs(fs1) / 2;
        const float sigx = (float)(hfx / 2), sigy = (float)(hfy / 2);
        const float sx = 2.0f * sigx * sigx, sy = 2.0f * sigy * sigy;
        std::vector<float> wxh(2 * hfx + 1), wyh(2 * hfy + 1);
        double sumx = 0.0, sumy = 0.0;
        for (int i = -hfx; i <= hfx; ++i) sumx += wxh[i + hfx] = (float)std::exp(-(double)(i * i) / sx);
        for (int j = -hfy; j <= hfy; ++j) sumy += wyh[j + hfy] = (float)std::exp(-(double)(j * j) / sy);
        for (auto &v : wxh) v = (float)(v / sumx);
        for (auto &v : wyh) v = (float)(v / sumy);
        dalloc(F, &F.wx, wxh.size()), dalloc(F, &F.wy, wyh.size());
        if (!F.err) {
            F.ck(cudaMemcpyAsync(F.wx, wxh.data(), sizeof(float) * wxh.size(), cudaMemcpyHostToDevice, F.st), "w");
            F.ck(cudaMemcpyAsync(F.wy, wyh.data(), sizeof(float) * wyh.size(), cudaMemcpyHostToDevice, F.st), "w");
            F.ck(cudaStreamSynchronize(F.st), "w");
        }
        F.o_hfx = hfx, F.o_hfy = hfy;
    }
    // horizontal taper (taper_grad.c:118-172): 0 above GRADT1, a Gaussian
    // window up to GRADT2, (depth)^EXP_TAPER_GRAD_HOR below (rows 1-based)
    if (o.taper_hor && !F.err) {
        const int t1 = o.gradt1, t2 = o.gradt2, tl = t2 - t1, ifw = t2 - t1 + 1;
        std::vector<float> win(std::max(ifw, 1) + 1, 1.0f), coef(ny, 0.0f);
        const float a = 3.0f;
        for (int i = 1; i <= ifw; ++i)
            if (i <= tl) {
                const double x = (double)(a * (float)(i - tl)) / (tl / 2.0);
                win[i] = (float)std::exp(-(1.0 / 2.0) * x * x);
            }
        int h = 1;
        for (int j = 1; j <= ny; ++j) {
            float tap = 0.0f;
            if (j >= t1 && j <= t2 && h <= ifw) tap = win[h];
            if (j > t2) tap = (float)std::pow((double)((float)j * dh), (double)o.exp_taper_grad_hor);
            coef[j - 1] = tap;
            if (j >= t1) ++h;
        }
        dalloc(F, &F.taper, coef.size());
        if (!F.err) {
            F.ck(cudaMemcpyAsync(F.taper, coef.data(), sizeof(float) * coef.size(), cudaMemcpyHostToDevice, F.st), "t");
            F.ck(cudaStreamSynchronize(F.st), "t");
        }
    }

}

}  // namespace

extern "C" {

int rz_fatt_defaults(rz_fatt_opts *o) {
    if (!o) return RZ_EINVAL;
    memset(o, 0, sizeof *o);
    o->itermax = 30;
    o->nlbfgs = 5;
    o->stepmax = 10;
    o->eps_scale = 0.01f;
    o->c1 = 1e-4f;
    o->c2 = 0.9f;
    o->scalefac = 2.0f;
    o->vp_lo = 300.0f;
    o->vp_hi = 6000.0f;
    o->pro = 0.0f;
    o->spatfilter = 0;
    o->filt_size_grad = 0;
    o->filt_size_grad1 = 0;
    o->taper_hor = 0;
    o->gradt1 = 0;
    o->gradt2 = 0;
    o->exp_taper_grad_hor = 0.0f;
    o->recursion = RZ_LBFGS_SLOT_ORDER;
    return RZ_OK;
}

int rz_precond(rz_context *ctx, const rz_fatt_opts *opts, float *grad, int flags) {
    if (!ctx || !opts || !grad) return RZ_EINVAL;
    Fatt F{};
    float dh = 0.f;
    int ntr = 0;
    int r = rz_context_query(ctx, &F.nx, &F.ny, &dh, &ntr, &F.st);
    if (r != RZ_OK) return r;
    F.ctx = ctx;
    F.n = (long)F.nx * F.ny;
    F.o = *opts;
    float *g = grad;
    dalloc(F, &F.tmp, (size_t)F.n);
    if (!(flags & RZ_DEVICE_PTRS)) {
        dalloc(F, &F.q, (size_t)F.n);
        if (!F.err) F.ck(cudaMemcpyAsync(F.q, grad, sizeof(float) * F.n, cudaMemcpyHostToDevice, F.st), "upload");
        g = F.q;
    }
    setup_precond(F, *opts, F.ny, dh);
    if (!F.err) F.precondition(g);
    if (!F.err && !(flags & RZ_DEVICE_PTRS))
        F.ck(cudaMemcpyAsync(grad, g, sizeof(float) * F.n, cudaMemcpyDeviceToHost, F.st), "download");
    if (!F.err) F.ck(cudaStreamSynchronize(F.st), "sync");
    for (float *p : {F.tmp, F.q, F.wx, F.wy, F.taper})
        if (p) cudaFree(p);
    if (F.err) rz_context_set_error(ctx, F.msg);
    return F.err;
}

int rz_fatt(rz_context *ctx, const rz_fatt_opts *opts, int nshots, const float *srcx, const float *srcz,
            const float *Tobs, float *vp_io, double *misfit, float *steps, int *iterations, int *evaluations) {
    if (!ctx || !opts || !srcx || !srcz || !Tobs || !vp_io || nshots < 1) return RZ_EINVAL;
    struct {
        int nx, ny;
        float dh;
    } g;
    int ntr = 0;
    cudaStream_t st = nullptr;
    int r = rz_context_query(ctx, &g.nx, &g.ny, &g.dh, &ntr, &st);
    if (r != RZ_OK) return r;
    if (opts->itermax < 1 || opts->nlbfgs < 0 || opts->stepmax < 1 || !(opts->scalefac > 0.0f) ||
        (opts->recursion != RZ_LBFGS_SLOT_ORDER && opts->recursion != RZ_LBFGS_CHRONOLOGICAL))
        return RZ_EINVAL;
    Fatt F{};
    F.ctx = ctx;
    F.st = st;
    F.nx = g.nx;
    F.ny = g.ny;
    F.n = (long)g.nx * g.ny;
    F.o = *opts;
    F.nshots = nshots;
    F.srcx = srcx;
    F.srcz = srcz;
    F.rho.assign(std::max(1, opts->nlbfgs), 0.0);
    F.alpha.assign(std::max(1, opts->nlbfgs), 0.0);
    const size_t n = (size_t)F.n, m = (size_t)opts->nlbfgs;
    dalloc(F, &F.vp, n), dalloc(F, &F.vp_old, n), dalloc(F, &F.vnp1, n), dalloc(F, &F.grad, n);
    dalloc(F, &F.grad_old, n), dalloc(F, &F.gt, n), dalloc(F, &F.hgrad, n), dalloc(F, &F.q, n);
    dalloc(F, &F.r, n), dalloc(F, &F.tmp, n), dalloc(F, &F.ys, 2 * m * n), dalloc(F, &F.l2, 1);
    dalloc(F, &F.part, kPartials), dalloc(F, &F.fpart, kPartials);
    dalloc(F, &F.tobs, (size_t)nshots * (ntr > 0 ? ntr : 1));
    if (!F.err && m) F.ck(cudaMemsetAsync(F.ys, 0, sizeof(float) * 2 * m * n, st), "memset");
    if (!F.err) F.ck(cudaMemcpyAsync(F.vp, vp_io, sizeof(float) * n, cudaMemcpyHostToDevice, st), "upload model");
    if (!F.err && ntr > 0)
        F.ck(cudaMemcpyAsync(F.tobs, Tobs, sizeof(float) * nshots * ntr, cudaMemcpyHostToDevice, st), "upload picks");

    setup_precond(F, *opts, g.ny, g.dh);

    // fatt.c:108-258, one workflow stage
    std::vector<double> hist;
    int iter = 1, ptr = 0, done_iters = 0;
    while (iter <= opts->itermax && !F.err) {
        if (iter > 2 && opts->nlbfgs > 0) ptr = (ptr + 1) % opts->nlbfgs;
        const double L2 = F.grad_obj(F.vp, F.grad);
        if (F.err) break;
        F.lbfgs(iter, ptr);
        F.check_descent();
        F.precondition_direction();
        const float step = F.wolfe(iter, L2);
        if (F.err) break;
        hist.push_back(L2);
        if (misfit) misfit[iter - 1] = L2;
        if (steps) steps[iter - 1] = step;
        model_step_kernel<<<grid_for(F.n), kThreads, 0, st>>>(F.n, F.vp, F.hgrad, step, opts->vp_lo, opts->vp_hi, F.vnp1);
        F.ck(cudaGetLastError(), "model update");
        F.copy(F.vp, F.vnp1);
        done_iters = iter;
        double diff = 1e20;
        if (iter > 2) diff = std::fabs((hist[iter - 3] - hist[iter - 1]) / hist[iter - 3]);
        if (diff <= opts->pro || step < 1e-10f) break;
        ++iter;
    }
    if (!F.err) F.ck(cudaMemcpyAsync(vp_io, F.vp, sizeof(float) * n, cudaMemcpyDeviceToHost, st), "download model");
    if (!F.err) F.ck(cudaStreamSynchronize(st), "sync");
    for (float *p : {F.vp, F.vp_old, F.vnp1, F.grad, F.grad_old, F.gt, F.hgrad, F.q, F.r, F.tmp, F.ys, F.tobs, F.wx,
                     F.wy, F.taper, F.fpart})
        if (p) cudaFree(p);
    if (F.l2) cudaFree(F.l2);
    if (F.part) cudaFree(F.part);
    if (iterations) *iterations = done_iters;
    if (evaluations) *evaluations = F.evaluations;
    if (F.err) rz_context_set_error(ctx, F.msg);
    return F.err;
}

}  // extern "C"
