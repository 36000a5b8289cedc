/*
 * rz_oracle.c -- CPU restatement of RAJZEL's forward + adjoint Eikonal path.
 *
 * TEST INFRASTRUCTURE ONLY (see rz_oracle.h).  Compile with
 * -ffp-contract=off: every expression below is evaluated exactly as written,
 * operation by operation, because the float variant must reproduce the
 * reference's float/double rounding sequence bit for bit.
 *
 * Sweep order and arithmetic follow sweep.c:24-102 and sweep_adj.c:25-75;
 * the drivers follow eikonal.c:31-57 and eikonal_adj.c:31-51; the stopping
 * rule follows norm1.c:20-29; receiver/adjoint initialisation follows
 * init_travel_adj.c:22-58 and init_recflag.c:18-33 (restated as an O(ntr)
 * scatter with the same "last receiver wins" result); residuals follow
 * calc_FA_res.c:34-72; gradient assembly follows ass_grad.c:20-46 and
 * cp_grad_frame.c:18-49; the shot loop follows grad_obj.c:27-73.
 */
#include "rz_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define IDX(g, h, k) ((size_t)(k) * (size_t)(g)->nx + (size_t)(h))

/* iround() of fd.h:18 applied to a float coordinate divided by DH. */
static int grid_index(float x, float dh) { return (int)floor((double)(x / dh) + 0.5); }
static int grid_index_f64(double x, double dh) { return (int)floor(x / dh + 0.5); }

static int check_grid(const rzo_grid *g) {
    if (!g || g->nx < 2 || g->ny < 2) return RZO_EINVAL;
    if (!(g->dh > 0.0f) || !(g->ttnorm > 0.0f)) return RZO_EINVAL;
    return RZO_OK;
}

/* ------------------------------------------------------------------------ */
/* forward, float variant                                                    */
/* ------------------------------------------------------------------------ */

/* One Godunov-upwind update (sweep.c:89-97).  a/b are the x/y neighbour
   minima, own the cell's current value. */
static inline float godunov_update(float a, float b, float s, float dh, float own) {
    float d = a - b;
    float sh = s * dh;
    float tt;
    if (fabs(d) >= sh) {
        tt = fminf(a, b) + sh;
    } else {
        double p = 2.0 * ((double)s * (double)s) * ((double)dh * (double)dh);
        double q = p - (double)d * (double)d;
        tt = (float)(((double)(a + b) + sqrt(q)) / 2.0);
    }
    return fminf(own, tt);
}

/* One directional Gauss-Seidel pass (sweep.c:24-102): x outer, depth inner,
   starting at (h0,k0) and stepping (dx,dy).  Missing neighbours at the grid
   border are replaced by the cell's own value. */
static void sweep_fwd(const rzo_grid *g, const float *S, float *T, int h0, int dx, int k0, int dy) {
    const int nx = g->nx, ny = g->ny;
    int h = h0;
    for (int i = 0; i < nx; i++, h += dx) {
        int k = k0;
        for (int j = 0; j < ny; j++, k += dy) {
            float own = T[IDX(g, h, k)];
            float w = (h > 0) ? T[IDX(g, h - 1, k)] : own;
            float e = (h < nx - 1) ? T[IDX(g, h + 1, k)] : own;
            float n = (k > 0) ? T[IDX(g, h, k - 1)] : own;
            float s = (k < ny - 1) ? T[IDX(g, h, k + 1)] : own;
            float a = fminf(w, e);
            float b = fminf(n, s);
            T[IDX(g, h, k)] = godunov_update(a, b, S[IDX(g, h, k)], g->dh, own);
        }
    }
}

/* norm1.c:20-29: float accumulator, x outer, each term added in double. */
static float mean_abs_change(const rzo_grid *g, const float *T, const float *Told) {
    float sum = 0.0f;
    for (int h = 0; h < g->nx; h++)
        for (int k = 0; k < g->ny; k++) sum = (float)((double)sum + fabs(T[IDX(g, h, k)] - Told[IDX(g, h, k)]));
    return sum / (g->nx * g->ny);
}

int rzo_eikonal(const rzo_grid *g, const float *S, float srcx, float srcz, float *TT, int *passes) {
    if (check_grid(g)) return RZO_EINVAL;
    const int nx = g->nx, ny = g->ny;
    int hs = grid_index(srcx, g->dh) - 1, ks = grid_index(srcz, g->dh) - 1;
    if (hs < 0 || hs >= nx || ks < 0 || ks >= ny) return RZO_EINVAL;
    size_t n = (size_t)nx * ny;
    float *Told = (float *)malloc(n * sizeof(float));
    if (!Told) return RZO_EINVAL;
    float init = (float)(2.0 * g->time); /* zero_travel.c:22 */
    for (size_t c = 0; c < n; c++) TT[c] = init;
    TT[IDX(g, hs, ks)] = 0.0f;
    float l1 = (float)(10.0 * g->time);
    int it = 0, status = RZO_OK;
    while (l1 >= g->ttnorm) {
        if (g->max_passes > 0 && it >= g->max_passes) { status = RZO_ENOCONV; break; }
        memcpy(Told, TT, n * sizeof(float));
        sweep_fwd(g, S, TT, 0, 1, 0, 1);           /* (+x,+y) */
        sweep_fwd(g, S, TT, nx - 1, -1, 0, 1);     /* (-x,+y) */
        sweep_fwd(g, S, TT, nx - 1, -1, ny - 1, -1); /* (-x,-y) */
        sweep_fwd(g, S, TT, 0, 1, ny - 1, -1);     /* (+x,-y) */
        l1 = mean_abs_change(g, TT, Told);
        it++;
    }
    free(Told);
    if (passes) *passes = it;
    return status;
}

void rzo_calc_fa(const rzo_grid *g, const float *TT, int ntr, const int *recx, const int *recz, float *Tmod) {
    for (int i = 0; i < ntr; i++) Tmod[i] = TT[IDX(g, recx[i] - 1, recz[i] - 1)];
}

/* ------------------------------------------------------------------------ */
/* forward, double variant                                                   */
/* ------------------------------------------------------------------------ */

static inline double godunov_update_f64(double a, double b, double s, double dh, double own) {
    double d = a - b;
    double sh = s * dh;
    double tt;
    if (fabs(d) >= sh) tt = fmin(a, b) + sh;
    else tt = (a + b + sqrt(2.0 * (s * s) * (dh * dh) - d * d)) / 2.0;
    return fmin(own, tt);
}

static void sweep_fwd_f64(const rzo_grid *g, const double *S, double *T, int h0, int dx, int k0, int dy) {
    const int nx = g->nx, ny = g->ny;
    int h = h0;
    for (int i = 0; i < nx; i++, h += dx) {
        int k = k0;
        for (int j = 0; j < ny; j++, k += dy) {
            double own = T[IDX(g, h, k)];
            double w = (h > 0) ? T[IDX(g, h - 1, k)] : own;
            double e = (h < nx - 1) ? T[IDX(g, h + 1, k)] : own;
            double n = (k > 0) ? T[IDX(g, h, k - 1)] : own;
            double s = (k < ny - 1) ? T[IDX(g, h, k + 1)] : own;
            T[IDX(g, h, k)] = godunov_update_f64(fmin(w, e), fmin(n, s), S[IDX(g, h, k)], g->dh, own);
        }
    }
}

static double mean_abs_change_f64(const rzo_grid *g, const double *T, const double *Told) {
    double sum = 0.0;
    for (int h = 0; h < g->nx; h++)
        for (int k = 0; k < g->ny; k++) sum += fabs(T[IDX(g, h, k)] - Told[IDX(g, h, k)]);
    return sum / ((double)g->nx * g->ny);
}

int rzo_eikonal_f64(const rzo_grid *g, const double *S, double srcx, double srcz, double *TT, int *passes) {
    if (check_grid(g)) return RZO_EINVAL;
    const int nx = g->nx, ny = g->ny;
    int hs = grid_index_f64(srcx, g->dh) - 1, ks = grid_index_f64(srcz, g->dh) - 1;
    if (hs < 0 || hs >= nx || ks < 0 || ks >= ny) return RZO_EINVAL;
    size_t n = (size_t)nx * ny;
    double *Told = (double *)malloc(n * sizeof(double));
    if (!Told) return RZO_EINVAL;
    for (size_t c = 0; c < n; c++) TT[c] = 2.0 * g->time;
    TT[IDX(g, hs, ks)] = 0.0;
    double l1 = 10.0 * g->time;
    int it = 0, status = RZO_OK;
    while (l1 >= g->ttnorm) {
        if (g->max_passes > 0 && it >= g->max_passes) { status = RZO_ENOCONV; break; }
        memcpy(Told, TT, n * sizeof(double));
        sweep_fwd_f64(g, S, TT, 0, 1, 0, 1);
        sweep_fwd_f64(g, S, TT, nx - 1, -1, 0, 1);
        sweep_fwd_f64(g, S, TT, nx - 1, -1, ny - 1, -1);
        sweep_fwd_f64(g, S, TT, 0, 1, ny - 1, -1);
        l1 = mean_abs_change_f64(g, TT, Told);
        it++;
    }
    free(Told);
    if (passes) *passes = it;
    return status;
}

/* ------------------------------------------------------------------------ */
/* residuals                                                                 */
/* ------------------------------------------------------------------------ */

double rzo_calc_res(const rzo_grid *g, const float *TT, const float *Tmod, const float *Tobs, float *Tres, int ntr,
                    const int *recx, const int *recz) {
    double l2 = 0.0;
    for (int i = 0; i < ntr; i++) {
        if (Tobs[i] >= 0.0f) {
            int h = recx[i] - 1, k = recz[i] - 1;
            Tres[i] = Tmod[i] - Tobs[i];
            l2 += Tres[i] * Tres[i];
            if (recz[i] <= g->ny - 1) {
                float grad = (TT[IDX(g, h, k + 1)] - TT[IDX(g, h, k)]) / g->dh;
                if (fabs(grad) > 0.0) Tres[i] = Tres[i] / grad;
                else Tres[i] = 0.0f;
            } else if (recz[i] == g->ny) {
                float grad = (TT[IDX(g, h, k)] - TT[IDX(g, h, k - 1)]) / g->dh;
                if (fabs(grad) > 0.0) Tres[i] = Tres[i] / grad;
                else Tres[i] = 0.0f;
            }
        }
    }
    return l2;
}

double rzo_calc_res_f64(const rzo_grid *g, const double *TT, const double *Tmod, const double *Tobs, double *Tres,
                        int ntr, const int *recx, const int *recz) {
    double l2 = 0.0;
    for (int i = 0; i < ntr; i++) {
        if (Tobs[i] >= 0.0) {
            int h = recx[i] - 1, k = recz[i] - 1;
            Tres[i] = Tmod[i] - Tobs[i];
            l2 += Tres[i] * Tres[i];
            double grad;
            if (recz[i] <= g->ny - 1) grad = (TT[IDX(g, h, k + 1)] - TT[IDX(g, h, k)]) / g->dh;
            else grad = (TT[IDX(g, h, k)] - TT[IDX(g, h, k - 1)]) / g->dh;
            Tres[i] = (fabs(grad) > 0.0) ? Tres[i] / grad : 0.0;
        }
    }
    return l2;
}

/* ------------------------------------------------------------------------ */
/* adjoint, float variant                                                    */
/* ------------------------------------------------------------------------ */

/* init_travel_adj.c:22-58 + init_recflag.c:18-33: frame 0, interior
   10*TIME, interior receiver cells Tres (last receiver wins); skip[] marks
   receiver cells anywhere on the grid. */
static void init_adjoint(const rzo_grid *g, float *lam, unsigned char *skip, const float *Tres, int ntr,
                         const int *recx, const int *recz) {
    const int nx = g->nx, ny = g->ny;
    float start = (float)(10.0 * g->time);
    for (int k = 0; k < ny; k++)
        for (int h = 0; h < nx; h++) {
            int interior = (h > 0 && h < nx - 1 && k > 0 && k < ny - 1);
            lam[IDX(g, h, k)] = interior ? start : 0.0f;
            skip[IDX(g, h, k)] = 0;
        }
    for (int l = 0; l < ntr; l++) {
        int h = recx[l] - 1, k = recz[l] - 1;
        if (h < 0 || h >= nx || k < 0 || k >= ny) continue;
        skip[IDX(g, h, k)] = 1;
        if (h > 0 && h < nx - 1 && k > 0 && k < ny - 1) lam[IDX(g, h, k)] = Tres[l];
    }
}

/* One Leung-Qian pass over the interior (sweep_adj.c:25-75). */
static void sweep_adj(const rzo_grid *g, const float *T, float *L, const unsigned char *skip, int h0, int dx, int k0,
                      int dy) {
    const int nx = g->nx, ny = g->ny;
    const float dh = g->dh;
    int h = h0;
    for (int i = 1; i < nx - 1; i++, h += dx) {
        int k = k0;
        for (int j = 1; j < ny - 1; j++, k += dy) {
            size_t c = IDX(g, h, k);
            if (skip[c]) continue;
            float tc = T[c], te = T[c + 1], tw = T[c - 1], ts = T[c + nx], tn = T[c - nx];
            float ap = -(te - tc) / dh;
            float am = -(tc - tw) / dh;
            float bp = -(ts - tc) / dh;
            float bm = -(tc - tn) / dh;
            float app = (ap + fabs(ap)) / 2.0;
            float apm = (ap - fabs(ap)) / 2.0;
            float amp = (am + fabs(am)) / 2.0;
            float amm = (am - fabs(am)) / 2.0;
            float bpp = (bp + fabs(bp)) / 2.0;
            float bpm = (bp - fabs(bp)) / 2.0;
            float bmp = (bm + fabs(bm)) / 2.0;
            float bmm = (bm - fabs(bm)) / 2.0;
            float lhs = (app - amm) / dh + (bpp - bmm) / dh;
            float rhs = (amp * L[c - 1] - apm * L[c + 1]) / dh + (bmp * L[c - nx] - bpm * L[c + nx]) / dh;
            float lt = (lhs > g->eps_adj) ? rhs / lhs : 0.0f;
            L[c] = fminf(L[c], lt);
            if (tc >= 9999999 || ts >= 9999999 || tn >= 9999999 || te >= 9999999 || tw >= 9999999) L[c] = 0.0f;
        }
    }
}

int rzo_eikonal_adj(const rzo_grid *g, const float *TT, const float *Tres, int ntr, const int *recx, const int *recz,
                    float *lam, int *passes) {
    if (check_grid(g)) return RZO_EINVAL;
    const int nx = g->nx, ny = g->ny;
    size_t n = (size_t)nx * ny;
    float *Lold = (float *)malloc(n * sizeof(float));
    unsigned char *skip = (unsigned char *)malloc(n);
    if (!Lold || !skip) { free(Lold); free(skip); return RZO_EINVAL; }
    init_adjoint(g, lam, skip, Tres, ntr, recx, recz);
    float l1 = (float)(10.0 * g->time);
    int it = 0, status = RZO_OK;
    while (l1 >= g->ttnorm) {
        if (g->max_passes > 0 && it >= g->max_passes) { status = RZO_ENOCONV; break; }
        memcpy(Lold, lam, n * sizeof(float));
        sweep_adj(g, TT, lam, skip, 1, 1, 1, 1);                /* (+x,+y) */
        sweep_adj(g, TT, lam, skip, 1, 1, ny - 2, -1);          /* (+x,-y) */
        sweep_adj(g, TT, lam, skip, nx - 2, -1, 1, 1);          /* (-x,+y) */
        sweep_adj(g, TT, lam, skip, nx - 2, -1, ny - 2, -1);    /* (-x,-y) */
        l1 = mean_abs_change(g, lam, Lold);
        it++;
    }
    free(Lold);
    free(skip);
    if (passes) *passes = it;
    return status;
}

/* ------------------------------------------------------------------------ */
/* adjoint, double variant                                                   */
/* ------------------------------------------------------------------------ */

static void sweep_adj_f64(const rzo_grid *g, const double *T, double *L, const unsigned char *skip, int h0, int dx,
                          int k0, int dy) {
    const int nx = g->nx, ny = g->ny;
    const double dh = g->dh;
    int h = h0;
    for (int i = 1; i < nx - 1; i++, h += dx) {
        int k = k0;
        for (int j = 1; j < ny - 1; j++, k += dy) {
            size_t c = IDX(g, h, k);
            if (skip[c]) continue;
            double tc = T[c];
            double ap = -(T[c + 1] - tc) / dh, am = -(tc - T[c - 1]) / dh;
            double bp = -(T[c + nx] - tc) / dh, bm = -(tc - T[c - nx]) / dh;
            double app = fmax(ap, 0.0), apm = fmin(ap, 0.0), amp = fmax(am, 0.0), amm = fmin(am, 0.0);
            double bpp = fmax(bp, 0.0), bpm = fmin(bp, 0.0), bmp = fmax(bm, 0.0), bmm = fmin(bm, 0.0);
            double lhs = (app - amm) / dh + (bpp - bmm) / dh;
            double rhs = (amp * L[c - 1] - apm * L[c + 1]) / dh + (bmp * L[c - nx] - bpm * L[c + nx]) / dh;
            double lt = (lhs > g->eps_adj) ? rhs / lhs : 0.0;
            L[c] = fmin(L[c], lt);
        }
    }
}

int rzo_eikonal_adj_f64(const rzo_grid *g, const double *TT, const double *Tres, int ntr, const int *recx,
                        const int *recz, double *lam, int *passes) {
    if (check_grid(g)) return RZO_EINVAL;
    const int nx = g->nx, ny = g->ny;
    size_t n = (size_t)nx * ny;
    double *Lold = (double *)malloc(n * sizeof(double));
    unsigned char *skip = (unsigned char *)calloc(n, 1);
    if (!Lold || !skip) { free(Lold); free(skip); return RZO_EINVAL; }
    for (int k = 0; k < ny; k++)
        for (int h = 0; h < nx; h++)
            lam[IDX(g, h, k)] = (h > 0 && h < nx - 1 && k > 0 && k < ny - 1) ? 10.0 * g->time : 0.0;
    for (int l = 0; l < ntr; l++) {
        int h = recx[l] - 1, k = recz[l] - 1;
        if (h < 0 || h >= nx || k < 0 || k >= ny) continue;
        skip[IDX(g, h, k)] = 1;
        if (h > 0 && h < nx - 1 && k > 0 && k < ny - 1) lam[IDX(g, h, k)] = Tres[l];
    }
    double l1 = 10.0 * g->time;
    int it = 0, status = RZO_OK;
    while (l1 >= g->ttnorm) {
        if (g->max_passes > 0 && it >= g->max_passes) { status = RZO_ENOCONV; break; }
        memcpy(Lold, lam, n * sizeof(double));
        sweep_adj_f64(g, TT, lam, skip, 1, 1, 1, 1);
        sweep_adj_f64(g, TT, lam, skip, 1, 1, ny - 2, -1);
        sweep_adj_f64(g, TT, lam, skip, nx - 2, -1, 1, 1);
        sweep_adj_f64(g, TT, lam, skip, nx - 2, -1, ny - 2, -1);
        l1 = mean_abs_change_f64(g, lam, Lold);
        it++;
    }
    free(Lold);
    free(skip);
    if (passes) *passes = it;
    return status;
}

/* ------------------------------------------------------------------------ */
/* gradient assembly                                                         */
/* ------------------------------------------------------------------------ */

/* cp_grad_frame.c:18-49, same copy sequence. */
void rzo_cp_grad_frame(const rzo_grid *g, float *A) {
    const int nx = g->nx, ny = g->ny;
    for (int h = 0; h < nx; h++) { A[IDX(g, h, 1)] = A[IDX(g, h, 2)]; A[IDX(g, h, 0)] = A[IDX(g, h, 1)]; }
    for (int h = 0; h < nx; h++) { A[IDX(g, h, ny - 2)] = A[IDX(g, h, ny - 3)]; A[IDX(g, h, ny - 1)] = A[IDX(g, h, ny - 2)]; }
    for (int k = 0; k < ny; k++) { A[IDX(g, 1, k)] = A[IDX(g, 2, k)]; A[IDX(g, 0, k)] = A[IDX(g, 1, k)]; }
    for (int k = 0; k < ny; k++) { A[IDX(g, nx - 2, k)] = A[IDX(g, nx - 3, k)]; A[IDX(g, nx - 1, k)] = A[IDX(g, nx - 2, k)]; }
}

void rzo_cp_grad_frame_f64(const rzo_grid *g, double *A) {
    const int nx = g->nx, ny = g->ny;
    for (int h = 0; h < nx; h++) { A[IDX(g, h, 1)] = A[IDX(g, h, 2)]; A[IDX(g, h, 0)] = A[IDX(g, h, 1)]; }
    for (int h = 0; h < nx; h++) { A[IDX(g, h, ny - 2)] = A[IDX(g, h, ny - 3)]; A[IDX(g, h, ny - 1)] = A[IDX(g, h, ny - 2)]; }
    for (int k = 0; k < ny; k++) { A[IDX(g, 1, k)] = A[IDX(g, 2, k)]; A[IDX(g, 0, k)] = A[IDX(g, 1, k)]; }
    for (int k = 0; k < ny; k++) { A[IDX(g, nx - 2, k)] = A[IDX(g, nx - 3, k)]; A[IDX(g, nx - 1, k)] = A[IDX(g, nx - 2, k)]; }
}

/* ass_grad.c:23 multiplies by pow(S,3.0) from the C library.  That value is
   faithful but not always the correctly rounded cube (rzo_pin_cube counts
   the floats where they differ by one double ulp), so the restatement calls
   pow exactly as the reference does. */
static inline double cube_ref(float s) { return pow((double)s, 3.0); }

/* correctly rounded S^3 (S*S is exact in double, one more multiply rounds once) */
static inline double cube_rn(float s) {
    double s2 = (double)s * (double)s;
    return s2 * (double)s;
}

void rzo_ass_grad(const rzo_grid *g, float *grad, const float *S, const float *lam) {
    const int nx = g->nx, ny = g->ny;
    size_t n = (size_t)nx * ny;
    float *gs = (float *)calloc(n, sizeof(float));
    for (int h = 1; h < nx - 1; h++)
        for (int k = 1; k < ny - 1; k++) gs[IDX(g, h, k)] = (float)((double)lam[IDX(g, h, k)] * cube_ref(S[IDX(g, h, k)]));
    rzo_cp_grad_frame(g, gs);
    for (size_t c = 0; c < n; c++) grad[c] += gs[c];
    free(gs);
}

void rzo_ass_grad_f64(const rzo_grid *g, double *grad, const double *S, const double *lam) {
    const int nx = g->nx, ny = g->ny;
    size_t n = (size_t)nx * ny;
    double *gs = (double *)calloc(n, sizeof(double));
    for (int h = 1; h < nx - 1; h++)
        for (int k = 1; k < ny - 1; k++) {
            double s = S[IDX(g, h, k)];
            gs[IDX(g, h, k)] = lam[IDX(g, h, k)] * s * s * s;
        }
    rzo_cp_grad_frame_f64(g, gs);
    for (size_t c = 0; c < n; c++) grad[c] += gs[c];
    free(gs);
}

/* ------------------------------------------------------------------------ */
/* shot loops                                                                */
/* ------------------------------------------------------------------------ */

int rzo_grad_obj(const rzo_grid *g, const float *S, int nshots, const float *srcx, const float *srcz, int ntr,
                 const int *recx, const int *recz, const float *Tobs, float *grad, double *L2, float *Tres_io,
                 int *fwd_passes, int *adj_passes) {
    if (check_grid(g)) return RZO_EINVAL;
    size_t n = (size_t)g->nx * g->ny;
    float *TT = (float *)malloc(n * sizeof(float));
    float *lam = (float *)malloc(n * sizeof(float));
    float *Tmod = (float *)malloc((ntr > 0 ? ntr : 1) * sizeof(float));
    float *Tres = Tres_io ? Tres_io : (float *)calloc(ntr > 0 ? ntr : 1, sizeof(float));
    int status = RZO_OK;
    double l2sum = 0.0;
    memset(grad, 0, n * sizeof(float));
    for (int s = 0; s < nshots && status == RZO_OK; s++) {
        int pf = 0, pa = 0;
        status = rzo_eikonal(g, S, srcx[s], srcz[s], TT, &pf);
        if (status) break;
        rzo_calc_fa(g, TT, ntr, recx, recz, Tmod);
        l2sum += rzo_calc_res(g, TT, Tmod, Tobs + (size_t)s * ntr, Tres, ntr, recx, recz);
        status = rzo_eikonal_adj(g, TT, Tres, ntr, recx, recz, lam, &pa);
        if (status) break;
        rzo_ass_grad(g, grad, S, lam);
        if (fwd_passes) fwd_passes[s] = pf;
        if (adj_passes) adj_passes[s] = pa;
    }
    if (status == RZO_OK) {
        /* grad_obj.c:60-73 on one rank: Allreduce and sum_grad_MPI are the
           identity (sum_grad_MPI's corner cell is rewritten by the frame
           copy), precond with all filters/tapers off is the identity. */
        rzo_cp_grad_frame(g, grad);
        if (L2) *L2 = 0.5 * l2sum;
    }
    free(TT); free(lam); free(Tmod);
    if (!Tres_io) free(Tres);
    return status;
}

int rzo_grad_obj_f64(const rzo_grid *g, const double *S, int nshots, const double *srcx, const double *srcz, int ntr,
                     const int *recx, const int *recz, const double *Tobs, double *grad, double *L2) {
    if (check_grid(g)) return RZO_EINVAL;
    size_t n = (size_t)g->nx * g->ny;
    double *TT = (double *)malloc(n * sizeof(double));
    double *lam = (double *)malloc(n * sizeof(double));
    double *Tmod = (double *)malloc((ntr > 0 ? ntr : 1) * sizeof(double));
    double *Tres = (double *)calloc(ntr > 0 ? ntr : 1, sizeof(double));
    int status = RZO_OK;
    double l2sum = 0.0;
    memset(grad, 0, n * sizeof(double));
    for (int s = 0; s < nshots && status == RZO_OK; s++) {
        status = rzo_eikonal_f64(g, S, srcx[s], srcz[s], TT, NULL);
        if (status) break;
        for (int i = 0; i < ntr; i++) Tmod[i] = TT[IDX(g, recx[i] - 1, recz[i] - 1)];
        l2sum += rzo_calc_res_f64(g, TT, Tmod, Tobs + (size_t)s * ntr, Tres, ntr, recx, recz);
        status = rzo_eikonal_adj_f64(g, TT, Tres, ntr, recx, recz, lam, NULL);
        if (status) break;
        rzo_ass_grad_f64(g, grad, S, lam);
    }
    if (status == RZO_OK) {
        rzo_cp_grad_frame_f64(g, grad);
        if (L2) *L2 = 0.5 * l2sum;
    }
    free(TT); free(lam); free(Tmod); free(Tres);
    return status;
}

int rzo_forward(const rzo_grid *g, const float *S, int nshots, const float *srcx, const float *srcz, int ntr,
                const int *recx, const int *recz, float *TT_all, float *Tmod_all, int *passes) {
    size_t n = (size_t)g->nx * g->ny;
    for (int s = 0; s < nshots; s++) {
        int st = rzo_eikonal(g, S, srcx[s], srcz[s], TT_all + (size_t)s * n, passes ? passes + s : NULL);
        if (st) return st;
        rzo_calc_fa(g, TT_all + (size_t)s * n, ntr, recx, recz, Tmod_all + (size_t)s * ntr);
    }
    return RZO_OK;
}

/* ------------------------------------------------------------------------ */
/* exact discrete adjoint (FP64; not in the reference)                       */
/* ------------------------------------------------------------------------ */
/* The converged forward field satisfies T_c = G(a_c, b_c, S_c) at every cell
   but the source, with a_c / b_c the smaller x / z neighbour (sweep.c:89-97).
   Linearising G: one-sided (|a-b| >= S*DH): dT_c = dT_argmin + DH dS_c;
   two-sided with r = sqrt(2 S^2 DH^2 - (a-b)^2):
   dT_c = (r-d)/(2r) dT_a + (r+d)/(2r) dT_b + S DH^2 / r dS_c,  d = a - b.
   Every dependency points to a strictly earlier-arriving cell, so the adjoint
   system mu = R + W^T mu is solved exactly by visiting cells in order of
   decreasing traveltime.  dJ/dVp = -S^2 dJ/dS (S = 1/Vp). */
typedef struct {
    double t;
    size_t c;
} rzo_tc;

static int cmp_desc(const void *x, const void *y) {
    double a = ((const rzo_tc *)x)->t, b = ((const rzo_tc *)y)->t;
    return (a < b) - (a > b);
}

static void exact_coef_f64(const rzo_grid *g, const double *T, const double *S, int h, int k, long *xn, double *wx,
                           long *zn, double *wz, double *gs) {
    const int nx = g->nx, ny = g->ny;
    const double inf = 1e300;
    double tw = h > 0 ? T[IDX(g, h - 1, k)] : inf, te = h < nx - 1 ? T[IDX(g, h + 1, k)] : inf;
    double tn = k > 0 ? T[IDX(g, h, k - 1)] : inf, ts = k < ny - 1 ? T[IDX(g, h, k + 1)] : inf;
    long ia = tw <= te ? (long)IDX(g, h - 1, k) : (long)IDX(g, h + 1, k);
    long ib = tn <= ts ? (long)IDX(g, h, k - 1) : (long)IDX(g, h, k + 1);
    double a = tw <= te ? tw : te, b = tn <= ts ? tn : ts;
    double s = S[IDX(g, h, k)], sh = s * g->dh, d = a - b;
    *xn = -1, *zn = -1, *wx = 0.0, *wz = 0.0;
    if (fabs(d) >= sh) {
        if (a <= b) *xn = ia, *wx = 1.0;
        else *zn = ib, *wz = 1.0;
        *gs = g->dh;
    } else {
        double r = sqrt(2.0 * sh * sh - d * d);
        *xn = ia, *wx = (r - d) / (2.0 * r);
        *zn = ib, *wz = (r + d) / (2.0 * r);
        *gs = s * (double)g->dh * (double)g->dh / r;
    }
}

int rzo_grad_exact_f64(const rzo_grid *g, const double *S, int nshots, const double *srcx, const double *srcz,
                       int ntr, const int *recx, const int *recz, const double *Tobs, double *grad_vp, double *L2) {
    if (check_grid(g)) return RZO_EINVAL;
    const size_t n = (size_t)g->nx * g->ny;
    double *T = (double *)malloc(n * sizeof(double));
    double *mu = (double *)malloc(n * sizeof(double));
    double *gS = (double *)calloc(n, sizeof(double));
    rzo_tc *ord = (rzo_tc *)malloc(n * sizeof(rzo_tc));
    int status = RZO_OK;
    double l2 = 0.0;
    for (int sh = 0; sh < nshots && status == RZO_OK; sh++) {
        status = rzo_eikonal_f64(g, S, srcx[sh], srcz[sh], T, NULL);
        if (status) break;
        const size_t src = IDX(g, grid_index_f64(srcx[sh], g->dh) - 1, grid_index_f64(srcz[sh], g->dh) - 1);
        memset(mu, 0, n * sizeof(double));
        for (int i = 0; i < ntr; i++) {
            const double tob = Tobs[(size_t)sh * ntr + i];
            if (tob < 0.0) continue; /* muted pick */
            const size_t c = IDX(g, recx[i] - 1, recz[i] - 1);
            const double res = T[c] - tob;
            mu[c] += res;
            l2 += res * res;
        }
        for (size_t c = 0; c < n; c++) ord[c].t = T[c], ord[c].c = c;
        qsort(ord, n, sizeof(rzo_tc), cmp_desc);
        for (size_t i = 0; i < n; i++) {
            const size_t c = ord[i].c;
            if (c == src) continue;
            long xn, zn;
            double wx, wz, gs;
            exact_coef_f64(g, T, S, (int)(c % g->nx), (int)(c / g->nx), &xn, &wx, &zn, &wz, &gs);
            if (xn >= 0) mu[xn] += wx * mu[c];
            if (zn >= 0) mu[zn] += wz * mu[c];
            gS[c] += mu[c] * gs;
        }
    }
    if (status == RZO_OK) {
        for (size_t c = 0; c < n; c++) grad_vp[c] = -S[c] * S[c] * gS[c];
        if (L2) *L2 = 0.5 * l2;
    }
    free(T); free(mu); free(gS); free(ord);
    return status;
}

/* misfit 0.5 * sum (Tmod - Tobs)^2 over unmuted picks, FP64 forward */
int rzo_misfit_f64(const rzo_grid *g, const double *S, int nshots, const double *srcx, const double *srcz, int ntr,
                   const int *recx, const int *recz, const double *Tobs, double *L2) {
    if (check_grid(g)) return RZO_EINVAL;
    const size_t n = (size_t)g->nx * g->ny;
    double *T = (double *)malloc(n * sizeof(double));
    double l2 = 0.0;
    int status = RZO_OK;
    for (int sh = 0; sh < nshots && status == RZO_OK; sh++) {
        status = rzo_eikonal_f64(g, S, srcx[sh], srcz[sh], T, NULL);
        for (int i = 0; i < ntr && status == RZO_OK; i++) {
            const double tob = Tobs[(size_t)sh * ntr + i];
            if (tob < 0.0) continue;
            const double res = T[IDX(g, recx[i] - 1, recz[i] - 1)] - tob;
            l2 += res * res;
        }
    }
    free(T);
    if (status == RZO_OK && L2) *L2 = 0.5 * l2;
    return status;
}

void rzo_shot_partition(int nshots, int np, int myid, int *s1, int *s2) {
    int a = (nshots / np) * myid, b;
    if (nshots % np > myid) {
        a += myid;
        b = a + (nshots / np) + 1;
    } else {
        a += nshots % np;
        b = a + (nshots / np);
    }
    *s1 = a + 1;
    *s2 = b + 1;
}

/* Exhaustive pin: count float s in [lo,hi] where libm's pow(s,3.0) differs
   from the once-rounded cube used above (ass_grad.c:23 calls pow). */
long rzo_pin_cube(float lo, float hi) {
    long bad = 0;
    for (float s = lo; s <= hi; s = nextafterf(s, 2.0f * hi))
        if (cube_ref(s) != cube_rn(s)) bad++;
    return bad;
}
