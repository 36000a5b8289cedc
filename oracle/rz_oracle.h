/*
 * rz_oracle -- CPU restatement of RAJZEL's forward + adjoint Eikonal path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity tests, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py use it as the checker.  The rajzel_gb300
 * product never calls, links or loads it.
 *
 * Layout: flat row-major fields, cell (h,k) (0-based x index h, depth index
 * k) at k*nx + h -- the memory order of the reference's NR matrices
 * A[k+1][h+1] (util.c:177-203).  Receiver and source grid positions are the
 * reference's 1-based indices (receiver.c:55-56, eikonal.c:31-32).
 *
 * Two arithmetic variants:
 *   rzo_*      float storage with the reference's exact float/double mix
 *              (bit-identical to the compiled reference on the same inputs);
 *   rzo_*_f64  the same algorithm and order carried out entirely in double
 *              (the FP64 oracle every float result is measured against).
 */
#ifndef RZ_ORACLE_H
#define RZ_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nx, ny;        /* NX, NY */
    float dh;          /* DH  [m] */
    float time;        /* TIME: 2*TIME is the forward "infinity", 10*TIME the adjoint start */
    float ttnorm;      /* TTNORM: stop when mean |change| < TTNORM */
    float eps_adj;     /* EPS_ADJ: water level of the adjoint sweep */
    int max_passes;    /* safety limit on outer passes (the reference has none) */
} rzo_grid;

/* status codes */
#define RZO_OK 0
#define RZO_EINVAL 1
#define RZO_ENOCONV 2

/* forward: returns status; *passes = outer iterations (4 sweeps each). */
int rzo_eikonal(const rzo_grid *g, const float *S, float srcx, float srcz, float *TT, int *passes);
int rzo_eikonal_f64(const rzo_grid *g, const double *S, double srcx, double srcz, double *TT, int *passes);

/* Tmod[i] = TT at receiver i (calc_FA.c:15-18). */
void rzo_calc_fa(const rzo_grid *g, const float *TT, int ntr, const int *recx, const int *recz, float *Tmod);

/* residuals, misfit and receiver scaling (calc_FA_res.c:34-72); Tres is
   in/out: muted picks (Tobs<0) leave their entry untouched. */
double rzo_calc_res(const rzo_grid *g, const float *TT, const float *Tmod, const float *Tobs, float *Tres, int ntr,
                    const int *recx, const int *recz);
double rzo_calc_res_f64(const rzo_grid *g, const double *TT, const double *Tmod, const double *Tobs, double *Tres,
                        int ntr, const int *recx, const int *recz);

/* adjoint: returns status; *passes as above. */
int rzo_eikonal_adj(const rzo_grid *g, const float *TT, const float *Tres, int ntr, const int *recx, const int *recz,
                    float *lam, int *passes);
int rzo_eikonal_adj_f64(const rzo_grid *g, const double *TT, const double *Tres, int ntr, const int *recx,
                        const int *recz, double *lam, int *passes);

/* per-shot gradient lam*S^3 + frame copy, added into grad (ass_grad.c:20-46). */
void rzo_ass_grad(const rzo_grid *g, float *grad, const float *S, const float *lam);
void rzo_ass_grad_f64(const rzo_grid *g, double *grad, const double *S, const double *lam);
void rzo_cp_grad_frame(const rzo_grid *g, float *A);
void rzo_cp_grad_frame_f64(const rzo_grid *g, double *A);

/* grad_obj on one rank over shots 0..nshots-1 (grad_obj.c:10-81):
   returns status; *L2 = 0.5*sum of shot misfits; grad = stacked gradient.
   Tobs is [nshots][ntr].  Tres_io carries the residual array between shots
   exactly like the reference's single Tres buffer (muted picks keep the
   previous shot's value); pass NULL to start from zeros. */
int rzo_grad_obj(const rzo_grid *g, const float *S, int nshots, const float *srcx, const float *srcz, int ntr,
                 const int *recx, const int *recz, const float *Tobs, float *grad, double *L2, float *Tres_io,
                 int *fwd_passes, int *adj_passes);
int rzo_grad_obj_f64(const rzo_grid *g, const double *S, int nshots, const double *srcx, const double *srcz, int ntr,
                     const int *recx, const int *recz, const double *Tobs, double *grad, double *L2);

/* forward() over shots: TT_all is [nshots][ny][nx], Tmod_all [nshots][ntr]. */
int rzo_forward(const rzo_grid *g, const float *S, int nshots, const float *srcx, const float *srcz, int ntr,
                const int *recx, const int *recz, float *TT_all, float *Tmod_all, int *passes);

/* init_MPIshot's block partition (init_MPIshot.c:19-30): 1-based [*s1,*s2). */
/* Exact discrete adjoint gradient dJ/dVp of J = 0.5 sum (Tmod-Tobs)^2 over
   unmuted picks (Tobs >= 0), FP64 forward; not in the reference. */
int rzo_grad_exact_f64(const rzo_grid *g, const double *S, int nshots, const double *srcx, const double *srcz,
                       int ntr, const int *recx, const int *recz, const double *Tobs, double *grad_vp, double *L2);
int rzo_misfit_f64(const rzo_grid *g, const double *S, int nshots, const double *srcx, const double *srcz, int ntr,
                   const int *recx, const int *recz, const double *Tobs, double *L2);

void rzo_shot_partition(int nshots, int np, int myid, int *s1, int *s2);

/* count floats in [lo,hi] where pow(s,3.0) != the once-rounded cube. */
long rzo_pin_cube(float lo, float hi);

#ifdef __cplusplus
}
#endif
#endif
