/*
 * rajzel_gb300.h -- C ABI of the GB300 forward + adjoint Eikonal engine.
 *
 * Drop-in for RAJZEL's hot path: the shot loop of grad_obj()/forward() and
 * the solvers eikonal()/eikonal_adj() (reference fd.h:60,62,68,72 and
 * grad_obj.c:10-81).  Plain C types only; every call returns an RZ_* status
 * (the reference aborts through err()/MPI_Abort instead, util.c:7-17).
 *
 * Conventions (identical to the reference's data, only the container
 * differs):
 *   - fields are row-major [ny][nx] float32, x fastest: cell (h,k) at
 *     k*nx+h, i.e. the memory order of the reference's NR matrix A[k+1][h+1]
 *     (util.c:177-203) with the row pointers dropped;
 *   - source positions are metres, like srcpos[1][s] (x) and srcpos[2][s]
 *     (depth) (sources.c:68-69); the grid index is iround(x/DH)
 *     (eikonal.c:31-32);
 *   - receiver positions are the reference's 1-based grid indices,
 *     recpos[1][i] (x) and recpos[2][i] (depth) (receiver.c:55-56);
 *   - rz_grid carries the process globals the path reads (NX, NY, DH, TIME,
 *     TTNORM, EPS_ADJ; globvar.h:12-15,96).
 *
 * Pointers are host pointers unless RZ_DEVICE_PTRS is passed in `flags`, in
 * which case every array argument of that call is a device pointer on the
 * context's device and the call returns without synchronising (results are
 * valid once the context stream reaches them).
 *
 * Threading: one context per host thread at a time; contexts are independent.
 */
#ifndef RAJZEL_GB300_H
#define RAJZEL_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RZ_ABI_VERSION 1

/* status codes */
#define RZ_OK 0
#define RZ_EINVAL 1          /* bad argument (the reference would read out of bounds or spin) */
#define RZ_ENOCONV 2         /* TTNORM not met within rz_grid.max_passes outer passes */
#define RZ_ECUDA 3           /* CUDA runtime/driver error (see rz_last_error) */
#define RZ_ENOMEM 4          /* device allocation failed */
#define RZ_ETIMEOUT 5        /* a bounded device-side wait gave up (kernel returned cleanly) */
#define RZ_ESTATE 6          /* call order: grid/model/receivers not set */
#define RZ_EUNSUPPORTED 7    /* grid shape beyond the kernels' limits */

/* arithmetic modes */
#define RZ_MODE_REFERENCE 0  /* bit-identical to the reference's float/double arithmetic */
#define RZ_MODE_FAST 1       /* FP32 sweeps, FP64 misfit and gradient stack */
#define RZ_MODE_FP64 2       /* FP64 oracle: every sweep, residual and stack in double (validation, slow) */

/* gradient kinds (rz_set_gradient) */
#define RZ_GRADIENT_REFERENCE 0 /* Leung-Qian adjoint, lambda*S^3 + frame copy (ass_grad.c) */
#define RZ_GRADIENT_EXACT 1     /* exact discrete adjoint: dJ/dVp of the float misfit */

/* flags */
#define RZ_DEVICE_PTRS 1

typedef struct rz_context rz_context;

/* The reference globals the hot path reads. */
typedef struct {
    int nx;          /* NX */
    int ny;          /* NY */
    float dh;        /* DH [m] */
    float time;      /* TIME: 2*TIME initialises traveltimes, 10*TIME lambda */
    float ttnorm;    /* TTNORM: stop when mean |change| < TTNORM; must be > 0 */
    float eps_adj;   /* EPS_ADJ: adjoint water level */
    int max_passes;  /* outer-pass limit (the reference loops forever); <=0 -> 10000 */
} rz_grid;

int rz_abi_version(void);
const char *rz_strerror(int status);

/* Context on CUDA device `device` (owns all device memory it allocates). */
int rz_create(rz_context **ctx, int device);
void rz_destroy(rz_context *ctx);
const char *rz_last_error(const rz_context *ctx);

/* cudaStream_t to issue work on (NULL = the context's own stream). */
int rz_set_stream(rz_context *ctx, void *cuda_stream);
/* RZ_MODE_REFERENCE (default) or RZ_MODE_FAST. */
int rz_set_mode(rz_context *ctx, int mode);

/* Which gradient rz_grad_obj returns (not in the reference, which has only
   the first):
     RZ_GRADIENT_REFERENCE  the reference's: Leung-Qian adjoint state
                            (sweep_adj.c), lambda*S^3 stacked and
                            frame-copied (ass_grad.c, cp_grad_frame.c);
     RZ_GRADIENT_EXACT      the exact derivative dJ/dVp of the discrete
                            misfit J = 0.5 sum (Tmod - Tobs)^2 over unmuted
                            picks: the adjoint of the Godunov update
                            linearised at the converged traveltimes, solved
                            by the same wavefront sweeps; no frame copy. */
int rz_set_gradient(rz_context *ctx, int kind);

/* Grid and solver constants (replaces the globals NX..EPS_ADJ). */
int rz_set_grid(rz_context *ctx, const rz_grid *grid);

/* Slowness model S [ny][nx] (the S matrix of eikonal(), fd.h:60). */
int rz_set_slowness(rz_context *ctx, const float *S, int flags);
/* Velocity model; S = 1/vp per cell as calc_S.c:21 (float division). */
int rz_set_velocity(rz_context *ctx, const float *vp, int flags);

/* Receiver geometry shared by all shots: ntr receivers at 1-based grid
   indices (recpos[1..2][1..ntr] of receiver.c).  Host pointers. */
int rz_set_receivers(rz_context *ctx, int ntr, const int *recx, const int *recz);

/* Autotuner (no counterpart in the reference): runs rz_grad_obj on the
   caller's batch once per candidate launch shape, times each with CUDA
   events, and keeps the fastest for later rz_grad_obj calls with the same
   number of shots, mode and gradient kind.  A shape is
     - the band width: warps that sweep, i.e. strips swept together -- the
       balanced width for the fewest bands of <= 16 strips and for one and
       two more bands;
     - the fixpoint checks' task height: at most 32, 64 or 128 rows of 128
       columns per warp task;
     - the CTA width: as many warps as fit at the same occupancy (the spare
       ones share the cell-parallel phases), or the sweeping warps alone.
   No shape changes a result.  Arguments as rz_grad_obj (grad receives the
   gradient); best_warps / best_ms (may be NULL) the chosen band width and
   its time; cand_warps / cand_ms [*ncand] (may be NULL) every band width
   with its fastest shape's time, *ncand set to their number.
   rz_tuned_shape returns the whole chosen shape. */
int rz_autotune(rz_context *ctx, int nshots, const float *srcx, const float *srcz, const float *Tobs, float *grad,
                int flags, int *best_warps, double *best_ms, int *cand_warps, double *cand_ms, int *ncand);
int rz_tuned_shape(rz_context *ctx, int nshots, int *warps, int *cta_warps, int *check_rows);

/* CUDA graphs (default on): rz_grad_obj captures its device sequence
   (per-shot resets, shot-kernel launches, stacks, frame copy, misfit sum)
   once and replays it while the buffers, shapes and settings it baked in are
   unchanged; inputs are uploaded before each replay.  Results are the same
   either way.  0 disables capture and frees the graph. */
int rz_set_graphs(rz_context *ctx, int enable);

/* Device memory the per-shot field slots (traveltimes, lambda, pass
   snapshot, skewed copies: about 28 bytes per padded cell) may occupy.
   A batch whose slots exceed it runs in chunks of as many shots as fit, in
   shot order, stacking each chunk onto the previous ones; results do not
   depend on the chunk size.  0 (the default) = 90% of free device memory.
   Not in the reference, whose MPI ranks each hold one shot's fields. */
int rz_set_memory_cap(rz_context *ctx, size_t bytes);

/* forward(): traveltimes for nshots sources (forward.c:19-24 over
   eikonal(), eikonal.c:10-76).
     srcx, srcz : [nshots] metres (host pointers)
     TT         : [nshots][ny][nx] or NULL
     Tmod       : [nshots][ntr]   or NULL (calc_FA.c:15-18)
     passes     : [nshots] outer passes per shot or NULL (host pointer) */
int rz_forward(rz_context *ctx, int nshots, const float *srcx, const float *srcz, float *TT, float *Tmod,
               int *passes, int flags);

/* grad_obj(): misfit and stacked gradient over nshots sources on one GPU
   (grad_obj.c:27-73 with sum_grad_MPI/MPI_Allreduce replaced by the
   in-device shot stack; preconditioning not applied).
     Tobs : [nshots][ntr] observed picks; Tobs<0 mutes a pick (calc_FA_res.c:39)
     grad : [ny][nx] stacked gradient
     L2   : misfit 0.5*sum(Tres^2) (grad_obj.c:61)
   A muted pick contributes a zero residual. */
int rz_grad_obj(rz_context *ctx, int nshots, const float *srcx, const float *srcz, const float *Tobs, float *grad,
                double *L2, int flags);

/* Backward of the forward map Vp -> Tmod (vector-Jacobian product, not in
   the reference): grad[ny][nx] = sum over shots of (dTmod/dVp)^T dTmod_s,
   with dTmod [nshots][ntr] the cotangents of the picks.  The forward fields
   are recomputed inside the call from the model and the sources (chunk by
   chunk under the memory cap); no earlier rz_forward is needed.
   rz_grad_obj with RZ_GRADIENT_EXACT equals rz_backward with
   dTmod = Tmod - Tobs (0 for muted picks). */
int rz_backward(rz_context *ctx, int nshots, const float *srcx, const float *srcz, const float *dTmod, float *grad,
                int flags);

/* ----------------------------------------------------------------------
 * FATT inversion (fatt.c:108-258): l-BFGS with a weak-Wolfe line search over
 * rz_grad_obj, on the GPU; one workflow stage.  Parameter names are the
 * reference's (RAJZEL .inp and workflow files).
 * ---------------------------------------------------------------------- */
#define RZ_LBFGS_SLOT_ORDER 0    /* history visited in slot order, as LBFGS.c:113-150 */
#define RZ_LBFGS_CHRONOLOGICAL 1 /* newest to oldest and back (Nocedal & Wright 7.4) */

typedef struct {
    int itermax;              /* ITERMAX: iterations of the stage */
    int nlbfgs;               /* NLBFGS: stored (s, y) pairs */
    int stepmax;              /* STEPMAX: gradient evaluations per line search */
    float eps_scale;          /* EPS_SCALE: first trial step = EPS_SCALE*max(Vp)/max(Hgrad) */
    float c1, c2;             /* C1, C2: Wolfe constants */
    float scalefac;           /* SCALEFAC: step growth / bisection factor */
    float vp_lo, vp_hi;       /* VPLOWERLIM, VPUPPERLIM: hard model limits */
    float pro;                /* PRO: stop once |L2(i-2)-L2(i)|/L2(i-2) <= PRO */
    int spatfilter;           /* SPATFILTER: 0 none, 4 Gaussian filter (gauss_filt.c) */
    int filt_size_grad;       /* FILT_SIZE_GRAD: filter length in x (grid points) */
    int filt_size_grad1;      /* FILT_SIZE_GRAD1: filter length in depth */
    int taper_hor;            /* SWS_TAPER_GRAD_HOR: horizontal gradient taper */
    int gradt1, gradt2;       /* GRADT1, GRADT2: taper rows (1-based) */
    float exp_taper_grad_hor; /* EXP_TAPER_GRAD_HOR: depth scaling exponent below GRADT2 */
    int recursion;            /* RZ_LBFGS_SLOT_ORDER or RZ_LBFGS_CHRONOLOGICAL */
} rz_fatt_opts;

/* The reference's example settings (par/RAJZEL_marm_OBC.inp) with NLBFGS 5,
   ITERMAX 30, no filter or taper, slot-order recursion. */
int rz_fatt_defaults(rz_fatt_opts *opts);

/* precond() (precond.c:12-58) for SPATFILTER 4 and the horizontal taper:
   grad [ny][nx] is filtered (gauss_filt.c) and tapered (taper_grad.c, sws 2)
   in place, as opts selects.  The context must hold the grid. */
int rz_precond(rz_context *ctx, const rz_fatt_opts *opts, float *grad, int flags);

/* Invert for Vp.  The context must hold the grid and receivers (the model is
   set by this call).  vp [ny][nx] is the start model on entry and the final
   model on return (host pointers); Tobs [nshots][ntr] the observed picks;
   misfit[itermax] and steps[itermax] receive L2 and the accepted step length
   per iteration (the columns of the reference's misfit log, fatt.c:202), or
   NULL; iterations and evaluations (or NULL) the iterations done and
   rz_grad_obj calls made.  Misfit, dot products and the l-BFGS scalars are
   FP64; vectors FP32. */
int rz_fatt(rz_context *ctx, const rz_fatt_opts *opts, int nshots, const float *srcx, const float *srcz,
            const float *Tobs, float *vp, double *misfit, float *steps, int *iterations, int *evaluations);

/* Several grids in one launch (no counterpart in the reference): each
   context holds one grid, its model and receivers; shot i of grid g is a job
   of one persistent kernel whose CTAs take jobs largest grid first, so small
   grids fill the SMs while the large ones run.  Per grid the results equal
   rz_grad_obj on that context (gradient kind and refinement included).  All
   contexts must use the same device and mode (FP64 excepted); the work runs
   on ctxs[0]'s stream.
     nshots[g], srcx[g], srcz[g], Tobs[g], grad[g]: as rz_grad_obj, per grid
     L2[ngrids]: misfit per grid */
int rz_grad_obj_multi(int ngrids, rz_context *const *ctxs, const int *nshots, const float *const *srcx,
                      const float *const *srcz, const float *const *Tobs, float *const *grad, double *L2, int flags);

/* Misfit only: forward solves and residuals of nshots sources, L2 =
   0.5*sum (Tmod - Tobs)^2 over unmuted picks (the objective of
   grid_search.c:62-80, calc_FA_res.c:34-47); no adjoint, no gradient. */
int rz_misfit(rz_context *ctx, int nshots, const float *srcx, const float *srcz, const float *Tobs, double *L2,
              int flags);

/* ----------------------------------------------------------------------
 * FP64 oracle on the GPU (not in the reference, which computes in float
 * with one double expression, sweep.c:94).  The same algorithm -- sweep.c,
 * sweep_adj.c, norm1.c's stopping rule, calc_FA_res.c, ass_grad.c,
 * cp_grad_frame.c -- carried out entirely in double, one CTA per shot; the
 * exact gradient kind solves the exact discrete adjoint in double.  It is the
 * yardstick of every float result:
 *   - RZ_MODE_FP64 (rz_set_mode) runs rz_forward, rz_grad_obj, rz_misfit and
 *     rz_backward in FP64 and rounds their results to float;
 *   - rz_forward_f64 / rz_grad_obj_f64 return the double results;
 *   - rz_set_error_check makes every later rz_forward / rz_grad_obj /
 *     rz_misfit of a float mode also run the FP64 oracle on the same inputs
 *     and record the error of its result (rz_error_report).
 * ---------------------------------------------------------------------- */
typedef struct {
    int shots;           /* shots whose traveltime fields were compared (those
                            kept in the field slots: all, unless the batch ran
                            in chunks under the memory cap) */
    double tt_rel;       /* worst shot's max|TT - TT64| / max|TT64| */
    double tt_rel_l2;    /* worst shot's ||TT - TT64||_2 / ||TT64||_2 */
    double tmod_rel;     /* max|Tmod - Tmod64| / max|Tmod64| over all picks */
    double grad_rel_l2;  /* ||grad - grad64||_2 / ||grad64||_2 (gradient calls) */
    double grad_rel_max; /* max|grad - grad64| / max|grad64| (gradient calls) */
    double misfit_rel;   /* |L2 - L2_64| / |L2_64| (gradient and misfit calls) */
} rz_error;

/* Traveltimes TT [nshots][ny][nx] and picks Tmod [nshots][ntr] (either may
   be NULL) of the FP64 oracle. */
int rz_forward_f64(rz_context *ctx, int nshots, const float *srcx, const float *srcz, double *TT, double *Tmod,
                   int flags);
/* Gradient [ny][nx] and misfit of the FP64 oracle, of the context's
   gradient kind (Leung-Qian with frame copy, or exact dJ/dVp). */
int rz_grad_obj_f64(rz_context *ctx, int nshots, const float *srcx, const float *srcz, const float *Tobs,
                    double *grad, double *L2, int flags);
/* 1: later float calls also run the FP64 oracle on their inputs (the call
   then synchronises and takes the oracle's time too); 0: off (default).  With
   refinement on (rz_set_refine) the oracle's forward runs to the fixpoint of
   the discrete equations (until a pass changes no cell) instead of stopping
   at TTNORM: on rough models the TTNORM-stopped iterate lies up to ~1e-5
   from that fixpoint, which a refined field reaches. */
int rz_set_error_check(rz_context *ctx, int enable);
/* The error of the last checked call's results against the FP64 oracle. */
int rz_error_report(rz_context *ctx, rz_error *err);

/* Traveltime refinement (not in the reference; default off).  Float32
   traveltimes carry the rounding of every update along their path: on a
   1700 x 350 grid the reference's own float arithmetic ends up to 2e-5
   (relative) from the FP64 fixpoint, and residuals of a few hundredths of a
   second inherit that.  With refinement on, every shot's converged field T
   is corrected by one linear solve, delta = r + W delta, with r the residual
   of the discrete equations evaluated in float-float and W the Godunov
   weights (the sweeps of the exact adjoint, in the forward orders), after
   which T + delta agrees with the FP64 fixpoint to float precision.  All
   results use the refined field: traveltimes and picks (rounded to float),
   residuals and misfit (in double), the Leung-Qian adjoint's inputs, and
   the exact gradient (weights of the refined field).  Costs one more linear
   solve per shot; in reference mode the results are then more accurate than
   the reference's rather than bit-identical to them. */
int rz_set_refine(rz_context *ctx, int enable);

/* Test hook for the failure path (no counterpart in the reference, which
   aborts through err()/MPI_Abort, util.c:7-17).  Every device wait for
   another warp is bounded: after spin_limit polls (0 = the default budget of
   2^21 polls) it records a status bit, raises the CTA's abort word so
   every later wait of the CTA returns at once, and the kernel ends normally;
   waits for the CTA's own tensor copies always let the copies land.  With
   withhold_handoff != 0 the first warp of every CTA withholds one hand-off
   signal in its first sweep, so the next warp's wait runs out: the call then
   returns RZ_ETIMEOUT (status bit 1) and the context stays usable.  0, 0
   restores normal operation. */
int rz_set_wait_test(rz_context *ctx, unsigned spin_limit, int withhold_handoff);

/* Per-shot results of the last rz_forward/rz_grad_obj (host pointers, any
   may be NULL): outer passes of forward/adjoint, device status bits. */
int rz_shot_info(rz_context *ctx, int shot, int *fwd_passes, int *adj_passes, int *status);

/* Device status bits, as rz_shot_info, rz_batch_status and
   rz_eikonal_noalloc's info[1] report them: bit 0 a bounded wait for a tensor
   copy gave up, bit 1 a bounded wait for another warp gave up (both
   RZ_ETIMEOUT), bit 2 / bit 3 the forward / adjoint did not meet TTNORM
   within max_passes (RZ_ENOCONV), bit 4 a source outside the grid, bit 5 an
   invalid slowness (RZ_EINVAL).  rz_status_code maps them to the RZ_* code a
   synchronous call would return. */
int rz_status_code(int bits);
/* OR of the status bits of every shot of the last batch: the check for
   calls made with RZ_DEVICE_PTRS, which return before the device is done
   (this call waits for the context stream). */
int rz_batch_status(rz_context *ctx, int *bits);

/* Directional sweeps of shot `shot` in the last batch that were actually
   run (forward, adjoint): 4 per swept pass.  A pass that a parallel fixpoint
   check proves to change no cell is counted in rz_shot_info's pass counts
   (the reference runs it) but not swept; after its first pass the exact
   adjoint stops at the first sweep that moves no cell's mu by more than 1e-6
   of its value, so its count need not be a multiple of 4. */
int rz_shot_work(rz_context *ctx, int shot, int *fwd_swept, int *adj_swept);

/* Fields of shot `shot` from the last rz_grad_obj: TT, lambda [ny][nx],
   Tres [ntr] (scaled residuals as passed to eikonal_adj).  TT and lambda
   are kept only for the shots of the last chunk (all shots when the batch
   fit the memory cap); Tres is kept for every shot. */
int rz_shot_fields(rz_context *ctx, int shot, float *TT, float *lam, float *Tres, int flags);

/* Accounting: kernels this context has launched so far, and the summed
   device time (CUDA events on the context stream) of the shot kernels
   launched since the previous call (the list is cleared by this call). */
int rz_kernel_stats(rz_context *ctx, long long *launches, double *shot_kernel_ms, int *shot_kernel_calls);

/* Diagnostics: device time stamps (ns, %globaltimer) of shot `shot` in the
   last batch: [0] start, [1] forward converged (and refined), [2] residuals
   done, [3] adjoint prepared, [4] adjoint converged, [5] first forward sweep
   done, [6] first adjoint sweep done, [7] refinement started (0 without
   refinement).  stamps has 8 entries. */
int rz_shot_timeline(rz_context *ctx, int shot, unsigned long long *stamps);

/* eikonal(): one source -> TT [ny][nx] and Tmod [ntr] (eikonal.c:10-76). */
int rz_eikonal(rz_context *ctx, float srcx, float srcz, float *TT, float *Tmod, int *passes, int flags);

/* eikonal_adj(): adjoint field lam [ny][nx] for a given traveltime field
   TT [ny][nx] and scaled residuals Tres [ntr] (eikonal_adj.c:10-59). */
int rz_eikonal_adj(rz_context *ctx, const float *TT, const float *Tres, float *lam, int *passes, int flags);

/* Allocation-free forward solve (no counterpart in the reference: RAJZEL
   always runs on the host and allocates its own scratch with matrix()).
   For callers that cannot allocate GPU memory -- a solver step working
   inside a fixed memory pool or a memory budget fixed up front, or a host
   with no allocator available -- this computes one shot's traveltimes
   exactly like rz_eikonal() in reference mode, with its working space in a
   static 32 MiB device array that every GPU loading this library holds until
   exit.  S (slowness [ny][nx]), TT (output [ny][nx]) and info (2 ints: outer
   passes, status bits as rz_status_code reads them) are device pointers; the
   call is asynchronous on `stream` (NULL = legacy default).  The slowness is
   checked on the device as rz_set_slowness checks it: a zero, negative or
   non-finite value sets bit 5 of info[1] (RZ_EINVAL), no solve runs and TT
   is undefined.  Grids needing more than the static space return
   RZ_EUNSUPPORTED.  The first call on a device sets up (looks up the array's
   address) and should come before any stream capture; calls that overlap on
   the GPU share the array and race. */
int rz_eikonal_noalloc(const rz_grid *grid, const float *S, float srcx, float srcz, float *TT, int *info,
                       void *stream);

#ifdef __cplusplus
}
#endif
#endif
