/*
 * rajzel_compat.h -- the reference's own entry points, served by the GB300
 * engine.  A RAJZEL build compiles rajzel_gb300/csrc/rz_compat.c in place of
 * eikonal.c, eikonal_adj.c, forward.c and grad_obj.c (and drops sweep.c,
 * sweep_adj.c, init_travel_adj.c, norm1.c, store_mat.c, zero_travel.c), and
 * links librajzel_gb300.so.  Signatures are exactly fd.h:60,62,68,72; the
 * functions read the reference's globals (NX, NY, DH, TIME, TTNORM, EPS_ADJ,
 * SNAP, SEISMO, NSHOT1, NSHOT2, DATA_DIR, SNAP_FILE) as the originals do.
 *
 * The host program provides, as RAJZEL does: the globals (globvar.h) and
 * err(), writemod(), write_picks(), precond() (util.c, writemod.c,
 * write_picks.c, precond.c).
 * Compile rz_compat.c with -DRZ_COMPAT_MPI (and mpi.h) to keep grad_obj's
 * MPI_Allreduce of the misfit and sum_grad_MPI() of the gradient
 * (grad_obj.c:58-68); without it the shim is single-rank.
 */
#ifndef RAJZEL_COMPAT_H
#define RAJZEL_COMPAT_H

#ifdef __cplusplus
extern "C" {
#endif

/* eikonal.c:10 */
void eikonal(float **S, float **TT, float *Tmod, float **srcpos, int ishot, int nshots, int **recpos, int ntr);
/* eikonal_adj.c:10 */
void eikonal_adj(float **TT, float *Tres, float **lam, int **recpos, int ntr, int ishot, int **recflag);
/* forward.c:10 */
void forward(float **S, float **TT, float *Tmod, float **srcpos, int nshots, int **recpos, int ntr);
/* grad_obj.c:10 */
double grad_obj(float **grad, float **S, float **TT, float **lam, float *Tmod, float *Tobs, float *Tres,
                float **srcpos, int nshots, int **recpos, int ntr, int iter);

/* Engine selection for the shim (not in the reference): CUDA device and
   arithmetic mode (RZ_MODE_REFERENCE = 0, RZ_MODE_FAST = 1).  Defaults:
   device 0, reference mode; the environment variables RAJZEL_GPU and
   RAJZEL_MODE=fast override them at first use. */
int rz_compat_configure(int device, int mode);

#ifdef __cplusplus
}
#endif
#endif
