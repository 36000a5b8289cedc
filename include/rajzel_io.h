/*
 * rajzel_io.h -- RAJZEL's file formats, so existing parameter directories
 * run on the GPU engine: the positional .inp parameter file (read_par.c),
 * the FATT workflow file (read_par_inv.c), source and receiver lists
 * (sources.c, receiver.c), binary models (readmod.c, writemod.c format 3)
 * and pick files (write_picks.c, calc_FA_res.c).  Plain C, host only.
 * All functions return RZ_OK (0) or RZ_EINVAL (1, with a message from
 * rz_io_error()).
 */
#ifndef RAJZEL_IO_H
#define RAJZEL_IO_H

#ifdef __cplusplus
extern "C" {
#endif

#define RZ_PATH 256

/* The parameters of a RAJZEL .inp file, in file order (read_par.c:72-270);
   names are the reference's globals. */
typedef struct {
    int INVMAT, NX, NY;
    float DH, TIME;
    char SOURCE_FILE[RZ_PATH];
    int READMOD;
    char MFILE[RZ_PATH];
    int SNAP, IDX, IDY, SNAP_FORMAT;
    char SNAP_FILE[RZ_PATH];
    int SEISMO;
    char REC_FILE[RZ_PATH];
    float REFREC[2];
    int N_STREAMER;
    float REC_INCR_X, REC_INCR_Y;
    char PICKS_FILE[RZ_PATH];
    float TTNORM;
    char LOG_FILE[RZ_PATH];
    int LOG, ITERMAX;
    float EPS_ADJ;
    char JACOBIAN[RZ_PATH], DATA_DIR[RZ_PATH];
    int TAPER, TAPERLENGTH, INVTYPE;
    int GRADT1, GRADT2, GRADT3, GRADT4;
    int SWS_TAPER_GRAD_VERT, SWS_TAPER_GRAD_HOR;
    float EXP_TAPER_GRAD_HOR;
    int SWS_TAPER_GRAD_SOURCES, SWS_TAPER_CIRCULAR_PER_SHOT, SRTSHAPE;
    float SRTRADIUS;
    int FILTSIZE, SWS_TAPER_FILE;
    char INV_MODELFILE[RZ_PATH];
    int nfstart, nf, nfstart_jac, nf_jac;
    float VPUPPERLIM, VPLOWERLIM;
    int GRAD_METHOD, NLBFGS, MODEL_FILTER, FILT_SIZE, LINESEARCH;
    float EPS_SCALE, C1, C2;
    int STEPMAX;
    float SCALEFAC;
    char MISFIT_LOG_FILE[RZ_PATH];
    int MIN_ITER, GRAD_FILTER, FILT_SIZE_GRAD;
    float VP0_1, VP0_2, DVP0, GRAD0_1, GRAD0_2, DGRAD0;
    char GRIDSEARCH_FILE[RZ_PATH];
    int nlines; /* parameter lines found (63 in a complete file) */
} rz_par;

/* message of the last failing call (thread-local) */
const char *rz_io_error(void);

/* read_par.c: positional "label = value" lines, '#' lines skipped */
int rz_read_par(const char *path, rz_par *par);

/* read_par_inv.c: workflow row `stage` (1-based) of a FATT workflow file;
   nstages (may be NULL) receives the number of rows */
int rz_read_workflow(const char *path, int stage, float *pro, int *spatfilter, float *wd_damp, float *wd_damp1,
                     int *filt_size_grad, int *filt_size_grad1, int *nstages);

/* sources.c:37-73: first line the number of sources, then one line each with
   at least 6 numbers: x, (unused), depth, tshift, fc, amp.  With cap == 0
   only *nshots is set; else up to cap positions (metres) are stored. */
int rz_read_sources(const char *path, int *nshots, float *srcx, float *srcz, int cap);

/* receiver.c:36-78: one "x depth" pair per line (metres); grid indices
   iround((x + REFREC)/DH), receivers with x index <= 0 dropped.  With cap == 0
   only *ntr is set. */
int rz_read_receivers(const char *path, float dh, const float refrec[2], int *ntr, int *recx, int *recz, int cap);

/* readmod.c:30-40 / writemod.c format 3: float32, x outer, depth inner;
   vp is [ny][nx] (depth-major, x fastest) in memory */
int rz_read_model(const char *path, int nx, int ny, float *vp);
int rz_write_model(const char *path, int nx, int ny, const float *vp);

/* write_picks.c / calc_FA_res.c:28-37: <prefix>_<shot>.dat, one "%e" per line */
int rz_read_picks(const char *prefix, int shot, int ntr, float *t);
int rz_write_picks(const char *prefix, int shot, int ntr, const float *t);

#ifdef __cplusplus
}
#endif
#endif
