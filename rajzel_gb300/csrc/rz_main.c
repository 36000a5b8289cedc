/*
 * rz_main.c -- `rajzel_gpu PARFILE [WORKFLOW]`: runs a RAJZEL parameter
 * directory on the GPU engine, as the reference's rajzel.c:70-170 does on
 * MPI ranks.
 *
 *   INVMAT 0  forward modelling: picks <PICKS_FILE>_<shot>.dat (SEISMO=1),
 *             traveltime fields <SNAP_FILE>_shot_<shot>.tt (SNAP=1)
 *   INVMAT 1  FATT: one l-BFGS stage per workflow row (fatt.c:98-258), models
 *             <INV_MODELFILE>_vp_stage_<n>.bin, misfit log MISFIT_LOG_FILE
 *   INVMAT 2  grid search over 1-D linear gradient models (grid_search.c),
 *             results in GRIDSEARCH_FILE
 *
 * Shots are numbered from 1 in file names, as in the reference.  The model
 * is read from <MFILE>.vp (READMOD=1) or built as the reference's start model
 * (1D_start_marm.c: water to row 23, then a linear gradient).  Environment:
 * RAJZEL_GPU=<device>, RAJZEL_MODE=fast|reference (default reference).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rajzel_gb300.h"
#include "rajzel_io.h"

static void die(const char *what, const char *msg) {
    fprintf(stderr, "rajzel_gpu: %s: %s\n", what, msg);
    exit(1);
}

static rz_context *g_ctx;

static void check(int st, const char *what) {
    if (st != RZ_OK) die(what, g_ctx ? rz_last_error(g_ctx) : rz_strerror(st));
}

static void io(int st) {
    if (st != 0) die("input/output", rz_io_error());
}

static void *xmalloc(size_t n) {
    void *p = malloc(n ? n : 1);
    if (!p) die("malloc", "out of host memory");
    return p;
}

/* 1D_start_marm.c:26-37 */
static void start_model(const rz_par *P, float *vp) {
    const int h = 23;
    const float vp_water = 1500.0f, vp0 = 1939.0f, grad0 = 1.0f;
    for (int i = 1; i <= P->NX; i++)
        for (int j = 1; j <= P->NY; j++) {
            float v = vp_water;
            if (j >= h) v = grad0 * ((float)(j - h - 1) * P->DH) + vp0;
            vp[(size_t)(j - 1) * P->NX + (i - 1)] = v;
        }
}

/* 1D_start_gridsearch.c:26-37 */
static void gridsearch_model(const rz_par *P, float vp0, float grad0, float *vp) {
    for (int j = 1; j <= P->NY; j++) {
        const float v = grad0 * ((float)(j - 1) * P->DH) + vp0;
        for (int i = 0; i < P->NX; i++) vp[(size_t)(j - 1) * P->NX + i] = v;
    }
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: rajzel_gpu PARFILE [WORKFLOW]\n");
        return 2;
    }
    rz_par P;
    io(rz_read_par(argv[1], &P));
    if (P.N_STREAMER > 0) die("receivers", "towed-streamer geometry (N_STREAMER > 0) is not supported");
    if (P.INVMAT == 1 && (P.SWS_TAPER_GRAD_VERT || P.SWS_TAPER_GRAD_SOURCES || P.SWS_TAPER_CIRCULAR_PER_SHOT ||
                          P.SWS_TAPER_FILE))
        die("FATT", "only the horizontal gradient taper (SWS_TAPER_GRAD_HOR) is built");
    if (P.INVMAT == 1 && (P.GRAD_FILTER || P.MODEL_FILTER))
        die("FATT", "GRAD_FILTER and MODEL_FILTER are not built");

    int ntr = 0, nshots = 0;
    io(rz_read_receivers(P.REC_FILE, P.DH, P.REFREC, &ntr, NULL, NULL, 0));
    int *recx = (int *)xmalloc(sizeof(int) * ntr), *recz = (int *)xmalloc(sizeof(int) * ntr);
    io(rz_read_receivers(P.REC_FILE, P.DH, P.REFREC, &ntr, recx, recz, ntr));
    io(rz_read_sources(P.SOURCE_FILE, &nshots, NULL, NULL, 0));
    float *srcx = (float *)xmalloc(sizeof(float) * nshots), *srcz = (float *)xmalloc(sizeof(float) * nshots);
    io(rz_read_sources(P.SOURCE_FILE, &nshots, srcx, srcz, nshots));

    const size_t ncell = (size_t)P.NX * P.NY;
    float *vp = (float *)xmalloc(sizeof(float) * ncell);
    if (P.READMOD) {
        char fn[RZ_PATH + 8];
        snprintf(fn, sizeof fn, "%s.vp", P.MFILE);
        io(rz_read_model(fn, P.NX, P.NY, vp));
    } else {
        start_model(&P, vp);
    }

    const char *dev = getenv("RAJZEL_GPU"), *mode = getenv("RAJZEL_MODE");
    check(rz_create(&g_ctx, dev ? atoi(dev) : 0), "rz_create");
    check(rz_set_mode(g_ctx, mode && !strcmp(mode, "fast") ? RZ_MODE_FAST : RZ_MODE_REFERENCE), "rz_set_mode");
    rz_grid g = {P.NX, P.NY, P.DH, P.TIME, P.TTNORM, P.EPS_ADJ, 0};
    check(rz_set_grid(g_ctx, &g), "rz_set_grid");
    check(rz_set_velocity(g_ctx, vp, 0), "rz_set_velocity");
    check(rz_set_receivers(g_ctx, ntr, recx, recz), "rz_set_receivers");

    if (P.INVMAT == 0) {
        /* forward.c / eikonal.c:58-66 */
        float *tmod = (float *)xmalloc(sizeof(float) * (size_t)nshots * (ntr ? ntr : 1));
        float *tt = P.SNAP == 1 ? (float *)xmalloc(sizeof(float) * ncell * nshots) : NULL;
        check(rz_forward(g_ctx, nshots, srcx, srcz, tt, tmod, NULL, 0), "rz_forward");
        for (int s = 0; s < nshots; s++) {
            if (P.SEISMO == 1) io(rz_write_picks(P.PICKS_FILE, s + 1, ntr, tmod + (size_t)s * ntr));
            if (tt) {
                char fn[RZ_PATH + 32];
                snprintf(fn, sizeof fn, "%s_shot_%d.tt", P.SNAP_FILE, s + 1);
                io(rz_write_model(fn, P.NX, P.NY, tt + (size_t)s * ncell));
            }
        }
        printf("rajzel_gpu: forward modelling of %d shots done\n", nshots);
        free(tmod);
        free(tt);
    } else if (P.INVMAT == 1 || P.INVMAT == 2) {
        float *tobs = (float *)xmalloc(sizeof(float) * (size_t)nshots * (ntr ? ntr : 1));
        for (int s = 0; s < nshots; s++) io(rz_read_picks(P.DATA_DIR, s + 1, ntr, tobs + (size_t)s * ntr));
        if (P.INVMAT == 1) {
            if (argc < 3) die("FATT", "a workflow file is required (second argument)");
            if (P.GRAD_METHOD != 2 || P.LINESEARCH != 1)
                die("FATT", "only GRAD_METHOD=2 (l-BFGS) with LINESEARCH=1 (Wolfe) is built");
            int nstages = 0;
            io(rz_read_workflow(argv[2], 1, NULL, NULL, NULL, NULL, NULL, NULL, &nstages));
            double *mis = (double *)xmalloc(sizeof(double) * (P.ITERMAX > 0 ? P.ITERMAX : 1));
            float *steps = (float *)xmalloc(sizeof(float) * (P.ITERMAX > 0 ? P.ITERMAX : 1));
            int first = 1;
            for (int stage = 1; stage <= nstages; stage++) {
                rz_fatt_opts o;
                rz_fatt_defaults(&o);
                float wd, wd1;
                io(rz_read_workflow(argv[2], stage, &o.pro, &o.spatfilter, &wd, &wd1, &o.filt_size_grad,
                                    &o.filt_size_grad1, NULL));
                o.itermax = P.ITERMAX;
                o.nlbfgs = P.NLBFGS;
                o.stepmax = P.STEPMAX;
                o.eps_scale = P.EPS_SCALE;
                o.c1 = P.C1;
                o.c2 = P.C2;
                o.scalefac = P.SCALEFAC;
                o.vp_lo = P.VPLOWERLIM;
                o.vp_hi = P.VPUPPERLIM;
                o.taper_hor = P.SWS_TAPER_GRAD_HOR;
                o.gradt1 = P.GRADT1;
                o.gradt2 = P.GRADT2;
                o.exp_taper_grad_hor = P.EXP_TAPER_GRAD_HOR;
                if (o.spatfilter != 0 && o.spatfilter != 4) die("FATT", "only SPATFILTER 0 and 4 are built");
                int iters = 0, evals = 0;
                check(rz_fatt(g_ctx, &o, nshots, srcx, srcz, tobs, vp, mis, steps, &iters, &evals), "rz_fatt");
                /* fatt.c:128-140,202: one line per iteration */
                FILE *fl = fopen(P.MISFIT_LOG_FILE, first ? "w" : "a");
                if (fl) {
                    for (int i = 0; i < iters; i++) fprintf(fl, "%e \t %e \t %d \n", steps[i], mis[i], stage);
                    fclose(fl);
                }
                first = 0;
                char fn[RZ_PATH + 32];
                snprintf(fn, sizeof fn, "%s_vp_stage_%d.bin", P.INV_MODELFILE, stage); /* model_out.c */
                io(rz_write_model(fn, P.NX, P.NY, vp));
                printf("rajzel_gpu: FATT stage %d of %d: %d iterations, %d gradients, misfit %e -> %e\n", stage,
                       nstages, iters, evals, iters ? mis[0] : 0.0, iters ? mis[iters - 1] : 0.0);
            }
            free(mis);
            free(steps);
        } else {
            /* grid_search.c:32-88 */
            const int nvp0 = (int)ceil((P.VP0_2 - P.VP0_1) / P.DVP0);
            const int ngrad0 = (int)ceil((P.GRAD0_2 - P.GRAD0_1) / P.DGRAD0);
            FILE *fg = fopen(P.GRIDSEARCH_FILE, "w");
            if (!fg) die("grid search", "cannot create GRIDSEARCH_FILE");
            fprintf(fg, "Objfcn \t         vp0 \t         grad0 \n");
            float vp0 = P.VP0_1;
            for (int i = 1; i <= nvp0; i++) {
                float grad0 = P.GRAD0_1;
                for (int j = 1; j <= ngrad0; j++) {
                    gridsearch_model(&P, vp0, grad0, vp);
                    check(rz_set_velocity(g_ctx, vp, 0), "rz_set_velocity");
                    double L2 = 0.0;
                    check(rz_misfit(g_ctx, nshots, srcx, srcz, tobs, &L2, 0), "rz_misfit");
                    fprintf(fg, "%e \t %e \t %e \n", (float)L2, vp0, grad0);
                    grad0 += P.DGRAD0;
                }
                vp0 += P.DVP0;
            }
            fclose(fg);
            printf("rajzel_gpu: grid search over %d x %d models done\n", nvp0, ngrad0);
        }
        free(tobs);
    } else {
        die("INVMAT", "must be 0, 1 or 2");
    }
    rz_destroy(g_ctx);
    free(recx);
    free(recz);
    free(srcx);
    free(srcz);
    free(vp);
    return 0;
}
