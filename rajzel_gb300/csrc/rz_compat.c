/*
 * rz_compat.c -- eikonal(), eikonal_adj(), forward() and grad_obj() with the
 * reference's signatures and globals, running on the GB300 engine through
 * the C ABI of rajzel_gb300.h.  See include/rajzel_compat.h for how a RAJZEL
 * build uses it.
 *
 * The NR matrices of the reference (util.c:177-203) store their elements in
 * one contiguous block starting at &A[1][1], row after row: exactly the
 * [NY][NX] layout of the C ABI, so they are passed without copying.
 */
#include "rajzel_compat.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rajzel_gb300.h"

#ifdef RZ_COMPAT_MPI
#include <mpi.h>
#endif

#define RZ_STRING_SIZE 74 /* STRING_SIZE of fd.h:25 */
/* a snapshot name: SNAP_FILE, "_shot_", the shot number and ".tt" (the
   reference formats it into STRING_SIZE bytes, which a long SNAP_FILE overruns) */
#define RZ_SNAP_NAME (RZ_STRING_SIZE + 24)

/* the reference's globals (globvar.h) and helpers (util.c, writemod.c, write_picks.c) */
extern float DH, TIME, TTNORM, EPS_ADJ;
extern int NX, NY, SNAP, SEISMO, NSHOT1, NSHOT2;
extern char SNAP_FILE[RZ_STRING_SIZE], DATA_DIR[RZ_STRING_SIZE];
extern void err(char err_text[]);
extern void writemod(char modfile[RZ_STRING_SIZE], float **array, int format);
extern void write_picks(float *Tmod, int ntr, int ishot);
extern void precond(float **grad, int nsrc, float **srcpos, int **recpos, int ntr, int iter);
#ifdef RZ_COMPAT_MPI
extern void sum_grad_MPI(float **grad);
extern void cp_grad_frame(float **A);
#endif

static rz_context *g_ctx = NULL;
static int g_device = -1, g_mode = -1;
/* the receiver geometry the engine holds (see receivers()) */
static int g_ntr = -1;
static int *g_recx = NULL, *g_recz = NULL;

int rz_compat_configure(int device, int mode) {
    g_device = device;
    g_mode = mode;
    if (g_ctx) {
        rz_destroy(g_ctx);
        g_ctx = NULL;
        g_ntr = -1;
    }
    return RZ_OK;
}

static void fail(const char *what, int st) {
    static char msg[512];
    snprintf(msg, sizeof msg, "GB300 engine: %s failed: %s (%s)", what, rz_strerror(st),
             g_ctx ? rz_last_error(g_ctx) : "no context");
    err(msg);
}

/* context + the globals of this call (set_grid keeps buffers when the shape is unchanged) */
static void engine(void) {
    if (!g_ctx) {
        int dev = g_device >= 0 ? g_device : (getenv("RAJZEL_GPU") ? atoi(getenv("RAJZEL_GPU")) : 0);
        int mode = g_mode >= 0 ? g_mode
                               : (getenv("RAJZEL_MODE") && !strcmp(getenv("RAJZEL_MODE"), "fast") ? RZ_MODE_FAST
                                                                                                  : RZ_MODE_REFERENCE);
        int st = rz_create(&g_ctx, dev);
        if (st) fail("rz_create", st);
        if ((st = rz_set_mode(g_ctx, mode))) fail("rz_set_mode", st);
    }
    rz_grid g;
    g.nx = NX;
    g.ny = NY;
    g.dh = DH;
    g.time = TIME;
    g.ttnorm = TTNORM;
    g.eps_adj = EPS_ADJ;
    g.max_passes = 0;
    static int last_nx = -1, last_ny = -1;
    int st = rz_set_grid(g_ctx, &g);
    if (st) fail("rz_set_grid", st);
    if (NX != last_nx || NY != last_ny) g_ntr = -1; /* a new shape drops the engine's receivers */
    last_nx = NX, last_ny = NY;
}

/* The receiver geometry is uploaded only when it differs from the last one
   the engine received: FATT calls grad_obj() for every line-search trial with
   the same recpos, and only the model changes between them. */
static void receivers(int **recpos, int ntr) {
    const size_t bytes = sizeof(int) * (size_t)(ntr > 0 ? ntr : 1);
    if (ntr == g_ntr && (ntr == 0 || (!memcmp(g_recx, &recpos[1][1], sizeof(int) * ntr) &&
                                      !memcmp(g_recz, &recpos[2][1], sizeof(int) * ntr))))
        return;
    int st = rz_set_receivers(g_ctx, ntr, ntr > 0 ? &recpos[1][1] : NULL, ntr > 0 ? &recpos[2][1] : NULL);
    if (st) fail("rz_set_receivers", st);
    free(g_recx), free(g_recz);
    g_recx = (int *)malloc(bytes), g_recz = (int *)malloc(bytes);
    if (!g_recx || !g_recz) err("rz_compat: host allocation failed");
    if (ntr > 0) memcpy(g_recx, &recpos[1][1], sizeof(int) * ntr), memcpy(g_recz, &recpos[2][1], sizeof(int) * ntr);
    g_ntr = ntr;
}

static void model_and_receivers(float **S, int **recpos, int ntr) {
    int st = rz_set_slowness(g_ctx, &S[1][1], 0);
    if (st) fail("rz_set_slowness", st);
    receivers(recpos, ntr);
}

/* eikonal.c:10-76 */
void eikonal(float **S, float **TT, float *Tmod, float **srcpos, int ishot, int nshots, int **recpos, int ntr) {
    (void)nshots;
    engine();
    model_and_receivers(S, recpos, ntr);
    int st = rz_eikonal(g_ctx, srcpos[1][ishot], srcpos[2][ishot], &TT[1][1], ntr > 0 ? &Tmod[1] : NULL, NULL, 0);
    if (st) fail("rz_eikonal", st);
    if (SNAP == 1) {
        char filename[RZ_SNAP_NAME];
        snprintf(filename, sizeof filename, "%s_shot_%d.tt", SNAP_FILE, ishot);
        writemod(filename, TT, 3);
    }
    if (SEISMO == 1) write_picks(Tmod, ntr, ishot);
}

/* eikonal_adj.c:10-59; recflag is rebuilt from recpos by the engine */
void eikonal_adj(float **TT, float *Tres, float **lam, int **recpos, int ntr, int ishot, int **recflag) {
    (void)ishot;
    (void)recflag;
    engine();
    receivers(recpos, ntr);
    int st = rz_eikonal_adj(g_ctx, &TT[1][1], ntr > 0 ? &Tres[1] : NULL, &lam[1][1], NULL, 0);
    if (st) fail("rz_eikonal_adj", st);
}

/* forward.c:10-26: this rank's shots NSHOT1..NSHOT2-1 in batched engine calls
   (chunks of kForwardChunk shots bound the host copy of their traveltime
   fields, which only the snapshot files need), then per shot in shot order
   what eikonal() does after its solve: the snapshot file (SNAP == 1) and the
   picks file (SEISMO == 1).  TT and Tmod are left holding the last shot's
   fields, as the reference's loop leaves them. */
enum { kForwardChunk = 64 };
void forward(float **S, float **TT, float *Tmod, float **srcpos, int nshots, int **recpos, int ntr) {
    (void)nshots;
    const int n = NSHOT2 - NSHOT1;
    if (n <= 0) return;
    engine();
    model_and_receivers(S, recpos, ntr);
    const size_t cells = (size_t)NX * NY, nt = (size_t)(ntr > 0 ? ntr : 1);
    const int chunk = n < kForwardChunk ? n : kForwardChunk;
    float *sx = (float *)malloc(sizeof(float) * chunk), *sz = (float *)malloc(sizeof(float) * chunk);
    float *tm = (float *)malloc(sizeof(float) * nt * chunk);
    float *tt = SNAP == 1 ? (float *)malloc(sizeof(float) * cells * chunk) : NULL;
    if (!sx || !sz || !tm || (SNAP == 1 && !tt)) err("forward: host allocation failed");
    int m = 0;
    for (int first = NSHOT1; first < NSHOT2; first += chunk) {
        m = NSHOT2 - first < chunk ? NSHOT2 - first : chunk;
        for (int s = 0; s < m; s++) sx[s] = srcpos[1][first + s], sz[s] = srcpos[2][first + s];
        int st = rz_forward(g_ctx, m, sx, sz, tt, ntr > 0 ? tm : NULL, NULL, 0);
        if (st) fail("rz_forward", st);
        for (int s = 0; s < m; s++) {
            const int ishot = first + s;
            for (int i = 0; i < ntr; i++) Tmod[i + 1] = tm[(size_t)s * ntr + i];
            if (SNAP == 1) {
                char filename[RZ_SNAP_NAME];
                memcpy(&TT[1][1], tt + (size_t)s * cells, sizeof(float) * cells);
                snprintf(filename, sizeof filename, "%s_shot_%d.tt", SNAP_FILE, ishot);
                writemod(filename, TT, 3);
            }
            if (SEISMO == 1) write_picks(Tmod, ntr, ishot);
        }
    }
    /* the last shot's traveltimes, where the reference's loop leaves them */
    if (SNAP != 1) {
        int st = rz_shot_fields(g_ctx, m - 1, &TT[1][1], NULL, NULL, 0);
        if (st) fail("rz_shot_fields", st);
    }
    free(sx), free(sz), free(tm), free(tt);
}

/* picks of one shot from DATA_DIR_<ishot>.dat, one value per line (calc_FA_res.c:28-37) */
static void read_picks(int ishot, int ntr, float *dst) {
    char fn[RZ_STRING_SIZE + 16];
    snprintf(fn, sizeof fn, "%s_%i.dat", DATA_DIR, ishot);
    FILE *fp = fopen(fn, "r");
    if (!fp) err(" picks_?.dat could not be opened !");
    for (int i = 0; i < ntr; i++)
        if (fscanf(fp, "%e", &dst[i]) != 1) err(" picks_?.dat is too short !");
    fclose(fp);
}

/* grad_obj.c:10-81: every local shot in one batched GPU call */
double grad_obj(float **grad, float **S, float **TT, float **lam, float *Tmod, float *Tobs, float *Tres,
                float **srcpos, int nshots, int **recpos, int ntr, int iter) {
    SEISMO = 0; /* grad_obj.c:24 */
    engine();
    model_and_receivers(S, recpos, ntr);
    const int n = NSHOT2 - NSHOT1;
    double L2 = 0.0;
    if (n > 0) {
        float *sx = (float *)malloc(sizeof(float) * n), *sz = (float *)malloc(sizeof(float) * n);
        float *obs = (float *)malloc(sizeof(float) * (size_t)n * (ntr > 0 ? ntr : 1));
        if (!sx || !sz || !obs) err("grad_obj: host allocation failed");
        for (int s = 0; s < n; s++) {
            sx[s] = srcpos[1][NSHOT1 + s];
            sz[s] = srcpos[2][NSHOT1 + s];
            read_picks(NSHOT1 + s, ntr, obs + (size_t)s * ntr);
        }
        double half = 0.0;
        int st = rz_grad_obj(g_ctx, n, sx, sz, obs, &grad[1][1], &half, 0);
        if (st) fail("rz_grad_obj", st);
        L2 = 2.0 * half; /* this rank's sum of shot misfits */
        /* leave the last shot's fields where the reference leaves them */
        st = rz_shot_fields(g_ctx, n - 1, &TT[1][1], &lam[1][1], ntr > 0 ? &Tres[1] : NULL, 0);
        if (st) fail("rz_shot_fields", st);
        for (int i = 0; i < ntr; i++) {
            Tmod[i + 1] = TT[recpos[2][i + 1]][recpos[1][i + 1]];
            Tobs[i + 1] = obs[(size_t)(n - 1) * ntr + i];
        }
        free(sx);
        free(sz);
        free(obs);
    } else {
        memset(&grad[1][1], 0, sizeof(float) * (size_t)NX * NY);
    }
#ifdef RZ_COMPAT_MPI
    double L2sum = 0.0;
    MPI_Barrier(MPI_COMM_WORLD);
    MPI_Allreduce(&L2, &L2sum, 1, MPI_DOUBLE, MPI_SUM, MPI_COMM_WORLD);
    L2 = L2sum;
    /* sum_grad_MPI reduces NX*NY floats from index 0 of a vector filled from
       index 1, so the corner cell grad[NY][NX] comes back uninitialised
       (sum_grad_MPI.c:24-36); the reference's frame copy after it
       (grad_obj.c:68-70) overwrites that corner, and so does this one */
    sum_grad_MPI(grad);
    cp_grad_frame(grad);
#endif
    /* single rank: the engine already applied cp_grad_frame (grad_obj.c:70) */
    precond(grad, nshots, srcpos, recpos, ntr, iter); /* grad_obj.c:73 */
    return 0.5 * L2;
}
