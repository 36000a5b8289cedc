/*
 * Test harness for the reference-signature shim (rz_compat.c): plays the
 * part of the RAJZEL host program -- it owns the globals, provides err(),
 * writemod(), write_picks(), precond(), builds 1-based NR matrices -- and
 * exposes flat-array wrappers that tests call through ctypes.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "rajzel_compat.h"

#ifdef RZ_COMPAT_MPI
#include <mpi.h>
#endif

float DH, TIME, TTNORM, EPS_ADJ;
int NX, NY, SNAP = 0, SEISMO = 0, NSHOT1 = 1, NSHOT2 = 1;
char SNAP_FILE[74], DATA_DIR[74];
static int g_err = 0;

void err(char err_text[]) {
    fprintf(stderr, "harness err(): %s\n", err_text);
    g_err = 1;
    exit(3);
}
void writemod(char modfile[74], float **array, int format) { (void)modfile, (void)array, (void)format; }

/* picks written through write_picks(), kept per shot for the tests */
#define H_MAX_SHOTS 32
#define H_MAX_TR 4096
static float g_picks[H_MAX_SHOTS + 1][H_MAX_TR];
static int g_picks_calls = 0;
void write_picks(float *Tmod, int ntr, int ishot) {
    g_picks_calls++;
    if (ishot < 0 || ishot > H_MAX_SHOTS || ntr > H_MAX_TR) return;
    for (int i = 0; i < ntr; i++) g_picks[ishot][i] = Tmod[i + 1];
}
int h_picks(int ishot, int ntr, float *out) {
    for (int i = 0; i < ntr; i++) out[i] = g_picks[ishot][i];
    return g_picks_calls;
}

#ifdef RZ_COMPAT_MPI
/* the reference's sum_grad_MPI on one rank (sum_grad_MPI.c:19-47): the
   reduction covers NX*NY floats from index 0 of a vector filled from index
   1, so the corner grad[NY][NX] receives an element nobody wrote -- made a
   NaN here so that a shim which does not repeat the frame copy fails */
void sum_grad_MPI(float **grad) {
    float *v = (float *)malloc(((size_t)NX + 1) * (NY + 1) * sizeof(float));
    float *r = (float *)malloc(((size_t)NX + 1) * (NY + 1) * sizeof(float));
    int h = 1;
    for (int i = 1; i <= NX; i++)
        for (int j = 1; j <= NY; j++) v[h++] = grad[j][i];
    for (size_t k = 0; k < ((size_t)NX + 1) * (NY + 1); k++) r[k] = NAN;
    MPI_Allreduce(v, r, NX * NY, MPI_FLOAT, MPI_SUM, MPI_COMM_WORLD);
    h = 1;
    for (int i = 1; i <= NX; i++)
        for (int j = 1; j <= NY; j++) grad[j][i] = r[h++];
    free(v), free(r);
}
/* cp_grad_frame.c:18-49: rows 2 -> 1 -> 0 at the top, NY-2 -> NY-1 -> NY at
   the bottom, then the same for the columns */
void cp_grad_frame(float **A) {
    for (int i = 1; i <= NX; i++) A[2][i] = A[3][i], A[1][i] = A[2][i];
    for (int i = 1; i <= NX; i++) A[NY - 1][i] = A[NY - 2][i], A[NY][i] = A[NY - 1][i];
    for (int j = 1; j <= NY; j++) A[j][2] = A[j][3], A[j][1] = A[j][2];
    for (int j = 1; j <= NY; j++) A[j][NX - 1] = A[j][NX - 2], A[j][NX] = A[j][NX - 1];
}
#endif
void precond(float **grad, int nsrc, float **srcpos, int **recpos, int ntr, int iter) {
    (void)grad, (void)nsrc, (void)srcpos, (void)recpos, (void)ntr, (void)iter;
}

static float **fmat(int nr, int nc) { /* [1..nr][1..nc], contiguous like util.c:177-203 */
    float **m = (float **)malloc((nr + 1) * sizeof(float *));
    m[1] = (float *)calloc((size_t)nr * nc + 1, sizeof(float));
    m[1] -= 1;
    for (int i = 2; i <= nr; i++) m[i] = m[i - 1] + nc;
    return m;
}
static int **imat(int nr, int nc) {
    int **m = (int **)malloc((nr + 1) * sizeof(int *));
    m[1] = (int *)calloc((size_t)nr * nc + 1, sizeof(int));
    m[1] -= 1;
    for (int i = 2; i <= nr; i++) m[i] = m[i - 1] + nc;
    return m;
}
static void ffree(float **m) { free(m[1] + 1), free(m); }
static void ifree(int **m) { free(m[1] + 1), free(m); }

void h_set(int nx, int ny, float dh, float time, float ttnorm, float eps_adj) {
    NX = nx, NY = ny, DH = dh, TIME = time, TTNORM = ttnorm, EPS_ADJ = eps_adj;
}

static int **recs(int ntr, const int *rx, const int *rz) {
    int **r = imat(3, ntr > 0 ? ntr : 1);
    for (int i = 0; i < ntr; i++) r[1][i + 1] = rx[i], r[2][i + 1] = rz[i];
    return r;
}

void h_eikonal(const float *S, float sx, float sz, int ntr, const int *rx, const int *rz, float *TT, float *Tmod) {
    float **s = fmat(NY, NX), **tt = fmat(NY, NX), **src = fmat(8, 1);
    float *tm = (float *)calloc(ntr + 2, sizeof(float));
    int **r = recs(ntr, rx, rz);
    memcpy(&s[1][1], S, sizeof(float) * NX * NY);
    src[1][1] = sx, src[2][1] = sz;
    eikonal(s, tt, tm, src, 1, 1, r, ntr);
    memcpy(TT, &tt[1][1], sizeof(float) * NX * NY);
    for (int i = 0; i < ntr; i++) Tmod[i] = tm[i + 1];
    ffree(s), ffree(tt), ffree(src), ifree(r), free(tm);
}

void h_eikonal_adj(const float *TT, const float *Tres, int ntr, const int *rx, const int *rz, float *lam) {
    float **tt = fmat(NY, NX), **l = fmat(NY, NX);
    float *tr = (float *)calloc(ntr + 2, sizeof(float));
    int **r = recs(ntr, rx, rz), **flag = imat(NY, NX);
    memcpy(&tt[1][1], TT, sizeof(float) * NX * NY);
    for (int i = 0; i < ntr; i++) tr[i + 1] = Tres[i];
    eikonal_adj(tt, tr, l, r, ntr, 1, flag);
    memcpy(lam, &l[1][1], sizeof(float) * NX * NY);
    ffree(tt), ffree(l), ifree(r), ifree(flag), free(tr);
}

/* grad_obj over shots 1..ns with picks written to DATA_DIR_<s>.dat */
double h_grad_obj(const char *datadir, const float *S, int ns, const float *sx, const float *sz, int ntr,
                  const int *rx, const int *rz, const float *Tobs, float *grad) {
    snprintf(DATA_DIR, sizeof DATA_DIR, "%s", datadir);
    for (int s = 0; s < ns; s++) {
        char fn[128];
        snprintf(fn, sizeof fn, "%s_%i.dat", DATA_DIR, s + 1);
        FILE *fp = fopen(fn, "w");
        for (int i = 0; i < ntr; i++) fprintf(fp, "%.9e\n", Tobs[(size_t)s * ntr + i]);
        fclose(fp);
    }
    float **s = fmat(NY, NX), **tt = fmat(NY, NX), **l = fmat(NY, NX), **g = fmat(NY, NX), **src = fmat(8, ns);
    float *tm = (float *)calloc(ntr + 2, sizeof(float)), *to = (float *)calloc(ntr + 2, sizeof(float)),
          *tr = (float *)calloc(ntr + 2, sizeof(float));
    int **r = recs(ntr, rx, rz);
    memcpy(&s[1][1], S, sizeof(float) * NX * NY);
    for (int i = 0; i < ns; i++) src[1][i + 1] = sx[i], src[2][i + 1] = sz[i];
    NSHOT1 = 1, NSHOT2 = ns + 1;
    double L2 = grad_obj(g, s, tt, l, tm, to, tr, src, ns, r, ntr, 1);
    memcpy(grad, &g[1][1], sizeof(float) * NX * NY);
    ffree(s), ffree(tt), ffree(l), ffree(g), ffree(src), ifree(r), free(tm), free(to), free(tr);
    return L2;
}

/* forward() over shots 1..ns with SEISMO = 1: TT / Tmod receive what the
   reference leaves there (the last shot's), the picks go to write_picks() */
void h_forward(const float *S, int ns, const float *sx, const float *sz, int ntr, const int *rx, const int *rz,
               float *TT, float *Tmod) {
    float **s = fmat(NY, NX), **tt = fmat(NY, NX), **src = fmat(8, ns);
    float *tm = (float *)calloc(ntr + 2, sizeof(float));
    int **r = recs(ntr, rx, rz);
    memcpy(&s[1][1], S, sizeof(float) * NX * NY);
    for (int i = 0; i < ns; i++) src[1][i + 1] = sx[i], src[2][i + 1] = sz[i];
    NSHOT1 = 1, NSHOT2 = ns + 1;
    SEISMO = 1;
    g_picks_calls = 0;
    forward(s, tt, tm, src, ns, r, ntr);
    SEISMO = 0;
    memcpy(TT, &tt[1][1], sizeof(float) * NX * NY);
    for (int i = 0; i < ntr; i++) Tmod[i] = tm[i + 1];
    ffree(s), ffree(tt), ffree(src), ifree(r), free(tm);
}
