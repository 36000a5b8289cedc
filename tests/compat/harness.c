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
void write_picks(float *Tmod, int ntr, int ishot) { (void)Tmod, (void)ntr, (void)ishot; }
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
