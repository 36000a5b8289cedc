/*
 * rz_io.c -- RAJZEL's parameter, workflow, source, receiver, model and pick
 * files (include/rajzel_io.h).
 *
 * The .inp file is positional: a parameter line is any line that does not
 * start with '#'; the n-th such line holds parameter n as "label = value"
 * (read_par.c:72-270).  The reader consumes the first character of each
 * counted line before scanning "label =value", exactly as the reference
 * does, so files the reference accepts parse to the same values.
 */
#include "rajzel_io.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define RZ_OK 0
#define RZ_EINVAL 1

static __thread char g_msg[512];

const char *rz_io_error(void) { return g_msg; }

static int io_fail(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_msg, sizeof g_msg, fmt, ap);
    va_end(ap);
    return RZ_EINVAL;
}

/* iround of fd.h:18 */
static int iround(float x) { return (int)floor(x + 0.5); }

/* ------------------------------------------------------------------------ */
/* .inp parameter file                                                      */
/* ------------------------------------------------------------------------ */
enum kind { K_INT, K_FLOAT, K_STR, K_F2, K_I4, K_F3 };

struct field {
    enum kind k;
    void *p[4];
};

static int scan_field(FILE *fp, const struct field *f) {
    char label[256];
    switch (f->k) {
        case K_INT: return fscanf(fp, "%255s =%i", label, (int *)f->p[0]) == 2;
        case K_FLOAT: return fscanf(fp, "%255s =%f", label, (float *)f->p[0]) == 2;
        case K_STR: return fscanf(fp, "%255s =%255s", label, (char *)f->p[0]) == 2;
        case K_F2: return fscanf(fp, "%255s =%f ,%f", label, (float *)f->p[0], (float *)f->p[1]) == 3;
        case K_I4:
            return fscanf(fp, "%255s =%i, %i, %i, %i", label, (int *)f->p[0], (int *)f->p[1], (int *)f->p[2],
                          (int *)f->p[3]) == 5;
        case K_F3:
            return fscanf(fp, "%255s =%f, %f, %f", label, (float *)f->p[0], (float *)f->p[1], (float *)f->p[2]) == 4;
    }
    return 0;
}

int rz_read_par(const char *path, rz_par *P) {
    if (!path || !P) return io_fail("rz_read_par: NULL argument");
    memset(P, 0, sizeof *P);
    /* file order of read_par.c:72-270; the two-value lines (REFREC, C1/C2) accept
       "a , b" and "a, b" alike, as the reference's formats do */
    const struct field f[] = {
        {K_INT, {&P->INVMAT}}, {K_INT, {&P->NX}}, {K_INT, {&P->NY}}, {K_FLOAT, {&P->DH}}, {K_FLOAT, {&P->TIME}},
        {K_STR, {P->SOURCE_FILE}}, {K_INT, {&P->READMOD}}, {K_STR, {P->MFILE}}, {K_INT, {&P->SNAP}},
        {K_INT, {&P->IDX}}, {K_INT, {&P->IDY}}, {K_INT, {&P->SNAP_FORMAT}}, {K_STR, {P->SNAP_FILE}},
        {K_INT, {&P->SEISMO}}, {K_STR, {P->REC_FILE}}, {K_F2, {&P->REFREC[0], &P->REFREC[1]}},
        {K_INT, {&P->N_STREAMER}}, {K_FLOAT, {&P->REC_INCR_X}}, {K_FLOAT, {&P->REC_INCR_Y}},
        {K_STR, {P->PICKS_FILE}}, {K_FLOAT, {&P->TTNORM}}, {K_STR, {P->LOG_FILE}}, {K_INT, {&P->LOG}},
        {K_INT, {&P->ITERMAX}}, {K_FLOAT, {&P->EPS_ADJ}}, {K_STR, {P->JACOBIAN}}, {K_STR, {P->DATA_DIR}},
        {K_INT, {&P->TAPER}}, {K_INT, {&P->TAPERLENGTH}}, {K_INT, {&P->INVTYPE}},
        {K_I4, {&P->GRADT1, &P->GRADT2, &P->GRADT3, &P->GRADT4}}, {K_INT, {&P->SWS_TAPER_GRAD_VERT}},
        {K_INT, {&P->SWS_TAPER_GRAD_HOR}}, {K_FLOAT, {&P->EXP_TAPER_GRAD_HOR}},
        {K_INT, {&P->SWS_TAPER_GRAD_SOURCES}}, {K_INT, {&P->SWS_TAPER_CIRCULAR_PER_SHOT}},
        {K_INT, {&P->SRTSHAPE}}, {K_FLOAT, {&P->SRTRADIUS}}, {K_INT, {&P->FILTSIZE}},
        {K_INT, {&P->SWS_TAPER_FILE}}, {K_STR, {P->INV_MODELFILE}}, {K_INT, {&P->nfstart}}, {K_INT, {&P->nf}},
        {K_INT, {&P->nfstart_jac}}, {K_INT, {&P->nf_jac}}, {K_FLOAT, {&P->VPUPPERLIM}},
        {K_FLOAT, {&P->VPLOWERLIM}}, {K_INT, {&P->GRAD_METHOD}}, {K_INT, {&P->NLBFGS}},
        {K_INT, {&P->MODEL_FILTER}}, {K_INT, {&P->FILT_SIZE}}, {K_INT, {&P->LINESEARCH}},
        {K_FLOAT, {&P->EPS_SCALE}}, {K_F2, {&P->C1, &P->C2}}, {K_INT, {&P->STEPMAX}}, {K_FLOAT, {&P->SCALEFAC}},
        {K_STR, {P->MISFIT_LOG_FILE}}, {K_INT, {&P->MIN_ITER}}, {K_INT, {&P->GRAD_FILTER}},
        {K_INT, {&P->FILT_SIZE_GRAD}}, {K_F3, {&P->VP0_1, &P->VP0_2, &P->DVP0}},
        {K_F3, {&P->GRAD0_1, &P->GRAD0_2, &P->DGRAD0}}, {K_STR, {P->GRIDSEARCH_FILE}},
    };
    const int nf = (int)(sizeof f / sizeof f[0]);
    FILE *fp = fopen(path, "r");
    if (!fp) return io_fail("cannot open parameter file %s", path);
    int c, line = 0;
    while ((c = getc(fp)) != EOF) {
        if (c != '\n') continue;
        c = getc(fp); /* first character of the next line (consumed, as read_par.c does) */
        if (c == EOF) break;
        if (c == '#') continue;
        if (line < nf && !scan_field(fp, &f[line])) {
            fclose(fp);
            return io_fail("%s: parameter line %d could not be read", path, line + 1);
        }
        ++line;
    }
    fclose(fp);
    P->nlines = line;
    if (line < 5) return io_fail("%s: only %d parameter lines", path, line);
    return RZ_OK;
}

/* ------------------------------------------------------------------------ */
/* workflow file                                                            */
/* ------------------------------------------------------------------------ */
int rz_read_workflow(const char *path, int stage, float *pro, int *spatfilter, float *wd_damp, float *wd_damp1,
                     int *filt_size_grad, int *filt_size_grad1, int *nstages) {
    FILE *fp = fopen(path, "r");
    if (!fp) return io_fail("cannot open workflow file %s", path);
    int c, lines = 0;
    while ((c = getc(fp)) != EOF)
        if (c == '\n') ++lines;
    if (nstages) *nstages = lines - 1; /* fatt.c:55-59 */
    rewind(fp);
    char h[6][128];
    if (fscanf(fp, "%127s%127s%127s%127s%127s%127s", h[0], h[1], h[2], h[3], h[4], h[5]) != 6) {
        fclose(fp);
        return io_fail("%s: no header line", path);
    }
    float a = 0, b = 0, d = 0;
    int e = 0, g = 0, k = 0;
    for (int i = 1; i <= stage; ++i)
        if (fscanf(fp, "%f%i%f%f%i%i", &a, &e, &b, &d, &g, &k) != 6) {
            fclose(fp);
            return io_fail("%s: workflow row %d could not be read", path, i);
        }
    fclose(fp);
    if (pro) *pro = a;
    if (spatfilter) *spatfilter = e;
    if (wd_damp) *wd_damp = b;
    if (wd_damp1) *wd_damp1 = d;
    if (filt_size_grad) *filt_size_grad = g;
    if (filt_size_grad1) *filt_size_grad1 = k;
    return RZ_OK;
}

/* ------------------------------------------------------------------------ */
/* sources and receivers                                                    */
/* ------------------------------------------------------------------------ */
int rz_read_sources(const char *path, int *nshots, float *srcx, float *srcz, int cap) {
    if (!nshots) return io_fail("rz_read_sources: NULL argument");
    FILE *fp = fopen(path, "r");
    if (!fp) return io_fail("Source file %s could not be opened", path);
    int n = 0;
    if (fscanf(fp, "%d", &n) != 1 || n < 0) {
        fclose(fp);
        return io_fail("%s: first line must hold the number of sources", path);
    }
    *nshots = n;
    if (cap == 0) {
        fclose(fp);
        return RZ_OK;
    }
    if (!srcx || !srcz || cap < n) {
        fclose(fp);
        return io_fail("%s: room for %d of %d sources", path, cap, n);
    }
    rewind(fp);
    char line[1024];
    if (!fgets(line, sizeof line, fp)) n = -1;
    for (int l = 0; l < n; ++l) {
        float v[8];
        if (!fgets(line, sizeof line, fp)) {
            fclose(fp);
            return io_fail("%s: source %d missing", path, l + 1);
        }
        const int got = sscanf(line, "%f%f%f%f%f%f%f%f", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &v[7]);
        if (got < 6) {
            fclose(fp);
            return io_fail("%s: source %d has %d of at least 6 values (Missing parameter in SOURCE_FILE)", path, l + 1,
                           got < 0 ? 0 : got);
        }
        srcx[l] = v[0]; /* sources.c:63-64: x is column 1, depth column 3 */
        srcz[l] = v[2];
    }
    fclose(fp);
    return RZ_OK;
}

int rz_read_receivers(const char *path, float dh, const float refrec[2], int *ntr, int *recx, int *recz, int cap) {
    if (!ntr || !(dh > 0.f)) return io_fail("rz_read_receivers: bad arguments");
    FILE *fp = fopen(path, "r");
    if (!fp) return io_fail("Receiver file %s could not be opened", path);
    int c, lines = 0;
    while ((c = getc(fp)) != EOF)
        if (c == '\n') ++lines;
    rewind(fp);
    const float rx = refrec ? refrec[0] : 0.f, rz = refrec ? refrec[1] : 0.f;
    int kept = 0;
    for (int i = 0; i < lines; ++i) {
        float x, z;
        if (fscanf(fp, "%f%f\n", &x, &z) != 2) {
            fclose(fp);
            return io_fail("%s: receiver line %d could not be read", path, i + 1);
        }
        const int ix = iround((x + rx) / dh), iz = iround((z + rz) / dh);
        if (ix <= 0) continue; /* receiver.c:66-72 keeps x index > 0 only */
        if (cap > 0) {
            if (kept >= cap) {
                fclose(fp);
                return io_fail("%s: more than %d receivers", path, cap);
            }
            recx[kept] = ix;
            recz[kept] = iz;
        }
        ++kept;
    }
    fclose(fp);
    *ntr = kept;
    return RZ_OK;
}

/* ------------------------------------------------------------------------ */
/* models and picks                                                         */
/* ------------------------------------------------------------------------ */
int rz_read_model(const char *path, int nx, int ny, float *vp) {
    FILE *fp = fopen(path, "rb");
    if (!fp) return io_fail("Could not open model file %s", path);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            if (fread(&vp[(size_t)j * nx + i], sizeof(float), 1, fp) != 1) {
                fclose(fp);
                return io_fail("%s: shorter than %d x %d floats", path, nx, ny);
            }
    fclose(fp);
    return RZ_OK;
}

int rz_write_model(const char *path, int nx, int ny, const float *vp) {
    FILE *fp = fopen(path, "wb");
    if (!fp) return io_fail("Could not create model file %s", path);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            if (fwrite(&vp[(size_t)j * nx + i], sizeof(float), 1, fp) != 1) {
                fclose(fp);
                return io_fail("%s: write failed", path);
            }
    fclose(fp);
    return RZ_OK;
}

int rz_read_picks(const char *prefix, int shot, int ntr, float *t) {
    char fn[RZ_PATH + 32];
    snprintf(fn, sizeof fn, "%s_%i.dat", prefix, shot);
    FILE *fp = fopen(fn, "r");
    if (!fp) return io_fail("pick file %s could not be opened", fn);
    for (int i = 0; i < ntr; ++i)
        if (fscanf(fp, "%e", &t[i]) != 1) {
            fclose(fp);
            return io_fail("%s: %d of %d picks", fn, i, ntr);
        }
    fclose(fp);
    return RZ_OK;
}

int rz_write_picks(const char *prefix, int shot, int ntr, const float *t) {
    char fn[RZ_PATH + 32];
    snprintf(fn, sizeof fn, "%s_%i.dat", prefix, shot);
    FILE *fp = fopen(fn, "w");
    if (!fp) return io_fail("pick file %s could not be created", fn);
    for (int i = 0; i < ntr; ++i) fprintf(fp, "%e \n", t[i]);
    fclose(fp);
    return RZ_OK;
}
