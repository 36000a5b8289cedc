/*
 * Test-only driver around the reference's own hot-path C sources.
 *
 * oracle/Makefile compiles this file together with the UNMODIFIED reference
 * sources (eikonal.c, sweep.c, eikonal_adj.c, sweep_adj.c, init_travel_adj.c,
 * init_recflag.c, norm1.c, store_mat.c, zero_travel.c, calc_FA.c,
 * calc_FA_res.c, ass_grad.c, cp_grad_frame.c, grad_obj.c, sum_grad_MPI.c,
 * precond.c, ...) into oracle/_ref/libref.so.  The reference's globals are
 * defined by including its globvar.h here exactly once, as rajzel.c does.
 *
 * The functions below only marshal flat row-major arrays ([NY][NX], x
 * fastest, cell (h,k) at k*NX+h, 0-based) to and from the reference's
 * 1-based NR matrices and call the reference entry points.  Sweep and
 * norm1 calls are counted through the linker's --wrap so tests can compare
 * pass counts, and the misfits grad_obj() returns are recorded in call order
 * (a FATT stage's trajectory).  This library is the oracle's pin, never the
 * product.
 */
#include "fd.h"
#include "globvar.h"

#include <unistd.h>
#include <sys/stat.h>

/* --- call counters via -Wl,--wrap ----------------------------------------- */
void __real_sweep(float **S, float **TT, int nxsrc, int nysrc, int nx1, int nx2, int ndx, int ny1, int ny2, int ndy);
void __real_sweep_adj(float **lam, float **TT, float *Tres, int **recpos, int ntr, int nx1, int nx2, int ndx, int ny1,
                      int ny2, int ndy, int **recflag);
float __real_norm1(float **TT, float **TTold);

static long g_sweeps = 0, g_sweeps_adj = 0, g_norm1 = 0;
static float g_last_norm1 = 0.0f;

/* every misfit grad_obj() returns, in call order (FATT trajectories) */
double __real_grad_obj(float **grad, float **S, float **TT, float **lam, float *Tmod, float *Tobs, float *Tres,
                       float **srcpos, int nshots, int **recpos, int ntr, int iter);
#define REF_MAX_EVALS 4096
static double g_evals[REF_MAX_EVALS];
static int g_nevals = 0;
double __wrap_grad_obj(float **grad, float **S, float **TT, float **lam, float *Tmod, float *Tobs, float *Tres,
                       float **srcpos, int nshots, int **recpos, int ntr, int iter) {
    double L2 = __real_grad_obj(grad, S, TT, lam, Tmod, Tobs, Tres, srcpos, nshots, recpos, ntr, iter);
    if (g_nevals < REF_MAX_EVALS) g_evals[g_nevals] = L2;
    g_nevals++;
    return L2;
}
int ref_evals(double *out, int cap) {
    for (int i = 0; i < g_nevals && i < cap; i++) out[i] = g_evals[i];
    return g_nevals;
}

void __wrap_sweep(float **S, float **TT, int nxsrc, int nysrc, int nx1, int nx2, int ndx, int ny1, int ny2, int ndy) {
    g_sweeps++;
    __real_sweep(S, TT, nxsrc, nysrc, nx1, nx2, ndx, ny1, ny2, ndy);
}
void __wrap_sweep_adj(float **lam, float **TT, float *Tres, int **recpos, int ntr, int nx1, int nx2, int ndx, int ny1,
                      int ny2, int ndy, int **recflag) {
    g_sweeps_adj++;
    __real_sweep_adj(lam, TT, Tres, recpos, ntr, nx1, nx2, ndx, ny1, ny2, ndy, recflag);
}
float __wrap_norm1(float **TT, float **TTold) {
    g_norm1++;
    g_last_norm1 = __real_norm1(TT, TTold);
    return g_last_norm1;
}

/* wavenumber.c needs FFTW, which is absent; SPATFILTER==1 is never used by
   the oracle, so the symbol only has to exist for precond.c to link. */
void wavenumber(float **grad) {
    (void)grad;
    err("wavenumber filtering (FFTW) is not built into the oracle");
}

long ref_counter(int which) {
    switch (which) {
        case 0: return g_sweeps;
        case 1: return g_sweeps_adj;
        case 2: return g_norm1;
        default: return 0;
    }
}
float ref_last_norm1(void) { return g_last_norm1; }
void ref_reset_counters(void) { g_sweeps = g_sweeps_adj = g_norm1 = 0; }

/* --- parameters ----------------------------------------------------------- */
void ref_set_params(int nx, int ny, float dh, float time, float ttnorm, float eps_adj) {
    NX = nx; NY = ny; DH = dh; TIME = time; TTNORM = ttnorm; EPS_ADJ = eps_adj;
    NP = 1; MYID = 0; INFO = 0; SNAP = 0; SEISMO = 0; LOG = 0;
    IDX = 1; IDY = 1;
    SPATFILTER = 0; GRAD_FILTER = 0;
    SWS_TAPER_GRAD_VERT = 0; SWS_TAPER_GRAD_HOR = 0; SWS_TAPER_GRAD_SOURCES = 0;
    SWS_TAPER_FILE = 0; SWS_TAPER_CIRCULAR_PER_SHOT = 0;
    FP = stdout;
}

static void flat_to_nr(const float *src, float **dst) {
    for (int k = 1; k <= NY; k++)
        for (int h = 1; h <= NX; h++) dst[k][h] = src[(size_t)(k - 1) * NX + (h - 1)];
}
static void nr_to_flat(float **src, float *dst) {
    for (int k = 1; k <= NY; k++)
        for (int h = 1; h <= NX; h++) dst[(size_t)(k - 1) * NX + (h - 1)] = src[k][h];
}
static int **make_recpos(int ntr, const int *recx, const int *recz) {
    int **recpos = imatrix(1, 3, 1, ntr > 0 ? ntr : 1);
    for (int i = 1; i <= ntr; i++) {
        recpos[1][i] = recx[i - 1];
        recpos[2][i] = recz[i - 1];
        recpos[3][i] = 0;
    }
    return recpos;
}

/* eikonal(): forward traveltimes for one source at (srcx, srcz) metres. */
int ref_eikonal(const float *S_flat, float srcx, float srcz, int ntr, const int *recx, const int *recz,
                float *TT_flat, float *Tmod_out) {
    float **S = matrix(1, NY, 1, NX), **TT = matrix(1, NY, 1, NX);
    float *Tmod = vector(1, ntr > 0 ? ntr : 1);
    float **srcpos = matrix(1, 8, 1, 1);
    int **recpos = make_recpos(ntr, recx, recz);
    flat_to_nr(S_flat, S);
    srcpos[1][1] = srcx;
    srcpos[2][1] = srcz;
    long n0 = g_norm1;
    eikonal(S, TT, Tmod, srcpos, 1, 1, recpos, ntr);
    nr_to_flat(TT, TT_flat);
    for (int i = 1; i <= ntr; i++) Tmod_out[i - 1] = Tmod[i];
    free_matrix(S, 1, NY, 1, NX);
    free_matrix(TT, 1, NY, 1, NX);
    free_vector(Tmod, 1, ntr > 0 ? ntr : 1);
    free_matrix(srcpos, 1, 8, 1, 1);
    free_imatrix(recpos, 1, 3, 1, ntr > 0 ? ntr : 1);
    return (int)(g_norm1 - n0);
}

/* eikonal_adj(): adjoint field for scaled residuals Tres (receiver order). */
int ref_eikonal_adj(const float *TT_flat, const float *Tres_in, int ntr, const int *recx, const int *recz,
                    float *lam_flat) {
    float **TT = matrix(1, NY, 1, NX), **lam = matrix(1, NY, 1, NX);
    float *Tres = vector(1, ntr > 0 ? ntr : 1);
    int **recpos = make_recpos(ntr, recx, recz);
    int **recflag = imatrix(1, NY, 1, NX);
    flat_to_nr(TT_flat, TT);
    for (int i = 1; i <= ntr; i++) Tres[i] = Tres_in[i - 1];
    init_recflag(recflag, recpos, ntr);
    long n0 = g_norm1;
    eikonal_adj(TT, Tres, lam, recpos, ntr, 1, recflag);
    nr_to_flat(lam, lam_flat);
    free_matrix(TT, 1, NY, 1, NX);
    free_matrix(lam, 1, NY, 1, NX);
    free_vector(Tres, 1, ntr > 0 ? ntr : 1);
    free_imatrix(recpos, 1, 3, 1, ntr > 0 ? ntr : 1);
    free_imatrix(recflag, 1, NY, 1, NX);
    return (int)(g_norm1 - n0);
}

/* Pick files: one "%.9e" per line so that fscanf("%e") round-trips floats. */
static char g_pickdir[64] = "";
static void write_pick_file(int ishot, int ntr, const float *tobs) {
    char fn[STRING_SIZE2];
    snprintf(fn, sizeof fn, "%s_%i.dat", DATA_DIR, ishot);
    FILE *fp = fopen(fn, "w");
    if (!fp) err("oracle driver: cannot write pick file");
    for (int i = 0; i < ntr; i++) fprintf(fp, "%.9e\n", tobs[i]);
    fclose(fp);
}
static void ensure_pickdir(void) {
    if (g_pickdir[0] == '\0') {
        char tmpl[] = "/tmp/rzrefXXXXXX";
        char *d = mkdtemp(tmpl);
        if (!d) err("oracle driver: mkdtemp failed");
        strncpy(g_pickdir, d, sizeof g_pickdir - 1);
    }
    snprintf(DATA_DIR, STRING_SIZE, "%s/p", g_pickdir);
}

/* calc_FA_res(): Tres is in/out (muted picks leave it untouched, as in the
   reference); returns the shot's l2.  The reference never initialises l2
   (calc_FA_res.c:21); oracle/Makefile builds the sources with
   -ftrivial-auto-var-init=zero so that it starts at 0.0, the value the
   rebuild defines. */
double ref_calc_FA_res(const float *TT_flat, const float *Tmod_in, const float *Tobs_in, float *Tres_io, int ntr,
                       const int *recx, const int *recz) {
    float **TT = matrix(1, NY, 1, NX);
    float *Tmod = vector(1, ntr), *Tobs = vector(1, ntr), *Tres = vector(1, ntr);
    int **recpos = make_recpos(ntr, recx, recz);
    flat_to_nr(TT_flat, TT);
    for (int i = 1; i <= ntr; i++) { Tmod[i] = Tmod_in[i - 1]; Tres[i] = Tres_io[i - 1]; }
    ensure_pickdir();
    write_pick_file(1, ntr, Tobs_in);
    double l2 = calc_FA_res(TT, Tmod, Tobs, Tres, ntr, 1, recpos);
    for (int i = 1; i <= ntr; i++) Tres_io[i - 1] = Tres[i];
    free_matrix(TT, 1, NY, 1, NX);
    free_vector(Tmod, 1, ntr); free_vector(Tobs, 1, ntr); free_vector(Tres, 1, ntr);
    free_imatrix(recpos, 1, 3, 1, ntr);
    return l2;
}

/* grad_obj(): misfit + stacked gradient over shots 1..nshots on one rank.
   Tobs is [nshots][ntr]; grad_out is the flat gradient after grad_obj's own
   cp_grad_frame and precond (all tapers/filters off).  Tres_out receives the
   Tres array as grad_obj leaves it (last shot). */
double ref_grad_obj(const float *S_flat, int nshots, const float *srcx, const float *srcz, int ntr, const int *recx,
                    const int *recz, const float *Tobs_all, float *grad_out, float *lam_last_out, float *Tres_out) {
    float **S = matrix(1, NY, 1, NX), **TT = matrix(1, NY, 1, NX), **lam = matrix(1, NY, 1, NX);
    float **grad = matrix(1, NY, 1, NX);
    float *Tmod = vector(1, ntr), *Tobs = vector(1, ntr), *Tres = vector(1, ntr);
    float **srcpos = matrix(1, 8, 1, nshots);
    int **recpos = make_recpos(ntr, recx, recz);
    flat_to_nr(S_flat, S);
    for (int s = 1; s <= nshots; s++) { srcpos[1][s] = srcx[s - 1]; srcpos[2][s] = srcz[s - 1]; }
    ensure_pickdir();
    for (int s = 1; s <= nshots; s++) write_pick_file(s, ntr, Tobs_all + (size_t)(s - 1) * ntr);
    NSHOT1 = 1;
    NSHOT2 = nshots + 1;
    double L2 = grad_obj(grad, S, TT, lam, Tmod, Tobs, Tres, srcpos, nshots, recpos, ntr, 1);
    nr_to_flat(grad, grad_out);
    if (lam_last_out) nr_to_flat(lam, lam_last_out);
    if (Tres_out) for (int i = 1; i <= ntr; i++) Tres_out[i - 1] = Tres[i];
    free_matrix(S, 1, NY, 1, NX); free_matrix(TT, 1, NY, 1, NX); free_matrix(lam, 1, NY, 1, NX);
    free_matrix(grad, 1, NY, 1, NX);
    free_vector(Tmod, 1, ntr); free_vector(Tobs, 1, ntr); free_vector(Tres, 1, ntr);
    free_matrix(srcpos, 1, 8, 1, nshots);
    free_imatrix(recpos, 1, 3, 1, ntr);
    return L2;
}

/* ass_grad() for one shot into a running gradient (grad_io is in/out). */
void ref_ass_grad(float *grad_io, const float *S_flat, const float *lam_flat) {
    float **S = matrix(1, NY, 1, NX), **lam = matrix(1, NY, 1, NX);
    float **grad = matrix(1, NY, 1, NX), **grad_shot = matrix(1, NY, 1, NX);
    float **srcpos = matrix(1, 8, 1, 1);
    int **recpos = imatrix(1, 3, 1, 1);
    flat_to_nr(S_flat, S);
    flat_to_nr(lam_flat, lam);
    flat_to_nr(grad_io, grad);
    init_grad(grad_shot);
    ass_grad(grad, grad_shot, S, lam, srcpos, 1, recpos, 0, 1);
    nr_to_flat(grad, grad_io);
    free_matrix(S, 1, NY, 1, NX); free_matrix(lam, 1, NY, 1, NX);
    free_matrix(grad, 1, NY, 1, NX); free_matrix(grad_shot, 1, NY, 1, NX);
    free_matrix(srcpos, 1, 8, 1, 1);
    free_imatrix(recpos, 1, 3, 1, 1);
}

/* cp_grad_frame() on a flat field. */
void ref_cp_grad_frame(float *A_flat) {
    float **A = matrix(1, NY, 1, NX);
    flat_to_nr(A_flat, A);
    cp_grad_frame(A);
    nr_to_flat(A, A_flat);
    free_matrix(A, 1, NY, 1, NX);
}

/* --- preconditioning and the FATT stage ------------------------------------ */
/* The reference writes files into the working directory (taper_grad.c's
   taper_coeff_hor.bin, fatt.c's logs and model files, LBFGS.c's history):
   these calls run inside a fresh temporary directory. */
static char g_cwd[4096];
static char g_tmpdir[64];
static void enter_tmpdir(void) {
    if (!getcwd(g_cwd, sizeof g_cwd)) err("oracle driver: getcwd failed");
    char tmpl[] = "/tmp/rzfattXXXXXX";
    char *d = mkdtemp(tmpl);
    if (!d) err("oracle driver: mkdtemp failed");
    strncpy(g_tmpdir, d, sizeof g_tmpdir - 1);
    if (chdir(g_tmpdir)) err("oracle driver: chdir failed");
}
static void leave_tmpdir(void) {
    if (chdir(g_cwd)) err("oracle driver: chdir back failed");
}

static void set_precond_globals(int spatfilter, int fs, int fs1, int taper_hor, int gradt1, int gradt2,
                                float exp_hor) {
    SPATFILTER = spatfilter;
    FILT_SIZE_GRAD = fs;
    FILT_SIZE_GRAD1 = fs1;
    SWS_TAPER_GRAD_HOR = taper_hor;
    SWS_TAPER_GRAD_VERT = 0;
    SWS_TAPER_GRAD_SOURCES = 0;
    SWS_TAPER_FILE = 0;
    GRADT1 = gradt1;
    GRADT2 = gradt2;
    EXP_TAPER_GRAD_HOR = exp_hor;
}

/* precond() (precond.c:12-58) on a flat gradient: SPATFILTER 4 (gauss_filt.c)
   and / or the horizontal taper (taper_grad.c, sws 2). */
void ref_precond(float *grad_flat, int spatfilter, int fs, int fs1, int taper_hor, int gradt1, int gradt2,
                 float exp_hor) {
    float **grad = matrix(1, NY, 1, NX);
    flat_to_nr(grad_flat, grad);
    set_precond_globals(spatfilter, fs, fs1, taper_hor, gradt1, gradt2, exp_hor);
    enter_tmpdir();
    precond(grad, 0, NULL, NULL, 0, 1);
    leave_tmpdir();
    set_precond_globals(0, 0, 0, 0, 0, 0, 0.0f);
    nr_to_flat(grad, grad_flat);
    free_matrix(grad, 1, NY, 1, NX);
}

/* One FATT workflow stage by the reference's own fatt() (fatt.c:10-258):
   l-BFGS (GRAD_METHOD 2, LBFGS.c) with the weak-Wolfe line search
   (LINESEARCH 1, wolfels.c), the workflow file holding one stage.  vp_flat:
   start model in, final model out.  misfit_out / step_out [itermax]: the
   columns of fatt.c's misfit log (L2 and the accepted step per iteration).
   Returns the number of iterations logged. */
int ref_fatt_stage(float *vp_flat, int nshots, const float *srcx, const float *srcz, int ntr, const int *recx,
                   const int *recz, const float *Tobs_all, int itermax, int nlbfgs, int stepmax, float eps_scale,
                   float c1, float c2, float scalefac, float vp_lo, float vp_hi, float pro, int spatfilter, int fs,
                   int fs1, int taper_hor, int gradt1, int gradt2, float exp_hor, double *misfit_out,
                   float *step_out) {
    float **Vp = matrix(1, NY, 1, NX), **S = matrix(1, NY, 1, NX), **TT = matrix(1, NY, 1, NX);
    float *Tmod = vector(1, ntr), *Tobs = vector(1, ntr), *Tres = vector(1, ntr);
    float **srcpos = matrix(1, 8, 1, nshots);
    int **recpos = make_recpos(ntr, recx, recz);
    flat_to_nr(vp_flat, Vp);
    for (int s = 1; s <= nshots; s++) { srcpos[1][s] = srcx[s - 1]; srcpos[2][s] = srcz[s - 1]; }
    ensure_pickdir();
    for (int s = 1; s <= nshots; s++) write_pick_file(s, ntr, Tobs_all + (size_t)(s - 1) * ntr);
    NSHOT1 = 1;
    NSHOT2 = nshots + 1;
    set_precond_globals(spatfilter, fs, fs1, taper_hor, gradt1, gradt2, exp_hor);
    GRAD_METHOD = 2; NLBFGS = nlbfgs; ITERMAX = itermax; LINESEARCH = 1; STEPMAX = stepmax;
    EPS_SCALE = eps_scale; C1 = c1; C2 = c2; SCALEFAC = scalefac; VPLOWERLIM = vp_lo; VPUPPERLIM = vp_hi;
    INVMAT = 1;
    enter_tmpdir();
    snprintf(MISFIT_LOG_FILE, STRING_SIZE, "misfit.log");
    snprintf(JACOBIAN, STRING_SIZE, "jac");
    snprintf(INV_MODELFILE, STRING_SIZE, "inv");
    FILE *fp = fopen("workflow.inp", "w");
    if (!fp) err("oracle driver: cannot write workflow file");
    fprintf(fp, "PRO SPATFILTER WD_DAMP WD_DAMP1 FILT_SIZE_GRAD FILT_SIZE_GRAD1\n");
    fprintf(fp, "%.9e %d 1e-3 1e-3 %d %d\n", pro, spatfilter, fs, fs1);
    fclose(fp);
    calc_S(Vp, S);
    g_nevals = 0;
    char wf[] = "workflow.inp";
    fatt(Vp, S, TT, Tmod, Tobs, Tres, srcpos, nshots, recpos, ntr, wf);
    int n = 0;
    fp = fopen("misfit.log", "r");
    if (fp) {
        float step;
        double l2;
        int stage;
        while (n < itermax && fscanf(fp, "%e %le %d", &step, &l2, &stage) == 3) {
            step_out[n] = step;
            misfit_out[n] = l2;
            n++;
        }
        fclose(fp);
    }
    leave_tmpdir();
    set_precond_globals(0, 0, 0, 0, 0, 0, 0.0f);
    nr_to_flat(Vp, vp_flat);
    free_matrix(Vp, 1, NY, 1, NX); free_matrix(S, 1, NY, 1, NX); free_matrix(TT, 1, NY, 1, NX);
    free_vector(Tmod, 1, ntr); free_vector(Tobs, 1, ntr); free_vector(Tres, 1, ntr);
    free_matrix(srcpos, 1, 8, 1, nshots);
    free_imatrix(recpos, 1, 3, 1, ntr);
    return n;
}
