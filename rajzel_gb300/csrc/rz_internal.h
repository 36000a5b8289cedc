// rz_internal.h -- parameter blocks and launcher declarations shared by the
// kernels (rz_shot.cu, rz_aux.cu) and the C-ABI implementation (rz_api.cu).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace rz {

// Strips are 32 grid rows; one warp sweeps one strip at a time.
constexpr int kStrip = 32;
// Column blocks moved by TMA are 32 columns wide; a warp keeps a ring of
// three blocks of its strip (+1 halo row) in shared memory.
constexpr int kBlk = 32;
constexpr int kRing = 3;
constexpr int kBoxRows = kStrip + 1;
constexpr int kSlotFloats = kBoxRows * kBlk;  // 1056 floats = 4224 B
// warp-to-warp hand-off ring (values of the strip boundary row), guarded by
// full/empty mbarrier pairs per group of kGroup columns
constexpr int kHandoff = 64;
constexpr int kGroup = 8;
constexpr int kGroups = kHandoff / kGroup;
constexpr int kGroupsLog2 = 3;
static_assert(kGroups == 1 << kGroupsLog2, "hand-off groups");
constexpr int kMaxWarps = 16;
constexpr int kTimelineSlots = 8;

// Skewed ("diagonal-major") copy of a per-cell field for one sweep family:
// X[s][q][j] holds the cell (row 32s+j, column h) with
//   family A (sweeps with dx == dy): q = h + j
//   family B (sweeps with dx != dy): q = h - j + 31
// so that the 32 cells a warp updates at one wavefront step are 32
// consecutive floats.  Line q is stored at index q + kSkewFront; qn =
// 32*nxb + 64 lines per strip leave room for the prefetch running up to ten
// lines past either end of a sweep.
constexpr int kSkewFront = 16;
__host__ __device__ inline int skew_lines(int nxb) { return 32 * nxb + 64; }
// Rows bordering a strip (adjoint traveltime halo) are stored with kEdgePad
// floats of padding on both sides of each row.
constexpr int kEdgePad = 48;
__host__ __device__ inline int edge_row(int nxp) { return nxp + 2 * kEdgePad; }

// kModeExact names the exact discrete adjoint sweeps (FP32), kModeTangent the
// traveltime refinement's linear sweeps (FP32); the forward of such a launch
// runs in the context's reference or fast arithmetic.
enum Mode : int { kModeReference = 0, kModeFast = 1, kModeExact = 2, kModeTangent = 3 };

struct ShotParams {
    // grid
    int nx, ny, nxp;        // NX, NY, row pitch (floats) of field buffers
    int nstrips, nxb, qn;   // ceil(NY/32), ceil(NX/32), skew lines per strip
    float dh, time, ttnorm, eps_adj;
    float dh_rcp;           // RN(1/DH)
    int div_fast;           // Markstein division by DH verified for this DH
    int max_passes;
    int nshots;             // shots in this launch (blockIdx.x < nshots)
    int do_residual;        // compute Tres and l2 from Tobs
    int do_adjoint;         // 0: forward (+ residuals) only
    int start_adjoint;      // 1: T and Tres are given; skip forward and residuals
    int exact;              // adjoint: 0 Leung-Qian (sweep_adj.c), 1 exact discrete adjoint
    int refine;             // refine the converged traveltimes to the FP64 fixpoint: T holds the
                            // refined values rounded to float, Told their low parts
    int cotangent;          // exact: Tobs holds dJ/dTmod itself (vector-Jacobian product)
    // model (shared by all shots)
    const float *S;         // slowness [ny][nx]
    const uint8_t *skip;    // cells the adjoint leaves unchanged [ny][nxp] (frame, receivers, padding), or null
    const float *SA, *SB;   // skewed slowness
    const uint32_t *MA, *MB;  // skewed adjoint skip bits (frame | receiver | outside)
    // per-shot fields; shot z at offset z*fstride (floats)
    float *T;               // traveltime  [nshots][ny][nxp]
    float *Told;            // reference-mode snapshot  [nshots][ny][nxp]
    float *L;               // adjoint field lambda [nshots][ny][nxp]
    float *TA, *TB;         // skewed traveltimes [nshots][nstrips][qn][32]
                            // (exact adjoint: signed x weights, see exact_coef)
    float *EU, *ED;         // rows above / below each strip [nshots][nstrips][edge_row(nxp)]
                            // (exact adjoint: their signed z weights)
    float *RA, *RB;         // exact adjoint: skewed dJ/dT at receiver cells, like TA/TB
    size_t fstride;         // ny*nxp
    size_t sstride;         // nstrips*qn*32
    size_t estride;         // nstrips*edge_row(nxp)
    // sources (0-based grid indices) for the shots of this launch
    const int *src_h, *src_k;
    // receivers (0-based)
    int ntr;
    const int *rec_h, *rec_k;
    // de-duplicated interior receiver cells and the receiver whose residual
    // initialises lambda there ("last receiver wins", init_travel_adj.c:49-54)
    int nrcell;
    const int *rcell_h, *rcell_k, *rcell_rec;
    // every receiver cell (frame included) with its receivers in index order:
    // cell i holds receivers xcell_rec[xcell_off[i] .. xcell_off[i+1]-1]
    int nxcell;
    const int *xcell_h, *xcell_k, *xcell_off, *xcell_rec;
    const float *Tobs;      // [nshots][ntr]
    float *Tmod, *Tres;     // [nshots][ntr]
    double *l2;             // [nshots]
    int *passes_fwd, *passes_adj, *status;  // [nshots]
    // passes actually swept [nshots][2] (forward, adjoint): a pass proven to
    // change nothing is counted in passes_* but not swept
    int *swept;
    unsigned long long *timeline;           // [nshots][kTimelineSlots] ns stamps, or null
    // change votes of the last sweep of a pass, [nshots][nstrips][4*(nxb+1)]
    // bytes: group G of strip s changed a cell (fixpoint checks skip the
    // tasks no change can reach), or null
    uint8_t *chg;
    size_t chg_stride;                      // nstrips*4*(nxb+1)
    // launch_prep_model's first-invalid-cell word (kModelOk: none), or null:
    // an invalid model ends every shot at once with ERR_BAD_MODEL
    const int *model_bad;
    // waits for another warp give up after `spin` polls (0: kSpinLimit);
    // withhold (test hook): warp 0 of every CTA withholds one hand-off
    // signal in its first sweep, so warp 1's bounded wait runs out
    uint32_t spin;
    int withhold;
    // fixpoint checks: most rows per task (0: kCheckRows), the autotuner's choice
    int check_rows;
};

// Tensor maps of a launch.  Field maps cover [shots][ny][nxp] floats with
// logical extent [shots][ny][nx]:
//   tld  traveltime, 32 x kBoxRows box (forward sweeps, adjoint preparation)
//   tst  traveltime, 32 x kStrip box (forward sweeps' write-back)
//   lld  lambda, 32 x kBoxRows box (adjoint sweeps)
//   lst  lambda, 32 x kStrip box (adjoint sweeps' write-back)
//   tchk traveltime, 136 x 4 box (fixpoint checks)
//   lchk lambda, 136 x 4 box (adjoint fixpoint check)
//   schk slowness in rows of nxp floats [1][ny][nxp], 128 x 4 box (forward check)
//   tlo  low parts of refined traveltimes, 32 x kBoxRows box (exact adjoint preparation)
constexpr int kCheckCols = 136, kCheckBoxRows = 4;  // box of tchk / lchk
struct ShotMaps {
    CUtensorMap tld, tst, lld, lst, tchk, lchk, schk, tlo;
};

// several grids in one persistent launch
constexpr int kMaxGrids = 8;
struct MultiGrid {
    ShotMaps maps;
    ShotParams P;
    int W;                        // warps of the CTA that sweep this grid's strips
};
struct MultiParams {
    MultiGrid grid[kMaxGrids];
    int ngrids, njobs;
    int *counter;       // zeroed before the launch
    const int2 *jobs;   // [njobs] (grid, shot), largest grids first
};

// launchers (rz_shot.cu)
size_t shot_kernel_smem(int nwarps);
int shot_kernel_warps(int nstrips);  // warps per CTA for a grid of nstrips strips
// persistent CTAs of at least W warps (W >= every grid's W); nctas receives the grid size
cudaError_t launch_multi_shot_kernel(const MultiParams &M, int mode, int W, int *nctas, cudaStream_t st);
// warps: strips swept together per band; 0 = the balanced choice of
// shot_kernel_warps.  The CTA may hold more warps than that (they share the
// cell-parallel phases) where this costs no occupancy: cta_warps caps them
// (0 = as many as fit).  No result changes.
cudaError_t launch_shot_kernel(const ShotParams &P, int mode, const ShotMaps &maps, cudaStream_t st, int warps = 0,
                               int cta_warps = 0);

// launchers (rz_aux.cu)
cudaError_t launch_skew_field(const float *src, int nx, int ny, int pitch, int nstrips, int nxb, float *dstA,
                              float *dstB, cudaStream_t st, const int *note_src = nullptr, int *note_dst = nullptr);
cudaError_t launch_skip_masks(const uint8_t *skip, int nx, int ny, int nstrips, int nxb, uint32_t *MA, uint32_t *MB,
                              cudaStream_t st);
// gradient stack: grad = sum_s RN32(lam_s * cube) on the interior
//   mode reference: per-shot float contribution RN32(RN64(lam*cube64)) added
//   in float in shot order; mode fast: lam summed exactly (shot_sum_fixed),
//   times S^3 in double.
//   accumulate: continue the sums already in grad / grad64 (chunked batches)
//   frame: also the frame cells, as cp_grad_frame leaves them (a single
//   chunk, nx, ny >= 5; else launch_cp_frame afterwards)
//   l2_out: also *l2_out = 0.5 * sum of l2[0..nl2) (as launch_sum_l2)
cudaError_t launch_stack(const float *L, size_t fstride, int nshots, const double *cube, const float *S, int nx,
                         int ny, int nxp, int mode, float *grad, int gpitch, double *grad64, bool accumulate,
                         cudaStream_t st, bool frame = false, const double *l2 = nullptr, int nl2 = 0,
                         double *l2_out = nullptr);
// exact-adjoint gradient dJ/dVp = -S^2 sum_s mu_s * dG/dS (G the Godunov
// update at the converged traveltimes T_s, or T_s + Tlo_s when refined);
// continues grad64 when accumulate
cudaError_t launch_stack_exact(const float *T, const float *L, size_t fstride, int nshots, const int *src_h,
                               const int *src_k, const float *S, int nx, int ny, int nxp, float dh, float *grad,
                               double *grad64, bool accumulate, cudaStream_t st, const float *Tlo = nullptr);
cudaError_t launch_cp_frame(float *A, double *A64, int nx, int ny, int pitch, int times, cudaStream_t st);
cudaError_t launch_copy_rows(const float *src, int src_pitch, float *dst, int dst_pitch, int nx, int ny,
                             size_t nbatch, size_t src_bstride, size_t dst_bstride, cudaStream_t st);
cudaError_t launch_check_div(float dh, float rcp, unsigned int *bad, cudaStream_t st);
// S = (float)(1.0/(double)vp) per cell (calc_S.c:21), its nxp-pitch copy and
// the first invalid cell, in one launch (after resetting *first_bad)
constexpr int kModelOk = 0x7f7f7f7f;  // launch_prep_model: no invalid cell (grids have fewer cells)
cudaError_t launch_prep_model(const float *src, bool is_vp, float *S, float *Sp, int nx, int ny, int nxp,
                              int *first_bad, cudaStream_t st);
// gout[0..n) = g, *l2_out = *l2, *status_out = OR of status[0..nshots): the
// end of a gradient call whose outputs are host memory the device writes
cudaError_t launch_finish_grad(const float *g, float *gout, long n, const double *l2, double *l2_out,
                               const int *status, int nshots, int *status_out, cudaStream_t st);
// *out = 0.5 * sum_z l2[z], summed in shot order in double (grad_obj.c:28,42,61)
cudaError_t launch_sum_l2(const double *l2, int n, double *out, cudaStream_t st);

// FP64 oracle (rz_fp64.cu): one CTA per shot, double fields [shot][ny][nx]
struct F64Params {
    int nx, ny, nxp;
    double dh, time, ttnorm, eps_adj;  // the float globals, widened
    int max_passes;
    int fixpoint;                // forward: sweep until a pass changes no cell (TTNORM not used)
    int nshots;
    int do_residual, do_adjoint;
    int exact;                   // adjoint: 0 Leung-Qian, 1 exact discrete adjoint
    int cotangent;               // exact: Tobs holds dJ/dTmod itself
    const float *S;              // slowness [ny][nx]
    const uint8_t *skip;         // [ny][nxp]: cells the Leung-Qian sweeps leave unchanged
    const int *src_h, *src_k;    // [nshots]
    int ntr;
    const int *rec_h, *rec_k;
    int nrcell;
    const int *rcell_h, *rcell_k, *rcell_rec;
    int nxcell;
    const int *xcell_h, *xcell_k, *xcell_off, *xcell_rec;
    const float *Tobs;           // [nshots][ntr]
    double *T, *A, *L;           // traveltime, snapshot (exact: R), adjoint field (exact: mu)
    double *WX, *WZ, *GS;        // exact: signed weights and dG/dS per cell
    double *Tmod, *Tres, *l2;    // [nshots][ntr], [nshots][ntr], [nshots]
    int *passes_fwd, *passes_adj, *status;
    size_t fstride;              // nx*ny
};
cudaError_t launch_fp64_shots(const F64Params &P, cudaStream_t st);
// gradient of the launch's shots added to grad64 [ny][nx] in shot order
cudaError_t launch_fp64_stack(const F64Params &P, double *grad64, bool accumulate, cudaStream_t st);
cudaError_t launch_fp64_vp_scale(const float *S, long n, double *grad64, cudaStream_t st);
// acc[4 z + 0..3] += sum (a-b)^2, sum b^2, max |a-b|, max |b| over rows of
// ncol values of batch entry z (a float with row pitch pa, b double with pb)
cudaError_t launch_compare(const float *a, int pa, const double *b, int pb, int ncol, long nrow, int nbatch,
                           size_t bstride_a, size_t bstride_b, double *acc, cudaStream_t st);
cudaError_t launch_d2f(const double *src, float *dst, long n, cudaStream_t st);

}  // namespace rz

// context accessors for code layered on the C ABI (rz_fatt.cu)
struct rz_context;
int rz_context_query(rz_context *c, int *nx, int *ny, float *dh, int *ntr, cudaStream_t *stream);
void rz_context_set_error(rz_context *c, const char *msg);
