// rz_api.cu -- implementation of the C ABI declared in include/rajzel_gb300.h.
//
// A context owns: the grid constants (the reference's globals), the model
// (slowness, its two skewed copies, the pow(S,3) table of the reference
// gradient), the receiver geometry (skewed adjoint skip bits, de-duplicated
// receiver cells), and per-shot work buffers sized for the largest batch
// seen so far, with their TMA descriptors.  All work is issued on one CUDA
// stream.  Host-side validation rejects every input on which the reference
// would index out of bounds or loop forever.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <array>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/rajzel_gb300.h"
#include "rz_internal.h"

using namespace rz;

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

struct rz_context {
    int device = 0;
    cudaStream_t own = nullptr, st = nullptr;
    int mode = RZ_MODE_REFERENCE;
    std::string err;

    // grid
    bool grid_set = false;
    rz_grid g{};
    int nxp = 0, nstrips = 0, nxb = 0, qn = 0;
    int div_fast = 0;
    float div_dh = -1.f;

    // model
    bool model_set = false;
    float *dS = nullptr, *dSA = nullptr, *dSB = nullptr, *dVp = nullptr;
    float *dSp = nullptr;  // slowness in rows of nxp floats (fixpoint checks)
    double *dCube = nullptr;
    bool cube_valid = false;
    int *dBad = nullptr;  // launch_prep_model result
    // words the device writes into mapped pinned host memory (host / device
    // address), read after a stream wait without a copy
    struct HostWords {
        double l2;   // misfit of a gradient call
        int status;  // OR of the shots' status words
        int bad;     // launch_prep_model result
    };
    HostWords *hw = nullptr, *hwDev = nullptr;
    bool host_coherent = false;  // the device reaches every host address coherently (Grace C2C)

    // receivers
    bool rec_set = false;
    int ntr = 0, nrcell = 0, nxcell = 0;
    int *dRecH = nullptr, *dRecK = nullptr, *dRcH = nullptr, *dRcK = nullptr, *dRcRec = nullptr;
    int *dXcH = nullptr, *dXcK = nullptr, *dXcOff = nullptr, *dXcRec = nullptr;  // all receiver cells
    uint8_t *dSkip = nullptr;
    uint8_t *dSkipP = nullptr;  // [ny][nxp]: frame, receiver and padding cells (adjoint fixpoint check)
    uint32_t *dMA = nullptr, *dMB = nullptr;

    // per-shot field slots (a batch larger than cap_f runs in chunks of cap_f shots)
    int cap_f = 0;
    size_t memcap = 0;  // bytes the field slots may occupy; 0 = 90% of free device memory
    float *dT = nullptr, *dTold = nullptr, *dL = nullptr, *dTA = nullptr, *dTB = nullptr, *dEU = nullptr,
          *dED = nullptr;
    uint8_t *dChg = nullptr;  // [slot][nstrips][4*(nxb+1)] change votes of a pass's last sweep
    float *dRA = nullptr, *dRB = nullptr;  // exact adjoint and refinement only
    bool fields_exact = false;
    ShotMaps maps{};  // tensor maps of the field buffers and the row-pitched slowness
    int grad_kind = RZ_GRADIENT_REFERENCE;
    // per-shot scalars and receiver arrays, sized for the whole batch
    int cap_s = 0;
    float *dTobs = nullptr, *dTmod = nullptr, *dTres = nullptr;
    double *dl2 = nullptr, *dL2 = nullptr;
    int *dPf = nullptr, *dPa = nullptr, *dStat = nullptr, *dSrcH = nullptr, *dSrcK = nullptr;
    int *dSwept = nullptr;  // [n][2] passes actually swept
    unsigned long long *dTl = nullptr;
    float *dGrad = nullptr;
    double *dGrad64 = nullptr;

    int last_n = 0;           // shots of the last batch
    int last_first = 0;       // first shot whose fields are still in the slots
    bool last_adj = false;

    // band width (warps per CTA) of the shot-kernel launches: 0 = balanced
    // default; rz_autotune records the fastest per (shots, mode, gradient kind)
    int warps = 0;
    bool tuning = false;
    // the launch shape: warps that sweep (warps), CTA width (cta_warps, 0 =
    // as wide as fits), most rows per fixpoint-check task (check_rows, 0 =
    // default); rz_autotune records the fastest per (shots, mode, gradient kind)
    int cta_warps = 0, check_rows = 0;
    struct Shape {
        int warps, cta_warps, check_rows;
    };
    std::map<std::array<int, 3>, Shape> tuned;

    // CUDA graph of the rz_grad_obj sequence, replayed while its key is unchanged
    bool use_graphs = true;
    bool capturing = false;
    struct GraphKey {
        ShotParams P0;  // parameters of the first chunk (pointers, constants)
        int nshots, chunk, mode, kind, cap_f, flags_dev, warps, cta_warps;
        const void *gdst, *grad64, *cube, *S, *L2;
    } gkey;
    cudaGraph_t graph = nullptr;          // kept: its nodes name the exec's event records
    cudaGraphExec_t gexec = nullptr;
    std::vector<cudaGraphNode_t> gevents;  // event-record nodes around each shot-kernel launch
    std::vector<cudaEvent_t> gcap_events;  // the events recorded at capture time
    std::vector<cudaEvent_t> ginstalled;   // events the exec's nodes hold now
    std::vector<cudaEvent_t> gretired;     // read by rz_kernel_stats, still installed
    long long glaunches = 0;               // kernels per replay

    // persistent multi-grid launches driven by this context
    int2 *dJobs = nullptr;
    int njobs_cap = 0;
    int *dCounter = nullptr;

    // accounting: kernels launched, and CUDA-event timing of every shot-kernel launch
    long long launches = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> shot_events;

    // FP64 oracle (rz_fp64.cu): double field slots, sized for the largest
    // chunk seen, and per-shot scalars for the whole batch
    int cap64 = 0;
    bool cap64_exact = false;
    double *d64T = nullptr, *d64A = nullptr, *d64L = nullptr, *d64WX = nullptr, *d64WZ = nullptr, *d64GS = nullptr;
    int cap64s = 0;
    double *d64Tmod = nullptr, *d64Tres = nullptr, *d64l2 = nullptr;
    int *d64Pf = nullptr, *d64Pa = nullptr, *d64Stat = nullptr;
    double *d64Grad = nullptr, *d64L2 = nullptr;
    double *dCmp = nullptr;  // comparison accumulators (4 doubles per entry)
    int ncmp = 0;
    const float *last_grad = nullptr;  // device gradient of the last rz_grad_obj
    // bounded waits: polls before a wait for another warp gives up (0 =
    // default) and the withheld hand-off of the timeout test (rz_set_wait_test)
    unsigned spin = 0;
    int withhold = 0;
    // traveltime refinement to the FP64 fixpoint (rz_set_refine)
    bool refine = false;
    // errors of float results against the FP64 oracle (rz_set_error_check)
    bool err_check = false;
    bool err_valid = false;
    rz_error err_rep{};
};

// ---------------------------------------------------------------------------
// helpers
// ---------------------------------------------------------------------------
static int fail(rz_context *c, int code, const char *fmt, ...) {
    if (c) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        c->err = buf;
    }
    return code;
}

// a failed call's error is reported and cleared, so that it does not
// resurface in the next call's launch check
#define CK(call)                                                                                         \
    do {                                                                                                 \
        cudaError_t e_ = (call);                                                                         \
        if (e_ != cudaSuccess) {                                                                         \
            (void)cudaGetLastError();                                                                    \
            return fail(c, e_ == cudaErrorMemoryAllocation ? RZ_ENOMEM : RZ_ECUDA, "%s: %s (%s:%d)", #call, \
                        cudaGetErrorString(e_), __FILE__, __LINE__);                                     \
        }                                                                                                \
    } while (0)

template <typename T>
static cudaError_t dalloc(T **p, size_t count) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (count == 0) count = 1;
    return cudaMalloc((void **)p, count * sizeof(T));
}

template <typename T>
static void dfree(T *&p) {
    if (p) cudaFree(p);
    p = nullptr;
}

static int iround_pos(float x, float dh) { return (int)std::floor((double)(x / dh) + 0.5); }

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, looked up once for all host threads
static EncodeTiledFn encode_fn() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
        else
            (void)cudaGetLastError();
    });
    return fn;
}

// 3-D map over [depth][ny][nxp] float fields, logical extent [depth][ny][nx]
static int make_map(rz_context *c, CUtensorMap *m, float *base, int depth, int box_cols, int box_rows) {
    EncodeTiledFn enc = encode_fn();
    if (!enc) return fail(c, RZ_ECUDA, "cuTensorMapEncodeTiled entry point unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)c->g.nx, (cuuint64_t)c->g.ny, (cuuint64_t)depth};
    cuuint64_t strides[2] = {(cuuint64_t)c->nxp * 4, (cuuint64_t)c->nxp * c->g.ny * 4};
    cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                     CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                     CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(c, RZ_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return RZ_OK;
}

static void free_fields(rz_context *c) {
    dfree(c->dT), dfree(c->dTold), dfree(c->dL), dfree(c->dTA), dfree(c->dTB), dfree(c->dEU), dfree(c->dED);
    dfree(c->dChg);
    dfree(c->dRA), dfree(c->dRB);
    c->fields_exact = false;
    c->cap_f = 0;
}

static void free_shots(rz_context *c) {
    dfree(c->dTobs), dfree(c->dTmod), dfree(c->dTres), dfree(c->dl2), dfree(c->dPf), dfree(c->dPa);
    dfree(c->dStat), dfree(c->dSrcH), dfree(c->dSrcK), dfree(c->dTl), dfree(c->dSwept);
    c->cap_s = 0;
}

static void free_fp64(rz_context *c) {
    dfree(c->d64T), dfree(c->d64A), dfree(c->d64L), dfree(c->d64WX), dfree(c->d64WZ), dfree(c->d64GS);
    c->cap64 = 0;
    c->cap64_exact = false;
    dfree(c->d64Tmod), dfree(c->d64Tres), dfree(c->d64l2), dfree(c->d64Pf), dfree(c->d64Pa), dfree(c->d64Stat);
    c->cap64s = 0;
    dfree(c->d64Grad), dfree(c->d64L2), dfree(c->dCmp);
    c->ncmp = 0;
}

static void free_batch(rz_context *c) {
    free_fields(c);
    free_shots(c);
    free_fp64(c);
}

// device bytes of one field slot: T, pass snapshot, lambda, two skewed T copies, border rows,
// change votes (the exact adjoint and the refinement add skewed receiver terms or residuals,
// two copies; their packed weights take the skewed T copies' place)
static size_t slot_bytes(const rz_context *c) {
    const size_t fs = (size_t)c->g.ny * c->nxp, ss = (size_t)c->nstrips * c->qn * 32,
                 es = (size_t)c->nstrips * edge_row(c->nxp);
    const size_t extra = (c->grad_kind == RZ_GRADIENT_EXACT || c->refine) ? 2 * ss : 0;
    return 4 * (3 * fs + 2 * ss + 2 * es + extra) + (size_t)c->nstrips * 4 * (c->nxb + 1);  // + change votes
}

static int ensure_fields(rz_context *c, int n) {
    const bool exact = c->grad_kind == RZ_GRADIENT_EXACT || c->refine;  // weight streams
    if (n <= c->cap_f && (!exact || c->fields_exact)) return RZ_OK;
    if (n < c->cap_f) n = c->cap_f;
    free_fields(c);
    const size_t fs = (size_t)c->g.ny * c->nxp, ss = (size_t)c->nstrips * c->qn * 32,
                 es = (size_t)c->nstrips * edge_row(c->nxp);
    CK(dalloc(&c->dT, fs * n));
    CK(dalloc(&c->dTold, fs * n));
    CK(dalloc(&c->dL, fs * n));
    CK(dalloc(&c->dChg, (size_t)c->nstrips * 4 * (c->nxb + 1) * n));
    CK(dalloc(&c->dTA, ss * n));
    CK(dalloc(&c->dTB, ss * n));
    CK(dalloc(&c->dEU, es * n));
    CK(dalloc(&c->dED, es * n));
    CK(cudaMemsetAsync(c->dEU, 0, es * n * 4, c->st));
    CK(cudaMemsetAsync(c->dED, 0, es * n * 4, c->st));
    if (exact) {
        CK(dalloc(&c->dRA, ss * n));
        CK(dalloc(&c->dRB, ss * n));
        c->fields_exact = true;
    }
    c->cap_f = n;
    int r;
    if ((r = make_map(c, &c->maps.tld, c->dT, n, kBlk, kBoxRows))) return r;
    if ((r = make_map(c, &c->maps.tst, c->dT, n, kBlk, kStrip))) return r;
    if ((r = make_map(c, &c->maps.lld, c->dL, n, kBlk, kBoxRows))) return r;
    if ((r = make_map(c, &c->maps.lst, c->dL, n, kBlk, kStrip))) return r;
    if ((r = make_map(c, &c->maps.tchk, c->dT, n, kCheckCols, kCheckBoxRows))) return r;
    if ((r = make_map(c, &c->maps.lchk, c->dL, n, kCheckCols, kCheckBoxRows))) return r;
    if ((r = make_map(c, &c->maps.tlo, c->dTold, n, kBlk, kBoxRows))) return r;
    return RZ_OK;
}

static int ensure_shots(rz_context *c, int n) {
    if (n <= c->cap_s) return RZ_OK;
    free_shots(c);
    const size_t nt = (size_t)(c->ntr > 0 ? c->ntr : 1);
    CK(dalloc(&c->dTobs, nt * n));
    CK(dalloc(&c->dTmod, nt * n));
    CK(dalloc(&c->dTres, nt * n));
    CK(dalloc(&c->dl2, (size_t)n));
    CK(dalloc(&c->dPf, (size_t)n));
    CK(dalloc(&c->dPa, (size_t)n));
    CK(dalloc(&c->dStat, (size_t)n));
    CK(dalloc(&c->dSrcH, (size_t)n));
    CK(dalloc(&c->dSrcK, (size_t)n));
    CK(dalloc(&c->dTl, (size_t)n * kTimelineSlots));
    CK(dalloc(&c->dSwept, (size_t)n * 2));
    c->cap_s = n;
    return RZ_OK;
}

// Shots per chunk for a batch of n: all of them when their field slots fit
// the memory cap, else as many as fit (at least one).  Allocates the slots.
static int plan_chunks(rz_context *c, int n, int *chunk) {
    const size_t per = slot_bytes(c);
    size_t limit = c->memcap;
    if (limit == 0) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        limit = (size_t)(0.9 * (double)(fr + per * (size_t)c->cap_f));
    }
    size_t fit = limit / per;
    if (fit < 1) fit = 1;
    int m = (size_t)n < fit ? n : (int)fit;
    if (m < n) {
        // whole waves: a chunk of a multiple of the SM count leaves no SM idle
        int sms = 0;
        CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device));
        if (sms > 0 && m > sms) m -= m % sms;
    }
    // keep existing slots when they already hold a whole chunk
    if (c->cap_f > m && (size_t)c->cap_f <= fit) m = n < c->cap_f ? n : c->cap_f;
    if (c->cap_f > 0 && (size_t)c->cap_f > fit) free_fields(c);  // slots of a larger kind no longer fit
    int r;
    if ((r = ensure_fields(c, m))) return r;
    *chunk = m;
    return RZ_OK;
}

static int ensure_div(rz_context *c) {
    if (c->div_dh == c->g.dh) return RZ_OK;
    unsigned int *dbad = nullptr, hbad = 1;
    CK(cudaMalloc(&dbad, sizeof(unsigned int)));
    CK(cudaMemsetAsync(dbad, 0, sizeof(unsigned int), c->st));
    const float rcp = (float)(1.0 / (double)c->g.dh);
    CK(launch_check_div(c->g.dh, rcp, dbad, c->st));
    CK(cudaMemcpyAsync(&hbad, dbad, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    cudaFree(dbad);
    // the check covers x in [1,2); it carries to every exponent the sweeps use
    // for DH within [2^-20, 2^20] (quotients and remainders stay normal)
    c->div_fast = (hbad == 0) && c->g.dh >= 0x1p-20f && c->g.dh <= 0x1p20f;
    c->div_dh = c->g.dh;
    return RZ_OK;
}

// reference-mode gradient needs pow(S,3.0) exactly as the host C library
// returns it (ass_grad.c:23); it is faithful but not always correctly rounded
static int ensure_cube(rz_context *c) {
    if (c->cube_valid) return RZ_OK;
    const size_t n = (size_t)c->g.nx * c->g.ny;
    std::vector<float> hS(n);
    CK(cudaMemcpyAsync(hS.data(), c->dS, n * 4, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    std::vector<double> cube(n);
    // pow of the host C library (reentrant), spread over the host cores
    auto cubes = [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i) cube[i] = std::pow((double)hS[i], 3.0);
    };
    const unsigned nt = n < (size_t)1 << 16 ? 1u : std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::thread> pool;
    const size_t chunk = (n + nt - 1) / nt;
    for (unsigned t = 1; t < nt; ++t)
        if (t * chunk < n) pool.emplace_back(cubes, t * chunk, std::min(n, (t + 1) * chunk));
    cubes(0, std::min(n, chunk));
    for (auto &th : pool) th.join();
    if (!c->dCube) CK(dalloc(&c->dCube, n));  // kept across models (graphs hold the pointer)
    CK(cudaMemcpyAsync(c->dCube, cube.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->cube_valid = true;
    return RZ_OK;
}

static bool have_dev(int flags) { return (flags & RZ_DEVICE_PTRS) != 0; }

// parameters for shots first..first+n-1 of the batch, their fields in slots 0..n-1
static void fill_params(rz_context *c, ShotParams &P, int first, int n) {
    memset(&P, 0, sizeof P);
    P.nx = c->g.nx;
    P.ny = c->g.ny;
    P.nxp = c->nxp;
    P.nstrips = c->nstrips;
    P.nxb = c->nxb;
    P.qn = c->qn;
    P.dh = c->g.dh;
    P.time = c->g.time;
    P.ttnorm = c->g.ttnorm;
    P.eps_adj = c->g.eps_adj;
    P.dh_rcp = (float)(1.0 / (double)c->g.dh);
    P.div_fast = c->div_fast;
    P.max_passes = c->g.max_passes > 0 ? c->g.max_passes : 10000;
    P.nshots = n;
    P.S = c->dS;
    P.skip = c->dSkipP;
    P.SA = c->dSA;
    P.SB = c->dSB;
    P.MA = c->dMA;
    P.MB = c->dMB;
    P.T = c->dT;
    P.Told = c->dTold;
    P.L = c->dL;
    P.TA = c->dTA;
    P.TB = c->dTB;
    P.EU = c->dEU;
    P.ED = c->dED;
    P.fstride = (size_t)c->g.ny * c->nxp;
    P.sstride = (size_t)c->nstrips * c->qn * 32;
    P.estride = (size_t)c->nstrips * edge_row(c->nxp);
    P.src_h = c->dSrcH + first;
    P.src_k = c->dSrcK + first;
    P.ntr = c->ntr;
    P.rec_h = c->dRecH;
    P.rec_k = c->dRecK;
    P.nrcell = c->nrcell;
    P.rcell_h = c->dRcH;
    P.rcell_k = c->dRcK;
    P.rcell_rec = c->dRcRec;
    P.nxcell = c->nxcell;
    P.xcell_h = c->dXcH;
    P.xcell_k = c->dXcK;
    P.xcell_off = c->dXcOff;
    P.xcell_rec = c->dXcRec;
    P.RA = c->dRA;
    P.RB = c->dRB;
    P.Tobs = c->dTobs + (size_t)first * c->ntr;
    P.Tmod = c->dTmod + (size_t)first * c->ntr;
    P.Tres = c->dTres + (size_t)first * c->ntr;
    P.l2 = c->dl2 + first;
    P.passes_fwd = c->dPf + first;
    P.passes_adj = c->dPa + first;
    P.status = c->dStat + first;
    P.timeline = c->dTl + (size_t)first * kTimelineSlots;
    P.swept = c->dSwept + (size_t)first * 2;
    P.chg = c->dChg;
    P.chg_stride = (size_t)c->nstrips * 4 * (c->nxb + 1);
    P.spin = c->spin;
    P.withhold = c->withhold;
    P.refine = c->refine ? 1 : 0;
    P.check_rows = c->check_rows;
}

static int status_to_code(int bits) {
    if (bits & 3) return RZ_ETIMEOUT;
    if (bits & 12) return RZ_ENOCONV;
    if (bits) return RZ_EINVAL;
    return RZ_OK;
}

// upload validated source indices for n shots
static int set_sources(rz_context *c, int n, const float *srcx, const float *srcz) {
    if (!srcx || !srcz) return fail(c, RZ_EINVAL, "source arrays are NULL");
    std::vector<int> hh(n), kk(n);
    for (int i = 0; i < n; ++i) {
        int h = iround_pos(srcx[i], c->g.dh) - 1, k = iround_pos(srcz[i], c->g.dh) - 1;
        if (!(std::isfinite(srcx[i]) && std::isfinite(srcz[i])) || h < 0 || h >= c->g.nx || k < 0 || k >= c->g.ny)
            return fail(c, RZ_EINVAL, "shot %d: source (%g, %g) m maps to grid index (%d, %d) outside 1..%d x 1..%d", i,
                        srcx[i], srcz[i], h + 1, k + 1, c->g.nx, c->g.ny);
        hh[i] = h;
        kk[i] = k;
    }
    CK(cudaMemcpyAsync(c->dSrcH, hh.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->dSrcK, kk.data(), n * sizeof(int), cudaMemcpyHostToDevice, c->st));
    return RZ_OK;
}

static int ready(rz_context *c, bool need_rec) {
    if (!c) return RZ_EINVAL;
    if (!c->grid_set) return fail(c, RZ_ESTATE, "rz_set_grid has not been called");
    if (!c->model_set) return fail(c, RZ_ESTATE, "no slowness/velocity model set");
    if (need_rec && !c->rec_set) return fail(c, RZ_ESTATE, "rz_set_receivers has not been called");
    return RZ_OK;
}

// copy a [n][ny][nxp] device field batch to a packed [n][ny][nx] destination
static int copy_out_fields(rz_context *c, const float *src, float *dst, int n, int flags) {
    const size_t fs = (size_t)c->g.ny * c->nxp;
    for (int z = 0; z < n; ++z) {
        CK(cudaMemcpy2DAsync(dst + (size_t)z * c->g.nx * c->g.ny, (size_t)c->g.nx * 4, src + z * fs,
                             (size_t)c->nxp * 4, (size_t)c->g.nx * 4, c->g.ny,
                             have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
    }
    return RZ_OK;
}

static int run_batch(rz_context *c, int first, int n, bool adjoint, bool residual, bool start_adj, bool exact = false,
                     bool cotangent = false) {
    int r;
    if ((r = ensure_div(c))) return r;
    ShotParams P;
    fill_params(c, P, first, n);
    P.do_residual = residual ? 1 : 0;
    P.do_adjoint = adjoint ? 1 : 0;
    P.start_adjoint = start_adj ? 1 : 0;
    P.exact = exact ? 1 : 0;
    P.cotangent = cotangent ? 1 : 0;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const unsigned evf = c->capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    CK(cudaEventRecordWithFlags(e0, c->st, evf));
    CK(launch_shot_kernel(P, c->mode, c->maps, c->st, c->warps, c->cta_warps));
    CK(cudaEventRecordWithFlags(e1, c->st, evf));
    c->shot_events.emplace_back(e0, e1);
    c->launches += 1;
    c->last_first = first;
    c->last_adj = adjoint;
    return RZ_OK;
}

// clear the per-shot counters of a whole batch before its chunks run
static int reset_shots(rz_context *c, int n) {
    CK(cudaMemsetAsync(c->dStat, 0, n * sizeof(int), c->st));
    CK(cudaMemsetAsync(c->dTl, 0, (size_t)n * kTimelineSlots * sizeof(unsigned long long), c->st));
    CK(cudaMemsetAsync(c->dPf, 0, n * sizeof(int), c->st));
    CK(cudaMemsetAsync(c->dPa, 0, n * sizeof(int), c->st));
    CK(cudaMemsetAsync(c->dSwept, 0, 2 * n * sizeof(int), c->st));
    c->last_n = n;
    return RZ_OK;
}

static int collect_status(rz_context *c, int n) {
    std::vector<int> st(n);
    CK(cudaMemcpyAsync(st.data(), c->dStat, n * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    int worst = 0;
    for (int i = 0; i < n; ++i) worst |= st[i];
    int code = status_to_code(worst);
    if (code != RZ_OK) return fail(c, code, "device status bits 0x%x", worst);
    return RZ_OK;
}

static void drop_graph(rz_context *c) {
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    if (c->graph) cudaGraphDestroy(c->graph);
    c->gexec = nullptr;
    c->graph = nullptr;
    c->gevents.clear();
    for (auto e : c->gcap_events) cudaEventDestroy(e);
    c->gcap_events.clear();
    for (auto e : c->gretired) cudaEventDestroy(e);
    c->gretired.clear();
    c->ginstalled.clear();  // still listed for rz_kernel_stats, which frees them
}

static bool contains(const std::vector<cudaEvent_t> &v, cudaEvent_t e) {
    return std::find(v.begin(), v.end(), e) != v.end();
}

// gradient contribution of the shots first..first+m-1 (fields in slots 0..m-1).
// whole: these are all the batch's shots.  *finished: the launch also wrote
// the frame cells and the misfit (a whole Leung-Qian batch), so neither the
// frame copy nor the misfit sum follows.
static int stack_chunk(rz_context *c, int first, int m, float *gdst, bool whole = false, bool *finished = nullptr) {
    const size_t fs = (size_t)c->g.ny * c->nxp;
    bool fin = false;
    if (c->grad_kind == RZ_GRADIENT_EXACT) {
        CK(launch_stack_exact(c->dT, c->dL, fs, m, c->dSrcH + first, c->dSrcK + first, c->dS, c->g.nx, c->g.ny,
                              c->nxp, c->g.dh, gdst, c->dGrad64, first > 0, c->st, c->refine ? c->dTold : nullptr));
    } else {
        fin = whole && first == 0 && c->g.nx >= 5 && c->g.ny >= 5 && c->dL2;
        CK(launch_stack(c->dL, fs, m, c->dCube, c->dS, c->g.nx, c->g.ny, c->nxp, c->mode, gdst, c->g.nx,
                        c->mode == RZ_MODE_FAST ? c->dGrad64 : nullptr, first > 0, c->st, fin,
                        fin ? c->dl2 : nullptr, fin ? m : 0, fin ? c->dL2 : nullptr));
    }
    c->launches += 1;
    if (finished) *finished = fin;
    return RZ_OK;
}

// ---------------------------------------------------------------------------
// FP64 oracle: the whole computation in double (rz_fp64.cu), for RZ_MODE_FP64,
// rz_forward_f64 / rz_grad_obj_f64 and the error of float results
// ---------------------------------------------------------------------------
// Per-shot scalars for n shots and field slots for a chunk of them: all n
// when they fit the memory cap (default 90% of free memory), else fewer.
static int ensure_fp64(rz_context *c, int n, bool exact, int *chunk) {
    const size_t fs = (size_t)c->g.nx * c->g.ny;
    if (n > c->cap64s) {
        dfree(c->d64Tmod), dfree(c->d64Tres), dfree(c->d64l2), dfree(c->d64Pf), dfree(c->d64Pa), dfree(c->d64Stat);
        c->cap64s = 0;
        const size_t nt = (size_t)(c->ntr > 0 ? c->ntr : 1) * n;
        CK(dalloc(&c->d64Tmod, nt));
        CK(dalloc(&c->d64Tres, nt));
        CK(dalloc(&c->d64l2, (size_t)n));
        CK(dalloc(&c->d64Pf, (size_t)n));
        CK(dalloc(&c->d64Pa, (size_t)n));
        CK(dalloc(&c->d64Stat, (size_t)n));
        c->cap64s = n;
    }
    if (!c->d64Grad) CK(dalloc(&c->d64Grad, fs));
    if (!c->d64L2) CK(dalloc(&c->d64L2, 1));
    const size_t per = (exact ? 6 : 3) * fs * sizeof(double);
    const size_t held = (size_t)c->cap64 * (c->cap64_exact ? 6 : 3) * fs * sizeof(double);
    size_t limit = c->memcap;
    if (limit == 0) {
        size_t fr = 0, tot = 0;
        CK(cudaMemGetInfo(&fr, &tot));
        limit = (size_t)(0.9 * (double)(fr + held));
    }
    const int fit = (int)std::max<size_t>(1, std::min<size_t>(limit / per, (size_t)n));
    if (c->cap64 < std::min(n, fit) || (exact && !c->cap64_exact) || (size_t)c->cap64 * per > limit) {
        dfree(c->d64T), dfree(c->d64A), dfree(c->d64L), dfree(c->d64WX), dfree(c->d64WZ), dfree(c->d64GS);
        c->cap64 = 0;
        const int m = std::min(n, fit);
        CK(dalloc(&c->d64T, fs * m));
        CK(dalloc(&c->d64A, fs * m));
        CK(dalloc(&c->d64L, fs * m));
        if (exact) {
            CK(dalloc(&c->d64WX, fs * m));
            CK(dalloc(&c->d64WZ, fs * m));
            CK(dalloc(&c->d64GS, fs * m));
        }
        c->cap64 = m;
        c->cap64_exact = exact;
    }
    *chunk = std::min(n, c->cap64);
    return RZ_OK;
}

static void fill_fp64(const rz_context *c, F64Params &P, int first, int m) {
    memset(&P, 0, sizeof P);
    P.nx = c->g.nx, P.ny = c->g.ny, P.nxp = c->nxp;
    P.dh = c->g.dh, P.time = c->g.time, P.ttnorm = c->g.ttnorm, P.eps_adj = c->g.eps_adj;
    P.max_passes = c->g.max_passes > 0 ? c->g.max_passes : 10000;
    P.nshots = m;
    P.S = c->dS;
    P.skip = c->dSkipP;
    P.src_h = c->dSrcH + first, P.src_k = c->dSrcK + first;
    P.ntr = c->ntr;
    P.rec_h = c->dRecH, P.rec_k = c->dRecK;
    P.nrcell = c->nrcell, P.rcell_h = c->dRcH, P.rcell_k = c->dRcK, P.rcell_rec = c->dRcRec;
    P.nxcell = c->nxcell, P.xcell_h = c->dXcH, P.xcell_k = c->dXcK, P.xcell_off = c->dXcOff, P.xcell_rec = c->dXcRec;
    P.Tobs = c->dTobs + (size_t)first * c->ntr;
    P.T = c->d64T, P.A = c->d64A, P.L = c->d64L, P.WX = c->d64WX, P.WZ = c->d64WZ, P.GS = c->d64GS;
    P.Tmod = c->d64Tmod + (size_t)first * c->ntr;
    P.Tres = c->d64Tres + (size_t)first * c->ntr;
    P.l2 = c->d64l2 + first;
    P.passes_fwd = c->d64Pf + first, P.passes_adj = c->d64Pa + first, P.status = c->d64Stat + first;
    P.fstride = (size_t)c->g.nx * c->g.ny;
}

// The FP64 computation over the n shots whose sources (and picks, for
// residual) are already on the device.  After each chunk's launch,
// on_chunk(first, m) sees the double traveltimes of shots first..first+m-1
// in the slots.  adjoint: gradient into d64Grad, misfit into d64L2 (also for
// residual alone).  fixpoint: the forward runs to the fixpoint of the
// discrete equations instead of stopping at TTNORM.  Returns the status of
// the shots.
template <class F>
static int run_fp64(rz_context *c, int n, bool adjoint, bool residual, bool exact, bool cotangent, F &&on_chunk,
                    bool fixpoint = false) {
    int chunk = 0, r;
    if ((r = ensure_fp64(c, n, adjoint && exact, &chunk))) return r;
    if (!c->rec_set && (r = rz_set_receivers(c, 0, nullptr, nullptr))) return r;
    CK(cudaMemsetAsync(c->d64Stat, 0, n * sizeof(int), c->st));
    for (int first = 0; first < n; first += chunk) {
        const int m = std::min(chunk, n - first);
        F64Params P;
        fill_fp64(c, P, first, m);
        P.do_residual = residual ? 1 : 0;
        P.do_adjoint = adjoint ? 1 : 0;
        P.exact = exact ? 1 : 0;
        P.cotangent = cotangent ? 1 : 0;
        P.fixpoint = fixpoint ? 1 : 0;
        CK(launch_fp64_shots(P, c->st));
        c->launches += 1;
        if ((r = on_chunk(first, m))) return r;
        if (adjoint) {
            CK(launch_fp64_stack(P, c->d64Grad, first > 0, c->st));
            c->launches += 1;
        }
    }
    const long ncell = (long)c->g.nx * c->g.ny;
    if (adjoint && exact) CK(launch_fp64_vp_scale(c->dS, ncell, c->d64Grad, c->st));
    if (adjoint && !exact) CK(launch_cp_frame(nullptr, c->d64Grad, c->g.nx, c->g.ny, c->g.nx, 1, c->st));
    if (residual) CK(launch_sum_l2(c->d64l2, n, c->d64L2, c->st));
    c->launches += (adjoint ? 1 : 0) + (residual ? 1 : 0);
    std::vector<int> st(n);
    CK(cudaMemcpyAsync(st.data(), c->d64Stat, n * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    int worst = 0;
    for (int v : st) worst |= v;
    const int code = status_to_code(worst);
    if (code != RZ_OK) return fail(c, code, "FP64 oracle: device status bits 0x%x", worst);
    return RZ_OK;
}

static int no_chunk_work(int, int) { return RZ_OK; }

static int ensure_cmp(rz_context *c, int entries) {
    if (entries > c->ncmp) {
        CK(dalloc(&c->dCmp, (size_t)4 * entries));
        c->ncmp = entries;
    }
    CK(cudaMemsetAsync(c->dCmp, 0, sizeof(double) * 4 * entries, c->st));
    return RZ_OK;
}

// Error of the float results of the last call against the FP64 oracle on the
// same inputs.  what: 0 forward (traveltimes, picks), 1 gradient (also the
// gradient and misfit), 2 misfit (picks and misfit).  Traveltimes are
// compared for the shots whose float fields are still in the slots (all of
// them unless the batch ran in chunks).  A refined call is compared with the
// FP64 fixpoint of the discrete equations, which its linear solve approximates;
// an unrefined one with the FP64 run of the same algorithm, TTNORM included.
static int error_check(rz_context *c, int n, int what) {
    const bool adjoint = what == 1, residual = what != 0;
    const bool exact = adjoint && c->grad_kind == RZ_GRADIENT_EXACT;
    const int t0 = c->last_first, t1 = c->last_n, ntt = std::max(0, t1 - t0);
    const size_t fsf = (size_t)c->g.ny * c->nxp, fs64 = (size_t)c->g.nx * c->g.ny;
    int r;
    if ((r = ensure_cmp(c, ntt + 2))) return r;
    r = run_fp64(c, n, adjoint, residual, exact, false, [&](int first, int m) -> int {
        const int a = std::max(first, t0), b = std::min(first + m, t1);
        if (a < b)
            CK(launch_compare(c->dT + (size_t)(a - t0) * fsf, c->nxp, c->d64T + (size_t)(a - first) * fs64, c->g.nx,
                              c->g.nx, c->g.ny, b - a, fsf, fs64, c->dCmp + 4 * (size_t)(a - t0), c->st));
        return RZ_OK;
    }, c->refine);
    if (r) return r;
    if (c->ntr > 0)
        CK(launch_compare(c->dTmod, c->ntr, c->d64Tmod, c->ntr, c->ntr, n, 1, 0, 0, c->dCmp + 4 * (size_t)ntt, c->st));
    if (adjoint)
        CK(launch_compare(c->last_grad, c->g.nx, c->d64Grad, c->g.nx, c->g.nx, c->g.ny, 1, 0, 0,
                          c->dCmp + 4 * (size_t)(ntt + 1), c->st));
    std::vector<double> acc(4 * (size_t)(ntt + 2));
    double l2[2] = {0.0, 0.0};
    CK(cudaMemcpyAsync(acc.data(), c->dCmp, acc.size() * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    if (residual) {
        CK(cudaMemcpyAsync(&l2[0], c->dL2, sizeof(double), cudaMemcpyDeviceToHost, c->st));
        CK(cudaMemcpyAsync(&l2[1], c->d64L2, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    }
    CK(cudaStreamSynchronize(c->st));
    rz_error e;
    memset(&e, 0, sizeof e);
    e.shots = ntt;
    for (int z = 0; z < ntt; ++z) {
        const double *q = &acc[4 * (size_t)z];
        e.tt_rel = std::max(e.tt_rel, q[3] > 0 ? q[2] / q[3] : 0.0);
        e.tt_rel_l2 = std::max(e.tt_rel_l2, q[1] > 0 ? std::sqrt(q[0] / q[1]) : 0.0);
    }
    const double *q = &acc[4 * (size_t)ntt];
    e.tmod_rel = q[3] > 0 ? q[2] / q[3] : 0.0;
    q = &acc[4 * (size_t)(ntt + 1)];
    e.grad_rel_l2 = adjoint && q[1] > 0 ? std::sqrt(q[0] / q[1]) : 0.0;
    e.grad_rel_max = adjoint && q[3] > 0 ? q[2] / q[3] : 0.0;
    e.misfit_rel = residual && l2[1] != 0.0 ? std::fabs(l2[0] - l2[1]) / std::fabs(l2[1]) : 0.0;
    c->err_rep = e;
    c->err_valid = true;
    return RZ_OK;
}

// copy n doubles from the device to dst as float (dst on the device with
// dev, else host memory)
static int out_as_float(rz_context *c, const double *src, float *dst, size_t n, bool dev) {
    if (dev) {
        CK(launch_d2f(src, dst, (long)n, c->st));
        c->launches += 1;
        return RZ_OK;
    }
    std::vector<double> h(n);
    CK(cudaMemcpyAsync(h.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    for (size_t i = 0; i < n; ++i) dst[i] = (float)h[i];
    return RZ_OK;
}

// upload sources (and picks) of an FP64 call; the float slots are not touched
static int fp64_inputs(rz_context *c, int n, const float *srcx, const float *srcz, const float *Tobs, int flags) {
    int r;
    if ((r = ensure_shots(c, n))) return r;
    if ((r = set_sources(c, n, srcx, srcz))) return r;
    const size_t nt = (size_t)n * c->ntr;
    if (Tobs && nt)
        CK(cudaMemcpyAsync(c->dTobs, Tobs, nt * 4,
                           have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->st));
    return RZ_OK;
}

int rz_context_query(rz_context *c, int *nx, int *ny, float *dh, int *ntr, cudaStream_t *stream) {
    if (!c) return RZ_EINVAL;
    if (!c->grid_set) return fail(c, RZ_ESTATE, "rz_set_grid has not been called");
    cudaSetDevice(c->device);
    *nx = c->g.nx;
    *ny = c->g.ny;
    *dh = c->g.dh;
    *ntr = c->rec_set ? c->ntr : 0;
    *stream = c->st;
    return RZ_OK;
}

void rz_context_set_error(rz_context *c, const char *msg) {
    if (c) c->err = msg;
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

int rz_abi_version(void) { return RZ_ABI_VERSION; }

const char *rz_strerror(int s) {
    switch (s) {
        case RZ_OK: return "ok";
        case RZ_EINVAL: return "invalid argument";
        case RZ_ENOCONV: return "no convergence within max_passes";
        case RZ_ECUDA: return "CUDA error";
        case RZ_ENOMEM: return "out of device memory";
        case RZ_ETIMEOUT: return "device-side wait timed out";
        case RZ_ESTATE: return "call order: grid/model/receivers not set";
        case RZ_EUNSUPPORTED: return "unsupported grid shape";
        default: return "unknown status";
    }
}

int rz_create(rz_context **out, int device) {
    if (!out) return RZ_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return RZ_ECUDA;
    rz_context *c = new rz_context();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return RZ_ECUDA;
    }
    c->st = c->own;
    int coherent = 0;
    if (cudaDeviceGetAttribute(&coherent, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device) != cudaSuccess)
        coherent = 0, (void)cudaGetLastError();
    c->host_coherent = coherent != 0;
    void *h = nullptr, *d = nullptr;
    if (cudaHostAlloc(&h, sizeof(rz_context::HostWords), cudaHostAllocMapped) == cudaSuccess &&
        cudaHostGetDevicePointer(&d, h, 0) == cudaSuccess) {
        c->hw = (rz_context::HostWords *)h, c->hwDev = (rz_context::HostWords *)d;
    } else {
        if (h) cudaFreeHost(h);
        (void)cudaGetLastError();  // results are then read back by copies
    }
    *out = c;
    return RZ_OK;
}

void rz_destroy(rz_context *c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->st) cudaStreamSynchronize(c->st);
    free_batch(c);
    for (auto &pr : c->shot_events) cudaEventDestroy(pr.first), cudaEventDestroy(pr.second);
    dfree(c->dS), dfree(c->dSA), dfree(c->dSB), dfree(c->dVp), dfree(c->dCube), dfree(c->dGrad), dfree(c->dL2);
    dfree(c->dBad);
    if (c->hw) cudaFreeHost(c->hw);
    dfree(c->dSp);
    dfree(c->dRecH), dfree(c->dRecK), dfree(c->dRcH), dfree(c->dRcK), dfree(c->dRcRec), dfree(c->dSkip);
    dfree(c->dSkipP);
    dfree(c->dMA), dfree(c->dMB), dfree(c->dGrad64);
    dfree(c->dXcH), dfree(c->dXcK), dfree(c->dXcOff), dfree(c->dXcRec);
    dfree(c->dJobs), dfree(c->dCounter);
    drop_graph(c);
    if (c->own) cudaStreamDestroy(c->own);
    delete c;
}

const char *rz_last_error(const rz_context *c) { return c ? c->err.c_str() : "no context"; }

int rz_set_stream(rz_context *c, void *stream) {
    if (!c) return RZ_EINVAL;
    c->st = stream ? (cudaStream_t)stream : c->own;
    return RZ_OK;
}

int rz_set_mode(rz_context *c, int mode) {
    if (!c) return RZ_EINVAL;
    if (mode != RZ_MODE_REFERENCE && mode != RZ_MODE_FAST && mode != RZ_MODE_FP64)
        return fail(c, RZ_EINVAL, "unknown mode %d", mode);
    c->mode = mode;
    return RZ_OK;
}

int rz_set_grid(rz_context *c, const rz_grid *g) {
    if (!c || !g) return RZ_EINVAL;
    if (g->nx < 3 || g->ny < 3) return fail(c, RZ_EINVAL, "grid %d x %d: NX and NY must be >= 3", g->nx, g->ny);
    if (!(g->dh > 0.f) || !std::isfinite(g->dh)) return fail(c, RZ_EINVAL, "DH must be > 0");
    if (!(g->ttnorm > 0.f))
        return fail(c, RZ_EINVAL, "TTNORM must be > 0 (the reference never terminates otherwise)");
    if (!std::isfinite(g->time) || !std::isfinite(g->eps_adj)) return fail(c, RZ_EINVAL, "TIME/EPS_ADJ not finite");
    const int nstrips = (g->ny + kStrip - 1) / kStrip;
    cudaSetDevice(c->device);
    const bool same_shape = c->grid_set && c->g.nx == g->nx && c->g.ny == g->ny;
    c->g = *g;
    c->grid_set = true;
    if (!same_shape) {
        c->nxb = (g->nx + kBlk - 1) / kBlk;
        c->nxp = c->nxb * kBlk;
        c->nstrips = nstrips;
        c->qn = skew_lines(c->nxb);
        free_batch(c);
        dfree(c->dCube);
        c->model_set = false;
        c->rec_set = false;
        c->cube_valid = false;
    }
    return RZ_OK;
}

// The device address of pinned host memory at p when the device reads host
// memory coherently (Grace's C2C link): a kernel then reads the caller's
// buffer directly instead of a staging copy.  Null otherwise.
static const float *coherent_host(const rz_context *c, const float *p) {
    if (!c->host_coherent) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost && a.devicePointer ? (const float *)a.devicePointer : nullptr;
}

// src: the velocity (is_vp) or slowness on the device, or pinned host memory
// from coherent_host; one preparation launch, the skewed copies, one wait
static int set_model_common(rz_context *c, const float *src, bool is_vp) {
    const int nx = c->g.nx, ny = c->g.ny;
    const size_t skew = (size_t)c->nstrips * c->qn * 32;
    if (!c->dSA) {
        CK(dalloc(&c->dSA, skew));
        CK(dalloc(&c->dSB, skew));
    }
    CK(launch_prep_model(src, is_vp, c->dS, c->dSp, nx, ny, c->nxp, c->dBad, c->st));
    // the skew launch hands the check's result to pinned host memory
    CK(launch_skew_field(c->dS, nx, ny, nx, c->nstrips, c->nxb, c->dSA, c->dSB, c->st, c->dBad,
                         c->hw ? &c->hwDev->bad : nullptr));
    int bad = kModelOk;
    if (!c->hw) CK(cudaMemcpyAsync(&bad, c->dBad, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (c->hw) bad = *(volatile int *)&c->hw->bad;
    if (bad != kModelOk) {
        c->model_set = false;
        return fail(c, RZ_EINVAL, "slowness at cell %d is not a positive finite number", bad);
    }
    c->model_set = true;
    c->cube_valid = false;
    return RZ_OK;
}

static int alloc_model(rz_context *c) {
    const size_t n = (size_t)c->g.nx * c->g.ny;
    if (!c->dS) CK(dalloc(&c->dS, n));
    if (!c->dBad) CK(dalloc(&c->dBad, 1));
    if (!c->dSp) {
        CK(dalloc(&c->dSp, (size_t)c->g.ny * c->nxp));
        CK(cudaMemsetAsync(c->dSp, 0, (size_t)c->g.ny * c->nxp * 4, c->st));
        int r;
        if ((r = make_map(c, &c->maps.schk, c->dSp, 1, 128, kCheckBoxRows))) return r;
    }
    return RZ_OK;
}

int rz_set_slowness(rz_context *c, const float *S, int flags) {
    if (!c || !S) return RZ_EINVAL;
    if (!c->grid_set) return fail(c, RZ_ESTATE, "rz_set_grid first");
    cudaSetDevice(c->device);
    // allocations follow the grid; they are dropped when the shape changes
    if (c->dS && !c->model_set) {
        dfree(c->dS), dfree(c->dSA), dfree(c->dSB), dfree(c->dSp);
    }
    int r;
    if ((r = alloc_model(c))) return r;
    const size_t n = (size_t)c->g.nx * c->g.ny;
    const float *src = S;
    if (!have_dev(flags) && !(src = coherent_host(c, S))) {
        CK(cudaMemcpyAsync(c->dS, S, n * 4, cudaMemcpyHostToDevice, c->st));
        src = c->dS;
    }
    return set_model_common(c, src, false);
}

int rz_set_velocity(rz_context *c, const float *vp, int flags) {
    if (!c || !vp) return RZ_EINVAL;
    if (!c->grid_set) return fail(c, RZ_ESTATE, "rz_set_grid first");
    cudaSetDevice(c->device);
    if (c->dS && !c->model_set) {
        dfree(c->dS), dfree(c->dSA), dfree(c->dSB), dfree(c->dSp), dfree(c->dVp);
    }
    int r;
    if ((r = alloc_model(c))) return r;
    const size_t n = (size_t)c->g.nx * c->g.ny;
    const float *src = vp;
    if (!have_dev(flags) && !(src = coherent_host(c, vp))) {
        if (!c->dVp) CK(dalloc(&c->dVp, n));
        CK(cudaMemcpyAsync(c->dVp, vp, n * 4, cudaMemcpyHostToDevice, c->st));
        src = c->dVp;
    }
    return set_model_common(c, src, true);
}

int rz_set_receivers(rz_context *c, int ntr, const int *recx, const int *recz) {
    if (!c) return RZ_EINVAL;
    if (!c->grid_set) return fail(c, RZ_ESTATE, "rz_set_grid first");
    if (ntr < 0 || (ntr > 0 && (!recx || !recz))) return fail(c, RZ_EINVAL, "bad receiver arrays");
    cudaSetDevice(c->device);
    const int nx = c->g.nx, ny = c->g.ny;
    std::vector<int> hh(ntr), kk(ntr);
    std::vector<uint8_t> skip((size_t)nx * ny, 0);
    std::map<long, int> last;  // interior receiver cell -> last receiver index
    for (int i = 0; i < ntr; ++i) {
        if (recx[i] < 1 || recx[i] > nx || recz[i] < 1 || recz[i] > ny)
            return fail(c, RZ_EINVAL, "receiver %d at grid index (%d, %d) outside 1..%d x 1..%d", i + 1, recx[i],
                        recz[i], nx, ny);
        hh[i] = recx[i] - 1;
        kk[i] = recz[i] - 1;
        skip[(size_t)kk[i] * nx + hh[i]] = 1;
        if (hh[i] > 0 && hh[i] < nx - 1 && kk[i] > 0 && kk[i] < ny - 1) last[(long)kk[i] * nx + hh[i]] = i;
    }
    std::vector<int> rh, rk, rr;
    for (auto &kv : last) {
        rk.push_back((int)(kv.first / nx));
        rh.push_back((int)(kv.first % nx));
        rr.push_back(kv.second);
    }
    // every receiver cell with its receivers in index order (exact adjoint)
    std::map<long, std::vector<int>> cells;
    for (int i = 0; i < ntr; ++i) cells[(long)kk[i] * nx + hh[i]].push_back(i);
    std::vector<int> xh, xk, xoff(1, 0), xrec;
    for (auto &kv : cells) {
        xk.push_back((int)(kv.first / nx));
        xh.push_back((int)(kv.first % nx));
        for (int i : kv.second) xrec.push_back(i);
        xoff.push_back((int)xrec.size());
    }
    c->ntr = ntr;
    c->nrcell = (int)rr.size();
    CK(dalloc(&c->dRecH, (size_t)ntr));
    CK(dalloc(&c->dRecK, (size_t)ntr));
    CK(dalloc(&c->dRcH, rr.size()));
    CK(dalloc(&c->dRcK, rr.size()));
    CK(dalloc(&c->dRcRec, rr.size()));
    CK(dalloc(&c->dSkip, skip.size()));
    if (ntr) {
        CK(cudaMemcpyAsync(c->dRecH, hh.data(), ntr * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(c->dRecK, kk.data(), ntr * sizeof(int), cudaMemcpyHostToDevice, c->st));
    }
    if (!rr.empty()) {
        CK(cudaMemcpyAsync(c->dRcH, rh.data(), rr.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(c->dRcK, rk.data(), rr.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(c->dRcRec, rr.data(), rr.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
    }
    c->nxcell = (int)xh.size();
    CK(dalloc(&c->dXcH, xh.size()));
    CK(dalloc(&c->dXcK, xk.size()));
    CK(dalloc(&c->dXcOff, xoff.size()));
    CK(dalloc(&c->dXcRec, xrec.size()));
    if (!xh.empty()) {
        CK(cudaMemcpyAsync(c->dXcH, xh.data(), xh.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(c->dXcK, xk.data(), xk.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
        CK(cudaMemcpyAsync(c->dXcRec, xrec.data(), xrec.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
    }
    CK(cudaMemcpyAsync(c->dXcOff, xoff.data(), xoff.size() * sizeof(int), cudaMemcpyHostToDevice, c->st));
    CK(cudaMemcpyAsync(c->dSkip, skip.data(), skip.size(), cudaMemcpyHostToDevice, c->st));
    {
        std::vector<uint8_t> sp((size_t)ny * c->nxp, 1);
        for (int k = 1; k < ny - 1; ++k)
            for (int h = 1; h < nx - 1; ++h) sp[(size_t)k * c->nxp + h] = skip[(size_t)k * nx + h];
        CK(dalloc(&c->dSkipP, sp.size()));
        CK(cudaMemcpyAsync(c->dSkipP, sp.data(), sp.size(), cudaMemcpyHostToDevice, c->st));
        CK(cudaStreamSynchronize(c->st));
    }
    const size_t lines = (size_t)c->nstrips * c->qn;
    CK(dalloc(&c->dMA, lines));
    CK(dalloc(&c->dMB, lines));
    CK(launch_skip_masks(c->dSkip, nx, ny, c->nstrips, c->nxb, c->dMA, c->dMB, c->st));
    CK(cudaStreamSynchronize(c->st));
    free_shots(c);  // receiver-sized buffers follow ntr
    c->rec_set = true;
    return RZ_OK;
}

int rz_set_memory_cap(rz_context *c, size_t bytes) {
    if (!c) return RZ_EINVAL;
    c->memcap = bytes;
    if (bytes && c->cap_f && slot_bytes(c) * (size_t)c->cap_f > bytes) {
        cudaSetDevice(c->device);
        cudaStreamSynchronize(c->st);
        free_fields(c);
    }
    return RZ_OK;
}

static int forward_impl(rz_context *c, int nshots, const float *srcx, const float *srcz, float *TT, float *Tmod,
                        int *passes, int flags) {
    int r;
    if ((r = ready(c, false))) return r;
    if (nshots < 1) return fail(c, RZ_EINVAL, "nshots must be >= 1");
    cudaSetDevice(c->device);
    if (!c->rec_set) {
        if ((r = rz_set_receivers(c, 0, nullptr, nullptr))) return r;
    }
    int chunk = 0;
    if ((r = ensure_shots(c, nshots))) return r;
    if ((r = plan_chunks(c, nshots, &chunk))) return r;
    if ((r = set_sources(c, nshots, srcx, srcz))) return r;
    if ((r = reset_shots(c, nshots))) return r;
    const size_t fpts = (size_t)c->g.nx * c->g.ny;
    for (int first = 0; first < nshots; first += chunk) {
        const int m = nshots - first < chunk ? nshots - first : chunk;
        if ((r = run_batch(c, first, m, false, false, false))) return r;
        if (TT && (r = copy_out_fields(c, c->dT, TT + (size_t)first * fpts, m, flags))) return r;
    }
    if (Tmod && c->ntr > 0)
        CK(cudaMemcpyAsync(Tmod, c->dTmod, (size_t)nshots * c->ntr * 4,
                           have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
    if (passes) CK(cudaMemcpyAsync(passes, c->dPf, nshots * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    if (have_dev(flags) && !passes) return RZ_OK;
    return collect_status(c, nshots);
}

static int grad_obj_impl(rz_context *c, int nshots, const float *srcx, const float *srcz, const float *Tobs,
                         float *grad, double *L2, int flags) {
    int r;
    if ((r = ready(c, true))) return r;
    if (nshots < 1 || !Tobs || !grad) return fail(c, RZ_EINVAL, "bad arguments");
    cudaSetDevice(c->device);
    int chunk = 0;
    if ((r = ensure_shots(c, nshots))) return r;
    if ((r = plan_chunks(c, nshots, &chunk))) return r;
    if ((r = set_sources(c, nshots, srcx, srcz))) return r;
    if (c->mode == RZ_MODE_REFERENCE && (r = ensure_cube(c))) return r;
    const size_t nt = (size_t)nshots * c->ntr;
    if (nt) CK(cudaMemcpyAsync(c->dTobs, Tobs, nt * 4, have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->st));
    float *gdst = grad;
    if (!have_dev(flags)) {
        if (!c->dGrad) CK(dalloc(&c->dGrad, (size_t)c->g.nx * c->g.ny));
        gdst = c->dGrad;
    }
    c->last_grad = gdst;
    const bool exact = c->grad_kind == RZ_GRADIENT_EXACT;
    if ((c->mode == RZ_MODE_FAST || exact) && !c->dGrad64) CK(dalloc(&c->dGrad64, (size_t)c->g.nx * c->g.ny));
    if (!c->dL2) CK(dalloc(&c->dL2, 1));
    if ((r = ensure_div(c))) return r;
    if (!c->tuning) {
        auto it = c->tuned.find({nshots, c->mode, c->grad_kind});
        const rz_context::Shape sh = it != c->tuned.end() ? it->second : rz_context::Shape{0, 0, 0};
        c->warps = sh.warps, c->cta_warps = sh.cta_warps, c->check_rows = sh.check_rows;
    }
    // the device sequence: chunks in shot order, each stack continuing the
    // previous chunk's sums (the result does not depend on the chunk size)
    auto sequence = [&]() -> int {
        int q;
        if ((q = reset_shots(c, nshots))) return q;
        bool finished = false;
        for (int first = 0; first < nshots; first += chunk) {
            const int m = nshots - first < chunk ? nshots - first : chunk;
            if ((q = run_batch(c, first, m, true, true, false, exact))) return q;
            if ((q = stack_chunk(c, first, m, gdst, m == nshots, &finished))) return q;
        }
        if (finished) return RZ_OK;
        if (!exact) {
            CK(launch_cp_frame(gdst, nullptr, c->g.nx, c->g.ny, c->g.nx, 2, c->st));
            c->launches += 1;
        }
        CK(launch_sum_l2(c->dl2, nshots, c->dL2, c->st));
        c->launches += 1;
        return RZ_OK;
    };
    if (!c->use_graphs) {
        if ((r = sequence())) return r;
    } else {
        rz_context::GraphKey key;
        memset(&key, 0, sizeof key);
        fill_params(c, key.P0, 0, nshots < chunk ? nshots : chunk);
        key.nshots = nshots, key.chunk = chunk, key.mode = c->mode, key.kind = c->grad_kind, key.cap_f = c->cap_f;
        key.flags_dev = have_dev(flags), key.gdst = gdst, key.grad64 = c->dGrad64, key.cube = c->dCube;
        key.S = c->dS, key.L2 = c->dL2, key.warps = c->warps, key.cta_warps = c->cta_warps;
        if (!c->gexec || memcmp(&key, &c->gkey, sizeof key) != 0) {
            drop_graph(c);
            const size_t ev0 = c->shot_events.size();
            const long long l0 = c->launches;
            CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
            c->capturing = true;
            r = sequence();
            c->capturing = false;
            cudaGraph_t graph = nullptr;
            const cudaError_t ce = cudaStreamEndCapture(c->st, &graph);
            // the capture's events are nodes of the graph, not recorded work
            std::vector<cudaEvent_t> cap_ev;
            for (size_t i = ev0; i < c->shot_events.size(); ++i)
                cap_ev.push_back(c->shot_events[i].first), cap_ev.push_back(c->shot_events[i].second);
            c->shot_events.resize(ev0);
            c->glaunches = c->launches - l0;
            c->launches = l0;
            if (r || ce != cudaSuccess) {
                (void)cudaGetLastError();
                if (graph) cudaGraphDestroy(graph);
                for (auto e : cap_ev) cudaEventDestroy(e);
                if (r) return r;
                return fail(c, RZ_ECUDA, "stream capture failed: %s", cudaGetErrorString(ce));
            }
            c->graph = graph;  // owned from here on (drop_graph frees it)
            c->gcap_events = cap_ev;
            size_t nn = 0;
            CK(cudaGraphGetNodes(graph, nullptr, &nn));
            std::vector<cudaGraphNode_t> nodes(nn);
            CK(cudaGraphGetNodes(graph, nodes.data(), &nn));
            c->gevents.assign(cap_ev.size(), nullptr);
            for (auto nd : nodes) {
                cudaGraphNodeType t;
                CK(cudaGraphNodeGetType(nd, &t));
                if (t != cudaGraphNodeTypeEventRecord) continue;
                cudaEvent_t e;
                CK(cudaGraphEventRecordNodeGetEvent(nd, &e));
                for (size_t i = 0; i < cap_ev.size(); ++i)
                    if (cap_ev[i] == e) c->gevents[i] = nd;
            }
            const cudaError_t ie = cudaGraphInstantiate(&c->gexec, graph, 0);
            if (ie != cudaSuccess) {
                c->gexec = nullptr;
                (void)cudaGetLastError();
                drop_graph(c);
                return fail(c, RZ_ECUDA, "graph instantiation failed: %s", cudaGetErrorString(ie));
            }
            c->gkey = key;
        }
        // fresh events for this replay's shot-kernel timings; the ones they
        // replace are freed once rz_kernel_stats has read them
        std::vector<cudaEvent_t> now;
        for (size_t i = 0; i + 1 < c->gevents.size(); i += 2) {
            cudaEvent_t e0, e1;
            CK(cudaEventCreate(&e0));
            CK(cudaEventCreate(&e1));
            if (c->gevents[i]) CK(cudaGraphExecEventRecordNodeSetEvent(c->gexec, c->gevents[i], e0));
            if (c->gevents[i + 1]) CK(cudaGraphExecEventRecordNodeSetEvent(c->gexec, c->gevents[i + 1], e1));
            c->shot_events.emplace_back(e0, e1);
            now.push_back(e0), now.push_back(e1);
        }
        for (auto e : c->gcap_events) cudaEventDestroy(e);
        c->gcap_events.clear();
        for (auto e : c->ginstalled)
            if (contains(c->gretired, e)) {
                cudaEventDestroy(e);
                c->gretired.erase(std::find(c->gretired.begin(), c->gretired.end(), e));
            }
        c->ginstalled = now;
        CK(cudaGraphLaunch(c->gexec, c->st));
        c->launches += c->glaunches;
        c->last_n = nshots;
        c->last_first = nshots - ((nshots - 1) % chunk + 1);
        c->last_adj = true;
    }
    if (have_dev(flags)) {
        if (L2) CK(cudaMemcpyAsync(L2, c->dL2, sizeof(double), cudaMemcpyDeviceToDevice, c->st));
        return RZ_OK;
    }
    float *gh = c->hw ? (float *)coherent_host(c, grad) : nullptr;
    if (gh) {
        // one launch writes the gradient into the caller's pinned buffer and
        // the misfit and status words into mapped host words: no copies
        CK(launch_finish_grad(gdst, gh, (long)c->g.nx * c->g.ny, c->dL2, &c->hwDev->l2, c->dStat, nshots,
                              &c->hwDev->status, c->st));
        c->launches += 1;
        CK(cudaStreamSynchronize(c->st));
        if (L2) *L2 = *(volatile double *)&c->hw->l2;
        const int worst = *(volatile int *)&c->hw->status;
        const int code = status_to_code(worst);
        if (code != RZ_OK) return fail(c, code, "device status bits 0x%x", worst);
        return RZ_OK;
    }
    CK(cudaMemcpyAsync(grad, gdst, (size_t)c->g.nx * c->g.ny * 4, cudaMemcpyDeviceToHost, c->st));
    if (L2) CK(cudaMemcpyAsync(L2, c->dL2, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    return collect_status(c, nshots);
}

static int misfit_impl(rz_context *c, int nshots, const float *srcx, const float *srcz, const float *Tobs,
                       double *L2, int flags) {
    int r;
    if ((r = ready(c, true))) return r;
    if (nshots < 1 || !Tobs || !L2) return fail(c, RZ_EINVAL, "bad arguments");
    cudaSetDevice(c->device);
    int chunk = 0;
    if ((r = ensure_shots(c, nshots))) return r;
    if ((r = plan_chunks(c, nshots, &chunk))) return r;
    if ((r = set_sources(c, nshots, srcx, srcz))) return r;
    const size_t nt = (size_t)nshots * c->ntr;
    if (nt) CK(cudaMemcpyAsync(c->dTobs, Tobs, nt * 4, have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->st));
    if ((r = reset_shots(c, nshots))) return r;
    for (int first = 0; first < nshots; first += chunk) {
        const int m = nshots - first < chunk ? nshots - first : chunk;
        if ((r = run_batch(c, first, m, false, true, false))) return r;
    }
    if (!c->dL2) CK(dalloc(&c->dL2, 1));
    CK(launch_sum_l2(c->dl2, nshots, c->dL2, c->st));
    c->launches += 1;
    if (have_dev(flags)) {
        CK(cudaMemcpyAsync(L2, c->dL2, sizeof(double), cudaMemcpyDeviceToDevice, c->st));
        return RZ_OK;
    }
    CK(cudaMemcpyAsync(L2, c->dL2, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    return collect_status(c, nshots);
}


int rz_forward(rz_context *c, int nshots, const float *srcx, const float *srcz, float *TT, float *Tmod, int *passes,
               int flags) {
    int r;
    if (c && c->mode == RZ_MODE_FP64) {
        if ((r = ready(c, false))) return r;
        if (nshots < 1) return fail(c, RZ_EINVAL, "nshots must be >= 1");
        cudaSetDevice(c->device);
        if ((r = fp64_inputs(c, nshots, srcx, srcz, nullptr, flags))) return r;
        const size_t fs = (size_t)c->g.nx * c->g.ny;
        r = run_fp64(c, nshots, false, false, false, false, [&](int first, int m) -> int {
            return TT ? out_as_float(c, c->d64T, TT + (size_t)first * fs, (size_t)m * fs, have_dev(flags)) : RZ_OK;
        });
        if (r) return r;
        if (Tmod && c->ntr > 0 && (r = out_as_float(c, c->d64Tmod, Tmod, (size_t)nshots * c->ntr, have_dev(flags))))
            return r;
        if (passes) CK(cudaMemcpyAsync(passes, c->d64Pf, nshots * sizeof(int), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        return RZ_OK;
    }
    if ((r = forward_impl(c, nshots, srcx, srcz, TT, Tmod, passes, flags))) return r;
    return c->err_check ? error_check(c, nshots, 0) : RZ_OK;
}

int rz_grad_obj(rz_context *c, int nshots, const float *srcx, const float *srcz, const float *Tobs, float *grad,
                double *L2, int flags) {
    int r;
    if (c && c->mode == RZ_MODE_FP64) {
        if ((r = ready(c, true))) return r;
        if (nshots < 1 || !Tobs || !grad) return fail(c, RZ_EINVAL, "bad arguments");
        cudaSetDevice(c->device);
        if ((r = fp64_inputs(c, nshots, srcx, srcz, Tobs, flags))) return r;
        if ((r = run_fp64(c, nshots, true, true, c->grad_kind == RZ_GRADIENT_EXACT, false, no_chunk_work))) return r;
        if ((r = out_as_float(c, c->d64Grad, grad, (size_t)c->g.nx * c->g.ny, have_dev(flags)))) return r;
        if (L2)
            CK(cudaMemcpyAsync(L2, c->d64L2, sizeof(double),
                               have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
        if (!have_dev(flags)) CK(cudaStreamSynchronize(c->st));
        return RZ_OK;
    }
    if ((r = grad_obj_impl(c, nshots, srcx, srcz, Tobs, grad, L2, flags))) return r;
    return c->err_check ? error_check(c, nshots, 1) : RZ_OK;
}

int rz_misfit(rz_context *c, int nshots, const float *srcx, const float *srcz, const float *Tobs, double *L2,
              int flags) {
    int r;
    if (c && c->mode == RZ_MODE_FP64) {
        if ((r = ready(c, true))) return r;
        if (nshots < 1 || !Tobs || !L2) return fail(c, RZ_EINVAL, "bad arguments");
        cudaSetDevice(c->device);
        if ((r = fp64_inputs(c, nshots, srcx, srcz, Tobs, flags))) return r;
        if ((r = run_fp64(c, nshots, false, true, false, false, no_chunk_work))) return r;
        CK(cudaMemcpyAsync(L2, c->d64L2, sizeof(double),
                           have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
        if (!have_dev(flags)) CK(cudaStreamSynchronize(c->st));
        return RZ_OK;
    }
    if ((r = misfit_impl(c, nshots, srcx, srcz, Tobs, L2, flags))) return r;
    return c->err_check ? error_check(c, nshots, 2) : RZ_OK;
}

int rz_forward_f64(rz_context *c, int nshots, const float *srcx, const float *srcz, double *TT, double *Tmod,
                   int flags) {
    int r;
    if ((r = ready(c, false))) return r;
    if (nshots < 1) return fail(c, RZ_EINVAL, "nshots must be >= 1");
    cudaSetDevice(c->device);
    if ((r = fp64_inputs(c, nshots, srcx, srcz, nullptr, flags))) return r;
    const size_t fs = (size_t)c->g.nx * c->g.ny;
    const cudaMemcpyKind k = have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    r = run_fp64(c, nshots, false, false, false, false, [&](int first, int m) -> int {
        if (TT) CK(cudaMemcpyAsync(TT + (size_t)first * fs, c->d64T, (size_t)m * fs * sizeof(double), k, c->st));
        return RZ_OK;
    });
    if (r) return r;
    if (Tmod && c->ntr > 0)
        CK(cudaMemcpyAsync(Tmod, c->d64Tmod, (size_t)nshots * c->ntr * sizeof(double), k, c->st));
    CK(cudaStreamSynchronize(c->st));
    return RZ_OK;
}

int rz_grad_obj_f64(rz_context *c, int nshots, const float *srcx, const float *srcz, const float *Tobs, double *grad,
                    double *L2, int flags) {
    int r;
    if ((r = ready(c, true))) return r;
    if (nshots < 1 || !Tobs || !grad) return fail(c, RZ_EINVAL, "bad arguments");
    cudaSetDevice(c->device);
    if ((r = fp64_inputs(c, nshots, srcx, srcz, Tobs, flags))) return r;
    if ((r = run_fp64(c, nshots, true, true, c->grad_kind == RZ_GRADIENT_EXACT, false, no_chunk_work))) return r;
    const cudaMemcpyKind k = have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    CK(cudaMemcpyAsync(grad, c->d64Grad, (size_t)c->g.nx * c->g.ny * sizeof(double), k, c->st));
    if (L2) CK(cudaMemcpyAsync(L2, c->d64L2, sizeof(double), k, c->st));
    CK(cudaStreamSynchronize(c->st));
    return RZ_OK;
}

int rz_set_wait_test(rz_context *c, unsigned spin_limit, int withhold_handoff) {
    if (!c) return RZ_EINVAL;
    c->spin = spin_limit;
    c->withhold = withhold_handoff != 0;
    return RZ_OK;
}

int rz_set_refine(rz_context *c, int enable) {
    if (!c) return RZ_EINVAL;
    c->refine = enable != 0;
    return RZ_OK;
}

int rz_set_error_check(rz_context *c, int enable) {
    if (!c) return RZ_EINVAL;
    c->err_check = enable != 0;
    c->err_valid = false;
    return RZ_OK;
}

int rz_error_report(rz_context *c, rz_error *err) {
    if (!c || !err) return RZ_EINVAL;
    if (!c->err_valid) return fail(c, RZ_ESTATE, "no error report: enable rz_set_error_check before the call");
    *err = c->err_rep;
    return RZ_OK;
}

int rz_grad_obj_multi(int ngrids, rz_context *const *ctxs, const int *nshots, const float *const *srcx,
                      const float *const *srcz, const float *const *Tobs, float *const *grad, double *L2, int flags) {
    if (ngrids < 1 || ngrids > kMaxGrids || !ctxs || !nshots || !srcx || !srcz || !Tobs || !grad || !L2)
        return RZ_EINVAL;
    rz_context *c0 = ctxs[0];
    if (!c0) return RZ_EINVAL;
    rz_context *c = c0;  // error reports of the CK() checks below
    for (int i = 0; i < ngrids; ++i) {
        rz_context *c = ctxs[i];
        int r;
        if (!c) return fail(c0, RZ_EINVAL, "context %d is NULL", i);
        if ((r = ready(c, true))) return fail(c0, r, "grid %d: %s", i, c->err.c_str());
        if (c->device != c0->device || c->mode != c0->mode)
            return fail(c0, RZ_EINVAL, "grid %d: every context must use the same device and mode", i);
        if (c->mode == RZ_MODE_FP64) return fail(c0, RZ_EUNSUPPORTED, "grid %d: FP64 mode has no multi-grid launch", i);
        if (nshots[i] < 1 || !Tobs[i] || !grad[i]) return fail(c0, RZ_EINVAL, "grid %d: bad arguments", i);
        for (int k = 0; k < i; ++k)
            if (ctxs[k] == c) return fail(c0, RZ_EINVAL, "context %d appears twice", i);
    }
    cudaSetDevice(c0->device);
    cudaStream_t st = c0->st;
    // every grid's work goes on the first context's stream for this call
    std::vector<cudaStream_t> saved(ngrids);
    for (int i = 0; i < ngrids; ++i) {
        saved[i] = ctxs[i]->st;
        if (ctxs[i]->st != st) CK(cudaStreamSynchronize(ctxs[i]->st));
        ctxs[i]->st = st;
    }
    struct Restore {
        rz_context *const *c;
        std::vector<cudaStream_t> &s;
        ~Restore() {
            for (size_t i = 0; i < s.size(); ++i) c[i]->st = s[i];
        }
    } restore{ctxs, saved};

    MultiParams M;
    memset(&M, 0, sizeof M);
    M.ngrids = ngrids;
    int Wb = 1, r;
    std::vector<std::pair<long, int2>> jobs;
    for (int i = 0; i < ngrids; ++i) {
        rz_context *c = ctxs[i];
        const int n = nshots[i];
        int chunk = 0;
        if ((r = ensure_shots(c, n)) || (r = plan_chunks(c, n, &chunk))) return fail(c0, r, "%s", c->err.c_str());
        if (chunk < n)
            return fail(c0, RZ_EUNSUPPORTED, "grid %d: %d shots do not fit the memory cap in one launch", i, n);
        if ((r = set_sources(c, n, srcx[i], srcz[i]))) return fail(c0, r, "%s", c->err.c_str());
        if (c->mode == RZ_MODE_REFERENCE && (r = ensure_cube(c))) return fail(c0, r, "%s", c->err.c_str());
        if ((r = ensure_div(c))) return fail(c0, r, "%s", c->err.c_str());
        const size_t nt = (size_t)n * c->ntr;
        if (nt)
            CK(cudaMemcpyAsync(c->dTobs, Tobs[i], nt * 4, have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                               st));
        if ((r = reset_shots(c, n))) return r;
        MultiGrid &G = M.grid[i];
        fill_params(c, G.P, 0, n);
        G.P.do_residual = 1;
        G.P.do_adjoint = 1;
        G.P.exact = c->grad_kind == RZ_GRADIENT_EXACT ? 1 : 0;
        G.maps = c->maps;
        G.W = shot_kernel_warps(c->nstrips);
        Wb = std::max(Wb, G.W);
        const long cost = (long)c->g.ny * c->nxp;  // cells per shot: the larger grids go first
        for (int z = 0; z < n; ++z) jobs.push_back({cost, make_int2(i, z)});
        c->last_first = 0;
        c->last_adj = true;
    }
    std::stable_sort(jobs.begin(), jobs.end(), [](const std::pair<long, int2> &a, const std::pair<long, int2> &b) {
        return a.first > b.first;
    });
    const int nj = (int)jobs.size();
    if (nj > c0->njobs_cap) {
        CK(dalloc(&c0->dJobs, (size_t)nj));
        c0->njobs_cap = nj;
    }
    if (!c0->dCounter) CK(dalloc(&c0->dCounter, 1));
    std::vector<int2> hj(nj);
    for (int k = 0; k < nj; ++k) hj[k] = jobs[k].second;
    CK(cudaMemcpyAsync(c0->dJobs, hj.data(), sizeof(int2) * nj, cudaMemcpyHostToDevice, st));
    CK(cudaMemsetAsync(c0->dCounter, 0, sizeof(int), st));
    M.njobs = nj;
    M.counter = c0->dCounter;
    M.jobs = c0->dJobs;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    CK(cudaEventRecord(e0, st));
    CK(launch_multi_shot_kernel(M, c0->mode, Wb, nullptr, st));
    CK(cudaEventRecord(e1, st));
    c0->shot_events.emplace_back(e0, e1);
    c0->launches += 1;
    // per grid: stack, frame copy, misfit
    for (int i = 0; i < ngrids; ++i) {
        rz_context *c = ctxs[i];
        float *gdst = grad[i];
        if (!have_dev(flags)) {
            if (!c->dGrad) CK(dalloc(&c->dGrad, (size_t)c->g.nx * c->g.ny));
            gdst = c->dGrad;
        }
        const bool exact = c->grad_kind == RZ_GRADIENT_EXACT;
        if ((c->mode == RZ_MODE_FAST || exact) && !c->dGrad64) CK(dalloc(&c->dGrad64, (size_t)c->g.nx * c->g.ny));
        if (!c->dL2) CK(dalloc(&c->dL2, 1));
        bool finished = false;
        if ((r = stack_chunk(c, 0, nshots[i], gdst, true, &finished))) return fail(c0, r, "%s", c->err.c_str());
        if (!finished) {
            if (!exact) {  // the exact gradient has no frame copy (dJ/dVp of every cell)
                CK(launch_cp_frame(gdst, nullptr, c->g.nx, c->g.ny, c->g.nx, 2, st));
                c->launches += 1;
            }
            CK(launch_sum_l2(c->dl2, nshots[i], c->dL2, st));
            c->launches += 1;
        }
        CK(cudaMemcpyAsync(L2 + i, c->dL2, sizeof(double),
                           have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
        if (!have_dev(flags))
            CK(cudaMemcpyAsync(grad[i], gdst, (size_t)c->g.nx * c->g.ny * 4, cudaMemcpyDeviceToHost, st));
    }
    if (have_dev(flags)) return RZ_OK;
    for (int i = 0; i < ngrids; ++i)
        if ((r = collect_status(ctxs[i], nshots[i]))) return fail(c0, r, "grid %d: %s", i, ctxs[i]->err.c_str());
    return RZ_OK;
}

int rz_autotune(rz_context *c, int nshots, const float *srcx, const float *srcz, const float *Tobs, float *grad,
                int flags, int *best_warps, double *best_ms, int *cand_warps, double *cand_ms, int *ncand) {
    int r;
    if ((r = ready(c, true))) return r;
    if (c->mode == RZ_MODE_FP64) return fail(c, RZ_EUNSUPPORTED, "the autotuner times the float kernels only");
    if (nshots < 1 || !grad) return fail(c, RZ_EINVAL, "bad arguments");
    cudaSetDevice(c->device);
    // band widths: the balanced width for the fewest bands and one or two more bands
    const int ns = c->nstrips, nb0 = (ns + kMaxWarps - 1) / kMaxWarps;
    std::vector<int> widths;
    for (int nb = nb0; nb <= nb0 + 2 && nb <= ns; ++nb) {
        const int W = (ns + nb - 1) / nb;
        if (std::find(widths.begin(), widths.end(), W) == widths.end()) widths.push_back(W);
    }
    // shapes: band width x fixpoint-check task height x CTA width (as wide as
    // fits, or the sweeping warps alone)
    std::vector<rz_context::Shape> shapes;
    for (int W : widths)
        for (int rows : {32, 64, 128})
            for (int cta : {0, W}) shapes.push_back({W, cta, rows});
    const bool graphs = c->use_graphs;
    c->use_graphs = false;
    c->tuning = true;
    double L2 = 0.0;
    std::vector<double> ms(shapes.size(), 0.0);
    int best = 0;
    for (size_t i = 0; i < shapes.size() && !r; ++i) {
        c->warps = shapes[i].warps, c->cta_warps = shapes[i].cta_warps, c->check_rows = shapes[i].check_rows;
        cudaEvent_t e0, e1;
        r = rz_grad_obj(c, nshots, srcx, srcz, Tobs, grad, &L2, flags);  // warm
        if (!r && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess) {
            cudaEventRecord(e0, c->st);
            r = rz_grad_obj(c, nshots, srcx, srcz, Tobs, grad, &L2, flags);
            cudaEventRecord(e1, c->st);
            cudaEventSynchronize(e1);
            float t = 0.f;
            cudaEventElapsedTime(&t, e0, e1);
            ms[i] = t;
            cudaEventDestroy(e0), cudaEventDestroy(e1);
            if (ms[i] < ms[best]) best = (int)i;
        }
    }
    c->tuning = false;
    c->use_graphs = graphs;
    c->warps = 0, c->cta_warps = 0, c->check_rows = 0;
    if (r) return r;
    c->tuned[{nshots, c->mode, c->grad_kind}] = shapes[best];
    if (best_warps) *best_warps = shapes[best].warps;
    if (best_ms) *best_ms = ms[best];
    if (ncand) {
        // per band width, its fastest shape's time
        const int cap = *ncand;
        for (int i = 0; i < (int)widths.size() && i < cap; ++i) {
            double t = 0.0;
            for (size_t k = 0; k < shapes.size(); ++k)
                if (shapes[k].warps == widths[i] && (t == 0.0 || ms[k] < t)) t = ms[k];
            if (cand_warps) cand_warps[i] = widths[i];
            if (cand_ms) cand_ms[i] = t;
        }
        *ncand = (int)widths.size();
    }
    return RZ_OK;
}

int rz_tuned_shape(rz_context *c, int nshots, int *warps, int *cta_warps, int *check_rows) {
    if (!c) return RZ_EINVAL;
    auto it = c->tuned.find({nshots, c->mode, c->grad_kind});
    if (it == c->tuned.end()) return fail(c, RZ_ESTATE, "no tuned shape for %d shots in this mode", nshots);
    if (warps) *warps = it->second.warps;
    if (cta_warps) *cta_warps = it->second.cta_warps;
    if (check_rows) *check_rows = it->second.check_rows;
    return RZ_OK;
}

int rz_set_graphs(rz_context *c, int enable) {
    if (!c) return RZ_EINVAL;
    c->use_graphs = enable != 0;
    if (!c->use_graphs) {
        cudaSetDevice(c->device);
        drop_graph(c);
    }
    return RZ_OK;
}

int rz_set_gradient(rz_context *c, int kind) {
    if (!c) return RZ_EINVAL;
    if (kind != RZ_GRADIENT_REFERENCE && kind != RZ_GRADIENT_EXACT)
        return fail(c, RZ_EINVAL, "unknown gradient kind %d", kind);
    c->grad_kind = kind;
    return RZ_OK;
}

int rz_backward(rz_context *c, int nshots, const float *srcx, const float *srcz, const float *dTmod, float *grad,
                int flags) {
    int r;
    if ((r = ready(c, true))) return r;
    if (nshots < 1 || !grad || (c->ntr > 0 && !dTmod)) return fail(c, RZ_EINVAL, "bad arguments");
    cudaSetDevice(c->device);
    if (c->mode == RZ_MODE_FP64) {
        if ((r = fp64_inputs(c, nshots, srcx, srcz, dTmod, flags))) return r;
        if ((r = run_fp64(c, nshots, true, true, true, true, no_chunk_work))) return r;
        if ((r = out_as_float(c, c->d64Grad, grad, (size_t)c->g.nx * c->g.ny, have_dev(flags)))) return r;
        if (!have_dev(flags)) CK(cudaStreamSynchronize(c->st));
        return RZ_OK;
    }
    const int kind = c->grad_kind;
    c->grad_kind = RZ_GRADIENT_EXACT;  // the slots need the exact-adjoint arrays
    int chunk = 0;
    r = ensure_shots(c, nshots);
    if (!r) r = plan_chunks(c, nshots, &chunk);
    if (!r) r = set_sources(c, nshots, srcx, srcz);
    if (r) {
        c->grad_kind = kind;
        return r;
    }
    const size_t nt = (size_t)nshots * c->ntr;
    if (nt) CK(cudaMemcpyAsync(c->dTobs, dTmod, nt * 4, have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->st));
    if ((r = reset_shots(c, nshots))) return r;
    float *gdst = grad;
    if (!have_dev(flags)) {
        if (!c->dGrad) CK(dalloc(&c->dGrad, (size_t)c->g.nx * c->g.ny));
        gdst = c->dGrad;
    }
    if (!c->dGrad64) CK(dalloc(&c->dGrad64, (size_t)c->g.nx * c->g.ny));
    // the forward fields are recomputed here, chunk by chunk, from the model
    // and the source positions: nothing of an earlier rz_forward is needed
    for (int first = 0; first < nshots && !r; first += chunk) {
        const int m = nshots - first < chunk ? nshots - first : chunk;
        r = run_batch(c, first, m, true, true, false, true, true);
        if (!r) r = stack_chunk(c, first, m, gdst);
    }
    c->grad_kind = kind;
    if (r) return r;
    if (have_dev(flags)) return RZ_OK;
    CK(cudaMemcpyAsync(grad, gdst, (size_t)c->g.nx * c->g.ny * 4, cudaMemcpyDeviceToHost, c->st));
    return collect_status(c, nshots);
}

int rz_status_code(int bits) { return status_to_code(bits); }

int rz_batch_status(rz_context *c, int *bits) {
    if (!c || !bits) return RZ_EINVAL;
    cudaSetDevice(c->device);
    const int n = c->last_n;
    std::vector<int> st(n > 0 ? n : 1, 0);
    if (n > 0) CK(cudaMemcpyAsync(st.data(), c->dStat, n * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    int worst = 0;
    for (int i = 0; i < n; ++i) worst |= st[i];
    *bits = worst;
    return RZ_OK;
}

int rz_shot_info(rz_context *c, int shot, int *fwd_passes, int *adj_passes, int *status) {
    if (!c) return RZ_EINVAL;
    if (shot < 0 || shot >= c->last_n) return fail(c, RZ_EINVAL, "shot %d not in the last batch", shot);
    cudaSetDevice(c->device);
    int v[3] = {0, 0, 0};
    CK(cudaMemcpyAsync(&v[0], c->dPf + shot, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(&v[1], c->dPa + shot, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemcpyAsync(&v[2], c->dStat + shot, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (fwd_passes) *fwd_passes = v[0];
    if (adj_passes) *adj_passes = v[1];
    if (status) *status = v[2];
    return RZ_OK;
}

int rz_shot_work(rz_context *c, int shot, int *fwd_swept, int *adj_swept) {
    if (!c) return RZ_EINVAL;
    if (shot < 0 || shot >= c->last_n) return fail(c, RZ_EINVAL, "shot %d not in the last batch", shot);
    cudaSetDevice(c->device);
    int v[2] = {0, 0};
    CK(cudaMemcpyAsync(v, c->dSwept + 2 * (size_t)shot, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    if (fwd_swept) *fwd_swept = v[0];
    if (adj_swept) *adj_swept = v[1];
    return RZ_OK;
}

int rz_shot_fields(rz_context *c, int shot, float *TT, float *lam, float *Tres, int flags) {
    if (!c) return RZ_EINVAL;
    if (shot < 0 || shot >= c->last_n) return fail(c, RZ_EINVAL, "shot %d not in the last batch", shot);
    cudaSetDevice(c->device);
    const size_t fs = (size_t)c->g.ny * c->nxp;
    const int slot = shot - c->last_first;
    if ((TT || lam) && slot < 0)
        return fail(c, RZ_EINVAL, "fields of shot %d were not kept: the batch ran in chunks of %d shots", shot,
                    c->cap_f);
    int r;
    if (TT && (r = copy_out_fields(c, c->dT + slot * fs, TT, 1, flags))) return r;
    if (lam && (r = copy_out_fields(c, c->dL + slot * fs, lam, 1, flags))) return r;
    if (Tres && c->ntr)
        CK(cudaMemcpyAsync(Tres, c->dTres + (size_t)shot * c->ntr, c->ntr * 4,
                           have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return RZ_OK;
}

int rz_kernel_stats(rz_context *c, long long *launches, double *shot_kernel_ms, int *shot_kernel_calls) {
    if (!c) return RZ_EINVAL;
    cudaSetDevice(c->device);
    double tot = 0.0;
    int n = 0;
    for (auto &pr : c->shot_events) {
        CK(cudaEventSynchronize(pr.second));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, pr.first, pr.second));
        tot += ms;
        ++n;
        for (cudaEvent_t e : {pr.first, pr.second}) {
            if (contains(c->ginstalled, e)) c->gretired.push_back(e);  // a graph node still holds it
            else cudaEventDestroy(e);
        }
    }
    c->shot_events.clear();
    if (launches) *launches = c->launches;
    if (shot_kernel_ms) *shot_kernel_ms = tot;
    if (shot_kernel_calls) *shot_kernel_calls = n;
    return RZ_OK;
}

int rz_shot_timeline(rz_context *c, int shot, unsigned long long *stamps) {
    if (!c || !stamps) return RZ_EINVAL;
    if (shot < 0 || shot >= c->last_n) return fail(c, RZ_EINVAL, "shot %d not in the last batch", shot);
    cudaSetDevice(c->device);
    CK(cudaMemcpyAsync(stamps, c->dTl + (size_t)shot * kTimelineSlots, kTimelineSlots * sizeof(unsigned long long),
                       cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return RZ_OK;
}

int rz_eikonal(rz_context *c, float srcx, float srcz, float *TT, float *Tmod, int *passes, int flags) {
    return rz_forward(c, 1, &srcx, &srcz, TT, Tmod, passes, flags);
}

int rz_eikonal_adj(rz_context *c, const float *TT, const float *Tres, float *lam, int *passes, int flags) {
    int r;
    if ((r = ready(c, true))) return r;
    if (c->mode == RZ_MODE_FP64) return fail(c, RZ_EUNSUPPORTED, "eikonal_adj takes float traveltimes; use rz_grad_obj");
    if (!TT || !lam || (c->ntr > 0 && !Tres)) return fail(c, RZ_EINVAL, "bad arguments");
    cudaSetDevice(c->device);
    if ((r = ensure_shots(c, 1)) || (r = ensure_fields(c, 1))) return r;
    const cudaMemcpyKind kin = have_dev(flags) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    CK(cudaMemcpy2DAsync(c->dT, (size_t)c->nxp * 4, TT, (size_t)c->g.nx * 4, (size_t)c->g.nx * 4, c->g.ny, kin, c->st));
    if (c->ntr) CK(cudaMemcpyAsync(c->dTres, Tres, c->ntr * 4, kin, c->st));
    if ((r = reset_shots(c, 1))) return r;
    if ((r = run_batch(c, 0, 1, true, false, true))) return r;
    if ((r = copy_out_fields(c, c->dL, lam, 1, flags))) return r;
    if (passes) CK(cudaMemcpyAsync(passes, c->dPa, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    return collect_status(c, 1);
}

}  // extern "C"
