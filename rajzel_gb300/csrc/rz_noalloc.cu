// rz_noalloc.cu -- forward Eikonal for callers that cannot allocate memory.
//
// Some callers must not allocate GPU memory at all: code working inside a
// pre-sized memory pool, allocator-less embedded hosts, or a time step of a
// larger solver that has fixed its memory budget up front.  rz_eikonal_noalloc() serves them: it computes one shot's
// traveltime field with the same kernels and reference-exact arithmetic as
// rz_eikonal(), but never calls cudaMalloc, cudaFree or any allocating
// routine.  Its working space (traveltimes in a pitched layout, the pass
// snapshot, two skewed copies of the slowness, two source indices) lives in
// one file-scope __device__ array of kNoAllocFloats floats (32 MiB), which
// every GPU that loads the library holds until the process exits.  The
// slowness is checked on the device (first invalid cell in the array); an
// invalid model sets status bit ERR_BAD_MODEL and no solve runs.
//
// Rules for callers:
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make this first call
//     before any stream capture;
//   * all calls share the one array, so calls whose work overlaps on the GPU
//     race; issue them on one stream or serialise them;
//   * grids whose working space exceeds the array are rejected with
//     RZ_EUNSUPPORTED before any GPU work.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/rajzel_gb300.h"
#include "rz_internal.h"

using namespace rz;

namespace {

constexpr size_t kNoAllocFloats = size_t(8) << 20;  // 8 Mi floats = 32 MiB
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_noalloc_scratch[kNoAllocFloats];

std::mutex g_mutex;
float *g_scratch[kMaxDevices] = {nullptr};

// device address of the scratch array on the current device (looked up once)
int scratch_address(float **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RZ_ECUDA;
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return RZ_ECUDA;
        g_scratch[dev] = static_cast<float *>(p);
    }
    *out = g_scratch[dev];
    return RZ_OK;
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// the driver's tensor-map encoder, looked up once for all host threads
EncodeTiledFn encoder() {
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        else
            (void)cudaGetLastError();
    });
    return fn;
}

bool encode_field_map(CUtensorMap *m, float *base, int nx, int ny, int nxp, int box_cols, int box_rows) {
    const EncodeTiledFn fn = encoder();
    if (!fn) return false;
    cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, 1};
    cuuint64_t strides[2] = {(cuuint64_t)nxp * 4, (cuuint64_t)nxp * ny * 4};
    cuuint32_t box[3] = {(cuuint32_t)box_cols, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// the shared array keeps the previous call's contents: set what the kernel
// reads before writing it (source index, pass count, status bits)
__global__ void noalloc_prologue(int *src, int hs, int ks, int *info) {
    src[0] = hs;
    src[1] = ks;
    info[0] = 0;
    info[1] = 0;
}

}  // namespace

extern "C" int rz_eikonal_noalloc(const rz_grid *grid, const float *S, float srcx, float srcz, float *TT, int *info,
                                  void *stream) {
    if (!grid || !S || !TT || !info) return RZ_EINVAL;
    const rz_grid g = *grid;
    if (g.nx < 3 || g.ny < 3 || !(g.dh > 0.f) || !(g.ttnorm > 0.f) || !std::isfinite(g.time)) return RZ_EINVAL;
    const int nstrips = (g.ny + kStrip - 1) / kStrip;
    const int hs = (int)std::floor((double)(srcx / g.dh) + 0.5) - 1;
    const int ks = (int)std::floor((double)(srcz / g.dh) + 0.5) - 1;
    if (!std::isfinite(srcx) || !std::isfinite(srcz) || hs < 0 || hs >= g.nx || ks < 0 || ks >= g.ny)
        return RZ_EINVAL;

    // working space inside the static array (offsets keep 128-byte alignment)
    const int nxb = (g.nx + kBlk - 1) / kBlk, nxp = nxb * kBlk, qn = skew_lines(nxb);
    const size_t field = (size_t)g.ny * nxp, skew = (size_t)nstrips * qn * 32;
    const size_t need = 3 * field + 2 * skew + 32;
    if (need > kNoAllocFloats) return RZ_EUNSUPPORTED;
    float *base = nullptr;
    if (int r = scratch_address(&base)) return r;
    float *T = base, *Told = base + field, *Sp = base + 2 * field, *SA = base + 3 * field, *SB = SA + skew;
    int *src = reinterpret_cast<int *>(SB + skew);  // [0..1] source index, [2] first invalid slowness cell

    ShotMaps M;
    if (!encode_field_map(&M.tld, T, g.nx, g.ny, nxp, kBlk, kBoxRows) ||
        !encode_field_map(&M.tst, T, g.nx, g.ny, nxp, kBlk, kStrip) ||
        !encode_field_map(&M.tchk, T, g.nx, g.ny, nxp, kCheckCols, kCheckBoxRows) ||
        !encode_field_map(&M.schk, Sp, g.nx, g.ny, nxp, 128, kCheckBoxRows))
        return RZ_ECUDA;
    M.lld = M.tld;  // no adjoint here
    M.lst = M.tst;
    M.lchk = M.tchk;
    M.tlo = M.tld;

    ShotParams P;
    memset(&P, 0, sizeof P);
    P.nx = g.nx;
    P.ny = g.ny;
    P.nxp = nxp;
    P.nstrips = nstrips;
    P.nxb = nxb;
    P.qn = qn;
    P.dh = g.dh;
    P.time = g.time;
    P.ttnorm = g.ttnorm;
    P.eps_adj = g.eps_adj;
    P.dh_rcp = (float)(1.0 / (double)g.dh);
    P.max_passes = g.max_passes > 0 ? g.max_passes : 10000;
    P.nshots = 1;
    P.S = S;
    P.SA = SA;
    P.SB = SB;
    P.T = T;
    P.Told = Told;
    P.fstride = field;
    P.src_h = src;
    P.src_k = src + 1;
    P.passes_fwd = info;
    P.status = info + 1;
    P.model_bad = src + 2;

    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // the row-pitched copy of S and its first invalid cell (as rz_set_slowness
    // checks it); with S given as both source and destination nothing is
    // written to the caller's array
    if (launch_prep_model(S, false, const_cast<float *>(S), Sp, g.nx, g.ny, nxp, src + 2, st) != cudaSuccess)
        return RZ_ECUDA;
    if (launch_skew_field(S, g.nx, g.ny, g.nx, nstrips, nxb, SA, SB, st) != cudaSuccess) return RZ_ECUDA;
    noalloc_prologue<<<1, 1, 0, st>>>(src, hs, ks, info);
    if (cudaGetLastError() != cudaSuccess) return RZ_ECUDA;
    if (launch_shot_kernel(P, kModeReference, M, st) != cudaSuccess) return RZ_ECUDA;
    if (launch_copy_rows(T, nxp, TT, g.nx, g.nx, g.ny, 1, 0, 0, st) != cudaSuccess) return RZ_ECUDA;
    return RZ_OK;
}
