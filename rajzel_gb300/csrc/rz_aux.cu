// rz_aux.cu -- per-model / per-geometry preparation and the gradient stack.
#include <algorithm>

#include "rz_device.cuh"
#include "rz_internal.h"

namespace rz {

// X[s][q][j] <- src(row 32s+j, column h) for both skew families (see
// rz_internal.h); cells outside the grid read as 0.  With note_dst, thread 0
// first copies *note_src there (a word an earlier launch on the stream wrote).
__global__ void skew_field_kernel(const float *src, int nx, int ny, int pitch, int nstrips, int qn, float *A,
                                  float *B, const int *note_src, int *note_dst) {
    if (note_dst && blockIdx.x == 0 && threadIdx.x == 0) *note_dst = *note_src;
    const int j = threadIdx.x & 31;
    const long gline = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (gline >= (long)nstrips * qn) return;
    const int s = (int)(gline / qn), qi = (int)(gline - (long)s * qn);
    const int q = qi - kSkewFront;  // skew position of stored line qi
    const long line = (long)s * qn + q;
    const int row = kStrip * s + j;
    const int ha = q - j, hb = q + j - 31;
    float va = 0.f, vb = 0.f;
    if (row < ny) {
        if (ha >= 0 && ha < nx) va = src[(size_t)row * pitch + ha];
        if (hb >= 0 && hb < nx) vb = src[(size_t)row * pitch + hb];
    }
    A[((size_t)line + kSkewFront) * 32 + j] = va;
    B[((size_t)line + kSkewFront) * 32 + j] = vb;
}

cudaError_t launch_skew_field(const float *src, int nx, int ny, int pitch, int nstrips, int nxb, float *dstA,
                              float *dstB, cudaStream_t st, const int *note_src, int *note_dst) {
    const int qn = skew_lines(nxb);
    const long lines = (long)nstrips * qn;
    const int wpb = 8;
    skew_field_kernel<<<(unsigned)((lines + wpb - 1) / wpb), 32 * wpb, 0, st>>>(src, nx, ny, pitch, nstrips, qn, dstA,
                                                                              dstB, note_src, note_dst);
    return cudaGetLastError();
}

// bit j of M[s][q]: the adjoint sweep leaves cell (row 32s+j, h) unchanged --
// outside the grid, on the frame (sweep_adj.c:26-28), or a receiver cell
// (sweep_adj.c:30).  skip[] is the per-cell receiver flag [ny][nx].
__global__ void skip_mask_kernel(const uint8_t *skip, int nx, int ny, int nstrips, int qn, uint32_t *MA,
                                 uint32_t *MB) {
    const int j = threadIdx.x & 31;
    const long line = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (line >= (long)nstrips * qn) return;
    const int s = (int)(line / qn), q = (int)(line - (long)s * qn) - kSkewFront;
    const int row = kStrip * s + j;
    auto skipped = [&](int h) -> bool {
        if (row >= ny || h < 0 || h >= nx) return true;
        if (row == 0 || row == ny - 1 || h == 0 || h == nx - 1) return true;
        return skip[(size_t)row * nx + h] != 0;
    };
    const uint32_t ba = __ballot_sync(0xffffffffu, skipped(q - j));
    const uint32_t bb = __ballot_sync(0xffffffffu, skipped(q + j - 31));
    if (j == 0) {
        MA[line] = ba;
        MB[line] = bb;
    }
}

cudaError_t launch_skip_masks(const uint8_t *skip, int nx, int ny, int nstrips, int nxb, uint32_t *MA, uint32_t *MB,
                              cudaStream_t st) {
    const int qn = skew_lines(nxb);
    const long lines = (long)nstrips * qn;
    const int wpb = 8;
    skip_mask_kernel<<<(unsigned)((lines + wpb - 1) / wpb), 32 * wpb, 0, st>>>(skip, nx, ny, nstrips, qn, MA, MB);
    return cudaGetLastError();
}

// Gradient stack over shots (ass_grad.c:20-46 summed as grad_obj.c:33-52).
// Interior cells only; frame cells stay 0 until the frame copy.
//   reference: per shot RN32(RN64(lam * cube)) with cube = pow(S,3) from the
//              host C library, summed in float in shot order
//   fast:      S^3 (double) times the shots' lam summed by shot_sum_fixed,
//              kept in double (grad64) and rounded into grad
// With `accumulate` the sums continue from grad (reference) / grad64 (fast),
// so a batch stacked chunk by chunk in shot order gives the same result
// (in fast mode up to the double roundings of the partial sums).
// With `frame` (one chunk only, nx, ny >= 5) every cell takes the stack of
// the cell nearest to it two cells inside the grid: what the frame copy
// (cp_grad_frame.c:18-49) leaves there.  With l2_out, thread 0 also writes
// 0.5 * the shot-order double sum of l2[0..nl2) (grad_obj.c:28,42,61).
__global__ void stack_kernel(const float *L, size_t fstride, int nshots, const double *cube, const float *S, int nx,
                             int ny, int nxp, int mode, float *grad, int gpitch, double *grad64, bool accumulate,
                             bool frame, const double *l2, int nl2, double *l2_out) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (l2_out && c == 0) {
        double sum = 0.0;
        for (int i = 0; i < nl2; ++i) sum = __dadd_rn(sum, l2[i]);
        *l2_out = __dmul_rn(0.5, sum);
    }
    if (c >= (long)nx * ny) return;
    int k = (int)(c / nx), h = (int)(c - (long)k * nx);
    const size_t og = (size_t)k * gpitch + h;
    if (frame) {
        k = min(max(k, 2), ny - 3);
        h = min(max(h, 2), nx - 3);
    }
    const size_t o = (size_t)k * nxp + h;
    const bool interior = (h > 0 && h < nx - 1 && k > 0 && k < ny - 1);
    if (mode == kModeReference) {
        float acc = accumulate ? grad[og] : 0.f;
        if (interior) {
            const double cb = cube[(size_t)k * nx + h];
            for (int z = 0; z < nshots; ++z) {
                const float lam = __ldg(L + (size_t)z * fstride + o);
                acc = __fadd_rn(acc, __double2float_rn(__dmul_rn((double)lam, cb)));
            }
        }
        grad[og] = acc;
    } else {
        double acc = 0.0;
        if (interior) {
            const float sv = S[(size_t)k * nx + h];
            const double cb = (double)sv * (double)sv * (double)sv;
            acc = shot_sum_fixed(L + o, fstride, nshots) * cb;
        }
        if (accumulate && grad64) acc += grad64[og];
        if (grad64) grad64[og] = acc;
        grad[og] = (float)acc;
    }
}

cudaError_t launch_stack(const float *L, size_t fstride, int nshots, const double *cube, const float *S, int nx,
                         int ny, int nxp, int mode, float *grad, int gpitch, double *grad64, bool accumulate,
                         cudaStream_t st, bool frame, const double *l2, int nl2, double *l2_out) {
    if (frame && (accumulate || nx < 5 || ny < 5)) return cudaErrorInvalidValue;
    const long n = (long)nx * ny;
    stack_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(L, fstride, nshots, cube, S, nx, ny, nxp, mode, grad,
                                                           gpitch, grad64, accumulate, frame, l2, nl2, l2_out);
    return cudaGetLastError();
}

// Exact-adjoint gradient (not in the reference): dJ/dVp of every cell,
//   -S^2 * sum over shots of mu * dG/dS,
// dG/dS from the shot's converged traveltimes (exact_coef), summed in double.
// With Tlo (refined traveltimes) dG/dS is that of T + Tlo.
__global__ void stack_exact_kernel(const float *T, const float *L, size_t fstride, int nshots, const int *src_h,
                                   const int *src_k, const float *S, int nx, int ny, int nxp, float dh, float *grad,
                                   double *grad64, bool accumulate, const float *Tlo) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nx * ny) return;
    const int k = (int)(c / nx), h = (int)(c - (long)k * nx);
    const size_t o = (size_t)k * nxp + h;
    const float s = S[c];
    double acc = 0.0;
    for (int z = 0; z < nshots; ++z) {
        const ExactCoef cf = exact_coef(T + (size_t)z * fstride, nxp, nx, ny, h, k, s, dh,
                                        h == src_h[z] && k == src_k[z], Tlo ? Tlo + (size_t)z * fstride : nullptr);
        acc += (double)__ldg(L + (size_t)z * fstride + o) * (double)cf.gs;
    }
    acc *= -((double)s * (double)s);
    if (accumulate) acc += grad64[c];
    grad64[c] = acc;
    grad[c] = (float)acc;
}

cudaError_t launch_stack_exact(const float *T, const float *L, size_t fstride, int nshots, const int *src_h,
                               const int *src_k, const float *S, int nx, int ny, int nxp, float dh, float *grad,
                               double *grad64, bool accumulate, cudaStream_t st, const float *Tlo) {
    const long n = (long)nx * ny;
    stack_exact_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(T, L, fstride, nshots, src_h, src_k, S, nx, ny,
                                                                   nxp, dh, grad, grad64, accumulate, Tlo);
    return cudaGetLastError();
}

// cp_grad_frame.c:18-49: top rows, bottom rows, left columns, right columns,
// each pass completing before the next reads it; applied `times` times.
template <typename V>
__device__ void cp_frame_pass(V *A, int nx, int ny, int nxp) {
    for (int h = threadIdx.x; h < nx; h += blockDim.x) {
        A[(size_t)1 * nxp + h] = A[(size_t)2 * nxp + h];
        A[h] = A[(size_t)1 * nxp + h];
    }
    __syncthreads();
    for (int h = threadIdx.x; h < nx; h += blockDim.x) {
        A[(size_t)(ny - 2) * nxp + h] = A[(size_t)(ny - 3) * nxp + h];
        A[(size_t)(ny - 1) * nxp + h] = A[(size_t)(ny - 2) * nxp + h];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < ny; k += blockDim.x) {
        A[(size_t)k * nxp + 1] = A[(size_t)k * nxp + 2];
        A[(size_t)k * nxp] = A[(size_t)k * nxp + 1];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < ny; k += blockDim.x) {
        A[(size_t)k * nxp + nx - 2] = A[(size_t)k * nxp + nx - 3];
        A[(size_t)k * nxp + nx - 1] = A[(size_t)k * nxp + nx - 2];
    }
    __syncthreads();
}

__global__ void cp_frame_kernel(float *A, double *A64, int nx, int ny, int nxp, int times) {
    for (int t = 0; t < times; ++t) {
        if (A) cp_frame_pass(A, nx, ny, nxp);
        if (A64) cp_frame_pass(A64, nx, ny, nxp);
    }
}

cudaError_t launch_cp_frame(float *A, double *A64, int nx, int ny, int nxp, int times, cudaStream_t st) {
    cp_frame_kernel<<<1, 1024, 0, st>>>(A, A64, nx, ny, nxp, times);
    return cudaGetLastError();
}

__global__ void copy_rows_kernel(const float *src, int sp, float *dst, int dp, int nx, int ny, size_t sb, size_t db) {
    const size_t z = blockIdx.y;
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= (long)nx * ny) return;
    const int k = (int)(c / nx), h = (int)(c - (long)k * nx);
    dst[z * db + (size_t)k * dp + h] = src[z * sb + (size_t)k * sp + h];
}

cudaError_t launch_copy_rows(const float *src, int src_pitch, float *dst, int dst_pitch, int nx, int ny,
                             size_t nbatch, size_t src_bstride, size_t dst_bstride, cudaStream_t st) {
    const long n = (long)nx * ny;
    dim3 grid((unsigned)((n + 255) / 256), (unsigned)nbatch);
    copy_rows_kernel<<<grid, 256, 0, st>>>(src, src_pitch, dst, dst_pitch, nx, ny, src_bstride, dst_bstride);
    return cudaGetLastError();
}

// Exhaustive check of Markstein's division by the constant DH against IEEE
// division for every float significand in [1,2) (scaling x by a power of two
// scales every intermediate exactly, so this covers all normal x).
__global__ void check_div_kernel(float dh, float rcp, unsigned int *bad) {
    const unsigned int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= (1u << 23)) return;
    const float x = __uint_as_float(0x3f800000u | m);
    DivDH fast{dh, rcp, true};
    const float a = fast(x), b = __fdiv_rn(x, dh);
    if (__float_as_uint(a) != __float_as_uint(b)) atomicAdd(bad, 1u);
}

cudaError_t launch_check_div(float dh, float rcp, unsigned int *bad, cudaStream_t st) {
    check_div_kernel<<<(1u << 23) / 256, 256, 0, st>>>(dh, rcp, bad);
    return cudaGetLastError();
}

// Model preparation, one pass over the cells: the slowness S (calc_S.c:21:
// 1/vp in double, rounded to float; or the caller's slowness as given), its
// copy Sp in rows of nxp floats (the fixpoint checks' layout), and the index
// of the first cell whose slowness is not a positive finite number
// (atomicMin into first_bad, set to kModelOk before the launch).  src may be
// pinned host memory that the device reads directly.
__global__ void prep_model_kernel(const float *src, bool is_vp, float *S, float *Sp, int nx, long n, int nxp,
                                  int *first_bad) {
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        const float v = src[c];
        const float s = is_vp ? __double2float_rn(__drcp_rn((double)v)) : v;
        if (S != src) S[c] = s;
        const long k = c / nx;
        Sp[k * nxp + (c - k * nx)] = s;
        if (!(s > 0.f) || !isfinite(s)) atomicMin(first_bad, (int)c);
    }
}

cudaError_t launch_prep_model(const float *src, bool is_vp, float *S, float *Sp, int nx, int ny, int nxp,
                              int *first_bad, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(first_bad, 0x7f, sizeof(int), st);  // kModelOk
    if (e != cudaSuccess) return e;
    const long n = (long)nx * ny;
    const long blocks = std::min((n + 255) / 256, 152L * 8);
    prep_model_kernel<<<(unsigned)std::max(blocks, 1L), 256, 0, st>>>(src, is_vp, S, Sp, nx, n, nxp, first_bad);
    return cudaGetLastError();
}

// The end of a gradient call into host memory the device writes directly:
// the n-float gradient g into gout, and from block 0 the misfit and the OR of
// the nshots status words into mapped host words.
__global__ void finish_grad_kernel(const float *g, float *gout, long n, const double *l2, double *l2_out,
                                   const int *status, int nshots, int *status_out) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        gout[i] = g[i];
    if (blockIdx.x != 0) return;
    __shared__ int worst;
    if (threadIdx.x == 0) worst = 0;
    __syncthreads();
    int v = 0;
    for (int i = threadIdx.x; i < nshots; i += blockDim.x) v |= status[i];
    if (v) atomicOr(&worst, v);
    __syncthreads();
    if (threadIdx.x == 0) {
        *status_out = worst;
        *l2_out = *l2;
    }
}

cudaError_t launch_finish_grad(const float *g, float *gout, long n, const double *l2, double *l2_out,
                               const int *status, int nshots, int *status_out, cudaStream_t st) {
    const long blocks = std::min((n + 255) / 256, 152L * 4);
    finish_grad_kernel<<<(unsigned)std::max(blocks, 1L), 256, 0, st>>>(g, gout, n, l2, l2_out, status, nshots,
                                                                         status_out);
    return cudaGetLastError();
}

__global__ void sum_l2_kernel(const double *l2, int n, double *out) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = __dadd_rn(s, l2[i]);
    *out = __dmul_rn(0.5, s);
}

cudaError_t launch_sum_l2(const double *l2, int n, double *out, cudaStream_t st) {
    sum_l2_kernel<<<1, 1, 0, st>>>(l2, n, out);
    return cudaGetLastError();
}

}  // namespace rz
