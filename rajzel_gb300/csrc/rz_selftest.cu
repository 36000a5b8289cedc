// rz_selftest.cu -- device self-tests of the point-update arithmetic and of
// the gradient stack's shot sum, built into librz_selftest.so for the GPU
// test-suite only.
//
// rz_selftest_godunov draws n seeded random update inputs (neighbour minima
// a, b within a few cell-times of each other, slowness 1/6000..1/1400 s/m,
// DH from the workload set) and compares the certified float-float evaluation
// of the reference's double branch (godunov_ref) with a direct evaluation of
// that branch in double.  Any mismatch is a defect.
//
// rz_selftest_div_tiny compares the divisions of tiny numerators (below
// 2^-96, down to the smallest subnormal; quotients normal and subnormal) with
// IEEE division bit for bit: DivDH::checked for a given DH (after the
// exhaustive check of Markstein's division for that DH that the engine runs
// before using it) and div_rn_tiny_scaled for divisors spread log-uniformly
// over [1e-9, 1e3].
#include <cuda_runtime.h>

#include "rz_device.cuh"

namespace {

__device__ __forceinline__ uint32_t mix(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return (uint32_t)x;
}
__device__ __forceinline__ float unif(uint64_t seed, uint64_t i, int k) {
    return (mix(seed * 0x9E3779B97F4A7C15ULL + i * 8 + k) >> 8) * (1.0f / 16777216.0f);
}

__global__ void godunov_check(uint64_t seed, long n, unsigned long long *bad, unsigned long long *slow) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float dhs[4] = {5.0f, 10.0f, 12.5f, 20.0f};
    const float dh = dhs[mix(seed + 17 * i) & 3];
    const float s = 1.0f / (1400.0f + 4600.0f * unif(seed, i, 0));
    const float sh = s * dh;
    const float a = 40.0f * unif(seed, i, 1);
    // b within [-1.2 sh, 1.2 sh] of a to exercise both branches
    float b = a + sh * (2.4f * unif(seed, i, 2) - 1.2f);
    if (b < 0.f) b = 0.f;
    const float got = rz::godunov_ref(a, b, s, dh);
    float want;
    const float d = __fsub_rn(a, b);
    if (fabsf(d) >= __fmul_rn(s, dh)) want = __fadd_rn(fminf(a, b), __fmul_rn(s, dh));
    else want = rz::godunov_branch2_f64(__fadd_rn(a, b), d, s, dh);
    if (__float_as_uint(got) != __float_as_uint(want)) atomicAdd(bad, 1ull);
    (void)slow;
}

}  // namespace

extern "C" int rz_selftest_godunov(unsigned long long seed, long n, unsigned long long *bad_out) {
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return 3;
    cudaMemset(d, 0, 2 * sizeof(unsigned long long));
    godunov_check<<<(unsigned)((n + 255) / 256), 256>>>(seed, n, d, d + 1);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h[2] = {0, 0};
    cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return 3;
    *bad_out = h[0];
    return 0;
}

namespace {

__global__ void shot_sum_check(const float *vals, long ncells, int nshots, double *out) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    out[c] = rz::shot_sum_fixed(vals + c, (size_t)ncells, nshots);
}

}  // namespace

// rz_selftest_shot_sum: out[c] = shot_sum_fixed over vals[z * ncells + c],
// z < nshots, for host arrays vals [nshots][ncells] and out [ncells].
extern "C" int rz_selftest_shot_sum(const float *vals, long ncells, int nshots, double *out) {
    if (ncells <= 0 || nshots < 0) return 1;
    float *dv = nullptr;
    double *dout = nullptr;
    const size_t nv = (size_t)ncells * (size_t)(nshots > 0 ? nshots : 1);
    if (cudaMalloc(&dv, nv * sizeof(float)) != cudaSuccess) return 3;
    if (cudaMalloc(&dout, (size_t)ncells * sizeof(double)) != cudaSuccess) {
        cudaFree(dv);
        return 3;
    }
    cudaError_t e = cudaSuccess;
    if (nshots > 0) e = cudaMemcpy(dv, vals, (size_t)ncells * nshots * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        shot_sum_check<<<(unsigned)((ncells + 255) / 256), 256>>>(dv, ncells, nshots, dout);
        e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, (size_t)ncells * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dv);
    cudaFree(dout);
    return e == cudaSuccess ? 0 : 3;
}

namespace {

__global__ void weights_check(const float *wx, const float *wz, long n, float *ox, float *oz, float *packed) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    rz::ExactCoef c{wx[i], wz[i], 0.f};
    const float p = rz::pack_weights(c);
    rz::unpack_weights(p, ox[i], oz[i]);
    packed[i] = p;
}

}  // namespace

// rz_selftest_weights: the exact adjoint's packed weight stream, round trip.
// For host arrays wx, wz [n] of one cell's signed weights (|wx| + |wz| = 1,
// or both 0), returns the unpacked weights ox, oz and the packed floats.
extern "C" int rz_selftest_weights(const float *wx, const float *wz, long n, float *ox, float *oz, float *packed) {
    if (n <= 0) return 1;
    float *d = nullptr;
    if (cudaMalloc(&d, 5 * (size_t)n * sizeof(float)) != cudaSuccess) return 3;
    cudaError_t e = cudaMemcpy(d, wx, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, wz, n * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        weights_check<<<(unsigned)((n + 255) / 256), 256>>>(d, d + n, n, d + 2 * n, d + 3 * n, d + 4 * n);
        e = cudaDeviceSynchronize();
    }
    if (e == cudaSuccess) e = cudaMemcpy(ox, d + 2 * n, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(oz, d + 3 * n, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(packed, d + 4 * n, n * sizeof(float), cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? 0 : 3;
}

namespace {

__global__ void div_check_dh(float dh, float rcp, unsigned long long *bad) {
    const unsigned int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= (1u << 23)) return;
    const float x = __uint_as_float(0x3f800000u | m);
    if (__float_as_uint(rz::DivDH{dh, rcp, true}.markstein(x)) != __float_as_uint(__fdiv_rn(x, dh)))
        atomicAdd(bad, 1ull);
}

// a nonzero float below 2^-96: half the draws subnormal bit patterns, half
// normal ones with exponents -126..-97
__device__ float tiny_float(uint64_t seed, uint64_t i, int k) {
    const uint32_t u = mix(seed * 0x9E3779B97F4A7C15ULL + i * 8 + k);
    const uint32_t sig = (u >> 9) & 0x7fffffu;
    uint32_t bits;
    if (u & 1u) bits = sig ? sig : 1u;
    else bits = ((1u + (mix(u) % 30u)) << 23) | sig;  // biased exponents 1..30
    return __uint_as_float(bits | ((u & 2u) << 30));
}

__global__ void div_tiny_check(uint64_t seed, long n, float dh, float rcp, unsigned long long *bad) {
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = tiny_float(seed, i, 0);
    const rz::DivDH d{dh, rcp, true};
    if (__float_as_uint(d.checked(x)) != __float_as_uint(__fdiv_rn(x, dh))) atomicAdd(bad, 1ull);
    const float a = tiny_float(seed, i, 1);
    const float b = exp2f(-29.9f + 39.9f * unif(seed, i, 2));  // ~1e-9 .. ~1e3
    if (__float_as_uint(rz::div_rn_tiny_scaled(a, b)) != __float_as_uint(__fdiv_rn(a, b))) atomicAdd(bad + 1, 1ull);
}

}  // namespace

// bad_out[0]: DivDH::checked mismatches, [1]: div_rn_tiny_scaled mismatches.
// Returns 4 when Markstein's division is not exact for this DH (the engine
// then uses IEEE division; nothing to test).
extern "C" int rz_selftest_div_tiny(unsigned long long seed, long n, float dh, unsigned long long *bad_out) {
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return 3;
    cudaMemset(d, 0, 3 * sizeof(unsigned long long));
    const float rcp = (float)(1.0 / (double)dh);
    div_check_dh<<<(1u << 23) / 256, 256>>>(dh, rcp, d + 2);
    div_tiny_check<<<(unsigned)((n + 255) / 256), 256>>>(seed, n, dh, rcp, d);
    cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h[3] = {0, 0, 0};
    cudaMemcpy(h, d, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return 3;
    if (h[2]) return 4;
    bad_out[0] = h[0];
    bad_out[1] = h[1];
    return 0;
}
