// rz_device.cuh -- device-side building blocks for the RAJZEL GB300 kernels:
// inline-PTX wrappers for TMA (cp.async.bulk.tensor), mbarriers, proxy fences
// and release/acquire flags, plus the point updates of the forward
// (Godunov-upwind, sweep.c:89-97) and adjoint (Leung-Qian, sweep_adj.c:33-68)
// sweeps in two arithmetic modes:
//   * reference mode: bit-identical to the reference's float/double mix;
//   * fast mode: plain FP32.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#define RZ_DEV __device__ __forceinline__

namespace rz {

// ---------------------------------------------------------------------------
// error bits written to the per-shot status word
// ---------------------------------------------------------------------------
enum : int {
    ERR_TMA_TIMEOUT = 1 << 0,    // an mbarrier wait for a TMA load gave up
    ERR_FLAG_TIMEOUT = 1 << 1,   // a warp-to-warp progress wait gave up
    ERR_NOCONV_FWD = 1 << 2,     // forward did not meet TTNORM within max passes
    ERR_NOCONV_ADJ = 1 << 3,     // adjoint did not meet TTNORM within max passes
    ERR_BAD_SOURCE = 1 << 4,     // source index outside the grid
    ERR_BAD_MODEL = 1 << 5,      // a slowness is not a positive finite number (no solve ran)
};

// Bounded waits.  Legitimate waits in these kernels last microseconds; a
// wait that exceeds its poll budget records an error bit, raises the CTA's
// abort word, and every later wait in that CTA returns at once, so a faulty
// launch still ends within about one budget per CTA.
constexpr uint32_t kSpinLimit = 1u << 21;

// ---------------------------------------------------------------------------
// shared-memory address helpers
// ---------------------------------------------------------------------------
RZ_DEV uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---------------------------------------------------------------------------
// mbarrier
// ---------------------------------------------------------------------------
RZ_DEV void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
RZ_DEV void mbar_inval(uint64_t *bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
RZ_DEV void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
RZ_DEV void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
RZ_DEV bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// predicated forms: one instruction, no branch in the caller's code
RZ_DEV void sts_if(uint32_t a, float v, bool p) {
    asm volatile("{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %2, 0;\n\t@q st.shared.f32 [%0], %1;\n\t}" ::"r"(a), "f"(v),
                 "r"((uint32_t)p));
}
RZ_DEV void sts4_if(uint32_t a, float x, float y, float z, float w, bool p) {
    asm volatile(
        "{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %5, 0;\n\t@q st.shared.v4.f32 [%0], {%1, %2, %3, %4};\n\t}" ::"r"(a),
        "f"(x), "f"(y), "f"(z), "f"(w), "r"((uint32_t)p));
}
RZ_DEV void mbar_arrive_if(uint32_t bar, bool p) {
    asm volatile(
        "{\n\t.reg .pred q;\n\tsetp.ne.u32 q, %1, 0;\n\t@q mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];\n\t}" ::"r"(
            bar),
        "r"((uint32_t)p)
        : "memory");
}

// the same operations on 32-bit shared-window addresses (kept in registers)
RZ_DEV void mbar_arrive_a(uint32_t bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
RZ_DEV bool mbar_try_wait_a(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for another warp's signal; returns false on timeout (after
// `limit` polls, raising the abort word) or at once when the CTA's abort word
// (shared memory) is up.
RZ_DEV bool mbar_wait_a(uint32_t bar, uint32_t parity, uint32_t abort_word, uint32_t limit = kSpinLimit) {
    if (mbar_try_wait_a(bar, parity)) return true;
    for (uint32_t i = 0; i < limit; ++i) {
        if (mbar_try_wait_a(bar, parity)) return true;
        int ab;
        asm volatile("ld.volatile.shared.b32 %0, [%1];" : "=r"(ab) : "r"(abort_word) : "memory");
        if (ab) return false;
    }
    asm volatile("st.volatile.shared.b32 [%0], %1;" ::"r"(abort_word), "r"(1) : "memory");
    return false;
}

// Bounded wait for a tensor copy issued by this warp.  A copy always lands,
// and a warp must not leave its copies in flight, so this wait ignores the
// abort word; false only if kSpinLimit polls pass (broken hardware).
RZ_DEV bool mbar_wait_copy(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kSpinLimit; ++i)
        if (mbar_try_wait_a(bar, parity)) return true;
    return false;
}

// ---------------------------------------------------------------------------
// fences
// ---------------------------------------------------------------------------
// make this thread's generic-proxy shared-memory writes visible to the async
// proxy (before a TMA store reads them)
RZ_DEV void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// order generic-proxy global accesses with later/earlier async-proxy (TMA)
// accesses to global memory
RZ_DEV void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// ---------------------------------------------------------------------------
// TMA: 3-D tiled tensor copies (x = column, y = row, z = shot slot)
// ---------------------------------------------------------------------------
RZ_DEV void tma_load_3d(void *smem_dst, const CUtensorMap *map, int x, int y, int z, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(smem_dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
RZ_DEV void tma_store_3d(const CUtensorMap *map, int x, int y, int z, const void *smem_src) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     (uint64_t)map),
                 "r"(x), "r"(y), "r"(z), "r"(smem_u32(smem_src))
                 : "memory");
}
// the same copies with 32-bit shared-window addresses
RZ_DEV void tma_load_3d_a(uint32_t smem_dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_dst),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}
RZ_DEV void tma_store_3d_a(const CUtensorMap *map, int x, int y, int z, uint32_t smem_src) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(
                     (uint64_t)map),
                 "r"(x), "r"(y), "r"(z), "r"(smem_src)
                 : "memory");
}
// untiled bulk copy global -> shared (16-byte aligned addresses, size a multiple of 16)
RZ_DEV void bulk_load_a(uint32_t smem_dst, const void *src, uint32_t bytes, uint32_t bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}
RZ_DEV void mbar_arrive_expect_tx_a(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
RZ_DEV void tma_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// wait until at most N committed store groups are still reading shared memory
template <int N>
RZ_DEV void tma_store_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
// wait until at most N committed store groups are still incomplete
template <int N>
RZ_DEV void tma_store_wait_all() {
    asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}
RZ_DEV void tma_prefetch_desc(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// ---------------------------------------------------------------------------
// release/acquire flags in this CTA's shared memory
// ---------------------------------------------------------------------------
RZ_DEV void st_release_smem(int *p, int v) {
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(p)), "r"(v) : "memory");
}
RZ_DEV int ld_acquire_smem(const int *p) {
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(smem_u32(p)) : "memory");
    return v;
}
// Bounded wait until *flag >= need.  Returns false on timeout or abort.
// Hand-off waits are short and frequent (a consumer warp trails its producer
// by a few dozen steps), so the first polls spin; only a long wait backs off
// with __nanosleep, whose wake-up latency is microseconds.
RZ_DEV bool wait_flag_ge(const int *flag, int need, volatile int *abort_word, uint32_t limit = kSpinLimit) {
    for (int i = 0; i < 2048; ++i)
        if (ld_acquire_smem(flag) >= need) return true;
    uint32_t ns = 32;
    for (uint32_t i = 0; i < limit; ++i) {
        __nanosleep(ns);
        if (ns < 256) ns <<= 1;
        if (ld_acquire_smem(flag) >= need) return true;
        if (*abort_word) return false;
    }
    *abort_word = 1;
    return false;
}

// read-only global load that bypasses L1 allocation rules for streaming data
RZ_DEV float ldg_nc(const float *p) { return __ldg(p); }
RZ_DEV uint32_t ldg_nc_u32(const uint32_t *p) { return __ldg(p); }

// (x >= y) ? u : v and (x > y) ? u : v as one predicated select.  The
// cells of a warp take either side; a branch would run the sides one after
// the other, which the compiler chooses when a side holds a division or a
// square root.  Comparisons with NaN are false, as in C.
RZ_DEV float sel_ge(float x, float y, float u, float v) {
    float r;
    asm("{\n\t.reg .pred p;\n\tsetp.ge.f32 p, %1, %2;\n\tselp.f32 %0, %3, %4, p;\n\t}"
        : "=f"(r)
        : "f"(x), "f"(y), "f"(u), "f"(v));
    return r;
}
RZ_DEV float sel_gt(float x, float y, float u, float v) {
    float r;
    asm("{\n\t.reg .pred p;\n\tsetp.gt.f32 p, %1, %2;\n\tselp.f32 %0, %3, %4, p;\n\t}"
        : "=f"(r)
        : "f"(x), "f"(y), "f"(u), "f"(v));
    return r;
}

// ---------------------------------------------------------------------------
// Forward point update (sweep.c:89-97)
//
// Reference arithmetic: d = a-b and sh = S*DH in float; branch 1 is float;
// branch 2 evaluates (a+b) in float and the rest in double:
//   Tt = (float)(((double)(a+b) + sqrt(2*S^2*DH^2 - d^2)) / 2).
// On GB300 double precision runs at a small fraction of the FP32 rate, so
// branch 2 is evaluated in float-float arithmetic with a certified error
// bound (about 2^-42 relative; the check uses 2^-38).  If the float-float
// value is farther than the bound from every float rounding midpoint, the
// reference's double computation (whose own error is below 2^-50) rounds to
// the same float.  Otherwise the exact double path runs; that happens for
// roughly one update in ten thousand.
// ---------------------------------------------------------------------------
// Out of line: inlined into the sweep step, its double-precision code made a
// reference-mode forward pass ~13% slower although it runs for one update in
// ten thousand.
static __device__ __noinline__ float godunov_branch2_f64(float sum, float d, float s, float dh) {
    double sd = (double)s, hd = (double)dh, dd = (double)d;
    double p = __dmul_rn(__dmul_rn(2.0, __dmul_rn(sd, sd)), __dmul_rn(hd, hd));
    double q = __dsub_rn(p, __dmul_rn(dd, dd));
    double u = __dadd_rn((double)sum, __dsqrt_rn(q));
    return __double2float_rn(__dmul_rn(u, 0.5));
}

RZ_DEV float godunov_ref(float a, float b, float s, float dh) {
    float d = __fsub_rn(a, b);
    float sh = __fmul_rn(s, dh);
    // branch 1 (|d| >= sh); branch 2 is evaluated for every cell and the
    // branch selected at the end (its float-float value is NaN or meaningless
    // where branch 1 holds, and is then not used)
    const float one_sided = __fadd_rn(fminf(a, b), sh);
    float sum = __fadd_rn(a, b);
    // S*h = sh + shl exactly
    float shl = __fmaf_rn(s, dh, -sh);
    // (S*h)^2 ~= p2 + p2l + 2*sh*shl  (shl^2 < 2^-48 relative is dropped)
    float p2 = __fmul_rn(sh, sh);
    float p2l = __fmaf_rn(sh, sh, -p2);
    float cross = __fmaf_rn(__fmul_rn(2.0f, sh), shl, p2l);
    // d^2 = d2 + d2l exactly
    float d2 = __fmul_rn(d, d);
    float d2l = __fmaf_rn(d, d, -d2);
    // D = 2*(S h)^2 - d^2 with 2*p2 >= d2 (|d| < sh): fast two-sum
    float P = __fmul_rn(2.0f, p2);
    float Dh = __fsub_rn(P, d2);
    float Dl = __fsub_rn(__fsub_rn(P, Dh), d2);
    Dl = __fadd_rn(Dl, __fsub_rn(__fmul_rn(2.0f, cross), d2l));
    // sqrt(D) ~= r0 + rl: one Newton correction on an rsqrt seed
    float rs = rsqrtf(Dh);
    float r0 = __fmul_rn(Dh, rs);
    float res = __fmaf_rn(-r0, r0, Dh);
    float rl = __fmul_rn(__fadd_rn(res, Dl), __fmul_rn(0.5f, rs));
    // u = sum + r0 + rl (two-sum on the leading terms)
    float uh = __fadd_rn(sum, r0);
    float bb = __fsub_rn(uh, sum);
    float ue = __fadd_rn(__fsub_rn(sum, __fsub_rn(uh, bb)), __fsub_rn(r0, bb));
    float ul = __fadd_rn(ue, rl);
    float z = __fadd_rn(uh, ul);
    float zr = __fadd_rn(__fsub_rn(uh, z), ul);
    // distance to the nearest rounding midpoint against the error bound; the
    // spacing below z (smaller at a power of two) is the conservative one
    float below = __fsub_rn(z, __int_as_float(__float_as_int(z) - 1));
    float tol = __fmul_rn(z, 0x1p-38f);
    bool safe = (fabsf(zr) < __fsub_rn(__fmul_rn(0.5f, below), tol)) && (Dh > 0x1p-100f) && (z < 0x1p+100f);
    if (__builtin_expect(!(fabsf(d) >= sh) && !safe, 0)) return godunov_branch2_f64(sum, d, s, dh);
    return sel_ge(fabsf(d), sh, one_sided, __fmul_rn(0.5f, z));
}

// fast mode: FP32 arithmetic throughout (error ~1 ulp per update), written
// without branches so that consecutive wavefront steps can be interleaved
RZ_DEV float godunov_fast(float a, float b, float s, float dh) {
    const float d = a - b;
    const float sh = s * dh;
    const float one_sided = fminf(a, b) + sh;
    const float q = fmaf(2.0f * sh, sh, -d * d);  // > 0 whenever it is selected
    const float two_sided = fmaf(0.5f * q, rsqrtf(q), 0.5f * (a + b));
    return fabsf(d) >= sh ? one_sided : two_sided;
}

// ---------------------------------------------------------------------------
// Adjoint point update (sweep_adj.c:33-68)
//
// All reference operations are float: differences, division by DH, the
// upwind splits (x+|x|)/2, (x-|x|)/2 (exact), lhs, rhs, rhs/lhs, fminf.
// Division by the constant DH uses Markstein's correction
//   q = x*y, r = fma(-q, DH, x), q' = fma(r, y, q),  y = RN(1/DH),
// which is correctly rounded for every x when it passes the exhaustive
// per-DH check the host runs before enabling it (rz_check_div); otherwise
// IEEE division is used.
// ---------------------------------------------------------------------------
// RN(a/b), b > 0, from qs = RN(a*2^64 / b) and its remainder rs = a*2^64 -
// qs*b (exact: the remainder of a correctly rounded quotient is representable
// when nothing underflows, true for |a*2^64| >= 2^-85).  qs*2^-64 is exact
// and equals RN(a/b) while it is normal.  For a subnormal result RN(qs*2^-64)
// rounds a second time, which can go wrong only where qs*2^-64 lies exactly
// halfway between two subnormals: every such midpoint is a 24-bit number at
// that scale, so none lies strictly between a/b and qs*2^-64.  At a midpoint
// the remainder's sign says on which side a/b lies (none: a tie, to even).
// Scaling numerators this way keeps tiny ones off IEEE division's slow path.
RZ_DEV float unscale_quotient(float qs, float rs) {
    const float q = __fmul_rn(qs, 0x1p-64f);
    const bool mid = fabsf(__fmaf_rn(q, 0x1p64f, -qs)) == 0x1p-86f;
    const float qm = __fmul_rn(__fadd_rn(qs, rs > 0.0f ? 0x1p-86f : -0x1p-86f), 0x1p-64f);
    return (mid && rs != 0.0f) ? qm : q;
}

// RN(a/b) for b > 0: a tiny numerator (|a| < 2^-96) is divided at 2^64 times
// its size (b within [2^-60, 2^40] keeps that quotient normal), any other one
// by IEEE division
RZ_DEV float div_rn_tiny_scaled(float a, float b) {
    const bool tiny = fabsf(a) < 0x1p-96f && b >= 0x1p-60f && b <= 0x1p40f;
    const float as = tiny ? __fmul_rn(a, 0x1p64f) : a;
    const float q = __fdiv_rn(as, b);
    return tiny ? unscale_quotient(q, __fmaf_rn(-q, b, as)) : q;
}

struct DivDH {
    float dh, rdh;
    bool fast;
    // numerators that are never tiny (differences of traveltimes): a zero
    // numerator may come out as +0 instead of -0, which no later operation
    // of the sweep can tell apart (no division by it, no sign test)
    RZ_DEV float operator()(float x) const { return fast ? markstein(x) : __fdiv_rn(x, dh); }
    // numerators built from lambda, which can be tiny.  The exhaustive check
    // tries every significand of x in [1,2); scaling by powers of two carries
    // it to every x whose quotient and Markstein remainder stay normal, which
    // holds for |x| >= 2^-96 (DH within [2^-20, 2^20]).  A smaller x (lambda
    // decays to tiny and subnormal values away from the rays, so such
    // numerators are common, and IEEE division of them is slow) is divided at
    // 2^64 times its size and brought back by unscale_quotient.  A zero
    // numerator gives a zero either way, at most with the other sign, which no
    // later operation tells apart.
    RZ_DEV float checked(float x) const {
        if (!fast) return __fdiv_rn(x, dh);
        const bool tiny = fabsf(x) < 0x1p-96f;
        const float xs = tiny ? __fmul_rn(x, 0x1p64f) : x;
        const float qs = markstein(xs);
        return tiny ? unscale_quotient(qs, __fmaf_rn(-qs, dh, xs)) : qs;
    }
    RZ_DEV float markstein(float x) const {
        float q = __fmul_rn(x, rdh);
        float r = __fmaf_rn(-q, dh, x);
        return __fmaf_rn(r, rdh, q);
    }
};

RZ_DEV float pos_part(float x) { return x > 0.0f ? x : 0.0f; }   // (x+|x|)/2
RZ_DEV float neg_part(float x) { return x <= 0.0f ? x : 0.0f; }  // (x-|x|)/2

// tc: TT at the cell; te/tw/ts/tn: TT at (h+1,k), (h-1,k), (h,k+1), (h,k-1)
// le/lw/ls/ln: lambda at the same neighbours; own: lambda at the cell.
RZ_DEV float leung_qian_ref(float tc, float te, float tw, float ts, float tn, float le, float lw, float ls, float ln,
                            float own, const DivDH &div, float eps_adj) {
    float ap = div(-__fsub_rn(te, tc));
    float am = div(-__fsub_rn(tc, tw));
    float bp = div(-__fsub_rn(ts, tc));
    float bm = div(-__fsub_rn(tc, tn));
    float app = pos_part(ap), apm = neg_part(ap);
    float amp = pos_part(am), amm = neg_part(am);
    float bpp = pos_part(bp), bpm = neg_part(bp);
    float bmp = pos_part(bm), bmm = neg_part(bm);
    float lhs = __fadd_rn(div(__fsub_rn(app, amm)), div(__fsub_rn(bpp, bmm)));
    float rhs = __fadd_rn(div.checked(__fsub_rn(__fmul_rn(amp, lw), __fmul_rn(apm, le))),
                          div.checked(__fsub_rn(__fmul_rn(bmp, ln), __fmul_rn(bpm, ls))));
    // rhs / lhs; a zero rhs is its own quotient (lhs > 0), sign included
    float lt = (lhs > eps_adj) ? (rhs == 0.0f ? rhs : div_rn_tiny_scaled(rhs, lhs)) : 0.0f;
    float r = fminf(own, lt);
    const float kInf = 9999999.0f;  // INF of fd.h:30
    if (tc >= kInf || ts >= kInf || tn >= kInf || te >= kInf || tw >= kInf) r = 0.0f;
    return r;
}

// Fast mode: the reference divides each difference and the sums by DH, a
// common factor 1/DH^2 of lhs and rhs that cancels in rhs/lhs; the
// differences stay unscaled and the threshold EPS_ADJ becomes EPS_ADJ*DH^2
// (lq_eps_h2).
RZ_DEV float lq_eps_h2(float eps_adj, float dh) { return eps_adj * (dh * dh); }
RZ_DEV float leung_qian_fast(float tc, float te, float tw, float ts, float tn, float le, float lw, float ls, float ln,
                             float own, float eps_h2) {
    const float ap = tc - te, am = tw - tc, bp = tc - ts, bm = tn - tc;
    const float lhs = (fmaxf(ap, 0.0f) - fminf(am, 0.0f)) + (fmaxf(bp, 0.0f) - fminf(bm, 0.0f));
    const float rhs = (fmaxf(am, 0.0f) * lw - fminf(ap, 0.0f) * le) + (fmaxf(bm, 0.0f) * ln - fminf(bp, 0.0f) * ls);
    const float lt = sel_gt(lhs, eps_h2, __fdividef(rhs, lhs), 0.0f);
    return fminf(own, lt);
}

// ---------------------------------------------------------------------------
// exact discrete adjoint: linearisation of the Godunov update at the
// converged traveltimes (not in the reference)
// ---------------------------------------------------------------------------
// Cell (h,k) with T its converged traveltime, a / b the smaller x / z
// neighbour, d = a - b, sh = S*DH.  One-sided (|d| >= sh): T = min(a,b) + sh,
// dT depends on the smaller neighbour with weight 1 and dT/dS = DH.
// Two-sided: with r = sqrt(2 sh^2 - d^2), T = (a + b + r)/2, so
//   dT/da = (r - d)/(2r),  dT/db = (r + d)/(2r),  dT/dS = S DH^2 / r,
// written without T - a or T - b, which would cancel.  The weights are
// returned signed: negative points to the lower-index neighbour (west /
// north), positive to the higher one (east / south), 0 to none.
struct ExactCoef {
    float wx, wz, gs;
};

// A cell's two weights in one float, for the skewed weight streams.  Every
// cell with an upwind neighbour has |wx| + |wz| = 1 (one-sided: 1 and 0;
// two-sided: (r-d)/2r and (r+d)/2r), so the smaller magnitude is stored and
// the larger is 1 minus it: the sign bit is the x direction (set: west),
// significand bit 0 the z direction (set: south), bit 1 whether the stored
// magnitude is |wz|; those two bits cost at most 3 ulp of the smaller weight.
// 2.0 marks a cell with no upwind neighbour (the source, cells outside the
// grid).
RZ_DEV float pack_weights(const ExactCoef &c) {
    if (c.wx == 0.f && c.wz == 0.f) return 2.0f;
    const float ax = fabsf(c.wx), az = fabsf(c.wz);
    const bool z_small = az < ax;
    uint32_t b = __float_as_uint(z_small ? az : ax) & ~3u;
    b |= (c.wz > 0.f ? 1u : 0u) | (z_small ? 2u : 0u) | (c.wx < 0.f ? 0x80000000u : 0u);
    return __uint_as_float(b);
}
RZ_DEV void unpack_weights(float p, float &wx, float &wz) {
    const uint32_t b = __float_as_uint(p);
    const float a = __uint_as_float(b & 0x7ffffffcu);
    const bool none = a > 1.5f;
    const float big = 1.0f - a;
    float ax = (b & 2u) ? big : a, az = (b & 2u) ? a : big;
    ax = none ? 0.f : ax, az = none ? 0.f : az;
    wx = (b >> 31) ? -ax : ax;
    wz = (b & 1u) ? az : -az;
}

// The values one cell's linearisation reads: its traveltime and those of its
// four neighbours (3e38 for a missing one) and, for refined traveltimes, the
// neighbours' low parts.  Loading them apart from the arithmetic lets a
// caller issue the loads of several cells before any of them is used.
struct CellNb {
    float tw, te, tn, ts, tc;
    float lw, le, ln, ls;
};
RZ_DEV CellNb load_cell_nb(const float *T, const float *Tlo, int nxp, int nx, int ny, int h, int k) {
    const float big = 3.0e38f;
    const size_t o = (size_t)k * nxp + h;
    const float *p = T + o;
    CellNb c;
    c.tw = h > 0 ? __ldcg(p - 1) : big, c.te = h < nx - 1 ? __ldcg(p + 1) : big;
    c.tn = k > 0 ? __ldcg(p - nxp) : big, c.ts = k < ny - 1 ? __ldcg(p + nxp) : big;
    c.tc = __ldcg(p);
    c.lw = c.le = c.ln = c.ls = 0.f;
    if (Tlo) {
        const float *q = Tlo + o;
        c.lw = h > 0 ? __ldcg(q - 1) : 0.f, c.le = h < nx - 1 ? __ldcg(q + 1) : 0.f;
        c.ln = k > 0 ? __ldcg(q - nxp) : 0.f, c.ls = k < ny - 1 ? __ldcg(q + nxp) : 0.f;
    }
    return c;
}

// With refined traveltimes (T + Tlo, see the traveltime refinement in
// rz_shot.cu) the neighbours are chosen by their rounded sums and d carries
// the low parts, so the weights are those of the refined field to float
// precision; the low parts are 0 otherwise.
RZ_DEV ExactCoef exact_coef_nb(const CellNb &n, float s, float dh, bool source) {
    // both cases are evaluated and one is selected: cells of a warp take
    // either, and a branch would run them one after the other
    const bool west = n.tw <= n.te, north = n.tn <= n.ts;
    const float a = west ? n.tw : n.te, b = north ? n.tn : n.ts;
    const float d = (a - b) + ((west ? n.lw : n.le) - (north ? n.ln : n.ls));
    const float sh = s * dh;
    const bool one = fabsf(d) >= sh;
    // two-sided: r = sqrt(q) and 1/r from one reciprocal square root (a few
    // ulp: the weights enter a linear solve whose float error is of that
    // order anyway); q <= 0 only where the one-sided case is taken
    const float q = fmaf(2.0f * sh, sh, -d * d);
    const float rr = rsqrtf(q);
    const float r = q * rr;
    const float half_rcp = 0.5f * rr;
    // one-sided: weight 1 on the smaller neighbour (x when d <= 0), dT/dS = DH
    const float wa = one ? (d <= 0.f ? 1.f : 0.f) : (r - d) * half_rcp;
    const float wb = one ? (d <= 0.f ? 0.f : 1.f) : (r + d) * half_rcp;
    ExactCoef c;
    c.wx = source ? 0.f : (west ? -wa : wa);
    c.wz = source ? 0.f : (north ? -wb : wb);
    c.gs = source ? 0.f : (one ? dh : s * dh * dh * rr);
    return c;
}

RZ_DEV ExactCoef exact_coef(const float *T, int nxp, int nx, int ny, int h, int k, float s, float dh, bool source,
                            const float *Tlo = nullptr) {
    if (source) return ExactCoef{0.f, 0.f, 0.f};
    return exact_coef_nb(load_cell_nb(T, Tlo, nxp, nx, ny, h, k), s, dh, false);
}

// Traveltime refinement (not in the reference).  A converged float field
// T32 satisfies T32_c = fl(G(a_c, b_c)) at every cell but the source, G the
// Godunov update and a_c / b_c the smaller x / z neighbour; the FP64 fixpoint
// T* = T32 + delta solves, to first order, delta_c = r_c + w_a delta_a +
// w_b delta_b with r_c = G(a_c, b_c) - T32_c and the weights of exact_coef.
// godunov_residual returns r_c with G evaluated in float-float (error about
// 2^-42 of the traveltime), a / b the smaller existing neighbours.
RZ_DEV float godunov_residual(float a, float b, float s, float dh, float t) {
    const float sh = __fmul_rn(s, dh);
    const float shl = __fmaf_rn(s, dh, -sh);  // sh + shl = s*dh exactly
    const float d = __fsub_rn(a, b);
    // one-sided: min(a, b) + s*dh - t; min - t is exact (t lies within a
    // factor two of min, or min is 0).  Both cases are evaluated and one is
    // selected (no divergent branch; the two-sided value is NaN where unused).
    const float one = __fadd_rn(__fadd_rn(__fsub_rn(fminf(a, b), t), sh), shl);
    // (a + b + sqrt(2 (s dh)^2 - d^2)) / 2 - t in float-float
    const float sum = __fadd_rn(a, b);
    const float sbb = __fsub_rn(sum, a);
    const float se = __fadd_rn(__fsub_rn(a, __fsub_rn(sum, sbb)), __fsub_rn(b, sbb));  // a + b = sum + se
    const float p2 = __fmul_rn(sh, sh);
    const float p2l = __fmaf_rn(sh, sh, -p2);
    const float cross = __fmaf_rn(__fmul_rn(2.0f, sh), shl, p2l);
    const float d2 = __fmul_rn(d, d);
    const float d2l = __fmaf_rn(d, d, -d2);
    const float P = __fmul_rn(2.0f, p2);
    const float Dh = __fsub_rn(P, d2);
    const float Dl = __fadd_rn(__fsub_rn(__fsub_rn(P, Dh), d2), __fsub_rn(__fmul_rn(2.0f, cross), d2l));
    const float rs = rsqrtf(Dh);
    const float r0 = __fmul_rn(Dh, rs);
    const float rl = __fmul_rn(__fadd_rn(__fmaf_rn(-r0, r0, Dh), Dl), __fmul_rn(0.5f, rs));
    const float uh = __fadd_rn(sum, r0);
    const float ubb = __fsub_rn(uh, sum);
    const float ue = __fadd_rn(__fsub_rn(sum, __fsub_rn(uh, ubb)), __fsub_rn(r0, ubb));
    const float ul = __fadd_rn(__fadd_rn(ue, rl), se);
    // uh - 2t is exact (uh lies within a factor two of 2t)
    const float two = __fmul_rn(0.5f, __fadd_rn(__fsub_rn(uh, __fmul_rn(2.0f, t)), ul));
    return fabsf(d) >= sh ? one : two;
}

// r_c of the traveltime refinement at a cell of the converged field
// (missing neighbours count as absent, as in exact_coef); 0 at the source
RZ_DEV float cell_residual_nb(const CellNb &n, float s, float dh, bool source) {
    if (source) return 0.f;
    return godunov_residual(fminf(n.tw, n.te), fminf(n.tn, n.ts), s, dh, n.tc);
}

// Sum of the n floats q[0], q[stride], ..., q[(n-1)*stride] as a double,
// accumulated on the integer pipe.  GB300 issues FP64 at about two operations
// per SM cycle, so a plain double sum (a float->double conversion and an add
// per value) is bound by the FP64 pipe; this sum costs one conversion per 128
// values.
//
// Each value m * 2^(e-150) (m the 24-bit significand, e the biased exponent,
// 1 for subnormals) is added as the integer (m << 31) >> (emax - e) to a
// 64-bit fixed-point word whose unit is 2^(emax-181), emax the largest
// exponent seen so far; a larger exponent first shifts the word right
// (arithmetic) by the difference.  Every term and every shift drops less than
// one unit, i.e. less than 2^-54 of the largest |value|; with an exponent
// span of at most 31 nothing is dropped and the word is the exact sum.
// Blocks of 128 values stay below 2^62 (|term| < 2^55) and are converted to
// double once each (one rounding), so the error is below
// n * 2^-53 * max|q| + 2^-53 per block of the block sum -- within the bound
// of a plain double sum, (n-1) * 2^-53 * sum|q|.  A block holding an Inf or
// NaN is summed in double instead, so non-finite values propagate as there.
RZ_DEV double shot_sum_fixed(const float *__restrict__ q, size_t stride, int n) {
    constexpr int kBlock = 128;
    double total = 0.0;
    for (int z0 = 0; z0 < n; z0 += kBlock) {
        const int z1 = min(n, z0 + kBlock);
        long long acc = 0;
        int emax = 1;
        uint32_t special = 0;
        auto add = [&](uint32_t u) {
            const int ef = (int)((u >> 23) & 0xffu);
            special |= (uint32_t)(ef == 0xff);
            const int e = max(ef, 1);
            const int up = max(e - emax, 0);
            acc >>= min(up, 63);
            emax += up;
            const long long m = (long long)((u & 0x7fffffu) | (ef ? 0x800000u : 0u)) << 31;
            const long long x = m >> min(emax - e, 63);
            acc += (u >> 31) ? -x : x;
        };
        int z = z0;
        for (; z + 7 < z1; z += 8) {
            uint32_t u[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) u[i] = __float_as_uint(__ldg(q + (size_t)(z + i) * stride));
#pragma unroll
            for (int i = 0; i < 8; ++i) add(u[i]);
        }
        for (; z < z1; ++z) add(__float_as_uint(__ldg(q + (size_t)z * stride)));
        if (special) {
            double s = 0.0;
            for (z = z0; z < z1; ++z) s += (double)__ldg(q + (size_t)z * stride);
            total += s;
        } else {
            // exact power-of-two scale 2^(emax-181), emax in [1, 254]
            total += (double)acc * __longlong_as_double((long long)(emax - 181 + 1023) << 52);
        }
    }
    return total;
}

}  // namespace rz
