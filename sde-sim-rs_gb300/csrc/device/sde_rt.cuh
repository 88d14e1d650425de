/*
 * sde_rt.cuh -- device runtime of the GB300 path-simulation engine.
 *
 * Included by the nvcc-built kernels (kernels.cu) and prepended to every
 * NVRTC-lowered step kernel.  It holds the per-path random streams, the
 * Sobol point construction, the inverse CDFs, the fasteval operator
 * semantics and the estimator reduction.  No system headers: NVRTC builds
 * it without an include path.
 */
#ifndef SDE_RT_CUH
#define SDE_RT_CUH

#define SDE_DEV static __device__ __forceinline__
#define SDE_FULL_MASK 0xffffffffu

/* the FP64 logarithm of the inverse CDF (prepended to the lowered kernels'
 * source, included here for the nvcc-built ones) */
#ifndef SDE_LOG_H
#include "sde_log.h"
#endif

/* ChaCha8 per scenario: sde_seed_from_u64, sde_chacha8_block and the
 * stream-precomputed sde_chacha8_block_s (prepended to the lowered
 * kernels' source, included here for the nvcc-built ones) */
#ifndef SDE_CHACHA_H
#include "sde_chacha.h"
#include "sde_shift.h"
#endif

SDE_DEV sde_u64 sde_pair(sde_u32 lo, sde_u32 hi) { return ((sde_u64)hi << 32) | (sde_u64)lo; }

/* rand's StandardUniform<f64>: (u64 >> 11) * 2^-53 */
SDE_DEV double sde_u64_to_f64(sde_u64 r) { return (double)(r >> 11) * 0x1p-53; }

/* ------------------------------------------------------------------------
 * Uniform tail probabilities for the FP32 kernels: q = min(p, 1-p) formed
 * exactly in integers, so the only rounding is the final float conversion.
 * up is p >= 0.5, gt is p > 0.5.
 * ---------------------------------------------------------------------- */

/* pseudo: p = U * 2^-53, U = r >> 11 */
SDE_DEV void sde_tail_u53(sde_u64 U, float& q, bool& up, bool& gt) {
    up = U >= (1ull << 52);
    gt = U > (1ull << 52);
    const sde_u64 Q = up ? (1ull << 53) - U : U;
    q = __ull2float_rn(Q) * 0x1p-53f;
}

/* Sobol with a random shift (src/rng/sobol.rs:62-79): u = fract(x*2^-32 + s)
 * in f64, s = (r >> 11)*2^-53.  Emulated exactly in 53-bit fixed point:
 * sums in [1,2) round to a multiple of 2^-52, ties to even. */
SDE_DEV sde_u64 sde_shift_u53(sde_u32 x, sde_u64 r) {
    const sde_u64 sum = ((sde_u64)x << 21) + (r >> 11);
    if (sum < (1ull << 53)) return sum;
    sde_u64 h = sum >> 1;
    if ((sum & 1ull) && (h & 1ull)) h += 1ull;
    return (h - (1ull << 52)) << 1;
}

/* XOR-scrambled Sobol: p = (y + 0.5) * 2^-32 */
SDE_DEV void sde_tail_xor(sde_u32 y, float& q, bool& up, bool& gt) {
    up = (y >> 31) != 0u;
    gt = up;
    const sde_u32 m = up ? ~y : y;
    q = __uint2float_rn(2u * m + 1u) * 0x1p-33f;
}

/* ------------------------------------------------------------------------
 * Sobol points (sobol crate, Joe-Kuo D6, Gray-code order):
 *   x_n[d] = xor of V[d][b] over the set bits b of gray(n) = n ^ (n >> 1).
 * ---------------------------------------------------------------------- */

SDE_DEV sde_u32 sde_gray(sde_u32 n) { return n ^ (n >> 1); }

SDE_DEV sde_u32 sde_sobol_direct(const sde_u32* __restrict__ V, int d, sde_u32 g) {
    const sde_u32* v = V + (sde_u64)d * 32u;
    sde_u32 x = 0u;
    while (g) {
        const int b = __ffs(g) - 1;
        x ^= __ldg(v + b);
        g &= g - 1u;
    }
    return x;
}

/* Warp-cooperative part of a point: for a warp whose 32 lanes hold points
 * 32w .. 32w+31, gray(n) >> 5 == gray(w) is the same on every lane.  Lane l
 * returns, for dimension 32*chunk + l, the xor of the direction numbers
 * 5.. selected by H = gray(w), xored with the scramble mask; lanes then
 * fetch a dimension's value with one shuffle. */
SDE_DEV sde_u32 sde_sobol_hi(const sde_u32* __restrict__ VT, const sde_u32* __restrict__ mask,
                             int dims, int chunk, sde_u32 H, int lane) {
    const int d = chunk * 32 + lane;
    if (d >= dims) return 0u;
    /* mask rows are padded to a multiple of 32 words */
    sde_u32 acc = mask ? __ldg(mask + d) : 0u;
    while (H) {
        const int b = __ffs(H) - 1;
        acc ^= __ldg(VT + (sde_u64)(b + 5) * (sde_u64)dims + (sde_u64)d);
        H &= H - 1u;
    }
    return acc;
}

/* ------------------------------------------------------------------------
 * Inverse CDFs (src/proc/increment.rs:161-200)
 * ---------------------------------------------------------------------- */

/* Abramowitz-Stegun 26.2.23 as the reference evaluates it; the logarithm
 * of the tail probability is sde_log_tail (within 0.52 ulp, so it agrees
 * with the reference's log to the last bit nearly always). */
SDE_DEV double sde_icdf_as26(double p) {
    const double t = p < 0.5 ? sqrt(-2.0 * sde_log_tail(p)) : sqrt(-2.0 * sde_log_tail(1.0 - p));
    const double x = t - ((0.010328 * t + 0.802853) * t + 2.515517) /
                             (((0.001308 * t + 0.189269) * t + 1.432788) * t + 1.0);
    return p < 0.5 ? -x : x;
}

SDE_DEV float sde_lg2_approx(float x) {
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
SDE_DEV float sde_rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
SDE_DEV float sde_rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

/* AS 26.2.23 in FP32 straight from an XOR-scrambled Sobol word y, with
 * p = (y + 0.5) 2^-32: q = min(p, 1-p) = (2 min(y, ~y) + 1) 2^-33 is exact
 * before its one rounding, log2 q = lg2(2m+1) - 33 folds into one FMA with
 * -2 ln 2, sqrt(a) = a * rsqrt(a) (a >= 2 ln 2 > 0), the rational term is
 * one reciprocal, and the sign (negative for p < 0.5) is one xor. */
/* |z| of AS 26.2.23 from a = -2 ln q > 0 */
SDE_DEV float sde_as26_abs(float a) {
    const float t = a * sde_rsqrt_approx(a);
    const float num = fmaf(fmaf(0.010328f, t, 0.802853f), t, 2.515517f);
    const float den = fmaf(fmaf(fmaf(0.001308f, t, 0.189269f), t, 1.432788f), t, 1.0f);
    return fmaf(-num, sde_rcp_approx(den), t);
}

SDE_DEV float sde_normal_xor(sde_u32 y) {
    const sde_u32 s = (sde_u32)((int)y >> 31);  /* all ones when p >= 0.5 */
    const sde_u32 m = y ^ s;                    /* min(y, ~y) */
    const float lg = sde_lg2_approx(__uint2float_rn(2u * m + 1u));
    const float x = sde_as26_abs(fmaf(lg, -1.3862943611198906f, 45.747713916956393f));  /* -2 ln q */
    return __int_as_float(__float_as_int(x) ^ (~s & 0x80000000u));
}

/* Two normals at once: the polynomial and scaling work of both runs as
 * paired FP32 operations (one fma.f32x2 per pair of FMAs); lg2 and rsqrt
 * stay per element.  The two denominators share one reciprocal: both lie in
 * [1, 28] (t <= 8.6 for q >= 2^-53), so r = 1/(den.x den.y) is far from
 * overflow and 1/den.x = den.y r, 1/den.y = den.x r, about two ulp of 1/den
 * against one for a reciprocal each, for one SFU operation fewer (SHARED;
 * kernels not bound by the SFU pipe keep one each).  The numerator is
 * formed negated so the final step is a plain paired FMA. */
template <bool SHARED = true>
SDE_DEV float2 sde_as26_abs2(float2 a) {
    const float2 r = make_float2(sde_rsqrt_approx(a.x), sde_rsqrt_approx(a.y));
    const float2 t = __fmul2_rn(a, r);
    const float2 nnum = __ffma2_rn(__ffma2_rn(make_float2(-0.010328f, -0.010328f), t,
                                              make_float2(-0.802853f, -0.802853f)),
                                   t, make_float2(-2.515517f, -2.515517f));
    const float2 den = __ffma2_rn(__ffma2_rn(__ffma2_rn(make_float2(0.001308f, 0.001308f), t,
                                                        make_float2(0.189269f, 0.189269f)),
                                             t, make_float2(1.432788f, 1.432788f)),
                                  t, make_float2(1.0f, 1.0f));
    float2 rc;
    if (SHARED) {
        const float rd = sde_rcp_approx(den.x * den.y);
        rc = __fmul2_rn(make_float2(rd, rd), make_float2(den.y, den.x));
    } else {
        rc = make_float2(sde_rcp_approx(den.x), sde_rcp_approx(den.y));
    }
    return __ffma2_rn(nnum, rc, t);
}

template <bool SHARED = true>
SDE_DEV float2 sde_normal_xor2(sde_u32 ya, sde_u32 yb) {
    const sde_u32 sa = (sde_u32)((int)ya >> 31), sb = (sde_u32)((int)yb >> 31);
    const float2 lg = make_float2(sde_lg2_approx(__uint2float_rn(2u * (ya ^ sa) + 1u)),
                                  sde_lg2_approx(__uint2float_rn(2u * (yb ^ sb) + 1u)));
    const float2 x = sde_as26_abs2<SHARED>(__ffma2_rn(lg, make_float2(-1.3862943611198906f, -1.3862943611198906f),
                                                      make_float2(45.747713916956393f, 45.747713916956393f)));
    return make_float2(__int_as_float(__float_as_int(x.x) ^ (~sa & 0x80000000u)),
                       __int_as_float(__float_as_int(x.y) ^ (~sb & 0x80000000u)));
}

/* float of a tail integer Q <= 2^52 from its two 32-bit halves: hi < 2^21
 * converts exactly, lo rounds by at most 2^7, and the FMA rounds once; within
 * one ulp of the correctly rounded value, without the 64-bit conversion,
 * which runs on the FP64 pipe */
SDE_DEV float sde_q53_to_float(sde_u64 Q) {
    return fmaf(__uint2float_rn((sde_u32)(Q >> 32)), 0x1p32f, __uint2float_rn((sde_u32)Q));
}

/* SPLIT_CVT: the tails convert with sde_q53_to_float (the shifted-Sobol
 * kernels, where the FP64 pipe is busy); else one 64-bit conversion each
 * (the ChaCha8 kernels, bound by issue, measured slower with the split) */
template <bool SHARED = true, bool SPLIT_CVT = false>
SDE_DEV float2 sde_normal_u53_2(sde_u64 Ua, sde_u64 Ub) {
    const bool upa = Ua >= (1ull << 52), upb = Ub >= (1ull << 52);
    const sde_u64 Qa = upa ? (1ull << 53) - Ua : Ua, Qb = upb ? (1ull << 53) - Ub : Ub;
    const float2 lg = SPLIT_CVT ? make_float2(sde_lg2_approx(sde_q53_to_float(Qa)), sde_lg2_approx(sde_q53_to_float(Qb)))
                                : make_float2(sde_lg2_approx(__ull2float_rn(Qa)), sde_lg2_approx(__ull2float_rn(Qb)));
    const float2 x = sde_as26_abs2<SHARED>(__ffma2_rn(lg, make_float2(-1.3862943611198906f, -1.3862943611198906f),
                                                      make_float2(73.473601139354201f, 73.473601139354201f)));
    return make_float2(upa ? x.x : -x.x, upb ? x.y : -x.y);
}

/* Two normals of the reference's shifted Sobol uniforms U = hi 2^21 + lo
 * (sde_shift_split): the tails Q = hq 2^21 + lq in 32-bit pieces
 * (sde_tail_split), float(Q) = fma(float(hq), 2^21, float(lq)) within one
 * ulp (hq <= 2^31 rounds once, lq < 2^21 is exact), then as
 * sde_normal_u53_2. */
template <bool SHARED = true>
SDE_DEV float2 sde_normal_split2(sde_u32 ha, sde_u32 la, sde_u32 hb, sde_u32 lb) {
    sde_u32 qha, qla, qhb, qlb;
    int upa, upb;
    sde_tail_split(ha, la, &qha, &qla, &upa);
    sde_tail_split(hb, lb, &qhb, &qlb, &upb);
    const float2 lg = make_float2(sde_lg2_approx(fmaf(__uint2float_rn(qha), 0x1p21f, __uint2float_rn(qla))),
                                  sde_lg2_approx(fmaf(__uint2float_rn(qhb), 0x1p21f, __uint2float_rn(qlb))));
    const float2 x = sde_as26_abs2<SHARED>(__ffma2_rn(lg, make_float2(-1.3862943611198906f, -1.3862943611198906f),
                                                      make_float2(73.473601139354201f, 73.473601139354201f)));
    return make_float2(upa ? x.x : -x.x, upb ? x.y : -x.y);
}

/* The same from a 53-bit uniform p = U 2^-53 (ChaCha doubles, or the
 * reference's shifted Sobol values through sde_shift_u53): q = min(U,
 * 2^53 - U) 2^-53, log2 q = lg2(Q) - 53. */
SDE_DEV float sde_normal_u53(sde_u64 U) {
    const bool up = U >= (1ull << 52);
    const sde_u64 Q = up ? (1ull << 53) - U : U;
    const float lg = sde_lg2_approx(__ull2float_rn(Q));
    const float x = sde_as26_abs(fmaf(lg, -1.3862943611198906f, 73.473601139354201f));
    return up ? x : -x;
}

/* The same rational approximation in FP32, from the exact tail q. */
SDE_DEV float sde_icdf_as26_q(float q, bool up) {
    const float t = sqrtf(-2.0f * __logf(q));
    const float num = (0.010328f * t + 0.802853f) * t + 2.515517f;
    const float den = ((0.001308f * t + 0.189269f) * t + 1.432788f) * t + 1.0f;
    const float x = t - __fdividef(num, den);
    return up ? x : -x;
}

/* "accurate" inverse normal (an option beside the reference's formula):
 * the AS 26.2.23 value refined by Halley steps on Phi(z) - p, with the
 * residual formed from the tail probability through erfc, so nothing
 * cancels in the tails:  u = r / phi(z),  z <- z - u / (1 + z u / 2).
 * FP64: two steps (|error| ~ 1e-16 from 4.5e-4); FP32: one step. */
SDE_DEV double sde_icdf_accurate(double p) {
    double z = sde_icdf_as26(p);
    const bool lower = p < 0.5;
    const double tail = lower ? p : 1.0 - p;
#pragma unroll
    for (int it = 0; it < 2; ++it) {
        const double ft = 0.5 * erfc((lower ? -z : z) * 0.70710678118654752);
        const double r = lower ? ft - tail : tail - ft;
        const double u = r * 2.5066282746310002 * exp(0.5 * z * z);
        z = z - u / (1.0 + 0.5 * z * u);
    }
    return z;
}

SDE_DEV float sde_icdf_accurate_q(float q, bool up) {
    float z = sde_icdf_as26_q(q, up);
    const float ft = 0.5f * erfcf((up ? z : -z) * 0.70710678f);
    const float r = up ? q - ft : ft - q;
    const float u = r * 2.50662827f * expf(0.5f * z * z);
    return z - u / (1.0f + 0.5f * z * u);
}

/* Poisson inverse CDF with the reference's cap of 200 (increment.rs:182-200) */
SDE_DEV double sde_poisson(double u, double lambda) {
    if (lambda <= 0.0) return 0.0;
    double p = exp(-lambda);
    double f = p;
    int k = 0;
    while (u > f && k < 200) {
        k += 1;
        p *= lambda / (double)k;
        f += p;
    }
    return (double)k;
}

SDE_DEV float sde_poisson(float u, float lambda) {
    if (lambda <= 0.0f) return 0.0f;
    float p = expf(-lambda);
    float f = p;
    int k = 0;
    while (u > f && k < 200) {
        k += 1;
        p *= lambda / (float)k;
        f += p;
    }
    return (float)k;
}

/* ------------------------------------------------------------------------
 * fasteval operator semantics (src/func.rs:18-42 evaluates with fasteval
 * 0.2.4): comparisons give 1/0, == != <= >= carry fasteval's 8*eps absolute
 * tolerance, && and || return an operand, log(x) is ln(x)/ln(10).
 * ---------------------------------------------------------------------- */

#define SDE_EPS8 0x1p-49

SDE_DEV double sde_b(bool b, double) { return b ? 1.0 : 0.0; }
SDE_DEV float sde_b(bool b, float) { return b ? 1.0f : 0.0f; }
template <class R> SDE_DEV R sde_eq(R l, R r) { return sde_b(fabs(l - r) <= (R)SDE_EPS8, l); }
template <class R> SDE_DEV R sde_ne(R l, R r) { return sde_b(fabs(l - r) > (R)SDE_EPS8, l); }
template <class R> SDE_DEV R sde_lt(R l, R r) { return sde_b(l < r, l); }
template <class R> SDE_DEV R sde_gt(R l, R r) { return sde_b(l > r, l); }
template <class R> SDE_DEV R sde_le(R l, R r) { return sde_b(l <= r + (R)SDE_EPS8, l); }
template <class R> SDE_DEV R sde_ge(R l, R r) { return sde_b(l + (R)SDE_EPS8 >= r, l); }
template <class R> SDE_DEV R sde_not(R x) { return sde_b(fabs(x) <= (R)SDE_EPS8, x); }
template <class R> SDE_DEV R sde_and(R l, R r) { return fabs(l) <= (R)SDE_EPS8 ? l : r; }
template <class R> SDE_DEV R sde_or(R l, R r) { return fabs(l) > (R)SDE_EPS8 ? l : r; }
template <class R> SDE_DEV R sde_sign(R x) { return isnan(x) ? x : (signbit(x) ? (R)-1 : (R)1); }
template <class R> SDE_DEV R sde_sq(R x) { return x * x; }
SDE_DEV double sde_rsqrt(double x) { return 1.0 / sqrt(x); }
SDE_DEV float sde_rsqrt(float x) { return rsqrtf(x); }
/* chain-rule product of symbolic derivatives: 0 where the inner derivative
 * is 0, even if the outer one is infinite there */
template <class R> SDE_DEV R sde_mul0(R a, R b) { return b == (R)0 ? (R)0 : a * b; }
SDE_DEV double sde_log10(double x) { return log(x) / 0x1.26bb1bbb55516p+1; }
SDE_DEV float sde_log10(float x) { return logf(x) / 0x1.26bb1cp+1f; }
template <class R> SDE_DEV R sde_logb(R b, R x) { return log(x) / log(b); }
template <class R> SDE_DEV R sde_round2(R m, R x) { return round(x / m) * m; }

/* ------------------------------------------------------------------------
 * 5th-generation tensor cores (tcgen05) for correlated diffusions: the
 * per-step increments d = K w of a universe whose diffusion terms are
 * constant * own state are one [paths x dims] x [dims x processes] product.
 * A (the paths' Wiener increments) and B (the constant matrix) sit in shared
 * memory in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes per
 * core matrix, LBO = next core matrix along K, SBO = next 8-row group); the
 * FP32 accumulator D lives in tensor memory and comes back one row (path)
 * per thread with tcgen05.ld 32x32b.
 * ---------------------------------------------------------------------- */

SDE_DEV sde_u32 sde_smem_addr(const void* p) { return (sde_u32)__cvta_generic_to_shared(p); }

/* matrix descriptor: start, LBO, SBO (bytes, >> 4), version 1, no swizzle */
SDE_DEV sde_u64 sde_smem_desc(sde_u32 saddr, sde_u32 lbo, sde_u32 sbo) {
    return (sde_u64)((saddr & 0x3FFFFu) >> 4) | ((sde_u64)((lbo >> 4) & 0x3FFFu) << 16) |
           ((sde_u64)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

/* instruction descriptor, kind::tf32: F32 accumulator, TF32 A and B, both
 * K-major, N >> 3 at bit 17, M >> 4 at bit 24 */
SDE_DEV sde_u32 sde_idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((sde_u32)(N >> 3) << 17) | ((sde_u32)(M >> 4) << 24);
}

SDE_DEV void sde_tmem_alloc(sde_u32 dst_smem, sde_u32 ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
SDE_DEV void sde_tmem_dealloc(sde_u32 taddr, sde_u32 ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
SDE_DEV void sde_mbar_init(sde_u32 mbar, sde_u32 count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count) : "memory");
}
/* suspends the thread until the phase completes or about 10 us pass (the
 * suspend-time hint, in ns), instead of returning at once: waiting warps
 * then take no issue slots from the other warps of the SM */
SDE_DEV bool sde_mbar_try_wait(sde_u32 mbar, sde_u32 parity) {
    sde_u32 ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(mbar), "r"(parity), "r"(10000u)
        : "memory");
    return ok != 0u;
}
/* waits for the barrier phase, giving up after ~1 s of SM clock */
SDE_DEV bool sde_mbar_wait_bounded(sde_u32 mbar, sde_u32 parity) {
    const long long t0 = clock64();
    while (!sde_mbar_try_wait(mbar, parity))
        if (clock64() - t0 > 2000000000ll) return false;
    return true;
}
/* the phase's state now, without suspending */
SDE_DEV bool sde_mbar_test_wait(sde_u32 mbar, sde_u32 parity) {
    sde_u32 ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0u;
}
/* sde_mbar_wait_bounded with a budget of `cycles` SM clocks (0: the ~1 s
 * default); a shorter budget polls without suspending, so it gives up once
 * the budget is spent even when the phase would complete soon after */
SDE_DEV bool sde_mbar_wait_budget(sde_u32 mbar, sde_u32 parity, sde_u64 cycles) {
    if (cycles == 0ull) return sde_mbar_wait_bounded(mbar, parity);
    const long long t0 = clock64();
    while (!sde_mbar_test_wait(mbar, parity))
        if (clock64() - t0 > (long long)cycles) return false;
    return true;
}
/* one arrival (release) on a CTA mbarrier */
SDE_DEV void sde_mbar_arrive(sde_u32 mbar) {
    asm volatile("{ .reg .b64 st; mbarrier.arrive.shared::cta.b64 st, [%0]; }" ::"r"(mbar) : "memory");
}
SDE_DEV void sde_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
/* one arrival on a CTA mbarrier that also expects `bytes` of asynchronous
 * copies to complete on it */
SDE_DEV void sde_mbar_arrive_expect_tx(sde_u32 mbar, sde_u32 bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}
/* bulk copy of `bytes` from global memory into this CTA's shared memory,
 * completing on mbar; both addresses 16-byte aligned, bytes a multiple of 16 */
SDE_DEV void sde_bulk_g2s(sde_u32 dst, const void* src, sde_u32 bytes, sde_u32 mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(mbar)
                 : "memory");
}
SDE_DEV void sde_tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
SDE_DEV void sde_tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

SDE_DEV void sde_mma_tf32(sde_u32 dtmem, sde_u64 adesc, sde_u64 bdesc, sde_u32 idesc, sde_u32 accumulate) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p; }" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
SDE_DEV void sde_mma_commit(sde_u32 mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}
/* 16 consecutive FP32 columns of this thread's TMEM lane */
SDE_DEV void sde_tmem_ld16(sde_u32 taddr, float* d) {
    sde_u32 r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) d[i] = __uint_as_float(r[i]);
}
SDE_DEV void sde_tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
/* the same load with its wait in one statement, so no use of the registers
 * can be scheduled between the two */
SDE_DEV void sde_tmem_ld16_wait(sde_u32 taddr, float* d) {
    sde_u32 r[16];
    asm volatile(
        "{\n\ttcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];\n\ttcgen05.wait::ld.sync.aligned;\n\t}"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) d[i] = __uint_as_float(r[i]);
}
/* makes an mbarrier.init visible to the async proxy (tensor-core commits) */
SDE_DEV void sde_fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

/* TF32 split x = hi + lo (hi keeps the 19 bits a TF32 operand reads) */
SDE_DEV float sde_tf32_hi(float x) { return __uint_as_float(__float_as_uint(x) & 0xFFFFE000u); }

/* instruction descriptor, kind::f16 with F16 A and B (both K-major) and an
 * F32 accumulator */
SDE_DEV sde_u32 sde_idesc_f16(int M, int N) {
    return (1u << 4) | ((sde_u32)(N >> 3) << 17) | ((sde_u32)(M >> 4) << 24);
}
SDE_DEV void sde_mma_f16(sde_u32 dtmem, sde_u64 adesc, sde_u64 bdesc, sde_u32 idesc, sde_u32 accumulate) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
/* FP16 split of two values: x = hi + lo with hi = f16(x) and lo = f16(x - hi)
 * (x - hi is exact in FP32), packed with the first value in the low half. */
SDE_DEV void sde_split_f16x2(float x0, float x1, sde_u32& hi, sde_u32& lo) {
    asm("{\n\t.reg .b16 h0, h1;\n\t.reg .f32 f0, f1;\n\t"
        "cvt.rn.f16x2.f32 %0, %3, %2;\n\t"
        "mov.b32 {h0, h1}, %0;\n\t"
        "cvt.f32.f16 f0, h0;\n\t"
        "cvt.f32.f16 f1, h1;\n\t"
        "sub.rn.f32 f0, %2, f0;\n\t"
        "sub.rn.f32 f1, %3, f1;\n\t"
        "cvt.rn.f16x2.f32 %1, f1, f0;\n\t}"
        : "=&r"(hi), "=&r"(lo)
        : "f"(x0), "f"(x1));
}

/* sde_sobol_hi with the direction-number loads issued eight bits of H at a
 * time (predicated), so up to eight are in flight together instead of one
 * per loop trip; batches stop where H has no bits left */
SDE_DEV sde_u32 sde_sobol_hi_unrolled(const sde_u32* __restrict__ VT, const sde_u32* __restrict__ mask, int dims,
                                      int chunk, sde_u32 H, int lane) {
    const int d = chunk * 32 + lane;
    if (d >= dims) return 0u;
    sde_u32 acc = mask ? __ldg(mask + d) : 0u;
    const sde_u32* col = VT + 5ull * (sde_u64)dims + (sde_u64)d;
#pragma unroll 1
    for (int b0 = 0; b0 < 27 && (H >> b0) != 0u; b0 += 8) {
#pragma unroll
        for (int b = 0; b < 8; ++b)
            if (b0 + b < 27 && ((H >> (b0 + b)) & 1u)) acc ^= __ldg(col + (sde_u64)(b0 + b) * (sde_u64)dims);
    }
    return acc;
}

/* ------------------------------------------------------------------------
 * Estimator reduction (fused epilogue): warp shuffles, then a Neumaier
 * compensated sum over the block's warps, in FP64.  out gets
 * {sum, compensation, sum of squares, compensation} per estimator.
 * ---------------------------------------------------------------------- */

SDE_DEV void sde_neumaier(double& s, double& c, double x) {
    const double t = s + x;
    if (fabs(s) >= fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
}

/* s[k], q[k]: this thread's sum and sum of squares of estimator k (a thread
 * may own several paths). */
template <int K>
SDE_DEV void sde_block_reduce_store(const double (&fs)[K], const double (&fq)[K],
                                    double* __restrict__ out) {
    __shared__ double sm[K][32][2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double s = fs[k], q = fq[k];
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            s += __shfl_down_sync(SDE_FULL_MASK, s, o);
            q += __shfl_down_sync(SDE_FULL_MASK, q, o);
        }
        if (lane == 0) { sm[k][warp][0] = s; sm[k][warp][1] = q; }
    }
    __syncthreads();
    if (threadIdx.x < K) {
        const int k = threadIdx.x;
        double s = 0.0, sc = 0.0, q = 0.0, qc = 0.0;
        for (int w = 0; w < nw; ++w) {
            sde_neumaier(s, sc, sm[k][w][0]);
            sde_neumaier(q, qc, sm[k][w][1]);
        }
        out[k * 4 + 0] = s; out[k * 4 + 1] = sc;
        out[k * 4 + 2] = q; out[k * 4 + 3] = qc;
    }
}

#endif
