/*
 * sde_shift.h -- the reference's shifted Sobol uniform in 32-bit integer
 * pieces (src/rng/sobol.rs:62-79): u = fract(x 2^-32 + s) in f64, with
 * x the 32-bit Sobol word and s = (r >> 11) 2^-53 the scenario's ChaCha8
 * double.  In units of 2^-53 the sum is S = x 2^21 + R (R = r >> 11, 53
 * bits).  Below 2^53 (a sum under 1) it is exact: U = S.  From 2^53 on the
 * f64 sum rounds to an even unit, ties to even, and fract takes 2^53 away:
 * U = 2 rhe(S / 2) - 2^53.  With R = Rh 2^21 + Rl (Rh = the high word of
 * r, Rl its bits 11..31) and c the carry of x + Rh: the high 32 bits of U
 * are x + Rh mod 2^32, and its low 21 bits are Rl, or, with the carry, Rl
 * rounded to even (an odd Rl moves to the even neighbour whose half is
 * even, which may carry into bit 21).  So U is formed without 64-bit
 * arithmetic, and so is the tail Q = min(U, 2^53 - U).
 *
 * Plain C as well as CUDA: the host tests compile this header with the
 * host compiler and check it against the f64 sum bit for bit.  sde_u32 /
 * sde_u64 come from sde_args.h, included first.
 */
#ifndef SDE_SHIFT_H
#define SDE_SHIFT_H

#ifdef __CUDACC__
#define SDE_SH_FN static __device__ __forceinline__
#else
#define SDE_SH_FN static inline
#endif

/* U = hi 2^21 + lo with lo < 2^21 (hi: bits 21..52 of U). */
SDE_SH_FN void sde_shift_split(sde_u32 x, sde_u64 r, sde_u32* hi, sde_u32* lo) {
    const sde_u32 rh = (sde_u32)(r >> 32);
    const sde_u32 rl = (sde_u32)r >> 11;
    const sde_u32 h = x + rh;
    const int carry = h < x;
    /* odd rl: +1 when bit 1 is set (rl / 2 rounds up to an even half),
     * else -1; even rl stays */
    const sde_u32 adj = (rl & 1u) ? ((rl & 2u) ? 1u : 0xFFFFFFFFu) : 0u;
    const sde_u32 l = carry ? rl + adj : rl;   /* <= 2^21 */
    *hi = h + (l >> 21);                       /* no wrap: h <= 2^32 - 2 with the carry */
    *lo = l & 0x1FFFFFu;
}

/* The tail of U = hi 2^21 + lo: up = (U >= 2^52), Q = up ? 2^53 - U : U =
 * hq 2^21 + lq with lq < 2^21 (hq < 2^31 + 1). */
SDE_SH_FN void sde_tail_split(sde_u32 hi, sde_u32 lo, sde_u32* hq, sde_u32* lq, int* up) {
    const int u = (int)(hi >> 31);
    *up = u;
    *hq = u ? ~hi + (lo == 0u) : hi;
    *lq = u ? (0x200000u - lo) & 0x1FFFFFu : lo;
}

#endif
