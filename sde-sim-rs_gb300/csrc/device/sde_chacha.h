/*
 * sde_chacha.h -- ChaCha8 per scenario (rand_chacha 0.9 as called at
 * src/rng/pseudo.rs:18 and src/rng/sobol.rs:68): 32-byte key from
 * rand_core's PCG32-based seed_from_u64, 64-bit block counter in words
 * 12-13 starting at 0, stream 0 in words 14-15, 8 rounds.  u64 number k of
 * the stream is words 2k (low) and 2k+1 (high).
 *
 * Plain C as well as CUDA: the host tests compile this header with the
 * host compiler and check its blocks against the oracle's ChaCha core,
 * including counters whose high word is not 0.  sde_u32 / sde_u64 come
 * from sde_args.h, included first.
 */
#ifndef SDE_CHACHA_H
#define SDE_CHACHA_H

#ifdef __CUDACC__
#define SDE_CC_FN static __device__ __forceinline__
#define SDE_CC_UNROLL _Pragma("unroll")
#define SDE_ROTL(x, n) __funnelshift_l((x), (x), (n))
#define SDE_ROTR(x, n) __funnelshift_r((x), (x), (n))
#else
#define SDE_CC_FN static inline
#define SDE_CC_UNROLL
#define SDE_ROTL(x, n) (((x) << ((n) & 31)) | ((x) >> ((32 - ((n) & 31)) & 31)))
#define SDE_ROTR(x, n) (((x) >> ((n) & 31)) | ((x) << ((32 - ((n) & 31)) & 31)))
#endif

SDE_CC_FN sde_u32 sde_rotl(sde_u32 x, int n) { return SDE_ROTL(x, n); }

SDE_CC_FN void sde_seed_from_u64(sde_u64 s, sde_u32 k[8]) {
    SDE_CC_UNROLL for (int i = 0; i < 8; ++i) {
        s = s * 6364136223846793005ull + 11634580027462260723ull;
        const sde_u32 xs = (sde_u32)(((s >> 18) ^ s) >> 27);
        const sde_u32 rot = (sde_u32)(s >> 59);
        k[i] = SDE_ROTR(xs, rot);
    }
}

#define SDE_QR(a, b, c, d)                          \
    a += b; d ^= a; d = sde_rotl(d, 16);            \
    c += d; b ^= c; b = sde_rotl(b, 12);            \
    a += b; d ^= a; d = sde_rotl(d, 8);             \
    c += d; b ^= c; b = sde_rotl(b, 7);

#define SDE_CC0 0x61707865u
#define SDE_CC1 0x3320646eu
#define SDE_CC2 0x79622d32u
#define SDE_CC3 0x6b206574u

SDE_CC_FN void sde_chacha8_block(const sde_u32 k[8], sde_u64 ctr, sde_u32 o[16]) {
    const sde_u32 c0 = (sde_u32)ctr, c1 = (sde_u32)(ctr >> 32);
    sde_u32 x0 = SDE_CC0, x1 = SDE_CC1, x2 = SDE_CC2, x3 = SDE_CC3;
    sde_u32 x4 = k[0], x5 = k[1], x6 = k[2], x7 = k[3];
    sde_u32 x8 = k[4], x9 = k[5], x10 = k[6], x11 = k[7];
    sde_u32 x12 = c0, x13 = c1, x14 = 0u, x15 = 0u;
    SDE_CC_UNROLL for (int r = 0; r < 4; ++r) {
        SDE_QR(x0, x4, x8, x12) SDE_QR(x1, x5, x9, x13)
        SDE_QR(x2, x6, x10, x14) SDE_QR(x3, x7, x11, x15)
        SDE_QR(x0, x5, x10, x15) SDE_QR(x1, x6, x11, x12)
        SDE_QR(x2, x7, x8, x13) SDE_QR(x3, x4, x9, x14)
    }
    o[0] = x0 + SDE_CC0; o[1] = x1 + SDE_CC1; o[2] = x2 + SDE_CC2; o[3] = x3 + SDE_CC3;
    o[4] = x4 + k[0]; o[5] = x5 + k[1]; o[6] = x6 + k[2]; o[7] = x7 + k[3];
    o[8] = x8 + k[4]; o[9] = x9 + k[5]; o[10] = x10 + k[6]; o[11] = x11 + k[7];
    o[12] = x12 + c0; o[13] = x13 + c1; o[14] = x14; o[15] = x15;
}

#endif
