/* x87.cuh -- x87 extended-precision arithmetic on whole numbers, for host and device.
 *
 * The reference forms a few scalars in `long double`, the x87 80-bit format (64-bit significand, round to nearest
 * even), and rounds them to F32: tk_build's contrast gain and offset (src/kern/track.c:603-614) and store_appearance's
 * mean (track.c:958). Where the operands are whole numbers these are a quotient and a product of integers, computed
 * here exactly and rounded the way the x87 unit rounds, so the F32 results are the reference's bits on any machine. */
#ifndef VTG_X87_CUH
#define VTG_X87_CUH

#include <math.h>
#include <stdint.h>

/* An x87 extended value on whole-number arithmetic: m x 2^e, 2^63 <= m < 2^64 (m = 0 for zero). Round to nearest even
 * at 64 bits, as the x87 unit does in its default precision. */
struct X87 {
    uint64_t m;
    int e;
};

/* num / den rounded to a 64-bit significand; 0 < num, den < 2^31. Long division, one quotient bit a step. */
__host__ __device__ static inline X87 x87_div(uint32_t num, uint32_t den)
{
    uint64_t R = num, D = den;
    int s = 0;
    while (D <= (R >> 1)) { /* D <= R < 2 D afterwards: the quotient is R / D x 2^s, R / D in [1, 2) */
        D <<= 1;
        s++;
    }
    while (R < D) {
        R <<= 1;
        s--;
    }
    uint64_t m = 0;
    for (int i = 0; i < 64; i++) { /* R < 2 D throughout */
        m <<= 1;
        if (R >= D) {
            m |= 1;
            R -= D;
        }
        R <<= 1;
    }
    const bool guard = R >= D;
    if (guard)
        R -= D;
    X87 r = {m, s - 63};
    if (guard && (R != 0 || (m & 1))) {
        r.m++;
        if (r.m == 0) {
            r.m = 1ull << 63;
            r.e++;
        }
    }
    return r;
}

/* a x k rounded to a 64-bit significand, k < 2^32: the 96-bit product in two words, then one rounding. */
__host__ __device__ static inline X87 x87_mul(X87 a, uint32_t k)
{
    if (a.m == 0 || k == 0)
        return X87{0, 0};
    const uint64_t lo32 = (a.m & 0xffffffffull) * k, hi32 = (a.m >> 32) * k;
    const uint64_t lo = lo32 + (hi32 << 32);
    const uint64_t hi = (hi32 >> 32) + (lo < lo32 ? 1u : 0u); /* product = hi x 2^64 + lo, hi < 2^32 */
    int sh = 0;
    while ((hi >> sh) != 0)
        sh++;
    if (sh == 0)
        return X87{lo, a.e};
    const uint64_t m = (lo >> sh) | (hi << (64 - sh));
    const uint64_t half = 1ull << (sh - 1), rest = lo & ((half << 1) - 1);
    X87 r = {m, a.e + sh};
    if (rest > half || (rest == half && (m & 1))) {
        r.m++;
        if (r.m == 0) {
            r.m = 1ull << 63;
            r.e++;
        }
    }
    return r;
}

/* An extended value rounded to F32 (to nearest even). */
__host__ __device__ static inline float x87_to_f32(X87 a)
{
    if (a.m == 0)
        return 0.0f;
    uint32_t t = (uint32_t)(a.m >> 40);
    const uint64_t rest = a.m & ((1ull << 40) - 1), half = 1ull << 39;
    int e = a.e + 40;
    if (rest > half || (rest == half && (t & 1)))
        t++;
    if (t == (1u << 24)) {
        t >>= 1;
        e++;
    }
    return ldexpf((float)t, e);
}

#endif
