/* lk.cu -- sparse pyramidal Lucas-Kanade, one warp per point, and the per-cell grid driver.
 *
 * Reference: lk_track / lk_flowback (src/kern/lk.h:46-53): the driver of src/kern/lk_driver.inc:7-121 around three patch
 * operations, build (src/kern/lk_vx.c:36-97), iterate (lk_vx.c:100-140) and residual (lk_vx.c:142-175); the per-cell
 * grid of still_vectors (src/kern/still.c:116-141); the tracker's point list OP_LK (src/kern/track.c:275-292).
 *
 * Mapping. A warp owns one point. Lane c holds patch column c - 1 (c = 1 .. W are the patch; lane 0 and lanes past W
 * hold the window's border columns or nothing, with zero gradients, so they add exactly nothing to any sum). A lane
 * walks the patch's rows, carrying the previous row's horizontally interpolated value, so one J load per lane per row
 * serves the bilinear sample (the right neighbour comes from the next lane by shuffle). The template T, Tx, Ty of the
 * current level lives in registers (3 x H floats a lane) from its build to its last iteration. Sums are per-lane FMA
 * chains folded across the warp by a butterfly of xor shuffles, so every lane ends with the same bits and the driver
 * runs warp-uniform, without divergence. Arithmetic follows the reference's lane model: lerps as fma(n - l, f, l),
 * Sobel as fma(2 dm, 2, du + dd) x 1/512, accumulation by fused multiply-add. This file is built with -fmad=false:
 * every fused operation is written out.
 *
 * The driver is F32 where the reference's is long double. A position is kept as a whole pixel plus a small float
 * offset from it (the sub-pixel phase of the level's start plus the flow so far), so the bilinear phase keeps ~1e-6 px
 * of precision at any picture size; the determinant is formed by Kahan's fused-multiply-add product difference, and the
 * smaller eigenvalue as det / lambda_max, so neither cancels. No FP64 anywhere. */
#include <limits.h>

#include "vtg_internal.cuh"

#define LK_GRAD_SCALE (1.0f / 512.0f)
#define LK_Q6_INV (1.0f / 64.0f)

/* The checked build (-DVTG_CHECKED: vtg_build.py's libvtg_checked.so). Each patch operation first tests the rectangle
 * of pixels its loads touch against the level; one that would leave the level records its site in g_vtg_check (bit 1
 * the template build, 2 the window pass, 4 the sample pass) and returns zero sums without reading. The production build
 * has no test: the driver's bounds tests keep every rectangle inside the level by construction, and the checked build
 * is how the tests confirm it. */
#ifdef VTG_CHECKED
__device__ unsigned int g_vtg_check[2]; /* failed sites (bits), failures */

__device__ __forceinline__ bool lk_window_ok(const DevLevel &L, int x0, int x1, int y0, int y1, unsigned site)
{
    if (x0 >= 0 && y0 >= 0 && x1 < L.w && y1 < L.h)
        return true;
    if ((threadIdx.x & 31) == 0) {
        atomicOr(&g_vtg_check[0], site);
        atomicAdd(&g_vtg_check[1], 1u);
    }
    return false;
}
#define LK_CHECK_WINDOW(L, x0, x1, y0, y1, site, ...)                                                                   \
    do {                                                                                                               \
        if (!lk_window_ok(L, x0, x1, y0, y1, site)) {                                                                  \
            __VA_ARGS__;                                                                                               \
            return;                                                                                                    \
        }                                                                                                              \
    } while (0)
#else
#define LK_CHECK_WINDOW(L, x0, x1, y0, y1, site, ...)                                                                   \
    do {                                                                                                               \
    } while (0)
#endif

extern "C" int vtg_check_read(uint32_t *out)
{
    if (!out)
        return VTG_EINVAL;
    out[0] = out[1] = 0;
#ifdef VTG_CHECKED
    unsigned h[2] = {0u, 0u};
    if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpyFromSymbol(h, g_vtg_check, sizeof h) != cudaSuccess)
        return VTG_ECUDA;
    const unsigned z[2] = {0u, 0u};
    if (cudaMemcpyToSymbol(g_vtg_check, z, sizeof z) != cudaSuccess)
        return VTG_ECUDA;
    out[0] = h[0];
    out[1] = h[1];
    return 1;
#else
    return 0;
#endif
}

/* Two floats in one 64-bit register (lo, hi), for the packed FP32 pair instructions (add/sub/mul/fma .f32x2): one
 * instruction moves two independent row chains of a patch. Each half rounds like its scalar instruction. */
typedef unsigned long long f2_t;

__device__ __forceinline__ f2_t f2_pack(float lo, float hi)
{
    f2_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_split(f2_t v, float &lo, float &hi)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ float f2_hi(f2_t v)
{
    float lo, hi;
    f2_split(v, lo, hi);
    return hi;
}
__device__ __forceinline__ float f2_sum(f2_t v)
{
    float lo, hi;
    f2_split(v, lo, hi);
    return lo + hi;
}
__device__ __forceinline__ f2_t f2_add(f2_t a, f2_t b)
{
    f2_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_sub(f2_t a, f2_t b)
{
    f2_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_mul(f2_t a, f2_t b)
{
    f2_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2_t f2_fma(f2_t a, f2_t b, f2_t c)
{
    f2_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
/* |lo|, |hi|: both sign bits cleared */
__device__ __forceinline__ f2_t f2_abs(f2_t v) { return v & 0x7fffffff7fffffffull; }

/* The template of the current level, patch rows paired as (r, HH + r), HH = MAXH / 2, so the sample walks the top and
 * bottom halves of the patch together; an odd MAXH's last row (2 HH) is kept apart. Tx, Ty are the unscaled Sobel sums
 * (the 1/512 is applied to the folded sums, an exact power of two). T is in registers or, with TS, in this warp's
 * rows of shared memory ([HH][32] pairs: a lane reads only what it wrote). */
template <int MAXH, bool TS>
struct Patch {
    static constexpr int HH = MAXH / 2;
    f2_t tx[HH], ty[HH];
    f2_t t[TS ? 1 : HH];
    float txl, tyl, tl;
    f2_t *ts;
};

template <int MAXH, bool TS>
__device__ __forceinline__ void put_t(Patch<MAXH, TS> &P, int r, int lane, f2_t v)
{
    if constexpr (TS)
        P.ts[r * 32 + lane] = v;
    else
        P.t[r] = v;
}

template <int MAXH, bool TS>
__device__ __forceinline__ f2_t get_t(const Patch<MAXH, TS> &P, int r, int lane)
{
    if constexpr (TS)
        return P.ts[r * 32 + lane];
    else
        return P.t[r];
}

__device__ __forceinline__ float warp_fold(float v)
{
#pragma unroll
    for (int s = 1; s < 32; s <<= 1)
        v = v + __shfl_xor_sync(VTG_FULL, v, s);
    return v;
}

/* Two butterfly folds at once (the same partners, the same order of additions as warp_fold on each half). */
__device__ __forceinline__ void warp_fold2(float &a, float &b)
{
    f2_t v = f2_pack(a, b);
#pragma unroll
    for (int s = 1; s < 32; s <<= 1) {
        float lo, hi;
        f2_split(v, lo, hi);
        v = f2_add(v, f2_pack(__shfl_xor_sync(VTG_FULL, lo, s), __shfl_xor_sync(VTG_FULL, hi, s)));
    }
    f2_split(v, a, b);
}

/* Eight butterfly folds at once, the same partners and the same order of additions as warp_fold on each (so the same
 * sums, bit for bit), in 17 shuffles instead of 40: over stride 1 a lane keeps the four values its bit 0 selects and
 * sends the other four, over stride 2 two of those by bit 1, over stride 4 one by bit 2; strides 8 and 16 fold the one
 * left. Value k's total then sits in the lanes whose bits 0, 1, 2 spell k (from its high bit down), and the first N are
 * broadcast. */
template <int N>
__device__ __forceinline__ void warp_fold8(float (&v)[8])
{
    const int lane = threadIdx.x & 31;
    const bool b0 = lane & 1, b1 = lane & 2, b2 = lane & 4;
    float a[4], c[2];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float keep = b0 ? v[4 + k] : v[k], send = b0 ? v[k] : v[4 + k];
        a[k] = keep + __shfl_xor_sync(VTG_FULL, send, 1);
    }
#pragma unroll
    for (int k = 0; k < 2; k++) {
        const float keep = b1 ? a[2 + k] : a[k], send = b1 ? a[k] : a[2 + k];
        c[k] = keep + __shfl_xor_sync(VTG_FULL, send, 2);
    }
    float t = (b2 ? c[1] : c[0]) + __shfl_xor_sync(VTG_FULL, b2 ? c[0] : c[1], 4);
    t = t + __shfl_xor_sync(VTG_FULL, t, 8);
    t = t + __shfl_xor_sync(VTG_FULL, t, 16);
#pragma unroll
    for (int k = 0; k < N; k++)
        v[k] = __shfl_sync(VTG_FULL, t, (k >> 2) | (((k >> 1) & 1) << 1) | ((k & 1) << 2));
}

/* The row's horizontal interpolation at this lane's column: l from this lane's load, n from the next lane's. Every lane
 * loads (a clamped column for lanes past the window), so the load needs no predicate. */
__device__ __forceinline__ float hlerp(const float *p, float fx)
{
    const float l = __ldg(p);
    const float n = __shfl_down_sync(VTG_FULL, l, 1);
    return __fmaf_rn(n - l, fx, l);
}

/* hlerp of two rows at once, (row a, row b); FX = (fx, fx) */
__device__ __forceinline__ f2_t hlerp2(const float *pa, const float *pb, f2_t FX)
{
    const float la = __ldg(pa), lb = __ldg(pb);
    const f2_t l = f2_pack(la, lb);
    const f2_t n = f2_pack(__shfl_down_sync(VTG_FULL, la, 1), __shfl_down_sync(VTG_FULL, lb, 1));
    return f2_fma(f2_sub(n, l), FX, l);
}

/* build: the window of I around pixel (ix + fx, iy + fy); T, Tx, Ty into the patch; the tensor's sums; tc (the
 * patch's centre value on its first row) and C = sum (T - tc) Tx, sum (T - tc) Ty for the correlation below.
 * S row s is the bilinear row between image rows y0 + s and y0 + s + 1; patch row k takes its Sobel from S rows k - 1,
 * k, k + 1. The top half (rows 0 .. HH - 1, S rows -1 .. HH) and the bottom half (rows HH .. 2 HH - 1, S rows HH - 1
 * .. 2 HH) run as the two halves of packed pairs, each with its own three-row window, so each pair of rows lands in
 * the patch's pair register directly; an odd height's last row continues the bottom half. Not EXACT: rows from H on
 * read the last image row again and are zero in Tx, Ty. */
template <int MAXH, bool EXACT, bool TS>
__device__ __forceinline__ void lk_build(const DevLevel &L, int ix, float fx, int iy, float fy, int W, int Hr, int lane,
                                         Patch<MAXH, TS> &P, float &gxx, float &gxy, float &gyy, float &tco,
                                         float &cxo, float &cyo)
{
    constexpr int HH = MAXH / 2;
    const int H = EXACT ? MAXH : Hr;
    const int x0 = ix - W / 2, y0 = iy - H / 2;
    LK_CHECK_WINDOW(L, x0 - 1, x0 + W + 1, y0 - 1, y0 + H + 1, 1u, gxx = gxy = gyy = tco = cxo = cyo = 0.0f);
    /* Lane c samples window column c - 1 (c = 0 .. W + 1; lane W + 2 feeds lane W + 1's right neighbour; the lanes past
     * it read a clamped column and feed nothing). Patch columns are lanes 1 .. W; the others' sums are dropped before
     * the fold. */
    const bool act = lane >= 1 && lane <= W;
    const float *col = L.p + (x0 - 1 + min(lane, W + 2));
    /* image row y0 + r, r in -1 .. H + 1 (rows past that are read as row H + 1) */
    auto img = [&](int r) { return col + (size_t)(y0 + (EXACT ? r : min(r, H + 1))) * L.pitch; };
    const f2_t FX = f2_pack(fx, fx), FY = f2_pack(fy, fy), TWO = f2_pack(2.0f, 2.0f);
    const float *pa = img(-1), *pb = img(HH - 1);
    f2_t prev = hlerp2(pa, pb, FX);
    /* S rows k - 1, k, k + 1 of each half: values, and their x + 1 minus x - 1 differences */
    f2_t u = 0ull, ul = 0ull, ur = 0ull, m = 0ull, ml = 0ull, mr = 0ull, mdx = 0ull, udx = 0ull;
    f2_t sxx = 0ull, sxy = 0ull, syy = 0ull, scx = 0ull, scy = 0ull, TC = 0ull, hu2 = 0ull, hm2 = 0ull;
    float tc = 0.0f;
#pragma unroll
    for (int t = 0; t < HH + 2; t++) {
        if (EXACT || t < H + 2) {
            if (EXACT) {
                pa += L.pitch;
                pb += L.pitch;
            } else {
                pa = img(t);
                pb = img(HH + t);
            }
            const f2_t cur = hlerp2(pa, pb, FX);
            const f2_t d = f2_fma(f2_sub(cur, prev), FY, prev);
            prev = cur;
            float dlo, dhi;
            f2_split(d, dlo, dhi);
            const f2_t dl = f2_pack(__shfl_up_sync(VTG_FULL, dlo, 1), __shfl_up_sync(VTG_FULL, dhi, 1));
            const f2_t dr = f2_pack(__shfl_down_sync(VTG_FULL, dlo, 1), __shfl_down_sync(VTG_FULL, dhi, 1));
            const f2_t ddx = f2_sub(dr, dl);
            if (t >= 2) {
                const int k = t - 2; /* rows k and HH + k */
                f2_t tx = f2_fma(mdx, TWO, f2_add(udx, ddx));
                /* Sobel y as the horizontal smoothing (l + 2 c + r) of S row k + 1 less that of S row k - 1, the
                 * latter kept from two steps back */
                f2_t ty = f2_sub(f2_fma(d, TWO, f2_add(dl, dr)), hu2);
                if (!EXACT) {
                    const f2_t keep = f2_pack(k < H ? 1.0f : 0.0f, HH + k < H ? 1.0f : 0.0f);
                    tx = f2_mul(tx, keep);
                    ty = f2_mul(ty, keep);
                }
                if (k == 0) {
                    float mlo, mhi;
                    f2_split(m, mlo, mhi);
                    tc = __shfl_sync(VTG_FULL, mlo, W / 2 + 1);
                    TC = f2_pack(tc, tc);
                }
                put_t(P, k, lane, m);
                P.tx[k] = tx;
                P.ty[k] = ty;
                sxx = f2_fma(tx, tx, sxx);
                sxy = f2_fma(tx, ty, sxy);
                syy = f2_fma(ty, ty, syy);
                const f2_t tt = f2_sub(m, TC);
                scx = f2_fma(tt, tx, scx);
                scy = f2_fma(tt, ty, scy);
            }
            hu2 = hm2; hm2 = f2_fma(d, TWO, f2_add(dl, dr));
            u = m; ul = ml; ur = mr; udx = mdx;
            m = d; ml = dl; mr = dr; mdx = ddx;
        }
    }
    float fxx = f2_sum(sxx), fxy = f2_sum(sxy), fyy = f2_sum(syy), fcx = f2_sum(scx), fcy = f2_sum(scy);
    if constexpr ((MAXH & 1) != 0) {
        /* the last row, 2 HH: one more step of the bottom half (S row 2 HH + 1, image rows H, H + 1) */
        if (EXACT || H == MAXH) {
            const float c1 = hlerp(EXACT ? pb + L.pitch : img(H + 1), fx);
            const float p1 = f2_hi(prev);
            const float d = __fmaf_rn(c1 - p1, fy, p1);
            const float dl = __shfl_up_sync(VTG_FULL, d, 1), dr = __shfl_down_sync(VTG_FULL, d, 1);
            const float tx = __fmaf_rn(f2_hi(mdx), 2.0f, f2_hi(udx) + (dr - dl));
            const float ty = __fmaf_rn(d - f2_hi(u), 2.0f, (dl - f2_hi(ul)) + (dr - f2_hi(ur)));
            const float mt = f2_hi(m);
            P.tl = mt;
            P.txl = tx;
            P.tyl = ty;
            fxx = __fmaf_rn(tx, tx, fxx);
            fxy = __fmaf_rn(tx, ty, fxy);
            fyy = __fmaf_rn(ty, ty, fyy);
            fcx = __fmaf_rn(mt - tc, tx, fcx);
            fcy = __fmaf_rn(mt - tc, ty, fcy);
        } else {
            P.tl = P.txl = P.tyl = 0.0f;
        }
    }
    if constexpr (!EXACT) {
        /* rows the loop did not reach (t >= H + 2): zero */
#pragma unroll
        for (int k = 0; k < HH; k++)
            if (k + 2 >= H + 2) {
                P.tx[k] = 0ull;
                P.ty[k] = 0ull;
                put_t(P, k, lane, 0ull);
            }
    }
    /* (Sobel / 512)^2 = Sobel^2 x 2^-18, exact */
    fxx = act ? fxx : 0.0f;
    fxy = act ? fxy : 0.0f;
    fyy = act ? fyy : 0.0f;
    fcx = act ? fcx : 0.0f;
    fcy = act ? fcy : 0.0f;
    float fv[8] = {fxx, fxy, fyy, fcx, fcy, 0.0f, 0.0f, 0.0f};
    warp_fold8<5>(fv);
    fxx = fv[0];
    fxy = fv[1];
    fyy = fv[2];
    fcx = fv[3];
    fcy = fv[4];
    gxx = fxx * (LK_GRAD_SCALE * LK_GRAD_SCALE);
    gxy = fxy * (LK_GRAD_SCALE * LK_GRAD_SCALE);
    gyy = fyy * (LK_GRAD_SCALE * LK_GRAD_SCALE);
    tco = tc;
    cxo = fcx;
    cyo = fcy;
}

/* iterate's sums for every sub-pixel phase at one whole-pixel position. Bilinear sampling is linear in J's four
 * whole-pixel shifts, so with J' = J - tc,
 *     sum (T - J(p + q)) Tx = C - [lerp_y(lerp_x(X00, X10, fx), lerp_x(X01, X11, fx), fy)],
 *     X_ab = sum over the patch of J'(x0 + col + a, y0 + row + b) Tx,   C = sum (T - tc) Tx
 * (the tc terms cancel, since the weights sum to 1). One pass over the window gives X for Tx (X[0..3]) and Ty
 * (X[4..7]); every iteration that stays at the same whole pixel then needs only these eight numbers. Subtracting tc
 * keeps the sums near the patch's contrast, not its brightness, so F32 rounding stays far below 1e-4 px. Rows as in
 * lk_sample: the top and bottom halves of the patch as the two halves of packed pairs. */
template <int MAXH, bool EXACT, bool TS>
__device__ __forceinline__ void lk_correlate(const DevLevel &L, int jx, int jy, int W, int Hr, int lane,
                                             const Patch<MAXH, TS> &P, float tc, float (&X)[8])
{
    constexpr int HH = MAXH / 2;
    const int H = EXACT ? MAXH : Hr;
    const int x0 = jx - W / 2, y0 = jy - H / 2;
    LK_CHECK_WINDOW(L, x0 - 1, x0 + W, y0, y0 + H, 2u, for (int k = 0; k < 8; k++) X[k] = 0.0f);
    const bool act = lane >= 1 && lane <= W;
    const float *col = L.p + (size_t)y0 * L.pitch + (x0 - 1 + min(lane, W + 1));
    const float *ra = col;
    const float *rb = col + (size_t)(EXACT ? HH : min(HH, H)) * L.pitch;
    const f2_t M = f2_pack(-tc, -tc);
    /* a row pair: l = J' at this lane's column, n = J' at the next column (the next lane's l) */
    auto load = [&](const float *pa, const float *pb, f2_t &l, f2_t &n) {
        l = f2_add(f2_pack(__ldg(pa), __ldg(pb)), M);
        float a, b;
        f2_split(l, a, b);
        n = f2_pack(__shfl_down_sync(VTG_FULL, a, 1), __shfl_down_sync(VTG_FULL, b, 1));
    };
    f2_t pl, pn;
    load(ra, rb, pl, pn);
    f2_t a00 = 0ull, a10 = 0ull, a01 = 0ull, a11 = 0ull, b00 = 0ull, b10 = 0ull, b01 = 0ull, b11 = 0ull;
#pragma unroll
    for (int r = 0; r < HH; r++) {
        if (EXACT || r < H) {
            ra += L.pitch;
            if (EXACT)
                rb += L.pitch;
            else
                rb = col + (size_t)min(HH + 1 + r, H) * L.pitch;
            f2_t cl, cn;
            load(ra, rb, cl, cn);
            a00 = f2_fma(pl, P.tx[r], a00);
            a10 = f2_fma(pn, P.tx[r], a10);
            a01 = f2_fma(cl, P.tx[r], a01);
            a11 = f2_fma(cn, P.tx[r], a11);
            b00 = f2_fma(pl, P.ty[r], b00);
            b10 = f2_fma(pn, P.ty[r], b10);
            b01 = f2_fma(cl, P.ty[r], b01);
            b11 = f2_fma(cn, P.ty[r], b11);
            pl = cl;
            pn = cn;
        }
    }
    X[0] = f2_sum(a00);
    X[1] = f2_sum(a10);
    X[2] = f2_sum(a01);
    X[3] = f2_sum(a11);
    X[4] = f2_sum(b00);
    X[5] = f2_sum(b10);
    X[6] = f2_sum(b01);
    X[7] = f2_sum(b11);
    if constexpr ((MAXH & 1) != 0) {
        if (EXACT || H == MAXH) {
            /* the last row follows the bottom half: its previous row is the pairs' high halves */
            const float l = __ldg(EXACT ? rb + L.pitch : col + (size_t)H * L.pitch) - tc;
            const float n = __shfl_down_sync(VTG_FULL, l, 1);
            const float ol = f2_hi(pl), on = f2_hi(pn);
            X[0] = __fmaf_rn(ol, P.txl, X[0]);
            X[1] = __fmaf_rn(on, P.txl, X[1]);
            X[2] = __fmaf_rn(l, P.txl, X[2]);
            X[3] = __fmaf_rn(n, P.txl, X[3]);
            X[4] = __fmaf_rn(ol, P.tyl, X[4]);
            X[5] = __fmaf_rn(on, P.tyl, X[5]);
            X[6] = __fmaf_rn(l, P.tyl, X[6]);
            X[7] = __fmaf_rn(n, P.tyl, X[7]);
        }
    }
#pragma unroll
    for (int k = 0; k < 8; k++)
        X[k] = act ? X[k] : 0.0f;
    warp_fold8<8>(X);
}

/* sum (T - J) T_grad at phase (fx, fy) from the correlation's four shifts and C, before the Sobel scale (which the
 * walk folds into G^-1: a power of two, so the products round the same). X holds the shifts (0, 0) and (0, 1) and the
 * x differences (1, 0) - (0, 0), (1, 1) - (0, 1), formed once a window pass (lk_phase_diffs): the same values each
 * iteration would form. */
__device__ __forceinline__ float lk_at_phase(const float *X, float C, float fx, float fy)
{
    const float r0 = __fmaf_rn(X[1], fx, X[0]), r1 = __fmaf_rn(X[3], fx, X[2]);
    return C - __fmaf_rn(r1 - r0, fy, r0);
}
__device__ __forceinline__ void lk_phase_diffs(float (&X)[8])
{
#pragma unroll
    for (int k = 0; k < 8; k += 2)
        X[k + 1] -= X[k];
}

/* iterate (RESID = false): J at pixel (jx + fx, jy + fy); the sums of It Tx and It Ty.
 * residual (RESID = true): the sums of |It| and It^2, It in 8-bit grey.
 * The top half's rows (image rows y0 .. y0 + HH) and the bottom half's (y0 + HH .. y0 + 2 HH) run as the two halves
 * of packed pairs, each carrying its own previous row; an odd height's last row follows the bottom half. With a height
 * below MAXH (not EXACT), bottom-half rows past H read row H again and count for nothing (zero Tx, Ty; masked It). */
template <int MAXH, bool EXACT, bool RESID, bool TS>
__device__ __forceinline__ void lk_sample(const DevLevel &L, int jx, float fx, int jy, float fy, int W, int Hr, int lane,
                                          const Patch<MAXH, TS> &P, float &b0, float &b1)
{
    constexpr int HH = MAXH / 2;
    const int H = EXACT ? MAXH : Hr;
    const int x0 = jx - W / 2, y0 = jy - H / 2;
    LK_CHECK_WINDOW(L, x0 - 1, x0 + W, y0, y0 + H, 4u, b0 = b1 = 0.0f);
    const bool act = lane >= 1 && lane <= W;
    const float q6 = act ? LK_Q6_INV : 0.0f;
    const float *col = L.p + (size_t)y0 * L.pitch + (x0 - 1 + min(lane, W + 1));
    const float *ra = col;
    const float *rb = col + (size_t)(EXACT ? HH : min(HH, H)) * L.pitch;
    const f2_t FX = f2_pack(fx, fx), FY = f2_pack(fy, fy);
    f2_t prev = hlerp2(ra, rb, FX);
    /* It Tx, It Ty: pairs of even and of odd r in separate chains */
    f2_t s0 = 0ull, s1 = 0ull, s2 = 0ull, s3 = 0ull; /* (+0, +0) */
#pragma unroll
    for (int r = 0; r < HH; r++) {
        if (EXACT || r < H) {
            ra += L.pitch;
            if (EXACT)
                rb += L.pitch;
            else
                rb = col + (size_t)min(HH + 1 + r, H) * L.pitch;
            const f2_t cur = hlerp2(ra, rb, FX);
            const f2_t it = f2_sub(get_t(P, r, lane), f2_fma(f2_sub(cur, prev), FY, prev));
            prev = cur;
            if (RESID) {
                const f2_t g = f2_mul(it, f2_pack(q6, (EXACT || HH + r < H) ? q6 : 0.0f));
                s0 = f2_add(s0, f2_abs(g));
                s1 = f2_fma(g, g, s1);
            } else if (r & 1) {
                s2 = f2_fma(it, P.tx[r], s2);
                s3 = f2_fma(it, P.ty[r], s3);
            } else {
                s0 = f2_fma(it, P.tx[r], s0);
                s1 = f2_fma(it, P.ty[r], s1);
            }
        }
    }
    if (!RESID) {
        s0 = f2_add(s0, s2);
        s1 = f2_add(s1, s3);
    }
    float t0 = f2_sum(s0), t1 = f2_sum(s1);
    if constexpr ((MAXH & 1) != 0) {
        if (EXACT || H == MAXH) {
            const float cur = hlerp(EXACT ? rb + L.pitch : col + (size_t)H * L.pitch, fx);
            const float pb = f2_hi(prev);
            const float it = P.tl - __fmaf_rn(cur - pb, fy, pb);
            if (RESID) {
                const float g = it * q6;
                t0 = t0 + fabsf(g);
                t1 = __fmaf_rn(g, g, t1);
            } else {
                t0 = __fmaf_rn(it, P.txl, t0);
                t1 = __fmaf_rn(it, P.tyl, t1);
            }
        }
    }
    if (!RESID) {
        t0 = act ? t0 : 0.0f;
        t1 = act ? t1 : 0.0f;
    }
    warp_fold2(t0, t1);
    /* iterate: It Tx / 512, the gradient scale applied to the folded sums (exact) */
    b0 = RESID ? t0 : t0 * LK_GRAD_SCALE;
    b1 = RESID ? t1 : t1 * LK_GRAD_SCALE;
}

/* Two warps on one point (NW = 2): each takes half the patch's rows, and after every pass over them the pair adds its
 * partial sums. Lane 0 of each posts its warp's N folded sums to the pair's slot, both wait at the pair's named barrier
 * (64 threads), every lane adds the two in one order (the top half's first), and a second wait frees the slot. Both
 * warps then hold the same totals, so they take the same decisions in the walk. */
struct LkPair {
    float *slot; /* [2][8] floats in shared memory */
    int bar;     /* the pair's named barrier */
    int half;    /* 0: the top rows, 1: the bottom rows */
};

template <int N>
__device__ __forceinline__ void pair_add(float (&v)[N], const LkPair &q, int lane)
{
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < N; k++)
            q.slot[q.half * 8 + k] = v[k];
    asm volatile("bar.sync %0, 64;" ::"r"(q.bar) : "memory");
#pragma unroll
    for (int k = 0; k < N; k++)
        v[k] = q.slot[k] + q.slot[8 + k];
    asm volatile("bar.sync %0, 64;" ::"r"(q.bar) : "memory");
}

/* A position as whole pixel + offset: floor and phase of base + t, base a whole number. */
__device__ __forceinline__ void split(int base, float t, int &i, float &f)
{
    const float ft = floorf(t);
    i = base + (int)ft;
    f = t - ft;
}

/* The pyramid walk (src/kern/lk_driver.inc:7-109), warp-uniform, F32. */
/* The work one point's walks did, for counting runs (vtg_batch_count): template builds, window passes, residual passes
 * and iterations, packed into one warp-uniform word (LK_WORK_* shifts). */
#define LK_WORK_BUILD 1u
#define LK_WORK_RESID (1u << 5)
#define LK_WORK_PASS (1u << 8)
#define LK_WORK_ITER (1u << 16)

template <int MAXH, bool EXACT, bool TS, int NW = 1>
__device__ __forceinline__ void lk_track(const DevPyr &I, const DevPyr &J, int top, const LkPrm &p, float x, float y,
                                         float gx0, float gy0, int lane, Patch<MAXH, TS> &P, vtg_lk_out &o,
                                         unsigned &work, const LkPair &q = LkPair{nullptr, 0, 0})
{
    /* NW = 2: the patch's rows split as Ht = ceil(H / 2) on top and the rest below; this warp's Hs rows start `off`
     * rows down, so its passes see a patch of Hs rows whose centre row sits dy rows below the point's */
    const int Hf = NW == 2 ? p.H : (EXACT ? MAXH : p.H);
    const int Ht = (Hf + 1) / 2, off = NW == 2 && q.half ? Ht : 0;
    const int W = p.W, H = NW == 2 ? (q.half ? Hf - Ht : Ht) : Hf;
    const int dy = NW == 2 ? off + H / 2 - Hf / 2 : 0;
    const int mx = W / 2 + 1, my = Hf / 2 + 1;
    /* scalings by 2^-L are products with an exact power of two (levels stay far from the exponent's limits): the
     * same bits as ldexpf, in one instruction */
    const float stop = __int_as_float((127 - top) << 23);
    float gx = gx0 * stop, gy = gy0 * stop;
    int status = 0, iters = 0;
    bool valid0 = false;
    float eig0 = 0.0f, idet0 = 0.0f, gxx0 = 0.0f, gxy0 = 0.0f, gyy0 = 0.0f;
    for (int L = top; L >= 0; L--) {
        const DevLevel IL = I.l[L], JL = J.l[L];
        const float sl = __int_as_float((127 - L) << 23);
        const float px = x * sl, py = y * sl; /* exact */
        /* written so that NaN fails it: a caller's NaN point is out, never a window at a garbage place */
        if (!(px >= (float)mx && py >= (float)my && px < (float)(IL.w - mx - 1) && py < (float)(IL.h - my - 1))) {
            if (L == 0)
                status |= VTG_LK_OUT;
            else {
                gx *= 2.0f;
                gy *= 2.0f;
            }
            continue;
        }
        const float fpx = floorf(px), fpy = floorf(py);
        const int bx = (int)fpx, by = (int)fpy;
        const float rx = px - fpx, ry = py - fpy; /* exact */
        float gxx, gxy, gyy, tc, cx, cy;
        lk_build<MAXH, EXACT, TS>(IL, bx, rx, by + dy, ry, W, H, lane, P, gxx, gxy, gyy, tc, cx, cy);
        if constexpr (NW == 2) { /* tc stays each half's own: its terms cancel within the half */
            float v[5] = {gxx, gxy, gyy, cx, cy};
            pair_add(v, q, lane);
            gxx = v[0];
            gxy = v[1];
            gyy = v[2];
            cx = v[3];
            cy = v[4];
        }
        work += LK_WORK_BUILD;
        /* det = gxx gyy - gxy^2 by Kahan's product difference; the smaller eigenvalue as det / lambda_max. */
        const float w2 = gxy * gxy;
        const float e2 = __fmaf_rn(gxy, gxy, -w2);
        const float det = __fmaf_rn(gxx, gyy, -w2) - e2;
        const float tr = gxx + gyy, df = gxx - gyy;
        const float root = sqrtf(__fmaf_rn(df, df, 4.0f * w2));
        const float lmax = 0.5f * (tr + root);
        /* the threshold test and min_eig's report need no correctly rounded quotient: the fast division's 2 ulp */
        const float eig = lmax > 0.0f ? __fdividef(det, lmax * p.area) : 0.0f;
        if (L == 0)
            eig0 = eig;
        if (eig < p.min_eig || det <= 0.0f) {
            if (L == 0)
                status |= VTG_LK_LOWEIG;
            else {
                gx *= 2.0f;
                gy *= 2.0f;
            }
            continue;
        }
        const float idet = __frcp_rn(det);
        if (L == 0) {
            idet0 = idet;
            gxx0 = gxx;
            gxy0 = gxy;
            gyy0 = gyy;
            valid0 = true;
        }
        /* G^-1 / 64: b arrives in Q6 grey x 8-bit grey per pixel; times the Sobel scale of b's sums, exact (a power of
         * two far from the exponent's limits at these magnitudes), so each product below rounds as it would with b
         * scaled first */
        const float ia = gyy * idet * LK_Q6_INV * LK_GRAD_SCALE, ib = -gxy * idet * LK_Q6_INV * LK_GRAD_SCALE,
                    ic = gxx * idet * LK_Q6_INV * LK_GRAD_SCALE;
        const float lo_x = (float)(mx - bx), lo_y = (float)(my - by);
        const float hi_x = (float)(JL.w - mx - 1 - bx), hi_y = (float)(JL.h - my - 1 - by);
        float vx = 0.0f, vy = 0.0f;
        /* the correlation at the last whole pixel sampled (none yet on this level) */
        float X[8];
        int cjx = INT_MIN, cjy = INT_MIN;
        for (int it = 0; it < p.max_iter; it++) {
            const float qx = (rx + gx) + vx, qy = (ry + gy) + vy; /* offsets from (bx, by) */
            if (!(qx >= lo_x && qy >= lo_y && qx < hi_x && qy < hi_y)) { /* NaN fails it too (a NaN guess) */
                if (L == 0) {
                    status |= VTG_LK_OUT;
                    valid0 = false;
                }
                break;
            }
            int jx, jy;
            float fx, fy;
            split(bx, qx, jx, fx);
            split(by, qy, jy, fy);
            if (jx != cjx || jy != cjy) {
                lk_correlate<MAXH, EXACT, TS>(JL, jx, jy + dy, W, H, lane, P, tc, X);
                if constexpr (NW == 2)
                    pair_add(X, q, lane);
                lk_phase_diffs(X);
                work += LK_WORK_PASS;
                cjx = jx;
                cjy = jy;
            }
            const float sx = lk_at_phase(X, cx, fx, fy), sy = lk_at_phase(X + 4, cy, fx, fy);
            const float ex = __fmaf_rn(ia, sx, ib * sy), ey = __fmaf_rn(ib, sx, ic * sy);
            vx += ex;
            vy += ey;
            iters++;
            work += LK_WORK_ITER;
            if (__fmaf_rn(ex, ex, ey * ey) < p.eps2)
                break;
        }
        gx += vx;
        gy += vy;
        if (L > 0) {
            gx *= 2.0f;
            gy *= 2.0f;
        }
    }
    o.x = x + gx;
    o.y = y + gy;
    o.min_eig = eig0;
    o.iters = (uint16_t)iters;
    o.residual = 0.0f;
    o.cov_xx = o.cov_xy = o.cov_yy = 0.0f;
    if (valid0 && !status) {
        const DevLevel J0 = J.l[0];
        const float fx0 = floorf(x), fy0 = floorf(y);
        const int bx = (int)fx0, by = (int)fy0;
        const float qx = (x - fx0) + gx, qy = (y - fy0) + gy;
        if (!(qx >= (float)(mx - bx) && qy >= (float)(my - by) && qx < (float)(J0.w - mx - 1 - bx) &&
              qy < (float)(J0.h - my - 1 - by))) {
            status |= VTG_LK_OUT;
        } else {
            int jx, jy;
            float fx, fy;
            split(bx, qx, jx, fx);
            split(by, qy, jy, fy);
            float sa, ss;
            lk_sample<MAXH, EXACT, true, TS>(J0, jx, fx, jy + dy, fy, W, H, lane, P, sa, ss);
            if constexpr (NW == 2) {
                float v[2] = {sa, ss};
                pair_add(v, q, lane);
                sa = v[0];
                ss = v[1];
            }
            work += LK_WORK_RESID;
            const float r0 = sa / p.area, r1 = ss / p.area;
            o.residual = r0;
            if (r0 > p.max_residual)
                status |= VTG_LK_RESIDUAL;
            const float s2 = r1 * p.area / (p.area - 2.0f);
            o.cov_xx = s2 * gyy0 * idet0;
            o.cov_xy = -s2 * gxy0 * idet0;
            o.cov_yy = s2 * gxx0 * idet0;
        }
    }
    o.status = (uint16_t)status;
}

/* lk_track then, when asked and the track is good, the forward-backward check (src/kern/lk_driver.inc:111-121): the
 * found point tracked back from J to I from minus the found flow. One copy of the walk serves both passes. */
template <int MAXH, bool EXACT, bool TS, int NW = 1>
__device__ __forceinline__ void lk_point(const DevPyr &I, const DevPyr &J, int top, const LkPrm &p, float x, float y,
                                         float gx, float gy, int lane, Patch<MAXH, TS> &P, vtg_lk_out &o,
                                         unsigned &work, const LkPair &q = LkPair{nullptr, 0, 0})
{
    const int passes = p.fb_max2 > 0.0f ? 2 : 1;
    float sx = x, sy = y;
    for (int pass = 0; pass < passes; pass++) {
        vtg_lk_out r;
        lk_track<MAXH, EXACT, TS, NW>(pass ? J : I, pass ? I : J, top, p, sx, sy, gx, gy, lane, P, r, work, q);
        if (pass == 0) {
            o = r;
            if (o.status)
                break;
            sx = o.x;
            sy = o.y;
            gx = x - o.x;
            gy = y - o.y;
        } else {
            const float ex = r.x - x, ey = r.y - y;
            if (r.status || !(__fmaf_rn(ex, ex, ey * ey) <= p.fb_max2))
                o.status |= VTG_LK_FLOWBACK;
        }
    }
}

__device__ __forceinline__ void store_out(vtg_lk_out *dst, const vtg_lk_out &o, int lane)
{
    /* eight 4-byte words, one per lane */
    const uint32_t *src = reinterpret_cast<const uint32_t *>(&o);
    uint32_t w = 0;
#pragma unroll
    for (int k = 0; k < 8; k++)
        w = lane == k ? src[k] : w;
    if (lane < 8)
        reinterpret_cast<uint32_t *>(dst)[lane] = w;
}

/* Mean |J - I| over one cell of level 0, 8-bit grey (still.c:105-114). The differences are whole Q6 numbers, their sum
 * below 2^24, so the F32 sum is exact and the mean is one rounding, as in the reference. */
__device__ __forceinline__ float cell_diff(const DevLevel &A, const DevLevel &B, int col, int row, const CellGrid &g,
                                           int lane)
{
    const int x = col * g.cell_w, y0 = row * g.cell_h, y1 = min(y0 + g.cell_h, A.h);
    float s = 0.0f;
    /* a cell's row and column of element k: a shift and a mask for power-of-two widths (the 16 x 8 grid) */
    const bool p2 = (g.cell_w & (g.cell_w - 1)) == 0;
    const int sh = __ffs(g.cell_w) - 1;
    for (int k = lane; k < g.cell_w * (y1 - y0); k += 32) {
        const int kr = p2 ? k >> sh : k / g.cell_w, kc = p2 ? k & (g.cell_w - 1) : k % g.cell_w;
        const int yy = y0 + kr, xx = min(x + kc, A.w - 1);
        s += fabsf(__ldg(B.p + (size_t)yy * B.pitch + xx) - __ldg(A.p + (size_t)yy * A.pitch + xx));
    }
    s = warp_fold(s);
    return __fdiv_rn(s, (float)((y1 - y0) * g.cell_w)) * LK_Q6_INV;
}

/* One cell of a grid: its centre (cw c + cw / 2, ch r + ch / 2), clamped to where the patch fits (still.c:127-130),
 * LK with the forward-backward check, and the cell record (still.c:132-140). The whole warp calls it. */
/* Adds one point's work word to the four counters (template builds, residual passes, window passes, iterations). */
__device__ __forceinline__ void lk_count(unsigned long long *count, unsigned work, int lane)
{
    if (count && lane == 0) {
        atomicAdd(count + 0, (unsigned long long)(work & 31u));
        atomicAdd(count + 1, (unsigned long long)((work >> 5) & 7u));
        atomicAdd(count + 2, (unsigned long long)((work >> 8) & 255u));
        atomicAdd(count + 3, (unsigned long long)(work >> 16));
    }
}

template <int MAXH, bool EXACT, bool TS>
__device__ __forceinline__ void lk_cell(const DevPyr &I, const DevPyr &J, int top, const LkPrm &p, const CellGrid &g,
                                        int base_w, int base_h, int i, int lane, vtg_lk_out *__restrict__ out,
                                        vtg_cell *__restrict__ cells, f2_t *ts, unsigned long long *count = nullptr)
{
    const int col = i % g.cols, row = i / g.cols;
    const float mx = (float)(p.W / 2 + 2), my = (float)(p.H / 2 + 2);
    float x = (float)(col * g.cell_w + g.cell_w / 2), y = (float)(row * g.cell_h + g.cell_h / 2);
    x = fminf(fmaxf(x, mx), (float)base_w - 1.0f - mx);
    y = fminf(fmaxf(y, my), (float)base_h - 1.0f - my);
    Patch<MAXH, TS> P;
    P.ts = ts;
    vtg_lk_out o;
    unsigned work = 0;
    lk_point<MAXH, EXACT, TS>(I, J, top, p, x, y, 0.0f, 0.0f, lane, P, o, work);
    lk_count(count, work, lane);
    if (out)
        store_out(out + i, o, lane);
    if (cells) {
        const float diff = cell_diff(I.l[0], J.l[0], col, row, g, lane);
        if (lane == 0) {
            vtg_cell c;
            c.u = o.x - x;
            c.v = o.y - y;
            c.diff = diff;
            c.state = o.status;
            c.sigma = o.status ? 0.0f : sqrtf(o.cov_xx + o.cov_yy);
            c.pad = 0.0f;
            cells[i] = c;
        }
    }
}

template <int MAXH, bool EXACT>
__global__ void __launch_bounds__(256, 2) lk_cells_kernel(const DevPyr *__restrict__ Ip, const DevPyr *__restrict__ Jp,
                                                          int top, LkPrm p, CellGrid g, int base_w, int base_h,
                                                          vtg_lk_out *__restrict__ out, vtg_cell *__restrict__ cells)
{
    extern __shared__ f2_t s_tc[]; /* the template's T: 8 warps x (MAXH / 2) x 32 pairs */
    const int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (i >= g.n)
        return;
    lk_cell<MAXH, EXACT, true>(*Ip, *Jp, top, p, g, base_w, base_h, i, lane, out, cells,
                               s_tc + (size_t)(threadIdx.x >> 5) * (MAXH / 2) * 32);
}

/* Many streams' cells in one launch. Work items are runs of `chunk` cells of one job; job j's items start at
 * item_start[j]. PERSISTENT: a fixed grid whose warps take items from `counter` until none is left, so uneven streams
 * balance themselves; otherwise one warp per item. The cell code is the single-stream kernel's: a cell's result does
 * not depend on what else is in the batch.
 *
 * TILED (persistent only): a job's cells are walked in tiles of LK_TILE_W x LK_TILE_H cells (row-major inside a tile,
 * the tiles row-major over the grid; cells past the grid's edge are skipped), and each CTA takes whole tiles, tile
 * g x gridDim.x + blockIdx.x for g = 0, 1, ..., its warps taking the tile's items from a counter in shared memory. So
 * the cells a CTA runs at once are neighbours, whose windows overlap (at level L cells are 16 / 2^L by 8 / 2^L pixels
 * apart, under a 23 x 23 window), and the SM's L1 serves one cell's rows to the next. The tiles are dealt to the CTAs
 * in a fixed order, with no global counter. */
#define LK_BATCH_MAX_JOBS 512
#define LK_TILE_W 8
#define LK_TILE_H 4
#define LK_TILE_CELLS (LK_TILE_W * LK_TILE_H)

/* Cell of work index w of a grid walked in tiles, or -1 past the grid's edge. */
__device__ __forceinline__ int lk_tile_cell(const CellGrid &g, int w)
{
    const int tiles_x = (g.cols + LK_TILE_W - 1) / LK_TILE_W;
    const int t = w / LK_TILE_CELLS, u = w - t * LK_TILE_CELLS;
    const int col = (t % tiles_x) * LK_TILE_W + u % LK_TILE_W, row = (t / tiles_x) * LK_TILE_H + u / LK_TILE_W;
    return (col < g.cols && row < g.rows) ? row * g.cols + col : -1;
}

template <int MAXH, bool EXACT, bool PERSISTENT, int WARPS, int MINB, bool TS>
__global__ void __launch_bounds__(WARPS * 32, MINB) lk_batch_kernel(const LkJob *__restrict__ jobs,
                                                                    const int *__restrict__ item_start, int njobs,
                                                                    int items, int chunk, LkPrm p,
                                                                    int *__restrict__ counter,
                                                                    unsigned long long *__restrict__ count,
                                                                    int tiled)
{
    __shared__ int s_start[LK_BATCH_MAX_JOBS + 1];
    __shared__ int s_taken; /* tiled: the CTA's items taken so far */
    extern __shared__ f2_t s_t[]; /* TS: WARPS x (MAXH / 2) x 32 pairs */
    f2_t *ts = TS ? s_t + (size_t)(threadIdx.x >> 5) * (MAXH / 2) * 32 : nullptr;
    for (int k = threadIdx.x; k <= njobs; k += blockDim.x)
        s_start[k] = item_start[k]; /* the step's own table, written when it was prepared */
    if (threadIdx.x == 0)
        s_taken = 0;
    __syncthreads();
    vtg_grid_dependency_wait(); /* the pyramids and the counter, when launched as a dependent of the pyramid */
    const int lane = threadIdx.x & 31;
    const int per_tile = LK_TILE_CELLS / chunk; /* items of a tile (tiled: chunk divides LK_TILE_CELLS) */
    int item = PERSISTENT ? 0 : (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    for (;;) {
        if (PERSISTENT) {
            int t = 0;
            if (lane == 0) {
                if (tiled) {
                    /* Whole tiles to each CTA in turn (tile g x CTAs + its index), its warps taking the tile's items
                     * from s_taken: neighbouring cells on one SM. All but the last round of tiles; those items any
                     * warp of any CTA takes one by one from the global counter, so SMs whose tiles cost less pick up
                     * the rest instead of idling at the launch's end. */
                    const int i = atomicAdd(&s_taken, 1), g = i / per_tile;
                    const int tiles = (items + per_tile - 1) / per_tile, rounds = tiles / (int)gridDim.x;
                    const int fixed = (rounds > 1 ? rounds - 1 : 0) * (int)gridDim.x;
                    const int tile = g * (int)gridDim.x + (int)blockIdx.x;
                    t = tile < fixed ? tile * per_tile + (i - g * per_tile) : fixed * per_tile + atomicAdd(counter, 1);
                } else {
                    t = atomicAdd(counter, 1);
                }
            }
            item = __shfl_sync(VTG_FULL, t, 0);
        }
        if (item >= items)
            break;
        int lo = 0, hi = njobs;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_start[mid] <= item)
                lo = mid;
            else
                hi = mid;
        }
        const LkJob &jb = jobs[lo];
        const int c0 = (item - s_start[lo]) * chunk;
        for (int c = c0; c < c0 + chunk; c++) {
            const int cell = tiled ? lk_tile_cell(jb.g, c) : (c < jb.g.n ? c : -1);
            if (cell >= 0)
                lk_cell<MAXH, EXACT, TS>(*jb.I, *jb.J, jb.top, p, jb.g, jb.base_w, jb.base_h, cell, lane, jb.out,
                                         jb.cells, ts, count);
        }
        if (!PERSISTENT)
            break;
    }
}

template <int MAXH, bool EXACT>
static cudaError_t lk_batch_launch(const LkJob *jobs, const int *item_start, int njobs, int items, const LkPrm &p,
                                   const LkTune &t, int sms, int *counter, cudaStream_t s, bool pdl,
                                   unsigned long long *count)
{
#define LKB(P, WARPS, MINB)                                                                                            \
    do {                                                                                                               \
        const int blocks = P ? sms * t.ctas_per_sm : (items + WARPS - 1) / WARPS;                                      \
        const cudaError_t e = vtg_launch_k(lk_batch_kernel<MAXH, EXACT, P, WARPS, MINB, false>, blocks, WARPS * 32, 0, \
                                           s, pdl, jobs, item_start, njobs, items, t.chunk, p, counter, count,         \
                                           P ? t.tiled : 0);                                                           \
        if (e != cudaSuccess)                                                                                          \
            return e;                                                                                                  \
    } while (0)
#define LKT(WARPS, MINB)                                                                                               \
    do {                                                                                                               \
        /* WARPS x (MAXH / 2) x 32 pairs: at most 60 KB (16 warps, MAXH 31) */                                       \
        const size_t smem = sizeof(f2_t) * WARPS * (MAXH / 2) * 32;                                                  \
        if (smem > 48 * 1024) {                                                                                        \
            const cudaError_t e = cudaFuncSetAttribute(lk_batch_kernel<MAXH, EXACT, true, WARPS, MINB, true>,          \
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);        \
            if (e != cudaSuccess)                                                                                      \
                return e;                                                                                              \
        }                                                                                                              \
        const cudaError_t e2 = vtg_launch_k(lk_batch_kernel<MAXH, EXACT, true, WARPS, MINB, true>,                    \
                                            sms * t.ctas_per_sm, WARPS * 32, smem, s, pdl, jobs, item_start, njobs,    \
                                            items, t.chunk, p, counter, count, t.tiled);                               \
        if (e2 != cudaSuccess)                                                                                         \
            return e2;                                                                                                 \
    } while (0)
    if (t.tsmem) {
        /* the template's T in shared memory: fewer registers, or more warps an SM */
        if (t.block_warps == 4)
            LKT(4, 5);
        else if (t.block_warps == 16)
            LKT(16, 1);
        else
            LKT(8, 3);
    } else if (t.persistent) {
        if (t.block_warps == 4)
            LKB(true, 4, 4);
        else if (t.block_warps == 16)
            LKB(true, 16, 1);
        else
            LKB(true, 8, 2);
    } else {
        if (t.block_warps == 4)
            LKB(false, 4, 4);
        else if (t.block_warps == 16)
            LKB(false, 16, 1);
        else
            LKB(false, 8, 2);
    }
#undef LKB
#undef LKT
    return cudaGetLastError();
}

cudaError_t vtg_launch_lk_batch(const LkJob *jobs, const int *item_start, int njobs, int items, const LkPrm &p,
                                const LkTune &tune, int sms, int *counter, cudaStream_t s, bool pdl,
                                unsigned long long *count)
{
    if (njobs < 1 || njobs > LK_BATCH_MAX_JOBS || items <= 0)
        return items <= 0 ? cudaSuccess : cudaErrorInvalidValue;
    if (p.H == 21)
        return lk_batch_launch<21, true>(jobs, item_start, njobs, items, p, tune, sms, counter, s, pdl, count);
    if (p.H == 15)
        return lk_batch_launch<15, true>(jobs, item_start, njobs, items, p, tune, sms, counter, s, pdl, count);
    return lk_batch_launch<31, false>(jobs, item_start, njobs, items, p, tune, sms, counter, s, pdl, count);
}

template <int MAXH, bool EXACT>
__global__ void __launch_bounds__(256, 2) lk_points_kernel(const DevPyr *__restrict__ Ip, const DevPyr *__restrict__ Jp,
                                                        int top, LkPrm p, int n, const float *__restrict__ xs,
                                                        const float *__restrict__ ys, const float *__restrict__ gxs,
                                                        const float *__restrict__ gys, vtg_lk_out *__restrict__ out)
{
    extern __shared__ f2_t s_tp[]; /* the template's T: 8 warps x (MAXH / 2) x 32 pairs */
    const int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (i >= n)
        return;
    Patch<MAXH, true> P;
    P.ts = s_tp + (size_t)(threadIdx.x >> 5) * (MAXH / 2) * 32;
    vtg_lk_out o;
    unsigned work = 0;
    lk_point<MAXH, EXACT, true>(*Ip, *Jp, top, p, xs[i], ys[i], gxs ? gxs[i] : 0.0f, gys ? gys[i] : 0.0f, lane, P, o,
                                work);
    store_out(out + i, o, lane);
}

/* The point list with two warps a point (consecutive warps of a CTA): each walks the same pyramid with half the patch's
 * rows, and the pair adds its sums after every pass. The warps-a-point choice of vtg_tracker_set_point_warps; not the
 * default, as a pass's latency is one round of row loads however many rows a warp takes. MAXH bounds a half's rows
 * (11 for a 21-row patch, 16 for any up to 31). */
template <int MAXH>
__global__ void __launch_bounds__(256, 2) lk_points_pair_kernel(const DevPyr *__restrict__ Ip,
                                                             const DevPyr *__restrict__ Jp, int top, LkPrm p, int n,
                                                             const float *__restrict__ xs, const float *__restrict__ ys,
                                                             const float *__restrict__ gxs,
                                                             const float *__restrict__ gys,
                                                             vtg_lk_out *__restrict__ out)
{
    extern __shared__ f2_t s_tp[]; /* the template's T: 8 warps x (MAXH / 2) x 32 pairs */
    __shared__ float s_pair[4][16];
    const int wg = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    const int i = wg >> 1, pr = (threadIdx.x >> 6) & 3;
    if (i >= n) /* both warps of a pair leave together */
        return;
    const LkPair q{s_pair[pr], 1 + pr, wg & 1};
    Patch<MAXH, true> P;
    P.ts = s_tp + (size_t)(threadIdx.x >> 5) * (MAXH / 2) * 32;
    vtg_lk_out o;
    unsigned work = 0;
    lk_point<MAXH, false, true, 2>(*Ip, *Jp, top, p, xs[i], ys[i], gxs ? gxs[i] : 0.0f, gys ? gys[i] : 0.0f, lane, P,
                                   o, work, q);
    if (q.half == 0)
        store_out(out + i, o, lane);
}

/* shared memory of a 256-thread single-stream CTA: its 8 warps' template intensities (at most 30 KB) */
static constexpr size_t lk_t_bytes(int maxh) { return sizeof(f2_t) * 8 * (size_t)(maxh / 2) * 32; }

cudaError_t vtg_launch_cells(const DevPyr *I, const DevPyr *J, int top, const LkPrm &p, const CellGrid &g, int base_w,
                             int base_h, vtg_lk_out *out, vtg_cell *cells, cudaStream_t s)
{
    const int blocks = (g.n + 7) / 8;
    if (p.H == 21)
        lk_cells_kernel<21, true><<<blocks, 256, lk_t_bytes(21), s>>>(I, J, top, p, g, base_w, base_h, out, cells);
    else if (p.H == 15)
        lk_cells_kernel<15, true><<<blocks, 256, lk_t_bytes(15), s>>>(I, J, top, p, g, base_w, base_h, out, cells);
    else
        lk_cells_kernel<31, false><<<blocks, 256, lk_t_bytes(31), s>>>(I, J, top, p, g, base_w, base_h, out, cells);
    return cudaGetLastError();
}

cudaError_t vtg_launch_points(const DevPyr *I, const DevPyr *J, int top, const LkPrm &p, int n, const float *xs,
                              const float *ys, const float *gx, const float *gy, vtg_lk_out *out, cudaStream_t s,
                              int warps)
{
    if (n <= 0)
        return cudaSuccess;
    if (warps < 0 || warps > 2)
        return cudaErrorInvalidValue;
    if (vtg_points_pair(n, warps)) {
        const int pblocks = (n + 3) / 4;
        if (p.H <= 22)
            lk_points_pair_kernel<11><<<pblocks, 256, lk_t_bytes(11), s>>>(I, J, top, p, n, xs, ys, gx, gy, out);
        else
            lk_points_pair_kernel<16><<<pblocks, 256, lk_t_bytes(16), s>>>(I, J, top, p, n, xs, ys, gx, gy, out);
        return cudaGetLastError();
    }
    const int blocks = (n + 7) / 8;
    if (p.H == 21)
        lk_points_kernel<21, true><<<blocks, 256, lk_t_bytes(21), s>>>(I, J, top, p, n, xs, ys, gx, gy, out);
    else if (p.H == 15)
        lk_points_kernel<15, true><<<blocks, 256, lk_t_bytes(15), s>>>(I, J, top, p, n, xs, ys, gx, gy, out);
    else
        lk_points_kernel<31, false><<<blocks, 256, lk_t_bytes(31), s>>>(I, J, top, p, n, xs, ys, gx, gy, out);
    return cudaGetLastError();
}
