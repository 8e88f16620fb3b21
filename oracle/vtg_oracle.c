/* vtg_oracle.c -- TEST INFRASTRUCTURE ONLY. Nothing in the library links or loads this file: tests/, the smoke
 * check and bench.py's cpu_baseline leg are its only users, and only as the checker.
 *
 * A CPU restatement of the reference's sparse pyramidal Lucas-Kanade path (Lasimeri/Intel-Phi-VisionTrack), in this
 * project's own code, for checking the CUDA kernels:
 *   - the pyramid: u8 -> Q6 (src/kern/img_ref.c:32-40) and the 5 x 5 binomial reduce with clamp-to-edge borders
 *     (src/kern/img_ref.c:9-30, 74-114); exact integers;
 *   - tk_build's optional input steps (src/kern/track.c:600-622): the contrast stretch (img_minmax, img_norm,
 *     img_ref.c:42-71, with the gain and offset formed as the x87 unit forms them, in exact integer arithmetic) and
 *     the 5 x 5 binomial at every pixel (img_gauss5, img_ref.c:83-96); and the M1 gate's img_sobel / img_absdiff
 *     (img_ref.c:116-137);
 *   - one point of pyramidal LK: the driver of src/kern/lk_driver.inc:7-109 and the three patch operations of
 *     src/kern/lk_vx.c:36-175, and the forward-backward check (src/kern/lk_driver.inc:111-121);
 *   - the per-cell grid of src/kern/still.c:116-141, generalised to any cell size and patch;
 *   - the appearance correlation of src/kern/track.c:184-206, its half-pixel form (track.c:1615-1647), the parabola
 *     (track.c:1650-1657), the per-cell map (track.c:301-329) and the top-8 search (track.c:1661-1726), generalised to
 *     a T_w x T_h template (T_w a multiple of 16); and the template cut of store_appearance (track.c:935-974);
 *   - corner detection: the Harris response over Sobel gradients on a 5 x 5 box and the cells' strongest responses
 *     in the reference's F32 operation order (src/kern/detect.c:68-141), exact in any IEEE arithmetic, and the
 *     selection of detect_finish (detect.c:175-258), long double as the reference;
 *   - the still picture's decision and update (src/kern/still.c:143-246): the noise median, each cell's evidence, the
 *     3 x 3 vote, the counts and weights, the drift statistics, and the running mean; long double as the reference.
 *   - frame generation (src/kern/framegen.c, as src/kern/track.c:847-888 runs it): the scene-change test, the block
 *     SAD search, filter and upscale over the field's pyramid, the middle-instant vectors and the blended frame;
 *     whole-number planes, so exact in any arithmetic.
 *
 * Two arithmetics for everything that is floating point:
 *   OR_LANE  the reference's replay arithmetic: F32 patch sums in 16 lanes, each lane a chain of fused multiply-adds in
 *            row order, the lanes folded by the butterfly i^1, i^2, i^4, i^8 (src/common/vx.h:158-221), and the
 *            driver in long double. With gcc on x86-64 long double is the x87 80-bit format the reference was built
 *            with, so this mode reproduces the reference's golden LK hashes (logs/m2/host/640x480.txt) bit for bit.
 *            On another architecture long double differs and the mode is only close.
 *   OR_F64   every sample, sum and driver step in double: the FP64 oracle that flow tolerances are stated against.
 *            Window sums of the correlation are exact integers (or exact quarter-integers) in this mode.
 * Integer work (u8 -> Q6, the reduce) is exact and mode-free.
 *
 * Must be built with -ffp-contract=off: a * b + c stays two roundings unless fmaf/fma is written out. */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_LANE 0
#define OR_F64 1
#define OR_MAX_LEVELS 8
#define OR_MAX_W 48
#define OR_MAX_H 31

enum { OR_OK = 0, OR_OUT = 1, OR_LOWEIG = 2, OR_RESIDUAL = 4, OR_FLOWBACK = 8 };

/* A pyramid: level k is w[k] x h[k] Q6 values, rows stride[k] floats apart. Level k + 1 is (w + 1) / 2 x (h + 1) / 2. */
struct or_pyr {
    int levels;
    int w[OR_MAX_LEVELS], h[OR_MAX_LEVELS], stride[OR_MAX_LEVELS];
    const float *lv[OR_MAX_LEVELS];
};

/* The LK parameters of struct lk_cfg (src/kern/lk.h:24-31). */
struct or_lk_cfg {
    int w, h, max_iter;
    float eps, min_eig, max_residual;
};

/* struct lk_out (src/kern/lk.h:33-40), byte for byte: 32 bytes. */
struct or_lk_out {
    float x, y, min_eig, residual, cov_xx, cov_xy, cov_yy;
    uint16_t iters, status;
};

/* struct vt_cell (src/common/vt_proto.h:395-402): 24 bytes. */
struct or_cell {
    float u, v, diff;
    uint32_t state;
    float sigma, pad;
};

/* ---------------------------------------------------------------- hashing, for the reference's golden logs */

/* 64-bit FNV-1a, the hash the reference's gates print (src/common/vt_util.h:29-38). */
uint64_t or_fnv(uint64_t h, const void *p, size_t n)
{
    const uint8_t *b = p;
    for (size_t i = 0; i < n; i++) {
        h ^= b[i];
        h *= 0x100000001b3ull;
    }
    return h;
}

/* ---------------------------------------------------------------- the pyramid, exact integers */

/* Q6 = byte x 64 (src/kern/img_ref.c:32-40). dst: w x h, rows dst_stride floats apart. */
void or_u8_to_q6(const uint8_t *src, int src_stride, int w, int h, float *dst, int dst_stride)
{
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            dst[(size_t)y * dst_stride + x] = (float)(src[(size_t)y * src_stride + x] * 64);
}

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : v > hi ? hi : v; }

/* One pyramid step: (1 4 6 4 1)^2 / 256 at every second pixel of every second row, rounded as (sum + 128) >> 8
 * (src/kern/img_ref.c:98-114). The reference reads its replicated border (img_pad_rows / img_pad_tb, img_ref.c:9-30):
 * here that is a clamped index. Every value is a whole number below 2^24, so the integer sum is the F32 sum exactly. */
void or_reduce(const float *src, int w, int h, int src_stride, float *dst, int dst_stride)
{
    static const int k[5] = {1, 4, 6, 4, 1};
    const int dw = (w + 1) / 2, dh = (h + 1) / 2;
    for (int y = 0; y < dh; y++)
        for (int x = 0; x < dw; x++) {
            int64_t s = 0;
            for (int j = -2; j <= 2; j++) {
                const float *row = src + (size_t)clampi(2 * y + j, 0, h - 1) * src_stride;
                for (int i = -2; i <= 2; i++)
                    s += (int64_t)k[j + 2] * k[i + 2] * (int64_t)row[clampi(2 * x + i, 0, w - 1)];
            }
            dst[(size_t)y * dst_stride + x] = (float)((s + 128) >> 8);
        }
}

/* ---------------------------------------------------------------- tk_build's optional input steps and the M1 gate's
 * other image kernels (src/kern/img_ref.c), on w x h planes read with clamped indices (the reference's replicated
 * border). */

/* Min and max of the plane's values, the first value as the start (img_minmax_ref, img_ref.c:57-71). */
void or_minmax(const float *src, int w, int h, int stride, float out[2])
{
    float mn = src[0], mx = mn;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const float v = src[(size_t)y * stride + x];
            if (v < mn)
                mn = v;
            if (v > mx)
                mx = v;
        }
    out[0] = mn;
    out[1] = mx;
}

/* dst = clamp(rint(src x gain + offset), 0, 16320) (img_norm_ref, img_ref.c:42-55). The reference rounds an x87
 * extended src x gain + offset to F32; its vector form (img_vx.c:49-59) rounds the exact value once with a fused
 * multiply-add, as here. The two agree whenever the extended sum is exact: always for tk_build's gains (whole-number
 * src, gain >= 1), and for the M1 gate's (0.75, 512). */
void or_norm(const float *src, int w, int h, int sstride, const float go[2], float *dst, int dstride)
{
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            float v = rintf(fmaf(src[(size_t)y * sstride + x], go[0], go[1]));
            v = v < 0.0f ? 0.0f : v > 16320.0f ? 16320.0f : v;
            dst[(size_t)y * dstride + x] = v;
        }
}

/* The 5 x 5 binomial at every pixel, (sum + 128) >> 8 (img_gauss5_ref, img_ref.c:73-96): whole numbers, exact. */
void or_gauss5(const float *src, int w, int h, int sstride, float *dst, int dstride)
{
    static const int k[5] = {1, 4, 6, 4, 1};
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            int64_t s = 0;
            for (int j = -2; j <= 2; j++) {
                const float *row = src + (size_t)clampi(y + j, 0, h - 1) * sstride;
                for (int i = -2; i <= 2; i++)
                    s += (int64_t)k[j + 2] * k[i + 2] * (int64_t)row[clampi(x + i, 0, w - 1)];
            }
            dst[(size_t)y * dstride + x] = (float)((s + 128) >> 8);
        }
}

/* Sobel x and y in the reference's F32 order (img_sobel_ref, img_ref.c:116-127). */
void or_sobel(const float *src, int w, int h, int sstride, float *ix, float *iy, int dstride)
{
    for (int y = 0; y < h; y++) {
        const float *r0 = src + (size_t)clampi(y - 1, 0, h - 1) * sstride, *r1 = src + (size_t)y * sstride,
                    *r2 = src + (size_t)clampi(y + 1, 0, h - 1) * sstride;
        for (int x = 0; x < w; x++) {
            const int xl = clampi(x - 1, 0, w - 1), xr = clampi(x + 1, 0, w - 1);
            const float a = r0[xl], b = r0[x], c = r0[xr], e = r1[xl], g = r1[xr], m = r2[xl], n = r2[x], o = r2[xr];
            ix[(size_t)y * dstride + x] = (c + 2.0f * g + o) - (a + 2.0f * e + m);
            iy[(size_t)y * dstride + x] = (m + 2.0f * n + o) - (a + 2.0f * b + c);
        }
    }
}

/* |a - b| (img_absdiff_ref, img_ref.c:129-137). */
void or_absdiff(const float *a, const float *b, int w, int h, int stride, float *dst, int dstride)
{
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++)
            dst[(size_t)y * dstride + x] = fabsf(a[(size_t)y * stride + x] - b[(size_t)y * stride + x]);
}

/* q / d rounded to nearest even at 64 significant bits: (m, e) with q / d = m 2^e, 2^63 <= m < 2^64. q, d > 0. */
static void x87_quot(unsigned __int128 q, unsigned __int128 d, uint64_t *m, int *e)
{
    int k = 0; /* q 2^k / d in [2^63, 2^64) */
    while (q / d < ((unsigned __int128)1 << 63)) {
        q <<= 1;
        k++;
    }
    while (q / d >= ((unsigned __int128)1 << 64)) {
        d <<= 1;
        k--;
    }
    unsigned __int128 t = q / d;
    const unsigned __int128 r = q % d;
    if (2 * r > d || (2 * r == d && (t & 1)))
        t++;
    if (t == ((unsigned __int128)1 << 64)) {
        t >>= 1;
        k--;
    }
    *m = (uint64_t)t;
    *e = -k;
}

/* m 2^e rounded to nearest even at `bits` significant bits, m below 2^127: the rounded significand and exponent. */
static void round_bits(unsigned __int128 m, int e, int bits, uint64_t *mo, int *eo)
{
    int len = 0;
    while (len < 128 && (m >> len) != 0)
        len++;
    if (len <= bits) {
        *mo = (uint64_t)m;
        *eo = e;
        return;
    }
    const int s = len - bits;
    unsigned __int128 t = m >> s;
    const unsigned __int128 rest = m & (((unsigned __int128)1 << s) - 1), half = (unsigned __int128)1 << (s - 1);
    if (rest > half || (rest == half && (t & 1)))
        t++;
    int ex = e + s;
    if (t >> bits) {
        t >>= 1;
        ex++;
    }
    *mo = (uint64_t)t;
    *eo = ex;
}

/* tk_build's stretch (src/kern/track.c:603-614): gain = 16320 / (hi - lo) (1 when hi == lo) and offset = -lo x gain,
 * each an x87 extended value (64-bit significand, to nearest even) rounded to F32. Whole numbers 0 <= lo <= hi < 2^24.
 * Exact integer arithmetic, so it is the same on every host. */
void or_contrast_gain(int lo, int hi, float go[2])
{
    if (hi <= lo) {
        go[0] = 1.0f;
        go[1] = -(float)lo;
        return;
    }
    uint64_t gm, om, fm;
    int ge, oe, fe;
    x87_quot(16320, (unsigned __int128)(hi - lo), &gm, &ge);
    round_bits(gm, ge, 24, &fm, &fe);
    go[0] = ldexpf((float)fm, fe);
    if (lo == 0) {
        go[1] = -0.0f;
        return;
    }
    round_bits((unsigned __int128)gm * (unsigned __int128)lo, ge, 64, &om, &oe);
    round_bits(om, oe, 24, &fm, &fe);
    go[1] = -ldexpf((float)fm, fe);
}

/* Level 0 as tk_build makes it from a frame's bytes (track.c:596-622): Q6, then with opts & 1 the stretch of its min ..
 * max, then with opts & 2 the binomial. dst: w x h, rows dstride floats apart. */
void or_build_input(const uint8_t *src, int sstride, int w, int h, int opts, float *dst, int dstride)
{
    float *a = calloc((size_t)w * h, sizeof(float)), *b = calloc((size_t)w * h, sizeof(float));
    if (!a || !b) {
        free(a);
        free(b);
        return;
    }
    or_u8_to_q6(src, sstride, w, h, a, w);
    if (opts & 1) {
        float mm[2], go[2];
        or_minmax(a, w, h, w, mm);
        or_contrast_gain((int)mm[0], (int)mm[1], go);
        or_norm(a, w, h, w, go, b, w);
        float *t = a;
        a = b;
        b = t;
    }
    if (opts & 2) {
        or_gauss5(a, w, h, w, b, w);
        float *t = a;
        a = b;
        b = t;
    }
    for (int y = 0; y < h; y++)
        memcpy(dst + (size_t)y * dstride, a + (size_t)y * w, sizeof(float) * (size_t)w);
    free(a);
    free(b);
}

/* ---------------------------------------------------------------- lane arithmetic */

static float hsum16(const float *in)
{
    float v[16], t[16];
    memcpy(v, in, sizeof v);
    for (int s = 1; s <= 8; s <<= 1) {
        for (int i = 0; i < 16; i++)
            t[i] = v[i] + v[i ^ s];
        memcpy(v, t, sizeof v);
    }
    return v[0];
}

static inline float px_at(const struct or_pyr *p, int L, long x, long y) { return p->lv[L][(size_t)y * p->stride[L] + x]; }

/* The patch state one level's build leaves for its iterations: T, Tx, Ty in lane-model F32, or in double. */
struct or_tile {
    float t[OR_MAX_H][OR_MAX_W], tx[OR_MAX_H][OR_MAX_W], ty[OR_MAX_H][OR_MAX_W];
    double dt[OR_MAX_H][OR_MAX_W], dtx[OR_MAX_H][OR_MAX_W], dty[OR_MAX_H][OR_MAX_W];
};

/* build_vx (src/kern/lk_vx.c:36-97): the window of I around (px, py) at the patch's sub-pixel phase, the Sobel
 * gradients scaled by 1/512, and the structure tensor's sums, lane by lane. */
static void build_lane(const struct or_pyr *I, int L, long double px, long double py, const struct or_lk_cfg *c, struct or_tile *t, float g[3])
{
    const long ix = (long)floorl(px), iy = (long)floorl(py);
    const float fx = (float)(px - (long double)ix), fy = (float)(py - (long double)iy);
    const int W = c->w, H = c->h;
    const long x0 = ix - W / 2, y0 = iy - H / 2;
    float s[OR_MAX_H + 2][OR_MAX_W + 2], prev[OR_MAX_W + 2];
    for (int j = -1; j <= W; j++) {
        const float l = px_at(I, L, x0 + j, y0 - 1), n = px_at(I, L, x0 + j + 1, y0 - 1);
        prev[j + 1] = fmaf(n - l, fx, l);
    }
    for (int r = 0; r < H + 2; r++)
        for (int j = -1; j <= W; j++) {
            const float l = px_at(I, L, x0 + j, y0 + r), n = px_at(I, L, x0 + j + 1, y0 + r);
            const float cur = fmaf(n - l, fx, l);
            s[r][j + 1] = fmaf(cur - prev[j + 1], fy, prev[j + 1]);
            prev[j + 1] = cur;
        }
    float gxx[16] = {0}, gxy[16] = {0}, gyy[16] = {0};
    const float gs = 1.0f / 512.0f;
    for (int r = 0; r < H; r++) {
        const float *u = s[r], *m = s[r + 1], *d = s[r + 2];
        for (int j = 0; j < W; j++) {
            const int i = j + 1, l = j & 15;
            const float dxu = u[i + 1] - u[i - 1], dxm = m[i + 1] - m[i - 1], dxd = d[i + 1] - d[i - 1];
            const float tx = fmaf(dxm, 2.0f, dxu + dxd) * gs;
            const float dyl = d[i - 1] - u[i - 1], dyc = d[i] - u[i], dyr = d[i + 1] - u[i + 1];
            const float ty = fmaf(dyc, 2.0f, dyl + dyr) * gs;
            t->t[r][j] = m[i];
            t->tx[r][j] = tx;
            t->ty[r][j] = ty;
            gxx[l] = fmaf(tx, tx, gxx[l]);
            gxy[l] = fmaf(tx, ty, gxy[l]);
            gyy[l] = fmaf(ty, ty, gyy[l]);
        }
    }
    g[0] = hsum16(gxx);
    g[1] = hsum16(gxy);
    g[2] = hsum16(gyy);
}

/* iterate_vx (src/kern/lk_vx.c:100-140): J sampled at (qx, qy), It = T - J, the sums of It Tx and It Ty. */
static void iterate_lane(const struct or_pyr *J, int L, long double qx, long double qy, const struct or_lk_cfg *c, const struct or_tile *t, float b[2])
{
    const long jx = (long)floorl(qx), jy = (long)floorl(qy);
    const float fx = (float)(qx - (long double)jx), fy = (float)(qy - (long double)jy);
    const int W = c->w, H = c->h;
    const long x0 = jx - W / 2, y0 = jy - H / 2;
    float prev[OR_MAX_W], bx[16] = {0}, by[16] = {0};
    for (int j = 0; j < W; j++) {
        const float l = px_at(J, L, x0 + j, y0), n = px_at(J, L, x0 + j + 1, y0);
        prev[j] = fmaf(n - l, fx, l);
    }
    for (int r = 0; r < H; r++)
        for (int j = 0; j < W; j++) {
            const int l = j & 15;
            const float a = px_at(J, L, x0 + j, y0 + r + 1), n = px_at(J, L, x0 + j + 1, y0 + r + 1);
            const float cur = fmaf(n - a, fx, a);
            const float it = t->t[r][j] - fmaf(cur - prev[j], fy, prev[j]);
            bx[l] = fmaf(it, t->tx[r][j], bx[l]);
            by[l] = fmaf(it, t->ty[r][j], by[l]);
            prev[j] = cur;
        }
    b[0] = hsum16(bx);
    b[1] = hsum16(by);
}

/* residual_vx (src/kern/lk_vx.c:142-175): mean |It| and mean It^2 in 8-bit grey. */
static void residual_lane(const struct or_pyr *J, long double qx, long double qy, const struct or_lk_cfg *c, const struct or_tile *t, float out[2])
{
    const long jx = (long)floorl(qx), jy = (long)floorl(qy);
    const float fx = (float)(qx - (long double)jx), fy = (float)(qy - (long double)jy);
    const int W = c->w, H = c->h;
    const long x0 = jx - W / 2, y0 = jy - H / 2;
    float prev[OR_MAX_W], sa[16] = {0}, ss[16] = {0};
    for (int j = 0; j < W; j++) {
        const float l = px_at(J, 0, x0 + j, y0), n = px_at(J, 0, x0 + j + 1, y0);
        prev[j] = fmaf(n - l, fx, l);
    }
    for (int r = 0; r < H; r++)
        for (int j = 0; j < W; j++) {
            const int l = j & 15;
            const float a = px_at(J, 0, x0 + j, y0 + r + 1), n = px_at(J, 0, x0 + j + 1, y0 + r + 1);
            const float cur = fmaf(n - a, fx, a);
            const float it = (t->t[r][j] - fmaf(cur - prev[j], fy, prev[j])) * (1.0f / 64.0f);
            sa[l] = sa[l] + fabsf(it);
            ss[l] = fmaf(it, it, ss[l]);
            prev[j] = cur;
        }
    const long double n = (long double)(W * H);
    out[0] = (float)((long double)hsum16(sa) / n);
    out[1] = (float)((long double)hsum16(ss) / n);
}

/* ---------------------------------------------------------------- the same three operations in double */

static inline double lerp2(const struct or_pyr *p, int L, long x, long y, double fx, double fy)
{
    const double a = px_at(p, L, x, y), b = px_at(p, L, x + 1, y), c = px_at(p, L, x, y + 1), d = px_at(p, L, x + 1, y + 1);
    const double top = a + fx * (b - a), bot = c + fx * (d - c);
    return top + fy * (bot - top);
}

static void build_f64(const struct or_pyr *I, int L, double px, double py, const struct or_lk_cfg *c, struct or_tile *t, double g[3])
{
    const long ix = (long)floor(px), iy = (long)floor(py);
    const double fx = px - (double)ix, fy = py - (double)iy;
    const int W = c->w, H = c->h;
    const long x0 = ix - W / 2, y0 = iy - H / 2;
    double s[OR_MAX_H + 2][OR_MAX_W + 2];
    for (int r = 0; r < H + 2; r++)
        for (int j = -1; j <= W; j++)
            s[r][j + 1] = lerp2(I, L, x0 + j, y0 - 1 + r, fx, fy);
    double gxx = 0, gxy = 0, gyy = 0;
    for (int r = 0; r < H; r++) {
        const double *u = s[r], *m = s[r + 1], *d = s[r + 2];
        for (int j = 0; j < W; j++) {
            const int i = j + 1;
            const double tx = ((u[i + 1] - u[i - 1]) + 2.0 * (m[i + 1] - m[i - 1]) + (d[i + 1] - d[i - 1])) / 512.0;
            const double ty = ((d[i - 1] - u[i - 1]) + 2.0 * (d[i] - u[i]) + (d[i + 1] - u[i + 1])) / 512.0;
            t->dt[r][j] = m[i];
            t->dtx[r][j] = tx;
            t->dty[r][j] = ty;
            gxx += tx * tx;
            gxy += tx * ty;
            gyy += ty * ty;
        }
    }
    g[0] = gxx;
    g[1] = gxy;
    g[2] = gyy;
}

static void iterate_f64(const struct or_pyr *J, int L, double qx, double qy, const struct or_lk_cfg *c, const struct or_tile *t, double b[2])
{
    const long jx = (long)floor(qx), jy = (long)floor(qy);
    const double fx = qx - (double)jx, fy = qy - (double)jy;
    const long x0 = jx - c->w / 2, y0 = jy - c->h / 2;
    double bx = 0, by = 0;
    for (int r = 0; r < c->h; r++)
        for (int j = 0; j < c->w; j++) {
            const double it = t->dt[r][j] - lerp2(J, L, x0 + j, y0 + r, fx, fy);
            bx += it * t->dtx[r][j];
            by += it * t->dty[r][j];
        }
    b[0] = bx;
    b[1] = by;
}

static void residual_f64(const struct or_pyr *J, double qx, double qy, const struct or_lk_cfg *c, const struct or_tile *t, double out[2])
{
    const long jx = (long)floor(qx), jy = (long)floor(qy);
    const double fx = qx - (double)jx, fy = qy - (double)jy;
    const long x0 = jx - c->w / 2, y0 = jy - c->h / 2;
    double sa = 0, ss = 0;
    for (int r = 0; r < c->h; r++)
        for (int j = 0; j < c->w; j++) {
            const double it = (t->dt[r][j] - lerp2(J, 0, x0 + j, y0 + r, fx, fy)) / 64.0;
            sa += fabs(it);
            ss += it * it;
        }
    const double n = (double)(c->w * c->h);
    out[0] = sa / n;
    out[1] = ss / n;
}

/* ---------------------------------------------------------------- the pyramid walk (src/kern/lk_driver.inc:7-109) */

/* The driver, once per arithmetic. REAL is the driver's scalar type, G the type of the patch sums. */
#define OR_DRIVER(NAME, REAL, G, BUILD, ITERATE, RESIDUAL, FLOOR, SQRT)                                                      \
    static void NAME(const struct or_pyr *I, const struct or_pyr *J, int top, const struct or_lk_cfg *c, float x, float y,  \
                     float gx0, float gy0, struct or_lk_out *o, struct or_tile *tile)                                        \
    {                                                                                                                         \
        const REAL scale_top = (REAL)1 / (REAL)(1 << top);                                                                   \
        REAL gx = (REAL)gx0 * scale_top, gy = (REAL)gy0 * scale_top;                                                         \
        const REAL area = (REAL)(c->w * c->h);                                                                               \
        const REAL eps2 = (REAL)c->eps * (REAL)c->eps;                                                                       \
        REAL det0 = 0, gxx0 = 0, gxy0 = 0, gyy0 = 0;                                                                         \
        int status = 0, iters = 0, valid0 = 0;                                                                               \
        float eig0 = 0.0f;                                                                                                    \
        const int mx = c->w / 2 + 1, my = c->h / 2 + 1;                                                                     \
        for (int L = top; L >= 0; L--) {                                                                                      \
            const REAL s = (REAL)1 / (REAL)(1 << L);                                                                         \
            const REAL px = (REAL)x * s, py = (REAL)y * s;                                                                   \
            const REAL last_x = (REAL)(I->w[L] - mx - 1), last_y = (REAL)(I->h[L] - my - 1);                                 \
            if (px < mx || py < my || px >= last_x || py >= last_y) {                                                        \
                if (L == 0)                                                                                                   \
                    status |= OR_OUT;                                                                                         \
                else {                                                                                                        \
                    gx *= 2;                                                                                                  \
                    gy *= 2;                                                                                                  \
                }                                                                                                             \
                continue;                                                                                                     \
            }                                                                                                                 \
            G g[3];                                                                                                           \
            BUILD(I, L, px, py, c, tile, g);                                                                                  \
            const REAL gxx = g[0], gxy = g[1], gyy = g[2];                                                                   \
            const REAL det = gxx * gyy - gxy * gxy;                                                                          \
            const REAL tr = gxx + gyy, diff = gxx - gyy;                                                                     \
            const REAL eig = (tr - SQRT(diff * diff + 4 * gxy * gxy)) * (REAL)0.5 / area;                                    \
            if (L == 0)                                                                                                       \
                eig0 = (float)eig;                                                                                            \
            if (eig < (REAL)c->min_eig || det <= 0) {                                                                        \
                if (L == 0)                                                                                                   \
                    status |= OR_LOWEIG;                                                                                      \
                else {                                                                                                        \
                    gx *= 2;                                                                                                  \
                    gy *= 2;                                                                                                  \
                }                                                                                                             \
                continue;                                                                                                     \
            }                                                                                                                 \
            if (L == 0) {                                                                                                     \
                det0 = det;                                                                                                   \
                gxx0 = gxx;                                                                                                   \
                gxy0 = gxy;                                                                                                   \
                gyy0 = gyy;                                                                                                   \
                valid0 = 1;                                                                                                   \
            }                                                                                                                 \
            const REAL ia = gyy / det, ib = -gxy / det, ic = gxx / det;                                                      \
            REAL vx = 0, vy = 0;                                                                                              \
            for (int it = 0; it < c->max_iter; it++) {                                                                        \
                const REAL qxl = px + gx + vx, qyl = py + gy + vy;                                                           \
                const REAL lx = (REAL)(J->w[L] - mx - 1), ly = (REAL)(J->h[L] - my - 1);                                     \
                if (qxl < mx || qyl < my || qxl >= lx || qyl >= ly) {                                                        \
                    if (L == 0) {                                                                                             \
                        status |= OR_OUT;                                                                                     \
                        valid0 = 0;                                                                                           \
                    }                                                                                                         \
                    break;                                                                                                    \
                }                                                                                                             \
                G b[2];                                                                                                       \
                ITERATE(J, L, qxl, qyl, c, tile, b);                                                                          \
                const REAL bx = (REAL)b[0] / 64, by = (REAL)b[1] / 64;                                                       \
                const REAL ex = ia * bx + ib * by, ey = ib * bx + ic * by;                                                   \
                vx += ex;                                                                                                     \
                vy += ey;                                                                                                     \
                iters++;                                                                                                      \
                if (ex * ex + ey * ey < eps2)                                                                                 \
                    break;                                                                                                    \
            }                                                                                                                 \
            gx += vx;                                                                                                         \
            gy += vy;                                                                                                         \
            if (L > 0) {                                                                                                      \
                gx *= 2;                                                                                                      \
                gy *= 2;                                                                                                      \
            }                                                                                                                 \
        }                                                                                                                     \
        const REAL qx = (REAL)x + gx, qy = (REAL)y + gy;                                                                     \
        o->x = (float)qx;                                                                                                     \
        o->y = (float)qy;                                                                                                     \
        o->min_eig = eig0;                                                                                                    \
        o->iters = (uint16_t)iters;                                                                                           \
        o->residual = 0.0f;                                                                                                   \
        o->cov_xx = o->cov_xy = o->cov_yy = 0.0f;                                                                             \
        if (valid0 && !status) {                                                                                              \
            if (qx < mx || qy < my || qx >= (REAL)(J->w[0] - mx - 1) || qy >= (REAL)(J->h[0] - my - 1)) {                    \
                status |= OR_OUT;                                                                                             \
            } else {                                                                                                          \
                G r[2];                                                                                                       \
                RESIDUAL(J, qx, qy, c, tile, r);                                                                              \
                o->residual = (float)r[0];                                                                                    \
                if (r[0] > c->max_residual)                                                                                   \
                    status |= OR_RESIDUAL;                                                                                    \
                const REAL s2 = (REAL)r[1] * area / (area - 2);                                                              \
                o->cov_xx = (float)(s2 * gyy0 / det0);                                                                        \
                o->cov_xy = (float)(-s2 * gxy0 / det0);                                                                       \
                o->cov_yy = (float)(s2 * gxx0 / det0);                                                                        \
            }                                                                                                                 \
        }                                                                                                                     \
        o->status = (uint16_t)status;                                                                                         \
    }

OR_DRIVER(track_lane, long double, float, build_lane, iterate_lane, residual_lane, floorl, sqrtl)
OR_DRIVER(track_f64, double, double, build_f64, iterate_f64, residual_f64, floor, sqrt)

static void track_mode(const struct or_pyr *I, const struct or_pyr *J, int top, const struct or_lk_cfg *c, float x, float y, float gx, float gy, struct or_lk_out *o, struct or_tile *tile, int mode)
{
    if (mode == OR_F64)
        track_f64(I, J, top, c, x, y, gx, gy, o, tile);
    else
        track_lane(I, J, top, c, x, y, gx, gy, o, tile);
}

/* lk_flowback (src/kern/lk_driver.inc:111-121): track the found point back from J to I, from minus the found flow; a
 * miss beyond max_fb, or a failed return, flags the point. */
static void flowback_mode(const struct or_pyr *I, const struct or_pyr *J, int top, const struct or_lk_cfg *c, float x, float y, float max_fb, struct or_lk_out *o, struct or_tile *tile, int mode)
{
    if (o->status)
        return;
    struct or_lk_out b;
    if (mode == OR_F64) {
        track_f64(J, I, top, c, o->x, o->y, (float)((double)x - (double)o->x), (float)((double)y - (double)o->y), &b, tile);
        const double ex = (double)b.x - (double)x, ey = (double)b.y - (double)y;
        if (b.status || ex * ex + ey * ey > (double)max_fb * (double)max_fb)
            o->status |= OR_FLOWBACK;
    } else {
        track_lane(J, I, top, c, o->x, o->y, (float)((long double)x - (long double)o->x), (float)((long double)y - (long double)o->y), &b, tile);
        const long double ex = (long double)b.x - (long double)x, ey = (long double)b.y - (long double)y;
        if (b.status || ex * ex + ey * ey > (long double)max_fb * (long double)max_fb)
            o->status |= OR_FLOWBACK;
    }
}

void or_lk_track(const struct or_pyr *I, const struct or_pyr *J, int top, const struct or_lk_cfg *c, float x, float y, float gx, float gy, float max_fb, struct or_lk_out *o, int mode)
{
    struct or_tile *tile = malloc(sizeof *tile);
    track_mode(I, J, top, c, x, y, gx, gy, o, tile, mode);
    if (max_fb > 0.0f)
        flowback_mode(I, J, top, c, x, y, max_fb, o, tile, mode);
    free(tile);
}

/* ---------------------------------------------------------------- points and cells, on a team of threads */

/* A cell's centre: (cw c + cw / 2, ch r + ch / 2), clamped to where the patch still fits (src/kern/still.c:127-130,
 * whose margin of 9 is a 15-pixel patch's half plus 2; here it is the configured patch's). */
void or_cell_centre(int w, int h, int cell_w, int cell_h, const struct or_lk_cfg *c, int col, int row, float *x, float *y)
{
    const float mx = (float)(c->w / 2 + 2), my = (float)(c->h / 2 + 2);
    const float x_max = (float)w - 1.0f - mx, y_max = (float)h - 1.0f - my;
    float cx = (float)(col * cell_w + cell_w / 2), cy = (float)(row * cell_h + cell_h / 2);
    cx = cx < mx ? mx : cx > x_max ? x_max : cx;
    cy = cy < my ? my : cy > y_max ? y_max : cy;
    *x = cx;
    *y = cy;
}

/* Mean |J - I| over a cell of level 0, 8-bit grey (src/kern/still.c:105-114): row sums folded as the lane model folds
 * 16 lanes, in long double across rows. A cell past the picture's edge reads the replicated border. */
static float cell_diff(const struct or_pyr *I, const struct or_pyr *J, int cell_w, int cell_h, int col, int row, int mode)
{
    const int w = I->w[0], h = I->h[0];
    const int x = col * cell_w, y0 = row * cell_h, y1 = y0 + cell_h < h ? y0 + cell_h : h;
    long double sum = 0.0L;
    for (int y = y0; y < y1; y++) {
        float lanes[16] = {0};
        double rs = 0.0;
        for (int k = 0; k < cell_w; k++) {
            const int xx = clampi(x + k, 0, w - 1);
            const float d = fabsf(px_at(J, 0, xx, y) - px_at(I, 0, xx, y));
            lanes[k & 15] = lanes[k & 15] + d;
            rs += d;
        }
        sum += mode == OR_F64 ? (long double)rs : (long double)hsum16(lanes);
    }
    return (float)(sum / (long double)((y1 - y0) * cell_w) / 64.0L);
}

struct team_job {
    const struct or_pyr *I, *J;
    const struct or_lk_cfg *c;
    int top, mode, n;
    float max_fb;
    /* points */
    const float *xs, *ys, *gxs, *gys;
    /* cells */
    int cell_w, cell_h, cols;
    struct or_lk_out *out;
    struct or_cell *cells;
    int next;
};

static void *team_points(void *arg)
{
    struct team_job *j = arg;
    struct or_tile *tile = malloc(sizeof *tile);
    for (;;) {
        const int i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (i >= j->n)
            break;
        track_mode(j->I, j->J, j->top, j->c, j->xs[i], j->ys[i], j->gxs ? j->gxs[i] : 0.0f, j->gys ? j->gys[i] : 0.0f, &j->out[i], tile, j->mode);
        if (j->max_fb > 0.0f)
            flowback_mode(j->I, j->J, j->top, j->c, j->xs[i], j->ys[i], j->max_fb, &j->out[i], tile, j->mode);
    }
    free(tile);
    return NULL;
}

/* The per-cell grid of still_vectors (src/kern/still.c:116-141): LK from I to J at each cell's centre, the
 * forward-backward check when max_fb > 0, then the cell record. */
static void *team_cells(void *arg)
{
    struct team_job *j = arg;
    struct or_tile *tile = malloc(sizeof *tile);
    for (;;) {
        const int i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (i >= j->n)
            break;
        const int col = i % j->cols, row = i / j->cols;
        float x, y;
        or_cell_centre(j->I->w[0], j->I->h[0], j->cell_w, j->cell_h, j->c, col, row, &x, &y);
        struct or_lk_out o;
        track_mode(j->I, j->J, j->top, j->c, x, y, 0.0f, 0.0f, &o, tile, j->mode);
        if (j->max_fb > 0.0f)
            flowback_mode(j->I, j->J, j->top, j->c, x, y, j->max_fb, &o, tile, j->mode);
        if (j->out)
            j->out[i] = o;
        if (j->cells) {
            struct or_cell *cl = &j->cells[i];
            cl->u = (float)((long double)o.x - (long double)x);
            cl->v = (float)((long double)o.y - (long double)y);
            cl->diff = cell_diff(j->I, j->J, j->cell_w, j->cell_h, col, row, j->mode);
            cl->state = o.status;
            cl->sigma = o.status ? 0.0f : (float)sqrtl((long double)o.cov_xx + (long double)o.cov_yy);
            cl->pad = 0.0f;
        }
    }
    free(tile);
    return NULL;
}

static void run_team(void *(*fn)(void *), struct team_job *j, int threads)
{
    if (threads < 1)
        threads = 1;
    j->next = 0;
    if (threads == 1) {
        fn(j);
        return;
    }
    pthread_t *th = malloc(sizeof *th * (size_t)threads);
    for (int i = 0; i < threads; i++)
        pthread_create(&th[i], NULL, fn, j);
    for (int i = 0; i < threads; i++)
        pthread_join(th[i], NULL);
    free(th);
}

/* Points with their own guesses (the tracker's OP_LK, src/kern/track.c:275-292). gxs / gys may be NULL. */
void or_lk_points(const struct or_pyr *I, const struct or_pyr *J, int top, const struct or_lk_cfg *c, int n, const float *xs, const float *ys, const float *gxs, const float *gys, float max_fb, struct or_lk_out *out, int mode, int threads)
{
    struct team_job j = {.I = I, .J = J, .c = c, .top = top, .mode = mode, .n = n, .max_fb = max_fb, .xs = xs, .ys = ys, .gxs = gxs, .gys = gys, .out = out};
    run_team(team_points, &j, threads);
}

/* The cell grid over level 0 of I and J: ceil(w / cell_w) x ceil(h / cell_h) cells, row-major. out or cells may be NULL. */
void or_cells(const struct or_pyr *I, const struct or_pyr *J, int top, const struct or_lk_cfg *c, int cell_w, int cell_h, float max_fb, struct or_lk_out *out, struct or_cell *cells, int mode, int threads)
{
    const int cols = (I->w[0] + cell_w - 1) / cell_w, rows = (I->h[0] + cell_h - 1) / cell_h;
    struct team_job j = {.I = I, .J = J, .c = c, .top = top, .mode = mode, .n = cols * rows, .max_fb = max_fb, .cell_w = cell_w, .cell_h = cell_h, .cols = cols, .out = out, .cells = cells};
    run_team(team_cells, &j, threads);
}

/* ---------------------------------------------------------------- the appearance correlation */

/* A plane for the correlation: Q6 (or 8-bit) whole-number values, w x h, rows stride floats apart. */
struct or_img {
    const float *p;
    int w, h, stride;
};

static inline float im_at(const struct or_img *m, int x, int y) { return m->p[(size_t)y * m->stride + x]; }

/* search_at (src/kern/track.c:184-206) for a T_w x T_h zero-mean template at corner (x, y): st = sum t v, with
 * v = J - J(x, y); var = sum v^2 - (sum v)^2 / n; 0 when var <= norm / 16 or norm <= 0, else st / sqrt(norm var);
 * -1 where the template does not fit inside a one-pixel margin. */
double or_ncc_at(const struct or_img *m, const float *app, int tw, int th, double norm, int x, int y, int mode)
{
    if (x < 1 || y < 1 || x + tw >= m->w - 1 || y + th >= m->h - 1)
        return -1.0;
    const int n = tw * th;
    if (mode == OR_F64) {
        /* Exact window sums of whole numbers, the product sum in double (each term exact, the sum all but exact). */
        int64_t s1 = 0, s2 = 0;
        double st = 0.0, ts = 0.0;
        for (int r = 0; r < th; r++)
            for (int k = 0; k < tw; k++) {
                const int64_t v = (int64_t)im_at(m, x + k, y + r);
                s1 += v;
                s2 += v * v;
                st += (double)app[r * tw + k] * (double)v;
                ts += (double)app[r * tw + k];
            }
        st -= ts * (double)im_at(m, x, y);
        const double nvar = (double)((int64_t)n * s2 - s1 * s1); /* n var, exact */
        if (nvar <= (double)n * norm * 0.0625 || norm <= 0.0)
            return 0.0;
        return st / sqrt(norm * (nvar / (double)n));
    }
    const float first = im_at(m, x, y);
    float st[16] = {0}, sj[16] = {0}, sjj[16] = {0};
    for (int r = 0; r < th; r++)
        for (int k = 0; k < tw; k++) {
            const int l = k & 15;
            const float v = im_at(m, x + k, y + r) - first;
            st[l] = fmaf(v, app[r * tw + k], st[l]);
            sj[l] = sj[l] + v;
            sjj[l] = fmaf(v, v, sjj[l]);
        }
    const long double nn = (long double)n, nt = (long double)norm;
    const long double a = hsum16(st), b = hsum16(sj), c = hsum16(sjj);
    const long double var = c - b * b / nn;
    return (double)((var <= nt * 0.0625L || nt <= 0.0L) ? 0.0L : a / sqrtl(nt * var));
}

/* search_half (src/kern/track.c:1615-1647): the corner in half pixels; an odd half step averages the two neighbours. */
double or_ncc_half(const struct or_img *m, const float *app, int tw, int th, double norm, int hx, int hy, int mode)
{
    const int x = hx >> 1, y = hy >> 1, ox = hx & 1, oy = hy & 1;
    if (x < 1 || y < 1 || x + tw + 1 >= m->w - 1 || y + th + 1 >= m->h - 1)
        return -1.0;
    const int n = tw * th;
    if (mode == OR_F64) {
        /* In quarters: every sample is a whole number of quarters, so the sums are exact. */
        int64_t s1 = 0, s2 = 0;
        double st = 0.0, ts = 0.0;
        for (int r = 0; r < th; r++)
            for (int k = 0; k < tw; k++) {
                int64_t q = 4 * (int64_t)im_at(m, x + k, y + r);
                if (ox)
                    q = 2 * ((int64_t)im_at(m, x + k, y + r) + (int64_t)im_at(m, x + k + 1, y + r));
                if (oy) {
                    int64_t b = 4 * (int64_t)im_at(m, x + k, y + r + 1);
                    if (ox)
                        b = 2 * ((int64_t)im_at(m, x + k, y + r + 1) + (int64_t)im_at(m, x + k + 1, y + r + 1));
                    q = (q + b) / 2;
                }
                s1 += q;
                s2 += q * q;
                st += (double)app[r * tw + k] * (double)q * 0.25;
                ts += (double)app[r * tw + k];
            }
        st -= ts * (double)im_at(m, x, y);
        const double nvar = (double)((int64_t)n * s2 - s1 * s1) / 16.0;
        if (nvar <= (double)n * norm * 0.0625 || norm <= 0.0)
            return 0.0;
        return st / sqrt(norm * (nvar / (double)n));
    }
    const float first = im_at(m, x, y);
    float st[16] = {0}, sj[16] = {0}, sjj[16] = {0};
    for (int r = 0; r < th; r++)
        for (int k = 0; k < tw; k++) {
            const int l = k & 15;
            float v = im_at(m, x + k, y + r);
            if (ox)
                v = (v + im_at(m, x + k + 1, y + r)) * 0.5f;
            if (oy) {
                float w = im_at(m, x + k, y + r + 1);
                if (ox)
                    w = (w + im_at(m, x + k + 1, y + r + 1)) * 0.5f;
                v = (v + w) * 0.5f;
            }
            v = v - first;
            st[l] = fmaf(v, app[r * tw + k], st[l]);
            sj[l] = sj[l] + v;
            sjj[l] = fmaf(v, v, sjj[l]);
        }
    const long double nn = (long double)n, nt = (long double)norm;
    const long double a = hsum16(st), b = hsum16(sj), c = hsum16(sjj);
    const long double var = c - b * b / nn;
    return (double)((var <= nt * 0.0625L || nt <= 0.0L) ? 0.0L : a / sqrtl(nt * var));
}

/* peak_offset (src/kern/track.c:1650-1657): the vertex of a parabola through three scores, within half a step. */
double or_peak_offset(double l, double c, double r)
{
    const long double den = (long double)l - 2.0L * (long double)c + (long double)r;
    if (den >= 0.0L)
        return 0.0;
    const long double o = 0.5L * ((long double)l - (long double)r) / den;
    return (double)(o < -0.5L ? -0.5L : o > 0.5L ? 0.5L : o);
}

/* The zero-mean template store_appearance cuts (src/kern/track.c:935-974): T_w x T_h pixels at corner (x0, y0), their
 * mean (lane sums, long double division) taken off, norm = the lane-folded sum of squares. */
/* (float)((long double)sum / n), the x87 quotient rounded to F32, for a whole-number sum: exact integer arithmetic, so
 * the same on every host. Other sums go through the host's long double. */
static float x87_mean(float sum, int n)
{
    if (sum == 0.0f)
        return 0.0f;
    if (!(sum > 0.0f && sum == floorf(sum)))
        return (float)((long double)sum / (long double)n);
    uint64_t m, fm;
    int e, fe;
    x87_quot((unsigned __int128)sum, (unsigned __int128)n, &m, &e);
    round_bits(m, e, 24, &fm, &fe);
    return ldexpf((float)fm, fe);
}

void or_cut_template(const struct or_img *m, int x0, int y0, int tw, int th, float *app, float *norm)
{
    float sum[16] = {0};
    for (int r = 0; r < th; r++)
        for (int k = 0; k < tw; k++) {
            const float v = im_at(m, x0 + k, y0 + r);
            app[r * tw + k] = v;
            sum[k & 15] = sum[k & 15] + v;
        }
    const float mean = x87_mean(hsum16(sum), tw * th);
    float ss[16] = {0};
    for (int r = 0; r < th; r++)
        for (int k = 0; k < tw; k++) {
            const float z = app[r * tw + k] - mean;
            app[r * tw + k] = z;
            ss[k & 15] = fmaf(z, z, ss[k & 15]);
        }
    *norm = hsum16(ss);
}

/* store_appearance (src/kern/track.c:935-974) on a pyramid: the coarsest level where a 32 x 21 template fits inside
 * the region rw x rh, the window around the centre (cx, cy) there (truncated to whole pixels), zero-mean, and its sum
 * of squares. info: norm, fx, fy, level, valid (valid 0: the window leaves the level's border; app untouched). */
void or_store_appearance(const struct or_pyr *p, float cx, float cy, float rw, float rh, float *app, float info[5])
{
    enum { AW = 32, AH = 21 };
    int L = 0;
    while (L < p->levels - 1 && (double)rw / (double)(1 << (L + 1)) >= AW && (double)rh / (double)(1 << (L + 1)) >= AH)
        L++;
    const double lx = ldexp((double)cx, -L), ly = ldexp((double)cy, -L);
    const int ix = (int)lx, iy = (int)ly;
    const int x0 = ix - AW / 2, y0 = iy - AH / 2;
    info[1] = (float)(lx - ix);
    info[2] = (float)(ly - iy);
    info[3] = (float)L;
    info[4] = 0.0f;
    if (x0 < 1 || y0 < 1 || x0 + AW >= p->w[L] - 1 || y0 + AH >= p->h[L] - 1)
        return;
    const struct or_img m = {p->lv[L], p->w[L], p->h[L], p->stride[L]};
    or_cut_template(&m, x0, y0, AW, AH, app, &info[0]);
    info[4] = 1.0f;
}

/* What one search found (struct found, src/kern/track.c:1608-1612): the best corner in half pixels, its score, the best
 * score clear of it, and the parabola's sub-half-pixel offsets around it (take_back, track.c:1741-1742). */
struct or_found {
    int hx, hy;
    double ncc, second, ox, oy;
};

#define OR_SEARCH_CELL 16
#define OR_SEARCH_TOP 8

/* search_slot (src/kern/track.c:1661-1726) with the per-cell map of OP_SEARCH (track.c:301-329): the best corner of
 * each 16 x 16 cell of corners at the given step, the eight best cells, each looked at again in half pixels within
 * +-(2 step - 1) (or +-1), the best of those, and the best of the rest that stands half a template away. map_v, map_x,
 * map_y (may be NULL) receive the per-cell map. */
void or_search_slot(const struct or_img *m, const float *app, int tw, int th, double norm, int x0, int x1, int y0, int y1, int step, int mode, struct or_found *f, float *map_v, int *map_x, int *map_y)
{
    const int lo_x = 1, hi_x = m->w - tw - 2, lo_y = 1, hi_y = m->h - th - 2;
    x0 = x0 < lo_x ? lo_x : x0;
    x1 = x1 > hi_x ? hi_x : x1;
    y0 = y0 < lo_y ? lo_y : y0;
    y1 = y1 > hi_y ? hi_y : y1;
    f->ncc = -2.0;
    f->second = -2.0;
    f->hx = f->hy = 0;
    f->ox = f->oy = 0.0;
    if (x1 < x0 || y1 < y0)
        return;
    const int ccols = (x1 - x0) / OR_SEARCH_CELL + 1, crows = (y1 - y0) / OR_SEARCH_CELL + 1, cells = ccols * crows;
    float *sv = malloc(sizeof(float) * (size_t)cells);
    int *sx = malloc(sizeof(int) * (size_t)cells), *sy = malloc(sizeof(int) * (size_t)cells);
    for (int cell = 0; cell < cells; cell++) {
        const int cy0 = y0 + (cell / ccols) * OR_SEARCH_CELL, cx0 = x0 + (cell % ccols) * OR_SEARCH_CELL;
        const int cy1 = cy0 + OR_SEARCH_CELL <= y1 + 1 ? cy0 + OR_SEARCH_CELL : y1 + 1, cx1 = cx0 + OR_SEARCH_CELL <= x1 + 1 ? cx0 + OR_SEARCH_CELL : x1 + 1;
        float best = -2.0f;
        int bx = cx0, by = cy0;
        for (int y = cy0; y < cy1; y += step)
            for (int x = cx0; x < cx1; x += step) {
                const float v = (float)or_ncc_at(m, app, tw, th, norm, x, y, mode);
                if (v > best) {
                    best = v;
                    bx = x;
                    by = y;
                }
            }
        sv[cell] = best;
        sx[cell] = bx;
        sy[cell] = by;
    }
    if (map_v)
        memcpy(map_v, sv, sizeof(float) * (size_t)cells);
    if (map_x)
        memcpy(map_x, sx, sizeof(int) * (size_t)cells);
    if (map_y)
        memcpy(map_y, sy, sizeof(int) * (size_t)cells);
    int top[OR_SEARCH_TOP], ntop = 0;
    for (int i = 0; i < cells; i++) {
        if (sv[i] <= -2.0f || (ntop == OR_SEARCH_TOP && sv[i] <= sv[top[ntop - 1]]))
            continue;
        int at = ntop < OR_SEARCH_TOP ? ntop++ : OR_SEARCH_TOP - 1;
        for (; at > 0 && sv[top[at - 1]] < sv[i]; at--)
            top[at] = top[at - 1];
        top[at] = i;
    }
    const int around = step > 1 ? 2 * step - 1 : 1;
    double score[OR_SEARCH_TOP];
    int shx[OR_SEARCH_TOP], shy[OR_SEARCH_TOP];
    for (int c = 0; c < ntop; c++) {
        const int cx = 2 * sx[top[c]], cy = 2 * sy[top[c]];
        score[c] = -2.0;
        shx[c] = cx;
        shy[c] = cy;
        for (int hy = cy - around; hy <= cy + around; hy++)
            for (int hx = cx - around; hx <= cx + around; hx++) {
                const double v = or_ncc_half(m, app, tw, th, norm, hx, hy, mode);
                if (v > score[c]) {
                    score[c] = v;
                    shx[c] = hx;
                    shy[c] = hy;
                }
            }
        if (score[c] > f->ncc) {
            f->ncc = score[c];
            f->hx = shx[c];
            f->hy = shy[c];
        }
    }
    for (int c = 0; c < ntop; c++) {
        const int dx = shx[c] - f->hx, dy = shy[c] - f->hy;
        if ((dx * dx > tw * tw || dy * dy > th * th) && score[c] > f->second)
            f->second = score[c];
    }
    if (ntop) {
        f->ox = or_peak_offset(or_ncc_half(m, app, tw, th, norm, f->hx - 1, f->hy, mode), f->ncc, or_ncc_half(m, app, tw, th, norm, f->hx + 1, f->hy, mode));
        f->oy = or_peak_offset(or_ncc_half(m, app, tw, th, norm, f->hx, f->hy - 1, mode), f->ncc, or_ncc_half(m, app, tw, th, norm, f->hx, f->hy + 1, mode));
    }
    free(sv);
    free(sx);
    free(sy);
}

/* Every corner's score over a window of corners (step 1), row-major: the dense map the whole-picture search computes.
 * out: (x1 - x0 + 1) x (y1 - y0 + 1). */
void or_ncc_map(const struct or_img *m, const float *app, int tw, int th, double norm, int x0, int x1, int y0, int y1, int mode, float *out, int threads)
{
    (void)threads;
    const int cols = x1 - x0 + 1;
    for (int y = y0; y <= y1; y++)
        for (int x = x0; x <= x1; x++)
            out[(size_t)(y - y0) * cols + (x - x0)] = (float)or_ncc_at(m, app, tw, th, norm, x, y, mode);
}

/* ---------------------------------------------------------------- the reference's deterministic test images */

/* xorshift64* (src/common/vt_util.h:40-49). */
static inline uint64_t or_rand(uint64_t *s)
{
    uint64_t x = *s;
    x ^= x >> 12;
    x ^= x << 25;
    x ^= x >> 27;
    *s = x;
    return x * 0x2545F4914F6CDD1Dull;
}

/* The M1 gate's frame (src/kern/m1_input.h:10-21): a ramp, 32-pixel blocks and 5 bits of noise, from integers. */
void or_m1_image(uint8_t *img, int w, int h, int stride)
{
    uint64_t s = 0x9e3779b97f4a7c15ull;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const int ramp = (x * 96) / w + (y * 64) / h;
            const int block = (((x >> 5) ^ (y >> 5)) & 7) * 8;
            const int noise = (int)(or_rand(&s) & 31);
            img[(size_t)y * (size_t)stride + (size_t)x] = (uint8_t)(ramp + block + noise);
        }
}

/* The M2 gate's pattern (src/kern/m2_input.h:12-50): two octaves of integer value noise on a grid four times finer
 * than the pixels, each pixel the rounded mean of its 4 x 4 fine cells, so an offset of (ox, oy) fine cells moves the
 * picture by exactly (ox / 4, oy / 4) pixels. */
static inline uint32_t m2_hash(int x, int y)
{
    uint32_t h = (uint32_t)x * 0x9E3779B1u ^ (uint32_t)y * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0xC2B2AE3Du;
    return h ^ (h >> 13);
}

static inline uint32_t m2_noise(int x, int y, int bits)
{
    const int xi = x >> bits, yi = y >> bits, m = (1 << bits) - 1;
    const uint32_t fx = (uint32_t)(x & m), fy = (uint32_t)(y & m), one = 1u << bits;
    const uint32_t a = m2_hash(xi, yi) & 255, b = m2_hash(xi + 1, yi) & 255, c = m2_hash(xi, yi + 1) & 255, d = m2_hash(xi + 1, yi + 1) & 255;
    return (a * (one - fx) + b * fx) * (one - fy) + (c * (one - fx) + d * fx) * fy;
}

void or_m2_render(uint8_t *img, int w, int h, int stride, int ox, int oy)
{
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            uint32_t sum = 0;
            for (int j = 0; j < 4; j++)
                for (int i = 0; i < 4; i++) {
                    const int fx = 4 * x + i + ox, fy = 4 * y + j + oy;
                    sum += ((m2_noise(fx, fy, 5) >> 6) * 3 + (m2_noise(fx, fy, 4) >> 4)) >> 2;
                }
            img[(size_t)y * stride + x] = (uint8_t)((sum + 128) >> 8);
        }
}

/* ---------------------------------------------------------------- corner detection */

/* A region laid out as detect_begin does (src/kern/detect.c:28-66): the rectangle in whole pixels, clamped to the
 * margin; columns from ax = x0 rounded down to 16, a whole number of 16-column groups; 16 x 16 cells. */
struct or_det_geo {
    int x0, y0, x1, y1, ax, cols, rows, nv, cell_rows;
};

/* 0 when nothing of the rectangle lies inside the margin (detect_begin's false). */
int or_detect_geometry(int w, int h, float rx, float ry, float rw, float rh, int margin, struct or_det_geo *g)
{
    int x0 = (int)rx, y0 = (int)ry, x1 = (int)(rx + rw), y1 = (int)(ry + rh);
    x0 = x0 < margin ? margin : x0;
    y0 = y0 < margin ? margin : y0;
    x1 = x1 > w - margin ? w - margin : x1;
    y1 = y1 > h - margin ? h - margin : y1;
    if (x1 <= x0 || y1 <= y0)
        return 0;
    g->x0 = x0;
    g->y0 = y0;
    g->x1 = x1;
    g->y1 = y1;
    g->ax = x0 & ~15;
    g->cols = (x1 - g->ax + 15) & ~15;
    g->rows = y1 - y0;
    g->nv = g->cols / 16;
    g->cell_rows = g->rows / 16 + 1;
    return 1;
}

/* The plane at (x, y), edges replicated (the reference reads its padding). */
static inline float det_px(const struct or_img *m, int x, int y)
{
    return m->p[(size_t)clampi(y, 0, m->h - 1) * m->stride + clampi(x, 0, m->w - 1)];
}

/* The Harris response of detect_tensor / detect_response (src/kern/detect.c:68-125) at resp[r * cols + c] (image row
 * y0 + r, column ax + c) and each 16 x 16 cell's strongest response, floored at 0 (detect_cells, detect.c:127-141),
 * at cell[cr * nv + k], in the reference's F32 operation order:
 *   gx = (2 (M(x+1) - M(x-1)) + ((U(x+1) - U(x-1)) + (D(x+1) - D(x-1)))) / 512 as one fused multiply-add, gy alike,
 *   the three products rounded; the 5-row sum added top to bottom; the 5-column box as (v + (v_-1 + v_+1)) +
 *   (v_-2 + v_+2), columns outside the region's 16-column groups reading 0; det - k trace^2 as two fused
 *   multiply-subtracts with k = 0.04. */
void or_detect_maps(const struct or_img *m, const struct or_det_geo *g, float *resp, float *cell)
{
    const int cols = g->cols, rows = g->rows, trows = rows + 4;
    const float two = 2.0f, gs = 1.0f / 512.0f, kh = 0.04f;
    float *t = malloc(sizeof(float) * 3 * (size_t)cols * (size_t)trows);
    float *xx = t, *xy = t + (size_t)cols * trows, *yy = t + 2 * (size_t)cols * trows;
    for (int r = 0; r < trows; r++) {
        const int sy = g->y0 - 2 + r;
        for (int c = 0; c < cols; c++) {
            const int x = g->ax + c;
            const float dxu = det_px(m, x + 1, sy - 1) - det_px(m, x - 1, sy - 1);
            const float dxm = det_px(m, x + 1, sy) - det_px(m, x - 1, sy);
            const float dxd = det_px(m, x + 1, sy + 1) - det_px(m, x - 1, sy + 1);
            const float gx = fmaf(dxm, two, dxu + dxd) * gs;
            const float dyl = det_px(m, x - 1, sy + 1) - det_px(m, x - 1, sy - 1);
            const float dyc = det_px(m, x, sy + 1) - det_px(m, x, sy - 1);
            const float dyr = det_px(m, x + 1, sy + 1) - det_px(m, x + 1, sy - 1);
            const float gy = fmaf(dyc, two, dyl + dyr) * gs;
            const size_t i = (size_t)r * cols + c;
            xx[i] = gx * gx;
            xy[i] = gx * gy;
            yy[i] = gy * gy;
        }
    }
    float *v = malloc(sizeof(float) * 3 * (size_t)(cols + 4));
    for (int r = 0; r < rows; r++) {
        for (int q = 0; q < 3; q++) {
            const float *p = q == 0 ? xx : q == 1 ? xy : yy;
            float *vq = v + (size_t)q * (cols + 4) + 2;
            vq[-2] = vq[-1] = vq[cols] = vq[cols + 1] = 0.0f;
            for (int c = 0; c < cols; c++) {
                const float *a = p + (size_t)r * cols + c;
                vq[c] = (((a[0] + a[cols]) + a[2 * (size_t)cols]) + a[3 * (size_t)cols]) + a[4 * (size_t)cols];
            }
        }
        const float *va = v + 2, *vb = v + (cols + 4) + 2, *vc = v + 2 * (cols + 4) + 2;
        for (int c = 0; c < cols; c++) {
            const float a = (va[c] + (va[c - 1] + va[c + 1])) + (va[c - 2] + va[c + 2]);
            const float b = (vb[c] + (vb[c - 1] + vb[c + 1])) + (vb[c - 2] + vb[c + 2]);
            const float cc = (vc[c] + (vc[c - 1] + vc[c + 1])) + (vc[c - 2] + vc[c + 2]);
            const float tr = a + cc;
            resp[(size_t)r * cols + c] = fmaf(-kh, tr * tr, fmaf(-b, b, a * cc));
        }
    }
    for (int cr = 0; cr < g->cell_rows; cr++)
        for (int k = 0; k < g->nv; k++) {
            float mx = 0.0f;
            const int r1 = (cr + 1) * 16 < rows ? (cr + 1) * 16 : rows;
            for (int r = cr * 16; r < r1; r++)
                for (int c = 16 * k; c < 16 * k + 16; c++)
                    mx = fmaxf(mx, resp[(size_t)r * cols + c]);
            cell[cr * g->nv + k] = mx;
        }
    free(v);
    free(t);
}

struct or_det_cand {
    float score;
    int order, x, y;
};

static int det_cand_cmp(const void *a, const void *b)
{
    const struct or_det_cand *p = a, *q = b;
    if (p->score != q->score)
        return p->score > q->score ? -1 : 1;
    return p->order - q->order;
}

/* detect_finish (src/kern/detect.c:175-258): the best cell, each cell's 3 x 3 neighbourhood strongest, the local
 * maxima of the response inside the rectangle above max(quality x their neighbourhood's strongest, 2500), at most
 * 8,192 in row-major scan order, scored v / local + 0.001 v / best in long double and rounded to F32; best first
 * (equal scores in scan order), then greedily those at least min_dist from every one taken, up to max. */
int or_detect_finish(const struct or_det_geo *g, const float *resp, const float *cell, int max, float min_dist,
                     float quality, float *xs, float *ys)
{
    const int nv = g->nv, ch = g->cell_rows, cols = g->cols;
    float best = 0.0f;
    for (int i = 0; i < nv * ch; i++)
        if (cell[i] > best)
            best = cell[i];
    if (best <= 0.0f)
        return 0;
    float *near = malloc(sizeof(float) * (size_t)nv * ch);
    for (int cr = 0; cr < ch; cr++)
        for (int k = 0; k < nv; k++) {
            float mx = 0.0f;
            for (int a = cr > 0 ? cr - 1 : 0; a <= cr + 1 && a < ch; a++)
                for (int b = k > 0 ? k - 1 : 0; b <= k + 1 && b < nv; b++)
                    if (cell[a * nv + b] > mx)
                        mx = cell[a * nv + b];
            near[cr * nv + k] = mx;
        }
    const int lane_lo = g->x0 - g->ax > 1 ? g->x0 - g->ax : 1, lane_hi = g->x1 - g->ax < cols - 1 ? g->x1 - g->ax : cols - 1;
    struct or_det_cand *cand = malloc(sizeof *cand * 8192);
    int nc = 0;
    for (int r = 1; r < g->rows - 1 && nc < 8192; r++) {
        const int cr = r / 16;
        for (int c = lane_lo; c < lane_hi && nc < 8192; c++) {
            const float v = resp[(size_t)r * cols + c];
            const long double local = (long double)near[cr * nv + c / 16], rel = local * (long double)quality;
            const float thresh = (float)(rel > 2500.0L ? rel : 2500.0L);
            if (!(thresh < v))
                continue;
            int keep = 1;
            for (int dr = -1; dr <= 1 && keep; dr++)
                for (int dc = -1; dc <= 1 && keep; dc++) {
                    if (!dr && !dc)
                        continue;
                    const int cc = c + dc;
                    const float nb = cc < 0 || cc >= cols ? 0.0f : resp[(size_t)(r + dr) * cols + cc];
                    keep = nb <= v;
                }
            if (!keep)
                continue;
            cand[nc].score = (float)((long double)v / local + 0.001L * (long double)v / (long double)best);
            cand[nc].order = nc;
            cand[nc].x = g->ax + c;
            cand[nc].y = g->y0 + r;
            nc++;
        }
    }
    qsort(cand, (size_t)nc, sizeof *cand, det_cand_cmp);
    const long double min2 = (long double)min_dist * (long double)min_dist;
    int need = (int)min2;
    if ((long double)need < min2)
        need++;
    int taken = 0;
    int *tx = malloc(sizeof(int) * (size_t)(max > 0 ? max : 1)), *ty = malloc(sizeof(int) * (size_t)(max > 0 ? max : 1));
    for (int i = 0; i < nc && taken < max; i++) {
        int far = 1;
        for (int k = 0; k < taken && far; k++) {
            const int dx = tx[k] - cand[i].x, dy = ty[k] - cand[i].y;
            far = dx * dx + dy * dy >= need;
        }
        if (far) {
            tx[taken] = cand[i].x;
            ty[taken] = cand[i].y;
            xs[taken] = (float)cand[i].x;
            ys[taken] = (float)cand[i].y;
            taken++;
        }
    }
    free(ty);
    free(tx);
    free(cand);
    free(near);
    return taken;
}

/* ---------------------------------------------------------------- the still picture (src/kern/still.c:143-242) */

/* One camera's still-picture state (struct still, src/kern/still.c:36-52, the fields the decision and the update use):
 * the frames in each cell's mean, this frame's weights, the usual noise, and the newest frame's statistics. */
struct or_still {
    int w, h, cols, rows, n, avg;
    float motion_px, motion_grey;
    uint64_t frames;
    long double noise_usual;
    uint16_t *count;
    float *weight;
    uint8_t *raw; /* (cols + 2) x (rows + 2), a zero border */
    uint32_t tracked, moving;
    float count_mean, drift_u, drift_v, drift_rms, diff_median, diff_limit;
};

/* What still_motion fills (src/kern/still.c:262-275), in the layout of the library's struct vtg_still_motion. */
struct or_still_motion {
    uint32_t cols, rows, tracked, moving;
    float count_mean, drift_u, drift_v, drift_rms, diff_median, diff_limit;
    uint64_t frames;
};

struct or_still *or_still_create(int w, int h, int avg, float motion_px, float motion_grey)
{
    struct or_still *s = calloc(1, sizeof *s);
    if (!s)
        return NULL;
    s->w = w;
    s->h = h;
    s->cols = (w + 15) / 16; /* VT_CELL_W x VT_CELL_H */
    s->rows = (h + 7) / 8;
    s->n = s->cols * s->rows;
    s->avg = avg;
    s->motion_px = motion_px;
    s->motion_grey = motion_grey;
    s->count = calloc((size_t)s->n, sizeof *s->count);
    s->weight = calloc((size_t)s->n, sizeof *s->weight);
    s->raw = calloc((size_t)(s->cols + 2) * (size_t)(s->rows + 2), 1);
    return s;
}

void or_still_destroy(struct or_still *s)
{
    if (!s)
        return;
    free(s->count);
    free(s->weight);
    free(s->raw);
    free(s);
}

int or_still_first(const struct or_still *s) { return s->frames == 0; }

/* still_decide (src/kern/still.c:143-222), long double as the reference: the median cell difference (a histogram of
 * 1/16 grey bins) is this camera's noise; a cell's own evidence is a good vector longer than max(12 sigma, motion_px),
 * a lost patch (LK_RESIDUAL) or a difference above max(3 noise, motion_grey); a cell moves when two cells of its 3 x 3
 * have evidence, or when the median leapt past 3x its usual value (everything moved). A moving cell's mean restarts
 * (count 1); a still one's count grows to avg. cells[].state gets the LK byte, CHANGED, MOVING and the count. */
void or_still_decide(struct or_still *s, struct or_cell *cells)
{
    const int cols = s->cols, rows = s->rows, wide = cols + 2, n = s->n;
    uint32_t hist[256] = {0};
    for (int i = 0; i < n; i++) {
        const long b = (long)((long double)cells[i].diff * 16.0L);
        hist[b < 255 ? b : 255]++;
    }
    uint32_t below = 0;
    int med = 0;
    while (med < 255 && below + hist[med] < (uint32_t)n / 2u)
        below += hist[med++];
    const long double noise = (long double)med / 16.0L, three = noise * 3.0L;
    const long double limit = three > (long double)s->motion_grey ? three : (long double)s->motion_grey;
    s->diff_median = (float)noise;
    s->diff_limit = (float)limit;
    const long double usual3 = s->noise_usual * 3.0L;
    const long double usual = usual3 > (long double)s->motion_grey ? usual3 : (long double)s->motion_grey;
    const int everything = s->frames >= 2 && noise > usual;
    if (!everything && s->frames >= 1)
        s->noise_usual = s->frames == 1 ? noise : s->noise_usual + (noise - s->noise_usual) / 32.0L;
    const long double px2 = (long double)s->motion_px * (long double)s->motion_px;
    for (int i = 0; i < n; i++) {
        const struct or_cell *c = &cells[i];
        const uint32_t lk = c->state & 0xffu;
        const long double u = c->u, v = c->v, sg = (long double)c->sigma * 12.0L;
        const long double need = sg * sg > px2 ? sg * sg : px2;
        const int moved = lk == 0 && u * u + v * v > need;
        const int failed = (lk & OR_RESIDUAL) != 0;
        const int changed = (long double)c->diff > limit;
        s->raw[(size_t)(i / cols + 1) * (size_t)wide + (size_t)(i % cols + 1)] = (uint8_t)(moved || failed || changed);
    }
    uint32_t tracked = 0, moving = 0, good = 0;
    long double su = 0.0L, sv = 0.0L, suu = 0.0L, counts = 0.0L;
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++) {
            const int i = r * cols + c;
            uint32_t votes = 0;
            for (int dy = 0; dy < 3; dy++)
                for (int dx = 0; dx < 3; dx++)
                    votes += s->raw[(size_t)(r + dy) * (size_t)wide + (size_t)(c + dx)];
            const int any = votes >= 2 || everything;
            const int own = s->raw[(size_t)(r + 1) * (size_t)wide + (size_t)(c + 1)] != 0;
            const uint32_t grown = (uint32_t)s->count[i] + 1u, cnt = any ? 1u : grown < (uint32_t)s->avg ? grown : (uint32_t)s->avg;
            s->count[i] = (uint16_t)cnt;
            s->weight[i] = (float)(1.0L / (long double)cnt);
            struct or_cell *cl = &cells[i];
            const uint32_t lk = cl->state & 0xffu;
            cl->state = lk | (own ? 0x100u : 0u) | (any ? 0x200u : 0u) | (cnt << 16);
            tracked += lk == 0;
            moving += any != 0;
            counts += (long double)cnt;
            if (lk == 0 && !any) {
                su += cl->u;
                sv += cl->v;
                suu += (long double)cl->u * cl->u + (long double)cl->v * cl->v;
                good++;
            }
        }
    s->tracked = tracked;
    s->moving = moving;
    s->count_mean = (float)(counts / (long double)n);
    const long double mu = good ? su / (long double)good : 0.0L, mv = good ? sv / (long double)good : 0.0L;
    s->drift_u = (float)mu;
    s->drift_v = (float)mv;
    const long double var = good ? suu / (long double)good - mu * mu - mv * mv : 0.0L;
    s->drift_rms = var > 0.0L ? (float)sqrtl(var) : 0.0f;
}

/* still_update (src/kern/still.c:224-246): each pixel of the mean moves toward the frame by its cell's weight,
 * m + w (f - m) as one fused multiply-add; a cell of weight 1 takes the frame exactly. Planes w x h, rows `pitch`
 * floats apart. */
void or_still_update(const struct or_still *s, float *mean, int mean_pitch, const float *cur, int cur_pitch)
{
    for (int y = 0; y < s->h; y++)
        for (int x = 0; x < s->w; x++) {
            const float wt = s->weight[(y / 8) * s->cols + x / 16];
            const float f = cur[(size_t)y * cur_pitch + x];
            float *m = &mean[(size_t)y * mean_pitch + x];
            *m = wt == 1.0f ? f : fmaf(f - *m, wt, *m);
        }
}

void or_still_finish(struct or_still *s) { s->frames++; }

void or_still_motion(const struct or_still *s, struct or_still_motion *m)
{
    m->cols = (uint32_t)s->cols;
    m->rows = (uint32_t)s->rows;
    m->tracked = s->tracked;
    m->moving = s->moving;
    m->count_mean = s->count_mean;
    m->drift_u = s->drift_u;
    m->drift_v = s->drift_v;
    m->drift_rms = s->drift_rms;
    m->diff_median = s->diff_median;
    m->diff_limit = s->diff_limit;
    m->frames = s->frames;
}

/* ---------------------------------------------------------------- frame generation (src/kern/framegen.c) */

/* The field's pyramid, the 16 x 16 SAD search of each 8 x 8 block around the coarser level's estimate, the 3 x 3
 * filter, the four-candidate upscale, the vectors at the middle instant and the blended frame, as the tracker runs
 * them for one generated frame (src/kern/track.c:847-888). Planes are whole-number Q6 values, so every sum is exact in
 * F32: the results are the reference's in any arithmetic. The reference reads its replicated padding; here that is a
 * clamped index, except where the search window's origin is clamped (that moves the offsets searched). */

#define OR_FG_LEVELS 7 /* FG_MAX_LEVELS */

struct or_fg_vec {
    int16_t x, y;
};

struct or_plane {
    const float *p;
    int w, h, stride;
};

static inline float fpx(const struct or_plane *q, int x, int y)
{
    return q->p[(size_t)clampi(y, 0, q->h - 1) * (size_t)q->stride + (size_t)clampi(x, 0, q->w - 1)];
}

/* The field's levels for w x h frames (track.c:547-556): level 0 is the frame's half size, each next half that, while
 * both sides are at least 16, seven at most. */
int or_fg_levels(int w, int h)
{
    int lw = (w + 1) / 2, lh = (h + 1) / 2, n = 0;
    while (n < OR_FG_LEVELS && lw >= 16 && lh >= 16) {
        n++;
        lw = (lw + 1) / 2;
        lh = (lh + 1) / 2;
    }
    return n;
}

/* fg_hist_section + fg_scene_verdict (framegen.c:85-113): 64 bins of 4 grey levels over every second row of nine
 * sections (columns cut to multiples of 16); the scene changed when more than half the samples moved bins. */
static void fg_hist(const struct or_plane *p, uint32_t *hist)
{
    memset(hist, 0, 9 * 64 * sizeof(uint32_t));
    for (int s = 0; s < 9; s++) {
        const int sx = s % 3, sy = s / 3;
        const int x0 = (p->w * sx / 3) & ~15, x1 = (p->w * (sx + 1) / 3) & ~15;
        const int y0 = p->h * sy / 3, y1 = p->h * (sy + 1) / 3;
        for (int y = y0; y < y1; y += 2)
            for (int x = x0; x < x1; x++)
                hist[s * 64 + ((int)(p->p[(size_t)y * p->stride + x] * (1.0f / 256.0f)) & 63)]++;
    }
}

/* The block search at one level (fg_search, framegen.c:117-214). */
static void fg_search_level(const struct or_plane *cur, const struct or_plane *old, const struct or_fg_vec *pred,
                            struct or_fg_vec *out, int bw, int bh, int level, int scene)
{
    const int lanes = (old->w + 15) & ~15;
    for (int i = 0; i < bw * bh; i++) {
        if (scene) {
            out[i].x = out[i].y = 0;
            continue;
        }
        const int px = (i % bw) * 8, py = (i / bw) * 8;
        const int wx = pred ? pred[i].x : 0, wy = pred ? pred[i].y : 0;
        const int x0 = clampi(px + wx - 8, -32, lanes), y0 = py + wy - 8;
        const int pvx = x0 - px + 8, pvy = wy;
        if (level == 0) {
            /* a block the estimate already explains is not searched (at most 2 grey levels a pixel) */
            float sum = 0.0f;
            for (int r = 0; r < 8; r++)
                for (int n = 0; n < 8; n++)
                    sum += fabsf(fpx(cur, px + n, py + r) - fpx(old, px + pvx + n, py + r + pvy));
            if (sum <= 8192.0f) {
                out[i].x = (int16_t)pvx;
                out[i].y = (int16_t)pvy;
                continue;
            }
        }
        /* 256 places, the cost of each with a tie-break toward less motion; the first lowest in row order */
        float best = 0.0f;
        int fx = 0, fy = 0;
        for (int dy = 0; dy < 16; dy++)
            for (int dx = 0; dx < 16; dx++) {
                float cost = (float)(dx > 8 ? dx - 8 : 8 - dx) + (float)(dy > 8 ? dy - 8 : 8 - dy);
                for (int r = 0; r < 8; r++)
                    for (int n = 0; n < 8; n++)
                        cost += fabsf(fpx(old, x0 + dx + n, y0 + dy + r) - fpx(cur, px + n, py + r));
                if ((dx == 0 && dy == 0) || cost < best) {
                    best = cost;
                    fx = dx;
                    fy = dy;
                }
            }
        int vx = x0 - px + fx, vy = wy + fy - 8;
        if (level == 0) {
            /* no motion, when it matches as well as the best: the finest level's fallback */
            float sum = 0.0f;
            for (int r = 0; r < 8; r++)
                for (int n = 0; n < 8; n++)
                    sum += fabsf(fpx(cur, px + n, py + r) - fpx(old, px + n, py + r));
            if (sum <= best)
                vx = vy = 0;
        }
        out[i].x = (int16_t)vx;
        out[i].y = (int16_t)vy;
    }
}

/* fg_filter (framegen.c:218-247): of the 3 x 3 around a block (clamped), the vector with the least sum of squared
 * differences from the other eight; ties to the first in column-major order. */
static void fg_filter_level(const struct or_fg_vec *in, struct or_fg_vec *out, int bw, int bh)
{
    for (int i = 0; i < bw * bh; i++) {
        const int bx = i % bw, by = i / bw;
        int mx[9], my[9], k = 0;
        for (int xx = -1; xx <= 1; xx++)
            for (int yy = -1; yy <= 1; yy++) {
                const struct or_fg_vec v = in[clampi(by + yy, 0, bh - 1) * bw + clampi(bx + xx, 0, bw - 1)];
                mx[k] = v.x;
                my[k] = v.y;
                k++;
            }
        int pick = 0;
        uint32_t least = 0;
        for (int a = 0; a < 9; a++) {
            uint32_t d = 0;
            for (int b = 0; b < 9; b++) {
                const int dx = mx[a] - mx[b], dy = my[a] - my[b];
                d += (uint32_t)(dx * dx + dy * dy);
            }
            if (a == 0 || d < least) {
                least = d;
                pick = a;
            }
        }
        out[i].x = (int16_t)mx[pick];
        out[i].y = (int16_t)my[pick];
    }
}

/* fg_upscale (framegen.c:251-288): each block of the finer level takes, of the four nearest blocks of this level, the
 * vector whose 4 x 4 SAD at this level is least (the first on a tie), doubled. */
static void fg_upscale_level(const struct or_plane *cur, const struct or_plane *old, const struct or_fg_vec *in,
                             int bw, int bh, struct or_fg_vec *out, int ow, int oh, int scene)
{
    for (int i = 0; i < ow * oh; i++) {
        if (scene) {
            out[i].x = out[i].y = 0;
            continue;
        }
        const int gx = i % ow, gy = i / ow;
        float best = 0.0f;
        int bx_ = 0, by_ = 0;
        for (int n = 0; n < 4; n++) {
            const int xo = n % 2 - 1 + gx % 2, yo = n / 2 - 1 + gy % 2;
            const struct or_fg_vec v = in[clampi(gy / 2 + yo, 0, bh - 1) * bw + clampi(gx / 2 + xo, 0, bw - 1)];
            float s = 0.0f;
            for (int r = 0; r < 4; r++)
                for (int c = 0; c < 4; c++)
                    s += fabsf(fpx(cur, gx * 4 + c, gy * 4 + r) - fpx(old, gx * 4 + c + v.x, gy * 4 + r + v.y));
            if (n == 0 || s < best) {
                best = s;
                bx_ = v.x;
                by_ = v.y;
            }
        }
        out[i].x = (int16_t)(bx_ * 2);
        out[i].y = (int16_t)(by_ * 2);
    }
}

/* How well the two frames agree over a block moved half way each (framegen.c:292-303). */
static float fg_sad_mid(const struct or_plane *a, const struct or_plane *b, int x, int y, int vx, int vy)
{
    const int ax = vx >> 1, ay = vy >> 1, bx = vx - ax, by = vy - ay;
    float s = 0.0f;
    for (int r = 0; r < 8; r++)
        for (int c = 0; c < 8; c++)
            s += fabsf(fpx(a, x + c + ax, y + r + ay) - fpx(b, x + c - bx, y + r - by));
    return s;
}

/* fg_mid_vectors (framegen.c:305-328): no motion first, favoured by one grey level over the block, then each vector
 * of the 3 x 3 that agrees better. */
static void fg_mid_level(const struct or_plane *a, const struct or_plane *b, const struct or_fg_vec *fil, int bw,
                         int bh, struct or_fg_vec *out)
{
    for (int i = 0; i < bw * bh; i++) {
        const int bx = i % bw, by = i / bw, px = bx * 8, py = by * 8;
        float best = fg_sad_mid(a, b, px, py, 0, 0) - 64.0f;
        int vx = 0, vy = 0;
        for (int yy = -1; yy <= 1; yy++)
            for (int xx = -1; xx <= 1; xx++) {
                const struct or_fg_vec v = fil[clampi(by + yy, 0, bh - 1) * bw + clampi(bx + xx, 0, bw - 1)];
                if ((v.x == vx && v.y == vy) || (v.x == 0 && v.y == 0))
                    continue;
                const float s = fg_sad_mid(a, b, px, py, v.x, v.y);
                if (s < best) {
                    best = s;
                    vx = v.x;
                    vy = v.y;
                }
            }
        out[i].x = (int16_t)vx;
        out[i].y = (int16_t)vy;
    }
}

/* fg_blend (framegen.c:332-357): 16 x 16 tiles of the full-size frame; where the nine vectors around a tile agree,
 * the two frames moved half way each, averaged; elsewhere a pixel takes from the tile's own row of vectors and the
 * row above or below, by triangles in 32nds across and down, 2048ths in all, as six fused multiply-adds in order.
 * Rounded to the nearest, ties to even. */
static void fg_blend_frame(const struct or_plane *a0, const struct or_plane *b0, const struct or_fg_vec *mid, int bw,
                           int bh, float *out, int out_stride)
{
    static const float WL[16] = {15, 13, 11, 9, 7, 5, 3, 1, 0, 0, 0, 0, 0, 0, 0, 0};
    static const float WS[16] = {17, 19, 21, 23, 25, 27, 29, 31, 31, 29, 27, 25, 23, 21, 19, 17};
    static const float WR[16] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 3, 5, 7, 9, 11, 13, 15};
    const float *wh[3] = {WL, WS, WR};
    const int w = a0->w, h = a0->h, tw = (w + 15) / 16, th = (h + 15) / 16;
    for (int t = 0; t < tw * th; t++) {
        const int tx = t % tw, ty = t / tw, x0 = tx * 16, y0 = ty * 16;
        struct or_fg_vec near[3][3];
        int same = 1;
        for (int yy = 0; yy < 3; yy++)
            for (int xx = 0; xx < 3; xx++) {
                near[yy][xx] = mid[clampi(ty + yy - 1, 0, bh - 1) * bw + clampi(tx + xx - 1, 0, bw - 1)];
                same &= near[yy][xx].x == near[0][0].x && near[yy][xx].y == near[0][0].y;
            }
        for (int y = y0; y < y0 + 16 && y < h; y++)
            for (int k = 0; k < 16 && x0 + k < w; k++) {
                const int x = x0 + k;
                float v;
                if (same) {
                    const int vx = near[0][0].x, vy = near[0][0].y;
                    v = rintf((fpx(a0, x + vx, y + vy) + fpx(b0, x - vx, y - vy)) * 0.5f);
                } else {
                    const int s = y - y0, other = s < 8 ? 0 : 2, wo = s < 8 ? 15 - 2 * s : 2 * s - 15;
                    const float vw[2] = {(float)(32 - wo), (float)wo};
                    const int rows[2] = {1, other};
                    float acc = 0.0f;
                    for (int a = 0; a < 2; a++)
                        for (int b = 0; b < 3; b++) {
                            const struct or_fg_vec q = near[rows[a]][b];
                            const float sum = fpx(a0, x + q.x, y + q.y) + fpx(b0, x - q.x, y - q.y);
                            acc = fmaf(sum, wh[b][k] * vw[a], acc);
                        }
                    v = rintf(acc * (1.0f / 2048.0f));
                }
                out[(size_t)y * out_stride + x] = v;
            }
    }
}

/* One generated frame between a0 (older) and b0 (newer), w x h Q6 planes rows `stride` floats apart. Outputs, any
 * may be NULL: the fields raw, fil and up of every level one after the other (level 0 first, each ceil(lw / 8) x
 * ceil(lh / 8); up of the top level is zero), mid (level 0's blocks), the frame out (w x h, Q6) and pic (w x h bytes,
 * img_q6_to_u8: clamp(rint(q / 64))). Returns the scene-change verdict, or -1 when the frames are smaller than
 * 64 x 64. */
int or_framegen(const float *a0, const float *b0, int w, int h, int stride, struct or_fg_vec *raw_out,
                struct or_fg_vec *fil_out, struct or_fg_vec *up_out, struct or_fg_vec *mid_out, float *out,
                uint8_t *pic)
{
    const int levels = or_fg_levels(w, h);
    if (levels < 2)
        return -1;
    float *pa[OR_FG_LEVELS], *pb[OR_FG_LEVELS];
    struct or_plane A[OR_FG_LEVELS], B[OR_FG_LEVELS];
    int bw[OR_FG_LEVELS], bh[OR_FG_LEVELS];
    size_t off[OR_FG_LEVELS + 1];
    off[0] = 0;
    int lw = w, lh = h;
    const float *sa = a0, *sb = b0;
    int ss = stride;
    for (int L = 0; L < levels; L++) {
        const int nw = (lw + 1) / 2, nh = (lh + 1) / 2;
        pa[L] = malloc(sizeof(float) * (size_t)nw * (size_t)nh);
        pb[L] = malloc(sizeof(float) * (size_t)nw * (size_t)nh);
        or_reduce(sa, lw, lh, ss, pa[L], nw);
        or_reduce(sb, lw, lh, ss, pb[L], nw);
        A[L] = (struct or_plane){pa[L], nw, nh, nw};
        B[L] = (struct or_plane){pb[L], nw, nh, nw};
        bw[L] = (nw + 7) / 8;
        bh[L] = (nh + 7) / 8;
        off[L + 1] = off[L] + (size_t)bw[L] * (size_t)bh[L];
        lw = nw;
        lh = nh;
        sa = pa[L];
        sb = pb[L];
        ss = nw;
    }
    struct or_fg_vec *raw = calloc(off[levels], sizeof *raw), *fil = calloc(off[levels], sizeof *fil);
    struct or_fg_vec *up = calloc(off[levels], sizeof *up), *mid = calloc(off[0 + 1], sizeof *mid);
    uint32_t ha[9 * 64], hb[9 * 64];
    fg_hist(&A[1], ha);
    fg_hist(&B[1], hb);
    uint64_t diff = 0, total = 0;
    for (int i = 0; i < 9 * 64; i++) {
        diff += ha[i] > hb[i] ? ha[i] - hb[i] : hb[i] - ha[i];
        total += hb[i];
    }
    const int scene = total && diff > total; /* diff / 2 / total > 0.5 */
    for (int L = levels - 1; L >= 0; L--) {
        fg_search_level(&B[L], &A[L], L == levels - 1 ? NULL : up + off[L], raw + off[L], bw[L], bh[L], L, scene);
        fg_filter_level(raw + off[L], fil + off[L], bw[L], bh[L]);
        if (L > 0)
            fg_upscale_level(&B[L], &A[L], fil + off[L], bw[L], bh[L], up + off[L - 1], bw[L - 1], bh[L - 1], scene);
    }
    fg_mid_level(&A[0], &B[0], fil, bw[0], bh[0], mid);
    float *frame = out ? out : malloc(sizeof(float) * (size_t)w * (size_t)h);
    const struct or_plane F0 = {a0, w, h, stride}, G0 = {b0, w, h, stride};
    fg_blend_frame(&F0, &G0, mid, bw[0], bh[0], frame, w);
    if (pic)
        for (size_t i = 0; i < (size_t)w * (size_t)h; i++) {
            const float s = rintf(frame[i] * (1.0f / 64.0f));
            pic[i] = s <= 0.0f ? 0u : s >= 255.0f ? 255u : (uint8_t)s;
        }
    if (raw_out)
        memcpy(raw_out, raw, sizeof *raw * off[levels]);
    if (fil_out)
        memcpy(fil_out, fil, sizeof *fil * off[levels]);
    if (up_out)
        memcpy(up_out, up, sizeof *up * off[levels]);
    if (mid_out)
        memcpy(mid_out, mid, sizeof *mid * off[1]);
    if (!out)
        free(frame);
    free(raw);
    free(fil);
    free(up);
    free(mid);
    for (int L = 0; L < levels; L++) {
        free(pa[L]);
        free(pb[L]);
    }
    return scene;
}
