/* still.cu -- one camera's still picture on the GPU: the running mean of the frames each 16 x 8 cell has held still,
 * gated by the camera's own per-cell vectors from that mean to the newest frame.
 *
 * Reference: still_vectors, still_decide, still_update and still_finish (src/kern/still.c:116-251), run in that order
 * once a frame (src/kern/still.h:11; src/host/m3_ref.c:272-277), the vectors skipped on the first frame.
 *
 * A frame is five launches on one stream, no host round trip:
 *   vectors   lk.cu's per-cell kernel: LK from the mean to the frame at every cell's centre, one level, a 15 x 15
 *             patch, 6 iterations, forward-backward 0.25 px (still.c:14-19), the cell's mean |frame - mean|;
 *   decide    three launches a thread a cell (still_decide, still.c:143-222): the noise median (a histogram of the
 *             cells' differences in 1/16 grey) and the scalars; each cell's evidence; the 3 x 3 vote, the counts,
 *             weights and states, and the drift statistics. Their FP64 work (below) is spread over every SM: GB300's
 *             FP64 rate is a small fraction of its FP32 rate, and one SM took 0.42 ms over 16,200 cells;
 *   update    a thread a pixel: m + w (f - m) as one fused multiply-add, or f where the weight is 1 (still.c:224-246).
 *
 * Exactness against the reference's long double:
 *   - the histogram, the median, the noise and its limit, the votes, the counts and the mean are exact;
 *   - the weight 1/n rounds to the same F32 through long double, double or an IEEE F32 division for every n up to
 *     65,535, so an F32 division gives it;
 *   - "a good vector longer than max(12 sigma, motion_px)" is decided exactly as the x87 does it: u^2 + v^2 is formed
 *     as an exact double-double, rounded to a 64-bit significand, and compared exactly with (12 sigma)^2;
 *   - the usual noise, a running mean over frames, is kept in FP64 (the reference: long double); it only enters the
 *     comparison of the median with three times itself;
 *   - the drift sums are exact fixed-point integers (units of 2^-60), divided and rounded to F32 once.
 * The last two agree with the reference's F32 results except where a value lies within 2^-53 of an F32 rounding
 * boundary. */
#include <math.h>
#include <stdint.h>

#include <new>

#include "vtg_ctx.h"
#include "vtg_internal.cuh"

#define STILL_BLOCK 256     /* threads a CTA, a cell each */
#define STILL_MAX_SIDE 4096 /* up to 256 x 512 cells */
#define STILL_HIST 256      /* HIST_BINS, src/kern/still.c:30 */
#define STILL_MAX_BLOCKS ((STILL_MAX_SIDE / 16) * (STILL_MAX_SIDE / 8) / STILL_BLOCK)
static_assert(STILL_BLOCK == STILL_HIST, "a thread a histogram bin");

/* The decision's state across frames, its newest statistics and the launches' hand-offs, in device memory. */
struct StillScal {
    double noise_usual;
    vtg_still_motion motion;
    double limit;      /* this frame's difference limit */
    int all;           /* this frame: everything moved */
    unsigned ticket;   /* CTAs done in the current launch; 0 between launches */
    int hist[STILL_HIST];
};

/* a double-double: hi + lo, |lo| at most half an ulp of hi */
struct DD {
    double hi, lo;
};

/* A CTA's share of the statistics: the drift sums as exact fixed-point integers, units of 2^-60. */
struct StillPart {
    int tracked, moving, good, pad;
    long long counts, pad2;
    __int128 su, sv, suu;
};

struct vtg_still {
    vtg_ctx *ctx;
    cudaStream_t stream;
    char *mem;
    size_t bytes;
    vtg_still_config c;
    int cols, rows, n, pitch;
    float *mean;
    vtg_cell *cells;
    unsigned *count;
    float *weight;
    StillScal *scal;
    unsigned char *raw; /* (cols + 2) x (rows + 2): each cell's evidence, a zero border */
    StillPart *part;
    DevPyr *dpyr; /* [0] the mean, [1] the frame: one level each */
    DevPyr hpyr[2];
    unsigned long long frames;
};

struct StillPrm {
    int cols, rows, n, avg;
    float motion_px, motion_grey;
    unsigned long long frames; /* before this one */
};

/* ---- double-double helpers: -fmad=false keeps every a * b + c here two roundings unless fma is written ---- */

__device__ __forceinline__ double two_sum_err(double a, double b, double s)
{
    const double bb = s - a;
    return (a - (s - bb)) + (b - bb);
}

__device__ __forceinline__ DD dd_add(DD a, DD b)
{
    const double s = a.hi + b.hi;
    const double e = two_sum_err(a.hi, b.hi, s) + (a.lo + b.lo);
    const double hi = s + e;
    return DD{hi, e - (hi - s)};
}

__device__ __forceinline__ DD dd_of(double a) { return DD{a, 0.0}; }

/* a / n, n > 0: a quotient and one correction term */
__device__ __forceinline__ DD dd_div(DD a, double n)
{
    const double q1 = a.hi / n;
    const double r = fma(-q1, n, a.hi) + a.lo;
    const double q2 = r / n;
    const double hi = q1 + q2;
    return DD{hi, q2 - (hi - q1)};
}

__device__ __forceinline__ DD dd_sqr(DD a)
{
    const double p = a.hi * a.hi;
    const double e = fma(a.hi, a.hi, -p) + 2.0 * a.hi * a.lo;
    const double hi = p + e;
    return DD{hi, e - (hi - p)};
}

__device__ __forceinline__ DD dd_neg(DD a) { return DD{-a.hi, -a.lo}; }

/* Whether a good vector moved (still.c:178-182): u^2 + v^2, rounded to a 64-bit significand as the x87 rounds the
 * long double sum, greater than need = max((12 sigma)^2, px^2), which is exact (56 bits at most). Both sides are
 * canonical double-doubles (head = the double nearest the sum), so they compare as (head, tail) pairs. */
__device__ bool still_longer(float u, float v, float sigma, float px)
{
    const double a = (double)u * (double)u, b = (double)v * (double)v; /* exact: 48-bit products */
    double s = a + b, t = two_sum_err(a, b, s);
    if (t != 0.0) {
        int e;
        const double m = frexp(s, &e); /* s = m 2^e, m in [0.5, 1): a 64-bit significand's unit is 2^(e - 64) */
        int k = 64 - e;
        if (m == 0.5 && t < 0.0)
            k++; /* just below a power of two: the binade below, half the unit */
        const double t64 = ldexp(rint(ldexp(t, k)), -k);
        const double s2 = s + t64;
        t = two_sum_err(s, t64, s2);
        s = s2;
    }
    const double sg = (double)sigma * 12.0; /* VEC_OVER_SIGMA, still.c:21; exact */
    double np = sg * sg, ne = fma(sg, sg, -np);
    const double p2 = (double)px * (double)px;
    if (p2 > np || (p2 == np && ne < 0.0)) {
        np = p2;
        ne = 0.0;
    }
    return s > np || (s == np && t > ne);
}

__device__ __forceinline__ int warp_sum_i(int v)
{
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1)
        v += __shfl_xor_sync(VTG_FULL, v, d);
    return v;
}

__device__ __forceinline__ DD warp_sum_dd(DD v)
{
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        DD o;
        o.hi = __shfl_xor_sync(VTG_FULL, v.hi, d);
        o.lo = __shfl_xor_sync(VTG_FULL, v.lo, d);
        v = dd_add(v, o);
    }
    return v;
}

/* The drift sums (su += u, sv += v, suu += u^2 + v^2, still.c:206-211) exactly: each F32 u, and its square (exact
 * in 48 bits), as an integer in units of 2^-60. A good vector lies on its plane (|u| < 2^13), so a square needs at
 * most 87 bits and 131,072 cells' sums fit 128; bits below 2^-60 (|u| < 2^-37, a square below 2^-60) are dropped. */
__device__ __forceinline__ __int128 fix60(float f)
{
    const unsigned b = __float_as_uint(f);
    const int ex = (int)((b >> 23) & 0xffu);
    if (ex == 0)
        return 0; /* zero, or below 2^-126 */
    const unsigned long long m = (b & 0x7fffffu) | 0x800000u;
    const int sh = min(ex - 90, 80); /* u = m 2^(ex - 150), in units of 2^-60: m 2^(ex - 90) */
    const __int128 v = sh >= 0 ? (__int128)m << sh : (__int128)(sh > -64 ? m >> -sh : 0ull);
    return (b >> 31) ? -v : v;
}

__device__ __forceinline__ __int128 fix60_sq(float f)
{
    const unsigned b = __float_as_uint(f);
    const int ex = (int)((b >> 23) & 0xffu);
    if (ex == 0)
        return 0;
    const unsigned long long m = (b & 0x7fffffu) | 0x800000u, m2 = m * m; /* 48 bits */
    const int sh = min(2 * ex - 240, 72);                                 /* u^2 = m2 2^(2 ex - 300) */
    return sh >= 0 ? (__int128)m2 << sh : (__int128)(sh > -64 ? m2 >> -sh : 0ull);
}

__device__ __forceinline__ __int128 warp_sum_i128(__int128 v)
{
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        const unsigned long long lo = __shfl_xor_sync(VTG_FULL, (unsigned long long)v, d);
        const long long hi = __shfl_xor_sync(VTG_FULL, (long long)(v >> 64), d);
        v += ((__int128)hi << 64) | (__int128)lo;
    }
    return v;
}

/* v x 2^-60 as a double-double: three 42-bit pieces of |v|, each exact in a double */
__device__ DD dd_of_fix60(__int128 v)
{
    const bool neg = v < 0;
    const unsigned __int128 a = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    const unsigned long long k = (1ull << 42) - 1ull;
    const double c0 = (double)(unsigned long long)(a & k), c1 = (double)(unsigned long long)((a >> 42) & k);
    const double c2 = (double)(unsigned long long)(a >> 84);
    DD r = dd_add(dd_add(dd_of(ldexp(c2, 24)), dd_of(ldexp(c1, -18))), dd_of(ldexp(c0, -60)));
    return neg ? dd_neg(r) : r;
}

/* still_decide (still.c:143-222) over the whole GPU in three launches, a thread a cell; the first and the last finish
 * in whichever CTA ends last (a ticket counter, no waiting): the histogram and then the scalars, the evidence, the
 * vote with the counts, weights and states and then the statistics. */

/* the camera's noise: the median cell difference, in 1/16 grey (HIST_PER_GREY); then, in the last CTA, the noise,
 * its limit, the usual noise and whether everything moved */
__global__ void __launch_bounds__(STILL_BLOCK) still_hist_kernel(StillPrm q, const vtg_cell *__restrict__ cells,
                                                                 StillScal *sc)
{
    __shared__ int s_hist[STILL_HIST];
    __shared__ bool s_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    s_hist[tid] = 0; /* STILL_BLOCK == STILL_HIST */
    __syncthreads();
    const int i = (int)(blockIdx.x * blockDim.x) + tid;
    if (i < q.n) {
        const int b = (int)(cells[i].diff * 16.0f); /* diff >= 0; x 16 is exact; the cast truncates as (long) does */
        atomicAdd(&s_hist[b < STILL_HIST - 1 ? b : STILL_HIST - 1], 1);
    }
    __syncthreads();
    if (s_hist[tid])
        atomicAdd(&sc->hist[tid], s_hist[tid]);
    __threadfence();
    __syncthreads();
    if (tid == 0)
        s_last = atomicAdd(&sc->ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!s_last || warp != 0)
        return;
    __threadfence();
    /* med = the first bin whose running count reaches n / 2, at most 255 (the reference's walk) */
    const int half = q.n / 2;
    int c[8], sum = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        c[j] = __ldcg(&sc->hist[8 * lane + j]);
        sum += c[j];
    }
    int inc = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(VTG_FULL, inc, d);
        if (lane >= d)
            inc += v;
    }
    int run = inc - sum, first = STILL_HIST - 1;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        run += c[j];
        if (run >= half && 8 * lane + j < first)
            first = 8 * lane + j;
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1)
        first = min(first, __shfl_xor_sync(VTG_FULL, first, d));
#pragma unroll
    for (int j = 0; j < 8; j++)
        sc->hist[8 * lane + j] = 0; /* ready for the next frame */
    if (lane == 0) {
        const double noise = (double)first / 16.0, three = noise * 3.0; /* DIFF_OVER_NOISE */
        const double grey = (double)q.motion_grey;
        const double limit = three > grey ? three : grey;
        const double nu = sc->noise_usual, usual3 = nu * 3.0;
        const double usual = usual3 > grey ? usual3 : grey;
        const int all = q.frames >= 2 && noise > usual;
        if (!all && q.frames >= 1)
            sc->noise_usual = q.frames == 1 ? noise : nu + (noise - nu) / 32.0; /* NOISE_FRAMES */
        sc->motion.diff_median = (float)noise;
        sc->motion.diff_limit = (float)limit;
        sc->limit = limit;
        sc->all = all;
        sc->ticket = 0;
    }
}

/* each cell's own evidence: a good vector that moved, a lost patch (LK_RESIDUAL), or a difference past the limit;
 * raw is (cols + 2) x (rows + 2) bytes whose border stays 0 */
__global__ void __launch_bounds__(STILL_BLOCK) still_evidence_kernel(StillPrm q, const vtg_cell *__restrict__ cells,
                                                                     const StillScal *__restrict__ sc,
                                                                     unsigned char *__restrict__ raw)
{
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= q.n)
        return;
    const vtg_cell c = cells[i];
    const unsigned lk = c.state & 0xffu;
    const bool moved = lk == 0 && still_longer(c.u, c.v, c.sigma, q.motion_px);
    const bool failed = (lk & 4u) != 0;
    const bool changed = (double)c.diff > sc->limit;
    raw[(i / q.cols + 1) * (q.cols + 2) + i % q.cols + 1] = (unsigned char)(moved || failed || changed);
}

/* a cell moves when two cells of its 3 x 3 have evidence (EVIDENCE_MIN) or everything moved: its mean restarts;
 * otherwise its count grows to avg. Then the statistics, in the last CTA. */
__global__ void __launch_bounds__(STILL_BLOCK) still_vote_kernel(StillPrm q, vtg_cell *__restrict__ cells,
                                                                 const unsigned char *__restrict__ raw,
                                                                 unsigned *__restrict__ count,
                                                                 float *__restrict__ weight, StillScal *sc,
                                                                 StillPart *__restrict__ part)
{
    __shared__ int s_wi[STILL_BLOCK / 32][3];
    __shared__ long long s_cnt[STILL_BLOCK / 32];
    __shared__ __int128 s_ws[STILL_BLOCK / 32][3];
    __shared__ bool s_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int i = (int)(blockIdx.x * blockDim.x) + tid;
    const bool all = sc->all != 0;
    int tracked = 0, moving = 0, good = 0;
    long long counts = 0;
    __int128 su = 0, sv = 0, suu = 0;
    if (i < q.n) {
        const int wide = q.cols + 2, r = i / q.cols, col = i - r * q.cols;
        const unsigned char *a = raw + r * wide + col;
        const int votes = a[0] + a[1] + a[2] + a[wide] + a[wide + 1] + a[wide + 2] + a[2 * wide] + a[2 * wide + 1] +
                          a[2 * wide + 2];
        const bool any = votes >= 2 || all;
        const bool own = a[wide + 1] != 0;
        const unsigned grown = count[i] + 1u;
        const unsigned n = any ? 1u : grown < (unsigned)q.avg ? grown : (unsigned)q.avg;
        count[i] = n;
        weight[i] = __fdiv_rn(1.0f, (float)n);
        const vtg_cell c = cells[i];
        const unsigned lk = c.state & 0xffu;
        cells[i].state = lk | (own ? 0x100u : 0u) | (any ? 0x200u : 0u) | (n << 16);
        tracked = lk == 0;
        moving = any;
        counts = n;
        if (lk == 0 && !any) {
            su = fix60(c.u);
            sv = fix60(c.v);
            suu = fix60_sq(c.u) + fix60_sq(c.v);
            good = 1;
        }
    }
    /* the CTA's share, then (in the CTA that ends last) every share: the same reduction twice */
    for (int pass = 0; pass < 2; pass++) {
        tracked = warp_sum_i(tracked);
        moving = warp_sum_i(moving);
        good = warp_sum_i(good);
#pragma unroll
        for (int d = 16; d >= 1; d >>= 1)
            counts += __shfl_xor_sync(VTG_FULL, counts, d);
        su = warp_sum_i128(su);
        sv = warp_sum_i128(sv);
        suu = warp_sum_i128(suu);
        if (lane == 0) {
            s_wi[warp][0] = tracked;
            s_wi[warp][1] = moving;
            s_wi[warp][2] = good;
            s_cnt[warp] = counts;
            s_ws[warp][0] = su;
            s_ws[warp][1] = sv;
            s_ws[warp][2] = suu;
        }
        __syncthreads();
        if (tid == 0) {
            StillPart P{};
            for (int w = 0; w < STILL_BLOCK / 32; w++) {
                P.tracked += s_wi[w][0];
                P.moving += s_wi[w][1];
                P.good += s_wi[w][2];
                P.counts += s_cnt[w];
                P.su += s_ws[w][0];
                P.sv += s_ws[w][1];
                P.suu += s_ws[w][2];
            }
            if (pass == 0) {
                part[blockIdx.x] = P;
                __threadfence();
                s_last = atomicAdd(&sc->ticket, 1u) == gridDim.x - 1;
            } else {
                vtg_still_motion &m = sc->motion;
                m.cols = (uint32_t)q.cols;
                m.rows = (uint32_t)q.rows;
                m.tracked = (uint32_t)P.tracked;
                m.moving = (uint32_t)P.moving;
                m.count_mean = (float)((double)P.counts / (double)q.n);
                if (P.good > 0) {
                    const double G = (double)P.good;
                    const DD mu = dd_div(dd_of_fix60(P.su), G), mv = dd_div(dd_of_fix60(P.sv), G);
                    const DD var =
                        dd_add(dd_add(dd_div(dd_of_fix60(P.suu), G), dd_neg(dd_sqr(mu))), dd_neg(dd_sqr(mv)));
                    m.drift_u = (float)(mu.hi + mu.lo);
                    m.drift_v = (float)(mv.hi + mv.lo);
                    const double vv = var.hi + var.lo;
                    m.drift_rms = vv > 0.0 ? (float)sqrt(vv) : 0.0f;
                } else {
                    m.drift_u = m.drift_v = m.drift_rms = 0.0f;
                }
                m.frames = q.frames + 1;
                sc->ticket = 0;
            }
        }
        __syncthreads();
        if (pass == 1 || !s_last)
            return;
        /* the last CTA: every CTA's share, a thread a share (read through L2, where the others' stores are) */
        __threadfence();
        tracked = moving = good = 0;
        counts = 0;
        su = sv = suu = 0;
        for (int b = tid; b < (int)gridDim.x; b += blockDim.x) {
            const StillPart *pb = part + b;
            tracked += __ldcg(&pb->tracked);
            moving += __ldcg(&pb->moving);
            good += __ldcg(&pb->good);
            counts += __ldcg(&pb->counts);
            const long long *w = reinterpret_cast<const long long *>(&pb->su);
            su += ((__int128)__ldcg(w + 1) << 64) | (__int128)(unsigned long long)__ldcg(w);
            sv += ((__int128)__ldcg(w + 3) << 64) | (__int128)(unsigned long long)__ldcg(w + 2);
            suu += ((__int128)__ldcg(w + 5) << 64) | (__int128)(unsigned long long)__ldcg(w + 4);
        }
    }
}

/* still_update (still.c:224-246): a thread a pixel of row blockIdx.y. */
__global__ void still_update_kernel(float *__restrict__ mean, int mpitch, const float *__restrict__ cur, int cpitch,
                                    const float *__restrict__ weight, int w, int cols)
{
    const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)blockIdx.y;
    if (x >= w)
        return;
    const float wt = weight[(y >> 3) * cols + (x >> 4)];
    const float f = cur[(size_t)y * cpitch + x];
    float *m = mean + (size_t)y * mpitch + x;
    *m = wt == 1.0f ? f : __fmaf_rn(f - *m, wt, *m);
}

/* ---- the C ABI ---- */

#define CU(call)                                                                                                       \
    do {                                                                                                               \
        const cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess) {                                                                                       \
            vtg_set_cuda_error(e_);                                                                                    \
            return VTG_ECUDA;                                                                                          \
        }                                                                                                              \
    } while (0)

static size_t up256(size_t n) { return (n + 255) & ~(size_t)255; }

struct StillLayout {
    size_t mean, cells, count, weight, scal, raw, part, dpyr, bytes;
};

static bool still_cfg_ok(const vtg_still_config *c)
{
    return c && c->w >= 32 && c->h >= 32 && c->w <= STILL_MAX_SIDE && c->h <= STILL_MAX_SIDE && c->avg >= 1 &&
           c->avg <= 65535 && c->motion_px >= 0.0f && c->motion_grey >= 0.0f;
}

static StillLayout still_layout(const vtg_still_config *c)
{
    const int cols = (c->w + 15) / 16, rows = (c->h + 7) / 8, n = cols * rows;
    StillLayout L;
    size_t b = 0;
    L.mean = b;
    b += up256(sizeof(float) * (size_t)vtg_pitch(c->w) * (size_t)c->h);
    L.cells = b;
    b += up256(sizeof(vtg_cell) * (size_t)n);
    L.count = b;
    b += up256(sizeof(unsigned) * (size_t)n);
    L.weight = b;
    b += up256(sizeof(float) * (size_t)n);
    L.scal = b;
    b += up256(sizeof(StillScal));
    L.raw = b;
    b += up256((size_t)(cols + 2) * (size_t)(rows + 2));
    L.part = b;
    b += up256(sizeof(StillPart) * (size_t)((n + STILL_BLOCK - 1) / STILL_BLOCK));
    L.dpyr = b;
    b += up256(2 * sizeof(DevPyr));
    L.bytes = b;
    return L;
}

extern "C" size_t vtg_still_bytes(const struct vtg_still_config *c)
{
    return still_cfg_ok(c) ? still_layout(c).bytes : 0;
}

extern "C" int vtg_still_create(vtg_ctx *ctx, const struct vtg_still_config *c, vtg_still **out)
{
    if (!ctx || !out || !still_cfg_ok(c))
        return VTG_EINVAL;
    *out = nullptr;
    const StillLayout L = still_layout(c);
    const int charged = vtg_ctx_charge(ctx, L.bytes);
    if (charged != VTG_OK)
        return charged;
    vtg_still *s = new (std::nothrow) vtg_still;
    if (!s) {
        vtg_ctx_release(ctx, L.bytes);
        return VTG_ENOMEM;
    }
    s->ctx = ctx;
    s->bytes = L.bytes;
    s->c = *c;
    s->cols = (c->w + 15) / 16;
    s->rows = (c->h + 7) / 8;
    s->n = s->cols * s->rows;
    s->pitch = vtg_pitch(c->w);
    s->frames = 0;
    cudaError_t e = cudaSetDevice(vtg_ctx_device(ctx));
    if (e == cudaSuccess)
        e = cudaMalloc(&s->mem, L.bytes);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        vtg_ctx_release(ctx, L.bytes);
        delete s;
        return VTG_ENOMEM;
    }
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    /* every field starts at zero, as still_create leaves them (still.c:82-87): the mean, the cells, the counts */
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s->mem, 0, L.bytes, s->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        if (s->stream)
            cudaStreamDestroy(s->stream);
        cudaFree(s->mem);
        vtg_ctx_release(ctx, L.bytes);
        delete s;
        return VTG_ECUDA;
    }
    s->mean = (float *)(s->mem + L.mean);
    s->cells = (vtg_cell *)(s->mem + L.cells);
    s->count = (unsigned *)(s->mem + L.count);
    s->weight = (float *)(s->mem + L.weight);
    s->scal = (StillScal *)(s->mem + L.scal);
    s->raw = (unsigned char *)(s->mem + L.raw);
    s->part = (StillPart *)(s->mem + L.part);
    s->dpyr = (DevPyr *)(s->mem + L.dpyr);
    for (int k = 0; k < 2; k++) {
        s->hpyr[k] = DevPyr{};
        s->hpyr[k].levels = 1;
        s->hpyr[k].l[0].w = c->w;
        s->hpyr[k].l[0].h = c->h;
    }
    s->hpyr[0].l[0].p = s->mean;
    s->hpyr[0].l[0].pitch = s->pitch;
    vtg_ctx_track(ctx, s->stream, true);
    *out = s;
    return VTG_OK;
}

extern "C" void vtg_still_destroy(vtg_still *s)
{
    if (!s)
        return;
    cudaSetDevice(vtg_ctx_device(s->ctx));
    cudaStreamSynchronize(s->stream);
    vtg_ctx_track(s->ctx, s->stream, false);
    cudaStreamDestroy(s->stream);
    cudaFree(s->mem);
    vtg_ctx_release(s->ctx, s->bytes);
    delete s;
}

extern "C" void *vtg_still_stream(const vtg_still *s) { return s ? (void *)s->stream : nullptr; }

extern "C" int vtg_still_frame(vtg_still *s, const float *cur, int pitch, const struct vtg_cell *cells_in, int where,
                               void *stream)
{
    if (!s || !cur || pitch < s->c.w || (cells_in && where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    CU(cudaSetDevice(vtg_ctx_device(s->ctx)));
    const int w = s->c.w, h = s->c.h;
    if (cells_in) {
        CU(cudaMemcpyAsync(s->cells, cells_in, sizeof(vtg_cell) * (size_t)s->n,
                           where == VTG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    } else if (s->frames > 0) {
        /* still_vectors (still.c:116-141): the mean to the frame, one level; PATCH, LK_ITER, LK_EPS, LK_MIN_EIG,
         * LK_MAX_RESIDUAL, FB_MAX (still.c:14-19) */
        s->hpyr[1].l[0].p = cur;
        s->hpyr[1].l[0].pitch = pitch;
        CU(cudaMemcpyAsync(s->dpyr, s->hpyr, sizeof(s->hpyr), cudaMemcpyHostToDevice, st));
        LkPrm p;
        p.W = 15;
        p.H = 15;
        p.max_iter = 6;
        p.eps2 = 0.01f * 0.01f;
        p.min_eig = 0.1f;
        p.max_residual = 16.0f;
        p.fb_max2 = 0.25f * 0.25f;
        p.area = 225.0f;
        CellGrid g;
        g.cell_w = 16;
        g.cell_h = 8;
        g.cols = s->cols;
        g.rows = s->rows;
        g.n = s->n;
        CU(vtg_launch_cells(s->dpyr, s->dpyr + 1, 0, p, g, w, h, nullptr, s->cells, st));
    }
    StillPrm q;
    q.cols = s->cols;
    q.rows = s->rows;
    q.n = s->n;
    q.avg = s->c.avg;
    q.motion_px = s->c.motion_px;
    q.motion_grey = s->c.motion_grey;
    q.frames = s->frames;
    const int nb = (s->n + STILL_BLOCK - 1) / STILL_BLOCK;
    still_hist_kernel<<<nb, STILL_BLOCK, 0, st>>>(q, s->cells, s->scal);
    still_evidence_kernel<<<nb, STILL_BLOCK, 0, st>>>(q, s->cells, s->scal, s->raw);
    still_vote_kernel<<<nb, STILL_BLOCK, 0, st>>>(q, s->cells, s->raw, s->count, s->weight, s->scal, s->part);
    still_update_kernel<<<dim3((w + 255) / 256, h), 256, 0, st>>>(s->mean, s->pitch, cur, pitch, s->weight, w,
                                                                  s->cols);
    CU(cudaGetLastError());
    s->frames++; /* still_finish (still.c:248-251) */
    return VTG_OK;
}

extern "C" int vtg_still_read(vtg_still *s, struct vtg_cell *cells, struct vtg_still_motion *motion, float *mean,
                              int mean_pitch, int where, void *stream)
{
    if (!s || (where != VTG_HOST && where != VTG_DEVICE) || (mean && mean_pitch < s->c.w))
        return VTG_EINVAL;
    const cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    const cudaMemcpyKind k = where == VTG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    CU(cudaSetDevice(vtg_ctx_device(s->ctx)));
    if (cells)
        CU(cudaMemcpyAsync(cells, s->cells, sizeof(vtg_cell) * (size_t)s->n, k, st));
    if (motion)
        CU(cudaMemcpyAsync(motion, &s->scal->motion, sizeof(vtg_still_motion), k, st));
    if (mean)
        CU(cudaMemcpy2DAsync(mean, sizeof(float) * (size_t)mean_pitch, s->mean, sizeof(float) * (size_t)s->pitch,
                             sizeof(float) * (size_t)s->c.w, (size_t)s->c.h, k, st));
    if (where == VTG_HOST)
        CU(cudaStreamSynchronize(st));
    return VTG_OK;
}

extern "C" int vtg_still_mean(const vtg_still *s, const float **plane, int *pitch)
{
    if (!s || !plane || !pitch)
        return VTG_EINVAL;
    *plane = s->mean;
    *pitch = s->pitch;
    return VTG_OK;
}
