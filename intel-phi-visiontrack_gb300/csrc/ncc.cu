/* ncc.cu -- the appearance search: zero-mean normalised cross-correlation of a T_w x T_h template over a window of
 * corners, the best corner of every 16 x 16 cell of corners, the eight best cells looked at again in half pixels, the
 * best and the second peak, and the parabola's sub-half-pixel offsets.
 *
 * Reference: search_at / tk_correlate (src/kern/track.c:184-208), OP_SEARCH (track.c:301-329), search_slot
 * (track.c:1661-1726), search_half (track.c:1615-1647), peak_offset (track.c:1650-1657), take_back (track.c:1737-1775).
 * The reference's template is 32 x 21 on a Q6 plane; here T_w (a multiple of 8, <= 128) x T_h (<= 128) on an 8-bit or
 * Q6 plane.
 *
 * Score at corner (x, y): st = sum t (J - J(x, y)); var = sum J^2 - (sum J)^2 / n; 0 when var <= norm / 16 or
 * norm <= 0, else st / sqrt(norm var). The window sums come from exact int64 integral images (sum J and sum J^2), so the
 * near-blank rule compares an exact integer n var with n norm / 16 and never lets a flat window through.
 *
 * Pipeline (all on one stream, no host round trip):
 *   integral_rows / integral_cols  int64 tables of J and J^2 ((h + 1) x (w + 1)), exact: for the F32 map at steps 4 to
 *                                 16, and at steps 1 and 2 where ncc_sums_in_map leaves the window sums to them (the
 *                                 tensor-core map's preparation (ncc_prep) sums the window bytes directly)
 *   ncc_map_f32q (steps 1 and 2), ncc_map_f32 (steps 4 to 16), or the tensor-core map in ncc_tc.cu
 *                                 per cell: best score and its corner
 *   ncc_top_ctas                  the eight best cells, value descending then cell index ascending (the reference's
 *                                 insertion order): a list a CTA, merged by the CTA that finishes last
 *   ncc_half_all (+ ncc_pick)     each candidate in half pixels within +-(2 step - 1) (or +-1) and one ring past it,
 *                                 one CTA per corner; then, in the CTA that finishes last, the best, the second peak
 *                                 clear of it by half a template, and the parabola offsets from the ring; F32 products
 *                                 with exact integer (quarter-pixel) window sums. */
#include <float.h>

#include <type_traits>

#include "vtg_internal.cuh"
#include "vtg_ncc.cuh"

/* ---- integral images ---- */

template <typename T>
__device__ __forceinline__ long long pix(const T *p, size_t i)
{
    return (long long)__ldg(p + i);
}

/* Row pass: table row y + 1, columns 1 .. w, holds the prefix of row y (and of its squares); row 0 and column 0 are
 * zero. One warp per row, 4 pixels a lane per round, sums in 64 bits. */
template <typename T>
__global__ void integral_rows(const T *__restrict__ plane, int pitch, int w, int h, long long *__restrict__ S1,
                              long long *__restrict__ S2, int tp)
{
    const int lane = threadIdx.x & 31;
    const int y = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (y > h)
        return;
    long long *r1 = S1 + (size_t)y * tp, *r2 = S2 + (size_t)y * tp;
    if (y == 0) {
        for (int x = lane; x <= w; x += 32)
            r1[x] = r2[x] = 0;
        return;
    }
    if (lane == 0)
        r1[0] = r2[0] = 0;
    long long c1 = 0, c2 = 0;
    const T *src = plane + (size_t)(y - 1) * pitch;
    for (int x0 = 0; x0 < w; x0 += 128) {
        long long v[4], q[4];
        long long a1 = 0, a2 = 0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int x = x0 + 4 * lane + k;
            const long long p = x < w ? pix(src, x) : 0;
            a1 += p;
            a2 += p * p;
            v[k] = a1;
            q[k] = a2;
        }
        long long s1 = a1, s2 = a2;
#pragma unroll
        for (int s = 1; s < 32; s <<= 1) {
            const long long b1 = __shfl_up_sync(VTG_FULL, s1, s), b2 = __shfl_up_sync(VTG_FULL, s2, s);
            if (lane >= s) {
                s1 += b1;
                s2 += b2;
            }
        }
        const long long e1 = c1 + s1 - a1, e2 = c2 + s2 - a2; /* exclusive prefix of this lane's four */
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int x = x0 + 4 * lane + k;
            if (x < w) {
                r1[x + 1] = e1 + v[k];
                r2[x + 1] = e2 + q[k];
            }
        }
        c1 += __shfl_sync(VTG_FULL, s1, 31);
        c2 += __shfl_sync(VTG_FULL, s2, 31);
    }
}

/* Column pass: running sums down the rows. A CTA takes 32 columns and splits the rows into 32 segments: each thread
 * sums its segment, the segments' totals are scanned in shared memory, and each thread adds its offset. */
#define IC_COLS 32
#define IC_SEGS 32
__global__ void __launch_bounds__(IC_COLS *IC_SEGS) integral_cols(int w, int h, long long *__restrict__ S1,
                                                                  long long *__restrict__ S2, int tp)
{
    __shared__ long long t1[IC_SEGS][IC_COLS + 1], t2[IC_SEGS][IC_COLS + 1];
    const int c = threadIdx.x % IC_COLS, g = threadIdx.x / IC_COLS;
    const int x = blockIdx.x * IC_COLS + c;
    const int rows = h + 1, seg = (rows + IC_SEGS - 1) / IC_SEGS;
    const int r0 = g * seg, r1 = min(r0 + seg, rows);
    long long a = 0, b = 0;
    if (x <= w)
        for (int y = r0; y < r1; y++) {
            const size_t i = (size_t)y * tp + x;
            a += S1[i];
            b += S2[i];
            S1[i] = a;
            S2[i] = b;
        }
    t1[g][c] = a;
    t2[g][c] = b;
    __syncthreads();
    if (g == 0) {
        long long o1 = 0, o2 = 0;
        for (int k = 0; k < IC_SEGS; k++) {
            const long long u1 = t1[k][c], u2 = t2[k][c];
            t1[k][c] = o1;
            t2[k][c] = o2;
            o1 += u1;
            o2 += u2;
        }
    }
    __syncthreads();
    const long long o1 = t1[g][c], o2 = t2[g][c];
    if (x <= w && (o1 | o2))
        for (int y = r0; y < r1; y++) {
            const size_t i = (size_t)y * tp + x;
            S1[i] += o1;
            S2[i] += o2;
        }
}

/* ---- the score, shared by every map kernel ---- */

__device__ __forceinline__ long long box(const long long *S, int tp, int x, int y, int tw, int th)
{
    const long long *a = S + (size_t)y * tp + x, *b = S + (size_t)(y + th) * tp + x;
    return b[tw] - b[0] - a[tw] + a[0];
}

/* score from st and the exact window sums; -1 where the corner is outside the reference's bounds. */
__device__ __forceinline__ float ncc_score(float st, long long s1, long long s2, const NccPrm &p)
{
    const long long nvar = (long long)p.n * s2 - s1 * s1; /* n var, exact */
    if (nvar <= p.nthr || p.norm <= 0.0f)
        return 0.0f;
    const float var = (float)nvar / (float)p.n;
    return st / sqrtf(p.norm * var);
}

/* ---- the map, F32 products: one CTA a cell (steps 4 to 16), or 32 x 32 corners a CTA (steps 1 and 2) ---- */

/* A cell's best: value descending, then row-major scan order (the first maximum wins, as OP_SEARCH's strict > does). */
__device__ __forceinline__ bool better(float v, int k, float bv, int bk) { return v > bv || (v == bv && k < bk); }

template <typename T>
__global__ void __launch_bounds__(256) ncc_map_f32(const T *__restrict__ plane, int pitch, const float *__restrict__ app,
                                                   NccPrm p, const long long *__restrict__ S1,
                                                   const long long *__restrict__ S2, int tp, float *__restrict__ map_v,
                                                   int *__restrict__ map_x, int *__restrict__ map_y)
{
    extern __shared__ __align__(16) float sm[];
    const int cell = blockIdx.x;
    const int cx0 = p.x0 + (cell % p.ccols) * NCC_CELL, cy0 = p.y0 + (cell / p.ccols) * NCC_CELL;
    const int cx1 = min(cx0 + NCC_CELL, p.x1 + 1), cy1 = min(cy0 + NCC_CELL, p.y1 + 1);
    const int iw = NCC_CELL + p.tw, ih = NCC_CELL + p.th;
    float *s_app = sm, *s_img = sm + p.tw * p.th;
    for (int i = threadIdx.x; i < p.tw * p.th; i += blockDim.x)
        s_app[i] = app[i];
    for (int i = threadIdx.x; i < iw * ih; i += blockDim.x) {
        const int r = i / iw, c = i - r * iw;
        const int yy = min(cy0 + r, p.h - 1), xx = min(cx0 + c, p.w - 1);
        s_img[i] = (float)__ldg(plane + (size_t)yy * pitch + xx);
    }
    __syncthreads();
    const int per = NCC_CELL / p.step;
    const int a = threadIdx.x % NCC_CELL, b = threadIdx.x / NCC_CELL;
    float v = -2.0f;
    int key = 1 << 30;
    if (a < per && b < per) {
        const int x = cx0 + a * p.step, y = cy0 + b * p.step;
        if (x < cx1 && y < cy1) {
            key = b * per + a;
            const float *im = s_img + (y - cy0) * iw + (x - cx0);
            const float first = im[0];
            float s0 = 0.f, s1 = 0.f;
            for (int i = 0; i < p.th; i++) {
                const float *row = im + i * iw, *t = s_app + i * p.tw;
                for (int j = 0; j < p.tw; j += 2) {
                    s0 = __fmaf_rn(row[j] - first, t[j], s0);
                    s1 = __fmaf_rn(row[j + 1] - first, t[j + 1], s1);
                }
            }
            v = ncc_score(s0 + s1, box(S1, tp, x, y, p.tw, p.th), box(S2, tp, x, y, p.tw, p.th), p);
        }
    }
    /* block argmax */
    __shared__ float rv[8];
    __shared__ int rk[8];
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const float ov = __shfl_xor_sync(VTG_FULL, v, s);
        const int ok = __shfl_xor_sync(VTG_FULL, key, s);
        if (better(ov, ok, v, key)) {
            v = ov;
            key = ok;
        }
    }
    const int warp = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        rv[warp] = v;
        rk[warp] = key;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float bv = rv[0];
        int bk = rk[0];
        for (int k = 1; k < 8; k++)
            if (better(rv[k], rk[k], bv, bk)) {
                bv = rv[k];
                bk = rk[k];
            }
        if (bk >= (1 << 30)) { /* no corner: the reference leaves top at -2 and the cell origin */
            map_v[cell] = -2.0f;
            map_x[cell] = cx0;
            map_y[cell] = cy0;
        } else {
            /* a cell whose every corner reads -1 (out of bounds) keeps -2 and its origin, as `v > top` never fires */
            const bool fired = bv > -2.0f;
            map_v[cell] = fired ? bv : -2.0f;
            map_x[cell] = fired ? cx0 + (bk % per) * p.step : cx0;
            map_y[cell] = fired ? cy0 + (bk / per) * p.step : cy0;
        }
    }
}

/* The F32 map at steps 1 and 2 (the steps the reference's searches take), four corners a thread. A CTA of 256 threads
 * takes 32 x 32 corners: 2 x 2 cells at step 1, 4 x 4 at step 2. It stages their window and the template in shared
 * memory, the window's rows at an odd pitch so that the four or eight picture rows a warp reads fall in different
 * banks. A thread scores four corners of one row, ST apart. As the column pair j advances by 2, the picture values
 * the four corners read are a window of M = 3 ST + 2 registers sliding along the row: two loads and one template load
 * feed eight products. Each corner's sums run in ncc_map_f32's order (rows, then columns in even and odd chains), so
 * the map is the same bits. A cell's best is a shared-memory atomicMax of (ordered score, inverted scan index): value
 * descending, then scan order, as `better`. A score that underflowed to -0 is taken as +0 first (adding +0), so the two
 * zeros tie as they compare in `better`.
 * With SUMS the window sums (sum J, sum J^2) come from the staged window too, in 64-bit integers, once the products are
 * done and the template's shared memory is free: a thread a column keeps the column's sum over the template's rows,
 * sliding down the corner rows, and writes eight corner rows of column sums at a time; each corner's thread adds its
 * row's T_w column sums, and slides ST columns to the next corner. The integers are the integral images' box sums, so
 * the scores are those of ncc_map_f32 bit for bit, and the search needs no integral images. Without SUMS they come from
 * the integral images (ncc_sums_in_map decides). */
#define NMQ_K 4       /* corners a thread */
#define NMQ_CORNERS 32 /* corners a CTA's side */

/* The window a CTA of ncc_map_f32q<ST> stages: columns (with the two values the sliding window reads past the last
 * corner's row on its last column pair), its odd pitch, and rows. */
__host__ __device__ inline int nmq_cols(int st, int tw) { return (NMQ_CORNERS - 1) * st + tw + 2; }
__host__ __device__ inline int nmq_pitch(int st, int tw) { return nmq_cols(st, tw) | 1; }
__host__ __device__ inline int nmq_rows(int st, int th) { return (NMQ_CORNERS - 1) * st + th; }
/* the columns a CTA's corners' windows cover, and the floats of shared memory before the window: the template, later
 * eight corner rows of column sums (two int64 tables) in the same place */
__host__ __device__ inline int nmq_sum_cols(int st, int tw) { return (NMQ_CORNERS - 1) * st + tw; }
__host__ __device__ inline int nmq_head(int st, int tw, int th)
{
    const int t = tw * th, c = 32 * nmq_sum_cols(st, tw);
    return t > c ? t : c;
}

/* A staged value as the integral images take it, (long long) of the plane's value: in 32 bits where it is known to fit
 * (bytes always; F32 planes when every value the CTA staged does), since the 64-bit conversion runs on the FP64 pipe. */
template <bool W32>
__device__ __forceinline__ long long nmq_int(float v)
{
    return W32 ? (long long)__float2int_rz(v) : __float2ll_rz(v);
}

/* Column t's sums (J, J^2) over rows 0 .. th - 1 of the staged window, as two chains. */
template <bool W32>
__device__ __forceinline__ void nmq_col_first(const float *s_img, int ip, int th, int t, long long &r1, long long &r2)
{
    long long a1 = 0, a2 = 0, b1 = 0, b2 = 0;
    int i = 0;
    for (; i + 1 < th; i += 2) {
        const long long u = nmq_int<W32>(s_img[i * ip + t]), v = nmq_int<W32>(s_img[(i + 1) * ip + t]);
        a1 += u;
        a2 += u * u;
        b1 += v;
        b2 += v * v;
    }
    if (i < th) {
        const long long u = nmq_int<W32>(s_img[i * ip + t]);
        a1 += u;
        a2 += u * u;
    }
    r1 = a1 + b1;
    r2 = a2 + b2;
}

/* Column t's sums one window row down: row ro leaves, row ro + th enters. */
template <bool W32>
__device__ __forceinline__ void nmq_col_slide(const float *s_img, int ip, int th, int t, int ro, long long &r1, long long &r2)
{
    const long long vo = nmq_int<W32>(s_img[ro * ip + t]), vn = nmq_int<W32>(s_img[(ro + th) * ip + t]);
    r1 += vn - vo;
    r2 += vn * vn - vo * vo;
}

/* With SUMS, six CTAs an SM: the sums' phase would otherwise take the registers to 48 and small templates to five CTAs
 * an SM. Without it no bound: the integral images' variant runs large templates, which shared memory already holds to
 * one or two CTAs an SM, and the bound slowed it (96 x 96 by 4 %). */
template <typename T, int ST, bool SUMS>
__global__ void __launch_bounds__(256, SUMS ? 6 : 1) ncc_map_f32q(const T *__restrict__ plane, int pitch, const float *__restrict__ app,
                                                    NccPrm p, const long long *__restrict__ S1,
                                                    const long long *__restrict__ S2, int tp, int bcols,
                                                    float *__restrict__ map_v, int *__restrict__ map_x,
                                                    int *__restrict__ map_y)
{
    constexpr int BC = NMQ_CORNERS * ST / NCC_CELL; /* cells a CTA's side */
    constexpr int PER = NCC_CELL / ST;             /* corners a cell's side */
    constexpr int M = (NMQ_K - 1) * ST + 2;        /* the sliding window */
    extern __shared__ __align__(16) float sm[];
    __shared__ unsigned long long s_best[BC * BC];
    const int bx = blockIdx.x % bcols, by = blockIdx.x / bcols;
    const int ccx0 = BC * bx, ccy0 = BC * by; /* the CTA's first cell column and row */
    const int X0 = p.x0 + ccx0 * NCC_CELL, Y0 = p.y0 + ccy0 * NCC_CELL;
    const int iw = nmq_cols(ST, p.tw), ip = nmq_pitch(ST, p.tw), ih = nmq_rows(ST, p.th);
    float *s_app = sm, *s_img = sm + nmq_head(ST, p.tw, p.th); /* a multiple of 8 floats: s_img stays 16-byte aligned */
    for (int i = threadIdx.x; i < p.tw * p.th; i += blockDim.x)
        s_app[i] = app[i];
    bool small = true; /* every value this thread staged converts to the same integer in 32 bits */
    for (int i = threadIdx.x; i < iw * ih; i += blockDim.x) {
        const int r = i / iw, c = i - r * iw;
        const int yy = min(Y0 + r, p.h - 1), xx = min(X0 + c, p.w - 1);
        const float v = (float)__ldg(plane + (size_t)yy * pitch + xx);
        s_img[r * ip + c] = v;
        small = small && fabsf(v) < 2147483648.0f;
    }
    if (threadIdx.x < BC * BC)
        s_best[threadIdx.x] = 0ull;
    const bool w32 = __syncthreads_and(small ? 1 : 0) != 0 || sizeof(T) == 1;
    constexpr int GROUPS = NMQ_CORNERS / NMQ_K;
    const int t = threadIdx.x;
    const int b = t / GROUPS, a0 = (t - b * GROUPS) * NMQ_K; /* corner row, first corner column in the CTA */
    const float *rowb = s_img + (b * ST) * ip + a0 * ST;
    float first[NMQ_K], s0[NMQ_K], s1[NMQ_K];
#pragma unroll
    for (int c = 0; c < NMQ_K; c++) {
        first[c] = rowb[c * ST];
        s0[c] = s1[c] = 0.0f;
    }
    for (int i = 0; i < p.th; i++) {
        const float *row = rowb + i * ip, *tt = s_app + i * p.tw;
        float w[M];
#pragma unroll
        for (int m = 0; m < M; m++)
            w[m] = row[m];
#pragma unroll 4
        for (int j = 0; j < p.tw; j += 2) {
            const float2 tv = *reinterpret_cast<const float2 *>(tt + j);
#pragma unroll
            for (int c = 0; c < NMQ_K; c++) {
                s0[c] = __fmaf_rn(w[c * ST] - first[c], tv.x, s0[c]);
                s1[c] = __fmaf_rn(w[c * ST + 1] - first[c], tv.y, s1[c]);
            }
#pragma unroll
            for (int m = 0; m < M - 2; m++)
                w[m] = w[m + 2];
            w[M - 2] = row[j + M];
            w[M - 1] = row[j + M + 1];
        }
    }
    float sc[NMQ_K]; /* the corners' st, then their scores */
#pragma unroll
    for (int c = 0; c < NMQ_K; c++)
        sc[c] = s0[c] + s1[c];
    const int y = Y0 + b * ST;
    if constexpr (!SUMS) {
        /* the window sums from the integral images */
#pragma unroll
        for (int c = 0; c < NMQ_K; c++) {
            const int x = X0 + (a0 + c) * ST;
            if (x <= p.x1 && y <= p.y1)
                sc[c] = ncc_score(sc[c], box(S1, tp, x, y, p.tw, p.th), box(S2, tp, x, y, p.tw, p.th), p) + 0.0f;
        }
    } else {
        /* the window sums, eight corner rows at a time, in the template's place */
        __syncthreads();
        const int ncols = nmq_sum_cols(ST, p.tw);
        long long *cs1 = reinterpret_cast<long long *>(sm), *cs2 = cs1 + 8 * ncols;
        long long r1 = 0, r2 = 0; /* thread t < ncols: column t's sums over the current corner row's window rows */
        if (t < ncols) {
            if (w32)
                nmq_col_first<true>(s_img, ip, p.th, t, r1, r2);
            else
                nmq_col_first<false>(s_img, ip, p.th, t, r1, r2);
        }
#pragma unroll 1
        for (int q = 0; q < NMQ_CORNERS / 8; q++) {
            if (t < ncols)
                for (int k = 0; k < 8; k++) {
                    const int rb = 8 * q + k;
                    if (rb > 0)
#pragma unroll
                        for (int u = 0; u < ST; u++) {
                            if (w32)
                                nmq_col_slide<true>(s_img, ip, p.th, t, (rb - 1) * ST + u, r1, r2);
                            else
                                nmq_col_slide<false>(s_img, ip, p.th, t, (rb - 1) * ST + u, r1, r2);
                        }
                    cs1[k * ncols + t] = r1;
                    cs2[k * ncols + t] = r2;
                }
            __syncthreads();
            if (b / 8 == q) {
                const long long *c1 = cs1 + (b % 8) * ncols + a0 * ST, *c2 = cs2 + (b % 8) * ncols + a0 * ST;
                long long x1 = 0, x2 = 0, y1 = 0, y2 = 0; /* two chains; tw is even */
                for (int j = 0; j < p.tw; j += 2) {
                    x1 += c1[j];
                    x2 += c2[j];
                    y1 += c1[j + 1];
                    y2 += c2[j + 1];
                }
                x1 += y1;
                x2 += y2;
                sc[0] = ncc_score(sc[0], x1, x2, p) + 0.0f;
#pragma unroll
                for (int c = 1; c < NMQ_K; c++) {
#pragma unroll
                    for (int u = 0; u < ST; u++) {
                        x1 += c1[(c - 1) * ST + p.tw + u] - c1[(c - 1) * ST + u];
                        x2 += c2[(c - 1) * ST + p.tw + u] - c2[(c - 1) * ST + u];
                    }
                    sc[c] = ncc_score(sc[c], x1, x2, p) + 0.0f;
                }
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int c = 0; c < NMQ_K; c++) {
        const int a = a0 + c, x = X0 + a * ST;
        const int ccx = ccx0 + a / PER, ccy = ccy0 + b / PER;
        if (x > p.x1 || y > p.y1 || ccx >= p.ccols || ccy >= p.crows)
            continue;
        const float v = sc[c];
        const int key = (b % PER) * PER + a % PER;
        unsigned u = __float_as_uint(v);
        u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
        atomicMax(&s_best[(b / PER) * BC + a / PER], ((unsigned long long)u << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)key));
    }
    __syncthreads();
    if (t < BC * BC) {
        const int ccx = ccx0 + t % BC, ccy = ccy0 + t / BC;
        if (ccx < p.ccols && ccy < p.crows) {
            const int cell = ccy * p.ccols + ccx;
            const int cx0 = p.x0 + ccx * NCC_CELL, cy0 = p.y0 + ccy * NCC_CELL;
            const unsigned long long wd = s_best[t];
            if (wd == 0ull) { /* no corner: the reference leaves top at -2 and the cell origin */
                map_v[cell] = -2.0f;
                map_x[cell] = cx0;
                map_y[cell] = cy0;
            } else {
                unsigned u = (unsigned)(wd >> 32);
                u = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
                const float bv = __uint_as_float(u);
                const int bk = (int)(0xFFFFFFFFu - (unsigned)(wd & 0xFFFFFFFFull));
                /* a cell whose every corner reads -1 (out of bounds) keeps -2 and its origin, as `v > top` never fires */
                const bool fired = bv > -2.0f;
                map_v[cell] = fired ? bv : -2.0f;
                map_x[cell] = fired ? cx0 + (bk % PER) * ST : cx0;
                map_y[cell] = fired ? cy0 + (bk / PER) * ST : cy0;
            }
        }
    }
}

template <typename T, int ST, bool SUMS>
static cudaError_t launch_map_f32q(const T *plane, int pitch, const float *app, const NccPrm &p, const NccScratch &s,
                                   cudaStream_t st)
{
    constexpr int BC = NMQ_CORNERS * ST / NCC_CELL;
    const int head = SUMS ? nmq_head(ST, p.tw, p.th) : p.tw * p.th;
    const size_t smem = sizeof(float) * ((size_t)head + (size_t)nmq_pitch(ST, p.tw) * nmq_rows(ST, p.th));
    cudaError_t e = cudaFuncSetAttribute(ncc_map_f32q<T, ST, SUMS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    const int bcols = (p.ccols + BC - 1) / BC, brows = (p.crows + BC - 1) / BC;
    ncc_map_f32q<T, ST, SUMS><<<bcols * brows, NMQ_CORNERS * NMQ_CORNERS / NMQ_K, smem, st>>>(
        plane, pitch, app, p, s.S1, s.S2, s.tp, bcols, s.map_v, s.map_x, s.map_y);
    return cudaGetLastError();
}

/* Where the F32 map at steps 1 and 2 takes its window sums. In the map kernel they cost a serial phase after the
 * products, which other CTAs' products hide while enough CTAs share an SM: up to 64 x 64 templates (measured at 1080p:
 * as fast or faster at every size up to there, 2-6 % slower at 96 x 96 and 128 x 128, where shared memory leaves one
 * or two CTAs an SM). The integral images cost two passes over the whole plane, whatever the window, so a window under
 * half the plane takes the in-kernel sums at any template size. */
static bool ncc_sums_in_map(const NccPrm &p)
{
    const long long win = (long long)(p.x1 - p.x0 + 1) * (long long)(p.y1 - p.y0 + 1);
    return p.tw * p.th <= 64 * 64 || 2 * win < (long long)p.w * (long long)p.h;
}

/* ---- the eight best cells ---- */

/* The eight best cells. Each CTA takes NCC_TOPB_PER x NCC_TOPB_THREADS cells (a thread keeps its best eight in
 * registers; the lists merge across each warp, then across the CTA's warps) and writes its eight to blk. The CTA that
 * arrives last merges every CTA's list into top / ntop and resets the counter, so the pass is one launch. WORDS: the
 * cells come as the tensor-core map's 64-bit words, which this pass also decodes into map_v / map_x / map_y. */
template <bool WORDS>
__global__ void __launch_bounds__(NCC_TOPB_THREADS) ncc_top_ctas(NccPrm p, const unsigned long long *__restrict__ cellw,
                                                                 float *__restrict__ map_v, int *__restrict__ map_x,
                                                                 int *__restrict__ map_y, int cells,
                                                                 unsigned long long *__restrict__ blk,
                                                                 unsigned *__restrict__ arrive, int *__restrict__ top,
                                                                 int *__restrict__ ntop)
{
    __shared__ unsigned long long s[NCC_TOPB_THREADS / 32][NCC_TOP];
    __shared__ bool s_last;
    vtg_grid_launch_dependents(); /* the half-pixel pass may start its CTAs and wait */
    vtg_grid_dependency_wait();   /* the map's cells, when launched as its programmatic dependent */
    unsigned long long t[NCC_TOP];
#pragma unroll
    for (int k = 0; k < NCC_TOP; k++)
        t[k] = 0ull;
    float v[NCC_TOPB_PER];
    const int i0 = blockIdx.x * NCC_TOPB_THREADS * NCC_TOPB_PER + threadIdx.x;
#pragma unroll
    for (int u = 0; u < NCC_TOPB_PER; u++) {
        const int i = i0 + u * NCC_TOPB_THREADS;
        if (WORDS) {
            const unsigned long long w = i < cells ? __ldca(cellw + i) : 0ull;
            if (i < cells) {
                int x, y;
                ncc_cell_decode(p, i, w, v[u], x, y);
                map_v[i] = v[u];
                map_x[i] = x;
                map_y[i] = y;
            } else {
                v[u] = -3.0f;
            }
        } else {
            v[u] = i < cells ? __ldca(map_v + i) : -3.0f;
        }
    }
#pragma unroll
    for (int u = 0; u < NCC_TOPB_PER; u++)
        top_insert(t, top_key(v[u], i0 + u * NCC_TOPB_THREADS));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    top_warp_merge(t);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < NCC_TOP; k++)
            s[warp][k] = t[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NCC_TOP; k++)
            t[k] = lane < NCC_TOPB_THREADS / 32 ? s[lane][k] : 0ull;
        top_warp_merge(t);
        /* every lane holds the list: lane 0 publishes it, then counts it */
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < NCC_TOP; k++)
                blk[(size_t)blockIdx.x * NCC_TOP + k] = t[k];
            __threadfence();
            s_last = atomicAdd(arrive, 1u) == gridDim.x - 1;
        }
    }
    __syncthreads();
    if (!s_last || warp != 0)
        return;
    __threadfence();
    ncc_top_final(blk, gridDim.x, arrive, top, ntop);
}

cudaError_t vtg_launch_ncc_top(const NccPrm &p, const NccScratch &s, bool words, cudaStream_t st, bool pdl)
{
    const int cells = p.ccols * p.crows;
    if (ncc_top_ctas(cells) > s.topblk_lists) /* each CTA leaves its best eight */
        return cudaErrorInvalidValue;
    const unsigned long long *w = words ? s.cellw : nullptr;
    return words ? vtg_launch_k(ncc_top_ctas<true>, dim3(ncc_top_ctas(cells)), dim3(NCC_TOPB_THREADS), 0, st, pdl, p, w,
                                s.map_v, s.map_x, s.map_y, cells, s.topblk, s.arrive, s.top, s.ntop)
                 : vtg_launch_k(ncc_top_ctas<false>, dim3(ncc_top_ctas(cells)), dim3(NCC_TOPB_THREADS), 0, st, pdl, p, w,
                                s.map_v, s.map_x, s.map_y, cells, s.topblk, s.arrive, s.top, s.ntop);
}

/* ---- half-pixel refinement (search_half, search_slot's second half, take_back's parabola) ---- */

/* A corner's score in half pixels (search_half), by a whole CTA of 256 threads: its 8 warps take template rows i = warp, warp + 8, .., its lanes the
 * columns, so one corner's latency is a few rows, not the whole template. The quarter-pixel sums are exact integers:
 * 32-bit a thread for byte planes (at most 64 terms of at most 1,020^2 each, for a 128 x 128 template), 64-bit for F32
 * planes and for every sum across threads. The F32 product sum is added in a fixed order (each thread's rows, the
 * warp's butterfly, then warps 0 .. 7), so a corner's score is the same every run. The result is thread 0's. */
template <typename T>
__device__ float half_score_cta(const T *__restrict__ plane, int pitch, const float *__restrict__ app, const NccPrm &p,
                                int hx, int hy)
{
    using Q = typename std::conditional<sizeof(T) == 1, int, long long>::type;
    __shared__ float s_st[8];
    __shared__ long long s_q1[8], s_q2[8];
    const int x = hx >> 1, y = hy >> 1, ox = hx & 1, oy = hy & 1;
    if (x < 1 || y < 1 || x + p.tw + 1 >= p.w - 1 || y + p.th + 1 >= p.h - 1)
        return -1.0f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float first = (float)__ldg(plane + (size_t)y * pitch + x);
    float st = 0.0f;
    Q a1 = 0, a2 = 0; /* in quarters */
    /* the columns of a row as four unrolled, predicated steps (T_w <= 128) and two rows at a time, so a thread's loads
     * are in flight together; the order of its sums is still rows, then columns, ascending */
#pragma unroll 2
    for (int i = warp; i < p.th; i += 8) {
        const T *r0 = plane + (size_t)(y + i) * pitch + x, *r1 = r0 + pitch;
        const float *ar = app + (size_t)i * p.tw;
#pragma unroll
        for (int u = 0; u < VTG_NCC_MAX_T / 32; u++) {
            const int j = lane + 32 * u;
            if (j >= p.tw)
                break;
            const Q a = (Q)__ldg(r0 + j), b = ox ? (Q)__ldg(r0 + j + 1) : a;
            Q q = 2 * (a + b);
            if (oy) {
                const Q c = (Q)__ldg(r1 + j), d = ox ? (Q)__ldg(r1 + j + 1) : c;
                q = (q + 2 * (c + d)) / 2;
            }
            a1 += q;
            a2 += q * q;
            st = __fmaf_rn((float)q * 0.25f - first, __ldg(ar + j), st);
        }
    }
    long long q1 = a1, q2 = a2;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        st += __shfl_xor_sync(VTG_FULL, st, s);
        q1 += __shfl_xor_sync(VTG_FULL, q1, s);
        q2 += __shfl_xor_sync(VTG_FULL, q2, s);
    }
    if (lane == 0) {
        s_st[warp] = st;
        s_q1[warp] = q1;
        s_q2[warp] = q2;
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return 0.0f;
    st = 0.0f;
    q1 = q2 = 0;
    for (int k = 0; k < 8; k++) {
        st += s_st[k];
        q1 += s_q1[k];
        q2 += s_q2[k];
    }
    const long long nvar16 = (long long)p.n * q2 - q1 * q1; /* 16 n var, exact */
    if (nvar16 <= p.nthr16 || p.norm <= 0.0f)
        return 0.0f;
    const float var = (float)nvar16 / (16.0f * (float)p.n);
    return st / sqrtf(p.norm * var);
}

__device__ __forceinline__ float parabola(float l, float c, float r)
{
    const float den = l - 2.0f * c + r;
    if (den >= 0.0f)
        return 0.0f;
    const float o = 0.5f * (l - r) / den;
    return fminf(fmaxf(o, -0.5f), 0.5f);
}

/* The best of each candidate's window (row-major first maximum, as search_slot's strict > over hy then hx: the
 * smallest index among equal scores), one warp a candidate; then, on one thread, the best over candidates in rank
 * order, the second peak half a template away, and the parabola through the four neighbours of the best (take_back's
 * peak_offset), all from hs (read through L2: other CTAs wrote it). Run by a CTA of NCC_TOP warps. */
__device__ void ncc_pick(const NccPrm &p, const int *__restrict__ map_x, const int *__restrict__ map_y,
                         const int *__restrict__ top, int n, const float *__restrict__ hs, vtg_found *__restrict__ out)
{
    __shared__ float s_score[NCC_TOP];
    __shared__ int s_hx[NCC_TOP], s_hy[NCC_TOP], s_at[NCC_TOP];
    const int around = p.step > 1 ? 2 * p.step - 1 : 1, side = 2 * around + 1, ring = side + 2;
    const int c = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (c < n) {
        const float *h = hs + (size_t)c * ring * ring;
        float best = -2.0f;
        int bo = side * side; /* scan index of the best; side^2: none */
        for (int o = lane; o < side * side; o += 32) {
            const float v = __ldcg(h + (o / side + 1) * ring + o % side + 1);
            if (v > best) {
                best = v;
                bo = o;
            }
        }
#pragma unroll
        for (int sh = 16; sh >= 1; sh >>= 1) {
            const float ov = __shfl_xor_sync(VTG_FULL, best, sh);
            const int oo = __shfl_xor_sync(VTG_FULL, bo, sh);
            if (ov > best || (ov == best && oo < bo)) {
                best = ov;
                bo = oo;
            }
        }
        if (lane == 0) {
            const int cell = __ldca(top + c);
            if (bo == side * side)
                bo = (side * side) / 2; /* no score above -2: the centre */
            s_score[c] = best;
            s_hx[c] = 2 * __ldca(map_x + cell) + bo % side - around;
            s_hy[c] = 2 * __ldca(map_y + cell) + bo / side - around;
            s_at[c] = (bo / side + 1) * ring + bo % side + 1;
        }
    }
    __syncthreads();
    if (threadIdx.x != 0)
        return;
    float ncc = -2.0f;
    int win = -1, hx = 0, hy = 0;
    for (int k = 0; k < n; k++)
        if (s_score[k] > ncc) {
            ncc = s_score[k];
            win = k;
            hx = s_hx[k];
            hy = s_hy[k];
        }
    float second = -2.0f;
    for (int k = 0; k < n; k++) {
        const int dx = s_hx[k] - hx, dy = s_hy[k] - hy;
        if ((dx * dx > p.tw * p.tw || dy * dy > p.th * p.th) && s_score[k] > second)
            second = s_score[k];
    }
    vtg_found f;
    f.hx = hx;
    f.hy = hy;
    f.ncc = ncc;
    f.second = second;
    f.ox = f.oy = 0.0f;
    if (win >= 0) {
        const float *h = hs + (size_t)win * ring * ring;
        const int k = s_at[win];
        f.ox = parabola(__ldcg(h + k - 1), ncc, __ldcg(h + k + 1));
        f.oy = parabola(__ldcg(h + k - ring), ncc, __ldcg(h + k + ring));
    }
    f.ntop = n;
    f.cells = p.ccols * p.crows;
    *out = f;
}

/* The half-pixel corners around every candidate, one CTA each: the window of +-around half pixels that
 * search_slot compares, and one ring past it, so the parabola's neighbours of any best are already scored. Scores go
 * to hs[candidate][(around + 1 + dy) ring + around + 1 + dx], ring = 2 around + 3. The CTA that arrives last (every
 * CTA counts, those past the candidates too) makes the pick and resets the counter. */
template <typename T>
__global__ void __launch_bounds__(NCC_TOP * 32) ncc_half_all(const T *__restrict__ plane, int pitch,
                                                             const float *__restrict__ app, NccPrm p,
                                                             const int *__restrict__ map_x, const int *__restrict__ map_y,
                                                             const int *__restrict__ top, const int *__restrict__ ntop,
                                                             float *__restrict__ hs, unsigned *__restrict__ arrive,
                                                             vtg_found *__restrict__ out)
{
    __shared__ bool s_last;
    vtg_grid_dependency_wait(); /* the candidates, when launched as the top-8 pass's programmatic dependent */
    const int around = p.step > 1 ? 2 * p.step - 1 : 1, ring = 2 * around + 3, r = around + 1;
    const int c = blockIdx.x / (ring * ring), o = blockIdx.x - c * ring * ring;
    /* what the top-8 pass wrote, by coherent loads: it was not read-only while this kernel ran */
    const int n = __ldca(ntop);
    if (c < n) {
        const int cell = __ldca(top + c);
        const int hx = 2 * __ldca(map_x + cell) + (o % ring) - r, hy = 2 * __ldca(map_y + cell) + (o / ring) - r;
        const float v = half_score_cta(plane, pitch, app, p, hx, hy);
        if (threadIdx.x == 0)
            hs[c * ring * ring + o] = v;
    }
    if (threadIdx.x == 0) {
        /* publish the score before counting it */
        __threadfence();
        s_last = atomicAdd(arrive, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    ncc_pick(p, map_x, map_y, top, n, hs, out);
    if (threadIdx.x == 0)
        *arrive = 0u;
}

/* ---- corners one by one (tk_correlate): one warp per corner ---- */

template <typename T>
__global__ void ncc_corners(const T *__restrict__ plane, int pitch, const float *__restrict__ app, NccPrm p, int count,
                            const int *__restrict__ xs, const int *__restrict__ ys, float *__restrict__ out)
{
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (i >= count)
        return;
    /* a whole-pixel corner is the half-pixel corner (2x, 2y) with the bounds of search_at */
    const int x = xs[i], y = ys[i];
    float v;
    if (x < 1 || y < 1 || x + p.tw >= p.w - 1 || y + p.th >= p.h - 1) {
        v = -1.0f;
    } else {
        const float first = (float)__ldg(plane + (size_t)y * pitch + x);
        float st = 0.0f;
        long long q1 = 0, q2 = 0;
        for (int k = lane; k < p.tw * p.th; k += 32) {
            const int r = k / p.tw, j = k - r * p.tw;
            const long long q = (long long)__ldg(plane + (size_t)(y + r) * pitch + x + j);
            q1 += q;
            q2 += q * q;
            st = __fmaf_rn((float)q - first, app[k], st);
        }
#pragma unroll
        for (int s = 16; s >= 1; s >>= 1) {
            st += __shfl_xor_sync(VTG_FULL, st, s);
            q1 += __shfl_xor_sync(VTG_FULL, q1, s);
            q2 += __shfl_xor_sync(VTG_FULL, q2, s);
        }
        v = ncc_score(st, q1, q2, p);
    }
    if (lane == 0)
        out[i] = v;
}

/* ---- launchers ---- */

template <typename T>
static cudaError_t launch_all(const T *plane, int pitch, const float *app, const NccPrm &p, const NccScratch &s,
                              int map_kind, vtg_found *out, cudaStream_t st)
{
    const int cells = p.ccols * p.crows;
    cudaError_t e = cudaSuccess;
    if (map_kind == VTG_NCC_F32) {
        /* steps 1 and 2: four corners a thread, the window sums from the staged window; the other steps one corner a
         * thread, a CTA a cell, the window sums from the integral images (the tensor-core map's prep sums the bytes) */
        const bool quad = p.step == 1 || p.step == 2;
        const bool sums = quad && ncc_sums_in_map(p);
        if (!sums) {
            integral_rows<T><<<(p.h + 1 + 7) / 8, 256, 0, st>>>(plane, pitch, p.w, p.h, s.S1, s.S2, s.tp);
            integral_cols<<<(p.w + 1 + IC_COLS - 1) / IC_COLS, IC_COLS * IC_SEGS, 0, st>>>(p.w, p.h, s.S1, s.S2, s.tp);
        }
        const size_t smem = sizeof(float) * ((size_t)p.tw * p.th + (size_t)(NCC_CELL + p.tw) * (NCC_CELL + p.th));
        if (!quad && (e = cudaFuncSetAttribute(ncc_map_f32<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
                         cudaSuccess)
            return e;
        if (s.map_ev0 && (e = cudaEventRecord(s.map_ev0, st)) != cudaSuccess)
            return e;
        if (quad)
            e = p.step == 1 ? (sums ? launch_map_f32q<T, 1, true>(plane, pitch, app, p, s, st)
                                    : launch_map_f32q<T, 1, false>(plane, pitch, app, p, s, st))
                            : (sums ? launch_map_f32q<T, 2, true>(plane, pitch, app, p, s, st)
                                    : launch_map_f32q<T, 2, false>(plane, pitch, app, p, s, st));
        else
            ncc_map_f32<T><<<cells, 256, smem, st>>>(plane, pitch, app, p, s.S1, s.S2, s.tp, s.map_v, s.map_x, s.map_y);
        if (e != cudaSuccess)
            return e;
        if (s.map_ev1 && (e = cudaEventRecord(s.map_ev1, st)) != cudaSuccess)
            return e;
    } else {
        e = vtg_launch_ncc_map_tc(plane, pitch, sizeof(T), p, s, map_kind, st);
        if (e != cudaSuccess)
            return e;
    }
    /* the tensor-core map's launcher ends with the top-8 pass over its cell words (ncc_tc.cu); the passes after the
     * map start as programmatic dependents, except when events around the map time it alone */
    const bool pdl = !s.map_ev1;
    if (map_kind == VTG_NCC_F32 && (e = vtg_launch_ncc_top(p, s, false, st, pdl)) != cudaSuccess)
        return e;
    const int around = p.step > 1 ? 2 * p.step - 1 : 1, ring = 2 * around + 3;
    return vtg_launch_k(ncc_half_all<T>, dim3(NCC_TOP * ring * ring), dim3(NCC_TOP * 32), 0, st, pdl, plane, pitch, app, p,
                        (const int *)s.map_x, (const int *)s.map_y, (const int *)s.top, (const int *)s.ntop, s.half,
                        s.arrive + 1, out);
}

cudaError_t vtg_launch_ncc(const void *plane, int pitch, int plane_type, const float *app, const NccPrm &p,
                           const NccScratch &s, int map_kind, vtg_found *out, cudaStream_t st)
{
    if (plane_type == VTG_PLANE_U8)
        return launch_all((const uint8_t *)plane, pitch, app, p, s, map_kind, out, st);
    return launch_all((const float *)plane, pitch, app, p, s, map_kind, out, st);
}

cudaError_t vtg_launch_ncc_corners(const void *plane, int pitch, int plane_type, const float *app, const NccPrm &p,
                                   int count, const int *xs, const int *ys, float *out, cudaStream_t st)
{
    const int blocks = (count + 7) / 8;
    if (count <= 0)
        return cudaSuccess;
    if (plane_type == VTG_PLANE_U8)
        ncc_corners<uint8_t><<<blocks, 256, 0, st>>>((const uint8_t *)plane, pitch, app, p, count, xs, ys, out);
    else
        ncc_corners<float><<<blocks, 256, 0, st>>>((const float *)plane, pitch, app, p, count, xs, ys, out);
    return cudaGetLastError();
}
