/* detect.cu -- corners inside a rectangle of a Q6 plane: the Harris response over Sobel gradients on a 5 x 5 box of
 * the structure tensor, each 16 x 16 cell's strongest response, and the selection of the strongest corners at a
 * spacing.
 *
 * Reference: detect_begin, detect_tensor, detect_response, detect_cells and detect_finish (src/kern/detect.h:21-37,
 * src/kern/detect.c:28-258), run in that order by the tracker's seed_at (src/kern/track.c:988-992).
 *
 * The response is the reference's bit for bit: every step is an IEEE F32 operation in the reference's order (the
 * Sobel sums of whole numbers, a fused multiply-add, the 1/512 scale, three rounded products, the five rows added top
 * to bottom, the box as (v + (v_-1 + v_+1)) + (v_-2 + v_+2) with the columns outside the region's 16-column groups
 * reading 0, and det - 0.04 trace^2 as two fused multiply-subtracts). No sqrt or division, so no arithmetic differs.
 *
 * Pipeline, one stream, no host round trip:
 *   det_response  a CTA a tile of 16 rows x 64 columns: the plane tile, the tensor, the row sums and the box in
 *                 shared memory; the response out, and the four cells' strongest (floored at 0)
 *   det_near      each cell's 3 x 3 neighbourhood strongest, a thread a cell, and the best cell
 *   det_count     a warp an eighth of a row: the local maxima above max(quality x neighbourhood, 2500), counted
 *   det_scan      the segments' counts scanned: each segment's first place in scan order
 *   det_collect   a warp a segment: the candidates in scan order, the first 8,192 kept (DETECT_MAX_CANDIDATES), each
 *                 scored v / local + 0.001 v / best in FP64 and rounded to F32 (the reference's long double rounds to
 *                 the same F32 but where the sum lies within 2^-53 of a rounding boundary)
 *   det_select    one CTA: the candidates sorted by (score descending, scan order) -- a stable radix sort of the 32-bit
 *                 score keys in shared memory, four 8-bit passes -- their places gathered, then the greedy spacing
 *                 in blocks of 1,024 candidates, a thread each, settled in parallel passes with the in-order result,
 *                 up to max corners. The corners taken and the block's candidates sit in grids of linked lists (cells
 *                 at least the spacing wide), so a candidate looks at its 3 x 3 grid cells only.
 * The threshold needs no long double: local x quality is an exact product of two F32s, so its F32 rounding is the
 * reference's (float)(rel) and max(fl(rel), 2500) equals its (float)(rel > 2500 ? rel : 2500). */
#include <math.h>
#include <stdint.h>

#include <new>

#include "vtg_ctx.h"
#include "vtg_internal.cuh"

#define DET_MAX_CAND 8192   /* DETECT_MAX_CANDIDATES, src/kern/detect.h:12 */
#define DET_TX 64           /* a response tile: four cells wide ... */
#define DET_TY 16           /* ... and one cell row high */
#define DET_SELECT_THREADS 1024
#define DET_SEGS 8          /* a row's candidate columns in this many segments, a warp each */
#define DET_GRID_MAX 16384  /* the taken corners' grid: at most this many cells (their list heads fill the keys' space) */
#define DET_RADIX 256       /* the sort's digit: 8 bits, four passes over the 32-bit score key */
#define DET_HIST_PITCH 257  /* a warp's digit counts: one word of padding against bank conflicts */
static_assert(DET_SELECT_THREADS / 32 * 256 == DET_MAX_CAND, "the sort: a warp 256 candidates, 8 a lane");
static_assert(DET_GRID_MAX <= 2 * DET_MAX_CAND, "grid heads in the spare keys' and places' space");
static_assert(DET_SELECT_THREADS * 2 <= DET_MAX_CAND, "a block's places in the keys' space");
static_assert(DET_GRID_MAX <= 2 * DET_HIST_PITCH * 32, "block grid heads in the counts' space");

struct DetGeo {
    int x0, y0, x1, y1, ax, cols, rows, nv, cell_rows;
};

struct DetPrm {
    const float *p; /* the plane, w x h, rows pitch floats apart */
    int w, h, pitch;
    DetGeo g;
    float quality;
    int need; /* ceil(min_dist^2): the spacing test on whole-pixel places */
    int max;
    int gs, gw, gh; /* the grid of corners taken: cells gs pixels square (gs^2 >= need), gw x gh of them */
};

struct vtg_detector {
    vtg_ctx *ctx;
    cudaStream_t stream;
    char *mem;
    size_t bytes;
    int max_w, max_h, max_cols, max_cells;
    float *resp, *cell, *near, *best;
    int *rowcount, *rowbase, *ncand;
    unsigned *keys;
    int2 *cxy;
    float *xs, *ys;
    int *count;
};

/* ---- the response and the cells ---- */

__global__ void __launch_bounds__(256) det_response(DetPrm q, float *__restrict__ resp, float *__restrict__ cell,
                                                    float *__restrict__ best)
{
    __shared__ float s_p[DET_TY + 6][DET_TX + 6];   /* image rows y0 - 3 + r0 + i, columns ax + c0 - 3 + j */
    __shared__ float s_t[3][DET_TY + 4][DET_TX + 4]; /* tensor rows r0 + i, region columns c0 - 2 + j */
    __shared__ float s_v[3][DET_TY][DET_TX + 4];     /* the five-row sums */
    __shared__ float s_m[8][4];                      /* each warp's strongest in the tile's four cells */
    const DetGeo &g = q.g;
    const int tid = threadIdx.x;
    const int r0 = blockIdx.y * DET_TY, c0 = blockIdx.x * DET_TX;
    if (tid == 0 && blockIdx.x == 0 && blockIdx.y == 0)
        *best = 0.0f; /* det_near's maximum starts here */
    for (int i = tid; i < (DET_TY + 6) * (DET_TX + 6); i += blockDim.x) {
        const int a = i / (DET_TX + 6), b = i - a * (DET_TX + 6);
        const int y = min(max(g.y0 - 3 + r0 + a, 0), q.h - 1), x = min(max(g.ax + c0 - 3 + b, 0), q.w - 1);
        s_p[a][b] = __ldg(q.p + (size_t)y * q.pitch + x);
    }
    __syncthreads();
    /* the tensor at region row r0 + a (image row y0 - 2 + r0 + a: staged row a + 1) and region column c0 - 2 + b
     * (staged column b + 1); 0 outside the region's columns, as the box's zero vectors read */
    for (int i = tid; i < (DET_TY + 4) * (DET_TX + 4); i += blockDim.x) {
        const int a = i / (DET_TX + 4), b = i - a * (DET_TX + 4);
        const int c = c0 - 2 + b;
        float xx = 0.0f, xy = 0.0f, yy = 0.0f;
        if (c >= 0 && c < g.cols) {
            const float *U = &s_p[a][b], *M = &s_p[a + 1][b], *D = &s_p[a + 2][b];
            const float dxu = U[2] - U[0], dxm = M[2] - M[0], dxd = D[2] - D[0];
            const float gx = __fmaf_rn(dxm, 2.0f, dxu + dxd) * (1.0f / 512.0f);
            const float dyl = D[0] - U[0], dyc = D[1] - U[1], dyr = D[2] - U[2];
            const float gy = __fmaf_rn(dyc, 2.0f, dyl + dyr) * (1.0f / 512.0f);
            xx = gx * gx;
            xy = gx * gy;
            yy = gy * gy;
        }
        s_t[0][a][b] = xx;
        s_t[1][a][b] = xy;
        s_t[2][a][b] = yy;
    }
    __syncthreads();
    for (int i = tid; i < 3 * DET_TY * (DET_TX + 4); i += blockDim.x) {
        const int t = i / (DET_TY * (DET_TX + 4)), rem = i - t * DET_TY * (DET_TX + 4);
        const int a = rem / (DET_TX + 4), b = rem - a * (DET_TX + 4);
        s_v[t][a][b] = (((s_t[t][a][b] + s_t[t][a + 1][b]) + s_t[t][a + 2][b]) + s_t[t][a + 3][b]) + s_t[t][a + 4][b];
    }
    __syncthreads();
    /* four outputs a thread: row a = tid / 16, columns j .. j + 3, all in cell j / 16 */
    const int a = tid >> 4, j = 4 * (tid & 15);
    const int r = r0 + a;
    float m = 0.0f;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int b = j + e + 2; /* s_v column of region column c0 + j + e */
        const float *A = &s_v[0][a][b], *B = &s_v[1][a][b], *C = &s_v[2][a][b];
        const float va = (A[0] + (A[-1] + A[1])) + (A[-2] + A[2]);
        const float vb = (B[0] + (B[-1] + B[1])) + (B[-2] + B[2]);
        const float vc = (C[0] + (C[-1] + C[1])) + (C[-2] + C[2]);
        const float tr = va + vc;
        const float v = __fmaf_rn(-0.04f, tr * tr, __fmaf_rn(-vb, vb, va * vc));
        const int c = c0 + j + e;
        if (r < g.rows && c < g.cols) {
            resp[(size_t)r * g.cols + c] = v;
            m = fmaxf(m, v);
        }
    }
    /* the lanes of a cell: 4 a half-warp row, the two rows of the warp */
    m = fmaxf(m, __shfl_xor_sync(VTG_FULL, m, 1));
    m = fmaxf(m, __shfl_xor_sync(VTG_FULL, m, 2));
    m = fmaxf(m, __shfl_xor_sync(VTG_FULL, m, 16));
    const int lane = tid & 31, warp = tid >> 5;
    if (lane < 16 && (lane & 3) == 0)
        s_m[warp][lane >> 2] = m;
    __syncthreads();
    if (tid < 4) {
        float c = 0.0f;
        for (int w = 0; w < 8; w++)
            c = fmaxf(c, s_m[w][tid]);
        const int k = 4 * blockIdx.x + tid;
        if (k < g.nv)
            cell[blockIdx.y * g.nv + k] = c;
    }
}

/* ---- the selection ---- */

/* Each cell's 3 x 3 neighbourhood strongest, a thread a cell, and the best cell over the CTAs: an integer atomicMax
 * on the F32 bits orders them as the floats, all being >= 0 (det_response zeroes the best first). */
__global__ void __launch_bounds__(256) det_near(DetGeo g, const float *__restrict__ cell, float *__restrict__ near,
                                                float *__restrict__ best)
{
    __shared__ float s_w[8];
    const int n = g.nv * g.cell_rows, i = (int)(blockIdx.x * blockDim.x + threadIdx.x), tid = threadIdx.x;
    float m = 0.0f;
    if (i < n) {
        const int cr = i / g.nv, k = i - cr * g.nv;
        for (int a = cr > 0 ? cr - 1 : 0; a <= cr + 1 && a < g.cell_rows; a++)
            for (int b = k > 0 ? k - 1 : 0; b <= k + 1 && b < g.nv; b++)
                m = fmaxf(m, cell[a * g.nv + b]);
        near[i] = m;
    }
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1)
        m = fmaxf(m, __shfl_xor_sync(VTG_FULL, m, s));
    if ((tid & 31) == 0)
        s_w[tid >> 5] = m;
    __syncthreads();
    if (tid == 0) {
        float b = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++)
            b = fmaxf(b, s_w[w]);
        if (b > 0.0f)
            atomicMax(reinterpret_cast<int *>(best), __float_as_int(b));
    }
}

/* A corner candidate: inside the rectangle's lanes, above its threshold, and no smaller than any of its 8 neighbours
 * (those past the region's columns read 0). */
__device__ __forceinline__ bool det_candidate(const DetPrm &q, const float *__restrict__ resp,
                                              const float *__restrict__ near, int r, int c)
{
    const DetGeo &g = q.g;
    const float *me = resp + (size_t)r * g.cols;
    const float v = me[c];
    const float thresh = fmaxf(near[(r >> 4) * g.nv + (c >> 4)] * q.quality, 2500.0f);
    if (!(thresh < v))
        return false;
    const float *up = me - g.cols, *dn = me + g.cols;
    const bool lo = c > 0, hi = c + 1 < g.cols;
    return (lo ? up[c - 1] : 0.0f) <= v && up[c] <= v && (hi ? up[c + 1] : 0.0f) <= v && (lo ? me[c - 1] : 0.0f) <= v &&
           (hi ? me[c + 1] : 0.0f) <= v && (lo ? dn[c - 1] : 0.0f) <= v && dn[c] <= v && (hi ? dn[c + 1] : 0.0f) <= v;
}

__device__ __forceinline__ void det_lanes(const DetGeo &g, int &lo, int &hi)
{
    lo = g.x0 - g.ax > 1 ? g.x0 - g.ax : 1;
    hi = g.x1 - g.ax < g.cols - 1 ? g.x1 - g.ax : g.cols - 1;
}

/* Segment s of a row's candidate columns [lo, hi): [a, b), consecutive segments in column order. */
__device__ __forceinline__ void det_segment(const DetGeo &g, int s, int &a, int &b)
{
    int lo, hi;
    det_lanes(g, lo, hi);
    const int len = hi > lo ? hi - lo : 0, per = (len + DET_SEGS - 1) / DET_SEGS;
    a = lo + s * per;
    b = min(a + per, lo + len);
}

__global__ void __launch_bounds__(256) det_count(DetPrm q, const float *__restrict__ resp,
                                                 const float *__restrict__ near, const float *__restrict__ best,
                                                 int *__restrict__ rowcount)
{
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    const int r = w / DET_SEGS, sg = w - r * DET_SEGS;
    if (r >= q.g.rows)
        return;
    int cnt = 0;
    if (*best > 0.0f && r >= 1 && r < q.g.rows - 1) {
        int a, b;
        det_segment(q.g, sg, a, b);
        for (int c0 = a; c0 < b; c0 += 32) {
            const int c = c0 + lane;
            cnt += __popc(__ballot_sync(VTG_FULL, c < b && det_candidate(q, resp, near, r, c)));
        }
    }
    if (lane == 0)
        rowcount[w] = cnt;
}

/* Each row's first place in scan order (exclusive scan over rows), and the candidates kept: at most 8,192. */
__global__ void __launch_bounds__(1024) det_scan(int rows, const int *__restrict__ rowcount, int *__restrict__ rowbase,
                                                 int *__restrict__ ncand)
{
    __shared__ int s[1024];
    const int tid = threadIdx.x, per = (rows + 1023) / 1024, a = tid * per, b = min(a + per, rows);
    int sum = 0;
    for (int r = a; r < b; r++)
        sum += rowcount[r];
    s[tid] = sum;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        const int v = tid >= d ? s[tid - d] : 0;
        __syncthreads();
        s[tid] += v;
        __syncthreads();
    }
    int run = s[tid] - sum;
    for (int r = a; r < b; r++) {
        rowbase[r] = run;
        run += rowcount[r];
    }
    if (tid == 1023)
        *ncand = min(s[1023], DET_MAX_CAND);
}

__global__ void __launch_bounds__(256) det_collect(DetPrm q, const float *__restrict__ resp,
                                                   const float *__restrict__ near, const float *__restrict__ best,
                                                   const int *__restrict__ rowbase, unsigned *__restrict__ keys,
                                                   int2 *__restrict__ cxy)
{
    const int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    const int r = w / DET_SEGS, sg = w - r * DET_SEGS;
    if (r < 1 || r >= q.g.rows - 1 || !(*best > 0.0f))
        return;
    int pos = rowbase[w];
    if (pos >= DET_MAX_CAND)
        return;
    const double bst = (double)*best;
    int a, b;
    det_segment(q.g, sg, a, b);
    for (int c0 = a; c0 < b && pos < DET_MAX_CAND; c0 += 32) {
        const int c = c0 + lane;
        const bool f = c < b && det_candidate(q, resp, near, r, c);
        const unsigned m = __ballot_sync(VTG_FULL, f);
        const int p = pos + __popc(m & ((1u << lane) - 1u));
        if (f && p < DET_MAX_CAND) {
            const double v = (double)resp[(size_t)r * q.g.cols + c];
            const double local = (double)near[(r >> 4) * q.g.nv + (c >> 4)];
            const float score = (float)(v / local + 0.001 * v / bst);
            keys[p] = ~__float_as_uint(score); /* ascending: the best first; the place is the index */
            cxy[p] = make_int2(q.g.ax + c, q.g.y0 + r);
        }
        pos += __popc(m);
    }
}

/* Whether the corner at (x, y) keeps the spacing from every corner in the grid: the 3 x 3 grid cells around its own
 * (a cell's side is at least the spacing, so no corner farther out can be too close). */
__device__ __forceinline__ bool det_far(const DetPrm &q, const int *s_head, const int *s_next, const int *s_tx,
                                        const int *s_ty, int x, int y)
{
    const int gx = (x - q.g.ax) / q.gs, gy = (y - q.g.y0) / q.gs;
    int h[9];
#pragma unroll
    for (int j = 0; j < 9; j++) {
        const int a = gx + j % 3 - 1, b = gy + j / 3 - 1;
        h[j] = a >= 0 && a < q.gw && b >= 0 && b < q.gh ? s_head[b * q.gw + a] : -1;
    }
#pragma unroll
    for (int j = 0; j < 9; j++)
        for (int t = h[j]; t >= 0; t = s_next[t]) {
            const int dx = s_tx[t] - x, dy = s_ty[t] - y;
            if (dx * dx + dy * dy < q.need)
                return false;
        }
    return true;
}

#define DET_OPEN 0
#define DET_TAKEN 1
#define DET_OUT 2

/* A block candidate's earlier neighbours within the spacing (the block grid's 3 x 3 cells around it): DET_OUT when
 * one of them is taken, DET_OPEN when none is but one is still open, else DET_TAKEN. The states are read while other
 * threads set theirs: a state once set never changes, so a stale read only defers the answer to the next pass. */
__device__ __forceinline__ int det_earlier(const DetPrm &q, const int *s_bhead, const int *s_bnext, const int2 *xy,
                                           const unsigned char *s_st, int me, int x, int y)
{
    const volatile unsigned char *st = s_st;
    const int gx = (x - q.g.ax) / q.gs, gy = (y - q.g.y0) / q.gs;
    bool pending = false;
    for (int j = 0; j < 9; j++) {
        const int a = gx + j % 3 - 1, b = gy + j / 3 - 1;
        if (a < 0 || a >= q.gw || b < 0 || b >= q.gh)
            continue;
        for (int u = s_bhead[b * q.gw + a]; u >= 0; u = s_bnext[u]) {
            if (u >= me)
                continue;
            const int dx = xy[u].x - x, dy = xy[u].y - y;
            if (dx * dx + dy * dy >= q.need)
                continue;
            const int su = st[u];
            if (su == DET_TAKEN)
                return DET_OUT;
            pending = pending || su == DET_OPEN;
        }
    }
    return pending ? DET_OPEN : DET_TAKEN;
}

/* One pass of the stable LSD radix sort over the candidates' score keys in shared memory: the 8-bit digit at shift,
 * from (ka, va) to (kb, vb). Warp w holds elements 256 w + 32 k + lane (k = 0..7), ranked in that order within the
 * warp (the lanes with the same digit found by eight ballots); the per-(digit, warp) counts, scanned in digit-major
 * order, place them. The counts sit at warp * DET_HIST_PITCH + digit: a warp's lanes and a scan step's lanes fall in
 * different banks. Two count buffers alternate: this pass counts in hist (zeroed by the pass before) and zeroes
 * next. Warps past the candidates (256 w >= n) count nothing. */
__device__ __forceinline__ void det_radix_pass(const unsigned *ka, const unsigned *va, unsigned *kb, unsigned *vb,
                                               int *hist, int *next, int *s_wsum, int n, int shift, bool first)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int i = tid; i < DET_HIST_PITCH * 32; i += blockDim.x)
        next[i] = 0;
    const bool active = 256 * warp < n;
    unsigned key[8], val[8];
    int rank[8];
    if (active) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const int i = 256 * warp + 32 * k + lane;
            key[k] = ka[i];
            val[k] = first ? (unsigned)i : va[i];
            const unsigned dig = (key[k] >> shift) & (DET_RADIX - 1);
            unsigned peers = VTG_FULL;
#pragma unroll
            for (int b = 0; b < 8; b++) {
                const unsigned m = __ballot_sync(VTG_FULL, (dig >> b) & 1u);
                peers &= ((dig >> b) & 1u) ? m : ~m;
            }
            const int lt = __popc(peers & ((1u << lane) - 1u));
            int *h = hist + warp * DET_HIST_PITCH + dig;
            const int base = *h;
            rank[k] = base + lt;
            __syncwarp();
            if (lt == 0)
                *h = base + __popc(peers);
            __syncwarp();
        }
    }
    __syncthreads();
    /* exclusive scan of the 8,192 counts: 8 a thread, across a warp, then across the warps (each warp scans the 32
     * warp totals itself) */
    int c[8], sum = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int e = 8 * tid + j; /* digit e / 32, warp e % 32 */
        c[j] = hist[(e & 31) * DET_HIST_PITCH + (e >> 5)];
        sum += c[j];
    }
    int inc = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(VTG_FULL, inc, d);
        if (lane >= d)
            inc += v;
    }
    if (lane == 31)
        s_wsum[warp] = inc;
    __syncthreads();
    const int t = s_wsum[lane];
    int ti = t;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(VTG_FULL, ti, d);
        if (lane >= d)
            ti += v;
    }
    int run = __shfl_sync(VTG_FULL, ti - t, warp) + inc - sum;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const int e = 8 * tid + j;
        hist[(e & 31) * DET_HIST_PITCH + (e >> 5)] = run;
        run += c[j];
    }
    __syncthreads();
    if (active) {
#pragma unroll
        for (int k = 0; k < 8; k++) {
            const unsigned dig = (key[k] >> shift) & (DET_RADIX - 1);
            const int dst = hist[warp * DET_HIST_PITCH + dig] + rank[k];
            kb[dst] = key[k];
            vb[dst] = val[k];
        }
    }
    __syncthreads();
}

__global__ void __launch_bounds__(DET_SELECT_THREADS, 1) det_select(DetPrm q, const int *__restrict__ ncand,
                                                                 const float *__restrict__ best,
                                                                 const unsigned *__restrict__ keys,
                                                                 const int2 *__restrict__ cxy,
                                                                 float *__restrict__ xs, float *__restrict__ ys,
                                                                 int *__restrict__ count)
{
    /* two buffers of keys and places (DET_MAX_CAND each), then two of radix counts. Once sorted (places in v0),
     * k1 and v1 hold the taken corners' grid heads, the counts the block grid's, and k0 a block's (x, y). */
    extern __shared__ unsigned s_buf[];
    __shared__ int s_tx[512], s_ty[512], s_next[512], s_wsum[32];
    __shared__ int s_bnext[DET_SELECT_THREADS];
    __shared__ unsigned char s_st[DET_SELECT_THREADS];
    unsigned *k0 = s_buf, *v0 = s_buf + DET_MAX_CAND, *k1 = s_buf + 2 * DET_MAX_CAND, *v1 = s_buf + 3 * DET_MAX_CAND;
    int *h0 = reinterpret_cast<int *>(s_buf + 4 * DET_MAX_CAND), *h1 = h0 + DET_HIST_PITCH * 32;
    int2 *s_xy = reinterpret_cast<int2 *>(k0);
    int *s_head = reinterpret_cast<int *>(k1);
    int *s_bhead = h0;
    const int tid = threadIdx.x;
    const int n = *best > 0.0f ? *ncand : 0;
    const int n256 = (n + 255) & ~255;
    for (int i = tid; i < n256; i += blockDim.x)
        k0[i] = i < n ? keys[i] : ~0u; /* past the candidates: after every score, and stable behind them */
    for (int i = tid; i < DET_HIST_PITCH * 32; i += blockDim.x)
        h0[i] = 0;
    __syncthreads();
    /* ascending ~score bits, ties in scan order: the order detect_finish's qsort gives (score descending, then order) */
    det_radix_pass(k0, v0, k1, v1, h0, h1, s_wsum, n, 0, true);
    det_radix_pass(k1, v1, k0, v0, h1, h0, s_wsum, n, 8, false);
    det_radix_pass(k0, v0, k1, v1, h0, h1, s_wsum, n, 16, false);
    det_radix_pass(k1, v1, k0, v0, h1, h0, s_wsum, n, 24, false);
    for (int i = tid; i < q.gw * q.gh; i += blockDim.x) {
        s_head[i] = -1;
        s_bhead[i] = -1;
    }
    __syncthreads();
    /* The greedy spacing in blocks of up to 1,024 candidates, a thread a candidate; the result is the one-by-one
     * order's. A candidate too close to a corner taken in an earlier block is out. Within the block the candidates
     * sit in a grid of their own, and each open one looks at its earlier neighbours within the spacing: out once one
     * of them is taken, taken once all of them are out. Every pass settles at least the earliest open one, so a block ends
     * within as many passes as it has candidates. The taken ones past max are dropped in order. */
    const int lane = tid & 31, warp = tid >> 5;
    int taken = 0;
    for (int base = 0, B = 0; base < n && taken < q.max; base += B) {
        /* twice the corners still wanted, 64 to 1,024: the greedy rarely looks further, and a shorter block settles
         * in fewer passes */
        B = min(n - base, min(DET_SELECT_THREADS, max(64, 2 * (q.max - taken))));
        int2 me = make_int2(0, 0);
        int cell = 0;
        if (tid < B) {
            me = cxy[v0[base + tid]]; /* the block's places, gathered as it starts */
            s_xy[tid] = me;
            cell = ((me.y - q.g.y0) / q.gs) * q.gw + (me.x - q.g.ax) / q.gs;
            s_st[tid] = det_far(q, s_head, s_next, s_tx, s_ty, me.x, me.y) ? DET_OPEN : DET_OUT;
            s_bnext[tid] = atomicExch(&s_bhead[cell], tid);
        }
        __syncthreads();
        bool open = tid < B && s_st[tid] == DET_OPEN;
        while (__syncthreads_or(open)) {
            if (open) {
                const int r = det_earlier(q, s_bhead, s_bnext, s_xy, s_st, tid, me.x, me.y);
                if (r != DET_OPEN) {
                    s_st[tid] = (unsigned char)r;
                    open = false;
                }
            }
        }
        /* the taken ones in order: their places in the list of corners */
        const bool yes = tid < B && s_st[tid] == DET_TAKEN;
        const unsigned bal = __ballot_sync(VTG_FULL, yes);
        if (lane == 0)
            s_wsum[warp] = __popc(bal);
        __syncthreads();
        const int wt = s_wsum[lane];
        int wi = wt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int v = __shfl_up_sync(VTG_FULL, wi, d);
            if (lane >= d)
                wi += v;
        }
        const int rank = __shfl_sync(VTG_FULL, wi - wt, warp) + __popc(bal & ((1u << lane) - 1u));
        const int total = __shfl_sync(VTG_FULL, wi, 31);
        if (yes && taken + rank < q.max) {
            const int at = taken + rank;
            s_tx[at] = me.x;
            s_ty[at] = me.y;
            xs[at] = (float)me.x;
            ys[at] = (float)me.y;
            s_next[at] = atomicExch(&s_head[cell], at);
        }
        taken = min(taken + total, q.max);
        __syncthreads();
        if (tid < B)
            s_bhead[cell] = -1;
        __syncthreads();
    }
    if (tid == 0)
        *count = taken;
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

/* detect_begin's layout (src/kern/detect.c:28-66); false when nothing of the rectangle lies inside the margin. */
static bool det_geometry(int w, int h, float rx, float ry, float rw, float rh, int margin, DetGeo &g)
{
    /* a region past any plane (or not a number) holds nothing; so does a negative margin's outside */
    const float lim = 1.0e8f;
    if (margin < 0 || !(fabsf(rx) < lim && fabsf(ry) < lim && fabsf(rw) < lim && fabsf(rh) < lim))
        return false;
    int x0 = (int)rx, y0 = (int)ry, x1 = (int)(rx + rw), y1 = (int)(ry + rh);
    x0 = x0 < margin ? margin : x0;
    y0 = y0 < margin ? margin : y0;
    x1 = x1 > w - margin ? w - margin : x1;
    y1 = y1 > h - margin ? h - margin : y1;
    if (x1 <= x0 || y1 <= y0)
        return false;
    g.x0 = x0;
    g.y0 = y0;
    g.x1 = x1;
    g.y1 = y1;
    g.ax = x0 & ~15;
    g.cols = (x1 - g.ax + 15) & ~15;
    g.rows = y1 - y0;
    g.nv = g.cols / 16;
    g.cell_rows = g.rows / 16 + 1;
    return true;
}

static size_t up256(size_t n) { return (n + 255) & ~(size_t)255; }

struct DetLayout {
    size_t resp, cell, near, best, rowcount, rowbase, ncand, keys, cxy, xs, ys, count, bytes;
};

static DetLayout det_layout(int max_w, int max_h, int &max_cols, int &max_cells)
{
    max_cols = ((max_w + 15) & ~15) + 16;
    max_cells = (max_h / 16 + 1) * (max_cols / 16);
    DetLayout L;
    size_t b = 0;
    L.resp = b;
    b += up256(sizeof(float) * (size_t)max_cols * max_h);
    L.cell = b;
    b += up256(sizeof(float) * (size_t)max_cells);
    L.near = b;
    b += up256(sizeof(float) * (size_t)max_cells);
    L.best = b;
    b += 256;
    L.rowcount = b;
    b += up256(sizeof(int) * (size_t)max_h * DET_SEGS);
    L.rowbase = b;
    b += up256(sizeof(int) * (size_t)max_h * DET_SEGS);
    L.ncand = b;
    b += 256;
    L.keys = b;
    b += up256(sizeof(unsigned) * DET_MAX_CAND);
    L.cxy = b;
    b += up256(sizeof(int2) * DET_MAX_CAND);
    L.xs = b;
    b += up256(sizeof(float) * 512);
    L.ys = b;
    b += up256(sizeof(float) * 512);
    L.count = b;
    b += 256;
    L.bytes = b;
    return L;
}

extern "C" size_t vtg_detector_bytes(int max_w, int max_h)
{
    if (max_w < 1 || max_h < 1 || max_w > 16384 || max_h > 16384)
        return 0;
    int mc, mcl;
    return det_layout(max_w, max_h, mc, mcl).bytes;
}

extern "C" int vtg_detector_create(vtg_ctx *ctx, int max_w, int max_h, vtg_detector **out)
{
    if (!ctx || !out || max_w < 1 || max_h < 1 || max_w > 16384 || max_h > 16384)
        return VTG_EINVAL;
    *out = nullptr;
    int max_cols, max_cells;
    const DetLayout L = det_layout(max_w, max_h, max_cols, max_cells);
    const int charged = vtg_ctx_charge(ctx, L.bytes);
    if (charged != VTG_OK)
        return charged;
    vtg_detector *d = new (std::nothrow) vtg_detector;
    if (!d) {
        vtg_ctx_release(ctx, L.bytes);
        return VTG_ENOMEM;
    }
    d->ctx = ctx;
    d->bytes = L.bytes;
    d->max_w = max_w;
    d->max_h = max_h;
    d->max_cols = max_cols;
    d->max_cells = max_cells;
    cudaError_t e = cudaSetDevice(vtg_ctx_device(ctx));
    if (e == cudaSuccess)
        e = cudaMalloc(&d->mem, L.bytes);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        vtg_ctx_release(ctx, L.bytes);
        delete d;
        return VTG_ENOMEM;
    }
    e = cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        cudaFree(d->mem);
        vtg_ctx_release(ctx, L.bytes);
        delete d;
        return VTG_ECUDA;
    }
    d->resp = (float *)(d->mem + L.resp);
    d->cell = (float *)(d->mem + L.cell);
    d->near = (float *)(d->mem + L.near);
    d->best = (float *)(d->mem + L.best);
    d->rowcount = (int *)(d->mem + L.rowcount);
    d->rowbase = (int *)(d->mem + L.rowbase);
    d->ncand = (int *)(d->mem + L.ncand);
    d->keys = (unsigned *)(d->mem + L.keys);
    d->cxy = (int2 *)(d->mem + L.cxy);
    d->xs = (float *)(d->mem + L.xs);
    d->ys = (float *)(d->mem + L.ys);
    d->count = (int *)(d->mem + L.count);
    vtg_ctx_track(ctx, d->stream, true);
    *out = d;
    return VTG_OK;
}

extern "C" void vtg_detector_destroy(vtg_detector *d)
{
    if (!d)
        return;
    cudaSetDevice(vtg_ctx_device(d->ctx));
    cudaStreamSynchronize(d->stream);
    vtg_ctx_track(d->ctx, d->stream, false);
    cudaStreamDestroy(d->stream);
    cudaFree(d->mem);
    vtg_ctx_release(d->ctx, d->bytes);
    delete d;
}

extern "C" void *vtg_detector_stream(const vtg_detector *d) { return d ? (void *)d->stream : nullptr; }

extern "C" int vtg_detect(vtg_detector *d, const float *plane, int w, int h, int pitch, float rx, float ry, float rw,
                          float rh, int margin, int max, float min_dist, float quality, float *xs, float *ys, int *count,
                          int where, void *stream)
{
    if (!d || !plane || w < 1 || h < 1 || pitch < w || max < 0 || max > 512 || !(min_dist >= 0.0f) ||
        !(quality >= 0.0f) || (max > 0 && (!xs || !ys)) || !count || (where != VTG_HOST && where != VTG_DEVICE) ||
        !(rx == rx && ry == ry && rw == rw && rh == rh))
        return VTG_EINVAL;
    const cudaStream_t st = stream ? (cudaStream_t)stream : d->stream;
    CU(cudaSetDevice(vtg_ctx_device(d->ctx)));
    DetPrm q;
    q.p = plane;
    q.w = w;
    q.h = h;
    q.pitch = pitch;
    q.quality = quality;
    q.max = max;
    /* exact: a product of two F32s; past 2^30 no two places in a 16384 x 16384 region are that far apart */
    const double min2 = (double)min_dist * (double)min_dist;
    q.need = min2 < (double)(1 << 30) ? (int)ceil(min2) : 1 << 30;
    const bool any = det_geometry(w, h, rx, ry, rw, rh, margin, q.g);
    if (any && (q.g.rows > d->max_h || q.g.cols > d->max_cols || q.g.nv * q.g.cell_rows > d->max_cells))
        return VTG_EINVAL;
    if (any) {
        /* the smallest side whose square reaches need, grown until the region's grid fits DET_GRID_MAX cells */
        long long gs = (long long)sqrt((double)q.need);
        while (gs * gs < q.need)
            gs++;
        gs = gs < 1 ? 1 : gs;
        while (((q.g.cols + gs - 1) / gs) * ((q.g.rows + gs - 1) / gs) > DET_GRID_MAX)
            gs++;
        q.gs = (int)gs;
        q.gw = (int)((q.g.cols + gs - 1) / gs);
        q.gh = (int)((q.g.rows + gs - 1) / gs);
    }
    if (!any || max == 0) {
        if (where == VTG_HOST) {
            *count = 0;
            return VTG_OK;
        }
        CU(cudaMemsetAsync(count, 0, sizeof(int), st));
        return VTG_OK;
    }
    const DetGeo &g = q.g;
    CU(cudaMemsetAsync(d->cell, 0, sizeof(float) * (size_t)g.nv * g.cell_rows, st));
    det_response<<<dim3((g.cols + DET_TX - 1) / DET_TX, (g.rows + DET_TY - 1) / DET_TY), 256, 0, st>>>(q, d->resp,
                                                                                                   d->cell, d->best);
    det_near<<<(g.nv * g.cell_rows + 255) / 256, 256, 0, st>>>(g, d->cell, d->near, d->best);
    const int rblocks = (g.rows * DET_SEGS * 32 + 255) / 256;
    det_count<<<rblocks, 256, 0, st>>>(q, d->resp, d->near, d->best, d->rowcount);
    det_scan<<<1, 1024, 0, st>>>(g.rows * DET_SEGS, d->rowcount, d->rowbase, d->ncand);
    det_collect<<<rblocks, 256, 0, st>>>(q, d->resp, d->near, d->best, d->rowbase, d->keys, d->cxy);
    const int smem = (int)(4 * sizeof(unsigned) * DET_MAX_CAND + 2 * sizeof(int) * DET_HIST_PITCH * 32);
    CU(cudaFuncSetAttribute(det_select, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    float *oxs = where == VTG_DEVICE ? xs : d->xs, *oys = where == VTG_DEVICE ? ys : d->ys;
    int *ocount = where == VTG_DEVICE ? count : d->count;
    det_select<<<1, DET_SELECT_THREADS, smem, st>>>(q, d->ncand, d->best, d->keys, d->cxy, oxs, oys, ocount);
    CU(cudaGetLastError());
    if (where == VTG_HOST) {
        CU(cudaMemcpyAsync(count, d->count, sizeof(int), cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(xs, d->xs, sizeof(float) * (size_t)max, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(ys, d->ys, sizeof(float) * (size_t)max, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
    }
    return VTG_OK;
}

/* The stages' planes, for checking: resp (rows x cols) and cells (cell_rows x nv) of the last vtg_detect, and its
 * layout (x0, y0, x1, y1, ax, cols, rows, nv, cell_rows). Waits for the detector's stream. */
extern "C" int vtg_detect_maps(vtg_detector *d, float rx, float ry, float rw, float rh, int w, int h, int margin,
                               int *geo, float *resp, float *cells)
{
    if (!d || !geo)
        return VTG_EINVAL;
    DetGeo g;
    if (!det_geometry(w, h, rx, ry, rw, rh, margin, g) || g.rows > d->max_h || g.cols > d->max_cols ||
        g.nv * g.cell_rows > d->max_cells)
        return VTG_EINVAL;
    const int v[9] = {g.x0, g.y0, g.x1, g.y1, g.ax, g.cols, g.rows, g.nv, g.cell_rows};
    for (int k = 0; k < 9; k++)
        geo[k] = v[k];
    CU(cudaSetDevice(vtg_ctx_device(d->ctx)));
    CU(cudaStreamSynchronize(d->stream));
    if (resp)
        CU(cudaMemcpy(resp, d->resp, sizeof(float) * (size_t)g.rows * g.cols, cudaMemcpyDeviceToHost));
    if (cells)
        CU(cudaMemcpy(cells, d->cell, sizeof(float) * (size_t)g.nv * g.cell_rows, cudaMemcpyDeviceToHost));
    return VTG_OK;
}
