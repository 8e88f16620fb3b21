/* framegen.cu -- a generated frame between two real ones on the GPU: the motion field of FidelityFX Optical Flow as
 * the reference restates it (block SAD search, filter, upscale over a pyramid), the vectors at the middle instant, and
 * the blended frame.
 *
 * Reference: src/kern/framegen.c (fg_hist_section, fg_scene_verdict, fg_search, fg_filter, fg_upscale,
 * fg_mid_vectors, fg_blend) and img_q6_to_u8_vx (src/kern/img_vx.c:36-47), run in the order of tk_generate_make
 * (src/kern/track.c:847-888).
 *
 * Every plane holds whole-number Q6 values, so every SAD is an exact F32 sum in any order and the fields are the
 * reference's bit for bit. The blend keeps the reference's six fused multiply-adds in their order (its sums pass 2^24)
 * and rounds to the nearest, ties to even. The reference reads replicated padding; here a read is a clamped index,
 * except the search window's origin, which the reference clamps into its padding (that moves the offsets searched)
 * and which is clamped here the same way.
 *
 * One call, on one stream:
 *   fg_reduce_kernel      the field's pyramid of both frames: level 0 is the frames' half size (x(levels))
 *   fg_hist_kernel        64-bin histograms of nine sections of both frames' level 1 (8 CTAs a section); the last
 *                         CTA's verdict
 *   fg_search_kernel      a warp an 8 x 8 block: the 24 x 24 window in shared memory, a lane 8 of the 256 offsets
 *   fg_filter_kernel      a thread a block: the 3 x 3's vector nearest the others
 *   fg_upscale_kernel     a thread a finer block: of four coarse vectors, the least 4 x 4 SAD, doubled
 *   fg_mid_kernel         a warp a block: the vectors at the middle instant
 *   fg_blend_kernel       a CTA a 16 x 16 tile of the full-size frame: the frame (Q6) and its bytes */
#include <math.h>
#include <stdint.h>

#include <new>

#include "vtg_ctx.h"
#include "vtg_internal.cuh"

#define FG_LEVELS 7 /* FG_MAX_LEVELS, src/kern/framegen.h:20 */
#define FG_WARPS 4  /* blocks a CTA in the search and the middle vectors */

/* one level of the field: both frames' planes there and its three fields */
struct FgLevel {
    const float *a, *b; /* older, newer */
    int w, h, pitch, bw, bh;
    short2 *raw, *fil, *up;
};

struct vtg_framegen {
    vtg_ctx *ctx;
    cudaStream_t stream;
    char *mem;
    size_t bytes;
    int w, h, levels, out_pitch;
    FgLevel L[FG_LEVELS];
    float *pa[FG_LEVELS], *pb[FG_LEVELS];
    short2 *mid;
    unsigned *hist; /* 2 x 9 x 64 */
    int *scene;     /* [0] the verdict, [1] the hist kernel's ticket */
    float *out;
    unsigned char *pic;
};

__device__ __forceinline__ float fg_at(const float *p, int pitch, int w, int h, int x, int y)
{
    return __ldg(p + (size_t)min(max(y, 0), h - 1) * pitch + min(max(x, 0), w - 1));
}

__device__ __forceinline__ float fg_warp_sum(float v)
{
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1)
        v += __shfl_xor_sync(VTG_FULL, v, d);
    return v;
}

/* One pyramid step of both frames (img_reduce, src/kern/img_ref.c:98-114): the 5 x 5 binomial, (sum + 128) >> 8,
 * clamped borders; blockIdx.z picks the frame. */
__global__ void fg_reduce_kernel(const float *__restrict__ sa, const float *__restrict__ sb, int sw, int sh,
                                 int spa, int spb, float *__restrict__ da, float *__restrict__ db, int dw, int dh,
                                 int dp)
{
    const int x = (int)(blockIdx.x * blockDim.x + threadIdx.x), y = (int)(blockIdx.y * blockDim.y + threadIdx.y);
    if (x >= dw || y >= dh)
        return;
    const float *s = blockIdx.z ? sb : sa;
    const int sp = blockIdx.z ? spb : spa;
    const int k[5] = {1, 4, 6, 4, 1};
    int sum = 0;
#pragma unroll
    for (int j = 0; j < 5; j++) {
        int row = 0;
#pragma unroll
        for (int i = 0; i < 5; i++)
            row += k[i] * (int)fg_at(s, sp, sw, sh, 2 * x + i - 2, 2 * y + j - 2);
        sum += k[j] * row;
    }
    (blockIdx.z ? db : da)[(size_t)y * dp + x] = (float)((sum + 128) >> 8);
}

/* fg_hist_section (framegen.c:85-101): section blockIdx.x % 9 of frame blockIdx.x / 9, its sampled rows split over
 * FG_HIST_SPLIT CTAs (blockIdx.y), added into the global counts; the last CTA compares the frames (fg_scene_verdict,
 * framegen.c:103-113: more than half the samples in other bins, i.e. sum |a - b| > sum b) and zeroes the counts for
 * the next call. */
#define FG_HIST_SPLIT 8
__global__ void __launch_bounds__(256) fg_hist_kernel(FgLevel lv, unsigned *__restrict__ hist, int *scene)
{
    __shared__ unsigned s_h[64];
    __shared__ bool s_last;
    const int tid = threadIdx.x, s = blockIdx.x % 9, f = blockIdx.x / 9;
    if (tid < 64)
        s_h[tid] = 0;
    __syncthreads();
    const float *p = f ? lv.b : lv.a;
    const int sx = s % 3, sy = s / 3;
    const int x0 = (lv.w * sx / 3) & ~15, x1 = (lv.w * (sx + 1) / 3) & ~15;
    const int y0 = lv.h * sy / 3, y1 = lv.h * (sy + 1) / 3;
    const int cols = x1 - x0, rows = (y1 - y0 + 1) / 2;
    for (int k = (int)blockIdx.y * blockDim.x + tid; k < cols * rows; k += FG_HIST_SPLIT * blockDim.x) {
        const int y = y0 + 2 * (k / cols), x = x0 + k % cols;
        atomicAdd(&s_h[(int)(p[(size_t)y * lv.pitch + x] * (1.0f / 256.0f)) & 63], 1u);
    }
    __syncthreads();
    if (tid < 64 && s_h[tid])
        atomicAdd(&hist[(f * 9 + s) * 64 + tid], s_h[tid]);
    __threadfence();
    __syncthreads();
    if (tid == 0)
        s_last = atomicAdd(&scene[1], 1) == (int)(gridDim.x * gridDim.y) - 1;
    __syncthreads();
    if (!s_last || tid >= 32)
        return;
    __threadfence();
    unsigned long long diff = 0, total = 0;
    for (int i = tid; i < 9 * 64; i += 32) {
        const unsigned a = __ldcg(&hist[i]), b = __ldcg(&hist[9 * 64 + i]);
        diff += a > b ? a - b : b - a;
        total += b;
        hist[i] = 0;
        hist[9 * 64 + i] = 0;
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        diff += __shfl_xor_sync(VTG_FULL, diff, d);
        total += __shfl_xor_sync(VTG_FULL, total, d);
    }
    if (tid == 0) {
        scene[0] = total && diff > total;
        scene[1] = 0;
    }
}

/* fg_search (framegen.c:117-214) at one level: a warp an 8 x 8 block. pred: the coarser level's estimate (NULL at the
 * top). The 256 offsets x0 - px + dx, wy + dy - 8 (dx, dy < 16) cost |dx - 8| + |dy - 8| plus the block's SAD; the
 * first lowest in row order wins. On the finest level a block the estimate explains (SAD <= 8192) is not searched, and
 * no motion wins when its SAD is no more than the best cost. */
__global__ void __launch_bounds__(32 * FG_WARPS) fg_search_kernel(FgLevel lv, const short2 *__restrict__ pred,
                                                                  int level, const int *__restrict__ scene)
{
    __shared__ float s_win[FG_WARPS][24][25];
    __shared__ float s_blk[FG_WARPS][8][8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (int)blockIdx.x * FG_WARPS + warp;
    if (i >= lv.bw * lv.bh)
        return;
    if (*scene) {
        if (lane == 0)
            lv.raw[i] = make_short2(0, 0);
        return;
    }
    const int px = (i % lv.bw) * 8, py = (i / lv.bw) * 8;
    const short2 want = pred ? pred[i] : make_short2(0, 0);
    const int wx = want.x, wy = want.y;
    const int lanes = (lv.w + 15) & ~15;
    const int x0 = min(max(px + wx - 8, -32), lanes), y0 = py + wy - 8;
    {
        /* every load of the window and the block in flight before the first store */
        float wv[18], bv[2];
#pragma unroll
        for (int j = 0; j < 18; j++) {
            const int k = lane + 32 * j;
            wv[j] = fg_at(lv.a, lv.pitch, lv.w, lv.h, x0 + k % 24, y0 + k / 24);
        }
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int k = lane + 32 * j;
            bv[j] = fg_at(lv.b, lv.pitch, lv.w, lv.h, px + (k & 7), py + (k >> 3));
        }
#pragma unroll
        for (int j = 0; j < 18; j++) {
            const int k = lane + 32 * j;
            s_win[warp][k / 24][k % 24] = wv[j];
        }
#pragma unroll
        for (int j = 0; j < 2; j++) {
            const int k = lane + 32 * j;
            s_blk[warp][k >> 3][k & 7] = bv[j];
        }
    }
    __syncwarp();
    if (level == 0) {
        /* the estimate's place is the window's centre: (x0 + 8, y0 + 8) */
        float s = 0.0f;
        for (int k = lane; k < 64; k += 32)
            s += fabsf(s_blk[warp][k >> 3][k & 7] - s_win[warp][8 + (k >> 3)][8 + (k & 7)]);
        s = fg_warp_sum(s);
        if (s <= 8192.0f) { /* FG_ENOUGH */
            if (lane == 0)
                lv.raw[i] = make_short2((short)(x0 - px + 8), (short)wy);
            return;
        }
    }
    const int dy = lane >> 1, dx0 = (lane & 1) * 8;
    float c[8];
#pragma unroll
    for (int k = 0; k < 8; k++)
        c[k] = (float)abs(dx0 + k - 8) + (float)abs(dy - 8); /* FG_TIE_UNIT */
#pragma unroll
    for (int r = 0; r < 8; r++) {
        float wv[15], bv[8];
#pragma unroll
        for (int k = 0; k < 15; k++)
            wv[k] = s_win[warp][dy + r][dx0 + k];
#pragma unroll
        for (int n = 0; n < 8; n++)
            bv[n] = s_blk[warp][r][n];
#pragma unroll
        for (int k = 0; k < 8; k++)
#pragma unroll
            for (int n = 0; n < 8; n++)
                c[k] += fabsf(wv[k + n] - bv[n]);
    }
    float best = c[0];
    int bi = dy * 16 + dx0;
#pragma unroll
    for (int k = 1; k < 8; k++)
        if (c[k] < best) {
            best = c[k];
            bi = dy * 16 + dx0 + k;
        }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) {
        const float ob = __shfl_xor_sync(VTG_FULL, best, d);
        const int oi = __shfl_xor_sync(VTG_FULL, bi, d);
        if (ob < best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    int vx = x0 - px + (bi & 15), vy = wy + (bi >> 4) - 8;
    if (level == 0) {
        float s = 0.0f;
        for (int k = lane; k < 64; k += 32)
            s += fabsf(s_blk[warp][k >> 3][k & 7] - fg_at(lv.a, lv.pitch, lv.w, lv.h, px + (k & 7), py + (k >> 3)));
        s = fg_warp_sum(s);
        if (s <= best)
            vx = vy = 0;
    }
    if (lane == 0)
        lv.raw[i] = make_short2((short)vx, (short)vy);
}

/* fg_filter (framegen.c:218-247): of the 3 x 3 around a block (clamped, column by column), the vector with the least
 * sum of squared differences from the nine; the first on a tie. */
__global__ void fg_filter_kernel(FgLevel lv)
{
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= lv.bw * lv.bh)
        return;
    const int bx = i % lv.bw, by = i / lv.bw;
    int mx[9], my[9];
#pragma unroll
    for (int xx = 0; xx < 3; xx++)
#pragma unroll
        for (int yy = 0; yy < 3; yy++) {
            const short2 v = lv.raw[min(max(by + yy - 1, 0), lv.bh - 1) * lv.bw + min(max(bx + xx - 1, 0), lv.bw - 1)];
            mx[xx * 3 + yy] = v.x;
            my[xx * 3 + yy] = v.y;
        }
    int pick = 0;
    unsigned least = 0;
#pragma unroll
    for (int a = 0; a < 9; a++) {
        unsigned d = 0;
#pragma unroll
        for (int b = 0; b < 9; b++) {
            const int dx = mx[a] - mx[b], dy = my[a] - my[b];
            d += (unsigned)(dx * dx + dy * dy);
        }
        if (a == 0 || d < least) {
            least = d;
            pick = a;
        }
    }
    lv.fil[i] = make_short2((short)mx[pick], (short)my[pick]);
}

/* fg_upscale (framegen.c:251-288): block (gx, gy) of the finer level (fine.bw x fine.bh) takes, of the four nearest
 * blocks of this level, the vector with the least SAD over the 4 x 4 of this level it covers (the first on a tie),
 * doubled. */
__global__ void fg_upscale_kernel(FgLevel lv, short2 *__restrict__ up, int fbw, int fbh, const int *__restrict__ scene)
{
    const int i = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= fbw * fbh)
        return;
    if (*scene) {
        up[i] = make_short2(0, 0);
        return;
    }
    const int gx = i % fbw, gy = i / fbw;
    /* the four candidates' SADs with all their loads in flight, then the first least */
    short2 v[4];
    float sad[4];
#pragma unroll
    for (int n = 0; n < 4; n++) {
        const int xo = n % 2 - 1 + gx % 2, yo = n / 2 - 1 + gy % 2;
        v[n] = lv.fil[min(max(gy / 2 + yo, 0), lv.bh - 1) * lv.bw + min(max(gx / 2 + xo, 0), lv.bw - 1)];
    }
    float cur[16];
#pragma unroll
    for (int k = 0; k < 16; k++)
        cur[k] = fg_at(lv.b, lv.pitch, lv.w, lv.h, gx * 4 + (k & 3), gy * 4 + (k >> 2));
#pragma unroll
    for (int n = 0; n < 4; n++) {
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < 16; k++)
            s += fabsf(cur[k] - fg_at(lv.a, lv.pitch, lv.w, lv.h, gx * 4 + (k & 3) + v[n].x, gy * 4 + (k >> 2) + v[n].y));
        sad[n] = s;
    }
    int pick = 0;
#pragma unroll
    for (int n = 1; n < 4; n++)
        if (sad[n] < sad[pick])
            pick = n;
    up[i] = make_short2((short)(2 * v[pick].x), (short)(2 * v[pick].y));
}

/* fg_mid_vectors (framegen.c:292-328) on the finest level: no motion first, favoured by one grey level over the block
 * (FG_MID_FAVOUR_ZERO), then each vector of the 3 x 3 (row by row) that agrees better when each frame moves half way.
 * A warp a block, a lane two of its pixels. */
__global__ void __launch_bounds__(32 * FG_WARPS) fg_mid_kernel(FgLevel lv, short2 *__restrict__ mid)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (int)blockIdx.x * FG_WARPS + warp;
    if (i >= lv.bw * lv.bh)
        return;
    const int bx = i % lv.bw, by = i / lv.bw, px = bx * 8, py = by * 8;
    auto sad = [&](int vx, int vy) {
        const int ax = vx >> 1, ay = vy >> 1, qx = vx - ax, qy = vy - ay;
        float s = 0.0f;
        for (int k = lane; k < 64; k += 32) {
            const int r = k >> 3, c = k & 7;
            s += fabsf(fg_at(lv.a, lv.pitch, lv.w, lv.h, px + c + ax, py + r + ay) -
                       fg_at(lv.b, lv.pitch, lv.w, lv.h, px + c - qx, py + r - qy));
        }
        return fg_warp_sum(s);
    };
    float best = sad(0, 0) - 64.0f;
    int vx = 0, vy = 0;
    for (int yy = 0; yy < 3; yy++)
        for (int xx = 0; xx < 3; xx++) {
            const short2 v = lv.fil[min(max(by + yy - 1, 0), lv.bh - 1) * lv.bw + min(max(bx + xx - 1, 0), lv.bw - 1)];
            if ((v.x == vx && v.y == vy) || (v.x == 0 && v.y == 0))
                continue;
            const float s = sad(v.x, v.y);
            if (s < best) {
                best = s;
                vx = v.x;
                vy = v.y;
            }
        }
    if (lane == 0)
        mid[i] = make_short2((short)vx, (short)vy);
}

/* fg_blend (framegen.c:332-357) and img_q6_to_u8_vx: a CTA a 16 x 16 tile, a thread a pixel. */
__global__ void __launch_bounds__(256) fg_blend_kernel(const float *__restrict__ a0, int pa, const float *__restrict__ b0,
                                                       int pb, int w, int h, const short2 *__restrict__ mid, int bw,
                                                       int bh, float *__restrict__ out, int po,
                                                       unsigned char *__restrict__ pic)
{
    __shared__ short2 s_near[3][3];
    __shared__ int s_same;
    const int tid = threadIdx.x, tx = blockIdx.x, ty = blockIdx.y;
    if (tid < 9)
        s_near[tid / 3][tid % 3] = mid[min(max(ty + tid / 3 - 1, 0), bh - 1) * bw + min(max(tx + tid % 3 - 1, 0), bw - 1)];
    __syncthreads();
    if (tid == 0) {
        int same = 1;
        for (int k = 0; k < 9; k++)
            same &= s_near[k / 3][k % 3].x == s_near[0][0].x && s_near[k / 3][k % 3].y == s_near[0][0].y;
        s_same = same;
    }
    __syncthreads();
    const int k = tid & 15, s = tid >> 4, x = tx * 16 + k, y = ty * 16 + s;
    if (x >= w || y >= h)
        return;
    float v;
    if (s_same) {
        const int vx = s_near[0][0].x, vy = s_near[0][0].y;
        v = rintf((fg_at(a0, pa, w, h, x + vx, y + vy) + fg_at(b0, pb, w, h, x - vx, y - vy)) * 0.5f);
    } else {
        /* in 32nds: across, the left, own and right blocks; down, the own row and the one above or below */
        const float wl = k < 8 ? (float)(15 - 2 * k) : 0.0f, wr = k < 8 ? 0.0f : (float)(2 * k - 15);
        const float ws = k < 8 ? (float)(17 + 2 * k) : (float)(47 - 2 * k);
        const float wh[3] = {wl, ws, wr};
        const int other = s < 8 ? 0 : 2, wo = s < 8 ? 15 - 2 * s : 2 * s - 15;
        const float vw[2] = {(float)(32 - wo), (float)wo};
        const int rows[2] = {1, other};
        float acc = 0.0f;
#pragma unroll
        for (int a = 0; a < 2; a++)
#pragma unroll
            for (int b = 0; b < 3; b++) {
                const short2 q = s_near[rows[a]][b];
                const float sum = fg_at(a0, pa, w, h, x + q.x, y + q.y) + fg_at(b0, pb, w, h, x - q.x, y - q.y);
                acc = __fmaf_rn(sum, wh[b] * vw[a], acc);
            }
        v = rintf(acc * (1.0f / 2048.0f));
    }
    out[(size_t)y * po + x] = v;
    if (pic) {
        const float q = rintf(v * (1.0f / 64.0f));
        pic[(size_t)y * w + x] = q <= 0.0f ? 0 : q >= 255.0f ? 255 : (unsigned char)q;
    }
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

static bool fg_size_ok(int w, int h) { return w >= 64 && h >= 64 && w <= 8192 && h <= 8192; }

/* The field's levels (src/kern/track.c:547-556): the frames' half size, then halves, while both sides are >= 16. */
static int fg_shapes(int w, int h, int lw[FG_LEVELS], int lh[FG_LEVELS])
{
    int n = 0, x = (w + 1) / 2, y = (h + 1) / 2;
    while (n < FG_LEVELS && x >= 16 && y >= 16) {
        lw[n] = x;
        lh[n] = y;
        n++;
        x = (x + 1) / 2;
        y = (y + 1) / 2;
    }
    return n;
}

static size_t fg_layout(int w, int h, size_t off_plane_a[FG_LEVELS], size_t off_plane_b[FG_LEVELS],
                        size_t off_f[FG_LEVELS][3], size_t *off_mid, size_t *off_hist, size_t *off_scene,
                        size_t *off_out, size_t *off_pic)
{
    int lw[FG_LEVELS], lh[FG_LEVELS];
    const int n = fg_shapes(w, h, lw, lh);
    size_t b = 0;
    for (int L = 0; L < n; L++) {
        const size_t plane = up256(sizeof(float) * (size_t)vtg_pitch(lw[L]) * (size_t)lh[L]);
        const size_t field = up256(sizeof(short2) * (size_t)((lw[L] + 7) / 8) * (size_t)((lh[L] + 7) / 8));
        off_plane_a[L] = b;
        b += plane;
        off_plane_b[L] = b;
        b += plane;
        for (int k = 0; k < 3; k++) {
            off_f[L][k] = b;
            b += field;
        }
    }
    *off_mid = b;
    b += up256(sizeof(short2) * (size_t)((lw[0] + 7) / 8) * (size_t)((lh[0] + 7) / 8));
    *off_hist = b;
    b += up256(sizeof(unsigned) * 2 * 9 * 64);
    *off_scene = b;
    b += 256;
    *off_out = b;
    b += up256(sizeof(float) * (size_t)vtg_pitch(w) * (size_t)h);
    *off_pic = b;
    b += up256((size_t)w * (size_t)h);
    return b;
}

extern "C" size_t vtg_framegen_bytes(int w, int h)
{
    if (!fg_size_ok(w, h))
        return 0;
    size_t a[FG_LEVELS], b[FG_LEVELS], f[FG_LEVELS][3], m, hi, s, o, p;
    return fg_layout(w, h, a, b, f, &m, &hi, &s, &o, &p);
}

extern "C" int vtg_framegen_create(vtg_ctx *ctx, int w, int h, vtg_framegen **out)
{
    if (!ctx || !out || !fg_size_ok(w, h))
        return VTG_EINVAL;
    *out = nullptr;
    size_t oa[FG_LEVELS], ob[FG_LEVELS], of[FG_LEVELS][3], om, oh, os, oo, op;
    const size_t bytes = fg_layout(w, h, oa, ob, of, &om, &oh, &os, &oo, &op);
    const int charged = vtg_ctx_charge(ctx, bytes);
    if (charged != VTG_OK)
        return charged;
    vtg_framegen *g = new (std::nothrow) vtg_framegen;
    if (!g) {
        vtg_ctx_release(ctx, bytes);
        return VTG_ENOMEM;
    }
    g->ctx = ctx;
    g->bytes = bytes;
    g->w = w;
    g->h = h;
    g->out_pitch = vtg_pitch(w);
    int lw[FG_LEVELS], lh[FG_LEVELS];
    g->levels = fg_shapes(w, h, lw, lh);
    g->stream = nullptr;
    cudaError_t e = cudaSetDevice(vtg_ctx_device(ctx));
    if (e == cudaSuccess)
        e = cudaMalloc(&g->mem, bytes);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        vtg_ctx_release(ctx, bytes);
        delete g;
        return VTG_ENOMEM;
    }
    e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(g->mem, 0, bytes, g->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(g->stream);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        if (g->stream)
            cudaStreamDestroy(g->stream);
        cudaFree(g->mem);
        vtg_ctx_release(ctx, bytes);
        delete g;
        return VTG_ECUDA;
    }
    for (int L = 0; L < g->levels; L++) {
        FgLevel &v = g->L[L];
        g->pa[L] = (float *)(g->mem + oa[L]);
        g->pb[L] = (float *)(g->mem + ob[L]);
        v.a = g->pa[L];
        v.b = g->pb[L];
        v.w = lw[L];
        v.h = lh[L];
        v.pitch = vtg_pitch(lw[L]);
        v.bw = (lw[L] + 7) / 8;
        v.bh = (lh[L] + 7) / 8;
        v.raw = (short2 *)(g->mem + of[L][0]);
        v.fil = (short2 *)(g->mem + of[L][1]);
        v.up = (short2 *)(g->mem + of[L][2]);
    }
    g->mid = (short2 *)(g->mem + om);
    g->hist = (unsigned *)(g->mem + oh);
    g->scene = (int *)(g->mem + os);
    g->out = (float *)(g->mem + oo);
    g->pic = (unsigned char *)(g->mem + op);
    vtg_ctx_track(ctx, g->stream, true);
    *out = g;
    return VTG_OK;
}

extern "C" void vtg_framegen_destroy(vtg_framegen *g)
{
    if (!g)
        return;
    cudaSetDevice(vtg_ctx_device(g->ctx));
    cudaStreamSynchronize(g->stream);
    vtg_ctx_track(g->ctx, g->stream, false);
    cudaStreamDestroy(g->stream);
    cudaFree(g->mem);
    vtg_ctx_release(g->ctx, g->bytes);
    delete g;
}

extern "C" void *vtg_framegen_stream(const vtg_framegen *g) { return g ? (void *)g->stream : nullptr; }

extern "C" int vtg_framegen_levels(const vtg_framegen *g) { return g ? g->levels : 0; }

extern "C" int vtg_framegen_run(vtg_framegen *g, const float *older, int older_pitch, const float *newer,
                                int newer_pitch, float *out, int out_pitch, uint8_t *pic, int where, void *stream)
{
    if (!g || !older || !newer || older_pitch < g->w || newer_pitch < g->w || (out && out_pitch < g->w) ||
        (pic && where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    CU(cudaSetDevice(vtg_ctx_device(g->ctx)));
    /* the field's pyramid: level 0 from the frames, each next from the last */
    const float *sa = older, *sb = newer;
    int sw = g->w, sh = g->h, spa = older_pitch, spb = newer_pitch;
    for (int L = 0; L < g->levels; L++) {
        const FgLevel &v = g->L[L];
        fg_reduce_kernel<<<dim3((v.w + 31) / 32, (v.h + 7) / 8, 2), dim3(32, 8), 0, st>>>(
            sa, sb, sw, sh, spa, spb, g->pa[L], g->pb[L], v.w, v.h, v.pitch);
        sa = g->pa[L];
        sb = g->pb[L];
        sw = v.w;
        sh = v.h;
        spa = spb = v.pitch;
    }
    fg_hist_kernel<<<dim3(18, FG_HIST_SPLIT), 256, 0, st>>>(g->L[1], g->hist, g->scene);
    for (int L = g->levels - 1; L >= 0; L--) {
        const FgLevel &v = g->L[L];
        const int nb = v.bw * v.bh;
        fg_search_kernel<<<(nb + FG_WARPS - 1) / FG_WARPS, 32 * FG_WARPS, 0, st>>>(
            v, L == g->levels - 1 ? nullptr : v.up, L, g->scene);
        fg_filter_kernel<<<(nb + 255) / 256, 256, 0, st>>>(v);
        if (L > 0) {
            const FgLevel &f = g->L[L - 1];
            fg_upscale_kernel<<<(f.bw * f.bh + 255) / 256, 256, 0, st>>>(v, f.up, f.bw, f.bh, g->scene);
        }
    }
    const FgLevel &z = g->L[0];
    fg_mid_kernel<<<(z.bw * z.bh + FG_WARPS - 1) / FG_WARPS, 32 * FG_WARPS, 0, st>>>(z, g->mid);
    float *dst = out ? out : g->out;
    const int dp = out ? out_pitch : g->out_pitch;
    unsigned char *pd = pic ? (where == VTG_DEVICE ? (unsigned char *)pic : g->pic) : nullptr;
    fg_blend_kernel<<<dim3((g->w + 15) / 16, (g->h + 15) / 16), 256, 0, st>>>(older, older_pitch, newer, newer_pitch,
                                                                            g->w, g->h, g->mid, z.bw, z.bh, dst, dp,
                                                                            pd);
    CU(cudaGetLastError());
    if (pic && where == VTG_HOST) {
        CU(cudaMemcpyAsync(pic, g->pic, (size_t)g->w * (size_t)g->h, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
    }
    return VTG_OK;
}

extern "C" int vtg_framegen_fields(vtg_framegen *g, int level, struct vtg_fg_vec *raw, struct vtg_fg_vec *fil,
                                   struct vtg_fg_vec *up, struct vtg_fg_vec *mid, int *scene, int where, void *stream)
{
    if (!g || level < 0 || level >= g->levels || (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    const cudaMemcpyKind k = where == VTG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    CU(cudaSetDevice(vtg_ctx_device(g->ctx)));
    const FgLevel &v = g->L[level];
    const size_t n = sizeof(short2) * (size_t)v.bw * (size_t)v.bh;
    if (raw)
        CU(cudaMemcpyAsync(raw, v.raw, n, k, st));
    if (fil)
        CU(cudaMemcpyAsync(fil, v.fil, n, k, st));
    if (up)
        CU(cudaMemcpyAsync(up, v.up, n, k, st));
    if (mid)
        CU(cudaMemcpyAsync(mid, g->mid, sizeof(short2) * (size_t)g->L[0].bw * (size_t)g->L[0].bh, k, st));
    if (scene)
        CU(cudaMemcpyAsync(scene, g->scene, sizeof(int), k, st));
    if (where == VTG_HOST)
        CU(cudaStreamSynchronize(st));
    return VTG_OK;
}

extern "C" int vtg_framegen_frame(const vtg_framegen *g, const float **plane, int *pitch)
{
    if (!g || !plane || !pitch)
        return VTG_EINVAL;
    *plane = g->out;
    *pitch = g->out_pitch;
    return VTG_OK;
}
