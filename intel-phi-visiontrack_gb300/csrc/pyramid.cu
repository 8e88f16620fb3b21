/* pyramid.cu -- the Gaussian pyramid of an 8-bit frame, bit-exact to the reference's Q6 planes.
 *
 * Reference: tk_build (src/kern/track.c:584-629) runs img_u8_to_q6 (src/kern/img_ref.c:32-40, img_vx.c:24-34) and
 * img_pad_rows / img_pad_tb (img_ref.c:9-30) for level 0, then img_reduce (img_ref.c:98-114, img_vx.c:129-162) per
 * level: the 5 x 5 binomial (1 4 6 4 1)^2 at every second pixel of every second row, rounded as (sum + 128) >> 8,
 * reading a replicated border. Every value is a whole number below 2^24, so the reference's F32 sums are exact; here
 * they are int32 sums, the border is a clamped index, and the results are the same bits.
 *
 * One launch per level: the first reads the bytes once from HBM and writes level 0 (byte x 64) and level 1 from the
 * same shared-memory tile; each further launch reduces the level below it (L2-resident at these sizes). A CTA of 256
 * threads makes a 64 x 16 tile of its output level from a 132 x 36 source tile staged in shared memory: the vertical
 * pass runs over the staged rows, the horizontal pass over the vertical sums, as the reference's vert5 / shift8 do. */
#include "vtg_internal.cuh"

#define RT_X 64 /* output tile */
#define RT_Y 16
#define RS_X (2 * RT_X + 4) /* source tile: two output pixels per step, two each side */
#define RS_Y (2 * RT_Y + 4)

/* One 64 x 16 tile of the output level at (ox, oy), from a 132 x 36 source tile in shared memory; with FROM_U8 the
 * source is the frame's bytes and level 0 (byte x 64) is written from the same tile. dst may be NULL (level 0 only). */
template <bool FROM_U8>
__device__ __forceinline__ void reduce_tile(const void *__restrict__ src_, int sw, int sh, int spitch,
                                            float *__restrict__ l0, int l0pitch, float *__restrict__ dst, int dw, int dh,
                                            int dpitch, int ox, int oy, int (*s_src)[RS_X + 1], int (*s_v)[RS_X + 1])
{
    const int tid = threadIdx.x;
    const int sx0 = 2 * ox - 2, sy0 = 2 * oy - 2;
    for (int i = tid; i < RS_Y * RS_X; i += blockDim.x) {
        const int r = i / RS_X, c = i - r * RS_X;
        const int sy = min(max(sy0 + r, 0), sh - 1), sx = min(max(sx0 + c, 0), sw - 1);
        int v;
        if (FROM_U8)
            v = 64 * (int)__ldg((const uint8_t *)src_ + (size_t)sy * spitch + sx);
        else
            v = (int)__ldg((const float *)src_ + (size_t)sy * spitch + sx);
        s_src[r][c] = v;
        /* Level 0 itself, from the same bytes: this tile's own 2 RT_X x 2 RT_Y pixels. */
        if (FROM_U8 && r >= 2 && r < RS_Y - 2 && c >= 2 && c < RS_X - 2 && sy0 + r < sh && sx0 + c < sw)
            l0[(size_t)(sy0 + r) * l0pitch + (sx0 + c)] = (float)v;
    }
    if (!dst)
        return;
    __syncthreads();
    for (int i = tid; i < RT_Y * RS_X; i += blockDim.x) {
        const int r = i / RS_X, c = i - r * RS_X;
        s_v[r][c] = s_src[2 * r][c] + s_src[2 * r + 4][c] + 4 * (s_src[2 * r + 1][c] + s_src[2 * r + 3][c]) + 6 * s_src[2 * r + 2][c];
    }
    __syncthreads();
    for (int i = tid; i < RT_Y * RT_X; i += blockDim.x) {
        const int r = i / RT_X, x = i - r * RT_X;
        const int c = 2 * x + 2;
        const int h = s_v[r][c - 2] + s_v[r][c + 2] + 4 * (s_v[r][c - 1] + s_v[r][c + 1]) + 6 * s_v[r][c];
        const int gy = oy + r, gx = ox + x;
        if (gy < dh && gx < dw)
            dst[(size_t)gy * dpitch + gx] = (float)((h + 128) >> 8);
    }
}

template <bool FROM_U8>
__global__ void __launch_bounds__(256) pyr_reduce_kernel(const void *__restrict__ src_, int sw, int sh, int spitch,
                                                         float *__restrict__ l0, int l0pitch, float *__restrict__ dst,
                                                         int dw, int dh, int dpitch)
{
    __shared__ int s_src[RS_Y][RS_X + 1];
    __shared__ int s_v[RT_Y][RS_X + 1];
    reduce_tile<FROM_U8>(src_, sw, sh, spitch, l0, l0pitch, dst, dw, dh, dpitch, blockIdx.x * RT_X, blockIdx.y * RT_Y,
                         s_src, s_v);
}

/* Many frames at once: the launch's tiles are every job's tiles of this level, back to back; a block finds its job by
 * binary search over the tile offsets. Level 1 (with level 0) from each job's bytes, or level L from level L - 1. */
template <bool FROM_U8>
__global__ void __launch_bounds__(256) pyr_batch_kernel(const PyrJob *__restrict__ jobs, const int *__restrict__ start,
                                                        int njobs, int level)
{
    __shared__ int s_src[RS_Y][RS_X + 1];
    __shared__ int s_v[RT_Y][RS_X + 1];
    const int b = blockIdx.x;
    int lo = 0, hi = njobs; /* start[lo] <= b < start[hi] */
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(start + mid) <= b)
            lo = mid;
        else
            hi = mid;
    }
    const PyrJob &j = jobs[lo];
    const int t = b - __ldg(start + lo);
    const int sw = FROM_U8 ? j.w : j.lw[level - 1], sh = FROM_U8 ? j.h : j.lh[level - 1];
    const int dw = (sw + 1) / 2, dh = (sh + 1) / 2;
    const int tiles_x = (dw + RT_X - 1) / RT_X;
    const int ox = (t % tiles_x) * RT_X, oy = (t / tiles_x) * RT_Y;
    if (FROM_U8)
        reduce_tile<true>(j.src, j.w, j.h, j.stride, j.lv[0], j.pitch[0], j.levels > 1 ? j.lv[1] : nullptr, dw, dh,
                          j.pitch[1], ox, oy, s_src, s_v);
    else
        reduce_tile<false>(j.lv[level - 1], sw, sh, j.pitch[level - 1], nullptr, 0, j.lv[level], dw, dh, j.pitch[level],
                           ox, oy, s_src, s_v);
}

int vtg_pyr_tiles(int w, int h, int level)
{
    /* tiles of the launch that makes `level` (1: levels 0 and 1) from a w x h frame */
    int sw = w, sh = h;
    for (int L = 1; L < level; L++) {
        sw = (sw + 1) / 2;
        sh = (sh + 1) / 2;
    }
    const int dw = (sw + 1) / 2, dh = (sh + 1) / 2;
    return ((dw + RT_X - 1) / RT_X) * ((dh + RT_Y - 1) / RT_Y);
}

cudaError_t vtg_launch_pyramid_batch(const PyrJob *jobs, const int *starts, const int *tiles_total, int njobs,
                                     int max_levels, cudaStream_t s)
{
    for (int L = 1; L < (max_levels > 1 ? max_levels : 2); L++) {
        const int tiles = tiles_total[L - 1];
        if (tiles <= 0)
            continue;
        if (L == 1)
            pyr_batch_kernel<true><<<tiles, 256, 0, s>>>(jobs, starts + (size_t)(L - 1) * (njobs + 1), njobs, L);
        else
            pyr_batch_kernel<false><<<tiles, 256, 0, s>>>(jobs, starts + (size_t)(L - 1) * (njobs + 1), njobs, L);
    }
    return cudaGetLastError();
}

cudaError_t vtg_launch_pyramid(const uint8_t *frame, int stride, int w, int h, float *const *levels, const int *pitches,
                               int nlevels, cudaStream_t s)
{
    /* Level 0 and level 1 from the bytes. */
    int sw = (w + 1) / 2, sh = (h + 1) / 2;
    {
        const dim3 grid((sw + RT_X - 1) / RT_X, (sh + RT_Y - 1) / RT_Y);
        pyr_reduce_kernel<true><<<grid, 256, 0, s>>>(frame, w, h, stride, levels[0], pitches[0],
                                                     nlevels > 1 ? levels[1] : nullptr, sw, sh, nlevels > 1 ? pitches[1] : 0);
    }
    for (int L = 2; L < nlevels; L++) {
        const int dw = (sw + 1) / 2, dh = (sh + 1) / 2;
        const dim3 grid((dw + RT_X - 1) / RT_X, (dh + RT_Y - 1) / RT_Y);
        pyr_reduce_kernel<false><<<grid, 256, 0, s>>>(levels[L - 1], sw, sh, pitches[L - 1], nullptr, 0, levels[L], dw, dh,
                                                      pitches[L]);
        sw = dw;
        sh = dh;
    }
    return cudaGetLastError();
}
