/* pyramid.cu -- the Gaussian pyramid of an 8-bit frame, bit-exact to the reference's Q6 planes.
 *
 * Reference: tk_build (src/kern/track.c:584-629) runs img_u8_to_q6 (src/kern/img_ref.c:32-40, img_vx.c:24-34) and
 * img_pad_rows / img_pad_tb (img_ref.c:9-30) for level 0, then img_reduce (img_ref.c:98-114, img_vx.c:129-162) per
 * level: the 5 x 5 binomial (1 4 6 4 1)^2 at every second pixel of every second row, rounded as (sum + 128) >> 8,
 * reading a replicated border. Every value is a whole number below 2^24, so the reference's F32 sums are exact; here
 * they are int32 sums, the border is a clamped index, and the results are the same bits.
 *
 * Levels 0 to 3 in one launch (pyr_fused_kernel, pyr_fused_batch_kernel): a CTA reads its block's bytes once and
 * reduces level by level in shared memory, halos included (below). Levels from 4 on, and level 1 when level 0 came
 * from tk_build's input steps, take one launch per level (pyr_reduce_kernel, pyr_batch_kernel): a CTA of 256 threads
 * makes a 64 x 16 tile of its output level from a 132 x 36 source tile staged in shared memory, the vertical pass over
 * the staged rows, the horizontal pass over the vertical sums, as the reference's vert5 / shift8 do. */
#include <math.h>

#include "vtg_internal.cuh"
#include "x87.cuh"

#define RT_X 64 /* output tile */
#define RT_Y 16
#define RS_Y (2 * RT_Y + 4) /* source rows of a tile: two each side */
/* Staged columns. A tile's source columns are 2 ox - 2 .. 2 ox + 129; staging starts 16-byte aligned before them:
 * bytes from 2 ox - 16 (160 of them), F32 values from 2 ox - 4 (136). Column k of the vertical sums is source column
 * 2 ox - 4 + k in both. */
#define SB_X 160
#define SF_X 136
#define SF_P 140 /* int row pitch of staged F32 values and of the vertical sums: 16-byte aligned rows */
#define PK_G (SF_X / 4) /* four-column groups of vertical sums in a row (the byte path's packed words) */

/* A whole number 0 <= v < 2^23 as a float without a conversion instruction: the bits of 2^23 + v, less 2^23. */
__device__ __forceinline__ float small_int_to_float(int v)
{
    return __int_as_float(0x4B000000 | v) - 8388608.0f;
}

/* Byte e of w times 64 (a Q6 value) as a float: the byte placed in the mantissa of 2^23 by one byte permute, then
 * (2^23 + b) x 64 - 2^29 = 64 b in one fused multiply-add, exact (2^29 + 64 b is a multiple of 64 below 2^30). */
__device__ __forceinline__ float q6_of(uint32_t w, int e)
{
    return __fmaf_rn(__int_as_float((int)__byte_perm(w, 0x4Bu, 0x4550u + (unsigned)e)), 64.0f, -536870912.0f);
}

/* One 64 x 16 tile of the output level at (ox, oy). With FROM_U8 the source is the frame's bytes (rows `spitch`
 * bytes apart), level 0 (byte x 64) is written from the same staged bytes, and the sums run on the bytes:
 * (64 h + 128) >> 8 = (h + 2) >> 2 exactly. Otherwise the source is level L - 1 (F32 Q6, whole numbers) and the result
 * is (h + 128) >> 8. vec: the source rows may be read 16 bytes at a time (base and pitch 16-byte aligned). dst may be
 * NULL (level 0 only). Staging reads whole 16-byte chunks inside the row and clamps the chunks that reach past an
 * edge element by element, so every read is inside the plane and the border is the reference's replicated edge. */
template <bool FROM_U8>
__device__ __forceinline__ void reduce_tile(const void *__restrict__ src_, int sw, int sh, int spitch, bool vec,
                                            float *__restrict__ l0, int l0pitch, float *__restrict__ dst, int dw, int dh,
                                            int dpitch, int ox, int oy, uint8_t (*s_b)[SB_X], int (*s_f)[SF_P],
                                            int (*s_v)[SF_P])
{
    const int tid = threadIdx.x;
    const int sy0 = 2 * oy - 2;
    if (FROM_U8) {
        const uint8_t *src = (const uint8_t *)src_;
        const int gx0 = 2 * ox - 16;
        for (int i = tid; i < RS_Y * (SB_X / 16); i += blockDim.x) {
            const int r = i / (SB_X / 16), k = i - r * (SB_X / 16);
            const int gy = min(max(sy0 + r, 0), sh - 1), gx = gx0 + 16 * k;
            const uint8_t *row = src + (size_t)gy * spitch;
            uint4 v;
            if (vec && gx >= 0 && gx + 16 <= sw) {
                v = __ldg(reinterpret_cast<const uint4 *>(row + gx));
            } else {
                uint32_t w[4];
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    uint32_t x = 0;
#pragma unroll
                    for (int e = 0; e < 4; e++)
                        x |= (uint32_t)__ldg(row + min(max(gx + 4 * q + e, 0), sw - 1)) << (8 * e);
                    w[q] = x;
                }
                v = make_uint4(w[0], w[1], w[2], w[3]);
            }
            *reinterpret_cast<uint4 *>(&s_b[r][16 * k]) = v;
        }
        __syncthreads();
        /* level 0: rows 2 oy .. 2 oy + 31, columns 2 ox .. 2 ox + 127 (staged columns 16 .. 143), four a thread */
        for (int i = tid; i < 2 * RT_Y * (2 * RT_X / 4); i += blockDim.x) {
            const int r = i / (2 * RT_X / 4), g = i - r * (2 * RT_X / 4);
            const int gy = 2 * oy + r, gx = 2 * ox + 4 * g;
            if (gy >= sh || gx >= sw)
                continue;
            const uint32_t w = *reinterpret_cast<const uint32_t *>(&s_b[r + 2][16 + 4 * g]);
            const float4 f = make_float4(q6_of(w, 0), q6_of(w, 1), q6_of(w, 2), q6_of(w, 3));
            float *d = l0 + (size_t)gy * l0pitch + gx;
            if (gx + 4 <= sw) {
                *reinterpret_cast<float4 *>(d) = f;
            } else {
                d[0] = f.x;
                if (gx + 1 < sw)
                    d[1] = f.y;
                if (gx + 2 < sw)
                    d[2] = f.z;
            }
        }
        if (!dst)
            return;
        /* vertical sums of staged byte columns 12 .. 147 (source 2 ox - 4 ..), four columns a thread, two to a word:
         * group g's even columns in the 16-bit halves of E_g, its odd columns in O_g. A sum is at most 16 x 255 =
         * 4080, so whole-word adds never carry from one half into the other. */
        uint32_t *s_e = reinterpret_cast<uint32_t *>(&s_v[0][0]), *s_o = s_e + RT_Y * PK_G;
        for (int i = tid; i < RT_Y * PK_G; i += blockDim.x) {
            const int r = i / PK_G, g = i - r * PK_G;
            uint32_t e[5], o[5];
#pragma unroll
            for (int t = 0; t < 5; t++) {
                const uint32_t w = *reinterpret_cast<const uint32_t *>(&s_b[2 * r + t][12 + 4 * g]);
                e[t] = w & 0x00FF00FFu;
                o[t] = (w >> 8) & 0x00FF00FFu;
            }
            s_e[i] = e[0] + e[4] + 4u * (e[1] + e[3]) + 6u * e[2];
            s_o[i] = o[0] + o[4] + 4u * (o[1] + o[3]) + 6u * o[2];
        }
        __syncthreads();
        /* horizontal, two outputs a word: outputs 2m and 2m + 1 take vertical sums 4m + 2 .. 4m + 6 and 4m + 4 ..
         * 4m + 8, i.e. the pairs (E_m hi, E_m+1 lo), (O_m hi, O_m+1 lo), E_m+1, O_m+1, (E_m+1 hi, E_m+2 lo) with
         * weights 1, 4, 6, 4, 1. A sum is at most 16 x 4080 = 65280 in each half; (h + 2) >> 2 is at most 16320, so
         * the mask drops exactly the bits the high half shifts into the low one. Four outputs a thread. */
        for (int i = tid; i < RT_Y * (RT_X / 4); i += blockDim.x) {
            const int r = i / (RT_X / 4), q = i - r * (RT_X / 4);
            const int gy = oy + r, gx = ox + 4 * q;
            if (gy >= dh || gx >= dw)
                continue;
            const uint32_t *E = s_e + r * PK_G + 2 * q, *O = s_o + r * PK_G + 2 * q;
            uint32_t res[2];
#pragma unroll
            for (int p = 0; p < 2; p++) {
                const uint32_t e1 = E[p + 1], o1 = O[p + 1];
                const uint32_t A = __byte_perm(E[p], e1, 0x5432), B = __byte_perm(O[p], o1, 0x5432);
                const uint32_t F = __byte_perm(e1, E[p + 2], 0x5432);
                const uint32_t h = A + F + 4u * (B + o1) + 6u * e1;
                res[p] = ((h + 0x00020002u) >> 2) & 0x3FFF3FFFu;
            }
            const float o[4] = {small_int_to_float((int)(res[0] & 0xFFFFu)), small_int_to_float((int)(res[0] >> 16)),
                                small_int_to_float((int)(res[1] & 0xFFFFu)), small_int_to_float((int)(res[1] >> 16))};
            float *d = dst + (size_t)gy * dpitch + gx;
            if (gx + 4 <= dw) {
                *reinterpret_cast<float4 *>(d) = make_float4(o[0], o[1], o[2], o[3]);
            } else {
                for (int e = 0; e < 4 && gx + e < dw; e++)
                    d[e] = o[e];
            }
        }
        return;
    } else {
        const float *src = (const float *)src_;
        const int gx0 = 2 * ox - 4;
        for (int i = tid; i < RS_Y * (SF_X / 4); i += blockDim.x) {
            const int r = i / (SF_X / 4), k = i - r * (SF_X / 4);
            const int gy = min(max(sy0 + r, 0), sh - 1), gx = gx0 + 4 * k;
            const float *row = src + (size_t)gy * spitch;
            float4 v;
            if (vec && gx >= 0 && gx + 4 <= sw) /* vec: the plane and its pitch are 16-byte aligned */
                v = __ldg(reinterpret_cast<const float4 *>(row + gx));
            else
                v = make_float4(__ldg(row + min(max(gx, 0), sw - 1)), __ldg(row + min(max(gx + 1, 0), sw - 1)),
                                __ldg(row + min(max(gx + 2, 0), sw - 1)), __ldg(row + min(max(gx + 3, 0), sw - 1)));
            *reinterpret_cast<float4 *>(&s_f[r][4 * k]) = v;
        }
        __syncthreads();
        for (int i = tid; i < RT_Y * (SF_X / 4); i += blockDim.x) {
            const int r = i / (SF_X / 4), g = i - r * (SF_X / 4);
            /* F32 as the reference sums: whole numbers below 2^24, so every sum is exact */
            float4 t[5];
#pragma unroll
            for (int q = 0; q < 5; q++)
                t[q] = *reinterpret_cast<const float4 *>(&s_f[2 * r + q][4 * g]);
            float4 o;
            o.x = t[0].x + t[4].x + 4.0f * (t[1].x + t[3].x) + 6.0f * t[2].x;
            o.y = t[0].y + t[4].y + 4.0f * (t[1].y + t[3].y) + 6.0f * t[2].y;
            o.z = t[0].z + t[4].z + 4.0f * (t[1].z + t[3].z) + 6.0f * t[2].z;
            o.w = t[0].w + t[4].w + 4.0f * (t[1].w + t[3].w) + 6.0f * t[2].w;
            *reinterpret_cast<float4 *>(&s_v[r][4 * g]) = o;
        }
    }
    __syncthreads();
    /* horizontal: output x takes vertical sums 2 x + 2 .. 2 x + 6; four outputs a thread (sums 8 g .. 8 g + 15) */
    for (int i = tid; i < RT_Y * (RT_X / 4); i += blockDim.x) {
        const int r = i / (RT_X / 4), g = i - r * (RT_X / 4);
        const int gy = oy + r, gx = ox + 4 * g;
        if (gy >= dh || gx >= dw)
            continue;
        int v[16];
#pragma unroll
        for (int q = 0; q < 4; q++)
            *reinterpret_cast<int4 *>(&v[4 * q]) = *reinterpret_cast<const int4 *>(&s_v[r][8 * g + 4 * q]);
        float o[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int c = 2 * e + 4;
            const float *f = reinterpret_cast<const float *>(v);
            const float h = f[c - 2] + f[c + 2] + 4.0f * (f[c - 1] + f[c + 1]) + 6.0f * f[c];
            o[e] = floorf((h + 128.0f) * (1.0f / 256.0f)); /* (h + 128) >> 8, exact */
        }
        float *d = dst + (size_t)gy * dpitch + gx;
        if (gx + 4 <= dw) {
            *reinterpret_cast<float4 *>(d) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
            for (int e = 0; e < 4 && gx + e < dw; e++)
                d[e] = o[e];
        }
    }
}

/* The staged source: bytes for the first launch, ints (F32 values) for the others. */
union TileSmem {
    __align__(16) uint8_t b[RS_Y][SB_X];
    __align__(16) int f[RS_Y][SF_P];
};

static __device__ __forceinline__ bool aligned16(const void *p, int pitch_bytes)
{
    return (((uintptr_t)p | (uintptr_t)pitch_bytes) & 15) == 0;
}

template <bool FROM_U8>
__global__ void __launch_bounds__(256) pyr_reduce_kernel(const void *__restrict__ src_, int sw, int sh, int spitch,
                                                         float *__restrict__ l0, int l0pitch, float *__restrict__ dst,
                                                         int dw, int dh, int dpitch)
{
    __shared__ TileSmem s_t;
    __shared__ __align__(16) int s_v[RT_Y][SF_P];
    reduce_tile<FROM_U8>(src_, sw, sh, spitch, aligned16(src_, FROM_U8 ? spitch : spitch * 4), l0, l0pitch, dst, dw, dh, dpitch,
                         blockIdx.x * RT_X, blockIdx.y * RT_Y, s_t.b, s_t.f, s_v);
}

/* Many frames at once: the launch's tiles are every job's tiles of this level, back to back; a block finds its job by
 * binary search over the tile offsets. Level 1 (with level 0) from each job's bytes, or level L from level L - 1. */
template <bool FROM_U8>
__global__ void __launch_bounds__(256) pyr_batch_kernel(const PyrJob *__restrict__ jobs, const int *__restrict__ start,
                                                        int njobs, int level, int *__restrict__ reset)
{
    __shared__ TileSmem s_t;
    __shared__ __align__(16) int s_v[RT_Y][SF_P];
    vtg_grid_dependency_wait(); /* the level below, when launched as a dependent of its launch */
    if (reset && blockIdx.x == 0 && threadIdx.x == 0)
        *reset = 0;
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
    if (FROM_U8 && j.opts) {
        /* level 0 came from the build options' launches: level 1 reduces it like any other level */
        if (j.levels > 1)
            reduce_tile<false>(j.lv[0], j.w, j.h, j.pitch[0], true, nullptr, 0, j.lv[1], dw, dh, j.pitch[1], ox, oy,
                               s_t.b, s_t.f, s_v);
    } else if (FROM_U8)
        reduce_tile<true>(j.src, j.w, j.h, j.stride, aligned16(j.src, j.stride), j.lv[0], j.pitch[0],
                          j.levels > 1 ? j.lv[1] : nullptr, dw, dh, j.pitch[1], ox, oy, s_t.b, s_t.f, s_v);
    else
        reduce_tile<false>(j.lv[level - 1], sw, sh, j.pitch[level - 1], true, nullptr, 0, j.lv[level], dw, dh,
                           j.pitch[level], ox, oy, s_t.b, s_t.f, s_v);
}

/* ---- levels 0 to 3 from the bytes in one launch ----
 *
 * A CTA owns a 128 x 64 block of level 0 and the blocks of levels 1, 2 and 3 under it (64 x 32, 32 x 16, 16 x 8). It
 * stages the bytes the block's level 3 depends on (rows Y0 - 14 .. Y0 + 70, columns X0 - 16 .. X0 + 143, each clamped
 * into the frame: the reference's replicated border), writes level 0 from them, and reduces in shared memory: level 1
 * over 73 x 41 values (the block and the halo level 2 needs), level 2 over 35 x 19, level 3 over its 16 x 8. A level's
 * reduce reads the level below at the reference's clamped indices, which always fall inside the computed halo, so the
 * values outside a level's plane that the halo holds are never read. Every sum is an exact integer: (sum of the bytes'
 * taps + 2) >> 2 for level 1 ((64 h + 128) >> 8 of the Q6 values), (h + 128) >> 8 above. Level 1 is then never read
 * back from memory, and three launches become one. */
#define FP_X 128 /* a CTA's level-0 block */
#define FP_Y 64
#define FB_R 85  /* staged byte rows: Y0 - 14 .. Y0 + 70 */
#define FB_C 160 /* staged byte columns: X0 - 16 .. X0 + 143 (16-byte chunks) */
#define F1_R 41  /* level 1 computed: rows Y0 / 2 - 6 .. Y0 / 2 + 34 */
#define F1_C 73  /*                   columns X0 / 2 - 6 .. X0 / 2 + 66 */
#define F1_P 76
#define F2_R 19  /* level 2: rows Y0 / 4 - 2 .. Y0 / 4 + 16 */
#define F2_C 35  /*          columns X0 / 4 - 2 .. X0 / 4 + 32 */
#define F2_P 36
#define F3_R 8   /* level 3: the block, rows Y0 / 8 .. + 7 */
#define F3_C 16  /*          columns X0 / 8 .. + 15 */

struct FusedSmem {
    __align__(16) uint8_t b[FB_R][FB_C];   /* the bytes */
    __align__(16) uint16_t v1[F1_R][FB_C]; /* level 1's vertical sums of the bytes (at most 16 x 255) */
    __align__(16) uint16_t l1[F1_R][F1_P]; /* level 1 (at most 16320) */
    __align__(16) int v2[F2_R][F1_P];      /* level 2's vertical sums of level 1 */
    __align__(16) uint16_t l2[F2_R][F2_P]; /* level 2 */
    __align__(16) int v3[F3_R][F2_P];      /* level 3's vertical sums of level 2 */
};

/* One frame of a fused launch: the bytes (rows `stride` apart), and levels 0 .. min(levels, 4) - 1. */
struct FusedFrame {
    const uint8_t *src;
    int stride, w, h, levels;
    float *lv[4];
    int pitch[4];
};

__device__ __forceinline__ int tap5(int a, int b, int c, int d, int e) { return a + e + 4 * (b + d) + 6 * c; }

/* A block is interior when every byte it stages lies inside the frame. Then no index of any level needs a clamp, and
 * every write of its blocks lies inside their planes. */
__device__ __forceinline__ bool fused_interior(const FusedFrame &f, int X0, int Y0)
{
    return X0 >= 16 && X0 + 144 <= f.w && Y0 >= 14 && Y0 + 71 <= f.h;
}

template <bool EDGE>
__device__ void fused_block(const FusedFrame &f, int X0, int Y0, FusedSmem &S)
{
    const int tid = threadIdx.x, nt = blockDim.x;
    const int w = f.w, h = f.h;
    const int w1 = (w + 1) / 2, h1 = (h + 1) / 2, w2 = (w1 + 1) / 2, h2 = (h1 + 1) / 2, w3 = (w2 + 1) / 2,
              h3 = (h2 + 1) / 2;
    const bool vec = (((uintptr_t)f.src | (uintptr_t)f.stride) & 15) == 0;
    /* the bytes: staged row r is frame row Y0 - 14 + r, staged column c frame column X0 - 16 + c, both clamped */
    for (int i = tid; i < FB_R * (FB_C / 16); i += nt) {
        const int r = i / (FB_C / 16), k = i - r * (FB_C / 16);
        const int gy = EDGE ? min(max(Y0 - 14 + r, 0), h - 1) : Y0 - 14 + r, gx = X0 - 16 + 16 * k;
        const uint8_t *row = f.src + (size_t)gy * f.stride;
        uint4 v;
        if (vec && (!EDGE || (gx >= 0 && gx + 16 <= w))) {
            v = __ldg(reinterpret_cast<const uint4 *>(row + gx));
        } else {
            uint32_t q[4];
#pragma unroll
            for (int a = 0; a < 4; a++) {
                uint32_t x = 0;
#pragma unroll
                for (int e = 0; e < 4; e++)
                    x |= (uint32_t)__ldg(row + min(max(gx + 4 * a + e, 0), w - 1)) << (8 * e);
                q[a] = x;
            }
            v = make_uint4(q[0], q[1], q[2], q[3]);
        }
        *reinterpret_cast<uint4 *>(&S.b[r][16 * k]) = v;
    }
    __syncthreads();
    /* level 0: the block's rows (staged 14 ..) and columns (staged 16 ..), four a thread */
    for (int i = tid; i < FP_Y * (FP_X / 4); i += nt) {
        const int r = i / (FP_X / 4), g = i - r * (FP_X / 4);
        const int gy = Y0 + r, gx = X0 + 4 * g;
        if (EDGE && (gy >= h || gx >= w))
            continue;
        const uint32_t q = *reinterpret_cast<const uint32_t *>(&S.b[r + 14][16 + 4 * g]);
        const float4 o = make_float4(q6_of(q, 0), q6_of(q, 1), q6_of(q, 2), q6_of(q, 3));
        float *d = f.lv[0] + (size_t)gy * f.pitch[0] + gx;
        if (!EDGE || gx + 4 <= w) {
            *reinterpret_cast<float4 *>(d) = o;
        } else {
            d[0] = o.x;
            if (gx + 1 < w)
                d[1] = o.y;
            if (gx + 2 < w)
                d[2] = o.z;
        }
    }
    if (f.levels < 2)
        return;
    /* level 1's vertical sums: local row y (frame row of level 1 Y0 / 2 - 6 + y) takes staged rows 2 y .. 2 y + 4;
     * four columns a thread, even and odd bytes in the 16-bit halves of two words (no half carries: at most 4080) */
    for (int i = tid; i < F1_R * (FB_C / 4); i += nt) {
        const int y = i / (FB_C / 4), g = i - y * (FB_C / 4);
        uint32_t e[5], o[5];
#pragma unroll
        for (int t = 0; t < 5; t++) {
            const uint32_t q = *reinterpret_cast<const uint32_t *>(&S.b[2 * y + t][4 * g]);
            e[t] = q & 0x00FF00FFu;
            o[t] = (q >> 8) & 0x00FF00FFu;
        }
        const uint32_t E = e[0] + e[4] + 4u * (e[1] + e[3]) + 6u * e[2];
        const uint32_t O = o[0] + o[4] + 4u * (o[1] + o[3]) + 6u * o[2];
        *reinterpret_cast<uint2 *>(&S.v1[y][4 * g]) = make_uint2((E & 0xFFFFu) | (O << 16), (E >> 16) | (O & 0xFFFF0000u));
    }
    __syncthreads();
    /* level 1: local column x (frame column X0 / 2 - 6 + x) centres on staged column 2 x + 4. Two columns a thread in
     * the halves of one word: with w_k = v1 columns 2 x + 2 + 2 k and 2 x + 3 + 2 k, column x takes (w_0 lo, w_0 hi,
     * w_1 lo, w_1 hi, w_2 lo) and column x + 1 the same one word on. A sum is at most 16 x 4080 = 65280 a half, and
     * (h + 2) >> 2 at most 16320, so the mask drops exactly what the high half shifts into the low one. */
    for (int i = tid; i < F1_R * ((F1_C + 1) / 2); i += nt) {
        const int y = i / ((F1_C + 1) / 2), x = 2 * (i - y * ((F1_C + 1) / 2));
        const uint32_t *v = reinterpret_cast<const uint32_t *>(&S.v1[y][2 * x + 2]);
        const uint32_t w0 = v[0], w1 = v[1], w2 = v[2], w3 = v[3];
        const uint32_t L0 = __byte_perm(w0, w1, 0x5410), H0 = __byte_perm(w0, w1, 0x7632);
        const uint32_t L1 = __byte_perm(w1, w2, 0x5410), H1 = __byte_perm(w1, w2, 0x7632);
        const uint32_t L2 = __byte_perm(w2, w3, 0x5410);
        const uint32_t hs = L0 + L2 + 4u * (H0 + H1) + 6u * L1;
        *reinterpret_cast<uint32_t *>(&S.l1[y][x]) = ((hs + 0x00020002u) >> 2) & 0x3FFF3FFFu;
    }
    __syncthreads();
    /* level 1's block (local rows and columns 6 ..), four columns a thread */
    const int o1x = X0 / 2 - 6, o1y = Y0 / 2 - 6; /* level 1's local origin */
    for (int i = tid; i < (FP_Y / 2) * (FP_X / 8); i += nt) {
        const int r = i / (FP_X / 8), c = 4 * (i - r * (FP_X / 8));
        const int gy = Y0 / 2 + r, gx = X0 / 2 + c;
        if (EDGE && (gy >= h1 || gx >= w1))
            continue;
        const uint32_t a = *reinterpret_cast<const uint32_t *>(&S.l1[r + 6][c + 6]);
        const uint32_t b = *reinterpret_cast<const uint32_t *>(&S.l1[r + 6][c + 8]);
        const float4 o = make_float4(small_int_to_float((int)(a & 0xFFFFu)), small_int_to_float((int)(a >> 16)),
                                     small_int_to_float((int)(b & 0xFFFFu)), small_int_to_float((int)(b >> 16)));
        float *d = f.lv[1] + (size_t)gy * f.pitch[1] + gx;
        if (!EDGE || gx + 4 <= w1) {
            *reinterpret_cast<float4 *>(d) = o;
        } else {
            d[0] = o.x;
            if (gx + 1 < w1)
                d[1] = o.y;
            if (gx + 2 < w1)
                d[2] = o.z;
        }
    }
    if (f.levels < 3)
        return;
    /* level 2's vertical sums over level 1's (clamped) rows */
    const int o2x = X0 / 4 - 2, o2y = Y0 / 4 - 2; /* level 2's local origin */
    for (int i = tid; i < F2_R * F1_C; i += nt) {
        const int y = i / F1_C, x = i - y * F1_C;
        int a[5];
#pragma unroll
        for (int t = 0; t < 5; t++)
            a[t] = S.l1[EDGE ? min(max(2 * (o2y + y) - 2 + t, 0), h1 - 1) - o1y : 2 * y + t][x];
        S.v2[y][x] = tap5(a[0], a[1], a[2], a[3], a[4]);
    }
    __syncthreads();
    for (int i = tid; i < F2_R * F2_C; i += nt) {
        const int y = i / F2_C, x = i - y * F2_C;
        int a[5];
#pragma unroll
        for (int t = 0; t < 5; t++)
            a[t] = S.v2[y][EDGE ? min(max(2 * (o2x + x) - 2 + t, 0), w1 - 1) - o1x : 2 * x + t];
        S.l2[y][x] = (uint16_t)((tap5(a[0], a[1], a[2], a[3], a[4]) + 128) >> 8);
    }
    __syncthreads();
    for (int i = tid; i < (FP_Y / 4) * (FP_X / 4); i += nt) {
        const int r = i / (FP_X / 4), c = i - r * (FP_X / 4);
        const int gy = Y0 / 4 + r, gx = X0 / 4 + c;
        if (!EDGE || (gy < h2 && gx < w2))
            f.lv[2][(size_t)gy * f.pitch[2] + gx] = small_int_to_float(S.l2[r + 2][c + 2]);
    }
    if (f.levels < 4)
        return;
    for (int i = tid; i < F3_R * F2_C; i += nt) {
        const int y = i / F2_C, x = i - y * F2_C;
        int a[5];
#pragma unroll
        for (int t = 0; t < 5; t++)
            a[t] = S.l2[EDGE ? min(max(2 * (Y0 / 8 + y) - 2 + t, 0), h2 - 1) - o2y : 2 * y + t][x];
        S.v3[y][x] = tap5(a[0], a[1], a[2], a[3], a[4]);
    }
    __syncthreads();
    for (int i = tid; i < F3_R * F3_C; i += nt) {
        const int y = i / F3_C, x = i - y * F3_C;
        const int gy = Y0 / 8 + y, gx = X0 / 8 + x;
        if (EDGE && (gy >= h3 || gx >= w3))
            continue;
        int a[5];
#pragma unroll
        for (int t = 0; t < 5; t++)
            a[t] = S.v3[y][EDGE ? min(max(2 * gx - 2 + t, 0), w2 - 1) - o2x : 2 * x + t];
        f.lv[3][(size_t)gy * f.pitch[3] + gx] = small_int_to_float((tap5(a[0], a[1], a[2], a[3], a[4]) + 128) >> 8);
    }
}

__device__ __forceinline__ void fused_any(const FusedFrame &f, int bx, int by, FusedSmem &S)
{
    const int X0 = bx * FP_X, Y0 = by * FP_Y;
    if (fused_interior(f, X0, Y0))
        fused_block<false>(f, X0, Y0, S);
    else
        fused_block<true>(f, X0, Y0, S);
}

__global__ void __launch_bounds__(256) pyr_fused_kernel(FusedFrame f)
{
    __shared__ FusedSmem S;
    fused_any(f, blockIdx.x, blockIdx.y, S);
}

/* Many frames: the launch's blocks are every job's blocks back to back; a CTA finds its job by binary search. */
__global__ void __launch_bounds__(256) pyr_fused_batch_kernel(const PyrJob *__restrict__ jobs, const int *__restrict__ start,
                                                              int njobs, int *__restrict__ reset)
{
    __shared__ FusedSmem S;
    if (reset && blockIdx.x == 0 && threadIdx.x == 0)
        *reset = 0;
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
    FusedFrame f;
    f.src = j.src;
    f.stride = j.stride;
    f.w = j.w;
    f.h = j.h;
    f.levels = j.levels;
#pragma unroll
    for (int L = 0; L < 4; L++) {
        f.lv[L] = L < j.levels ? j.lv[L] : nullptr;
        f.pitch[L] = L < j.levels ? j.pitch[L] : 0;
    }
    const int t = b - __ldg(start + lo), bcols = (j.w + FP_X - 1) / FP_X;
    fused_any(f, t % bcols, t / bcols, S);
}

int vtg_pyr_fused_tiles(int w, int h) { return ((w + FP_X - 1) / FP_X) * ((h + FP_Y - 1) / FP_Y); }

/* ---- tk_build's optional input steps (src/kern/track.c:600-622) ----
 *
 * CONTRAST: the min and max of the frame (img_minmax_ref, img_ref.c:57-71), the gain 16320 / (max - min) and the offset
 * -min x gain in x87 extended precision (track.c:603-614), each rounded to F32, then per pixel
 * clamp(rint(Q6 x gain + offset), 0, 16320) (img_norm, img_ref.c:42-55). PRE_GAUSS: the 5 x 5 binomial of that with
 * (h + 128) >> 8 (img_gauss5, img_ref.c:83-96). The result is level 0. The stretch runs on the bytes through a table:
 * a frame has 256 byte values, each mapped once per CTA. */

/* tk_build's gain and offset (track.c:606-614) for Q6 minimum lo and maximum hi: gain = 16320 / (hi - lo) or 1, offset
 * = -lo x gain, both formed in extended precision and rounded to F32. */
__host__ __device__ static inline void contrast_gain(int lo, int hi, float *go)
{
    if (hi > lo) {
        const X87 g = x87_div(16320u, (uint32_t)(hi - lo));
        go[0] = x87_to_f32(g);
        go[1] = -x87_to_f32(x87_mul(g, (uint32_t)lo));
    } else {
        go[0] = 1.0f;
        go[1] = -(float)lo;
    }
}

extern "C" int vtg_contrast_gain(int lo, int hi, float *gain_offset)
{
    if (!gain_offset || lo < 0 || hi < lo || hi >= (1 << 24))
        return VTG_EINVAL;
    contrast_gain(lo, hi, gain_offset);
    return VTG_OK;
}

/* The minimum and maximum over a CTA of per-thread values (min in the low byte of the result, max in the next). */
__device__ __forceinline__ uint32_t block_minmax(uint32_t mn, uint32_t mx, uint32_t *s_w)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    mn = __reduce_min_sync(VTG_FULL, mn);
    mx = __reduce_max_sync(VTG_FULL, mx);
    if (lane == 0)
        s_w[warp] = mn | (mx << 8);
    __syncthreads();
    if (warp == 0) {
        const uint32_t v = lane < (int)(blockDim.x >> 5) ? s_w[lane] : 255u;
        mn = __reduce_min_sync(VTG_FULL, v & 255u);
        mx = __reduce_max_sync(VTG_FULL, (v >> 8) & 255u);
        if (lane == 0)
            s_w[32] = mn | (mx << 8);
    }
    __syncthreads();
    const uint32_t r = s_w[32];
    __syncthreads();
    return r;
}

/* The frame's byte min and max (x 64 = img_minmax of its Q6 plane): CTA b scans rows b, b + grid, ... four bytes at a
 * time (16 with an aligned frame) and writes its partial to mm[b]; the last CTA to finish (a ticket in
 * mm[VTG_MM_BLOCKS]) combines the partials, writes gain and offset to mm[VTG_MM_BLOCKS + 1 ..] and resets the ticket. */
__global__ void __launch_bounds__(256) pyr_minmax_kernel(const uint8_t *__restrict__ src, int w, int h, int stride,
                                                         uint32_t *__restrict__ mm)
{
    __shared__ uint32_t s_w[33];
    __shared__ bool s_last;
    uint32_t mn4 = 0xffffffffu, mx4 = 0u;
    const bool vec = (((uintptr_t)src | (uintptr_t)stride) & 15) == 0;
    for (int y = blockIdx.x; y < h; y += gridDim.x) {
        const uint8_t *row = src + (size_t)y * stride;
        for (int x = 16 * (int)threadIdx.x; x < w; x += 16 * (int)blockDim.x) {
            uint32_t v[4];
            if (vec && x + 16 <= w) {
                const uint4 q = __ldg(reinterpret_cast<const uint4 *>(row + x));
                v[0] = q.x;
                v[1] = q.y;
                v[2] = q.z;
                v[3] = q.w;
            } else {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    uint32_t word = 0;
#pragma unroll
                    for (int e = 0; e < 4; e++) /* past the row's end: its last byte again, which changes nothing */
                        word |= (uint32_t)__ldg(row + min(x + 4 * k + e, w - 1)) << (8 * e);
                    v[k] = word;
                }
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                mn4 = __vminu4(mn4, v[k]);
                mx4 = __vmaxu4(mx4, v[k]);
            }
        }
    }
    uint32_t mn = min(min(mn4 & 255u, (mn4 >> 8) & 255u), min((mn4 >> 16) & 255u, mn4 >> 24));
    uint32_t mx = max(max(mx4 & 255u, (mx4 >> 8) & 255u), max((mx4 >> 16) & 255u, mx4 >> 24));
    const uint32_t part = block_minmax(mn, mx, s_w);
    if (threadIdx.x == 0) {
        mm[blockIdx.x] = part;
        __threadfence();
        s_last = atomicAdd(&mm[VTG_MM_BLOCKS], 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!s_last)
        return;
    __threadfence();
    mn = 255u;
    mx = 0u;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) {
        const uint32_t p = __ldcg(&mm[i]);
        mn = min(mn, p & 255u);
        mx = max(mx, (p >> 8) & 255u);
    }
    const uint32_t all = block_minmax(mn, mx, s_w);
    if (threadIdx.x == 0) {
        float go[2];
        contrast_gain(64 * (int)(all & 255u), 64 * (int)((all >> 8) & 255u), go);
        reinterpret_cast<float *>(mm)[VTG_MM_BLOCKS + 1] = go[0];
        reinterpret_cast<float *>(mm)[VTG_MM_BLOCKS + 2] = go[1];
        mm[VTG_MM_BLOCKS] = 0u; /* the next frame's ticket; this kernel's CTAs have all taken theirs */
    }
}

#define PT_X 64 /* level-0 tile of the input steps */
#define PT_Y 16

/* Level 0 under the build options, one 64 x 16 tile a CTA: the bytes mapped through the stretch's table (or x 64),
 * staged with a two-pixel clamped border, then the binomial's vertical and horizontal passes on whole numbers
 * (at most 16320 x 256, exact in int) when GAUSS. */
template <bool CONTRAST, bool GAUSS>
__global__ void __launch_bounds__(256) pyr_input_kernel(const uint8_t *__restrict__ src, int w, int h, int stride,
                                                        const uint32_t *__restrict__ mm, float *__restrict__ l0,
                                                        int pitch)
{
    __shared__ float s_lut[256];
    __shared__ __align__(16) int s_n[PT_Y + 4][PT_X + 4];
    __shared__ __align__(16) int s_v[PT_Y][PT_X + 4];
    const int tid = threadIdx.x;
    const int ox = blockIdx.x * PT_X, oy = blockIdx.y * PT_Y;
    if (CONTRAST) {
        const float g = __ldcg(reinterpret_cast<const float *>(mm) + VTG_MM_BLOCKS + 1);
        const float o = __ldcg(reinterpret_cast<const float *>(mm) + VTG_MM_BLOCKS + 2);
        /* the reference's x87 form rounds Q6 x gain + offset to F32 from an exact extended sum (the product has 38
         * bits, the sum's lowest bit is at least 2^-23 and its size below 2^23); one fused multiply-add rounds the
         * same exact value once */
        const float v = rintf(__fmaf_rn((float)(64 * tid), g, o));
        /* the reference's select, which keeps the -0 that rint gives a small negative value (the level's bits) */
        s_lut[tid] = v < 0.0f ? 0.0f : v > 16320.0f ? 16320.0f : v;
    } else {
        s_lut[tid] = (float)(64 * tid);
    }
    __syncthreads();
    if (GAUSS) {
        for (int i = tid; i < (PT_Y + 4) * (PT_X + 4); i += blockDim.x) {
            const int r = i / (PT_X + 4), c = i - r * (PT_X + 4);
            const int gy = min(max(oy - 2 + r, 0), h - 1), gx = min(max(ox - 2 + c, 0), w - 1);
            s_n[r][c] = (int)s_lut[__ldg(src + (size_t)gy * stride + gx)];
        }
        __syncthreads();
        for (int i = tid; i < PT_Y * (PT_X + 4); i += blockDim.x) {
            const int r = i / (PT_X + 4), c = i - r * (PT_X + 4);
            s_v[r][c] = s_n[r][c] + s_n[r + 4][c] + 4 * (s_n[r + 1][c] + s_n[r + 3][c]) + 6 * s_n[r + 2][c];
        }
        __syncthreads();
    }
    for (int i = tid; i < PT_Y * (PT_X / 4); i += blockDim.x) {
        const int r = i / (PT_X / 4), g = i - r * (PT_X / 4);
        const int gy = oy + r, gx = ox + 4 * g;
        if (gy >= h || gx >= w)
            continue;
        float o[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            if (GAUSS) {
                const int c = 4 * g + e; /* vertical sums c .. c + 4 around output column c + 2 of the staged tile */
                const int hs = s_v[r][c] + s_v[r][c + 4] + 4 * (s_v[r][c + 1] + s_v[r][c + 3]) + 6 * s_v[r][c + 2];
                o[e] = small_int_to_float((hs + 128) >> 8);
            } else {
                o[e] = s_lut[__ldg(src + (size_t)gy * stride + min(gx + e, w - 1))];
            }
        }
        float *d = l0 + (size_t)gy * pitch + gx;
        if (gx + 4 <= w) {
            *reinterpret_cast<float4 *>(d) = make_float4(o[0], o[1], o[2], o[3]);
        } else {
            for (int e = 0; e < 4 && gx + e < w; e++)
                d[e] = o[e];
        }
    }
}

cudaError_t vtg_launch_build_input(const uint8_t *frame, int stride, int w, int h, int opts, uint32_t *mm, float *l0,
                                   int pitch0, cudaStream_t s)
{
    const bool contrast = (opts & VTG_BUILD_CONTRAST) != 0, gauss = (opts & VTG_BUILD_PRE_GAUSS) != 0;
    if (contrast)
        pyr_minmax_kernel<<<min(h, VTG_MM_BLOCKS), 256, 0, s>>>(frame, w, h, stride, mm);
    const dim3 grid((w + PT_X - 1) / PT_X, (h + PT_Y - 1) / PT_Y);
    if (contrast && gauss)
        pyr_input_kernel<true, true><<<grid, 256, 0, s>>>(frame, w, h, stride, mm, l0, pitch0);
    else if (contrast)
        pyr_input_kernel<true, false><<<grid, 256, 0, s>>>(frame, w, h, stride, mm, l0, pitch0);
    else if (gauss)
        pyr_input_kernel<false, true><<<grid, 256, 0, s>>>(frame, w, h, stride, mm, l0, pitch0);
    return cudaGetLastError();
}

cudaError_t vtg_launch_pyramid_opts(const uint8_t *frame, int stride, int w, int h, float *const *levels,
                                    const int *pitches, int nlevels, int opts, uint32_t *mm, cudaStream_t s)
{
    if (!(opts & (VTG_BUILD_CONTRAST | VTG_BUILD_PRE_GAUSS)))
        return vtg_launch_pyramid(frame, stride, w, h, levels, pitches, nlevels, s);
    cudaError_t e = vtg_launch_build_input(frame, stride, w, h, opts, mm, levels[0], pitches[0], s);
    int sw = w, sh = h;
    for (int L = 1; L < nlevels && e == cudaSuccess; L++) {
        const int dw = (sw + 1) / 2, dh = (sh + 1) / 2;
        const dim3 grid((dw + RT_X - 1) / RT_X, (dh + RT_Y - 1) / RT_Y);
        pyr_reduce_kernel<false><<<grid, 256, 0, s>>>(levels[L - 1], sw, sh, pitches[L - 1], nullptr, 0, levels[L], dw,
                                                      dh, pitches[L]);
        e = cudaGetLastError();
        sw = dw;
        sh = dh;
    }
    return e;
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
                                     int max_levels, cudaStream_t s, int *reset, bool pdl, bool fused)
{
    const int top = max_levels > 1 ? max_levels : 2;
    int last = 1; /* the last level launched (level 1's launch always has tiles) */
    for (int L = fused ? 4 : 1; L < top; L++)
        if (tiles_total[L - 1] > 0)
            last = L;
    if (fused) {
        /* levels 0 .. 3 of every job in one launch (row VTG_MAX_LEVELS - 1 of the tables), then levels 4 .. */
        const cudaError_t e = vtg_launch_k(pyr_fused_batch_kernel, tiles_total[VTG_MAX_LEVELS - 1], 256, 0, s, false,
                                           jobs, (const int *)(starts + (size_t)(VTG_MAX_LEVELS - 1) * (njobs + 1)),
                                           njobs, last < 4 ? reset : (int *)nullptr);
        if (e != cudaSuccess)
            return e;
    }
    for (int L = fused ? 4 : 1; L < top; L++) {
        const int tiles = tiles_total[L - 1];
        if (tiles <= 0)
            continue;
        const int *st = starts + (size_t)(L - 1) * (njobs + 1);
        int *r = L == last ? reset : nullptr;
        const cudaError_t e = L == 1 ? vtg_launch_k(pyr_batch_kernel<true>, tiles, 256, 0, s, false, jobs, st, njobs, L, r)
                                     : vtg_launch_k(pyr_batch_kernel<false>, tiles, 256, 0, s, pdl, jobs, st, njobs, L, r);
        if (e != cudaSuccess)
            return e;
    }
    return cudaGetLastError();
}

cudaError_t vtg_launch_pyramid(const uint8_t *frame, int stride, int w, int h, float *const *levels, const int *pitches,
                               int nlevels, cudaStream_t s)
{
    /* Levels 0 .. 3 from the bytes in one launch, then one launch per further level. */
    FusedFrame f;
    f.src = frame;
    f.stride = stride;
    f.w = w;
    f.h = h;
    f.levels = nlevels;
    for (int L = 0; L < 4; L++) {
        f.lv[L] = L < nlevels ? levels[L] : nullptr;
        f.pitch[L] = L < nlevels ? pitches[L] : 0;
    }
    pyr_fused_kernel<<<dim3((w + FP_X - 1) / FP_X, (h + FP_Y - 1) / FP_Y), 256, 0, s>>>(f);
    int sw = w, sh = h;
    for (int L = 1; L < 4 && L < nlevels; L++) {
        sw = (sw + 1) / 2;
        sh = (sh + 1) / 2;
    }
    for (int L = 4; L < nlevels; L++) {
        const int dw = (sw + 1) / 2, dh = (sh + 1) / 2;
        const dim3 grid((dw + RT_X - 1) / RT_X, (dh + RT_Y - 1) / RT_Y);
        pyr_reduce_kernel<false><<<grid, 256, 0, s>>>(levels[L - 1], sw, sh, pitches[L - 1], nullptr, 0, levels[L], dw, dh,
                                                      pitches[L]);
        sw = dw;
        sh = dh;
    }
    return cudaGetLastError();
}
