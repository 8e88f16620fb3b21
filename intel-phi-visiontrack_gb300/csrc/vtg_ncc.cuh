/* vtg_ncc.cuh -- what the appearance search's kernels share (ncc.cu, ncc_tc.cu) and the C ABI (api_ncc.cu). */
#ifndef VTG_NCC_CUH
#define VTG_NCC_CUH

#include <math.h>

#include "vtg_internal.cuh"

#define NCC_CELL 16 /* SEARCH_CELL, src/kern/track.c:61: corners to a cell of the map */
#define NCC_TOP 8   /* SEARCH_TOP, src/kern/track.c:62: cells looked at again in half pixels */
#define NCC_HALF_MAX (NCC_TOP * 65 * 65) /* half-pixel scores of the candidates at the largest step (16), with
                                          * the ring around each window */

/* One search: the plane, the template and the clamped window of corners. */
struct NccPrm {
    int w, h;        /* the plane */
    int tw, th, n;   /* template, n = tw th */
    float norm;      /* sum of the template's squares */
    float sum_t;     /* sum of the template as the tensor-core map multiplies it (its rounded values) */
    int x0, x1, y0, y1, step;
    int ccols, crows; /* the map's cells */
    /* the near-blank rule on exact integers: n var <= nthr, 16 n var <= nthr16 (half pixels) */
    long long nthr, nthr16;
    float rnorm; /* sqrt(n / norm): the tensor-core map's factor is rnorm / sqrt(n var) */
};

/* nthr = floor(n norm / 16) and nthr16 = floor(n norm): n norm is exact in double (n <= 2^14, norm an F32), so an
 * integer n var compares with them exactly as with n norm / 16 itself, and no kernel needs FP64 for the rule. */
static inline void ncc_thresholds(NccPrm &p)
{
    const double nn = (double)p.n * (double)p.norm;
    p.nthr = (long long)floor(nn * 0.0625);
    p.nthr16 = (long long)floor(nn);
    p.rnorm = p.norm > 0.0f ? (float)sqrt((double)p.n / (double)p.norm) : 0.0f;
}

/* Scratch of a search context, in device memory. */
struct NccScratch {
    long long *S1, *S2; /* integral images of J and J^2, (h + 1) rows of tp */
    int tp;
    float *map_v;
    int *map_x, *map_y;
    int *top, *ntop;
    float *half;          /* the candidates' half-pixel scores: NCC_TOP x (2 around + 3)^2, around <= 2 x 16 - 1 */
    const uint16_t *band; /* the template band for the tensor-core map (ncc_tc.cu), NULL if unset */
    int *err;             /* device status word: nonzero when a bounded wait gave up */
    /* the tensor-core map's own scratch: the 16-bit picture (shifted so a tile's row starts 16-byte aligned), each
     * corner's normalisation factor, and one 64-bit (score, corner) word per cell */
    uint16_t *conv;
    size_t conv_elems;
    float *fac;
    size_t fac_elems;
    unsigned long long *cellw;
    /* the top-8 pass's per-CTA lists (NCC_TOP keys a CTA, ncc_top_ctas(cells) CTAs) and two arrival counters, one for
     * it and one for the half-pixel pass: zero between searches, each reset by the CTA that arrives last */
    unsigned long long *topblk;
    int topblk_lists; /* lists topblk holds */
    unsigned *arrive;
    /* vtg_search_profile: events recorded just before and just after the map kernel (NULL: none) */
    cudaEvent_t map_ev0, map_ev1;
};

/* The top-8 pass: NCC_TOPB_THREADS threads a CTA, NCC_TOPB_PER cells a thread; it needs ncc_top_ctas(cells) lists. */
#define NCC_TOPB_THREADS 256
#define NCC_TOPB_PER 4
static inline int ncc_top_ctas(int cells) { return (cells + NCC_TOPB_THREADS * NCC_TOPB_PER - 1) / (NCC_TOPB_THREADS * NCC_TOPB_PER); }

/* A cell of the tensor-core map from its 64-bit word (ordered score, inverted scan index): value and corner, or -2 and
 * the cell's origin where no corner was scored (the F32 map's convention). */
__device__ __forceinline__ void ncc_cell_decode(const NccPrm &p, int cell, unsigned long long w, float &v, int &x, int &y)
{
    const int cx0 = p.x0 + (cell % p.ccols) * NCC_CELL, cy0 = p.y0 + (cell / p.ccols) * NCC_CELL;
    const int per = NCC_CELL / p.step;
    if (w == 0ull) {
        v = -2.0f;
        x = cx0;
        y = cy0;
        return;
    }
    unsigned u = (unsigned)(w >> 32);
    u = (u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u;
    const int key = (int)(0xFFFFFFFFu - (unsigned)(w & 0xFFFFFFFFull));
    v = __uint_as_float(u);
    x = cx0 + (key % per) * p.step;
    y = cy0 + (key / per) * p.step;
}

/* ---- the eight best cells: keys, a register list, a warp's merge ---- */

/* A cell's key: its value in ascending float order as unsigned, then the inverted cell index (the earlier cell first
 * among equal values); 0 for no value (-2). */
__device__ __forceinline__ unsigned long long top_key(float v, int i)
{
    if (!(v > -2.0f))
        return 0ull;
    unsigned u = __float_as_uint(v);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u); /* ascending float order as unsigned */
    return ((unsigned long long)u << 32) | (unsigned long long)(0xFFFFFFFFu - (unsigned)i);
}

/* k into the descending list t, keeping its NCC_TOP largest: one compare-exchange a place, unrolled, so t stays in
 * registers. Keys are distinct (the cell index is in their low bits). */
__device__ __forceinline__ void top_insert(unsigned long long (&t)[NCC_TOP], unsigned long long k)
{
    if (k <= t[NCC_TOP - 1])
        return;
#pragma unroll
    for (int j = 0; j < NCC_TOP; j++) {
        const unsigned long long hi = t[j] > k ? t[j] : k;
        k = t[j] > k ? k : t[j];
        t[j] = hi;
    }
}

/* Two descending lists' best eight: max(a_k, b_(7 - k)) is their top eight as a bitonic sequence, which three
 * compare-exchange layers sort. Across the warp by xor partners, so every lane ends with the warp's best eight. */
__device__ __forceinline__ void top_warp_merge(unsigned long long (&t)[NCC_TOP])
{
#pragma unroll 1
    for (int sh = 1; sh < 32; sh <<= 1) {
        unsigned long long c[NCC_TOP];
#pragma unroll
        for (int k = 0; k < NCC_TOP; k++) {
            const unsigned long long o = __shfl_xor_sync(VTG_FULL, t[NCC_TOP - 1 - k], sh);
            c[k] = t[k] > o ? t[k] : o;
        }
#pragma unroll
        for (int d = NCC_TOP / 2; d >= 1; d >>= 1)
#pragma unroll
            for (int k = 0; k < NCC_TOP; k++)
                if ((k & d) == 0) {
                    const unsigned long long hi = c[k] > c[k + d] ? c[k] : c[k + d];
                    const unsigned long long lo = c[k] > c[k + d] ? c[k + d] : c[k];
                    c[k] = hi;
                    c[k + d] = lo;
                }
#pragma unroll
        for (int k = 0; k < NCC_TOP; k++)
            t[k] = c[k];
    }
}

/* The last CTA of a top-8 pass, its warp 0: the best eight of the n CTAs' lists in blk (read through L2) into top /
 * ntop, and the arrival counter back to zero. */
__device__ __forceinline__ void ncc_top_final(const unsigned long long *blk, int n, unsigned *arrive, int *top, int *ntop)
{
    const int lane = threadIdx.x & 31;
    unsigned long long t[NCC_TOP];
#pragma unroll
    for (int k = 0; k < NCC_TOP; k++)
        t[k] = 0ull;
    for (int b = lane; b < n; b += 32)
#pragma unroll
        for (int k = 0; k < NCC_TOP; k++)
            top_insert(t, __ldcg(blk + (size_t)b * NCC_TOP + k));
    top_warp_merge(t);
    if (lane == 0) {
        int c = 0;
        for (int k = 0; k < NCC_TOP; k++) {
            if (t[k] == 0ull)
                break;
            top[c++] = (int)(0xFFFFFFFFu - (unsigned)(t[k] & 0xFFFFFFFFull));
        }
        *ntop = c;
        *arrive = 0u;
    }
}

/* Elements of the tensor-core map's scratch for planes up to max_w x max_h and templates up to max_tw x max_th. */
size_t vtg_ncc_conv_elems(int max_w, int max_h, int max_th);
size_t vtg_ncc_fac_elems(int max_w, int max_h);

/* The top-8 pass on its own launch: over map_v, or (words) over the tensor-core map's cell words, which it decodes;
 * with pdl as a programmatic dependent of the kernel before it. */
cudaError_t vtg_launch_ncc_top(const NccPrm &p, const NccScratch &s, bool words, cudaStream_t st, bool pdl);
cudaError_t vtg_launch_ncc(const void *plane, int pitch, int plane_type, const float *app, const NccPrm &p,
                           const NccScratch &s, int map_kind, vtg_found *out, cudaStream_t st);
cudaError_t vtg_launch_ncc_corners(const void *plane, int pitch, int plane_type, const float *app, const NccPrm &p,
                                   int count, const int *xs, const int *ys, float *out, cudaStream_t st);
/* The tensor-core map (ncc_tc.cu): the same map_v / map_x / map_y as ncc_map_f32, products in BF16 or FP16. */
cudaError_t vtg_launch_ncc_map_tc(const void *plane, int pitch, int elem_bytes, const NccPrm &p, const NccScratch &s,
                                  int kind, cudaStream_t st);
/* Builds the template band for the tensor-core map from a zero-mean template. */
cudaError_t vtg_launch_ncc_band(const float *app, int tw, int th, int kind, uint16_t *band, float *sum_t, cudaStream_t st);
size_t vtg_ncc_band_bytes(int tw, int th);

#endif
