/* vtg_compat.h -- libvtg behind the reference's own kernel signatures.
 *
 * The reference reaches its hot path through kernel pairs of identical signatures, picked per frame by
 * enum vt_algorithm: img_u8_to_q6_{ref,vx}, img_reduce_{ref,vx} (with img_norm, img_minmax and img_gauss5 for
 * tk_build's optional steps, and img_sobel / img_absdiff beside them), lk_track_{ref,vx}, lk_flowback_{ref,vx},
 * lk_tile_bytes, still_vectors and tk_correlate (src/kern/img.h:17-45, src/kern/lk.h:42-53, src/kern/still.h:37,
 * src/kern/track.h:59; the pick: src/kern/track.c:214, src/common/vt_proto.h:156). The functions here are the third
 * member of each pair, with a _cuda suffix: the same arguments with the same meaning, computed on the GPU. A
 * VT_ALG_CUDA branch calls them where the reference calls its _vx kernels today.
 *
 * Planes are the reference's struct vt_plane (src/kern/plane.h:20-24): `p` is pixel (0, 0) of F32 Q6 values, rows
 * `stride` floats apart. struct vtg_ref_plane has that layout under a name of its own, so this header and the
 * reference's plane.h can be included together; the reference passes its planes with a cast. A plane may be in host
 * memory (staged through device memory on every call) or in device or managed memory (used in place). Reads past
 * the edges are clamped to the edge, which is what the reference's replicated padding gives, so padding is not needed;
 * outputs are written inside the plane only, and the caller pads them as before (img_pad_rows / img_pad_tb).
 *
 * Every call is synchronous: its outputs are in place when it returns. Calls from many threads are serialised. The
 * batched entry points of vtg.h are the fast path; these exist so the reference's callers run unchanged.
 *
 * A call that cannot run (no GPU, a CUDA error, an argument out of range such as a patch wider than VTG_MAX_PATCH_W)
 * leaves image outputs untouched, marks an LK result VTG_LK_OUT (no measurement is invented, as lk.h says), returns
 * -1 from tk_correlate_cuda and 0 corners from detect_run_cuda, and records its status for vtg_compat_error. */
#ifndef VTG_COMPAT_H
#define VTG_COMPAT_H

#include <stddef.h>
#include <stdint.h>

#include "vtg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* struct vt_plane, src/kern/plane.h:20-24 */
struct vtg_ref_plane {
    float *p;   /* pixel (0, 0) */
    int w, h;
    int stride; /* floats a row */
};

/* struct lk_cfg, src/kern/lk.h:24-31 (prefetch changes timing only; it is ignored here) */
struct vtg_ref_lk_cfg {
    int w, h;
    int max_iter;
    float eps;
    float min_eig;
    float max_residual;
    int prefetch;
};

/* lk_tile_bytes (src/kern/lk.h:42-43): the per-thread scratch the caller allocates. The GPU path needs none; one
 * 64-byte line keeps callers that allocate it working. */
size_t lk_tile_bytes_cuda(void);

/* img_u8_to_q6_ref / _vx (src/kern/img.h:17-18, img_ref.c:32-40): rows y0 .. y1 - 1 of dst = src x 64. src holds
 * dst->h rows of dst->w bytes, src_stride apart. */
void img_u8_to_q6_cuda(const struct vtg_ref_plane *dst, const uint8_t *src, int src_stride, int y0, int y1);

/* img_reduce_ref / _vx (src/kern/img.h:30-33, img_ref.c:98-114): rows y0 .. y1 - 1 of dst, which is
 * (src->w + 1) / 2 x (src->h + 1) / 2, from the 5 x 5 binomial of src at every second pixel, (h + 128) >> 8. */
void img_reduce_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *src, int y0, int y1);

/* The rest of img.h's kernels, which tk_build's optional steps (src/kern/track.c:600-622) and the M1 gate
 * (src/card/m1_gate.c:182-210) run. dst and src have the same size; rows y0 .. y1 - 1 are written. Planes hold whole
 * numbers, as every plane of the reference does. */
/* img_norm_ref / _vx (img.h:20-22, img_ref.c:42-55): dst = clamp(rint(src x gain_offset[0] + gain_offset[1]),
 * 0, 16320), rounded once from the exact value as img_norm_vx does (img_norm_ref's x87 sum rounds the same value
 * whenever that sum is exact, as it is for tk_build's gains). */
void img_norm_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *src, const float *gain_offset, int y0,
                   int y1);
/* img_minmax_ref / _vx (img.h:24-26, img_ref.c:57-71): out[0] = min, out[1] = max over rows y0 .. y1 - 1. */
void img_minmax_cuda(const struct vtg_ref_plane *src, float *out, int y0, int y1);
/* img_gauss5_ref / _vx (img.h:28-30, img_ref.c:83-96): the 5 x 5 binomial at every pixel, (h + 128) >> 8. */
void img_gauss5_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *src, int y0, int y1);
/* img_sobel_ref / _vx (img.h:40-41, img_ref.c:116-127): the 3 x 3 Sobel x into ix, y into iy. */
void img_sobel_cuda(const struct vtg_ref_plane *ix, const struct vtg_ref_plane *iy, const struct vtg_ref_plane *src,
                    int y0, int y1);
/* img_absdiff_ref / _vx (img.h:44-45, img_ref.c:129-137): dst = |a - b|. */
void img_absdiff_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *a, const struct vtg_ref_plane *b,
                      int y0, int y1);

/* lk_track_ref / _vx (src/kern/lk.h:45-47): tracks (x, y) from pyramid I to pyramid J (planes I[0 .. top],
 * J[0 .. top]), starting at level top with guess (gx, gy) in level-0 pixels. `tile` is not used. */
void lk_track_cuda(const struct vtg_ref_plane *I, const struct vtg_ref_plane *J, int top, const struct vtg_ref_lk_cfg *c,
                   float x, float y, float gx, float gy, struct vtg_lk_out *o, void *tile);

/* lk_flowback_ref / _vx (src/kern/lk.h:49-53, lk_driver.inc:111-121): when o has no status, tracks o's estimate back
 * from J to I from minus the found flow, and sets VTG_LK_FLOWBACK when the round trip fails or misses (x, y) by more
 * than max_fb pixels. */
void lk_flowback_cuda(const struct vtg_ref_plane *I, const struct vtg_ref_plane *J, int top,
                      const struct vtg_ref_lk_cfg *c, float x, float y, float max_fb, struct vtg_lk_out *o, void *tile);

/* still_vectors (src/kern/still.h:37, still.c:116-141) over the fields of its struct still, which is private to
 * still.c: every cell of the 16 x 8 grid over `cur`, its centre clamped to where the patch fits, tracked from the
 * running mean to cur on one level with the forward-backward check, into cells[] (struct vt_cell). The GPU does every
 * cell on the call with tid 0; the team's other threads return at once. */
void still_vectors_cuda(const struct vtg_ref_plane *mean, const struct vtg_ref_plane *cur,
                        const struct vtg_ref_lk_cfg *lk, float max_fb, struct vtg_cell *cells, int tid, int n);

/* tk_correlate (src/kern/track.h:59, track.c:184-208): the NCC of a zero-mean 32 x 21 template `app` (sum of squares
 * `norm`) against the plane at corner (x, y); -1 outside the valid corners, 0 for a near-blank window. */
long double tk_correlate_cuda(const struct vtg_ref_plane *pl, const float *app, long double norm, int x, int y);

/* Corner detection as seed_at runs it (src/kern/track.c:988-992): detect_begin (src/kern/detect.h:27), the three
 * stages detect_tensor / detect_response / detect_cells (detect.h:30-32) and detect_finish (detect.h:35) in one call.
 * The same arguments as detect_begin without the job and its scratch, and detect_finish's outputs: up to max (at most
 * 512) corners in x and y (host memory), best first, at least min_dist apart; returns how many, 0 when nothing of the
 * rectangle lies inside the plane's margin. The plane may be in host or device memory. */
int detect_run_cuda(const struct vtg_ref_plane *pl, float rx, float ry, float rw, float rh, int margin, int max,
                    float min_dist, float quality, float *x, float *y);

/* The status of this thread's last call above: VTG_OK or a VTG_E* code. */
int vtg_compat_error(void);

#ifdef __cplusplus
}
#endif

#endif
