/* dropin_shim.c -- TEST INFRASTRUCTURE ONLY: the reference's own m2_ref program (src/host/m2_ref.c, unmodified) run on
 * the GPU through the library's reference-signature entry points (include/vtg_compat.h), each call checked against
 * the reference's own kernel on the same arguments.
 *
 * oracle/Makefile compiles m2_ref.c with
 *     -Dimg_u8_to_q6_vx=vtg_dropin_u8_to_q6 -Dimg_reduce_vx=vtg_dropin_reduce -Dlk_track_vx=vtg_dropin_lk_track
 * and links this file, the reference's kernels (compiled as they are) and libvtg.so. So every pyramid row and every
 * LK track m2_ref asks for is computed by img_u8_to_q6_cuda / img_reduce_cuda / lk_track_cuda, and its result is what
 * m2_ref hashes and prints. Beside each call the shim runs the reference's _vx kernel on a copy and keeps score:
 * pyramid rows whose bits differ, and for LK the points both call good, the status agreement and the largest flow
 * difference. At exit it prints one line on stderr:
 *     dropin rows R rows_differ D points P both_ok B status_agree S max_err_px E compat_errors C */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "img.h"
#include "lk.h"
#include "plane.h"

#include "vtg_compat.h"

static long g_rows, g_rows_differ, g_points, g_both_ok, g_status_agree, g_compat_err;
static double g_max_err;

static void report(void)
{
    fprintf(stderr, "dropin rows %ld rows_differ %ld points %ld both_ok %ld status_agree %ld max_err_px %.9f "
                    "compat_errors %ld\n",
            g_rows, g_rows_differ, g_points, g_both_ok, g_status_agree, g_max_err, g_compat_err);
}

static void once(void)
{
    static int done;
    if (!done) {
        done = 1;
        atexit(report);
    }
}

static const struct vtg_ref_plane *as_vtg(const struct vt_plane *p) { return (const struct vtg_ref_plane *)p; }

/* a plane of the same size as `like`, its rows y0 .. y1 - 1 copied from `src` */
static struct vt_plane scratch_like(const struct vt_plane *like)
{
    void *m = aligned_alloc(64, (plane_bytes(like->w, like->h) + 63) & ~(size_t)63);
    if (!m)
        exit(3);
    memset(m, 0, plane_bytes(like->w, like->h));
    return plane_at(m, like->w, like->h);
}

static void free_scratch(struct vt_plane *p) { free(p->p - (size_t)p->stride * VT_PAD_Y - VT_PAD_X); }

static void compare_rows(const struct vt_plane *a, const struct vt_plane *b, int y0, int y1)
{
    for (int y = y0; y < y1; y++) {
        g_rows++;
        g_rows_differ += memcmp(plane_row(a, y), plane_row(b, y), sizeof(float) * (size_t)a->w) != 0;
    }
}

void vtg_dropin_u8_to_q6(const struct vt_plane *dst, const uint8_t *src, int src_stride, int y0, int y1)
{
    once();
    img_u8_to_q6_cuda(as_vtg(dst), src, src_stride, y0, y1);
    g_compat_err += vtg_compat_error() != 0;
    struct vt_plane r = scratch_like(dst);
    img_u8_to_q6_vx(&r, src, src_stride, y0, y1);
    compare_rows(dst, &r, y0, y1);
    free_scratch(&r);
}

void vtg_dropin_reduce(const struct vt_plane *dst, const struct vt_plane *src, int y0, int y1)
{
    once();
    img_reduce_cuda(as_vtg(dst), as_vtg(src), y0, y1);
    g_compat_err += vtg_compat_error() != 0;
    struct vt_plane r = scratch_like(dst);
    img_reduce_vx(&r, src, y0, y1);
    compare_rows(dst, &r, y0, y1);
    free_scratch(&r);
}

void vtg_dropin_lk_track(const struct vt_plane *I, const struct vt_plane *J, int top, const struct lk_cfg *c, float x,
                         float y, float gx, float gy, struct lk_out *o, void *tile)
{
    once();
    lk_track_cuda(as_vtg(I), as_vtg(J), top, (const struct vtg_ref_lk_cfg *)c, x, y, gx, gy, (struct vtg_lk_out *)o,
                  tile);
    g_compat_err += vtg_compat_error() != 0;
    struct lk_out r;
    lk_track_vx(I, J, top, c, x, y, gx, gy, &r, tile);
    g_points++;
    g_status_agree += r.status == o->status;
    if (r.status == 0 && o->status == 0) {
        g_both_ok++;
        const double e = fmax(fabs((double)r.x - (double)o->x), fabs((double)r.y - (double)o->y));
        g_max_err = e > g_max_err ? e : g_max_err;
    }
}
