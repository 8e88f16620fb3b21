/* ref_driver.c -- TEST INFRASTRUCTURE ONLY: this project's own harness around the reference's unmodified sources.
 *
 * oracle/Makefile compiles the reference's kernel sources (the C files of src/kern in Lasimeri/Intel-Phi-VisionTrack,
 * read in place) together with this file into oracle/_ref/libvtref.so. The functions here only arrange inputs, call the
 * reference's own public functions (and, through ref_track_tu.c, two static ones of track.c) and copy results out. They
 * are used to pin the oracle restatement (vtg_oracle.c) and to generate the golden fixtures under tests/golden/.
 *
 * The reference's planes are padded F32 (src/kern/plane.h:16-35); here every plane handed in or out is its w x h
 * interior, rows w floats apart. */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "detect.h"
#include "framegen.h"
#include "img.h"
#include "lk.h"
#include "plane.h"
#include "still.h"
#include "track.h"

#define REF_MAX_LEVELS 8

struct ref_pyr {
    int levels;
    struct vt_plane l[REF_MAX_LEVELS];
};

static struct vt_plane new_plane(int w, int h)
{
    void *m = aligned_alloc(64, (plane_bytes(w, h) + 63) & ~(size_t)63);
    memset(m, 0, plane_bytes(w, h));
    return plane_at(m, w, h);
}

static void free_plane(struct vt_plane *pl) { free(pl->p - (size_t)pl->stride * VT_PAD_Y - VT_PAD_X); }

/* tk_build's pyramid with the vector kernels (src/kern/track.c:584-629, OP_U8 and OP_REDUCE of job_main). */
static void build(struct ref_pyr *p, const uint8_t *img, int stride, int w, int h, int levels, int use_ref)
{
    p->levels = levels;
    for (int i = 0; i < levels; i++) {
        p->l[i] = new_plane(w, h);
        w = (w + 1) / 2;
        h = (h + 1) / 2;
    }
    if (use_ref)
        img_u8_to_q6_ref(&p->l[0], img, stride, 0, p->l[0].h);
    else
        img_u8_to_q6_vx(&p->l[0], img, stride, 0, p->l[0].h);
    img_pad_rows(&p->l[0], 0, p->l[0].h);
    img_pad_tb(&p->l[0]);
    for (int i = 1; i < levels; i++) {
        if (use_ref)
            img_reduce_ref(&p->l[i], &p->l[i - 1], 0, p->l[i].h);
        else
            img_reduce_vx(&p->l[i], &p->l[i - 1], 0, p->l[i].h);
        img_pad_rows(&p->l[i], 0, p->l[i].h);
        img_pad_tb(&p->l[i]);
    }
}

static void release(struct ref_pyr *p)
{
    for (int i = 0; i < p->levels; i++)
        free_plane(&p->l[i]);
}

/* The pyramid of one frame: every level's interior, level after level. src rows are stride bytes apart (a multiple
 * of 16, as img.h asks). */
void ref_pyramid(const uint8_t *src, int stride, int w, int h, int levels, int use_ref, float *out)
{
    struct ref_pyr p;
    build(&p, src, stride, w, h, levels, use_ref);
    for (int i = 0; i < levels; i++) {
        for (int y = 0; y < p.l[i].h; y++)
            memcpy(out + (size_t)y * p.l[i].w, plane_row(&p.l[i], y), sizeof(float) * (size_t)p.l[i].w);
        out += (size_t)p.l[i].w * p.l[i].h;
    }
    release(&p);
}

struct ref_team {
    const struct ref_pyr *I, *J;
    const struct lk_cfg *c;
    int top, n, use_ref, base;
    float max_fb;
    const float *xs, *ys, *gxs, *gys;
    struct lk_out *out;
    int next;
};

static void *ref_points_thread(void *arg)
{
    struct ref_team *j = arg;
    void *tile = aligned_alloc(64, (lk_tile_bytes() + 63) & ~(size_t)63);
    for (;;) {
        const int i = __atomic_fetch_add(&j->next, 1, __ATOMIC_RELAXED);
        if (i >= j->n)
            break;
        const float gx = j->gxs ? j->gxs[i] : 0.0f, gy = j->gys ? j->gys[i] : 0.0f;
        if (j->use_ref) {
            lk_track_ref(j->I->l + j->base, j->J->l + j->base, j->top, j->c, j->xs[i], j->ys[i], gx, gy, &j->out[i], tile);
            if (j->max_fb > 0.0f)
                lk_flowback_ref(j->I->l + j->base, j->J->l + j->base, j->top, j->c, j->xs[i], j->ys[i], j->max_fb, &j->out[i], tile);
        } else {
            lk_track_vx(j->I->l + j->base, j->J->l + j->base, j->top, j->c, j->xs[i], j->ys[i], gx, gy, &j->out[i], tile);
            if (j->max_fb > 0.0f)
                lk_flowback_vx(j->I->l + j->base, j->J->l + j->base, j->top, j->c, j->xs[i], j->ys[i], j->max_fb, &j->out[i], tile);
        }
    }
    free(tile);
    return NULL;
}

/* OP_LK of job_main (src/kern/track.c:275-292): every point through lk_track_{vx,ref} and, when max_fb > 0,
 * lk_flowback_{vx,ref}, on a team of threads taking points by an atomic counter. Pyramids are built from the two frames
 * with the vector kernels, as tk_build does; LK runs on the pyramid from level `base` up (points in that level's
 * pixels), as the per-cell flow does at a flow level above 0. */
void ref_lk_points(const uint8_t *f0, const uint8_t *f1, int stride, int w, int h, int levels, int base, int top, int pw, int ph, int max_iter, float eps, float min_eig, float max_residual, float max_fb, int n, const float *xs, const float *ys, const float *gxs, const float *gys, int use_ref, int threads, struct lk_out *out)
{
    struct ref_pyr I, J;
    build(&I, f0, stride, w, h, levels, 0);
    build(&J, f1, stride, w, h, levels, 0);
    const struct lk_cfg c = {.w = pw, .h = ph, .max_iter = max_iter, .eps = eps, .min_eig = min_eig, .max_residual = max_residual, .prefetch = 0};
    struct ref_team j = {.I = &I, .J = &J, .c = &c, .top = top, .n = n, .use_ref = use_ref, .base = base, .max_fb = max_fb, .xs = xs, .ys = ys, .gxs = gxs, .gys = gys, .out = out, .next = 0};
    if (threads <= 1) {
        ref_points_thread(&j);
    } else {
        pthread_t th[64];
        threads = threads > 64 ? 64 : threads;
        for (int i = 0; i < threads; i++)
            pthread_create(&th[i], NULL, ref_points_thread, &j);
        for (int i = 0; i < threads; i++)
            pthread_join(th[i], NULL);
    }
    release(&I);
    release(&J);
}

static void *host_alloc(void *ctx, size_t bytes)
{
    (void)ctx;
    return aligned_alloc(64, (bytes + 63) & ~(size_t)63);
}

/* still_vectors itself (src/kern/still.c:116-141): one frame of the reference's per-cell flow, with the still's mean
 * set to frame f0 (as after its first frame) and f1 the current frame, both at native resolution. cells receives
 * ceil(w / 16) x ceil(h / 8) records. */
int ref_still_vectors(const uint8_t *f0, const uint8_t *f1, int stride, int w, int h, struct vt_cell *cells)
{
    const struct still_cfg sc = {.w = w, .h = h, .avg = 8, .motion_px = 1.0f, .motion_grey = 4.0f, .threads = 1};
    struct still *s = still_create(&sc, host_alloc, NULL);
    if (!s)
        return -1;
    struct ref_pyr A, B;
    build(&A, f0, stride, w, h, 1, 0);
    build(&B, f1, stride, w, h, 1, 0);
    const struct vt_plane *mean = still_mean(s);
    for (int y = -VT_PAD_Y; y < h + VT_PAD_Y; y++)
        memcpy(plane_row(mean, y) - VT_PAD_X, plane_row(&A.l[0], y) - VT_PAD_X, sizeof(float) * (size_t)mean->stride);
    still_vectors(s, &B.l[0], 0, 1);
    const int n = ((w + VT_CELL_W - 1) / VT_CELL_W) * ((h + VT_CELL_H - 1) / VT_CELL_H);
    memcpy(cells, still_cells(s), sizeof(struct vt_cell) * (size_t)n);
    release(&A);
    release(&B);
    return n;
}

/* A padded plane from an interior of whole-number values, its border replicated as img_pad_rows / img_pad_tb do. */
static struct vt_plane plane_from(const float *interior, int w, int h)
{
    struct vt_plane pl = new_plane(w, h);
    for (int y = 0; y < h; y++)
        memcpy(plane_row(&pl, y), interior + (size_t)y * w, sizeof(float) * (size_t)w);
    img_pad_rows(&pl, 0, h);
    img_pad_tb(&pl);
    return pl;
}

/* tk_correlate (src/kern/track.c:208) at each of n corners of a 32 x 21 template. */
void ref_correlate(const float *interior, int w, int h, const float *app, double norm, int n, const int *xs, const int *ys, double *out)
{
    struct vt_plane pl = plane_from(interior, w, h);
    for (int i = 0; i < n; i++)
        out[i] = (double)tk_correlate(&pl, app, (long double)norm, xs[i], ys[i]);
    free_plane(&pl);
}

/* Corner detection as the tracker's seed_at runs it (src/kern/track.c:988-992): detect_begin, the three stages over
 * their whole ranges on one thread, detect_finish. geo gets x0, y0, x1, y1, ax, cols, rows, nv, cell_rows; resp
 * (rows x cols) and cell (cell_rows x nv) get the stages' planes when not NULL. Returns the corners found (-1: the
 * rectangle is empty). */
int ref_detect(const float *interior, int w, int h, float rx, float ry, float rw, float rh, int margin, int max, float min_dist, float quality,
               int *geo, float *resp, float *cell, float *xs, float *ys)
{
    struct vt_plane pl = plane_from(interior, w, h);
    void *scratch = aligned_alloc(64, (detect_scratch_bytes(w, h) + 63) & ~(size_t)63);
    struct detect_job j;
    int n = -1;
    if (detect_begin(&j, &pl, rx, ry, rw, rh, margin, max, min_dist, quality, scratch)) {
        detect_tensor(&j, 0, j.rows + 4);
        detect_response(&j, 0, j.rows);
        detect_cells(&j, 0, j.cell_rows);
        const int g[9] = {j.x0, j.y0, j.x1, j.y1, j.ax, j.cols, j.rows, j.nv, j.cell_rows};
        memcpy(geo, g, sizeof g);
        if (resp)
            memcpy(resp, j.resp, sizeof(float) * (size_t)j.rows * (size_t)j.cols);
        if (cell)
            memcpy(cell, j.cell, sizeof(float) * (size_t)j.nv * (size_t)j.cell_rows);
        n = detect_finish(&j, xs, ys);
    }
    free(scratch);
    free_plane(&pl);
    return n;
}

/* What still_motion fills (src/kern/still.c:262-275), in the layout of the library's struct vtg_still_motion. */
struct ref_still_motion {
    uint32_t cols, rows, tracked, moving;
    float count_mean, drift_u, drift_v, drift_rms, diff_median, diff_limit;
    uint64_t frames;
};

/* The reference's still picture over a sequence of 8-bit frames, in the order m3_ref runs it (src/host/m3_ref.c:
 * 272-283): each frame's Q6 plane, still_vectors unless it is the first frame, still_decide, still_update,
 * still_finish. Per frame: the cells after the decision, still_motion, and still_hash from the FNV basis
 * 0xcbf29ce484222325; after the last frame, the mean's w x h interior. Returns the cells a frame. */
int ref_still_run(const uint8_t *frames, int nframes, int stride, int w, int h, int avg, float motion_px,
                  float motion_grey, struct vt_cell *cells, struct ref_still_motion *motion, uint64_t *hash,
                  float *mean_out)
{
    const struct still_cfg sc = {.w = w, .h = h, .avg = avg, .motion_px = motion_px, .motion_grey = motion_grey, .threads = 1};
    struct still *s = still_create(&sc, host_alloc, NULL);
    if (!s)
        return -1;
    const int n = ((w + VT_CELL_W - 1) / VT_CELL_W) * ((h + VT_CELL_H - 1) / VT_CELL_H);
    for (int f = 0; f < nframes; f++) {
        struct ref_pyr P;
        build(&P, frames + (size_t)f * (size_t)stride * (size_t)h, stride, w, h, 1, 0);
        if (!still_first(s))
            still_vectors(s, &P.l[0], 0, 1);
        still_decide(s);
        still_update(s, &P.l[0], 0, 1);
        still_finish(s);
        memcpy(cells + (size_t)f * (size_t)n, still_cells(s), sizeof(struct vt_cell) * (size_t)n);
        struct vt_motion m;
        memset(&m, 0, sizeof m);
        still_motion(s, &m);
        motion[f] = (struct ref_still_motion){m.cols, m.rows, m.tracked, m.moving, m.count_mean, m.drift_u, m.drift_v,
                                              m.drift_rms, m.diff_median, m.diff_limit, m.frames};
        hash[f] = still_hash(s, 0xcbf29ce484222325ull);
        release(&P);
    }
    const struct vt_plane *mp = still_mean(s);
    for (int y = 0; y < h; y++)
        memcpy(mean_out + (size_t)y * (size_t)w, plane_row(mp, y), sizeof(float) * (size_t)w);
    return n;
}


/* The reference's frame generation between two 8-bit frames, in the order tk_generate_make runs it
 * (src/kern/track.c:847-888, without the tracker): the field's pyramid from the frames' Q6 pyramids (levels 1 ..),
 * fg_hist_section over the nine sections of each frame's field level 1, fg_scene_verdict, then coarsest first
 * fg_search, fg_filter and fg_upscale, fg_mid_vectors, fg_blend, the padding and img_q6_to_u8_vx. Outputs as the
 * oracle's or_framegen (fields level by level, up of the top level zero). Returns the verdict, or -1. */
int ref_framegen(const uint8_t *fa, const uint8_t *fb, int stride, int w, int h, struct fg_vec *raw_out,
                 struct fg_vec *fil_out, struct fg_vec *up_out, struct fg_vec *mid_out, float *out, uint8_t *pic)
{
    int lw = (w + 1) / 2, lh = (h + 1) / 2, levels = 0;
    for (int i = 0; i < FG_MAX_LEVELS && lw >= 16 && lh >= 16; i++) {
        levels++;
        lw = (lw + 1) / 2;
        lh = (lh + 1) / 2;
    }
    if (levels < 2)
        return -1;
    struct ref_pyr A, B;
    build(&A, fa, stride, w, h, levels + 1, 0);
    build(&B, fb, stride, w, h, levels + 1, 0);
    struct fg_job j;
    memset(&j, 0, sizeof j);
    const size_t bytes = fg_bytes((w + 1) / 2, (h + 1) / 2, levels);
    void *mem = aligned_alloc(64, (bytes + 63) & ~(size_t)63);
    memset(mem, 0, bytes);
    fg_init(&j, mem, (w + 1) / 2, (h + 1) / 2, levels);
    for (int i = 0; i < levels; i++) {
        j.a[i] = A.l[i + 1];
        j.b[i] = B.l[i + 1];
    }
    j.a0 = A.l[0];
    j.b0 = B.l[0];
    j.out = new_plane(w, h);
    for (int s = 0; s < FG_SECTIONS; s++) {
        fg_hist_section(&j.a[1], j.hist_a, s);
        fg_hist_section(&j.b[1], j.hist_b, s);
    }
    j.scene_changed = fg_scene_verdict(&j);
    for (int L = levels - 1; L >= 0; L--) {
        fg_search(&j, L, 0, j.raw[L].w * j.raw[L].h);
        fg_filter(&j, L, 0, j.fil[L].w * j.fil[L].h);
        if (L > 0)
            fg_upscale(&j, L, 0, j.up[L - 1].w * j.up[L - 1].h);
    }
    fg_mid_vectors(&j, 0, j.mid.w * j.mid.h);
    fg_blend(&j, 0, fg_tiles(&j));
    img_pad_rows(&j.out, 0, h);
    img_pad_tb(&j.out);
    uint8_t *buf = malloc((size_t)w * (size_t)h + 64);
    img_q6_to_u8_vx(&j.out, buf, 0, h);
    size_t off = 0;
    for (int L = 0; L < levels; L++) {
        const size_t n = (size_t)j.raw[L].w * (size_t)j.raw[L].h;
        memcpy(raw_out + off, j.raw[L].v, n * sizeof(struct fg_vec));
        memcpy(fil_out + off, j.fil[L].v, n * sizeof(struct fg_vec));
        memcpy(up_out + off, j.up[L].v, n * sizeof(struct fg_vec));
        off += n;
    }
    memcpy(mid_out, j.mid.v, (size_t)j.mid.w * (size_t)j.mid.h * sizeof(struct fg_vec));
    for (int y = 0; y < h; y++)
        memcpy(out + (size_t)y * (size_t)w, plane_row(&j.out, y), sizeof(float) * (size_t)w);
    memcpy(pic, buf, (size_t)w * (size_t)h);
    const int scene = j.scene_changed;
    free(buf);
    free_plane(&j.out);
    free(mem);
    release(&A);
    release(&B);
    return scene;
}
