/* ref_bench.c -- TIMING HARNESS ONLY: the reference's own CPU implementation of the path, timed on the host's cores.
 *
 * oracle/Makefile links this file with the reference's unmodified kernel sources (img_ref.c, img_vx.c, lk_ref.c,
 * lk_vx.c of its src/kern, read where they lie) into oracle/_ref/vtref_bench. bench.py runs it for its reference arm and
 * CPU baseline; nothing of the product calls it.
 *
 * One step is one frame pair of the per-cell flow: the new frame's pyramid (img_u8_to_q6 and img_reduce per level with
 * their edge padding, rows split over the threads as tk_build's team splits them, src/kern/track.c:179, 584-629), then
 * every cell's LK with the forward-backward check (lk_track + lk_flowback, src/kern/lk.h:45-53), the cells taken from
 * an atomic counter by every thread (the reference's own fan-out, src/kern/still.c:116-141, track.c:275-292).
 * The kernels are the reference's plain-C pair (`ref`: img_*_ref, lk_*_ref) or its vector pair (`vx`: img_*_vx,
 * lk_*_vx, which on a host runs the 16-lane model of src/common/vx.h).
 *
 *   vtref_bench FILE [--lk ref|vx] [--pyr ref|vx] [--threads T] [--steps K] [--warmup W] [--every N]
 *               [--interleave R] [--out FILE]
 *
 * FILE holds int32 w, h, levels, ncells, then frame 0 and frame 1 (h rows of w bytes), then ncells float x and ncells
 * float y (level-0 cell centres). --every N tracks every Nth cell. --interleave R times R rounds of the `ref` and `vx`
 * kernels alternately (the reference's median-of-interleaved method, src/card/m2_gate.c:193-228) instead of K steps of
 * one pair. Prints one JSON line. */
#define _GNU_SOURCE
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "img.h"
#include "lk.h"
#include "plane.h"

#define MAXL 6
#define MAXT 256

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

struct pyr {
    struct vt_plane l[MAXL];
    int levels;
};

static struct pyr new_pyr(int w, int h, int levels)
{
    struct pyr p;
    p.levels = levels;
    for (int i = 0; i < levels; i++) {
        void *m = aligned_alloc(64, (plane_bytes(w, h) + 63) & ~(size_t)63);
        if (!m)
            exit(2);
        memset(m, 0, plane_bytes(w, h));
        p.l[i] = plane_at(m, w, h);
        w = (w + 1) / 2;
        h = (h + 1) / 2;
    }
    return p;
}

/* the team: fn(arg, tid, n) on every thread, then join */
typedef void (*team_fn)(void *arg, int tid, int n);
struct team_job {
    team_fn fn;
    void *arg;
    int tid, n;
};
static void *team_main(void *p)
{
    struct team_job *j = p;
    j->fn(j->arg, j->tid, j->n);
    return NULL;
}
static void team_run(team_fn fn, void *arg, int n)
{
    pthread_t th[MAXT];
    struct team_job jobs[MAXT];
    for (int t = 1; t < n; t++) {
        jobs[t] = (struct team_job){fn, arg, t, n};
        pthread_create(&th[t], NULL, team_main, &jobs[t]);
    }
    fn(arg, 0, n);
    for (int t = 1; t < n; t++)
        pthread_join(th[t], NULL);
}

static int row_of(int rows, int tid, int n) { return (int)((long)rows * tid / n); }

struct build_arg {
    const struct pyr *p;
    const uint8_t *img;
    int stride, level, vx;
};

static void build_rows(void *a_, int tid, int n)
{
    const struct build_arg *a = a_;
    const struct vt_plane *d = &a->p->l[a->level];
    const int y0 = row_of(d->h, tid, n), y1 = row_of(d->h, tid + 1, n);
    if (a->level == 0) {
        if (a->vx)
            img_u8_to_q6_vx(d, a->img, a->stride, y0, y1);
        else
            img_u8_to_q6_ref(d, a->img, a->stride, y0, y1);
    } else {
        if (a->vx)
            img_reduce_vx(d, &a->p->l[a->level - 1], y0, y1);
        else
            img_reduce_ref(d, &a->p->l[a->level - 1], y0, y1);
    }
    img_pad_rows(d, y0, y1);
}

static void build(const struct pyr *p, const uint8_t *img, int stride, int vx, int threads)
{
    for (int L = 0; L < p->levels; L++) {
        struct build_arg a = {p, img, stride, L, vx};
        team_run(build_rows, &a, threads);
        img_pad_tb(&p->l[L]);
    }
}

struct lk_arg {
    const struct pyr *I, *J;
    const float *xs, *ys;
    int ncells, every, vx;
    struct lk_cfg cfg;
    struct lk_out *out;
    int next; /* the cell counter */
    void *tiles[MAXT];
};

static void lk_cells(void *a_, int tid, int n)
{
    struct lk_arg *a = a_;
    (void)n;
    void *tile = a->tiles[tid];
    const int top = a->I->levels - 1;
    for (;;) {
        const int k = __atomic_fetch_add(&a->next, 1, __ATOMIC_RELAXED);
        const int i = k * a->every;
        if (i >= a->ncells)
            break;
        struct lk_out *o = &a->out[i];
        if (a->vx) {
            lk_track_vx(a->I->l, a->J->l, top, &a->cfg, a->xs[i], a->ys[i], 0.0f, 0.0f, o, tile);
            lk_flowback_vx(a->I->l, a->J->l, top, &a->cfg, a->xs[i], a->ys[i], 0.5f, o, tile);
        } else {
            lk_track_ref(a->I->l, a->J->l, top, &a->cfg, a->xs[i], a->ys[i], 0.0f, 0.0f, o, tile);
            lk_flowback_ref(a->I->l, a->J->l, top, &a->cfg, a->xs[i], a->ys[i], 0.5f, o, tile);
        }
    }
}

static int cmp_dbl(const void *a, const void *b)
{
    const double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

static double median(double *v, int n)
{
    qsort(v, (size_t)n, sizeof *v, cmp_dbl);
    return n ? v[n / 2] : 0.0;
}

int main(int argc, char **argv)
{
    if (argc < 2) {
        fprintf(stderr, "usage: %s FILE [--lk ref|vx] [--pyr ref|vx] [--threads T] [--steps K] [--warmup W] "
                        "[--every N] [--interleave R] [--out FILE]\n", argv[0]);
        return 2;
    }
    int lk_vx = 0, pyr_vx = 1, threads = 1, steps = 5, warmup = 1, every = 1, inter = 0;
    const char *out_path = NULL;
    for (int i = 2; i + 1 < argc; i += 2) {
        if (!strcmp(argv[i], "--lk"))
            lk_vx = !strcmp(argv[i + 1], "vx");
        else if (!strcmp(argv[i], "--pyr"))
            pyr_vx = !strcmp(argv[i + 1], "vx");
        else if (!strcmp(argv[i], "--threads"))
            threads = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "--steps"))
            steps = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "--warmup"))
            warmup = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "--every"))
            every = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "--interleave"))
            inter = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "--out"))
            out_path = argv[i + 1];
    }
    if (threads < 1 || threads > MAXT || steps < 1 || every < 1 || warmup < 0)
        return 2;
    FILE *f = fopen(argv[1], "rb");
    if (!f)
        return 2;
    int32_t hd[4];
    if (fread(hd, sizeof hd, 1, f) != 1)
        return 2;
    const int w = hd[0], h = hd[1], levels = hd[2], ncells = hd[3];
    if (w < 32 || h < 32 || levels < 1 || levels > MAXL || ncells < 1)
        return 2;
    const int stride = (w + 15) & ~15; /* the reference's frames: rows a multiple of 16 bytes (src/kern/img.h) */
    uint8_t *f0 = aligned_alloc(64, (size_t)stride * h), *f1 = aligned_alloc(64, (size_t)stride * h);
    float *xs = malloc(sizeof(float) * (size_t)ncells), *ys = malloc(sizeof(float) * (size_t)ncells);
    struct lk_out *out = calloc((size_t)ncells, sizeof *out);
    if (!f0 || !f1 || !xs || !ys || !out)
        return 2;
    for (int y = 0; y < h; y++)
        if (fread(f0 + (size_t)y * stride, 1, (size_t)w, f) != (size_t)w)
            return 2;
    for (int y = 0; y < h; y++)
        if (fread(f1 + (size_t)y * stride, 1, (size_t)w, f) != (size_t)w)
            return 2;
    if (fread(xs, sizeof(float), (size_t)ncells, f) != (size_t)ncells ||
        fread(ys, sizeof(float), (size_t)ncells, f) != (size_t)ncells)
        return 2;
    fclose(f);
    const struct pyr P0 = new_pyr(w, h, levels), P1 = new_pyr(w, h, levels);
    build(&P0, f0, stride, pyr_vx, threads);
    struct lk_arg a;
    memset(&a, 0, sizeof a);
    a.I = &P0;
    a.J = &P1;
    a.xs = xs;
    a.ys = ys;
    a.ncells = ncells;
    a.every = every;
    a.cfg = (struct lk_cfg){.w = 21, .h = 21, .max_iter = 10, .eps = 0.01f, .min_eig = 0.1f, .max_residual = 25.0f};
    a.out = out;
    for (int t = 0; t < threads; t++) {
        a.tiles[t] = aligned_alloc(64, (lk_tile_bytes() + 63) & ~(size_t)63);
        if (!a.tiles[t])
            return 2;
    }
    const int tracked = (ncells + every - 1) / every;
    if (inter > 0) {
        /* R rounds of ref then vx, each a whole step (pyramid + LK); the medians of each */
        double *tr = malloc(sizeof(double) * (size_t)inter), *tv = malloc(sizeof(double) * (size_t)inter);
        for (int r = 0; r < inter; r++)
            for (int v = 0; v < 2; v++) {
                const double t0 = now_s();
                build(&P1, f1, stride, v, threads);
                a.vx = v;
                a.next = 0;
                team_run(lk_cells, &a, threads);
                (v ? tv : tr)[r] = now_s() - t0;
            }
        const double mr = median(tr, inter), mv = median(tv, inter);
        printf("{\"cells_per_step\": %d, \"threads\": %d, \"rounds\": %d, \"ref_median_s\": %.6f, \"vx_median_s\": %.6f, "
               "\"ref_cells_per_s\": %.3f, \"vx_cells_per_s\": %.3f}\n",
               tracked, threads, inter, mr, mv, tracked / mr, tracked / mv);
        return 0;
    }
    a.vx = lk_vx;
    for (int k = 0; k < warmup; k++) {
        build(&P1, f1, stride, pyr_vx, threads);
        a.next = 0;
        team_run(lk_cells, &a, threads);
    }
    double *ts = malloc(sizeof(double) * (size_t)steps), total = 0.0;
    for (int k = 0; k < steps; k++) {
        const double t0 = now_s();
        build(&P1, f1, stride, pyr_vx, threads);
        a.next = 0;
        team_run(lk_cells, &a, threads);
        ts[k] = now_s() - t0;
        total += ts[k];
    }
    if (out_path) {
        FILE *o = fopen(out_path, "wb");
        if (!o || fwrite(out, sizeof *out, (size_t)ncells, o) != (size_t)ncells)
            return 2;
        fclose(o);
    }
    printf("{\"cells_per_step\": %d, \"threads\": %d, \"steps\": %d, \"total_s\": %.6f, \"median_s\": %.6f, "
           "\"cells_per_s\": %.3f, \"lk\": \"%s\", \"pyr\": \"%s\"}\n",
           tracked, threads, steps, total, median(ts, steps), tracked * steps / total, lk_vx ? "vx" : "ref",
           pyr_vx ? "vx" : "ref");
    return 0;
}
