/* ref_track_tu.c -- TEST INFRASTRUCTURE ONLY. The reference's src/kern/track.c, compiled unmodified as part of this
 * translation unit (it is included by path, not copied), so that this project's harness can call two of its static
 * functions: search_half (track.c:1615-1647) and search_slot (track.c:1661-1726) with its OP_SEARCH map
 * (track.c:301-329). oracle/Makefile builds this file in place of track.c. */
#include "track.c"

static void *tu_alloc(void *ctx, size_t bytes)
{
    (void)ctx;
    return aligned_alloc(64, (bytes + 63) & ~(size_t)63);
}

static void tu_run(void *ctx, tk_fn fn, void *arg)
{
    (void)ctx;
    fn(arg, 0, 1);
}

/* A tracker holding one plane of whole-number values (w a multiple of 16) as level `level` of its current set, and a
 * 32 x 21 zero-mean appearance in slot 0. */
static struct tracker *tu_tracker(const float *interior, int w, int h, int level, const float *app, float norm)
{
    struct vt_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.width = (uint32_t)(w << level);
    cfg.height = (uint32_t)(h << level);
    cfg.levels = (uint32_t)(level + 1);
    cfg.patch_w = 21;
    cfg.patch_h = 21;
    cfg.max_iter = 10;
    cfg.pipelines = 1;
    struct tracker *t = tk_create(&cfg, 1, 1, tu_alloc, NULL, tu_run, NULL, tu_run, NULL);
    if (!t)
        return NULL;
    t->cur = 0;
    struct vt_plane *pl = &t->pyr[0][0].l[level];
    if (pl->w != w || pl->h != h)
        return NULL;
    for (int y = 0; y < h; y++)
        memcpy(plane_row(pl, y), interior + (size_t)y * w, sizeof(float) * (size_t)w);
    img_pad_rows(pl, 0, h);
    img_pad_tb(pl);
    memcpy(t->app[0].pix, app, sizeof(float) * APP_W * APP_H);
    t->app[0].norm = norm;
    t->app[0].level = level;
    t->app[0].valid = 1;
    return t;
}

/* search_slot over corners [x0, x1] x [y0, y1] at `step`: the found corner in half pixels, its score and the second
 * peak; the per-cell map (cells = its length) into map_v / map_x / map_y. Returns the number of map cells, or -1. */
int ref_search_slot(const float *interior, int w, int h, int level, const float *app, float norm, int x0, int x1, int y0, int y1, int step, int *hx, int *hy, double *ncc, double *second, float *map_v, int *map_x, int *map_y, int max_cells)
{
    struct tracker *t = tu_tracker(interior, w, h, level, app, norm);
    if (!t)
        return -1;
    struct found f;
    search_slot(t, 0, x0, x1, y0, y1, step, VT_ALG_MVEX, &f);
    *hx = f.hx;
    *hy = f.hy;
    *ncc = (double)f.ncc;
    *second = (double)f.second;
    const int cells = t->jt->cell_cols * t->jt->cell_rows;
    for (int i = 0; i < cells && i < max_cells; i++) {
        map_v[i] = t->sc_v[i];
        map_x[i] = t->sc_x[i];
        map_y[i] = t->sc_y[i];
    }
    return cells;
}

/* search_half at each of n half-pixel corners, and peak_offset of the triples (l, c, r) given. */
void ref_search_half(const float *interior, int w, int h, const float *app, float norm, int n, const int *hx, const int *hy, double *out)
{
    struct tracker *t = tu_tracker(interior, w, h, 0, app, norm);
    for (int i = 0; i < n; i++)
        out[i] = t ? (double)search_half(&t->pyr[0][0].l[0], &t->app[0], hx[i], hy[i]) : -3.0;
}

double ref_peak_offset(double l, double c, double r) { return (double)peak_offset((long double)l, (long double)c, (long double)r); }

/* tk_build (track.c:584-629) of one frame (w a multiple of 16, rows w bytes apart) with struct vt_config's contrast and
 * pre_gauss as given, on the x87 kernels (alg 1) or the vector ones (alg 0): every level's w_L x h_L values, level 0
 * first, into out. Returns 0, or -1 when the tracker cannot be made. */
int ref_tk_build(const uint8_t *frame, int w, int h, int levels, int contrast, int pre_gauss, int alg, float *out)
{
    struct vt_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.width = (uint32_t)w;
    cfg.height = (uint32_t)h;
    cfg.levels = (uint32_t)levels;
    cfg.patch_w = 21;
    cfg.patch_h = 21;
    cfg.max_iter = 10;
    cfg.pipelines = 1;
    cfg.contrast = (uint32_t)contrast;
    cfg.pre_gauss = (uint32_t)pre_gauss;
    struct tracker *t = tk_create(&cfg, 1, 1, tu_alloc, NULL, tu_run, NULL, tu_run, NULL);
    if (!t)
        return -1;
    struct vt_msg m;
    memset(&m, 0, sizeof m);
    m.algorithm = alg ? VT_ALG_X87 : VT_ALG_MVEX;
    tk_build(t, 0, frame, NULL, &m);
    for (int L = 0; L < levels; L++) {
        const struct vt_plane *pl = &t->pyr[0][0].l[L];
        for (int y = 0; y < pl->h; y++) {
            memcpy(out, plane_row(pl, y), sizeof(float) * (size_t)pl->w);
            out += pl->w;
        }
    }
    return 0;
}

/* store_appearance (track.c:935-974) on the pyramid tk_build makes of a frame (w a multiple of 16, rows w bytes apart),
 * for the region centred at (cx, cy) of size rw x rh: the template into pix (32 x 21) and info = norm, fx, fy, level,
 * valid. Returns 0, or -1 when the tracker cannot be made. */
int ref_store_appearance(const uint8_t *frame, int w, int h, int levels, float cx, float cy, float rw, float rh,
                         float *pix, float *info)
{
    struct vt_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.width = (uint32_t)w;
    cfg.height = (uint32_t)h;
    cfg.levels = (uint32_t)levels;
    cfg.patch_w = 21;
    cfg.patch_h = 21;
    cfg.max_iter = 10;
    cfg.pipelines = 1;
    struct tracker *t = tk_create(&cfg, 1, 1, tu_alloc, NULL, tu_run, NULL, tu_run, NULL);
    if (!t)
        return -1;
    struct vt_msg m;
    memset(&m, 0, sizeof m);
    m.algorithm = VT_ALG_MVEX;
    tk_build(t, 0, frame, NULL, &m);
    t->cur = 0;
    t->cx = cx;
    t->cy = cy;
    t->rw = rw;
    t->rh = rh;
    store_appearance(t, 0);
    const struct app_slot *a = &t->app[0];
    if (a->valid)
        memcpy(pix, a->pix, sizeof(float) * APP_W * APP_H);
    info[0] = a->norm;
    info[1] = a->fx;
    info[2] = a->fy;
    info[3] = (float)a->level;
    info[4] = (float)a->valid;
    return 0;
}
