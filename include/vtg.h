/* vtg.h -- the C ABI of libvtg: the sparse pyramidal Lucas-Kanade path of Lasimeri/Intel-Phi-VisionTrack on one GB300
 * (sm_103a), for C host code.
 *
 * Plain C types only: pointers, sizes, ints and floats. CUDA streams are passed as `void *` (a cudaStream_t, or NULL for
 * the library's own stream of the context). Every entry point returns an int status (VTG_OK = 0, negative on error);
 * none traps, and no device wait is unbounded.
 *
 * Reference interfaces each entry point replaces are cited as path:line inside the reference tree. */
#ifndef VTG_H
#define VTG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define VTG_MAX_LEVELS 6 /* VT_MAX_LEVELS, src/common/vt_proto.h:59 */
#define VTG_MAX_PATCH_W 29
#define VTG_MAX_PATCH_H 31 /* LK_MAX_H, src/kern/lk.h:19 */

/* Status codes. */
enum {
    VTG_OK = 0,
    VTG_EINVAL = -1,   /* an argument or configuration out of range */
    VTG_ENOMEM = -2,   /* device or host allocation failed */
    VTG_ECUDA = -3,    /* a CUDA call failed (vtg_last_cuda_error gives its code) */
    VTG_ETIMEOUT = -4, /* a bounded device wait gave up */
    VTG_EBUSY = -5,    /* the object is in use by work not yet finished */
    VTG_ENODEV = -6,   /* no usable CUDA device */
    VTG_EBUDGET = -7   /* the request does not fit the context's device-memory budget */
};

/* Where a buffer lives. */
enum { VTG_HOST = 0, VTG_DEVICE = 1 };

/* LK status bits: enum in src/kern/lk.h:22, bit for bit. */
enum { VTG_LK_OK = 0, VTG_LK_OUT = 1, VTG_LK_LOWEIG = 2, VTG_LK_RESIDUAL = 4, VTG_LK_FLOWBACK = 8 };

/* One tracked point: struct lk_out (src/kern/lk.h:33-40), byte for byte (32 bytes). */
struct vtg_lk_out {
    float x, y;         /* the estimate at level 0 */
    float min_eig;      /* smaller eigenvalue of the structure tensor per patch pixel, at level 0 */
    float residual;     /* mean |T - J|, 8-bit grey */
    float cov_xx, cov_xy, cov_yy;
    uint16_t iters;     /* summed over levels */
    uint16_t status;    /* VTG_LK_* bits */
};

/* One cell of the per-cell flow grid: struct vt_cell (src/common/vt_proto.h:395-402), byte for byte (24 bytes). */
struct vtg_cell {
    float u, v;     /* flow, pixels of the cells' level */
    float diff;     /* mean |J - I| over the cell, 8-bit grey */
    uint32_t state; /* LK status bits in the low byte */
    float sigma;    /* sqrt(cov_xx + cov_yy) when the status is 0 */
    float pad;
};

/* A stream's configuration: the LK fields of struct vt_config (src/common/vt_proto.h:67-127) plus the cell grid
 * (VT_CELL_W / VT_CELL_H, vt_proto.h:385-386) and the level it lives on (flow_level, vt_proto.h:115). */
struct vtg_config {
    uint32_t width, height; /* level 0, pixels; any size >= 32 x 32 */
    uint32_t levels;        /* pyramid levels, 1 .. VTG_MAX_LEVELS */
    uint32_t patch_w, patch_h; /* odd, 5 .. VTG_MAX_PATCH_W / VTG_MAX_PATCH_H */
    uint32_t max_iter;
    float eps;          /* stop when a step is below this, pixels of the level */
    float min_eig;      /* per patch pixel, 8-bit grey per pixel */
    float max_residual; /* mean |T - J| in 8-bit grey */
    float fb_max;       /* forward-backward miss, pixels; 0 = no check */
    uint32_t cell_w, cell_h; /* the cell grid, pixels of flow_level */
    uint32_t flow_level;     /* the pyramid level the cells live on */
};

typedef struct vtg_ctx vtg_ctx;
typedef struct vtg_tracker vtg_tracker;

/* ---- library and context ---- */

const char *vtg_strerror(int status);
/* The last CUDA error code a VTG_ECUDA came from, in this thread. */
int vtg_last_cuda_error(void);
/* A context on CUDA device `device`, holding at most `hbm_budget` bytes of device memory for its trackers (0 = no limit
 * beyond the device's own). */
int vtg_ctx_create(int device, size_t hbm_budget, vtg_ctx **out);
void vtg_ctx_destroy(vtg_ctx *ctx);
/* Bytes of the budget in use. */
size_t vtg_ctx_used(const vtg_ctx *ctx);
/* Waits for all of the context's work, at most timeout_ms (VTG_ETIMEOUT after that). */
int vtg_ctx_sync(vtg_ctx *ctx, int timeout_ms);
/* The bounds record of the checked build (libvtg_checked.so, built with VTG_CHECKED): after the device is idle,
 * out[0] = the LK patch operations whose pixel rectangle would have left its level (bit 1 template build, 2 window
 * pass, 4 sample pass), out[1] = how many times; then clears it. Returns 1 in the checked build, 0 (out zeroed) in the
 * production build, which has no checks. */
int vtg_check_read(uint32_t *out);

/* ---- a tracker: one camera stream's device-resident state (tk_create, src/kern/track.h:22 / track.c:447-572) ---- */

/* Device bytes one tracker of this configuration holds: two pyramid sets, a frame staging buffer, the cell results. */
size_t vtg_tracker_bytes(const struct vtg_config *cfg);
int vtg_tracker_create(vtg_ctx *ctx, const struct vtg_config *cfg, vtg_tracker **out);
void vtg_tracker_destroy(vtg_tracker *t);
/* Pyramid sets (tk_sets, src/kern/track.h:26): frame k goes to set k mod this. */
int vtg_tracker_sets(const vtg_tracker *t);
/* Cells of the grid: ceil(w_f / cell_w) x ceil(h_f / cell_h) at the flow level's size w_f x h_f. Returns their
 * number (cols x rows), or a negative status. */
int vtg_tracker_cells(const vtg_tracker *t, int *cols, int *rows);
/* The tracker's stream (a cudaStream_t) -- work of one tracker is ordered on it. */
void *vtg_tracker_stream(const vtg_tracker *t);

/* ---- the hot path ---- */

/* The pyramid of one 8-bit frame into set `set` (tk_build, src/kern/track.c:584-629: img_u8_to_q6 + img_reduce per
 * level, src/kern/img_ref.c:32-40 / 98-114). Levels hold the reference's Q6 values (byte x 64, then the 5 x 5 binomial
 * with (h + 128) >> 8) bit for bit. frame: height rows of width bytes, `stride` bytes apart, in host (pinned or
 * pageable) or device memory as `where` says. Asynchronous on `stream` (NULL: the tracker's). The build options below
 * change level 0 first, as tk_build's do. */
int vtg_build(vtg_tracker *t, int set, const uint8_t *frame, int stride, int where, void *stream);

/* tk_build's optional steps on the input frame: struct vt_config's contrast and pre_gauss
 * (src/common/vt_proto.h:89-90), switched per frame by the VT_SC_CONTRAST / VT_SC_PRE_GAUSS keys
 * (src/kern/track.c:586-589). In the reference's order (track.c:600-622):
 *   - VTG_BUILD_CONTRAST: the frame's Q6 min .. max stretched onto 0 .. 16320 (img_minmax + img_norm,
 *     src/kern/img_ref.c:42-71), with vtg_contrast_gain's gain and offset;
 *   - VTG_BUILD_PRE_GAUSS: then the 5 x 5 binomial with (h + 128) >> 8 (img_gauss5, img_ref.c:83-96).
 * Level 0 is the result and the levels above reduce from it, bit for bit as the reference. The flags apply to the
 * tracker's later vtg_build calls and batch steps. */
#define VTG_BUILD_CONTRAST 1
#define VTG_BUILD_PRE_GAUSS 2
int vtg_tracker_set_build(vtg_tracker *t, int flags);
int vtg_tracker_build_flags(const vtg_tracker *t);
/* The stretch's gain_offset[0..1] for a frame whose Q6 minimum and maximum are lo and hi (whole numbers,
 * 0 <= lo <= hi < 2^24), as tk_build forms them in x87 extended precision (track.c:603-614): gain = 16320 / (hi - lo)
 * (1 when hi == lo), offset = -lo x gain, each rounded to F32 from the extended value. */
int vtg_contrast_gain(int lo, int hi, float *gain_offset);

/* Per-cell flow from set `prev` to set `cur` (still_vectors, src/kern/still.c:116-141, with the tracker's LK settings):
 * one LK vector per cell centre, the forward-backward check when fb_max > 0, and the cell record. `cells` (may be
 * NULL) receives cols x rows struct vtg_cell, `lk` (may be NULL) the struct vtg_lk_out of each cell, both row-major, in
 * host or device memory as `where` says. Host results are complete when the stream is. */
int vtg_cells(vtg_tracker *t, int prev, int cur, struct vtg_cell *cells, struct vtg_lk_out *lk, int where, void *stream);

/* LK for a list of points from set `prev` to set `cur` (OP_LK, src/kern/track.c:275-292: lk_track + lk_flowback,
 * src/kern/lk.h:46-53): n points (xs, ys) in level-0 pixels, each with its own guess (gx, gy may be NULL: no guess);
 * `top` the first level (-1: the tracker's top). Arrays in host or device memory as `where` says. */
int vtg_points(vtg_tracker *t, int prev, int cur, int top, int n, const float *xs, const float *ys, const float *gx,
               const float *gy, struct vtg_lk_out *out, int where, void *stream);
/* Warps a point for the tracker's later vtg_points calls: 1 (a warp walks the whole patch), 2 (two warps each walk half
 * the patch's rows and add their sums after every pass), or 0, the default, which is 1: on the GB300 two warps were
 * slower at every list length measured (128 to 2,048 points). The two differ only in the F32 rounding of the sums. */
int vtg_tracker_set_point_warps(vtg_tracker *t, int warps);

/* Copies one level of a set out (tk_level, src/kern/track.h:61): h_L rows of w_L floats, Q6. */
int vtg_level(vtg_tracker *t, int set, int level, float *out, int where, void *stream);
/* A level's size. */
int vtg_level_size(const vtg_tracker *t, int level, int *w, int *h);
/* The device address of a level of a set (F32 Q6, rows `pitch` floats apart), for searching it in place. Valid until
 * the tracker is destroyed; its contents change with every vtg_build of that set. */
int vtg_level_device(const vtg_tracker *t, int set, int level, const float **plane, int *w, int *h, int *pitch);

/* The appearance template of a region (store_appearance, src/kern/track.c:935-974), cut from a set's resident
 * pyramid: the coarsest level where a 32 x 21 template still fits inside the region rw x rh, the 32 x 21 window there
 * around the centre (cx, cy) (level-0 pixels, truncated to whole pixels of that level), made zero-mean, and its sum of
 * squares, in the reference's F32 arithmetic bit for bit (its 16-lane sums and folds, the x87 mean). `a` (host memory)
 * gets the level, the centre's fraction (fx, fy) and `valid`, at once; with valid = 0 (the window does not fit inside
 * the level's border) nothing is written and nothing runs. Otherwise pix (VTG_APP_W x VTG_APP_H floats, row-major) and
 * norm (one float) are written in host or device memory as `where` says, complete when the stream is; the pair is
 * what vtg_search_template takes. */
#define VTG_APP_W 32
#define VTG_APP_H 21
struct vtg_appearance {
    float fx, fy;
    int32_t level, valid;
};
int vtg_store_appearance(vtg_tracker *t, int set, float cx, float cy, float rw, float rh, float *pix, float *norm,
                         struct vtg_appearance *a, int where, void *stream);

/* The cell results of a tracker's last vtg_cells or batch step: cols x rows records each (either may be NULL). */
int vtg_tracker_results(vtg_tracker *t, struct vtg_cell *cells, struct vtg_lk_out *lk, int where, void *stream);

/* ---- many streams in one step: the batched form of tk_build + still_vectors ---- */

/* How the batched LK launch runs (its autotuner's choices): warps per CTA (4, 8 or 16), cells per work item, a
 * persistent grid of ctas_per_sm CTAs per SM pulling items from a device counter (persistent = 1) or one warp per item
 * (persistent = 0); tsmem = 1 keeps the template's intensities in shared memory instead of registers, for more warps
 * an SM (persistent only; 4 warps with ctas_per_sm <= 5, 8 with <= 3, 16 with 1); tiled = 1 walks each stream's cells
 * in tiles of 8 x 4 and gives a CTA whole tiles, so the cells an SM runs at once are neighbours that share their
 * windows in its L1 (persistent only; chunk must divide 32). */
struct vtg_tune {
    int block_warps, chunk, persistent, ctas_per_sm, tsmem, tiled;
};

typedef struct vtg_batch vtg_batch;

/* A batch of up to max_jobs streams (all of one context, one LK setting). Two slots hold two prepared steps. */
int vtg_batch_create(vtg_ctx *ctx, int max_jobs, vtg_batch **out);
void vtg_batch_destroy(vtg_batch *b);
void *vtg_batch_stream(const vtg_batch *b);
/* Prepares one step into `slot`: for each of n trackers, frames[j] (height rows of width bytes, strides[j] apart, or
 * NULL strides: width) becomes the pyramid of set cur_sets[j], and the cells flow from set 1 - cur_sets[j] to it
 * (tk_build + still_vectors, src/kern/track.c:584-629, src/kern/still.c:116-141). Host frames must stay valid (and
 * pinned, to be captured in a graph) for every launch of the slot. */
int vtg_batch_prepare(vtg_batch *b, int slot, int n, vtg_tracker *const *trackers, const uint8_t *const *frames,
                      const int *strides, int where, const int *cur_sets);
/* Runs a prepared step: the batched pyramid launches, then one LK launch over every stream's cells. Results stay in
 * each tracker (vtg_tracker_results). */
int vtg_batch_launch(vtg_batch *b, int slot, void *stream);
/* The same, with the steps that wrote these trackers' pyramid sets and results before still in flight on other
 * streams: host frames are uploaded at once (each set has its own staging buffer), then the kernels wait for the
 * `nwait` CUDA events (cudaEvent_t) recorded after those steps. */
int vtg_batch_launch_after(vtg_batch *b, int slot, void *stream, int nwait, void *const *events);
/* As vtg_batch_launch_after, with `nwait_lk` more events that only the step's LK launch waits for, after its pyramid:
 * e.g. the copies of earlier results out of the result buffers this LK launch writes, which may then overlap this
 * step's pyramid. */
int vtg_batch_launch_split(vtg_batch *b, int slot, void *stream, int nwait, void *const *events, int nwait_lk,
                           void *const *events_lk);
/* Captures a prepared step into a CUDA graph, and replays it. */
int vtg_batch_capture(vtg_batch *b, int slot);
int vtg_batch_replay(vtg_batch *b, int slot, void *stream);
/* Cells of a prepared step. */
int vtg_batch_cells(const vtg_batch *b, int slot);
int vtg_batch_set_tune(vtg_batch *b, const struct vtg_tune *t);
int vtg_batch_get_tune(const vtg_batch *b, struct vtg_tune *t);
/* Times every candidate launch shape on the prepared step (median of reps) and keeps the fastest for this mix of
 * stream sizes; reports it, its time and the default shape's time. */
int vtg_batch_autotune(vtg_batch *b, int slot, int reps, struct vtg_tune *best, float *best_ms, float *default_ms);
/* Runs a prepared step reps times with events between its phases: the median time of the pyramids (with any host
 * frames' upload) and of the LK launch. For rooflines. */
int vtg_batch_profile(vtg_batch *b, int slot, int reps, float *pyr_ms, float *lk_ms);
/* Runs a prepared step's LK launch once more (its pyramids as they stand) and counts the work of every cell's walks,
 * forward and backward: counts[0] template builds, [1] residual passes, [2] window passes, [3] iterations. With the
 * reference's operation counts per patch operation (src/kern/lk_ref.c) they give the launch's algorithmic FLOPs.
 * Waits for the result. */
int vtg_batch_count(vtg_batch *b, int slot, uint64_t *counts);

/* ---- the appearance search (reacquisition) ---- */

/* Plane element types. */
enum { VTG_PLANE_U8 = 0, VTG_PLANE_F32 = 1 };
/* Arithmetic of the correlation map: F32 products (CUDA cores), or BF16 / FP16 products with F32 accumulation on the
 * tensor cores (U8 planes). Window sums are exact in every case; the final scores of the eight candidates are always
 * F32. */
enum { VTG_NCC_F32 = 0, VTG_NCC_BF16 = 1, VTG_NCC_FP16 = 2 };
#define VTG_NCC_MAX_T 128

/* What a search found: struct found (src/kern/track.c:1608-1612) plus take_back's parabola offsets
 * (track.c:1741-1742). hx, hy: the template's corner in half pixels of the plane; ncc: its score; second: the best
 * score clear of it by half a template (-2 if none); ox, oy: sub-half-pixel offsets in [-0.5, 0.5]; ntop: candidates
 * looked at; cells: cells of the map. */
struct vtg_found {
    int hx, hy;
    float ncc, second, ox, oy;
    int ntop, cells;
};

typedef struct vtg_search vtg_search;

/* Device bytes of a search context for planes up to max_w x max_h and templates up to max_tw x max_th. */
size_t vtg_search_bytes(int max_w, int max_h, int max_tw, int max_th);
/* A search context: its template, the integral images, the per-cell map and the candidates, in one allocation charged
 * to the context's budget. */
int vtg_search_create(vtg_ctx *ctx, int max_w, int max_h, int max_tw, int max_th, vtg_search **out);
void vtg_search_destroy(vtg_search *s);
void *vtg_search_stream(const vtg_search *s);
/* The template (store_appearance, src/kern/track.c:935-974): th rows of tw zero-mean floats (tw a multiple of 8) and
 * norm, the sum of their squares. Host or device memory as `where` says. */
int vtg_search_template(vtg_search *s, const float *app, int tw, int th, float norm, int where, void *stream);
/* search_slot (src/kern/track.c:1661-1726) over corners [x0, x1] x [y0, y1] of a plane (w x h, rows `pitch` elements
 * apart, device memory, type VTG_PLANE_*), at `step`; the window is clamped to where the template fits as the
 * reference clamps it. `precision` VTG_NCC_*. *found (and, if not NULL, the per-cell map of `cells` entries) in host
 * or device memory as `where` says. */
int vtg_search_run(vtg_search *s, const void *plane, int w, int h, int pitch, int plane_type, int x0, int x1, int y0,
                   int y1, int step, int precision, struct vtg_found *found, float *map_v, int *map_x, int *map_y,
                   int where, void *stream);
/* Runs vtg_search_run's work reps times (after one warm-up) on the search's stream and reports the median CUDA-event
 * time of the correlation map's kernel alone and of the whole search (window sums, map, candidates, half-pixel
 * re-score). Each rep runs it twice: once with events around the map kernel, once with events around the whole
 * search only, launched as vtg_search_run launches it. For rooflines. */
int vtg_search_profile(vtg_search *s, const void *plane, int w, int h, int pitch, int plane_type, int x0, int x1,
                       int y0, int y1, int step, int precision, int reps, float *map_ms, float *total_ms);
/* tk_correlate (src/kern/track.c:208, track.h:59) at n corners: the score of each, -1 where the template does not fit. */
int vtg_correlate(vtg_search *s, const void *plane, int w, int h, int pitch, int plane_type, int n, const int *xs,
                  const int *ys, float *out, int where, void *stream);

/* ---- the appearance search without any allocation ---- */

#define VTG_NOALLOC_SCRATCH_BYTES (5u << 20) /* held on every GPU that loads the library, until exit */
#define VTG_NOALLOC_MAX_PIXELS 320000        /* (w + 1) (h + 1) at most: a 640 x 480 plane fits */
#define VTG_NOALLOC_MAX_T 64                 /* template sides at most */

/* No counterpart in the reference: an extra entry point for callers that cannot allocate device memory when they search
 * (a real-time loop that cannot absorb a cudaMalloc, a host runtime that owns every byte of device memory). The same
 * search as vtg_search_run with an F32 map, but nothing is allocated: no context, no search context; the caller
 * passes the plane, the template (th rows of tw zero-mean floats, tw a multiple of 8) and its norm, and *found (and the
 * optional per-cell map) in device memory; the scratch lives in one fixed device array of VTG_NOALLOC_SCRATCH_BYTES.
 * Larger planes or templates than the limits above, or a step other than 1, 2 or 4, return VTG_EINVAL. All calls
 * share that array: calls whose work overlaps on the GPU race, so order them on one stream. The first call on a device
 * looks the array's address up and keeps it for the life of the process; make it before any stream capture, and do
 * not call this entry point on a device after cudaDeviceReset of that device. Asynchronous on `stream` (a
 * cudaStream_t, NULL for the legacy default). */
int vtg_search_run_noalloc(const void *plane, int w, int h, int pitch, int plane_type, const float *app, int tw, int th,
                           float norm, int x0, int x1, int y0, int y1, int step, struct vtg_found *found, float *map_v,
                           int *map_x, int *map_y, void *stream);

/* ---- corner detection: seed_at's detect_begin, detect_tensor / detect_response / detect_cells, detect_finish
 *      (src/kern/track.c:988-992; src/kern/detect.h:21-37, src/kern/detect.c:28-258) ---- */

typedef struct vtg_detector vtg_detector;

/* Device bytes of a detector for regions up to max_w x max_h: the response map, the cells, 8,192 candidates. */
size_t vtg_detector_bytes(int max_w, int max_h);
int vtg_detector_create(vtg_ctx *ctx, int max_w, int max_h, vtg_detector **out);
void vtg_detector_destroy(vtg_detector *d);
void *vtg_detector_stream(const vtg_detector *d);
/* Corners inside the rectangle (rx, ry, rw, rh) of a Q6 plane (w x h, rows `pitch` floats apart, device memory), kept
 * `margin` pixels from its edges: the Harris response on a 5 x 5 box over Sobel gradients, the local maxima above
 * max(quality x the strongest of their 3 x 3 cells of 16 x 16, 2500), best first, and greedily those at least min_dist
 * from every one taken, up to max (<= 512). xs, ys get the corners, *count their number. where: VTG_HOST (xs, ys,
 * count in host memory; the call waits) or VTG_DEVICE (asynchronous on `stream`, or the detector's). */
int vtg_detect(vtg_detector *d, const float *plane, int w, int h, int pitch, float rx, float ry, float rw, float rh,
               int margin, int max, float min_dist, float quality, float *xs, float *ys, int *count, int where,
               void *stream);
/* For checking, after vtg_detect: its region's layout (geo: x0, y0, x1, y1, ax, cols, rows, nv, cell_rows), its
 * response map (rows x cols) and its cells' strongest responses (cell_rows x nv), as detect_begin, detect_response
 * and detect_cells leave them; resp and cells may be NULL. Waits for the detector's stream. */
int vtg_detect_maps(vtg_detector *d, float rx, float ry, float rw, float rh, int w, int h, int margin, int *geo,
                    float *resp, float *cells);

/* ---- the still picture: one camera's mean over the frames each cell held still (src/kern/still.h:1-53,
 *      src/kern/still.c) ---- */

typedef struct vtg_still vtg_still;

/* struct still_cfg (src/kern/still.h:21-27) without its thread count: the plane size (32 to 4096 a side), frames at
 * most in a cell's mean (avg, 1 to 65,535: weight 1 / min(count, avg)), the good-vector length past which a cell
 * moved (motion_px, pixels) and the mean |frame - mean| over a cell past which it changed (motion_grey, 8-bit grey). */
struct vtg_still_config {
    int w, h, avg;
    float motion_px, motion_grey;
};

/* What still_motion fills (src/kern/still.c:262-275) of struct vt_motion (src/common/vt_proto.h:403-415), for the
 * newest frame: 48 bytes. */
struct vtg_still_motion {
    uint32_t cols, rows, tracked, moving;
    float count_mean, drift_u, drift_v, drift_rms, diff_median, diff_limit;
    uint64_t frames;
};

/* still_bytes / still_create (still.h:31-32, still.c:55-99): the mean, the 16 x 8 cells, their counts, all zero. */
size_t vtg_still_bytes(const struct vtg_still_config *c);
int vtg_still_create(vtg_ctx *ctx, const struct vtg_still_config *c, vtg_still **out);
void vtg_still_destroy(vtg_still *s);
void *vtg_still_stream(const vtg_still *s);

/* One frame, as the reference runs it (still.h:11): still_vectors unless it is the first frame (LK from the mean to
 * the frame at every cell, 15 x 15, 6 iterations, forward-backward 0.25 px), still_decide, still_update, still_finish.
 * cur: the frame's Q6 plane (w x h, rows `pitch` floats apart) in device memory, e.g. a tracker's resident level
 * (vtg_level_device). cells_in (host or device memory as `where` says) replaces the vectors with the caller's own
 * cells; NULL runs them. Asynchronous on `stream` (NULL: the still's own). */
int vtg_still_frame(vtg_still *s, const float *cur, int pitch, const struct vtg_cell *cells_in, int where,
                    void *stream);

/* still_cells / still_motion / still_mean (still.h:45-51) of the newest frame: any of cells (cols x rows), motion and
 * mean (w x h, rows mean_pitch floats apart) may be NULL. VTG_HOST waits for the copies; VTG_DEVICE does not. */
int vtg_still_read(vtg_still *s, struct vtg_cell *cells, struct vtg_still_motion *motion, float *mean, int mean_pitch,
                   int where, void *stream);

/* The mean plane in device memory (still_mean, still.h:45), valid until the next frame. */
int vtg_still_mean(const vtg_still *s, const float **plane, int *pitch);

/* ---- frame generation: a frame between two real ones (src/kern/framegen.h, src/kern/framegen.c; run as
 *      tk_generate_make runs it, src/kern/track.c:847-888) ---- */

typedef struct vtg_framegen vtg_framegen;

/* struct fg_vec (src/kern/framegen.h:24-26): a block's vector, from the newer frame to the older, in pixels of its
 * level. */
struct vtg_fg_vec {
    int16_t x, y;
};

/* For frames of w x h (64 to 8192 a side): the field's pyramid of both frames (their half size, then halves while
 * both sides are >= 16, seven levels at most: track.c:547-556), its fields, the generated frame. */
size_t vtg_framegen_bytes(int w, int h);
int vtg_framegen_create(vtg_ctx *ctx, int w, int h, vtg_framegen **out);
void vtg_framegen_destroy(vtg_framegen *g);
void *vtg_framegen_stream(const vtg_framegen *g);
int vtg_framegen_levels(const vtg_framegen *g);

/* One generated frame between older and newer, w x h Q6 planes in device memory (e.g. two sets' level 0 of a tracker,
 * vtg_level_device). The scene-change test (fg_hist_section, fg_scene_verdict), then coarsest first fg_search,
 * fg_filter, fg_upscale, then fg_mid_vectors and fg_blend. out (device, rows out_pitch floats apart) receives the
 * frame in Q6, or NULL keeps it inside (vtg_framegen_frame); pic (NULL, or host or device memory as `where` says)
 * receives its bytes (img_q6_to_u8_vx, src/kern/img_vx.c:36-47), w a row. VTG_HOST waits for pic; otherwise
 * asynchronous on `stream` (NULL: the generator's own). */
int vtg_framegen_run(vtg_framegen *g, const float *older, int older_pitch, const float *newer, int newer_pitch,
                     float *out, int out_pitch, uint8_t *pic, int where, void *stream);

/* The last run's fields at `level` (raw = fg_search's, fil = fg_filter's, up = what the level started from; each
 * ceil(level w / 8) x ceil(level h / 8)), the middle-instant field (level 0's blocks) and the scene verdict; any may
 * be NULL. */
int vtg_framegen_fields(vtg_framegen *g, int level, struct vtg_fg_vec *raw, struct vtg_fg_vec *fil,
                        struct vtg_fg_vec *up, struct vtg_fg_vec *mid, int *scene, int where, void *stream);

/* The generated frame inside the generator (device memory), valid until the next run. */
int vtg_framegen_frame(const vtg_framegen *g, const float **plane, int *pitch);

#ifdef __cplusplus
}
#endif

#endif
