/* vtg_serve.h -- the served request loop of libvtg (host C, over the C ABI of vtg.h).
 *
 * The reference's card session is the precedent: frames from many cameras arrive over a DMA ring, are admitted
 * while device memory lasts and processed as they come (src/card/session_track.c:1-10, 37-53). Here: many streams'
 * frame pairs arrive on a Poisson schedule, streams are admitted by device-memory footprint, requests are batched as
 * they arrive with up to two batches in flight, and latency is measured from arrival to results on the host. */
#ifndef VTG_SERVE_H
#define VTG_SERVE_H

#include "vtg.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- the request API: a host pushes each frame as it arrives and polls for its cells ----
 *
 * The card session's loop, for hosts that run their own: frames arrive in device memory as the host publishes them,
 * each is built and tracked as soon as the device has room, results go back with a status word, a LIVE stream skips
 * the frames queued ahead of its newest one and counts them (src/card/session_track.c:1-10, 187-225; frames_skipped,
 * src/common/vt_proto.h:346), and a session with no frame for a while ends (session_track.c:1031-1033).
 *
 * A server holds streams (one tracker each, admitted against the context's budget) and two batch slots. Every
 * vtg_server_poll collects the steps that finished and launches what is ready: the oldest queued frame of every stream
 * with room on the device, up to max_batch streams a step (continuous batching; a step of one frame runs as the plain
 * calls). A stream's cells flow from the last frame built for it to the new one, so a stream's results are the same
 * bits alone and in any mix. All calls on one server must come from one thread at a time. */

enum { VTG_PRIO_ORDERED = 0, VTG_PRIO_LIVE = 1 }; /* enum vt_priority, src/common/vt_proto.h:154 */

/* Request flags. */
#define VTG_REQ_SEARCH 1 /* after its cells, an appearance search of the frame's level 1 (level 0 with one level) */

/* What a poll delivers for a request (or, with ticket -1, for a stream the server retired). */
enum {
    VTG_RES_DONE = 0,    /* its cells are in the caller's buffer */
    VTG_RES_SKIPPED = 1, /* a LIVE stream's newer frame went ahead of it: nothing was computed */
    VTG_RES_RETIRED = 2  /* the stream sent nothing for idle_timeout_s and was closed; its memory is free */
};

struct vtg_server_cfg {
    struct vtg_config lk; /* LK settings and cell grid of every stream (width, height, flow_level come per stream) */
    int max_batch;        /* streams in one step at most (1 .. 512) */
    int inflight;         /* steps on the GPU at once, 1 or 2 */
    int plain;            /* 1: one frame at a time in submission order, no batching (the plain form) */
    int max_queue;        /* frames a stream may have queued (1 .. 64) */
    double idle_timeout_s; /* a stream with nothing queued or on the GPU and no frame for this long is retired; 0: never */
};

struct vtg_server_result {
    int stream;
    int status;              /* VTG_RES_* */
    int64_t ticket;          /* vtg_server_submit's return (-1 for VTG_RES_RETIRED) */
    uint64_t tag;            /* the caller's tag */
    uint32_t frames_skipped; /* VTG_RES_DONE: frames of this stream skipped just before it */
    int searched;            /* 1 when `found` holds an appearance search's result */
    double latency_ms;       /* submission to results on the host */
    struct vtg_found found;
};

typedef struct vtg_server vtg_server;

int vtg_server_create(vtg_ctx *ctx, const struct vtg_server_cfg *cfg, vtg_server **out);
/* Waits (at most 10 s) for the steps on the GPU, then frees everything, streams included. */
void vtg_server_destroy(vtg_server *s);
/* The template of the appearance searches (vtg_search_template's arguments, host memory; at most 32 x 21). The searches'
 * device scratch is allocated here for the streams already open, and by vtg_server_open for each later one, never in
 * a step; it is charged to the context's budget. */
int vtg_server_template(vtg_server *s, const float *app, int tw, int th, float norm);
/* Admits a stream of width x height frames whose cells live on flow_level, with priority VTG_PRIO_*; `first` (host
 * memory, `stride` bytes a row; it must stay valid until the stream's first result is polled) is its first frame,
 * whose pyramid is queued at once and which the stream's first step waits for on the GPU. Returns the stream's id
 * (>= 0), VTG_EINVAL for a size or level the tracker does not take (the server goes on), VTG_EBUDGET when its memory
 * (with a template set, the searches' scratch for its size too) does not fit the budget now (retry when streams
 * close). */
int vtg_server_open(vtg_server *s, uint32_t width, uint32_t height, uint32_t flow_level, int priority,
                    const uint8_t *first, int stride);
/* Closes a stream: at once if nothing of it is queued or on the GPU, else as soon as that is done (queued frames are
 * still served). Its memory goes back to the budget. */
int vtg_server_close(vtg_server *s, int stream);
/* Queues a frame of a stream: `frame` (host memory, pinned for the upload to overlap, `stride` bytes a row) must stay
 * valid until its result is polled; `cells` (host memory, the stream's cols x rows records, or NULL) receives its
 * cells. Returns the request's ticket (>= 0), VTG_EBUSY when the stream's queue is full, VTG_EINVAL for a closed or
 * unknown stream. */
int64_t vtg_server_submit(vtg_server *s, int stream, const uint8_t *frame, int stride, struct vtg_cell *cells,
                          uint64_t tag, int flags);
/* Collects finished steps and launches ready ones; then returns up to max results (>= 0), waiting up to timeout_us for
 * the first one when none is ready, or a negative status (VTG_ECUDA). */
int vtg_server_poll(vtg_server *s, struct vtg_server_result *out, int max, int timeout_us);
/* Frames queued or on the GPU, over all streams. */
int vtg_server_pending(const vtg_server *s);
/* Steps launched so far and the frames they held (their ratio is the mean batch). */
int vtg_server_counts(const vtg_server *s, long *steps, long *frames);

/* ---- the Poisson driver of the request API ---- */

/* One stream: its picture, frame rate, when it starts and how many frame pairs it sends. */
struct vtg_serve_stream {
    uint32_t width, height;
    uint32_t flow_level; /* the level its cells live on */
    float fps;           /* Poisson arrival rate */
    float start_s;       /* seconds after the run starts */
    int frames;          /* frame pairs it sends */
};

struct vtg_serve_cfg {
    int nstreams;
    const struct vtg_serve_stream *streams;
    /* two frames per stream (frames[2 s], frames[2 s + 1]), width bytes a row, pinned host memory; a stream's frame
     * pairs alternate between them */
    const uint8_t *const *frames;
    struct vtg_config lk;  /* LK settings and cell grid of every stream (width, height, flow_level per stream) */
    double duration_s;     /* the arrival window; the loop gives up 10 s after it */
    int max_batch;         /* streams in one batch at most */
    int inflight;          /* batches on the GPU at once, 1 or 2 */
    size_t hbm_budget;     /* device bytes for the streams' trackers; 0: no limit */
    float ncc_share;       /* share of frame pairs followed by an appearance search on their level 1 */
    int plain;             /* 1: the plain form, one frame pair at a time in arrival order, no batching */
    uint64_t seed;
    /* optional (NULL, or NULL entries): per stream, host memory for its cols x rows cell records, which receives the
     * results of each of its frame pairs as it completes, so it ends with its last one's */
    struct vtg_cell *const *last_cells;
    int live;               /* 1: every stream has LIVE priority (frames queued behind a newer one are skipped) */
    int max_queue;          /* frames a stream may have queued (0: 64); a frame arriving at a full queue is dropped */
    /* host-side fault injection and its bound: the producer stops submitting at stall_at_s (0: never), and the run
     * ends with VTG_ETIMEOUT once no frame has come for stall_timeout_s (0: 2 s), after every step on the GPU has
     * delivered its results */
    double stall_at_s, stall_timeout_s;
};

struct vtg_serve_stats {
    int streams_admitted, streams_waited, streams_rejected;
    long requests, served, cells, ncc;
    double wall_s, cells_per_s, p50_ms, p99_ms, max_ms, mean_batch;
    long skipped;  /* frames LIVE streams skipped */
    long dropped;  /* frames that arrived at a full queue */
    long submitted; /* frames handed to the server */
};

/* Runs the loop to the end of the schedule (every frame pair served, skipped or dropped) or to its time limit, or to
 * a stalled producer's bound (VTG_ETIMEOUT, with the stats of everything delivered). A stream whose description is
 * malformed (a size, level or rate the tracker does not take, no frames) is refused and counted in
 * streams_rejected; the others run. */
int vtg_serve_run(vtg_ctx *ctx, const struct vtg_serve_cfg *cfg, struct vtg_serve_stats *out);

#ifdef __cplusplus
}
#endif

#endif
