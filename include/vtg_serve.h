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
};

struct vtg_serve_stats {
    int streams_admitted, streams_waited, streams_rejected;
    long requests, served, cells, ncc;
    double wall_s, cells_per_s, p50_ms, p99_ms, max_ms, mean_batch;
};

/* Runs the loop to the end of the schedule (every frame pair served) or to its time limit (VTG_ETIMEOUT). */
int vtg_serve_run(vtg_ctx *ctx, const struct vtg_serve_cfg *cfg, struct vtg_serve_stats *out);

#ifdef __cplusplus
}
#endif

#endif
