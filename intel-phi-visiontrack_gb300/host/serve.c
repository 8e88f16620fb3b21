/* serve.c -- the served loop's Poisson driver: frame-pair requests from many camera streams pushed through the request
 * API (server.c) as they arrive.
 *
 * The reference's card session takes frames from a DMA ring as the host publishes them, skips frames under LIVE
 * priority and backs off when device memory is full (src/card/session_track.c:1-10, 37-53, 187-225). This drives the
 * request API the same way, on the host, in C:
 *   - streams start over time; each is admitted when its tracker's device memory fits the budget (vtg_tracker_bytes),
 *     else it waits for a stream that finishes to free memory; a stream whose description is malformed is refused and
 *     the run goes on;
 *   - each stream's frame pairs arrive on a seeded Poisson schedule at its rate and are submitted when they arrive
 *     (a frame that meets a full queue is dropped); with `live`, a stream's newer frame goes ahead of its queued older
 *     ones, which are skipped;
 *   - a share of the frames asks for an appearance search of its level 1 after its cells;
 *   - latency of a frame pair = its results on the host minus its arrival; p50 / p99 over all pairs served.
 * The plain form runs the same schedule one frame pair at a time (the server's plain mode, one step in flight).
 * Every wait is bounded: the run ends at duration + 10 s whatever the GPU does, and a producer that stops submitting
 * (stall_at_s, a host-side fault injection) ends it with VTG_ETIMEOUT after stall_timeout_s, once the steps on the GPU
 * have delivered their results. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "vtg_serve.h"

#define SERVE_DRAIN_S 10.0
#define SERVE_POLL 256

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* xorshift64*: a reproducible arrival schedule. */
static double urand(uint64_t *s)
{
    uint64_t x = *s;
    x ^= x >> 12;
    x ^= x << 25;
    x ^= x >> 27;
    *s = x;
    return (double)((x * 0x2545F4914F6CDD1Dull) >> 11) * (1.0 / 9007199254740992.0);
}

struct req {
    int stream, k;
    double t_arrive;
};

struct sstate {
    int id;          /* the server's stream id, -1 before admission */
    int valid, waiting, finished, cells;
    int first, count, next; /* its requests in arrival order: order[first .. first + count), submitted up to next */
    int settled;            /* served, skipped or dropped */
};

static int cmp_req(const void *a, const void *b)
{
    const struct req *x = a, *y = b;
    return x->t_arrive < y->t_arrive ? -1 : x->t_arrive > y->t_arrive;
}

static int cmp_dbl(const void *a, const void *b)
{
    const double x = *(const double *)a, y = *(const double *)b;
    return x < y ? -1 : x > y;
}

static struct vtg_config stream_cfg(const struct vtg_serve_cfg *c, int s)
{
    struct vtg_config g = c->lk;
    g.width = c->streams[s].width;
    g.height = c->streams[s].height;
    g.flow_level = c->streams[s].flow_level;
    return g;
}

/* Cells of a stream's grid: ceil(w_f / cell_w) x ceil(h_f / cell_h) at its flow level's size (each level (n + 1) / 2
 * of the one below, as the pyramid's). */
static int grid_cells(const struct vtg_config *g)
{
    uint32_t w = g->width, h = g->height;
    for (uint32_t L = 0; L < g->flow_level; L++) {
        w = (w + 1) / 2;
        h = (h + 1) / 2;
    }
    return (int)(((w + g->cell_w - 1) / g->cell_w) * ((h + g->cell_h - 1) / g->cell_h));
}

/* A stream description the loop can run: a size and level the tracker takes, a rate, frames. */
static int stream_ok(const struct vtg_serve_cfg *c, int s)
{
    const struct vtg_serve_stream *d = &c->streams[s];
    if (!(d->fps > 0.0f) || !isfinite(d->fps) || d->frames < 1 || !(d->start_s >= 0.0f) || !isfinite(d->start_s) ||
        !c->frames[2 * s] || !c->frames[2 * s + 1])
        return 0;
    struct vtg_config g = stream_cfg(c, s);
    return vtg_tracker_bytes(&g) > 0;
}

int vtg_serve_run(vtg_ctx *ctx, const struct vtg_serve_cfg *c, struct vtg_serve_stats *out)
{
    if (!ctx || !c || !out || c->nstreams < 1 || !c->streams || !c->frames || !(c->duration_s > 0.0) ||
        c->max_batch < 1 || c->max_batch > 512 || c->inflight < 1 || c->inflight > 2 || c->max_queue < 0 ||
        c->max_queue > 64 || !(c->stall_at_s >= 0.0) || !(c->stall_timeout_s >= 0.0))
        return VTG_EINVAL;
    memset(out, 0, sizeof *out);
    const int ns = c->nstreams;
    uint64_t seed = c->seed ? c->seed : 0x9E3779B97F4A7C15ull;
    struct sstate *st = calloc((size_t)(unsigned)ns, sizeof *st);
    if (!st)
        return VTG_ENOMEM;
    int total = 0;
    for (int s = 0; s < ns; s++) {
        st[s].id = -1;
        st[s].valid = stream_ok(c, s);
        if (st[s].valid)
            total += c->streams[s].frames;
        else
            out->streams_rejected++;
    }
    struct req *rq = calloc((size_t)total + 1, sizeof *rq);
    double *lat = calloc((size_t)total + 1, sizeof *lat);
    int *order = calloc((size_t)total + 1, sizeof *order);
    struct vtg_server_result *res = calloc(SERVE_POLL, sizeof *res);
    if (!rq || !lat || !order || !res) {
        free(st);
        free(rq);
        free(lat);
        free(order);
        free(res);
        return VTG_ENOMEM;
    }
    /* the arrival schedule */
    int n = 0;
    for (int s = 0; s < ns; s++) {
        if (!st[s].valid)
            continue;
        double t = c->streams[s].start_s;
        for (int k = 0; k < c->streams[s].frames; k++) {
            t += -log(1.0 - urand(&seed)) / (double)c->streams[s].fps;
            rq[n].stream = s;
            rq[n].k = k;
            rq[n].t_arrive = t;
            n++;
        }
    }
    qsort(rq, (size_t)n, sizeof *rq, cmp_req);
    for (int i = 0; i < n; i++)
        st[rq[i].stream].count++;
    for (int s = 0, acc = 0; s < ns; s++) {
        st[s].first = acc;
        acc += st[s].count;
    }
    {
        int *fill = calloc((size_t)(unsigned)ns, sizeof *fill);
        if (!fill) {
            free(st);
            free(rq);
            free(lat);
            free(order);
            free(res);
            return VTG_ENOMEM;
        }
        for (int i = 0; i < n; i++) {
            const int s = rq[i].stream;
            order[st[s].first + fill[s]++] = i;
        }
        free(fill);
    }
    struct vtg_server_cfg scfg;
    memset(&scfg, 0, sizeof scfg);
    scfg.lk = c->lk;
    scfg.max_batch = c->max_batch;
    scfg.inflight = c->plain ? 1 : c->inflight;
    scfg.plain = c->plain;
    scfg.max_queue = c->max_queue ? c->max_queue : 64;
    vtg_server *srv = NULL;
    int rc = vtg_server_create(ctx, &scfg, &srv);
    if (rc == VTG_OK && c->ncc_share > 0.0f) {
        /* a template for the searches: 32 x 21 zero-mean values (its contents do not change the cost) */
        float app[32 * 21];
        for (int i = 0; i < 32 * 21; i++)
            app[i] = (float)((int)(urand(&seed) * 255.0) - 127) * 64.0f;
        rc = vtg_server_template(srv, app, 32, 21, 1.0e9f);
    }
    const size_t used0 = vtg_ctx_used(ctx);
    const double stall_to = c->stall_timeout_s > 0.0 ? c->stall_timeout_s : 2.0;
    long served = 0, cells = 0, ncc = 0, skipped = 0, dropped = 0, submitted = 0;
    const double t0 = now_s();
    double t_last = t0, t_last_submit = t0;
    int next_arrival = 0; /* arrivals before this index have come */
    int stalled = 0;
    while (rc == VTG_OK) {
        const double now = now_s() - t0;
        if (now > c->duration_s + SERVE_DRAIN_S) {
            rc = VTG_ETIMEOUT;
            break;
        }
        long settled = 0;
        for (int s = 0; s < ns; s++)
            settled += st[s].settled;
        if (settled >= n)
            break;
        const int producing = !(c->stall_at_s > 0.0 && now >= c->stall_at_s);
        /* streams that have begun: admit in start order while the budget allows */
        for (int s = 0; s < ns && rc == VTG_OK; s++) {
            if (!st[s].valid || st[s].id >= 0 || st[s].finished || c->streams[s].start_s > now || !producing)
                continue;
            struct vtg_config g = stream_cfg(c, s);
            const size_t need = vtg_tracker_bytes(&g);
            if (c->hbm_budget && vtg_ctx_used(ctx) - used0 + need > c->hbm_budget) {
                if (!st[s].waiting)
                    out->streams_waited++;
                st[s].waiting = 1;
                continue;
            }
            const int id = vtg_server_open(srv, g.width, g.height, g.flow_level,
                                           c->live ? VTG_PRIO_LIVE : VTG_PRIO_ORDERED, c->frames[2 * s],
                                           (int)g.width);
            if (id == VTG_EBUDGET) {
                if (!st[s].waiting)
                    out->streams_waited++;
                st[s].waiting = 1;
                continue;
            }
            if (id == VTG_EINVAL) { /* refused: the others run */
                st[s].valid = 0;
                st[s].finished = 1;
                st[s].settled = st[s].count;
                out->streams_rejected++;
                continue;
            }
            if (id < 0) {
                rc = id;
                break;
            }
            st[s].id = id;
            st[s].waiting = 0;
            st[s].cells = grid_cells(&g);
            out->streams_admitted++;
        }
        if (rc != VTG_OK)
            break;
        /* arrivals: every admitted stream's frames that have come, in arrival order */
        while (next_arrival < n && rq[next_arrival].t_arrive <= now)
            next_arrival++;
        if (producing) {
            for (int s = 0; s < ns && rc == VTG_OK; s++) {
                struct sstate *ss = &st[s];
                if (ss->id < 0 || ss->finished)
                    continue;
                while (ss->next < ss->count && rq[order[ss->first + ss->next]].t_arrive <= now) {
                    const int ri = order[ss->first + ss->next];
                    const int kk = rq[ri].k;
                    const int search = c->ncc_share > 0.0f && urand(&seed) < (double)c->ncc_share;
                    struct vtg_cell *dst = c->last_cells ? c->last_cells[s] : NULL;
                    const int64_t tk = vtg_server_submit(srv, ss->id, c->frames[2 * s + ((kk + 1) & 1)],
                                                         (int)c->streams[s].width, dst, (uint64_t)ri,
                                                         search ? VTG_REQ_SEARCH : 0);
                    ss->next++;
                    if (tk == VTG_EBUSY) {
                        dropped++;
                        ss->settled++;
                    } else if (tk < 0) {
                        rc = (int)tk;
                        break;
                    } else {
                        submitted++;
                        t_last_submit = now_s();
                    }
                }
            }
        } else if (!stalled && now_s() - t_last_submit > stall_to) {
            stalled = 1;
        }
        if (rc != VTG_OK)
            break;
        const int got = vtg_server_poll(srv, res, SERVE_POLL, 0);
        if (got < 0) {
            rc = got;
            break;
        }
        for (int i = 0; i < got; i++) {
            const struct vtg_server_result *r = &res[i];
            if (r->status == VTG_RES_RETIRED)
                continue;
            const struct req *q = &rq[r->tag];
            struct sstate *ss = &st[q->stream];
            ss->settled++;
            if (r->status == VTG_RES_SKIPPED) {
                skipped++;
            } else {
                const double td = now_s() - t0;
                lat[served++] = 1e3 * (td - q->t_arrive);
                t_last = td + t0;
                cells += ss->cells;
                ncc += r->searched;
            }
            if (ss->settled == ss->count && !ss->finished) {
                vtg_server_close(srv, ss->id); /* its memory goes back to the budget */
                ss->finished = 1;
            }
        }
        if (stalled) {
            /* the producer stopped: deliver what the GPU holds, then give up */
            const double d0 = now_s();
            while (vtg_server_pending(srv) > 0 && now_s() - d0 < SERVE_DRAIN_S) {
                const int g2 = vtg_server_poll(srv, res, SERVE_POLL, 1000);
                if (g2 < 0) {
                    rc = g2;
                    break;
                }
                for (int i = 0; i < g2; i++) {
                    const struct vtg_server_result *r = &res[i];
                    if (r->status == VTG_RES_RETIRED)
                        continue;
                    const struct req *q = &rq[r->tag];
                    st[q->stream].settled++;
                    if (r->status == VTG_RES_SKIPPED) {
                        skipped++;
                    } else {
                        const double td = now_s() - t0;
                        lat[served++] = 1e3 * (td - q->t_arrive);
                        t_last = td + t0;
                        cells += st[q->stream].cells;
                        ncc += r->searched;
                    }
                }
            }
            if (rc == VTG_OK)
                rc = VTG_ETIMEOUT;
            break;
        }
        if (got == 0 && vtg_server_pending(srv) == 0 && next_arrival < n) {
            /* nothing queued or on the GPU and nothing to do until the next arrival: a short pause keeps the loop from
             * burning a core. With work in flight the loop keeps polling, so a completion is seen at once. */
            const double wait = rq[next_arrival].t_arrive - (now_s() - t0);
            if (wait > 200e-6) {
                struct timespec ts = {0, 100000};
                nanosleep(&ts, NULL);
            }
        }
    }
    long steps = 0, frames = 0;
    if (srv)
        vtg_server_counts(srv, &steps, &frames);
    vtg_server_destroy(srv); /* waits for what is left on the GPU */
    const double wall = t_last - t0 - (n ? rq[0].t_arrive : 0.0);
    qsort(lat, (size_t)served, sizeof *lat, cmp_dbl);
    out->requests = n;
    out->served = served;
    out->skipped = skipped;
    out->dropped = dropped;
    out->submitted = submitted;
    out->ncc = ncc;
    out->cells = cells;
    out->wall_s = wall;
    out->cells_per_s = wall > 0.0 ? (double)cells / wall : 0.0;
    out->p50_ms = served ? lat[(long)(0.50 * (double)(served - 1))] : 0.0;
    out->p99_ms = served ? lat[(long)(0.99 * (double)(served - 1))] : 0.0;
    out->max_ms = served ? lat[served - 1] : 0.0;
    out->mean_batch = steps ? (double)frames / (double)steps : 0.0;
    for (int s = 0; s < ns; s++)
        if (st[s].valid && st[s].id < 0 && !st[s].finished)
            out->streams_rejected++; /* never admitted */
    free(st);
    free(rq);
    free(lat);
    free(order);
    free(res);
    return rc;
}
