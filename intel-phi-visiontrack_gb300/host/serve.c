/* serve.c -- the served request loop: frame-pair requests from many camera streams, continuously batched on one GPU.
 *
 * The reference's card session takes frames from a DMA ring, drops frames under LIVE priority and backs off when
 * device memory is full (src/card/session_track.c:1-10, 37-53). This is that loop for the GPU path, on the host, in C:
 *   - streams arrive over time; each is admitted when its trackers' device memory fits the budget
 *     (vtg_tracker_bytes), else it waits for a stream that finishes to free memory;
 *   - each stream's frames arrive on a Poisson schedule at its rate;
 *   - continuous batching: whenever one of `inflight` batch slots is free, the oldest waiting frame of every admitted
 *     stream that has nothing on the GPU is taken (up to max_batch streams), their pyramids and cells run as one batched
 *     step (vtg_batch_*), and their cell records are copied back; frames that arrive meanwhile wait for the next slot,
 *     so batches overlap on the device;
 *   - a share of the frames is followed by an appearance search on that stream's level 1 (vtg_search_run);
 *   - latency of a frame pair = its results on the host minus its arrival; p50 / p99 over all pairs.
 * The plain form for comparison runs one frame pair at a time, in arrival order: vtg_build, vtg_cells, wait.
 * Every wait is bounded: the run ends at duration + 10 s whatever the GPU does. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime.h>

#include "vtg_serve.h"

#define SERVE_SLOTS 2
#define SERVE_DRAIN_S 10.0

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
    double t_arrive, t_done;
};

struct sstate {
    vtg_tracker *t;
    int admitted, waiting, finished, cells, cols, rows;
    int in_flight;              /* frame pairs on the GPU, at most one a slot */
    int last_slot;              /* the slot that holds its latest one */
    int first, count, next;     /* this stream's requests in the sorted list: pending from `next` */
    int done;                   /* served */
    struct vtg_cell *host_cells[SERVE_SLOTS]; /* results, one buffer a slot */
    size_t bytes;
};

struct slot {
    vtg_batch *b;
    vtg_search *s;
    struct vtg_found *d_found;
    cudaEvent_t ev;    /* the step done: its results on the host */
    cudaEvent_t ev_lk; /* its LK done (batched steps): the pyramid sets it read are free again */
    int busy, n;
    int *reqs;                  /* indices into the request list */
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

/* Admits stream s if its tracker fits: creates it, builds its first frame (set 0) and its result buffer. */
static int admit(vtg_ctx *ctx, const struct vtg_serve_cfg *c, struct sstate *st, int s)
{
    struct vtg_config g = stream_cfg(c, s);
    int rc = vtg_tracker_create(ctx, &g, &st[s].t);
    if (rc != VTG_OK)
        return rc;
    vtg_tracker_cells(st[s].t, &st[s].cols, &st[s].rows);
    st[s].cells = st[s].cols * st[s].rows;
    for (int k = 0; k < c->inflight; k++)
        if (cudaHostAlloc((void **)&st[s].host_cells[k], sizeof(struct vtg_cell) * (size_t)st[s].cells,
                          cudaHostAllocDefault) != cudaSuccess) {
            for (int j = 0; j < k; j++) {
                cudaFreeHost(st[s].host_cells[j]);
                st[s].host_cells[j] = NULL;
            }
            vtg_tracker_destroy(st[s].t);
            st[s].t = NULL;
            return VTG_ENOMEM;
        }
    rc = vtg_build(st[s].t, 0, c->frames[2 * s], (int)g.width, VTG_HOST, NULL);
    if (rc == VTG_OK)
        rc = vtg_ctx_sync(ctx, 10000);
    st[s].admitted = 1;
    st[s].waiting = 0;
    return rc;
}

static void retire(struct sstate *st, int s)
{
    if (st[s].t) {
        vtg_tracker_destroy(st[s].t);
        st[s].t = NULL;
    }
    for (int k = 0; k < SERVE_SLOTS; k++)
        if (st[s].host_cells[k]) {
            cudaFreeHost(st[s].host_cells[k]);
            st[s].host_cells[k] = NULL;
        }
    st[s].finished = 1;
}

int vtg_serve_run(vtg_ctx *ctx, const struct vtg_serve_cfg *c, struct vtg_serve_stats *out)
{
    if (!ctx || !c || !out || c->nstreams < 1 || !c->streams || !c->frames || c->duration_s <= 0.0 || c->max_batch < 1 ||
        c->inflight < 1 || c->inflight > SERVE_SLOTS)
        return VTG_EINVAL;
    memset(out, 0, sizeof *out);
    const int ns = c->nstreams;
    uint64_t seed = c->seed ? c->seed : 0x9E3779B97F4A7C15ull;
    /* the arrival schedule */
    int total = 0;
    for (int s = 0; s < ns; s++)
        total += c->streams[s].frames;
    struct req *rq = calloc((size_t)total + 1, sizeof *rq);
    struct sstate *st = calloc((size_t)(unsigned)ns, sizeof *st);
    double *lat = calloc((size_t)total + 1, sizeof *lat);
    if (!rq || !st || !lat) {
        free(rq);
        free(st);
        free(lat);
        return VTG_ENOMEM;
    }
    int n = 0;
    for (int s = 0; s < ns; s++) {
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
    /* each stream's requests, in arrival order, are a FIFO over the sorted list: keep per-stream index lists */
    int *order = calloc((size_t)n + 1, sizeof *order);
    int *fill = calloc((size_t)(unsigned)ns, sizeof *fill);
    for (int i = 0; i < n; i++)
        st[rq[i].stream].count++;
    int acc = 0;
    for (int s = 0; s < ns; s++) {
        st[s].first = acc;
        acc += st[s].count;
    }
    for (int i = 0; i < n; i++) {
        const int s = rq[i].stream;
        order[st[s].first + fill[s]++] = i;
    }
    free(fill);
    struct slot sl[SERVE_SLOTS];
    memset(sl, 0, sizeof sl);
    int rc = VTG_OK;
    int max_w = 0, max_h = 0;
    for (int s = 0; s < ns; s++) {
        max_w = c->streams[s].width > (uint32_t)max_w ? (int)c->streams[s].width : max_w;
        max_h = c->streams[s].height > (uint32_t)max_h ? (int)c->streams[s].height : max_h;
    }
    for (int k = 0; k < c->inflight && rc == VTG_OK; k++) {
        sl[k].reqs = calloc((size_t)c->max_batch, sizeof(int));
        rc = vtg_batch_create(ctx, c->max_batch, &sl[k].b);
        if (rc == VTG_OK && c->ncc_share > 0.0f)
            rc = vtg_search_create(ctx, max_w / 2 + 1, max_h / 2 + 1, 32, 21, &sl[k].s);
        if (rc == VTG_OK && cudaMalloc((void **)&sl[k].d_found, sizeof(struct vtg_found)) != cudaSuccess)
            rc = VTG_ENOMEM;
        if (rc == VTG_OK && cudaEventCreateWithFlags(&sl[k].ev, cudaEventDisableTiming) != cudaSuccess)
            rc = VTG_ECUDA;
        if (rc == VTG_OK && cudaEventCreateWithFlags(&sl[k].ev_lk, cudaEventDisableTiming) != cudaSuccess)
            rc = VTG_ECUDA;
    }
    /* a template for the searches: 32 x 21 zero-mean values in 8-bit grey (its contents do not change the cost) */
    float app[32 * 21];
    for (int i = 0; i < 32 * 21; i++)
        app[i] = (float)((int)(urand(&seed) * 255.0) - 127) * 64.0f;
    for (int k = 0; k < c->inflight && rc == VTG_OK; k++)
        if (sl[k].s)
            rc = vtg_search_template(sl[k].s, app, 32, 21, 1.0e9f, VTG_HOST, NULL);
    size_t used0 = vtg_ctx_used(ctx);
    vtg_tracker **tr = calloc((size_t)c->max_batch, sizeof *tr);
    const uint8_t **fr = calloc((size_t)c->max_batch, sizeof *fr);
    int *cur = calloc((size_t)c->max_batch, sizeof *cur);
    int *stream_of = calloc((size_t)c->max_batch, sizeof *stream_of);
    long served = 0, cells = 0, ncc = 0, batches = 0, batched = 0;
    const double t0 = now_s();
    double t_last = t0;
    int next_req = 0;
    while (rc == VTG_OK && served < n) {
        const double now = now_s() - t0;
        if (now > c->duration_s + SERVE_DRAIN_S)
            break;
        int idle = 1;
        /* streams that have begun: admit in start order while the budget allows */
        for (int s = 0; s < ns; s++) {
            if (st[s].admitted || st[s].finished || c->streams[s].start_s > now || st[s].count == 0)
                continue;
            struct vtg_config g = stream_cfg(c, s);
            const size_t need = vtg_tracker_bytes(&g);
            if (c->hbm_budget && vtg_ctx_used(ctx) - used0 + need > c->hbm_budget) {
                if (!st[s].waiting)
                    out->streams_waited++;
                st[s].waiting = 1;
                continue;
            }
            rc = admit(ctx, c, st, s);
            if (rc != VTG_OK)
                break;
            out->streams_admitted++;
            idle = 0;
        }
        /* arrivals */
        while (next_req < n && rq[next_req].t_arrive <= now)
            next_req++;
        /* completions */
        for (int k = 0; k < c->inflight; k++) {
            if (!sl[k].busy)
                continue;
            const cudaError_t q = cudaEventQuery(sl[k].ev);
            if (q == cudaErrorNotReady)
                continue;
            if (q != cudaSuccess) {
                rc = VTG_ECUDA;
                break;
            }
            const double td = now_s() - t0;
            for (int i = 0; i < sl[k].n; i++) {
                struct req *r = &rq[sl[k].reqs[i]];
                r->t_done = td;
                lat[served++] = 1e3 * (td - r->t_arrive);
                struct sstate *ss = &st[r->stream];
                if (c->last_cells && c->last_cells[r->stream])
                    memcpy(c->last_cells[r->stream], ss->host_cells[k], sizeof(struct vtg_cell) * (size_t)ss->cells);
                ss->in_flight--;
                ss->done++;
                cells += ss->cells;
                if (ss->done == ss->count)
                    retire(st, r->stream); /* its memory goes back to the budget */
            }
            sl[k].busy = 0;
            t_last = td + t0;
            idle = 0;
        }
        if (rc != VTG_OK)
            break;
        /* launches: one step per free slot, from what has arrived */
        for (int k = 0; k < c->inflight && rc == VTG_OK; k++) {
            if (sl[k].busy)
                continue;
            int m = 0;
            unsigned wait_slots = 0; /* slots holding the previous frame of a stream in this batch */
            /* the oldest arrived frame of each stream with a slot to spare, oldest first. A stream's next frame may
             * go to one slot while its previous one is on the GPU in another: the new step then waits on the GPU
             * for that slot's work (its pyramid set and result buffers are reused), with no host round trip. */
            for (;;) {
                int best = -1;
                double bt = 1e300;
                for (int s = 0; s < ns; s++) {
                    struct sstate *ss = &st[s];
                    if (!ss->admitted || ss->finished || ss->in_flight >= c->inflight || ss->next >= ss->count)
                        continue;
                    const struct req *r = &rq[order[ss->first + ss->next]];
                    if (r->t_arrive > now || r->t_arrive >= bt)
                        continue;
                    int taken = 0;
                    for (int i = 0; i < m; i++)
                        taken |= stream_of[i] == s;
                    if (taken)
                        continue;
                    best = s;
                    bt = r->t_arrive;
                }
                if (best < 0 || m >= c->max_batch)
                    break;
                struct sstate *ss = &st[best];
                const int ri = order[ss->first + ss->next];
                const int kk = rq[ri].k;
                if (ss->in_flight)
                    wait_slots |= 1u << ss->last_slot;
                stream_of[m] = best;
                sl[k].reqs[m] = ri;
                tr[m] = ss->t;
                cur[m] = (kk + 1) & 1;
                fr[m] = c->frames[2 * best + ((kk + 1) & 1)];
                m++;
                if (c->plain)
                    break; /* the plain form: one frame pair at a time */
            }
            if (m == 0)
                break;
            cudaStream_t bs = (cudaStream_t)vtg_batch_stream(sl[k].b);
            void *waits[SERVE_SLOTS];
            int nw = 0;
            for (int j = 0; j < c->inflight; j++)
                if (wait_slots >> j & 1u)
                    waits[nw++] = (void *)sl[j].ev;
            if (c->plain || m == 1) {
                /* one frame pair: vtg_build + vtg_cells on the slot's stream (the plain form always; the served form
                 * when only one request is ready, where the batched step's tables and persistent grid only add
                 * latency; the cells are the same bits either way) */
                const int s = stream_of[0];
                for (int j = 0; j < nw && rc == VTG_OK; j++)
                    if (cudaStreamWaitEvent(bs, (cudaEvent_t)waits[j], 0) != cudaSuccess)
                        rc = VTG_ECUDA;
                if (rc == VTG_OK)
                    rc = vtg_build(tr[0], cur[0], fr[0], (int)c->streams[s].width, VTG_HOST, bs);
                if (rc == VTG_OK)
                    rc = vtg_cells(tr[0], cur[0] ^ 1, cur[0], st[s].host_cells[k], NULL, VTG_HOST, bs);
            } else {
                rc = vtg_batch_prepare(sl[k].b, 0, m, tr, fr, NULL, VTG_HOST, cur);
                /* the uploads overlap the other slot's step. On the GPU the pyramid waits for that step's LK (it
                 * rewrites the sets that LK read), and the LK launch for that step's result copies (it rewrites the
                 * buffers they read), so those copies overlap this step's pyramid */
                void *waits_lk[SERVE_SLOTS];
                int nl = 0;
                for (int j = 0; j < c->inflight; j++)
                    if (wait_slots >> j & 1u)
                        waits_lk[nl++] = (void *)sl[j].ev_lk;
                if (rc == VTG_OK)
                    rc = vtg_batch_launch_split(sl[k].b, 0, NULL, nl, waits_lk, nw, waits);
                if (rc == VTG_OK && cudaEventRecord(sl[k].ev_lk, bs) != cudaSuccess)
                    rc = VTG_ECUDA;
                for (int i = 0; i < m && rc == VTG_OK; i++)
                    rc = vtg_tracker_results(tr[i], st[stream_of[i]].host_cells[k], NULL, VTG_HOST, bs);
            }
            for (int i = 0; i < m && rc == VTG_OK; i++) {
                if (sl[k].s && urand(&seed) < (double)c->ncc_share) {
                    const float *plane;
                    int lw, lh, lp;
                    const int lev = c->lk.levels > 1 ? 1 : 0;
                    rc = vtg_level_device(tr[i], cur[i], lev, &plane, &lw, &lh, &lp);
                    if (rc == VTG_OK)
                        rc = vtg_search_run(sl[k].s, plane, lw, lh, lp, VTG_PLANE_F32, 1, lw, 1, lh, 2, VTG_NCC_F32,
                                            sl[k].d_found, NULL, NULL, NULL, VTG_DEVICE, bs);
                    ncc++;
                }
                st[stream_of[i]].in_flight++;
                st[stream_of[i]].last_slot = k;
                st[stream_of[i]].next++;
            }
            if (rc == VTG_OK && cudaEventRecord(sl[k].ev, bs) != cudaSuccess)
                rc = VTG_ECUDA;
            /* a one-pair step's LK copies its results on its way out: later steps wait for all of it */
            if (rc == VTG_OK && (c->plain || m == 1) && cudaEventRecord(sl[k].ev_lk, bs) != cudaSuccess)
                rc = VTG_ECUDA;
            sl[k].n = m;
            sl[k].busy = 1;
            batches++;
            batched += m;
            idle = 0;
        }
        int busy = 0;
        for (int k = 0; k < c->inflight; k++)
            busy |= sl[k].busy;
        if (idle && !busy && next_req < n) {
            /* nothing on the GPU and nothing to do until the next arrival: a short pause keeps the loop from burning a
             * core. With a step in flight the loop keeps polling its event, so a completion is seen at once. */
            const double wait = rq[next_req].t_arrive - (now_s() - t0);
            if (wait > 200e-6) {
                struct timespec ts = {0, 100000};
                nanosleep(&ts, NULL);
            }
        }
    }
    /* drain: at most SERVE_DRAIN_S */
    for (int k = 0; k < c->inflight; k++)
        if (sl[k].busy) {
            const double d0 = now_s();
            while (cudaEventQuery(sl[k].ev) == cudaErrorNotReady && now_s() - d0 < SERVE_DRAIN_S)
                ;
        }
    const double wall = t_last - t0 - (n ? rq[0].t_arrive : 0.0);
    qsort(lat, (size_t)served, sizeof *lat, cmp_dbl);
    out->requests = n;
    out->served = served;
    out->cells = cells;
    out->ncc = ncc;
    out->wall_s = wall;
    out->cells_per_s = wall > 0.0 ? (double)cells / wall : 0.0;
    out->p50_ms = served ? lat[(long)(0.50 * (double)(served - 1))] : 0.0;
    out->p99_ms = served ? lat[(long)(0.99 * (double)(served - 1))] : 0.0;
    out->max_ms = served ? lat[served - 1] : 0.0;
    out->mean_batch = batches ? (double)batched / (double)batches : 0.0;
    for (int s = 0; s < ns; s++)
        if (!st[s].admitted && !st[s].finished)
            out->streams_rejected++;
    for (int s = 0; s < ns; s++)
        if (st[s].admitted && !st[s].finished)
            retire(st, s);
    for (int k = 0; k < c->inflight; k++) {
        if (sl[k].b)
            vtg_batch_destroy(sl[k].b);
        if (sl[k].s)
            vtg_search_destroy(sl[k].s);
        if (sl[k].d_found)
            cudaFree(sl[k].d_found);
        if (sl[k].ev)
            cudaEventDestroy(sl[k].ev);
        if (sl[k].ev_lk)
            cudaEventDestroy(sl[k].ev_lk);
        free(sl[k].reqs);
    }
    free(tr);
    free(fr);
    free(cur);
    free(stream_of);
    free(order);
    free(rq);
    free(st);
    free(lat);
    if (rc == VTG_OK && served < n)
        rc = VTG_ETIMEOUT;
    return rc;
}
