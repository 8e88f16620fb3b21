/* server.c -- the request API of the served loop (include/vtg_serve.h): a host pushes each frame of each camera stream
 * as it arrives and polls for its cell records; the server batches what is ready on one GPU.
 *
 * The reference's card session is the precedent (src/card/session_track.c:1-10, 187-225): frames land in device
 * memory as the host publishes them, each is built and tracked when the device has room, results go back with a status
 * word, a LIVE frame goes ahead of the frames queued before it and they are counted as skipped
 * (src/common/vt_proto.h:154, 346), and a session that gets no frame for a while ends (session_track.c:1031-1033).
 *
 * Here a stream is one tracker (its two pyramid sets, staging buffers and cell results on the device) and a FIFO of
 * queued frames on the host. Two batch slots alternate on the GPU. Every poll:
 *   - collects the slots whose step finished (their event), copies each frame's cells to the caller's buffer and
 *     queues its result;
 *   - retires streams that were closed, or idle past idle_timeout_s, once nothing of theirs is queued or in flight;
 *   - fills every free slot with one step: the oldest queued frame of every stream that has room on the GPU (up to
 *     max_batch), a LIVE stream's newest frame in place of its older ones. A step of one frame runs as the plain calls
 *     (vtg_build + vtg_cells), a step of more as one batched step (vtg_batch_*);
 *   - delivers up to `max` results, waiting up to timeout_us for the first.
 * A stream's next frame may go to one slot while its previous one is still on the GPU in the other: the new step's
 * pyramid waits on the GPU for the other step's LK (it rewrites the set that LK reads), and its LK for the other step's
 * result copies (it rewrites the buffers they read), with no host round trip. A stream's cells always flow from the
 * last frame built for it to the new one, so its results are the same bits alone and in any batch. Every host wait is
 * bounded. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime.h>

#include "vtg_serve.h"

#define SRV_SLOTS 2
#define SRV_QMAX 64
#define SRV_WAIT_S 10.0
#define SRV_APP_MAX (32 * 21)

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

struct srv_req {
    int64_t ticket;
    uint64_t tag;
    const uint8_t *frame;
    int stride, flags;
    struct vtg_cell *cells;
    double t_submit;
};

struct srv_stream {
    int used, closing;
    vtg_tracker *t;
    uint32_t w, h, fl;
    int prio, ncells;
    int last_set;  /* the set holding the last frame built */
    int in_flight; /* frames on the GPU */
    int last_slot; /* the slot holding the latest of them */
    struct srv_req q[SRV_QMAX];
    int qh, qn; /* the queue: a ring */
    uint32_t skipped; /* frames skipped since the last one served */
    struct vtg_cell *host_cells[SRV_SLOTS]; /* pinned, one a slot */
    double last_t;                          /* last submission */
    cudaEvent_t first_built;                /* its first frame's pyramid, which its first step waits for on the GPU */
    int first_pending;
};

struct srv_entry {
    int stream, searched;
    uint32_t skipped;
    struct srv_req r;
};

struct srv_slot {
    vtg_batch *b;
    vtg_search *srch;
    int srch_w, srch_h;
    struct vtg_found *d_found, *h_found; /* max_batch each: device, pinned host */
    cudaEvent_t ev;                      /* the step's results are on the host */
    cudaEvent_t ev_lk;                   /* its LK is done: the sets it read are free */
    int busy, n;
    struct srv_entry *e;
};

struct vtg_server {
    vtg_ctx *ctx;
    struct vtg_server_cfg cfg;
    struct srv_stream *st;
    int nst, cap;
    struct srv_slot sl[SRV_SLOTS];
    struct vtg_server_result *ready;
    int nready, rcap;
    int64_t next_ticket;
    long steps, frames;
    float app[SRV_APP_MAX];
    int tw, th, has_template;
    float norm;
    vtg_tracker **tr;
    const uint8_t **fr;
    int *strides, *cur, *pick;
    cudaEvent_t *first_ev; /* a step's new streams' first pyramids: max_batch entries */
    int *cand;             /* streams that can take a step: cap entries */
};

static int push_result(vtg_server *s, const struct vtg_server_result *r)
{
    if (s->nready == s->rcap) {
        const int cap = s->rcap ? 2 * s->rcap : 64;
        struct vtg_server_result *p = realloc(s->ready, sizeof *p * (size_t)cap);
        if (!p)
            return VTG_ENOMEM;
        s->ready = p;
        s->rcap = cap;
    }
    s->ready[s->nready++] = *r;
    return VTG_OK;
}

/* Waits for an event, at most SRV_WAIT_S. */
static int wait_event(cudaEvent_t ev)
{
    const double t0 = now_s();
    for (;;) {
        const cudaError_t q = cudaEventQuery(ev);
        if (q == cudaSuccess)
            return VTG_OK;
        if (q != cudaErrorNotReady)
            return VTG_ECUDA;
        if (now_s() - t0 > SRV_WAIT_S)
            return VTG_ETIMEOUT;
    }
}

static void free_stream(struct srv_stream *ss)
{
    if (ss->first_built)
        cudaEventDestroy(ss->first_built);
    if (ss->t)
        vtg_tracker_destroy(ss->t);
    for (int k = 0; k < SRV_SLOTS; k++)
        if (ss->host_cells[k])
            cudaFreeHost(ss->host_cells[k]);
    memset(ss, 0, sizeof *ss);
}

int vtg_server_create(vtg_ctx *ctx, const struct vtg_server_cfg *cfg, vtg_server **out)
{
    if (!ctx || !cfg || !out || cfg->max_batch < 1 || cfg->max_batch > 512 || cfg->inflight < 1 ||
        cfg->inflight > SRV_SLOTS || cfg->max_queue < 1 || cfg->max_queue > SRV_QMAX || !(cfg->idle_timeout_s >= 0.0))
        return VTG_EINVAL;
    *out = NULL;
    vtg_server *s = calloc(1, sizeof *s);
    if (!s)
        return VTG_ENOMEM;
    s->ctx = ctx;
    s->cfg = *cfg;
    int rc = VTG_OK;
    const int mb = cfg->max_batch;
    s->tr = calloc((size_t)mb, sizeof *s->tr);
    s->fr = calloc((size_t)mb, sizeof *s->fr);
    s->strides = calloc((size_t)mb, sizeof *s->strides);
    s->cur = calloc((size_t)mb, sizeof *s->cur);
    s->pick = calloc((size_t)mb, sizeof *s->pick);
    s->first_ev = calloc((size_t)mb, sizeof *s->first_ev);
    if (!s->tr || !s->fr || !s->strides || !s->cur || !s->pick || !s->first_ev)
        rc = VTG_ENOMEM;
    for (int k = 0; k < cfg->inflight && rc == VTG_OK; k++) {
        struct srv_slot *sl = &s->sl[k];
        sl->e = calloc((size_t)mb, sizeof *sl->e);
        if (!sl->e) {
            rc = VTG_ENOMEM;
            break;
        }
        rc = vtg_batch_create(ctx, mb, &sl->b);
        if (rc == VTG_OK && cudaMalloc((void **)&sl->d_found, sizeof(struct vtg_found) * (size_t)mb) != cudaSuccess)
            rc = VTG_ENOMEM;
        if (rc == VTG_OK &&
            cudaHostAlloc((void **)&sl->h_found, sizeof(struct vtg_found) * (size_t)mb, cudaHostAllocDefault) !=
                cudaSuccess)
            rc = VTG_ENOMEM;
        if (rc == VTG_OK && cudaEventCreateWithFlags(&sl->ev, cudaEventDisableTiming) != cudaSuccess)
            rc = VTG_ECUDA;
        if (rc == VTG_OK && cudaEventCreateWithFlags(&sl->ev_lk, cudaEventDisableTiming) != cudaSuccess)
            rc = VTG_ECUDA;
    }
    if (rc != VTG_OK) {
        vtg_server_destroy(s);
        return rc;
    }
    *out = s;
    return VTG_OK;
}

void vtg_server_destroy(vtg_server *s)
{
    if (!s)
        return;
    for (int k = 0; k < SRV_SLOTS; k++) {
        struct srv_slot *sl = &s->sl[k];
        if (sl->busy)
            wait_event(sl->ev);
        if (sl->b)
            vtg_batch_destroy(sl->b);
        if (sl->srch)
            vtg_search_destroy(sl->srch);
        if (sl->d_found)
            cudaFree(sl->d_found);
        if (sl->h_found)
            cudaFreeHost(sl->h_found);
        if (sl->ev)
            cudaEventDestroy(sl->ev);
        if (sl->ev_lk)
            cudaEventDestroy(sl->ev_lk);
        free(sl->e);
    }
    for (int i = 0; i < s->nst; i++)
        if (s->st[i].used)
            free_stream(&s->st[i]);
    free(s->st);
    free(s->ready);
    free(s->tr);
    free(s->fr);
    free(s->strides);
    free(s->cur);
    free(s->pick);
    free(s->first_ev);
    free(s->cand);
    free(s);
}

static int ensure_search(vtg_server *s, int w, int h);

int vtg_server_template(vtg_server *s, const float *app, int tw, int th, float norm)
{
    if (!s || !app || tw < 8 || th < 1 || (tw % 8) || tw * th > SRV_APP_MAX || !(norm >= 0.0f))
        return VTG_EINVAL;
    memcpy(s->app, app, sizeof(float) * (size_t)(tw * th));
    s->tw = tw;
    s->th = th;
    s->norm = norm;
    s->has_template = 1;
    for (int k = 0; k < SRV_SLOTS; k++)
        if (s->sl[k].srch) {
            if (s->sl[k].busy && wait_event(s->sl[k].ev) != VTG_OK)
                return VTG_ETIMEOUT;
            const int rc = vtg_search_template(s->sl[k].srch, s->app, tw, th, norm, VTG_HOST, NULL);
            if (rc != VTG_OK)
                return rc;
        }
    for (int i = 0; i < s->nst; i++)
        if (s->st[i].used) {
            const int rc = ensure_search(s, (int)s->st[i].w, (int)s->st[i].h);
            if (rc != VTG_OK)
                return rc;
        }
    return VTG_OK;
}

int vtg_server_open(vtg_server *s, uint32_t width, uint32_t height, uint32_t flow_level, int priority,
                    const uint8_t *first, int stride)
{
    if (!s || !first || stride < (int)width || (priority != VTG_PRIO_ORDERED && priority != VTG_PRIO_LIVE))
        return VTG_EINVAL;
    struct vtg_config g = s->cfg.lk;
    g.width = width;
    g.height = height;
    g.flow_level = flow_level;
    int id = -1;
    for (int i = 0; i < s->nst; i++)
        if (!s->st[i].used) {
            id = i;
            break;
        }
    if (id < 0) {
        if (s->nst == s->cap) {
            const int cap = s->cap ? 2 * s->cap : 16;
            struct srv_stream *p = realloc(s->st, sizeof *p * (size_t)cap);
            if (!p)
                return VTG_ENOMEM;
            memset(p + s->cap, 0, sizeof *p * (size_t)(cap - s->cap));
            s->st = p;
            int *c = realloc(s->cand, sizeof *c * (size_t)cap);
            if (!c)
                return VTG_ENOMEM;
            s->cand = c;
            s->cap = cap;
        }
        id = s->nst++;
    }
    struct srv_stream *ss = &s->st[id];
    memset(ss, 0, sizeof *ss);
    int rc = vtg_tracker_create(s->ctx, &g, &ss->t); /* VTG_EINVAL (malformed) or VTG_EBUDGET (no room now) */
    if (rc != VTG_OK) {
        ss->t = NULL;
        return rc;
    }
    int cols = 0, rows = 0;
    vtg_tracker_cells(ss->t, &cols, &rows);
    ss->ncells = cols * rows;
    for (int k = 0; k < s->cfg.inflight && rc == VTG_OK; k++)
        if (cudaHostAlloc((void **)&ss->host_cells[k], sizeof(struct vtg_cell) * (size_t)ss->ncells,
                          cudaHostAllocDefault) != cudaSuccess)
            rc = VTG_ENOMEM;
    /* the first frame's pyramid on the tracker's stream; the stream's first step waits for it on the GPU, so
     * admitting a stream costs the loop no host wait */
    if (rc == VTG_OK && cudaEventCreateWithFlags(&ss->first_built, cudaEventDisableTiming) != cudaSuccess)
        rc = VTG_ECUDA;
    if (rc == VTG_OK)
        rc = vtg_build(ss->t, 0, first, stride, VTG_HOST, NULL);
    if (rc == VTG_OK && cudaEventRecord(ss->first_built, (cudaStream_t)vtg_tracker_stream(ss->t)) != cudaSuccess)
        rc = VTG_ECUDA;
    if (rc == VTG_OK)
        rc = ensure_search(s, (int)width, (int)height); /* searches of this stream allocate nothing in a step */
    if (rc != VTG_OK) {
        free_stream(ss);
        return rc;
    }
    ss->used = 1;
    ss->w = width;
    ss->h = height;
    ss->fl = flow_level;
    ss->prio = priority;
    ss->first_pending = 1;
    ss->last_set = 0;
    ss->last_t = now_s();
    return id;
}

static int retire(vtg_server *s, int id)
{
    free_stream(&s->st[id]);
    (void)s;
    return VTG_OK;
}

int vtg_server_close(vtg_server *s, int stream)
{
    if (!s || stream < 0 || stream >= s->nst || !s->st[stream].used)
        return VTG_EINVAL;
    struct srv_stream *ss = &s->st[stream];
    ss->closing = 1;
    if (ss->qn == 0 && ss->in_flight == 0)
        return retire(s, stream);
    return VTG_OK;
}

int64_t vtg_server_submit(vtg_server *s, int stream, const uint8_t *frame, int stride, struct vtg_cell *cells,
                          uint64_t tag, int flags)
{
    if (!s || stream < 0 || stream >= s->nst || !s->st[stream].used || s->st[stream].closing || !frame ||
        stride < (int)s->st[stream].w || (flags & ~VTG_REQ_SEARCH))
        return VTG_EINVAL;
    struct srv_stream *ss = &s->st[stream];
    if (ss->qn >= s->cfg.max_queue)
        return VTG_EBUSY;
    struct srv_req *r = &ss->q[(ss->qh + ss->qn) % SRV_QMAX];
    r->ticket = s->next_ticket++;
    r->tag = tag;
    r->frame = frame;
    r->stride = stride;
    r->flags = flags;
    r->cells = cells;
    r->t_submit = now_s();
    ss->qn++;
    ss->last_t = r->t_submit;
    return r->ticket;
}

int vtg_server_pending(const vtg_server *s)
{
    if (!s)
        return VTG_EINVAL;
    int n = 0;
    for (int i = 0; i < s->nst; i++)
        if (s->st[i].used)
            n += s->st[i].qn + s->st[i].in_flight;
    return n;
}

int vtg_server_counts(const vtg_server *s, long *steps, long *frames)
{
    if (!s)
        return VTG_EINVAL;
    if (steps)
        *steps = s->steps;
    if (frames)
        *frames = s->frames;
    return VTG_OK;
}

/* The slots whose step finished: results, cells to the callers' buffers, streams closed once drained. */
static int collect(vtg_server *s)
{
    for (int k = 0; k < s->cfg.inflight; k++) {
        struct srv_slot *sl = &s->sl[k];
        if (!sl->busy)
            continue;
        const cudaError_t q = cudaEventQuery(sl->ev);
        if (q == cudaErrorNotReady)
            continue;
        if (q != cudaSuccess)
            return VTG_ECUDA;
        const double td = now_s();
        for (int i = 0; i < sl->n; i++) {
            const struct srv_entry *e = &sl->e[i];
            struct srv_stream *ss = &s->st[e->stream];
            if (e->r.cells)
                memcpy(e->r.cells, ss->host_cells[k], sizeof(struct vtg_cell) * (size_t)ss->ncells);
            struct vtg_server_result r;
            memset(&r, 0, sizeof r);
            r.stream = e->stream;
            r.status = VTG_RES_DONE;
            r.ticket = e->r.ticket;
            r.tag = e->r.tag;
            r.frames_skipped = e->skipped;
            r.searched = e->searched;
            r.latency_ms = 1e3 * (td - e->r.t_submit);
            if (e->searched)
                r.found = sl->h_found[i];
            const int rc = push_result(s, &r);
            if (rc != VTG_OK)
                return rc;
            ss->in_flight--;
            if (ss->closing && ss->qn == 0 && ss->in_flight == 0)
                retire(s, e->stream);
        }
        sl->busy = 0;
        sl->n = 0;
    }
    return VTG_OK;
}

static int retire_idle(vtg_server *s)
{
    if (s->cfg.idle_timeout_s <= 0.0)
        return VTG_OK;
    const double t = now_s();
    for (int i = 0; i < s->nst; i++) {
        struct srv_stream *ss = &s->st[i];
        if (!ss->used || ss->qn || ss->in_flight || t - ss->last_t <= s->cfg.idle_timeout_s)
            continue;
        retire(s, i);
        struct vtg_server_result r;
        memset(&r, 0, sizeof r);
        r.stream = i;
        r.status = VTG_RES_RETIRED;
        r.ticket = -1;
        const int rc = push_result(s, &r);
        if (rc != VTG_OK)
            return rc;
    }
    return VTG_OK;
}

/* The search context of a slot, large enough for a w x h plane. */
static int slot_search(vtg_server *s, struct srv_slot *sl, int w, int h)
{
    if (sl->srch && sl->srch_w >= w && sl->srch_h >= h)
        return VTG_OK;
    const int nw = w > sl->srch_w ? w : sl->srch_w, nh = h > sl->srch_h ? h : sl->srch_h;
    if (sl->srch) {
        vtg_search_destroy(sl->srch);
        sl->srch = NULL;
    }
    int rc = vtg_search_create(s->ctx, nw, nh, 32, 21, &sl->srch);
    if (rc != VTG_OK)
        return rc;
    sl->srch_w = nw;
    sl->srch_h = nh;
    return vtg_search_template(sl->srch, s->app, s->tw, s->th, s->norm, VTG_HOST, NULL);
}

/* Every slot's search context sized for a w x h stream's search plane (its level 1, or level 0 with one level), so
 * that no step allocates: called when a stream is admitted and when the template is set, never inside a step. A busy
 * slot is waited for first, as its context may be replaced. */
static int ensure_search(vtg_server *s, int w, int h)
{
    if (!s->has_template)
        return VTG_OK;
    const int lw = s->cfg.lk.levels > 1 ? (w + 1) / 2 : w, lh = s->cfg.lk.levels > 1 ? (h + 1) / 2 : h;
    for (int k = 0; k < SRV_SLOTS; k++) {
        struct srv_slot *sl = &s->sl[k];
        if (sl->srch && sl->srch_w >= lw && sl->srch_h >= lh)
            continue;
        if (sl->busy && wait_event(sl->ev) != VTG_OK)
            return VTG_ETIMEOUT;
        const int rc = slot_search(s, sl, lw, lh);
        if (rc != VTG_OK)
            return rc;
    }
    return VTG_OK;
}

/* The server whose streams cmp_head orders (qsort takes no context; calls on one server come from one thread). */
static _Thread_local const vtg_server *g_sort_server;

static int cmp_head(const void *a, const void *b)
{
    const struct srv_stream *x = &g_sort_server->st[*(const int *)a], *y = &g_sort_server->st[*(const int *)b];
    const double tx = x->q[x->qh].t_submit, ty = y->q[y->qh].t_submit;
    if (tx != ty)
        return tx < ty ? -1 : 1;
    return *(const int *)a - *(const int *)b;
}

/* Fills free slots with steps of what is queued. */
static int launch(vtg_server *s)
{
    for (int k = 0; k < s->cfg.inflight; k++) {
        struct srv_slot *sl = &s->sl[k];
        if (sl->busy)
            continue;
        /* the streams with a queued frame and room on the GPU, oldest queued frame first */
        int nc = 0;
        for (int i = 0; i < s->nst; i++) {
            const struct srv_stream *ss = &s->st[i];
            if (ss->used && ss->qn > 0 && ss->in_flight < s->cfg.inflight)
                s->cand[nc++] = i;
        }
        if (nc == 0)
            break;
        g_sort_server = s;
        qsort(s->cand, (size_t)nc, sizeof *s->cand, cmp_head);
        const int take = s->cfg.plain ? 1 : (nc < s->cfg.max_batch ? nc : s->cfg.max_batch);
        int m = 0, nfirst = 0;
        unsigned wait_slots = 0;
        for (int c = 0; c < take; c++) {
            const int best = s->cand[c];
            struct srv_stream *ss = &s->st[best];
            /* LIVE: the newest queued frame goes ahead of the older ones, which are skipped */
            while (ss->prio == VTG_PRIO_LIVE && ss->qn > 1) {
                const struct srv_req *old = &ss->q[ss->qh];
                struct vtg_server_result r;
                memset(&r, 0, sizeof r);
                r.stream = best;
                r.status = VTG_RES_SKIPPED;
                r.ticket = old->ticket;
                r.tag = old->tag;
                r.latency_ms = 1e3 * (now_s() - old->t_submit);
                const int rc = push_result(s, &r);
                if (rc != VTG_OK)
                    return rc;
                ss->qh = (ss->qh + 1) % SRV_QMAX;
                ss->qn--;
                ss->skipped++;
            }
            struct srv_entry *e = &sl->e[m];
            e->stream = best;
            e->r = ss->q[ss->qh];
            e->skipped = ss->skipped;
            e->searched = 0;
            if (ss->in_flight)
                wait_slots |= 1u << ss->last_slot;
            if (ss->first_pending)
                s->first_ev[nfirst++] = ss->first_built;
            s->pick[m] = best;
            s->tr[m] = ss->t;
            s->fr[m] = e->r.frame;
            s->strides[m] = e->r.stride;
            s->cur[m] = ss->last_set ^ 1;
            m++;
        }
        cudaStream_t bs = (cudaStream_t)vtg_batch_stream(sl->b);
        void *waits[SRV_SLOTS], *waits_lk[SRV_SLOTS];
        int nw = 0;
        for (int j = 0; j < s->cfg.inflight; j++)
            if (wait_slots >> j & 1u) {
                waits[nw] = (void *)s->sl[j].ev;
                waits_lk[nw] = (void *)s->sl[j].ev_lk;
                nw++;
            }
        int rc = VTG_OK;
        /* the new streams' first pyramids come before anything of this step */
        for (int j = 0; j < nfirst && rc == VTG_OK; j++)
            if (cudaStreamWaitEvent(bs, s->first_ev[j], 0) != cudaSuccess)
                rc = VTG_ECUDA;
        if (m == 1) {
            /* one frame: vtg_build + vtg_cells on the slot's stream, after the other slot's step of this stream */
            for (int j = 0; j < nw && rc == VTG_OK; j++)
                if (cudaStreamWaitEvent(bs, (cudaEvent_t)waits[j], 0) != cudaSuccess)
                    rc = VTG_ECUDA;
            if (rc == VTG_OK)
                rc = vtg_build(s->tr[0], s->cur[0], s->fr[0], s->strides[0], VTG_HOST, bs);
            if (rc == VTG_OK)
                rc = vtg_cells(s->tr[0], s->cur[0] ^ 1, s->cur[0], s->st[s->pick[0]].host_cells[k], NULL, VTG_HOST,
                               bs);
        } else {
            rc = vtg_batch_prepare(sl->b, 0, m, s->tr, s->fr, s->strides, VTG_HOST, s->cur);
            if (rc == VTG_OK)
                rc = vtg_batch_launch_split(sl->b, 0, NULL, nw, waits_lk, nw, waits);
            if (rc == VTG_OK && cudaEventRecord(sl->ev_lk, bs) != cudaSuccess)
                rc = VTG_ECUDA;
            for (int i = 0; i < m && rc == VTG_OK; i++)
                rc = vtg_tracker_results(s->tr[i], s->st[s->pick[i]].host_cells[k], NULL, VTG_HOST, bs);
        }
        /* appearance searches asked for: the new frame's level 1, step 2, the whole plane */
        for (int i = 0; i < m && rc == VTG_OK; i++) {
            struct srv_entry *e = &sl->e[i];
            if (!(e->r.flags & VTG_REQ_SEARCH) || !s->has_template)
                continue;
            const float *plane;
            int lw, lh, lp;
            const int lev = s->cfg.lk.levels > 1 ? 1 : 0;
            rc = vtg_level_device(s->tr[i], s->cur[i], lev, &plane, &lw, &lh, &lp);
            if (rc == VTG_OK)
                rc = slot_search(s, sl, lw, lh);
            if (rc == VTG_OK)
                rc = vtg_search_run(sl->srch, plane, lw, lh, lp, VTG_PLANE_F32, 1, lw, 1, lh, 2, VTG_NCC_F32,
                                    sl->d_found + i, NULL, NULL, NULL, VTG_DEVICE, bs);
            if (rc == VTG_OK && cudaMemcpyAsync(sl->h_found + i, sl->d_found + i, sizeof(struct vtg_found),
                                                cudaMemcpyDeviceToHost, bs) != cudaSuccess)
                rc = VTG_ECUDA;
            e->searched = rc == VTG_OK;
        }
        if (rc == VTG_OK && cudaEventRecord(sl->ev, bs) != cudaSuccess)
            rc = VTG_ECUDA;
        /* a one-frame step copies its results on its LK's way out: later steps wait for all of it */
        if (rc == VTG_OK && m == 1 && cudaEventRecord(sl->ev_lk, bs) != cudaSuccess)
            rc = VTG_ECUDA;
        if (rc != VTG_OK)
            return rc;
        for (int i = 0; i < m; i++) {
            struct srv_stream *ss = &s->st[s->pick[i]];
            ss->qh = (ss->qh + 1) % SRV_QMAX;
            ss->qn--;
            ss->skipped = 0;
            ss->in_flight++;
            ss->last_slot = k;
            ss->last_set = s->cur[i];
            ss->first_pending = 0;
        }
        sl->n = m;
        sl->busy = 1;
        s->steps++;
        s->frames += m;
    }
    return VTG_OK;
}

static int deliver(vtg_server *s, struct vtg_server_result *out, int max)
{
    const int n = s->nready < max ? s->nready : max;
    if (n > 0) {
        memcpy(out, s->ready, sizeof *out * (size_t)n);
        memmove(s->ready, s->ready + n, sizeof *out * (size_t)(s->nready - n));
        s->nready -= n;
    }
    return n;
}

int vtg_server_poll(vtg_server *s, struct vtg_server_result *out, int max, int timeout_us)
{
    if (!s || (max > 0 && !out) || max < 0 || timeout_us < 0)
        return VTG_EINVAL;
    const double t0 = now_s();
    for (;;) {
        int rc = collect(s);
        if (rc == VTG_OK)
            rc = retire_idle(s);
        if (rc == VTG_OK)
            rc = launch(s);
        if (rc != VTG_OK)
            return rc;
        if (s->nready > 0 || max == 0 || now_s() - t0 >= 1e-6 * (double)timeout_us)
            return deliver(s, out, max);
        int busy = 0;
        for (int k = 0; k < s->cfg.inflight; k++)
            busy |= s->sl[k].busy;
        if (!busy) {
            /* nothing on the GPU: nothing can finish before a new submission, so do not burn the core */
            struct timespec ts = {0, 20000};
            nanosleep(&ts, NULL);
        }
    }
}
