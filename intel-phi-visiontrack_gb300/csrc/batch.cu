/* batch.cu -- many streams' frame pairs in one step: the batched form of tk_build + still_vectors.
 *
 * A batch step takes one new frame for each of n trackers (uneven sizes and cell counts) and runs, on one CUDA
 * stream:
 *   - the pyramids of all n frames, one launch per level for all of them (pyr_batch_kernel, a tile table per level);
 *   - the per-cell flow of all n streams in one LK launch (lk_batch_kernel): work items of `chunk` cells of one
 *     stream, taken from a device counter by a persistent grid of warps, so short and long streams balance.
 * The step's tables (per-frame level pointers, tile offsets, per-stream cell grids, item offsets) are prepared once
 * into one of two slots and uploaded; a prepared slot launches with no host work and no host-to-device copy of its
 * own, so it can be captured into a CUDA graph and replayed (two slots: frame k and frame k + 1 write alternate sets).
 * The LK launch's shape (warps per CTA, cells per item, persistent or one warp per item, CTAs per SM) is a tuning
 * choice; vtg_batch_autotune times the candidates on the prepared step and keeps the fastest for that mix of sizes.
 *
 * Every stream's cells are computed by the same code as a single-stream vtg_cells, so a stream's results are the same
 * bits alone and in any batch. */
#include <algorithm>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "vtg_ctx.h"
#include "vtg_internal.cuh"
#include "vtg_tracker.h"

#define BATCH_SLOTS 2

struct BatchSlot {
    PyrJob *d_pyr;
    int *d_tiles;   /* [VTG_MAX_LEVELS][max_jobs + 1] tile offsets per level launch, the fused launch's last */
    LkJob *d_lk;
    int *d_items;   /* [max_jobs + 1] */
    int *d_counter;
    unsigned long long *d_count; /* vtg_batch_count's four totals, in the counter's 256-byte block */
    int njobs, max_levels, items, cells;
    int chunk; /* cells per work item the item table was laid out for */
    int tiled; /* and its order: row-major or 8 x 4 tiles */
    int tiles[VTG_MAX_LEVELS];
    LkPrm prm;
    bool ready;
    /* host frames: copied to the trackers' staging buffers at launch */
    std::vector<const uint8_t *> h_src;
    std::vector<uint8_t *> h_dst;
    std::vector<int> h_stride, h_w, h_h;
    std::string key; /* the size mix, for the tuning cache */
    /* frames under build options: their level 0 is made by launches of their own before the batched pyramid */
    struct Input {
        const uint8_t *src;
        int stride, w, h, opts;
        uint32_t *mm;
        float *l0;
        int pitch0;
    };
    std::vector<Input> inputs;
    cudaGraphExec_t graph;
    bool has_graph;
};

struct vtg_batch {
    vtg_ctx *ctx;
    int max_jobs, sms;
    cudaStream_t stream;
    char *mem;
    size_t bytes;
    BatchSlot slot[BATCH_SLOTS];
    LkTune tune;
    std::map<std::string, LkTune> tuned;
    std::mutex mu;
};

static size_t up256(size_t n) { return (n + 255) & ~(size_t)255; }

static size_t slot_bytes(int max_jobs)
{
    return up256(sizeof(PyrJob) * (size_t)max_jobs) + up256(sizeof(int) * (size_t)VTG_MAX_LEVELS * (max_jobs + 1)) +
           up256(sizeof(LkJob) * (size_t)max_jobs) + up256(sizeof(int) * (size_t)(max_jobs + 1)) + 256;
}

static const LkTune k_default_tune = {16, 2, 1, 1, 1, 1};

#define CU(call)                                                                                                       \
    do {                                                                                                               \
        const cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess) {                                                                                       \
            vtg_set_cuda_error(e_);                                                                                    \
            return VTG_ECUDA;                                                                                          \
        }                                                                                                              \
    } while (0)

extern "C" int vtg_batch_create(vtg_ctx *ctx, int max_jobs, vtg_batch **out)
{
    if (!ctx || !out || max_jobs < 1 || max_jobs > 512)
        return VTG_EINVAL;
    *out = nullptr;
    const size_t bytes = BATCH_SLOTS * slot_bytes(max_jobs);
    const int charged = vtg_ctx_charge(ctx, bytes);
    if (charged != VTG_OK)
        return charged;
    vtg_batch *b = new (std::nothrow) vtg_batch;
    if (!b) {
        vtg_ctx_release(ctx, bytes);
        return VTG_ENOMEM;
    }
    b->ctx = ctx;
    b->max_jobs = max_jobs;
    b->bytes = bytes;
    b->tune = k_default_tune;
    cudaError_t e = cudaSetDevice(vtg_ctx_device(ctx));
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, vtg_ctx_device(ctx));
    if (e == cudaSuccess)
        e = cudaMalloc(&b->mem, bytes);
    if (e == cudaSuccess)
        e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        vtg_ctx_release(ctx, bytes);
        delete b;
        return VTG_ECUDA;
    }
    for (int s = 0; s < BATCH_SLOTS; s++) {
        char *m = b->mem + (size_t)s * slot_bytes(max_jobs);
        BatchSlot &sl = b->slot[s];
        sl.d_pyr = (PyrJob *)m;
        m += up256(sizeof(PyrJob) * (size_t)max_jobs);
        sl.d_tiles = (int *)m;
        m += up256(sizeof(int) * (size_t)VTG_MAX_LEVELS * (max_jobs + 1));
        sl.d_lk = (LkJob *)m;
        m += up256(sizeof(LkJob) * (size_t)max_jobs);
        sl.d_items = (int *)m;
        m += up256(sizeof(int) * (size_t)(max_jobs + 1));
        sl.d_counter = (int *)m;
        sl.d_count = (unsigned long long *)(m + 64);
        sl.ready = false;
        sl.has_graph = false;
        sl.njobs = sl.items = sl.cells = 0;
    }
    vtg_ctx_track(ctx, b->stream, true);
    *out = b;
    return VTG_OK;
}

static void drop_graph(BatchSlot &sl)
{
    if (sl.has_graph) {
        cudaGraphExecDestroy(sl.graph);
        sl.has_graph = false;
    }
}

extern "C" void vtg_batch_destroy(vtg_batch *b)
{
    if (!b)
        return;
    cudaSetDevice(vtg_ctx_device(b->ctx));
    cudaStreamSynchronize(b->stream);
    for (int s = 0; s < BATCH_SLOTS; s++)
        drop_graph(b->slot[s]);
    vtg_ctx_track(b->ctx, b->stream, false);
    cudaStreamDestroy(b->stream);
    cudaFree(b->mem);
    vtg_ctx_release(b->ctx, b->bytes);
    delete b;
}

extern "C" void *vtg_batch_stream(const vtg_batch *b) { return b ? (void *)b->stream : nullptr; }

static bool same_prm(const LkPrm &a, const LkPrm &b)
{
    return a.W == b.W && a.H == b.H && a.max_iter == b.max_iter && a.eps2 == b.eps2 && a.min_eig == b.min_eig &&
           a.max_residual == b.max_residual && a.fb_max2 == b.fb_max2;
}

extern "C" int vtg_batch_prepare(vtg_batch *b, int slot, int n, vtg_tracker *const *trackers,
                                 const uint8_t *const *frames, const int *strides, int where, const int *cur_sets)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || n < 1 || n > b->max_jobs || !trackers || !frames || !cur_sets ||
        (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    BatchSlot &sl = b->slot[slot];
    std::vector<PyrJob> pj((size_t)n);
    std::vector<LkJob> lj((size_t)n);
    std::vector<int> tiles((size_t)VTG_MAX_LEVELS * (n + 1), 0);
    std::vector<int> items((size_t)n + 1, 0);
    sl.h_src.clear();
    sl.h_dst.clear();
    sl.h_stride.clear();
    sl.h_w.clear();
    sl.h_h.clear();
    sl.inputs.clear();
    int max_levels = 1;
    std::vector<std::string> keys;
    for (int j = 0; j < n; j++) {
        vtg_tracker *t = trackers[j];
        if (!t || t->ctx != b->ctx || cur_sets[j] < 0 || cur_sets[j] > 1 || !frames[j])
            return VTG_EINVAL;
        for (int k = 0; k < j; k++)
            if (trackers[k] == t)
                return VTG_EINVAL; /* one frame per stream per step */
        if (j > 0 && !same_prm(t->prm, trackers[0]->prm))
            return VTG_EINVAL; /* one LK setting per batch */
        const int w = (int)t->cfg.width, h = (int)t->cfg.height;
        const int stride = strides ? strides[j] : w;
        if (stride < w)
            return VTG_EINVAL;
        const int cur = cur_sets[j], prev = cur ^ 1;
        PyrJob &p = pj[(size_t)j];
        if (where == VTG_HOST) {
            sl.h_src.push_back(frames[j]);
            uint8_t *stage = t->staging + (size_t)cur * t->staging_set;
            sl.h_dst.push_back(stage);
            sl.h_stride.push_back(stride);
            sl.h_w.push_back(w);
            sl.h_h.push_back(h);
            p.src = stage;
            p.stride = w;
        } else {
            p.src = frames[j];
            p.stride = stride;
        }
        p.w = w;
        p.h = h;
        p.levels = t->levels;
        p.opts = t->build_opts;
        if (p.opts)
            sl.inputs.push_back({p.src, p.stride, w, h, p.opts, t->d_mm + (size_t)cur * VTG_MM_WORDS,
                                 t->sets[cur] + t->loff[0], t->lpitch[0]});
        for (int L = 0; L < VTG_MAX_LEVELS; L++) {
            p.lv[L] = L < t->levels ? t->sets[cur] + t->loff[L] : nullptr;
            p.pitch[L] = t->lpitch[L];
            p.lw[L] = t->lw[L];
            p.lh[L] = t->lh[L];
        }
        max_levels = std::max(max_levels, t->levels);
        const int fl = (int)t->cfg.flow_level;
        LkJob &l = lj[(size_t)j];
        l.I = t->desc + 2 * prev + 1;
        l.J = t->desc + 2 * cur + 1;
        l.top = t->levels - 1 - fl;
        l.g.cols = t->cols;
        l.g.rows = t->rows;
        l.g.n = t->cols * t->rows;
        l.g.cell_w = (int)t->cfg.cell_w;
        l.g.cell_h = (int)t->cfg.cell_h;
        l.base_w = t->lw[fl];
        l.base_h = t->lh[fl];
        l.out = t->d_lk;
        l.cells = t->d_cells;
        keys.push_back(std::to_string(w) + "x" + std::to_string(h) + "/" + std::to_string(l.g.n));
    }
    std::sort(keys.begin(), keys.end());
    std::string key;
    for (auto &k : keys)
        key += k + ";";
    {
        std::lock_guard<std::mutex> g(b->mu);
        auto it = b->tuned.find(key);
        sl.key = key;
        if (it != b->tuned.end())
            b->tune = it->second;
    }
    /* tile offsets per level launch (level L of the launch makes level L, L = 1 also level 0) */
    for (int L = 1; L < VTG_MAX_LEVELS; L++) {
        int acc = 0;
        int *row = tiles.data() + (size_t)(L - 1) * (n + 1);
        for (int j = 0; j < n; j++) {
            row[j] = acc;
            const PyrJob &p = pj[(size_t)j];
            if (L == 1 || L < p.levels)
                acc += vtg_pyr_tiles(p.w, p.h, L);
        }
        row[n] = acc;
        sl.tiles[L - 1] = acc;
    }
    {
        /* the fused launch's blocks (levels 0 .. 3 at once), the last row */
        int acc = 0;
        int *row = tiles.data() + (size_t)(VTG_MAX_LEVELS - 1) * (n + 1);
        for (int j = 0; j < n; j++) {
            row[j] = acc;
            acc += vtg_pyr_fused_tiles(pj[(size_t)j].w, pj[(size_t)j].h);
        }
        row[n] = acc;
        sl.tiles[VTG_MAX_LEVELS - 1] = acc;
    }
    int acc = 0, cells = 0;
    const int chunk = std::max(1, b->tune.chunk), tiled = b->tune.tiled;
    for (int j = 0; j < n; j++) {
        items[(size_t)j] = acc;
        acc += vtg_lk_items(lj[(size_t)j].g.cols, lj[(size_t)j].g.rows, chunk, tiled);
        cells += lj[(size_t)j].g.n;
    }
    items[(size_t)n] = acc;
    sl.items = acc;
    sl.chunk = chunk;
    sl.tiled = tiled;
    sl.cells = cells;
    sl.njobs = n;
    sl.max_levels = max_levels;
    sl.prm = trackers[0]->prm;
    CU(cudaSetDevice(vtg_ctx_device(b->ctx)));
    CU(cudaMemcpyAsync(sl.d_pyr, pj.data(), sizeof(PyrJob) * (size_t)n, cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(sl.d_tiles, tiles.data(), sizeof(int) * tiles.size(), cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(sl.d_lk, lj.data(), sizeof(LkJob) * (size_t)n, cudaMemcpyHostToDevice, b->stream));
    CU(cudaMemcpyAsync(sl.d_items, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice, b->stream));
    CU(cudaStreamSynchronize(b->stream)); /* the host vectors go out of scope */
    drop_graph(sl);
    sl.ready = true;
    return VTG_OK;
}

/* The tiles table is laid out with the prepared n; the batched pyramid launcher wants one row per level. */
static int launch_slot(vtg_batch *b, BatchSlot &sl, cudaStream_t s, int nwait = 0, void *const *wait = nullptr,
                       int nwait_lk = 0, void *const *wait_lk = nullptr)
{
    for (size_t k = 0; k < sl.h_src.size(); k++)
        CU(cudaMemcpy2DAsync(sl.h_dst[k], (size_t)sl.h_w[k], sl.h_src[k], (size_t)sl.h_stride[k], (size_t)sl.h_w[k],
                             (size_t)sl.h_h[k], cudaMemcpyHostToDevice, s));
    /* the uploads went to each frame's own set's staging buffer; the kernels reuse pyramid sets and result buffers */
    for (int k = 0; k < nwait; k++)
        CU(cudaStreamWaitEvent(s, (cudaEvent_t)wait[k], 0));
    for (const BatchSlot::Input &in : sl.inputs)
        CU(vtg_launch_build_input(in.src, in.stride, in.w, in.h, in.opts, in.mm, in.l0, in.pitch0, s));
    /* the pyramid's levels and the LK launch as a chain of programmatic dependents: each starts as the one before
     * drains; the last pyramid launch zeroes the LK launch's work counter */
    CU(vtg_launch_pyramid_batch(sl.d_pyr, sl.d_tiles, sl.tiles, sl.njobs, sl.max_levels, s, sl.d_counter, true,
                                sl.inputs.empty()));
    /* what only the LK launch must wait for (earlier reads of the result buffers it writes) */
    for (int k = 0; k < nwait_lk; k++)
        CU(cudaStreamWaitEvent(s, (cudaEvent_t)wait_lk[k], 0));
    LkTune t = b->tune;
    t.chunk = sl.chunk;
    t.tiled = sl.tiled;
    CU(vtg_launch_lk_batch(sl.d_lk, sl.d_items, sl.njobs, sl.items, sl.prm, t, b->sms, sl.d_counter, s,
                           nwait_lk == 0));
    return VTG_OK;
}

extern "C" int vtg_batch_launch(vtg_batch *b, int slot, void *stream)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready)
        return VTG_EINVAL;
    return launch_slot(b, b->slot[slot], stream ? (cudaStream_t)stream : b->stream);
}

extern "C" int vtg_batch_launch_after(vtg_batch *b, int slot, void *stream, int nwait, void *const *events)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready || nwait < 0 || (nwait > 0 && !events))
        return VTG_EINVAL;
    CU(cudaSetDevice(vtg_ctx_device(b->ctx)));
    return launch_slot(b, b->slot[slot], stream ? (cudaStream_t)stream : b->stream, nwait, events);
}

extern "C" int vtg_batch_launch_split(vtg_batch *b, int slot, void *stream, int nwait, void *const *events,
                                      int nwait_lk, void *const *events_lk)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready || nwait < 0 || (nwait > 0 && !events) ||
        nwait_lk < 0 || (nwait_lk > 0 && !events_lk))
        return VTG_EINVAL;
    CU(cudaSetDevice(vtg_ctx_device(b->ctx)));
    return launch_slot(b, b->slot[slot], stream ? (cudaStream_t)stream : b->stream, nwait, events, nwait_lk,
                       events_lk);
}

extern "C" int vtg_batch_capture(vtg_batch *b, int slot)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready)
        return VTG_EINVAL;
    BatchSlot &sl = b->slot[slot];
    drop_graph(sl);
    cudaGraph_t g;
    CU(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = launch_slot(b, sl, b->stream);
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc != VTG_OK)
        return rc;
    CU(e);
    const cudaError_t e2 = cudaGraphInstantiate(&sl.graph, g, 0);
    cudaGraphDestroy(g);
    CU(e2);
    sl.has_graph = true;
    return VTG_OK;
}

extern "C" int vtg_batch_replay(vtg_batch *b, int slot, void *stream)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].has_graph)
        return VTG_EINVAL;
    CU(cudaGraphLaunch(b->slot[slot].graph, stream ? (cudaStream_t)stream : b->stream));
    return VTG_OK;
}

extern "C" int vtg_batch_cells(const vtg_batch *b, int slot)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready)
        return VTG_EINVAL;
    return b->slot[slot].cells;
}

extern "C" int vtg_batch_set_tune(vtg_batch *b, const struct vtg_tune *t)
{
    if (!b || !t || (t->block_warps != 4 && t->block_warps != 8 && t->block_warps != 16) || t->chunk < 1 ||
        t->chunk > 64 || t->ctas_per_sm < 1 || t->ctas_per_sm > 8)
        return VTG_EINVAL;
    if (t->tiled && (!t->persistent || 32 % t->chunk))
        return VTG_EINVAL;
    if (t->tsmem && (!t->persistent || t->ctas_per_sm > (t->block_warps == 4 ? 5 : t->block_warps == 8 ? 3 : 1)))
        return VTG_EINVAL;
    std::lock_guard<std::mutex> g(b->mu);
    b->tune.block_warps = t->block_warps;
    b->tune.chunk = t->chunk;
    b->tune.persistent = t->persistent ? 1 : 0;
    b->tune.ctas_per_sm = t->ctas_per_sm;
    b->tune.tsmem = t->tsmem ? 1 : 0;
    b->tune.tiled = t->tiled ? 1 : 0;
    return VTG_OK;
}

extern "C" int vtg_batch_get_tune(const vtg_batch *b, struct vtg_tune *t)
{
    if (!b || !t)
        return VTG_EINVAL;
    t->block_warps = b->tune.block_warps;
    t->chunk = b->tune.chunk;
    t->persistent = b->tune.persistent;
    t->ctas_per_sm = b->tune.ctas_per_sm;
    t->tsmem = b->tune.tsmem;
    t->tiled = b->tune.tiled;
    return VTG_OK;
}

/* Re-lays the prepared slot's item table for a new chunk and order (items depend on them). */
static int relay_items(vtg_batch *b, BatchSlot &sl, int chunk, int tiled)
{
    std::vector<LkJob> lj((size_t)sl.njobs);
    CU(cudaMemcpyAsync(lj.data(), sl.d_lk, sizeof(LkJob) * (size_t)sl.njobs, cudaMemcpyDeviceToHost, b->stream));
    CU(cudaStreamSynchronize(b->stream));
    std::vector<int> items((size_t)sl.njobs + 1);
    int acc = 0;
    for (int j = 0; j < sl.njobs; j++) {
        items[(size_t)j] = acc;
        acc += vtg_lk_items(lj[(size_t)j].g.cols, lj[(size_t)j].g.rows, chunk, tiled);
    }
    items[(size_t)sl.njobs] = acc;
    sl.items = acc;
    sl.chunk = chunk;
    sl.tiled = tiled;
    CU(cudaMemcpyAsync(sl.d_items, items.data(), sizeof(int) * items.size(), cudaMemcpyHostToDevice, b->stream));
    CU(cudaStreamSynchronize(b->stream));
    drop_graph(sl);
    return VTG_OK;
}

extern "C" int vtg_batch_autotune(vtg_batch *b, int slot, int reps, struct vtg_tune *best, float *best_ms,
                                  float *default_ms)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready || reps < 1)
        return VTG_EINVAL;
    BatchSlot &sl = b->slot[slot];
    std::vector<LkTune> cands;
    cands.push_back(k_default_tune);
    for (int pers = 0; pers <= 1; pers++)
        for (int warps : {4, 8, 16})
            for (int chunk : {1, 2, 4, 8}) {
                if (pers) {
                    const int max_ctas = 16 / warps; /* 128 registers a thread: 16 warps an SM */
                    for (int c = 1; c <= max_ctas; c *= 2)
                        for (int tl = 0; tl <= 1; tl++)
                            cands.push_back({warps, chunk, 1, c, 0, tl});
                } else if (chunk <= 2) {
                    cands.push_back({warps, chunk, 0, 1, 0, 0});
                }
            }
    /* the template's intensities in shared memory: 20 or 24 warps an SM */
    for (int chunk : {1, 2, 4})
        for (int tl = 0; tl <= 1; tl++) {
            cands.push_back({4, chunk, 1, 5, 1, tl});
            cands.push_back({8, chunk, 1, 3, 1, tl});
            cands.push_back({16, chunk, 1, 1, 1, tl});
        }
    cudaEvent_t e0, e1;
    CU(cudaEventCreate(&e0));
    CU(cudaEventCreate(&e1));
    float best_t = 1e30f, def_t = 0.0f;
    LkTune best_c = k_default_tune;
    int cur_chunk = -1, cur_tiled = -1;
    for (size_t ci = 0; ci < cands.size(); ci++) {
        const LkTune &c = cands[ci];
        if (c.chunk != cur_chunk || c.tiled != cur_tiled) {
            const int rc = relay_items(b, sl, c.chunk, c.tiled);
            if (rc != VTG_OK)
                return rc;
            cur_chunk = c.chunk;
            cur_tiled = c.tiled;
        }
        b->tune = c;
        std::vector<float> t;
        for (int r = 0; r < reps + 1; r++) {
            CU(cudaEventRecord(e0, b->stream));
            const int rc = launch_slot(b, sl, b->stream);
            if (rc != VTG_OK)
                return rc;
            CU(cudaEventRecord(e1, b->stream));
            CU(cudaEventSynchronize(e1));
            float ms = 0.0f;
            CU(cudaEventElapsedTime(&ms, e0, e1));
            if (r > 0)
                t.push_back(ms); /* the first run warms up */
        }
        std::sort(t.begin(), t.end());
        const float med = t[t.size() / 2];
        if (ci == 0)
            def_t = med;
        if (med < best_t) {
            best_t = med;
            best_c = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    {
        std::lock_guard<std::mutex> g(b->mu);
        b->tune = best_c;
        b->tuned[sl.key] = best_c;
    }
    const int rc = relay_items(b, sl, best_c.chunk, best_c.tiled);
    if (rc != VTG_OK)
        return rc;
    if (best) {
        best->block_warps = best_c.block_warps;
        best->chunk = best_c.chunk;
        best->persistent = best_c.persistent;
        best->ctas_per_sm = best_c.ctas_per_sm;
        best->tsmem = best_c.tsmem;
        best->tiled = best_c.tiled;
    }
    if (best_ms)
        *best_ms = best_t;
    if (default_ms)
        *default_ms = def_t;
    return VTG_OK;
}

extern "C" int vtg_tracker_results(vtg_tracker *t, struct vtg_cell *cells, struct vtg_lk_out *lk, int where,
                                   void *stream)
{
    if (!t || (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t s = stream ? (cudaStream_t)stream : t->stream;
    const size_t n = (size_t)t->cols * t->rows;
    const cudaMemcpyKind k = where == VTG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (cells)
        CU(cudaMemcpyAsync(cells, t->d_cells, n * sizeof(vtg_cell), k, s));
    if (lk)
        CU(cudaMemcpyAsync(lk, t->d_lk, n * sizeof(vtg_lk_out), k, s));
    return VTG_OK;
}

extern "C" int vtg_batch_profile(vtg_batch *b, int slot, int reps, float *pyr_ms, float *lk_ms)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready || reps < 1)
        return VTG_EINVAL;
    BatchSlot &sl = b->slot[slot];
    cudaEvent_t e[3];
    for (int i = 0; i < 3; i++)
        CU(cudaEventCreate(&e[i]));
    std::vector<float> tp, tl;
    LkTune t = b->tune;
    t.chunk = sl.chunk;
    t.tiled = sl.tiled;
    for (int r = 0; r < reps; r++) {
        CU(cudaEventRecord(e[0], b->stream));
        for (size_t k = 0; k < sl.h_src.size(); k++)
            CU(cudaMemcpy2DAsync(sl.h_dst[k], (size_t)sl.h_w[k], sl.h_src[k], (size_t)sl.h_stride[k], (size_t)sl.h_w[k],
                                 (size_t)sl.h_h[k], cudaMemcpyHostToDevice, b->stream));
        for (const BatchSlot::Input &in : sl.inputs)
            CU(vtg_launch_build_input(in.src, in.stride, in.w, in.h, in.opts, in.mm, in.l0, in.pitch0, b->stream));
        CU(vtg_launch_pyramid_batch(sl.d_pyr, sl.d_tiles, sl.tiles, sl.njobs, sl.max_levels, b->stream, nullptr, false,
                                    sl.inputs.empty()));
        CU(cudaMemsetAsync(sl.d_counter, 0, sizeof(int), b->stream));
        CU(cudaEventRecord(e[1], b->stream));
        CU(vtg_launch_lk_batch(sl.d_lk, sl.d_items, sl.njobs, sl.items, sl.prm, t, b->sms, sl.d_counter, b->stream));
        CU(cudaEventRecord(e[2], b->stream));
        CU(cudaEventSynchronize(e[2]));
        float a = 0.0f, c = 0.0f;
        CU(cudaEventElapsedTime(&a, e[0], e[1]));
        CU(cudaEventElapsedTime(&c, e[1], e[2]));
        tp.push_back(a);
        tl.push_back(c);
    }
    for (int i = 0; i < 3; i++)
        cudaEventDestroy(e[i]);
    std::sort(tp.begin(), tp.end());
    std::sort(tl.begin(), tl.end());
    if (pyr_ms)
        *pyr_ms = tp[tp.size() / 2];
    if (lk_ms)
        *lk_ms = tl[tl.size() / 2];
    return VTG_OK;
}

extern "C" int vtg_batch_count(vtg_batch *b, int slot, uint64_t *counts)
{
    if (!b || slot < 0 || slot >= BATCH_SLOTS || !b->slot[slot].ready || !counts)
        return VTG_EINVAL;
    BatchSlot &sl = b->slot[slot];
    LkTune t = b->tune;
    t.chunk = sl.chunk;
    t.tiled = sl.tiled;
    CU(cudaSetDevice(vtg_ctx_device(b->ctx)));
    CU(cudaMemsetAsync(sl.d_count, 0, 4 * sizeof(unsigned long long), b->stream));
    CU(cudaMemsetAsync(sl.d_counter, 0, sizeof(int), b->stream));
    CU(vtg_launch_lk_batch(sl.d_lk, sl.d_items, sl.njobs, sl.items, sl.prm, t, b->sms, sl.d_counter, b->stream, false,
                           sl.d_count));
    unsigned long long h[4];
    CU(cudaMemcpyAsync(h, sl.d_count, sizeof h, cudaMemcpyDeviceToHost, b->stream));
    CU(cudaStreamSynchronize(b->stream));
    for (int k = 0; k < 4; k++)
        counts[k] = h[k];
    return VTG_OK;
}
