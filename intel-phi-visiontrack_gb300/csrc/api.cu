/* api.cu -- the C ABI (include/vtg.h): contexts, trackers, and the hot-path entry points.
 *
 * A tracker is one camera stream's device-resident state, the GPU form of the reference's struct tracker
 * (src/kern/track.c:75-160) as far as this path goes: two pyramid sets (the ring tk_sets describes), the frame staging
 * buffer, the pyramids' descriptors, and the cell results, all in one device allocation charged to the context's
 * budget, with the build options' scratch and the appearance template's. Each tracker owns a CUDA stream; its work is
 * ordered there. The appearance template cut (store_appearance, track.c:935-974) is here too, as one warp's kernel on
 * the resident pyramid. */
#include <chrono>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "vtg_ctx.h"
#include "vtg_internal.cuh"
#include "vtg_tracker.h"
#include "x87.cuh"

static thread_local int g_last_cuda = 0;

void vtg_set_cuda_error(cudaError_t e) { g_last_cuda = (int)e; }

#define CU(call)                                                                                                       \
    do {                                                                                                               \
        const cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess) {                                                                                       \
            g_last_cuda = (int)e_;                                                                                     \
            return VTG_ECUDA;                                                                                          \
        }                                                                                                              \
    } while (0)

struct vtg_ctx {
    int device;
    size_t budget, used;
    std::mutex mu;
    std::vector<vtg_tracker *> trackers;
    std::vector<cudaStream_t> streams; /* of the other objects (search contexts, batches) */
};

int vtg_ctx_charge(vtg_ctx *ctx, size_t bytes)
{
    std::lock_guard<std::mutex> g(ctx->mu);
    if (ctx->budget && ctx->used + bytes > ctx->budget)
        return VTG_EBUDGET;
    ctx->used += bytes;
    return VTG_OK;
}

void vtg_ctx_release(vtg_ctx *ctx, size_t bytes)
{
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->used -= bytes;
}

int vtg_ctx_device(const vtg_ctx *ctx) { return ctx->device; }

void vtg_ctx_track(vtg_ctx *ctx, cudaStream_t s, bool add)
{
    std::lock_guard<std::mutex> g(ctx->mu);
    if (add) {
        ctx->streams.push_back(s);
        return;
    }
    for (size_t i = 0; i < ctx->streams.size(); i++)
        if (ctx->streams[i] == s) {
            ctx->streams.erase(ctx->streams.begin() + (long)i);
            return;
        }
}



extern "C" const char *vtg_strerror(int status)
{
    switch (status) {
    case VTG_OK: return "ok";
    case VTG_EINVAL: return "invalid argument or configuration";
    case VTG_ENOMEM: return "out of memory";
    case VTG_ECUDA: return "CUDA error";
    case VTG_ETIMEOUT: return "timed out";
    case VTG_EBUSY: return "busy";
    case VTG_ENODEV: return "no CUDA device";
    case VTG_EBUDGET: return "over the device-memory budget";
    default: return "unknown status";
    }
}

extern "C" int vtg_last_cuda_error(void) { return g_last_cuda; }

extern "C" int vtg_ctx_create(int device, size_t hbm_budget, vtg_ctx **out)
{
    if (!out)
        return VTG_EINVAL;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0)
        return VTG_ENODEV;
    if (device < 0 || device >= n)
        return VTG_EINVAL;
    CU(cudaSetDevice(device));
    CU(cudaFree(nullptr)); /* the primary context, now */
    vtg_ctx *c = new (std::nothrow) vtg_ctx;
    if (!c)
        return VTG_ENOMEM;
    c->device = device;
    c->budget = hbm_budget;
    c->used = 0;
    *out = c;
    return VTG_OK;
}

extern "C" void vtg_ctx_destroy(vtg_ctx *ctx)
{
    if (!ctx)
        return;
    std::vector<vtg_tracker *> left;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        left = ctx->trackers;
    }
    for (vtg_tracker *t : left)
        vtg_tracker_destroy(t);
    delete ctx;
}

extern "C" size_t vtg_ctx_used(const vtg_ctx *ctx) { return ctx ? ctx->used : 0; }

extern "C" int vtg_ctx_sync(vtg_ctx *ctx, int timeout_ms)
{
    if (!ctx)
        return VTG_EINVAL;
    CU(cudaSetDevice(ctx->device));
    std::vector<cudaStream_t> streams;
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        for (vtg_tracker *t : ctx->trackers)
            streams.push_back(t->stream);
        for (cudaStream_t s : ctx->streams)
            streams.push_back(s);
    }
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
    for (cudaStream_t s : streams) {
        for (;;) {
            const cudaError_t e = cudaStreamQuery(s);
            if (e == cudaSuccess)
                break;
            if (e != cudaErrorNotReady) {
                g_last_cuda = (int)e;
                return VTG_ECUDA;
            }
            if (std::chrono::steady_clock::now() > deadline)
                return VTG_ETIMEOUT;
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
    }
    return VTG_OK;
}

/* ---- trackers ---- */

static int check_config(const vtg_config *c)
{
    if (!c || c->width < 32 || c->height < 32 || c->width > 16384 || c->height > 16384)
        return VTG_EINVAL;
    if (c->levels < 1 || c->levels > VTG_MAX_LEVELS || c->flow_level >= c->levels)
        return VTG_EINVAL;
    if (c->patch_w < 5 || c->patch_w > VTG_MAX_PATCH_W || c->patch_h < 5 || c->patch_h > VTG_MAX_PATCH_H)
        return VTG_EINVAL;
    if (c->max_iter < 1 || c->max_iter > 1000 || !(c->eps >= 0.0f) || !(c->fb_max >= 0.0f))
        return VTG_EINVAL;
    if (c->cell_w < 1 || c->cell_h < 1 || c->cell_w > 256 || c->cell_h > 256)
        return VTG_EINVAL;
    return VTG_OK;
}

struct Layout {
    int lw[VTG_MAX_LEVELS], lh[VTG_MAX_LEVELS], lpitch[VTG_MAX_LEVELS];
    size_t loff[VTG_MAX_LEVELS], set_floats, staging_off, desc_off, lk_off, cells_off, mm_off, app_off, bytes;
    int cols, rows;
};

static size_t up256(size_t n) { return (n + 255) & ~(size_t)255; }

static void layout(const vtg_config *c, Layout *L)
{
    int w = (int)c->width, h = (int)c->height;
    size_t off = 0;
    for (int i = 0; i < (int)c->levels; i++) {
        L->lw[i] = w;
        L->lh[i] = h;
        L->lpitch[i] = vtg_pitch(w);
        L->loff[i] = off;
        off += up256((size_t)L->lpitch[i] * (size_t)h * sizeof(float)) / sizeof(float);
        w = (w + 1) / 2;
        h = (h + 1) / 2;
    }
    L->set_floats = off;
    const int fw = L->lw[c->flow_level], fh = L->lh[c->flow_level];
    L->cols = (fw + (int)c->cell_w - 1) / (int)c->cell_w;
    L->rows = (fh + (int)c->cell_h - 1) / (int)c->cell_h;
    size_t b = 2 * off * sizeof(float);
    /* one staging buffer a set: a frame's upload never waits for the previous frame's pyramid to finish reading */
    L->staging_off = b;
    b += 2 * up256((size_t)c->width * c->height);
    L->desc_off = b;
    b += up256(4 * sizeof(DevPyr));
    L->lk_off = b;
    const size_t n = (size_t)L->cols * L->rows;
    b += up256(n * sizeof(vtg_lk_out));
    L->cells_off = b;
    b += up256(n * sizeof(vtg_cell));
    L->mm_off = b;
    b += up256(2 * VTG_MM_WORDS * sizeof(uint32_t)); /* one block a set, like the staging */
    L->app_off = b;
    b += up256((VTG_APP_W * VTG_APP_H + 1) * sizeof(float));
    L->bytes = b;
}

extern "C" size_t vtg_tracker_bytes(const vtg_config *cfg)
{
    if (check_config(cfg) != VTG_OK)
        return 0;
    Layout L;
    layout(cfg, &L);
    return L.bytes;
}

static DevPyr pyr_from(const vtg_tracker *t, int set, int from)
{
    DevPyr p;
    p.levels = t->levels - from;
    for (int i = 0; i < VTG_MAX_LEVELS; i++) {
        const int L = from + i;
        if (L < t->levels) {
            p.l[i].p = t->sets[set] + t->loff[L];
            p.l[i].w = t->lw[L];
            p.l[i].h = t->lh[L];
            p.l[i].pitch = t->lpitch[L];
        } else {
            p.l[i].p = nullptr;
            p.l[i].w = p.l[i].h = p.l[i].pitch = 0;
        }
    }
    return p;
}

extern "C" int vtg_tracker_create(vtg_ctx *ctx, const vtg_config *cfg, vtg_tracker **out)
{
    if (!ctx || !out)
        return VTG_EINVAL;
    *out = nullptr;
    const int chk = check_config(cfg);
    if (chk != VTG_OK)
        return chk;
    Layout L;
    layout(cfg, &L);
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        if (ctx->budget && ctx->used + L.bytes > ctx->budget)
            return VTG_EBUDGET;
        ctx->used += L.bytes;
    }
    vtg_tracker *t = new (std::nothrow) vtg_tracker;
    auto undo = [&](int code) {
        std::lock_guard<std::mutex> g(ctx->mu);
        ctx->used -= L.bytes;
        delete t;
        return code;
    };
    if (!t)
        return undo(VTG_ENOMEM);
    t->ctx = ctx;
    t->cfg = *cfg;
    t->levels = (int)cfg->levels;
    t->cols = L.cols;
    t->rows = L.rows;
    for (int i = 0; i < VTG_MAX_LEVELS; i++) {
        t->lw[i] = i < t->levels ? L.lw[i] : 0;
        t->lh[i] = i < t->levels ? L.lh[i] : 0;
        t->lpitch[i] = i < t->levels ? L.lpitch[i] : 0;
        t->loff[i] = i < t->levels ? L.loff[i] : 0;
    }
    t->set_floats = L.set_floats;
    t->bytes = L.bytes;
    if (cudaSetDevice(ctx->device) != cudaSuccess)
        return undo(VTG_ECUDA);
    cudaError_t e = cudaMalloc(&t->mem, L.bytes);
    if (e != cudaSuccess) {
        g_last_cuda = (int)e;
        return undo(VTG_ENOMEM);
    }
    e = cudaStreamCreateWithFlags(&t->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaFree(t->mem);
        g_last_cuda = (int)e;
        return undo(VTG_ECUDA);
    }
    t->sets[0] = (float *)t->mem;
    t->sets[1] = (float *)t->mem + L.set_floats;
    t->staging = (uint8_t *)(t->mem + L.staging_off);
    t->staging_set = up256((size_t)cfg->width * cfg->height);
    t->desc = (DevPyr *)(t->mem + L.desc_off);
    t->d_lk = (vtg_lk_out *)(t->mem + L.lk_off);
    t->d_cells = (vtg_cell *)(t->mem + L.cells_off);
    t->d_mm = (uint32_t *)(t->mem + L.mm_off);
    t->d_app = (float *)(t->mem + L.app_off);
    t->build_opts = 0;
    t->point_warps = 0;
    DevPyr d[4] = {pyr_from(t, 0, 0), pyr_from(t, 0, (int)cfg->flow_level), pyr_from(t, 1, 0),
                   pyr_from(t, 1, (int)cfg->flow_level)};
    /* Pyramid planes start zeroed, as the reference's do (track.c:493-503). */
    e = cudaMemsetAsync(t->mem, 0, 2 * L.set_floats * sizeof(float), t->stream);
    if (e == cudaSuccess) /* the build options' ticket starts at 0 */
        e = cudaMemsetAsync(t->d_mm, 0, 2 * VTG_MM_WORDS * sizeof(uint32_t), t->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(t->desc, d, sizeof d, cudaMemcpyHostToDevice, t->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(t->stream);
    if (e != cudaSuccess) {
        cudaStreamDestroy(t->stream);
        cudaFree(t->mem);
        g_last_cuda = (int)e;
        return undo(VTG_ECUDA);
    }
    t->prm.W = (int)cfg->patch_w;
    t->prm.H = (int)cfg->patch_h;
    t->prm.max_iter = (int)cfg->max_iter;
    t->prm.eps2 = cfg->eps * cfg->eps;
    t->prm.min_eig = cfg->min_eig;
    t->prm.max_residual = cfg->max_residual;
    t->prm.fb_max2 = cfg->fb_max > 0.0f ? cfg->fb_max * cfg->fb_max : 0.0f;
    t->prm.area = (float)(cfg->patch_w * cfg->patch_h);
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        ctx->trackers.push_back(t);
    }
    *out = t;
    return VTG_OK;
}

extern "C" void vtg_tracker_destroy(vtg_tracker *t)
{
    if (!t)
        return;
    vtg_ctx *ctx = t->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(t->stream);
    cudaStreamDestroy(t->stream);
    cudaFree(t->mem);
    {
        std::lock_guard<std::mutex> g(ctx->mu);
        ctx->used -= t->bytes;
        for (size_t i = 0; i < ctx->trackers.size(); i++)
            if (ctx->trackers[i] == t) {
                ctx->trackers.erase(ctx->trackers.begin() + (long)i);
                break;
            }
    }
    delete t;
}

extern "C" int vtg_tracker_sets(const vtg_tracker *t) { return t ? 2 : VTG_EINVAL; }

extern "C" int vtg_tracker_cells(const vtg_tracker *t, int *cols, int *rows)
{
    if (!t)
        return VTG_EINVAL;
    if (cols)
        *cols = t->cols;
    if (rows)
        *rows = t->rows;
    return t->cols * t->rows;
}

extern "C" void *vtg_tracker_stream(const vtg_tracker *t) { return t ? (void *)t->stream : nullptr; }

extern "C" int vtg_level_size(const vtg_tracker *t, int level, int *w, int *h)
{
    if (!t || level < 0 || level >= t->levels)
        return VTG_EINVAL;
    if (w)
        *w = t->lw[level];
    if (h)
        *h = t->lh[level];
    return VTG_OK;
}

static cudaStream_t pick(const vtg_tracker *t, void *stream) { return stream ? (cudaStream_t)stream : t->stream; }

/* ---- the hot path ---- */

extern "C" int vtg_build(vtg_tracker *t, int set, const uint8_t *frame, int stride, int where, void *stream)
{
    if (!t || !frame || set < 0 || set > 1 || stride < (int)t->cfg.width || (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t s = pick(t, stream);
    const int w = (int)t->cfg.width, h = (int)t->cfg.height;
    const uint8_t *src = frame;
    int sstride = stride;
    if (where == VTG_HOST) {
        uint8_t *stage = t->staging + (size_t)set * t->staging_set;
        CU(cudaMemcpy2DAsync(stage, (size_t)w, frame, (size_t)stride, (size_t)w, (size_t)h, cudaMemcpyHostToDevice, s));
        src = stage;
        sstride = w;
    }
    float *lv[VTG_MAX_LEVELS];
    for (int i = 0; i < t->levels; i++)
        lv[i] = t->sets[set] + t->loff[i];
    CU(vtg_launch_pyramid_opts(src, sstride, w, h, lv, t->lpitch, t->levels, t->build_opts,
                               t->d_mm + (size_t)set * VTG_MM_WORDS, s));
    return VTG_OK;
}

extern "C" int vtg_tracker_set_build(vtg_tracker *t, int flags)
{
    if (!t || (flags & ~(VTG_BUILD_CONTRAST | VTG_BUILD_PRE_GAUSS)))
        return VTG_EINVAL;
    t->build_opts = flags;
    return VTG_OK;
}

extern "C" int vtg_tracker_build_flags(const vtg_tracker *t) { return t ? t->build_opts : 0; }

extern "C" int vtg_tracker_set_point_warps(vtg_tracker *t, int warps)
{
    if (!t || warps < 0 || warps > 2)
        return VTG_EINVAL;
    t->point_warps = warps;
    return VTG_OK;
}

extern "C" int vtg_cells(vtg_tracker *t, int prev, int cur, vtg_cell *cells, vtg_lk_out *lk, int where, void *stream)
{
    if (!t || prev < 0 || prev > 1 || cur < 0 || cur > 1 || (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t s = pick(t, stream);
    const int fl = (int)t->cfg.flow_level;
    CellGrid g;
    g.cols = t->cols;
    g.rows = t->rows;
    g.n = t->cols * t->rows;
    g.cell_w = (int)t->cfg.cell_w;
    g.cell_h = (int)t->cfg.cell_h;
    vtg_cell *dc = where == VTG_DEVICE ? cells : (cells ? t->d_cells : nullptr);
    vtg_lk_out *dl = where == VTG_DEVICE ? lk : (lk ? t->d_lk : nullptr);
    CU(vtg_launch_cells(t->desc + 2 * prev + 1, t->desc + 2 * cur + 1, t->levels - 1 - fl, t->prm, g, t->lw[fl], t->lh[fl],
                        dl, dc, s));
    if (where == VTG_HOST) {
        if (cells)
            CU(cudaMemcpyAsync(cells, t->d_cells, (size_t)g.n * sizeof(vtg_cell), cudaMemcpyDeviceToHost, s));
        if (lk)
            CU(cudaMemcpyAsync(lk, t->d_lk, (size_t)g.n * sizeof(vtg_lk_out), cudaMemcpyDeviceToHost, s));
    }
    return VTG_OK;
}

extern "C" int vtg_points(vtg_tracker *t, int prev, int cur, int top, int n, const float *xs, const float *ys,
                          const float *gx, const float *gy, vtg_lk_out *out, int where, void *stream)
{
    if (!t || prev < 0 || prev > 1 || cur < 0 || cur > 1 || n < 0 || (n > 0 && (!xs || !ys || !out)) ||
        (where != VTG_HOST && where != VTG_DEVICE) || top < -1 || top >= t->levels)
        return VTG_EINVAL;
    if (n == 0)
        return VTG_OK;
    const cudaStream_t s = pick(t, stream);
    if (top < 0)
        top = t->levels - 1;
    if (where == VTG_DEVICE) {
        CU(vtg_launch_points(t->desc + 2 * prev, t->desc + 2 * cur, top, t->prm, n, xs, ys, gx, gy, out, s,
                             t->point_warps));
        return VTG_OK;
    }
    /* Host arrays: one stream-ordered scratch allocation for the call. */
    const size_t fbytes = (size_t)n * sizeof(float);
    char *d = nullptr;
    CU(cudaMallocAsync((void **)&d, 4 * fbytes + (size_t)n * sizeof(vtg_lk_out), s));
    float *dx = (float *)d, *dy = dx + n, *dgx = gx ? dy + n : nullptr, *dgy = gy ? dy + 2 * (size_t)n : nullptr;
    vtg_lk_out *dout = (vtg_lk_out *)(d + 4 * fbytes);
    CU(cudaMemcpyAsync(dx, xs, fbytes, cudaMemcpyHostToDevice, s));
    CU(cudaMemcpyAsync(dy, ys, fbytes, cudaMemcpyHostToDevice, s));
    if (gx)
        CU(cudaMemcpyAsync(dgx, gx, fbytes, cudaMemcpyHostToDevice, s));
    if (gy)
        CU(cudaMemcpyAsync(dgy, gy, fbytes, cudaMemcpyHostToDevice, s));
    CU(vtg_launch_points(t->desc + 2 * prev, t->desc + 2 * cur, top, t->prm, n, dx, dy, dgx, dgy, dout, s,
                         t->point_warps));
    CU(cudaMemcpyAsync(out, dout, (size_t)n * sizeof(vtg_lk_out), cudaMemcpyDeviceToHost, s));
    CU(cudaFreeAsync(d, s));
    return VTG_OK;
}

extern "C" int vtg_level_device(const vtg_tracker *t, int set, int level, const float **plane, int *w, int *h, int *pitch)
{
    if (!t || !plane || set < 0 || set > 1 || level < 0 || level >= t->levels)
        return VTG_EINVAL;
    *plane = t->sets[set] + t->loff[level];
    if (w)
        *w = t->lw[level];
    if (h)
        *h = t->lh[level];
    if (pitch)
        *pitch = t->lpitch[level];
    return VTG_OK;
}

/* store_appearance's cut (track.c:947-965) in one warp. Lane l < 16 is the reference's vector lane l: it sums, then
 * squares, columns l and 16 + l of each row in row order, and the lanes fold as vx_hsum does (i ^ 1, ^ 2, ^ 4, ^ 8).
 * The sum is a whole number below 2^24 (672 Q6 values), so the mean is the x87 quotient rounded to F32 exactly. */
__global__ void __launch_bounds__(32) app_kernel(const float *__restrict__ plane, int pitch, float *__restrict__ out)
{
    const int lane = threadIdx.x;
    float s = 0.0f;
    if (lane < 16)
        for (int r = 0; r < VTG_APP_H; r++) {
            const float v0 = plane[(size_t)r * pitch + lane], v1 = plane[(size_t)r * pitch + 16 + lane];
            out[r * VTG_APP_W + lane] = v0;
            out[r * VTG_APP_W + 16 + lane] = v1;
            s = s + v0;
            s = s + v1;
        }
#pragma unroll
    for (int k = 1; k < 16; k <<= 1)
        s = s + __shfl_xor_sync(VTG_FULL, s, k);
    const uint32_t whole = (uint32_t)s; /* exact: a sum of whole numbers below 2^24 */
    const float mean = whole ? x87_to_f32(x87_div(whole, VTG_APP_W * VTG_APP_H)) : 0.0f;
    float ss = 0.0f;
    if (lane < 16)
        for (int r = 0; r < VTG_APP_H; r++) {
            const float z0 = out[r * VTG_APP_W + lane] - mean, z1 = out[r * VTG_APP_W + 16 + lane] - mean;
            out[r * VTG_APP_W + lane] = z0;
            out[r * VTG_APP_W + 16 + lane] = z1;
            ss = __fmaf_rn(z0, z0, ss);
            ss = __fmaf_rn(z1, z1, ss);
        }
#pragma unroll
    for (int k = 1; k < 16; k <<= 1)
        ss = ss + __shfl_xor_sync(VTG_FULL, ss, k);
    if (lane == 0)
        out[VTG_APP_W * VTG_APP_H] = ss;
}

extern "C" int vtg_store_appearance(vtg_tracker *t, int set, float cx, float cy, float rw, float rh, float *pix,
                                    float *norm, struct vtg_appearance *a, int where, void *stream)
{
    if (!t || !a || set < 0 || set > 1 || (where != VTG_HOST && where != VTG_DEVICE) || !(rw >= 0.0f) ||
        !(rh >= 0.0f) || !isfinite(cx) || !isfinite(cy))
        return VTG_EINVAL;
    /* the coarsest level where the template fits inside the region (track.c:939-941); every quotient is exact */
    int L = 0;
    while (L < t->levels - 1 && (double)rw / (double)(1 << (L + 1)) >= VTG_APP_W &&
           (double)rh / (double)(1 << (L + 1)) >= VTG_APP_H)
        L++;
    const double lx = ldexp((double)cx, -L), ly = ldexp((double)cy, -L);
    if (!(fabs(lx) < 1e9 && fabs(ly) < 1e9))
        return VTG_EINVAL;
    const int ix = (int)lx, iy = (int)ly; /* truncation, as the reference's (int) */
    const int x0 = ix - VTG_APP_W / 2, y0 = iy - VTG_APP_H / 2;
    a->level = L;
    a->fx = (float)(lx - ix);
    a->fy = (float)(ly - iy);
    a->valid = !(x0 < 1 || y0 < 1 || x0 + VTG_APP_W >= t->lw[L] - 1 || y0 + VTG_APP_H >= t->lh[L] - 1);
    if (!a->valid)
        return VTG_OK;
    if (!pix || !norm)
        return VTG_EINVAL;
    const cudaStream_t s = pick(t, stream);
    const float *plane = t->sets[set] + t->loff[L] + (size_t)y0 * t->lpitch[L] + x0;
    const size_t n = VTG_APP_W * VTG_APP_H;
    if (where == VTG_DEVICE && norm == pix + n) {
        app_kernel<<<1, 32, 0, s>>>(plane, t->lpitch[L], pix);
        CU(cudaGetLastError());
        return VTG_OK;
    }
    app_kernel<<<1, 32, 0, s>>>(plane, t->lpitch[L], t->d_app);
    CU(cudaGetLastError());
    const cudaMemcpyKind k = where == VTG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    CU(cudaMemcpyAsync(pix, t->d_app, n * sizeof(float), k, s));
    CU(cudaMemcpyAsync(norm, t->d_app + n, sizeof(float), k, s));
    return VTG_OK;
}

extern "C" int vtg_level(vtg_tracker *t, int set, int level, float *out, int where, void *stream)
{
    if (!t || !out || set < 0 || set > 1 || level < 0 || level >= t->levels || (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t s = pick(t, stream);
    CU(cudaMemcpy2DAsync(out, (size_t)t->lw[level] * sizeof(float), t->sets[set] + t->loff[level],
                         (size_t)t->lpitch[level] * sizeof(float), (size_t)t->lw[level] * sizeof(float),
                         (size_t)t->lh[level], where == VTG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s));
    return VTG_OK;
}
