/* api_ncc.cu -- the C ABI of the appearance search (include/vtg.h): search contexts, their template, the search and
 * tk_correlate. */
#include <algorithm>
#include <mutex>
#include <new>
#include <vector>

#include "vtg_ncc.cuh"
#include "vtg_ctx.h"

struct vtg_search {
    vtg_ctx *ctx;
    int max_w, max_h, max_tw, max_th;
    cudaStream_t stream;
    char *mem;
    size_t bytes;
    float *app;       /* the template, max_tw x max_th floats */
    float *sum_t;     /* [0]: BF16 band sum, [1]: FP16 band sum (device) */
    NccScratch sc;
    uint16_t *band[2]; /* BF16 and FP16 bands */
    vtg_found *found;  /* device result slot for host callers */
    int *xy;           /* corners for vtg_correlate from the host */
    float *vals;
    int tw, th;
    float norm;
    float host_sum[2];
    bool has_template;
};

static size_t up256(size_t n) { return (n + 255) & ~(size_t)255; }

struct SearchLayout {
    size_t app, sum, S1, S2, map_v, map_x, map_y, top, ntop, err, half, band0, band1, found, conv, fac, cellw, topblk,
        arrive, bytes;
    size_t conv_elems, fac_elems;
    int tp, cells, lists;
};

static bool search_dims_ok(int max_w, int max_h, int max_tw, int max_th)
{
    return max_w >= 8 && max_h >= 8 && max_w <= 16384 && max_h <= 16384 && max_tw >= 8 && max_th >= 1 &&
           max_tw <= VTG_NCC_MAX_T && max_th <= VTG_NCC_MAX_T && (max_tw % 8) == 0;
}

static SearchLayout search_layout(int max_w, int max_h, int max_tw, int max_th)
{
    SearchLayout L;
    L.tp = max_w + 1;
    L.cells = (max_w / NCC_CELL + 2) * (max_h / NCC_CELL + 2);
    size_t b = 0;
    L.app = b;
    b += up256(sizeof(float) * (size_t)max_tw * max_th);
    L.sum = b;
    b += 256;
    L.S1 = b;
    b += up256(sizeof(long long) * (size_t)L.tp * (max_h + 1));
    L.S2 = b;
    b += up256(sizeof(long long) * (size_t)L.tp * (max_h + 1));
    L.map_v = b;
    b += up256(sizeof(float) * (size_t)L.cells);
    L.map_x = b;
    b += up256(sizeof(int) * (size_t)L.cells);
    L.map_y = b;
    b += up256(sizeof(int) * (size_t)L.cells);
    L.top = b;
    b += 256;
    L.ntop = b;
    b += 256;
    L.err = b;
    b += 256;
    L.half = b;
    b += up256(sizeof(float) * NCC_HALF_MAX);
    L.band0 = b;
    b += up256(vtg_ncc_band_bytes(max_tw, max_th));
    L.band1 = b;
    b += up256(vtg_ncc_band_bytes(max_tw, max_th));
    L.found = b;
    b += 256;
    L.conv_elems = vtg_ncc_conv_elems(max_w, max_h, max_th);
    L.conv = b;
    b += up256(sizeof(uint16_t) * L.conv_elems);
    L.fac_elems = vtg_ncc_fac_elems(max_w, max_h);
    L.fac = b;
    b += up256(sizeof(float) * L.fac_elems);
    L.cellw = b;
    b += up256(sizeof(unsigned long long) * (size_t)L.cells);
    L.topblk = b;
    L.lists = ncc_top_ctas(L.cells);
    b += up256(sizeof(unsigned long long) * NCC_TOP * (size_t)L.lists);
    L.arrive = b; /* zeroed with the rest at creation */
    b += 256;
    L.bytes = b;
    return L;
}

extern "C" size_t vtg_search_bytes(int max_w, int max_h, int max_tw, int max_th)
{
    if (!search_dims_ok(max_w, max_h, max_tw, max_th))
        return 0;
    return search_layout(max_w, max_h, max_tw, max_th).bytes;
}

extern "C" int vtg_search_create(vtg_ctx *ctx, int max_w, int max_h, int max_tw, int max_th, vtg_search **out)
{
    if (!ctx || !out || !search_dims_ok(max_w, max_h, max_tw, max_th))
        return VTG_EINVAL;
    *out = nullptr;
    const SearchLayout L = search_layout(max_w, max_h, max_tw, max_th);
    const int charged = vtg_ctx_charge(ctx, L.bytes);
    if (charged != VTG_OK)
        return charged;
    vtg_search *s = new (std::nothrow) vtg_search;
    if (!s) {
        vtg_ctx_release(ctx, L.bytes);
        return VTG_ENOMEM;
    }
    s->ctx = ctx;
    s->max_w = max_w;
    s->max_h = max_h;
    s->max_tw = max_tw;
    s->max_th = max_th;
    s->bytes = L.bytes;
    s->has_template = false;
    cudaError_t e = cudaSetDevice(vtg_ctx_device(ctx));
    if (e == cudaSuccess)
        e = cudaMalloc(&s->mem, L.bytes);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        vtg_ctx_release(ctx, L.bytes);
        delete s;
        return VTG_ENOMEM;
    }
    e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(s->mem, 0, L.bytes, s->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        cudaFree(s->mem);
        vtg_ctx_release(ctx, L.bytes);
        delete s;
        return VTG_ECUDA;
    }
    s->app = (float *)(s->mem + L.app);
    s->sum_t = (float *)(s->mem + L.sum);
    s->sc.S1 = (long long *)(s->mem + L.S1);
    s->sc.S2 = (long long *)(s->mem + L.S2);
    s->sc.tp = L.tp;
    s->sc.map_v = (float *)(s->mem + L.map_v);
    s->sc.map_x = (int *)(s->mem + L.map_x);
    s->sc.map_y = (int *)(s->mem + L.map_y);
    s->sc.top = (int *)(s->mem + L.top);
    s->sc.ntop = (int *)(s->mem + L.ntop);
    s->sc.err = (int *)(s->mem + L.err);
    s->sc.half = (float *)(s->mem + L.half);
    s->band[0] = (uint16_t *)(s->mem + L.band0);
    s->band[1] = (uint16_t *)(s->mem + L.band1);
    s->sc.band = nullptr;
    s->sc.conv = (uint16_t *)(s->mem + L.conv);
    s->sc.conv_elems = L.conv_elems;
    s->sc.fac = (float *)(s->mem + L.fac);
    s->sc.fac_elems = L.fac_elems;
    s->sc.cellw = (unsigned long long *)(s->mem + L.cellw);
    s->sc.topblk = (unsigned long long *)(s->mem + L.topblk);
    s->sc.topblk_lists = L.lists;
    s->sc.arrive = (unsigned *)(s->mem + L.arrive);
    s->sc.map_ev0 = s->sc.map_ev1 = nullptr;
    s->found = (vtg_found *)(s->mem + L.found);
    s->xy = nullptr;
    s->vals = nullptr;
    vtg_ctx_track(ctx, s->stream, true);
    *out = s;
    return VTG_OK;
}

extern "C" void vtg_search_destroy(vtg_search *s)
{
    if (!s)
        return;
    cudaSetDevice(vtg_ctx_device(s->ctx));
    cudaStreamSynchronize(s->stream);
    vtg_ctx_track(s->ctx, s->stream, false);
    cudaStreamDestroy(s->stream);
    cudaFree(s->mem);
    vtg_ctx_release(s->ctx, s->bytes);
    delete s;
}

extern "C" void *vtg_search_stream(const vtg_search *s) { return s ? (void *)s->stream : nullptr; }

#define CU(call)                                                                                                       \
    do {                                                                                                               \
        const cudaError_t e_ = (call);                                                                                 \
        if (e_ != cudaSuccess) {                                                                                       \
            vtg_set_cuda_error(e_);                                                                                    \
            return VTG_ECUDA;                                                                                          \
        }                                                                                                              \
    } while (0)

extern "C" int vtg_search_template(vtg_search *s, const float *app, int tw, int th, float norm, int where, void *stream)
{
    if (!s || !app || tw < 8 || th < 1 || tw > s->max_tw || th > s->max_th || (tw % 8) || !(norm >= 0.0f) ||
        (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    const cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    CU(cudaMemcpyAsync(s->app, app, sizeof(float) * (size_t)tw * th,
                       where == VTG_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    CU(vtg_launch_ncc_band(s->app, tw, th, VTG_NCC_BF16, s->band[0], s->sum_t + 0, st));
    CU(vtg_launch_ncc_band(s->app, tw, th, VTG_NCC_FP16, s->band[1], s->sum_t + 1, st));
    CU(cudaMemcpyAsync(s->host_sum, s->sum_t, 2 * sizeof(float), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st)); /* the band sums are kernel parameters of every later search */
    s->tw = tw;
    s->th = th;
    s->norm = norm;
    s->has_template = true;
    return VTG_OK;
}

static int make_prm(const vtg_search *s, int w, int h, int x0, int x1, int y0, int y1, int step, int precision, NccPrm *p,
                    bool *empty)
{
    if (!s->has_template || w < 8 || h < 8 || w > s->max_w || h > s->max_h || step < 1 || step > 16 ||
        (NCC_CELL % step) || precision < VTG_NCC_F32 || precision > VTG_NCC_FP16)
        return VTG_EINVAL;
    p->w = w;
    p->h = h;
    p->tw = s->tw;
    p->th = s->th;
    p->n = s->tw * s->th;
    p->norm = s->norm;
    ncc_thresholds(*p);
    p->sum_t = precision == VTG_NCC_BF16 ? s->host_sum[0] : precision == VTG_NCC_FP16 ? s->host_sum[1] : 0.0f;
    /* the reference's clamp of the window (search_slot, track.c:1665-1670) */
    const int lo_x = 1, hi_x = w - s->tw - 2, lo_y = 1, hi_y = h - s->th - 2;
    p->x0 = x0 < lo_x ? lo_x : x0;
    p->x1 = x1 > hi_x ? hi_x : x1;
    p->y0 = y0 < lo_y ? lo_y : y0;
    p->y1 = y1 > hi_y ? hi_y : y1;
    p->step = step;
    *empty = p->x1 < p->x0 || p->y1 < p->y0;
    p->ccols = *empty ? 0 : (p->x1 - p->x0) / NCC_CELL + 1;
    p->crows = *empty ? 0 : (p->y1 - p->y0) / NCC_CELL + 1;
    return VTG_OK;
}

extern "C" int vtg_search_run(vtg_search *s, const void *plane, int w, int h, int pitch, int plane_type, int x0, int x1,
                              int y0, int y1, int step, int precision, vtg_found *found, float *map_v, int *map_x,
                              int *map_y, int where, void *stream)
{
    if (!s || !plane || !found || pitch < w || (plane_type != VTG_PLANE_U8 && plane_type != VTG_PLANE_F32) ||
        (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    if (precision != VTG_NCC_F32 && plane_type != VTG_PLANE_U8)
        return VTG_EINVAL; /* the tensor-core map reads 8-bit planes */
    NccPrm p;
    bool empty = false;
    const int chk = make_prm(s, w, h, x0, x1, y0, y1, step, precision, &p, &empty);
    if (chk != VTG_OK)
        return chk;
    const cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    vtg_found *dst = where == VTG_DEVICE ? found : s->found;
    if (empty) {
        vtg_found f = {0, 0, -2.0f, -2.0f, 0.0f, 0.0f, 0, 0};
        if (where == VTG_HOST)
            *found = f;
        else
            CU(cudaMemcpyAsync(found, &f, sizeof f, cudaMemcpyHostToDevice, st));
        return VTG_OK;
    }
    NccScratch sc = s->sc;
    sc.band = precision == VTG_NCC_BF16 ? s->band[0] : precision == VTG_NCC_FP16 ? s->band[1] : nullptr;
    CU(vtg_launch_ncc(plane, pitch, plane_type, s->app, p, sc, precision, dst, st));
    const size_t cells = (size_t)p.ccols * p.crows;
    const cudaMemcpyKind k = where == VTG_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (map_v)
        CU(cudaMemcpyAsync(map_v, sc.map_v, cells * sizeof(float), k, st));
    if (map_x)
        CU(cudaMemcpyAsync(map_x, sc.map_x, cells * sizeof(int), k, st));
    if (map_y)
        CU(cudaMemcpyAsync(map_y, sc.map_y, cells * sizeof(int), k, st));
    if (where == VTG_HOST) {
        CU(cudaMemcpyAsync(found, dst, sizeof(vtg_found), cudaMemcpyDeviceToHost, st));
        int err = 0;
        CU(cudaMemcpyAsync(&err, sc.err, sizeof(int), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        if (err) {
            CU(cudaMemsetAsync(sc.err, 0, sizeof(int), st));
            return VTG_ETIMEOUT;
        }
    }
    return VTG_OK;
}

extern "C" int vtg_correlate(vtg_search *s, const void *plane, int w, int h, int pitch, int plane_type, int n,
                             const int *xs, const int *ys, float *out, int where, void *stream)
{
    if (!s || !plane || n < 0 || (n > 0 && (!xs || !ys || !out)) || pitch < w ||
        (plane_type != VTG_PLANE_U8 && plane_type != VTG_PLANE_F32) || (where != VTG_HOST && where != VTG_DEVICE))
        return VTG_EINVAL;
    NccPrm p;
    bool empty = false;
    const int chk = make_prm(s, w, h, 0, w, 0, h, 1, VTG_NCC_F32, &p, &empty);
    if (chk != VTG_OK)
        return chk;
    if (n == 0)
        return VTG_OK;
    const cudaStream_t st = stream ? (cudaStream_t)stream : s->stream;
    if (where == VTG_DEVICE) {
        CU(vtg_launch_ncc_corners(plane, pitch, plane_type, s->app, p, n, xs, ys, out, st));
        return VTG_OK;
    }
    char *d = nullptr;
    CU(cudaMallocAsync((void **)&d, (size_t)n * (2 * sizeof(int) + sizeof(float)), st));
    int *dx = (int *)d, *dy = dx + n;
    float *dv = (float *)(dy + n);
    CU(cudaMemcpyAsync(dx, xs, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st));
    CU(cudaMemcpyAsync(dy, ys, (size_t)n * sizeof(int), cudaMemcpyHostToDevice, st));
    CU(vtg_launch_ncc_corners(plane, pitch, plane_type, s->app, p, n, dx, dy, dv, st));
    CU(cudaMemcpyAsync(out, dv, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st));
    CU(cudaFreeAsync(d, st));
    CU(cudaStreamSynchronize(st));
    return VTG_OK;
}

extern "C" int vtg_search_profile(vtg_search *s, const void *plane, int w, int h, int pitch, int plane_type, int x0,
                                  int x1, int y0, int y1, int step, int precision, int reps, float *map_ms,
                                  float *total_ms)
{
    if (!s || !plane || reps < 1 || pitch < w || (plane_type != VTG_PLANE_U8 && plane_type != VTG_PLANE_F32) ||
        (precision != VTG_NCC_F32 && plane_type != VTG_PLANE_U8))
        return VTG_EINVAL;
    NccPrm p;
    bool empty = false;
    const int chk = make_prm(s, w, h, x0, x1, y0, y1, step, precision, &p, &empty);
    if (chk != VTG_OK)
        return chk;
    if (empty)
        return VTG_EINVAL;
    CU(cudaSetDevice(vtg_ctx_device(s->ctx)));
    cudaEvent_t ev[4];
    for (int k = 0; k < 4; k++)
        CU(cudaEventCreate(&ev[k]));
    NccScratch sc = s->sc;
    sc.band = precision == VTG_NCC_BF16 ? s->band[0] : precision == VTG_NCC_FP16 ? s->band[1] : nullptr;
    sc.map_ev0 = ev[1];
    sc.map_ev1 = ev[2];
    std::vector<float> tm, tt;
    int rc = VTG_OK;
    /* each rep runs the search twice: with events around the map (the map's time; its launch and the next one's are then
     * ordinary), and with events around the whole search only (its time, the passes after the map launched as
     * programmatic dependents as vtg_search_run launches them) */
    NccScratch whole = sc;
    whole.map_ev0 = whole.map_ev1 = nullptr;
    for (int r = 0; r < reps + 1 && rc == VTG_OK; r++) {
        cudaError_t e = vtg_launch_ncc(plane, pitch, plane_type, s->app, p, sc, precision, s->found, s->stream);
        if (e == cudaSuccess)
            e = cudaEventRecord(ev[3], s->stream);
        if (e == cudaSuccess)
            e = cudaEventSynchronize(ev[3]);
        float a = 0.0f, b = 0.0f;
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&a, ev[1], ev[2]);
        if (e == cudaSuccess)
            e = cudaEventRecord(ev[0], s->stream);
        if (e == cudaSuccess)
            e = vtg_launch_ncc(plane, pitch, plane_type, s->app, p, whole, precision, s->found, s->stream);
        if (e == cudaSuccess)
            e = cudaEventRecord(ev[3], s->stream);
        if (e == cudaSuccess)
            e = cudaEventSynchronize(ev[3]);
        if (e == cudaSuccess)
            e = cudaEventElapsedTime(&b, ev[0], ev[3]);
        if (e != cudaSuccess) {
            vtg_set_cuda_error(e);
            rc = VTG_ECUDA;
        } else if (r > 0) { /* the first run warms up */
            tm.push_back(a);
            tt.push_back(b);
        }
    }
    for (int k = 0; k < 4; k++)
        cudaEventDestroy(ev[k]);
    if (rc != VTG_OK)
        return rc;
    std::sort(tm.begin(), tm.end());
    std::sort(tt.begin(), tt.end());
    if (map_ms)
        *map_ms = tm[tm.size() / 2];
    if (total_ms)
        *total_ms = tt[tt.size() / 2];
    return VTG_OK;
}
