/* noalloc.cu -- the appearance search for callers that cannot allocate device memory.
 *
 * vtg_search_run needs a search context, and creating one calls cudaMalloc. Some callers cannot do that at the moment
 * they search: a real-time serving loop whose frame budget cannot absorb an allocation (cudaMalloc may synchronize the
 * device and take milliseconds), or a host runtime that accounts for every byte of device memory itself and forbids
 * libraries to allocate behind its back (the reference's own tracker takes all of its memory from its caller's
 * allocator and never frees it, src/kern/track.h:15-16). vtg_search_run_noalloc serves them: the caller passes the
 * plane, the template and the result buffers, and the search's scratch (the two int64 integral images, the per-cell
 * map and the candidate list) lives in one fixed array in this file's device memory.
 *
 * What that costs and what it limits:
 *   - VTG_NOALLOC_SCRATCH_BYTES (5 MiB) of device memory on every GPU that loads this library, held until the process
 *     exits, whether or not the entry point is ever called;
 *   - planes with (w + 1) (h + 1) <= VTG_NOALLOC_MAX_PIXELS (320,000: 640 x 480 fits), templates up to 64 x 64, steps 1,
 *     2 or 4 (the reference searches at 1 and 2; a step must divide the map's 16-corner cells), F32 map only; other
 *     requests are refused with VTG_EINVAL, before anything runs;
 *   - every call shares the one array, so calls whose work overlaps on the GPU (different streams, or different host
 *     threads) race and corrupt each other's results: order them on one stream, or serialize them;
 *   - the first call on a device looks the array's device address up (cudaGetSymbolAddress, once per device, with that
 *     device current); make that first call before any stream capture begins;
 *   - that address is kept for the life of the process. cudaDeviceReset destroys the context the array lives in, and
 *     the array may sit elsewhere in the next one, so a process that resets a device must not call this entry point on
 *     that device afterwards.
 * Of the array only the two arrival counters (the last CTA of a pass does its final step) need to start at zero: the
 * first call on a device zeroes them, and every search leaves them at zero. Every call writes all the other scratch it
 * reads (both integral images in full, every cell of its map, the candidate list and its count) before reading it. */
#include <mutex>

#include "vtg_ctx.h"
#include "vtg_ncc.cuh"

#define VTG_NOALLOC_MAX_CELLS 2048

/* The scratch: two integral images of VTG_NOALLOC_MAX_PIXELS int64 each, then the map and the candidates, the top-8
 * pass's per-CTA lists and the two arrival counters. */
static __device__ __align__(256) unsigned char g_noalloc_scratch[VTG_NOALLOC_SCRATCH_BYTES];

#define VTG_NOALLOC_MAX_STEP 4
#define VTG_NOALLOC_HALF (NCC_TOP * (4 * VTG_NOALLOC_MAX_STEP + 1) * (4 * VTG_NOALLOC_MAX_STEP + 1))

#define VTG_NOALLOC_TOPB ((VTG_NOALLOC_MAX_CELLS + NCC_TOPB_THREADS * NCC_TOPB_PER - 1) / (NCC_TOPB_THREADS * NCC_TOPB_PER))
#define VTG_NOALLOC_REST (2 * sizeof(long long) * (size_t)VTG_NOALLOC_MAX_PIXELS)
#define VTG_NOALLOC_HALF_AT (VTG_NOALLOC_REST + sizeof(float) * VTG_NOALLOC_MAX_CELLS + 2 * sizeof(int) * VTG_NOALLOC_MAX_CELLS + 256)
#define VTG_NOALLOC_TOPB_AT (((VTG_NOALLOC_HALF_AT + sizeof(float) * VTG_NOALLOC_HALF) + 255) & ~(size_t)255)
#define VTG_NOALLOC_ARRIVE_AT (VTG_NOALLOC_TOPB_AT + sizeof(unsigned long long) * NCC_TOP * VTG_NOALLOC_TOPB)
static_assert(VTG_NOALLOC_ARRIVE_AT + 2 * sizeof(unsigned) <= VTG_NOALLOC_SCRATCH_BYTES,
              "the scratch array holds the largest search it accepts");

#define VTG_NOALLOC_DEVICES 64

static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[VTG_NOALLOC_DEVICES];

/* The array's device address on the current device, looked up once per device; that first lookup also zeroes the
 * arrival counters, on the call's stream, ahead of the search it launches there. */
static cudaError_t noalloc_scratch(unsigned char **out, cudaStream_t st)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= VTG_NOALLOC_DEVICES)
        return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        /* the arrival counters start at zero; every search leaves them there */
        if (e == cudaSuccess)
            e = cudaMemsetAsync((unsigned char *)p + VTG_NOALLOC_ARRIVE_AT, 0, 2 * sizeof(unsigned), st);
        if (e != cudaSuccess)
            return e;
        g_noalloc_ptr[dev] = (unsigned char *)p;
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

extern "C" int vtg_search_run_noalloc(const void *plane, int w, int h, int pitch, int plane_type, const float *app,
                                      int tw, int th, float norm, int x0, int x1, int y0, int y1, int step,
                                      struct vtg_found *found, float *map_v, int *map_x, int *map_y, void *stream)
{
    if (!plane || !app || !found || w < 8 || h < 8 || pitch < w || (plane_type != VTG_PLANE_U8 && plane_type != VTG_PLANE_F32))
        return VTG_EINVAL;
    if (tw < 8 || th < 1 || (tw % 8) || tw > VTG_NOALLOC_MAX_T || th > VTG_NOALLOC_MAX_T || !(norm >= 0.0f))
        return VTG_EINVAL;
    if (w > VTG_NOALLOC_MAX_PIXELS || h > VTG_NOALLOC_MAX_PIXELS ||
        ((long long)w + 1) * ((long long)h + 1) > VTG_NOALLOC_MAX_PIXELS || step < 1 || step > VTG_NOALLOC_MAX_STEP ||
        (NCC_CELL % step))
        return VTG_EINVAL;
    NccPrm p;
    p.w = w;
    p.h = h;
    p.tw = tw;
    p.th = th;
    p.n = tw * th;
    p.norm = norm;
    ncc_thresholds(p);
    p.sum_t = 0.0f;
    /* the reference's clamp of the window (search_slot, src/kern/track.c:1665-1670) */
    const int lo_x = 1, hi_x = w - tw - 2, lo_y = 1, hi_y = h - th - 2;
    p.x0 = x0 < lo_x ? lo_x : x0;
    p.x1 = x1 > hi_x ? hi_x : x1;
    p.y0 = y0 < lo_y ? lo_y : y0;
    p.y1 = y1 > hi_y ? hi_y : y1;
    p.step = step;
    const cudaStream_t st = (cudaStream_t)stream;
    if (p.x1 < p.x0 || p.y1 < p.y0) {
        static const vtg_found none = {0, 0, -2.0f, -2.0f, 0.0f, 0.0f, 0, 0};
        const cudaError_t e = cudaMemcpyAsync(found, &none, sizeof none, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            vtg_set_cuda_error(e);
            return VTG_ECUDA;
        }
        return VTG_OK;
    }
    p.ccols = (p.x1 - p.x0) / NCC_CELL + 1;
    p.crows = (p.y1 - p.y0) / NCC_CELL + 1;
    if (p.ccols * p.crows > VTG_NOALLOC_MAX_CELLS)
        return VTG_EINVAL;
    unsigned char *base = nullptr;
    cudaError_t e = noalloc_scratch(&base, st);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        return VTG_ECUDA;
    }
    const size_t table = sizeof(long long) * (size_t)(w + 1) * (size_t)(h + 1);
    NccScratch s;
    s.tp = w + 1;
    s.S1 = (long long *)base;
    s.S2 = (long long *)(base + table);
    unsigned char *rest = base + VTG_NOALLOC_REST;
    s.map_v = (float *)rest;
    s.map_x = (int *)(rest + sizeof(float) * VTG_NOALLOC_MAX_CELLS);
    s.map_y = s.map_x + VTG_NOALLOC_MAX_CELLS;
    s.top = s.map_y + VTG_NOALLOC_MAX_CELLS;
    s.ntop = s.top + NCC_TOP;
    s.band = nullptr;
    s.err = s.ntop + 1;
    s.half = (float *)(base + VTG_NOALLOC_HALF_AT);
    s.topblk = (unsigned long long *)(base + VTG_NOALLOC_TOPB_AT);
    s.topblk_lists = VTG_NOALLOC_TOPB;
    s.arrive = (unsigned *)(base + VTG_NOALLOC_ARRIVE_AT);
    s.conv = nullptr; /* the F32 map needs none of the tensor-core map's scratch */
    s.conv_elems = 0;
    s.fac = nullptr;
    s.fac_elems = 0;
    s.cellw = nullptr;
    s.map_ev0 = s.map_ev1 = nullptr;
    e = vtg_launch_ncc(plane, pitch, plane_type, app, p, s, VTG_NCC_F32, found, st);
    const size_t cells = (size_t)p.ccols * p.crows;
    if (e == cudaSuccess && map_v)
        e = cudaMemcpyAsync(map_v, s.map_v, cells * sizeof(float), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && map_x)
        e = cudaMemcpyAsync(map_x, s.map_x, cells * sizeof(int), cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess && map_y)
        e = cudaMemcpyAsync(map_y, s.map_y, cells * sizeof(int), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) {
        vtg_set_cuda_error(e);
        return VTG_ECUDA;
    }
    return VTG_OK;
}
