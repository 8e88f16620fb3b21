/* compat.cu -- the reference-signature entry points of include/vtg_compat.h.
 *
 * Each call takes the reference's arguments (planes in its padded layout, host or device memory), moves what is in
 * host memory to device scratch, runs the same kernels as the native API (lk.cu's point and cell kernels, the
 * search's corner kernel) or a small kernel of its own for the image rows, and brings the outputs back before it
 * returns. One lock serialises the calls; the scratch and the stream belong to the device of the first call. Corner
 * detection runs detect.cu's pipeline through a detector kept for the largest plane seen. */
#include <math.h>

#include <mutex>

#include "vtg_ctx.h"
#include "vtg_internal.cuh"

#include "../../include/vtg_compat.h"

namespace {

thread_local int t_status = VTG_OK;

struct Compat {
    std::mutex mu;
    int device = -1;
    cudaStream_t stream = nullptr;
    char *scratch = nullptr;
    size_t scratch_bytes = 0;
    vtg_ctx *ctx = nullptr;       /* for the correlation's search context */
    vtg_search *search = nullptr; /* sized sw x sh, 32 x 21 templates */
    int sw = 0, sh = 0;
    vtg_detector *det = nullptr; /* sized dw x dh */
    int dw = 0, dh = 0;
};
Compat g_c;

#define TRY(x)                                                                                                         \
    do {                                                                                                               \
        const cudaError_t e_ = (x);                                                                                    \
        if (e_ != cudaSuccess) {                                                                                       \
            vtg_set_cuda_error(e_);                                                                                    \
            return VTG_ECUDA;                                                                                          \
        }                                                                                                              \
    } while (0)

/* The stream and scratch of the current device, made on first use. */
int ready()
{
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return VTG_ENODEV;
    }
    if (g_c.device == dev && g_c.stream)
        return VTG_OK;
    if (g_c.device >= 0)
        return VTG_EINVAL; /* one device per process for these entry points */
    TRY(cudaStreamCreateWithFlags(&g_c.stream, cudaStreamNonBlocking));
    g_c.device = dev;
    return VTG_OK;
}

/* At least `bytes` of device scratch, 256-byte aligned. */
int scratch(size_t bytes, char **out)
{
    if (bytes > g_c.scratch_bytes) {
        if (g_c.scratch) {
            TRY(cudaStreamSynchronize(g_c.stream));
            TRY(cudaFree(g_c.scratch));
            g_c.scratch = nullptr;
            g_c.scratch_bytes = 0;
        }
        const size_t want = bytes + (bytes >> 2);
        if (cudaMalloc((void **)&g_c.scratch, want) != cudaSuccess) {
            cudaGetLastError();
            return VTG_ENOMEM;
        }
        g_c.scratch_bytes = want;
    }
    *out = g_c.scratch;
    return VTG_OK;
}

size_t up256(size_t n) { return (n + 255) & ~(size_t)255; }

/* Device or managed memory: the kernels read it in place. Anything else is staged. */
bool on_device(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool plane_ok(const vtg_ref_plane *pl)
{
    return pl && pl->p && pl->w >= 1 && pl->h >= 1 && pl->stride >= pl->w;
}

__global__ void q6_rows_kernel(float *__restrict__ dst, int dpitch, const uint8_t *__restrict__ src, int spitch, int w,
                               int rows)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (x < w && r < rows)
        dst[(size_t)r * dpitch + x] = (float)(64 * (int)src[(size_t)r * spitch + x]);
}

/* Rows [y0, y1) of the reduce of src (rows srow0 .. of the full plane are at src), edges clamped to the plane's
 * sh rows and sw columns; out row y - y0. Whole-number sums, as img_reduce. */
__global__ void reduce_rows_kernel(float *__restrict__ dst, int dpitch, const float *__restrict__ src, int spitch,
                                   int sw, int sh, int srow0, int dw, int y0, int y1)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = y0 + (int)blockIdx.y;
    if (x >= dw || y >= y1)
        return;
    const int k[5] = {1, 4, 6, 4, 1};
    int h = 0;
    for (int i = 0; i < 5; i++) {
        const int sy = min(max(2 * y + i - 2, 0), sh - 1) - srow0;
        int v = 0;
        for (int j = 0; j < 5; j++)
            v += k[j] * (int)src[(size_t)sy * spitch + min(max(2 * x + j - 2, 0), sw - 1)];
        h += k[i] * v;
    }
    dst[(size_t)(y - y0) * dpitch + x] = (float)((h + 128) >> 8);
}

LkPrm lk_prm(const vtg_ref_lk_cfg *c, float fb_max)
{
    LkPrm p;
    p.W = c->w;
    p.H = c->h;
    p.max_iter = c->max_iter;
    p.eps2 = c->eps * c->eps;
    p.min_eig = c->min_eig;
    p.max_residual = c->max_residual;
    p.fb_max2 = fb_max > 0.0f ? fb_max * fb_max : 0.0f;
    p.area = (float)(c->w * c->h);
    return p;
}

bool cfg_ok(const vtg_ref_lk_cfg *c)
{
    return c && c->w >= 5 && c->w <= VTG_MAX_PATCH_W && c->h >= 5 && c->h <= VTG_MAX_PATCH_H && c->max_iter >= 1 &&
           c->max_iter <= 1000 && c->eps >= 0.0f;
}

/* The device view of planes pl[0 .. n - 1]: in place, or their rows copied into scratch starting at *off. */
int stage_levels(const vtg_ref_plane *pl, int n, DevPyr *d, char *base, size_t *off)
{
    d->levels = n;
    for (int L = 0; L < n; L++) {
        const vtg_ref_plane &q = pl[L];
        if (!plane_ok(&q))
            return VTG_EINVAL;
        d->l[L].w = q.w;
        d->l[L].h = q.h;
        if (on_device(q.p)) {
            d->l[L].p = q.p;
            d->l[L].pitch = q.stride;
        } else {
            const int pitch = (q.w + 31) & ~31;
            float *dst = (float *)(base + *off);
            *off += up256((size_t)pitch * (size_t)q.h * sizeof(float));
            TRY(cudaMemcpy2DAsync(dst, (size_t)pitch * sizeof(float), q.p, (size_t)q.stride * sizeof(float),
                                  (size_t)q.w * sizeof(float), (size_t)q.h, cudaMemcpyHostToDevice, g_c.stream));
            d->l[L].p = dst;
            d->l[L].pitch = pitch;
        }
    }
    return VTG_OK;
}

size_t levels_bytes(const vtg_ref_plane *pl, int n)
{
    size_t b = 0;
    for (int L = 0; L < n; L++)
        if (plane_ok(&pl[L]))
            b += up256((size_t)((pl[L].w + 31) & ~31) * (size_t)pl[L].h * sizeof(float));
    return b;
}

/* One point from pyramid I to pyramid J (levels 0 .. top), as lk_track: the result in *o. */
int track_one(const vtg_ref_plane *I, const vtg_ref_plane *J, int top, const vtg_ref_lk_cfg *c, float x, float y,
              float gx, float gy, vtg_lk_out *o)
{
    if (!I || !J || !o || !cfg_ok(c) || top < 0 || top >= VTG_MAX_LEVELS)
        return VTG_EINVAL;
    int rc = ready();
    if (rc != VTG_OK)
        return rc;
    const size_t fixed = up256(2 * sizeof(DevPyr)) + up256(4 * sizeof(float)) + up256(sizeof(vtg_lk_out));
    char *base = nullptr;
    rc = scratch(fixed + levels_bytes(I, top + 1) + levels_bytes(J, top + 1), &base);
    if (rc != VTG_OK)
        return rc;
    DevPyr h[2];
    size_t off = fixed;
    if ((rc = stage_levels(I, top + 1, &h[0], base, &off)) != VTG_OK ||
        (rc = stage_levels(J, top + 1, &h[1], base, &off)) != VTG_OK)
        return rc;
    DevPyr *dp = (DevPyr *)base;
    float *pt = (float *)(base + up256(2 * sizeof(DevPyr)));
    vtg_lk_out *dout = (vtg_lk_out *)(base + up256(2 * sizeof(DevPyr)) + up256(4 * sizeof(float)));
    const float hp[4] = {x, y, gx, gy};
    TRY(cudaMemcpyAsync(dp, h, sizeof(h), cudaMemcpyHostToDevice, g_c.stream));
    TRY(cudaMemcpyAsync(pt, hp, sizeof(hp), cudaMemcpyHostToDevice, g_c.stream));
    TRY(vtg_launch_points(dp, dp + 1, top, lk_prm(c, 0.0f), 1, pt, pt + 1, pt + 2, pt + 3, dout, g_c.stream, 1));
    TRY(cudaMemcpyAsync(o, dout, sizeof(vtg_lk_out), cudaMemcpyDeviceToHost, g_c.stream));
    TRY(cudaStreamSynchronize(g_c.stream));
    return VTG_OK;
}

void lost(vtg_lk_out *o, float x, float y)
{
    if (!o)
        return;
    o->x = x;
    o->y = y;
    o->min_eig = o->residual = o->cov_xx = o->cov_xy = o->cov_yy = 0.0f;
    o->iters = 0;
    o->status = VTG_LK_OUT;
}

} // namespace

extern "C" size_t lk_tile_bytes_cuda(void) { return 64; }

extern "C" int vtg_compat_error(void) { return t_status; }

extern "C" void img_u8_to_q6_cuda(const struct vtg_ref_plane *dst, const uint8_t *src, int src_stride, int y0, int y1)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = [&]() -> int {
        if (!plane_ok(dst) || !src || src_stride < dst->w || y0 < 0 || y1 > dst->h)
            return VTG_EINVAL;
        if (y0 >= y1)
            return VTG_OK;
        int rc = ready();
        if (rc != VTG_OK)
            return rc;
        const int w = dst->w, rows = y1 - y0;
        const bool sdev = on_device(src), ddev = on_device(dst->p);
        const size_t sbytes = sdev ? 0 : up256((size_t)w * rows), dbytes = ddev ? 0 : (size_t)w * rows * sizeof(float);
        char *base = nullptr;
        if (sbytes + dbytes > 0 && (rc = scratch(sbytes + dbytes + 256, &base)) != VTG_OK)
            return rc;
        const uint8_t *s = src + (size_t)y0 * src_stride;
        int spitch = src_stride;
        if (!sdev) {
            TRY(cudaMemcpy2DAsync(base, (size_t)w, s, (size_t)src_stride, (size_t)w, (size_t)rows,
                                  cudaMemcpyHostToDevice, g_c.stream));
            s = (const uint8_t *)base;
            spitch = w;
        }
        float *d = ddev ? dst->p + (size_t)y0 * dst->stride : (float *)(base + sbytes);
        const int dpitch = ddev ? dst->stride : w;
        q6_rows_kernel<<<dim3((w + 127) / 128, rows), 128, 0, g_c.stream>>>(d, dpitch, s, spitch, w, rows);
        TRY(cudaGetLastError());
        if (!ddev)
            TRY(cudaMemcpy2DAsync(dst->p + (size_t)y0 * dst->stride, (size_t)dst->stride * sizeof(float), d,
                                  (size_t)w * sizeof(float), (size_t)w * sizeof(float), (size_t)rows,
                                  cudaMemcpyDeviceToHost, g_c.stream));
        TRY(cudaStreamSynchronize(g_c.stream));
        return VTG_OK;
    }();
}

extern "C" void img_reduce_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *src, int y0, int y1)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = [&]() -> int {
        if (!plane_ok(dst) || !plane_ok(src) || dst->w != (src->w + 1) / 2 || dst->h != (src->h + 1) / 2 || y0 < 0 ||
            y1 > dst->h)
            return VTG_EINVAL;
        if (y0 >= y1)
            return VTG_OK;
        int rc = ready();
        if (rc != VTG_OK)
            return rc;
        const int dw = dst->w, rows = y1 - y0;
        /* the source rows these output rows read */
        const int s0 = max(2 * y0 - 2, 0), s1 = min(2 * (y1 - 1) + 2, src->h - 1);
        const bool sdev = on_device(src->p), ddev = on_device(dst->p);
        const size_t sbytes = sdev ? 0 : up256((size_t)src->w * (size_t)(s1 - s0 + 1) * sizeof(float));
        const size_t dbytes = ddev ? 0 : (size_t)dw * rows * sizeof(float);
        char *base = nullptr;
        if (sbytes + dbytes > 0 && (rc = scratch(sbytes + dbytes + 256, &base)) != VTG_OK)
            return rc;
        const float *s = src->p + (size_t)s0 * src->stride;
        int spitch = src->stride;
        if (!sdev) {
            TRY(cudaMemcpy2DAsync(base, (size_t)src->w * sizeof(float), s, (size_t)src->stride * sizeof(float),
                                  (size_t)src->w * sizeof(float), (size_t)(s1 - s0 + 1), cudaMemcpyHostToDevice,
                                  g_c.stream));
            s = (const float *)base;
            spitch = src->w;
        }
        float *d = ddev ? dst->p + (size_t)y0 * dst->stride : (float *)(base + sbytes);
        const int dpitch = ddev ? dst->stride : dw;
        reduce_rows_kernel<<<dim3((dw + 127) / 128, rows), 128, 0, g_c.stream>>>(d, dpitch, s, spitch, src->w, src->h,
                                                                                  s0, dw, y0, y1);
        TRY(cudaGetLastError());
        if (!ddev)
            TRY(cudaMemcpy2DAsync(dst->p + (size_t)y0 * dst->stride, (size_t)dst->stride * sizeof(float), d,
                                  (size_t)dw * sizeof(float), (size_t)dw * sizeof(float), (size_t)rows,
                                  cudaMemcpyDeviceToHost, g_c.stream));
        TRY(cudaStreamSynchronize(g_c.stream));
        return VTG_OK;
    }();
}

namespace {

/* The same-size image kernels of img.h, on rows [y0, y0 + rows) of a w x h plane. Sources a and b point at their row
 * srow0, `spitch` floats a row; rows and columns past the plane are clamped (the reference's replicated border). */
enum { IMG_NORM, IMG_GAUSS5, IMG_SOBEL, IMG_ABSDIFF };

template <int OP>
__global__ void img_rows_kernel(const float *__restrict__ a, int apitch, const float *__restrict__ b, int bpitch, int w,
                                int h, int srow0, int y0, int rows, float gain, float offset, float *__restrict__ d1,
                                float *__restrict__ d2, int dpitch)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y, y = y0 + r;
    if (x >= w || r >= rows)
        return;
    auto A = [&](int yy, int xx) {
        return a[(size_t)(min(max(yy, 0), h - 1) - srow0) * apitch + min(max(xx, 0), w - 1)];
    };
    float *o1 = d1 + (size_t)r * dpitch + x;
    if (OP == IMG_NORM) {
        /* img_norm_vx (img_vx.c:49-59): one rounding of the exact value; img_norm_ref's x87 form rounds the same value
         * whenever its extended sum is exact */
        const float v = rintf(__fmaf_rn(A(y, x), gain, offset));
        *o1 = v < 0.0f ? 0.0f : v > 16320.0f ? 16320.0f : v; /* keeps a -0 from rint, as the reference does */
    } else if (OP == IMG_GAUSS5) {
        /* img_gauss5_ref (img_ref.c:73-96) in its F32 order: vert5 per column, then the horizontal taps, shift8 */
        float v[5];
#pragma unroll
        for (int k = 0; k < 5; k++) {
            const int c = x + k - 2;
            v[k] = A(y - 2, c) + A(y + 2, c) + 4.0f * (A(y - 1, c) + A(y + 1, c)) + 6.0f * A(y, c);
        }
        const float hs = v[0] + v[4] + 4.0f * (v[1] + v[3]) + 6.0f * v[2];
        *o1 = (float)((__float2int_rn(hs) + 128) >> 8);
    } else if (OP == IMG_SOBEL) {
        /* img_sobel_ref (img_ref.c:116-127) */
        const float pa = A(y - 1, x - 1), pb = A(y - 1, x), pc = A(y - 1, x + 1), pe = A(y, x - 1), pg = A(y, x + 1),
                    pm = A(y + 1, x - 1), pn = A(y + 1, x), po = A(y + 1, x + 1);
        *o1 = (pc + 2.0f * pg + po) - (pa + 2.0f * pe + pm);
        d2[(size_t)r * dpitch + x] = (pm + 2.0f * pn + po) - (pa + 2.0f * pb + pc);
    } else {
        /* img_absdiff_ref (img_ref.c:129-137) */
        *o1 = fabsf(A(y, x) - b[(size_t)(y - srow0) * bpitch + x]);
    }
}

/* Min and max over rows [y0, y1) of a plane (img_minmax_ref, img_ref.c:57-71), one CTA: out[0..1]. */
__global__ void __launch_bounds__(1024) img_minmax_kernel(const float *__restrict__ a, int pitch, int w, int rows,
                                                          float *__restrict__ out)
{
    __shared__ float s_mn[32], s_mx[32];
    float mn = a[0], mx = mn;
    for (int r = 0; r < rows; r++)
        for (int x = threadIdx.x; x < w; x += blockDim.x) {
            const float v = a[(size_t)r * pitch + x];
            mn = fminf(mn, v);
            mx = fmaxf(mx, v);
        }
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(VTG_FULL, mn, s));
        mx = fmaxf(mx, __shfl_xor_sync(VTG_FULL, mx, s));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_mn[warp] = mn;
        s_mx[warp] = mx;
    }
    __syncthreads();
    if (warp == 0) {
        mn = lane < (int)(blockDim.x >> 5) ? s_mn[lane] : s_mn[0];
        mx = lane < (int)(blockDim.x >> 5) ? s_mx[lane] : s_mx[0];
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) {
            mn = fminf(mn, __shfl_xor_sync(VTG_FULL, mn, s));
            mx = fmaxf(mx, __shfl_xor_sync(VTG_FULL, mx, s));
        }
        if (lane == 0) {
            out[0] = mn;
            out[1] = mx;
        }
    }
}

/* Stages rows [r0, r1] of a plane in device memory (or uses it in place): the rows' device address and pitch. */
int stage_rows(const vtg_ref_plane *pl, int r0, int r1, char *base, size_t *off, const float **out, int *pitch)
{
    if (on_device(pl->p)) {
        *out = pl->p + (size_t)r0 * pl->stride;
        *pitch = pl->stride;
        return VTG_OK;
    }
    float *d = (float *)(base + *off);
    *off += up256((size_t)pl->w * (size_t)(r1 - r0 + 1) * sizeof(float));
    TRY(cudaMemcpy2DAsync(d, (size_t)pl->w * sizeof(float), pl->p + (size_t)r0 * pl->stride,
                          (size_t)pl->stride * sizeof(float), (size_t)pl->w * sizeof(float), (size_t)(r1 - r0 + 1),
                          cudaMemcpyHostToDevice, g_c.stream));
    *out = d;
    *pitch = pl->w;
    return VTG_OK;
}

/* Rows y0 .. y1 - 1 of d1 (and d2) from a (and b) by kernel OP, a's rows read `halo` rows each side. */
template <int OP>
int img_rows(const vtg_ref_plane *d1, const vtg_ref_plane *d2, const vtg_ref_plane *a, const vtg_ref_plane *b, int halo,
             float gain, float offset, int y0, int y1)
{
    if (!plane_ok(d1) || !plane_ok(a) || a->w != d1->w || a->h != d1->h || y0 < 0 || y1 > d1->h)
        return VTG_EINVAL;
    if ((d2 && (!plane_ok(d2) || d2->w != d1->w || d2->h != d1->h)) || (OP == IMG_SOBEL && !d2))
        return VTG_EINVAL;
    if ((b && (!plane_ok(b) || b->w != d1->w || b->h != d1->h)) || (OP == IMG_ABSDIFF && !b))
        return VTG_EINVAL;
    if (y0 >= y1)
        return VTG_OK;
    int rc = ready();
    if (rc != VTG_OK)
        return rc;
    const int w = d1->w, rows = y1 - y0;
    const int s0 = max(y0 - halo, 0), s1 = min(y1 - 1 + halo, a->h - 1);
    const size_t rows_bytes = up256((size_t)w * (size_t)(s1 - s0 + 1) * sizeof(float));
    const size_t out_bytes = up256((size_t)w * (size_t)rows * sizeof(float));
    char *base = nullptr;
    if ((rc = scratch(2 * rows_bytes + 2 * out_bytes, &base)) != VTG_OK)
        return rc;
    size_t off = 0;
    const float *pa = nullptr, *pb = nullptr;
    int apitch = 0, bpitch = 0;
    if ((rc = stage_rows(a, s0, s1, base, &off, &pa, &apitch)) != VTG_OK)
        return rc;
    if (b && (rc = stage_rows(b, s0, s1, base, &off, &pb, &bpitch)) != VTG_OK)
        return rc;
    const vtg_ref_plane *dst[2] = {d1, d2};
    float *dd[2] = {nullptr, nullptr};
    int dpitch = w;
    const bool in_place = on_device(d1->p) && (!d2 || (on_device(d2->p) && d2->stride == d1->stride));
    for (int k = 0; k < 2; k++) {
        if (!dst[k])
            continue;
        if (in_place) {
            dd[k] = dst[k]->p + (size_t)y0 * dst[k]->stride;
            dpitch = dst[k]->stride;
        } else {
            dd[k] = (float *)(base + off);
            off += out_bytes;
        }
    }
    img_rows_kernel<OP><<<dim3((w + 127) / 128, rows), 128, 0, g_c.stream>>>(pa, apitch, pb, bpitch, w, a->h, s0, y0,
                                                                             rows, gain, offset, dd[0], dd[1], dpitch);
    TRY(cudaGetLastError());
    if (!in_place)
        for (int k = 0; k < 2; k++)
            if (dst[k])
                TRY(cudaMemcpy2DAsync(dst[k]->p + (size_t)y0 * dst[k]->stride, (size_t)dst[k]->stride * sizeof(float),
                                      dd[k], (size_t)w * sizeof(float), (size_t)w * sizeof(float), (size_t)rows,
                                      on_device(dst[k]->p) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                      g_c.stream));
    TRY(cudaStreamSynchronize(g_c.stream));
    return VTG_OK;
}

} // namespace

extern "C" void img_norm_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *src,
                              const float *gain_offset, int y0, int y1)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = gain_offset ? img_rows<IMG_NORM>(dst, nullptr, src, nullptr, 0, gain_offset[0], gain_offset[1], y0, y1)
                           : VTG_EINVAL;
}

extern "C" void img_gauss5_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *src, int y0, int y1)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = img_rows<IMG_GAUSS5>(dst, nullptr, src, nullptr, 2, 0.0f, 0.0f, y0, y1);
}

extern "C" void img_sobel_cuda(const struct vtg_ref_plane *ix, const struct vtg_ref_plane *iy,
                               const struct vtg_ref_plane *src, int y0, int y1)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = img_rows<IMG_SOBEL>(ix, iy, src, nullptr, 1, 0.0f, 0.0f, y0, y1);
}

extern "C" void img_absdiff_cuda(const struct vtg_ref_plane *dst, const struct vtg_ref_plane *a,
                                 const struct vtg_ref_plane *b, int y0, int y1)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = img_rows<IMG_ABSDIFF>(dst, nullptr, a, b, 0, 0.0f, 0.0f, y0, y1);
}

extern "C" void img_minmax_cuda(const struct vtg_ref_plane *src, float *out, int y0, int y1)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = [&]() -> int {
        if (!plane_ok(src) || !out || y0 < 0 || y1 > src->h || y0 >= y1)
            return VTG_EINVAL;
        int rc = ready();
        if (rc != VTG_OK)
            return rc;
        char *base = nullptr;
        const size_t rows_bytes = up256((size_t)src->w * (size_t)(y1 - y0) * sizeof(float));
        if ((rc = scratch(rows_bytes + 256, &base)) != VTG_OK)
            return rc;
        size_t off = 256; /* the result pair first */
        const float *pa = nullptr;
        int pitch = 0;
        if ((rc = stage_rows(src, y0, y1 - 1, base, &off, &pa, &pitch)) != VTG_OK)
            return rc;
        img_minmax_kernel<<<1, 1024, 0, g_c.stream>>>(pa, pitch, src->w, y1 - y0, (float *)base);
        TRY(cudaGetLastError());
        TRY(cudaMemcpyAsync(out, base, 2 * sizeof(float), cudaMemcpyDeviceToHost, g_c.stream));
        TRY(cudaStreamSynchronize(g_c.stream));
        return VTG_OK;
    }();
}

extern "C" void lk_track_cuda(const struct vtg_ref_plane *I, const struct vtg_ref_plane *J, int top,
                              const struct vtg_ref_lk_cfg *c, float x, float y, float gx, float gy,
                              struct vtg_lk_out *o, void *tile)
{
    (void)tile;
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = track_one(I, J, top, c, x, y, gx, gy, o);
    if (t_status != VTG_OK)
        lost(o, x, y);
}

extern "C" void lk_flowback_cuda(const struct vtg_ref_plane *I, const struct vtg_ref_plane *J, int top,
                                 const struct vtg_ref_lk_cfg *c, float x, float y, float max_fb, struct vtg_lk_out *o,
                                 void *tile)
{
    (void)tile;
    if (!o)
        return;
    if (o->status) {
        t_status = VTG_OK;
        return;
    }
    std::lock_guard<std::mutex> g(g_c.mu);
    /* back from J to I, from the estimate, with minus the found flow as the guess */
    vtg_lk_out b;
    t_status = track_one(J, I, top, c, o->x, o->y, (float)((double)x - (double)o->x), (float)((double)y - (double)o->y),
                         &b);
    if (t_status != VTG_OK) {
        o->status |= VTG_LK_FLOWBACK;
        return;
    }
    const double ex = (double)b.x - (double)x, ey = (double)b.y - (double)y;
    if (b.status || ex * ex + ey * ey > (double)max_fb * (double)max_fb)
        o->status |= VTG_LK_FLOWBACK;
}

extern "C" void still_vectors_cuda(const struct vtg_ref_plane *mean, const struct vtg_ref_plane *cur,
                                   const struct vtg_ref_lk_cfg *lk, float max_fb, struct vtg_cell *cells, int tid, int n)
{
    (void)n;
    if (tid != 0)
        return;
    std::lock_guard<std::mutex> g(g_c.mu);
    t_status = [&]() -> int {
        if (!plane_ok(mean) || !plane_ok(cur) || mean->w != cur->w || mean->h != cur->h || !cells || !cfg_ok(lk) ||
            !(max_fb >= 0.0f))
            return VTG_EINVAL;
        int rc = ready();
        if (rc != VTG_OK)
            return rc;
        CellGrid gr;
        gr.cell_w = 16; /* VT_CELL_W x VT_CELL_H, src/common/vt_proto.h */
        gr.cell_h = 8;
        gr.cols = (cur->w + gr.cell_w - 1) / gr.cell_w;
        gr.rows = (cur->h + gr.cell_h - 1) / gr.cell_h;
        gr.n = gr.cols * gr.rows;
        const bool cdev = on_device(cells);
        const size_t fixed = up256(2 * sizeof(DevPyr)) + (cdev ? 0 : up256((size_t)gr.n * sizeof(vtg_cell)));
        char *base = nullptr;
        if ((rc = scratch(fixed + levels_bytes(mean, 1) + levels_bytes(cur, 1), &base)) != VTG_OK)
            return rc;
        DevPyr h[2];
        size_t off = fixed;
        if ((rc = stage_levels(mean, 1, &h[0], base, &off)) != VTG_OK ||
            (rc = stage_levels(cur, 1, &h[1], base, &off)) != VTG_OK)
            return rc;
        DevPyr *dp = (DevPyr *)base;
        vtg_cell *dc = cdev ? cells : (vtg_cell *)(base + up256(2 * sizeof(DevPyr)));
        TRY(cudaMemcpyAsync(dp, h, sizeof(h), cudaMemcpyHostToDevice, g_c.stream));
        TRY(vtg_launch_cells(dp, dp + 1, 0, lk_prm(lk, max_fb), gr, cur->w, cur->h, nullptr, dc, g_c.stream));
        if (!cdev)
            TRY(cudaMemcpyAsync(cells, dc, (size_t)gr.n * sizeof(vtg_cell), cudaMemcpyDeviceToHost, g_c.stream));
        TRY(cudaStreamSynchronize(g_c.stream));
        return VTG_OK;
    }();
}

extern "C" long double tk_correlate_cuda(const struct vtg_ref_plane *pl, const float *app, long double norm, int x,
                                         int y)
{
    enum { APP_W = 32, APP_H = 21 }; /* src/kern/track.c:21-22 */
    std::lock_guard<std::mutex> g(g_c.mu);
    float v = -1.0f;
    t_status = [&]() -> int {
        if (!plane_ok(pl) || !app)
            return VTG_EINVAL;
        /* search_at's bounds (track.c:187-188): no GPU work outside them */
        if (x < 1 || y < 1 || x + APP_W >= pl->w - 1 || y + APP_H >= pl->h - 1)
            return VTG_OK;
        int rc = ready();
        if (rc != VTG_OK)
            return rc;
        if (!g_c.ctx && (rc = vtg_ctx_create(g_c.device, 0, &g_c.ctx)) != VTG_OK)
            return rc;
        /* a plane in host memory: only the corner's window moves, one pixel around it and two past its far edges, so
         * the corner is (1, 1) of a window where search_at's bounds hold as they do in the whole plane */
        const bool pdev = on_device(pl->p);
        const int ww = pdev ? pl->w : APP_W + 3, wh = pdev ? pl->h : APP_H + 3;
        if (!g_c.search || g_c.sw < ww || g_c.sh < wh) {
            if (g_c.search)
                vtg_search_destroy(g_c.search);
            g_c.search = nullptr;
            if ((rc = vtg_search_create(g_c.ctx, max(ww, 64), max(wh, 64), APP_W, APP_H, &g_c.search)) != VTG_OK)
                return rc;
            g_c.sw = max(ww, 64);
            g_c.sh = max(wh, 64);
        }
        if ((rc = vtg_search_template(g_c.search, app, APP_W, APP_H, (float)norm,
                                      on_device(app) ? VTG_DEVICE : VTG_HOST, g_c.stream)) != VTG_OK)
            return rc;
        const float *plane = pl->p;
        int pitch = pl->stride, cx = x, cy = y;
        if (!pdev) {
            char *base = nullptr;
            if ((rc = scratch(up256((size_t)ww * wh * sizeof(float)), &base)) != VTG_OK)
                return rc;
            TRY(cudaMemcpy2DAsync(base, (size_t)ww * sizeof(float), pl->p + (size_t)(y - 1) * pl->stride + (x - 1),
                                  (size_t)pl->stride * sizeof(float), (size_t)ww * sizeof(float), (size_t)wh,
                                  cudaMemcpyHostToDevice, g_c.stream));
            plane = (const float *)base;
            pitch = ww;
            cx = cy = 1;
        }
        if ((rc = vtg_correlate(g_c.search, plane, ww, wh, pitch, VTG_PLANE_F32, 1, &cx, &cy, &v, VTG_HOST,
                                g_c.stream)) != VTG_OK)
            return rc;
        TRY(cudaStreamSynchronize(g_c.stream));
        return VTG_OK;
    }();
    return t_status == VTG_OK ? (long double)v : -1.0L;
}

extern "C" int detect_run_cuda(const struct vtg_ref_plane *pl, float rx, float ry, float rw, float rh, int margin,
                               int want, float min_dist, float quality, float *x, float *y)
{
    std::lock_guard<std::mutex> g(g_c.mu);
    int found = 0;
    t_status = [&]() -> int {
        if (!plane_ok(pl) || want < 0 || want > 512 || (want > 0 && (!x || !y)))
            return VTG_EINVAL;
        int rc = ready();
        if (rc != VTG_OK)
            return rc;
        if (!g_c.ctx && (rc = vtg_ctx_create(g_c.device, 0, &g_c.ctx)) != VTG_OK)
            return rc;
        if (!g_c.det || g_c.dw < pl->w || g_c.dh < pl->h) {
            const int dw = max(pl->w, g_c.dw), dh = max(pl->h, g_c.dh);
            if (g_c.det)
                vtg_detector_destroy(g_c.det);
            g_c.det = nullptr;
            if ((rc = vtg_detector_create(g_c.ctx, dw, dh, &g_c.det)) != VTG_OK)
                return rc;
            g_c.dw = dw;
            g_c.dh = dh;
        }
        const float *plane = pl->p;
        int pitch = pl->stride;
        if (!on_device(pl->p)) {
            /* the whole plane: detect_begin's margins and the clamped reads are the plane's own */
            pitch = (pl->w + 31) & ~31;
            char *base = nullptr;
            if ((rc = scratch(up256((size_t)pitch * (size_t)pl->h * sizeof(float)), &base)) != VTG_OK)
                return rc;
            TRY(cudaMemcpy2DAsync(base, (size_t)pitch * sizeof(float), pl->p, (size_t)pl->stride * sizeof(float),
                                  (size_t)pl->w * sizeof(float), (size_t)pl->h, cudaMemcpyHostToDevice, g_c.stream));
            plane = (const float *)base;
        }
        return vtg_detect(g_c.det, plane, pl->w, pl->h, pitch, rx, ry, rw, rh, margin, want, min_dist, quality, x, y,
                          &found, VTG_HOST, g_c.stream);
    }();
    return t_status == VTG_OK ? found : 0;
}
