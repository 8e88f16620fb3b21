/* track_pair.c -- TEST PROGRAM: the C ABI from C, as the reference's host code would call it.
 *
 * Two 1280 x 720 frames of a smooth analytic pattern, the second moved by (DX, DY) pixels; a tracker (4 levels,
 * 21 x 21, 16 x 8 cells, flowback 0.5) builds both pyramids from host memory and computes every cell's flow
 * (vtg_build, vtg_cells). Prints one line: the cells, how many are good, and the median flow, which must be the shift.
 * Exit status 0 when the library answered every call. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "vtg.h"

#define W 1280
#define H 720
#define DX 1.5
#define DY -0.75

static unsigned char pattern(double x, double y)
{
    const double v = 128.0 + 50.0 * sin(x / 7.3) * cos(y / 9.1) + 30.0 * sin((x + 2.0 * y) / 13.7) +
                     20.0 * cos((x - y) / 5.9);
    return (unsigned char)(v < 0.0 ? 0.0 : v > 255.0 ? 255.0 : v + 0.5);
}

static int cmp_float(const void *a, const void *b)
{
    const float x = *(const float *)a, y = *(const float *)b;
    return (x > y) - (x < y);
}

#define CHECK(call)                                                                                                    \
    do {                                                                                                               \
        const int rc_ = (call); /* a status, or a count for the calls that return one */                            \
        if (rc_ < 0) {                                                                                                 \
            fprintf(stderr, "%s: %s\n", #call, vtg_strerror(rc_));                                                     \
            return 1;                                                                                                  \
        }                                                                                                              \
    } while (0)

int main(void)
{
    unsigned char *f0 = malloc((size_t)W * H), *f1 = malloc((size_t)W * H);
    if (!f0 || !f1)
        return 1;
    for (int y = 0; y < H; y++)
        for (int x = 0; x < W; x++) {
            f0[(size_t)y * W + x] = pattern(x, y);
            f1[(size_t)y * W + x] = pattern(x - DX, y - DY); /* the picture moved by (DX, DY) */
        }
    vtg_ctx *ctx = NULL;
    CHECK(vtg_ctx_create(0, 0, &ctx));
    struct vtg_config cfg = {.width = W, .height = H, .levels = 4, .patch_w = 21, .patch_h = 21, .max_iter = 10,
                             .eps = 0.01f, .min_eig = 0.1f, .max_residual = 25.0f, .fb_max = 0.5f, .cell_w = 16,
                             .cell_h = 8, .flow_level = 0};
    vtg_tracker *t = NULL;
    CHECK(vtg_tracker_create(ctx, &cfg, &t));
    int cols = 0, rows = 0;
    CHECK(vtg_tracker_cells(t, &cols, &rows));
    const int n = cols * rows;
    struct vtg_cell *cells = malloc(sizeof *cells * (size_t)n);
    float *u = malloc(sizeof *u * (size_t)n), *v = malloc(sizeof *v * (size_t)n);
    if (!cells || !u || !v)
        return 1;
    CHECK(vtg_build(t, 0, f0, W, VTG_HOST, NULL));
    CHECK(vtg_build(t, 1, f1, W, VTG_HOST, NULL));
    CHECK(vtg_cells(t, 0, 1, cells, NULL, VTG_HOST, NULL));
    CHECK(vtg_ctx_sync(ctx, 10000));
    int good = 0;
    for (int i = 0; i < n; i++)
        if (cells[i].state == 0) {
            u[good] = cells[i].u;
            v[good] = cells[i].v;
            good++;
        }
    qsort(u, (size_t)good, sizeof *u, cmp_float);
    qsort(v, (size_t)good, sizeof *v, cmp_float);
    printf("{\"cells\": %d, \"good\": %d, \"median_u\": %.6f, \"median_v\": %.6f, \"dx\": %.3f, \"dy\": %.3f}\n", n,
           good, good ? u[good / 2] : 0.0, good ? v[good / 2] : 0.0, DX, DY);
    vtg_tracker_destroy(t);
    vtg_ctx_destroy(ctx);
    free(cells);
    free(u);
    free(v);
    free(f0);
    free(f1);
    return 0;
}
