/* vtg_internal.cuh -- what the kernels and the C ABI share: device descriptors, LK parameters, launchers.
 *
 * Layout in HBM. A pyramid set is one allocation: level L is a w_L x h_L plane of F32 Q6 values (the reference's own
 * plane values, src/kern/plane.h:1-9: byte x 64 at level 0, the binomial reduce above it), rows `pitch` floats apart,
 * pitch a multiple of 32 floats (128-byte rows). No border is stored: every read that the reference makes into its
 * replicated border is a clamped index here, and LK's reads never leave the plane (its bounds tests keep the window
 * inside). Levels of one set follow each other, each starting on a 256-byte boundary. */
#ifndef VTG_INTERNAL_CUH
#define VTG_INTERNAL_CUH

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/vtg.h"

#define VTG_FULL 0xffffffffu

struct DevLevel {
    const float *p;
    int w, h, pitch;
};

struct DevPyr {
    DevLevel l[VTG_MAX_LEVELS];
    int levels;
};

/* The LK settings a kernel needs, derived once from struct vtg_config. */
struct LkPrm {
    int W, H, max_iter;
    float eps2;     /* eps^2 */
    float min_eig;
    float max_residual;
    float fb_max2;  /* fb_max^2; <= 0: no forward-backward check */
    float area;     /* W H */
};

/* A cell grid on level 0 of the pyramids handed to the kernel. */
struct CellGrid {
    int cols, rows, n;
    int cell_w, cell_h;
};

static inline int vtg_pitch(int w) { return (w + 31) & ~31; }

/* tk_build's optional input steps (VTG_BUILD_CONTRAST / VTG_BUILD_PRE_GAUSS) keep a frame's partial minima and maxima,
 * a ticket and the gain / offset in VTG_MM_WORDS words of device memory. */
#define VTG_MM_BLOCKS 304
#define VTG_MM_WORDS (VTG_MM_BLOCKS + 4)

/* One frame's pyramid in a batched build: its bytes and its set's level planes. lw / lh: level sizes. opts: build
 * options; a job with options has its level 0 written by vtg_launch_build_input before the batched launches. */
struct PyrJob {
    const uint8_t *src;
    int stride, w, h, levels, opts;
    float *lv[VTG_MAX_LEVELS];
    int pitch[VTG_MAX_LEVELS], lw[VTG_MAX_LEVELS], lh[VTG_MAX_LEVELS];
};

/* One stream's per-cell flow in a batched step (the LK settings are the batch's, shared by every job). */
struct LkJob {
    const DevPyr *I, *J;
    int top;
    CellGrid g;
    int base_w, base_h;
    vtg_lk_out *out;
    vtg_cell *cells;
};

/* How a batched step runs its LK (the autotuner's choices). */
struct LkTune {
    int block_warps;   /* warps per CTA: 4, 8 or 16 */
    int chunk;         /* cells per work item */
    int persistent;    /* 1: a grid of ctas_per_sm x SMs pulling items from a counter; 0: one warp per item */
    int ctas_per_sm;   /* for the persistent form */
    int tsmem;         /* 1: the template's T in shared memory (persistent; 4 warps x <= 5, 8 x <= 3 or 16 x 1 CTAs an SM) */
    int tiled;         /* 1: cells in tiles of 8 x 4, whole tiles a CTA (persistent; chunk divides 32) */
};

/* Work items of one job's grid of cols x rows cells in runs of `chunk`: row-major, or (tiled) whole 8 x 4 tiles. */
static inline int vtg_lk_items(int cols, int rows, int chunk, int tiled)
{
    if (tiled)
        return ((cols + 7) / 8) * ((rows + 3) / 4) * (32 / chunk);
    return (cols * rows + chunk - 1) / chunk;
}

/* Launchers (pyramid.cu, lk.cu). All asynchronous on `s`; each returns a cudaError_t. */
cudaError_t vtg_launch_pyramid(const uint8_t *frame, int stride, int w, int h, float *const *levels, const int *pitches,
                               int nlevels, cudaStream_t s);
/* Level 0 of a frame under build options (the contrast stretch and / or the 5 x 5 binomial); `mm`: VTG_MM_WORDS words
 * of device memory whose ticket word (mm[VTG_MM_BLOCKS]) is 0. */
cudaError_t vtg_launch_build_input(const uint8_t *frame, int stride, int w, int h, int opts, uint32_t *mm, float *l0,
                                   int pitch0, cudaStream_t s);
/* The whole pyramid under build options: level 0 as above, then the reduce per level. */
cudaError_t vtg_launch_pyramid_opts(const uint8_t *frame, int stride, int w, int h, float *const *levels,
                                    const int *pitches, int nlevels, int opts, uint32_t *mm, cudaStream_t s);
cudaError_t vtg_launch_cells(const DevPyr *I, const DevPyr *J, int top, const LkPrm &p, const CellGrid &g, int base_w,
                             int base_h, vtg_lk_out *out, vtg_cell *cells, cudaStream_t s);
int vtg_pyr_tiles(int w, int h, int level);
/* Blocks of the fused launch that makes levels 0 .. 3 of a w x h frame at once. */
int vtg_pyr_fused_tiles(int w, int h);
/* The batched pyramid: one launch per level for all jobs. With pdl, each level after the first is launched as a
 * programmatic dependent of the one before (it starts as the previous level drains and waits in griddepcontrol.wait
 * until that level's writes are visible). reset (may be NULL): a device int the last launch sets to 0, for a
 * programmatic dependent launched after it (the LK launch's work counter). fused (no job with build options): levels 0
 * .. 3 of every job in one launch, whose tiles are row VTG_MAX_LEVELS - 1 of starts / tiles_total, then a launch per
 * further level. */
cudaError_t vtg_launch_pyramid_batch(const PyrJob *jobs, const int *starts, const int *tiles_total, int njobs,
                                     int max_levels, cudaStream_t s, int *reset = nullptr, bool pdl = false,
                                     bool fused = false);
/* Batched LK over jobs: items of `chunk` cells, job j's items from item_start[j]; `counter` must be 0 at launch.
 * count (NULL, or four device words): adds the launch's template builds, residual passes, window passes and
 * iterations, both walks of every cell, for the algorithmic operation count. */
cudaError_t vtg_launch_lk_batch(const LkJob *jobs, const int *item_start, int njobs, int items, const LkPrm &p,
                                const LkTune &tune, int sms, int *counter, cudaStream_t s, bool pdl = false,
                                unsigned long long *count = nullptr);

/* A kernel launch, as a programmatic dependent of the stream's previous kernel when pdl (the kernel itself runs
 * griddepcontrol.wait before it reads what that kernel wrote). */
template <typename... KArgs, typename... Args>
static inline cudaError_t vtg_launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                                       bool pdl, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

/* Waits until the kernels this launch programmatically depends on have finished and their writes are visible (at
 * once when there are none). */
__device__ __forceinline__ void vtg_grid_dependency_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
/* Lets the stream's next kernel, when launched as a programmatic dependent, start once every CTA of this launch has
 * called it (or exited): a CTA that calls it at its start is resident, so the dependent's waiting CTAs can take only
 * the room this launch no longer needs. */
__device__ __forceinline__ void vtg_grid_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
/* The point list. warps: warps a point (1 or 2), or 0 for the default (vtg_points_pair). */
cudaError_t vtg_launch_points(const DevPyr *I, const DevPyr *J, int top, const LkPrm &p, int n, const float *xs,
                              const float *ys, const float *gx, const float *gy, vtg_lk_out *out, cudaStream_t s,
                              int warps = 0);
/* Two warps a point only when asked: measured on the GB300 it was slower at every list length (128 points at 640 x
 * 480: 0.037 against 0.029 ms; 2,048 at 1080p: 0.104 against 0.047 ms), because a pass's latency is one round of row
 * loads however many rows a warp takes, and the pair's exchanges add to it. */
static inline bool vtg_points_pair(int n, int warps) { return warps == 2 && n > 0; }

#endif
