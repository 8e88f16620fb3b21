/* vtg_tracker.h -- the tracker's device state, shared by the C ABI's translation units (api.cu, batch.cu).
 *
 * A tracker is one camera stream's device-resident state, the GPU form of the reference's struct tracker
 * (src/kern/track.c:75-160) as far as this path goes: two pyramid sets (the ring tk_sets describes), the frame staging
 * buffer, the pyramids' descriptors, and the cell results, all in one device allocation charged to the context's
 * budget. */
#ifndef VTG_TRACKER_H
#define VTG_TRACKER_H

#include "vtg_internal.cuh"

struct vtg_tracker {
    vtg_ctx *ctx;
    vtg_config cfg;
    cudaStream_t stream;
    int levels, cols, rows;
    int lw[VTG_MAX_LEVELS], lh[VTG_MAX_LEVELS], lpitch[VTG_MAX_LEVELS];
    size_t loff[VTG_MAX_LEVELS]; /* float offset of each level inside a set */
    size_t set_floats;
    size_t bytes;
    char *mem;            /* the one allocation */
    float *sets[2];       /* pyramid sets */
    uint8_t *staging;     /* frames uploaded from the host: one buffer per set, staging_set bytes apart */
    size_t staging_set;
    DevPyr *desc;         /* [set][0: from level 0, 1: from flow_level] */
    vtg_lk_out *d_lk;     /* cells x lk_out */
    vtg_cell *d_cells;    /* cells x vt_cell */
    uint32_t *d_mm;       /* the build options' VTG_MM_WORDS words a set (min / max partials, ticket, gain / offset) */
    int build_opts;       /* VTG_BUILD_CONTRAST | VTG_BUILD_PRE_GAUSS */
    float *d_app;         /* an appearance template and its norm (VTG_APP_W x VTG_APP_H + 1 floats), for host reads */
    LkPrm prm;
    int point_warps; /* warps a point of the point list: 0 by the list's length, 1 or 2 */
};

#endif
