/* vtg_ctx.h -- the context's bookkeeping shared by the C ABI's translation units: the device-memory budget, the
 * streams that vtg_ctx_sync waits for, and the thread's last CUDA error. */
#ifndef VTG_CTX_H
#define VTG_CTX_H

#include <cuda_runtime.h>
#include <stddef.h>

#include "../../include/vtg.h"

/* Charges `bytes` to the budget: VTG_OK, or VTG_EBUDGET when it does not fit. */
int vtg_ctx_charge(vtg_ctx *ctx, size_t bytes);
void vtg_ctx_release(vtg_ctx *ctx, size_t bytes);
int vtg_ctx_device(const vtg_ctx *ctx);
/* Adds (or removes) a stream that vtg_ctx_sync waits for. */
void vtg_ctx_track(vtg_ctx *ctx, cudaStream_t s, bool add);
void vtg_set_cuda_error(cudaError_t e);

#endif
