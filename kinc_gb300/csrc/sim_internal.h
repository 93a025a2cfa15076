/*
 * sim_internal.h -- entry points shared between the library's own translation
 * units (not part of the public C ABI in include/).
 */
#ifndef KINC_SIM_INTERNAL_H
#define KINC_SIM_INTERNAL_H

#include <cuda_runtime.h>

#include <stdint.h>

#include "../../include/kinc_sim.h"

/* Stream-ordered copy of the context's kernel status word into dst (zero = no
 * kernel reported an error), so a pipelined caller can check each device block
 * without synchronising the context. */
int kinc_sim_status_copy_async(kinc_sim_ctx* ctx, uint64_t* dst, cudaStream_t stream);

#endif
