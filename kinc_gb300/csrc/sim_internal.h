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

/* Record the message kinc_pm_last_error returns on this thread; returns code. */
int kinc_pm_fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));

#ifdef __cplusplus
#include <string>
#include <vector>

/* Names one per line (a trailing '\r' dropped); exactly `expected` of them, else
 * KINC_SIM_EINVAL naming `what`.  path NULL: the indices 0..expected-1. */
int kinc_pm_read_names(const char* path, int64_t expected, const char* what, std::vector<std::string>& names);
#endif

#endif
