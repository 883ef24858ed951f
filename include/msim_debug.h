/*
 * msim_debug.h - host-side fault injection for tests of the failure paths.
 *
 * No counterpart in the reference (it has no failure detection: its README asks
 * users to turn off the GPU hang check).  Every fault here is made on the host or
 * by withholding work, never by faulting the GPU: a launch that reports an error
 * without being issued, a device allocation that reports failure, or a look-back
 * chain whose first tile is never handed out, so that a bounded device wait runs
 * out and reports MSIM_ERR_TIMEOUT.  Production code never calls these.
 */
#ifndef MSIM_DEBUG_H
#define MSIM_DEBUG_H

#include <stdint.h>

#include "msim.h"

#ifdef __cplusplus
extern "C" {
#endif

#define MSIM_FAULT_NONE 0u
/* The next index update's first look-back chain (the split of an incremental update,
 * or the first radix pass of a full sort) starts handing out tiles at tile 1: tile 1
 * waits for tile 0, which never publishes, until its bounded wait (msim_set_wait_limit)
 * runs out.  Needs a chain of at least two tiles (4,096 entities for either). */
#define MSIM_FAULT_SORT_TILE 1u
/* The (arg+1)-th kernel launch of the following msim_step calls reports
 * cudaErrorLaunchFailure instead of being issued; msim_step returns MSIM_ERR_CUDA. */
#define MSIM_FAULT_LAUNCH 2u

/* Arms one fault on the context (one shot; MSIM_FAULT_NONE disarms). */
int msim_debug_inject(msim_ctx* ctx, uint32_t fault, uint32_t arg);

/* Process-wide: the next `after` device allocations made by the library succeed and
 * every one after them fails (MSIM_ERR_NOMEM from the call that needed it) until
 * this is called again; after < 0 turns the injection off. */
int msim_debug_fail_device_alloc(int64_t after);

#ifdef __cplusplus
}
#endif

#endif /* MSIM_DEBUG_H */
