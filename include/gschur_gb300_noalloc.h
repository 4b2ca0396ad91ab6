/*
 * gschur_gb300_noalloc - allocation-free entry point of the GB300 Schur engine.
 * Companion of gschur_gb300.h (same return codes and flags).
 */
#ifndef GSCHUR_GB300_NOALLOC_H
#define GSCHUR_GB300_NOALLOC_H

#include "gschur_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------
 * Allocation-free batched real Schur.  No counterpart in the reference.
 * For callers that cannot allocate device memory when they call: code running
 * under a host program or framework that owns every device allocation (a pooled
 * or arena allocator that forbids raw cudaMalloc), and launch sequences being
 * recorded for replay, where an allocation would fall outside the recorded work.
 * Same computation as gs_schur_batched_f64 with GS_DEVICE; of `flags` only GS_WANTZ
 * and GS_SCALE are read (GS_GRAPH and the others are ignored).  All arrays are device
 * pointers on the current device and the call is asynchronous on `stream` (a
 * cudaStream_t as void*); the four size bins run one after another on that stream
 * (the regular entry point forks them onto auxiliary streams), so throughput can be
 * somewhat lower.  Orders must lie in [0, 128]: they are read on the device only, and
 * a matrix whose order is outside that range is left untouched with status[b] =
 * GS_BADARG (the other matrices are unaffected).  It calls no
 * cudaMalloc/cudaFree: the work-queue scratch lives in a static device array
 * sized for GS_NOALLOC_MAX_BATCH matrices, which every GPU that loads the library
 * holds until the process exits.  count > GS_NOALLOC_MAX_BATCH returns GS_BADARG.
 * The first call on each device looks up that array's device address; make that
 * first call before any stream capture.  The address is cached per device ordinal
 * for the life of the process, so cudaDeviceReset (or anything else that replaces
 * the device's primary context) is not supported after the first call.  Calls share the array, so calls whose
 * work overlaps on the GPU race; order them on one stream.  Returns GS_OK once the
 * work is enqueued (per-matrix status as in gs_schur_batched_f64), GS_BADARG, or
 * GS_CUDA. */
#define GS_NOALLOC_MAX_BATCH 65536
GS_API int gs_schur_batched_f64_noalloc(void* stream, int64_t count, const int32_t* ns, const int64_t* offs,
                                        const int64_t* woffs, double* A, double* Z, double* wr, double* wi,
                                        int32_t* status, unsigned flags);

#ifdef __cplusplus
}
#endif

#endif /* GSCHUR_GB300_NOALLOC_H */
