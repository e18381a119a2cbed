/* tdag_diag.h — diagnostics of libtdag.so (no counterpart in the reference).
 *
 * The translation search's probe kernel is bound by random 4-byte loads from its membership filter,
 * which lives in L2, not by HBM bandwidth. tdag_l2_probe_peak measures that ceiling on the current
 * GPU: a kernel that does nothing but independent random word loads from an L2-resident buffer of
 * the given size, at full occupancy, eight loads in flight per thread. tdag_device_pool_usage reports
 * the device memory pool's usage.
 */
#ifndef TDAG_DIAG_H
#define TDAG_DIAG_H

#include <stddef.h>
#include <stdint.h>

#include "tdag.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Runs `loads` random 4-byte loads (rounded up to whole threads) from a device buffer of
 * buffer_bytes (a power of two, 4 KiB .. 1 GiB) on the context's stream, after one untimed warm-up
 * launch, and writes the loads per second of the timed launch to *loads_per_s. */
int tdag_l2_probe_peak(tdag_ctx* ctx, uint64_t buffer_bytes, uint64_t loads, double* loads_per_s);

/* Bytes of the context device's default memory pool (the stream-ordered pool the library allocates
 * from) in use by allocations and reserved from the driver (cudaMemPoolAttrUsedMemCurrent,
 * cudaMemPoolAttrReservedMemCurrent). Lets a caller check that a call allocated nothing. */
int tdag_device_pool_usage(tdag_ctx* ctx, uint64_t* used_bytes, uint64_t* reserved_bytes);

#ifdef __cplusplus
}
#endif

#endif
