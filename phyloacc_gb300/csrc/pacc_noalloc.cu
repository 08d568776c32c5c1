// Device scratch of the allocation-free entry point pacc_pmatrix_noalloc.
//
// The scratch is a file-scope device array, so it exists as soon as this
// module is loaded on a device and never goes through cudaMalloc/cudaFree.
// Layout (doubles): d[MAX] | r[MAX] | out[MAX][16].  One scratch per device:
// calls that overlap on the same device (from two threads, or on two streams
// without a synchronisation between them) race on it.
#include <cuda_runtime.h>

#include "../../include/pacc.h"

namespace pacc {

static __device__ __align__(256) double g_noalloc_scratch[(size_t)PACC_NOALLOC_MAX_PAIRS * 18];

// Device address of the scratch on the current device (the caller makes the
// device current).  The first lookup on a device loads this module there.
cudaError_t noalloc_scratch_address(double** p) { return cudaGetSymbolAddress((void**)p, g_noalloc_scratch); }

size_t noalloc_scratch_bytes() { return sizeof(g_noalloc_scratch); }

}  // namespace pacc
