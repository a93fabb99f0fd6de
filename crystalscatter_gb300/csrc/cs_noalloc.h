// cs_noalloc.h — fixed device scratch of the allocation-free mixed launch (internal).
#ifndef CS_NOALLOC_H
#define CS_NOALLOC_H

#include <cuda_runtime.h>

#include "../../include/crystalscatter.h"
#include "cs_mixed.h"

#define CS_NOALLOC_MAX_DEVICES 64

namespace cs {

// The static redo list (counter + CS_NOALLOC_MAX_PIXELS entries) of `device`,
// which must be the current device. The first call for a device looks the
// addresses up with cudaGetSymbolAddress; later calls return them.
cudaError_t noalloc_scratch(int device, MixedScratch &S);

}  // namespace cs

#endif
