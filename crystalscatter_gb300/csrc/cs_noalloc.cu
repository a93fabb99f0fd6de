// cs_noalloc.cu — fixed device scratch of the allocation-free mixed launch
// (cs_launch_prepared_mixed_noalloc in include/crystalscatter.h).
//
// The mixed image kernel appends the pixels it cannot settle in FP32 to a redo
// list that a second kernel recomputes in FP64. The regular entry points keep
// that list in memory the handle allocates when it first needs it. For callers
// that must not allocate on the calculation path, the list lives here instead,
// in statically sized device memory that exists once the library's module is
// loaded: a counter and CS_NOALLOC_MAX_PIXELS pixel indices (4 MiB per device).
#include <cuda_runtime.h>

#include <mutex>

#include "cs_noalloc.h"

static __device__ __align__(256) int g_noalloc_count[64];  // [0] redo counter, [1] pixel queue; padded to 256 B
static __device__ __align__(256) int g_noalloc_list[CS_NOALLOC_MAX_PIXELS];

namespace cs {

cudaError_t noalloc_scratch(int device, MixedScratch &S) {
    static std::mutex mtx;
    static int *count_addr[CS_NOALLOC_MAX_DEVICES] = {nullptr};
    static int *list_addr[CS_NOALLOC_MAX_DEVICES] = {nullptr};
    if (device < 0 || device >= CS_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(mtx);
    if (!count_addr[device]) {
        // once per device, with that device current (the caller checks it):
        // the addresses of the static arrays in this device's copy of the module
        int *c = nullptr, *l = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void **)&c, g_noalloc_count);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress((void **)&l, g_noalloc_list);
        if (e != cudaSuccess) return e;
        count_addr[device] = c;
        list_addr[device] = l;
    }
    S.d_count = count_addr[device];
    S.d_list = list_addr[device];
    S.cap = CS_NOALLOC_MAX_PIXELS;
    return cudaSuccess;
}

}  // namespace cs
