// cs_batch.cuh — device side of the tile queue shared by the batch kernels.
#ifndef CS_BATCH_CUH
#define CS_BATCH_CUH

#include "cs_batch.h"

namespace cs {

// Thread 0 of the block takes the next tile of the group from the counter and
// finds its set: consecutive tiles mostly stay in one set, so the set of the
// previous tile is tried first, then the set after it, then a binary search
// over the group's tile_begin values. Returns false when the group has no
// tiles left. Every thread of the block must call it (two barriers).
__device__ __forceinline__ bool batch_next_tile(const BatchSetDev *__restrict__ sets, int set_begin, int set_end,
                                                long tiles, unsigned long long *counter, int &cur, long &tile,
                                                int &set) {
    __shared__ long s_tile;
    __shared__ int s_set;
    if (threadIdx.x == 0) {
        const long t = (long)atomicAdd(counter, 1ull);
        if (t < tiles) {
            auto inside = [&](int k) {
                return t >= sets[k].tile_begin && (k + 1 == set_end || t < sets[k + 1].tile_begin);
            };
            if (!inside(cur)) {
                if (cur + 1 < set_end && inside(cur + 1)) {
                    cur = cur + 1;
                } else {
                    int lo = set_begin, hi = set_end - 1;  // last set with tile_begin <= t
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (sets[mid].tile_begin <= t) lo = mid;
                        else hi = mid - 1;
                    }
                    cur = lo;
                }
            }
        }
        s_tile = t;
        s_set = cur;
    }
    __syncthreads();
    tile = s_tile;
    set = s_set;
    __syncthreads();  // s_tile/s_set are rewritten by the next call
    return tile < tiles;
}

}  // namespace cs

#endif
