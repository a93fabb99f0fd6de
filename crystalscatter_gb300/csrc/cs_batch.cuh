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

// Warp-level form of the queue: lane 0 of a warp takes the next chunk of
// `chunk` pixels (a multiple of 32 dividing CS_BATCH_TILE; the counter counts
// chunks) and finds its set as above; no barrier, so a warp that finishes
// early takes the next chunk at once instead of waiting for the slowest warp
// of its block. Returns false when the group's chunks (tiles * TILE/chunk)
// or the first `limit` of them are taken. pix0: first pixel of the chunk in
// the set's calculated region.
__device__ __forceinline__ bool batch_next_chunk(const BatchSetDev *__restrict__ sets, int set_begin, int set_end,
                                                 long tiles, int chunk, long limit, unsigned long long *counter,
                                                 int &cur, long &pix0, int &set) {
    const int lane = threadIdx.x & 31;
    const long per_tile = CS_BATCH_TILE / chunk;
    long nchunks = tiles * per_tile;
    if (limit > 0 && limit < nchunks) nchunks = limit;
    long c = 0;
    if (lane == 0) {
        c = (long)atomicAdd(counter, 1ull);
        if (c < nchunks) {
            const long t = c / per_tile;
            auto inside = [&](int k) {
                return t >= sets[k].tile_begin && (k + 1 == set_end || t < sets[k + 1].tile_begin);
            };
            if (!inside(cur)) {
                if (cur + 1 < set_end && inside(cur + 1)) {
                    cur = cur + 1;
                } else {
                    int lo = set_begin, hi = set_end - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (sets[mid].tile_begin <= t) lo = mid;
                        else hi = mid - 1;
                    }
                    cur = lo;
                }
            }
        }
    }
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= nchunks) return false;
    set = __shfl_sync(0xffffffffu, cur, 0);
    const long t = c / per_tile;
    pix0 = (t - sets[set].tile_begin) * CS_BATCH_TILE + (c % per_tile) * chunk;
    return true;
}

// q of pixel (ihex, i) from the set's shared geometry table; false when the
// set has none (the caller computes q itself).
__device__ __forceinline__ bool batch_q_from_table(const BatchSetDev &S, int ihex, int i, double &qx, double &qy,
                                                   double &qz) {
    if (!S.qtab) return false;
    const long n = (long)S.qw * S.qw;
    const long j = (long)(i + S.qhalf) * S.qw + (ihex + S.qhalf);
    qx = __ldg(S.qtab + j);
    qy = __ldg(S.qtab + j + n);
    qz = __ldg(S.qtab + j + 2 * n);
    return true;
}

}  // namespace cs

#endif
