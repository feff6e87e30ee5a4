// Work queue of the ragged-batch kernels (ragged.cu, stencil3d.cu,
// bitmorph.cu): a batch's output tiles are numbered item after item, and
// persistent CTAs take tile numbers from an atomic counter in the plan.
//
// Two latencies sit on every tile's critical path unless hidden: the atomic
// that hands out the tile, and the search for the tile's item over the
// plan's first-tile column.  TileQueue takes the NEXT tile number while the
// current tile is being computed (thread 0 issues the atomic and reads the
// result only at the next tile), and searches a shared-memory copy of the
// first-tile column (items beyond kQueueCache are searched in global memory).
#pragma once

#include "tm_common.cuh"

namespace tmc {

constexpr int kQueueCache = 1024;  // items whose first tile is cached per CTA

// Item: a plan descriptor with an `int tile_begin` field.
template <typename Item>
struct TileQueue {
    int *counter;
    int ntiles, nitems;
    const Item *items;
    int *s_tb;    // shared: tile_begin of the first min(nitems, kQueueCache) items
    int *s_slot;  // shared: {tile, item} of the CTA's current tile
    int next;     // thread 0: the tile number taken for the next iteration

    // All threads: fill the cache and take the first tile number.
    __device__ __forceinline__ void init() {
        const int nc = nitems < kQueueCache ? nitems : kQueueCache;
        for (int i = threadIdx.x; i < nc; i += blockDim.x) s_tb[i] = items[i].tile_begin;
        if (threadIdx.x == 0) next = atomicAdd(counter, 1);
        __syncthreads();
    }

    __device__ __forceinline__ int find(int t) const {
        int lo = 0, hi = nitems - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            const int tb = mid < kQueueCache ? s_tb[mid] : items[mid].tile_begin;
            if (tb <= t) lo = mid;
            else hi = mid - 1;
        }
        return lo;
    }

    // All threads: the next tile into s_slot; false when the queue is empty.
    // Callers separate consecutive calls with a block barrier after their last
    // use of s_slot and of the tile's shared buffers.
    __device__ __forceinline__ bool take() {
        if (threadIdx.x == 0) {
            const int t = next;  // taken during the previous tile
            const int it = t < ntiles ? find(t) : -1;
            s_slot[0] = t;
            s_slot[1] = it;
            if (it >= 0) next = atomicAdd(counter, 1);  // awaited only at the next take()
        }
        __syncthreads();
        return s_slot[1] >= 0;
    }
};

}  // namespace tmc
