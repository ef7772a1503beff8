// Single-pass decoupled look-back (Merrill & Garland, 2016) used by the outlier compaction, the
// Huffman encoder and the generic device-wide exclusive scan.  Tiles take their index from an
// atomic ticket, so a tile only ever waits on tiles that are already running; every wait is
// bounded by g_spin_limit polls and reports VSZ_ERR_TIMEOUT instead of hanging.
#pragma once

#include "vsz_device.cuh"

namespace vsz {

// Polls a look-back wait makes before it gives up: kSpinLimit unless the test hook
// vsz_debug_set_spin_limit lowers it.  A static device variable, so every translation unit that
// includes this header has its own copy, which set_spin_limit_this_unit sets.
static __device__ long long g_spin_limit = kSpinLimit;
[[maybe_unused]] static int set_spin_limit_this_unit(long long polls) {
    return cudaMemcpyToSymbol(g_spin_limit, &polls, sizeof(polls)) == cudaSuccess ? VSZ_OK : VSZ_ERR_CUDA;
}

constexpr unsigned long long kFlagAgg = 1ull << 62;
constexpr unsigned long long kFlagPre = 2ull << 62;
constexpr unsigned long long kValMask = (1ull << 62) - 1;

// Called by ONE thread of the tile.  Publishes the tile aggregate, walks back to the nearest
// inclusive prefix and publishes this tile's inclusive prefix.  Returns the exclusive prefix.
__device__ __forceinline__ unsigned long long lookback_publish(unsigned long long* tile_status, uint32_t tile,
                                                               unsigned long long agg, int* status) {
    if (tile == 0) {
        st_release_u64(&tile_status[0], kFlagPre | agg);
        return 0;
    }
    st_release_u64(&tile_status[tile], kFlagAgg | agg);
    unsigned long long excl = 0;
    long long spins         = 0;
    int t                   = (int)tile - 1;
    while (t >= 0) {
        unsigned long long s = ld_acquire_u64(&tile_status[t]);
        unsigned long long f = s & (3ull << 62);
        if (f == 0) {
            if (++spins > g_spin_limit) {
                set_status(status, VSZ_ERR_TIMEOUT);
                break;
            }
            continue;
        }
        excl += s & kValMask;
        if (f == kFlagPre) break;
        t--;
    }
    st_release_u64(&tile_status[tile], kFlagPre | (excl + agg));
    return excl;
}

// Warp-parallel variant: called by all 32 lanes of ONE warp of the tile.  Each step inspects the
// 32 nearest predecessors at once and stops at the nearest one that published its inclusive
// prefix, so the walk is short even when many predecessors only published aggregates.
// Returns the exclusive prefix in every lane.
__device__ __forceinline__ unsigned long long lookback_publish_warp(unsigned long long* tile_status, uint32_t tile,
                                                                    unsigned long long agg, int* status) {
    const unsigned lane = threadIdx.x & 31u;
    if (tile == 0) {
        if (lane == 0) st_release_u64(&tile_status[0], kFlagPre | agg);
        return 0;
    }
    if (lane == 0) st_release_u64(&tile_status[tile], kFlagAgg | agg);
    unsigned long long excl = 0;
    long long base          = (long long)tile - 1;
    long long spins         = 0;
    while (true) {
        const long long idx   = base - (long long)lane;
        unsigned long long sv = (idx >= 0) ? ld_acquire_u64(&tile_status[idx]) : kFlagPre;  // before tile 0: 0
        const unsigned long long f = sv & (3ull << 62);
        const unsigned pmask = __ballot_sync(0xffffffffu, f == kFlagPre);
        const unsigned zmask = __ballot_sync(0xffffffffu, f == 0);
        const int first_p    = pmask ? (__ffs(pmask) - 1) : 32;
        const unsigned need  = (first_p >= 31) ? 0xffffffffu : ((2u << first_p) - 1u);
        if (zmask & need) {
            if (++spins > g_spin_limit) {  // a predecessor never published: give up, report
                if (lane == 0) set_status(status, VSZ_ERR_TIMEOUT);
                break;
            }
            continue;
        }
        unsigned long long v = ((int)lane <= first_p) ? (sv & kValMask) : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        excl += v;
        if (first_p < 32) break;
        base -= 32;
    }
    if (lane == 0) st_release_u64(&tile_status[tile], kFlagPre | (excl + agg));
    return excl;
}

// Block-wide exclusive scan of one value per thread (blockDim.x <= 1024, multiple of 32).
// Returns the exclusive prefix; *total receives the block sum.  Uses `warp_sums` (33 entries).
template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T* warp_sums, T* total) {
    const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (unsigned)o) incl += n;
    }
    if (lane == 31) warp_sums[w] = incl;
    __syncthreads();
    if (w == 0) {
        T s = (lane < nw) ? warp_sums[lane] : T(0);
        T si = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T n = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= (unsigned)o) si += n;
        }
        if (lane < nw) warp_sums[lane] = si - s;
        if (lane == nw - 1) warp_sums[32] = si;
    }
    __syncthreads();
    T res  = incl - v + warp_sums[w];
    *total = warp_sums[32];
    __syncthreads();
    return res;
}

}  // namespace vsz
