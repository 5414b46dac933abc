// eg_scan.cuh — single-pass prefix scan (decoupled look-back) over u32 items with u64 sums.
//
// Each 256-thread CTA takes the next 4096-item tile from a ticket counter (so every tile it waits
// on belongs to a CTA that is already running), loads the tile striped (coalesced) into shared
// memory, scans it, publishes its aggregate, looks back over predecessor descriptors with warp 0,
// publishes its inclusive prefix and hands (index, exclusive prefix, value) of every item to an
// epilogue functor.  Descriptor: status in bits 63..62 (1 aggregate, 2 inclusive), value in 61..0.
// The look-back spin is bounded: on exhaustion the CTA raises err[0] and publishes anyway.
#pragma once

#include "eg_common.cuh"

namespace eg {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
constexpr uint64_t kStAgg = 1ull << 62;
constexpr uint64_t kStInc = 2ull << 62;
constexpr uint64_t kValMask = (1ull << 62) - 1;
constexpr uint32_t kLookbackSpinCap = 1u << 22;

__device__ __forceinline__ uint64_t ld_volatile_u64(const uint64_t* p) {
    return *reinterpret_cast<const volatile uint64_t*>(p);
}

__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

template <class Load, class Epi>
__global__ void __launch_bounds__(kScanThreads) k_scan(Load load, Epi epi, uint64_t n, uint64_t* desc,
                                                        uint32_t* ticket, int* err, uint64_t* total_out,
                                                        uint32_t spin_cap) {
    __shared__ uint32_t s_vals[kScanTile + kScanTile / 32];
    __shared__ uint64_t s_warp[kScanThreads / 32];
    __shared__ uint64_t s_prefix;
    __shared__ uint32_t s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint64_t base = (uint64_t)tile * kScanTile;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        uint32_t li = threadIdx.x + j * kScanThreads;
        uint64_t gi = base + li;
        s_vals[li + li / 32] = gi < n ? load(gi) : 0u;
    }
    __syncthreads();
    uint32_t v[kScanItems];
    uint64_t tsum = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        uint32_t li = threadIdx.x * kScanItems + j;
        v[j] = s_vals[li + li / 32];
        tsum += v[j];
    }
    // block exclusive scan of per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t inc = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    uint64_t warp_base = 0, tile_agg = 0;
#pragma unroll
    for (int w = 0; w < kScanThreads / 32; ++w) {
        uint64_t x = s_warp[w];
        if (w < warp) warp_base += x;
        tile_agg += x;
    }
    const uint64_t texcl = warp_base + inc - tsum;
    // look-back
    if (warp == 0) {
        uint64_t prefix = 0;
        if (tile == 0) {
            if (lane == 0) atomicExch((unsigned long long*)&desc[0], (unsigned long long)(kStInc | tile_agg));
        } else {
            if (lane == 0) atomicExch((unsigned long long*)&desc[tile], (unsigned long long)(kStAgg | tile_agg));
            int64_t pred = (int64_t)tile - 1;
            uint32_t spins = 0;
            bool timed_out = false;
            while (true) {
                int64_t idx = pred - lane;
                uint64_t d = idx >= 0 ? ld_volatile_u64(&desc[idx]) : kStInc;
                uint32_t st = (uint32_t)(d >> 62);
                if (__any_sync(0xffffffffu, st == 0)) {
                    if (++spins > spin_cap) {
                        timed_out = true;
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                uint32_t inc_mask = __ballot_sync(0xffffffffu, st == 2);
                uint64_t val = d & kValMask;
                if (idx < 0) val = 0;
                if (inc_mask) {
                    int k = __ffs(inc_mask) - 1;
                    prefix += warp_sum_u64(lane <= k ? val : 0);
                    break;
                }
                prefix += warp_sum_u64(val);
                pred -= 32;
            }
            if (timed_out && lane == 0) atomicExch(err, 1);
            if (lane == 0)
                atomicExch((unsigned long long*)&desc[tile], (unsigned long long)(kStInc | ((prefix + tile_agg) & kValMask)));
        }
        if (lane == 0) s_prefix = prefix;
    }
    __syncthreads();
    uint64_t run = s_prefix + texcl;
    const uint64_t first = base + (uint64_t)threadIdx.x * kScanItems;
#pragma unroll
    for (int j = 0; j < kScanItems; ++j) {
        if (first + j < n) epi(first + j, run, v[j]);
        run += v[j];
    }
    if (total_out && threadIdx.x == 0 && base + kScanTile >= n) *total_out = s_prefix + tile_agg;
}

// host launcher: scratch sized for the tile count; stream-ordered
template <class Load, class Epi>
int launch_scan(eg_graph* g, Load load, Epi epi, uint64_t n, uint64_t* total_out, const char* name) {
    uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0) tiles = 1;
    EG_TRY(g->scan.desc.reserve(tiles * sizeof(uint64_t)));
    EG_TRY(g->scan.counter.reserve(16));
    EG_CUDA(cudaMemsetAsync(g->scan.desc.ptr, 0, tiles * sizeof(uint64_t), g->stream));
    EG_CUDA(cudaMemsetAsync(g->scan.counter.ptr, 0, 4, g->stream));
    Timed t(&g->prof, g->stream, name);
    k_scan<<<(unsigned)tiles, kScanThreads, 0, g->stream>>>(load, epi, n, g->scan.desc.as<uint64_t>(),
                                                            g->scan.counter.as<uint32_t>(), g->err.as<int>(),
                                                            total_out, kLookbackSpinCap);
    EG_CHECK_LAUNCH(name);
    return EG_OK;
}

}  // namespace eg
