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
#include "../../include/endgraph_gb300_kernels.cuh"

namespace eg {

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
