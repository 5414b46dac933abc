// eg_scan.cuh — host launcher of the decoupled look-back scan (k_scan, in
// include/endgraph_gb300_kernels.cuh) on a graph handle's scratch and stream.
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
