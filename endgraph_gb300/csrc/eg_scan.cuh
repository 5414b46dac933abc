// eg_scan.cuh — host launcher of the decoupled look-back scan (k_scan, in
// include/endgraph_gb300_kernels.cuh) on a graph handle's scratch and stream.
#pragma once

#include "eg_common.cuh"
#include "../../include/endgraph_gb300_kernels.cuh"

namespace eg {

// ---- loads and epilogues shared by the scans --------------------------------------------------
struct LoadU32 {
    const uint32_t* p;
    __device__ uint32_t operator()(uint64_t i) const { return p[i]; }
};
struct EpiExclusive {
    uint64_t* out;
    __device__ void operator()(uint64_t i, uint64_t excl, uint32_t) const { out[i] = excl; }
};
// compressed incoming index (core/graph.hpp:1144-1188): flag of every vertex with in-edges, plus
// the sentinel slot V of each partition
struct LoadFlag {
    const uint32_t* cnt;
    uint32_t V;
    int single;  // P == 1: cnt has V entries, slot V is the sentinel
    __device__ uint32_t operator()(uint64_t i) const {
        uint64_t r = single ? i : i % ((uint64_t)V + 1);
        if (r == V) return 1u;
        return cnt[i] > 0 ? 1u : 0u;
    }
};
struct EpiCompress {
    const uint64_t* off;
    uint32_t* cvert;
    uint64_t* cidx;
    uint64_t* cstart;
    uint32_t V;
    int single;
    const uint32_t* cnt;
    __device__ void operator()(uint64_t i, uint64_t excl, uint32_t flag) const {
        if (!flag) return;
        uint64_t r = single ? i : i % ((uint64_t)V + 1);
        cvert[excl] = r == V ? V : (uint32_t)r;
        cidx[excl] = off[i];
        if (r == V) cstart[single ? 1 : i / ((uint64_t)V + 1) + 1] = excl + 1;
    }
};

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
