// eg_pull.cuh — host-side launchers of the traversal kernels (include/endgraph_gb300_kernels.cuh)
// on a graph handle: pull setup (first compressed entry per 4096-edge chunk, entries crossing
// chunks), the chunked pull sweeps, engine scratch, and one push level over a frontier queue
// (look-back rank of the frontier's edges, then the rank-balanced expansion).  Shared by the
// toolkits (eg_engine.cu) and the batched operators (eg_batch.cu).
#pragma once

#include <algorithm>

#include "eg_common.cuh"
#include "eg_scan.cuh"

namespace eg {

// adj: the CSC source ids to gather through (default: the built CSC's)
// max_grid (optional): a persistent grid that strides over the chunks instead of a CTA per chunk
template <class Op>
static int launch_pull_direct(eg_graph* g, const Op& op, const char* name, const uint32_t* adj = nullptr,
                              unsigned max_grid = 0) {
    EngineState& s = g->eng;
    if (s.pull_nchunks == 0) return EG_OK;
    const uint64_t nitems = g->ncompressed - 1;
    // a chunk holds at most one item per edge plus the zero-length sentinels of empty partitions
    const size_t smem = 6 * ((size_t)kPullChunk + g->partitions + 3);
    EG_CUDA(cudaFuncSetAttribute(k_pull_direct<Op>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    Timed t(&g->prof, g->stream, name);
    const unsigned grid = max_grid ? (unsigned)std::min<uint64_t>(s.pull_nchunks, max_grid) : (unsigned)s.pull_nchunks;
    k_pull_direct<Op><<<grid, kPullThreads, smem, g->stream>>>(
        op, adj ? adj : g->csc_adj.as<uint32_t>(), g->cidx.as<uint64_t>(), g->cvert.as<uint32_t>(),
        s.pull_chunk_item.as<uint32_t>(), g->E, nitems, g->V);
    EG_CHECK_LAUNCH(name);
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
static int setup_pull(eg_graph* g) {
    EngineState& s = g->eng;
    if (s.pull_ready) return EG_OK;
    const uint64_t nitems = g->ncompressed - 1;  // the last sentinel closes the final item
    const uint64_t nchunks = (g->E + kPullChunk - 1) / kPullChunk;
    EG_TRY(s.pull_chunk_item.reserve(sizeof(uint32_t) * (nchunks + 2)));
    EG_TRY(s.pull_split.reserve(sizeof(uint32_t) * (nchunks + 2)));
    EG_TRY(s.counters.reserve(64));
    unsigned long long* nsplit = s.counters.as<unsigned long long>();
    EG_CUDA(cudaMemsetAsync(nsplit, 0, 8, g->stream));
    // mark sentinels so they never join the split list (their cvert is V, which is not a vertex)
    {
        Timed t(&g->prof, g->stream, "pull_setup");
        k_pull_chunks<<<grid_for(nitems, 256), 256, 0, g->stream>>>(g->cidx.as<uint64_t>(), g->cvert.as<uint32_t>(), nitems,
                                                                    nchunks, s.pull_chunk_item.as<uint32_t>(),
                                                                    s.pull_split.as<uint32_t>(), nsplit);
        EG_CHECK_LAUNCH("k_pull_chunks");
    }
    unsigned long long h = 0;
    EG_CUDA(cudaMemcpyAsync(&h, nsplit, 8, cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    s.pull_nsplit = h;
    s.pull_nchunks = nchunks;
    s.pull_ready = true;
    return EG_OK;
}

// adj: the CSC source ids to gather through (default: the built CSC's)
template <class Op>
static int launch_pull(eg_graph* g, const Op& op, const char* name, const uint32_t* adj = nullptr) {
    EngineState& s = g->eng;
    const uint64_t nitems = g->ncompressed - 1;
    if (s.pull_nchunks == 0) return EG_OK;
    // a chunk holds at most one item per edge plus the zero-length sentinels of empty partitions
    const int cap = (int)kPullChunk + g->partitions + 2;
    const size_t smem = pull_acc_offset(cap) + sizeof(typename Op::Acc) * cap + (Op::kFilter ? cap : 0);
    // gathers through renumbered sources mostly hit L2: six CTAs per SM (2.40 against 2.49 ms per
    // PageRank sweep at 2^25 / 2^29); in vertex order they need the larger L1 of five (3.13 / 3.61)
    auto kern = adj ? k_pull<Op, 6> : k_pull<Op, 5>;
    EG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    EG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPullThreads, smem));
    if (g->pull_blocks_per_sm > 0) per_sm = std::min(per_sm, g->pull_blocks_per_sm);
    unsigned grid = (unsigned)std::min<uint64_t>(s.pull_nchunks, (uint64_t)g->num_sms * (uint64_t)std::max(per_sm, 1));
    Timed t(&g->prof, g->stream, name);
    kern<<<grid, kPullThreads, smem, g->stream>>>(op, adj ? adj : g->csc_adj.as<uint32_t>(), g->cidx.as<uint64_t>(),
                                                  g->cvert.as<uint32_t>(), s.pull_chunk_item.as<uint32_t>(), g->E,
                                                  nitems, s.pull_nchunks, g->V, cap);
    EG_CHECK_LAUNCH(name);
    return EG_OK;
}

static int ensure_engine(eg_graph* g) {
    EngineState& s = g->eng;
    const uint64_t V = g->V;
    const uint64_t nitems_max = V * (uint64_t)g->partitions + 1;
    EG_TRY(s.q0.reserve(sizeof(uint32_t) * (V + 1)));
    EG_TRY(s.q1.reserve(sizeof(uint32_t) * (V + 1)));
    EG_TRY(s.qdeg.reserve(sizeof(uint64_t) * (nitems_max + 1)));
    EG_TRY(s.chunk_item.reserve(sizeof(uint32_t) * (g->E / kPushChunk + 4)));
    EG_TRY(s.bm_visit.reserve(sizeof(uint64_t) * (V / 64 + 1)));
    EG_TRY(s.bm_next.reserve(sizeof(uint64_t) * (V / 64 + 1)));
    EG_TRY(s.bm_front.reserve(sizeof(uint64_t) * (V / 64 + 1)));
    EG_TRY(s.counters.reserve(64));
    EG_TRY(s.acc.reserve(sizeof(float) * (V + 1)));
    EG_TRY(s.vals0.reserve(sizeof(float) * (V + 1)));
    EG_TRY(s.vals1.reserve(sizeof(float) * (V + 1)));
    return EG_OK;
}

// one push level over queue `q` of n vertices; returns the new queue length via *n_out_host
template <class Op>
static int push_level(eg_graph* g, const Op& op, uint32_t* q, uint64_t n, uint32_t* q_out, uint32_t* n_out_host,
                      uint64_t* edges_host, unsigned long long* act_edges_host, const uint32_t* act_deg,
                      const char* name) {
    EngineState& s = g->eng;
    const int P = g->partitions;
    const uint64_t nitems = n * (uint64_t)P;
    uint64_t* ipref = s.qdeg.as<uint64_t>();
    uint32_t* d_nout = reinterpret_cast<uint32_t*>(s.counters.as<unsigned long long>() + 2);
    unsigned long long* d_act = s.counters.as<unsigned long long>() + 3;
    EG_CUDA(cudaMemsetAsync(s.counters.as<unsigned long long>() + 2, 0, 16, g->stream));
    LoadItemLen ld{q, P, (uint64_t)g->V + 1, g->csr_off.as<uint64_t>()};
    EpiItemRank ep{ipref, s.chunk_item.as<uint32_t>()};
    EG_TRY(launch_scan(g, ld, ep, nitems, ipref + nitems, "push_rank"));
    PushArgs a;
    a.q = q;
    a.nitems = nitems;
    a.P = P;
    a.stride = (uint64_t)g->V + 1;
    a.off = g->csr_off.as<uint64_t>();
    a.adj = g->csr_adj.as<uint32_t>();
    a.w = g->csr_w.as<float>();
    a.ipref = ipref;
    a.chunk_item = s.chunk_item.as<uint32_t>();
    a.q_out = q_out;
    a.n_out = d_nout;
    a.act_edges = act_deg ? d_act : nullptr;
    a.deg = act_deg;
    {
        Timed t(&g->prof, g->stream, name);
        k_push<Op><<<kPersistentGrid, kPushThreads, 0, g->stream>>>(op, a);
        EG_CHECK_LAUNCH(name);
    }
    // queue length, active out-edges and the level's edge total, into pinned host words
    uint64_t* hw = s.host_words;
    EG_CUDA(cudaMemcpyAsync(hw, d_nout, 16, cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaMemcpyAsync(hw + 2, ipref + nitems, 8, cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    *n_out_host = (uint32_t)(hw[0] & 0xFFFFFFFFu);
    if (edges_host) *edges_host = hw[2];
    if (act_edges_host) *act_edges_host = hw[1];
    return EG_OK;
}

static inline int copy_out(eg_graph* g, void* dst, const void* src, size_t bytes, int where) {
    if (!dst) return EG_OK;
    EG_CUDA(cudaMemcpyAsync(dst, src, bytes, where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            g->stream));
    return EG_OK;
}
}  // namespace eg
