// eg_pull.cuh — the traversal machinery shared by the toolkits (eg_engine.cu) and the batched
// operators (eg_batch.cu): the chunked pull sweep over the compressed CSC, the rank-balanced push
// expansion over a frontier queue, and their host-side launchers.
//
// Push (sparse, core/graph.hpp:1505-1655): the frontier is a queue of vertices; a look-back scan
// over the frontier's list lengths gives every frontier edge a global rank, and the expansion
// kernel hands each CTA a fixed run of 2048 ranks (8 contiguous edges per thread), so hubs and
// leaves cost the same per edge.  Activations are de-duplicated in a bitmap and appended with
// warp-aggregated atomics.
// Pull (dense, :1656-1802): the CSC is swept in fixed 4096-edge chunks (16 contiguous ids per
// thread, 128-bit loads); a chunk's compressed entries are staged in shared memory and each thread
// reduces its edges per destination into shared accumulators.  Destinations wholly inside a chunk
// are finalised in place; the few whose list crosses a chunk boundary are combined afterwards.
#pragma once

#include <algorithm>

#include "eg_common.cuh"
#include "eg_scan.cuh"

namespace eg {

constexpr int kPullThreads = 256;
constexpr int kPullPerThread = 16;
constexpr uint64_t kPullChunk = kPullThreads * kPullPerThread;  // 4096 edges
constexpr int kPushThreads = 256;
constexpr int kPushPerThread = 8;
constexpr uint64_t kPushChunk = kPushThreads * kPushPerThread;  // 2048 edges
constexpr unsigned kPersistentGrid = 152u * 8u;

// ---------------------------------------------------------------------------------------------
// pull setup: chunk -> first compressed item, and the list of destinations split across chunks
static __global__ void k_pull_chunks(const uint64_t* __restrict__ cidx, const uint32_t* __restrict__ cvert, uint64_t nitems,
                              uint64_t nchunks, uint32_t* __restrict__ chunk_item, uint32_t* __restrict__ split,
                              unsigned long long* nsplit) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nitems; i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t s = cidx[i], e = cidx[i + 1];
        if (e <= s) continue;
        uint64_t c0 = (s + kPullChunk - 1) / kPullChunk, c1 = (e + kPullChunk - 1) / kPullChunk;
        for (uint64_t c = c0; c < c1; ++c) chunk_item[c] = (uint32_t)i;
        if (s / kPullChunk != (e - 1) / kPullChunk && cvert[i] != 0xFFFFFFFFu) {
            unsigned long long k = atomicAdd(nsplit, 1ull);
            split[k] = (uint32_t)i;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) chunk_item[nchunks] = (uint32_t)nitems;
}

// Generic segmented pull over compressed CSC entries.  Op provides:
//   Acc identity(); Acc gather(uint32_t src, uint64_t epos); Acc combine(Acc, Acc);
//   void smem_add(Acc* slot, Acc v); void finish(uint32_t v, Acc a, bool whole)
template <class Op>
__global__ void __launch_bounds__(kPullThreads) k_pull(Op op, const uint32_t* __restrict__ adj,
                                                        const uint64_t* __restrict__ cidx,
                                                        const uint32_t* __restrict__ cvert,
                                                        const uint32_t* __restrict__ chunk_item, uint64_t E,
                                                        uint64_t nitems, uint64_t nchunks, uint32_t V, int cap) {
    using Acc = typename Op::Acc;
    if (op.stopped()) return;  // a captured loop whose traversal already finished
    extern __shared__ __align__(16) unsigned char s_raw[];
    // item boundaries relative to the chunk start, clamped to [0, chunk]: 4 bytes per item
    uint32_t* s_idx = reinterpret_cast<uint32_t*>(s_raw);
    Acc* s_acc = reinterpret_cast<Acc*>(s_idx + cap + 1);
    uint8_t* s_on = reinterpret_cast<uint8_t*>(s_acc + cap);  // per-item filter (Op::kFilter)
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint64_t e0 = c * kPullChunk;
        const uint64_t e1 = e0 + kPullChunk < E ? e0 + kPullChunk : E;
        const uint32_t i0 = chunk_item[c];
        const uint32_t j = chunk_item[c + 1];
        const uint32_t iend = (j < nitems && cidx[j] < e1) ? j + 1 : j;
        const int nit = (int)(iend - i0);
        const bool first_open = cidx[i0] < e0;     // first item began in an earlier chunk
        const bool last_open = cidx[iend] > e1;    // last item continues into a later chunk
        for (int k = threadIdx.x; k <= nit; k += blockDim.x) {
            const uint64_t x = cidx[i0 + k];
            s_idx[k] = x <= e0 ? 0u : (x >= e1 ? (uint32_t)(e1 - e0) : (uint32_t)(x - e0));
            if (k < nit) {
                s_acc[k] = op.identity();
                if (Op::kFilter) {
                    const uint32_t v = cvert[i0 + k];
                    s_on[k] = v < V && op.item_active(v);
                }
            }
        }
        __syncthreads();
        const uint64_t eb = e0 + (uint64_t)threadIdx.x * kPullPerThread;
        int fin_key = 0x7fffffff;  // destination of this thread's last (open) segment
        Acc fin = op.identity();
        // item holding eb: last k with s_idx[k] <= eb - e0
        const uint32_t rb = (uint32_t)(eb - e0);
        int k0 = 0;
        uint32_t act = 0;  // edges of this thread whose destination passes the filter
        if (eb < e1) {
            int lo = 0, hi = nit;
            while (hi - lo > 1) {
                int mid = (lo + hi) >> 1;
                if (s_idx[mid] <= rb) lo = mid; else hi = mid;
            }
            k0 = lo;
            const uint32_t re = (uint32_t)((eb + kPullPerThread < e1 ? eb + kPullPerThread : e1) - e0);
            if (Op::kFilter) {
                int k = k0;
                uint32_t nb = s_idx[k + 1];
#pragma unroll
                for (int q = 0; q < kPullPerThread; ++q) {
                    const uint32_t e = rb + q;
                    if (e < re) {
                        while (e >= nb) nb = s_idx[++k + 1];
                        if (s_on[k]) act |= 1u << q;
                    }
                }
            } else {
                act = re - rb >= 32 ? 0xFFFFFFFFu : ((1u << (re - rb)) - 1u);
            }
        }
        if (act) {
            const uint64_t ee = eb + kPullPerThread < e1 ? eb + kPullPerThread : e1;
            uint32_t ids[kPullPerThread];
            if (ee - eb == kPullPerThread) {
                const uint4* p = reinterpret_cast<const uint4*>(adj + eb);
#pragma unroll
                for (int q = 0; q < kPullPerThread / 4; ++q) {
                    uint4 x = __ldcs(p + q);
                    ids[4 * q] = x.x; ids[4 * q + 1] = x.y; ids[4 * q + 2] = x.z; ids[4 * q + 3] = x.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < kPullPerThread; ++q) ids[q] = eb + q < ee ? adj[eb + q] : 0u;
            }
            Acc vals[kPullPerThread];
#pragma unroll
            for (int q = 0; q < kPullPerThread; ++q) vals[q] = (act >> q) & 1u ? op.gather(ids[q], eb + q) : op.identity();
            int k = k0;
            uint32_t nb = s_idx[k + 1];
            Acc a = op.identity();
            const uint32_t re = (uint32_t)(ee - e0);
#pragma unroll
            for (int q = 0; q < kPullPerThread; ++q) {
                const uint32_t e = rb + q;
                if (e < re) {
                    while (e >= nb) {
                        op.smem_add(&s_acc[k], a);
                        a = op.identity();
                        ++k;
                        nb = s_idx[k + 1];
                    }
                    a = op.combine(a, vals[q]);
                }
            }
            fin_key = k;
            fin = a;
        }
        // the open segments of consecutive threads share destinations (a hub spans whole warps):
        // segmented inclusive scan over lanes (keys are non-decreasing in lane order), one shared
        // update per run and warp
        {
            const int lane = threadIdx.x & 31;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                Acc vo = __shfl_up_sync(0xffffffffu, fin, o);
                int ko = __shfl_up_sync(0xffffffffu, fin_key, o);
                if (lane >= o && ko == fin_key) fin = op.combine(fin, vo);
            }
            const int knext = __shfl_down_sync(0xffffffffu, fin_key, 1);
            if (fin_key != 0x7fffffff && (lane == 31 || knext != fin_key)) op.smem_add(&s_acc[fin_key], fin);
        }
        __syncthreads();
        const int rounds = (nit + (int)blockDim.x - 1) / (int)blockDim.x;
        for (int r = 0; r < rounds; ++r) {
            int k = r * blockDim.x + threadIdx.x;
            bool ok = k < nit;
            uint32_t v = ok ? cvert[i0 + k] : V;
            if (v >= V) ok = false;  // partition sentinels
            Acc a = ok ? s_acc[k] : op.identity();
            bool whole = ok && !(k == 0 && first_open) && !(k == nit - 1 && last_open);
            op.finish(ok, v, a, whole);
        }
        __syncthreads();
    }
}

// Pull without shared accumulators, for operators whose reduction is an idempotent OR that may be
// applied to a destination in pieces (Op::finish_direct(v, part) any number of times per level).
// One CTA per chunk: the chunk's item boundaries and filtered destinations are staged in shared
// memory (6 bytes per item, so eight CTAs fit an SM); a segment closed inside a thread's 16 edges
// is applied at once, and the open segments at the ends of threads are merged along the warp
// first.  No second barrier, so CTAs retire as soon as their own chunk is done.
template <class Op>
__global__ void __launch_bounds__(kPullThreads) k_pull_direct(Op op, const uint32_t* __restrict__ adj,
                                                               const uint64_t* __restrict__ cidx,
                                                               const uint32_t* __restrict__ cvert,
                                                               const uint32_t* __restrict__ chunk_item, uint64_t E,
                                                               uint64_t nitems, uint32_t V) {
    using Acc = typename Op::Acc;
    if (op.stopped()) return;
    extern __shared__ __align__(16) unsigned char s_raw[];
    const uint64_t c = blockIdx.x;
    const uint64_t e0 = c * kPullChunk;
    const uint64_t e1 = e0 + kPullChunk < E ? e0 + kPullChunk : E;
    const uint32_t i0 = chunk_item[c];
    const uint32_t j = chunk_item[c + 1];
    const uint32_t iend = (j < nitems && cidx[j] < e1) ? j + 1 : j;
    const int nit = (int)(iend - i0);
    uint32_t* s_v = reinterpret_cast<uint32_t*>(s_raw);    // destination, or ~0u when filtered out
    uint16_t* s_idx = reinterpret_cast<uint16_t*>(s_v + nit);  // nit + 1 boundaries relative to e0
    for (int k = threadIdx.x; k <= nit; k += blockDim.x) {
        const uint64_t x = cidx[i0 + k];
        s_idx[k] = (uint16_t)(x <= e0 ? 0u : (x >= e1 ? (uint32_t)(e1 - e0) : (uint32_t)(x - e0)));
        if (k < nit) {
            const uint32_t v = cvert[i0 + k];
            s_v[k] = (v < V && op.item_active(v)) ? v : 0xFFFFFFFFu;
        }
    }
    __syncthreads();
    const uint64_t eb = e0 + (uint64_t)threadIdx.x * kPullPerThread;
    const uint32_t rb = (uint32_t)(eb - e0);
    int fin_key = 0x7fffffff;
    Acc fin = op.identity();
    if (eb < e1) {
        int lo = 0, hi = nit;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_idx[mid] <= rb) lo = mid; else hi = mid;
        }
        const uint64_t ee = eb + kPullPerThread < e1 ? eb + kPullPerThread : e1;
        const uint32_t re = (uint32_t)(ee - e0);
        uint32_t act = 0;
        {
            int k = lo;
            uint32_t nb = s_idx[k + 1];
#pragma unroll
            for (int q = 0; q < kPullPerThread; ++q) {
                const uint32_t e = rb + q;
                if (e < re) {
                    while (e >= nb) nb = s_idx[++k + 1];
                    if (s_v[k] != 0xFFFFFFFFu) act |= 1u << q;
                }
            }
        }
        if (act) {
            uint32_t ids[kPullPerThread];
            if (ee - eb == kPullPerThread) {
                const uint4* p = reinterpret_cast<const uint4*>(adj + eb);
#pragma unroll
                for (int q = 0; q < kPullPerThread / 4; ++q) {
                    const uint4 x = __ldcs(p + q);
                    ids[4 * q] = x.x; ids[4 * q + 1] = x.y; ids[4 * q + 2] = x.z; ids[4 * q + 3] = x.w;
                }
            } else {
#pragma unroll
                for (int q = 0; q < kPullPerThread; ++q) ids[q] = eb + q < ee ? adj[eb + q] : 0u;
            }
            Acc vals[kPullPerThread];
#pragma unroll
            for (int q = 0; q < kPullPerThread; ++q) vals[q] = (act >> q) & 1u ? op.gather(ids[q]) : op.identity();
            int k = lo;
            uint32_t nb = s_idx[k + 1];
            Acc a = op.identity();
#pragma unroll
            for (int q = 0; q < kPullPerThread; ++q) {
                const uint32_t e = rb + q;
                if (e < re) {
                    while (e >= nb) {
                        if (a != op.identity()) op.finish_direct(s_v[k], a);
                        a = op.identity();
                        ++k;
                        nb = s_idx[k + 1];
                    }
                    a = op.combine(a, vals[q]);
                }
            }
            fin_key = k;
            fin = a;
        }
    }
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const Acc vo = __shfl_up_sync(0xffffffffu, fin, o);
        const int ko = __shfl_up_sync(0xffffffffu, fin_key, o);
        if (lane >= o && ko == fin_key) fin = op.combine(fin, vo);
    }
    const int knext = __shfl_down_sync(0xffffffffu, fin_key, 1);
    if (fin_key != 0x7fffffff && (lane == 31 || knext != fin_key) && fin != op.identity())
        op.finish_direct(s_v[fin_key], fin);
}

template <class Op>
static int launch_pull_direct(eg_graph* g, const Op& op, const char* name) {
    EngineState& s = g->eng;
    if (s.pull_nchunks == 0) return EG_OK;
    const uint64_t nitems = g->ncompressed - 1;
    // a chunk holds at most one item per edge plus the zero-length sentinels of empty partitions
    const size_t smem = 6 * ((size_t)kPullChunk + g->partitions + 3);
    EG_CUDA(cudaFuncSetAttribute(k_pull_direct<Op>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    Timed t(&g->prof, g->stream, name);
    k_pull_direct<Op><<<(unsigned)s.pull_nchunks, kPullThreads, smem, g->stream>>>(
        op, g->csc_adj.as<uint32_t>(), g->cidx.as<uint64_t>(), g->cvert.as<uint32_t>(), s.pull_chunk_item.as<uint32_t>(),
        g->E, nitems, g->V);
    EG_CHECK_LAUNCH(name);
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
// warp-aggregated append of activated vertices to a queue
__device__ __forceinline__ void append_active(bool act, uint32_t w, uint32_t* q_out, uint32_t* n_out,
                                              unsigned long long* act_edges, const uint32_t* deg) {
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    if (!mask) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(n_out, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (act) q_out[base + __popc(mask & ((1u << lane) - 1u))] = w;
    if (act_edges) {  // one add per warp: a single counter takes every warp's activations
        unsigned long long d = act ? (unsigned long long)deg[w] : 0ull;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (lane == leader) atomicAdd(act_edges, d);
    }
}

// push expansion over the frontier items (vertex q[i / P], partition i % P)
struct PushArgs {
    const uint32_t* q;
    uint64_t nitems;
    int P;
    uint64_t stride;
    const uint64_t* off;
    const uint32_t* adj;
    const float* w;
    const uint64_t* ipref;  // exclusive prefix of item lengths, ipref[nitems] = total
    const uint32_t* chunk_item;
    uint32_t* q_out;
    uint32_t* n_out;
    unsigned long long* act_edges;
    const uint32_t* deg;
};

template <class Op>
__global__ void __launch_bounds__(kPushThreads) k_push(Op op, PushArgs a) {
    const uint64_t T = a.ipref[a.nitems];
    const uint64_t nchunks = (T + kPushChunk - 1) / kPushChunk;
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        const uint64_t e0 = c * kPushChunk;
        const uint64_t e1 = e0 + kPushChunk < T ? e0 + kPushChunk : T;
        const uint64_t eb = e0 + (uint64_t)threadIdx.x * kPushPerThread;
        const uint64_t ee = eb + kPushPerThread < e1 ? eb + kPushPerThread : e1;
        // item holding rank eb: last i in [i0, i1] with ipref[i] <= eb
        uint64_t lo = a.chunk_item[c];
        uint64_t hi = (c + 1 < nchunks) ? (uint64_t)a.chunk_item[c + 1] + 1 : a.nitems;
        if (eb < ee) {
            while (hi - lo > 1) {
                uint64_t mid = (lo + hi) >> 1;
                if (a.ipref[mid] <= eb) lo = mid; else hi = mid;
            }
        }
        uint64_t it = lo;
        uint64_t ibeg = a.ipref[it], iend = a.ipref[it + 1];
        uint32_t u = a.q[it / a.P];
        uint64_t lbase = a.off[(it % a.P) * a.stride + u];
        auto pay = op.payload(u);
#pragma unroll
        for (int q = 0; q < kPushPerThread; ++q) {
            const uint64_t e = eb + q;
            bool act = false;
            uint32_t wv = 0;
            if (e < ee) {
                while (e >= iend) {
                    ++it;
                    ibeg = iend;
                    iend = a.ipref[it + 1];
                    u = a.q[it / a.P];
                    lbase = a.off[(it % a.P) * a.stride + u];
                    pay = op.payload(u);
                }
                const uint64_t pos = lbase + (e - ibeg);
                wv = a.adj[pos];
                act = op.relax(u, pay, wv, pos);
            }
            append_active(act, wv, a.q_out, a.n_out, a.act_edges, a.deg);
        }
    }
}

// scan over frontier items: item length -> exclusive rank, and chunk -> first item
struct LoadItemLen {
    const uint32_t* q;
    int P;
    uint64_t stride;
    const uint64_t* off;
    __device__ uint32_t operator()(uint64_t i) const {
        uint32_t u = q[i / P];
        uint64_t b = (i % P) * stride + u;
        return (uint32_t)(off[b + 1] - off[b]);
    }
};
struct EpiItemRank {
    uint64_t* ipref;
    uint32_t* chunk_item;
    __device__ void operator()(uint64_t i, uint64_t excl, uint32_t len) const {
        ipref[i] = excl;
        uint64_t c0 = (excl + kPushChunk - 1) / kPushChunk, c1 = (excl + len + kPushChunk - 1) / kPushChunk;
        for (uint64_t c = c0; c < c1; ++c) chunk_item[c] = (uint32_t)i;
    }
};

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

template <class Op>
static int launch_pull(eg_graph* g, const Op& op, const char* name) {
    EngineState& s = g->eng;
    const uint64_t nitems = g->ncompressed - 1;
    if (s.pull_nchunks == 0) return EG_OK;
    // a chunk holds at most one item per edge plus the zero-length sentinels of empty partitions
    const int cap = (int)kPullChunk + g->partitions + 2;
    const size_t smem = sizeof(uint32_t) * (cap + 1) + sizeof(typename Op::Acc) * cap + (Op::kFilter ? cap : 0);
    EG_CUDA(cudaFuncSetAttribute(k_pull<Op>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    EG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pull<Op>, kPullThreads, smem));
    if (g->pull_blocks_per_sm > 0) per_sm = std::min(per_sm, g->pull_blocks_per_sm);
    unsigned grid = (unsigned)std::min<uint64_t>(s.pull_nchunks, (uint64_t)g->num_sms * (uint64_t)std::max(per_sm, 1));
    Timed t(&g->prof, g->stream, name);
    k_pull<Op><<<grid, kPullThreads, smem, g->stream>>>(op, g->csc_adj.as<uint32_t>(), g->cidx.as<uint64_t>(),
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
    struct {
        uint32_t n;
        uint32_t pad;
        unsigned long long act;
    } h;
    uint64_t T = 0;
    EG_CUDA(cudaMemcpyAsync(&h, d_nout, 16, cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaMemcpyAsync(&T, ipref + nitems, 8, cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    *n_out_host = h.n;
    if (edges_host) *edges_host = T;
    if (act_edges_host) *act_edges_host = h.act;
    return EG_OK;
}

static int copy_out(eg_graph* g, void* dst, const void* src, size_t bytes, int where) {
    if (!dst) return EG_OK;
    EG_CUDA(cudaMemcpyAsync(dst, src, bytes, where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            g->stream));
    return EG_OK;
}
}  // namespace eg
