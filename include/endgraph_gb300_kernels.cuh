// endgraph_gb300_kernels.cuh — the device side of the traversal engine, shared by
// libendgraph_gb300 and by programs that run their own operators on a built graph
// (endgraph_gb300_engine.cuh).  CUDA C++ for sm_103a; no host state.
//
//  * k_scan: single-pass prefix scan (decoupled look-back) over u32 items with u64 sums.  Each
//    256-thread CTA takes 4096-item tiles from a ticket counter until they run out (so every tile
//    it waits on belongs to a CTA that is already running), scans each in shared memory, publishes its
//    aggregate, looks back over predecessor descriptors with warp 0, publishes its inclusive prefix
//    and hands (index, exclusive prefix, value) of every item to an epilogue functor.  Descriptor:
//    status in bits 63..62 (1 aggregate, 2 inclusive), value in 61..0.  The look-back spin is
//    bounded: on exhaustion the CTA raises err[0] and publishes anyway.
//  * Push (sparse, core/graph.hpp:1505-1655): the frontier is a queue of vertices; the scan over
//    the frontier's list lengths gives every frontier edge a global rank, and k_push hands each CTA
//    a fixed run of 2048 ranks (8 contiguous edges per thread), so hubs and leaves cost the same
//    per edge.  Activations are appended with warp-aggregated atomics.
//  * Pull (dense, :1656-1802): the CSC is swept in fixed 4096-edge chunks (16 contiguous ids per
//    thread, 128-bit loads); a chunk's compressed entries are staged in shared memory and each
//    thread reduces its edges per destination into shared accumulators (k_pull), or, for
//    idempotent OR reductions, applies them directly (k_pull_direct).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace eg {

// shared-memory sub-arrays start on 16-byte boundaries (vector and 8-byte accesses)
__host__ __device__ constexpr size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

// Gathers from a vertex array (ranks, labels, frontier words) ask L2 to keep half of what they
// touch ahead of the streamed adjacency: a 128 MiB rank array then stays mostly resident.
// Loads are L2-coherent (.cg), like __ldcg.
__device__ __forceinline__ unsigned long long l2_keep_policy() {
    unsigned long long p;
    asm("createpolicy.fractional.L2::evict_last.b64 %0, 0.5;" : "=l"(p));
    return p;
}
__device__ __forceinline__ float ld_keep(const float* a) {
    float v;
    asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(l2_keep_policy()));
    return v;
}
__device__ __forceinline__ uint32_t ld_keep(const uint32_t* a) {
    uint32_t v;
    asm volatile("ld.global.cg.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(l2_keep_policy()));
    return v;
}
__device__ __forceinline__ unsigned long long ld_keep(const unsigned long long* a) {
    unsigned long long v;
    asm volatile("ld.global.cg.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(l2_keep_policy()));
    return v;
}

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

// The scan's work for one CTA of 256 threads: tiles by ticket until they run out (callable from
// a persistent kernel, whose CTAs are all resident, as well as from k_scan)
template <class Load, class Epi>
__device__ __forceinline__ void scan_tiles(Load load, Epi epi, uint64_t n, uint64_t* desc, uint32_t* ticket, int* err,
                                           uint64_t* total_out, uint32_t spin_cap) {
    __shared__ uint32_t s_vals[kScanTile + kScanTile / 32];
    __shared__ uint64_t s_warp[kScanThreads / 32];
    __shared__ uint64_t s_prefix;
    __shared__ uint32_t s_tile;
    // a CTA takes tiles by ticket until they run out, so a grid smaller than the tile count works
    // too (tiles are taken in order by running CTAs, so every wait is on a running tile)
    while (true) {
        if (threadIdx.x == 0) s_tile = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t tile = s_tile;
        const uint64_t base = (uint64_t)tile * kScanTile;
        if (tile > 0 && base >= n) return;
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
        if (base + kScanTile >= n) return;  // the last tile: nothing left to take
        __syncthreads();                    // s_tile, s_vals and s_prefix are reused by the next tile
    }
}

template <class Load, class Epi>
__global__ void __launch_bounds__(kScanThreads) k_scan(Load load, Epi epi, uint64_t n, uint64_t* desc,
                                                        uint32_t* ticket, int* err, uint64_t* total_out,
                                                        uint32_t spin_cap, const uint32_t* n_dev = nullptr,
                                                        uint32_t n_mult = 1) {
    // n_dev: the item count is read on the device (at most n), for launches whose grid is sized for
    // the largest count (a captured graph); the tiles past it leave at once.  No tile waits on a
    // later tile, and tile 0 always runs, so the total is written even for zero items.
    if (n_dev) {
        const uint64_t nd = (uint64_t)__ldcg(n_dev) * n_mult;
        n = nd < n ? nd : n;
    }
    scan_tiles(load, epi, n, desc, ticket, err, total_out, spin_cap);
}


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

// k_pull's shared memory: cap + 1 item boundaries (u16, relative to the chunk start, <= kPullChunk),
// then cap accumulators, then cap filter bytes when Op::kFilter.  The smaller the footprint, the
// larger the L1 share of the SM's unified L1/shared memory that caches the gathers.
__host__ __device__ constexpr size_t pull_acc_offset(int cap) { return align16(sizeof(uint16_t) * (cap + 1)); }

// Generic segmented pull over compressed CSC entries.  Op provides:
//   Acc identity(); Acc gather(uint32_t src, uint64_t epos); Acc combine(Acc, Acc);
//   void smem_add(Acc* slot, Acc v); void finish(uint32_t v, Acc a, bool whole)
// kMinBlocks: CTAs per SM the registers are sized for (5: 48 registers; 6: 40, for gathers that
// mostly hit L2, which gain more from the sixth CTA than they lose to the smaller L1)
template <class Op, int kMinBlocks = 5>
__global__ void __launch_bounds__(kPullThreads, kMinBlocks) k_pull(Op op, const uint32_t* __restrict__ adj,
                                                        const uint64_t* __restrict__ cidx,
                                                        const uint32_t* __restrict__ cvert,
                                                        const uint32_t* __restrict__ chunk_item, uint64_t E,
                                                        uint64_t nitems, uint64_t nchunks, uint32_t V, int cap) {
    using Acc = typename Op::Acc;
    if (op.stopped()) return;  // a captured loop whose traversal already finished
    extern __shared__ __align__(16) unsigned char s_raw[];
    // item boundaries relative to the chunk start, clamped to [0, chunk]: 4 bytes per item
    uint16_t* s_idx = reinterpret_cast<uint16_t*>(s_raw);
    Acc* s_acc = reinterpret_cast<Acc*>(s_raw + pull_acc_offset(cap));
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
            s_idx[k] = (uint16_t)(x <= e0 ? 0u : (x >= e1 ? (uint32_t)(e1 - e0) : (uint32_t)(x - e0)));
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
// The chunks of one CTA (chunk blockIdx.x, then every gridDim.x-th), staging in s_raw
// ticket (optional): chunks are taken from this counter instead of by stride, which balances
// uneven chunks when a persistent grid runs the sweep
template <class Op>
__device__ __forceinline__ void pull_direct_chunks(const Op& op, const uint32_t* __restrict__ adj,
                                                   const uint64_t* __restrict__ cidx, const uint32_t* __restrict__ cvert,
                                                   const uint32_t* __restrict__ chunk_item, uint64_t E, uint64_t nitems,
                                                   uint32_t V, unsigned char* s_raw, uint32_t* ticket = nullptr) {
    using Acc = typename Op::Acc;
    __shared__ uint32_t s_chunk;
    // one chunk per CTA when launched with a CTA per chunk; a smaller (persistent) grid strides
    const uint64_t nchunks = (E + kPullChunk - 1) / kPullChunk;
    auto take = [&](uint64_t dflt) -> uint64_t {
        if (!ticket) return dflt;
        if (threadIdx.x == 0) s_chunk = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint64_t t = s_chunk;
        __syncthreads();
        return t;
    };
    for (uint64_t c = take(blockIdx.x); c < nchunks; c = take(c + gridDim.x)) {
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
        if (ticket || c + gridDim.x < nchunks) __syncthreads();  // the next chunk reuses the staged entries
    }
}

// sized for six CTAs per SM (40 registers): the 64-root pull level takes 7.41 ms against 7.66 ms
// at the five that 48 registers allow, at 2^25 / 2^29
template <class Op>
__global__ void __launch_bounds__(kPullThreads, 6) k_pull_direct(Op op, const uint32_t* __restrict__ adj,
                                                               const uint64_t* __restrict__ cidx,
                                                               const uint32_t* __restrict__ cvert,
                                                               const uint32_t* __restrict__ chunk_item, uint64_t E,
                                                               uint64_t nitems, uint32_t V) {
    if (op.stopped()) return;
    extern __shared__ __align__(16) unsigned char s_raw[];
    pull_direct_chunks(op, adj, cidx, cvert, chunk_item, E, nitems, V, s_raw);
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

// CTA-aggregated append for loops that are uniform across the CTA: one global atomic per CTA
// step instead of one per warp (a single queue counter takes every step's activations).
// s_cnt: 2 * (warps + 1) shared words; parity alternates between steps so that one barrier
// pair per step suffices.
__device__ __forceinline__ void append_block(bool act, uint32_t w, uint32_t* q_out, uint32_t* n_out, uint32_t* s_cnt,
                                             int parity) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t* c = s_cnt + parity * (nw + 1);
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    if (lane == 0) c[warp] = (uint32_t)__popc(mask);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int i = 0; i < nw; ++i) {
            const uint32_t x = c[i];
            c[i] = t;
            t += x;
        }
        c[nw] = t ? atomicAdd(n_out, t) : 0u;
    }
    __syncthreads();
    if (act) q_out[c[nw] + c[warp] + (uint32_t)__popc(mask & ((1u << lane) - 1u))] = w;
}

// The same with the activated vertices' out-degrees summed per CTA into *act_edges.
// s_cnt: 2 * (warps + 1) words, s_deg: warps words of shared memory.
__device__ __forceinline__ void append_block_deg(bool act, uint32_t w, uint32_t* q_out, uint32_t* n_out,
                                                 unsigned long long* act_edges, const uint32_t* deg, uint32_t* s_cnt,
                                                 unsigned long long* s_deg, int parity) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint32_t* c = s_cnt + parity * (nw + 1);
    const unsigned mask = __ballot_sync(0xffffffffu, act);
    unsigned long long d = act ? (unsigned long long)deg[w] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
    if (lane == 0) {
        c[warp] = (uint32_t)__popc(mask);
        s_deg[warp] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        unsigned long long dt = 0;
        for (int i = 0; i < nw; ++i) {
            const uint32_t x = c[i];
            c[i] = t;
            t += x;
            dt += s_deg[i];
        }
        c[nw] = t ? atomicAdd(n_out, t) : 0u;
        if (dt) atomicAdd(act_edges, dt);
    }
    __syncthreads();
    if (act) q_out[c[nw] + c[warp] + (uint32_t)__popc(mask & ((1u << lane) - 1u))] = w;
}

// push expansion over the frontier items (vertex q[i / P], partition i % P)
struct PushArgs {
    const uint32_t* q;
    uint64_t nitems;
    // optional: the queue length read on the device (items = *n_dev * P) and the edge total the
    // scan wrote at *total_dev, for launches made before the count is known on the host
    const uint32_t* n_dev = nullptr;
    const uint64_t* total_dev = nullptr;
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

// An operator with a `Value` type reduces a value over the edges it relaxes:
// relax(u, payload, w, pos, Value& acc) adds to a per-thread sum, and reduce_out(Value) receives one
// warp's total.  Operators without it use relax(u, payload, w, pos).
template <class Op, class = void>
struct push_value {
    using type = void;
};
template <class Op>
struct push_value<Op, std::void_t<typename Op::Value>> {
    using type = typename Op::Value;
};

// The rank-balanced expansion for one CTA of kPushThreads (chunks blockIdx.x, +gridDim.x, ...)
template <class Op>
__device__ __forceinline__ void push_chunks(const Op& op, PushArgs a) {
    using Val = typename push_value<Op>::type;
    constexpr bool kReduce = !std::is_void<Val>::value;
    std::conditional_t<kReduce, Val, int> acc{};
    __shared__ uint32_t s_cnt[kPushThreads / 32 + 1];
    unsigned long long my_act = 0;  // out-edges of the vertices this thread activated
    if (a.n_dev) a.nitems = (uint64_t)__ldcg(a.n_dev) * (uint64_t)a.P;
    const uint64_t T = a.total_dev ? __ldcg(a.total_dev) : a.ipref[a.nitems];
    // item starts; the end of the last item is the total (the scan writes it at ipref[nitems], or
    // at *total_dev when the count came from the device)
    auto pref = [&](uint64_t i) -> uint64_t { return i >= a.nitems ? T : a.ipref[i]; };
    const uint64_t nchunks = (T + kPushChunk - 1) / kPushChunk;
    for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
        uint32_t got[kPushPerThread];  // activated vertices of this thread's edges (slot q: edge q)
        uint32_t got_mask = 0;
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
        uint64_t ibeg = pref(it), iend = pref(it + 1);
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
                    iend = pref(it + 1);
                    u = a.q[it / a.P];
                    lbase = a.off[(it % a.P) * a.stride + u];
                    pay = op.payload(u);
                }
                const uint64_t pos = lbase + (e - ibeg);
                wv = a.adj[pos];
                if constexpr (kReduce) act = op.relax(u, pay, wv, pos, acc);
                else act = op.relax(u, pay, wv, pos);
            }
            got[q] = wv;
            if (act) got_mask |= 1u << q;
        }
        // one queue reservation per CTA and chunk (a single counter takes every activation)
        if (a.q_out) {
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = kPushThreads / 32;
            const uint32_t cnt = (uint32_t)__popc(got_mask);
            uint32_t incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            if (lane == 31) s_cnt[warp] = incl;
            __syncthreads();
            if (threadIdx.x == 0) {
                uint32_t t = 0;
                for (int i = 0; i < nw; ++i) {
                    const uint32_t x = s_cnt[i];
                    s_cnt[i] = t;
                    t += x;
                }
                s_cnt[nw] = t ? atomicAdd(a.n_out, t) : 0u;
            }
            __syncthreads();
            uint32_t at = s_cnt[nw] + s_cnt[warp] + incl - cnt;
#pragma unroll
            for (int q = 0; q < kPushPerThread; ++q) {
                if ((got_mask >> q) & 1u) {
                    a.q_out[at++] = got[q];
                    if (a.act_edges) my_act += a.deg[got[q]];
                }
            }
            __syncthreads();  // s_cnt is reused by the next chunk
        }
    }
    if (a.act_edges) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) my_act += __shfl_xor_sync(0xffffffffu, my_act, o);
        if ((threadIdx.x & 31) == 0 && my_act) atomicAdd(a.act_edges, my_act);
    }
    if constexpr (kReduce) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) op.reduce_out(acc);
    }
}

template <class Op>
__global__ void __launch_bounds__(kPushThreads) k_push(Op op, PushArgs a) {
    push_chunks(op, a);
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

// next frontier bitmap -> vertex queue, its length and the out-edges of the queued vertices;
// one warp per 32 words
__device__ __forceinline__ void bm_compact_words(const unsigned long long* __restrict__ bm, uint64_t nwords, uint32_t* q,
                                                 uint32_t* nq, unsigned long long* act_edges,
                                                 const uint32_t* __restrict__ deg) {
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < nwords; base += stride) {
        const uint64_t w = base + lane;
        unsigned long long word = w < nwords ? bm[w] : 0ull;
        const uint32_t cnt = (uint32_t)__popcll(word);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
        if (!tot) continue;
        uint32_t at = 0;
        if (lane == 31) at = atomicAdd(nq, tot);
        at = __shfl_sync(0xffffffffu, at, 31) + incl - cnt;
        unsigned long long d = 0;
        while (word) {
            const uint32_t v = (uint32_t)(w * 64 + (uint64_t)(__ffsll((long long)word) - 1));
            word &= word - 1;
            q[at++] = v;
            d += deg[v];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        if (lane == 0 && act_edges && d) atomicAdd(act_edges, d);
    }
}

static __global__ void k_bm_compact(const unsigned long long* __restrict__ bm, uint64_t nwords, uint32_t* q, uint32_t* nq,
                                    unsigned long long* act_edges, const uint32_t* __restrict__ deg) {
    bm_compact_words(bm, nwords, q, nq, act_edges, deg);
}


}  // namespace eg
