// eg_batch.cu — batched operators over one built graph (no reference counterpart; they batch the
// toolkits of toolkits/{bfs,sssp}.cpp and a personalised PageRank built on pagerank.cpp):
//
//  * eg_msbfs: bit-parallel BFS from up to 64 roots.  Every vertex keeps a u64 of the roots that
//    reached it and a u64 of the roots whose frontier it is in; a level either pushes the queued
//    frontier's words along the CSR or is one chunked pull over the CSC that ORs the
//    in-neighbours' frontier words (exact integer work, levels identical to 64 separate BFS runs).
//  * 64-column row engine: a destination's 64 values (one per seed / source) sit in one 256-byte
//    row; one warp reduces a task of <= kTaskEdges in-edges, each lane owning two columns, so every
//    gathered row is a single coalesced 256-byte read.  Lists longer than a task are split and
//    their partial rows combined in a small per-heavy-vertex buffer.  Used by
//      - eg_ppr: personalised PageRank x_{k+1} = a*e_seed + (1-a) * A^T x_k, A = row-normalised
//        edge weights, FP32;
//      - eg_ppr_backward: the adjoint of K unrolled iterations.  lambda_k = (1-a) A lambda_{k+1} is
//        a pull over the CSR (the transpose of the forward CSC); the same sweep accumulates
//        dL/dA_uv = (1-a) sum_k <x_k[u], lambda_{k+1}[v]>; iterates x_k are recomputed from
//        checkpoints kept every ceil(sqrt(K)) steps;
//      - eg_sssp_batch: Bellman-Ford from up to 64 sources, in place, skipping sources whose
//        distance did not change in the previous sweep (bit-exact least fixpoint).
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "eg_pull.cuh"

namespace eg {

constexpr uint32_t kTaskEdges = 512;
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------------------------
// MS-BFS.  A level is a pull sweep over the CSC when the frontier's out-edges reach E / divisor
// (the switch of core/graph.hpp:1484-1491) and a push over the frontier queue otherwise.  Roots
// whose traversal has ended can add nothing, so a destination whose visited word already holds
// every root still running (`alive`) is skipped, and while the frontier is small a source outside
// the frontier bitmap is not gathered at all.  The traversal kernels only set bits; the next
// frontier is then listed once (k_bm_compact) and its level bytes written from that list
// (k_queue_levels), so no traversal thread loops over the bits of a word.
// L2-coherent (.cg): the persistent traversal reads bitmaps that the same launch wrote
__device__ __forceinline__ bool bm_has(const unsigned long long* bm, uint32_t v) {
    return (__ldcg(bm + (v >> 6)) >> (v & 63)) & 1ull;
}

struct MsBfsPullOp {  // k_pull_direct operator
    using Acc = unsigned long long;
    const unsigned long long* front;
    const unsigned long long* front_bm;  // 1 bit per vertex: front[v] != 0
    int screen;                          // consult front_bm before gathering
    unsigned long long* visit;
    unsigned long long* next;
    unsigned long long* next_bm;
    const unsigned long long* alive;
    const int* stop;  // captured level loops: set once a level found nothing new
    __device__ bool stopped() const { return stop && *(volatile const int*)stop; }
    __device__ bool item_active(uint32_t v) const {
        const unsigned long long al = __ldg(alive);
        return (__ldcg(visit + v) & al) != al;
    }
    __device__ Acc identity() const { return 0ull; }
    __device__ Acc combine(Acc a, Acc b) const { return a | b; }
    __device__ Acc gather(uint32_t u) const {
        if (screen && !bm_has(front_bm, u)) return 0ull;
        return ld_keep(front + u);
    }
    __device__ __forceinline__ void finish_direct(uint32_t v, Acc m) const {
        const unsigned long long fresh = m & ~__ldcg(visit + v);
        if (!fresh) return;
        const unsigned long long nb = fresh & ~atomicOr(visit + v, fresh);
        if (nb && atomicOr(next + v, nb) == 0ull) atomicOr(next_bm + (v >> 6), 1ull << (v & 63));
    }
};

// Early-exit dense level: a destination stops reading in-edges as soon as its visited word holds
// every root still running (nothing more can reach it in this level).  One thread per compressed
// entry reads the first kMsHead in-edges; longer lists continue as kMsSeg-edge segments, one warp
// each, that apply their partial OR every 128 edges so that other segments of the same
// destination see the coverage.  Partial ORs are applied like finish_direct (idempotent).
constexpr uint32_t kMsHead = 8;
constexpr uint32_t kMsSeg = 1024;

struct MsBuArgs {
    const uint32_t* adj;
    const uint64_t* cidx;
    const uint32_t* cvert;
    uint64_t nitems;
    uint32_t V;
    const unsigned long long* front;
    unsigned long long* visit;
    unsigned long long* next;
    unsigned long long* next_bm;
    const unsigned long long* alive;
    unsigned long long* seg;  // (segment << 32) | compressed entry
    uint32_t* nseg;
    const int* stop;  // captured level loops: set once a level found nothing new
};

__device__ __forceinline__ void ms_apply(const MsBuArgs& a, uint32_t v, unsigned long long m) {
    const unsigned long long fresh = m & ~__ldcg(a.visit + v);
    if (!fresh) return;
    const unsigned long long nb = fresh & ~atomicOr(a.visit + v, fresh);
    if (nb && atomicOr(a.next + v, nb) == 0ull) atomicOr(a.next_bm + (v >> 6), 1ull << (v & 63));
}

__device__ __forceinline__ void ms_head_work(const MsBuArgs& a) {
    const int lane = threadIdx.x & 31;
    const unsigned long long al = __ldg(a.alive);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < a.nitems; base += stride) {
        const uint64_t i = base + threadIdx.x;
        uint32_t nsg = 0;
        if (i < a.nitems) {
            const uint32_t v = a.cvert[i];
            const unsigned long long need = v < a.V ? al & ~__ldcg(a.visit + v) : 0ull;
            if (need) {
                const uint64_t s = a.cidx[i], e = a.cidx[i + 1];
                const uint64_t h = e - s > kMsHead ? s + kMsHead : e;
                unsigned long long acc = 0;
                for (uint64_t p = s; p < h && (acc & need) != need; p += 4) {
                    uint32_t u[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) u[q] = p + q < h ? __ldg(a.adj + p + q) : a.V;
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (u[q] < a.V) acc |= ld_keep(a.front + u[q]);
                }
                if (acc & need) ms_apply(a, v, acc);
                if ((acc & need) != need && e > h) nsg = (uint32_t)((e - h + kMsSeg - 1) / kMsSeg);
            }
        }
        uint32_t incl = nsg;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
        if (tot) {
            uint32_t at = 0;
            if (lane == 31) at = atomicAdd(a.nseg, tot);
            at = __shfl_sync(0xffffffffu, at, 31) + incl - nsg;
            for (uint32_t k = 0; k < nsg; ++k) a.seg[at + k] = ((unsigned long long)k << 32) | (uint32_t)i;
        }
    }
}

__global__ void __launch_bounds__(256) k_ms_head(MsBuArgs a) {
    if (a.stop && *(volatile const int*)a.stop) return;
    ms_head_work(a);
}

__device__ __forceinline__ void ms_tail_work(const MsBuArgs& a) {
    const uint32_t n = __ldcg(a.nseg);
    const int lane = threadIdx.x & 31;
    const unsigned long long al = __ldg(a.alive);
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < n; t += nwarps) {
        const unsigned long long ent = a.seg[t];
        const uint32_t i = (uint32_t)ent;
        const uint32_t v = a.cvert[i];
        const uint64_t e = a.cidx[i + 1];
        uint64_t p = a.cidx[i] + kMsHead + (ent >> 32) * kMsSeg;
        const uint64_t pe = p + kMsSeg < e ? p + kMsSeg : e;
        for (; p < pe; p += 128) {
            const unsigned long long vis = __shfl_sync(0xffffffffu, __ldcg(a.visit + v), 0);
            if ((vis & al) == al) break;  // every running root already reached v
            unsigned long long acc = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint64_t x = p + 32 * q + lane;
                if (x < pe) acc |= ld_keep(a.front + __ldg(a.adj + x));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) acc |= __shfl_xor_sync(0xffffffffu, acc, o);
            if (lane == 0 && (acc & ~vis)) ms_apply(a, v, acc);
        }
    }
}

__global__ void __launch_bounds__(256) k_ms_tail(MsBuArgs a) {
    if (a.stop && *(volatile const int*)a.stop) return;
    ms_tail_work(a);
}

struct MsBfsPushOp {
    const unsigned long long* front;
    unsigned long long* visit;
    unsigned long long* next;
    unsigned long long* next_bm;
    __device__ unsigned long long payload(uint32_t u) const { return __ldcg(front + u); }
    __device__ bool relax(uint32_t, unsigned long long pay, uint32_t w, uint64_t) const {
        const unsigned long long m = pay & ~__ldcg(visit + w);
        if (!m) return false;
        const unsigned long long nb = m & ~atomicOr(visit + w, m);
        if (!nb || atomicOr(next + w, nb) != 0ull) return false;
        atomicOr(next_bm + (w >> 6), 1ull << (w & 63));
        return true;  // w joins the next frontier's queue
    }
};

// level bytes of the queued vertices' new bits (row v of [V][64]: 2 threads, two 16-byte quarters
// each, a quarter rewritten only where one of its roots is new) and the OR of their words, i.e.
// the roots whose traversal is still running
// With new_id, the words are also copied to renumbered positions (next_r[new_id[v]]) for the pull
// gathers that go through the renumbered CSC sources.
__device__ __forceinline__ void queue_levels_work(const uint32_t* __restrict__ q, uint32_t n,
                                                  const unsigned long long* __restrict__ next, uint8_t* levels,
                                                  uint32_t lvl, unsigned long long* alive_out,
                                                  const uint32_t* __restrict__ new_id,
                                                  unsigned long long* __restrict__ next_r) {
    const uint32_t sub = threadIdx.x & 1u;
    const uint32_t fill = (lvl & 0xFFu) * 0x01010101u;
    unsigned long long orr = 0;
    for (uint64_t i = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 1; i < n;
         i += ((uint64_t)gridDim.x * blockDim.x) >> 1) {
        const uint32_t v = q[i];
        const unsigned long long nb = next[v];
        if (new_id && sub == 0) next_r[new_id[v]] = nb;
        orr |= nb;
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const uint32_t quarter = sub * 2 + c;
            const uint32_t h = (uint32_t)(nb >> (16 * quarter)) & 0xFFFFu;
            if (levels && h) {
                uint4* p = reinterpret_cast<uint4*>(levels + (uint64_t)v * 64) + quarter;
                uint4 x = *p;
                uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    // bit j of the nibble -> byte j all ones (the shifted copies never overlap)
                    const uint32_t nib = (h >> (4 * k)) & 0xFu;
                    const uint32_t m = ((nib * 0x00204081u) & 0x01010101u) * 0xFFu;
                    w[k] = (w[k] & ~m) | (fill & m);
                }
                *p = make_uint4(w[0], w[1], w[2], w[3]);
            }
        }
    }
    if (!alive_out) return;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) orr |= __shfl_xor_sync(0xffffffffu, orr, o);
    if ((threadIdx.x & 31) == 0 && orr) atomicOr(alive_out, orr);
}

__global__ void k_queue_levels(const uint32_t* __restrict__ q, const uint32_t* n_dev,
                               const unsigned long long* __restrict__ next, uint8_t* levels, uint32_t lvl,
                               unsigned long long* alive_out, const uint32_t* __restrict__ new_id,
                               unsigned long long* __restrict__ next_r) {
    queue_levels_work(q, __ldcg(n_dev), next, levels, lvl, alive_out, new_id, next_r);
}

// zero the frontier words (and their renumbered copies) of the vertices a queue lists: the only
// non-zero entries of a frontier array, cheaper than clearing all of it while frontiers are small
__global__ void k_clear_front(const uint32_t* __restrict__ q, uint32_t n, unsigned long long* __restrict__ word,
                              const uint32_t* __restrict__ new_id, unsigned long long* __restrict__ word_r) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = q[i];
        word[v] = 0ull;
        if (word_r) word_r[new_id[v]] = 0ull;
    }
}

// the renumbered copy of the first frontier (the roots), which no level has listed
__global__ void k_front_renumber(const uint32_t* __restrict__ q, const uint32_t* n_dev,
                                 const unsigned long long* __restrict__ word, const uint32_t* __restrict__ new_id,
                                 unsigned long long* __restrict__ word_r) {
    const uint32_t n = __ldcg(n_dev);
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        word_r[new_id[q[i]]] = word[q[i]];
}

// sum over vertices of popcount(visited word) * out-degree: the edges 64 single-root runs scan
__global__ void k_reach_edges(const unsigned long long* __restrict__ visit, const uint32_t* __restrict__ deg, uint64_t V,
                              unsigned long long* out) {
    unsigned long long acc = 0;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x)
        acc += (unsigned long long)__popcll(visit[v]) * deg[v];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// [V][64] level rows -> [n][V] root rows for the first n roots, 64 vertices per CTA: rows come in
// as 16-byte loads, leave as 16-byte stores of 16 consecutive vertices (vec: V % 16 == 0 and out
// 16-byte aligned; bytes otherwise).  A byte whose root never reached the vertex (its visited bit
// is clear) becomes 0xFF, so the level rows need no initialisation.
__global__ void __launch_bounds__(256) k_levels_out(const uint8_t* __restrict__ lev,
                                                    const unsigned long long* __restrict__ visit, uint32_t V, int n,
                                                    uint8_t* __restrict__ out, int vec) {
    __shared__ __align__(16) uint8_t t[64][68];  // 68-byte rows: column reads spread over banks
    const uint64_t v0 = (uint64_t)blockIdx.x * 64;
    {
        const int r = threadIdx.x >> 2, q = threadIdx.x & 3;
        const uint64_t v = v0 + r;
        uint32_t w[4] = {~0u, ~0u, ~0u, ~0u};
        if (v < V) {
            const uint4 x = *reinterpret_cast<const uint4*>(lev + v * 64 + 16 * q);
            const unsigned long long vis = visit[v];
            w[0] = x.x;
            w[1] = x.y;
            w[2] = x.z;
            w[3] = x.w;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint32_t nib = (uint32_t)(vis >> (16 * q + 4 * j)) & 0xFu;
                const uint32_t m = ((nib * 0x00204081u) & 0x01010101u) * 0xFFu;  // bit k -> byte k
                w[j] = (w[j] & m) | ~m;
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) *reinterpret_cast<uint32_t*>(&t[r][16 * q + 4 * j]) = w[j];
    }
    __syncthreads();
    const int s = threadIdx.x >> 2, k = threadIdx.x & 3;
    if (s >= n) return;
    const uint64_t vb = v0 + 16 * (uint64_t)k;
    uint8_t* o = out + (uint64_t)s * V + vb;
    if (vec && vb + 16 <= V) {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int b = 16 * k + 4 * j;
            w[j] = (uint32_t)t[b][s] | ((uint32_t)t[b + 1][s] << 8) | ((uint32_t)t[b + 2][s] << 16) |
                   ((uint32_t)t[b + 3][s] << 24);
        }
        *reinterpret_cast<uint4*>(o) = make_uint4(w[0], w[1], w[2], w[3]);
    } else {
        for (int j = 0; j < 16; ++j)
            if (vb + j < V) o[j] = t[16 * k + j][s];
    }
}

template <typename T>
__global__ void k_transpose_rows(const T* __restrict__ in, uint32_t V, int n, T* __restrict__ out) {
    __shared__ T t[64][33];
    const uint64_t v0 = (uint64_t)blockIdx.x * 32;
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const uint64_t v = v0 + i;
        for (int s = threadIdx.x; s < 64; s += blockDim.x) t[s][i] = v < V ? in[v * 64 + s] : T(0);
    }
    __syncthreads();
    for (int s = threadIdx.y; s < n; s += blockDim.y) {
        const uint64_t v = v0 + threadIdx.x;
        if (v < V) out[(uint64_t)s * V + v] = t[s][threadIdx.x];
    }
}

template <typename T>
__global__ void k_untranspose_rows(const T* __restrict__ in, uint32_t V, int n, T* __restrict__ out) {
    __shared__ T t[64][33];
    const uint64_t v0 = (uint64_t)blockIdx.x * 32;
    for (int s = threadIdx.y; s < 64; s += blockDim.y) {
        const uint64_t v = v0 + threadIdx.x;
        t[s][threadIdx.x] = (s < n && v < V) ? in[(uint64_t)s * V + v] : T(0);
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += blockDim.y) {
        const uint64_t v = v0 + i;
        for (int s = threadIdx.x; s < 64; s += blockDim.x)
            if (v < V) out[v * 64 + s] = t[s][i];
    }
}

// ---------------------------------------------------------------------------------------------
// tasks: item i of a list index (begin[i], begin[i+1]) split into pieces of <= kTaskEdges edges
struct TaskLoad {
    const uint64_t* begin;
    __device__ uint32_t operator()(uint64_t i) const {
        const uint64_t n = begin[i + 1] - begin[i];
        return (uint32_t)((n + kTaskEdges - 1) / kTaskEdges);
    }
};
struct TaskEpi {
    uint32_t* t_item;
    uint32_t* t_part;
    uint32_t* heavy_slot;     // per item
    uint32_t* heavy_item;     // per slot
    uint32_t* nheavy;
    __device__ void operator()(uint64_t i, uint64_t excl, uint32_t cnt) const {
        for (uint32_t p = 0; p < cnt; ++p) {
            t_item[excl + p] = (uint32_t)i;
            t_part[excl + p] = p;
        }
        uint32_t slot = kNoSlot;
        if (cnt > 1) {
            slot = atomicAdd(nheavy, 1u);
            heavy_item[slot] = (uint32_t)i;
        }
        heavy_slot[i] = slot;
    }
};

struct RowTasks {
    DevBuf item, part, heavy_slot, heavy_item, counts;
    uint64_t ntasks = 0;
    uint32_t nheavy = 0;
    uint64_t nitems = 0;
    const uint64_t* begin = nullptr;
};

static int make_tasks(eg_graph* g, RowTasks& t, const uint64_t* begin, uint64_t nitems) {
    // upper bound on tasks: items + E / kTaskEdges
    const uint64_t cap = nitems + g->E / kTaskEdges + 2;
    EG_TRY(t.item.reserve(sizeof(uint32_t) * cap));
    EG_TRY(t.part.reserve(sizeof(uint32_t) * cap));
    EG_TRY(t.heavy_slot.reserve(sizeof(uint32_t) * (nitems + 1)));
    EG_TRY(t.heavy_item.reserve(sizeof(uint32_t) * (g->E / kTaskEdges + 2)));
    EG_TRY(t.counts.reserve(32));
    EG_CUDA(cudaMemsetAsync(t.counts.ptr, 0, 32, g->stream));
    uint64_t* d_total = t.counts.as<uint64_t>();
    uint32_t* d_nheavy = reinterpret_cast<uint32_t*>(t.counts.as<uint64_t>() + 1);
    TaskEpi ep{t.item.as<uint32_t>(), t.part.as<uint32_t>(), t.heavy_slot.as<uint32_t>(), t.heavy_item.as<uint32_t>(),
               d_nheavy};
    EG_TRY(launch_scan(g, TaskLoad{begin}, ep, nitems, d_total, "row_tasks"));
    uint64_t h[2] = {0, 0};
    EG_CUDA(cudaMemcpyAsync(h, t.counts.ptr, 16, cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    t.ntasks = nitems ? h[0] : 0;
    t.nheavy = (uint32_t)(h[1] & 0xFFFFFFFFu);
    t.nitems = nitems;
    t.begin = begin;
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
// row kernels: warp per task, lane l owns columns 2l, 2l+1 of a 64-column row (float2)
struct RowArgs {
    const uint32_t* t_item;
    const uint32_t* t_part;
    uint64_t ntasks;
    const uint32_t* heavy_slot;
    const uint32_t* item_vertex;  // null: item index is the vertex
    const uint64_t* begin;        // list offsets per item (item i: [begin[i], begin[i+1]))
    const uint32_t* adj;
    const float* w;               // per-edge weight (normalised for PPR, raw for SSSP)
};

// PPR forward: y[v] = (1-a) * sum_{u in in(v)} wn_uv * x[u]
// rows gathered together per warp in the row sweeps (independent 256-byte loads in flight).  The
// PPR adjoint at 2^22/2^26, K = 50: 717 ms one row at a time, 650 ms at 4, 575 ms at 8, 616 ms at 16
// (78 registers); the forward 176 ms at 4, 174 ms at 8
constexpr int kRowGather = 8;

__global__ void __launch_bounds__(256) k_row_spmm(RowArgs a, const float2* __restrict__ x, float2* __restrict__ y,
                                                   float2* __restrict__ heavy_acc, float scale) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = warp; t < a.ntasks; t += nwarps) {
        const uint32_t it = a.t_item[t];
        const uint64_t lb = a.begin[it], le = a.begin[it + 1];
        const uint64_t e0 = lb + (uint64_t)a.t_part[t] * kTaskEdges;
        const uint64_t e1 = e0 + kTaskEdges < le ? e0 + kTaskEdges : le;
        float2 acc = make_float2(0.f, 0.f);
        uint64_t e = e0;
        for (; e + kRowGather <= e1; e += kRowGather) {
            uint32_t u[kRowGather];
            float wv[kRowGather];
#pragma unroll
            for (int j = 0; j < kRowGather; ++j) {
                u[j] = __ldg(a.adj + e + j);
                wv[j] = __ldg(a.w + e + j);
            }
            float2 r[kRowGather];
#pragma unroll
            for (int j = 0; j < kRowGather; ++j) r[j] = __ldcg(x + (uint64_t)u[j] * 32 + lane);
#pragma unroll
            for (int j = 0; j < kRowGather; ++j) {
                acc.x = fmaf(wv[j], r[j].x, acc.x);
                acc.y = fmaf(wv[j], r[j].y, acc.y);
            }
        }
        for (; e < e1; ++e) {
            const uint32_t u = __ldg(a.adj + e);
            const float wv = __ldg(a.w + e);
            const float2 r = __ldcg(x + (uint64_t)u * 32 + lane);
            acc.x = fmaf(wv, r.x, acc.x);
            acc.y = fmaf(wv, r.y, acc.y);
        }
        const uint32_t v = a.item_vertex ? a.item_vertex[it] : it;
        const uint32_t slot = a.heavy_slot[it];
        if (slot == kNoSlot) {
            y[(uint64_t)v * 32 + lane] = make_float2(scale * acc.x, scale * acc.y);
        } else {
            atomicAdd(&heavy_acc[(uint64_t)slot * 32 + lane].x, acc.x);
            atomicAdd(&heavy_acc[(uint64_t)slot * 32 + lane].y, acc.y);
        }
    }
}

__global__ void k_row_heavy_finish(const uint32_t* __restrict__ heavy_item, const uint32_t* __restrict__ item_vertex,
                                   uint32_t nheavy, float2* __restrict__ heavy_acc, float2* __restrict__ y, float scale) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    const uint64_t slot = i >> 5;
    const int lane = threadIdx.x & 31;
    if (slot >= nheavy) return;
    const uint32_t it = heavy_item[slot];
    const uint32_t v = item_vertex ? item_vertex[it] : it;
    const float2 a = heavy_acc[slot * 32 + lane];
    heavy_acc[slot * 32 + lane] = make_float2(0.f, 0.f);
    y[(uint64_t)v * 32 + lane] = make_float2(scale * a.x, scale * a.y);
}

// y[seed_s][s] += a
__global__ void k_ppr_teleport(const uint32_t* seeds, int n, float* y, float alpha) {
    const int s = threadIdx.x;
    if (s < n) atomicAdd(y + (uint64_t)seeds[s] * 64 + s, alpha);
}
__global__ void k_ppr_init(const uint32_t* seeds, int n, float* x) {
    const int s = threadIdx.x;
    if (s < n) x[(uint64_t)seeds[s] * 64 + s] = 1.0f;
}

// normalised weights: wn[e] = w[eid[e]] / s[src], s[u] = sum of u's out-weights
__global__ void k_out_weight_sums(const uint64_t* __restrict__ csr_off, const float* __restrict__ csr_eid,
                                  const float* __restrict__ w_in, uint32_t V, float* __restrict__ s) {
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < V; u += (uint64_t)gridDim.x * blockDim.x) {
        double acc = 0;
        for (uint64_t e = csr_off[u]; e < csr_off[u + 1]; ++e) acc += w_in[__float_as_uint(csr_eid[e])];
        s[u] = (float)acc;
    }
}
__global__ void k_gather_norm_w(const uint32_t* __restrict__ nbr_is_src, const float* __restrict__ eid,
                                const float* __restrict__ w_in, const float* __restrict__ s, uint64_t E,
                                float* __restrict__ wn) {
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t id = __float_as_uint(eid[e]);
        wn[e] = w_in[id] / s[nbr_is_src[e]];
    }
}
// CSR positions: the source of position e is the row it sits in
__global__ void k_row_of(const uint64_t* __restrict__ off, uint32_t V, uint32_t* __restrict__ row) {
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < V; u += (uint64_t)gridDim.x * blockDim.x)
        for (uint64_t e = off[u]; e < off[u + 1]; ++e) row[e] = (uint32_t)u;
}

// ---- adjoint sweep over the CSR: for a source row u,
//   lam_out[u] = (1-a) * sum_{v in out(u)} wn_uv * lam_in[v]
//   gA[e]     += (1-a) * <x_k[u], lam_in[v]>      (per CSR edge e = (u, v))
__global__ void __launch_bounds__(256) k_row_adjoint(RowArgs a, const float2* __restrict__ lam_in,
                                                      const float2* __restrict__ xk, float2* __restrict__ lam_out,
                                                      float2* __restrict__ heavy_acc, float* __restrict__ gA,
                                                      float scale) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = warp; t < a.ntasks; t += nwarps) {
        const uint32_t u = a.t_item[t];  // CSR items are vertices
        const uint64_t lb = a.begin[u], le = a.begin[u + 1];
        const uint64_t e0 = lb + (uint64_t)a.t_part[t] * kTaskEdges;
        const uint64_t e1 = e0 + kTaskEdges < le ? e0 + kTaskEdges : le;
        const float2 xu = __ldcg(xk + (uint64_t)u * 32 + lane);
        float2 acc = make_float2(0.f, 0.f);
        uint64_t e = e0;
        // kRowGather edges at a time: their rows are gathered together (as in k_row_spmm), and the
        // first kRowGather lanes hold their gA entries; each dot product is summed over the warp
        // in the same order as for a single edge, so the result does not depend on the grouping
        for (; e + kRowGather <= e1; e += kRowGather) {
            uint32_t v[kRowGather];
            float wv[kRowGather];
#pragma unroll
            for (int j = 0; j < kRowGather; ++j) {
                v[j] = __ldg(a.adj + e + j);
                wv[j] = __ldg(a.w + e + j);
            }
            const float g_old = lane < kRowGather ? gA[e + lane] : 0.f;
            float2 l[kRowGather];
#pragma unroll
            for (int j = 0; j < kRowGather; ++j) l[j] = __ldcg(lam_in + (uint64_t)v[j] * 32 + lane);
            float d[kRowGather];
#pragma unroll
            for (int j = 0; j < kRowGather; ++j) {
                acc.x = fmaf(wv[j], l[j].x, acc.x);
                acc.y = fmaf(wv[j], l[j].y, acc.y);
                d[j] = fmaf(xu.x, l[j].x, xu.y * l[j].y);
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
#pragma unroll
                for (int j = 0; j < kRowGather; ++j) d[j] += __shfl_xor_sync(0xffffffffu, d[j], o);
            }
            float dl = d[0];
#pragma unroll
            for (int j = 1; j < kRowGather; ++j) dl = lane == j ? d[j] : dl;
            if (lane < kRowGather) gA[e + lane] = fmaf(scale, dl, g_old);
        }
        for (; e < e1; ++e) {
            const uint32_t v = __ldg(a.adj + e);
            const float wv = __ldg(a.w + e);
            const float2 l = __ldcg(lam_in + (uint64_t)v * 32 + lane);
            acc.x = fmaf(wv, l.x, acc.x);
            acc.y = fmaf(wv, l.y, acc.y);
            float d = fmaf(xu.x, l.x, xu.y * l.y);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
            if (lane == 0) gA[e] = fmaf(scale, d, gA[e]);
        }
        const uint32_t slot = a.heavy_slot[u];
        if (slot == kNoSlot) {
            lam_out[(uint64_t)u * 32 + lane] = make_float2(scale * acc.x, scale * acc.y);
        } else {
            atomicAdd(&heavy_acc[(uint64_t)slot * 32 + lane].x, acc.x);
            atomicAdd(&heavy_acc[(uint64_t)slot * 32 + lane].y, acc.y);
        }
    }
}

// dL/dw_e = (gA_e - sum_{e' in row(u)} wn_e' gA_e') / s_u, scattered to the input edge order
__global__ void k_weight_grad(const uint64_t* __restrict__ off, uint32_t V, const float* __restrict__ wn,
                              const float* __restrict__ gA, const float* __restrict__ s,
                              const float* __restrict__ eid, float* __restrict__ dw) {
    for (uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; u < V; u += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t b = off[u], e1 = off[u + 1];
        if (b == e1) continue;
        double dot = 0;
        for (uint64_t e = b; e < e1; ++e) dot += (double)wn[e] * gA[e];
        const float inv = 1.0f / s[u];
        for (uint64_t e = b; e < e1; ++e) dw[__float_as_uint(eid[e])] = (float)(((double)gA[e] - dot) * inv);
    }
}

// lam_K = dL/dx_K given in [V][64]; nothing else to seed
// ---- batched SSSP: in place, skipping sources whose row did not change in the last sweep --------
__global__ void __launch_bounds__(256) k_row_sssp(RowArgs a, float2* __restrict__ dist,
                                                   const uint8_t* __restrict__ changed_prev,
                                                   uint8_t* __restrict__ changed_next, int* __restrict__ any) {
    const int lane = threadIdx.x & 31;
    const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = warp; t < a.ntasks; t += nwarps) {
        const uint32_t it = a.t_item[t];
        const uint64_t lb = a.begin[it], le = a.begin[it + 1];
        const uint64_t e0 = lb + (uint64_t)a.t_part[t] * kTaskEdges;
        const uint64_t e1 = e0 + kTaskEdges < le ? e0 + kTaskEdges : le;
        float2 best = make_float2(1e9f, 1e9f);
        // 32 in-edges per step: ids, weights and "source changed" flags are loaded one per lane,
        // then the rows of the changed sources are gathered four at a time (min is exact, so the
        // order does not matter)
        for (uint64_t eb = e0; eb < e1; eb += 32) {
            const uint64_t e = eb + lane;
            uint32_t u = 0;
            float wv = 0.f;
            bool ch = false;
            if (e < e1) {
                u = __ldg(a.adj + e);
                wv = __ldg(a.w + e);
                ch = __ldcg(changed_prev + u) != 0;
            }
            unsigned m = __ballot_sync(0xffffffffu, ch);
            while (m) {  // m is the same in every lane
                int sl[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    sl[j] = m ? __ffs(m) - 1 : -1;
                    if (m) m &= m - 1;
                }
                float2 r[4];
                float wj[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (sl[j] >= 0) {
                        const uint32_t uj = __shfl_sync(0xffffffffu, u, sl[j]);
                        wj[j] = __shfl_sync(0xffffffffu, wv, sl[j]);
                        r[j] = __ldcg(dist + (uint64_t)uj * 32 + lane);
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (sl[j] >= 0) {
                        best.x = fminf(best.x, r[j].x + wj[j]);  // toolkits/sssp.cpp:55: relax_dist = msg + w
                        best.y = fminf(best.y, r[j].y + wj[j]);
                    }
                }
            }
        }
        const uint32_t v = a.item_vertex[it];
        float2* dv = dist + (uint64_t)v * 32 + lane;
        bool lowered = false;
        if (best.x < __ldcg(&dv->x)) lowered |= best.x < __int_as_float(atomicMin(reinterpret_cast<int*>(&dv->x), __float_as_int(best.x)));
        if (best.y < __ldcg(&dv->y)) lowered |= best.y < __int_as_float(atomicMin(reinterpret_cast<int*>(&dv->y), __float_as_int(best.y)));
        if (__any_sync(0xffffffffu, lowered) && lane == 0) {
            changed_next[v] = 1;
            *any = 1;
        }
    }
}

__global__ void k_fill_f32_rows(float* p, uint64_t n, float v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) p[i] = v;
}

// {src, dst} records -> {src, dst, index} records: the index rides through the build in the weight
// slot, so every CSR / CSC position knows which input edge it holds
__global__ void k_expand_ids(const uint2* __restrict__ in, uint64_t E, uint32_t* __restrict__ out) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint2 r = in[i];
        out[3 * i] = r.x;
        out[3 * i + 1] = r.y;
        out[3 * i + 2] = (uint32_t)i;
    }
}

int expand_with_ids(eg_graph* g, const uint8_t* rec8_dev, uint64_t E) {
    if (!E) return EG_OK;
    k_expand_ids<<<grid_for(E, 256, 152u * 16u), 256, 0, g->stream>>>(reinterpret_cast<const uint2*>(rec8_dev), E,
                                                                      g->edges.as<uint32_t>());
    EG_CHECK_LAUNCH("k_expand_ids");
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
struct BatchState {
    DevBuf a64, b64, c64, lev, rows0, rows1, heavy, tmp_out, seeds, wn_csc, wn_csr, s_out, gA, row_of, ck, seg;
    DevBuf ch0, ch1, flag, level_cnt, entries, n_entries, bm0, bm1, alive, ms_seg;
    DevBuf cap;      // captured level loop: per-level direction decisions and frontier edge counts
    DevBuf persist;  // persistent traversal: per-level counts, barrier words, error flag
    DevBuf wr0, wr1;  // frontier words in renumbered order (pull gathers through renumbered sources)
    RowTasks csc_tasks, csr_tasks;
    bool csc_ready = false, csr_ready = false;
    // captured MS-BFS level loop and the shapes it was captured for
    void* graph_exec = nullptr;
    uint64_t graph_V = 0;
    bool graph_lev = false;
    uint32_t graph_entries = 0;
    int graph_nbits = 0;
    int graph_div = 0;  // the switch's divisor the captured levels compare with
    ~BatchState() {
        if (graph_exec) cudaGraphExecDestroy((cudaGraphExec_t)graph_exec);
    }
};

static BatchState& bstate(eg_graph* g) {
    if (!g->batch) g->batch = new BatchState();
    return *static_cast<BatchState*>(g->batch);
}

void free_batch_state(eg_graph* g) {
    delete static_cast<BatchState*>(g->batch);
    g->batch = nullptr;
}

static int copy_small_in(eg_graph* g, DevBuf& dst, const uint32_t* src, int n, int where) {
    EG_TRY(dst.reserve(sizeof(uint32_t) * 64));
    EG_CUDA(cudaMemcpyAsync(dst.ptr, src, sizeof(uint32_t) * n,
                            where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, g->stream));
    return EG_OK;
}

static int check_roots(eg_graph* g, const uint32_t* roots, int n, int where, const char* fn) {
    if (!roots || n < 1 || n > 64) {
        set_error("%s: need 1..64 roots", fn);
        return EG_ERR_INVALID;
    }
    std::vector<uint32_t> h(n);
    EG_CUDA(cudaMemcpy(h.data(), roots, sizeof(uint32_t) * n,
                       where == EG_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    for (int i = 0; i < n; ++i)
        if (h[i] >= g->V) {
            set_error("%s: root %u >= V %u", fn, h[i], g->V);
            return EG_ERR_INVALID;
        }
    return EG_OK;
}

// root entries (global vertex, bit) from n roots: entry s = (roots[s] + base, s)
__global__ void k_root_entries(const uint32_t* roots, int n, uint32_t base, uint2* ent) {
    const int s = threadIdx.x;
    if (s < n) ent[s] = make_uint2(roots[s] + base, (uint32_t)s);
}

// per-graph roots of a graph batch: entry (g * nper + s) = (voff[g] + roots[g * nper + s], s)
__global__ void k_root_entries_graphs(const uint32_t* roots, const uint64_t* voff, uint32_t ngraphs, int nper,
                                      uint2* ent) {
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i < (uint64_t)ngraphs * nper) {
        const uint64_t gi = i / nper;
        ent[i] = make_uint2((uint32_t)(voff[gi] + roots[i]), (uint32_t)(i % nper));
    }
}

__global__ void k_msbfs_init_entries(const uint2* ent, const uint32_t* n_dev, unsigned long long* visit,
                                     unsigned long long* front, unsigned long long* front_bm, uint8_t* levels,
                                     uint32_t* q, uint32_t* nq, unsigned long long* act_edges, const uint32_t* deg) {
    const uint32_t n = *n_dev;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t v = ent[i].x, s = ent[i].y;
        const unsigned long long bit = 1ull << s;
        const unsigned long long old = atomicOr(visit + v, bit);
        if (atomicOr(front + v, bit) == 0ull) {
            atomicOr(front_bm + (v >> 6), 1ull << (v & 63));
            q[atomicAdd(nq, 1u)] = v;
            atomicAdd(act_edges, (unsigned long long)deg[v]);
        }
        if (!(old & bit) && levels) levels[(uint64_t)v * 64 + s] = 0;
    }
}

constexpr int kGraphLevels = 16;

// The captured level loop makes, on the device, the choice the host loop makes per level: each
// level's first kernel reads the frontier's length and out-edges and arms either the pull kernels
// (the chunked sweep for the first dense level, the early-exit pair after it on one graph) or the
// push (a scan and expansion whose item count it sets); the kernels of the other path find
// nothing to do.  After an empty frontier every later level is disarmed.
struct CapLevel {
    uint32_t n_push;   // queue length handed to the push scan and expansion (0: pull level)
    int skip_direct;   // k_pull_direct (MsBfsPullOp::stop)
    int skip_early;    // k_ms_head / k_ms_tail (MsBuArgs::stop)
    int pad;
};
struct CapState {
    CapLevel lv[kGraphLevels];
    unsigned long long act[kGraphLevels];  // out-edges of the frontier level L produced
    uint64_t push_total;                   // edges of the current push level (scan total)
    int dense_count;
    int stop;
};

__global__ void k_cap_decide(CapState* st, int L, const uint32_t* n_src, const unsigned long long* act_src,
                             unsigned long long dense_min, int early_after_first, int built_csr) {
    CapLevel& c = st->lv[L];
    const uint32_t n = *n_src;
    if (st->stop || n == 0) {
        st->stop = 1;
        c.n_push = 0;
        c.skip_direct = c.skip_early = 1;
        return;
    }
    const bool dense = !built_csr || *act_src >= dense_min;
    const bool early = dense && early_after_first && st->dense_count > 0;
    c.n_push = dense ? 0u : n;
    c.skip_direct = !(dense && !early);
    c.skip_early = !(dense && early);
    if (dense) ++st->dense_count;
}

// zero the frontier words a queue lists (its length read on the device), or the whole array when
// the queue is long; nothing once the loop has stopped
__global__ void k_clear_front_dev(const uint32_t* __restrict__ q, const uint32_t* n_dev, unsigned long long* word,
                                  uint64_t V, const CapState* st) {
    if (st->stop) return;
    const uint32_t n = __ldcg(n_dev);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    if ((uint64_t)n > V / 32) {
        for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += stride) word[v] = 0ull;
    } else {
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += stride) word[q[i]] = 0ull;
    }
}

// ---------------------------------------------------------------------------------------------
// The whole bit-parallel traversal in one persistent launch (EG_OPT_BATCH_LAUNCH = 1): every
// resident CTA runs every level, phase by phase, with a grid barrier between phases -- the same
// phases as the host-driven loop (clear, push or pull by the E / divisor switch, list the next
// frontier, level bytes), with the switch and the queue lengths read on the device.  A launch
// that could not keep all its CTAs resident is refused by the cooperative launch, and every
// barrier wait is bounded: on exhaustion the error flag is raised and the kernel returns.
constexpr int kMaxLevels = 256;

struct PersistWords {
    uint32_t cnt[kMaxLevels];          // queue length produced by level L
    unsigned long long act[kMaxLevels];  // out-edges of that queue
    uint32_t nseg[kMaxLevels];         // early-exit segments of level L
    uint32_t ticket[kMaxLevels];       // scan tile tickets of level L
    uint32_t chunk[kMaxLevels];        // pull chunk tickets of level L
    uint64_t total[kMaxLevels];        // push edges of level L
    unsigned bar_count, bar_gen;
    int err;
    uint32_t levels, pushes;
};

struct MsPersistArgs {
    uint64_t V, nwords;
    int P;
    const uint64_t* csr_off;
    const uint32_t* csr_adj;
    const uint32_t* gather_adj;
    const uint64_t* cidx;
    const uint32_t* cvert;
    uint64_t nitems;
    const uint32_t* pull_chunk_item;
    uint64_t E;
    const uint32_t* deg;
    unsigned long long* visit;
    unsigned long long* word0;
    unsigned long long* word1;
    unsigned long long* bm0;
    unsigned long long* bm1;
    uint32_t* q0;
    uint32_t* q1;
    const unsigned long long* alive_all;
    uint8_t* lev;
    unsigned long long* ms_seg;
    uint64_t* desc;
    uint64_t* ipref;
    uint32_t* push_chunk_item;
    const uint32_t* init_n;
    const unsigned long long* init_act;
    unsigned long long dense_min;
    int early_after_first, built_csr;
    PersistWords* w;
};

// bounded grid barrier (all CTAs resident): false when a wait ran out
__device__ __forceinline__ bool grid_barrier(PersistWords* w) {
    return grid_sync_bounded(&w->bar_count, &w->bar_gen, &w->err);
}

__global__ void __launch_bounds__(256, 4) k_msbfs_persistent(MsPersistArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    PersistWords* w = a.w;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t n = __ldcg(a.init_n);
    unsigned long long act = __ldcg(a.init_act);
    int dense_count = 0;
    for (uint32_t L = 0; L < 254 && n > 0; ++L) {
        const int c = L & 1;
        unsigned long long* front = c ? a.word1 : a.word0;
        unsigned long long* next = c ? a.word0 : a.word1;
        const unsigned long long* front_bm = c ? a.bm1 : a.bm0;
        unsigned long long* next_bm = c ? a.bm0 : a.bm1;
        const uint32_t* q = c ? a.q1 : a.q0;
        uint32_t* q_next = c ? a.q0 : a.q1;
        const bool dense = !a.built_csr || act >= a.dense_min;
        const bool early = dense && a.early_after_first && dense_count > 0;
        // clear: the next-frontier words (set two levels back, listed by q_next; level 0: all of
        // them), its bitmap, and the scan descriptors of a push level
        {
            const uint32_t n_old = L == 0 ? 0xFFFFFFFFu : (L == 1 ? __ldcg(a.init_n) : __ldcg(&w->cnt[L - 2]));
            if (n_old > a.V / 32) {
                for (uint64_t v = tid; v < a.V; v += stride) next[v] = 0ull;
            } else {
                for (uint64_t i = tid; i < n_old; i += stride) next[q_next[i]] = 0ull;
            }
            for (uint64_t i = tid; i < a.nwords; i += stride) next_bm[i] = 0ull;
            if (!dense) {
                const uint64_t tiles = ((uint64_t)n * a.P + kScanTile - 1) / kScanTile + 1;
                for (uint64_t i = tid; i < tiles; i += stride) a.desc[i] = 0ull;
            }
        }
        if (!grid_barrier(w)) return;
        if (dense && early) {
            MsBuArgs ma{a.gather_adj, a.cidx, a.cvert, a.nitems, (uint32_t)a.V, front, a.visit, next, next_bm,
                        a.alive_all, a.ms_seg, &w->nseg[L], nullptr};
            ms_head_work(ma);
            if (!grid_barrier(w)) return;
            ms_tail_work(ma);
        } else if (dense) {
            MsBfsPullOp op{front, front_bm, (uint64_t)n * 16 < a.V ? 1 : 0, a.visit, next, next_bm, a.alive_all, nullptr};
            pull_direct_chunks(op, a.gather_adj, a.cidx, a.cvert, a.pull_chunk_item, a.E, a.nitems, (uint32_t)a.V,
                               s_raw, &w->chunk[L]);
        } else {
            const uint64_t items = (uint64_t)n * a.P;
            scan_tiles(LoadItemLen{q, a.P, a.V + 1, a.csr_off}, EpiItemRank{a.ipref, a.push_chunk_item}, items, a.desc,
                       &w->ticket[L], &w->err, &w->total[L], kLookbackSpinCap);
            if (!grid_barrier(w)) return;
            PushArgs pa;
            pa.q = q;
            pa.nitems = items;
            pa.total_dev = &w->total[L];
            pa.P = a.P;
            pa.stride = a.V + 1;
            pa.off = a.csr_off;
            pa.adj = a.csr_adj;
            pa.w = nullptr;
            pa.ipref = a.ipref;
            pa.chunk_item = a.push_chunk_item;
            pa.q_out = nullptr;
            pa.n_out = nullptr;
            pa.act_edges = nullptr;
            pa.deg = nullptr;
            push_chunks(MsBfsPushOp{front, a.visit, next, next_bm}, pa);
        }
        if (!grid_barrier(w)) return;
        bm_compact_words(next_bm, a.nwords, q_next, &w->cnt[L], &w->act[L], a.deg);
        if (!grid_barrier(w)) return;
        n = __ldcg(&w->cnt[L]);
        act = __ldcg(&w->act[L]);
        if (dense) ++dense_count;
        if (a.lev) queue_levels_work(q_next, n, next, a.lev, L + 1, nullptr, nullptr, nullptr);
        if (tid == 0) {
            w->levels = L + 1;
            w->pushes += dense ? 0u : 1u;
        }
    }
}

// MS-BFS over root entries already in b.entries (count in b.n_entries device word)
// lev_filled: the level rows start as 0xFF (callers that hand them out as they are); otherwise
// their unreached bytes are left as they are and masked by k_levels_out
static int msbfs_core(eg_graph* g, uint32_t n_entries, int nbits, uint8_t* lev, uint64_t* reach_out, int* sweeps_out,
                      int* pushes_out, bool lev_filled) {
    BatchState& b = bstate(g);
    EngineState& s = g->eng;
    const uint64_t V = g->V;
    const uint64_t nwords = V / 64 + 1;
    const size_t bm_bytes = 8 * nwords;
    unsigned long long* visit = b.a64.as<unsigned long long>();
    unsigned long long* word[2] = {b.b64.as<unsigned long long>(), b.c64.as<unsigned long long>()};
    unsigned long long* bm[2] = {b.bm0.as<unsigned long long>(), b.bm1.as<unsigned long long>()};
    uint32_t* queue[2] = {s.q0.as<uint32_t>(), s.q1.as<uint32_t>()};
    unsigned long long* alive = b.alive.as<unsigned long long>();  // [0..1] per level parity, [2] all roots
    uint32_t* cnt = b.level_cnt.as<uint32_t>();  // [kGraphLevels + 1]
    unsigned long long* d_reach = s.counters.as<unsigned long long>() + 4;
    uint32_t* d_nq = reinterpret_cast<uint32_t*>(s.counters.as<unsigned long long>() + 2);
    unsigned long long* d_act = s.counters.as<unsigned long long>() + 3;
    const unsigned long long full = nbits == 64 ? ~0ull : ((1ull << nbits) - 1ull);
    const uint32_t* deg = g->outdeg.as<uint32_t>();
    const unsigned init_grid = std::max(1u, std::min<unsigned>((n_entries + 255) / 256, 4096u));
    const unsigned grid = (unsigned)g->num_sms * 8u;
    const bool one_graph = g->batch_voff.empty();
    constexpr uint64_t kUnknownQueue = ~0ull;
    // pull gathers through the CSC sources renumbered by out-degree class (hot frontier words share
    // cache lines), with a renumbered copy of each frontier; on one graph with the host-driven loop
    const bool renum = one_graph && !(g->use_cuda_graph & 1) && g->batch_launch != 1 && g->E > 0 && want_relabel(g);
    if (renum) {
        EG_TRY(setup_relabel(g));
        EG_TRY(b.wr0.reserve(8 * V + 8));
        EG_TRY(b.wr1.reserve(8 * V + 8));
    }
    unsigned long long* word_r[2] = {b.wr0.as<unsigned long long>(), b.wr1.as<unsigned long long>()};
    const uint32_t* new_id = s.pr_new_id.as<uint32_t>();
    const uint32_t* gather_adj = renum ? s.pr_adj.as<uint32_t>() : g->csc_adj.as<uint32_t>();

    auto enqueue_init = [&]() -> int {
        EG_CUDA(cudaMemsetAsync(visit, 0, 8 * V, g->stream));
        EG_CUDA(cudaMemsetAsync(word[0], 0, 8 * V, g->stream));
        EG_CUDA(cudaMemsetAsync(bm[0], 0, bm_bytes, g->stream));
        EG_CUDA(cudaMemsetAsync(d_nq, 0, 16, g->stream));
        EG_CUDA(cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * (kGraphLevels + 2), g->stream));
        EG_CUDA(cudaMemcpyAsync(alive + 2, &full, 8, cudaMemcpyHostToDevice, g->stream));
        EG_CUDA(cudaMemcpyAsync(alive, &full, 8, cudaMemcpyHostToDevice, g->stream));
        if (lev && lev_filled) EG_CUDA(cudaMemsetAsync(lev, 0xFF, 64 * V, g->stream));
        k_msbfs_init_entries<<<init_grid, 256, 0, g->stream>>>(b.entries.as<uint2>(), b.n_entries.as<uint32_t>(), visit,
                                                               word[0], bm[0], lev, queue[0], d_nq, d_act, deg);
        EG_CHECK_LAUNCH("k_msbfs_init_entries");
        if (renum) {
            EG_CUDA(cudaMemsetAsync(word_r[0], 0, 8 * V, g->stream));
            k_front_renumber<<<init_grid, 256, 0, g->stream>>>(queue[0], d_nq, word[0], new_id, word_r[0]);
            EG_CHECK_LAUNCH("k_front_renumber");
        }
        return EG_OK;
    };
    // one level L: frontier word[L&1] / bm[L&1] / queue[L&1] -> the same of parity (L+1)&1.  The
    // queue length lands in *count; captured loops (stop_flag set) pull every level and keep the
    // alive mask at "all roots".
    // The first dense level follows the frontier's explosion: most destinations miss most roots and
    // read all their in-edges, which the balanced chunked sweep (k_pull_direct) does best.  Later
    // dense levels find most destinations nearly covered and use the early-exit pair -- on one
    // graph.  In a batch of graphs the running-root mask is shared by all graphs, so a vertex
    // waits for bits its own graph can never deliver, and every level keeps the chunked sweep.
    // clear_n: how many vertices queue[x] lists from two levels back (the non-zero words of
    // word[x]); kUnknownQueue when not known on the host, and the arrays are cleared whole
    auto enqueue_level = [&](uint32_t L, uint64_t n_host, bool dense, bool screen, uint32_t* count, const int* stop_flag,
                             uint32_t* nout_host, unsigned long long* act_host, bool early_exit, uint64_t clear_n) -> int {
        const int c = L & 1, x = c ^ 1;
        if (clear_n <= V / 32) {
            if (clear_n) {
                Timed t(&g->prof, g->stream, "msbfs_vertex");
                k_clear_front<<<grid_for(clear_n, 256, grid), 256, 0, g->stream>>>(
                    queue[x], (uint32_t)clear_n, word[x], renum ? new_id : nullptr, renum ? word_r[x] : nullptr);
                EG_CHECK_LAUNCH("k_clear_front");
            }
        } else {
            EG_CUDA(cudaMemsetAsync(word[x], 0, 8 * V, g->stream));
            if (renum) EG_CUDA(cudaMemsetAsync(word_r[x], 0, 8 * V, g->stream));
        }
        EG_CUDA(cudaMemsetAsync(bm[x], 0, bm_bytes, g->stream));
        // renumbered gathers skip the frontier-bitmap screen (dense levels rarely screen)
        const unsigned long long* gather_word = renum ? word_r[c] : word[c];
        if (renum) screen = false;
        unsigned long long* alive_next = stop_flag ? nullptr : alive + x;
        if (alive_next) EG_CUDA(cudaMemsetAsync(alive_next, 0, 8, g->stream));
        if (dense) {
            EG_CUDA(cudaMemsetAsync(count, 0, 4, g->stream));
            if (!stop_flag) EG_CUDA(cudaMemsetAsync(d_act, 0, 8, g->stream));
            if (early_exit) {
                uint32_t* d_nseg = reinterpret_cast<uint32_t*>(cnt + kGraphLevels + 2);
                EG_CUDA(cudaMemsetAsync(d_nseg, 0, 4, g->stream));
                MsBuArgs ma{gather_adj, g->cidx.as<uint64_t>(), g->cvert.as<uint32_t>(),
                            g->ncompressed - 1, (uint32_t)V, gather_word, visit, word[x], bm[x],
                            stop_flag ? alive + 2 : alive + c, b.ms_seg.as<unsigned long long>(), d_nseg, stop_flag};
                Timed t(&g->prof, g->stream, "msbfs_pull");
                k_ms_head<<<grid_for(ma.nitems, 256, grid), 256, 0, g->stream>>>(ma);
                EG_CHECK_LAUNCH("k_ms_head");
                k_ms_tail<<<grid, 256, 0, g->stream>>>(ma);
                EG_CHECK_LAUNCH("k_ms_tail");
            } else {
                MsBfsPullOp op{gather_word, bm[c], screen ? 1 : 0, visit, word[x], bm[x],
                               stop_flag ? alive + 2 : alive + c, stop_flag};
                EG_TRY(launch_pull_direct(g, op, "msbfs_pull", gather_adj));
            }
            Timed t(&g->prof, g->stream, "msbfs_vertex");
            k_bm_compact<<<grid_for(nwords, 256, grid), 256, 0, g->stream>>>(bm[x], nwords, queue[x], count,
                                                                            stop_flag ? nullptr : d_act, deg);
            EG_CHECK_LAUNCH("k_bm_compact");
        } else {
            MsBfsPushOp op{word[c], visit, word[x], bm[x]};
            EG_TRY(push_level(g, op, queue[c], n_host, queue[x], nout_host, nullptr, act_host, deg, "msbfs_push"));
        }
        if (lev || alive_next || renum) {
            Timed t(&g->prof, g->stream, "msbfs_vertex");
            k_queue_levels<<<grid, 256, 0, g->stream>>>(queue[x], count, word[x], lev, L + 1, alive_next,
                                                        renum ? new_id : nullptr, word_r[x]);
            EG_CHECK_LAUNCH("k_queue_levels");
        }
        return EG_OK;
    };

    int sweeps = 0, pushes = 0;
    uint32_t lvl = 0;
    // the host-driven level loop from level lvl on: the frontier (queue[lvl & 1]) lists n vertices
    // with act out-edges; q0len / q1len are how many vertices queue[0] / queue[1] list
    auto host_levels = [&](uint64_t n, unsigned long long act, uint64_t q0len, uint64_t q1len,
                           int dense_levels) -> int {
        struct {
            uint32_t n;
            uint32_t pad;
            unsigned long long act;
        } h;
        uint64_t qlen[2] = {q0len, q1len};
        while (n > 0) {
            if (lvl >= 254) {
                set_error("eg_msbfs: more than 254 levels");
                return EG_ERR_UNSUPPORTED;
            }
            // the Gemini switch on the union frontier; EG_OPT_BFS_DIRECTION concerns single-root BFS
            const bool dense = !g->built_csr || act >= g->E / (uint64_t)batch_divisor(g);
            uint32_t nout = 0;
            // a bitmap test before each gather pays only while the frontier is a small part of V
            EG_TRY(enqueue_level(lvl, n, dense, n * 16 < V, d_nq, nullptr, &nout, &act, one_graph && dense_levels > 0,
                                 qlen[(lvl & 1) ^ 1]));
            if (dense) {
                ++dense_levels;
                EG_CUDA(cudaMemcpyAsync(&h, d_nq, 16, cudaMemcpyDeviceToHost, g->stream));
                EG_CUDA(cudaStreamSynchronize(g->stream));
                nout = h.n;
                act = h.act;
            } else {
                ++pushes;
            }
            qlen[(lvl & 1) ^ 1] = nout;
            ++sweeps;
            n = nout;
            ++lvl;
        }
        return EG_OK;
    };
    if (g->batch_launch == 1) {
        // the whole traversal in one persistent cooperative launch
        EG_TRY(enqueue_init());
        EG_TRY(b.persist.reserve(sizeof(PersistWords)));
        PersistWords* pw = b.persist.as<PersistWords>();
        EG_CUDA(cudaMemsetAsync(pw, 0, sizeof(PersistWords), g->stream));
        const int P = g->partitions;
        const uint64_t max_tiles = ((V + 1) * (uint64_t)P + kScanTile - 1) / kScanTile + 2;
        EG_TRY(g->scan.desc.reserve(max_tiles * sizeof(uint64_t)));
        const size_t smem = 6 * ((size_t)kPullChunk + P + 3);
        EG_CUDA(cudaFuncSetAttribute(k_msbfs_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int per_sm = 0;
        EG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_msbfs_persistent, 256, smem));
        if (per_sm < 1) {
            set_error("eg_msbfs: the persistent traversal does not fit an SM");
            return EG_ERR_UNSUPPORTED;
        }
        MsPersistArgs pa;
        pa.V = V;
        pa.nwords = nwords;
        pa.P = P;
        pa.csr_off = g->csr_off.as<uint64_t>();
        pa.csr_adj = g->csr_adj.as<uint32_t>();
        pa.gather_adj = gather_adj;
        pa.cidx = g->cidx.as<uint64_t>();
        pa.cvert = g->cvert.as<uint32_t>();
        pa.nitems = g->ncompressed - 1;
        pa.pull_chunk_item = s.pull_chunk_item.as<uint32_t>();
        pa.E = g->E;
        pa.deg = deg;
        pa.visit = visit;
        pa.word0 = word[0];
        pa.word1 = word[1];
        pa.bm0 = bm[0];
        pa.bm1 = bm[1];
        pa.q0 = queue[0];
        pa.q1 = queue[1];
        pa.alive_all = alive + 2;
        pa.lev = lev;
        pa.ms_seg = b.ms_seg.as<unsigned long long>();
        pa.desc = g->scan.desc.as<uint64_t>();
        pa.ipref = s.qdeg.as<uint64_t>();
        pa.push_chunk_item = s.chunk_item.as<uint32_t>();
        pa.init_n = d_nq;
        pa.init_act = d_act;
        pa.dense_min = g->E / (uint64_t)batch_divisor(g);
        pa.early_after_first = one_graph ? 1 : 0;
        pa.built_csr = g->built_csr ? 1 : 0;
        pa.w = pw;
        void* kargs[] = {&pa};
        {
            Timed t(&g->prof, g->stream, "msbfs_persistent");
            EG_CUDA(cudaLaunchCooperativeKernel((const void*)k_msbfs_persistent, dim3((unsigned)g->num_sms * per_sm),
                                                dim3(256), kargs, smem, g->stream));
            EG_CHECK_LAUNCH("k_msbfs_persistent");
        }
        PersistWords hw;
        EG_CUDA(cudaMemcpyAsync(&hw, pw, sizeof(PersistWords), cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        if (hw.err) {
            set_error("eg_msbfs: a bounded wait of the persistent traversal gave up");
            return EG_ERR_TIMEOUT;
        }
        if (hw.levels >= 254 && hw.cnt[253] > 0) {
            set_error("eg_msbfs: more than 254 levels");
            return EG_ERR_UNSUPPORTED;
        }
        sweeps = (int)hw.levels;
        pushes = (int)hw.pushes;
        lvl = hw.levels;
    } else if (g->use_cuda_graph & 1) {
        // init + kGraphLevels levels replayed as one CUDA graph, each level choosing push or pull
        // on the device (k_cap_decide); levels after an empty frontier do nothing
        const bool key_ok = b.graph_exec && b.graph_V == V && b.graph_lev == (lev != nullptr) &&
                            b.graph_entries >= n_entries && b.graph_nbits == nbits &&
                            b.graph_div == batch_divisor(g);
        if (!key_ok) {
            if (b.graph_exec) cudaGraphExecDestroy((cudaGraphExec_t)b.graph_exec);
            b.graph_exec = nullptr;
            EG_TRY(b.cap.reserve(sizeof(CapState)));
            const int P = g->partitions;
            const uint64_t max_items = (V + 1) * (uint64_t)P;
            const uint64_t max_tiles = (max_items + kScanTile - 1) / kScanTile;
            EG_TRY(g->scan.desc.reserve(max_tiles * sizeof(uint64_t)));
            EG_TRY(g->scan.counter.reserve(16));
            const bool prof = g->prof.enabled;
            g->prof.enabled = false;
            EG_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
            CapState* cs = b.cap.as<CapState>();
            int st = enqueue_init();
            auto ok = [&](cudaError_t e) {
                if (st == EG_OK && e != cudaSuccess) st = EG_ERR_CUDA;
            };
            ok(cudaMemsetAsync(cs, 0, sizeof(CapState), g->stream));
            ok(cudaMemsetAsync(word[1], 0, 8 * V, g->stream));
            const unsigned long long dense_min = g->E / (uint64_t)batch_divisor(g);
            for (uint32_t L = 0; st == EG_OK && L < (uint32_t)kGraphLevels; ++L) {
                const int c = L & 1, x = c ^ 1;
                const uint32_t* n_cur = L == 0 ? d_nq : cnt + L - 1;
                const unsigned long long* act_cur = L == 0 ? d_act : cs->act + L - 1;
                k_cap_decide<<<1, 1, 0, g->stream>>>(cs, (int)L, n_cur, act_cur, dense_min, one_graph ? 1 : 0,
                                                     g->built_csr ? 1 : 0);
                ok(cudaGetLastError());
                if (L >= 1) {  // the frontier words written two levels back (level 1: the roots)
                    const uint32_t* n_old = L == 1 ? d_nq : cnt + L - 2;
                    k_clear_front_dev<<<grid, 256, 0, g->stream>>>(queue[x], n_old, word[x], V, cs);
                    ok(cudaGetLastError());
                }
                ok(cudaMemsetAsync(bm[x], 0, bm_bytes, g->stream));
                // pull: the chunked sweep or the early-exit pair, whichever the level armed
                {
                    MsBfsPullOp op{word[c], bm[c], 1, visit, word[x], bm[x], alive + 2, &cs->lv[L].skip_direct};
                    if (st == EG_OK) st = launch_pull_direct(g, op, "msbfs_pull", gather_adj, 16 * grid);
                    uint32_t* d_nseg = reinterpret_cast<uint32_t*>(cnt + kGraphLevels + 2);
                    ok(cudaMemsetAsync(d_nseg, 0, 4, g->stream));
                    MsBuArgs ma{gather_adj, g->cidx.as<uint64_t>(), g->cvert.as<uint32_t>(), g->ncompressed - 1,
                                (uint32_t)V, word[c], visit, word[x], bm[x], alive + 2,
                                b.ms_seg.as<unsigned long long>(), d_nseg, &cs->lv[L].skip_early};
                    k_ms_head<<<grid_for(ma.nitems, 256, grid), 256, 0, g->stream>>>(ma);
                    ok(cudaGetLastError());
                    k_ms_tail<<<grid, 256, 0, g->stream>>>(ma);
                    ok(cudaGetLastError());
                }
                // push: scan of the queued lists' lengths and the rank-balanced expansion, sized on
                // the device (zero items on pull levels)
                if (g->built_csr) {
                    const uint32_t* n_push = &cs->lv[L].n_push;
                    uint64_t* ipref = s.qdeg.as<uint64_t>();
                    ok(cudaMemsetAsync(g->scan.desc.ptr, 0, max_tiles * sizeof(uint64_t), g->stream));
                    ok(cudaMemsetAsync(g->scan.counter.ptr, 0, 4, g->stream));
                    LoadItemLen ld{queue[c], P, V + 1, g->csr_off.as<uint64_t>()};
                    EpiItemRank ep{ipref, s.chunk_item.as<uint32_t>()};
                    k_scan<<<(unsigned)std::min<uint64_t>(max_tiles, grid), kScanThreads, 0, g->stream>>>(
                        ld, ep, max_items, g->scan.desc.as<uint64_t>(), g->scan.counter.as<uint32_t>(),
                        g->err.as<int>(), &cs->push_total, kLookbackSpinCap, n_push, (uint32_t)P);
                    ok(cudaGetLastError());
                    PushArgs a;
                    a.q = queue[c];
                    a.nitems = 0;
                    a.n_dev = n_push;
                    a.total_dev = &cs->push_total;
                    a.P = P;
                    a.stride = V + 1;
                    a.off = g->csr_off.as<uint64_t>();
                    a.adj = g->csr_adj.as<uint32_t>();
                    a.w = nullptr;
                    a.ipref = ipref;
                    a.chunk_item = s.chunk_item.as<uint32_t>();
                    a.q_out = nullptr;
                    a.n_out = nullptr;
                    a.act_edges = nullptr;
                    a.deg = nullptr;
                    MsBfsPushOp pop{word[c], visit, word[x], bm[x]};
                    k_push<MsBfsPushOp><<<kPersistentGrid, kPushThreads, 0, g->stream>>>(pop, a);
                    ok(cudaGetLastError());
                }
                // the next frontier from its bitmap (either path), its out-edges and level bytes
                k_bm_compact<<<grid_for(nwords, 256, grid), 256, 0, g->stream>>>(bm[x], nwords, queue[x], cnt + L,
                                                                                cs->act + L, deg);
                ok(cudaGetLastError());
                if (lev) {
                    k_queue_levels<<<grid, 256, 0, g->stream>>>(queue[x], cnt + L, word[x], lev, L + 1, nullptr,
                                                                nullptr, nullptr);
                    ok(cudaGetLastError());
                }
            }
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamEndCapture(g->stream, &graph);
            g->prof.enabled = prof;
            EG_TRY(st);
            if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
            cudaGraphExec_t exec = nullptr;
            e = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate", __FILE__, __LINE__);
            b.graph_exec = exec;
            b.graph_V = V;
            b.graph_lev = lev != nullptr;
            b.graph_entries = n_entries;
            b.graph_nbits = nbits;
            b.graph_div = batch_divisor(g);
        }
        {
            Timed t(&g->prof, g->stream, "msbfs_graph");
            EG_CUDA(cudaGraphLaunch((cudaGraphExec_t)b.graph_exec, g->stream));
        }
        std::vector<uint32_t> h(kGraphLevels);
        CapState hs;
        EG_CUDA(cudaMemcpyAsync(h.data(), cnt, sizeof(uint32_t) * kGraphLevels, cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaMemcpyAsync(&hs, b.cap.ptr, sizeof(CapState), cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        bool done = false;
        for (int L = 0; L < kGraphLevels && !done; ++L) {
            ++sweeps;
            if (hs.lv[L].n_push) ++pushes;
            done = h[L] == 0;
        }
        if (!done) {
            // deeper than the captured levels: the host-driven loop takes over at level
            // kGraphLevels (queue[0] lists level 31's output, queue[1] level 30's); the captured
            // levels kept no running-root masks, so every root counts as running
            lvl = kGraphLevels;
            EG_CUDA(cudaMemcpyAsync(alive + (lvl & 1), &full, 8, cudaMemcpyHostToDevice, g->stream));
            EG_TRY(host_levels(h[kGraphLevels - 1], hs.act[kGraphLevels - 1], h[kGraphLevels - 1], h[kGraphLevels - 2],
                               hs.dense_count));
        }
    } else {
        EG_TRY(enqueue_init());
        struct {
            uint32_t n;
            uint32_t pad;
            unsigned long long act;
        } h;
        EG_CUDA(cudaMemcpyAsync(&h, d_nq, 16, cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        // queue[1] still holds an earlier call's list: its length is unknown
        EG_TRY(host_levels(h.n, h.act, h.n, kUnknownQueue, 0));
    }
    if (reach_out) {
        EG_CUDA(cudaMemsetAsync(d_reach, 0, 8, g->stream));
        Timed t(&g->prof, g->stream, "msbfs_vertex");
        k_reach_edges<<<grid_for(V, 256, grid), 256, 0, g->stream>>>(visit, deg, V, d_reach);
        EG_CHECK_LAUNCH("k_reach_edges");
        EG_CUDA(cudaMemcpyAsync(reach_out, d_reach, 8, cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
    }
    *sweeps_out = sweeps;
    if (pushes_out) *pushes_out = pushes;
    return EG_OK;
}

static int msbfs_buffers(eg_graph* g, uint32_t n_entries, bool with_levels) {
    BatchState& b = bstate(g);
    const uint64_t V = g->V;
    EG_TRY(ensure_engine(g));
    EG_TRY(setup_pull(g));
    EG_TRY(b.a64.reserve(8 * V + 8));
    EG_TRY(b.b64.reserve(8 * V + 8));
    EG_TRY(b.c64.reserve(8 * V + 8));
    EG_TRY(b.level_cnt.reserve(sizeof(uint32_t) * (kGraphLevels + 4)));
    EG_TRY(b.bm0.reserve(8 * (V / 64 + 1)));
    EG_TRY(b.bm1.reserve(8 * (V / 64 + 1)));
    EG_TRY(b.alive.reserve(64));
    {  // early-exit dense levels: at most one segment per entry longer than kMsHead plus one per kMsSeg
        const uint64_t nitems = g->ncompressed - 1;
        const uint64_t heavy = std::min<uint64_t>(nitems, g->E / (kMsHead + 1));
        EG_TRY(b.ms_seg.reserve(sizeof(unsigned long long) * (heavy + g->E / kMsSeg + 2)));
    }
    EG_TRY(b.entries.reserve(sizeof(uint2) * (n_entries + 1)));
    EG_TRY(b.n_entries.reserve(16));
    if (with_levels) EG_TRY(b.lev.reserve(64 * V + 64));
    EG_CUDA(cudaMemcpyAsync(b.n_entries.ptr, &n_entries, 4, cudaMemcpyHostToDevice, g->stream));
    return EG_OK;
}

int run_msbfs(eg_graph* g, const uint32_t* roots, int n, uint8_t* levels, int where, uint64_t* edges) {
    if (!g->built_csc) { set_error("eg_msbfs: CSC not built"); return EG_ERR_STATE; }
    EG_TRY(check_roots(g, roots, n, where, "eg_msbfs"));
    BatchState& b = bstate(g);
    const uint64_t V = g->V;
    EG_TRY(msbfs_buffers(g, (uint32_t)n, levels != nullptr));
    EG_TRY(copy_small_in(g, b.seeds, roots, n, where));
    k_root_entries<<<1, 64, 0, g->stream>>>(b.seeds.as<uint32_t>(), n, 0, b.entries.as<uint2>());
    EG_CHECK_LAUNCH("k_root_entries");
    uint8_t* lev = levels ? b.lev.as<uint8_t>() : nullptr;
    uint64_t reach = 0;
    int sweeps = 0, pushes = 0;
    EG_TRY(msbfs_core(g, (uint32_t)n, n, lev, &reach, &sweeps, &pushes, false));
    if (levels) {
        uint8_t* out = levels;
        if (where != EG_DEVICE) {
            EG_TRY(b.tmp_out.reserve((size_t)n * V + 64));
            out = b.tmp_out.as<uint8_t>();
        }
        {
            Timed t(&g->prof, g->stream, "msbfs_levels_out");
            const int vec = (V % 16 == 0) && (((uintptr_t)out & 15u) == 0);
            k_levels_out<<<(unsigned)((V + 63) / 64), 256, 0, g->stream>>>(lev, b.a64.as<unsigned long long>(),
                                                                          (uint32_t)V, n, out, vec);
            EG_CHECK_LAUNCH("k_levels_out");
        }
        if (where != EG_DEVICE)
            EG_CUDA(cudaMemcpyAsync(levels, out, (size_t)n * V, cudaMemcpyDeviceToHost, g->stream));
    }
    EG_CUDA(cudaStreamSynchronize(g->stream));
    if (edges) *edges = reach;
    g->last_edges_processed = reach;
    g->last_iterations = sweeps;
    g->last_pushes = pushes;
    g->last_pulls = sweeps - pushes;
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
static int ensure_tasks(eg_graph* g, bool csr) {
    BatchState& b = bstate(g);
    if (csr) {
        if (!b.csr_ready) {
            EG_TRY(make_tasks(g, b.csr_tasks, g->csr_off.as<uint64_t>(), g->V));
            b.csr_ready = true;
        }
    } else if (!b.csc_ready) {
        EG_TRY(make_tasks(g, b.csc_tasks, g->cidx.as<uint64_t>(), g->ncompressed - 1));
        b.csc_ready = true;
    }
    return EG_OK;
}

static unsigned row_grid(eg_graph* g) { return (unsigned)g->num_sms * 8u; }

static RowArgs row_args(const RowTasks& t, const uint32_t* item_vertex, const uint32_t* adj, const float* w) {
    RowArgs a;
    a.t_item = t.item.as<uint32_t>();
    a.t_part = t.part.as<uint32_t>();
    a.ntasks = t.ntasks;
    a.heavy_slot = t.heavy_slot.as<uint32_t>();
    a.item_vertex = item_vertex;
    a.begin = t.begin;
    a.adj = adj;
    a.w = w;
    return a;
}

// weights in CSR and CSC order, row-normalised by the source's out-weight sum
static int prepare_ppr_weights(eg_graph* g, const float* w_in_dev) {
    BatchState& b = bstate(g);
    const uint64_t E = g->E, V = g->V;
    EG_TRY(b.wn_csc.reserve(4 * E + 64));
    EG_TRY(b.wn_csr.reserve(4 * E + 64));
    EG_TRY(b.s_out.reserve(4 * V + 64));
    EG_TRY(b.row_of.reserve(4 * E + 64));
    const unsigned gv = grid_for(V, 256, 152u * 16u), ge = grid_for(E, 256, 152u * 16u);
    Timed t(&g->prof, g->stream, "ppr_weights");
    k_out_weight_sums<<<gv, 256, 0, g->stream>>>(g->csr_off.as<uint64_t>(), g->csr_w.as<float>(), w_in_dev, (uint32_t)V,
                                                 b.s_out.as<float>());
    EG_CHECK_LAUNCH("k_out_weight_sums");
    // CSC: the neighbour is the source
    k_gather_norm_w<<<ge, 256, 0, g->stream>>>(g->csc_adj.as<uint32_t>(), g->csc_w.as<float>(), w_in_dev,
                                               b.s_out.as<float>(), E, b.wn_csc.as<float>());
    EG_CHECK_LAUNCH("k_gather_norm_w");
    // CSR: the source is the row
    k_row_of<<<gv, 256, 0, g->stream>>>(g->csr_off.as<uint64_t>(), (uint32_t)V, b.row_of.as<uint32_t>());
    EG_CHECK_LAUNCH("k_row_of");
    k_gather_norm_w<<<ge, 256, 0, g->stream>>>(b.row_of.as<uint32_t>(), g->csr_w.as<float>(), w_in_dev,
                                               b.s_out.as<float>(), E, b.wn_csr.as<float>());
    EG_CHECK_LAUNCH("k_gather_norm_w");
    return EG_OK;
}

// one forward step: y = a*e + (1-a) A^T x
static int ppr_step(eg_graph* g, const float* x, float* y, float alpha, int n) {
    BatchState& b = bstate(g);
    const uint64_t V = g->V;
    const RowTasks& t = b.csc_tasks;
    EG_CUDA(cudaMemsetAsync(y, 0, 256 * V, g->stream));
    RowArgs a = row_args(t, g->cvert.as<uint32_t>(), g->csc_adj.as<uint32_t>(), b.wn_csc.as<float>());
    Timed tm(&g->prof, g->stream, "ppr_spmm");
    k_row_spmm<<<row_grid(g), 256, 0, g->stream>>>(a, reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(y),
                                                  b.heavy.as<float2>(), 1.0f - alpha);
    EG_CHECK_LAUNCH("k_row_spmm");
    if (t.nheavy) {
        k_row_heavy_finish<<<(unsigned)((t.nheavy * 32ull + 255) / 256), 256, 0, g->stream>>>(
            t.heavy_item.as<uint32_t>(), g->cvert.as<uint32_t>(), t.nheavy, b.heavy.as<float2>(),
            reinterpret_cast<float2*>(y), 1.0f - alpha);
        EG_CHECK_LAUNCH("k_row_heavy_finish");
    }
    k_ppr_teleport<<<1, 64, 0, g->stream>>>(b.seeds.as<uint32_t>(), n, y, alpha);
    EG_CHECK_LAUNCH("k_ppr_teleport");
    return EG_OK;
}

static int ppr_common(eg_graph* g, const float* w_in, const uint32_t* seeds, int n, float alpha, int K, int where,
                      const float** w_dev) {
    if (!g->built_csc || !g->built_csr) { set_error("eg_ppr: graph not built"); return EG_ERR_STATE; }
    if (!g->weighted || !g->edge_ids) {
        set_error("eg_ppr: load the graph with eg_load_directed_with_ids (per-edge ids select the weights)");
        return EG_ERR_STATE;
    }
    if (!w_in || K < 0 || !(alpha > 0.f && alpha <= 1.f)) { set_error("eg_ppr: need weights, K >= 0, 0 < alpha <= 1"); return EG_ERR_INVALID; }
    EG_TRY(check_roots(g, seeds, n, where, "eg_ppr"));
    BatchState& b = bstate(g);
    const uint64_t V = g->V, E = g->E_input;
    EG_TRY(copy_small_in(g, b.seeds, seeds, n, where));
    const float* wd = w_in;
    if (where != EG_DEVICE) {
        EG_TRY(b.tmp_out.reserve(4 * E + 64));
        EG_CUDA(cudaMemcpyAsync(b.tmp_out.ptr, w_in, 4 * E, cudaMemcpyHostToDevice, g->stream));
        wd = b.tmp_out.as<float>();
    }
    *w_dev = wd;
    EG_TRY(ensure_tasks(g, false));
    EG_TRY(ensure_tasks(g, true));
    EG_TRY(b.heavy.reserve(256ull * (std::max(b.csc_tasks.nheavy, b.csr_tasks.nheavy) + 1)));
    EG_CUDA(cudaMemsetAsync(b.heavy.ptr, 0, b.heavy.bytes, g->stream));
    EG_TRY(b.rows0.reserve(256 * V + 256));
    EG_TRY(b.rows1.reserve(256 * V + 256));
    return prepare_ppr_weights(g, wd);
}

// one seed: the scalar chunked pull (4-byte gathers of x[src] times the normalised weight)
struct PprPullOp {
    using Acc = float;
    static constexpr bool kFilter = false;
    __device__ bool stopped() const { return false; }
    __device__ bool item_active(uint32_t) const { return true; }
    const float* x;
    const float* wn;
    float* y;
    float* acc;
    float scale;
    __device__ Acc identity() const { return 0.f; }
    __device__ Acc gather(uint32_t u, uint64_t e) const { return ld_keep(x + u) * __ldg(wn + e); }
    __device__ Acc combine(Acc a, Acc b) const { return a + b; }
    __device__ void smem_add(Acc* slot, Acc v) const { atomicAdd(slot, v); }
    __device__ void finish(bool ok, uint32_t v, Acc a, bool whole) const {
        if (!ok) return;
        if (whole) y[v] = scale * a;
        else atomicAdd(acc + v, a);
    }
};

__global__ void k_ppr_split(const uint32_t* __restrict__ split, const uint32_t* __restrict__ cvert, uint64_t nsplit,
                            float* y, float* acc, float scale) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nsplit; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = cvert[split[i]];
        y[v] = scale * acc[v];
        acc[v] = 0.f;
    }
}

__global__ void k_ppr_seed1(uint32_t seed, float* y, float value, int add) {
    if (add) y[seed] += value;
    else y[seed] = value;
}

static int run_ppr_single(eg_graph* g, uint32_t seed, float alpha, int K, float* out, int where) {
    BatchState& b = bstate(g);
    EngineState& s = g->eng;
    const uint64_t V = g->V;
    EG_TRY(ensure_engine(g));
    EG_TRY(setup_pull(g));
    float* x = s.vals0.as<float>();
    float* y = s.vals1.as<float>();
    EG_CUDA(cudaMemsetAsync(x, 0, 4 * V, g->stream));
    EG_CUDA(cudaMemsetAsync(s.acc.ptr, 0, 4 * V, g->stream));
    k_ppr_seed1<<<1, 1, 0, g->stream>>>(seed, x, 1.0f, 0);
    EG_CHECK_LAUNCH("k_ppr_seed1");
    for (int k = 0; k < K; ++k) {
        EG_CUDA(cudaMemsetAsync(y, 0, 4 * V, g->stream));
        // single = true: whole items write y directly, split items go through acc
        PprPullOp op{x, b.wn_csc.as<float>(), y, s.acc.as<float>(), 1.0f - alpha};
        EG_TRY(launch_pull(g, op, "ppr1_pull"));
        if (s.pull_nsplit) {
            k_ppr_split<<<grid_for(s.pull_nsplit, 256), 256, 0, g->stream>>>(s.pull_split.as<uint32_t>(), g->cvert.as<uint32_t>(),
                                                                             s.pull_nsplit, y, s.acc.as<float>(), 1.0f - alpha);
            EG_CHECK_LAUNCH("k_ppr_split");
        }
        k_ppr_seed1<<<1, 1, 0, g->stream>>>(seed, y, alpha, 1);
        EG_CHECK_LAUNCH("k_ppr_seed1");
        std::swap(x, y);
    }
    if (out)
        EG_CUDA(cudaMemcpyAsync(out, x, 4 * V, where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->last_edges_processed = g->E * (uint64_t)K;
    g->last_iterations = K;
    return EG_OK;
}

int run_ppr(eg_graph* g, const float* w_in, const uint32_t* seeds, int n, float alpha, int K, float* out, int where) {
    const float* wd = nullptr;
    EG_TRY(ppr_common(g, w_in, seeds, n, alpha, K, where, &wd));
    BatchState& b = bstate(g);
    const uint64_t V = g->V;
    if (n == 1 && g->partitions == 1) {
        uint32_t seed = 0;
        EG_CUDA(cudaMemcpyAsync(&seed, b.seeds.ptr, 4, cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        return run_ppr_single(g, seed, alpha, K, out, where);
    }
    float* x = b.rows0.as<float>();
    float* y = b.rows1.as<float>();
    EG_CUDA(cudaMemsetAsync(x, 0, 256 * V, g->stream));
    k_ppr_init<<<1, 64, 0, g->stream>>>(b.seeds.as<uint32_t>(), n, x);
    EG_CHECK_LAUNCH("k_ppr_init");
    for (int k = 0; k < K; ++k) {
        EG_TRY(ppr_step(g, x, y, alpha, n));
        std::swap(x, y);
    }
    if (out) {
        float* dst = out;
        if (where != EG_DEVICE) {
            EG_TRY(b.tmp_out.reserve(4ull * n * V + 64));
            dst = b.tmp_out.as<float>();
        }
        dim3 blk(32, 8);
        k_transpose_rows<float><<<(unsigned)((V + 31) / 32), blk, 0, g->stream>>>(x, (uint32_t)V, n, dst);
        EG_CHECK_LAUNCH("k_transpose_rows");
        if (where != EG_DEVICE) EG_CUDA(cudaMemcpyAsync(out, dst, 4ull * n * V, cudaMemcpyDeviceToHost, g->stream));
    }
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->last_edges_processed = g->E * (uint64_t)K;
    g->last_iterations = K;
    return EG_OK;
}

// adjoint of K forward steps from x_0 = e_seed; dL/dx_K given as [n][V]; dL/dw in input edge order
int run_ppr_backward(eg_graph* g, const float* w_in, const uint32_t* seeds, int n, float alpha, int K,
                     const float* dl_dx, float* dl_dw, int where) {
    const float* wd = nullptr;
    EG_TRY(ppr_common(g, w_in, seeds, n, alpha, K, where, &wd));
    if (!dl_dx || !dl_dw) { set_error("eg_ppr_backward: need dL/dx and the dL/dw output"); return EG_ERR_INVALID; }
    BatchState& b = bstate(g);
    const uint64_t V = g->V, E = g->E, Ein = g->E_input;
    const int C = std::max(1, (int)ceil(sqrt((double)std::max(K, 1))));  // checkpoint stride
    const int ncp = K / C + 1;
    const size_t row = 256 * V;
    EG_TRY(b.ck.reserve(row * ncp + 256));
    EG_TRY(b.seg.reserve(row * (C + 1) + 256));
    EG_TRY(b.gA.reserve(4 * E + 64));
    // forward with checkpoints x_0, x_C, x_2C, ...
    float* ck = b.ck.as<float>();
    EG_CUDA(cudaMemsetAsync(ck, 0, row, g->stream));
    k_ppr_init<<<1, 64, 0, g->stream>>>(b.seeds.as<uint32_t>(), n, ck);
    EG_CHECK_LAUNCH("k_ppr_init");
    {
        float* x = b.rows0.as<float>();
        float* y = b.rows1.as<float>();
        EG_CUDA(cudaMemcpyAsync(x, ck, row, cudaMemcpyDeviceToDevice, g->stream));
        for (int k = 0; k < K; ++k) {
            EG_TRY(ppr_step(g, x, y, alpha, n));
            std::swap(x, y);
            if ((k + 1) % C == 0 && (k + 1) / C < ncp)
                EG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(ck) + row * ((k + 1) / C), x, row, cudaMemcpyDeviceToDevice,
                                        g->stream));
        }
    }
    // lambda_K from dL/dx_K ([n][V] -> [V][64])
    float* lam = b.rows0.as<float>();
    float* lam2 = b.rows1.as<float>();
    {
        const float* src = dl_dx;
        if (where != EG_DEVICE) {
            EG_TRY(b.tmp_out.reserve(4ull * n * V + 64));
            EG_CUDA(cudaMemcpyAsync(b.tmp_out.ptr, dl_dx, 4ull * n * V, cudaMemcpyHostToDevice, g->stream));
            src = b.tmp_out.as<float>();
        }
        dim3 blk(32, 8);
        k_untranspose_rows<float><<<(unsigned)((V + 31) / 32), blk, 0, g->stream>>>(src, (uint32_t)V, n, lam);
        EG_CHECK_LAUNCH("k_untranspose_rows");
    }
    EG_CUDA(cudaMemsetAsync(b.gA.ptr, 0, 4 * E, g->stream));
    const RowTasks& tr = b.csr_tasks;
    RowArgs ar = row_args(tr, nullptr, g->csr_adj.as<uint32_t>(), b.wn_csr.as<float>());
    float* seg = b.seg.as<float>();
    for (int cp = (K - 1) / C; cp >= 0 && K > 0; --cp) {
        const int k0 = cp * C, k1 = std::min(K, k0 + C);
        // recompute x_k0 .. x_{k1-1} into the segment buffer
        EG_CUDA(cudaMemcpyAsync(seg, reinterpret_cast<char*>(ck) + row * cp, row, cudaMemcpyDeviceToDevice, g->stream));
        for (int k = k0 + 1; k < k1; ++k)
            EG_TRY(ppr_step(g, seg + (size_t)(k - 1 - k0) * 64 * V, seg + (size_t)(k - k0) * 64 * V, alpha, n));
        for (int k = k1 - 1; k >= k0; --k) {
            // lam holds lambda_{k+1}; gA += (1-a) <x_k[u], lam[v]>; lam2 = (1-a) A lam
            EG_CUDA(cudaMemsetAsync(lam2, 0, row, g->stream));
            {
                Timed tm(&g->prof, g->stream, "ppr_adjoint");
                k_row_adjoint<<<row_grid(g), 256, 0, g->stream>>>(
                    ar, reinterpret_cast<const float2*>(lam), reinterpret_cast<const float2*>(seg + (size_t)(k - k0) * 64 * V),
                    reinterpret_cast<float2*>(lam2), b.heavy.as<float2>(), b.gA.as<float>(), 1.0f - alpha);
                EG_CHECK_LAUNCH("k_row_adjoint");
            }
            if (tr.nheavy) {
                k_row_heavy_finish<<<(unsigned)((tr.nheavy * 32ull + 255) / 256), 256, 0, g->stream>>>(
                    tr.heavy_item.as<uint32_t>(), nullptr, tr.nheavy, b.heavy.as<float2>(), reinterpret_cast<float2*>(lam2),
                    1.0f - alpha);
                EG_CHECK_LAUNCH("k_row_heavy_finish");
            }
            std::swap(lam, lam2);
        }
    }
    // dL/dw
    float* dw = dl_dw;
    if (where != EG_DEVICE) {
        EG_TRY(b.tmp_out.reserve(4 * Ein + 64));
        dw = b.tmp_out.as<float>();
    }
    EG_CUDA(cudaMemsetAsync(dw, 0, 4 * Ein, g->stream));
    k_weight_grad<<<grid_for(V, 256, 152u * 16u), 256, 0, g->stream>>>(g->csr_off.as<uint64_t>(), (uint32_t)V,
                                                                       b.wn_csr.as<float>(), b.gA.as<float>(),
                                                                       b.s_out.as<float>(), g->csr_w.as<float>(), dw);
    EG_CHECK_LAUNCH("k_weight_grad");
    if (where != EG_DEVICE) EG_CUDA(cudaMemcpyAsync(dl_dw, dw, 4 * Ein, cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
__global__ void k_sssp_init_entries(const uint2* ent, uint32_t n, float* dist, uint8_t* changed) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dist[(uint64_t)ent[i].x * 64 + ent[i].y] = 0.f;
        changed[ent[i].x] = 1;
    }
}

// Bellman-Ford sweeps from the root entries in b.entries; leaves dist [V][64] in b.rows0
static int sssp_core(eg_graph* g, uint32_t n_entries, int* sweeps_out) {
    EG_TRY(ensure_tasks(g, false));
    BatchState& b = bstate(g);
    const uint64_t V = g->V;
    EG_TRY(b.rows0.reserve(256 * V + 256));
    EG_TRY(b.ch0.reserve(V + 64));
    EG_TRY(b.ch1.reserve(V + 64));
    EG_TRY(b.flag.reserve(16));
    float* dist = b.rows0.as<float>();
    {
        Timed t(&g->prof, g->stream, "sssp_batch_init");
        k_fill_f32_rows<<<grid_for(64 * V, 256, 152u * 16u), 256, 0, g->stream>>>(dist, 64 * V, 1e9f);
        EG_CHECK_LAUNCH("k_fill_f32_rows");
        EG_CUDA(cudaMemsetAsync(b.ch0.ptr, 0, V, g->stream));
        k_sssp_init_entries<<<std::max(1u, std::min<unsigned>((n_entries + 255) / 256, 4096u)), 256, 0, g->stream>>>(
            b.entries.as<uint2>(), n_entries, dist, b.ch0.as<uint8_t>());
        EG_CHECK_LAUNCH("k_sssp_init_entries");
    }
    RowArgs a = row_args(b.csc_tasks, g->cvert.as<uint32_t>(), g->csc_adj.as<uint32_t>(), g->csc_w.as<float>());
    uint8_t* prev = b.ch0.as<uint8_t>();
    uint8_t* nxt = b.ch1.as<uint8_t>();
    int sweeps = 0;
    while (true) {
        EG_CUDA(cudaMemsetAsync(nxt, 0, V, g->stream));
        EG_CUDA(cudaMemsetAsync(b.flag.ptr, 0, 4, g->stream));
        {
            Timed t(&g->prof, g->stream, "sssp_batch_sweep");
            k_row_sssp<<<row_grid(g), 256, 0, g->stream>>>(a, reinterpret_cast<float2*>(dist), prev, nxt, b.flag.as<int>());
            EG_CHECK_LAUNCH("k_row_sssp");
        }
        ++sweeps;
        int any = 0;
        EG_CUDA(cudaMemcpyAsync(&any, b.flag.ptr, 4, cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        if (!any) break;
        std::swap(prev, nxt);
    }
    *sweeps_out = sweeps;
    return EG_OK;
}

static int sssp_ready(eg_graph* g, const char* fn) {
    if (!g->built_csc) { set_error("%s: CSC not built", fn); return EG_ERR_STATE; }
    if (!g->weighted || g->edge_ids) { set_error("%s: graph needs float edge weights", fn); return EG_ERR_STATE; }
    return EG_OK;
}

int run_sssp_batch(eg_graph* g, const uint32_t* srcs, int n, float* out, int where) {
    EG_TRY(sssp_ready(g, "eg_sssp_batch"));
    EG_TRY(check_roots(g, srcs, n, where, "eg_sssp_batch"));
    BatchState& b = bstate(g);
    const uint64_t V = g->V;
    EG_TRY(copy_small_in(g, b.seeds, srcs, n, where));
    EG_TRY(b.entries.reserve(sizeof(uint2) * 64));
    k_root_entries<<<1, 64, 0, g->stream>>>(b.seeds.as<uint32_t>(), n, 0, b.entries.as<uint2>());
    EG_CHECK_LAUNCH("k_root_entries");
    int sweeps = 0;
    EG_TRY(sssp_core(g, (uint32_t)n, &sweeps));
    if (out) {
        float* dst = out;
        if (where != EG_DEVICE) {
            EG_TRY(b.tmp_out.reserve(4ull * n * V + 64));
            dst = b.tmp_out.as<float>();
        }
        dim3 blk(32, 8);
        k_transpose_rows<float><<<(unsigned)((V + 31) / 32), blk, 0, g->stream>>>(b.rows0.as<float>(), (uint32_t)V, n, dst);
        EG_CHECK_LAUNCH("k_transpose_rows");
        if (where != EG_DEVICE) EG_CUDA(cudaMemcpyAsync(out, dst, 4ull * n * V, cudaMemcpyDeviceToHost, g->stream));
    }
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->last_iterations = sweeps;
    g->last_pulls = sweeps;
    g->last_pushes = 0;
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
// many small graphs: roots are local ids, nper per graph; outputs stay vertex-major [V_total][64]
static int graph_roots(eg_graph* g, const uint32_t* roots, int nper, int where, const char* fn, uint32_t* n_entries) {
    const uint64_t G = g->batch_voff.size() ? g->batch_voff.size() - 1 : 0;
    if (!G) { set_error("%s: no graph batch loaded (eg_load_graph_batch)", fn); return EG_ERR_STATE; }
    if (!roots || nper < 1 || nper > 64) { set_error("%s: need 1..64 roots per graph", fn); return EG_ERR_INVALID; }
    const uint64_t n = G * (uint64_t)nper;
    std::vector<uint32_t> h(n);
    EG_CUDA(cudaMemcpy(h.data(), roots, 4 * n, where == EG_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost));
    for (uint64_t i = 0; i < n; ++i) {
        const uint64_t gi = i / nper;
        if (h[i] >= g->batch_voff[gi + 1] - g->batch_voff[gi]) {
            set_error("%s: root %u of graph %llu out of range", fn, h[i], (unsigned long long)gi);
            return EG_ERR_INVALID;
        }
    }
    BatchState& b = bstate(g);
    EG_TRY(b.entries.reserve(sizeof(uint2) * (n + 1)));
    EG_TRY(b.tmp_out.reserve(4 * n + 64));
    EG_CUDA(cudaMemcpyAsync(b.tmp_out.ptr, h.data(), 4 * n, cudaMemcpyHostToDevice, g->stream));
    k_root_entries_graphs<<<(unsigned)((n + 255) / 256), 256, 0, g->stream>>>(
        b.tmp_out.as<uint32_t>(), g->d_batch_voff.as<uint64_t>(), (uint32_t)G, nper, b.entries.as<uint2>());
    EG_CHECK_LAUNCH("k_root_entries_graphs");
    EG_CUDA(cudaStreamSynchronize(g->stream));
    *n_entries = (uint32_t)n;
    return EG_OK;
}

int run_msbfs_graphs(eg_graph* g, const uint32_t* roots, int nper, uint8_t* levels, int where, uint64_t* edges) {
    if (!g->built_csc) { set_error("eg_msbfs_graphs: CSC not built"); return EG_ERR_STATE; }
    uint32_t n = 0;
    const uint64_t G = g->batch_voff.size() ? g->batch_voff.size() - 1 : 0;
    EG_TRY(msbfs_buffers(g, (uint32_t)(G * (uint64_t)std::max(nper, 1)), levels != nullptr));
    EG_TRY(graph_roots(g, roots, nper, where, "eg_msbfs_graphs", &n));
    BatchState& b = bstate(g);
    EG_CUDA(cudaMemcpyAsync(b.n_entries.ptr, &n, 4, cudaMemcpyHostToDevice, g->stream));
    uint64_t reach = 0;
    int sweeps = 0, pushes = 0;
    EG_TRY(msbfs_core(g, n, nper, levels ? b.lev.as<uint8_t>() : nullptr, &reach, &sweeps, &pushes, true));
    if (levels)
        EG_CUDA(cudaMemcpyAsync(levels, b.lev.ptr, 64ull * g->V,
                                where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    if (edges) *edges = reach;
    g->last_edges_processed = reach;
    g->last_iterations = sweeps;
    g->last_pulls = sweeps - pushes;
    g->last_pushes = pushes;
    return EG_OK;
}

int run_sssp_graphs(eg_graph* g, const uint32_t* sources, int nper, float* dist, int where) {
    EG_TRY(sssp_ready(g, "eg_sssp_graphs"));
    uint32_t n = 0;
    EG_TRY(graph_roots(g, sources, nper, where, "eg_sssp_graphs", &n));
    int sweeps = 0;
    EG_TRY(sssp_core(g, n, &sweeps));
    if (dist)
        EG_CUDA(cudaMemcpyAsync(dist, bstate(g).rows0.ptr, 256ull * g->V,
                                where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->last_iterations = sweeps;
    g->last_pulls = sweeps;
    g->last_pushes = 0;
    return EG_OK;
}

// graph i's edges occupy [eoff[i], eoff[i+1]); its vertex v becomes voff[i] + v
__global__ void k_relabel_batch(uint8_t* edges, int rec, uint64_t E, const uint64_t* __restrict__ eoff,
                                const uint64_t* __restrict__ voff, uint32_t G, int* bad) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = G;  // last graph with eoff <= i
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(eoff + mid) <= i) lo = mid; else hi = mid;
        }
        uint32_t* r = reinterpret_cast<uint32_t*>(edges + i * (uint64_t)rec);
        const uint64_t base = voff[lo], nv = voff[lo + 1] - base;
        if (r[0] >= nv || r[1] >= nv) {
            atomicExch(bad, 1);
            continue;
        }
        r[0] = (uint32_t)(base + r[0]);
        r[1] = (uint32_t)(base + r[1]);
    }
}

int load_graph_batch(eg_graph* g, const void* edges, int rec, const uint64_t* eoff, const uint32_t* nverts, int G,
                     int where) {
    if ((rec != 8 && rec != 12) || G < 1 || !eoff || !nverts || eoff[0] != 0 || (where != EG_HOST && where != EG_DEVICE)) {
        set_error("eg_load_graph_batch: need 8/12-byte records, G >= 1, edge offsets starting at 0, vertex counts");
        return EG_ERR_INVALID;
    }
    std::vector<uint64_t> voff(G + 1, 0), eo(eoff, eoff + G + 1);
    for (int i = 0; i < G; ++i) {
        if (nverts[i] == 0 || eo[i + 1] < eo[i]) {
            set_error("eg_load_graph_batch: graph %d has no vertices or negative edge count", i);
            return EG_ERR_INVALID;
        }
        voff[i + 1] = voff[i] + nverts[i];
    }
    if (voff[G] >= (1ull << 32)) {
        set_error("eg_load_graph_batch: more than 2^32 vertices in total");
        return EG_ERR_INVALID;
    }
    const uint64_t E = eo[G];
    EG_TRY(load_edges_impl(g, edges, E, (uint32_t)voff[G], rec, 0, where, false));
    EG_TRY(g->d_batch_voff.reserve(8 * (G + 1)));
    EG_TRY(g->tmp64.reserve(8 * (G + 1)));
    EG_CUDA(cudaMemcpyAsync(g->d_batch_voff.ptr, voff.data(), 8 * (G + 1), cudaMemcpyHostToDevice, g->stream));
    EG_CUDA(cudaMemcpyAsync(g->tmp64.ptr, eo.data(), 8 * (G + 1), cudaMemcpyHostToDevice, g->stream));
    if (g->build_launch && persistent_build_fits(g)) {  // ids moved to the union inside the one launch
        EG_TRY(build_persistent(g, g->tmp64.as<uint64_t>(), g->d_batch_voff.as<uint64_t>(), (uint32_t)G));
        g->batch_voff = voff;
        g->batch_eoff = eo;
        return EG_OK;
    }
    EG_CUDA(cudaMemsetAsync(g->err.as<int>() + 1, 0, sizeof(int), g->stream));
    if (E) {
        Timed t(&g->prof, g->stream, "relabel_batch");
        k_relabel_batch<<<grid_for(E, 256, 152u * 16u), 256, 0, g->stream>>>(
            g->edges.as<uint8_t>(), rec, E, g->tmp64.as<uint64_t>(), g->d_batch_voff.as<uint64_t>(), (uint32_t)G,
            g->err.as<int>() + 1);
        EG_CHECK_LAUNCH("k_relabel_batch");
    }
    int bad = 0;
    EG_CUDA(cudaMemcpyAsync(&bad, g->err.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    if (bad) {
        set_error("eg_load_graph_batch: a record holds a vertex id >= its graph's vertex count");
        return EG_ERR_INVALID;
    }
    g->batch_voff = voff;
    g->batch_eoff = eo;
    return build_structures(g, 1, 1);
}

}  // namespace eg
