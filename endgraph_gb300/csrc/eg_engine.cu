// eg_engine.cu — process_edges on the GPU (core/graph.hpp:1376-1817) for the four toolkits.
//
// Push (sparse, :1505-1655): the frontier is a queue of vertices; a look-back scan over the
// frontier's list lengths gives every frontier edge a global rank, and the expansion kernel hands
// each CTA a fixed run of 2048 ranks (8 contiguous edges per thread), so hubs and leaves cost the
// same per edge.  Activations are de-duplicated in a bitmap and appended with warp-aggregated
// atomics.
// Pull (dense, :1656-1802): the CSC is swept in fixed 4096-edge chunks (16 contiguous ids per
// thread, 128-bit loads); a chunk's compressed entries are staged in shared memory and each thread
// reduces its edges per destination into shared accumulators.  Destinations wholly inside a chunk
// are finalised in place; the few whose list crosses a chunk boundary are combined afterwards.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "eg_pull.cuh"

namespace eg {

// ---------------------------------------------------------------------------------------------
// toolkit operators
struct BfsOp {  // toolkits/bfs.cpp:52-58: first visitor of dst becomes its parent
    unsigned long long* visited;
    unsigned long long* next_front;
    uint32_t* level;
    uint32_t* parent;
    uint32_t next_level;
    const uint32_t* next_level_dev = nullptr;  // a replayed graph reads the level number here
    __device__ uint32_t payload(uint32_t) const { return 0; }
    __device__ bool relax(uint32_t u, uint32_t, uint32_t w, uint64_t) const {
        const unsigned long long bit = 1ull << (w & 63);
        unsigned long long* word = visited + (w >> 6);
        if (__ldcg(word) & bit) return false;
        if (atomicOr(word, bit) & bit) return false;
        if (level) level[w] = next_level_dev ? __ldcg(next_level_dev) : next_level;
        if (parent) parent[w] = u;
        atomicOr(next_front + (w >> 6), bit);
        return true;
    }
};

// dense BFS step (toolkits/bfs.cpp:60-76): every unvisited destination looks for an in-neighbour
// in the current frontier and stops at the first one, which becomes its parent.  Stage one gives
// each compressed CSC entry a thread that reads at most kBuHead in-edges; an entry with a longer
// list that found nothing there is cut into kBuSeg-edge segments, and in stage two a warp reads a
// segment 128 ids per step and leaves as soon as any segment of that destination has claimed it.
constexpr uint32_t kBuHead = 8;
constexpr uint32_t kBuSeg = 1024;

struct BuArgs {
    const uint32_t* adj;
    const uint64_t* cidx;
    const uint32_t* cvert;
    uint64_t nitems;
    uint32_t V;
    const unsigned long long* front;
    unsigned long long* visited;
    unsigned long long* next_front;
    uint32_t* level;
    uint32_t* parent;
    uint32_t next_level;
    uint32_t* q_out;
    uint32_t* n_out;
    unsigned long long* act_edges;
    const uint32_t* deg;
    unsigned long long* seg;  // (segment << 32) | compressed entry
    uint32_t* nseg;
    const uint32_t* next_level_dev = nullptr;  // a replayed graph reads the level number here
};

__device__ __forceinline__ bool bu_in_front(const BuArgs& a, uint32_t u) {
    return (__ldg(a.front + (u >> 6)) >> (u & 63)) & 1ull;
}
__device__ __forceinline__ bool bu_claim(const BuArgs& a, uint32_t v, uint32_t par) {
    const unsigned long long bit = 1ull << (v & 63);
    if (atomicOr(a.visited + (v >> 6), bit) & bit) return false;  // another entry of v won
    if (a.level) a.level[v] = a.next_level_dev ? __ldcg(a.next_level_dev) : a.next_level;
    if (a.parent) a.parent[v] = par;
    atomicOr(a.next_front + (v >> 6), bit);
    return true;
}

__global__ void __launch_bounds__(256) k_bu_head(BuArgs a) {
    __shared__ uint32_t s_cnt[2 * (256 / 32 + 1)];
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    unsigned long long my_act = 0;  // out-edges of the vertices this thread activated
    int parity = 0;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x; base < a.nitems; base += stride, parity ^= 1) {
        const uint64_t i = base + threadIdx.x;
        bool act = false;
        uint32_t v = a.V, nsg = 0;
        if (i < a.nitems) {
            v = a.cvert[i];
            if (v < a.V && !((__ldcg(a.visited + (v >> 6)) >> (v & 63)) & 1ull)) {
                const uint64_t s = a.cidx[i], e = a.cidx[i + 1];
                const uint64_t h = e - s > kBuHead ? s + kBuHead : e;
                uint32_t par = 0xFFFFFFFFu;
                // four independent id loads, then four independent frontier probes per round
                for (uint64_t p = s; p < h && par == 0xFFFFFFFFu; p += 4) {
                    uint32_t u[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) u[q] = p + q < h ? __ldg(a.adj + p + q) : 0xFFFFFFFFu;
                    bool hit[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) hit[q] = u[q] != 0xFFFFFFFFu && bu_in_front(a, u[q]);
#pragma unroll
                    for (int q = 3; q >= 0; --q)
                        if (hit[q]) par = u[q];
                }
                if (par != 0xFFFFFFFFu) act = bu_claim(a, v, par);
                else if (e > h) nsg = (uint32_t)((e - h + kBuSeg - 1) / kBuSeg);
            }
        }
        append_block(act, v, a.q_out, a.n_out, s_cnt, parity);
        if (act) my_act += a.deg[v];
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
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_act += __shfl_xor_sync(0xffffffffu, my_act, o);
    if (lane == 0 && my_act) atomicAdd(a.act_edges, my_act);
}

__global__ void __launch_bounds__(256) k_bu_tail(BuArgs a) {
    const uint32_t n = __ldcg(a.nseg);
    const int lane = threadIdx.x & 31;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t t = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < n; t += nwarps) {
        const unsigned long long ent = a.seg[t];
        const uint32_t i = (uint32_t)ent;
        const uint32_t v = a.cvert[i];
        const uint64_t e = a.cidx[i + 1];
        uint64_t p = a.cidx[i] + kBuHead + (ent >> 32) * kBuSeg;
        const uint64_t pe = p + kBuSeg < e ? p + kBuSeg : e;
        const unsigned long long bit = 1ull << (v & 63);
        bool act = false;
        for (; p < pe; p += 128) {
            if (__any_sync(0xffffffffu, (__ldcg(a.visited + (v >> 6)) & bit) != 0)) break;
            uint32_t u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const uint64_t x = p + 32 * q + lane;
                u[q] = x < pe ? __ldg(a.adj + x) : 0xFFFFFFFFu;
            }
            uint32_t cand = 0xFFFFFFFFu;
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (cand == 0xFFFFFFFFu && u[q] != 0xFFFFFFFFu && bu_in_front(a, u[q])) cand = u[q];
            const unsigned m = __ballot_sync(0xffffffffu, cand != 0xFFFFFFFFu);
            if (m) {
                const uint32_t par = __shfl_sync(0xffffffffu, cand, __ffs(m) - 1);
                if (lane == 0) act = bu_claim(a, v, par);
                break;
            }
        }
        append_active(act, v, a.q_out, a.n_out, a.act_edges, a.deg);
    }
}

// toolkits/sssp.cpp:52-64: relax_dist = dist[src] + w; write_min.  With a near/far split a
// lowered vertex joins the next frontier only if its distance is below the current threshold;
// otherwise it is parked in the far bitmap until the threshold passes it.  Every relaxation is
// the reference's, only their order changes, and the least fixpoint of the float relaxations is
// unique, so distances are the same bit for bit.
struct SsspOp {
    float* dist;
    const float* wts;
    unsigned long long* next_bm;
    unsigned long long* far_bm;  // nullptr: plain Bellman-Ford sweeps
    float thr;
    __device__ uint32_t payload(uint32_t u) const { return __float_as_uint(__ldcg(dist + u)); }
    __device__ bool relax(uint32_t, uint32_t pay, uint32_t w, uint64_t pos) const {
        const float nd = __uint_as_float(pay) + wts[pos];
        if (!(nd < __ldcg(dist + w))) return false;
        const int old = atomicMin(reinterpret_cast<int*>(dist + w), __float_as_int(nd));
        if (!(nd < __int_as_float(old))) return false;
        const unsigned long long bit = 1ull << (w & 63);
        if (far_bm && !(nd < thr)) {
            if (!(__ldcg(far_bm + (w >> 6)) & bit)) atomicOr(far_bm + (w >> 6), bit);
            return false;
        }
        return !(atomicOr(next_bm + (w >> 6), bit) & bit);
    }
};

// far vertices whose distance is now below thr move to the near queue; the others stay, and
// their smallest distance (non-negative floats order like their bit patterns) and count are
// reported so that an empty phase can jump straight to the next occupied one
__global__ void k_far_split(unsigned long long* far_bm, uint64_t nwords, const float* __restrict__ dist, float thr,
                            uint32_t* q, uint32_t* nq, unsigned int* min_far_bits, unsigned int* n_far) {
    const int lane = threadIdx.x & 31;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t base = (uint64_t)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < nwords; base += stride) {
        const uint64_t w = base + lane;
        const unsigned long long word = w < nwords ? far_bm[w] : 0ull;
        unsigned long long move = 0;
        unsigned int mn = 0x7F800000u, left = 0;  // +inf
        for (unsigned long long x = word; x;) {
            const int b = __ffsll((long long)x) - 1;
            x &= x - 1;
            const float d = __ldcg(dist + w * 64 + b);
            if (d < thr) {
                move |= 1ull << b;
            } else {
                ++left;
                mn = min(mn, __float_as_uint(d));
            }
        }
        if (move) far_bm[w] = word & ~move;
        const uint32_t cnt = (uint32_t)__popcll(move);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            left += __shfl_xor_sync(0xffffffffu, left, o);
        }
        if (lane == 0 && left) {
            atomicMin(min_far_bits, mn);
            atomicAdd(n_far, left);
        }
        if (!tot) continue;
        uint32_t at = 0;
        if (lane == 31) at = atomicAdd(nq, tot);
        at = __shfl_sync(0xffffffffu, at, 31) + incl - cnt;
        for (unsigned long long x = move; x; x &= x - 1) q[at++] = (uint32_t)(w * 64 + (uint64_t)(__ffsll((long long)x) - 1));
    }
}

struct CcPushOp {  // toolkits/cc.cpp:50-60: msg = label[src]; write_min(label[dst], msg)
    uint32_t* label;
    unsigned long long* next_bm;
    __device__ uint32_t payload(uint32_t u) const { return __ldcg(label + u); }
    __device__ bool relax(uint32_t, uint32_t pay, uint32_t w, uint64_t) const {
        if (!(pay < __ldcg(label + w))) return false;
        const uint32_t old = atomicMin(label + w, pay);
        if (!(pay < old)) return false;
        const unsigned long long bit = 1ull << (w & 63);
        return !(atomicOr(next_bm + (w >> 6), bit) & bit);
    }
};

struct PrPullOp {  // toolkits/pagerank.cpp:64-97: sum curr[src]; next = 1-d+d*sum (/ outdeg)
    using Acc = float;
    static constexpr bool kFilter = false;
    __device__ bool stopped() const { return false; }
    __device__ bool item_active(uint32_t) const { return true; }
    const float* curr;
    float* next;
    float* acc;
    const uint32_t* outdeg;
    const uint32_t* slot;  // null: next in vertex order; else next[slot[v]] (renumbered order)
    float base, d;
    int divide, single;
    __device__ Acc identity() const { return 0.f; }
    __device__ Acc gather(uint32_t src, uint64_t) const { return ld_keep(curr + src); }
    __device__ Acc combine(Acc a, Acc b) const { return a + b; }
    __device__ void smem_add(Acc* slot, Acc v) const { atomicAdd(slot, v); }
    __device__ void finish(bool ok, uint32_t v, Acc a, bool whole) const {
        if (!ok) return;
        if (whole && single) {
            float x = base + d * a;
            if (divide) {
                uint32_t dg = outdeg[v];
                if (dg > 0) x /= (float)dg;
            }
            next[slot ? slot[v] : v] = x;
        } else {
            atomicAdd(acc + v, a);
        }
    }
};

struct CcPullOp {  // toolkits/cc.cpp:62-80: min label over in-neighbours, write_min + activate
    using Acc = uint32_t;
    static constexpr bool kFilter = false;
    __device__ bool stopped() const { return false; }
    __device__ bool item_active(uint32_t) const { return true; }
    uint32_t* label;
    unsigned long long* next_bm;
    uint32_t* q_out;
    uint32_t* n_out;
    unsigned long long* act_edges;
    const uint32_t* deg;
    __device__ Acc identity() const { return 0xFFFFFFFFu; }
    __device__ Acc gather(uint32_t src, uint64_t) const { return ld_keep(label + src); }
    __device__ Acc combine(Acc a, Acc b) const { return a < b ? a : b; }
    __device__ void smem_add(Acc* slot, Acc v) const { atomicMin(slot, v); }
    __device__ void finish(bool ok, uint32_t v, Acc m, bool) const {
        bool act = false;
        if (ok && m < __ldcg(label + v)) {
            uint32_t old = atomicMin(label + v, m);
            if (m < old) {
                const unsigned long long bit = 1ull << (v & 63);
                act = !(atomicOr(next_bm + (v >> 6), bit) & bit);
            }
        }
        // finish runs in a loop that is uniform across the CTA: one queue reservation per CTA
        __shared__ uint32_t s_cnt[2 * (kPullThreads / 32 + 1)];
        __shared__ unsigned long long s_deg[kPullThreads / 32];
        append_block_deg(act, v, q_out, n_out, act_edges, deg, s_cnt, s_deg, 0);
    }
};

// ---------------------------------------------------------------------------------------------
// vertex passes
__global__ void k_fill_u32(uint32_t* p, uint64_t n, uint32_t v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) p[i] = v;
}
__global__ void k_fill_f32(float* p, uint64_t n, float v) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) p[i] = v;
}
__global__ void k_iota(uint32_t* p, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) p[i] = (uint32_t)i;
}
// PageRank vectors are kept in vertex order, or (slot non-null) at slot[v]: the renumbering by
// out-degree class that the gathers go through
__global__ void k_pr_init(float* curr, const uint32_t* __restrict__ outdeg, uint32_t V,
                          const uint32_t* __restrict__ slot) {  // pagerank.cpp:36-45
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t dg = outdeg[v];
        curr[slot ? slot[v] : v] = dg > 0 ? 1.0f / (float)dg : 1.0f;
    }
}
// vertices without in-edges: next = 1-d (/ outdeg)
__global__ void k_pr_zero_in(float* buf, const uint32_t* __restrict__ indeg, const uint32_t* __restrict__ outdeg,
                             uint32_t V, float base, int divide, const uint32_t* __restrict__ slot) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x) {
        if (indeg[v] == 0) {
            uint32_t dg = outdeg[v];
            buf[slot ? slot[v] : v] = (divide && dg > 0) ? base / (float)dg : base;
        }
    }
}
// destinations whose list crossed a chunk boundary (P == 1)
__global__ void k_pr_split(const uint32_t* __restrict__ split, const uint32_t* __restrict__ cvert, uint64_t nsplit,
                           float* next, float* acc, const uint32_t* __restrict__ outdeg, float base, float d, int divide,
                           const uint32_t* __restrict__ slot) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nsplit; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = cvert[split[i]];
        float x = base + d * acc[v];
        acc[v] = 0.f;
        if (divide) {
            uint32_t dg = outdeg[v];
            if (dg > 0) x /= (float)dg;
        }
        next[slot ? slot[v] : v] = x;
    }
}
// P > 1: every destination with in-edges combines its partial sums
__global__ void k_pr_finish_all(const uint32_t* __restrict__ indeg, uint32_t V, float* next, float* acc,
                                const uint32_t* __restrict__ outdeg, float base, float d, int divide,
                                const uint32_t* __restrict__ slot) {
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x) {
        if (indeg[v] == 0) continue;
        float x = base + d * acc[v];
        acc[v] = 0.f;
        if (divide) {
            uint32_t dg = outdeg[v];
            if (dg > 0) x /= (float)dg;
        }
        next[slot ? slot[v] : v] = x;
    }
}

// ---- renumbering by out-degree class for the PageRank gathers ----------------------------------
// class = __clz(outdeg): 0 for the largest degrees, 31 for degree 1, 32 for no out-edges (never
// gathered).  new_id = the vertex's position in class order, tile by tile (tiles of 8,192
// vertices, classes counted per tile and scanned class-major), in any order inside a tile.
constexpr uint32_t kRelabelTile = 8192;
constexpr uint32_t kRelabelClasses = 33;
constexpr uint32_t kRelabelHot = 1u << 21;  // ranks spread round-robin over the hot region's lines

__global__ void __launch_bounds__(256) k_relabel_hist(const uint32_t* __restrict__ outdeg, uint32_t V, uint32_t ntiles,
                                                      uint32_t* __restrict__ cnt) {
    __shared__ uint32_t h[kRelabelClasses];
    if (threadIdx.x < kRelabelClasses) h[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t v0 = (uint64_t)blockIdx.x * kRelabelTile;
    for (uint32_t i = threadIdx.x; i < kRelabelTile; i += blockDim.x) {
        const uint64_t v = v0 + i;
        const uint32_t c = v < V ? (uint32_t)__clz(outdeg[v]) : kRelabelClasses;
        const uint32_t same = __match_any_sync(0xffffffffu, c);
        if (c < kRelabelClasses && (threadIdx.x & 31) == (uint32_t)(__ffs(same) - 1)) atomicAdd(&h[c], __popc(same));
    }
    __syncthreads();
    if (threadIdx.x < kRelabelClasses) cnt[(uint64_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(256) k_relabel_assign(const uint32_t* __restrict__ outdeg, uint32_t V, uint32_t ntiles,
                                                        const uint64_t* __restrict__ off, uint32_t lines,
                                                        uint32_t* __restrict__ new_id) {
    __shared__ uint32_t cur[kRelabelClasses];
    if (threadIdx.x < kRelabelClasses) cur[threadIdx.x] = (uint32_t)off[(uint64_t)threadIdx.x * ntiles + blockIdx.x];
    __syncthreads();
    const uint64_t v0 = (uint64_t)blockIdx.x * kRelabelTile;
    const uint32_t lane = threadIdx.x & 31;
    for (uint32_t i = threadIdx.x; i < kRelabelTile; i += blockDim.x) {
        const uint64_t v = v0 + i;
        const uint32_t c = v < V ? (uint32_t)__clz(outdeg[v]) : kRelabelClasses;
        const uint32_t same = __match_any_sync(0xffffffffu, c);
        const uint32_t leader = (uint32_t)(__ffs(same) - 1);
        uint32_t base = 0;
        if (c < kRelabelClasses && lane == leader) base = atomicAdd(&cur[c], __popc(same));
        base = __shfl_sync(same, base, leader);
        if (c < kRelabelClasses) {
            uint32_t r = base + __popc(same & ((1u << lane) - 1u));
            // the first 32 x lines ranks go round-robin over `lines` 128-byte lines: line j holds
            // ranks j, j + lines, ... (one vertex per heat stratum), so no line carries all hubs
            if (r < 32u * lines) r = (r % lines) * 32u + r / lines;
            new_id[v] = r;
        }
    }
}

// pr_adj[e] = new_id[csc_adj[e]]
__global__ void __launch_bounds__(256) k_relabel_adj(const uint32_t* __restrict__ adj, uint64_t E,
                                                     const uint32_t* __restrict__ new_id, uint32_t* __restrict__ out) {
    const uint64_t nq = E / 4;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < nq; q += stride) {
        const uint4 s = __ldcs(reinterpret_cast<const uint4*>(adj) + q);
        __stcs(reinterpret_cast<uint4*>(out) + q, make_uint4(__ldg(new_id + s.x), __ldg(new_id + s.y),
                                                            __ldg(new_id + s.z), __ldg(new_id + s.w)));
    }
    for (uint64_t e = 4 * nq + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += stride)
        out[e] = __ldg(new_id + adj[e]);
}

int scan_exclusive_u32(eg_graph* g, const uint32_t* in, uint64_t n, uint64_t* out);

bool want_relabel(const eg_graph* g) {
    return g->pr_relabel > 0 || (g->pr_relabel < 0 && g->V > (1u << 22));
}

int setup_relabel(eg_graph* g) {
    EngineState& s = g->eng;
    if (s.pr_ready) return EG_OK;
    const uint32_t V = g->V;
    const uint64_t E = g->E;
    const uint32_t ntiles = (uint32_t)(((uint64_t)V + kRelabelTile - 1) / kRelabelTile);
    const uint64_t ncnt = (uint64_t)kRelabelClasses * ntiles;
    EG_TRY(s.pr_new_id.reserve(sizeof(uint32_t) * ((size_t)V + 1)));
    EG_TRY(s.pr_adj.reserve(sizeof(uint32_t) * (E + 32)));
    EG_TRY(s.pr_cnt.reserve(sizeof(uint32_t) * ncnt));
    EG_TRY(s.pr_off.reserve(sizeof(uint64_t) * (ncnt + 1)));
    if (ntiles) {
        Timed t(&g->prof, g->stream, "pr_relabel");
        k_relabel_hist<<<ntiles, 256, 0, g->stream>>>(g->outdeg.as<uint32_t>(), V, ntiles, s.pr_cnt.as<uint32_t>());
        EG_CHECK_LAUNCH("k_relabel_hist");
    }
    if (ntiles) EG_TRY(scan_exclusive_u32(g, s.pr_cnt.as<uint32_t>(), ncnt, s.pr_off.as<uint64_t>()));
    {
        Timed t(&g->prof, g->stream, "pr_relabel");
        if (ntiles) {
            const uint32_t lines = std::min<uint32_t>(V, kRelabelHot) / 32u;
            k_relabel_assign<<<ntiles, 256, 0, g->stream>>>(g->outdeg.as<uint32_t>(), V, ntiles, s.pr_off.as<uint64_t>(),
                                                            lines, s.pr_new_id.as<uint32_t>());
            EG_CHECK_LAUNCH("k_relabel_assign");
        }
        if (E) {
            k_relabel_adj<<<grid_for(E / 4 + 1, 256, 152u * 16u), 256, 0, g->stream>>>(
                g->csc_adj.as<uint32_t>(), E, s.pr_new_id.as<uint32_t>(), s.pr_adj.as<uint32_t>());
            EG_CHECK_LAUNCH("k_relabel_adj");
        }
    }
    s.pr_ready = true;
    return EG_OK;
}

__global__ void k_bfs_root(uint32_t* level, uint32_t* parent, unsigned long long* visited, unsigned long long* front,
                           uint32_t root, uint32_t* q) {
    if (level) level[root] = 0;
    if (parent) parent[root] = root;
    visited[root >> 6] |= 1ull << (root & 63);
    front[root >> 6] |= 1ull << (root & 63);
    q[0] = root;
}
__global__ void k_sssp_root(float* dist, uint32_t root, uint32_t* q) {
    dist[root] = 0.f;
    q[0] = root;
}


// ---------------------------------------------------------------------------------------------
// Single-root BFS replayed as one CUDA graph with device-side control flow (EG_OPT_CUDA_GRAPH): a
// WHILE conditional node whose body runs two levels (the even one from queue 0 and frontier bitmap
// 0 into queue 1 and bitmap 1, the odd one back).  Each level is a one-thread kernel that arms one
// of two IF conditional nodes — the push (scan of the queued lists' lengths, rank-balanced
// expansion) or the dense step (early-exit head and tail) — or neither once the frontier is empty,
// then a one-thread kernel that moves the level's counters into the state; the odd level's also
// sets the loop condition.  No host round trip per level; the graph is built once per handle and
// structure and replayed for every root.  A traversal deeper than kBfsGraphLevels continues in the
// host loop from the state the graph leaves.
constexpr uint32_t kBfsGraphLevels = 4096;

struct BfsGraphState {
    uint32_t n;           // frontier length of the next level
    uint32_t lvl;         // levels done
    uint32_t next_level;  // level number of the vertices the running level reaches
    uint32_t ran;         // the running level was armed
    unsigned long long act;    // out-edges of the frontier
    unsigned long long reach;  // vertices reached
    unsigned long long total;  // out-edges of the reached vertices
    uint64_t scan_total;       // the push scan's edge total
    uint32_t pushes, pulls;
    uint32_t nout, pad0;       // the running level's queue length and out-edges
    unsigned long long nact;
    uint32_t nseg, pad1;       // the dense step's segments
};

static_assert(sizeof(BfsGraphState) <= 256, "the state is read back through the 256-byte pinned block");

__global__ void k_bfsg_init(BfsGraphState* st, const uint32_t* __restrict__ outdeg, uint32_t root) {
    const unsigned long long d = outdeg[root];
    st->n = 1;
    st->lvl = 0;
    st->next_level = 1;
    st->ran = 0;
    st->act = d;
    st->reach = 1;
    st->total = d;
    st->scan_total = 0;
    st->pushes = st->pulls = 0;
    st->nout = 0;
    st->nact = 0;
    st->nseg = 0;
}

// core/graph.hpp:1484-1491 (Gemini's switch) on the device: sparse iff the frontier's out-edges < E/div
__global__ void k_bfsg_decide(BfsGraphState* st, cudaGraphConditionalHandle h_push, cudaGraphConditionalHandle h_pull,
                              unsigned long long dense_min, int direction, int has_csc) {
    const bool go = st->n > 0 && st->lvl < kBfsGraphLevels;
    const bool dense = go && (direction == 2 || (direction == 0 && has_csc && st->act >= dense_min));
    st->ran = go ? 1u : 0u;
    st->next_level = st->lvl + 1;
    st->nout = 0;
    st->nact = 0;
    st->nseg = 0;
    if (go) {
        if (dense) ++st->pulls;
        else ++st->pushes;
    }
    cudaGraphSetConditional(h_push, go && !dense ? 1u : 0u);
    cudaGraphSetConditional(h_pull, dense ? 1u : 0u);
}

__global__ void k_bfsg_post(BfsGraphState* st, cudaGraphConditionalHandle h_loop, int odd) {
    if (st->ran) {
        st->n = st->nout;
        st->act = st->nact;
        st->reach += st->nout;
        st->total += st->nact;
        ++st->lvl;
    }
    if (odd) cudaGraphSetConditional(h_loop, st->n > 0 && st->lvl < kBfsGraphLevels ? 1u : 0u);
}

// the key a built graph is valid for: sizes, switch settings and every buffer it was captured with
static std::vector<uint64_t> bfs_graph_key(eg_graph* g) {
    EngineState& s = g->eng;
    auto p = [](const void* x) { return (uint64_t)(uintptr_t)x; };
    return {g->V, g->E, g->ncompressed, (uint64_t)g->partitions, (uint64_t)g->dense_div, (uint64_t)g->bfs_direction,
            (uint64_t)g->built_csc, p(g->csr_off.ptr), p(g->csr_adj.ptr), p(g->csc_adj.ptr), p(g->cidx.ptr),
            p(g->cvert.ptr), p(g->outdeg.ptr), p(s.q0.ptr), p(s.q1.ptr), p(s.bm_visit.ptr), p(s.bm_next.ptr),
            p(s.bm_front.ptr), p(s.vals0.ptr), p(s.vals1.ptr), p(s.qdeg.ptr), p(s.chunk_item.ptr), p(s.bu_seg.ptr),
            p(g->scan.desc.ptr), p(g->scan.counter.ptr), p(g->err.ptr), p(s.bfs_state.ptr)};
}

static int build_bfs_graph(eg_graph* g) {
    EngineState& s = g->eng;
    const uint32_t V = g->V;
    const int P = g->partitions;
    const uint64_t max_items = (uint64_t)V * P;
    const uint64_t max_tiles = (max_items + kScanTile - 1) / kScanTile + 1;
    EG_TRY(g->scan.desc.reserve(max_tiles * sizeof(uint64_t)));
    EG_TRY(g->scan.counter.reserve(16));
    EG_TRY(s.bfs_state.reserve(sizeof(BfsGraphState)));
    std::vector<uint64_t> key = bfs_graph_key(g);
    if (s.bfs_exec && key == s.bfs_key) return EG_OK;
    if (s.bfs_exec) cudaGraphExecDestroy(s.bfs_exec);
    if (s.bfs_graph) cudaGraphDestroy(s.bfs_graph);
    s.bfs_exec = nullptr;
    s.bfs_graph = nullptr;
    BfsGraphState* st = s.bfs_state.as<BfsGraphState>();
    uint32_t* q[2] = {s.q0.as<uint32_t>(), s.q1.as<uint32_t>()};
    unsigned long long* F[2] = {s.bm_next.as<unsigned long long>(), s.bm_front.as<unsigned long long>()};
    unsigned long long* visit = s.bm_visit.as<unsigned long long>();
    uint32_t* d_level = s.vals0.as<uint32_t>();
    uint32_t* d_parent = s.vals1.as<uint32_t>();
    const size_t bm_bytes = sizeof(uint64_t) * (V / 64 + 1);
    const unsigned long long dense_min = g->E / (uint64_t)g->dense_div;
    // captured on a stream of its own, so that nothing else the caller queued is recorded
    cudaStream_t cs = nullptr;
    EG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    struct StreamGuard {
        cudaStream_t s;
        ~StreamGuard() { cudaStreamDestroy(s); }
    } guard{cs};
    cudaGraph_t G = nullptr;
    EG_CUDA(cudaGraphCreate(&G, 0));
    s.bfs_graph = G;
    cudaGraphConditionalHandle h_loop;
    EG_CUDA(cudaGraphConditionalHandleCreate(&h_loop, G, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode;
    EG_CUDA(cudaGraphAddNode(&wnode, G, nullptr, nullptr, 0, &wp));
    cudaGraph_t body = wp.conditional.phGraph_out[0];
    cudaGraphConditionalHandle h_push[2], h_pull[2];
    for (int k = 0; k < 2; ++k) {
        EG_CUDA(cudaGraphConditionalHandleCreate(&h_push[k], body, 0, 0));
        EG_CUDA(cudaGraphConditionalHandleCreate(&h_pull[k], body, 0, 0));
    }
    // an IF node after the capture's current dependencies; returns its (empty) body graph
    auto add_if = [&](cudaGraphConditionalHandle h, cudaGraph_t* out) -> int {
        cudaStreamCaptureStatus cst;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        const cudaGraphEdgeData* ed = nullptr;
        size_t nd = 0;
        EG_CUDA(cudaStreamGetCaptureInfo(cs, &cst, nullptr, &cg, &deps, &ed, &nd));
        cudaGraphNodeParams ip = {};
        ip.type = cudaGraphNodeTypeConditional;
        ip.conditional.handle = h;
        ip.conditional.type = cudaGraphCondTypeIf;
        ip.conditional.size = 1;
        cudaGraphNode_t node;
        EG_CUDA(cudaGraphAddNode(&node, cg, deps, ed, nd, &ip));
        *out = ip.conditional.phGraph_out[0];
        EG_CUDA(cudaStreamUpdateCaptureDependencies(cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
        return EG_OK;
    };
    cudaGraph_t push_body[2], pull_body[2];
    EG_CUDA(cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < 2; ++k) {
        k_bfsg_decide<<<1, 1, 0, cs>>>(st, h_push[k], h_pull[k], dense_min, g->bfs_direction, g->built_csc ? 1 : 0);
        EG_TRY(add_if(h_push[k], &push_body[k]));
        EG_TRY(add_if(h_pull[k], &pull_body[k]));
        k_bfsg_post<<<1, 1, 0, cs>>>(st, h_loop, k);
    }
    cudaGraph_t captured = nullptr;
    EG_CUDA(cudaStreamEndCapture(cs, &captured));
    const unsigned scan_grid = (unsigned)std::min<uint64_t>(max_tiles, (uint64_t)g->num_sms * 8u);
    for (int k = 0; k < 2; ++k) {
        // push: queue q[k] -> q[k^1], new frontier bits in F[k^1]; F[k] cleared for the level after
        EG_CUDA(cudaStreamBeginCaptureToGraph(cs, push_body[k], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        EG_CUDA(cudaMemsetAsync(g->scan.desc.ptr, 0, max_tiles * sizeof(uint64_t), cs));
        EG_CUDA(cudaMemsetAsync(g->scan.counter.ptr, 0, 4, cs));
        uint64_t* ipref = s.qdeg.as<uint64_t>();
        LoadItemLen ld{q[k], P, (uint64_t)V + 1, g->csr_off.as<uint64_t>()};
        EpiItemRank ep{ipref, s.chunk_item.as<uint32_t>()};
        k_scan<<<scan_grid, kScanThreads, 0, cs>>>(ld, ep, max_items, g->scan.desc.as<uint64_t>(),
                                                   g->scan.counter.as<uint32_t>(), g->err.as<int>(), &st->scan_total,
                                                   kLookbackSpinCap, &st->n, (uint32_t)P);
        PushArgs a;
        a.q = q[k];
        a.nitems = 0;
        a.n_dev = &st->n;
        a.total_dev = &st->scan_total;
        a.P = P;
        a.stride = (uint64_t)V + 1;
        a.off = g->csr_off.as<uint64_t>();
        a.adj = g->csr_adj.as<uint32_t>();
        a.w = g->csr_w.as<float>();
        a.ipref = ipref;
        a.chunk_item = s.chunk_item.as<uint32_t>();
        a.q_out = q[k ^ 1];
        a.n_out = &st->nout;
        a.act_edges = &st->nact;
        a.deg = g->outdeg.as<uint32_t>();
        BfsOp op{visit, F[k ^ 1], d_level, d_parent, 0u, &st->next_level};
        k_push<BfsOp><<<kPersistentGrid, kPushThreads, 0, cs>>>(op, a);
        EG_CUDA(cudaMemsetAsync(F[k], 0, bm_bytes, cs));
        EG_CUDA(cudaStreamEndCapture(cs, &captured));
        // dense step: every unvisited destination looks for a parent in F[k]
        EG_CUDA(cudaStreamBeginCaptureToGraph(cs, pull_body[k], nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        if (g->built_csc) {
            BuArgs ba{g->csc_adj.as<uint32_t>(), g->cidx.as<uint64_t>(), g->cvert.as<uint32_t>(), g->ncompressed - 1, V,
                      F[k], visit, F[k ^ 1], d_level, d_parent, 0u, q[k ^ 1], &st->nout, &st->nact,
                      g->outdeg.as<uint32_t>(), s.bu_seg.as<unsigned long long>(), &st->nseg, &st->next_level};
            k_bu_head<<<grid_for(ba.nitems, 256, (unsigned)g->num_sms * 8u), 256, 0, cs>>>(ba);
            k_bu_tail<<<(unsigned)g->num_sms * 8u, 256, 0, cs>>>(ba);
        }
        EG_CUDA(cudaMemsetAsync(F[k], 0, bm_bytes, cs));
        EG_CUDA(cudaStreamEndCapture(cs, &captured));
    }
    EG_CUDA(cudaGraphInstantiate(&s.bfs_exec, G, 0));
    s.bfs_key = key;
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
int run_pagerank(eg_graph* g, int iterations, float damping, float* out, int where) {
    if (!g->built_csc) { set_error("eg_pagerank: CSC not built"); return EG_ERR_STATE; }
    if (iterations < 0) { set_error("eg_pagerank: iterations must be >= 0"); return EG_ERR_INVALID; }
    EG_TRY(ensure_engine(g));
    EG_TRY(setup_pull(g));
    const uint32_t V = g->V;
    EngineState& s = g->eng;
    float* A = s.vals0.as<float>();
    float* B = s.vals1.as<float>();
    const float base = 1.0f - damping;
    const int single = g->partitions == 1;
    const unsigned gv = grid_for(V, 256, 152u * 16u);
    // with renumbered gathers every vector but the final one is kept in class order
    const bool relabel = iterations > 0 && g->E > 0 && want_relabel(g);
    if (relabel) EG_TRY(setup_relabel(g));
    const uint32_t* order = relabel ? s.pr_new_id.as<uint32_t>() : nullptr;
    const uint32_t* gather_adj = relabel ? s.pr_adj.as<uint32_t>() : nullptr;
    {
        Timed t(&g->prof, g->stream, "pr_vertex");
        k_pr_init<<<gv, 256, 0, g->stream>>>(A, g->outdeg.as<uint32_t>(), V, order);
        EG_CHECK_LAUNCH("k_pr_init");
        EG_CUDA(cudaMemsetAsync(s.acc.ptr, 0, sizeof(float) * (size_t)V, g->stream));
    }
    for (int it = 0; it < iterations; ++it) {
        const int last = it == iterations - 1;
        float* curr = (it & 1) ? B : A;
        float* next = (it & 1) ? A : B;
        const uint32_t* slot = last ? nullptr : order;
        if (it < 2 || last) {
            Timed t(&g->prof, g->stream, "pr_vertex");
            k_pr_zero_in<<<gv, 256, 0, g->stream>>>(next, g->indeg.as<uint32_t>(), g->outdeg.as<uint32_t>(), V, base, !last,
                                                    slot);
            EG_CHECK_LAUNCH("k_pr_zero_in");
        }
        PrPullOp op{curr, next, s.acc.as<float>(), g->outdeg.as<uint32_t>(), slot, base, damping, !last, single};
        EG_TRY(launch_pull(g, op, "pr_pull", gather_adj));
        Timed t(&g->prof, g->stream, "pr_finish");
        if (single) {
            if (s.pull_nsplit) {
                k_pr_split<<<grid_for(s.pull_nsplit, 256), 256, 0, g->stream>>>(
                    s.pull_split.as<uint32_t>(), g->cvert.as<uint32_t>(), s.pull_nsplit, next, s.acc.as<float>(),
                    g->outdeg.as<uint32_t>(), base, damping, !last, slot);
                EG_CHECK_LAUNCH("k_pr_split");
            }
        } else {
            k_pr_finish_all<<<gv, 256, 0, g->stream>>>(g->indeg.as<uint32_t>(), V, next, s.acc.as<float>(),
                                                       g->outdeg.as<uint32_t>(), base, damping, !last, slot);
            EG_CHECK_LAUNCH("k_pr_finish_all");
        }
    }
    float* result = (iterations & 1) ? B : A;
    EG_TRY(copy_out(g, out, result, sizeof(float) * (size_t)V, where));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->last_edges_processed = g->E * (uint64_t)iterations;
    g->last_iterations = iterations;
    g->last_pushes = 0;
    g->last_pulls = iterations;
    return EG_OK;
}

int run_bfs(eg_graph* g, uint32_t root, uint32_t* level, uint32_t* parent, int where, uint64_t* reached) {
    if (!g->built_csr) { set_error("eg_bfs: CSR not built"); return EG_ERR_STATE; }
    if (root >= g->V) { set_error("eg_bfs: root %u >= V %u", root, g->V); return EG_ERR_INVALID; }
    EG_TRY(ensure_engine(g));
    const uint32_t V = g->V;
    EngineState& s = g->eng;
    uint32_t* d_level = s.vals0.as<uint32_t>();
    uint32_t* d_parent = s.vals1.as<uint32_t>();
    const unsigned gv = grid_for(V, 256, 152u * 16u);
    const size_t bm_bytes = sizeof(uint64_t) * (V / 64 + 1);
    unsigned long long* front = s.bm_next.as<unsigned long long>();
    unsigned long long* next_front = s.bm_front.as<unsigned long long>();
    {
        Timed t(&g->prof, g->stream, "bfs_init");
        k_fill_u32<<<gv, 256, 0, g->stream>>>(d_level, V, 0xFFFFFFFFu);
        EG_CHECK_LAUNCH("k_fill_u32");
        k_fill_u32<<<gv, 256, 0, g->stream>>>(d_parent, V, V);
        EG_CHECK_LAUNCH("k_fill_u32");
        EG_CUDA(cudaMemsetAsync(s.bm_visit.ptr, 0, bm_bytes, g->stream));
        EG_CUDA(cudaMemsetAsync(front, 0, bm_bytes, g->stream));
        EG_CUDA(cudaMemsetAsync(next_front, 0, bm_bytes, g->stream));
        k_bfs_root<<<1, 1, 0, g->stream>>>(d_level, d_parent, s.bm_visit.as<unsigned long long>(), front, root,
                                           s.q0.as<uint32_t>());
        EG_CHECK_LAUNCH("k_bfs_root");
    }
    if (g->built_csc) {
        // segment list of the dense step: at most one segment per entry with more than kBuHead
        // in-edges plus one per kBuSeg edges
        const uint64_t nitems = g->ncompressed - 1;
        const uint64_t heavy = std::min<uint64_t>(nitems, g->E / (kBuHead + 1));
        EG_TRY(s.bu_seg.reserve(sizeof(unsigned long long) * (heavy + g->E / kBuSeg + 2)));
    }
    uint32_t* qa = s.q0.as<uint32_t>();
    uint32_t* qb = s.q1.as<uint32_t>();
    uint64_t n = 1, reach = 1;
    unsigned long long active_edges = 0, total_edges = 0;
    uint32_t lvl = 0;
    int pushes = 0, pulls = 0;
    if (g->use_cuda_graph & 2) {
        // the whole level loop as one graph replay; the state it leaves says where it stopped
        EG_TRY(build_bfs_graph(g));
        BfsGraphState* st = s.bfs_state.as<BfsGraphState>();
        k_bfsg_init<<<1, 1, 0, g->stream>>>(st, g->outdeg.as<uint32_t>(), root);
        EG_CHECK_LAUNCH("k_bfsg_init");
        {
            Timed t(&g->prof, g->stream, "bfs_graph");
            EG_CUDA(cudaGraphLaunch(s.bfs_exec, g->stream));
        }
        BfsGraphState* hs = reinterpret_cast<BfsGraphState*>(s.host_words);  // pinned
        EG_CUDA(cudaMemcpyAsync(hs, st, sizeof(BfsGraphState), cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        EG_TRY(check_device_error(g, "eg_bfs"));
        n = hs->n;
        lvl = hs->lvl;
        reach = hs->reach;
        active_edges = hs->act;
        total_edges = hs->total;
        pushes = (int)hs->pushes;
        pulls = (int)hs->pulls;
        if (lvl & 1) {  // level lvl reads queue lvl & 1 and frontier bitmap lvl & 1
            std::swap(qa, qb);
            std::swap(front, next_front);
        }
    } else {
        uint32_t* hroot = reinterpret_cast<uint32_t*>(s.host_words + 3);  // pinned
        EG_CUDA(cudaMemcpyAsync(hroot, g->outdeg.as<uint32_t>() + root, 4, cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        active_edges = total_edges = *hroot;
    }
    while (n > 0) {
        // core/graph.hpp:1484-1491 (Gemini's switch): sparse iff the frontier's out-edges < E / div
        const bool dense = g->bfs_direction == 2 ||
                           (g->bfs_direction == 0 && g->built_csc && active_edges >= g->E / (uint64_t)g->dense_div);
        uint32_t nout = 0;
        unsigned long long act = 0;
        if (!dense) {
            BfsOp op{s.bm_visit.as<unsigned long long>(), next_front, d_level, d_parent, lvl + 1};
            EG_TRY(push_level(g, op, qa, n, qb, &nout, nullptr, &act, g->outdeg.as<uint32_t>(), "bfs_push"));
            ++pushes;
        } else {
            uint32_t* d_nout = reinterpret_cast<uint32_t*>(s.counters.as<unsigned long long>() + 2);
            unsigned long long* d_act = s.counters.as<unsigned long long>() + 3;
            uint32_t* d_nseg = reinterpret_cast<uint32_t*>(s.counters.as<unsigned long long>() + 5);
            EG_CUDA(cudaMemsetAsync(d_nout, 0, 16, g->stream));
            EG_CUDA(cudaMemsetAsync(d_nseg, 0, 8, g->stream));
            BuArgs a{g->csc_adj.as<uint32_t>(), g->cidx.as<uint64_t>(), g->cvert.as<uint32_t>(), g->ncompressed - 1, V,
                     front, s.bm_visit.as<unsigned long long>(), next_front, d_level, d_parent, lvl + 1, qb, d_nout,
                     d_act, g->outdeg.as<uint32_t>(), s.bu_seg.as<unsigned long long>(), d_nseg};
            {
                Timed t(&g->prof, g->stream, "bfs_pull");
                k_bu_head<<<grid_for(a.nitems, 256, (unsigned)g->num_sms * 8u), 256, 0, g->stream>>>(a);
                EG_CHECK_LAUNCH("k_bu_head");
            }
            {
                Timed t(&g->prof, g->stream, "bfs_pull_tail");
                k_bu_tail<<<(unsigned)g->num_sms * 8u, 256, 0, g->stream>>>(a);
                EG_CHECK_LAUNCH("k_bu_tail");
            }
            uint64_t* hw = s.host_words;  // pinned: queue length, active out-edges
            EG_CUDA(cudaMemcpyAsync(hw, d_nout, 16, cudaMemcpyDeviceToHost, g->stream));
            EG_CUDA(cudaStreamSynchronize(g->stream));
            nout = (uint32_t)(hw[0] & 0xFFFFFFFFu);
            act = hw[1];
            ++pulls;
        }
        EG_CUDA(cudaMemsetAsync(front, 0, bm_bytes, g->stream));
        std::swap(front, next_front);
        total_edges += act;
        active_edges = act;
        reach += nout;
        std::swap(qa, qb);
        n = nout;
        ++lvl;
    }
    EG_TRY(copy_out(g, level, d_level, sizeof(uint32_t) * (size_t)V, where));
    EG_TRY(copy_out(g, parent, d_parent, sizeof(uint32_t) * (size_t)V, where));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    if (reached) *reached = reach;
    g->last_edges_processed = total_edges;  // sum of out-degrees of the reached vertices
    g->last_iterations = (int)lvl;
    g->last_pushes = pushes;
    g->last_pulls = pulls;
    return EG_OK;
}

// mean of a strided sample of the weights, for the automatic near/far threshold step
__global__ void k_weight_sample(const float* __restrict__ w, uint64_t E, uint64_t step, uint32_t n, float* out) {
    float acc = 0.f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint64_t e = (uint64_t)i * step;
        if (e < E) acc += w[e];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, acc);
}

int run_sssp(eg_graph* g, uint32_t root, float* dist, int where) {
    if (!g->built_csr) { set_error("eg_sssp: CSR not built"); return EG_ERR_STATE; }
    if (!g->weighted) { set_error("eg_sssp: graph has no edge weights (load 12-byte records)"); return EG_ERR_STATE; }
    if (root >= g->V) { set_error("eg_sssp: root %u >= V %u", root, g->V); return EG_ERR_INVALID; }
    EG_TRY(ensure_engine(g));
    const uint32_t V = g->V;
    EngineState& s = g->eng;
    float* d_dist = s.vals0.as<float>();
    const uint64_t nwords = (uint64_t)V / 64 + 1;
    const size_t bm_bytes = sizeof(uint64_t) * nwords;
    unsigned long long* far_bm = s.bm_visit.as<unsigned long long>();
    unsigned int* d_small = reinterpret_cast<unsigned int*>(s.counters.as<unsigned long long>() + 6);
    {
        Timed t(&g->prof, g->stream, "sssp_init");
        k_fill_f32<<<grid_for(V, 256, 152u * 16u), 256, 0, g->stream>>>(d_dist, V, 1e9f);
        EG_CHECK_LAUNCH("k_fill_f32");
        EG_CUDA(cudaMemsetAsync(s.bm_next.ptr, 0, bm_bytes, g->stream));
        EG_CUDA(cudaMemsetAsync(far_bm, 0, bm_bytes, g->stream));
        k_sssp_root<<<1, 1, 0, g->stream>>>(d_dist, root, s.q0.as<uint32_t>());
        EG_CHECK_LAUNCH("k_sssp_root");
    }
    // threshold step: the option (millionths), or 0.7 x mean weight / mean out-degree (the best
    // of a sweep on the 41.6 M-vertex, 1.47 B-edge R-MAT: 0.01 there, 2.3x faster than plain
    // sweeps), or none
    float delta = 0.f;
    if (g->sssp_delta > 0) {
        delta = (float)((double)g->sssp_delta * 1e-6);
    } else if (g->sssp_delta < 0 && g->E > 0) {
        const uint32_t ns = 65536;
        const uint64_t step = std::max<uint64_t>(g->E / ns, 1);
        float* d_sum = reinterpret_cast<float*>(d_small);
        EG_CUDA(cudaMemsetAsync(d_sum, 0, 4, g->stream));
        k_weight_sample<<<64, 256, 0, g->stream>>>(g->csr_w.as<float>(), g->E, step, ns, d_sum);
        EG_CHECK_LAUNCH("k_weight_sample");
        float sum = 0.f;
        EG_CUDA(cudaMemcpyAsync(&sum, d_sum, 4, cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        const uint64_t taken = std::min<uint64_t>(ns, (g->E + step - 1) / step);
        const double mean_w = taken ? sum / (double)taken : 0.0;
        const double mean_deg = (double)g->E / (double)V;
        delta = (float)(mean_w * 0.7 / std::max(mean_deg, 1.0));
    }
    const bool split = delta > 0.f;
    float thr = split ? delta : INFINITY;
    uint32_t* qa = s.q0.as<uint32_t>();
    uint32_t* qb = s.q1.as<uint32_t>();
    uint64_t n = 1, total_edges = 0;
    int iters = 0, phases = 1;
    while (true) {
        while (n > 0) {
            SsspOp op{d_dist, g->csr_w.as<float>(), s.bm_next.as<unsigned long long>(), split ? far_bm : nullptr, thr};
            uint32_t nout = 0;
            uint64_t T = 0;
            EG_TRY(push_level(g, op, qa, n, qb, &nout, &T, nullptr, nullptr, "sssp_push"));
            EG_CUDA(cudaMemsetAsync(s.bm_next.ptr, 0, bm_bytes, g->stream));
            total_edges += T;
            std::swap(qa, qb);
            n = nout;
            ++iters;
        }
        if (!split) break;
        // next phase: raise the threshold by delta, or to the nearest parked distance + delta
        struct {
            unsigned int nq, min_bits, n_far, pad;
        } h = {0, 0, 0, 0};
        float next = thr + delta;
        for (int attempt = 0; attempt < 2; ++attempt) {
            const unsigned int init[4] = {0u, 0x7F800000u, 0u, 0u};
            EG_CUDA(cudaMemcpyAsync(d_small, init, 16, cudaMemcpyHostToDevice, g->stream));
            {
                Timed t(&g->prof, g->stream, "sssp_far_split");
                k_far_split<<<grid_for(nwords, 256, (unsigned)g->num_sms * 8u), 256, 0, g->stream>>>(
                    far_bm, nwords, d_dist, next, qa, d_small, d_small + 1, d_small + 2);
                EG_CHECK_LAUNCH("k_far_split");
            }
            EG_CUDA(cudaMemcpyAsync(&h, d_small, 16, cudaMemcpyDeviceToHost, g->stream));
            EG_CUDA(cudaStreamSynchronize(g->stream));
            if (h.nq > 0 || h.n_far == 0) break;
            float mn;
            memcpy(&mn, &h.min_bits, 4);
            next = std::max(next, mn) + delta;  // skip the empty phases
        }
        thr = next;
        n = h.nq;
        ++phases;
        if (n == 0) break;  // nothing parked: done
    }
    EG_TRY(copy_out(g, dist, d_dist, sizeof(float) * (size_t)V, where));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->last_edges_processed = total_edges;
    g->last_iterations = iters;
    g->last_pushes = iters;
    g->last_pulls = 0;
    return EG_OK;
}

int run_cc(eg_graph* g, uint32_t* label, int where) {
    if (!g->built_csr || !g->built_csc) { set_error("eg_cc: CSR and CSC must be built"); return EG_ERR_STATE; }
    EG_TRY(ensure_engine(g));
    EG_TRY(setup_pull(g));
    const uint32_t V = g->V;
    EngineState& s = g->eng;
    uint32_t* d_label = s.vals0.as<uint32_t>();
    const size_t bm_bytes = sizeof(uint64_t) * (V / 64 + 1);
    const unsigned gv = grid_for(V, 256, 152u * 16u);
    uint32_t* qa = s.q0.as<uint32_t>();
    uint32_t* qb = s.q1.as<uint32_t>();
    {
        Timed t(&g->prof, g->stream, "cc_init");
        k_iota<<<gv, 256, 0, g->stream>>>(d_label, V);  // cc.cpp:31-37
        EG_CHECK_LAUNCH("k_iota");
        k_iota<<<gv, 256, 0, g->stream>>>(qa, V);       // active_in->fill()
        EG_CHECK_LAUNCH("k_iota");
        EG_CUDA(cudaMemsetAsync(s.bm_next.ptr, 0, bm_bytes, g->stream));
    }
    uint64_t n = V;
    unsigned long long active_edges = g->E;  // every vertex active: sum of out-degrees
    uint64_t total_edges = 0;
    int iters = 0, pushes = 0, pulls = 0;
    uint32_t* d_nout = reinterpret_cast<uint32_t*>(s.counters.as<unsigned long long>() + 2);
    unsigned long long* d_act = s.counters.as<unsigned long long>() + 3;
    while (n > 0) {
        uint32_t nout = 0;
        unsigned long long act = 0;
        // core/graph.hpp:1484-1491: sparse iff active_edges < edges / 20
        const bool sparse = active_edges < g->E / (uint64_t)g->dense_div;
        if (sparse) {
            CcPushOp op{d_label, s.bm_next.as<unsigned long long>()};
            uint64_t T = 0;
            EG_TRY(push_level(g, op, qa, n, qb, &nout, &T, &act, g->outdeg.as<uint32_t>(), "cc_push"));
            total_edges += T;
            ++pushes;
        } else {
            EG_CUDA(cudaMemsetAsync(s.counters.as<unsigned long long>() + 2, 0, 16, g->stream));
            CcPullOp op{d_label, s.bm_next.as<unsigned long long>(), qb, d_nout, d_act, g->outdeg.as<uint32_t>()};
            EG_TRY(launch_pull(g, op, "cc_pull"));
            struct {
                uint32_t n;
                uint32_t pad;
                unsigned long long act;
            } h;
            EG_CUDA(cudaMemcpyAsync(&h, d_nout, 16, cudaMemcpyDeviceToHost, g->stream));
            EG_CUDA(cudaStreamSynchronize(g->stream));
            nout = h.n;
            act = h.act;
            total_edges += g->E;
            ++pulls;
        }
        EG_CUDA(cudaMemsetAsync(s.bm_next.ptr, 0, bm_bytes, g->stream));
        std::swap(qa, qb);
        n = nout;
        active_edges = act;
        ++iters;
    }
    EG_TRY(copy_out(g, label, d_label, sizeof(uint32_t) * (size_t)V, where));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->last_edges_processed = total_edges;
    g->last_iterations = iters;
    g->last_pushes = pushes;
    g->last_pulls = pulls;
    return EG_OK;
}

}  // namespace eg
