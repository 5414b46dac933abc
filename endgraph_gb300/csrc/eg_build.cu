// eg_build.cu — preprocessing on the GPU: degree histogram, CPBT partitioning, partition
// bucketing and the two structures of split_graph (core/graph.hpp:981-1009):
//   CSR  (prepare_push_mode :1248-1355): partition p = edges whose dst p owns, keyed by src
//   CSC  (prepare_pull_mode :1098-1242): partition p = edges whose src p owns, keyed by dst,
//        plus the compressed incoming index (:1144-1188)
//
// Layout in HBM (P partitions, V vertices, E edges):
//   outdeg/indeg      u32[V]
//   csr_off/csc_off   u64[P*(V+1)]   list (p,v) = [off[p*(V+1)+v], off[p*(V+1)+v+1])
//   csr_adj/csc_adj   u32[E]         neighbour ids (structure of arrays; weights in f32[E])
//   csr_bitmap        u64[P*(V/64+1)]
//   cvert/cidx        u32/u64 per non-empty CSC list + one sentinel per partition
// Construction is a counting sort: the scan writes INCLUSIVE offsets and the scatter claims
// positions by atomically decrementing them, which leaves exactly the exclusive offsets behind
// (no cursor array, no copy).  Intra-list order is therefore not the reference's; parity is
// defined on per-list sorted neighbours, as the reference's own order is thread-dependent.
#include <string.h>

#include <algorithm>

#include "eg_common.cuh"
#include "eg_scan.cuh"

namespace eg {

template <int REC>
__device__ __forceinline__ void load_edge(const uint8_t* __restrict__ base, uint64_t i, uint32_t& s, uint32_t& d,
                                          float& w) {
    if (REC == 8) {
        uint2 x = __ldg(reinterpret_cast<const uint2*>(base) + i);
        s = x.x;
        d = x.y;
        w = 0.f;
    } else {
        const uint32_t* r = reinterpret_cast<const uint32_t*>(base + i * 12u);
        s = __ldg(r);
        d = __ldg(r + 1);
        w = __uint_as_float(__ldg(r + 2));
    }
}

// ---- degree histogram (core/graph.hpp:689-707, both directions in one pass) ------------------
template <int REC>
__global__ void __launch_bounds__(256) k_degrees(const uint8_t* __restrict__ edges, uint64_t E,
                                                  uint32_t* __restrict__ outdeg, uint32_t* __restrict__ indeg) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s, d;
        float w;
        load_edge<REC>(edges, i, s, d, w);
        atomicAdd(&outdeg[s], 1u);
        atomicAdd(&indeg[d], 1u);
    }
}

// ids >= V are rejected before any structure is built
template <int REC>
__global__ void k_validate(const uint8_t* __restrict__ edges, uint64_t E, uint32_t V, int* bad) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s, d;
        float w;
        load_edge<REC>(edges, i, s, d, w);
        if (s >= V || d >= V) atomicExch(bad, 1);
    }
}

// symmetric load: records [E, 2E) = reversed copies of [0, E) (core/graph.hpp:1057-1078)
template <int REC>
__global__ void k_symmetrize(uint8_t* __restrict__ edges, uint64_t E) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t* r = reinterpret_cast<const uint32_t*>(edges + i * REC);
        uint32_t* o = reinterpret_cast<uint32_t*>(edges + (E + i) * REC);
        o[0] = r[1];
        o[1] = r[0];
        if (REC == 12) o[2] = r[2];
    }
}

// ---- CPBT page weights (core/graph.hpp:718-741) ----------------------------------------------
// (1 + (P-1)/16) * deg in 32-bit unsigned arithmetic, + eta * (32-bit unsigned)(P - 1 + T * deg)
__global__ void __launch_bounds__(256) k_page_weights(const uint32_t* __restrict__ deg, uint32_t V, uint32_t c1,
                                                       uint32_t pm1, uint32_t T, uint64_t eta,
                                                       uint64_t* __restrict__ out, uint32_t pages) {
    __shared__ uint64_t s_red[8];
    for (uint32_t pg = blockIdx.x; pg < pages; pg += gridDim.x) {
        uint64_t acc = 0;
        uint32_t vb = pg * kPageSize;
        for (uint32_t k = threadIdx.x; k < kPageSize; k += blockDim.x) {
            uint32_t v = vb + k;
            if (v < V) {
                uint32_t dv = deg[v];
                uint32_t t1 = c1 * dv;
                uint32_t t2 = pm1 + T * dv;
                acc += (uint64_t)t1 + eta * (uint64_t)t2;
            }
        }
        acc = warp_sum_u64(acc);
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint64_t t = 0;
            for (int w = 0; w < 8; ++w) t += s_red[w];
            out[pg] = t;
        }
        __syncthreads();
    }
}

// ---- optimal_offset / judge (core/graph.hpp:586-626) on one CTA ------------------------------
// prefix view: value(j) = p[j] - base for j in [0, n]
__device__ __forceinline__ uint32_t last_le(const uint64_t* p, uint64_t base, uint32_t n, uint64_t x) {
    // std::upper_bound(prefix, prefix + n + 1, x) - 1
    uint64_t lim = x + base;
    uint32_t lo = 0, hi = n + 1;
    while (lo < hi) {
        uint32_t mid = lo + ((hi - lo) >> 1);
        if (p[mid] <= lim) lo = mid + 1; else hi = mid;
    }
    return lo - 1;
}

__device__ bool judge(uint64_t s, const uint64_t* p, uint64_t base, uint32_t n, uint32_t k) {
    uint64_t sum = 0;
    for (uint32_t i = 0; i < k; ++i) sum = p[last_le(p, base, n, sum + s)] - base;
    return sum == p[n] - base;
}

// minimal feasible s by a (blockDim+1)-ary search (judge is monotone in s, so this is the value
// the reference's bisection `while (lb + 1 < ub)` converges to), then the greedy boundaries.
__device__ void optimal_offset_block(const uint64_t* p, uint64_t base, uint32_t n, uint32_t k, uint32_t* out,
                                     uint64_t* s_lohi, int* s_first) {
    const uint32_t T = blockDim.x;
    if (threadIdx.x == 0) {
        s_lohi[0] = 0;
        s_lohi[1] = p[n] - base;
    }
    __syncthreads();
    while (true) {
        uint64_t lo = s_lohi[0], hi = s_lohi[1];
        if (lo >= hi) break;
        __syncthreads();
        if (threadIdx.x == 0) *s_first = (int)T;
        __syncthreads();
        uint64_t st = lo + (uint64_t)(((unsigned __int128)(hi - lo) * threadIdx.x) / T);
        if (judge(st, p, base, n, k)) atomicMin(s_first, (int)threadIdx.x);
        __syncthreads();
        if (threadIdx.x == 0) {
            int f = *s_first;
            if (f == (int)T) {
                s_lohi[0] = lo + (uint64_t)(((unsigned __int128)(hi - lo) * (T - 1)) / T) + 1;
            } else {
                s_lohi[1] = lo + (uint64_t)(((unsigned __int128)(hi - lo) * (uint32_t)f) / T);
                if (f > 0) s_lohi[0] = lo + (uint64_t)(((unsigned __int128)(hi - lo) * (uint32_t)(f - 1)) / T) + 1;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        uint64_t ub = s_lohi[1];
        out[0] = 0;
        out[k] = n;
        uint64_t sum = 0;
        for (uint32_t i = 0; i + 1 < k; ++i) {
            uint32_t j = last_le(p, base, n, sum + ub);
            out[i + 1] = j;
            sum = p[j] - base;
        }
    }
    __syncthreads();
}

// one CTA: prefix of the page weights, partition boundaries (in pages), then each partition's
// sub-partition boundaries (core/graph.hpp:774-780, evaluated for every partition)
__global__ void __launch_bounds__(1024) k_cpbt(const uint64_t* __restrict__ pw, uint32_t n, uint32_t P, uint32_t S,
                                                uint64_t* prefix_g, uint32_t* page_off, uint32_t* local_page_off,
                                                int use_smem) {
    extern __shared__ uint64_t s_dyn[];
    __shared__ uint64_t s_warp[32];
    __shared__ uint64_t s_lohi[2];
    __shared__ int s_first;
    uint64_t* prefix = use_smem ? s_dyn : prefix_g;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint64_t running = 0;
    if (threadIdx.x == 0) prefix[0] = 0;
    for (uint32_t c = 0; c < n; c += blockDim.x) {
        uint64_t x = c + threadIdx.x < n ? pw[c + threadIdx.x] : 0;
        uint64_t inc = x;
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) s_warp[warp] = inc;
        __syncthreads();
        uint64_t wb = 0, tot = 0;
        for (int w = 0; w < nw; ++w) {
            if (w < warp) wb += s_warp[w];
            tot += s_warp[w];
        }
        if (c + threadIdx.x < n) prefix[c + threadIdx.x + 1] = running + wb + inc;
        running += tot;
        __syncthreads();
    }
    __syncthreads();
    __shared__ uint32_t s_page_off[kMaxPartitions + 1];
    optimal_offset_block(prefix, 0, n, P, s_page_off, s_lohi, &s_first);
    for (uint32_t i = threadIdx.x; i <= P; i += blockDim.x) page_off[i] = s_page_off[i];
    __syncthreads();
    for (uint32_t p = 0; p < P; ++p) {
        uint32_t pb = s_page_off[p], pe = s_page_off[p + 1];
        uint32_t cnt = pe >= pb ? pe - pb : 0;
        optimal_offset_block(prefix + pb, prefix[pb], cnt, S, local_page_off + (size_t)p * (S + 1), s_lohi, &s_first);
    }
}

// ---- partition bucketing counts for P > 1 (replaces shuffle_edge_list :798-973) --------------
template <int REC>
__global__ void __launch_bounds__(256) k_part_counts(const uint8_t* __restrict__ edges, uint64_t E,
                                                      const uint32_t* __restrict__ poff, int P, uint32_t V,
                                                      uint32_t* cnt_csr, uint32_t* cnt_csc) {
    __shared__ uint32_t s_off[kMaxPartitions + 1];
    for (int i = threadIdx.x; i <= P; i += blockDim.x) s_off[i] = poff[i];
    __syncthreads();
    const uint64_t stride = (uint64_t)V + 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s, d;
        float w;
        load_edge<REC>(edges, i, s, d, w);
        if (cnt_csr) atomicAdd(&cnt_csr[part_of(s_off, P, d) * stride + s], 1u);
        if (cnt_csc) atomicAdd(&cnt_csc[part_of(s_off, P, s) * stride + d], 1u);
    }
}

// ---- counting-sort scatter into both structures ----------------------------------------------
template <int REC>
__global__ void __launch_bounds__(256) k_scatter(const uint8_t* __restrict__ edges, uint64_t E,
                                                  const uint32_t* __restrict__ poff, int P, uint32_t V,
                                                  unsigned long long* csr_off, uint32_t* __restrict__ csr_adj,
                                                  float* __restrict__ csr_w, unsigned long long* csc_off,
                                                  uint32_t* __restrict__ csc_adj, float* __restrict__ csc_w) {
    __shared__ uint32_t s_off[kMaxPartitions + 1];
    for (int i = threadIdx.x; i <= P; i += blockDim.x) s_off[i] = poff[i];
    __syncthreads();
    const uint64_t stride = (uint64_t)V + 1;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s, d;
        float w;
        load_edge<REC>(edges, i, s, d, w);
        if (csr_off) {
            uint64_t key = P == 1 ? s : part_of(s_off, P, d) * stride + s;
            uint64_t pos = atomicAdd(&csr_off[key], ~0ull) - 1ull;
            csr_adj[pos] = d;
            if (REC == 12) csr_w[pos] = w;
        }
        if (csc_off) {
            uint64_t key = P == 1 ? d : part_of(s_off, P, s) * stride + d;
            uint64_t pos = atomicAdd(&csc_off[key], ~0ull) - 1ull;
            csc_adj[pos] = s;
            if (REC == 12) csc_w[pos] = w;
        }
    }
}

// ---- outgoing_adj_bitmap (core/graph.hpp:1304-1352): one warp per 64-bit word ---------------
__global__ void __launch_bounds__(256) k_bitmap(const uint32_t* __restrict__ cnt, uint32_t V, int P,
                                                 uint64_t* __restrict__ bitmap, uint64_t nwords) {
    const int lane = threadIdx.x & 31;
    const uint64_t nwarps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const uint64_t stride = P == 1 ? 0 : (uint64_t)V + 1;
    for (uint64_t wi = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; wi < nwords * (uint64_t)P; wi += nwarps) {
        uint64_t p = wi / nwords, w = wi % nwords;
        uint64_t v0 = w * 64 + lane, v1 = v0 + 32;
        uint32_t c0 = v0 < V ? cnt[p * stride + v0] : 0u;
        uint32_t c1 = v1 < V ? cnt[p * stride + v1] : 0u;
        uint32_t b0 = __ballot_sync(0xffffffffu, c0 > 0);
        uint32_t b1 = __ballot_sync(0xffffffffu, c1 > 0);
        if (lane == 0) bitmap[wi] = ((uint64_t)b1 << 32) | b0;
    }
}

// part_edges[p] = off[p*(V+1)] (after the scatter: start of partition p), part_edges[P] = E
__global__ void k_part_edges(const uint64_t* off, uint32_t V, int P, uint64_t E, uint64_t* out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) out[p] = off[(uint64_t)p * ((uint64_t)V + 1)];
    if (p == P) out[P] = E;
}

// ---------------------------------------------------------------------------------------------
int compute_degrees(eg_graph* g) {
    const uint64_t E = g->E;
    const uint32_t V = g->V;
    EG_TRY(g->outdeg.reserve(sizeof(uint32_t) * (size_t)V));
    EG_TRY(g->indeg.reserve(sizeof(uint32_t) * (size_t)V));
    EG_CUDA(cudaMemsetAsync(g->outdeg.ptr, 0, sizeof(uint32_t) * (size_t)V, g->stream));
    EG_CUDA(cudaMemsetAsync(g->indeg.ptr, 0, sizeof(uint32_t) * (size_t)V, g->stream));
    if (E == 0) return EG_OK;
    Timed t(&g->prof, g->stream, "degrees");
    unsigned grid = grid_for(E, 256, 152u * 16u);
    if (g->edge_bytes == 8)
        k_degrees<8><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->outdeg.as<uint32_t>(), g->indeg.as<uint32_t>());
    else
        k_degrees<12><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->outdeg.as<uint32_t>(), g->indeg.as<uint32_t>());
    EG_CHECK_LAUNCH("k_degrees");
    return EG_OK;
}

int validate_edges(eg_graph* g, uint64_t E) {
    if (E == 0) return EG_OK;
    EG_CUDA(cudaMemsetAsync(g->err.as<int>() + 1, 0, sizeof(int), g->stream));
    unsigned grid = grid_for(E, 256, 152u * 16u);
    if (g->edge_bytes == 8)
        k_validate<8><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->V, g->err.as<int>() + 1);
    else
        k_validate<12><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->V, g->err.as<int>() + 1);
    EG_CHECK_LAUNCH("k_validate");
    int bad = 0;
    EG_CUDA(cudaMemcpyAsync(&bad, g->err.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    if (bad) {
        set_error("edge list holds a vertex id >= V (%u)", g->V);
        return EG_ERR_INVALID;
    }
    return EG_OK;
}

int symmetrize_edges(eg_graph* g, uint64_t E) {
    if (E == 0) return EG_OK;
    unsigned grid = grid_for(E, 256, 152u * 16u);
    Timed t(&g->prof, g->stream, "symmetrize");
    if (g->edge_bytes == 8) k_symmetrize<8><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E);
    else k_symmetrize<12><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E);
    EG_CHECK_LAUNCH("k_symmetrize");
    return EG_OK;
}

// optimal_offset over n device weights for P parts (and S parts inside every part); results in
// page units to host arrays po[P+1], lpo[P*(S+1)].  The weights live in g->tmp64 or elsewhere.
int cpbt_search(eg_graph* g, const uint64_t* d_w, uint32_t n, int P, int S, uint32_t* po, uint32_t* lpo) {
    if (P < 1 || P > kMaxPartitions || S < 1) {
        set_error("CPBT: need 1 <= P <= %d and S >= 1", kMaxPartitions);
        return EG_ERR_INVALID;
    }
    size_t need = sizeof(uint64_t) * ((size_t)n + 1) + sizeof(uint32_t) * ((size_t)P + 1 + (size_t)P * (S + 1)) + 64;
    EG_TRY(g->cpbt_scratch.reserve(need));
    uint64_t* prefix = g->cpbt_scratch.as<uint64_t>();
    uint32_t* page_off = reinterpret_cast<uint32_t*>(prefix + n + 1);
    uint32_t* local_page_off = page_off + P + 1;
    size_t smem = sizeof(uint64_t) * ((size_t)n + 1);
    int use_smem = smem <= 160 * 1024;
    if (use_smem) EG_CUDA(cudaFuncSetAttribute(k_cpbt, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    {
        Timed t(&g->prof, g->stream, "cpbt_search");
        k_cpbt<<<1, 1024, use_smem ? smem : 0, g->stream>>>(d_w, n, (uint32_t)P, (uint32_t)S, prefix, page_off,
                                                             local_page_off, use_smem);
        EG_CHECK_LAUNCH("k_cpbt");
    }
    EG_CUDA(cudaMemcpyAsync(po, page_off, sizeof(uint32_t) * (P + 1), cudaMemcpyDeviceToHost, g->stream));
    if (lpo)
        EG_CUDA(cudaMemcpyAsync(lpo, local_page_off, sizeof(uint32_t) * (size_t)P * (S + 1), cudaMemcpyDeviceToHost,
                                g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    return EG_OK;
}

// CPBT on a device degree array; results to host arrays (P+1 and P*(S+1))
int cpbt_device(eg_graph* g, const uint32_t* d_deg, uint32_t V, int P, int S, uint64_t eta, int T, int dense,
                uint32_t* h_part, uint32_t* h_local) {
    if (P < 1 || P > kMaxPartitions || S < 1) {
        set_error("CPBT: need 1 <= P <= %d and S >= 1", kMaxPartitions);
        return EG_ERR_INVALID;
    }
    uint32_t pages = (uint32_t)(((uint64_t)V + kPageSize - 1) / kPageSize);
    EG_TRY(g->tmp64.reserve(sizeof(uint64_t) * ((size_t)pages + 1)));
    uint64_t* pw = g->tmp64.as<uint64_t>();
    {
        Timed t(&g->prof, g->stream, "cpbt_page_weights");
        if (pages) {
            k_page_weights<<<std::min<uint32_t>(pages, 152u * 8u), 256, 0, g->stream>>>(
                d_deg, V, (uint32_t)(1 + (P - 1) / 16), (uint32_t)(P - 1), dense ? (uint32_t)T : 1u, eta, pw, pages);
            EG_CHECK_LAUNCH("k_page_weights");
        }
    }
    std::vector<uint32_t> po(P + 1), lpo((size_t)P * (S + 1));
    EG_TRY(cpbt_search(g, pw, pages, P, S, po.data(), lpo.data()));
    // boundaries in vertices, with the reference's 32-bit arithmetic (core/graph.hpp:743-749, :774-780)
    h_part[0] = 0;
    h_part[P] = V;
    for (int i = 0; i < P - 1; ++i) h_part[i + 1] = po[i + 1] * kPageSize;
    if (h_local) {
        for (int p = 0; p < P; ++p) {
            uint32_t* lo = h_local + (size_t)p * (S + 1);
            lo[0] = h_part[p];
            lo[S] = h_part[p + 1];
            for (int i = 0; i < S - 1; ++i) lo[i + 1] = lpo[(size_t)p * (S + 1) + i + 1] * kPageSize + h_part[p];
        }
    }
    return EG_OK;
}

int build_structures(eg_graph* g, int want_csr, int want_csc) {
    const uint32_t V = g->V;
    const uint64_t E = g->E;
    const int P = g->partitions, S = g->sub_partitions;
    const uint64_t stride = (uint64_t)V + 1;
    const uint64_t nwords = (uint64_t)V / 64 + 1;
    g->built_csr = g->built_csc = false;
    g->eng.pull_ready = false;

    EG_TRY(compute_degrees(g));
    // assign_vertices: dense (out-degree) weights with T = max_iterations
    g->part_off.assign(P + 1, 0);
    g->local_off.assign((size_t)P * (S + 1), 0);
    EG_TRY(cpbt_device(g, g->outdeg.as<uint32_t>(), V, P, S, g->eta, g->max_iterations, 1, g->part_off.data(),
                       g->local_off.data()));
    std::vector<uint32_t> clamped(P + 1);
    for (int i = 0; i <= P; ++i) clamped[i] = std::min(g->part_off[i], V);
    for (int i = 1; i <= P; ++i) clamped[i] = std::max(clamped[i], clamped[i - 1]);
    EG_TRY(g->d_part_off.reserve(sizeof(uint32_t) * (P + 1)));
    EG_CUDA(cudaMemcpyAsync(g->d_part_off.ptr, clamped.data(), sizeof(uint32_t) * (P + 1), cudaMemcpyHostToDevice,
                            g->stream));

    const uint32_t* cnt_csr = g->outdeg.as<uint32_t>();
    const uint32_t* cnt_csc = g->indeg.as<uint32_t>();
    uint64_t n_scan = P == 1 ? V : P * stride;
    if (P > 1) {
        if (want_csr) {
            EG_TRY(g->cnt_csr.reserve(sizeof(uint32_t) * P * stride));
            EG_CUDA(cudaMemsetAsync(g->cnt_csr.ptr, 0, sizeof(uint32_t) * P * stride, g->stream));
        }
        if (want_csc) {
            EG_TRY(g->cnt_csc.reserve(sizeof(uint32_t) * P * stride));
            EG_CUDA(cudaMemsetAsync(g->cnt_csc.ptr, 0, sizeof(uint32_t) * P * stride, g->stream));
        }
        if (E) {
            Timed t(&g->prof, g->stream, "part_counts");
            unsigned grid = grid_for(E, 256, 152u * 16u);
            uint32_t* a = want_csr ? g->cnt_csr.as<uint32_t>() : nullptr;
            uint32_t* b = want_csc ? g->cnt_csc.as<uint32_t>() : nullptr;
            if (g->edge_bytes == 8)
                k_part_counts<8><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->d_part_off.as<uint32_t>(), P, V, a, b);
            else
                k_part_counts<12><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->d_part_off.as<uint32_t>(), P, V, a, b);
            EG_CHECK_LAUNCH("k_part_counts");
        }
        cnt_csr = g->cnt_csr.as<uint32_t>();
        cnt_csc = g->cnt_csc.as<uint32_t>();
    }
    // offsets: inclusive scans (P == 1: entry V receives the total)
    const size_t off_bytes = sizeof(uint64_t) * (size_t)P * stride;
    if (want_csr) {
        EG_TRY(g->csr_off.reserve(off_bytes));
        EG_TRY(g->csr_adj.reserve(sizeof(uint32_t) * (E + 32)));
        if (g->weighted) EG_TRY(g->csr_w.reserve(sizeof(float) * E));
        EG_TRY(scan_u32_to_u64(g, cnt_csr, n_scan, g->csr_off.as<uint64_t>(),
                               P == 1 ? g->csr_off.as<uint64_t>() + V : nullptr));
    }
    if (want_csc) {
        EG_TRY(g->csc_off.reserve(off_bytes));
        EG_TRY(g->csc_adj.reserve(sizeof(uint32_t) * (E + 32)));
        if (g->weighted) EG_TRY(g->csc_w.reserve(sizeof(float) * E));
        EG_TRY(scan_u32_to_u64(g, cnt_csc, n_scan, g->csc_off.as<uint64_t>(),
                               P == 1 ? g->csc_off.as<uint64_t>() + V : nullptr));
    }
    if (E) {
        Timed t(&g->prof, g->stream, "scatter");
        unsigned grid = grid_for(E, 256, 152u * 16u);
        auto a_off = want_csr ? g->csr_off.as<unsigned long long>() : nullptr;
        auto b_off = want_csc ? g->csc_off.as<unsigned long long>() : nullptr;
        if (g->edge_bytes == 8)
            k_scatter<8><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->d_part_off.as<uint32_t>(), P, V, a_off,
                                                      g->csr_adj.as<uint32_t>(), nullptr, b_off, g->csc_adj.as<uint32_t>(), nullptr);
        else
            k_scatter<12><<<grid, 256, 0, g->stream>>>(g->edges.as<uint8_t>(), E, g->d_part_off.as<uint32_t>(), P, V, a_off,
                                                       g->csr_adj.as<uint32_t>(), g->csr_w.as<float>(), b_off,
                                                       g->csc_adj.as<uint32_t>(), g->csc_w.as<float>());
        EG_CHECK_LAUNCH("k_scatter");
    }
    EG_TRY(g->tmp64.reserve(sizeof(uint64_t) * (size_t)(2 * P + 4)));
    uint64_t* d_small = g->tmp64.as<uint64_t>();
    if (want_csr) {
        EG_TRY(g->csr_bitmap.reserve(sizeof(uint64_t) * nwords * P));
        {
            Timed t(&g->prof, g->stream, "bitmap");
            k_bitmap<<<grid_for(nwords * P * 32, 256, 152u * 32u), 256, 0, g->stream>>>(cnt_csr, V, P, g->csr_bitmap.as<uint64_t>(), nwords);
            EG_CHECK_LAUNCH("k_bitmap");
        }
        g->part_edges_csr.assign(P + 1, 0);
        k_part_edges<<<1, 1024, 0, g->stream>>>(g->csr_off.as<uint64_t>(), V, P, E, d_small);
        EG_CHECK_LAUNCH("k_part_edges");
        EG_CUDA(cudaMemcpyAsync(g->part_edges_csr.data(), d_small, sizeof(uint64_t) * (P + 1), cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
    }
    if (want_csc) {
        uint64_t cap = std::min<uint64_t>(E, (uint64_t)P * V) + P;
        EG_TRY(g->cvert.reserve(sizeof(uint32_t) * cap));
        EG_TRY(g->cidx.reserve(sizeof(uint64_t) * cap));
        EG_CUDA(cudaMemsetAsync(d_small, 0, sizeof(uint64_t) * (P + 1), g->stream));
        EG_TRY(compress_index(g, cnt_csc, P == 1 ? (uint64_t)V + 1 : P * stride, V, g->csc_off.as<uint64_t>(),
                              g->cvert.as<uint32_t>(), g->cidx.as<uint64_t>(), d_small));
        g->cstart.assign(P + 1, 0);
        EG_CUDA(cudaMemcpyAsync(g->cstart.data(), d_small, sizeof(uint64_t) * (P + 1), cudaMemcpyDeviceToHost, g->stream));
        g->part_edges_csc.assign(P + 1, 0);
        k_part_edges<<<1, 1024, 0, g->stream>>>(g->csc_off.as<uint64_t>(), V, P, E, d_small + P + 1);
        EG_CHECK_LAUNCH("k_part_edges");
        EG_CUDA(cudaMemcpyAsync(g->part_edges_csc.data(), d_small + P + 1, sizeof(uint64_t) * (P + 1), cudaMemcpyDeviceToHost,
                                g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        g->ncompressed = g->cstart[P];
    }
    EG_TRY(check_device_error(g, "eg_build"));
    g->built_csr = want_csr != 0;
    g->built_csc = want_csc != 0;
    return EG_OK;
}

}  // namespace eg
