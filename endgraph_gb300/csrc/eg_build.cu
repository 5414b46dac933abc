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
#include <cstddef>
#include <thread>

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
__device__ __forceinline__ void bitmap_words(const uint32_t* __restrict__ cnt, uint32_t V, int P,
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
__global__ void __launch_bounds__(256) k_bitmap(const uint32_t* __restrict__ cnt, uint32_t V, int P,
                                                 uint64_t* __restrict__ bitmap, uint64_t nwords) {
    bitmap_words(cnt, V, P, bitmap, nwords);
}

// part_edges[p] = off[p*(V+1)] (after the scatter: start of partition p), part_edges[P] = E
__global__ void k_part_edges(const uint64_t* off, uint32_t V, int P, uint64_t E, uint64_t* out) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < P) out[p] = off[(uint64_t)p * ((uint64_t)V + 1)];
    if (p == P) out[P] = E;
}

// =============================================================================================
// One-partition build without per-edge global atomics: a counting sort in three passes.
//   A  per-block shared-memory histograms of the bucket (vertex >> shift) of src and of dst
//   B  each block re-reads its edges and writes them bucket by bucket to offsets given by an
//      exclusive scan of A's (bucket, block) counts; the 2 x nb x nblk write frontiers advance
//      sequentially, so L2 merges the scattered record stores into full sectors
//   C  one CTA per bucket: shared-memory degree histogram of the bucket's vertex range, block scan
//      (degrees and offsets written coalesced), then the scatter into the bucket's contiguous
//      output range through shared-memory cursors
// =============================================================================================
constexpr int kBucketThreads = 1024;
constexpr int kBuildThreads = 1024;
constexpr uint32_t kMaxBucketVerts = 32768;  // 128 KiB of shared-memory counters in pass C
constexpr int kBuildUnroll = 4;

// Records holding an id >= V are counted nowhere (pass B skips the same records) and raise *bad:
// a load that uploads and builds in one pipeline validates here instead of in a separate pass.
// One block `blk` of pass A (s_h: 2 nb shared counters)
template <int REC>
__device__ __forceinline__ void bucket_hist_block(const uint8_t* __restrict__ edges, uint64_t E, uint64_t chunk,
                                                  int shift, uint32_t nb, uint32_t nblk, uint32_t* __restrict__ cnt,
                                                  uint32_t V, int* bad, uint32_t blk, uint32_t* s_h) {
    for (uint32_t i = threadIdx.x; i < 2 * nb; i += blockDim.x) s_h[i] = 0;
    __syncthreads();
    const uint64_t e0 = blk * chunk;
    const uint64_t e1 = e0 + chunk < E ? e0 + chunk : E;
    bool out_of_range = false;
    auto count = [&](uint32_t s, uint32_t d) {
        if (s < V && d < V) {
            atomicAdd(&s_h[s >> shift], 1u);
            atomicAdd(&s_h[nb + (d >> shift)], 1u);
        } else {
            out_of_range = true;
        }
    };
    if (REC == 8) {
        // two records per 16-byte load (chunk is even, the buffer is 16-byte aligned)
        const uint4* p = reinterpret_cast<const uint4*>(edges);
        for (uint64_t e = e0 + 2 * threadIdx.x; e < e1; e += 2 * blockDim.x) {
            if (e + 1 < e1) {
                uint4 x = __ldcs(p + e / 2);
                count(x.x, x.y);
                count(x.z, x.w);
            } else {
                uint2 x = reinterpret_cast<const uint2*>(edges)[e];
                count(x.x, x.y);
            }
        }
    } else {
        for (uint64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
            uint32_t s, d;
            float w;
            load_edge<REC>(edges, e, s, d, w);
            count(s, d);
        }
    }
    if (out_of_range) atomicExch(bad, 1);
    __syncthreads();
    // bucket-major layout: [half][bucket][block]
    for (uint32_t i = threadIdx.x; i < 2 * nb; i += blockDim.x) cnt[(uint64_t)i * nblk + blk] = s_h[i];
}

template <int REC>
__global__ void __launch_bounds__(kBucketThreads) k_bucket_hist(const uint8_t* __restrict__ edges, uint64_t E,
                                                                 uint64_t chunk, int shift, uint32_t nb, uint32_t nblk,
                                                                 uint32_t* __restrict__ cnt, uint32_t V, int* bad) {
    extern __shared__ uint32_t s_h[];  // [2][nb]
    bucket_hist_block<REC>(edges, E, chunk, shift, nb, nblk, cnt, V, bad, blockIdx.x, s_h);
}

// in-place exclusive scan of s[0..n) by the whole block; returns the total.  s_warp: 33 words
__device__ uint32_t block_exclusive_scan(uint32_t* s, uint32_t n, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t tsum = 0;
    for (uint32_t j = 0; j < per; ++j)
        if (b0 + j < n) tsum += s[b0 + j];
    uint32_t inc = tsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) s_warp[warp] = inc;
    __syncthreads();
    if (warp == 0) {  // exclusive scan of the warp totals, the block total in s_warp[32]
        const uint32_t x = lane < nw ? s_warp[lane] : 0u;
        uint32_t y = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += z;
        }
        if (lane < nw) s_warp[lane] = y - x;
        if (lane == 31) s_warp[32] = y;
    }
    __syncthreads();
    const uint32_t total = s_warp[32];
    uint32_t run = s_warp[warp] + inc - tsum;
    for (uint32_t j = 0; j < per; ++j) {
        if (b0 + j < n) {
            uint32_t c = s[b0 + j];
            s[b0 + j] = run;
            run += c;
        }
    }
    __syncthreads();
    return total;
}

// B: tiles of scatter_per(REC) x 1024 edges are counting-sorted by bucket in shared memory and then
// stored in that order, so consecutive threads store consecutive addresses of a bucket's run
// (whole sectors instead of one partial sector per record).  The block's running base per bucket
// starts at its exclusive (bucket, block) offset from the scan of pass A.
constexpr int kScatterThreads = 1024;
// 16 records per thread for 8-byte records (128 KiB tile: longer runs per bucket, fewer partial
// sectors), 8 for 12-byte records so that the tile and the bucket tables still fit 200 KiB
__host__ __device__ constexpr int scatter_per(int rec) { return rec == 8 ? 16 : 8; }
__host__ __device__ constexpr int scatter_tile(int rec) { return kScatterThreads * scatter_per(rec); }

// kCheck: skip records with an id >= V as pass A did (an upload validated in pass A); edge lists
// validated at load leave it off
// One block `blk` of pass B (s_raw: the bucket tables and the staging tile)
template <int REC, bool kCheck>
__device__ __forceinline__ void bucket_scatter_block(const uint8_t* __restrict__ edges, uint64_t E, uint64_t chunk,
                                                     int shift, uint32_t nb, uint32_t nblk,
                                                     const uint64_t* __restrict__ excl, uint8_t* __restrict__ out,
                                                     uint32_t V, uint32_t blk, unsigned char* s_raw) {
    constexpr int W = REC / 4;  // words per record
    unsigned long long* s_base = reinterpret_cast<unsigned long long*>(s_raw);  // [2][nb]
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_base + 2 * nb);            // [nb]
    uint32_t* s_stage = reinterpret_cast<uint32_t*>(s_raw + align16(20ull * nb));  // [tile][W]
    __shared__ uint32_t s_warp[33];
    for (uint32_t i = threadIdx.x; i < 2 * nb; i += blockDim.x) s_base[i] = excl[(uint64_t)i * nblk + blk];
    const uint64_t e0 = blk * chunk;
    const uint64_t e1 = e0 + chunk < E ? e0 + chunk : E;
    constexpr int kPer = scatter_per(REC);
    unsigned long long keep;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
    for (uint64_t t0 = e0; t0 < e1; t0 += scatter_tile(REC)) {
        uint32_t rec[kPer][W];
        bool valid[kPer];
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            const uint64_t e = t0 + (uint64_t)j * blockDim.x + threadIdx.x;
            valid[j] = e < e1;
            if (valid[j]) {
                if (W == 2) {
                    const uint2 x = __ldcs(reinterpret_cast<const uint2*>(edges) + e);
                    rec[j][0] = x.x;
                    rec[j][1] = x.y;
                } else {
                    const uint32_t* r = reinterpret_cast<const uint32_t*>(edges + e * REC);
#pragma unroll
                    for (int w = 0; w < W; ++w) rec[j][w] = __ldcs(r + w);
                }
                if (kCheck) valid[j] = rec[j][0] < V && rec[j][1] < V;  // pass A skipped it too
            }
        }
#pragma unroll
        for (int half = 0; half < 2; ++half) {
            for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) s_cnt[i] = 0;
            __syncthreads();
            uint32_t rank[kPer];
#pragma unroll
            for (int j = 0; j < kPer; ++j)
                rank[j] = valid[j] ? atomicAdd(&s_cnt[rec[j][half] >> shift], 1u) : 0u;
            __syncthreads();
            // tile-local exclusive starts; s_cnt keeps the counts in a copy inside s_stage's tail
            const uint32_t n_tile = block_exclusive_scan(s_cnt, nb, s_warp);
#pragma unroll
            for (int j = 0; j < kPer; ++j) {
                if (valid[j]) {
                    const uint32_t slot = s_cnt[rec[j][half] >> shift] + rank[j];
                    if (W == 2) {
                        reinterpret_cast<uint2*>(s_stage)[slot] = make_uint2(rec[j][0], rec[j][1]);
                    } else {
#pragma unroll
                        for (int w = 0; w < W; ++w) s_stage[slot * W + w] = rec[j][w];
                    }
                }
            }
            __syncthreads();
            unsigned long long* base = s_base + (size_t)half * nb;
            for (uint32_t i = threadIdx.x; i < n_tile; i += blockDim.x) {
                const uint32_t* r = s_stage + i * W;
                const uint32_t b = r[half] >> shift;
                const uint64_t pos = base[b] + (i - s_cnt[b]);
                uint32_t* o = reinterpret_cast<uint32_t*>(out + pos * REC);
                if (W == 2) {  // 8-byte records: one 8-byte store, kept in L2 (the next tile's run
                               // of the same bucket completes its partial sectors)
                    const uint2 q = *reinterpret_cast<const uint2*>(r);
                    asm volatile("st.global.L2::cache_hint.v2.u32 [%0], {%1, %2}, %3;" ::"l"(o), "r"(q.x), "r"(q.y),
                                 "l"(keep)
                                 : "memory");
                } else {
#pragma unroll
                    for (int w = 0; w < W; ++w) o[w] = r[w];
                }
            }
            __syncthreads();
            // advance the block's running bases by this tile's counts (start[b+1] - start[b])
            for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) {
                const uint32_t next = b + 1 < nb ? s_cnt[b + 1] : n_tile;
                base[b] += next - s_cnt[b];
            }
            __syncthreads();
        }
    }
}

template <int REC, bool kCheck>
__global__ void __launch_bounds__(kScatterThreads) k_bucket_scatter(const uint8_t* __restrict__ edges, uint64_t E,
                                                                    uint64_t chunk, int shift, uint32_t nb, uint32_t nblk,
                                                                    const uint64_t* __restrict__ excl,
                                                                    uint8_t* __restrict__ out, uint32_t V) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    bucket_scatter_block<REC, kCheck>(edges, E, chunk, shift, nb, nblk, excl, out, V, blockIdx.x, s_raw);
}

// Visit records [r0, r1) of a bucket with several loads in flight per thread.  8-byte records go
// as 16-byte pairs when the buffer is 16-byte aligned (vec); a pair straddling r0 or r1 visits
// only its in-range half.
template <int REC, class F>
__device__ __forceinline__ void for_records(const uint8_t* __restrict__ rec, uint64_t r0, uint64_t r1, bool vec, F f) {
    if (REC == 8 && vec) {
        const uint4* p = reinterpret_cast<const uint4*>(rec);
        const uint64_t q1 = (r1 + 1) / 2;
        for (uint64_t q = r0 / 2 + threadIdx.x; q < q1; q += (uint64_t)blockDim.x * kBuildUnroll) {
            uint4 x[kBuildUnroll];
#pragma unroll
            for (int u = 0; u < kBuildUnroll; ++u) {
                const uint64_t qq = q + (uint64_t)u * blockDim.x;
                if (qq < q1) x[u] = __ldcs(p + qq);
            }
#pragma unroll
            for (int u = 0; u < kBuildUnroll; ++u) {
                const uint64_t r = 2 * (q + (uint64_t)u * blockDim.x);
                if (r < 2 * q1) {
                    if (r >= r0) f(x[u].x, x[u].y, 0u);
                    if (r + 1 < r1) f(x[u].z, x[u].w, 0u);
                }
            }
        }
    } else {
        for (uint64_t r = r0 + threadIdx.x; r < r1; r += (uint64_t)blockDim.x * kBuildUnroll) {
            uint32_t s[kBuildUnroll], d[kBuildUnroll], w[kBuildUnroll];
#pragma unroll
            for (int u = 0; u < kBuildUnroll; ++u) {
                const uint64_t ru = r + (uint64_t)u * blockDim.x;
                if (ru < r1) {
                    const uint32_t* p = reinterpret_cast<const uint32_t*>(rec + ru * REC);
                    s[u] = __ldcs(p);
                    d[u] = __ldcs(p + 1);
                    w[u] = REC == 12 ? __ldcs(p + 2) : 0u;
                }
            }
#pragma unroll
            for (int u = 0; u < kBuildUnroll; ++u)
                if (r + (uint64_t)u * blockDim.x < r1) f(s[u], d[u], w[u]);
        }
    }
}

__device__ __forceinline__ void st_keep_u32(uint32_t* p, uint32_t v, unsigned long long policy) {
    asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(policy) : "memory");
}

// The bucketed records of a build come in K parts (an upload in pieces scatters each piece as it
// lands): part k holds 2 x E_k records from record 2 * e0_k on, bucket-sorted per half, with
// excl[k] its exclusive scan over (half, bucket, block) of nblk[k] blocks (entry 2 * nb * nblk[k]
// the part's total).  Bucket b of half h is the union over k of
// [2 e0_k + excl_k[(h nb + b) nblk_k], 2 e0_k + excl_k[(h nb + b + 1) nblk_k]).
constexpr int kMaxParts = 8;
struct BuildParts {
    int K;
    uint64_t base2[kMaxParts];          // 2 * e0_k
    const uint64_t* excl[kMaxParts];
    uint32_t nblk[kMaxParts];
};

// C: one bucket per CTA iteration (persistent CTAs take buckets from a ticket); s_cnt: LB counters
template <int REC>
__device__ __forceinline__ void bucket_build_loop(const uint8_t* __restrict__ rec, const BuildParts& parts, int half,
                                                  uint32_t nb, uint32_t LB, uint32_t V, uint32_t* __restrict__ deg,
                                                  uint64_t* __restrict__ off, uint32_t* __restrict__ adj,
                                                  float* __restrict__ wout, uint32_t* ticket, uint32_t* s_cnt) {
    const bool vec = REC == 8;  // the bucketed buffer is 16-byte aligned
    const bool key_is_src = half == 0;
    // the 4-byte placement stores land at random positions of the bucket's window: ask L2 to keep
    // those lines so that a partly written sector is usually completed before it is evicted
    unsigned long long keep;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(keep));
    __shared__ uint32_t s_warp[33];
    __shared__ uint32_t s_b;
    __shared__ uint64_t s_lo[kMaxParts], s_hi[kMaxParts];
    __shared__ uint64_t s_r0, s_r1;
    while (true) {
        if (threadIdx.x == 0) s_b = atomicAdd(ticket, 1u);
        __syncthreads();
        const uint32_t b = s_b;
        if (b >= nb) break;
        if (threadIdx.x == 0) {
            uint64_t r0 = 0, len = 0;
            for (int k = 0; k < parts.K; ++k) {
                const uint64_t* ex = parts.excl[k];
                const uint64_t nbk = parts.nblk[k];
                const uint64_t lo = ex[((uint64_t)half * nb + b) * nbk], hi = ex[((uint64_t)half * nb + b + 1) * nbk];
                r0 += lo - ex[(uint64_t)half * nb * nbk];  // this part's records of earlier buckets
                len += hi - lo;
                s_lo[k] = parts.base2[k] + lo;
                s_hi[k] = parts.base2[k] + hi;
            }
            s_r0 = r0;
            s_r1 = r0 + len;
        }
        const uint32_t v0 = b * LB;
        const uint32_t nv = V - v0 < LB ? V - v0 : LB;
        for (uint32_t i = threadIdx.x; i < nv; i += blockDim.x) s_cnt[i] = 0;
        __syncthreads();
        const uint64_t r0 = s_r0, r1 = s_r1;
        for (int k = 0; k < parts.K; ++k)
            for_records<REC>(rec, s_lo[k], s_hi[k], vec, [&](uint32_t s, uint32_t d, uint32_t) {
                atomicAdd(&s_cnt[(key_is_src ? s : d) - v0], 1u);
            });
        __syncthreads();
        // degrees out, then offsets from the block scan
        for (uint32_t i = threadIdx.x; i < nv; i += blockDim.x) deg[v0 + i] = s_cnt[i];
        __syncthreads();
        block_exclusive_scan(s_cnt, nv, s_warp);
        for (uint32_t i = threadIdx.x; i < nv; i += blockDim.x) off[v0 + i] = r0 + s_cnt[i];
        if (threadIdx.x == 0 && v0 + nv == V) off[V] = r1;
        __syncthreads();
        for (int k = 0; k < parts.K; ++k)
            for_records<REC>(rec, s_lo[k], s_hi[k], vec, [&](uint32_t s, uint32_t d, uint32_t wb) {
                const uint64_t pos = r0 + atomicAdd(&s_cnt[(key_is_src ? s : d) - v0], 1u);
                st_keep_u32(adj + pos, key_is_src ? d : s, keep);
                if (REC == 12) st_keep_u32(reinterpret_cast<uint32_t*>(wout) + pos, wb, keep);
            });
        __syncthreads();
    }
}

template <int REC>
__global__ void __launch_bounds__(kBuildThreads) k_bucket_build(const uint8_t* __restrict__ rec, BuildParts parts,
                                                                 int half, uint32_t nb, uint32_t LB, uint32_t V,
                                                                 uint32_t* __restrict__ deg, uint64_t* __restrict__ off,
                                                                 uint32_t* __restrict__ adj, float* __restrict__ wout,
                                                                 uint32_t* ticket) {
    extern __shared__ uint32_t s_cnt[];  // LB counters
    bucket_build_loop<REC>(rec, parts, half, nb, LB, V, deg, off, adj, wout, ticket, s_cnt);
}

struct BucketPlan {
    int shift;
    uint32_t LB, nb, nblk;
    uint64_t chunk;
};

static BucketPlan plan_buckets(uint32_t V, uint64_t E) {
    BucketPlan p;
    uint32_t lb = 256;
    while (lb < kMaxBucketVerts && (uint64_t)lb * 1024 < V) lb <<= 1;  // aim for >= 1024 buckets
    p.LB = lb;
    p.shift = 0;
    while ((1u << p.shift) < lb) ++p.shift;
    p.nb = (uint32_t)(((uint64_t)V + lb - 1) / lb);
    uint64_t want = (E + 65535) / 65536;
    p.nblk = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, 304));
    p.chunk = (E + p.nblk - 1) / p.nblk;
    p.chunk = (p.chunk + 63) & ~63ull;
    p.nblk = (uint32_t)std::max<uint64_t>(1, (E + p.chunk - 1) / p.chunk);
    return p;
}

int scan_exclusive_u32(eg_graph* g, const uint32_t* in, uint64_t n, uint64_t* out);

// the handle's stream waits for part k of an upload (once the uploader has recorded its event)
static int wait_upload_part(eg_graph* g, const UploadParts* up, int k) {
    if (up->issued) {
        while (up->issued->load(std::memory_order_acquire) <= k) {
            if (up->failed && up->failed->load(std::memory_order_acquire)) {
                set_error("eg_load_directed: the upload of part %d stopped", k);
                return EG_ERR_CUDA;
            }
            std::this_thread::yield();
        }
    }
    EG_CUDA(cudaStreamWaitEvent(g->stream, up->ready[k], 0));
    return EG_OK;
}

// up (optional): the records are still being uploaded in parts; part k may be read once up->ready[k]
// has completed.  Passes A and B of each part run as soon as it lands (so the upload of the next
// parts overlaps them) and validate the ids on the way; pass C needs every part.
static int build_single(eg_graph* g, const UploadParts* up) {
    const uint32_t V = g->V;
    const uint64_t E = g->E;
    const int rec = g->edge_bytes;
    EG_TRY(g->outdeg.reserve(sizeof(uint32_t) * (size_t)V));
    EG_TRY(g->indeg.reserve(sizeof(uint32_t) * (size_t)V));
    EG_TRY(g->csr_off.reserve(sizeof(uint64_t) * ((size_t)V + 1)));
    EG_TRY(g->csc_off.reserve(sizeof(uint64_t) * ((size_t)V + 1)));
    EG_TRY(g->csr_adj.reserve(sizeof(uint32_t) * (E + 32)));
    EG_TRY(g->csc_adj.reserve(sizeof(uint32_t) * (E + 32)));
    if (g->weighted) {
        EG_TRY(g->csr_w.reserve(sizeof(float) * (E + 32)));
        EG_TRY(g->csc_w.reserve(sizeof(float) * (E + 32)));
    }
    if (E == 0) {
        EG_CUDA(cudaMemsetAsync(g->outdeg.ptr, 0, sizeof(uint32_t) * (size_t)V, g->stream));
        EG_CUDA(cudaMemsetAsync(g->indeg.ptr, 0, sizeof(uint32_t) * (size_t)V, g->stream));
        EG_CUDA(cudaMemsetAsync(g->csr_off.ptr, 0, sizeof(uint64_t) * ((size_t)V + 1), g->stream));
        EG_CUDA(cudaMemsetAsync(g->csc_off.ptr, 0, sizeof(uint64_t) * ((size_t)V + 1), g->stream));
        return EG_OK;
    }
    const int K = up ? up->K : 1;
    std::vector<uint64_t> e0(K + 1, 0);
    for (int k = 0; k <= K; ++k) e0[k] = up ? up->e0[k] : (k ? E : 0);
    std::vector<BucketPlan> pl(K);
    std::vector<uint64_t> co(K + 1, 0), oo(K + 1, 0);  // count / offset table positions per part
    for (int k = 0; k < K; ++k) {
        pl[k] = plan_buckets(V, e0[k + 1] - e0[k]);
        co[k + 1] = co[k] + 2ull * pl[k].nb * pl[k].nblk;
        oo[k + 1] = oo[k] + 2ull * pl[k].nb * pl[k].nblk + 1;
    }
    const uint32_t nb = pl[0].nb, LB = pl[0].LB;
    const int shift = pl[0].shift;
    EG_TRY(g->bucket_cnt.reserve(sizeof(uint32_t) * co[K]));
    EG_TRY(g->bucket_off.reserve(sizeof(uint64_t) * oo[K]));
    EG_TRY(g->bucketed.reserve((size_t)2 * E * rec + 64));
    EG_TRY(g->scan.counter.reserve(16));
    int* bad = g->err.as<int>() + 1;
    EG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), g->stream));
    const size_t smem_a = sizeof(uint32_t) * 2 * nb;
    const size_t smem_b = align16(20ull * nb) + (size_t)scatter_tile(rec) * rec;  // [2][nb] u64, [nb] u32, tile
    auto scatter_fn = [&]() -> const void* {
        if (rec == 8) return up ? (const void*)k_bucket_scatter<8, true> : (const void*)k_bucket_scatter<8, false>;
        return up ? (const void*)k_bucket_scatter<12, true> : (const void*)k_bucket_scatter<12, false>;
    };
    EG_CUDA(cudaFuncSetAttribute(scatter_fn(), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_b));
    if (rec == 8)
        EG_CUDA(cudaFuncSetAttribute(k_bucket_hist<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_a));
    else
        EG_CUDA(cudaFuncSetAttribute(k_bucket_hist<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_a));
    BuildParts parts{};
    parts.K = K;
    for (int k = 0; k < K; ++k) {
        if (up) EG_TRY(wait_upload_part(g, up, k));
        const uint64_t Ek = e0[k + 1] - e0[k];
        const uint8_t* src = g->edges.as<uint8_t>() + (size_t)e0[k] * rec;
        uint32_t* cnt = g->bucket_cnt.as<uint32_t>() + co[k];
        uint64_t* ex = g->bucket_off.as<uint64_t>() + oo[k];
        uint8_t* out = g->bucketed.as<uint8_t>() + (size_t)2 * e0[k] * rec;
        const BucketPlan& q = pl[k];
        {
            Timed t(&g->prof, g->stream, "bucket_hist");
            if (rec == 8)
                k_bucket_hist<8><<<q.nblk, kBucketThreads, smem_a, g->stream>>>(src, Ek, q.chunk, shift, nb, q.nblk, cnt,
                                                                                 V, bad);
            else
                k_bucket_hist<12><<<q.nblk, kBucketThreads, smem_a, g->stream>>>(src, Ek, q.chunk, shift, nb, q.nblk,
                                                                                  cnt, V, bad);
            EG_CHECK_LAUNCH("k_bucket_hist");
        }
        EG_TRY(scan_exclusive_u32(g, cnt, co[k + 1] - co[k], ex));
        {
            Timed t(&g->prof, g->stream, "bucket_scatter");
            if (rec == 8 && up)
                k_bucket_scatter<8, true><<<q.nblk, kScatterThreads, smem_b, g->stream>>>(src, Ek, q.chunk, shift, nb,
                                                                                          q.nblk, ex, out, V);
            else if (rec == 8)
                k_bucket_scatter<8, false><<<q.nblk, kScatterThreads, smem_b, g->stream>>>(src, Ek, q.chunk, shift, nb,
                                                                                           q.nblk, ex, out, V);
            else if (up)
                k_bucket_scatter<12, true><<<q.nblk, kScatterThreads, smem_b, g->stream>>>(src, Ek, q.chunk, shift, nb,
                                                                                           q.nblk, ex, out, V);
            else
                k_bucket_scatter<12, false><<<q.nblk, kScatterThreads, smem_b, g->stream>>>(src, Ek, q.chunk, shift,
                                                                                            nb, q.nblk, ex, out, V);
            EG_CHECK_LAUNCH("k_bucket_scatter");
        }
        parts.base2[k] = 2 * e0[k];
        parts.excl[k] = ex;
        parts.nblk[k] = q.nblk;
    }
    if (up) {  // an upload validates in pass A: ids >= V stop the build here
        int h = 0;
        EG_CUDA(cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
        EG_CUDA(cudaStreamSynchronize(g->stream));
        if (h) {
            set_error("edge list holds a vertex id >= V (%u)", V);
            return EG_ERR_INVALID;
        }
    }
    const size_t smem_c = sizeof(uint32_t) * LB;
    if (rec == 8) EG_CUDA(cudaFuncSetAttribute(k_bucket_build<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_c));
    else EG_CUDA(cudaFuncSetAttribute(k_bucket_build<12>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_c));
    int per_sm = 1;
    if (rec == 8)
        EG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bucket_build<8>, kBuildThreads, smem_c));
    else
        EG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bucket_build<12>, kBuildThreads, smem_c));
    const unsigned grid = std::min<uint32_t>(nb, (uint32_t)g->num_sms * (uint32_t)std::max(per_sm, 1));
    for (int half = 0; half < 2; ++half) {
        EG_CUDA(cudaMemsetAsync(g->scan.counter.ptr, 0, 4, g->stream));
        Timed t(&g->prof, g->stream, "bucket_build");
        uint32_t* deg = half == 0 ? g->outdeg.as<uint32_t>() : g->indeg.as<uint32_t>();
        uint64_t* off = half == 0 ? g->csr_off.as<uint64_t>() : g->csc_off.as<uint64_t>();
        uint32_t* adj = half == 0 ? g->csr_adj.as<uint32_t>() : g->csc_adj.as<uint32_t>();
        float* w = half == 0 ? g->csr_w.as<float>() : g->csc_w.as<float>();
        if (rec == 8)
            k_bucket_build<8><<<grid, kBuildThreads, smem_c, g->stream>>>(g->bucketed.as<uint8_t>(), parts, half, nb, LB,
                                                                          V, deg, off, adj, w,
                                                                          g->scan.counter.as<uint32_t>());
        else
            k_bucket_build<12><<<grid, kBuildThreads, smem_c, g->stream>>>(g->bucketed.as<uint8_t>(), parts, half, nb,
                                                                           LB, V, deg, off, adj, w,
                                                                           g->scan.counter.as<uint32_t>());
        EG_CHECK_LAUNCH("k_bucket_build");
    }
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
// The one-partition bucketed build in one cooperative launch: every phase of build_single and of
// the index kernels of build_structures, separated by bounded grid barriers (grid_sync_bounded),
// with one 1,024-thread CTA per SM taking pass-A and pass-B blocks by stride, pass-C buckets by
// ticket and the scans as contiguous ranges.  A graph batch's ids are moved to the union first.
constexpr int kPersistBuildMaxCtas = 1024;

struct BuildWords {
    unsigned bar_count, bar_gen;
    int err;              // a bounded barrier wait gave up
    int bad;              // a record holds an id out of range
    uint32_t ticket[2];   // pass-C bucket tickets, per half
    uint64_t cstart[2];   // entry ranges of the compressed index (cstart[1]: entries + sentinel)
    uint64_t tot[kPersistBuildMaxCtas];  // per-CTA sums of a grid scan
};

struct PersistBuildArgs {
    uint8_t* edges;
    uint64_t E;
    uint32_t V;
    const uint64_t* eoff;  // graph batch: record offsets (G + 1), null for one graph
    const uint64_t* voff;  // graph batch: vertex offsets (G + 1)
    uint32_t G;
    uint64_t chunk;
    int shift;
    uint32_t nb, nblk, LB;
    uint32_t* cnt;
    uint64_t* ex;
    uint8_t* bucketed;
    BuildParts parts;
    uint32_t *outdeg, *indeg;
    uint64_t *csr_off, *csc_off;
    uint32_t *csr_adj, *csc_adj;
    float *csr_w, *csc_w;
    uint64_t* bitmap;
    uint64_t nwords;
    uint32_t* cvert;
    uint64_t* cidx;
    BuildWords* w;
};

__device__ __forceinline__ bool build_barrier(BuildWords* w) { return grid_sync_bounded(&w->bar_count, &w->bar_gen, &w->err); }

__device__ __forceinline__ uint64_t block_sum_u64(uint64_t v, uint64_t* s_red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum_u64(v);
    if (lane == 0) s_red[warp] = v;
    __syncthreads();
    if (warp == 0) {
        uint64_t x = lane < (int)(blockDim.x >> 5) ? s_red[lane] : 0ull;
        x = warp_sum_u64(x);
        if (lane == 0) s_red[32] = x;
    }
    __syncthreads();
    const uint64_t r = s_red[32];
    __syncthreads();
    return r;
}

// exclusive prefix of one value per thread over the block; *total: the block's sum
__device__ __forceinline__ uint64_t block_excl_u64(uint64_t v, uint64_t* s_red, uint64_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    uint64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) s_red[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        const uint64_t x = lane < nw ? s_red[lane] : 0ull;
        uint64_t y = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t z = __shfl_up_sync(0xffffffffu, y, o);
            if (lane >= o) y += z;
        }
        if (lane < nw) s_red[lane] = y - x;
        if (lane == 31) s_red[32] = y;
    }
    __syncthreads();
    const uint64_t r = s_red[warp] + inc - v;
    *total = s_red[32];
    __syncthreads();
    return r;
}

// Exclusive scan of n u32 values over the whole grid without look-back: each CTA sums its own
// contiguous range, a grid barrier, then each CTA rescans its range from the sum of the earlier
// ranges and hands every item its exclusive prefix (epi(i, excl, value)).  *total_out (optional)
// gets the sum of all.  False when the barrier gave up.
template <class Load, class Epi>
__device__ bool grid_scan(Load load, Epi epi, uint64_t n, BuildWords* w, uint64_t* total_out) {
    __shared__ uint64_t s_red[33];
    const uint64_t L = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t lo = min(n, (uint64_t)blockIdx.x * L), hi = min(n, lo + L);
    uint64_t sum = 0;
    for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) sum += load(i);
    sum = block_sum_u64(sum, s_red);
    if (threadIdx.x == 0) w->tot[blockIdx.x] = sum;
    if (!build_barrier(w)) return false;
    uint64_t p = 0;
    for (uint32_t c = threadIdx.x; c < blockIdx.x; c += blockDim.x) p += __ldcg(&w->tot[c]);
    p = block_sum_u64(p, s_red);
    if (total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *total_out = p + __ldcg(&w->tot[blockIdx.x]);
    constexpr int kPer = 4;
    for (uint64_t t0 = lo; t0 < hi; t0 += (uint64_t)blockDim.x * kPer) {
        const uint64_t b = t0 + (uint64_t)threadIdx.x * kPer;
        uint32_t v[kPer];
        uint64_t ts = 0;
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            v[j] = b + j < hi ? load(b + j) : 0u;
            ts += v[j];
        }
        uint64_t tile_total;
        uint64_t run = p + block_excl_u64(ts, s_red, &tile_total);
#pragma unroll
        for (int j = 0; j < kPer; ++j) {
            if (b + j < hi) epi(b + j, run, v[j]);
            run += v[j];
        }
        p += tile_total;
    }
    return true;
}

// Union ids of a graph batch: record i of graph k (eoff[k] <= i < eoff[k+1]) gets voff[k] added to
// both ids, once they are checked against the graph's vertex count (*bad otherwise).  Loads and
// stores go to L2 only, so that no SM holds a stale L1 line of the records for the passes that
// read them later in the same launch.
template <int REC>
__device__ void relabel_union(uint8_t* edges, uint64_t E, const uint64_t* __restrict__ eoff,
                              const uint64_t* __restrict__ voff, uint32_t G, int* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    bool out_of_range = false;
    uint32_t lo = 0;  // graph of the previous record of this thread (records only move forward)
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += stride) {
        if (lo + 1 < G && __ldg(eoff + lo + 1) <= i) {
            uint32_t hi = G;  // last graph with eoff <= i, searched in (lo, G)
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (__ldg(eoff + mid) <= i) lo = mid; else hi = mid;
            }
        }
        uint32_t* r = reinterpret_cast<uint32_t*>(edges + i * (uint64_t)REC);
        const uint32_t s = __ldcg(r), d = __ldcg(r + 1);
        const uint64_t base = __ldg(voff + lo), nv = __ldg(voff + lo + 1) - base;
        if (s >= nv || d >= nv) {
            out_of_range = true;
            continue;
        }
        __stcg(r, (uint32_t)(base + s));
        __stcg(r + 1, (uint32_t)(base + d));
    }
    if (out_of_range) atomicExch(bad, 1);
}

template <int REC>
__global__ void __launch_bounds__(kBuildThreads, 1) k_build_persistent(PersistBuildArgs a) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    BuildWords* w = a.w;
    if (a.eoff) {
        relabel_union<REC>(a.edges, a.E, a.eoff, a.voff, a.G, &w->bad);
        if (!build_barrier(w)) return;
    }
    // A: bucket counts per (half, bucket, block)
    for (uint32_t blk = blockIdx.x; blk < a.nblk; blk += gridDim.x) {
        bucket_hist_block<REC>(a.edges, a.E, a.chunk, a.shift, a.nb, a.nblk, a.cnt, a.V, &w->bad, blk,
                               reinterpret_cast<uint32_t*>(s_raw));
        __syncthreads();
    }
    if (!build_barrier(w)) return;
    if (*(volatile int*)&w->bad) return;  // every CTA reads the same flag after the barrier
    const uint64_t ncnt = 2ull * a.nb * a.nblk;
    if (!grid_scan(LoadU32{a.cnt}, EpiExclusive{a.ex}, ncnt, w, a.ex + ncnt)) return;
    if (!build_barrier(w)) return;
    // B: records bucket-sorted per half
    for (uint32_t blk = blockIdx.x; blk < a.nblk; blk += gridDim.x) {
        bucket_scatter_block<REC, false>(a.edges, a.E, a.chunk, a.shift, a.nb, a.nblk, a.ex, a.bucketed, a.V, blk,
                                         s_raw);
        __syncthreads();
    }
    if (!build_barrier(w)) return;
    // C: both halves (independent outputs, no barrier between them)
    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_raw);
    bucket_build_loop<REC>(a.bucketed, a.parts, 0, a.nb, a.LB, a.V, a.outdeg, a.csr_off, a.csr_adj, a.csr_w,
                           &w->ticket[0], s_cnt);
    __syncthreads();  // every thread has read the last ticket of half 0 before thread 0 takes one of half 1
    bucket_build_loop<REC>(a.bucketed, a.parts, 1, a.nb, a.LB, a.V, a.indeg, a.csc_off, a.csc_adj, a.csc_w,
                           &w->ticket[1], s_cnt);
    if (!build_barrier(w)) return;
    // outgoing_adj_bitmap and the compressed incoming index
    bitmap_words(a.outdeg, a.V, 1, a.bitmap, a.nwords);
    grid_scan(LoadFlag{a.indeg, a.V, 1}, EpiCompress{a.csc_off, a.cvert, a.cidx, w->cstart, a.V, 1, a.indeg},
              (uint64_t)a.V + 1, w, nullptr);
}

bool persistent_build_fits(const eg_graph* g) {
    return g->partitions == 1 && g->sub_partitions == 1 && g->E > 0 &&
           align16(20ull * plan_buckets(g->V, g->E).nb) + (uint64_t)scatter_tile(g->edge_bytes) * g->edge_bytes <=
               200ull * 1024;
}

int build_persistent(eg_graph* g, const uint64_t* eoff, const uint64_t* voff, uint32_t G) {
    const uint32_t V = g->V;
    const uint64_t E = g->E;
    const int rec = g->edge_bytes;
    if (!persistent_build_fits(g)) {
        set_error("eg_build: the one-launch build needs one partition, one sub-partition and edges");
        return EG_ERR_UNSUPPORTED;
    }
    g->built_csr = g->built_csc = false;
    g->eng.pull_ready = false;
    g->eng.pr_ready = false;
    const BucketPlan q = plan_buckets(V, E);
    const uint64_t ncnt = 2ull * q.nb * q.nblk;
    const uint64_t nwords = (uint64_t)V / 64 + 1;
    EG_TRY(g->outdeg.reserve(sizeof(uint32_t) * (size_t)V));
    EG_TRY(g->indeg.reserve(sizeof(uint32_t) * (size_t)V));
    EG_TRY(g->csr_off.reserve(sizeof(uint64_t) * ((size_t)V + 1)));
    EG_TRY(g->csc_off.reserve(sizeof(uint64_t) * ((size_t)V + 1)));
    EG_TRY(g->csr_adj.reserve(sizeof(uint32_t) * (E + 32)));
    EG_TRY(g->csc_adj.reserve(sizeof(uint32_t) * (E + 32)));
    if (g->weighted) {
        EG_TRY(g->csr_w.reserve(sizeof(float) * (E + 32)));
        EG_TRY(g->csc_w.reserve(sizeof(float) * (E + 32)));
    }
    EG_TRY(g->bucket_cnt.reserve(sizeof(uint32_t) * ncnt));
    EG_TRY(g->bucket_off.reserve(sizeof(uint64_t) * (ncnt + 1)));
    EG_TRY(g->bucketed.reserve((size_t)2 * E * rec + 64));
    EG_TRY(g->csr_bitmap.reserve(sizeof(uint64_t) * nwords));
    const uint64_t cap = std::min<uint64_t>(E, V) + 1;
    EG_TRY(g->cvert.reserve(sizeof(uint32_t) * cap));
    EG_TRY(g->cidx.reserve(sizeof(uint64_t) * cap));
    EG_TRY(g->build_words.reserve(sizeof(BuildWords)));
    BuildWords* w = g->build_words.as<BuildWords>();
    EG_CUDA(cudaMemsetAsync(w, 0, sizeof(BuildWords), g->stream));

    const size_t smem = std::max({sizeof(uint32_t) * 2 * q.nb, align16(20ull * q.nb) + (size_t)scatter_tile(rec) * rec,
                                  sizeof(uint32_t) * (size_t)q.LB});
    const void* fn = rec == 8 ? (const void*)k_build_persistent<8> : (const void*)k_build_persistent<12>;
    EG_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    EG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBuildThreads, smem));
    const int grid = std::min(g->num_sms * per_sm, kPersistBuildMaxCtas);
    if (grid < 1) {
        set_error("eg_build: the one-launch build does not fit an SM");
        return EG_ERR_UNSUPPORTED;
    }
    PersistBuildArgs a;
    a.edges = g->edges.as<uint8_t>();
    a.E = E;
    a.V = V;
    a.eoff = eoff;
    a.voff = voff;
    a.G = G;
    a.chunk = q.chunk;
    a.shift = q.shift;
    a.nb = q.nb;
    a.nblk = q.nblk;
    a.LB = q.LB;
    a.cnt = g->bucket_cnt.as<uint32_t>();
    a.ex = g->bucket_off.as<uint64_t>();
    a.bucketed = g->bucketed.as<uint8_t>();
    a.parts = BuildParts{};
    a.parts.K = 1;
    a.parts.base2[0] = 0;
    a.parts.excl[0] = a.ex;
    a.parts.nblk[0] = q.nblk;
    a.outdeg = g->outdeg.as<uint32_t>();
    a.indeg = g->indeg.as<uint32_t>();
    a.csr_off = g->csr_off.as<uint64_t>();
    a.csc_off = g->csc_off.as<uint64_t>();
    a.csr_adj = g->csr_adj.as<uint32_t>();
    a.csc_adj = g->csc_adj.as<uint32_t>();
    a.csr_w = g->csr_w.as<float>();
    a.csc_w = g->csc_w.as<float>();
    a.bitmap = g->csr_bitmap.as<uint64_t>();
    a.nwords = nwords;
    a.cvert = g->cvert.as<uint32_t>();
    a.cidx = g->cidx.as<uint64_t>();
    a.w = w;
    void* kargs[] = {&a};
    {
        Timed t(&g->prof, g->stream, "build_persistent");
        EG_CUDA(cudaLaunchCooperativeKernel(fn, dim3((unsigned)grid), dim3(kBuildThreads), kargs, smem, g->stream));
        EG_CHECK_LAUNCH("k_build_persistent");
    }
    BuildWords hw;  // the flags and the index range (the per-CTA sums are not needed)
    EG_CUDA(cudaMemcpyAsync(&hw, w, offsetof(BuildWords, tot), cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    if (hw.err) {
        set_error("eg_build: a bounded grid barrier of the one-launch build gave up");
        return EG_ERR_TIMEOUT;
    }
    if (hw.bad) {
        set_error(eoff ? "eg_load_graph_batch: a record holds a vertex id >= its graph's vertex count"
                       : "edge list holds a vertex id >= V (%u)", V);
        return EG_ERR_INVALID;
    }
    // one partition, one sub-partition: the CPBT boundaries are [0, V]
    g->part_off.assign({0u, V});
    g->local_off.assign({0u, V});
    EG_TRY(g->d_part_off.reserve(sizeof(uint32_t) * 2));
    EG_CUDA(cudaMemcpyAsync(g->d_part_off.ptr, g->part_off.data(), sizeof(uint32_t) * 2, cudaMemcpyHostToDevice, g->stream));
    g->part_edges_csr.assign({0ull, E});
    g->part_edges_csc.assign({0ull, E});
    g->cstart.assign({0ull, hw.cstart[1]});
    g->ncompressed = hw.cstart[1];
    EG_CUDA(cudaStreamSynchronize(g->stream));
    g->built_csr = g->built_csc = true;
    return EG_OK;
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

int build_structures(eg_graph* g, int want_csr, int want_csc, const UploadParts* up) {
    const uint32_t V = g->V;
    const uint64_t E = g->E;
    const int P = g->partitions, S = g->sub_partitions;
    const uint64_t stride = (uint64_t)V + 1;
    const uint64_t nwords = (uint64_t)V / 64 + 1;
    g->built_csr = g->built_csc = false;
    g->eng.pull_ready = false;
    g->eng.pr_ready = false;

    if (g->build_launch && !up && persistent_build_fits(g)) return build_persistent(g, nullptr, nullptr, 0);
    // the bucket tables and a staging tile must fit one CTA's shared memory
    const bool bucketed =
        P == 1 && align16(20ull * plan_buckets(V, E).nb) + (uint64_t)scatter_tile(g->edge_bytes) * g->edge_bytes <=
                      200ull * 1024;
    if (bucketed) {
        // one partition: both structures (and both degree arrays) from the bucketed build
        want_csr = want_csc = 1;
        EG_TRY(build_single(g, up));
    } else {
        if (up) {  // the generic path reads the whole list: wait for every part
            for (int k = 0; k < up->K; ++k) EG_TRY(wait_upload_part(g, up, k));
            EG_TRY(validate_edges(g, E));
        }
        EG_TRY(compute_degrees(g));
    }
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
    // offsets: inclusive scans, then the atomic scatter (generic path, P > 1)
    const size_t off_bytes = sizeof(uint64_t) * (size_t)P * stride;
    if (!bucketed && want_csr) {
        EG_TRY(g->csr_off.reserve(off_bytes));
        EG_TRY(g->csr_adj.reserve(sizeof(uint32_t) * (E + 32)));
        if (g->weighted) EG_TRY(g->csr_w.reserve(sizeof(float) * E));
        EG_TRY(scan_u32_to_u64(g, cnt_csr, n_scan, g->csr_off.as<uint64_t>(),
                               P == 1 ? g->csr_off.as<uint64_t>() + V : nullptr));
    }
    if (!bucketed && want_csc) {
        EG_TRY(g->csc_off.reserve(off_bytes));
        EG_TRY(g->csc_adj.reserve(sizeof(uint32_t) * (E + 32)));
        if (g->weighted) EG_TRY(g->csc_w.reserve(sizeof(float) * E));
        EG_TRY(scan_u32_to_u64(g, cnt_csc, n_scan, g->csc_off.as<uint64_t>(),
                               P == 1 ? g->csc_off.as<uint64_t>() + V : nullptr));
    }
    if (!bucketed && E) {
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
