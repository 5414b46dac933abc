// eg_common.cuh — shared internals of libendgraph_gb300: status handling, device buffers,
// the graph handle, per-kernel CUDA-event profiling, and small device helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <map>
#include <string>
#include <vector>

#include "../../include/endgraph_gb300.h"

namespace eg {

constexpr uint32_t kPageSize = 4096;  // vertices per CPBT page (core/constants.hpp:21)
constexpr int kMaxPartitions = 1024;  // virtual partitions on one GPU

// ---------------------------------------------------------------------------------------------
// status
void set_error(const char* fmt, ...);
const char* error_text();
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define EG_CUDA(call)                                                          \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) return ::eg::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

// every kernel launch of the library is followed by this check, which also counts it
#define EG_CHECK_LAUNCH(name)                                                  \
    do {                                                                       \
        ::eg::g_launches.fetch_add(1, std::memory_order_relaxed);              \
        cudaError_t e_ = cudaGetLastError();                                   \
        if (e_ != cudaSuccess) return ::eg::cuda_fail(e_, name, __FILE__, __LINE__); \
    } while (0)

extern std::atomic<unsigned long long> g_launches;

#define EG_TRY(expr)                                                           \
    do {                                                                       \
        int s_ = (expr);                                                       \
        if (s_ != EG_OK) return s_;                                            \
    } while (0)

// ---------------------------------------------------------------------------------------------
// device memory: one owning buffer type; grows, never shrinks unless released
struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    int reserve(size_t n);  // ensure capacity >= n bytes (contents not preserved)
    void release();
    template <typename T> T* as() const { return static_cast<T*>(ptr); }
};

// ---------------------------------------------------------------------------------------------
// per-kernel timing with CUDA events on the handle's stream
struct KernelStat {
    uint64_t launches = 0;
    double ms = 0;
};

struct Profiler {
    bool enabled = false;
    struct Pending {
        std::string name;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    std::map<std::string, KernelStat> stats;
    cudaEvent_t get();
    void begin(cudaStream_t s, const char* name);
    void end(cudaStream_t s);
    void collect();  // synchronises pending events into stats
    void clear();
    ~Profiler();
};

// RAII launch bracket: records events around a launch when profiling is on
struct Timed {
    Profiler* p;
    cudaStream_t s;
    Timed(Profiler* prof, cudaStream_t st, const char* name) : p(prof), s(st) {
        if (p && p->enabled) p->begin(s, name);
    }
    ~Timed() {
        if (p && p->enabled) p->end(s);
    }
};

// ---------------------------------------------------------------------------------------------
// scan (decoupled look-back) scratch
struct ScanScratch {
    DevBuf desc;     // u64 per tile
    DevBuf counter;  // u32 tile ticket + i32 error flag
};

// engine scratch
struct EngineState {
    DevBuf q0, q1;         // frontier queues (u32 vertex ids)
    DevBuf qdeg;           // u64 prefix of frontier item degrees
    DevBuf chunk_item;     // u32 first item per edge chunk
    DevBuf bm_visit, bm_next, bm_front;  // bitmaps (u64 words)
    DevBuf counters;       // u64 small device counters
    DevBuf acc;            // float / u32 per-vertex accumulator for split items
    DevBuf vals0, vals1;   // per-vertex values
    DevBuf pull_chunk_item;  // u32 per CSC chunk: first compressed item
    DevBuf pull_split;     // u32 list of vertices whose list spans a chunk boundary
    DevBuf bu_seg;         // u64 segments of the early-exit dense BFS step
    DevBuf pr_new_id;      // u32 per vertex: position in out-degree-class order (PageRank gathers)
    DevBuf pr_adj;         // u32 per CSC edge: the source renumbered through pr_new_id
    DevBuf pr_cnt, pr_off; // class counts per vertex tile and their exclusive scan
    uint64_t pull_nsplit = 0;
    uint64_t pull_nchunks = 0;
    bool pull_ready = false;
    bool pr_ready = false;  // pr_new_id / pr_adj match the built CSC
    uint64_t* host_words = nullptr;  // pinned host block (256 bytes) for the readbacks of counters
    // single-root BFS replayed as a CUDA graph (eg_engine.cu): the instantiated graph, its state
    // words on the device and what it was built for
    cudaGraphExec_t bfs_exec = nullptr;
    cudaGraph_t bfs_graph = nullptr;
    std::vector<uint64_t> bfs_key;
    DevBuf bfs_state;
};

}  // namespace eg

// the opaque handle of the C ABI
struct eg_graph {
    int device = 0;
    int num_sms = 152;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // construction parameters (Graph(int eta), toolkit flags)
    uint64_t eta = 1;
    int partitions = 1;
    int sub_partitions = 1;
    int max_iterations = 20;
    // loaded edge list
    uint32_t V = 0;
    uint64_t E = 0;       // edges after symmetrisation
    int weighted = 0;
    int symmetric = 0;
    eg::DevBuf edges;     // packed records as loaded (8 or 12 bytes each)
    int edge_bytes = 8;
    // degrees (u32 V)
    eg::DevBuf outdeg, indeg;
    // CPBT
    std::vector<uint32_t> part_off;   // P+1
    std::vector<uint32_t> local_off;  // P*(S+1)
    eg::DevBuf d_part_off;            // P+1 clamped (monotone) copy on device
    bool built_csr = false, built_csc = false;
    // partition counts for P > 1 (u32 P*(V+1))
    eg::DevBuf cnt_csr, cnt_csc;
    // CSR: P*(V+1) u64 offsets, E u32 dst, E f32 w, P*nwords u64 bitmap
    eg::DevBuf csr_off, csr_adj, csr_w, csr_bitmap;
    // CSC: offsets, src, w, compressed (vertex u32, index u64)
    eg::DevBuf csc_off, csc_adj, csc_w, cvert, cidx;
    uint64_t ncompressed = 0;
    std::vector<uint64_t> cstart;  // P+1 entry ranges of the compressed index
    std::vector<uint64_t> part_edges_csr, part_edges_csc;  // P+1 edge ranges
    // scratch
    eg::ScanScratch scan;
    eg::DevBuf tmp64;  // generic u64 scratch
    eg::DevBuf cpbt_scratch;
    eg::DevBuf bucket_cnt, bucket_off, bucketed;  // one-partition bucketed build
    eg::DevBuf build_words;  // barrier, tickets and flags of the one-launch build
    eg::DevBuf err;    // device error flags (int)
    eg::EngineState eng;
    eg::Profiler prof;
    // pinned staging for host inputs
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    // pipelined host loads: the upload stream, its per-part events and the gate on prior work
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t part_ready[8] = {};
    cudaEvent_t copy_gate = nullptr;
    int pageable_direct = -1;  // the device reads pageable host memory at the link's rate (-1: not asked yet)
    // batched operators (eg_batch.cu): opaque state, dropped at every load/build
    void* batch = nullptr;
    bool edge_ids = false;   // the weight slot of each record holds the record's input index
    uint64_t E_input = 0;    // records as loaded (before symmetrisation)
    // engine options (eg_set_option)
    int bfs_direction = 0;  // 0: Gemini threshold switch, 1: push only, 2: pull only
    int dense_div = 20;     // sparse iff active_edges < E / dense_div (core/graph.hpp:1491)
    int use_cuda_graph = 0; // bit 0: batched BFS level loop as a captured graph; bit 1: single-root BFS
    int batch_launch = 0;   // batched BFS: 1 runs every level inside one persistent launch
    int batch_div = 0;      // batched BFS switch divisor; 0: the same as dense_div
    int build_launch = 1;   // 1: a one-partition build runs as one persistent cooperative launch
    int pull_blocks_per_sm = 0;  // pull-sweep grid; 0 = occupancy limit
    int batch_width = 64;        // roots per bit-parallel pass (eg_bfs_many)
    int pr_relabel = -1;         // PageRank gathers through renumbered sources: 1 on, 0 off, -1 automatic
    int64_t sssp_delta = -1;     // SSSP near/far step in millionths; 0 = Bellman-Ford, -1 = automatic
    // many small graphs in one handle (eg_load_graph_batch): per-graph vertex / edge offsets
    std::vector<uint64_t> batch_voff, batch_eoff;
    eg::DevBuf d_batch_voff;
    // last operator statistics
    uint64_t last_edges_processed = 0;
    int last_iterations = 0;
    int last_pushes = 0, last_pulls = 0;
};

namespace eg {
// ---------------------------------------------------------------------------------------------
// internal entry points shared between translation units
int scan_u32_to_u64(eg_graph* g, const uint32_t* in, uint64_t n, uint64_t* out_incl, uint64_t* total_dev);
int compress_index(eg_graph* g, const uint32_t* cnt, uint64_t n, uint32_t V, const uint64_t* off,
                   uint32_t* cvert, uint64_t* cidx, uint64_t* count_dev);
// records uploaded in parts on another stream: part k = records [e0[k], e0[k+1]) is resident once
// ready[k] has completed
// ready[k]: an upload thread that records the events as it goes publishes how many are recorded
// in *issued (null: all recorded up front) and raises *failed if it stops early
struct UploadParts {
    int K;
    uint64_t e0[9];
    cudaEvent_t ready[8];
    const std::atomic<int>* issued = nullptr;
    const std::atomic<bool>* failed = nullptr;
};
int build_structures(eg_graph* g, int want_csr, int want_csc, const UploadParts* up = nullptr);
// the one-partition, one-sub-partition build as one cooperative launch; eoff / voff (device, G + 1
// entries each, optional): a graph batch whose ids are moved to the union inside the launch
bool persistent_build_fits(const eg_graph* g);
int build_persistent(eg_graph* g, const uint64_t* eoff, const uint64_t* voff, uint32_t G);
// eg_load_directed of host records from this many records on: upload and build pipelined
constexpr uint64_t kPipelinedLoadMin = 1ull << 22;
int load_build_pipelined(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes);
int load_build_file(eg_graph* g, const char* path, uint32_t V, int edge_bytes);
int compute_degrees(eg_graph* g);
int cpbt_device(eg_graph* g, const uint32_t* d_deg, uint32_t V, int P, int S, uint64_t eta, int T, int dense,
                uint32_t* h_part, uint32_t* h_local);
int cpbt_search(eg_graph* g, const uint64_t* d_w, uint32_t n, int P, int S, uint32_t* po, uint32_t* lpo);
int check_device_error(eg_graph* g, const char* what);
int selftest_bounded_wait(eg_graph* g, uint32_t spin_cap);
int selftest_grid_barrier(eg_graph* g, uint32_t spin_cap);
int validate_edges(eg_graph* g, uint64_t E);
int symmetrize_edges(eg_graph* g, uint64_t E);
int run_pagerank(eg_graph* g, int iterations, float damping, float* out, int where);
// renumbering of the CSC sources by out-degree class (eng.pr_new_id / eng.pr_adj), built once per
// structure build and shared by the PageRank and bit-parallel BFS pull gathers
bool want_relabel(const eg_graph* g);
int setup_relabel(eg_graph* g);
int run_bfs(eg_graph* g, uint32_t root, uint32_t* level, uint32_t* parent, int where, uint64_t* reached);
int run_sssp(eg_graph* g, uint32_t root, float* dist, int where);
int run_cc(eg_graph* g, uint32_t* label, int where);
int run_msbfs(eg_graph* g, const uint32_t* roots, int n, uint8_t* levels, int where, uint64_t* edges);
int run_ppr(eg_graph* g, const float* w_in, const uint32_t* seeds, int n, float alpha, int K, float* out, int where);
int run_ppr_backward(eg_graph* g, const float* w_in, const uint32_t* seeds, int n, float alpha, int K,
                     const float* dl_dx, float* dl_dw, int where);
int run_sssp_batch(eg_graph* g, const uint32_t* srcs, int n, float* out, int where);
void free_batch_state(eg_graph* g);
int load_edges_impl(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes, int symmetric, int where,
                    bool validate);
int load_file_impl(eg_graph* g, const char* path, uint32_t V, int edge_bytes, int symmetric);
int load_graph_batch(eg_graph* g, const void* edges, int rec, const uint64_t* eoff, const uint32_t* nverts, int G,
                     int where);
int run_msbfs_graphs(eg_graph* g, const uint32_t* roots, int nper, uint8_t* levels, int where, uint64_t* edges);
int run_sssp_graphs(eg_graph* g, const uint32_t* sources, int nper, float* dist, int where);
int expand_with_ids(eg_graph* g, const uint8_t* rec8_dev, uint64_t E);

// Bounded grid barrier of a cooperative launch (every CTA resident).  count and gen start at zero;
// the last CTA to arrive resets count and advances gen, the others poll gen.  A poll that runs
// past kBarrierSpinCap, or that sees *err already raised by another CTA, raises *err and returns
// false: the caller leaves the kernel, so no CTA waits forever on one that left.
constexpr uint32_t kBarrierSpinCap = 1u << 22;
__device__ __forceinline__ bool grid_sync_bounded(unsigned* count, unsigned* gen, int* err,
                                                  uint32_t spin_cap = kBarrierSpinCap) {
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        const unsigned nblocks = gridDim.x;
        const unsigned g0 = *(volatile unsigned*)gen;
        __threadfence();
        int ok = 1;
        if (atomicAdd(count, 1u) == nblocks - 1) {
            atomicExch(count, 0u);
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            uint32_t spins = 0;
            while (*(volatile unsigned*)gen == g0) {
                if (++spins > spin_cap || *(volatile int*)err) {
                    atomicExch(err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// the push/pull switch of the batched traversals: sparse iff the frontier's out-edges < E / this
inline int batch_divisor(const eg_graph* g) { return g->batch_div > 0 ? g->batch_div : g->dense_div; }

// device helpers
__device__ __forceinline__ uint32_t part_of(const uint32_t* __restrict__ off, int P, uint32_t v) {
    // off: P+1 clamped monotone offsets; last index i with off[i] <= v (v < off[P] = V)
    int lo = 0, hi = P;  // answer in [0, P)
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (off[mid] <= v) lo = mid; else hi = mid;
    }
    return (uint32_t)lo;
}

inline unsigned grid_for(uint64_t n, unsigned block, unsigned cap = 152u * 64u) {
    uint64_t g = (n + block - 1) / block;
    if (g == 0) g = 1;
    return (unsigned)(g < cap ? g : cap);
}

}  // namespace eg
