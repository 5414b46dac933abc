/*
 * endgraph_gb300.h — C ABI of libendgraph_gb300.so: EndGraph preprocessing (CPBT partitioning,
 * two-level CSR/CSC construction) and the Gemini process_edges toolkits on one GB300 GPU.
 *
 * The reference exposes these as the C++ template class Graph<EdgeData> (core/graph.hpp:100) and
 * the toolkits' compute() functions; it has no C ABI.  Each entry point below names the reference
 * interface it replaces.  include/core/graph.hpp re-creates the Graph<EdgeData> surface on top of
 * this ABI.
 *
 * Conventions
 *  - Every function returns an eg_status; eg_last_error() gives the message of the calling
 *    thread's last failure.  Invalid sizes / pointers are rejected before any GPU work.
 *  - A handle owns one graph resident in device memory and one CUDA stream; calls on a handle
 *    are stream-ordered and must be serialised by the caller (handles are not thread-safe).
 *  - `where` arguments say where a caller buffer lives: EG_HOST (pageable or pinned host memory,
 *    copies happen inside the call) or EG_DEVICE (device memory of the handle's GPU).
 *  - Vertex ids are uint32 (UINT, core/type.hpp:26); edge counts and offsets are uint64.
 *  - Edge records are the reference's binary format (core/type.hpp:29-43): packed
 *    {uint32 src, uint32 dst} (8 bytes) or {uint32 src, uint32 dst, float w} (12 bytes).
 */
#ifndef ENDGRAPH_GB300_H
#define ENDGRAPH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum eg_status {
    EG_OK = 0,
    EG_ERR_INVALID = 1,       /* bad argument (size, pointer, id out of range) */
    EG_ERR_CUDA = 2,          /* CUDA runtime error */
    EG_ERR_NOMEM = 3,         /* device or pinned allocation failed */
    EG_ERR_STATE = 4,         /* call out of order (e.g. analytics before eg_build) */
    EG_ERR_TIMEOUT = 5,       /* a bounded device wait gave up; context stays usable */
    EG_ERR_HOST_CALLBACK = 6, /* host std::function callbacks cannot run on the device engine */
    EG_ERR_UNSUPPORTED = 7
} eg_status;

enum { EG_HOST = 0, EG_DEVICE = 1 };

typedef struct eg_graph eg_graph;

typedef struct eg_config {
    uint64_t eta;          /* CPBT coefficient, Graph(int eta) core/graph.hpp:202-212 */
    int32_t partitions;    /* virtual partitions k (MPI world size in the reference), >= 1 */
    int32_t sub_partitions;/* second-level split per partition (sockets_num), >= 1 */
    int32_t max_iterations;/* T of the CPBT page weight (core/graph.hpp:733-738) */
    int32_t device;        /* CUDA device ordinal */
    void* stream;          /* cudaStream_t to run on; NULL: the handle creates its own */
} eg_config;

typedef struct eg_info {
    uint32_t V;
    uint32_t partitions;
    uint64_t E;            /* edges after symmetrisation */
    uint64_t ncompressed;  /* compressed CSC entries incl. one sentinel per partition */
    int32_t weighted;
    int32_t built_csr;
    int32_t built_csc;
    int32_t symmetric;
} eg_info;

/* Device views of the built structures (pointers into the handle's memory; valid until the next
 * load/build or eg_destroy).  Partition p of the CSR holds the edges whose dst it owns, keyed by
 * src (prepare_push_mode core/graph.hpp:1248-1355); partition p of the CSC holds the edges whose
 * src it owns, keyed by dst (prepare_pull_mode :1098-1242). */
typedef struct eg_csr_view {
    const uint64_t* off;     /* [P*(V+1)] absolute edge positions; list (p,v) = [off[p*(V+1)+v], off[p*(V+1)+v+1]) */
    const uint32_t* adj;     /* [E] neighbour (dst) */
    const float* w;          /* [E] or NULL */
    const uint64_t* bitmap;  /* [P*(V/64+1)] outgoing_adj_bitmap: bit u set iff list (p,u) is non-empty */
} eg_csr_view;

typedef struct eg_csc_view {
    const uint64_t* off;     /* [P*(V+1)] dense offsets */
    const uint32_t* adj;     /* [E] neighbour (src) */
    const float* w;          /* [E] or NULL */
    const uint32_t* cvert;   /* [ncompressed] compressed_incoming_adj_index .vertex (sentinel: V) */
    const uint64_t* cidx;    /* [ncompressed] .index (absolute edge position; sentinel: partition end) */
} eg_csc_view;

typedef struct eg_kernel_stat {
    char name[48];
    uint64_t launches;
    double ms;
} eg_kernel_stat;

/* ---- lifetime: Graph(int eta) + init(), core/graph.hpp:202-285 ------------------------------ */
int eg_create(eg_graph** out, const eg_config* cfg);
int eg_destroy(eg_graph* g);
const char* eg_last_error(void);
int eg_version(void);
/* kernels this process has launched through the library (all handles); no reference counterpart */
unsigned long long eg_launch_count(void);
void* eg_stream(eg_graph* g); /* the cudaStream_t all work of g is ordered on */
int eg_sync(eg_graph* g);

/* ---- loading: preload_graph_file core/graph.hpp:1011-1084 --------------------------------- */
/* Copies E records (edge_bytes 8 or 12) into device memory; symmetric appends reversed copies
 * (load_undirected_from_directed, :629-646, :1057-1078).  Ids >= V are rejected (EG_ERR_INVALID). */
int eg_load_edges(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes, int symmetric,
                  int where);

/* The same from a binary edge file (the reference's input format, read whole as preload_graph_file
 * does for one rank, core/graph.hpp:1011-1084): 128 MiB pieces are read by a pool of reader threads
 * into pinned staging buffers while the previous piece is copied to the device.  The file size must be a multiple of
 * edge_bytes. */
int eg_load_file(eg_graph* g, const char* path, uint32_t V, int edge_bytes, int symmetric);
/* load_directed(path, V) in one call: eg_load_file(..., 0) + eg_build(g, 1, 1), with the file read
 * and uploaded in parts while the first build passes consume them (ids validated on the way). */
int eg_load_directed_file(eg_graph* g, const char* path, uint32_t V, int edge_bytes);

/* ---- preprocessing: split_graph core/graph.hpp:981-1009 ---------------------------------- */
/* Degree histogram, CPBT partition (assign_vertices :662-792, dense out-degree weights with
 * T = max_iterations), then the CSR (:1248-1355) and/or CSC (:1098-1242). */
int eg_build(eg_graph* g, int want_csr, int want_csc);
/* load_directed core/graph.hpp:1358-1373 = eg_load_edges + eg_build(1, 1) */
int eg_load_directed(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes, int where);
/* load_undirected_from_directed core/graph.hpp:629-646 */
int eg_load_undirected_from_directed(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes,
                                     int where);

int eg_get_info(eg_graph* g, eg_info* out);
/* partition_offset [P+1] (core/graph.hpp:743-749) and local_partition_offset [P*(S+1)] (:774-780,
 * evaluated for every partition).  Host buffers; either may be NULL. */
int eg_get_partition(eg_graph* g, uint32_t* partition_offset, uint32_t* local_offset);
/* out-degree / in-degree arrays [V] (degree[], core/graph.hpp:689-707); either may be NULL. */
int eg_get_degrees(eg_graph* g, uint32_t* outdeg, uint32_t* indeg, int where);
int eg_get_csr(eg_graph* g, eg_csr_view* out);
int eg_get_csc(eg_graph* g, eg_csc_view* out);
/* Copies of the structures into caller buffers (sizes as in the views; NULL skips an array).
 * The reference hands these out as per-socket arrays: outgoing_adj_index / _list / _bitmap
 * (core/graph.hpp:160-163) and incoming_adj_list + compressed_incoming_adj_index (:158-168). */
int eg_copy_csr(eg_graph* g, uint64_t* off, uint32_t* adj, float* w, uint64_t* bitmap, int where);
int eg_copy_csc(eg_graph* g, uint64_t* off, uint32_t* adj, float* w, uint32_t* cvert, uint64_t* cidx, int where);

/* ---- CPBT on its own: assign_vertices / optimal_offset core/graph.hpp:586-792 ------------- */
/* deg: [V] degrees (where says host or device).  dense selects T = max_iterations. */
int eg_cpbt_partition(const uint32_t* deg, uint32_t V, int P, int S, uint64_t eta, int max_iterations, int dense,
                      int where, uint32_t* partition_offset, uint32_t* local_offset);
/* optimal_offset(a, n, k) core/graph.hpp:597-626 on the GPU; a on the host, offset[k+1] on host. */
int eg_optimal_offset(const uint64_t* a, uint32_t n, uint32_t k, uint32_t* offset);

/* eg_cpbt_partition for callers that cannot allocate device memory.  No counterpart in the
 * reference.  Same boundaries as eg_cpbt_partition, but deg, partition_offset[P+1] and
 * local_offset[P*(S+1)] (may be NULL) are all DEVICE pointers and the work is only enqueued on
 * `stream` (a cudaStream_t; NULL is the legacy default stream).  It calls no cudaMalloc / cudaFree:
 * its scratch is a fixed array inside the library, EG_NOALLOC_SCRATCH_BYTES per GPU, kept until
 * process exit, which caps V, P and S at the limits below (larger requests return EG_ERR_INVALID).
 * The first call on a device looks up that array's device address (again after a device reset
 * replaced the context); make that call before any stream capture.  Calls share the array: calls
 * that overlap on the GPU race and must be serialised. */
#define EG_NOALLOC_MAX_V (1u << 28)
#define EG_NOALLOC_MAX_PARTITIONS 64
#define EG_NOALLOC_MAX_SUB_PARTITIONS 16
#define EG_NOALLOC_SCRATCH_BYTES (((1u << 28) / 4096u) * 16u + 16u * 1024u)
int eg_cpbt_partition_noalloc(const uint32_t* deg, uint32_t V, int P, int S, uint64_t eta, int max_iterations,
                              int dense, uint32_t* partition_offset, uint32_t* local_offset, void* stream);

/* ---- toolkits: process_edges / process_vertices core/graph.hpp:1376-1817 ------------------ */
/* Gemini PageRank (toolkits/pagerank.cpp:26-98): dense pull every iteration, FP32 ranks.
 * out[V] receives the final curr array. */
int eg_pagerank(eg_graph* g, int iterations, float damping, float* out, int where);
/* BFS (toolkits/bfs.cpp:22-84), push.  level[V] (0xFFFFFFFF unreached) and parent[V] (V when
 * unreached; parent[root] = root); either may be NULL.  *reached (may be NULL) = reached count. */
int eg_bfs(eg_graph* g, uint32_t root, uint32_t* level, uint32_t* parent, int where, uint64_t* reached);
/* CC (toolkits/cc.cpp:22-84) on a graph loaded with eg_load_undirected_from_directed: min-label
 * propagation, push/pull switched per iteration on active_edges < E/20 (core/graph.hpp:1484-1491). */
int eg_cc(eg_graph* g, uint32_t* label, int where);
/* SSSP (toolkits/sssp.cpp:24-84), push Bellman-Ford on float weights; unreached = 1e9. */
int eg_sssp(eg_graph* g, uint32_t root, float* dist, int where);

/* Engine options.  EG_OPT_DENSE_DIVISOR: process_edges runs sparse (push) iff the active
 * vertices' out-edges < E / divisor (core/graph.hpp:1484-1491; the reference uses 20).
 * EG_OPT_BFS_DIRECTION: 0 applies that switch to single-root BFS with the toolkit's dense
 * callbacks (toolkits/bfs.cpp:60-76), 1 forces push every level as the reference's use_root flag
 * does (core/graph.hpp:1496-1498), 2 forces pull.  Results are identical in every mode.  The
 * bit-parallel BFS always switches on its union frontier with the same divisor.
 * EG_OPT_CUDA_GRAPH: 1 replays the batched-BFS level loop (eg_msbfs, eg_msbfs_graphs) as one
 * captured CUDA graph of 16 levels, each choosing push or pull on the device from its frontier's
 * out-edges (the same switch as the host loop), instead of one host round trip per level; deeper
 * traversals continue from the host (bit 1, value 1).  Bit 2 (value 2; 3 for both) replays the
 * single-root eg_bfs level loop as one graph with device-side control flow (a WHILE conditional
 * node over the levels, IF conditional nodes for push or pull), up to 4,096 levels per replay;
 * eg_autotune sets bit 1 only. */
enum {
    EG_OPT_BFS_DIRECTION = 1,
    EG_OPT_DENSE_DIVISOR = 2,
    EG_OPT_CUDA_GRAPH = 3,
    EG_OPT_PULL_BLOCKS_PER_SM = 4, /* pull-sweep CTAs per SM, 0 = occupancy limit */
    EG_OPT_BATCH_WIDTH = 5,        /* roots per bit-parallel pass of eg_bfs_many, 1..64 */
    EG_OPT_SSSP_DELTA = 6,         /* eg_sssp near/far step in millionths of a weight unit; 0 = plain
                                      Bellman-Ford sweeps (the reference's order), -1 = automatic
                                      (0.7 x mean weight / mean out-degree; the default) */
    EG_OPT_PR_RELABEL = 7,         /* eg_pagerank gathers through a copy of the CSC source ids
                                      renumbered by out-degree class, high degrees first, so that
                                      the values most gathered share cache lines; the same values
                                      are summed per destination.  1 on, 0 off, -1 automatic (on
                                      for V > 2^22; the default) */
    EG_OPT_MAX_ITERATIONS = 8,     /* T of the CPBT page weight for the next build (the public
                                      max_iterations field of Graph, core/graph.hpp:733-738);
                                      eg_config.max_iterations sets it at creation */
    EG_OPT_BATCH_LAUNCH = 9,       /* batched BFS (eg_msbfs, eg_msbfs_graphs): 1 runs the whole
                                      traversal in one persistent cooperative launch (every level,
                                      with the push/pull switch and the queue lengths on the
                                      device; bounded grid barriers); 0 the host-driven loop or,
                                      with EG_OPT_CUDA_GRAPH, the captured one */
    EG_OPT_BATCH_DIVISOR = 10,     /* the switch of the batched BFS (push iff the union frontier's
                                      out-edges < E / divisor); 0 (the default): EG_OPT_DENSE_DIVISOR */
    EG_OPT_BUILD_LAUNCH = 11       /* the next one-partition, one-sub-partition build from device
                                      records (eg_build, eg_load_graph_batch): 1 runs it as one
                                      persistent cooperative launch (the default: batch id relabel,
                                      the three bucket passes, bitmap and compressed index between
                                      bounded grid barriers); 0: one launch per pass */
};
int eg_set_option(eg_graph* g, int option, int64_t value);

/* ---- batched operators (no reference counterpart: batched forms of the toolkits) ---------- */
/* Bit-parallel BFS from nroots <= 64 roots (toolkits/bfs.cpp semantics per root): levels[n][V]
 * bytes (0xFF unreached; may be NULL), *edges = sum over roots of the out-edges of the vertices
 * each root reaches.  Identical levels to nroots separate eg_bfs calls. */
int eg_msbfs(eg_graph* g, const uint32_t* roots, int nroots, uint8_t* levels, int where, uint64_t* edges);
/* Bellman-Ford from nsources <= 64 sources on a weighted graph (toolkits/sssp.cpp per source):
 * dist[n][V] floats, 1e9 when unreachable; bit-identical to separate eg_sssp calls. */
int eg_sssp_batch(eg_graph* g, const uint32_t* sources, int nsources, float* dist, int where);
/* Load {src, dst} records keeping each record's input index with it, for operators that take
 * per-edge values at call time (eg_ppr*).  Builds CPBT + CSR + CSC like eg_load_directed. */
int eg_load_directed_with_ids(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int where);
/* Personalised PageRank for nseeds <= 64 seeds over the learnable weights w[E] (input edge order):
 * x_0 = e_seed, x_{k+1} = alpha e_seed + (1 - alpha) A^T x_k with A_uv = w_uv / sum_v' w_uv',
 * FP32; out[n][V] = x_iterations.  Graph loaded with eg_load_directed_with_ids. */
int eg_ppr(eg_graph* g, const float* weights, const uint32_t* seeds, int nseeds, float alpha, int iterations,
           float* out, int where);
/* Adjoint of eg_ppr: given dL/dx_iterations (dl_dx[n][V]) writes dL/dw (dl_dw[E], input edge
 * order).  The transposed iteration runs over the CSR; iterates are recomputed from checkpoints
 * stored every ceil(sqrt(iterations)) steps. */
int eg_ppr_backward(eg_graph* g, const float* weights, const uint32_t* seeds, int nseeds, float alpha, int iterations,
                    const float* dl_dx, float* dl_dw, int where);

/* Many independent graphs in one handle: graph i's records are edges[graph_edges[i] ..
 * graph_edges[i+1]) with local ids < graph_vertices[i]; the handle holds their disjoint union (graph
 * i's vertex v is union vertex voff[i] + v) and preprocesses all of them with one build (one launch
 * per build pass for the whole batch).  graph_edges[G+1] and graph_vertices[G] are host arrays. */
int eg_load_graph_batch(eg_graph* g, const void* edges, int edge_bytes, const uint64_t* graph_edges,
                        const uint32_t* graph_vertices, int ngraphs, int where);
/* voff[G+1] and the edge offsets [G+1] of the loaded batch (host arrays; either may be NULL) */
int eg_get_graph_batch(eg_graph* g, uint64_t* vertex_offsets, uint64_t* edge_offsets);
/* Bit-parallel BFS with roots_per_graph <= 64 roots in every graph of the batch (roots[G * n],
 * local ids): levels[V_total][64] bytes, row = union vertex, column = root index, 0xFF unreached. */
int eg_msbfs_graphs(eg_graph* g, const uint32_t* roots, int roots_per_graph, uint8_t* levels, int where,
                    uint64_t* edges);
/* Bellman-Ford with sources_per_graph <= 64 sources in every graph (weighted batch):
 * dist[V_total][64] floats, row = union vertex, column = source index, 1e9 unreachable. */
int eg_sssp_graphs(eg_graph* g, const uint32_t* sources, int sources_per_graph, float* dist, int where);

/* BFS from many roots in bit-parallel passes of the tuned batch width (EG_OPT_BATCH_WIDTH, default
 * 64): levels[nroots][V] bytes (may be NULL), *edges summed over roots. */
int eg_bfs_many(eg_graph* g, const uint32_t* roots, int nroots, uint8_t* levels, int where, uint64_t* edges);

/* Autotuner (no reference counterpart): times candidate settings on the built graph and keeps the
 * fastest — BFS push/pull divisor or push-only, pull-sweep CTAs per SM, CUDA-graph replay of the
 * batched BFS loop, and roots per bit-parallel pass.  sample_roots: host array. */
typedef struct eg_tuning {
    int32_t bfs_direction;      /* EG_OPT_BFS_DIRECTION chosen */
    int32_t dense_divisor;      /* EG_OPT_DENSE_DIVISOR chosen */
    int32_t pull_blocks_per_sm; /* EG_OPT_PULL_BLOCKS_PER_SM chosen (0: occupancy limit) */
    int32_t cuda_graph;         /* EG_OPT_CUDA_GRAPH chosen */
    int32_t batch_width;        /* EG_OPT_BATCH_WIDTH chosen */
    int32_t batch_divisor;      /* EG_OPT_BATCH_DIVISOR chosen */
    double bfs_ms;              /* best single-root BFS time */
    double pull_sweep_ms;       /* best pull-sweep time (one PageRank iteration) */
    double msbfs_ms_per_root;   /* best batched BFS time per root */
} eg_tuning;
int eg_autotune(eg_graph* g, const uint32_t* sample_roots, int nroots, eg_tuning* out);

/* statistics of the last toolkit call: edges traversed, iterations, push / pull iterations */
int eg_last_run(eg_graph* g, uint64_t* edges_processed, int* iterations, int* push_iters, int* pull_iters);

/* ---- synthetic input (no reference counterpart; include/endgraph_rmat.h) ------------------ */
/* Writes E records of the seeded R-MAT stream into device memory (edge_bytes 8 or 12). */
int eg_generate_rmat(void* d_edges, int edge_bytes, uint64_t E, uint32_t V, double a, double b, double c,
                     uint64_t seed, int permute, float w_lo, float w_hi, void* stream);

/* ---- profiling: per-kernel CUDA-event timing on the handle's stream ----------------------- */
int eg_profile_enable(eg_graph* g, int enable);
int eg_profile_reset(eg_graph* g);
/* fills up to cap entries, returns the number of kernels via *count */
int eg_profile_read(eg_graph* g, eg_kernel_stat* out, int cap, int* count);

/* ---- failure handling, exercised without a fault ------------------------------------------- */
/* Every device-side wait of the library is bounded (the reference instead asserts or exits,
 * core/graph.hpp:87,227,764-771).  This call runs the decoupled look-back scan with its first tile
 * withheld, so the wait of the second tile runs out after spin_cap polls (1 .. 2^22).  Returns
 * EG_ERR_TIMEOUT, as any exhausted wait does, and leaves the handle and its context usable. */
int eg_selftest_bounded_wait(eg_graph* g, uint32_t spin_cap);
/* The grid barrier of the persistent launches (the one-launch build, the persistent batched BFS)
 * is bounded the same way: this call makes a cooperative launch in which one CTA never arrives,
 * so the others give up after spin_cap polls (1 .. 2^22).  Returns EG_ERR_TIMEOUT and leaves the
 * handle and its context usable. */
int eg_selftest_grid_barrier(eg_graph* g, uint32_t spin_cap);

#ifdef __cplusplus
}
#endif

#endif /* ENDGRAPH_GB300_H */
