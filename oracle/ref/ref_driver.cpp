/*
 * ref_driver.cpp — C entry points over the reference's OWN engine (core/graph.hpp of
 * leodestiny/EndGraph, compiled unmodified at one rank with the MPI/NUMA stand-ins in this
 * folder and the compile-time fixes listed in oracle/build_ref.sh).  Test oracle and timed CPU
 * baseline only; the product never links it.
 *
 * Load sequence (the reference's load_directed, core/graph.hpp:1358-1373, split so that both
 * structures exist at one rank): in-memory equivalent of preload_graph_file (:1011-1084), then
 * assign_vertices with sparse = false (out-degree, :689-707) and max_iterations defined,
 * shuffle_edge_list(key dst) + prepare_push_mode, then shuffle_edge_list(key src) +
 * prepare_pull_mode (push first: pull frees the aliased edge list, :1239 and :809-813).
 * The analytics restate the toolkits' callbacks (toolkits/{pagerank,bfs,cc,sssp}.cpp) on the
 * reference's process_edges / process_vertices.
 */
#include <stdint.h>
#include <unistd.h>
#include <fcntl.h>
#include <cmath>
#include <functional>
#include <type_traits>

#include "core/graph.hpp"
#include "endgraph_rmat.h"  // eg_mix64, the signature mixing the oracle uses

namespace {

struct Quiet {  // silences the reference's unconditional printf traffic (PRINT_DEBUG_MESSAGES)
    int saved = -1;
    explicit Quiet(bool on) {
        if (!on) return;
        fflush(stdout);
        saved = dup(1);
        int devnull = open("/dev/null", O_WRONLY);
        if (devnull >= 0) { dup2(devnull, 1); close(devnull); }
    }
    ~Quiet() {
        if (saved < 0) return;
        fflush(stdout);
        dup2(saved, 1);
        close(saved);
    }
};

struct Handle {
    int weighted;
    int quiet;
    int symmetric;
    double prep_time;
    void* g;
};

template <typename E>
Graph<E>* make_graph(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t n, uint32_t V,
                     int symmetric, int eta, int max_iterations) {
    Graph<E>* g = new Graph<E>(eta);
    // preload_graph_file (:1011-1084) from memory: one rank reads every edge; symmetric appends
    // the reversed copies and doubles both counts (:1057-1078).
    g->vertices_num = V;
    g->edges_num = n;
    g->read_edges_num = n;
    size_t cap = (symmetric ? 2 : 1) * n;
    g->edge_list = (EdgeType<E>*)numa_alloc_interleaved(sizeof(EdgeType<E>) * (cap ? cap : 1));
#pragma omp parallel for schedule(static)
    for (uint64_t i = 0; i < n; ++i) {
        g->edge_list[i].src = src[i];
        g->edge_list[i].dst = dst[i];
        if (!std::is_same<E, Empty>::value) memcpy((char*)&g->edge_list[i] + 8, &w[i], sizeof(float));
    }
    if (symmetric) {
#pragma omp parallel for schedule(static)
        for (uint64_t i = 0; i < n; ++i) {
            g->edge_list[n + i].src = g->edge_list[i].dst;
            g->edge_list[n + i].dst = g->edge_list[i].src;
            if (!std::is_same<E, Empty>::value)
                memcpy((char*)&g->edge_list[n + i] + 8, (char*)&g->edge_list[i] + 8, sizeof(float));
        }
        g->read_edges_num *= 2;
        g->edges_num *= 2;
    }
    g->max_iterations = max_iterations;
    g->sparse = false;
    g->use_undirected = false;
    return g;
}

// prepare_pull_mode sizes the per-thread dense chunks (tuned_chunks_dense) from `new ULLONG[length]`
// that it never zeroes before `a[cnt] += eta` (core/graph.hpp:1191-1237).  With non-zero heap
// contents the u64 prefix inside optimal_offset can wrap, the chunks then overlap and destinations
// are signalled twice.  Recompute them the way the code evidently intends (a[i] = 0 + eta), which
// is what the reference computes whenever its heap happens to be zeroed.
template <typename E>
void fix_dense_chunks(Graph<E>* g) {
    for (int i = 0; i < g->partitions_num; ++i) {
        for (int s_i = 0; s_i < g->sockets_num; ++s_i) {
            const UINT n = g->compressed_incoming_adj_vertices[s_i];
            const CompressedAdjIndexType* idx = g->compressed_incoming_adj_index[s_i];
            UINT p = 0;
            while (p < n && idx[p].vertex < g->partition_offset[i]) p++;
            const UINT last = p;
            while (p < n && idx[p].vertex < g->partition_offset[i + 1]) p++;
            const UINT length = p - last;
            std::vector<ULLONG> a(length + 1, (ULLONG)g->eta);
            UINT* off = g->optimal_offset(a.data(), length, g->threads_per_socket);
            for (int s_j = 0; s_j < g->threads_per_socket; ++s_j) {
                ThreadState& ts = g->tuned_chunks_dense[i][s_i * g->threads_per_socket + s_j];
                ts.status = WORKING;
                ts.curr = last + off[s_j];
                ts.end = last + off[s_j + 1];
            }
            delete[] off;
        }
    }
}

template <typename E>
double build(Graph<E>* g) {
    double t = -MPI_Wtime();
    g->sparse = false;
    g->assign_vertices();
    g->shuffle_edge_list(g->inter_outgoing_edge_array, g->inter_outgoing_edge_array_size,
                         [](EdgeType<E> e) { return e.dst; });
    g->prepare_push_mode();
    g->shuffle_edge_list(g->inter_incoming_edge_array, g->inter_incoming_edge_array_size,
                         [](EdgeType<E> e) { return e.src; });
    g->prepare_pull_mode();
    t += MPI_Wtime();
    fix_dense_chunks(g);
    return t;
}

template <typename E>
void destroy(Graph<E>* g) {
    size_t V = g->vertices_num;
    for (int s = 0; s < g->sockets_num; ++s) {
        numa_free(g->outgoing_adj_list[s], sizeof(EdgeType<E>) * g->outgoing_edges[s]);
        numa_free(g->incoming_adj_list[s], sizeof(EdgeType<E>) * g->incoming_edges[s]);
        numa_free(g->outgoing_adj_index[s], sizeof(ULLONG) * (V + 1));
        numa_free(g->compressed_incoming_adj_index[s],
                  sizeof(CompressedAdjIndexType) * (g->compressed_incoming_adj_vertices[s] + 1));
        delete g->outgoing_adj_bitmap[s];
    }
    for (int i = 0; i < g->partitions_num; ++i)
        for (int s = 0; s < g->sockets_num; ++s) {
            numa_free(g->send_buffer[i][s]->data, g->send_buffer[i][s]->capacity);
            numa_free(g->recv_buffer[i][s]->data, g->recv_buffer[i][s]->capacity);
        }
    numa_free(g->degree, sizeof(UINT) * V);
    delete g;
}

template <typename T>
T* vertex_array(Graph<Empty>* g) { return g->template alloc_vertex_array<T>(); }

}  // namespace

extern "C" {

int ref_threads() { return numa_num_configured_cpus(); }

/* optimal_offset, core/graph.hpp:597-626, called on a scratch Graph. */
void ref_optimal_offset(const uint64_t* a, uint32_t n, uint32_t k, uint32_t* out) {
    Quiet q(true);
    static Graph<Empty>* g = nullptr;
    if (!g) g = new Graph<Empty>(1);
    std::vector<ULLONG> tmp(a, a + n);
    UINT* off = g->optimal_offset(tmp.data(), n, k);
    memcpy(out, off, sizeof(uint32_t) * (k + 1));
    delete[] off;
}

/* assign_vertices (core/graph.hpp:662-792) for P partitions / S sockets, evaluated once per
 * partition index so that every partition's socket split is returned.  dense_mode selects the
 * out-degree histogram and T = max_iterations; sparse the in-degree histogram and T = 1. */
void ref_cpbt(const uint32_t* src, const uint32_t* dst, uint64_t n, uint32_t V, int P, int S, int eta,
              int max_iterations, int dense_mode, uint32_t* partition_offset, uint32_t* local_offset,
              uint32_t* degree_out) {
    Quiet q(true);
    Graph<Empty>* g = make_graph<Empty>(src, dst, nullptr, n, V, 0, eta, max_iterations);
    g->partitions_num = P;
    g->sockets_num = S;
    g->sparse = !dense_mode;
    for (int p = 0; p < P; ++p) {
        g->partition_idx = p;
        g->assign_vertices();
        if (p == 0) {
            memcpy(partition_offset, g->partition_offset, sizeof(uint32_t) * (P + 1));
            if (degree_out) memcpy(degree_out, g->degree, sizeof(uint32_t) * V);
        }
        memcpy(local_offset + (size_t)p * (S + 1), g->local_partition_offset, sizeof(uint32_t) * (S + 1));
    }
    // edge_list and the per-call arrays are left to process exit (tests only; small graphs).
}

void* ref_create(const uint32_t* src, const uint32_t* dst, const float* w, uint64_t n, uint32_t V,
                 int symmetric, int eta, int max_iterations, int quiet) {
    Quiet q(quiet != 0);
    Handle* h = new Handle();
    h->weighted = w != nullptr;
    h->quiet = quiet;
    h->symmetric = symmetric;
    if (h->weighted) h->g = make_graph<float>(src, dst, w, n, V, symmetric, eta, max_iterations);
    else h->g = make_graph<Empty>(src, dst, nullptr, n, V, symmetric, eta, max_iterations);
    return h;
}

/* CPBT + CSR + CSC; returns seconds spent (the span of split_graph, like prep_time :1367-1371). */
double ref_build(void* hp) {
    Handle* h = (Handle*)hp;
    Quiet q(h->quiet != 0);
    h->prep_time = h->weighted ? build((Graph<float>*)h->g) : build((Graph<Empty>*)h->g);
    return h->prep_time;
}

void ref_destroy(void* hp) {
    Handle* h = (Handle*)hp;
    if (h->weighted) destroy((Graph<float>*)h->g); else destroy((Graph<Empty>*)h->g);
    delete h;
}

uint64_t ref_num_edges(void* hp) {
    Handle* h = (Handle*)hp;
    return h->weighted ? ((Graph<float>*)h->g)->edges_num : ((Graph<Empty>*)h->g)->edges_num;
}

}  // extern "C"

template <typename E>
static void get_structure(Graph<E>* g, uint32_t* degree, uint32_t* partition_offset, uint32_t* csr_src,
                          uint32_t* csr_dst, float* csr_w, uint64_t* csr_index, uint64_t* csr_bitmap,
                          uint32_t* csc_src, uint32_t* csc_dst, float* csc_w, uint32_t* cvert, uint64_t* cidx) {
    size_t V = g->vertices_num;
    if (degree) memcpy(degree, g->degree, sizeof(uint32_t) * V);
    if (partition_offset) memcpy(partition_offset, g->partition_offset, sizeof(uint32_t) * 2);
    for (uint64_t i = 0; csr_src && i < g->outgoing_edges[0]; ++i) {
        EdgeType<E>& e = g->outgoing_adj_list[0][i];
        csr_src[i] = e.src;
        csr_dst[i] = e.dst;
        if (csr_w && !std::is_same<E, Empty>::value) memcpy(&csr_w[i], (char*)&e + 8, sizeof(float));
    }
    if (csr_index) memcpy(csr_index, g->outgoing_adj_index[0], sizeof(uint64_t) * (V + 1));
    if (csr_bitmap) memcpy(csr_bitmap, g->outgoing_adj_bitmap[0]->data, sizeof(uint64_t) * (V / 64 + 1));
    for (uint64_t i = 0; csc_src && i < g->incoming_edges[0]; ++i) {
        EdgeType<E>& e = g->incoming_adj_list[0][i];
        csc_src[i] = e.src;
        csc_dst[i] = e.dst;
        if (csc_w && !std::is_same<E, Empty>::value) memcpy(&csc_w[i], (char*)&e + 8, sizeof(float));
    }
    for (uint32_t i = 0; cvert && i <= g->compressed_incoming_adj_vertices[0]; ++i) {
        cvert[i] = g->compressed_incoming_adj_index[0][i].vertex;
        cidx[i] = g->compressed_incoming_adj_index[0][i].index;
    }
}

// Order-independent signature of every vertex's lists in the reference's own structures:
// hout[v] = sum of mix(dst | wbits<<32) over v's outgoing list, hin[v] likewise over v's
// incoming list (found through the compressed index).  Same mixing as the oracle's list hash.
// outgoing_adj_index is written only at sources and one past them (core/graph.hpp:1329-1353), so
// a list is read only where outgoing_adj_bitmap has the vertex.
template <typename E>
static void list_hashes(Graph<E>* g, uint64_t* hout, uint64_t* hin) {
    const int64_t V = g->vertices_num;
    const ULLONG* oi = g->outgoing_adj_index[0];
    const EdgeType<E>* ol = g->outgoing_adj_list[0];
    BitmapType* bm = g->outgoing_adj_bitmap[0];
    auto wbits = [](const EdgeType<E>& e) -> uint64_t {
        if (std::is_same<E, Empty>::value) return 0;
        uint32_t b;
        memcpy(&b, (const char*)&e + 8, 4);
        return (uint64_t)b << 32;
    };
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < V; ++v) {
        uint64_t acc = 0;
        if (bm->get_bit((UINT)v))
            for (ULLONG e = oi[v]; e < oi[v + 1]; ++e) acc += eg_mix64(ol[e].dst | wbits(ol[e]));
        hout[v] = acc;
        hin[v] = 0;
    }
    const int64_t nc = g->compressed_incoming_adj_vertices[0];
    const CompressedAdjIndexType* ci = g->compressed_incoming_adj_index[0];
    const EdgeType<E>* il = g->incoming_adj_list[0];
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t i = 0; i < nc; ++i) {
        uint64_t acc = 0;
        for (ULLONG e = ci[i].index; e < ci[i + 1].index; ++e) acc += eg_mix64(il[e].src | wbits(il[e]));
        hin[ci[i].vertex] = acc;
    }
}

extern "C" {

void ref_list_hashes(void* hp, uint64_t* hout, uint64_t* hin) {
    Handle* h = (Handle*)hp;
    if (h->weighted) list_hashes((Graph<float>*)h->g, hout, hin);
    else list_hashes((Graph<Empty>*)h->g, hout, hin);
}

/* number of compressed CSC entries including the sentinel (core/graph.hpp:1144-1188) */
uint64_t ref_num_compressed(void* hp) {
    Handle* h = (Handle*)hp;
    return 1 + (h->weighted ? ((Graph<float>*)h->g)->compressed_incoming_adj_vertices[0]
                            : ((Graph<Empty>*)h->g)->compressed_incoming_adj_vertices[0]);
}

void ref_get_structure(void* hp, uint32_t* degree, uint32_t* partition_offset, uint32_t* csr_src,
                       uint32_t* csr_dst, float* csr_w, uint64_t* csr_index, uint64_t* csr_bitmap,
                       uint32_t* csc_src, uint32_t* csc_dst, float* csc_w, uint32_t* cvert, uint64_t* cidx) {
    Handle* h = (Handle*)hp;
    if (h->weighted)
        get_structure((Graph<float>*)h->g, degree, partition_offset, csr_src, csr_dst, csr_w, csr_index,
                      csr_bitmap, csc_src, csc_dst, csc_w, cvert, cidx);
    else
        get_structure((Graph<Empty>*)h->g, degree, partition_offset, csr_src, csr_dst, csr_w, csr_index,
                      csr_bitmap, csc_src, csc_dst, csc_w, cvert, cidx);
}

/* toolkits/pagerank.cpp:26-103 (one compute() call); returns exec seconds, out[V] = curr. */
double ref_pagerank(void* hp, int iterations, double* out) {
    Handle* h = (Handle*)hp;
    Quiet q(h->quiet != 0);
    Graph<Empty>* graph = (Graph<Empty>*)h->g;
    const double d = 0.85;
    graph->use_undirected = false;
    graph->use_iteration = true;
    graph->use_root = false;
    graph->max_iterations = iterations;
    double exec_time = -get_time();
    double* curr = graph->alloc_vertex_array<double>();
    double* next = graph->alloc_vertex_array<double>();
    VertexSubset* active = graph->alloc_vertex_subset();
    active->fill();
    graph->process_vertices<double>(
        [&](UINT vtx) {
            curr[vtx] = (double)1;
            if (graph->degree[vtx] > 0) curr[vtx] /= graph->degree[vtx];
            return (double)1;
        },
        active);
    for (int i_i = 0; i_i < iterations; i_i++) {
        graph->fill_vertex_array(next, (double)0);
        graph->process_edges<int, double>(
            [&](UINT src) { graph->emit(src, curr[src]); },
            [&](UINT src, double msg, AdjacentListType<Empty> outgoing_adj) {
                for (EdgeType<Empty>* ptr = outgoing_adj.begin; ptr != outgoing_adj.end; ptr++)
                    write_add(&next[ptr->dst], msg);
                return 0;
            },
            [&](UINT dst, AdjacentListType<Empty> incoming_adj) {
                double sum = 0;
                for (EdgeType<Empty>* ptr = incoming_adj.begin; ptr != incoming_adj.end; ptr++) sum += curr[ptr->src];
                graph->emit(dst, sum);
            },
            [&](UINT dst, double msg) {
                write_add(&next[dst], msg);
                return 0;
            },
            active);
        if (i_i == iterations - 1) {
            graph->process_vertices<double>(
                [&](UINT vtx) {
                    next[vtx] = 1 - d + d * next[vtx];
                    return 0;
                },
                active);
        } else {
            graph->process_vertices<double>(
                [&](UINT vtx) {
                    next[vtx] = 1 - d + d * next[vtx];
                    if (graph->degree[vtx] > 0) {
                        next[vtx] /= graph->degree[vtx];
                        return fabs(next[vtx] - curr[vtx]) * graph->degree[vtx];
                    }
                    return fabs(next[vtx] - curr[vtx]);
                },
                active);
        }
        std::swap(curr, next);
    }
    exec_time += get_time();
    if (out) memcpy(out, curr, sizeof(double) * graph->vertices_num);
    graph->dealloc_vertex_array(curr);
    graph->dealloc_vertex_array(next);
    delete active;
    return exec_time;
}

/* toolkits/bfs.cpp:22-84; level[v] = iteration that activated v (root 0), parent as the toolkit. */
double ref_bfs(void* hp, uint32_t root, uint32_t* level, uint32_t* parent_out) {
    Handle* h = (Handle*)hp;
    Quiet q(h->quiet != 0);
    Graph<Empty>* graph = (Graph<Empty>*)h->g;
    graph->use_undirected = false;
    graph->use_iteration = false;
    graph->use_root = true;
    double exec_time = -get_time();
    UINT* parent = graph->alloc_vertex_array<UINT>();
    VertexSubset* visited = graph->alloc_vertex_subset();
    VertexSubset* active_in = graph->alloc_vertex_subset();
    VertexSubset* active_out = graph->alloc_vertex_subset();
    visited->clear();
    visited->set_bit(root);
    active_in->clear();
    active_in->set_bit(root);
    graph->fill_vertex_array(parent, graph->vertices_num);
    parent[root] = root;
    if (level) {
        for (UINT v = 0; v < graph->vertices_num; ++v) level[v] = 0xFFFFFFFFu;
        level[root] = 0;
    }
    UINT active_vertices = 1;
    for (int i_i = 0; active_vertices > 0; i_i++) {
        active_out->clear();
        active_vertices = graph->process_edges<UINT, UINT>(
            [&](UINT src) { graph->emit(src, src); },
            [&](UINT src, UINT msg, AdjacentListType<Empty> outgoing_adj) {
                UINT activated = 0;
                for (EdgeType<Empty>* ptr = outgoing_adj.begin; ptr != outgoing_adj.end; ptr++) {
                    UINT dst = ptr->dst;
                    if (parent[dst] == graph->vertices_num && cas(&parent[dst], graph->vertices_num, src)) {
                        active_out->set_bit(dst);
                        activated += 1;
                    }
                }
                return activated;
            },
            [&](UINT dst, AdjacentListType<Empty> incoming_adj) {
                if (visited->get_bit(dst)) return;
                for (EdgeType<Empty>* ptr = incoming_adj.begin; ptr != incoming_adj.end; ptr++) {
                    UINT src = ptr->src;
                    if (active_in->get_bit(src)) {
                        graph->emit(dst, src);
                        break;
                    }
                }
            },
            [&](UINT dst, UINT msg) {
                if (cas(&parent[dst], graph->vertices_num, msg)) {
                    active_out->set_bit(dst);
                    return 1;
                }
                return 0;
            },
            active_in, visited);
        active_vertices = graph->process_vertices<UINT>(
            [&](UINT vtx) {
                visited->set_bit(vtx);
                if (level) level[vtx] = (uint32_t)(i_i + 1);
                return 1;
            },
            active_out);
        std::swap(active_in, active_out);
    }
    exec_time += get_time();
    if (parent_out) memcpy(parent_out, parent, sizeof(UINT) * graph->vertices_num);
    graph->dealloc_vertex_array(parent);
    delete active_in;
    delete active_out;
    delete visited;
    return exec_time;
}

/* toolkits/cc.cpp:22-84 on a graph created with symmetric = 1 */
double ref_cc(void* hp, uint32_t* label_out, int* iterations_out) {
    Handle* h = (Handle*)hp;
    Quiet q(h->quiet != 0);
    Graph<Empty>* graph = (Graph<Empty>*)h->g;
    graph->use_undirected = true;
    graph->use_iteration = false;
    graph->use_root = false;
    double exec_time = -get_time();
    UINT* label = graph->alloc_vertex_array<UINT>();
    VertexSubset* active_in = graph->alloc_vertex_subset();
    active_in->fill();
    VertexSubset* active_out = graph->alloc_vertex_subset();
    UINT active_vertices = graph->process_vertices<UINT>(
        [&](UINT vtx) {
            label[vtx] = vtx;
            return 1;
        },
        active_in);
    int iters = 0;
    for (int i_i = 0; active_vertices > 0; i_i++) {
        active_out->clear();
        active_vertices = graph->process_edges<UINT, UINT>(
            [&](UINT src) { graph->emit(src, label[src]); },
            [&](UINT src, UINT msg, AdjacentListType<Empty> outgoing_adj) {
                UINT activated = 0;
                for (EdgeType<Empty>* ptr = outgoing_adj.begin; ptr != outgoing_adj.end; ptr++) {
                    UINT dst = ptr->dst;
                    if (msg < label[dst]) {
                        write_min(&label[dst], msg);
                        active_out->set_bit(dst);
                        activated += 1;
                    }
                }
                return activated;
            },
            [&](UINT dst, AdjacentListType<Empty> incoming_adj) {
                UINT msg = dst;
                for (EdgeType<Empty>* ptr = incoming_adj.begin; ptr != incoming_adj.end; ptr++) {
                    UINT src = ptr->src;
                    if (label[src] < msg) msg = label[src];
                }
                if (msg < dst) graph->emit(dst, msg);
            },
            [&](UINT dst, UINT msg) {
                if (msg < label[dst]) {
                    write_min(&label[dst], msg);
                    active_out->set_bit(dst);
                    return 1u;
                }
                return 0u;
            },
            active_in);
        std::swap(active_in, active_out);
        iters = i_i + 1;
    }
    exec_time += get_time();
    if (label_out) memcpy(label_out, label, sizeof(UINT) * graph->vertices_num);
    if (iterations_out) *iterations_out = iters;
    graph->dealloc_vertex_array(label);
    delete active_in;
    delete active_out;
    return exec_time;
}

/* toolkits/sssp.cpp:24-84 on a weighted graph */
double ref_sssp(void* hp, uint32_t root, float* dist_out) {
    Handle* h = (Handle*)hp;
    Quiet q(h->quiet != 0);
    typedef float Weight;
    Graph<Weight>* graph = (Graph<Weight>*)h->g;
    graph->use_undirected = false;
    graph->use_iteration = false;
    graph->use_root = true;
    double exec_time = -get_time();
    Weight* distance = graph->alloc_vertex_array<Weight>();
    VertexSubset* active_in = graph->alloc_vertex_subset();
    VertexSubset* active_out = graph->alloc_vertex_subset();
    active_in->clear();
    active_in->set_bit(root);
    graph->fill_vertex_array(distance, (Weight)1e9);
    distance[root] = (Weight)0;
    UINT active_vertices = 1;
    for (int i_i = 0; active_vertices > 0; i_i++) {
        active_out->clear();
        active_vertices = graph->process_edges<UINT, Weight>(
            [&](UINT src) { graph->emit(src, distance[src]); },
            [&](UINT src, Weight msg, AdjacentListType<Weight> outgoing_adj) {
                UINT activated = 0;
                for (EdgeType<Weight>* ptr = outgoing_adj.begin; ptr != outgoing_adj.end; ptr++) {
                    UINT dst = ptr->dst;
                    Weight relax_dist = msg + ptr->edge_data;
                    if (relax_dist < distance[dst]) {
                        if (write_min(&distance[dst], relax_dist)) {
                            active_out->set_bit(dst);
                            activated += 1;
                        }
                    }
                }
                return activated;
            },
            [&](UINT dst, AdjacentListType<Weight> incoming_adj) {
                Weight msg = 1e9;
                for (EdgeType<Weight>* ptr = incoming_adj.begin; ptr != incoming_adj.end; ptr++) {
                    Weight relax_dist = distance[ptr->src] + ptr->edge_data;
                    if (relax_dist < msg) msg = relax_dist;
                }
                if (msg < 1e9) graph->emit(dst, msg);
            },
            [&](UINT dst, Weight msg) {
                if (msg < distance[dst]) {
                    write_min(&distance[dst], msg);
                    active_out->set_bit(dst);
                    return 1;
                }
                return 0;
            },
            active_in);
        std::swap(active_in, active_out);
    }
    exec_time += get_time();
    if (dist_out) memcpy(dist_out, distance, sizeof(Weight) * graph->vertices_num);
    graph->dealloc_vertex_array(distance);
    delete active_in;
    delete active_out;
    return exec_time;
}

}  // extern "C"
