// The four reference toolkits (toolkits/{pagerank,bfs,cc,sssp}.cpp) written against the device
// operator API of endgraph_gb300_engine.cuh, in the reference's own shape: signal/slot pairs passed
// to process_edges, vertex updates through process_vertices, the same iteration structure.
//
//   engine_toolkits pagerank|bfs|cc|sssp <edge file> <V> <iterations|root> <out file> [partitions]
//
// Writes the result array (double ranks, u32 levels + u32 parents, u32 labels, f32 distances)
// to <out file> for the test to compare with the oracle.
#include <stdio.h>
#include <stdlib.h>

#include <string>
#include <vector>

#include "endgraph_gb300_engine.cuh"

using eg::engine::Engine;
using eg::engine::Mode;
using eg::engine::Subset;

// ---- PageRank, toolkits/pagerank.cpp:26-132 (FP64 ranks like the reference) --------------------
struct PrEdges {
    using Msg = double;
    using Acc = double;
    using R = int;
    const double* curr;
    double* next;
    __device__ bool sparse_signal(uint32_t, double&) const { return false; }
    __device__ int sparse_slot(uint32_t, const double&, uint32_t, float) const { return 0; }
    __device__ bool dense_active(uint32_t) const { return true; }
    __device__ double dense_identity() const { return 0.0; }
    __device__ double dense_signal(uint32_t src, float) const { return curr[src]; }
    __device__ double dense_combine(double a, double b) const { return a + b; }
    // write_add (toolkits/pagerank.cpp:91-94): with several partitions the partials of one
    // destination arrive as separate messages
    __device__ int dense_slot(uint32_t dst, double sum) const {
        atomicAdd(next + dst, sum);
        return 0;
    }
};
struct PrApply {  // next = 1 - d + d * next, divided by the out-degree except in the last iteration
    double* next;
    const uint32_t* deg;
    double d;
    int last;
    __device__ double operator()(uint32_t v) const {
        double x = 1.0 - d + d * next[v];
        if (!last && deg[v] > 0) x /= (double)deg[v];
        next[v] = x;
        return 0.0;
    }
};
struct PrInit {
    double* curr;
    const uint32_t* deg;
    __device__ double operator()(uint32_t v) const {
        curr[v] = deg[v] > 0 ? 1.0 / (double)deg[v] : 1.0;
        return 0.0;
    }
};
struct Zero {
    double* a;
    __device__ double operator()(uint32_t v) const {
        a[v] = 0.0;
        return 0.0;
    }
};

// ---- BFS, toolkits/bfs.cpp:22-112 ------------------------------------------------------------
// visited is the dense_selective subset (bfs.cpp passes it to process_edges): the dense signals of
// every partition skip visited destinations; the slots claim a parent with cas, so the first of
// several partials wins
struct BfsEdges {
    using Msg = uint32_t;
    using Acc = uint32_t;
    using R = unsigned int;
    uint32_t* parent;
    uint32_t V;
    Subset active_in, active_out, visited;
    __device__ bool sparse_signal(uint32_t v, uint32_t& msg) const {
        msg = v;
        return true;
    }
    __device__ unsigned sparse_slot(uint32_t, const uint32_t& src, uint32_t dst, float) const {
        if (__ldcg(parent + dst) == V && atomicCAS(parent + dst, V, src) == V) {
            active_out.set_bit(dst);
            return 1u;
        }
        return 0u;
    }
    __device__ bool dense_active(uint32_t dst) const { return !visited.get_bit(dst); }
    __device__ uint32_t dense_identity() const { return 0xFFFFFFFFu; }
    __device__ uint32_t dense_signal(uint32_t src, float) const { return active_in.get_bit(src) ? src : 0xFFFFFFFFu; }
    __device__ uint32_t dense_combine(uint32_t a, uint32_t b) const { return a < b ? a : b; }
    __device__ unsigned dense_slot(uint32_t dst, uint32_t src) const {
        if (src == 0xFFFFFFFFu) return 0u;
        if (atomicCAS(parent + dst, V, src) == V) {
            active_out.set_bit(dst);
            return 1u;
        }
        return 0u;
    }
};
struct BfsVisit {  // bfs.cpp:77-84: mark the new frontier visited and record its level
    Subset visited;
    uint32_t* level;
    uint32_t lvl;
    __device__ unsigned operator()(uint32_t v) const {
        visited.set_bit(v);
        level[v] = lvl;
        return 1u;
    }
};

// ---- CC, toolkits/cc.cpp:22-112: min-label propagation, push/pull switched on E/20 ----------------
struct CcEdges {
    using Msg = uint32_t;
    using Acc = uint32_t;
    using R = unsigned int;
    uint32_t* label;
    Subset active_out;
    __device__ bool sparse_signal(uint32_t v, uint32_t& msg) const {
        msg = __ldcg(label + v);
        return true;
    }
    __device__ unsigned sparse_slot(uint32_t, const uint32_t& msg, uint32_t dst, float) const {
        if (msg < __ldcg(label + dst) && msg < atomicMin(label + dst, msg)) {
            active_out.set_bit(dst);
            return 1u;
        }
        return 0u;
    }
    // the reference's dense_signal starts from msg = dst and emits only when an in-neighbour's
    // label is smaller (toolkits/cc.cpp:61-71)
    __device__ bool dense_active(uint32_t) const { return true; }
    __device__ uint32_t dense_identity() const { return 0xFFFFFFFFu; }
    __device__ uint32_t dense_signal(uint32_t src, float) const { return __ldcg(label + src); }
    __device__ uint32_t dense_combine(uint32_t a, uint32_t b) const { return a < b ? a : b; }
    __device__ unsigned dense_slot(uint32_t dst, uint32_t m) const {
        const uint32_t msg = m < dst ? m : dst;
        if (!(msg < dst)) return 0u;
        if (msg < __ldcg(label + dst) && msg < atomicMin(label + dst, msg)) {
            active_out.set_bit(dst);
            return 1u;
        }
        return 0u;
    }
};

// ---- SSSP, toolkits/sssp.cpp:24-108: push Bellman-Ford, write_min on float distances ----------
struct SsspEdges {
    using Msg = float;
    using Acc = float;
    using R = unsigned int;
    float* dist;
    Subset active_out;
    __device__ bool sparse_signal(uint32_t v, float& msg) const {
        msg = __ldcg(dist + v);
        return true;
    }
    __device__ unsigned sparse_slot(uint32_t, const float& d, uint32_t dst, float w) const {
        const float relax = d + w;
        // non-negative floats order like their bit patterns
        if (relax < __ldcg(dist + dst) &&
            relax < __int_as_float(atomicMin(reinterpret_cast<int*>(dist + dst), __float_as_int(relax)))) {
            active_out.set_bit(dst);
            return 1u;
        }
        return 0u;
    }
    __device__ bool dense_active(uint32_t) const { return false; }
    __device__ float dense_identity() const { return 0.f; }
    __device__ float dense_signal(uint32_t, float) const { return 0.f; }
    __device__ float dense_combine(float a, float) const { return a; }
    __device__ unsigned dense_slot(uint32_t, float) const { return 0u; }
};
struct Count {
    __device__ unsigned operator()(uint32_t) const { return 1u; }
};

static std::vector<char> read_file(const char* path) {
    FILE* f = fopen(path, "rb");
    if (!f) {
        perror(path);
        exit(2);
    }
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::vector<char> b((size_t)n + 1);
    if (n && fread(b.data(), 1, (size_t)n, f) != (size_t)n) exit(2);
    fclose(f);
    b.resize((size_t)n);
    return b;
}

template <class T>
static void write_out(FILE* f, const T* d, size_t n) {
    std::vector<T> h(n);
    eg::engine::check(cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost), "copy out");
    fwrite(h.data(), sizeof(T), n, f);
}

// messages the master/mirror path put in the partitions' buffers over the whole run
static unsigned long long g_messages = 0, g_bytes = 0, g_selective = 0;
static void tally(const Engine& g) {
    g_messages += g.message_stats().messages;
    g_bytes += g.message_stats().bytes;
    g_selective += g.message_stats().selective_bytes;
}

int main(int argc, char** argv) {
    if (argc < 6) {
        fprintf(stderr, "usage: %s pagerank|bfs|cc|sssp <edge file> <V> <iterations|root> <out file>\n", argv[0]);
        return 2;
    }
    const std::string algo = argv[1];
    const uint32_t V = (uint32_t)strtoul(argv[3], nullptr, 10);
    const uint32_t arg = (uint32_t)strtoul(argv[4], nullptr, 10);
    const int rec = algo == "sssp" ? 12 : 8;
    std::vector<char> buf = read_file(argv[2]);
    const uint64_t E = buf.size() / rec;
    const int parts = argc > 6 ? atoi(argv[6]) : 1;  // CPBT partitions (virtual, on this GPU)
    eg_config cfg = {1, parts, 1, 20, 0, nullptr};
    eg_graph* h = nullptr;
    eg::engine::check_eg(eg_create(&h, &cfg), "eg_create");
    eg::engine::check_eg(eg_load_edges(h, buf.data(), E, V, rec, algo == "cc" ? 1 : 0, EG_HOST), "eg_load_edges");
    eg::engine::check_eg(eg_build(h, 1, 1), "eg_build");
    FILE* out = fopen(argv[5], "wb");
    int dense_steps = 0, sparse_steps = 0;
    {
        Engine g(h);
        Subset all = g.alloc_subset();
        g.fill(all);
        if (algo == "pagerank") {
            double* curr = g.alloc_vertex_array<double>();
            double* next = g.alloc_vertex_array<double>();
            g.process_vertices<double>(PrInit{curr, g.out_degree()}, all);
            for (uint32_t it = 0; it < arg; ++it) {
                g.process_vertices<double>(Zero{next}, all);
                g.process_edges(PrEdges{curr, next}, all, Mode::Dense);  // use_iteration: always dense
                tally(g);
                ++dense_steps;
                g.process_vertices<double>(PrApply{next, g.out_degree(), 0.85, it == arg - 1}, all);
                std::swap(curr, next);
            }
            write_out(out, curr, V);
        } else if (algo == "bfs") {
            uint32_t* parent = g.alloc_vertex_array<uint32_t>();
            uint32_t* level = g.alloc_vertex_array<uint32_t>();
            g.fill_vertex_array<uint32_t>(parent, V);
            g.fill_vertex_array<uint32_t>(level, 0xFFFFFFFFu);
            eg::engine::check(cudaMemcpy(parent + arg, &arg, 4, cudaMemcpyHostToDevice), "root");
            const uint32_t zero = 0;
            eg::engine::check(cudaMemcpy(level + arg, &zero, 4, cudaMemcpyHostToDevice), "root");
            Subset a = g.alloc_subset(), b = g.alloc_subset(), visited = g.alloc_subset();
            g.set_bit(a, arg);
            g.set_bit(visited, arg);
            uint32_t active = 1;
            for (uint32_t lvl = 1; active > 0; ++lvl) {
                g.clear(b);
                // Gemini's switch: push while the frontier's out-edges stay below E/20
                g.process_edges(BfsEdges{parent, V, a, b, visited}, a, Mode::Auto, 20, &visited);
                tally(g);
                (g.last_was_dense() ? dense_steps : sparse_steps)++;
                active = g.process_vertices<unsigned>(BfsVisit{visited, level, lvl}, b);
                std::swap(a, b);
            }
            write_out(out, level, V);
            write_out(out, parent, V);
        } else if (algo == "cc") {
            uint32_t* label = g.alloc_vertex_array<uint32_t>();
            std::vector<uint32_t> init(V);
            for (uint32_t v = 0; v < V; ++v) init[v] = v;
            eg::engine::check(cudaMemcpy(label, init.data(), 4ull * V, cudaMemcpyHostToDevice), "labels");
            Subset a = g.alloc_subset(), b = g.alloc_subset();
            g.fill(a);
            uint32_t active = V;
            while (active > 0) {
                g.clear(b);
                active = g.process_edges(CcEdges{label, b}, a, Mode::Auto);
                tally(g);
                (g.last_was_dense() ? dense_steps : sparse_steps)++;
                std::swap(a, b);
            }
            write_out(out, label, V);
        } else if (algo == "sssp") {
            float* dist = g.alloc_vertex_array<float>();
            g.fill_vertex_array<float>(dist, 1e9f);
            const float zero = 0.f;
            eg::engine::check(cudaMemcpy(dist + arg, &zero, 4, cudaMemcpyHostToDevice), "root");
            Subset a = g.alloc_subset(), b = g.alloc_subset();
            g.set_bit(a, arg);
            uint32_t active = 1;
            while (active > 0) {
                g.clear(b);
                active = g.process_edges(SsspEdges{dist, b}, a, Mode::Sparse);  // always sparse
                tally(g);
                ++sparse_steps;
                std::swap(a, b);
            }
            const uint32_t reached = g.process_vertices<unsigned>(Count{}, b);  // b is empty here
            (void)reached;
            write_out(out, dist, V);
        } else {
            fprintf(stderr, "unknown algorithm %s\n", algo.c_str());
            return 2;
        }
    }
    fclose(out);
    printf("{\"dense_steps\": %d, \"sparse_steps\": %d, \"messages\": %llu, \"message_bytes\": %llu, "
           "\"selective_bytes\": %llu}\n",
           dense_steps, sparse_steps, g_messages, g_bytes, g_selective);
    eg_destroy(h);
    return 0;
}
