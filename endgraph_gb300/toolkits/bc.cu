// bc.cu — single-source betweenness centrality as a toolkit program (the reference README names a
// BC toolkit, README.md:24,37, that its tree does not contain).  Brandes' two sweeps written as
// device operators for process_edges (include/endgraph_gb300_engine.cuh):
//   forward  — level-synchronous BFS from the root that sums shortest-path counts (sigma) into
//              each newly reached vertex, push or pull per level by the E/20 switch;
//   backward — on the transposed graph, level by level from the deepest, every vertex v one level
//              above a vertex w gains sigma[v] / sigma[w] * (1 + delta[w]).
//
//   bc [file] [vertices] [root] [eta] [dump]
//
// Prints the summary and times like the reference toolkits (four runs); with a fifth argument
// writes sigma (V doubles) followed by delta (V doubles) to that file.
#include <stdio.h>
#include <stdlib.h>

#include <vector>

#include "core/graph.hpp"
#include "endgraph_gb300_engine.cuh"

using eg::engine::Engine;
using eg::engine::Mode;
using eg::engine::Subset;

struct BcForward {
    using Msg = double;
    using Acc = double;
    using R = unsigned int;
    double* paths;
    Subset visited, front, next;
    __device__ bool sparse_signal(uint32_t v, double& m) const {
        m = paths[v];
        return true;
    }
    __device__ unsigned sparse_slot(uint32_t, const double& m, uint32_t dst, float) const {
        if (visited.get_bit(dst)) return 0u;
        atomicAdd(paths + dst, m);  // integer-valued sums: exact in any order below 2^53
        const unsigned long long bit = 1ull << (dst & 63);
        return (atomicOr(next.words + (dst >> 6), bit) & bit) ? 0u : 1u;
    }
    __device__ bool dense_active(uint32_t dst) const { return !visited.get_bit(dst); }
    __device__ double dense_identity() const { return 0.0; }
    __device__ double dense_signal(uint32_t src, float) const { return front.get_bit(src) ? paths[src] : 0.0; }
    __device__ double dense_combine(double a, double b) const { return a + b; }
    __device__ unsigned dense_slot(uint32_t dst, double sum) const {
        if (sum == 0.0) return 0u;
        paths[dst] = sum;
        next.set_bit(dst);
        return 1u;
    }
};

struct Reached {  // newly reached vertices: visited, with their level
    Subset visited;
    uint32_t* level;
    uint32_t lvl;
    __device__ unsigned operator()(uint32_t v) const {
        visited.set_bit(v);
        level[v] = lvl;
        return 1u;
    }
};

// on the transposed graph: sources are the level-l vertices w, destinations their in-neighbours v
struct BcBackward {
    using Msg = double;
    using Acc = double;
    using R = unsigned int;
    const double* paths;
    double* dep;
    const uint32_t* level;
    uint32_t l;
    __device__ bool sparse_signal(uint32_t w, double& m) const {
        m = (1.0 + dep[w]) / paths[w];
        return true;
    }
    __device__ unsigned sparse_slot(uint32_t, const double& m, uint32_t v, float) const {
        if (level[v] == l - 1) atomicAdd(dep + v, paths[v] * m);
        return 0u;
    }
    __device__ bool dense_active(uint32_t v) const { return level[v] == l - 1; }
    __device__ double dense_identity() const { return 0.0; }
    __device__ double dense_signal(uint32_t w, float) const { return level[w] == l ? (1.0 + dep[w]) / paths[w] : 0.0; }
    __device__ double dense_combine(double a, double b) const { return a + b; }
    __device__ unsigned dense_slot(uint32_t v, double sum) const {
        dep[v] += paths[v] * sum;
        return 0u;
    }
};

struct Sum {
    const double* a;
    __device__ double operator()(uint32_t v) const { return a[v]; }
};

int main(int argc, char** argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s [file] [vertices] [root] [eta] [dump]\n", argv[0]);
        return 2;
    }
    try {
        Graph<Empty> g(std::atoi(argv[4]));
        g.load_directed(argv[1], (UINT)std::atoi(argv[2]));
        const uint32_t V = g.vertices_num;
        const uint32_t root = (uint32_t)std::atoi(argv[3]);
        if (root >= V) {
            fprintf(stderr, "root %u out of range\n", root);
            return 2;
        }
        Engine eng(g.native());
        double* paths = eng.alloc_vertex_array<double>();
        double* dep = eng.alloc_vertex_array<double>();
        uint32_t* level = eng.alloc_vertex_array<uint32_t>();
        Subset visited = eng.alloc_subset(), all = eng.alloc_subset();
        eng.fill(all);
        double exec = 0;
        for (int run = 0; run < 4; ++run) {
            double t = -get_time();
            eng.set_transposed(false);
            eng.fill_vertex_array(paths, 0.0);
            eng.fill_vertex_array(dep, 0.0);
            eng.fill_vertex_array(level, 0xFFFFFFFFu);
            eng.clear(visited);
            std::vector<Subset> fronts;  // fronts[l]: the vertices at BFS level l
            fronts.push_back(eng.alloc_subset());
            eng.set_bit(fronts[0], root);
            eng.set_bit(visited, root);
            const double one = 1.0;
            const uint32_t zero = 0;
            eg::engine::check(cudaMemcpy(paths + root, &one, 8, cudaMemcpyHostToDevice), "root");
            eg::engine::check(cudaMemcpy(level + root, &zero, 4, cudaMemcpyHostToDevice), "root");
            for (uint32_t lvl = 1;; ++lvl) {
                Subset next = eng.alloc_subset();
                const unsigned found = eng.process_edges(BcForward{paths, visited, fronts.back(), next}, fronts.back());
                if (!found) {
                    eng.free_subset(next);
                    break;
                }
                eng.process_vertices<unsigned>(Reached{visited, level, lvl}, next);
                fronts.push_back(next);
            }
            eng.set_transposed(true);
            for (uint32_t l = (uint32_t)fronts.size() - 1; l >= 1; --l)
                eng.process_edges(BcBackward{paths, dep, level, l}, fronts[l]);
            for (Subset& f : fronts) eng.free_subset(f);
            t += get_time();
            exec = t;
            const double total = eng.process_vertices<double>(Sum{dep}, all);
            printf("levels=%zu dependency_sum=%lf\npre time: %lf s exec time: %lf s\n", fronts.size(), total,
                   g.prep_time, t);
        }
        (void)exec;
        if (argc > 5) {
            std::vector<double> h((size_t)V);
            FILE* f = fopen(argv[5], "wb");
            if (!f) {
                perror(argv[5]);
                return 2;
            }
            eg::engine::check(cudaMemcpy(h.data(), paths, 8ull * V, cudaMemcpyDeviceToHost), "dump");
            fwrite(h.data(), 8, V, f);
            eg::engine::check(cudaMemcpy(h.data(), dep, 8ull * V, cudaMemcpyDeviceToHost), "dump");
            fwrite(h.data(), 8, V, f);
            fclose(f);
        }
    } catch (const std::exception& e) {
        fprintf(stderr, "bc: %s\n", e.what());
        return 1;
    }
    return 0;
}
