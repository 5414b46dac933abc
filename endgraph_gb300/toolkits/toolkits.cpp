// toolkits.cpp — the four Gemini toolkits as command-line programs on the GPU, with the
// reference's arguments (toolkits/{pagerank,bfs,cc,sssp}.cpp:main):
//
//   pagerank [file] [vertices] [iterations] [eta] [dump]
//   bfs      [file] [vertices] [root] [eta] [dump]
//   cc       [file] [vertices] [null] [eta] [dump]
//   sssp     [file] [vertices] [root] [eta] [dump]      (12-byte records with a float weight)
//
// The program name (argv[0] basename, or EG_TOOLKIT) selects the toolkit.  Like the reference it
// loads the graph once, runs the computation four times, prints the toolkit's summary line
// (pr_sum / found_vertices / components / distance[argmax]) and the prep / exec times; with a
// fifth argument the result array is written there as a raw vertex array (dump_vertex_array).
#include <libgen.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "core/graph.hpp"

static int run_pagerank(int argc, char** argv) {
    Graph<Empty> g(std::atoi(argv[4]));
    g.load_directed(argv[1], (UINT)std::atoi(argv[2]));
    const int iterations = std::atoi(argv[3]);
    g.use_iteration = true;
    g.max_iterations = iterations;
    std::vector<float> pr(g.vertices_num);
    for (int run = 0; run < 4; ++run) {
        double t = -get_time();
        g.pagerank(iterations, pr.data());
        t += get_time();
        double sum = 0;
        UINT best = 0;
        for (UINT v = 0; v < g.vertices_num; ++v) {
            sum += pr[v];
            if (pr[v] > pr[best]) best = v;
        }
        printf("pr_sum=%lf\npr[%u]=%lf\npre time: %lf s exec time: %lf s\n", sum, best, (double)pr[best], g.prep_time, t);
    }
    if (argc > 5) g.dump_vertex_array(pr.data(), argv[5]);
    return 0;
}

static int run_bfs(int argc, char** argv) {
    Graph<Empty> g(std::atoi(argv[4]));
    const UINT root = (UINT)std::atoi(argv[3]);
    g.load_directed(argv[1], (UINT)std::atoi(argv[2]));
    g.use_root = true;
    std::vector<UINT> parent(g.vertices_num), level(g.vertices_num);
    for (int run = 0; run < 4; ++run) {
        double t = -get_time();
        g.bfs(root, level.data(), parent.data());
        t += get_time();
        UINT found = 0;
        for (UINT v = 0; v < g.vertices_num; ++v) found += parent[v] < g.vertices_num;
        printf("found_vertices = %u\npre time: %lf s, exec time: %lf\n", found, g.prep_time, t);
    }
    if (argc > 5) g.dump_vertex_array(level.data(), argv[5]);
    return 0;
}

static int run_cc(int argc, char** argv) {
    Graph<Empty> g(std::atoi(argv[4]));
    g.load_undirected_from_directed(argv[1], (UINT)std::atoi(argv[2]));
    g.use_undirected = true;
    std::vector<UINT> label(g.vertices_num);
    for (int run = 0; run < 4; ++run) {
        double t = -get_time();
        g.cc(label.data());
        t += get_time();
        std::vector<UINT> count(g.vertices_num, 0);
        UINT components = 0;
        for (UINT v = 0; v < g.vertices_num; ++v) components += count[label[v]]++ == 0;
        printf("components = %u\npre time: %lf s, exec time: %lf s\n", components, g.prep_time, t);
    }
    if (argc > 5) g.dump_vertex_array(label.data(), argv[5]);
    return 0;
}

static int run_sssp(int argc, char** argv) {
    Graph<float> g(std::atoi(argv[4]));
    g.load_directed(argv[1], (UINT)std::atoi(argv[2]));
    const UINT root = (UINT)std::atoi(argv[3]);
    g.use_root = true;
    std::vector<float> dist(g.vertices_num);
    for (int run = 0; run < 4; ++run) {
        double t = -get_time();
        g.sssp(root, dist.data());
        t += get_time();
        UINT best = root;
        for (UINT v = 0; v < g.vertices_num; ++v)
            if (dist[v] < 1e9f && dist[v] > dist[best]) best = v;
        printf("distance[%u]=%f\npre time: %lfs, exec time: %lf s\n", best, (double)dist[best], g.prep_time, t);
    }
    if (argc > 5) g.dump_vertex_array(dist.data(), argv[5]);
    return 0;
}

int main(int argc, char** argv) {
    std::string name = getenv("EG_TOOLKIT") ? getenv("EG_TOOLKIT") : basename(argv[0]);
    if (argc < 5) {
        fprintf(stderr, "%s [file] [vertices] [iterations|root|null] [eta] [dump]\n", name.c_str());
        return 1;
    }
    try {
        if (name == "pagerank") return run_pagerank(argc, argv);
        if (name == "bfs") return run_bfs(argc, argv);
        if (name == "cc") return run_cc(argc, argv);
        if (name == "sssp") return run_sssp(argc, argv);
        fprintf(stderr, "unknown toolkit %s\n", name.c_str());
        return 1;
    } catch (const EndGraphError& e) {
        fprintf(stderr, "%s: %s\n", name.c_str(), e.what());
        return 2;
    }
}
