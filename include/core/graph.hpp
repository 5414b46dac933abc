// graph.hpp — the Graph<EdgeData> API of EndGraph/Gemini (core/graph.hpp:100-1819 of the
// reference) on one GB300 GPU, implemented over the C ABI of libendgraph_gb300 (endgraph_gb300.h).
//
// The reference's toolkits (toolkits/{pagerank,bfs,cc,sssp}.cpp) compile unchanged against this
// header: it keeps the names, signatures, public fields and types they use.  What runs:
//   - load_directed / load_undirected_from_directed stream the binary edge file to the GPU
//     (eg_load_file) and build CPBT partition + CSR + CSC there; prep_time times the build only
//     (like :1367-1371);
//   - vertex arrays, subsets, gather/dump/restore are host-side helpers as in the reference;
//   - the toolkits themselves run on the GPU through pagerank() / bfs() / cc() / sssp();
//   - process_vertices / process_edges / emit with host std::function callbacks are accepted by the
//     compiler but refused at run time (std::runtime_error, status EG_ERR_HOST_CALLBACK): host
//     closures cannot execute on the device engine, and this library has no CPU engine to run them.
// One GPU is one rank: partitions_num = 1, partition_idx = 0.
#ifndef EG_CORE_GRAPH_HPP
#define EG_CORE_GRAPH_HPP

#include <fcntl.h>
#include <sys/mman.h>
#include <unistd.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "core/atomic.hpp"
#include "core/bitmap.hpp"
#include "core/constants.hpp"
#include "core/filesystem.hpp"
#include "core/mpi.hpp"
#include "core/time.hpp"
#include "core/type.hpp"
#include "endgraph_gb300.h"

class EndGraphError : public std::runtime_error {
   public:
    int status;
    EndGraphError(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void eg_throw_if(int status, const char* what) {
    if (status != EG_OK) throw EndGraphError(status, std::string(what) + ": " + eg_last_error());
}

template <typename EdgeData = Empty>
class Graph {
    static_assert(std::is_same<EdgeData, Empty>::value || sizeof(EdgeData) == 4,
                  "the GPU structures hold no edge data or one 4-byte value per edge");

   public:
    // flags the toolkits set (core/graph.hpp:102-106; use_iteration / use_root are what the
    // toolkits assign and the mode switch reads)
    bool has_iterations = false, has_root = false;
    bool use_undirected = false, use_iteration = false, use_root = false;
    int max_iterations = 0;
    size_t eta;
    // one rank, one socket
    int partitions_num = 1, partition_idx = 0, threads_num = 1, sockets_num = 1, threads_per_socket = 1;
    UINT vertices_num = 0;
    ULLONG read_edges_num = 0, edges_num = 0;
    ULLONG exe_data = 0, prep_data = 0;
    double prep_time = 0, exec_time = 0;
    bool sparse = false;
    UINT owned_vertices = 0;
    UINT* degree = nullptr;                  // out-degree per vertex (host copy after load)
    UINT partition_offset_storage[2] = {0, 0};
    std::vector<UINT> local_partition_offset_storage = std::vector<UINT>(2, 0);  // [sockets_num + 1]
    UINT* partition_offset = partition_offset_storage;
    UINT* local_partition_offset = local_partition_offset_storage.data();

    // The reference takes the rank count from MPI and the socket count from libnuma (init(),
    // core/graph.hpp:202-285).  Here one process drives one GPU as one rank: EG_DEVICE picks the
    // GPU (default 0) and EG_SUB_PARTITIONS the second-level CPBT split that sockets_num gives
    // (default 1).  max_iterations is read at load time, as the reference reads it inside
    // assign_vertices (:733-738).
    explicit Graph(int eta_) : eta((size_t)eta_) {
        eg_config cfg;
        cfg.eta = (uint64_t)eta_;
        cfg.partitions = 1;
        cfg.sub_partitions = env_int("EG_SUB_PARTITIONS", 1, 1, 64);
        cfg.max_iterations = 0;
        cfg.device = env_int("EG_DEVICE", 0, 0, 1023);
        cfg.stream = nullptr;
        sockets_num = cfg.sub_partitions;
        local_partition_offset_storage.assign((size_t)sockets_num + 1, 0);
        local_partition_offset = local_partition_offset_storage.data();
        eg_throw_if(eg_create(&handle_, &cfg), "eg_create");
    }
    ~Graph() {
        delete[] degree;
        eg_destroy(handle_);
    }
    Graph(const Graph&) = delete;
    Graph& operator=(const Graph&) = delete;

    eg_graph* native() { return handle_; }

    // ---- loading (core/graph.hpp:629-646, :1011-1084, :1358-1373) --------------------------
    void load_directed(std::string path, UINT vertices) { load(path, vertices, false); }
    void load_undirected_from_directed(std::string path, UINT vertices) { load(path, vertices, true); }

    // ---- vertex arrays and subsets (core/graph.hpp:288-402) ----------------------------------
    template <typename T>
    T* alloc_vertex_array() {
        void* p = mmap(nullptr, sizeof(T) * (size_t)vertices_num, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS,
                       -1, 0);
        if (p == MAP_FAILED) throw EndGraphError(EG_ERR_NOMEM, "alloc_vertex_array");
        return (T*)p;
    }
    template <typename T>
    void dealloc_vertex_array(T* array) {
        munmap(array, sizeof(T) * (size_t)vertices_num);
    }
    template <typename T>
    void fill_vertex_array(T* array, T value) {
        for (UINT v = 0; v < vertices_num; ++v) array[v] = value;
    }
    VertexSubset* alloc_vertex_subset() { return new VertexSubset(vertices_num); }
    // One rank holds every vertex, so there is nothing to gather (core/graph.hpp:381-397 sends
    // each rank's owned range to the root).
    template <typename T>
    void gather_vertex_array(T*, int) {}
    // The reference's persistence format (core/graph.hpp:325-378): a raw file of sizeof(T) * V
    // bytes.  dump creates it at that size when it is missing or has another size, then writes
    // this rank's range [partition_offset[idx], partition_offset[idx + 1]) in place; restore
    // refuses a file of another size and reads the same range.
    template <typename T>
    void dump_vertex_array(T* array, std::string path) {
        const long file_length = (long)(sizeof(T) * (size_t)vertices_num);
        if (!file_exists(path) || file_size(path) != file_length) {
            int fd = open(path.c_str(), O_RDWR | O_CREAT | O_TRUNC, 0644);
            if (fd < 0) throw EndGraphError(EG_ERR_INVALID, "dump_vertex_array: cannot create " + path);
            const bool ok = ftruncate(fd, file_length) == 0;
            close(fd);
            if (!ok) throw EndGraphError(EG_ERR_INVALID, "dump_vertex_array: cannot size " + path);
        }
        io_range(array, path, true);
    }
    template <typename T>
    void restore_vertex_array(T* array, std::string path) {
        if (!file_exists(path) || file_size(path) != (long)(sizeof(T) * (size_t)vertices_num))
            throw EndGraphError(EG_ERR_INVALID, "restore_vertex_array: missing or size mismatch " + path);
        io_range(array, path, false);
    }

    // ---- host-callback engine entry points: compile-compatible, refused at run time ----------
    template <typename R>
    R process_vertices(std::function<R(UINT)>, VertexSubset*) {
        refuse("process_vertices");
        return R();
    }
    template <typename R, typename M>
    R process_edges(std::function<void(UINT)>, std::function<R(UINT, M, AdjacentListType<EdgeData>)>,
                    std::function<void(UINT, AdjacentListType<EdgeData>)>, std::function<R(UINT, M)>, VertexSubset*,
                    VertexSubset* = nullptr) {
        refuse("process_edges");
        return R();
    }
    template <typename M>
    void emit(UINT, M) {
        refuse("emit");
    }

    // ---- the toolkits on the GPU (host output arrays of vertices_num entries) ------------------
    // toolkits/pagerank.cpp:26-98 (FP32 ranks); returns the final curr array
    void pagerank(int iterations, float* out, float damping = 0.85f) {
        eg_throw_if(eg_pagerank(handle_, iterations, damping, out, EG_HOST), "eg_pagerank");
    }
    // toolkits/bfs.cpp:22-84; level and/or parent may be null
    ULLONG bfs(UINT root, UINT* level, UINT* parent) {
        uint64_t reached = 0;
        eg_throw_if(eg_bfs(handle_, root, level, parent, EG_HOST, &reached), "eg_bfs");
        return reached;
    }
    // toolkits/cc.cpp:22-84 (load_undirected_from_directed first)
    void cc(UINT* label) { eg_throw_if(eg_cc(handle_, label, EG_HOST), "eg_cc"); }
    // toolkits/sssp.cpp:24-84 (Graph<float>)
    void sssp(UINT root, float* dist) { eg_throw_if(eg_sssp(handle_, root, dist, EG_HOST), "eg_sssp"); }

   private:
    eg_graph* handle_ = nullptr;

    // pwrite / pread of this rank's range of a vertex array at its own offset in the file
    template <typename T>
    void io_range(T* array, const std::string& path, bool write_out) {
        int fd = open(path.c_str(), O_RDWR);
        if (fd < 0) throw EndGraphError(EG_ERR_INVALID, "vertex array file: cannot open " + path);
        long offset = (long)(sizeof(T) * (size_t)partition_offset[partition_idx]);
        const long end_offset = (long)(sizeof(T) * (size_t)partition_offset[partition_idx + 1]);
        char* data = reinterpret_cast<char*>(array);
        while (offset < end_offset) {
            ssize_t n = write_out ? pwrite(fd, data + offset, end_offset - offset, offset)
                                  : pread(fd, data + offset, end_offset - offset, offset);
            if (n <= 0) {
                close(fd);
                throw EndGraphError(EG_ERR_INVALID, std::string("vertex array file: short ") +
                                                        (write_out ? "write " : "read ") + path);
            }
            offset += n;
        }
        close(fd);
    }

    static int env_int(const char* name, int dflt, int lo, int hi) {
        const char* v = getenv(name);
        if (!v || !*v) return dflt;
        char* end = nullptr;
        long x = strtol(v, &end, 10);
        if (*end || x < lo || x > hi)
            throw EndGraphError(EG_ERR_INVALID, std::string(name) + ": expected an integer in [" + std::to_string(lo) +
                                                    ", " + std::to_string(hi) + "], got '" + v + "'");
        return (int)x;
    }

    [[noreturn]] void refuse(const char* what) {
        throw EndGraphError(EG_ERR_HOST_CALLBACK,
                            std::string(what) +
                                ": host std::function callbacks cannot run on the GB300 engine; use "
                                "Graph::pagerank/bfs/cc/sssp or the eg_* C ABI");
    }

    void load(const std::string& path, UINT vertices, bool symmetric) {
        const size_t rec = sizeof(EdgeType<EdgeData>);
        eg_throw_if(eg_set_option(handle_, EG_OPT_MAX_ITERATIONS, max_iterations), "eg_set_option");
        eg_throw_if(eg_load_file(handle_, path.c_str(), vertices, (int)rec, symmetric ? 1 : 0), "eg_load_file");
        eg_info info;
        eg_throw_if(eg_get_info(handle_, &info), "eg_get_info");
        vertices_num = vertices;
        edges_num = info.E;
        read_edges_num = edges_num;
        owned_vertices = vertices;
        double t = -MPI_Wtime();
        eg_throw_if(eg_build(handle_, 1, 1), "eg_build");
        t += MPI_Wtime();
        prep_time = t;
        delete[] degree;
        degree = new UINT[vertices];
        eg_throw_if(eg_get_degrees(handle_, degree, nullptr, EG_HOST), "eg_get_degrees");
        eg_throw_if(eg_get_partition(handle_, partition_offset_storage, local_partition_offset_storage.data()),
                    "eg_get_partition");
    }
};

#endif
