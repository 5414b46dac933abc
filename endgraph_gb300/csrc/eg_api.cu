// eg_api.cu — the extern "C" boundary of libendgraph_gb300.so (include/endgraph_gb300.h).
#include <errno.h>
#include <fcntl.h>
#include <string.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "eg_common.cuh"

using namespace eg;

namespace {

int check_graph(eg_graph* g, const char* fn) {
    if (!g) {
        set_error("%s: null handle", fn);
        return EG_ERR_INVALID;
    }
    cudaError_t e = cudaSetDevice(g->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice", __FILE__, __LINE__);
    return EG_OK;
}

int init_handle(eg_graph* g, const eg_config* cfg) {
    eg_config c = {1, 1, 1, 20, 0, nullptr};
    if (cfg) c = *cfg;
    if (c.partitions < 1 || c.partitions > kMaxPartitions) {
        set_error("eg_create: partitions must be in [1, %d]", kMaxPartitions);
        return EG_ERR_INVALID;
    }
    if (c.sub_partitions < 1 || c.sub_partitions > kMaxPartitions) {
        set_error("eg_create: sub_partitions must be in [1, %d]", kMaxPartitions);
        return EG_ERR_INVALID;
    }
    int ndev = 0;
    EG_CUDA(cudaGetDeviceCount(&ndev));
    if (c.device < 0 || c.device >= ndev) {
        set_error("eg_create: device %d not present (%d devices)", c.device, ndev);
        return EG_ERR_INVALID;
    }
    g->device = c.device;
    EG_CUDA(cudaSetDevice(g->device));
    EG_CUDA(cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, g->device));
    g->eta = c.eta;
    g->partitions = c.partitions;
    g->sub_partitions = c.sub_partitions;
    g->max_iterations = c.max_iterations;
    if (c.stream) {
        g->stream = (cudaStream_t)c.stream;
        g->own_stream = false;
    } else {
        EG_CUDA(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
        g->own_stream = true;
    }
    EG_TRY(g->err.reserve(64));
    EG_CUDA(cudaMemsetAsync(g->err.ptr, 0, 64, g->stream));
    EG_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&g->eng.host_words), 256, cudaHostAllocDefault));
    return EG_OK;
}

void free_handle(eg_graph* g) {
    if (!g) return;
    cudaSetDevice(g->device);
    if (g->stream) cudaStreamSynchronize(g->stream);
    g->prof.clear();
    free_batch_state(g);
    if (g->pinned) cudaFreeHost(g->pinned);
    if (g->eng.host_words) cudaFreeHost(g->eng.host_words);
    if (g->eng.bfs_exec) cudaGraphExecDestroy(g->eng.bfs_exec);
    if (g->eng.bfs_graph) cudaGraphDestroy(g->eng.bfs_graph);
    if (g->copy_stream) {
        cudaStreamSynchronize(g->copy_stream);
        cudaStreamDestroy(g->copy_stream);
    }
    for (cudaEvent_t e : g->part_ready)
        if (e) cudaEventDestroy(e);
    if (g->copy_gate) cudaEventDestroy(g->copy_gate);
    cudaStream_t s = g->stream;
    bool own = g->own_stream;
    delete g;  // DevBuf destructors free device memory
    if (own && s) cudaStreamDestroy(s);
}

struct HandleDeleter {
    void operator()(eg_graph* g) const { free_handle(g); }
};

}  // namespace

extern "C" {

int eg_version(void) { return 1; }

unsigned long long eg_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

const char* eg_last_error(void) { return error_text(); }

int eg_create(eg_graph** out, const eg_config* cfg) {
    if (!out) {
        set_error("eg_create: null output");
        return EG_ERR_INVALID;
    }
    *out = nullptr;
    eg_graph* g = new eg_graph();
    int s = init_handle(g, cfg);
    if (s != EG_OK) {
        free_handle(g);
        return s;
    }
    *out = g;
    return EG_OK;
}

int eg_destroy(eg_graph* g) {
    if (!g) return EG_OK;
    free_handle(g);
    return EG_OK;
}

void* eg_stream(eg_graph* g) { return g ? (void*)g->stream : nullptr; }

int eg_sync(eg_graph* g) {
    EG_TRY(check_graph(g, "eg_sync"));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    return EG_OK;
}

int eg_load_edges(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes, int symmetric, int where) {
    EG_TRY(check_graph(g, "eg_load_edges"));
    return load_edges_impl(g, edges, E, V, edge_bytes, symmetric, where, true);
}

int eg_load_directed_file(eg_graph* g, const char* path, uint32_t V, int edge_bytes) {
    EG_TRY(check_graph(g, "eg_load_directed_file"));
    free_batch_state(g);
    return eg::load_build_file(g, path, V, edge_bytes);
}

int eg_load_file(eg_graph* g, const char* path, uint32_t V, int edge_bytes, int symmetric) {
    EG_TRY(check_graph(g, "eg_load_file"));
    return load_file_impl(g, path, V, edge_bytes, symmetric);
}

int eg_load_graph_batch(eg_graph* g, const void* edges, int edge_bytes, const uint64_t* graph_edges,
                        const uint32_t* graph_vertices, int ngraphs, int where) {
    EG_TRY(check_graph(g, "eg_load_graph_batch"));
    return load_graph_batch(g, edges, edge_bytes, graph_edges, graph_vertices, ngraphs, where);
}

int eg_get_graph_batch(eg_graph* g, uint64_t* vertex_offsets, uint64_t* edge_offsets) {
    EG_TRY(check_graph(g, "eg_get_graph_batch"));
    if (g->batch_voff.empty()) {
        set_error("eg_get_graph_batch: no graph batch loaded");
        return EG_ERR_STATE;
    }
    if (vertex_offsets) memcpy(vertex_offsets, g->batch_voff.data(), 8 * g->batch_voff.size());
    if (edge_offsets) memcpy(edge_offsets, g->batch_eoff.data(), 8 * g->batch_eoff.size());
    return EG_OK;
}

int eg_msbfs_graphs(eg_graph* g, const uint32_t* roots, int roots_per_graph, uint8_t* levels, int where,
                    uint64_t* edges) {
    EG_TRY(check_graph(g, "eg_msbfs_graphs"));
    return run_msbfs_graphs(g, roots, roots_per_graph, levels, where, edges);
}

int eg_sssp_graphs(eg_graph* g, const uint32_t* sources, int sources_per_graph, float* dist, int where) {
    EG_TRY(check_graph(g, "eg_sssp_graphs"));
    return run_sssp_graphs(g, sources, sources_per_graph, dist, where);
}

}  // extern "C"

namespace eg {
static int prepare_load(eg_graph* g, uint64_t E, uint32_t V, int edge_bytes, int symmetric);

int load_edges_impl(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes, int symmetric, int where,
                    bool validate) {
    if (E > 0 && !edges) {
        set_error("eg_load_edges: null edge pointer");
        return EG_ERR_INVALID;
    }
    if (where != EG_HOST && where != EG_DEVICE) {
        set_error("eg_load_edges: where must be EG_HOST or EG_DEVICE");
        return EG_ERR_INVALID;
    }
    EG_TRY(prepare_load(g, E, V, edge_bytes, symmetric));
    if (E) {
        EG_CUDA(cudaMemcpyAsync(g->edges.ptr, edges, (size_t)E * edge_bytes,
                                where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, g->stream));
    }
    if (validate) EG_TRY(validate_edges(g, E));
    if (symmetric) EG_TRY(symmetrize_edges(g, E));
    return EG_OK;
}

// argument checks, state reset and the record buffer of a new edge list
static int prepare_load(eg_graph* g, uint64_t E, uint32_t V, int edge_bytes, int symmetric) {
    if (edge_bytes != 8 && edge_bytes != 12) {
        set_error("eg_load_edges: edge_bytes must be 8 ({src,dst}) or 12 ({src,dst,float})");
        return EG_ERR_INVALID;
    }
    if (V == 0) {
        set_error("eg_load_edges: V must be positive");
        return EG_ERR_INVALID;
    }
    const uint64_t total = symmetric ? 2 * E : E;
    if (total > (1ull << 40)) {
        set_error("eg_load_edges: too many edges");
        return EG_ERR_INVALID;
    }
    g->built_csr = g->built_csc = false;
    g->eng.pull_ready = false;
    g->eng.pr_ready = false;
    free_batch_state(g);
    g->batch_voff.clear();
    g->batch_eoff.clear();
    g->V = V;
    g->E = total;
    g->E_input = E;
    g->edge_ids = false;
    g->edge_bytes = edge_bytes;
    g->weighted = edge_bytes == 12;
    g->symmetric = symmetric != 0;
    EG_TRY(g->edges.reserve((size_t)total * edge_bytes + 64));
    return EG_OK;
}

// preload_graph_file (core/graph.hpp:1011-1084) for one rank: the whole file, read in 128 MiB
// pieces into two pinned staging buffers, so that reading piece i+1 overlaps the host-to-device
// copy of piece i; then the same validation and symmetrisation as eg_load_edges.
constexpr size_t kIngestPiece = 128ull << 20;

// Reader threads started once per file (or per host buffer, mem != null): each piece is split into
// one slice per thread (page-cache and pageable-memory copies are bound per thread), and the caller
// waits until every slice of the piece is in.
class ReaderPool {
   public:
    ReaderPool(int fd, unsigned nt, const uint8_t* mem = nullptr) : fd_(fd), nt_(nt), mem_(mem) {
        try {
            for (unsigned t = 0; t < nt; ++t) threads_.emplace_back([this, t] { run(t); });
        } catch (...) {  // fewer threads than asked (none: the caller's thread reads)
        }
        std::lock_guard<std::mutex> lk(m_);
        nt_ = (unsigned)threads_.size();
    }
    ~ReaderPool() {
        {
            std::lock_guard<std::mutex> lk(m_);
            stop_ = true;
            ++gen_;
        }
        cv_.notify_all();
        for (auto& th : threads_) th.join();
    }
    // bytes [off, off + n) of the file into buf; false on a short read
    bool read(uint8_t* buf, uint64_t off, size_t n) {
        if (nt_ == 0) return slice(buf, off, 0, n);
        {
            std::lock_guard<std::mutex> lk(m_);
            buf_ = buf;
            off_ = off;
            n_ = n;
            pending_ = nt_;
            ok_ = true;
            ++gen_;
        }
        cv_.notify_all();
        std::unique_lock<std::mutex> lk(m_);
        done_.wait(lk, [&] { return pending_ == 0; });
        return ok_;
    }

   private:
    void run(unsigned t) {
        uint64_t seen = 0;
        while (true) {
            uint8_t* buf;
            uint64_t off;
            size_t n;
            {
                std::unique_lock<std::mutex> lk(m_);
                cv_.wait(lk, [&] { return gen_ != seen; });
                seen = gen_;
                if (stop_) return;
                buf = buf_;
                off = off_;
                n = n_;
            }
            const size_t part = (n + nt_ - 1) / nt_;
            const size_t a = std::min(n, t * part), z = std::min(n, a + part);
            const bool good = slice(buf, off, a, z);
            std::lock_guard<std::mutex> lk(m_);
            if (!good) ok_ = false;
            if (--pending_ == 0) done_.notify_one();
        }
    }
    // bytes [a, z) of the piece at off
    bool slice(uint8_t* buf, uint64_t off, size_t a, size_t z) const {
        if (mem_) {
            memcpy(buf + a, mem_ + off + a, z - a);
            return true;
        }
        size_t got = 0;
        while (a + got < z) {
            const ssize_t r = pread(fd_, buf + a + got, z - a - got, (off_t)(off + a + got));
            if (r < 0 && errno == EINTR) continue;
            if (r <= 0) return false;
            got += (size_t)r;
        }
        return true;
    }
    int fd_;
    unsigned nt_;
    const uint8_t* mem_;
    std::vector<std::thread> threads_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    uint64_t gen_ = 0;
    bool stop_ = false, ok_ = true;
    unsigned pending_ = 0;
    uint8_t* buf_ = nullptr;
    uint64_t off_ = 0;
    size_t n_ = 0;
};

// Whether the device reads pageable host memory through the host's page tables (Grace with
// NVLink-C2C: a copy from an ordinary allocation or a page-cached file mapping runs at the link's
// rate), so that uploads need no pinned staging copy on the host.
static bool pageable_at_link_rate(eg_graph* g) {
    if (g->pageable_direct < 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, g->device) != cudaSuccess) v = 0;
        cudaGetLastError();
        g->pageable_direct = v ? 1 : 0;
    }
    return g->pageable_direct == 1;
}

// Reads one byte of every page of [off, off + n) of a file mapping on up to 16 host threads, so
// that the page-cached pages are mapped before the device reads them.
static void touch_pages(const uint8_t* src, size_t off, size_t n) {
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t page = (size_t)std::max(4096L, sysconf(_SC_PAGESIZE));
    std::atomic<unsigned long long> sink{0};
    auto run = [&](size_t a, size_t z) {
        unsigned long long acc = 0;
        for (size_t p = a & ~(page - 1); p < z; p += page) acc += *reinterpret_cast<const volatile uint8_t*>(src + std::max(p, a));
        sink += acc;
    };
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < nt; ++t) {
        const size_t a = off + n * t / nt, z = off + n * (t + 1) / nt;
        try {
            ts.emplace_back(run, a, z);
        } catch (...) {
            run(a, z);
        }
    }
    for (auto& th : ts) th.join();
}

// the two pinned staging buffers of file reads and pageable uploads
static int ensure_staging(eg_graph* g) {
    if (g->pinned_bytes >= 2 * kIngestPiece) return EG_OK;
    if (g->pinned) cudaFreeHost(g->pinned);
    g->pinned = nullptr;
    g->pinned_bytes = 0;
    cudaError_t e = cudaHostAlloc(&g->pinned, 2 * kIngestPiece, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        g->pinned = nullptr;
        return cuda_fail(e, "cudaHostAlloc", __FILE__, __LINE__);
    }
    g->pinned_bytes = 2 * kIngestPiece;
    return EG_OK;
}

// Host records uploaded in up to 8 parts on the handle's copy stream while the build consumes
// them: passes A and B of part k (and the id validation, in pass A) run on the handle's stream as
// soon as part k has landed, so only the last part's passes and pass C follow the upload.  The
// caller's buffer is read until this returns.
// mem: the records in host memory; else fd: a binary record file read by the staging thread
// touch: mem is a fresh file mapping; its pages are read once by host threads just before each
// part goes up, so that the device finds them mapped instead of faulting them in one by one
static int pipelined_load(eg_graph* g, const uint8_t* mem, int fd, uint64_t E, uint32_t V, int edge_bytes,
                          bool touch = false) {
    EG_TRY(prepare_load(g, E, V, edge_bytes, 0));
    if (!g->copy_stream) EG_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    if (!g->copy_gate) EG_CUDA(cudaEventCreateWithFlags(&g->copy_gate, cudaEventDisableTiming));
    for (cudaEvent_t& e : g->part_ready)
        if (!e) EG_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    UploadParts up{};
    const int want = (int)std::max<uint64_t>(1, std::min<uint64_t>(8, E / (kPipelinedLoadMin / 2)));
    // the last part's passes follow the copy, so it is the smallest (1/32 of the records); the
    // others share the rest; parts start on 64-record boundaries
    const uint64_t last = want > 1 ? E / 32 : 0;
    const uint64_t per = want > 1 ? ((E - last + want - 2) / (want - 1) + 63) & ~63ull : E;
    int K = 0;
    for (uint64_t a = 0; a < E && K < want - 1; a += per) up.e0[K++] = a;
    if (want > 1) {
        const uint64_t tail = (E - last) & ~63ull;
        if (K == 0 || tail > up.e0[K - 1]) up.e0[K++] = tail;
    } else if (K == 0) {
        up.e0[K++] = 0;
    }
    up.K = K;
    up.e0[K] = E;
    // the records buffer may still be read by earlier work on the handle's stream
    EG_CUDA(cudaEventRecord(g->copy_gate, g->stream));
    EG_CUDA(cudaStreamWaitEvent(g->copy_stream, g->copy_gate, 0));
    const uint8_t* src = mem;
    for (int k = 0; k < K; ++k) up.ready[k] = g->part_ready[k];
    // pinned host memory (or device / managed memory handed over as host: unified addressing
    // copies it the same way) goes to the copy engines directly; pageable memory is staged
    cudaPointerAttributes attr{};
    const bool direct = mem && cudaPointerGetAttributes(&attr, mem) == cudaSuccess &&
                        (attr.type == cudaMemoryTypeHost || attr.type == cudaMemoryTypeDevice ||
                         attr.type == cudaMemoryTypeManaged);
    cudaGetLastError();  // a pageable pointer may leave an error behind on older drivers
    free_batch_state(g);
    if (direct) {  // every part queued now
        cudaError_t e = cudaSuccess;
        for (int k = 0; k < K && e == cudaSuccess; ++k) {
            const size_t off = (size_t)up.e0[k] * edge_bytes, n = (size_t)(up.e0[k + 1] - up.e0[k]) * edge_bytes;
            e = cudaMemcpyAsync(g->edges.as<uint8_t>() + off, src + off, n, cudaMemcpyDefault, g->copy_stream);
            if (e == cudaSuccess) e = cudaEventRecord(g->part_ready[k], g->copy_stream);
        }
        if (e != cudaSuccess) {  // copies already queued may still read the caller's buffer
            cudaStreamSynchronize(g->copy_stream);
            g->V = 0;
            return cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__);
        }
        const int st = build_structures(g, 1, 1, &up);
        e = cudaStreamSynchronize(g->copy_stream);  // never return with the buffer in use
        if (st != EG_OK) {
            g->V = 0;  // no usable edge list
            return st;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize", __FILE__, __LINE__);
        return EG_OK;
    }
    // pageable memory or a file: a staging thread copies each part through the two pinned buffers
    // (reader threads memcpy or pread a piece while the previous piece goes up) and records the
    // part's event; the build waits for each event only after it has been recorded.  Where the
    // device reads pageable memory at the link's rate, the thread copies each part straight from
    // the caller's pages (or the file's mapping) instead.
    const bool from_pages = src && pageable_at_link_rate(g);
    if (!from_pages) EG_TRY(ensure_staging(g));
    std::atomic<int> issued{0};
    std::atomic<bool> failed{false};
    up.issued = &issued;
    up.failed = &failed;
    cudaError_t stage_err = cudaSuccess;
    uint64_t short_at = ~0ull;  // a short file read at this byte
    auto stage = [&]() {
        cudaSetDevice(g->device);
        if (from_pages) {
            cudaError_t e = cudaSuccess;
            for (int k = 0; k < K && e == cudaSuccess; ++k) {
                const size_t off = (size_t)up.e0[k] * edge_bytes, n = (size_t)(up.e0[k + 1] - up.e0[k]) * edge_bytes;
                if (touch) touch_pages(src, off, n);  // this part's pages mapped before its copy
                e = cudaMemcpyAsync(g->edges.as<uint8_t>() + off, src + off, n, cudaMemcpyDefault, g->copy_stream);
                if (e == cudaSuccess) e = cudaEventRecord(g->part_ready[k], g->copy_stream);
                if (e == cudaSuccess) issued.store(k + 1, std::memory_order_release);
            }
            if (e != cudaSuccess) {
                stage_err = e;
                failed.store(true, std::memory_order_release);
            }
            cudaStreamSynchronize(g->copy_stream);  // the caller's pages are read until this returns
            return;
        }
        cudaEvent_t done[2] = {nullptr, nullptr};
        cudaError_t e = cudaSuccess;
        for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
        ReaderPool pool(fd, std::max(1u, std::min(16u, std::thread::hardware_concurrency())), src);
        uint64_t piece = 0;
        for (int k = 0; k < K && e == cudaSuccess && short_at == ~0ull; ++k) {
            const uint64_t a = up.e0[k] * (uint64_t)edge_bytes, z = up.e0[k + 1] * (uint64_t)edge_bytes;
            for (uint64_t off = a; off < z && e == cudaSuccess; off += kIngestPiece, ++piece) {
                const int slot = (int)(piece & 1);
                uint8_t* buf = static_cast<uint8_t*>(g->pinned) + slot * kIngestPiece;
                if (piece >= 2) e = cudaEventSynchronize(done[slot]);  // the copy that last used it
                if (e != cudaSuccess) break;
                const size_t n = (size_t)std::min<uint64_t>(kIngestPiece, z - off);
                if (!pool.read(buf, off, n)) {
                    short_at = off;
                    break;
                }
                e = cudaMemcpyAsync(g->edges.as<uint8_t>() + off, buf, n, cudaMemcpyHostToDevice, g->copy_stream);
                if (e == cudaSuccess) e = cudaEventRecord(done[slot], g->copy_stream);
            }
            if (short_at != ~0ull) break;
            if (e == cudaSuccess) e = cudaEventRecord(g->part_ready[k], g->copy_stream);
            if (e == cudaSuccess) issued.store(k + 1, std::memory_order_release);
        }
        if (e != cudaSuccess || short_at != ~0ull) {
            stage_err = e;
            failed.store(true, std::memory_order_release);
        }
        cudaStreamSynchronize(g->copy_stream);  // the staging buffers are reused by the next call
        for (int i = 0; i < 2; ++i)
            if (done[i]) cudaEventDestroy(done[i]);
    };
    std::thread stager;
    try {
        stager = std::thread(stage);
    } catch (...) {  // no thread to spare: upload everything first, then build
        stage();
    }
    const int st = build_structures(g, 1, 1, &up);
    if (stager.joinable()) stager.join();
    if (st != EG_OK || stage_err != cudaSuccess || short_at != ~0ull) {
        g->V = 0;  // no usable edge list
        if (stage_err != cudaSuccess) return cuda_fail(stage_err, "eg_load_directed upload", __FILE__, __LINE__);
        if (short_at != ~0ull) {
            set_error("eg_load_directed_file: short read in the piece at byte %llu", (unsigned long long)short_at);
            return EG_ERR_INVALID;
        }
        return st;
    }
    return EG_OK;
}

int load_build_pipelined(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes) {
    return pipelined_load(g, static_cast<const uint8_t*>(edges), -1, E, V, edge_bytes);
}

// binary records of a file, read and uploaded in parts while the build consumes them (directed)
int load_build_file(eg_graph* g, const char* path, uint32_t V, int edge_bytes) {
    if (!path) {
        set_error("eg_load_directed_file: null path");
        return EG_ERR_INVALID;
    }
    if (edge_bytes != 8 && edge_bytes != 12) {
        set_error("eg_load_directed_file: edge_bytes must be 8 or 12");
        return EG_ERR_INVALID;
    }
    const int fd = open(path, O_RDONLY);
    if (fd < 0) {
        set_error("eg_load_directed_file: cannot open %s", path);
        return EG_ERR_INVALID;
    }
    struct stat st {};
    if (fstat(fd, &st) != 0 || (uint64_t)st.st_size % (uint64_t)edge_bytes != 0) {
        close(fd);
        set_error("eg_load_directed_file: %s is not a whole number of %d-byte records", path, edge_bytes);
        return EG_ERR_INVALID;
    }
    const uint64_t E = (uint64_t)st.st_size / (uint64_t)edge_bytes;
    if (E < kPipelinedLoadMin) {  // small: read it, then build
        close(fd);
        EG_TRY(load_file_impl(g, path, V, edge_bytes, 0));
        return build_structures(g, 1, 1);
    }
    // where the device reads pageable memory at the link's rate, the file's mapping goes up
    // directly, each part's pages touched by host threads just before its copy (a mapping the
    // device faults in page by page was slower than staging); else reader threads stage the file
    // through pinned buffers
    if (pageable_at_link_rate(g)) {
        const size_t bytes = (size_t)E * edge_bytes;
        void* map = mmap(nullptr, bytes, PROT_READ, MAP_SHARED, fd, 0);
        if (map != MAP_FAILED) {
            const int r = pipelined_load(g, static_cast<const uint8_t*>(map), -1, E, V, edge_bytes, true);
            munmap(map, bytes);
            close(fd);
            return r;
        }
    }
    const int r = pipelined_load(g, nullptr, fd, E, V, edge_bytes);
    close(fd);
    return r;
}

int load_file_impl(eg_graph* g, const char* path, uint32_t V, int edge_bytes, int symmetric) {
    if (!path) {
        set_error("eg_load_file: null path");
        return EG_ERR_INVALID;
    }
    const int fd = open(path, O_RDONLY);
    if (fd < 0) {
        set_error("eg_load_file: cannot open %s", path);
        return EG_ERR_INVALID;
    }
    struct stat st;
    if (fstat(fd, &st) != 0 || st.st_size < 0) {
        close(fd);
        set_error("eg_load_file: cannot stat %s", path);
        return EG_ERR_INVALID;
    }
    const uint64_t bytes = (uint64_t)st.st_size;
    if (edge_bytes > 0 && bytes % (uint64_t)edge_bytes) {
        close(fd);
        set_error("eg_load_file: %s holds %llu bytes, not a whole number of %d-byte records", path,
                  (unsigned long long)bytes, edge_bytes);
        return EG_ERR_INVALID;
    }
    const uint64_t E = edge_bytes > 0 ? bytes / (uint64_t)edge_bytes : 0;
    int st_load = prepare_load(g, E, V, edge_bytes, symmetric);
    if (st_load != EG_OK) {
        close(fd);
        return st_load;
    }
    // where the device reads pageable memory at the link's rate: the file's mapping goes up in
    // pieces, a helper thread touching the pages of piece i + 1 while piece i is copied
    if (bytes && pageable_at_link_rate(g)) {
        void* map = mmap(nullptr, (size_t)bytes, PROT_READ, MAP_SHARED, fd, 0);
        if (map != MAP_FAILED) {
            const uint8_t* src = static_cast<const uint8_t*>(map);
            constexpr size_t kPiece = 2 * kIngestPiece;
            const uint64_t npieces = (bytes + kPiece - 1) / kPiece;
            std::atomic<uint64_t> touched{0};
            std::atomic<bool> stop{false};
            auto toucher = [&] {
                for (uint64_t i = 0; i < npieces && !stop.load(std::memory_order_relaxed); ++i) {
                    const size_t off = (size_t)(i * kPiece);
                    touch_pages(src, off, (size_t)std::min<uint64_t>(kPiece, bytes - off));
                    touched.store(i + 1, std::memory_order_release);
                }
            };
            std::thread th;
            try {
                th = std::thread(toucher);
            } catch (...) {
                toucher();
            }
            cudaError_t e = cudaSuccess;
            for (uint64_t i = 0; i < npieces && e == cudaSuccess; ++i) {
                while (touched.load(std::memory_order_acquire) <= i) std::this_thread::yield();
                const size_t off = (size_t)(i * kPiece), n = (size_t)std::min<uint64_t>(kPiece, bytes - off);
                e = cudaMemcpyAsync(g->edges.as<uint8_t>() + off, src + off, n, cudaMemcpyDefault, g->stream);
            }
            stop.store(true, std::memory_order_relaxed);
            if (th.joinable()) th.join();
            const cudaError_t e2 = cudaStreamSynchronize(g->stream);  // the mapping is read until here
            munmap(map, (size_t)bytes);
            close(fd);
            if (e == cudaSuccess) e = e2;
            if (e != cudaSuccess) {
                g->V = 0;
                return cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__);
            }
            EG_TRY(validate_edges(g, E));
            if (symmetric) EG_TRY(symmetrize_edges(g, E));
            return EG_OK;
        }
    }
    {
        const int st = ensure_staging(g);
        if (st != EG_OK) {
            close(fd);
            return st;
        }
    }
    cudaEvent_t done[2] = {nullptr, nullptr};
    int status = EG_OK;
    for (int i = 0; i < 2 && status == EG_OK; ++i) {
        cudaError_t e = cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming);
        if (e != cudaSuccess) status = cuda_fail(e, "cudaEventCreate", __FILE__, __LINE__);
    }
    uint8_t* dst = g->edges.as<uint8_t>();
    ReaderPool pool(fd, std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
    for (uint64_t off = 0, piece = 0; status == EG_OK && off < bytes; off += kIngestPiece, ++piece) {
        const int slot = (int)(piece & 1);
        uint8_t* buf = static_cast<uint8_t*>(g->pinned) + slot * kIngestPiece;
        if (piece >= 2) {  // the copy that last used this buffer must have finished
            cudaError_t e = cudaEventSynchronize(done[slot]);
            if (e != cudaSuccess) {
                status = cuda_fail(e, "cudaEventSynchronize", __FILE__, __LINE__);
                break;
            }
        }
        const size_t n = (size_t)std::min<uint64_t>(kIngestPiece, bytes - off);
        if (!pool.read(buf, off, n)) {
            set_error("eg_load_file: short read of %s in the piece at byte %llu", path, (unsigned long long)off);
            status = EG_ERR_INVALID;
            break;
        }
        cudaError_t e = cudaMemcpyAsync(dst + off, buf, n, cudaMemcpyHostToDevice, g->stream);
        if (e == cudaSuccess) e = cudaEventRecord(done[slot], g->stream);
        if (e != cudaSuccess) status = cuda_fail(e, "cudaMemcpyAsync", __FILE__, __LINE__);
    }
    close(fd);
    cudaStreamSynchronize(g->stream);  // the staging buffers may be reused by the next call
    for (int i = 0; i < 2; ++i)
        if (done[i]) cudaEventDestroy(done[i]);
    if (status != EG_OK) {
        g->V = 0;  // no usable edge list
        return status;
    }
    EG_TRY(validate_edges(g, E));
    if (symmetric) EG_TRY(symmetrize_edges(g, E));
    return EG_OK;
}
}  // namespace eg

extern "C" {

int eg_build(eg_graph* g, int want_csr, int want_csc) {
    EG_TRY(check_graph(g, "eg_build"));
    if (g->V == 0) {
        set_error("eg_build: no edge list loaded");
        return EG_ERR_STATE;
    }
    free_batch_state(g);
    return build_structures(g, want_csr, want_csc);
}

int eg_load_directed_with_ids(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int where) {
    EG_TRY(check_graph(g, "eg_load_directed_with_ids"));
    if (V == 0 || (E > 0 && !edges) || E >= (1ull << 32) || (where != EG_HOST && where != EG_DEVICE)) {
        set_error("eg_load_directed_with_ids: need V > 0, an edge pointer, E < 2^32 and a valid `where`");
        return EG_ERR_INVALID;
    }
    g->built_csr = g->built_csc = false;
    g->eng.pull_ready = false;
    g->eng.pr_ready = false;
    free_batch_state(g);
    g->V = V;
    g->E = E;
    g->E_input = E;
    g->edge_bytes = 12;
    g->weighted = 1;
    g->symmetric = 0;
    g->edge_ids = true;
    EG_TRY(g->edges.reserve((size_t)E * 12 + 64));
    EG_TRY(g->bucketed.reserve((size_t)E * 8 + 64));
    if (E) {
        EG_CUDA(cudaMemcpyAsync(g->bucketed.ptr, edges, (size_t)E * 8,
                                where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, g->stream));
        EG_TRY(expand_with_ids(g, g->bucketed.as<uint8_t>(), E));
    }
    EG_TRY(validate_edges(g, E));
    return build_structures(g, 1, 1);
}

int eg_msbfs(eg_graph* g, const uint32_t* roots, int nroots, uint8_t* levels, int where, uint64_t* edges) {
    EG_TRY(check_graph(g, "eg_msbfs"));
    return run_msbfs(g, roots, nroots, levels, where, edges);
}

int eg_ppr(eg_graph* g, const float* weights, const uint32_t* seeds, int nseeds, float alpha, int iterations,
           float* out, int where) {
    EG_TRY(check_graph(g, "eg_ppr"));
    return run_ppr(g, weights, seeds, nseeds, alpha, iterations, out, where);
}

int eg_ppr_backward(eg_graph* g, const float* weights, const uint32_t* seeds, int nseeds, float alpha, int iterations,
                    const float* dl_dx, float* dl_dw, int where) {
    EG_TRY(check_graph(g, "eg_ppr_backward"));
    return run_ppr_backward(g, weights, seeds, nseeds, alpha, iterations, dl_dx, dl_dw, where);
}

int eg_sssp_batch(eg_graph* g, const uint32_t* sources, int nsources, float* dist, int where) {
    EG_TRY(check_graph(g, "eg_sssp_batch"));
    return run_sssp_batch(g, sources, nsources, dist, where);
}

int eg_load_directed(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes, int where) {
    if (where == EG_HOST && E >= eg::kPipelinedLoadMin && edges) {
        EG_TRY(check_graph(g, "eg_load_directed"));
        return eg::load_build_pipelined(g, edges, E, V, edge_bytes);
    }
    EG_TRY(eg_load_edges(g, edges, E, V, edge_bytes, 0, where));
    return eg_build(g, 1, 1);
}

int eg_load_undirected_from_directed(eg_graph* g, const void* edges, uint64_t E, uint32_t V, int edge_bytes,
                                     int where) {
    EG_TRY(eg_load_edges(g, edges, E, V, edge_bytes, 1, where));
    return eg_build(g, 1, 1);
}

int eg_get_info(eg_graph* g, eg_info* out) {
    EG_TRY(check_graph(g, "eg_get_info"));
    if (!out) {
        set_error("eg_get_info: null output");
        return EG_ERR_INVALID;
    }
    out->V = g->V;
    out->partitions = (uint32_t)g->partitions;
    out->E = g->E;
    out->ncompressed = g->built_csc ? g->ncompressed : 0;
    out->weighted = g->weighted;
    out->built_csr = g->built_csr;
    out->built_csc = g->built_csc;
    out->symmetric = g->symmetric;
    return EG_OK;
}

int eg_get_partition(eg_graph* g, uint32_t* partition_offset, uint32_t* local_offset) {
    EG_TRY(check_graph(g, "eg_get_partition"));
    if (g->part_off.empty()) {
        set_error("eg_get_partition: graph not built");
        return EG_ERR_STATE;
    }
    if (partition_offset) memcpy(partition_offset, g->part_off.data(), sizeof(uint32_t) * g->part_off.size());
    if (local_offset) memcpy(local_offset, g->local_off.data(), sizeof(uint32_t) * g->local_off.size());
    return EG_OK;
}

int eg_get_degrees(eg_graph* g, uint32_t* outdeg, uint32_t* indeg, int where) {
    EG_TRY(check_graph(g, "eg_get_degrees"));
    if (!g->built_csr && !g->built_csc) {
        set_error("eg_get_degrees: graph not built");
        return EG_ERR_STATE;
    }
    cudaMemcpyKind k = where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (outdeg) EG_CUDA(cudaMemcpyAsync(outdeg, g->outdeg.ptr, sizeof(uint32_t) * (size_t)g->V, k, g->stream));
    if (indeg) EG_CUDA(cudaMemcpyAsync(indeg, g->indeg.ptr, sizeof(uint32_t) * (size_t)g->V, k, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    return EG_OK;
}

int eg_get_csr(eg_graph* g, eg_csr_view* out) {
    EG_TRY(check_graph(g, "eg_get_csr"));
    if (!out) { set_error("eg_get_csr: null output"); return EG_ERR_INVALID; }
    if (!g->built_csr) { set_error("eg_get_csr: CSR not built"); return EG_ERR_STATE; }
    out->off = g->csr_off.as<uint64_t>();
    out->adj = g->csr_adj.as<uint32_t>();
    out->w = g->weighted ? g->csr_w.as<float>() : nullptr;
    out->bitmap = g->csr_bitmap.as<uint64_t>();
    return EG_OK;
}

int eg_get_csc(eg_graph* g, eg_csc_view* out) {
    EG_TRY(check_graph(g, "eg_get_csc"));
    if (!out) { set_error("eg_get_csc: null output"); return EG_ERR_INVALID; }
    if (!g->built_csc) { set_error("eg_get_csc: CSC not built"); return EG_ERR_STATE; }
    out->off = g->csc_off.as<uint64_t>();
    out->adj = g->csc_adj.as<uint32_t>();
    out->w = g->weighted ? g->csc_w.as<float>() : nullptr;
    out->cvert = g->cvert.as<uint32_t>();
    out->cidx = g->cidx.as<uint64_t>();
    return EG_OK;
}

static int copy_dev(eg_graph* g, void* dst, const void* src, size_t bytes, int where) {
    if (!dst || !bytes) return EG_OK;
    EG_CUDA(cudaMemcpyAsync(dst, src, bytes, where == EG_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            g->stream));
    return EG_OK;
}

int eg_copy_csr(eg_graph* g, uint64_t* off, uint32_t* adj, float* w, uint64_t* bitmap, int where) {
    EG_TRY(check_graph(g, "eg_copy_csr"));
    if (!g->built_csr) { set_error("eg_copy_csr: CSR not built"); return EG_ERR_STATE; }
    const size_t P = (size_t)g->partitions, V = g->V;
    EG_TRY(copy_dev(g, off, g->csr_off.ptr, sizeof(uint64_t) * P * (V + 1), where));
    EG_TRY(copy_dev(g, adj, g->csr_adj.ptr, sizeof(uint32_t) * g->E, where));
    if (g->weighted) EG_TRY(copy_dev(g, w, g->csr_w.ptr, sizeof(float) * g->E, where));
    EG_TRY(copy_dev(g, bitmap, g->csr_bitmap.ptr, sizeof(uint64_t) * P * (V / 64 + 1), where));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    return EG_OK;
}

int eg_copy_csc(eg_graph* g, uint64_t* off, uint32_t* adj, float* w, uint32_t* cvert, uint64_t* cidx, int where) {
    EG_TRY(check_graph(g, "eg_copy_csc"));
    if (!g->built_csc) { set_error("eg_copy_csc: CSC not built"); return EG_ERR_STATE; }
    const size_t P = (size_t)g->partitions, V = g->V;
    EG_TRY(copy_dev(g, off, g->csc_off.ptr, sizeof(uint64_t) * P * (V + 1), where));
    EG_TRY(copy_dev(g, adj, g->csc_adj.ptr, sizeof(uint32_t) * g->E, where));
    if (g->weighted) EG_TRY(copy_dev(g, w, g->csc_w.ptr, sizeof(float) * g->E, where));
    EG_TRY(copy_dev(g, cvert, g->cvert.ptr, sizeof(uint32_t) * g->ncompressed, where));
    EG_TRY(copy_dev(g, cidx, g->cidx.ptr, sizeof(uint64_t) * g->ncompressed, where));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    return EG_OK;
}

int eg_cpbt_partition(const uint32_t* deg, uint32_t V, int P, int S, uint64_t eta, int max_iterations, int dense,
                      int where, uint32_t* partition_offset, uint32_t* local_offset) {
    if (!deg || !partition_offset || V == 0) {
        set_error("eg_cpbt_partition: need degrees, output and V > 0");
        return EG_ERR_INVALID;
    }
    eg_graph* raw = nullptr;
    eg_config cfg = {eta, 1, 1, max_iterations, 0, nullptr};
    int dev = 0;
    cudaGetDevice(&dev);
    cfg.device = dev;
    EG_TRY(eg_create(&raw, &cfg));
    std::unique_ptr<eg_graph, HandleDeleter> g(raw);
    const uint32_t* d_deg = deg;
    DevBuf copy;
    if (where == EG_HOST) {
        EG_TRY(copy.reserve(sizeof(uint32_t) * (size_t)V));
        EG_CUDA(cudaMemcpyAsync(copy.ptr, deg, sizeof(uint32_t) * (size_t)V, cudaMemcpyHostToDevice, g->stream));
        d_deg = copy.as<uint32_t>();
    }
    std::vector<uint32_t> lo((size_t)P * (std::max(S, 1) + 1));
    EG_TRY(cpbt_device(g.get(), d_deg, V, P, S, eta, max_iterations, dense, partition_offset, lo.data()));
    if (local_offset) memcpy(local_offset, lo.data(), sizeof(uint32_t) * lo.size());
    return EG_OK;
}

int eg_optimal_offset(const uint64_t* a, uint32_t n, uint32_t k, uint32_t* offset) {
    if ((!a && n) || !offset || k < 1 || k > (uint32_t)kMaxPartitions) {
        set_error("eg_optimal_offset: need weights, output and 1 <= k <= %d", kMaxPartitions);
        return EG_ERR_INVALID;
    }
    eg_graph* raw = nullptr;
    eg_config cfg = {1, 1, 1, 1, 0, nullptr};
    int dev = 0;
    cudaGetDevice(&dev);
    cfg.device = dev;
    EG_TRY(eg_create(&raw, &cfg));
    std::unique_ptr<eg_graph, HandleDeleter> g(raw);
    DevBuf w;
    EG_TRY(w.reserve(sizeof(uint64_t) * ((size_t)n + 1)));
    if (n) EG_CUDA(cudaMemcpyAsync(w.ptr, a, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, g->stream));
    return cpbt_search(g.get(), w.as<uint64_t>(), n, (int)k, 1, offset, nullptr);
}

int eg_pagerank(eg_graph* g, int iterations, float damping, float* out, int where) {
    EG_TRY(check_graph(g, "eg_pagerank"));
    return run_pagerank(g, iterations, damping, out, where);
}

int eg_bfs(eg_graph* g, uint32_t root, uint32_t* level, uint32_t* parent, int where, uint64_t* reached) {
    EG_TRY(check_graph(g, "eg_bfs"));
    return run_bfs(g, root, level, parent, where, reached);
}

int eg_cc(eg_graph* g, uint32_t* label, int where) {
    EG_TRY(check_graph(g, "eg_cc"));
    return run_cc(g, label, where);
}

int eg_sssp(eg_graph* g, uint32_t root, float* dist, int where) {
    EG_TRY(check_graph(g, "eg_sssp"));
    return run_sssp(g, root, dist, where);
}

int eg_set_option(eg_graph* g, int option, int64_t value) {
    EG_TRY(check_graph(g, "eg_set_option"));
    switch (option) {
        case EG_OPT_BFS_DIRECTION:
            if (value < 0 || value > 2) break;
            g->bfs_direction = (int)value;
            return EG_OK;
        case EG_OPT_DENSE_DIVISOR:
            if (value < 1 || value > (1 << 30)) break;
            g->dense_div = (int)value;
            return EG_OK;
        case EG_OPT_CUDA_GRAPH:
            if (value < 0 || value > 3) break;
            g->use_cuda_graph = (int)value;
            return EG_OK;
        case EG_OPT_PULL_BLOCKS_PER_SM:
            if (value < 0 || value > 64) break;
            g->pull_blocks_per_sm = (int)value;
            return EG_OK;
        case EG_OPT_BATCH_WIDTH:
            if (value < 1 || value > 64) break;
            g->batch_width = (int)value;
            return EG_OK;
        case EG_OPT_SSSP_DELTA:
            if (value < -1 || value > (1ll << 40)) break;
            g->sssp_delta = value;
            return EG_OK;
        case EG_OPT_PR_RELABEL:
            if (value < -1 || value > 1) break;
            g->pr_relabel = (int)value;
            return EG_OK;
        case EG_OPT_BATCH_LAUNCH:
            if (value < 0 || value > 1) break;
            g->batch_launch = (int)value;
            return EG_OK;
        case EG_OPT_BATCH_DIVISOR:
            if (value < 0 || value > (1 << 30)) break;
            g->batch_div = (int)value;
            return EG_OK;
        case EG_OPT_MAX_ITERATIONS:
            if (value < 0 || value > INT32_MAX) break;
            g->max_iterations = (int)value;
            return EG_OK;
        case EG_OPT_BUILD_LAUNCH:
            if (value != 0 && value != 1) break;
            g->build_launch = (int)value;
            return EG_OK;
        default:
            set_error("eg_set_option: unknown option %d", option);
            return EG_ERR_INVALID;
    }
    set_error("eg_set_option: value %lld out of range for option %d", (long long)value, option);
    return EG_ERR_INVALID;
}

int eg_last_run(eg_graph* g, uint64_t* edges_processed, int* iterations, int* push_iters, int* pull_iters) {
    EG_TRY(check_graph(g, "eg_last_run"));
    if (edges_processed) *edges_processed = g->last_edges_processed;
    if (iterations) *iterations = g->last_iterations;
    if (push_iters) *push_iters = g->last_pushes;
    if (pull_iters) *pull_iters = g->last_pulls;
    return EG_OK;
}

int eg_profile_enable(eg_graph* g, int enable) {
    EG_TRY(check_graph(g, "eg_profile_enable"));
    g->prof.enabled = enable != 0;
    return EG_OK;
}

int eg_profile_reset(eg_graph* g) {
    EG_TRY(check_graph(g, "eg_profile_reset"));
    g->prof.clear();
    return EG_OK;
}

int eg_profile_read(eg_graph* g, eg_kernel_stat* out, int cap, int* count) {
    EG_TRY(check_graph(g, "eg_profile_read"));
    g->prof.collect();
    int i = 0;
    for (auto& kv : g->prof.stats) {
        if (out && i < cap) {
            memset(out[i].name, 0, sizeof(out[i].name));
            strncpy(out[i].name, kv.first.c_str(), sizeof(out[i].name) - 1);
            out[i].launches = kv.second.launches;
            out[i].ms = kv.second.ms;
        }
        ++i;
    }
    if (count) *count = i;
    return EG_OK;
}

int eg_selftest_bounded_wait(eg_graph* g, uint32_t spin_cap) {
    EG_TRY(check_graph(g, "eg_selftest_bounded_wait"));
    if (spin_cap < 1 || spin_cap > (1u << 22)) {
        set_error("eg_selftest_bounded_wait: spin_cap must be in 1..2^22");
        return EG_ERR_INVALID;
    }
    return selftest_bounded_wait(g, spin_cap);
}

int eg_selftest_grid_barrier(eg_graph* g, uint32_t spin_cap) {
    EG_TRY(check_graph(g, "eg_selftest_grid_barrier"));
    if (spin_cap < 1 || spin_cap > (1u << 22)) {
        set_error("eg_selftest_grid_barrier: spin_cap must be in 1..2^22");
        return EG_ERR_INVALID;
    }
    EG_CUDA(cudaSetDevice(g->device));
    return selftest_grid_barrier(g, spin_cap);
}

}  // extern "C"
