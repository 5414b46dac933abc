// eg_util.cu — status messages, device buffers, CUDA-event profiler, the R-MAT generator kernel.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include "../../include/endgraph_rmat.h"
#include "eg_common.cuh"
#include "eg_scan.cuh"

namespace eg {

static thread_local char t_err[512] = "";
std::atomic<unsigned long long> g_launches{0};

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
}

const char* error_text() { return t_err; }

int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    set_error("%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    return e == cudaErrorMemoryAllocation ? EG_ERR_NOMEM : EG_ERR_CUDA;
}

int DevBuf::reserve(size_t n) {
    if (n <= bytes && ptr) return EG_OK;
    release();
    size_t want = n ? n : 16;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e != cudaSuccess) {
        ptr = nullptr;
        bytes = 0;
        cudaGetLastError();
        set_error("device allocation of %zu bytes failed: %s", want, cudaGetErrorString(e));
        return EG_ERR_NOMEM;
    }
    bytes = want;
    return EG_OK;
}

void DevBuf::release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
}

cudaEvent_t Profiler::get() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

void Profiler::begin(cudaStream_t s, const char* name) {
    Pending p;
    p.name = name;
    p.a = get();
    p.b = get();
    cudaEventRecord(p.a, s);
    pending.push_back(p);
}

void Profiler::end(cudaStream_t s) {
    if (!pending.empty()) cudaEventRecord(pending.back().b, s);
}

void Profiler::collect() {
    for (auto& p : pending) {
        cudaEventSynchronize(p.b);
        float ms = 0;
        cudaEventElapsedTime(&ms, p.a, p.b);
        KernelStat& k = stats[p.name];
        k.launches += 1;
        k.ms += ms;
        pool.push_back(p.a);
        pool.push_back(p.b);
    }
    pending.clear();
}

void Profiler::clear() {
    collect();
    stats.clear();
}

Profiler::~Profiler() {
    for (auto& p : pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : pool) cudaEventDestroy(e);
}

int check_device_error(eg_graph* g, const char* what) {
    int h = 0;
    EG_CUDA(cudaMemcpyAsync(&h, g->err.ptr, sizeof(int), cudaMemcpyDeviceToHost, g->stream));
    EG_CUDA(cudaStreamSynchronize(g->stream));
    if (h) {
        cudaMemsetAsync(g->err.ptr, 0, sizeof(int), g->stream);
        set_error("%s: a bounded device wait gave up (code %d)", what, h);
        return EG_ERR_TIMEOUT;
    }
    return EG_OK;
}

// ---------------------------------------------------------------------------------------------
// scan of u32 counts into inclusive u64 offsets: out[i] = sum(in[0..i]), out[n] = total
struct EpiInclusive {
    uint64_t* out;
    __device__ void operator()(uint64_t i, uint64_t excl, uint32_t v) const { out[i] = excl + v; }
};

int scan_u32_to_u64(eg_graph* g, const uint32_t* in, uint64_t n, uint64_t* out_incl, uint64_t* total_dev) {
    return launch_scan(g, LoadU32{in}, EpiInclusive{out_incl}, n, total_dev, "scan_offsets");
}


// out[i] = sum(in[0..i)), out[n] = total
int scan_exclusive_u32(eg_graph* g, const uint32_t* in, uint64_t n, uint64_t* out) {
    return launch_scan(g, LoadU32{in}, EpiExclusive{out}, n, out + n, "scan_buckets");
}

// The bounded look-back wait, exercised: one CTA is launched for a two-tile scan with the ticket
// counter already at 1, so it takes tile 1 and waits for a tile-0 descriptor that nothing
// publishes.  After spin_cap polls it raises the error flag and finishes; the caller sees
// EG_ERR_TIMEOUT and the handle stays usable.
int selftest_bounded_wait(eg_graph* g, uint32_t spin_cap) {
    const uint64_t n = 2ull * kScanTile;
    EG_TRY(g->tmp64.reserve(sizeof(uint64_t) * n + sizeof(uint32_t) * n));
    uint64_t* out = g->tmp64.as<uint64_t>();
    uint32_t* in = reinterpret_cast<uint32_t*>(out + n);
    EG_TRY(g->scan.desc.reserve(2 * sizeof(uint64_t)));
    EG_TRY(g->scan.counter.reserve(16));
    EG_CUDA(cudaMemsetAsync(in, 0, sizeof(uint32_t) * n, g->stream));
    EG_CUDA(cudaMemsetAsync(g->scan.desc.ptr, 0, 2 * sizeof(uint64_t), g->stream));
    const uint32_t one = 1;
    EG_CUDA(cudaMemcpyAsync(g->scan.counter.ptr, &one, 4, cudaMemcpyHostToDevice, g->stream));
    k_scan<<<1, kScanThreads, 0, g->stream>>>(LoadU32{in}, EpiExclusive{out}, n, g->scan.desc.as<uint64_t>(),
                                              g->scan.counter.as<uint32_t>(), g->err.as<int>(), nullptr, spin_cap);
    EG_CHECK_LAUNCH("k_scan");
    return check_device_error(g, "eg_selftest_bounded_wait");
}

// The bounded grid barrier of the persistent kernels, exercised: a cooperative launch of four CTAs
// in which CTA 0 never arrives, so the other three poll until spin_cap runs out, raise the error
// flag and leave; the caller sees EG_ERR_TIMEOUT and the handle stays usable.
__global__ void k_grid_barrier_selftest(unsigned* words, int* err, uint32_t spin_cap) {
    if (blockIdx.x == 0) return;
    grid_sync_bounded(words, words + 1, err, spin_cap);
}

int selftest_grid_barrier(eg_graph* g, uint32_t spin_cap) {
    EG_TRY(g->tmp64.reserve(16));
    unsigned* words = reinterpret_cast<unsigned*>(g->tmp64.ptr);
    EG_CUDA(cudaMemsetAsync(words, 0, 16, g->stream));
    EG_CUDA(cudaMemsetAsync(g->err.ptr, 0, sizeof(int), g->stream));
    int* err = g->err.as<int>();
    void* kargs[] = {&words, &err, &spin_cap};
    EG_CUDA(cudaLaunchCooperativeKernel((const void*)k_grid_barrier_selftest, dim3(4), dim3(32), kargs, 0, g->stream));
    EG_CHECK_LAUNCH("k_grid_barrier_selftest");
    return check_device_error(g, "eg_selftest_grid_barrier");
}

// ---------------------------------------------------------------------------------------------
// compressed incoming index (core/graph.hpp:1144-1188): one (vertex, start) per non-empty list
// (p, v) plus a sentinel (V, partition end) per partition; cnt holds P*(V+1) counts with the
// (V+1)-th slot of each partition as the sentinel slot.
int compress_index(eg_graph* g, const uint32_t* cnt, uint64_t n, uint32_t V, const uint64_t* off, uint32_t* cvert,
                   uint64_t* cidx, uint64_t* cstart_dev) {
    int single = n == (uint64_t)V + 1;
    return launch_scan(g, LoadFlag{cnt, V, single}, EpiCompress{off, cvert, cidx, cstart_dev, V, single, cnt}, n,
                       nullptr, "compress_index");
}

// ---------------------------------------------------------------------------------------------
// R-MAT generator
__global__ void k_rmat(eg_rmat_params p, uint8_t* out, int rec, uint64_t E) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < E; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s, d;
        float w = 0.f;
        eg_rmat_edge(&p, i, &s, &d, rec == 12 ? &w : nullptr);
        uint32_t* r = reinterpret_cast<uint32_t*>(out + i * (uint64_t)rec);
        r[0] = s;
        r[1] = d;
        if (rec == 12) r[2] = __float_as_uint(w);
    }
}

}  // namespace eg

extern "C" int eg_generate_rmat(void* d_edges, int edge_bytes, uint64_t E, uint32_t V, double a, double b, double c,
                                uint64_t seed, int permute, float w_lo, float w_hi, void* stream) {
    if (!d_edges && E) { eg::set_error("eg_generate_rmat: null output"); return EG_ERR_INVALID; }
    if (edge_bytes != 8 && edge_bytes != 12) { eg::set_error("eg_generate_rmat: edge_bytes must be 8 or 12"); return EG_ERR_INVALID; }
    if (V == 0) { eg::set_error("eg_generate_rmat: V must be positive"); return EG_ERR_INVALID; }
    if (!(a >= 0 && b >= 0 && c >= 0 && a + b + c < 1.0)) { eg::set_error("eg_generate_rmat: need a,b,c >= 0, a+b+c < 1"); return EG_ERR_INVALID; }
    if (E == 0) return EG_OK;
    eg_rmat_params p;
    eg_rmat_init(&p, V, E, a, b, c, seed, (uint32_t)(permute != 0), w_lo, w_hi);
    eg::k_rmat<<<eg::grid_for(E, 256, 152u * 32u), 256, 0, (cudaStream_t)stream>>>(p, (uint8_t*)d_edges, edge_bytes, E);
    EG_CHECK_LAUNCH("k_rmat");
    return EG_OK;
}
