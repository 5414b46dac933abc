// eg_noalloc.cu — CPBT partitioning that allocates nothing.
//
// eg_cpbt_partition_noalloc is the partitioner of eg_cpbt_partition for callers that cannot call
// cudaMalloc: a caller that runs inside a fixed, pre-reserved device-memory budget, or that embeds
// the library in a process whose own allocator owns the device memory, or that must not pay the
// device-wide synchronisation cudaMalloc / cudaFree imply in the middle of its pipeline.  The caller
// passes the degree array and both outputs in device memory; every intermediate (page weights, their
// prefix, page boundaries) lives in the file-scope array below, which each GPU that loads the
// library holds until the process exits.
//
// The array is shared by all calls: calls on one device that overlap on the GPU (different streams,
// different host threads) race on it and must be serialised by the caller.  Its device address is
// looked up on the first call on a device, and again on the first call after a device reset (a
// new context); those calls should come before any stream capture.  Nothing in it has to
// start at zero: every element a call reads was written earlier in the same call.
#include <cuda.h>

#include <mutex>

#include "eg_common.cuh"

namespace eg {

// kernels of eg_build.cu
__global__ void k_page_weights(const uint32_t* __restrict__ deg, uint32_t V, uint32_t c1, uint32_t pm1, uint32_t T,
                               uint64_t eta, uint64_t* __restrict__ out, uint32_t pages);
__global__ void k_cpbt(const uint64_t* __restrict__ pw, uint32_t n, uint32_t P, uint32_t S, uint64_t* prefix_g,
                       uint32_t* page_off, uint32_t* local_page_off, int use_smem);

constexpr uint32_t kNaPages = (uint32_t)((EG_NOALLOC_MAX_V + kPageSize - 1) / kPageSize);
constexpr size_t kNaWeightsOff = 0;                                            // u64[pages]
constexpr size_t kNaPrefixOff = kNaWeightsOff + sizeof(uint64_t) * kNaPages;  // u64[pages + 1]
constexpr size_t kNaPageOffOff = kNaPrefixOff + sizeof(uint64_t) * (kNaPages + 1);
constexpr size_t kNaLocalOff = kNaPageOffOff + sizeof(uint32_t) * (EG_NOALLOC_MAX_PARTITIONS + 1);
constexpr size_t kNaBytes =
    kNaLocalOff + sizeof(uint32_t) * EG_NOALLOC_MAX_PARTITIONS * (EG_NOALLOC_MAX_SUB_PARTITIONS + 1);

static_assert(kNaBytes <= EG_NOALLOC_SCRATCH_BYTES, "scratch layout exceeds the documented size");
static __device__ __align__(256) unsigned char g_noalloc_scratch[EG_NOALLOC_SCRATCH_BYTES];

// page units -> vertex boundaries, with the reference's 32-bit arithmetic (core/graph.hpp:743-749,
// :774-780); one thread per partition
__global__ void k_cpbt_to_vertices(const uint32_t* __restrict__ page_off, const uint32_t* __restrict__ local_page_off,
                                   uint32_t V, int P, int S, uint32_t* __restrict__ part, uint32_t* __restrict__ local) {
    for (int p = threadIdx.x; p <= P; p += blockDim.x)
        part[p] = p == 0 ? 0u : (p == P ? V : page_off[p] * kPageSize);
    if (!local) return;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        const uint32_t pb = p == 0 ? 0u : page_off[p] * kPageSize;
        const uint32_t pe = p + 1 == P ? V : page_off[p + 1] * kPageSize;
        uint32_t* lo = local + (size_t)p * (S + 1);
        lo[0] = pb;
        lo[S] = pe;
        for (int i = 0; i < S - 1; ++i) lo[i + 1] = local_page_off[(size_t)p * (S + 1) + i + 1] * kPageSize + pb;
    }
}

// Device address of the scratch array, looked up with the device current and kept per device
// together with the unique id of the context it belongs to.  A context that is not the cached one
// (after cudaDeviceReset the runtime makes a new primary context and loads the module again) gets
// a fresh lookup, and the shared-memory attribute of k_cpbt is set again.  The context id comes
// from the driver (cuCtxGetCurrent / cuCtxGetId, reached through the runtime's entry-point query,
// so the library does not link libcuda); where it cannot be read, the first lookup per device is
// kept.
typedef CUresult (*PfnCtxGetCurrent)(CUcontext*);
typedef CUresult (*PfnCtxGetId)(CUcontext, unsigned long long*);

struct NaDevice {
    void* addr = nullptr;
    unsigned long long ctx_id = 0;
};
static std::mutex g_na_mutex;
static NaDevice g_na[128];

static unsigned long long current_context_id() {
    static bool queried = false;
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    if (!queried) {
        queried = true;
        cudaDriverEntryPointQueryResult q;
        void* f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PfnCtxGetCurrent>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(f);
    }
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
        return id;
    return 0;
}

static int noalloc_setup(int dev, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (dev < 0 || dev >= 128) {
        set_error("eg_cpbt_partition_noalloc: device ordinal %d unsupported", dev);
        return EG_ERR_INVALID;
    }
    NaDevice& d = g_na[dev];
    const unsigned long long id = current_context_id();
    if (!d.addr || (id != 0 && id != d.ctx_id)) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)", __FILE__, __LINE__);
        e = cudaFuncSetAttribute(k_cpbt, cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_cpbt)", __FILE__, __LINE__);
        d.addr = p;
        d.ctx_id = id ? id : current_context_id();  // the lookup above made the context current
    }
    *out = static_cast<unsigned char*>(d.addr);
    return EG_OK;
}

}  // namespace eg

extern "C" int eg_cpbt_partition_noalloc(const uint32_t* d_deg, uint32_t V, int P, int S, uint64_t eta,
                                         int max_iterations, int dense, uint32_t* d_partition_offset,
                                         uint32_t* d_local_offset, void* stream) {
    using namespace eg;
    if (!d_deg || !d_partition_offset || V == 0) {
        set_error("eg_cpbt_partition_noalloc: need a device degree array, a device output and V > 0");
        return EG_ERR_INVALID;
    }
    if (V > EG_NOALLOC_MAX_V || P < 1 || P > EG_NOALLOC_MAX_PARTITIONS || S < 1 || S > EG_NOALLOC_MAX_SUB_PARTITIONS) {
        set_error("eg_cpbt_partition_noalloc: limits are V <= %u, 1 <= P <= %d, 1 <= S <= %d (got V=%u P=%d S=%d); "
                  "use eg_cpbt_partition beyond them",
                  (unsigned)EG_NOALLOC_MAX_V, EG_NOALLOC_MAX_PARTITIONS, EG_NOALLOC_MAX_SUB_PARTITIONS, V, P, S);
        return EG_ERR_INVALID;
    }
    int dev = 0;
    EG_CUDA(cudaGetDevice(&dev));
    unsigned char* base = nullptr;
    EG_TRY(noalloc_setup(dev, &base));
    cudaStream_t st = (cudaStream_t)stream;
    uint64_t* pw = reinterpret_cast<uint64_t*>(base + kNaWeightsOff);
    uint64_t* prefix = reinterpret_cast<uint64_t*>(base + kNaPrefixOff);
    uint32_t* page_off = reinterpret_cast<uint32_t*>(base + kNaPageOffOff);
    uint32_t* local_page_off = reinterpret_cast<uint32_t*>(base + kNaLocalOff);
    const uint32_t pages = (uint32_t)(((uint64_t)V + kPageSize - 1) / kPageSize);
    k_page_weights<<<pages < 152u * 8u ? pages : 152u * 8u, 256, 0, st>>>(
        d_deg, V, (uint32_t)(1 + (P - 1) / 16), (uint32_t)(P - 1), dense ? (uint32_t)max_iterations : 1u, eta, pw, pages);
    EG_CHECK_LAUNCH("k_page_weights");
    const size_t smem = sizeof(uint64_t) * ((size_t)pages + 1);
    const int use_smem = smem <= 160 * 1024;
    k_cpbt<<<1, 1024, use_smem ? smem : 0, st>>>(pw, pages, (uint32_t)P, (uint32_t)S, prefix, page_off, local_page_off,
                                                 use_smem);
    EG_CHECK_LAUNCH("k_cpbt");
    k_cpbt_to_vertices<<<1, 128, 0, st>>>(page_off, local_page_off, V, P, S, d_partition_offset, d_local_offset);
    EG_CHECK_LAUNCH("k_cpbt_to_vertices");
    return EG_OK;
}
