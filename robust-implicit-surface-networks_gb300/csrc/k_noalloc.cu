// ria_compute_arrangement_batch_noalloc: the per-tet arrangement of ria_compute_arrangement_batch
// for callers that cannot allocate device memory.
//
// Who needs it: a caller whose device memory is entirely managed by someone else (for example a
// framework whose caching allocator already holds the GPU's memory, or an application that carves
// every buffer out of one arena reserved at start-up), and a caller in a latency-critical loop where
// cudaMalloc / cudaFree, which may synchronize the device, are not allowed.  Such a caller passes
// device buffers for the inputs and the outputs; every intermediate buffer (the record heaps, the
// deferred list, the counters) lives in one fixed array in this file, `g_noalloc_scratch`, which
// every GPU that loads the library holds until the process exits.
//
// Limits and behaviour:
//   * at most kNoAllocMaxTets tets per call (RIA_EINVAL beyond), and at most kNoAllocHeapBytes of
//     records per call (RIA_ECAPACITY beyond);
//   * the first call on a device looks up the array's device address there (cudaGetSymbolAddress);
//     make that first call before any stream capture;
//   * all calls share the array: the counters and the call's record descriptors are cleared at the
//     start of each call, the rest keeps the previous call's contents; the per-tet cuts' status is
//     checked before any record is sized or copied, so a failed call writes no records; calls that
//     overlap on the GPU (different streams, or different host threads) race on it and must be
//     serialized by the caller;
//   * nothing in this path calls cudaMalloc, cudaFree or an allocating library routine.  The
//     one-plane lookup table (allocated on first use by the other entry points) is not used here;
//     the result is the same.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "device_common.cuh"
#include "launch.hpp"

namespace ria {

namespace {

constexpr int64_t kNoAllocMaxTets = 4096;
constexpr int64_t kNoAllocHeapBytes = 8 << 20;  // records of both variants, per call

// layout of the scratch array (byte offsets)
constexpr size_t kOffHeap = 0;
constexpr size_t kOffDesc = kOffHeap + kNoAllocHeapBytes;
constexpr size_t kOffSum = kOffDesc + 8 * kNoAllocMaxTets;
constexpr size_t kOffList = kOffSum + sizeof(IASum4) * kNoAllocMaxTets;
constexpr size_t kOffDeferred = kOffList + 4 * kNoAllocMaxTets;
constexpr size_t kOffSizes = kOffDeferred + 4 * kNoAllocMaxTets;
constexpr size_t kOffCnt = kOffSizes + 4 * kNoAllocMaxTets;
constexpr size_t kScratchBytes = kOffCnt + 8 * 8;  // about 8.5 MB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// counters (cleared before this kernel): 0 status word, 1 record heap used, 2 deferred count,
// 4 malformed value_offsets
__global__ void k_na_init(unsigned char* scr, const uint32_t* __restrict__ off, int64_t n) {
    uint32_t* list = (uint32_t*)(scr + kOffList);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        list[i] = (uint32_t)i;
        if (off[i + 1] < off[i] || off[i + 1] - off[i] > 60) atomicOr((uint32_t*)(scr + kOffCnt + 8 * 4), 1u);
    }
}

__global__ void k_na_sizes(unsigned char* scr, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t d = ((const uint64_t*)(scr + kOffDesc))[i];
    RecSrc rs{scr + kOffHeap, scr + kOffHeap, nullptr, nullptr};
    ((uint32_t*)(scr + kOffSizes))[i] = (uint32_t)ia_record_size(rs.get(d));
}

// exclusive scan of the n <= kNoAllocMaxTets record sizes in one block of 1024 threads
__global__ void __launch_bounds__(1024) k_na_offsets(unsigned char* scr, int64_t n, uint64_t* __restrict__ out_off,
                                                     uint64_t capacity) {
    __shared__ uint64_t part[1024];
    const uint32_t* sz = (const uint32_t*)(scr + kOffSizes);
    constexpr int per = kNoAllocMaxTets / 1024;
    const int t = threadIdx.x;
    uint64_t local[per];
    uint64_t s = 0;
    for (int j = 0; j < per; ++j) {
        const int64_t i = (int64_t)t * per + j;
        local[j] = s;
        s += i < n ? sz[i] : 0;
    }
    part[t] = s;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        uint64_t v = t >= d ? part[t - d] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    const uint64_t base = part[t] - s;
    for (int j = 0; j < per; ++j) {
        const int64_t i = (int64_t)t * per + j;
        if (i < n) out_off[i] = base + local[j];
    }
    if (t == 1023) {
        out_off[n] = part[1023];
        if (part[1023] > capacity) atomicOr((uint32_t*)(scr + kOffCnt), ST_CAPACITY);
    }
}

// one warp per tet: the lanes copy consecutive bytes, so a heavy tet's record (tens of KB) is copied
// 32 bytes per step and both sides are accessed in contiguous runs
__global__ void k_na_copy(unsigned char* scr, int64_t n, const uint64_t* __restrict__ off, uint8_t* __restrict__ dst,
                          uint64_t capacity) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= n || off[n] > capacity) return;
    const uint64_t d = ((const uint64_t*)(scr + kOffDesc))[i];
    RecSrc rs{scr + kOffHeap, scr + kOffHeap, nullptr, nullptr};
    const uint8_t* src = rs.get(d);
    const uint64_t o = off[i];
    const uint32_t len = (uint32_t)(off[i + 1] - o);
    for (uint32_t b = lane; b < len; b += 32) dst[o + b] = src[b];
}

std::mutex g_na_mu;
std::vector<unsigned char*> g_na_ptr;  // per device: address of g_noalloc_scratch there

}  // namespace

// Device address of the scratch array on the current device (looked up once per device).
static cudaError_t noalloc_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_na_mu);
    if ((int)g_na_ptr.size() <= dev) g_na_ptr.resize(dev + 1, nullptr);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_na_ptr[dev] = (unsigned char*)p;
    }
    *out = g_na_ptr[dev];
    return cudaSuccess;
}

// Returns a ria_status value; *msg receives a static message on failure.
int run_batch_noalloc(const double* d_values, const uint32_t* d_value_offsets, uint64_t n_tets, uint8_t* d_records,
                      uint64_t capacity, uint64_t* d_record_offsets, cudaStream_t s, const char** msg) {
    if (n_tets > (uint64_t)kNoAllocMaxTets) {
        *msg = "n_tets exceeds the 4096 tets of the no-allocation path";
        return RIA_EINVAL;
    }
    if (!d_values || !d_value_offsets || !d_records || !d_record_offsets) {
        *msg = "null argument";
        return RIA_EINVAL;
    }
    unsigned char* scr = nullptr;
    if (noalloc_scratch(&scr) != cudaSuccess) {
        *msg = "cudaGetSymbolAddress of the scratch array failed";
        return RIA_ECUDA;
    }
    const int64_t n = (int64_t)n_tets;
    unsigned long long* cnt = (unsigned long long*)(scr + kOffCnt);
    uint32_t* status = (uint32_t*)cnt;
    // the descriptors are cleared too: a tet whose cut fails writes none, and no later kernel may
    // read an offset left by an earlier call
    if (cudaMemsetAsync(cnt, 0, 8 * 8, s) != cudaSuccess ||
        (n_tets > 0 && cudaMemsetAsync(scr + kOffDesc, 0, 8 * n_tets, s) != cudaSuccess)) {
        *msg = "CUDA error";
        return RIA_ECUDA;
    }
    if (n > 0) {
        k_na_init<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(scr, d_value_offsets, n);
        note_launch();
    }
    unsigned long long h[8];
    if (cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "CUDA error";
        return RIA_ECUDA;
    }
    if (h[4]) {
        *msg = "value_offsets must be non-decreasing with at most 60 rows per tet";
        return RIA_EINVAL;
    }
    CutArgs ca{};
    ca.mi = false;
    ca.list = (const uint32_t*)(scr + kOffList);
    ca.n = n;
    ca.act_desc = (uint64_t*)(scr + kOffDesc);
    ca.act_sum = (IASum4*)(scr + kOffSum);
    ca.heap = scr + kOffHeap;
    ca.heap_used = cnt + 1;
    ca.heap_cap = (uint64_t)kNoAllocHeapBytes;
    ca.desc_bit = 0;
    ca.deferred = (uint32_t*)(scr + kOffDeferred);
    ca.n_deferred = (unsigned int*)(cnt + 2);
    ca.status = status;
    ca.values = d_values;
    ca.value_off = d_value_offsets;
    launch_cut_fast(ca, s);
    if (cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "CUDA error";
        return RIA_ECUDA;
    }
    const int64_t n_def = (int64_t)(h[2] & 0xFFFFFFFFull);
    if (n_def > 0) {
        CutArgs cb = ca;
        cb.list = (const uint32_t*)(scr + kOffDeferred);
        cb.n = n_def;
        // both variants append to the one record heap
        launch_cut_big(cb, s);
    }
    // every record must exist before the sizes are read: a failed cut leaves its descriptor unset
    if (cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "CUDA error";
        return RIA_ECUDA;
    }
    if ((uint32_t)h[0] & ST_INTERNAL) {
        *msg = "per-tet cut: internal consistency check failed";
        return RIA_EINTERNAL;
    }
    if ((uint32_t)h[0] & ST_EXACT) {
        *msg = "an exact predicate exceeded its expansion capacity";
        return RIA_EDEGENERATE;
    }
    if ((uint32_t)h[0] & ST_CAPACITY) {
        *msg = "the records exceed the 8 MiB record space of the no-allocation path, or a tet exceeds the "
               "per-tet capacity";
        return RIA_ECAPACITY;
    }
    if (n > 0) {
        k_na_sizes<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(scr, n);
        note_launch();
    }
    k_na_offsets<<<1, 1024, 0, s>>>(scr, n, d_record_offsets, capacity);
    note_launch();
    if (n > 0) {
        k_na_copy<<<(unsigned)((n * 32 + 127) / 128), 128, 0, s>>>(scr, n, d_record_offsets, d_records, capacity);
        note_launch();
    }
    if (cudaMemcpyAsync(h, cnt, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
        *msg = "CUDA error";
        return RIA_ECUDA;
    }
    const uint32_t st = (uint32_t)h[0];
    if (st & ST_INTERNAL) {
        *msg = "per-tet cut: internal consistency check failed";
        return RIA_EINTERNAL;
    }
    if (st & ST_CAPACITY) {
        *msg = "record buffer too small";
        return RIA_ECAPACITY;
    }
    return RIA_OK;
}

}  // namespace ria
