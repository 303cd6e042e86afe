// Helpers shared by the implicit-arrangement and material-interface extraction kernels.
#pragma once
#include <cub/cub.cuh>

#include <vector>

#include "device_common.cuh"
#include "launch.hpp"

namespace ria {
namespace xc {

constexpr int kBs = 256;

enum : uint64_t { OCC_SELF = 0, OCC_CORNER = 1, OCC_EDGE = 2, OCC_FACE = 3 };

struct U4 {
    uint32_t a, b, c, d;
};
struct U4Sum {
    __host__ __device__ U4 operator()(const U4& x, const U4& y) const {
        return U4{x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d};
    }
};

__device__ __forceinline__ int local_func(uint64_t mask, int j) {  // j-th set bit of mask
    for (int i = 0; i < j; ++i) mask &= mask - 1;
    return __ffsll((long long)mask) - 1;
}

// per-active-tet extraction counts widened for the scans
static __global__ void k_base_in(int64_t A, const IASum4* __restrict__ sum, U4* __restrict__ out) {
    int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= A) return;
    IASum4 s = sum[a];
    out[a] = U4{s.a, s.b, s.c, s.d};
}

// p[idx] = a[n-1] + b[n-1] (the total of an exclusive scan), or 0 when n == 0
static __global__ void k_set_last(int64_t* p, int64_t idx, const uint32_t* a, const uint32_t* b, int64_t n) {
    p[idx] = n ? (int64_t)a[n - 1] + (int64_t)b[n - 1] : 0;
}

inline unsigned nblk(int64_t n) { return (unsigned)((n + kBs - 1) / kBs); }

inline uint64_t pow2_at_least(uint64_t x) {
    uint64_t p = 1024;
    while (p < x) p <<= 1;
    return p;
}

// stream-ordered device allocations released when the pool goes out of scope
struct Pool {
    cudaStream_t s;
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    template <class T>
    T* get(int64_t n) {
        void* p = nullptr;
        if (n <= 0) n = 1;
        cudaError_t e = cudaMallocAsync(&p, sizeof(T) * (size_t)n, s);
        if (e != cudaSuccess) {
            err = e;
            return nullptr;
        }
        ptrs.push_back(p);
        return (T*)p;
    }
    ~Pool() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
};

inline cudaError_t exscan_u32(const uint32_t* in, uint32_t* out, int64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, s);
    void* tmp = nullptr;
    cudaError_t e = cudaMallocAsync(&tmp, bytes, s);
    if (e != cudaSuccess) return e;
    cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, n, s);
    return cudaFreeAsync(tmp, s);
}

// total of an exclusive scan: out[n-1] + in[n-1] (synchronizes the stream)
inline cudaError_t scan_total(const uint32_t* in, const uint32_t* out, int64_t n, int64_t* total, cudaStream_t s) {
    if (n == 0) {
        *total = 0;
        return cudaSuccess;
    }
    uint32_t h[2];
    cudaError_t e = cudaMemcpyAsync(&h[0], in + n - 1, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h[1], out + n - 1, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    *total = (int64_t)h[0] + (int64_t)h[1];
    return e;
}

// Totals of several exclusive scans (out[n-1] + in[n-1] each), read with one synchronization.
struct ScanTotals {
    const uint32_t* in[8];
    const uint32_t* out[8];
    int64_t n[8];
    int count = 0;
    void add(const uint32_t* i, const uint32_t* o, int64_t len) {
        in[count] = i;
        out[count] = o;
        n[count] = len;
        ++count;
    }
};

static __global__ void k_scan_totals(ScanTotals r, int64_t* __restrict__ dst) {
    const int i = threadIdx.x;
    if (i < r.count) dst[i] = r.n[i] ? (int64_t)r.in[i][r.n[i] - 1] + (int64_t)r.out[i][r.n[i] - 1] : 0;
}

inline cudaError_t read_totals(const ScanTotals& r, int64_t* host, Pool& pool, cudaStream_t s) {
    int64_t* d = pool.get<int64_t>(8);
    if (pool.err) return pool.err;
    k_scan_totals<<<1, 32, 0, s>>>(r, d);
    note_launch();
    cudaError_t e = cudaMemcpyAsync(host, d, sizeof(int64_t) * (size_t)r.count, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e;
}

// exclusive scan of per-item U4 counts; returns the totals (synchronizes the stream)
inline cudaError_t exscan_u4(const U4* in, U4* out, int64_t n, U4* total, Pool& pool, cudaStream_t s) {
    *total = U4{0, 0, 0, 0};
    if (n == 0) return cudaSuccess;
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveScan(nullptr, bytes, in, out, U4Sum(), U4{0, 0, 0, 0}, n, s);
    void* tmp = pool.get<uint8_t>((int64_t)bytes);
    if (pool.err) return pool.err;
    cub::DeviceScan::ExclusiveScan(tmp, bytes, in, out, U4Sum(), U4{0, 0, 0, 0}, n, s);
    U4 h[2];
    cudaMemcpyAsync(&h[0], in + n - 1, sizeof(U4), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&h[1], out + n - 1, sizeof(U4), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    *total = U4Sum()(h[0], h[1]);
    return e;
}

}  // namespace xc
}  // namespace ria
