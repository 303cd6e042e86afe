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

// ---- per-vertex keys of the records: the reference's dedup keys (implicit arrangement
// src/extract_mesh.cpp:94-230, material interface :654-819)

// iso flags of the local vertices of an IA record (vertex ids below 256)
__device__ __forceinline__ void iso_vertex_flags(const IAView& r, uint64_t iso[4]) {
    iso[0] = iso[1] = iso[2] = iso[3] = 0;
    int off = 0;
    for (int f = 0; f < r.nf; ++f) {
        int L = r.len(f);
        if (r.plane_is_iso(r.supp(f)))
            for (int t = 0; t < L; ++t) {
                int v = r.loopv(off + t);
                iso[v >> 6] |= 1ull << (v & 63);
            }
        off += L;
    }
}

__device__ __forceinline__ int iso_rank(const uint64_t iso[4], int v) {
    int n = 0;
    for (int w = 0; w < (v >> 6); ++w) n += __popcll(iso[w]);
    return n + __popcll(iso[v >> 6] & ((1ull << (v & 63)) - 1));
}

struct VertKey {
    int type;       // 1 corner, 2 edge, 3 face, 4 interior (simplex size)
    int64_t sv[4];  // simplex vertex ids
    int fn[3];      // global function ids
};

__device__ __forceinline__ VertKey ia_vertex_key(const IAView& r, int j, const int64_t tv[4], uint64_t mask) {
    VertKey k;
    const uint8_t* lab = r.vlab + 3 * j;
    int nb = 0, bnd[3];
    int ni = 0;
    k.fn[0] = k.fn[1] = k.fn[2] = -1;
    for (int t = 0; t < 3; ++t) {
        if (lab[t] > 3)
            k.fn[ni++] = local_func(mask, lab[t] - 4);
        else
            bnd[nb++] = lab[t];
    }
    for (int c = 0; c < 4; ++c) k.sv[c] = -1;
    switch (nb) {
        case 3: {
            int c0 = 0;
            for (int c = 0; c < 4; ++c)
                if (c != bnd[0] && c != bnd[1] && c != bnd[2]) c0 = c;
            k.type = 1;
            k.sv[0] = tv[c0];
            break;
        }
        case 2: {
            int n = 0;
            for (int c = 0; c < 4; ++c)
                if (c != bnd[0] && c != bnd[1]) k.sv[n++] = tv[c];
            if (k.sv[0] > k.sv[1]) {
                int64_t x = k.sv[0];
                k.sv[0] = k.sv[1];
                k.sv[1] = x;
            }
            k.type = 2;
            break;
        }
        case 1: {
            int n = 0;
            for (int c = 0; c < 4; ++c)
                if (c != bnd[0]) k.sv[n++] = tv[c];
            for (int x = 1; x < 3; ++x)
                for (int y = x; y > 0 && k.sv[y - 1] > k.sv[y]; --y) {
                    int64_t s = k.sv[y];
                    k.sv[y] = k.sv[y - 1];
                    k.sv[y - 1] = s;
                }
            k.type = 3;
            break;
        }
        default:
            for (int c = 0; c < 4; ++c) k.sv[c] = tv[c];
            k.type = 4;
    }
    return k;
}

// ia_vertex_key's result computed on registers only (no locally indexed arrays): the labels are
// sorted, so the tet-face labels (below 4) come first and the function labels after them in order.
__device__ __forceinline__ int64_t pick4(int64_t t0, int64_t t1, int64_t t2, int64_t t3, int c) {
    return c == 0 ? t0 : (c == 1 ? t1 : (c == 2 ? t2 : t3));
}

__device__ __forceinline__ VertKey ia_vertex_key_r(const uint8_t* lab, int64_t t0, int64_t t1, int64_t t2,
                                                   int64_t t3, uint64_t mask) {
    VertKey k;
    const int l0 = lab[0], l1 = lab[1], l2 = lab[2];
    const int nb = (l0 < 4 ? 1 : 0) + (l1 < 4 ? 1 : 0) + (l2 < 4 ? 1 : 0);
    k.fn[0] = nb <= 2 ? local_func(mask, (nb == 0 ? l0 : (nb == 1 ? l1 : l2)) - 4) : -1;
    k.fn[1] = nb <= 1 ? local_func(mask, (nb == 0 ? l1 : l2) - 4) : -1;
    k.fn[2] = nb == 0 ? local_func(mask, l2 - 4) : -1;
    const uint32_t fm = (l0 < 4 ? 1u << l0 : 0u) | (l1 < 4 ? 1u << l1 : 0u) | (l2 < 4 ? 1u << l2 : 0u);
    const uint32_t cm = 0xFu & ~fm;  // the corners off every face label, ascending
    const int ca = __ffs(cm) - 1;
    const uint32_t cm2 = cm & (cm - 1);
    const int cb = __ffs(cm2) - 1;
    const int cc = __ffs(cm2 & (cm2 - 1)) - 1;
    k.sv[0] = k.sv[1] = k.sv[2] = k.sv[3] = -1;
    if (nb == 3) {
        k.type = 1;
        k.sv[0] = pick4(t0, t1, t2, t3, ca);
    } else if (nb == 2) {
        const int64_t x = pick4(t0, t1, t2, t3, ca), y = pick4(t0, t1, t2, t3, cb);
        k.type = 2;
        k.sv[0] = x < y ? x : y;
        k.sv[1] = x < y ? y : x;
    } else if (nb == 1) {
        int64_t x = pick4(t0, t1, t2, t3, ca), y = pick4(t0, t1, t2, t3, cb), z = pick4(t0, t1, t2, t3, cc);
        if (y < x) {
            const int64_t u = x;
            x = y;
            y = u;
        }
        if (z < y) {
            const int64_t u = y;
            y = z;
            z = u;
        }
        if (y < x) {
            const int64_t u = x;
            x = y;
            y = u;
        }
        k.type = 3;
        k.sv[0] = x;
        k.sv[1] = y;
        k.sv[2] = z;
    } else {
        k.type = 4;
        k.sv[0] = t0;
        k.sv[1] = t1;
        k.sv[2] = t2;
        k.sv[3] = t3;
    }
    return k;
}

struct MIKey {
    int type;  // 1 corner, 2 edge, 3 face, 4 interior, 0 not on an interface
    int64_t sv[4];
    int mats[4];
};

__device__ __forceinline__ int corner_of(const uint8_t* lab, int nb) {
    for (int c = 0; c < 4; ++c) {
        bool used = false;
        for (int t = 0; t < nb; ++t) used = used || lab[t] == c;
        if (!used) return c;
    }
    return 0;
}

__device__ __forceinline__ MIKey mi_vertex_key(const MIView& r, int j, const int64_t tv[4], uint64_t mask) {
    MIKey k;
    const uint8_t* lab = r.vlab + 4 * j;
    int nb = 0, nm = 0;
    uint8_t bnd[4];
    for (int t = 0; t < 4; ++t) {
        k.sv[t] = -1;
        k.mats[t] = -1;
    }
    int ms[4];
    for (int t = 0; t < 4; ++t) {
        if (lab[t] > 3)
            ms[nm++] = local_func(mask, lab[t] - 4);
        else
            bnd[nb++] = lab[t];
    }
    switch (nb) {
        case 3:
            k.type = 1;
            k.sv[0] = tv[corner_of(bnd, 3)];
            break;
        case 2: {
            int n = 0;
            for (int c = 0; c < 4; ++c)
                if (c != bnd[0] && c != bnd[1]) k.sv[n++] = tv[c];
            if (k.sv[0] > k.sv[1]) {
                int64_t x = k.sv[0];
                k.sv[0] = k.sv[1];
                k.sv[1] = x;
            }
            k.mats[0] = ms[0] < ms[1] ? ms[0] : ms[1];
            k.mats[1] = ms[0] < ms[1] ? ms[1] : ms[0];
            k.type = 2;
            break;
        }
        case 1: {
            int n = 0;
            for (int c = 0; c < 4; ++c)
                if (c != bnd[0]) k.sv[n++] = tv[c];
            for (int x = 1; x < 3; ++x)
                for (int y = x; y > 0 && k.sv[y - 1] > k.sv[y]; --y) {
                    int64_t s = k.sv[y];
                    k.sv[y] = k.sv[y - 1];
                    k.sv[y - 1] = s;
                }
            for (int x = 0; x < 3; ++x) k.mats[x] = ms[x];
            for (int x = 1; x < 3; ++x)
                for (int y = x; y > 0 && k.mats[y - 1] > k.mats[y]; --y) {
                    int s = k.mats[y];
                    k.mats[y] = k.mats[y - 1];
                    k.mats[y - 1] = s;
                }
            k.type = 3;
            break;
        }
        default:
            for (int c = 0; c < 4; ++c) {
                k.sv[c] = tv[c];
                k.mats[c] = ms[c];
            }
            k.type = 4;
    }
    return k;
}

// per-active-tet extraction counts widened for the scans
static __global__ void k_base_in(int64_t A, const IASum4* __restrict__ sum, U4* __restrict__ out) {
    int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= A) return;
    IASum4 s = sum[a];
    out[a] = U4{s.a, s.b, s.c, s.d};
}

// per-tet offsets from per-active-tet offsets: off[t] = exclusive total before tet t
static __global__ void k_expand_offsets(int64_t T, int64_t A, const uint32_t* __restrict__ act_tet,
                                 const uint32_t* __restrict__ aoff, const uint32_t* __restrict__ asz,
                                 int64_t* __restrict__ toff) {
    const int64_t t = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (t > T) return;
    // number of active tets before t (binary search in the sorted act_tet)
    int64_t lo = 0, hi = A;
    while (lo < hi) {
        int64_t mid = (lo + hi) >> 1;
        if ((int64_t)act_tet[mid] < t) lo = mid + 1;
        else hi = mid;
    }
    toff[t] = lo == 0 ? 0 : (int64_t)aoff[lo - 1] + (int64_t)asz[lo - 1];
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

// stream-ordered device allocations released when the pool goes out of scope.  Buffers are carved,
// 256-byte aligned, out of chunks of at least 32 MB: a stage allocates its dozens of buffers with a
// few cudaMallocAsync calls (after a synchronization the device waits while the host issues them).
struct Pool {
    cudaStream_t s;
    std::vector<void*> ptrs;
    cudaError_t err = cudaSuccess;
    char* cur = nullptr;
    size_t left = 0;
    bool measuring = false;  // get() only adds up the bytes (reserve() then takes them in one allocation)
    size_t measured = 0;
    static constexpr size_t kChunk = 32ull << 20;
    template <class T>
    T* get(int64_t n) {
        if (n <= 0) n = 1;
        const size_t bytes = (sizeof(T) * (size_t)n + 255) & ~(size_t)255;
        if (measuring) {
            measured += bytes;
            return nullptr;
        }
        if (bytes <= left) {
            T* p = (T*)cur;
            cur += bytes;
            left -= bytes;
            return p;
        }
        const size_t size = bytes < kChunk ? kChunk : bytes;
        void* p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, size, s);
        if (e != cudaSuccess) {
            err = e;
            return nullptr;
        }
        ptrs.push_back(p);
        cur = (char*)p + bytes;
        left = size - bytes;
        return (T*)p;
    }
    // one chunk for `bytes` more (a call's buffers carved from it with no further allocation)
    void reserve(size_t bytes) {
        if (bytes <= left) return;
        void* p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, bytes, s);
        if (e != cudaSuccess) {
            err = e;
            return;
        }
        ptrs.push_back(p);
        cur = (char*)p;
        left = bytes;
    }
    ~Pool() {
        for (void* p : ptrs) cudaFreeAsync(p, s);
    }
};

// Several buffers filled with a 32-bit pattern in one launch (the dedup tables' empty keys and
// owners, the duplicate counters): one wide grid-stride pass instead of a memset per buffer.
// Buffers start 16-byte aligned (Pool hands out 256-byte aligned blocks) and hold whole words.
struct FillList {
    static constexpr int kMax = 16;
    uint32_t* p[kMax];
    uint64_t words[kMax];
    uint32_t val[kMax];
    int n = 0;
    bool overflow = false;  // more buffers than kMax: launch_fill fills none and reports it
    void add(void* ptr, uint64_t bytes, uint32_t v) {
        if (n >= kMax) {
            overflow = true;
            return;
        }
        p[n] = (uint32_t*)ptr;
        words[n] = bytes / 4;
        val[n] = v;
        ++n;
    }
};

static __global__ void __launch_bounds__(256) k_fill(FillList L) {
    const uint64_t tid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, nth = (uint64_t)gridDim.x * blockDim.x;
    for (int i = 0; i < L.n; ++i) {
        uint32_t* p = L.p[i];
        const uint64_t w = L.words[i], n4 = w / 4;
        const uint32_t v = L.val[i];
        uint4* q = reinterpret_cast<uint4*>(p);
        for (uint64_t u = tid; u < n4; u += nth) q[u] = make_uint4(v, v, v, v);
        for (uint64_t u = 4 * n4 + tid; u < w; u += nth) p[u] = v;
    }
}

inline cudaError_t launch_fill(const FillList& L, cudaStream_t s) {
    if (L.overflow) return cudaErrorInvalidValue;
    if (L.n == 0) return cudaSuccess;
    k_fill<<<152 * 8, 256, 0, s>>>(L);
    note_launch();
    return cudaSuccess;
}

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
