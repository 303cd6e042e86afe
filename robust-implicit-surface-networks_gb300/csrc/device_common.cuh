// Device infrastructure shared by the kernels: status word, tet5 grid, record views, hash table.
#pragma once
#include <cstdint>

#include "variants.cuh"

namespace ria {

// status bits raised by kernels; the host maps them to ria_status values
enum : uint32_t {
    ST_CAPACITY = 1u << 0,      // a per-tet record needed more room than the big variant has
    ST_EXACT = 1u << 1,         // an exact predicate overflowed its expansion capacity
    ST_HASH_FULL = 1u << 2,     // a dedup hash table ran out of slots
    ST_INTERNAL = 1u << 3,      // an inconsistency that exact arithmetic rules out
    ST_NONMANIFOLD = 1u << 4,   // a tet face shared by more than two tets
    ST_BADINPUT = 1u << 5,      // a tet refers to a vertex outside 0..n_pts-1
};

__device__ __forceinline__ void raise_status(uint32_t* st, uint32_t bits) { atomicOr(st, bits); }

// tet t of the tet5 grid with `res` cubes per axis (src/io.cpp:125-147).  Calls keep t below 2^31
// (the pipeline's limit on tets), so the cube and its coordinates come from 32-bit divisions (a
// 64-bit division is a long software sequence on the GPU); larger indices take the 64-bit path.
__device__ __forceinline__ void grid_tet(int64_t t, int64_t res, int64_t v[4]) {
    const int64_t N = res + 1;
    int64_t i, j, k;
    int sub;
    if (((uint64_t)t >> 31) == 0 && ((uint64_t)res >> 15) == 0) {
        const uint32_t tt = (uint32_t)t, R = (uint32_t)res;
        const uint32_t c = tt / 5u;
        sub = (int)(tt - 5u * c);
        const uint32_t rr = R * R;
        const uint32_t ii = c / rr;
        const uint32_t rem = c - ii * rr;
        const uint32_t jj = rem / R;
        i = ii;
        j = jj;
        k = rem - jj * R;
    } else {
        const int64_t c = t / 5;
        sub = (int)(t - 5 * c);
        i = c / (res * res);
        j = (c / res) % res;
        k = c % res;
    }
    int64_t v0 = i * N * N + j * N + k, v1 = (i + 1) * N * N + j * N + k;
    int64_t v2 = (i + 1) * N * N + (j + 1) * N + k, v3 = i * N * N + (j + 1) * N + k;
    int64_t v4 = v0 + 1, v5 = v1 + 1, v6 = v2 + 1, v7 = v3 + 1;
    if (((i + j + k) & 1) == 0) {
        switch (sub) {
            case 0: v[0] = v4; v[1] = v6; v[2] = v1; v[3] = v3; break;
            case 1: v[0] = v6; v[1] = v3; v[2] = v4; v[3] = v7; break;
            case 2: v[0] = v1; v[1] = v3; v[2] = v0; v[3] = v4; break;
            case 3: v[0] = v3; v[1] = v1; v[2] = v2; v[3] = v6; break;
            default: v[0] = v4; v[1] = v1; v[2] = v6; v[3] = v5; break;
        }
    } else {
        switch (sub) {
            case 0: v[0] = v7; v[1] = v0; v[2] = v2; v[3] = v5; break;
            case 1: v[0] = v2; v[1] = v3; v[2] = v0; v[3] = v7; break;
            case 2: v[0] = v5; v[1] = v7; v[2] = v0; v[3] = v4; break;
            case 3: v[0] = v7; v[1] = v2; v[2] = v6; v[3] = v5; break;
            default: v[0] = v0; v[1] = v1; v[2] = v2; v[3] = v5; break;
        }
    }
}

// Tet source: an explicit T x 4 array or the tet5 grid.
struct TetSrc {
    const int64_t* tets;  // nullptr for the grid
    int64_t res;
    __device__ __forceinline__ void get(int64_t t, int64_t v[4]) const {
        if (tets) {
            for (int c = 0; c < 4; ++c) v[c] = tets[4 * t + c];
        } else {
            grid_tet(t, res, v);
        }
    }
};

// Point source: an explicit V x 3 array or the per-axis grid coordinates (src/io.cpp:104-106),
// coords[a * N + n] with N = res + 1.
struct PtSrc {
    const double* pts;     // nullptr for the grid
    const double* coords;
    int N;
    __device__ __forceinline__ void get(int64_t v, double p[3]) const {
        if (pts) {
            p[0] = pts[3 * v];
            p[1] = pts[3 * v + 1];
            p[2] = pts[3 * v + 2];
        } else {
            const int vi = (int)v;
            p[0] = coords[vi / (N * N)];
            p[1] = coords[N + (vi / N) % N];
            p[2] = coords[2 * N + vi % N];
        }
    }
};

__device__ __forceinline__ int rd16(const uint8_t* p) { return p[0] | (p[1] << 8); }

// ---- canonical record views (layout in include/ria.h)
struct IAView {
    int k, nv, nf, nc;
    const uint8_t* rep;
    const uint8_t* vlab;
    const uint8_t* faces;
    const uint8_t* loops;
    __device__ __forceinline__ void init(const uint8_t* b) {
        k = b[1];
        nv = rd16(b + 2);
        nf = rd16(b + 4);
        nc = rd16(b + 6);
        rep = b + 10;
        vlab = rep + k;
        faces = vlab + 3 * nv;
        loops = faces + 8 * nf;
    }
    __device__ __forceinline__ int supp(int f) const { return faces[8 * f]; }
    __device__ __forceinline__ bool bnd(int f) const { return faces[8 * f + 1] & 1; }
    __device__ __forceinline__ int pos(int f) const { return rd16(faces + 8 * f + 2); }
    __device__ __forceinline__ int neg(int f) const { return rd16(faces + 8 * f + 4); }
    __device__ __forceinline__ int len(int f) const { return rd16(faces + 8 * f + 6); }
    // sign vector of cell c (bit 4+j: positive side of inserted plane 4+j); b is the record start
    __device__ __forceinline__ uint64_t cell(const uint8_t* b, int c) const {
        const uint8_t* p = loops + 2 * rd16(b + 8) + 8 * c;
        uint64_t x = 0;
        for (int i = 7; i >= 0; --i) x = (x << 8) | p[i];
        return x;
    }
    __device__ __forceinline__ int loopv(int idx) const { return rd16(loops + 2 * idx); }
    __device__ __forceinline__ bool plane_is_iso(int p) const {
        if (p > 3) return true;
        for (int j = 0; j < k; ++j)
            if (rep[j] == p) return true;
        return false;
    }
    // local implicit index (0-based) of the function carried by supporting plane p
    __device__ __forceinline__ int plane_func_local(int p) const {
        if (p > 3) return p - 4;
        for (int j = 0; j < k; ++j)
            if (rep[j] == p) return j;
        return -1;
    }
};

struct MIView {
    int k, nv, nf, nc;
    const uint8_t* rep;
    const uint8_t* vlab;
    const uint8_t* faces;
    const uint8_t* loops;
    const uint8_t* cells;
    __device__ __forceinline__ void init(const uint8_t* b) {
        k = b[1];
        nv = rd16(b + 2);
        nf = rd16(b + 4);
        nc = rd16(b + 6);
        int nloop = rd16(b + 8);
        rep = b + 10;
        vlab = rep + k;
        faces = vlab + 4 * nv;
        loops = faces + 4 * nf;
        cells = loops + 2 * nloop;
    }
    __device__ __forceinline__ int pos(int f) const { return faces[4 * f]; }
    __device__ __forceinline__ int neg(int f) const { return faces[4 * f + 1]; }
    __device__ __forceinline__ int len(int f) const { return rd16(faces + 4 * f + 2); }
    __device__ __forceinline__ int loopv(int idx) const { return rd16(loops + 2 * idx); }
};

__device__ __forceinline__ int ia_record_size(const uint8_t* b) {
    int k = b[1], nv = rd16(b + 2), nf = rd16(b + 4), nc = rd16(b + 6), nl = rd16(b + 8);
    return 10 + k + 3 * nv + 8 * nf + 2 * nl + 8 * nc;
}
__device__ __forceinline__ int mi_record_size(const uint8_t* b) {
    int k = b[1], nv = rd16(b + 2), nf = rd16(b + 4), nc = rd16(b + 6), nl = rd16(b + 8);
    return 10 + k + 4 * nv + 4 * nf + 2 * nl + nc;
}

// A record descriptor: bit 63 set -> entry of the per-device lookup table; bit 62 set -> offset in
// the heap of the exact (big) variant; else an offset in the heap of the fast variant.
constexpr uint64_t kTableBit = 1ull << 63;
constexpr uint64_t kBigHeapBit = 1ull << 62;

struct RecSrc {
    const uint8_t* heap;
    const uint8_t* heap_big;
    const uint8_t* table;
    const uint32_t* table_off;
    __device__ __forceinline__ const uint8_t* get(uint64_t d) const {
        if (d & kTableBit) return table + table_off[d & 0xFFFFFFFFull];
        if (d & kBigHeapBit) return heap_big + (d & ~kBigHeapBit);
        return heap + d;
    }
};

// ---- open-addressing hash table with 128-bit keys (first occurrence by atomicMin)
struct HashTab {
    ulonglong2* keys;  // all bits set = empty
    uint32_t* owner;   // smallest occurrence position seen for the key
    uint64_t cap_mask;
    uint64_t probe_limit = 0;  // probes before an insert gives up (0: the whole table)
};

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return x;
}

__device__ __forceinline__ bool cas128(ulonglong2* addr, uint64_t new_lo, uint64_t new_hi, uint64_t& old_lo,
                                       uint64_t& old_hi) {
    uint64_t olo, ohi;
    const uint64_t cmp = ~0ull;
    asm volatile(
        "{\n\t.reg .b128 c, n, o;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 n, {%4, %5};\n\t"
        "atom.global.cas.b128 o, [%6], c, n;\n\t"
        "mov.b128 {%0, %1}, o;\n\t}"
        : "=l"(olo), "=l"(ohi)
        : "l"(cmp), "l"(cmp), "l"(new_lo), "l"(new_hi), "l"(addr)
        : "memory");
    old_lo = olo;
    old_hi = ohi;
    return olo == cmp && ohi == cmp;
}

// Open addressing with 64-bit keys (all bits set = empty), for keys that pack into one word.
struct HashTab64 {
    unsigned long long* keys;
    uint32_t* owner;
    uint64_t cap_mask;
    uint64_t probe_limit = 0;  // probes before an insert gives up (0: the whole table)
};

__device__ __forceinline__ int64_t ht64_insert_min(const HashTab64& h, uint64_t key, uint32_t pos) {
    uint64_t slot = mix64(key) & h.cap_mask;
    const uint64_t lim = h.probe_limit ? h.probe_limit : h.cap_mask + 1;
    for (uint64_t probe = 0; probe < lim; ++probe) {
        const unsigned long long old = atomicCAS(&h.keys[slot], ~0ull, (unsigned long long)key);
        if (old == ~0ull || old == key) {
            atomicMin(&h.owner[slot], pos);
            return (int64_t)slot;
        }
        slot = (slot + 1) & h.cap_mask;
    }
    return -1;
}

// Insert (k0, k1) and lower its owner to `pos`; returns the slot or -1 when the table is full.
__device__ __forceinline__ int64_t ht_insert_min(const HashTab& h, uint64_t k0, uint64_t k1, uint32_t pos) {
    uint64_t slot = mix64(k0 * 0x9E3779B97F4A7C15ull ^ mix64(k1)) & h.cap_mask;
    const uint64_t lim = h.probe_limit ? h.probe_limit : h.cap_mask + 1;
    for (uint64_t probe = 0; probe < lim; ++probe) {
        uint64_t olo, ohi;
        if (cas128(&h.keys[slot], k0, k1, olo, ohi) || (olo == k0 && ohi == k1)) {
            atomicMin(&h.owner[slot], pos);
            return (int64_t)slot;
        }
        slot = (slot + 1) & h.cap_mask;
    }
    return -1;
}

}  // namespace ria
