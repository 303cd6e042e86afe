// Stage (c): the per-tet cut (src/implicit_arrangement.cpp:244-306, src/material_interface.cpp:288-351).
//
//   k_cut_fast   one thread per tet, state in local memory, FP64-filtered predicates only.  A tet
//                whose predicate the filter cannot decide, or that outgrows the small capacities,
//                is appended to a deferred list.
//   k_cut_big    one tet per block at a time, its state in dynamic shared memory, exact
//                predicates and large capacities; walks the deferred list.
//   k_build_table  the 81-pattern lookup tables (IA: one active plane; MI: two active
//                materials), computed on the device by the exact variant from one representative
//                tet per sign pattern (corner values in {-1, 0, 1}).
// Records are appended to a byte heap with an atomic bump pointer; their placement does not affect
// the result, which only depends on the per-tet record contents.
#include <type_traits>

#include "device_common.cuh"
#include "launch.hpp"
#include "lookup2.cuh"
#include "robust.cuh"
#include "cut_mi_warp.cuh"

namespace ria {

namespace {

constexpr int kFastMaxK = 8;

template <class Sum>
__device__ __forceinline__ IASum4 pack_sum(const Sum& s);
template <>
__device__ __forceinline__ IASum4 pack_sum<IASummary>(const IASummary& s) {
    return IASum4{s.n_iso_v, s.n_iso_f, s.n_iso_loop, s.n_bnd_f};
}
template <>
__device__ __forceinline__ IASum4 pack_sum<MISummary>(const MISummary& s) {
    return IASum4{s.n_mi_v, s.n_mi_f, s.n_mi_loop, s.n_bnd_f};
}

template <bool MI>
struct Traits;
template <>
struct Traits<false> {
    using Fast = IACutFast;
    using Mid = IACutMid;
    using Big = IACutBig;
    using Sum = IASummary;
};
template <>
struct Traits<true> {
    using Fast = MICutFast;
    using Mid = MICutMid;
    using Big = MICutBig;
    using Sum = MISummary;
};
constexpr int kMidMaxK = 16;

template <bool MI>
struct BigSlot {
    typename Traits<MI>::Big cut;
    double planes[4 * 64];
};

__device__ __forceinline__ int gather_planes(const CutArgs& a, uint32_t ai, double* planes, int kmax) {
    if (a.values) {
        const uint32_t r0 = a.value_off[ai], r1 = a.value_off[ai + 1];
        const int k = (int)(r1 - r0);
        if (k > kmax) return k;
        for (int i = 0; i < 4 * k; ++i) planes[i] = a.values[4 * (size_t)r0 + i];
        return k;
    }
    const uint32_t t = a.act_tet[ai];
    uint64_t m = a.act_mask[ai];
    const int k = __popcll(m);
    if (k > kmax) return k;
    int64_t v[4];
    TetSrc ts{a.d_tets, a.g.res};
    ts.get(t, v);
    int i = 0;
    while (m) {
        int j = __ffsll((long long)m) - 1;
        m &= m - 1;
        for (int c = 0; c < 4; ++c) planes[4 * i + c] = a.fv[v[c] * a.F + j];
        ++i;
    }
    return k;
}

// heap space for a record of `size` bytes; allocations are multiples of 8 bytes, so every record
// starts 8-byte aligned (the template relabels write whole words)
__device__ __forceinline__ unsigned long long heap_alloc(const CutArgs& a, int size) {
    return atomicAdd(a.heap_used, (unsigned long long)((size + 7) & ~7));
}

// returns the record's place in the heap; nullptr when the heap is full (the exact kernel then
// reports the capacity; the filtered kernels hand the tet to the exact kernel, whose heap is sized
// by the record bound)
template <class Cut, class Sum>
__device__ __forceinline__ const uint8_t* finish_cut(const CutArgs& a, uint32_t ai, Cut& c, int* size_out,
                                                     IASum4* sum_out, bool defer_when_full = false) {
    c.canonicalize();
    const int size = c.record_size();
    unsigned long long off = heap_alloc(a, size);
    if (off + size > a.heap_cap) {
        if (!defer_when_full) raise_status(a.status, ST_CAPACITY);
        return nullptr;
    }
    Sum s;
    c.emit(a.heap + off, s);
    const IASum4 ps = pack_sum<Sum>(s);
    a.act_desc[ai] = off | a.desc_bit;
    a.act_sum[ai] = ps;
    *size_out = size;
    *sum_out = ps;
    return a.heap + off;
}

// ---- secondary lookup: a device-wide cache of canonical records keyed by the combinatorial type
// (lookup2.cuh), kept for the life of the process.  A slot holds (key + 1) << 32 and either the
// entry of the published record or a claim (kClaim | call number): the lookup pass lets the first
// tet of a key claim it, that tet's cut publishes the record, and the key's other tets take the
// record afterwards, so a key is cut once per call however many tets share it.  A record is
// published after its bytes (fence, then CAS of its slot); readers fence after seeing the slot.
// Records depend only on the key, so racing publications of one key are interchangeable.  A claim
// left by another call (whose cut could not publish) may be taken over.
constexpr int kCacheProbes = 32;
constexpr uint32_t kClaim = 0xFFFF0000u;  // entries stay far below (kCacheEntries)

__device__ __forceinline__ uint32_t cache_hash(uint32_t key, uint32_t mask) {
    return (uint32_t)mix64((uint64_t)key) & mask;
}

// the entry of the key's record; -1 when absent, -2 when claimed and not yet published
__device__ __forceinline__ int cache_find(const CutArgs::Cache& c, uint32_t key) {
    const unsigned long long tag = (unsigned long long)(key + 1u) << 32;
    const uint32_t h = cache_hash(key, c.slot_mask);
    for (int p = 0; p < kCacheProbes; ++p) {
        const unsigned long long v = *reinterpret_cast<volatile const unsigned long long*>(&c.slots[(h + p) & c.slot_mask]);
        if (v == 0) return -1;
        if ((v & 0xFFFFFFFF00000000ull) == tag) {
            if ((uint32_t)v >= kClaim) return -2;
            __threadfence();
            return (int)(v & 0xFFFFFFFFull);
        }
    }
    return -1;
}

enum : int { CLAIM_OWNER = 0, CLAIM_PUBLISHED = 1, CLAIM_WAIT = 2, CLAIM_NONE = 3 };

// CLAIM_OWNER: this tet claimed the key (its cut publishes the record); CLAIM_PUBLISHED: the record
// is entry *j; CLAIM_WAIT: another tet of this call claimed it; CLAIM_NONE: no free slot in reach.
__device__ __forceinline__ int cache_claim(const CutArgs::Cache& c, uint32_t key, int* j) {
    const unsigned long long tag = (unsigned long long)(key + 1u) << 32;
    const unsigned long long mine = tag | (kClaim | (c.gen & 0xFFFFu));
    const uint32_t h = cache_hash(key, c.slot_mask);
    for (int p = 0; p < kCacheProbes; ++p) {
        unsigned long long* slot = &c.slots[(h + p) & c.slot_mask];
        unsigned long long v = *reinterpret_cast<volatile unsigned long long*>(slot);
        if (v == 0) {
            v = atomicCAS(slot, 0ull, mine);
            if (v == 0) return CLAIM_OWNER;
        }
        if ((v & 0xFFFFFFFF00000000ull) != tag) continue;
        if ((uint32_t)v < kClaim) {
            __threadfence();
            *j = (int)(uint32_t)v;
            return CLAIM_PUBLISHED;
        }
        if (v == mine) return CLAIM_WAIT;
        // a claim of another call: take it over, or learn what replaced it
        const unsigned long long w = atomicCAS(slot, v, mine);
        if (w == v) return CLAIM_OWNER;
        if (w == mine) return CLAIM_WAIT;
        if ((uint32_t)w < kClaim) {
            __threadfence();
            *j = (int)(uint32_t)w;
            return CLAIM_PUBLISHED;
        }
        return CLAIM_NONE;
    }
    return CLAIM_NONE;
}

// publish a record for the key: into an empty slot, over a claim, or not at all when the key is
// already published
__device__ __forceinline__ void cache_insert(const CutArgs::Cache& c, uint32_t key, const uint8_t* rec, int size,
                                             IASum4 sum) {
    const unsigned long long j = atomicAdd(c.next, 1ull);
    if (j >= c.cap) return;
    const unsigned long long off = atomicAdd(c.heap_used, (unsigned long long)((size + 7) & ~7));
    if (off + size > c.heap_cap) return;
    uint8_t* dst = c.table + c.heap_base + off;
    for (int i = 0; i < size; ++i) dst[i] = rec[i];
    c.table_off[kTablePatterns + j] = (uint32_t)(c.heap_base + off);
    c.table_sum[kTablePatterns + j] = sum;
    __threadfence();
    const unsigned long long tag = (unsigned long long)(key + 1u) << 32;
    const unsigned long long v = tag | j;
    const uint32_t h = cache_hash(key, c.slot_mask);
    for (int p = 0; p < kCacheProbes; ++p) {
        unsigned long long* slot = &c.slots[(h + p) & c.slot_mask];
        unsigned long long old = atomicCAS(slot, 0ull, v);
        if (old == 0) return;
        for (int t = 0; t < 4 && (old & 0xFFFFFFFF00000000ull) == tag; ++t) {
            if ((uint32_t)old < kClaim) return;  // published already
            const unsigned long long w = atomicCAS(slot, old, v);
            if (w == old) return;
            old = w;
        }
        if ((old & 0xFFFFFFFF00000000ull) == tag) return;
    }
}

// ---- seeding: the secondary lookup is filled once per process, when the mode's table is built,
// from synthetic configurations (the reference ships its two-plane and three-material tables
// precomputed): every row set with entries in {-2, ..., 2} (two planes: 5^8 sets) or {-1, 0, 1}
// (three materials: 3^12 sets), then pseudo-random real rows with some exact zeros.  A new key is
// claimed, cut by the small filtered variant and published; a key that variant cannot decide stays
// claimed, and a call takes it over.
constexpr int64_t kSeedRandom = 1 << 20;

__device__ __forceinline__ double seed_value(uint64_t t, int i) {
    const uint64_t h = mix64(t * 0x9E3779B97F4A7C15ull + (uint64_t)(i + 1) * 0xD1B54A32D192ED03ull);
    if ((h & 7) == 0) return 0.0;
    const double m = 1.0 + (double)((h >> 12) & ((1ull << 52) - 1)) * 2.220446049250313e-16;  // [1, 2)
    const int e = (int)((h >> 3) & 7) - 4;
    return ((h >> 6) & 1 ? -m : m) * ldexp(1.0, e);
}

template <bool MI>
__global__ void __launch_bounds__(128) k_seed_cache(CutArgs a, int64_t n_int) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_int + kSeedRandom) return;
    constexpr int nr = MI ? 12 : 8;
    double rows[12];
    if (t < n_int) {
        int64_t q = t;
        for (int i = 0; i < nr; ++i) {
            rows[i] = MI ? (double)(q % 3) - 1.0 : (double)(q % 5) - 2.0;
            q /= MI ? 3 : 5;
        }
    } else {
        for (int i = 0; i < nr; ++i) rows[i] = seed_value((uint64_t)t, i);
    }
    uint32_t key = 0;
    if (!MI) {
        uint8_t rep[2];
        int first;
        if (ia_group_planes(rows, 2, rep, first) != 2 || !ia_key2(rows, key)) return;
    } else {
        if (!mi_distinct3(rows) || !mi_key3(rows, key)) return;
    }
    int j = -1;
    if (cache_claim(a.cache, key, &j) != CLAIM_OWNER) return;
    typename Traits<MI>::Fast c;
    if (c.run(rows, MI ? 3 : 2) != CUT_OK) return;
    c.canonicalize();
    const int size = c.record_size();
    uint8_t rec[1024];
    if (size > (int)sizeof(rec)) return;
    typename Traits<MI>::Sum sum;
    c.emit(rec, sum);
    cache_insert(a.cache, key, rec, size, pack_sum<typename Traits<MI>::Sum>(sum));
}

// writes a relabelled two-plane record for tet ai (false: the heap is full)
__device__ __forceinline__ bool ia_emit_template2(const CutArgs& a, uint32_t ai, const uint8_t* tmpl, int k,
                                                  const uint8_t* rep, int r1, int r2) {
    const int size = ia_template_record_size(tmpl, k);
    unsigned long long off = heap_alloc(a, size);
    if (off + size > a.heap_cap) return false;
    uint8_t* dst = a.heap + off;
    if (((uintptr_t)dst & 7) == 0) {
        WordSink o{reinterpret_cast<uint64_t*>(dst)};
        ia_template_relabel2(tmpl, k, rep, r1, r2, o);
    } else {
        ia_record_from_template2(tmpl, k, rep, r1, r2, dst);
    }
    IASummary s;
    ia_record_summary(tmpl, s, rep, k);  // from the template: the relabel keeps every count
    a.act_desc[ai] = off | a.desc_bit;
    a.act_sum[ai] = pack_sum<IASummary>(s);
    return true;
}

// the two representatives of a tet whose planes form two groups, and the key of their pair
__device__ __forceinline__ bool ia_two_group_key(const double* planes, int k, const uint8_t* rep, int r[2],
                                                 double two[8], uint32_t& key) {
    int n = 0;
    for (int i = 0; i < k; ++i)
        if (rep[i] == 4 + i) {
            if (n == 2) return false;
            r[n++] = i;
        }
    if (n != 2) return false;
    for (int c = 0; c < 4; ++c) {
        two[c] = planes[4 * r[0] + c];
        two[4 + c] = planes[4 * r[1] + c];
    }
    return ia_key2(two, key);
}

// the tet's record from published entry j of its two-group key
__device__ __forceinline__ bool ia_from_entry(const CutArgs& a, uint32_t ai, int j, int k, const uint8_t* rep, int r0,
                                              int r1) {
    if (k == 2) {  // the record itself
        a.act_desc[ai] = kTableBit | (uint64_t)(kTablePatterns + j);
        a.act_sum[ai] = a.cache.table_sum[kTablePatterns + j];
        return true;
    }
    const uint8_t* tmpl = a.cache.table + a.cache.table_off[kTablePatterns + j];
    return ia_emit_template2(a, ai, tmpl, k, rep, r0, r1);
}

// Tets whose planes reduce to two groups (duplicates, multiples, planes on a tet face, zero planes
// besides two distinct planes): the secondary lookup of the two representatives, whose record is
// relabelled for the tet (on a miss, with `cut_on_miss`, the two planes alone are cut and the record
// published).  Returns CUT_OK when the tet's record is written, CUT_DEFER to fall back to the
// general cut.
__device__ int ia_try_two_groups(const CutArgs& a, uint32_t ai, const double* planes, int k, const uint8_t* rep,
                                 bool cut_on_miss) {
    int r[2];
    double two[8];
    uint32_t key = 0;
    if (!ia_two_group_key(planes, k, rep, r, two, key)) return CUT_DEFER;
    const int j = cache_find(a.cache, key);
    if (j >= 0) return ia_from_entry(a, ai, j, k, rep, r[0], r[1]) ? CUT_OK : CUT_DEFER;
    if (!cut_on_miss) return CUT_DEFER;
    IACutFast c;
    if (c.run(two, 2) != CUT_OK) return CUT_DEFER;
    c.canonicalize();
    const int size = c.record_size();
    uint8_t rec2[1024];
    if (size > (int)sizeof(rec2)) return CUT_DEFER;
    IASummary s2;
    c.emit(rec2, s2);
    cache_insert(a.cache, key, rec2, size, pack_sum<IASummary>(s2));
    return ia_emit_template2(a, ai, rec2, k, rep, r[0], r[1]) ? CUT_OK : CUT_DEFER;
}

// Tets whose planes reduce to at most one after grouping (duplicates, planes coincident with a tet
// face, zero planes): the record comes from the one-plane lookup table, relabelled.  `two` reports
// exactly two groups with distinct representatives (secondary lookup).
__device__ __forceinline__ bool ia_try_template(const CutArgs& a, uint32_t ai, const double* planes, int k,
                                                bool* two, uint8_t* rep) {
    int first;
    const int eff = ia_group_planes(planes, k, rep, first);
    *two = eff == 2;
    if (eff > 1 || !a.table) return false;
    const int pattern = eff ? ia_sign_pattern(planes + 4 * first) : kTablePatterns - 1;  // all positive: uncut
    const uint8_t* tmpl = a.table + a.table_off[pattern];
    const int size = ia_template_record_size(tmpl, k);
    unsigned long long off = heap_alloc(a, size);
    if (off + size > a.heap_cap) {
        raise_status(a.status, ST_CAPACITY);
        return true;
    }
    uint8_t* dst = a.heap + off;
    if (((uintptr_t)dst & 7) == 0) {
        WordSink o{reinterpret_cast<uint64_t*>(dst)};
        ia_template_relabel1(tmpl, k, rep, eff, first, o);
    } else {
        ia_record_from_template(tmpl, k, rep, eff, first, dst);
    }
    IASummary s;
    ia_record_summary(tmpl, s, rep, k);  // from the template: the relabel keeps every count
    a.act_desc[ai] = off | a.desc_bit;
    a.act_sum[ai] = pack_sum<IASummary>(s);
    return true;
}

template <bool MI, bool MID>
__device__ __forceinline__ void cut_one(const CutArgs& a, int64_t i) {
    using Fast = typename std::conditional<MID, typename Traits<MI>::Mid, typename Traits<MI>::Fast>::type;
    using Sum = typename Traits<MI>::Sum;
    constexpr int kMax = MID ? kMidMaxK : kFastMaxK;
    const uint32_t ai = a.list[i];
    double planes[4 * kMax];
    const int k = gather_planes(a, ai, planes, kMax);
    bool keyed = false;
    if (!MI && k <= kMax && k <= kFastMaxK) {
        uint8_t rep[kFastMaxK];
        if (ia_try_template(a, ai, planes, k, &keyed, rep)) return;
        if (keyed && a.cache.slots && ia_try_two_groups(a, ai, planes, k, rep, true) == CUT_OK) return;
        keyed = false;  // the general cut below; its record is not a two-plane template
    }
    if (MI) keyed = k == 3 && mi_distinct3(planes);
    uint32_t key = 0;
    if (keyed && a.cache.slots) {
        keyed = MI ? mi_key3(planes, key) : ia_key2(planes, key);
        if (keyed) {
            const int j = cache_find(a.cache, key);
            if (j >= 0) {
                a.act_desc[ai] = kTableBit | (uint64_t)(kTablePatterns + j);
                a.act_sum[ai] = a.cache.table_sum[kTablePatterns + j];
                return;
            }
        }
    } else {
        keyed = false;
    }
    int st = CUT_DEFER;
    Fast c;
    if (k <= kMax) st = c.run(planes, k);
    if (st == CUT_OK) {
        int size = 0;
        IASum4 sum;
        const uint8_t* rec = finish_cut<Fast, Sum>(a, ai, c, &size, &sum, true);
        if (rec && keyed) cache_insert(a.cache, key, rec, size, sum);
        if (!rec) st = CUT_DEFER;
    }
    if (st == CUT_OK) {
    } else if (st == CUT_DEFER) {
        unsigned int d = atomicAdd(a.n_deferred, 1u);
        a.deferred[d] = ai;
    } else {
        raise_status(a.status, ST_INTERNAL);
    }
}

// One thread per tet.
template <bool MI, bool MID>
__global__ void __launch_bounds__(128) k_cut_fast(CutArgs a) {
    const int64_t n = a.n_dev ? (a.n < (int64_t)*a.n_dev ? a.n : (int64_t)*a.n_dev) : a.n;
    if (a.route_at && n <= a.route_at) return;  // the warp kernel takes a short list
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    cut_one<MI, MID>(a, i);
}

// The lookup pass.  A tet the one-plane table finishes, or whose secondary-lookup key is published,
// is done here.  The first tet of an unpublished key claims it and goes on to the cut kernels,
// whose cut publishes the record; the key's other tets wait (a.wait) for launch_cut_wait.  Every
// other tet is appended to a.deferred for the cut kernels (one atomic per warp, so the list keeps
// its heaviest-first order per warp).  A warp of the cut kernels then holds cuts only, and a key is
// cut once per call.
__device__ __forceinline__ void append_warp(bool mine, uint32_t ai, uint32_t* list, unsigned int* count) {
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, mine);
    if (mine) {
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(m) - 1;
        unsigned int base = 0;
        if (lane == leader) base = atomicAdd(count, (unsigned int)__popc(m));
        base = __shfl_sync(m, base, leader);
        list[base + __popc(m & ((1u << lane) - 1u))] = ai;
    }
}

// the rows of a tet with exactly K active functions (K known at compile time: the rows stay in
// registers)
template <int K>
__device__ __forceinline__ void gather_k(const CutArgs& a, uint32_t ai, double* planes) {
    if (a.values) {
        const uint32_t r0 = a.value_off[ai];
#pragma unroll
        for (int i = 0; i < 4 * K; ++i) planes[i] = a.values[4 * (size_t)r0 + i];
        return;
    }
    uint64_t m = a.act_mask[ai];
    int64_t v[4];
    TetSrc ts{a.d_tets, a.g.res};
    ts.get(a.act_tet[ai], v);
#pragma unroll
    for (int i = 0; i < K; ++i) {
        const int j = __ffsll((long long)m) - 1;
        m &= m - 1;
#pragma unroll
        for (int c = 0; c < 4; ++c) planes[4 * i + c] = a.fv[v[c] * a.F + j];
    }
}

// one tet of the lookup pass: done (record written), waiting (w filled), owner, or none of these
template <bool MI, int K>
__device__ __forceinline__ void prep_tet(const CutArgs& a, uint32_t ai, const double* planes, int k, bool& done,
                                         bool& wait, bool& owner, WaitRec& w) {
    if (!MI) {
        uint8_t rep[kFastMaxK];
        bool two = false;
        done = ia_try_template(a, ai, planes, k, &two, rep);
        int r[2];
        double tw[8];
        uint32_t key = 0;
        if (!done && two && a.cache.slots && ia_two_group_key(planes, k, rep, r, tw, key)) {
            int j = -1;
            const int c = cache_claim(a.cache, key, &j);
            if (c == CLAIM_PUBLISHED) {
                done = ia_from_entry(a, ai, j, k, rep, r[0], r[1]);
            } else if (c == CLAIM_OWNER) {
                owner = a.owners != nullptr;
            } else if (c == CLAIM_WAIT) {
                wait = true;
                w.ai = ai;
                w.key = key;
                w.k = (uint8_t)k;
                w.r0 = (uint8_t)r[0];
                w.r1 = (uint8_t)r[1];
                for (int t = 0; t < k; ++t) w.rep[t] = rep[t];
            }
        }
    } else if (k == 3 && a.cache.slots && mi_distinct3(planes)) {
        uint32_t key = 0;
        if (mi_key3(planes, key)) {
            int j = -1;
            const int c = cache_claim(a.cache, key, &j);
            if (c == CLAIM_PUBLISHED) {
                a.act_desc[ai] = kTableBit | (uint64_t)(kTablePatterns + j);
                a.act_sum[ai] = a.cache.table_sum[kTablePatterns + j];
                done = true;
            } else if (c == CLAIM_OWNER) {
                owner = a.owners != nullptr;
            } else if (c == CLAIM_WAIT) {
                wait = true;
                w.ai = ai;
                w.key = key;
                w.k = 3;
            }
        }
    }
}

template <bool MI>
__global__ void __launch_bounds__(128) k_cut_prep(CutArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const uint32_t ai = a.list[i];
    const int k = a.values ? (int)(a.value_off[ai + 1] - a.value_off[ai]) : __popcll(a.act_mask[ai]);
    bool done = false, wait = false, owner = false;
    WaitRec w{};
    if (k == 2) {  // most tets of the light bins: rows in registers
        double planes[8];
        gather_k<2>(a, ai, planes);
        prep_tet<MI, 2>(a, ai, planes, 2, done, wait, owner, w);
    } else if (k == 3) {
        double planes[12];
        gather_k<3>(a, ai, planes);
        prep_tet<MI, 3>(a, ai, planes, 3, done, wait, owner, w);
    } else if (k <= kFastMaxK) {
        double planes[4 * kFastMaxK];
        gather_planes(a, ai, planes, kFastMaxK);
        prep_tet<MI, 0>(a, ai, planes, k, done, wait, owner, w);
    }
    if (wait) a.wait[atomicAdd(a.n_wait, 1u)] = w;
    if (a.owners) append_warp(owner, ai, a.owners, a.n_owners);
    append_warp(!done && !wait && !owner, ai, a.deferred, a.n_deferred);
}

// The waiting tets: their keys' records are published by now (or the claiming tet's cut could not
// publish, and the tet goes to the exact kernel).
template <bool MI>
__global__ void __launch_bounds__(128) k_cut_wait(CutArgs a) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n || i >= (int64_t)*a.n_wait) return;
    const WaitRec w = a.wait[i];
    const int j = cache_find(a.cache, w.key);
    bool done = false;
    if (j >= 0) {
        if (MI) {
            a.act_desc[w.ai] = kTableBit | (uint64_t)(kTablePatterns + j);
            a.act_sum[w.ai] = a.cache.table_sum[kTablePatterns + j];
            done = true;
        } else {
            done = ia_from_entry(a, w.ai, j, w.k, w.rep, w.r0, w.r1);
        }
    }
    if (!done) a.deferred[atomicAdd(a.n_deferred, 1u)] = w.ai;
}

// Material interface with four or more materials: one block per tet, one warp per material.  A
// material's cell is the tet clipped by its half-spaces against every other material, independent of
// the other cells, so the warps clip the cells in parallel, each step of a clip across the lanes
// (MIWarpClip, cut_mi_warp.cuh); warp 0 then merges the cells (MIMerge, cut_mi_merge.cuh) into the
// bytes the serial cut emits.  A cell beyond the clipper's capacities sends the tet to the next
// variant.
constexpr int kSplitMaxK = 32;
constexpr int kSplitWarps = 8;
using SplitClip = MIWarpClip<32, 32, 192>;
using SplitCell = MICell<32, 32, 192>;
struct SplitSmem {
    double planes[4 * kSplitMaxK];
    MIPrep prep;
    SplitClip clip[kSplitWarps];
    SplitCell cells[kSplitMaxK];
    MIMerge<SplitCell> mg;
    int8_t cst[kSplitMaxK];  // 0 cell, 1 no cell, 2 defer
    uint8_t has[kSplitMaxK];
    int kk;
};

__global__ void __launch_bounds__(32 * kSplitWarps) k_cut_mi_split(CutArgs a) {
    extern __shared__ __align__(16) unsigned char split_smem[];
    SplitSmem& S = *reinterpret_cast<SplitSmem*>(split_smem);
    const int warp = threadIdx.x >> 5;
    const Lanes L = Lanes::of_thread(threadIdx.x & 31);
    SplitClip& c = S.clip[warp];
    for (int64_t i = blockIdx.x; i < a.n; i += gridDim.x) {
        const uint32_t ai = a.list[i];
        if (threadIdx.x == 0) S.kk = gather_planes(a, ai, S.planes, kSplitMaxK);
        __syncthreads();
        const int k = S.kk;
        if (k > kSplitMaxK) {
            if (threadIdx.x == 0) a.deferred[atomicAdd(a.n_deferred, 1u)] = ai;
            __syncthreads();
            continue;
        }
        if (warp == 0) mi_prepare_lanes(L, S.planes, k, S.prep);
        __syncthreads();
        for (int m = warp; m < k; m += kSplitWarps) {
            int8_t cs = 1;
            if (S.prep.has_cell(4 + m)) {
                bool empty = false;
                int st = c.clip(L, S.planes, k, S.prep, 4 + m, empty);
                if (st == CUT_OK && !empty) st = c.export_cell(L, S.cells[m]);
                cs = st != CUT_OK ? 2 : (empty ? 1 : 0);
            }
            if (L.lane == 0) {
                S.cst[m] = cs;
                S.has[m] = cs == 0 ? 1 : 0;
            }
        }
        __syncthreads();
        if (warp == 0) {
            bool ok = true;
            for (int j = 0; j < k; ++j) ok = ok && S.cst[j] != 2;
            // the merge across the lanes (cut_mi_merge.cuh)
            const int merged = ok ? S.mg.run(L, S.cells, S.has, k) : CUT_DEFER;
            bool done = false;
            if (merged == CUT_OK) {
                const int size = S.mg.record_size(k);
                unsigned long long off = 0;
                if (L.lane == 0) off = heap_alloc(a, size);
                off = __shfl_sync(0xFFFFFFFFu, off, 0);
                if (off + size <= a.heap_cap) {
                    MISummary sum;
                    S.mg.emit(L, S.cells, k, S.prep.rep, a.heap + off, sum);
                    if (L.lane == 0) {
                        a.act_desc[ai] = off | a.desc_bit;
                        a.act_sum[ai] = pack_sum<MISummary>(sum);
                    }
                    done = true;
                }
            }
            if (!done && L.lane == 0) a.deferred[atomicAdd(a.n_deferred, 1u)] = ai;
        }
        __syncthreads();
    }
}

// One warp per tet, its state in shared memory (IAWarpCutDev or IAWarpCutLight, cut_ia_warp.cuh): the
// heavy bins of the implicit arrangement, and the light bins' leftovers.  A tet beyond the state's
// capacity goes to the deferred list.
constexpr int kCutWarps = 4;  // warps per block

template <int G, class State>
__global__ void __launch_bounds__(32 * kCutWarps) k_cut_warp(CutArgs a) {
    constexpr int kGroups = 32 * kCutWarps / G;  // groups (one tet each) per block
    extern __shared__ __align__(16) unsigned char warp_smem[];
    const int gib = threadIdx.x / G;
    State& S = reinterpret_cast<State*>(warp_smem)[gib];
    const LanesG<G> L = LanesG<G>::of_thread((int)(threadIdx.x & 31));
    const int lane = L.lane;
    const int64_t n = a.n_dev ? (a.n < (int64_t)*a.n_dev ? a.n : (int64_t)*a.n_dev) : a.n;
    if (a.route_at && n > a.route_at) return;  // the thread kernel takes a long list
    const int64_t groups = (int64_t)gridDim.x * kGroups;
    int64_t i = (int64_t)blockIdx.x * kGroups + gib;
    for (;;) {
        if (a.next) {  // take the next tet in list order: the heaviest first, and no group idles early
            unsigned int t = 0;
            if (lane == 0) t = atomicAdd(a.next, 1u);
            i = (int64_t)L.bcast(t);
        }
        if (i >= n) break;
        const uint32_t ai = a.list[i];
        int k;
        if (a.values) {
            const uint32_t r0 = a.value_off[ai];
            k = (int)(a.value_off[ai + 1] - r0);
            if (k <= kWarpMaxK)
                for (int x = lane; x < 4 * k; x += G) S.pl[x] = a.values[4 * (size_t)r0 + x];
        } else {
            const uint64_t m = a.act_mask[ai];
            k = __popcll(m);
            if (k <= kWarpMaxK) {
                int64_t v[4];
                TetSrc ts{a.d_tets, a.g.res};
                ts.get(a.act_tet[ai], v);
                for (int x = lane; x < 4 * k; x += G) {
                    // plane x/4 is the (x/4)-th active function, at corner x%4
                    uint64_t mm = m;
                    for (int p = 0; p < (x >> 2); ++p) mm &= mm - 1;
                    const int fn = __ffsll((long long)mm) - 1;
                    S.pl[x] = a.fv[v[x & 3] * a.F + fn];
                }
            }
        }
        L.sync();
        int st = k <= kWarpMaxK ? S.run(L, k) : CUT_DEFER;
        unsigned long long off = 0;
        int size = 0;
        if (st == CUT_OK) {
            S.canonicalize(L);
            size = S.record_size();
            if (lane == 0) off = heap_alloc(a, size);
            off = L.bcast(off);
            if (off + size > a.heap_cap) st = CUT_DEFER;
        }
        if (st == CUT_OK) {
            IASummary sum;
            S.emit(L, a.heap + off, sum);
            if (lane == 0) {
                a.act_desc[ai] = off | a.desc_bit;
                a.act_sum[ai] = pack_sum<IASummary>(sum);
            }
        } else if (lane == 0) {
            // capacity, or an exact evaluation out of range: the exact kernel takes it (and reports)
            a.deferred[atomicAdd(a.n_deferred, 1u)] = ai;
        }
        L.sync();
        if (!a.next) i += groups;
    }
}

// One tet per block at a time; its state lives in shared memory (the exact variant is a long serial
// computation, so the latency of its state accesses sets the time of the whole stage).
template <bool MI>
__global__ void __launch_bounds__(32) k_cut_big(CutArgs a) {
    using Sum = typename Traits<MI>::Sum;
    extern __shared__ __align__(16) unsigned char big_smem[];
    if (threadIdx.x != 0) return;
    BigSlot<MI>& S = *reinterpret_cast<BigSlot<MI>*>(big_smem);
    for (int64_t i = blockIdx.x; i < a.n; i += gridDim.x) {
        const uint32_t ai = a.list[i];
        const int k = gather_planes(a, ai, S.planes, 60);
        if (k > 60) {
            raise_status(a.status, ST_CAPACITY);
            continue;
        }
        int st = S.cut.run(S.planes, k);
        if (st != CUT_OK) {
            raise_status(a.status, ST_CAPACITY);
            continue;
        }
        int size = 0;
        IASum4 sum;
        finish_cut<typename Traits<MI>::Big, Sum>(a, ai, S.cut, &size, &sum);
    }
}

template <bool MI>
__global__ void k_build_table(uint8_t* table, uint32_t* table_off, IASum4* table_sum, BigSlot<MI>* scratch,
                              uint32_t* status) {
    using Sum = typename Traits<MI>::Sum;
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= kTablePatterns) return;
    BigSlot<MI>& S = scratch[p];
    int q = p;
    for (int c = 0; c < 4; ++c) {
        double sgn = (double)(q % 3) - 1.0;
        q /= 3;
        if (MI) {
            S.planes[c] = 0.0;      // material a
            S.planes[4 + c] = sgn;  // material b: b - a has the pattern's signs
        } else {
            S.planes[c] = sgn;
        }
    }
    int st = S.cut.run(S.planes, MI ? 2 : 1);
    if (st != CUT_OK) {
        raise_status(status, ST_INTERNAL);
        return;
    }
    S.cut.canonicalize();
    if (S.cut.record_size() > kTableStride) {
        raise_status(status, ST_INTERNAL);
        return;
    }
    Sum s;
    S.cut.emit(table + p * kTableStride, s);
    table_off[p] = (uint32_t)(p * kTableStride);
    table_sum[p] = pack_sum<Sum>(s);
}

// The reference's robustness mode (src/implicit_arrangement.cpp:137-243,
// src/material_interface.cpp:174-287): every listed tet through robust_tet (robust.cuh) with the
// exact variant; n_fail[0..2] count the tets of type 1 (counts differ), type 2 (the cut fails in the
// given order) and type 3 (it fails in the reversed order).
template <bool MI>
__global__ void __launch_bounds__(64) k_robust(CutArgs a, BigSlot<MI>* scratch, int64_t slots,
                                               unsigned long long* n_fail) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= slots) return;
    BigSlot<MI>& S = scratch[tid];
    for (int64_t i = tid; i < a.n; i += slots) {
        const uint32_t ai = a.list[i];
        const int k = gather_planes(a, ai, S.planes, 30);
        if (k > 30) {
            raise_status(a.status, ST_CAPACITY);
            continue;
        }
        const int r = robust_tet(S.cut, S.planes, k);
        if (r == ROBUST_CAPACITY) raise_status(a.status, ST_CAPACITY);
        else if (r != ROBUST_OK) atomicAdd(n_fail + (r - ROBUST_TYPE1), 1ull);
    }
}

}  // namespace

void launch_robust(const CutArgs& a, void* scratch, int64_t slots, unsigned long long* n_fail, cudaStream_t s) {
    if (a.n == 0) return;
    const int bs = 64;
    const int64_t use = a.n < slots ? a.n : slots;
    const unsigned nb = (unsigned)((use + bs - 1) / bs);
    if (a.mi)
        {
            k_robust<true><<<nb, bs, 0, s>>>(a, (BigSlot<true>*)scratch, use, n_fail);
            note_launch();
        }
    else
        {
            k_robust<false><<<nb, bs, 0, s>>>(a, (BigSlot<false>*)scratch, use, n_fail);
            note_launch();
        }
}

size_t cut_big_slot_bytes(bool mi) { return mi ? sizeof(BigSlot<true>) : sizeof(BigSlot<false>); }

void launch_cut_mi_split(const CutArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    static const bool attr =  // once per process (thread-safe static initialisation)
        cudaFuncSetAttribute(k_cut_mi_split, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(SplitSmem)) ==
        cudaSuccess;
    (void)attr;
    const int64_t blocks = a.n < 152 * 4 ? a.n : 152 * 4;
    k_cut_mi_split<<<(unsigned)blocks, 32 * kSplitWarps, sizeof(SplitSmem), s>>>(a);
    note_launch();
}

void launch_seed_cache(const CutArgs& a, cudaStream_t s) {
    const int64_t n_int = a.mi ? 531441 : 390625;  // 3^12, 5^8
    const unsigned nb = (unsigned)((n_int + kSeedRandom + 127) / 128);
    if (a.mi)
        k_seed_cache<true><<<nb, 128, 0, s>>>(a, n_int);
    else
        k_seed_cache<false><<<nb, 128, 0, s>>>(a, n_int);
    note_launch();
}

void launch_cut_wait(const CutArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    const unsigned nb = (unsigned)((a.n + 127) / 128);
    if (a.mi)
        k_cut_wait<true><<<nb, 128, 0, s>>>(a);
    else
        k_cut_wait<false><<<nb, 128, 0, s>>>(a);
    note_launch();
}

void launch_cut_prep(const CutArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    const unsigned nb = (unsigned)((a.n + 127) / 128);
    if (a.mi)
        k_cut_prep<true><<<nb, 128, 0, s>>>(a);
    else
        k_cut_prep<false><<<nb, 128, 0, s>>>(a);
    note_launch();
}

template <int G, class State>
void launch_warp_groups(const CutArgs& a, cudaStream_t s) {
    constexpr int kGroups = 32 * kCutWarps / G;
    constexpr size_t smem = sizeof(State) * kGroups;
    // the shared-memory size, then the resident blocks on the device: once per process
    // (thread-safe static initialisation); the groups take tets from the list
    static const int2 occ = [] {  // (SMs, resident blocks per SM)
        cudaFuncSetAttribute(k_cut_warp<G, State>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cut_warp<G, State>, 32 * kCutWarps, smem);
        return make_int2(sms > 0 ? sms : 152, per_sm > 0 ? per_sm : 1);
    }();
    const int per_sm = a.warp_blocks_per_sm > 0 && a.warp_blocks_per_sm < occ.y ? a.warp_blocks_per_sm : occ.y;
    const int64_t resident = (int64_t)occ.x * per_sm;
    const int64_t want = (a.n + kGroups - 1) / kGroups;
    const int64_t blocks = want < resident ? want : resident;
    k_cut_warp<G, State><<<(unsigned)blocks, 32 * kCutWarps, smem, s>>>(a);
    note_launch();
}

// Whole warps: half-warp groups (two tets per warp) measured slower on the large config, as the
// two halves' data-dependent phases diverge.
void launch_cut_warp(const CutArgs& a, cudaStream_t s, bool light) {
    if (a.n == 0) return;
    if (light)
        launch_warp_groups<32, IAWarpCutLight>(a, s);
    else
        launch_warp_groups<32, IAWarpCutDev>(a, s);
}

void launch_cut_fast(const CutArgs& a, cudaStream_t s, bool mid) {
    if (a.n == 0) return;
    // each thread runs one long serial cut: with few tets, smaller blocks spread them over all SMs
    int bs = 128;
    if (a.fast_block >= 32 && a.fast_block <= 128 && (a.fast_block & 31) == 0)  // __launch_bounds__(128)
        bs = a.fast_block;
    else
        while (bs > 32 && (a.n + bs - 1) / bs < 4 * 152) bs >>= 1;
    const unsigned nb = (unsigned)((a.n + bs - 1) / bs);
    // the per-thread state lives in local memory: ask for the largest L1 (no shared memory used)
    static const bool carve = [] {  // once per process (thread-safe static initialisation)
        cudaFuncSetAttribute(k_cut_fast<true, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        cudaFuncSetAttribute(k_cut_fast<true, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        cudaFuncSetAttribute(k_cut_fast<false, true>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        cudaFuncSetAttribute(k_cut_fast<false, false>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        cudaFuncSetAttribute(k_cut_prep<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        cudaFuncSetAttribute(k_cut_prep<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        return true;
    }();
    (void)carve;
    if (a.mi) {
        if (mid) k_cut_fast<true, true><<<nb, bs, 0, s>>>(a);
        else k_cut_fast<true, false><<<nb, bs, 0, s>>>(a);
    } else {
        if (mid) k_cut_fast<false, true><<<nb, bs, 0, s>>>(a);
        else k_cut_fast<false, false><<<nb, bs, 0, s>>>(a);
    }
    note_launch();
}

template <bool MI>
void launch_big(const CutArgs& a, cudaStream_t s) {
    const size_t smem = sizeof(BigSlot<MI>);
    static const bool attr =  // once per process (thread-safe static initialisation)
        cudaFuncSetAttribute(k_cut_big<MI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess;
    (void)attr;
    const int64_t blocks = a.n < 152 * 8 ? a.n : 152 * 8;
    k_cut_big<MI><<<(unsigned)blocks, 32, smem, s>>>(a);
    note_launch();
}

void launch_cut_big(const CutArgs& a, cudaStream_t s) {
    if (a.n == 0) return;
    if (a.mi)
        launch_big<true>(a, s);
    else
        launch_big<false>(a, s);
}

void launch_build_table(bool mi, uint8_t* table, uint32_t* table_off, IASum4* table_sum, void* scratch,
                        uint32_t* status, cudaStream_t s) {
    const int bs = 32;
    const unsigned nb = (kTablePatterns + bs - 1) / bs;
    if (mi)
        {
            k_build_table<true><<<nb, bs, 0, s>>>(table, table_off, table_sum, (BigSlot<true>*)scratch, status);
            note_launch();
        }
    else
        {
            k_build_table<false><<<nb, bs, 0, s>>>(table, table_off, table_sum, (BigSlot<false>*)scratch, status);
            note_launch();
        }
}

}  // namespace ria
