// Stage (d): mesh extraction (src/extract_mesh.cpp:10-265 extract_iso_mesh) and vertex coordinates
// (src/extract_mesh.cpp:1446-1538 compute_iso_vert_xyz, src/extract_mesh.h:111-159).
//
// The reference walks the tets in order and numbers a vertex or face at its first occurrence,
// deduplicating through hash maps keyed by
//   tet vertex v | tet edge (v1, v2, f) | tet face (v1, v2, v3, f1, f2)   (vertices)
//   (smallest, second smallest, largest vertex id)                        (faces on the tet boundary)
// Here every occurrence gets its position in that serial order from exclusive scans of the
// per-tet counts; keyed occurrences lower their key's owner to their position with atomicMin
// (a direct-mapped array for tet vertices, a 128-bit open-addressing hash otherwise); an occurrence
// is new iff it owns its key, and the new occurrences are numbered by one more scan.  The result is
// the reference's numbering exactly.
#include "div_rn.cuh"
#include "extract_common.cuh"
#include "launch.hpp"

namespace ria {

using namespace xc;

namespace {

struct ExtractCtx {
    ExtractArgs a;
    RecSrc rs;
    const U4* base;        // per active tet: occurrence bases (vert, face, loop, boundary face)
    uint32_t* corner_owner;
    HashTab he, hf, hb;
    HashTab64 he64;        // edge keys packed in one word (vertex ids below 2^28, functions below 256)
    bool edge64;
    uint64_t* vocc;        // per vertex occurrence: type << 62 | payload
    uint64_t* vsrc;        // per vertex occurrence: active index << 8 | local vertex
    uint32_t* vowner;      // per vertex occurrence: owner position
    uint32_t* vflag;       // 1 if new
    uint32_t* vgid_new;    // exclusive scan of vflag
    uint32_t* occ_gid;     // per vertex occurrence: global vertex id
    uint64_t* focc;        // per face occurrence: OCC_SELF or slot in hb
    uint32_t* fowner;
    uint32_t* flen;
    uint32_t* fdup;
    U4* fsz;    // per face occurrence: (new, loop length if new, tets if new, 0)
    U4* fscan;  // its exclusive scan: (face id, offset in face_verts, offset in face_tets, 0)
    // per face occurrence, from the vertex pass: loop start in fgids, loop offset in the record,
    // (active tet, record face), function
    uint32_t* floop;
    uint32_t* frec;
    uint64_t* fsrc;
    int32_t* ffunc;
    uint32_t* fgids;  // global vertex ids of every iso face loop, in occurrence order
    uint64_t* iso0;   // per active tet: iso flags of its first 64 record vertices, from the vertex pass
    // per table record (the one-plane entries and the secondary lookup's records, shared by many tets):
    // what the vertex pass reads from its walk, summarised once per call for the entries its tets use
    uint32_t* tsum_state;  // 0 unused, 1 used (walked by each tet: too many vertices or faces), 2 summarised
    uint64_t* tsum;        // kTsumWords words per entry: iso flags, iso face count, then one word per face
    uint32_t tsum_n;
    U4 tot;  // totals of the bases (vertex occurrences, face occurrences, loop vertices, boundary faces)
};

constexpr int kTsumFaces = 6;
constexpr int kTsumWords = 2 + kTsumFaces;

// the table entries this call's tets use
__global__ void k_tsum_mark(ExtractCtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.a.A) return;
    const uint64_t d = C.a.act_desc[a];
    const uint32_t e = (uint32_t)(d & 0xFFFFFFFFull);
    // most tets share a few entries: a store only while the entry is unmarked
    if ((d & kTableBit) && e < C.tsum_n && C.tsum_state[e] == 0u) C.tsum_state[e] = 1u;
}

// one walk per used entry: its iso flags and iso faces (record face, loop length, loop offset, local
// function), when they fit the summary
__global__ void k_tsum_build(ExtractCtx C) {
    const uint32_t e = blockIdx.x * kBs + threadIdx.x;
    if (e >= C.tsum_n || C.tsum_state[e] != 1u) return;
    IAView r;
    r.init(C.rs.get(kTableBit | (uint64_t)e));
    uint64_t i0 = 0, rest = 0;
    uint64_t fw[kTsumFaces];
    int nfc = 0, off = 0;
    for (int f = 0; f < r.nf; ++f) {
        const int L = r.len(f);
        if (r.plane_is_iso(r.supp(f))) {
            for (int t = 0; t < L; ++t) {
                const int v = r.loopv(off + t);
                if (v < 64) i0 |= 1ull << v;
                else rest = 1;
            }
            if (nfc < kTsumFaces)
                fw[nfc] = (uint64_t)f | ((uint64_t)L << 16) | ((uint64_t)off << 32) |
                          ((uint64_t)(uint8_t)(int8_t)r.plane_func_local(r.supp(f)) << 48);
            ++nfc;
        }
        off += L;
    }
    if (nfc > kTsumFaces || rest || off >= 0x10000) return;  // stays 1: walked by each tet
    uint64_t* sd = C.tsum + (size_t)kTsumWords * e;
    sd[0] = i0;
    sd[1] = (uint64_t)nfc;
    for (int k = 0; k < nfc; ++k) sd[2 + k] = fw[k];
    C.tsum_state[e] = 2u;
}

// one iso face occurrence of the vertex pass: (record face, loop length, loop offset, local function)
__device__ __forceinline__ void list_iso_face(const ExtractCtx& C, int64_t a, uint64_t mask, uint32_t& fpos,
                                              uint32_t& lpos, int f, int L, int off, int lf) {
    if (fpos >= C.tot.b || lpos + (uint32_t)L > C.tot.c) {  // counts and record disagree: never written
        raise_status(C.a.status, ST_INTERNAL);
        return;
    }
    C.flen[fpos] = (uint32_t)L;
    C.floop[fpos] = lpos;
    C.frec[fpos] = (uint32_t)off;
    C.fsrc[fpos] = ((uint64_t)a << 16) | (uint64_t)f;
    C.ffunc[fpos] = lf < 0 ? -1 : local_func(mask, lf);
    ++fpos;
    lpos += (uint32_t)L;
}

__device__ __forceinline__ void list_iso_vertices(const ExtractCtx& C, int64_t a, uint32_t p, uint64_t i0, uint64_t i1,
                                                  uint64_t i2, uint64_t i3) {
#pragma unroll
    for (int w = 0; w < 4; ++w) {
        uint64_t x = w == 0 ? i0 : (w == 1 ? i1 : (w == 2 ? i2 : i3));
        while (x) {
            const int bit = __ffsll((long long)x) - 1;
            x &= x - 1;
            if (p >= C.tot.a) {  // counts and record disagree: never written
                raise_status(C.a.status, ST_INTERNAL);
                return;
            }
            C.vsrc[p++] = ((uint64_t)a << 8) | (uint64_t)(64 * w + bit);
        }
    }
}

// D2a: one thread per active tet.  One walk over the record's faces gives the iso flags of its
// vertices and the list of its iso face occurrences for the face pass; the tet's iso vertex
// occurrences are listed at their serial positions (consecutive per tet, in local vertex order).  A
// table record (most tets: one plane, or two planes through the secondary lookup) was walked once
// for the call (k_tsum_build); its tets read that summary.
__global__ void __launch_bounds__(kBs) k_ia_vert_list(ExtractCtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.a.A) return;
    const uint64_t d = C.a.act_desc[a];
    const uint64_t mask = C.a.act_mask[a];
    const U4 b = C.base[a];
    uint32_t fpos = b.b, lpos = b.c;
    const uint32_t e = (uint32_t)(d & 0xFFFFFFFFull);
    const bool tab = (d & kTableBit) && e < C.tsum_n;
    bool summ = tab && C.tsum_state[e] == 2u;
    const U4 bn = a + 1 < C.a.A ? C.base[a + 1] : C.tot;  // the next tet's bases: this tet's counts
    const uint64_t* sd = C.tsum + (size_t)kTsumWords * e;
    uint64_t s0 = 0, s1 = 0;
    if (summ) {
        s0 = sd[0];
        s1 = sd[1];
        // the summary must agree with the counts this tet's bases were scanned from
        if (s1 > (uint64_t)kTsumFaces || s1 != (uint64_t)(bn.b - b.b) || (uint32_t)__popcll(s0) != bn.a - b.a)
            summ = false;
    }
    uint64_t fws[kTsumFaces];
    if (summ) {
        uint32_t loops = 0;
        for (int k = 0; k < kTsumFaces; ++k) {
            fws[k] = k < (int)s1 ? sd[2 + k] : 0;
            loops += (uint32_t)((fws[k] >> 16) & 0xFFFF);
        }
        if (loops != bn.c - b.c) summ = false;
    }
    if (summ) {
        const uint64_t i0 = s0;
        for (int k = 0; k < kTsumFaces; ++k) {
            if (k >= (int)s1) break;
            const uint64_t fw = fws[k];
            list_iso_face(C, a, mask, fpos, lpos, (int)(fw & 0xFFFF), (int)((fw >> 16) & 0xFFFF),
                          (int)((fw >> 32) & 0xFFFF), (int)(int8_t)(fw >> 48));
        }
        C.iso0[a] = i0;
        list_iso_vertices(C, a, b.a, i0, 0, 0, 0);
        return;
    }
    IAView r;
    r.init(C.rs.get(d));
    uint64_t i0 = 0, i1 = 0, i2 = 0, i3 = 0;  // iso flags of local vertices 0..255
    int off = 0;
    for (int f = 0; f < r.nf; ++f) {
        const int L = r.len(f);
        if (r.plane_is_iso(r.supp(f))) {
            for (int t = 0; t < L; ++t) {
                const int v = r.loopv(off + t);
                const uint64_t bit = 1ull << (v & 63);
                const int w = v >> 6;
                i0 |= w == 0 ? bit : 0;
                i1 |= w == 1 ? bit : 0;
                i2 |= w == 2 ? bit : 0;
                i3 |= w == 3 ? bit : 0;
            }
            list_iso_face(C, a, mask, fpos, lpos, f, L, off, r.plane_func_local(r.supp(f)));
        }
        off += L;
    }
    C.iso0[a] = i0;
    list_iso_vertices(C, a, b.a, i0, i1, i2, i3);
}

__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
    const uint32_t lo = __shfl_sync(0xFFFFFFFFu, (uint32_t)v, src);
    const uint32_t hi = __shfl_sync(0xFFFFFFFFu, (uint32_t)(v >> 32), src);
    return ((uint64_t)hi << 32) | lo;
}

// D2b: keys of the iso vertex occurrences, one thread per occurrence (a warp's occurrences belong to
// one tet or to neighbouring ones, which share edges and faces).  Lanes with equal keys are grouped
// (__match_any_sync) and only the group's lowest lane, which holds the group's smallest position,
// inserts the key and lowers the owner; the others take its slot.  So each key reaches the global
// tables about once per warp.
__global__ void __launch_bounds__(kBs) k_ia_vert_keys(ExtractCtx C, int64_t NV) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool has = p < NV;
    const uint64_t src = has ? C.vsrc[p] : 0;
    const int64_t a = (int64_t)(src >> 8);
    if (has && a >= C.a.A) {  // an occurrence the list pass could not write (status raised there)
        raise_status(C.a.status, ST_INTERNAL);
        has = false;
    }
    int type = 0;
    VertKey k;
    uint64_t k0 = (uint64_t)lane, k1 = ~0ull;  // lanes without a keyed occurrence match no one
    if (has) {
        const int j = (int)(src & 0xFF);
        IAView r;
        r.init(C.rs.get(C.a.act_desc[a]));
        int64_t tv[4];
        TetSrc ts{C.a.d_tets, C.a.g.res};
        ts.get(C.a.act_tet[a], tv);
        k = ia_vertex_key_r(r.vlab + 3 * j, tv[0], tv[1], tv[2], tv[3], C.a.act_mask[a]);
        type = k.type;
        if (type == 1) {
            k0 = (uint64_t)k.sv[0];
            k1 = 1;
        } else if (type == 2) {
            k0 = ((uint64_t)k.sv[0] << 32) | (uint64_t)k.sv[1];
            k1 = ((uint64_t)k.fn[0] << 8) | 2;
        } else if (type == 3) {
            k0 = ((uint64_t)k.sv[0] << 32) | (uint64_t)k.sv[1];
            k1 = ((uint64_t)k.sv[2] << 32) | ((uint64_t)k.fn[0] << 16) | ((uint64_t)k.fn[1] << 4) | 3;
        }
    }
    const unsigned grp = __match_any_sync(0xFFFFFFFFu, k0) & __match_any_sync(0xFFFFFFFFu, k1);
    const int leader = __ffs(grp) - 1;
    const uint32_t pos = (uint32_t)p;
    int64_t slot = 0;
    if (has && leader == lane) {
        if (type == 1) {
            atomicMin(&C.corner_owner[k.sv[0]], pos);
        } else if (type == 2) {
            slot = C.edge64 ? ht64_insert_min(C.he64, ((uint64_t)k.sv[0] << 36) | ((uint64_t)k.sv[1] << 8) |
                                                          (uint64_t)k.fn[0], pos)
                            : ht_insert_min(C.he, ((uint64_t)k.sv[0] << 32) | (uint64_t)k.sv[1],
                                            (uint64_t)k.fn[0] + 1, pos);
            if (slot < 0) raise_status(C.a.status, ST_HASH_FULL);
        } else if (type == 3) {
            slot = ht_insert_min(C.hf, ((uint64_t)k.sv[0] << 32) | (uint64_t)k.sv[1],
                                 ((uint64_t)k.sv[2] << 32) | ((uint64_t)k.fn[0] << 16) | (uint64_t)k.fn[1], pos);
            if (slot < 0) raise_status(C.a.status, ST_HASH_FULL);
        }
    }
    slot = (int64_t)shfl64((uint64_t)slot, leader);
    if (has) {
        uint64_t occ;
        if (type == 1) occ = (OCC_CORNER << 62) | (uint64_t)k.sv[0];
        else if (type == 2) occ = (OCC_EDGE << 62) | (uint64_t)(slot < 0 ? 0 : slot);
        else if (type == 3) occ = (OCC_FACE << 62) | (uint64_t)(slot < 0 ? 0 : slot);
        else occ = OCC_SELF << 62;
        C.vocc[p] = occ;
    }
}

// D3: owner and new flag of each vertex occurrence
__global__ void k_vert_owner(ExtractCtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint64_t occ = C.vocc[p];
    const uint64_t ty = occ >> 62, pay = occ & ((1ull << 62) - 1);
    uint32_t own;
    if (ty == OCC_SELF) own = (uint32_t)p;
    else if (ty == OCC_CORNER) own = C.corner_owner[pay];
    else if (ty == OCC_EDGE) own = C.edge64 ? C.he64.owner[pay] : C.he.owner[pay];
    else own = C.hf.owner[pay];
    if (own > (uint32_t)p) own = (uint32_t)p;  // only after a failed insert (ST_HASH_FULL already raised)
    C.vowner[p] = own;
    C.vflag[p] = own == (uint32_t)p ? 1u : 0u;
}

// D4a: global vertex id of every occurrence; the occurrence of each new vertex, by id
__global__ void k_vert_gid(ExtractCtx C, int64_t n, uint32_t* __restrict__ gid_src) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint32_t own = C.vowner[p];
    const uint32_t gid = C.vgid_new[own];
    C.occ_gid[p] = gid;
    if (own == (uint32_t)p) gid_src[gid] = (uint32_t)p;
}

// D4b: vertex records and coordinates, one thread per new vertex (no idle lanes in the long path).
// The key of a vertex on the tet boundary is read back from the hash slot its owner inserted (corner:
// the vertex id itself), so only a vertex inside its tet goes back to the tet's record.
__device__ __forceinline__ void vert_emit_one(const ExtractCtx& C, uint32_t p, int64_t* rec, double* xyz) {
    const uint64_t occ = C.vocc[p], src = C.vsrc[p];
    const int64_t a = (int64_t)(src >> 8);
    const int j = (int)(src & 0xFF);
    if (a >= C.a.A) {
        raise_status(C.a.status, ST_INTERNAL);
        for (int c = 0; c < 11; ++c) rec[c] = -1;
        for (int c = 0; c < 3; ++c) xyz[c] = 0.0;
        return;
    }
    const uint32_t tet = C.a.act_tet[a];
    const uint64_t ty = occ >> 62, pay = occ & ((1ull << 62) - 1);
    VertKey k;
    for (int c = 0; c < 4; ++c) k.sv[c] = -1;
    k.fn[0] = k.fn[1] = k.fn[2] = -1;
    if (ty == OCC_CORNER) {
        k.type = 1;
        k.sv[0] = (int64_t)pay;
    } else if (ty == OCC_EDGE) {
        k.type = 2;
        if (C.edge64) {
            const uint64_t key = C.he64.keys[pay];
            k.sv[0] = (int64_t)(key >> 36);
            k.sv[1] = (int64_t)((key >> 8) & ((1ull << 28) - 1));
            k.fn[0] = (int)(key & 0xFF);
        } else {
            const ulonglong2 key = C.he.keys[pay];
            k.sv[0] = (int64_t)(key.x >> 32);
            k.sv[1] = (int64_t)(key.x & 0xFFFFFFFFull);
            k.fn[0] = (int)key.y - 1;
        }
    } else if (ty == OCC_FACE) {
        k.type = 3;
        const ulonglong2 key = C.hf.keys[pay];
        k.sv[0] = (int64_t)(key.x >> 32);
        k.sv[1] = (int64_t)(key.x & 0xFFFFFFFFull);
        k.sv[2] = (int64_t)(key.y >> 32);
        k.fn[0] = (int)((key.y >> 16) & 0xFFFF);
        k.fn[1] = (int)(key.y & 0xFFFF);
    } else {
        IAView r;
        r.init(C.rs.get(C.a.act_desc[a]));
        int64_t tv[4];
        TetSrc ts{C.a.d_tets, C.a.g.res};
        ts.get(tet, tv);
        k = ia_vertex_key_r(r.vlab + 3 * j, tv[0], tv[1], tv[2], tv[3], C.a.act_mask[a]);
    }
    // a key read back from a slot is in range unless its insertion failed (status already raised)
    if (k.sv[0] >= C.a.V || k.sv[1] >= C.a.V || k.sv[2] >= C.a.V || k.fn[0] >= C.a.F || k.fn[1] >= C.a.F) {
        raise_status(C.a.status, ST_INTERNAL);
        for (int c = 0; c < 11; ++c) rec[c] = -1;
        for (int c = 0; c < 3; ++c) xyz[c] = 0.0;
        return;
    }
    rec[0] = tet;
    rec[1] = j;
    rec[2] = k.type;
    for (int c = 0; c < 4; ++c) rec[3 + c] = k.sv[c];
    for (int c = 0; c < 3; ++c) rec[7 + c] = k.fn[c];
    rec[10] = -1;
    // coordinates, with the reference's formulas and operation order (divisions correctly rounded on the
    // integer pipe, div_rn.cuh: the same bits as the FP64 division)
    PtSrc ps{C.a.d_pts, C.a.coords, (int)C.a.g.res + 1};
    const double* fv = C.a.fv;
    const int F = C.a.F;
    double out[3];
    switch (k.type) {
        case 2: {
            double p1[3], p2[3];
            ps.get(k.sv[0], p1);
            ps.get(k.sv[1], p2);
            double f1 = fv[k.sv[0] * F + k.fn[0]], f2 = fv[k.sv[1] * F + k.fn[0]];
            double b0 = div_rn(f2, f2 - f1);
            double b1 = 1 - b0;
            for (int c = 0; c < 3; ++c) out[c] = b0 * p1[c] + b1 * p2[c];
            break;
        }
        case 3: {
            double P[3][3];
            for (int t = 0; t < 3; ++t) ps.get(k.sv[t], P[t]);
            double a1[3], a2[3];
            for (int t = 0; t < 3; ++t) {
                a1[t] = fv[k.sv[t] * F + k.fn[0]];
                a2[t] = fv[k.sv[t] * F + k.fn[1]];
            }
            double n1 = a1[2] * a2[1] - a1[1] * a2[2];
            double n2 = a1[0] * a2[2] - a1[2] * a2[0];
            double n3 = a1[1] * a2[0] - a1[0] * a2[1];
            double d = n1 + n2 + n3;
            double w0 = div_rn(n1, d), w1 = div_rn(n2, d), w2 = div_rn(n3, d);
            for (int c = 0; c < 3; ++c) out[c] = w0 * P[0][c] + w1 * P[1][c] + w2 * P[2][c];
            break;
        }
        case 4: {
            double P[4][3];
            for (int t = 0; t < 4; ++t) ps.get(k.sv[t], P[t]);
            double p1[4], p2[4], p3[4];
            for (int t = 0; t < 4; ++t) {
                p1[t] = fv[k.sv[t] * F + k.fn[0]];
                p2[t] = fv[k.sv[t] * F + k.fn[1]];
                p3[t] = fv[k.sv[t] * F + k.fn[2]];
            }
            double n1 = p1[3] * (p2[2] * p3[1] - p2[1] * p3[2]) + p1[2] * (p2[1] * p3[3] - p2[3] * p3[1]) +
                        p1[1] * (p2[3] * p3[2] - p2[2] * p3[3]);
            double n2 = p1[3] * (p2[0] * p3[2] - p2[2] * p3[0]) + p1[2] * (p2[3] * p3[0] - p2[0] * p3[3]) +
                        p1[0] * (p2[2] * p3[3] - p2[3] * p3[2]);
            double n3 = p1[3] * (p2[1] * p3[0] - p2[0] * p3[1]) + p1[1] * (p2[0] * p3[3] - p2[3] * p3[0]) +
                        p1[0] * (p2[3] * p3[1] - p2[1] * p3[3]);
            double n4 = p1[2] * (p2[0] * p3[1] - p2[1] * p3[0]) + p1[1] * (p2[2] * p3[0] - p2[0] * p3[2]) +
                        p1[0] * (p2[1] * p3[2] - p2[2] * p3[1]);
            double d = n1 + n2 + n3 + n4;
            double w0 = div_rn(n1, d), w1 = div_rn(n2, d), w2 = div_rn(n3, d), w3 = div_rn(n4, d);
            for (int c = 0; c < 3; ++c) out[c] = w0 * P[0][c] + w1 * P[1][c] + w2 * P[2][c] + w3 * P[3][c];
            break;
        }
        default:
            ps.get(k.sv[0], out);
    }
    for (int c = 0; c < 3; ++c) xyz[c] = out[c];
}

// The block's records and coordinates are staged in shared memory and stored as contiguous runs.
__global__ void __launch_bounds__(kBs) k_vert_emit(ExtractCtx C, int64_t n_new, const uint32_t* __restrict__ gid_src,
                                                   int64_t* __restrict__ verts, double* __restrict__ xyz) {
    __shared__ int64_t srec[kBs * 11];
    __shared__ double sxyz[kBs * 3];
    const int64_t g0 = (int64_t)blockIdx.x * kBs;
    const int64_t g = g0 + threadIdx.x;
    if (g < n_new) vert_emit_one(C, gid_src[g], srec + 11 * threadIdx.x, sxyz + 3 * threadIdx.x);
    __syncthreads();
    const int nb = (int)(n_new - g0 < kBs ? n_new - g0 : kBs);
    for (int i = threadIdx.x; i < 11 * nb; i += kBs) verts[11 * g0 + i] = srec[i];
    for (int i = threadIdx.x; i < 3 * nb; i += kBs) xyz[3 * g0 + i] = sxyz[i];
}

// D5: one thread per iso face occurrence (listed by the vertex pass): the global vertex ids of its
// loop, staged for D7; a face on
// the tet boundary is keyed by its (smallest, second smallest, largest) vertex id
// (src/extract_mesh.h:68-92).  The two occurrences of a shared tet face are often in one warp (the
// tets of a cube are consecutive): lanes with equal keys are grouped and only the lowest, which holds
// the smaller position, inserts the key.
__global__ void __launch_bounds__(kBs) k_ia_face_keys(ExtractCtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool has = p < n;
    bool bnd = false;
    uint64_t k0 = (uint64_t)lane, k1 = ~0ull;  // no boundary key: matches no other lane
    int64_t mn = 0, second = 0, mx = 0;
    if (has) {
        const uint64_t src = C.fsrc[p];
        const int64_t a = (int64_t)(src >> 16) < C.a.A ? (int64_t)(src >> 16) : 0;  // (a list-pass failure is already raised)
        const int f = (int)(src & 0xFFFF);
        IAView r;
        r.init(C.rs.get(C.a.act_desc[a]));
        uint64_t iso[4] = {0, 0, 0, 0};
        if (r.nv <= 64)
            iso[0] = C.iso0[a];  // computed by the vertex pass
        else
            iso_vertex_flags(r, iso);
        const uint32_t vb = C.base[a].a;
        const int L = (uint64_t)C.floop[p] + C.flen[p] <= (uint64_t)C.tot.c ? (int)C.flen[p] : 0;  // (else already raised)
        const int off = (int)C.frec[p];
        uint32_t* g = C.fgids + C.floop[p];
        for (int t = 0; t < L; ++t) g[t] = C.occ_gid[vb + iso_rank(iso, r.loopv(off + t))];
        bnd = r.bnd(f);
        if (bnd) {
            int mpos = 0;
            for (int t = 0; t < L; ++t) {
                const int64_t v = g[t];
                if (t == 0 || v < mn) {
                    mn = v;
                    mpos = t;
                }
                if (t == 0 || v > mx) mx = v;
            }
            second = mx + 1;
            for (int t = 0; t < L; ++t)
                if (t != mpos && (int64_t)g[t] < second) second = g[t];
            k0 = ((uint64_t)mn << 32) | (uint64_t)second;
            k1 = (uint64_t)mx + 1;
        }
    }
    const unsigned grp = __match_any_sync(0xFFFFFFFFu, k0) & __match_any_sync(0xFFFFFFFFu, k1);
    const int leader = __ffs(grp) - 1;
    int64_t sl = 0;
    if (has && bnd && leader == lane) {
        sl = ht_insert_min(C.hb, k0, k1, (uint32_t)p);
        if (sl < 0) raise_status(C.a.status, ST_HASH_FULL);
    }
    const uint32_t slo = __shfl_sync(0xFFFFFFFFu, (uint32_t)sl, leader);
    const uint32_t shi = __shfl_sync(0xFFFFFFFFu, (uint32_t)((uint64_t)sl >> 32), leader);
    sl = (int64_t)(((uint64_t)shi << 32) | slo);
    if (has) C.focc[p] = bnd ? ((OCC_EDGE << 62) | (uint64_t)(sl < 0 ? 0 : sl)) : (OCC_SELF << 62);
}

// D6: owners of the face occurrences, duplicate counts
__global__ void k_face_owner(ExtractCtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint64_t occ = C.focc[p];
    uint32_t own = (occ >> 62) == OCC_SELF ? (uint32_t)p : C.hb.owner[occ & ((1ull << 62) - 1)];
    if (own > (uint32_t)p) own = (uint32_t)p;  // only after a failed insert (ST_HASH_FULL already raised)
    C.fowner[p] = own;
    if (own != (uint32_t)p) atomicAdd(&C.fdup[own], 1u);
}

// the counts the three face numberings scan, as one U4 per occurrence (one scan for all three)
__global__ void k_face_sizes(ExtractCtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const bool isnew = C.fowner[p] == (uint32_t)p;
    const uint32_t dup = isnew ? C.fdup[p] : 0;
    C.fsz[p] = U4{isnew ? 1u : 0u, isnew ? C.flen[p] : 0u, isnew ? 1 + dup : 0u, 0u};
    if (dup > 1) raise_status(C.a.status, ST_NONMANIFOLD);
}

// totals of the vertex numbering and of the three face numberings: (vertices, faces, face vertices,
// face tets)
__global__ void k_ia_totals(ExtractCtx C, int64_t NV, int64_t NF, int64_t* __restrict__ d) {
    if (threadIdx.x != 0) return;
    d[0] = NV ? (int64_t)C.vflag[NV - 1] + (int64_t)C.vgid_new[NV - 1] : 0;
    const U4 z{0, 0, 0, 0};
    const U4 f = NF ? U4Sum()(C.fsz[NF - 1], C.fscan[NF - 1]) : z;
    d[1] = f.a;
    d[2] = f.b;
    d[3] = f.c;
}

// D7: face vertex lists, function ids and tet-face lists, one thread per face occurrence
__global__ void __launch_bounds__(kBs) k_ia_face_emit(ExtractCtx C, int64_t n, int64_t* __restrict__ face_offsets,
                                                      int64_t* __restrict__ face_verts,
                                                      int64_t* __restrict__ face_tet_offsets,
                                                      int64_t* __restrict__ face_tets, int64_t* __restrict__ face_func,
                                                      int64_t n_faces, int64_t n_fv, int64_t n_ft) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    if (p == 0) {  // the closing entries of the two offset arrays
        face_offsets[n_faces] = n_fv;
        face_tet_offsets[n_faces] = n_ft;
    }
    const uint32_t own = C.fowner[p];
    const uint64_t src = C.fsrc[p];
    const int64_t tet = C.a.act_tet[(int64_t)(src >> 16) < C.a.A ? (int64_t)(src >> 16) : 0];
    const int64_t f = (int64_t)(src & 0xFFFF);
    if (own == (uint32_t)p) {
        const U4 sc = C.fscan[p];
        const uint32_t gid = sc.a;
        const uint32_t vo = sc.b;
        const uint32_t L = C.flen[p];
        const uint32_t* g = C.fgids + C.floop[p];
        face_offsets[gid] = vo;
        for (uint32_t t = 0; t < L; ++t) face_verts[vo + t] = g[t];
        const uint32_t to = sc.c;
        face_tet_offsets[gid] = to;
        face_tets[2 * (int64_t)to] = tet;
        face_tets[2 * (int64_t)to + 1] = f;
        face_func[2 * (int64_t)gid] = C.ffunc[p];
        face_func[2 * (int64_t)gid + 1] = -1;
    } else {
        const uint32_t to = C.fscan[own].c + 1;
        face_tets[2 * (int64_t)to] = tet;
        face_tets[2 * (int64_t)to + 1] = f;
    }
}

}  // namespace

cudaError_t run_extract_mi(const ExtractArgs& a, const IASum4* act_sum, const ExtractBases* pre, ExtractOut& out,
                           cudaStream_t s);

namespace {

__global__ void k_bases_total(int64_t A, const U4* __restrict__ bin, const U4* __restrict__ base,
                              unsigned long long* __restrict__ totals) {
    const U4 t = U4Sum()(bin[A - 1], base[A - 1]);
    totals[0] = t.a;
    totals[1] = t.b;
    totals[2] = t.c;
    totals[3] = t.d;
}

size_t bases_scan_bytes(int64_t A) {
    size_t bytes = 0;
    cub::DeviceScan::ExclusiveScan(nullptr, bytes, (const U4*)nullptr, (U4*)nullptr, U4Sum(), U4{0, 0, 0, 0}, A,
                                   (cudaStream_t)0);
    return bytes;
}

}  // namespace

namespace {
constexpr uint32_t kTsumEntries = (uint32_t)(kTablePatterns + kCacheEntries);
constexpr size_t kTsumStateBytes = (sizeof(uint32_t) * kTsumEntries + 255) & ~(size_t)255;
constexpr size_t kTsumBytes = sizeof(uint64_t) * kTsumWords * (size_t)kTsumEntries;
}  // namespace

size_t extract_bases_bytes(int64_t A, bool summaries) {
    const size_t extra = summaries ? kTsumStateBytes + kTsumBytes : 0;
    if (A <= 0) return 256 + extra;
    const size_t arr = (sizeof(U4) * (size_t)A + 255) & ~(size_t)255;
    return 2 * arr + ((bases_scan_bytes(A) + 255) & ~(size_t)255) + extra;
}

void launch_extract_bases(int64_t A, const IASum4* act_sum, void* buf, unsigned long long* totals, ExtractBases* out,
                          cudaStream_t s) {
    out->base = nullptr;
    out->tsum_state = nullptr;
    out->tsum = nullptr;
    if (A <= 0) {
        cudaMemsetAsync(totals, 0, 4 * sizeof(unsigned long long), s);
        return;
    }
    const size_t arr = (sizeof(U4) * (size_t)A + 255) & ~(size_t)255;
    U4* bin = (U4*)buf;
    U4* base = (U4*)((char*)buf + arr);
    void* tmp = (char*)buf + 2 * arr;
    size_t bytes = bases_scan_bytes(A);
    k_base_in<<<nblk(A), kBs, 0, s>>>(A, act_sum, bin);
    note_launch();
    cub::DeviceScan::ExclusiveScan(tmp, bytes, bin, base, U4Sum(), U4{0, 0, 0, 0}, A, s);
    k_bases_total<<<1, 1, 0, s>>>(A, bin, base, totals);
    note_launch();
    out->base = base;
}

void launch_table_summaries(int64_t A, const uint64_t* act_desc, const uint8_t* table, const uint32_t* table_off,
                            void* buf, ExtractBases* out, cudaStream_t s) {
    out->tsum_state = nullptr;
    out->tsum = nullptr;
    if (A <= 0 || !act_desc || !table || !table_off) return;
    const size_t arr = (sizeof(U4) * (size_t)A + 255) & ~(size_t)255;
    char* t = (char*)buf + 2 * arr + ((bases_scan_bytes(A) + 255) & ~(size_t)255);
    ExtractCtx C{};
    C.a.A = A;
    C.a.act_desc = act_desc;
    C.rs = RecSrc{nullptr, nullptr, table, table_off};
    C.tsum_n = kTsumEntries;
    C.tsum_state = (uint32_t*)t;
    C.tsum = (uint64_t*)(t + kTsumStateBytes);
    cudaMemsetAsync(C.tsum_state, 0, sizeof(uint32_t) * kTsumEntries, s);
    k_tsum_mark<<<nblk(A), kBs, 0, s>>>(C);
    note_launch();
    k_tsum_build<<<nblk(kTsumEntries), kBs, 0, s>>>(C);
    note_launch();
    out->tsum_state = C.tsum_state;
    out->tsum = C.tsum;
}

cudaError_t run_extract(const ExtractArgs& a, const IASum4* act_sum, const ExtractBases* pre, ExtractOut& out,
                        cudaStream_t s) {
    if (a.mi) return run_extract_mi(a, act_sum, pre, out, s);
    Pool pool{s};
    ExtractCtx C;
    C.a = a;
    C.rs = RecSrc{a.heap, a.heap_big, a.table, a.table_off};
    const int64_t A = a.A;
    out = ExtractOut();
    // bases: prepared by the caller (their totals read with the cut stage's synchronization), or here
    U4 tot{0, 0, 0, 0};
    const U4* base = nullptr;
    if (pre && (pre->base || A == 0)) {
        base = (const U4*)pre->base;
        tot = U4{(uint32_t)pre->total[0], (uint32_t)pre->total[1], (uint32_t)pre->total[2], (uint32_t)pre->total[3]};
    } else if (A > 0) {
        U4* bin = pool.get<U4>(A);
        U4* b = pool.get<U4>(A);
        if (pool.err) return pool.err;
        k_base_in<<<nblk(A), kBs, 0, s>>>(A, act_sum, bin);
        note_launch();
        const cudaError_t e = exscan_u4(bin, b, A, &tot, pool, s);
        if (e != cudaSuccess) return e;
        base = b;
    }
    C.base = base;
    C.tot = tot;
    const int64_t NV = tot.a, NF = tot.b, NB = tot.d;
    // tables: tight, sized for the usual share of distinct keys (bounded probing; an overflow raises
    // ST_HASH_FULL and the caller runs the extraction again with worst-case sizes), or worst case: a
    // slot per occurrence that could hold a distinct key
    const bool tight = a.tight_tables;
    const uint64_t cap_e = pow2_at_least(tight ? (uint64_t)NV / 2 + 1 : (uint64_t)NV);
    const uint64_t cap_f = pow2_at_least(tight ? (uint64_t)NV / 16 + 1 : (uint64_t)NV / 2 + 1);
    const uint64_t cap_b = pow2_at_least(tight ? (uint64_t)NB + 1 : 2 * (uint64_t)NB + 1);
    const uint64_t probes = tight ? 4096 : 0;
    C.edge64 = a.V < (1ll << 28) && a.F <= 256;
    C.tsum_n = (uint32_t)(kTablePatterns + kCacheEntries);
    const bool tsum_ready = pre && pre->tsum_state;  // summarised before the cut stage's synchronization
    uint32_t* gid_src = nullptr;  // the occurrence of each new vertex, by id
    int64_t* d_tots = nullptr;
    void* scan_tmp = nullptr;
    size_t vscan_bytes = 0, fscan_bytes = 0;
    if (NV > 0) cub::DeviceScan::ExclusiveSum(nullptr, vscan_bytes, C.vflag, C.vgid_new, NV, s);
    if (NF > 0)
        cub::DeviceScan::ExclusiveScan(nullptr, fscan_bytes, C.fsz, C.fscan, U4Sum(), U4{0, 0, 0, 0}, NF, s);
    // every buffer of the call carved from one allocation: the sizes are added up first
    auto carve = [&](Pool& P) {
        C.corner_owner = P.get<uint32_t>(a.V);
        if (C.edge64) {
            C.he = HashTab{nullptr, nullptr, 0};
            C.he64 = HashTab64{P.get<unsigned long long>((int64_t)cap_e), P.get<uint32_t>((int64_t)cap_e), cap_e - 1,
                               probes};
        } else {
            C.he = HashTab{P.get<ulonglong2>((int64_t)cap_e), P.get<uint32_t>((int64_t)cap_e), cap_e - 1, probes};
            C.he64 = HashTab64{nullptr, nullptr, 0};
        }
        C.hf = HashTab{P.get<ulonglong2>((int64_t)cap_f), P.get<uint32_t>((int64_t)cap_f), cap_f - 1, probes};
        C.hb = HashTab{P.get<ulonglong2>((int64_t)cap_b), P.get<uint32_t>((int64_t)cap_b), cap_b - 1, probes};
        C.vocc = P.get<uint64_t>(NV);
        C.vsrc = P.get<uint64_t>(NV);
        C.vowner = P.get<uint32_t>(NV);
        C.vflag = P.get<uint32_t>(NV);
        C.vgid_new = P.get<uint32_t>(NV);
        C.occ_gid = P.get<uint32_t>(NV);
        C.focc = P.get<uint64_t>(NF);
        C.fowner = P.get<uint32_t>(NF);
        C.flen = P.get<uint32_t>(NF);
        C.fdup = P.get<uint32_t>(NF);
        C.fsz = P.get<U4>(NF);
        C.fscan = P.get<U4>(NF);
        C.floop = P.get<uint32_t>(NF);
        C.fsrc = P.get<uint64_t>(NF);
        C.ffunc = P.get<int32_t>(NF);
        C.frec = P.get<uint32_t>(NF);
        C.fgids = P.get<uint32_t>((int64_t)tot.c);
        C.iso0 = P.get<uint64_t>(A);
        if (tsum_ready) {
            C.tsum_state = pre->tsum_state;
            C.tsum = pre->tsum;
        } else {
            C.tsum_state = P.get<uint32_t>(C.tsum_n);
            C.tsum = P.get<uint64_t>((int64_t)kTsumWords * C.tsum_n);
        }
        gid_src = P.get<uint32_t>(NV);
        d_tots = P.get<int64_t>(8);
        scan_tmp = P.get<uint8_t>((int64_t)std::max(vscan_bytes, fscan_bytes));
    };
    pool.measuring = true;
    carve(pool);
    pool.measuring = false;
    pool.reserve(pool.measured);
    carve(pool);
    if (pool.err) return pool.err;
    FillList fill;
    fill.add(C.corner_owner, sizeof(uint32_t) * (size_t)(a.V > 0 ? a.V : 1), ~0u);
    for (HashTab* h : {&C.he, &C.hf, &C.hb}) {
        if (!h->keys) continue;
        fill.add(h->keys, sizeof(ulonglong2) * (h->cap_mask + 1), ~0u);
        fill.add(h->owner, sizeof(uint32_t) * (h->cap_mask + 1), ~0u);
    }
    if (C.edge64) {
        fill.add(C.he64.keys, sizeof(unsigned long long) * (C.he64.cap_mask + 1), ~0u);
        fill.add(C.he64.owner, sizeof(uint32_t) * (C.he64.cap_mask + 1), ~0u);
    }
    fill.add(C.fdup, sizeof(uint32_t) * (size_t)(NF > 0 ? NF : 1), 0u);
    uint64_t* pin = nullptr;
    AuxStream* aux = nullptr;
    cudaError_t e = pinned_words(&pin);
    if (e == cudaSuccess) e = aux_stream(&aux);
    if (e != cudaSuccess) return e;
    // whatever path leaves this function, the call's stream waits for the second stream's work before
    // the temporaries are released on it (this guard is destroyed before the pool)
    struct JoinAux {
        cudaStream_t s;
        AuxStream* aux;
        bool armed = false;
        ~JoinAux() {
            if (armed) cudaStreamWaitEvent(s, aux->join, 0);
        }
    } join_aux{s, aux};
    // the tables are filled on the second stream (bound by HBM bandwidth) while the occurrence list is
    // built (bound by memory latency); the key pass waits for both
    cudaEventRecord(aux->fork, s);
    cudaStreamWaitEvent(aux->s, aux->fork, 0);
    if ((e = launch_fill(fill, aux->s)) != cudaSuccess) return e;
    cudaEventRecord(aux->join, aux->s);
    join_aux.armed = true;
    // vertices: the table entries in use summarised (unless that was done with the bases), then the
    // occurrence list
    if (!tsum_ready) cudaMemsetAsync(C.tsum_state, 0, sizeof(uint32_t) * C.tsum_n, s);
    if (A > 0) {
        if (!tsum_ready) {
            k_tsum_mark<<<nblk(A), kBs, 0, s>>>(C);
            note_launch();
            k_tsum_build<<<nblk(C.tsum_n), kBs, 0, s>>>(C);
            note_launch();
        }
        k_ia_vert_list<<<nblk(A), kBs, 0, s>>>(C);
        note_launch();
    }
    cudaStreamWaitEvent(s, aux->join, 0);
    if (NV > 0) {
        k_ia_vert_keys<<<nblk(NV), kBs, 0, s>>>(C, NV);
        note_launch();
        k_vert_owner<<<nblk(NV), kBs, 0, s>>>(C, NV);
        note_launch();
        cub::DeviceScan::ExclusiveSum(scan_tmp, vscan_bytes, C.vflag, C.vgid_new, NV, s);
        k_vert_gid<<<nblk(NV), kBs, 0, s>>>(C, NV, gid_src);
        note_launch();
    }
    // The vertex count goes to pinned host memory while the face pass runs; as soon as it arrives the
    // vertex outputs are allocated and the vertex records (bound by the FP64 pipe: divisions) are
    // emitted on the second stream, beside the face pass (bound by memory latency).
    k_ia_totals<<<1, 32, 0, s>>>(C, NV, 0, d_tots);
    note_launch();
    cudaMemcpyAsync(pin, d_tots, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaEventRecord(aux->fork, s);
    // faces
    if (NF > 0) {
        k_ia_face_keys<<<nblk(NF), kBs, 0, s>>>(C, NF);
        note_launch();
        k_face_owner<<<nblk(NF), kBs, 0, s>>>(C, NF);
        note_launch();
        k_face_sizes<<<nblk(NF), kBs, 0, s>>>(C, NF);
        note_launch();
        cub::DeviceScan::ExclusiveScan(scan_tmp, fscan_bytes, C.fsz, C.fscan, U4Sum(), U4{0, 0, 0, 0}, NF, s);
    }
    k_ia_totals<<<1, 32, 0, s>>>(C, 0, NF, d_tots + 4);
    note_launch();
    cudaMemcpyAsync(pin + 1, d_tots + 5, 3 * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    if ((e = cudaEventSynchronize(aux->fork)) != cudaSuccess) return e;
    const int64_t n_verts = (int64_t)pin[0];
    out.n_verts = n_verts;
    cudaStreamWaitEvent(aux->s, aux->fork, 0);
    if ((e = cudaMallocAsync((void**)&out.xyz, sizeof(double) * 3 * (size_t)(n_verts > 0 ? n_verts : 1), aux->s)) !=
        cudaSuccess)
        return e;
    if ((e = cudaMallocAsync((void**)&out.verts, sizeof(int64_t) * 11 * (size_t)(n_verts > 0 ? n_verts : 1),
                             aux->s)) != cudaSuccess)
        return e;
    if (n_verts > 0) {
        k_vert_emit<<<nblk(n_verts), kBs, 0, aux->s>>>(C, n_verts, gid_src, out.verts, out.xyz);
        note_launch();
    }
    cudaEventRecord(aux->join, aux->s);
    cudaEventRecord(aux->fork, s);  // after the face totals' copy
    if ((e = cudaEventSynchronize(aux->fork)) != cudaSuccess) return e;
    const int64_t n_faces = (int64_t)pin[1], n_fv = (int64_t)pin[2], n_ft = (int64_t)pin[3];
    out.n_faces = n_faces;
    out.n_face_verts = n_fv;
    out.n_face_tets = n_ft;
    if ((e = cudaMallocAsync((void**)&out.face_offsets, sizeof(int64_t) * (size_t)(n_faces + 1), s)) != cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_verts, sizeof(int64_t) * (size_t)(n_fv > 0 ? n_fv : 1), s)) !=
            cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_tet_offsets, sizeof(int64_t) * (size_t)(n_faces + 1), s)) !=
            cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_tets, sizeof(int64_t) * 2 * (size_t)(n_ft > 0 ? n_ft : 1), s)) !=
            cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_func, sizeof(int64_t) * 2 * (size_t)(n_faces > 0 ? n_faces : 1), s)) !=
            cudaSuccess)
        return e;
    if (NF > 0) {
        k_ia_face_emit<<<nblk(NF), kBs, 0, s>>>(C, NF, out.face_offsets, out.face_verts, out.face_tet_offsets,
                                                out.face_tets, out.face_func, n_faces, n_fv, n_ft);
        note_launch();
    } else {
        cudaMemsetAsync(out.face_offsets, 0, sizeof(int64_t), s);
        cudaMemsetAsync(out.face_tet_offsets, 0, sizeof(int64_t), s);
    }
    return cudaGetLastError();  // the guard joins the second stream: the call's stream then owns every output
}

// ---- CSG pruning (src/csg.cpp:55-116): a face separates the shape's inside from its outside when the
// CSG membership differs on its two sides.  The signs of every function on one side come from the
// face's tet: inserted planes from the record's cell sign vector, grouped duplicates from their
// representative and the sign of the ratio, planes on a tet face from the opposite corner, inactive
// functions from any corner (their sign is constant in the tet).  The other side differs exactly in
// the functions coincident with the face.

namespace {

__device__ __forceinline__ int local_sign(const IAView& r, uint64_t cs, int li, uint64_t mask, const double* fv,
                                          int F, const int64_t v[4]) {
    const int rp = r.rep[li];
    if (rp == 4 + li) return (cs >> rp) & 1 ? 1 : -1;
    const int gj = local_func(mask, li);
    if (rp == 0xFF) return -1;  // the zero function: never inside
    if (rp < 4) return fv[v[rp] * F + gj] > 0.0 ? 1 : -1;
    const int g0 = local_func(mask, rp - 4);
    const int s0 = (cs >> rp) & 1 ? 1 : -1;
    for (int c = 0; c < 4; ++c) {
        const double x0 = fv[v[c] * F + g0];
        if (x0 != 0.0) return ((x0 > 0.0) == (fv[v[c] * F + gj] > 0.0)) ? s0 : -s0;
    }
    return -1;
}

__device__ __forceinline__ bool csg_inside(const CsgArgs& a, uint64_t S, uint64_t full) {
    const uint64_t in = a.pos_inside ? S : (~S & full);
    if (a.nprog == 0) return in != 0;
    uint64_t st = 0;  // stack of booleans, top at bit depth-1
    int depth = 0;
    for (int i = 0; i < a.nprog; ++i) {
        const int t = a.prog[i];
        if (t >= 0) {
            st = (st & ~bit64(depth)) | (((in >> t) & 1) << depth);
            ++depth;
        } else if (t == -3) {
            st ^= bit64(depth - 1);
        } else {
            const uint64_t x = (st >> (depth - 2)) & 1, y = (st >> (depth - 1)) & 1;
            const uint64_t z = t == -1 ? (x & y) : (x | y);
            --depth;
            st = (st & ~bit64(depth - 1)) | (z << (depth - 1));
        }
    }
    return st & 1;
}

__global__ void k_csg(CsgArgs a) {
    const int64_t g = a.f0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= a.f1) return;
    const int64_t to = a.face_tet_offsets[g];
    const int64_t t = a.face_tets[2 * to];
    const int rf = (int)a.face_tets[2 * to + 1];
    int64_t lo = 0, hi = a.A;  // active index of t (the active list is in tet order)
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((int64_t)a.act_tet[mid] < t) lo = mid + 1;
        else hi = mid;
    }
    const RecSrc rs{a.heap, a.heap_big, a.table, a.table_off};
    const uint8_t* b = rs.get(a.act_desc[lo]);
    IAView r;
    r.init(b);
    const uint64_t mask = a.act_mask[lo];
    int64_t v[4];
    TetSrc ts{a.d_tets, a.res};
    ts.get(t - a.tbase, v);
    for (int q = 0; q < 4; ++q) v[q] += a.vbase;
    const int c = r.pos(rf) != 0xFFFF ? r.pos(rf) : r.neg(rf);
    const uint64_t cs = r.cell(b, c);
    const uint64_t full = a.nfunc == 64 ? ~0ull : (bit64(a.nfunc) - 1);
    uint64_t S = 0;
    int li = 0;
    for (int j = 0; j < a.nfunc; ++j) {
        int sg;
        if (mask & bit64(j)) sg = local_sign(r, cs, li++, mask, a.fv, a.F, v);
        else sg = a.fv[v[0] * a.F + j] > 0.0 ? 1 : -1;
        if (sg > 0) S |= bit64(j);
    }
    const int jstar = (int)a.face_func[2 * g];
    if (jstar < 0) {
        if (a.sides) a.sides[2 * (g - a.f0)] = a.sides[2 * (g - a.f0) + 1] = S;
        else a.out[g - a.f0] = 0;
        return;
    }
    const int ls = __popcll(mask & (bit64(jstar) - 1));
    const int grp = r.rep[ls];
    uint64_t X = 0;
    for (int l = 0; l < r.k; ++l)
        if (r.rep[l] == grp) X |= bit64(local_func(mask, l));
    const uint64_t Sp = (S >> jstar) & 1 ? S : (S ^ X);
    if (a.sides) {
        a.sides[2 * (g - a.f0)] = Sp;
        a.sides[2 * (g - a.f0) + 1] = Sp ^ X;
        return;
    }
    const bool ip = csg_inside(a, Sp, full), in_ = csg_inside(a, Sp ^ X, full);
    a.out[g - a.f0] = ip == in_ ? 0 : (ip ? 1 : 2);
}

}  // namespace

void launch_csg(const CsgArgs& a, cudaStream_t s) {
    const int64_t n = a.f1 - a.f0;
    if (n <= 0) return;
    k_csg<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
    note_launch();
}

// ---- per-tet records and the active-function CRS, in tet order

namespace {

__global__ void k_rec_sizes(bool mi, int64_t A, const uint64_t* __restrict__ desc, RecSrc rs,
                            uint32_t* __restrict__ sz) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= A) return;
    const uint8_t* b = rs.get(desc[a]);
    sz[a] = mi ? mi_record_size(b) : ia_record_size(b);
}

__global__ void k_rec_copy(bool mi, int64_t A, const uint64_t* __restrict__ desc, RecSrc rs,
                           const uint32_t* __restrict__ off, uint8_t* __restrict__ dst) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= A) return;
    const uint8_t* b = rs.get(desc[a]);
    const int n = mi ? mi_record_size(b) : ia_record_size(b);
    for (int i = 0; i < n; ++i) dst[off[a] + i] = b[i];
}

__global__ void k_popc(int64_t A, const uint64_t* __restrict__ mask, uint32_t* __restrict__ k) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a < A) k[a] = __popcll(mask[a]);
}

__global__ void k_crs_fill(int64_t A, const uint64_t* __restrict__ mask, const uint32_t* __restrict__ off,
                           int64_t* __restrict__ vals) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= A) return;
    uint64_t m = mask[a];
    int64_t o = off[a];
    while (m) {
        vals[o++] = __ffsll((long long)m) - 1;
        m &= m - 1;
    }
}

}  // namespace

cudaError_t gather_records(bool mi, int64_t A, int64_t T, const uint32_t* act_tet, const uint64_t* act_desc,
                           const uint8_t* heap, const uint8_t* heap_big, const uint8_t* table,
                           const uint32_t* table_off, int64_t* d_rec_offsets, uint8_t** d_rec_bytes, int64_t* n_bytes,
                           cudaStream_t s) {
    Pool pool{s};
    RecSrc rs{heap, heap_big, table, table_off};
    uint32_t* sz = pool.get<uint32_t>(A);
    uint32_t* off = pool.get<uint32_t>(A);
    if (pool.err) return pool.err;
    if (A > 0) {
        k_rec_sizes<<<nblk(A), kBs, 0, s>>>(mi, A, act_desc, rs, sz);
        note_launch();
    }
    cudaError_t e = exscan_u32(sz, off, A, s);
    if (e != cudaSuccess) return e;
    int64_t total = 0;
    if ((e = scan_total(sz, off, A, &total, s)) != cudaSuccess) return e;
    *n_bytes = total;
    if ((e = cudaMallocAsync((void**)d_rec_bytes, (size_t)(total > 0 ? total : 1), s)) != cudaSuccess) return e;
    if (A > 0) {
        k_rec_copy<<<nblk(A), kBs, 0, s>>>(mi, A, act_desc, rs, off, *d_rec_bytes);
        note_launch();
    }
    {
        k_expand_offsets<<<nblk(T + 1), kBs, 0, s>>>(T, A, act_tet, off, sz, d_rec_offsets);
        note_launch();
    }
    return cudaGetLastError();
}

cudaError_t gather_func_in_tet(int64_t A, int64_t T, const uint32_t* act_tet, const uint64_t* act_mask,
                               int64_t* d_start, int64_t** d_vals, int64_t* n_vals, cudaStream_t s) {
    Pool pool{s};
    uint32_t* k = pool.get<uint32_t>(A);
    uint32_t* off = pool.get<uint32_t>(A);
    if (pool.err) return pool.err;
    if (A > 0) {
        k_popc<<<nblk(A), kBs, 0, s>>>(A, act_mask, k);
        note_launch();
    }
    cudaError_t e = exscan_u32(k, off, A, s);
    if (e != cudaSuccess) return e;
    int64_t total = 0;
    if ((e = scan_total(k, off, A, &total, s)) != cudaSuccess) return e;
    *n_vals = total;
    if ((e = cudaMallocAsync((void**)d_vals, sizeof(int64_t) * (size_t)(total > 0 ? total : 1), s)) != cudaSuccess)
        return e;
    if (A > 0) {
        k_crs_fill<<<nblk(A), kBs, 0, s>>>(A, act_mask, off, *d_vals);
        note_launch();
    }
    {
        k_expand_offsets<<<nblk(T + 1), kBs, 0, s>>>(T, A, act_tet, off, k, d_start);
        note_launch();
    }
    return cudaGetLastError();
}

}  // namespace ria
