// Stage (d) for the material interface: src/extract_mesh.cpp:569-986 (extract_MI_mesh) and
// :1541-1637 (compute_MI_vert_xyz).
//
// The reference walks the tets in order.  Per tet it
//   phase 0: numbers the vertices that lie on an interface face (keys: tet vertex v, tet edge
//            (v1, v2, m1, m2), tet face (v1, v2, v3, m1, m2, m3); vertices inside the tet are new);
//   phase 1: walks the faces: interface faces are always new; a face on the tet boundary is matched
//            with the face of the neighbouring tet (key: smallest, second smallest, largest vertex id,
//            tet vertices encoded as -v-1) and becomes an interface face, at its second occurrence,
//            when the two sides share no material; its tet-vertex corners may then be numbered.
// Here: phase-0 occurrences find their key's first occurrence by atomicMin on provisional
// positions; those owners serve as vertex identities to match the boundary faces (which needs only
// a consistent identity); only when some boundary face becomes an interface (degenerate inputs) are
// the positions recomputed with the phase-1 corners in place.  Scans number the new vertices and the
// faces in the reference's order.
#include "div_rn.cuh"
#include "extract_common.cuh"
#include "launch.hpp"

namespace ria {

using namespace xc;

namespace {

struct MICtx {
    ExtractArgs a;
    RecSrc rs;
    const U4* base0;        // per tet: phase-0 vertex, interface face, interface loop, boundary face bases
    uint32_t* corner_owner;
    HashTab he, hf, hb;
    uint32_t* hb_count;     // occurrences per boundary-face key
    // phase-0 occurrences (provisional positions)
    uint64_t* vocc0;
    uint64_t* vsrc0;
    uint32_t* ident;        // owner position = identity of the vertex
    // boundary-face occurrences
    uint64_t* bslot;
    uint64_t* bmask;        // materials of the cell inside the tet (bit set per global material)
    uint32_t* bemit;        // 1: becomes an interface face here
    // per tet: phase-1 corner occurrences, emitted faces, emitted loop lengths
    U4* extra;
    // final positions
    const U4* vbase;        // per tet: vertex occurrence base, face base, loop base
    uint64_t* vocc;
    uint64_t* vsrc;
    uint32_t* vowner;
    uint32_t* vflag;
    uint32_t* vgid_new;
    uint32_t* occ_gid;
    uint32_t* any_emit;
};


// flags of the local vertices on an interface face (vertex ids below 256)
__device__ __forceinline__ void mi_vertex_flags(const MIView& r, uint64_t f[4]) {
    f[0] = f[1] = f[2] = f[3] = 0;
    int off = 0;
    for (int i = 0; i < r.nf; ++i) {
        const int L = r.len(i);
        if (r.pos(i) > 3)
            for (int t = 0; t < L; ++t) {
                int v = r.loopv(off + t);
                f[v >> 6] |= 1ull << (v & 63);
            }
        off += L;
    }
}

__device__ __forceinline__ int flag_rank(const uint64_t f[4], int v) {
    int n = 0;
    for (int w = 0; w < (v >> 6); ++w) n += __popcll(f[w]);
    return n + __popcll(f[v >> 6] & ((1ull << (v & 63)) - 1));
}

__device__ __forceinline__ bool is_corner(const MIView& r, int v) {
    const uint8_t* lab = r.vlab + 4 * v;
    return lab[0] <= 3 && lab[1] <= 3 && lab[2] <= 3;
}

// materials (global ids) of the cell labelled `lab` (the group of identical materials)
__device__ __forceinline__ uint64_t group_mask(const MIView& r, int lab, uint64_t mask) {
    uint64_t m = 0;
    for (int j = 0; j < r.k; ++j)
        if (r.rep[j] == lab) m |= 1ull << local_func(mask, j);
    return m;
}

// M1: phase-0 keys
__global__ void __launch_bounds__(kBs) k_mi_vert_keys(MICtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.a.A) return;
    MIView r;
    r.init(C.rs.get(C.a.act_desc[a]));
    int64_t tv[4];
    TetSrc ts{C.a.d_tets, C.a.g.res};
    ts.get(C.a.act_tet[a], tv);
    const uint64_t mask = C.a.act_mask[a];
    uint64_t fl[4];
    mi_vertex_flags(r, fl);
    uint32_t pos = C.base0[a].a;
    for (int j = 0; j < r.nv; ++j) {
        if (!((fl[j >> 6] >> (j & 63)) & 1)) continue;
        MIKey k = mi_vertex_key(r, j, tv, mask);
        uint64_t occ;
        if (k.type == 1) {
            atomicMin(&C.corner_owner[k.sv[0]], pos);
            occ = (OCC_CORNER << 62) | (uint64_t)k.sv[0];
        } else if (k.type == 2) {
            int64_t s = ht_insert_min(C.he, ((uint64_t)k.sv[0] << 32) | (uint64_t)k.sv[1],
                                      ((uint64_t)k.mats[0] << 16) | (uint64_t)k.mats[1], pos);
            if (s < 0) raise_status(C.a.status, ST_HASH_FULL);
            occ = (OCC_EDGE << 62) | (uint64_t)(s < 0 ? 0 : s);
        } else if (k.type == 3) {
            int64_t s = ht_insert_min(C.hf, ((uint64_t)k.sv[0] << 32) | (uint64_t)k.sv[1],
                                      ((uint64_t)k.sv[2] << 32) | ((uint64_t)k.mats[0] << 20) |
                                          ((uint64_t)k.mats[1] << 10) | (uint64_t)k.mats[2],
                                      pos);
            if (s < 0) raise_status(C.a.status, ST_HASH_FULL);
            occ = (OCC_FACE << 62) | (uint64_t)(s < 0 ? 0 : s);
        } else {
            occ = OCC_SELF << 62;
        }
        C.vocc0[pos] = occ;
        C.vsrc0[pos] = ((uint64_t)a << 8) | (uint64_t)j;
        ++pos;
    }
}

__device__ __forceinline__ uint32_t owner_of(const MICtx& C, uint64_t occ, uint32_t self) {
    const uint64_t ty = occ >> 62, pay = occ & ((1ull << 62) - 1);
    if (ty == OCC_SELF) return self;
    if (ty == OCC_CORNER) return C.corner_owner[pay];
    if (ty == OCC_EDGE) return C.he.owner[pay];
    return C.hf.owner[pay];
}

// M2: identity of each phase-0 occurrence
__global__ void k_mi_ident(MICtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p < n) C.ident[p] = owner_of(C, C.vocc0[p], (uint32_t)p);
}

// 3 codes of at most 33 bits (tet vertices -v-1, identities >= 0) packed into 128 bits
__device__ __forceinline__ void pack3(int64_t a, int64_t b, int64_t c, uint64_t& k0, uint64_t& k1) {
    const uint64_t off = 1ull << 40;
    const uint64_t ua = (uint64_t)(a + (int64_t)off), ub = (uint64_t)(b + (int64_t)off), uc = (uint64_t)(c + (int64_t)off);
    k0 = ua | (ub << 41);
    k1 = (ub >> 23) | (uc << 18);
}

// encoded vertex of a boundary-face loop: tet corners -v-1, interface vertices their identity
__device__ __forceinline__ int64_t bnd_code(const MICtx& C, const MIView& r, int lv, const int64_t tv[4],
                                            const uint64_t fl[4], uint32_t b0) {
    if (is_corner(r, lv)) return -tv[corner_of(r.vlab + 4 * lv, 3)] - 1;
    if (!((fl[lv >> 6] >> (lv & 63)) & 1)) {  // every other boundary vertex lies on an interface
        raise_status(C.a.status, ST_INTERNAL);
        return 0;
    }
    return (int64_t)C.ident[b0 + flag_rank(fl, lv)];
}

// M3: keys of the boundary faces
__global__ void __launch_bounds__(kBs) k_mi_bnd_keys(MICtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.a.A) return;
    MIView r;
    r.init(C.rs.get(C.a.act_desc[a]));
    int64_t tv[4];
    TetSrc ts{C.a.d_tets, C.a.g.res};
    ts.get(C.a.act_tet[a], tv);
    const uint64_t mask = C.a.act_mask[a];
    uint64_t fl[4];
    mi_vertex_flags(r, fl);
    const uint32_t b0 = C.base0[a].a;
    uint32_t bpos = C.base0[a].d;
    int off = 0;
    for (int f = 0; f < r.nf; ++f) {
        const int L = r.len(f);
        if (r.pos(f) <= 3) {
            // smallest, second smallest (of the other vertices) and largest code in one walk
            int64_t mn = 0, mx = 0, second = INT64_MAX;
            for (int t = 0; t < L; ++t) {
                const int64_t c = bnd_code(C, r, r.loopv(off + t), tv, fl, b0);
                if (t == 0) {
                    mn = mx = c;
                    continue;
                }
                if (c < mn) {
                    second = mn;
                    mn = c;
                } else if (c < second) {
                    second = c;
                }
                if (c > mx) mx = c;
            }
            if (L < 2) second = mx + 1;
            uint64_t k0, k1;
            pack3(mn, second, mx, k0, k1);
            int64_t s = ht_insert_min(C.hb, k0, k1, bpos);
            if (s < 0) {
                raise_status(C.a.status, ST_HASH_FULL);
                s = 0;
            } else {
                atomicAdd(&C.hb_count[s], 1u);
            }
            C.bslot[bpos] = (uint64_t)s;
            C.bmask[bpos] = group_mask(r, r.neg(f), mask);
            ++bpos;
        }
        off += L;
    }
}

// M4: a boundary face becomes an interface face at the second occurrence of its key when the two
// sides share no material (src/extract_mesh.cpp:866-950, with at most two tets per face)
__global__ void k_mi_bnd_emit(MICtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint64_t s = C.bslot[p];
    const uint32_t cnt = C.hb_count[s];
    const uint32_t own = C.hb.owner[s];
    if (cnt > 2) raise_status(C.a.status, ST_NONMANIFOLD);
    uint32_t e = (cnt == 2 && own != (uint32_t)p && (C.bmask[p] & C.bmask[own]) == 0) ? 1u : 0u;
    C.bemit[p] = e;
    if (e) atomicOr(C.any_emit, 1u);
}

// M5 (only with emitted faces): per tet, phase-1 corner occurrences and emitted faces/loops
__global__ void __launch_bounds__(kBs) k_mi_extra(MICtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.a.A) return;
    MIView r;
    r.init(C.rs.get(C.a.act_desc[a]));
    uint32_t bpos = C.base0[a].d;
    uint32_t n1 = 0, ne = 0, nl = 0;
    int off = 0;
    for (int f = 0; f < r.nf; ++f) {
        const int L = r.len(f);
        if (r.pos(f) <= 3) {
            if (C.bemit[bpos]) {
                ++ne;
                nl += L;
                for (int t = 0; t < L; ++t) n1 += is_corner(r, r.loopv(off + t));
            }
            ++bpos;
        }
        off += L;
    }
    C.extra[a] = U4{n1, ne, nl, 0};
}

__global__ void k_mi_final_counts(int64_t A, const IASum4* __restrict__ sum, const U4* __restrict__ extra,
                                  U4* __restrict__ out) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= A) return;
    const IASum4 s = sum[a];
    const U4 e = extra ? extra[a] : U4{0, 0, 0, 0};
    out[a] = U4{(uint32_t)s.a + e.a, (uint32_t)s.b + e.b, (uint32_t)s.c + e.c, 0};
}

// totals of the final positions (vertex occurrences, faces, loop vertices) and whether any boundary
// face became an interface; with `nv`, the number of new vertices as well
__global__ void k_mi_totals(int64_t A, const U4* __restrict__ fin, const U4* __restrict__ vbase,
                            const uint32_t* __restrict__ any_emit, int64_t nv, const uint32_t* __restrict__ vflag,
                            const uint32_t* __restrict__ vgid_new, int64_t* __restrict__ d) {
    if (nv >= 0) {
        d[4] = nv ? (int64_t)vflag[nv - 1] + (int64_t)vgid_new[nv - 1] : 0;
        return;
    }
    const U4 t = A ? U4Sum()(fin[A - 1], vbase[A - 1]) : U4{0, 0, 0, 0};
    d[0] = t.a;
    d[1] = t.b;
    d[2] = t.c;
    d[3] = *any_emit;
}

// closing entries of the two offset arrays
__global__ void k_mi_close(int64_t* __restrict__ face_offsets, int64_t* __restrict__ face_tet_offsets, int64_t NF,
                           int64_t NL) {
    face_offsets[NF] = NL;
    face_tet_offsets[NF] = NF;
}

// M6 (only with emitted faces): occurrences at their final positions; owners recomputed
__global__ void __launch_bounds__(kBs) k_mi_final_occ(MICtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.a.A) return;
    MIView r;
    r.init(C.rs.get(C.a.act_desc[a]));
    int64_t tv[4];
    TetSrc ts{C.a.d_tets, C.a.g.res};
    ts.get(C.a.act_tet[a], tv);
    const uint32_t b0 = C.base0[a].a;
    uint32_t pos = C.vbase[a].a;
    uint64_t fl[4];
    mi_vertex_flags(r, fl);
    const int cnt0 = __popcll(fl[0]) + __popcll(fl[1]);
    for (int i = 0; i < cnt0; ++i) {
        const uint64_t occ = C.vocc0[b0 + i];
        C.vocc[pos] = occ;
        C.vsrc[pos] = C.vsrc0[b0 + i];
        const uint64_t ty = occ >> 62, pay = occ & ((1ull << 62) - 1);
        if (ty == OCC_CORNER) atomicMin(&C.corner_owner[pay], pos);
        else if (ty == OCC_EDGE) atomicMin(&C.he.owner[pay], pos);
        else if (ty == OCC_FACE) atomicMin(&C.hf.owner[pay], pos);
        ++pos;
    }
    uint32_t bpos = C.base0[a].d;
    int off = 0;
    for (int f = 0; f < r.nf; ++f) {
        const int L = r.len(f);
        if (r.pos(f) <= 3) {
            if (C.bemit[bpos]) {
                for (int t = 0; t < L; ++t) {
                    const int lv = r.loopv(off + t);
                    if (!is_corner(r, lv)) continue;
                    const int64_t v = tv[corner_of(r.vlab + 4 * lv, 3)];
                    atomicMin(&C.corner_owner[v], pos);
                    C.vocc[pos] = (OCC_CORNER << 62) | (uint64_t)v;
                    C.vsrc[pos] = ((uint64_t)a << 8) | (uint64_t)lv;
                    ++pos;
                }
            }
            ++bpos;
        }
        off += L;
    }
}

__global__ void k_mi_owner(MICtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint32_t own = owner_of(C, C.vocc[p], (uint32_t)p);
    C.vowner[p] = own;
    C.vflag[p] = own == (uint32_t)p;
}

// M7: vertex records and coordinates (compute_MI_vert_xyz: differences of consecutive materials)
// the global vertex id of every occurrence (the face pass reads them)
__global__ void k_mi_gid(MICtx C, int64_t n) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    C.occ_gid[p] = C.vgid_new[C.vowner[p]];
}

__global__ void k_mi_vert_emit(MICtx C, int64_t n, int64_t* __restrict__ verts, double* __restrict__ xyz) {
    const int64_t p = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (p >= n) return;
    const uint32_t own = C.vowner[p];
    if (own != (uint32_t)p) return;
    const uint32_t gid = C.vgid_new[p];
    const uint64_t src = C.vsrc[p];
    const int64_t a = (int64_t)(src >> 8);
    const int j = (int)(src & 0xFF);
    MIView r;
    r.init(C.rs.get(C.a.act_desc[a]));
    int64_t tv[4];
    TetSrc ts{C.a.d_tets, C.a.g.res};
    const uint32_t tet = C.a.act_tet[a];
    ts.get(tet, tv);
    MIKey k = mi_vertex_key(r, j, tv, C.a.act_mask[a]);
    int64_t* rec = verts + 11 * (int64_t)gid;
    rec[0] = tet;
    rec[1] = j;
    rec[2] = k.type;
    for (int c = 0; c < 4; ++c) rec[3 + c] = k.sv[c];
    for (int c = 0; c < 4; ++c) rec[7 + c] = k.type == 1 ? -1 : k.mats[c];
    PtSrc ps{C.a.d_pts, C.a.coords, (int)C.a.g.res + 1};
    const double* fv = C.a.fv;
    const int F = C.a.F;
    double out[3];
    auto diff = [&](int64_t v, int i0, int i1) { return fv[v * F + k.mats[i0]] - fv[v * F + k.mats[i1]]; };
    switch (k.type) {
        case 2: {
            double p1[3], p2[3];
            ps.get(k.sv[0], p1);
            ps.get(k.sv[1], p2);
            double f1 = diff(k.sv[0], 0, 1), f2 = diff(k.sv[1], 0, 1);
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
                a1[t] = diff(k.sv[t], 0, 1);
                a2[t] = diff(k.sv[t], 1, 2);
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
                p1[t] = diff(k.sv[t], 0, 1);
                p2[t] = diff(k.sv[t], 1, 2);
                p3[t] = diff(k.sv[t], 2, 3);
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
    for (int c = 0; c < 3; ++c) xyz[3 * (int64_t)gid + c] = out[c];
}

// M8: faces in the reference's order: interface faces, and boundary faces that became interfaces
__global__ void __launch_bounds__(kBs) k_mi_face_emit(MICtx C, bool with_extra, int64_t* __restrict__ face_offsets,
                                                      int64_t* __restrict__ face_verts,
                                                      int64_t* __restrict__ face_tet_offsets,
                                                      int64_t* __restrict__ face_tets,
                                                      int64_t* __restrict__ face_func) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.a.A) return;
    MIView r;
    r.init(C.rs.get(C.a.act_desc[a]));
    int64_t tv[4];
    TetSrc ts{C.a.d_tets, C.a.g.res};
    const uint32_t tet = C.a.act_tet[a];
    ts.get(tet, tv);
    const uint64_t mask = C.a.act_mask[a];
    uint64_t fl[4];
    mi_vertex_flags(r, fl);
    const uint32_t vb = C.vbase[a].a;
    uint32_t fpos = C.vbase[a].b;
    uint32_t lpos = C.vbase[a].c;
    uint32_t bpos = C.base0[a].d;
    int off = 0;
    for (int f = 0; f < r.nf; ++f) {
        const int L = r.len(f);
        const int pl = r.pos(f), ng = r.neg(f);
        bool emit = pl > 3;
        uint64_t other = 0;
        if (pl <= 3) {
            if (with_extra && C.bemit[bpos]) {
                emit = true;
                other = C.bmask[C.hb.owner[C.bslot[bpos]]];
            }
        }
        if (emit) {
            face_offsets[fpos] = lpos;
            face_tet_offsets[fpos] = fpos;
            face_tets[2 * (int64_t)fpos] = tet;
            face_tets[2 * (int64_t)fpos + 1] = f;
            for (int t = 0; t < L; ++t) {
                const int lv = r.loopv(off + t);
                int64_t g;
                if (pl <= 3 && is_corner(r, lv)) {
                    g = C.occ_gid[C.corner_owner[tv[corner_of(r.vlab + 4 * lv, 3)]]];
                } else {
                    g = C.occ_gid[vb + flag_rank(fl, lv)];
                }
                face_verts[lpos + t] = g;
            }
            if (pl > 3) {
                face_func[2 * (int64_t)fpos] = local_func(mask, pl - 4);
                face_func[2 * (int64_t)fpos + 1] = local_func(mask, ng - 4);
            } else {
                // the reference indexes material_in_tet with a tet-face label here
                // (src/extract_mesh.cpp:979); this build reports (larger, smaller) of the two sides
                const uint64_t here = C.bmask[bpos];
                const int mh = __ffsll((long long)here) - 1, mo = __ffsll((long long)other) - 1;
                face_func[2 * (int64_t)fpos] = mh > mo ? mh : mo;
                face_func[2 * (int64_t)fpos + 1] = mh > mo ? mo : mh;
            }
            ++fpos;
            lpos += L;
        }
        if (pl <= 3) ++bpos;
        off += L;
    }
}

}  // namespace

cudaError_t run_extract_mi(const ExtractArgs& a, const IASum4* act_sum, const ExtractBases* pre, ExtractOut& out,
                           cudaStream_t s) {
    Pool pool{s};
    MICtx C;
    C.a = a;
    C.rs = RecSrc{a.heap, a.heap_big, a.table, a.table_off};
    const int64_t A = a.A;
    out = ExtractOut();
    // phase-0 bases: prepared by the caller (their totals read with the cut stage's synchronization),
    // or here
    U4 tot{0, 0, 0, 0};
    if (pre && (pre->base || A == 0)) {
        C.base0 = (const U4*)pre->base;
        tot = U4{(uint32_t)pre->total[0], (uint32_t)pre->total[1], (uint32_t)pre->total[2], (uint32_t)pre->total[3]};
    } else {
        U4* bin = pool.get<U4>(A);
        U4* base0 = pool.get<U4>(A);
        if (pool.err) return pool.err;
        if (A > 0) {
            k_base_in<<<nblk(A), kBs, 0, s>>>(A, act_sum, bin);
            note_launch();
        }
        cudaError_t e = exscan_u4(bin, base0, A, &tot, pool, s);
        if (e != cudaSuccess) return e;
        C.base0 = base0;
    }
    const int64_t NV0 = tot.a, NB = tot.d;
    const uint64_t cap_e = pow2_at_least((uint64_t)NV0), cap_f = pow2_at_least((uint64_t)NV0 / 2 + 1);
    const uint64_t cap_b = pow2_at_least(2 * (uint64_t)NB + 1);
    uint64_t* pin = nullptr;
    AuxStream* aux = nullptr;
    cudaError_t e = pinned_words(&pin);
    if (e == cudaSuccess) e = aux_stream(&aux);
    if (e != cudaSuccess) return e;
    // every buffer of the first phases carved from one allocation (the sizes are added up first)
    U4 *fin = nullptr, *vbase = nullptr;
    int64_t* d_tot = nullptr;
    void* scan_tmp = nullptr;
    size_t fscan_bytes = 0;
    if (A > 0) cub::DeviceScan::ExclusiveScan(nullptr, fscan_bytes, fin, vbase, U4Sum(), U4{0, 0, 0, 0}, A, s);
    auto carve = [&](Pool& P) {
        C.corner_owner = P.get<uint32_t>(a.V);
        C.he = HashTab{P.get<ulonglong2>((int64_t)cap_e), P.get<uint32_t>((int64_t)cap_e), cap_e - 1};
        C.hf = HashTab{P.get<ulonglong2>((int64_t)cap_f), P.get<uint32_t>((int64_t)cap_f), cap_f - 1};
        C.hb = HashTab{P.get<ulonglong2>((int64_t)cap_b), P.get<uint32_t>((int64_t)cap_b), cap_b - 1};
        C.hb_count = P.get<uint32_t>((int64_t)cap_b);
        C.vocc0 = P.get<uint64_t>(NV0);
        C.vsrc0 = P.get<uint64_t>(NV0);
        C.ident = P.get<uint32_t>(NV0);
        C.bslot = P.get<uint64_t>(NB);
        C.bmask = P.get<uint64_t>(NB);
        C.bemit = P.get<uint32_t>(NB);
        C.any_emit = P.get<uint32_t>(1);
        C.extra = P.get<U4>(A);
        fin = P.get<U4>(A);
        vbase = P.get<U4>(A);
        d_tot = P.get<int64_t>(8);
        scan_tmp = P.get<uint8_t>((int64_t)fscan_bytes);
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
        fill.add(h->keys, sizeof(ulonglong2) * (h->cap_mask + 1), ~0u);
        fill.add(h->owner, sizeof(uint32_t) * (h->cap_mask + 1), ~0u);
    }
    fill.add(C.hb_count, sizeof(uint32_t) * cap_b, 0u);
    fill.add(C.any_emit, sizeof(uint32_t), 0u);
    if ((e = launch_fill(fill, s)) != cudaSuccess) return e;
    if (A > 0) {
        k_mi_vert_keys<<<nblk(A), kBs, 0, s>>>(C);
        note_launch();
    }
    if (NV0 > 0) {
        k_mi_ident<<<nblk(NV0), kBs, 0, s>>>(C, NV0);
        note_launch();
    }
    if (A > 0) {
        k_mi_bnd_keys<<<nblk(A), kBs, 0, s>>>(C);
        note_launch();
    }
    if (NB > 0) {
        k_mi_bnd_emit<<<nblk(NB), kBs, 0, s>>>(C, NB);
        note_launch();
    }
    // final positions: the emitted boundary faces' counts (zero when none became an interface) added
    // to the phase-0 counts; their totals and the emission flag come back in one synchronization
    if (A > 0) {
        k_mi_extra<<<nblk(A), kBs, 0, s>>>(C);
        note_launch();
        k_mi_final_counts<<<nblk(A), kBs, 0, s>>>(A, act_sum, C.extra, fin);
        note_launch();
        cub::DeviceScan::ExclusiveScan(scan_tmp, fscan_bytes, fin, vbase, U4Sum(), U4{0, 0, 0, 0}, A, s);
    }
    k_mi_totals<<<1, 1, 0, s>>>(A, fin, vbase, C.any_emit, -1, nullptr, nullptr, d_tot);
    note_launch();
    cudaMemcpyAsync(pin, d_tot, 4 * sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    const int64_t NV = (int64_t)pin[0], NF = (int64_t)pin[1], NL = (int64_t)pin[2];
    const bool h_emit = pin[3] != 0;
    C.vbase = vbase;
    size_t vscan_bytes = 0;
    if (NV > 0) cub::DeviceScan::ExclusiveSum(nullptr, vscan_bytes, (const uint32_t*)nullptr, (uint32_t*)nullptr, NV, s);
    void* vscan_tmp = nullptr;
    auto carve2 = [&](Pool& P) {
        if (h_emit) {
            C.vocc = P.get<uint64_t>(NV);
            C.vsrc = P.get<uint64_t>(NV);
        }
        C.vowner = P.get<uint32_t>(NV);
        C.vflag = P.get<uint32_t>(NV);
        C.vgid_new = P.get<uint32_t>(NV);
        C.occ_gid = P.get<uint32_t>(NV);
        vscan_tmp = P.get<uint8_t>((int64_t)vscan_bytes);
    };
    pool.measuring = true;
    pool.measured = 0;
    carve2(pool);
    pool.measuring = false;
    pool.reserve(pool.measured);
    carve2(pool);
    if (pool.err) return pool.err;
    if (h_emit) {
        FillList refill;
        refill.add(C.corner_owner, sizeof(uint32_t) * (size_t)(a.V > 0 ? a.V : 1), ~0u);
        refill.add(C.he.owner, sizeof(uint32_t) * (C.he.cap_mask + 1), ~0u);
        refill.add(C.hf.owner, sizeof(uint32_t) * (C.hf.cap_mask + 1), ~0u);
        if ((e = launch_fill(refill, s)) != cudaSuccess) return e;
        k_mi_final_occ<<<nblk(A), kBs, 0, s>>>(C);
        note_launch();
    } else {
        C.vocc = C.vocc0;
        C.vsrc = C.vsrc0;
    }
    if (NV > 0) {
        k_mi_owner<<<nblk(NV), kBs, 0, s>>>(C, NV);
        note_launch();
        cub::DeviceScan::ExclusiveSum(vscan_tmp, vscan_bytes, C.vflag, C.vgid_new, NV, s);
        k_mi_gid<<<nblk(NV), kBs, 0, s>>>(C, NV);
        note_launch();
    }
    // the vertex count goes to pinned memory while the faces are emitted; the vertex outputs are
    // allocated when it arrives
    k_mi_totals<<<1, 1, 0, s>>>(A, nullptr, nullptr, nullptr, NV, C.vflag, C.vgid_new, d_tot);
    note_launch();
    cudaMemcpyAsync(pin + 4, d_tot + 4, sizeof(int64_t), cudaMemcpyDeviceToHost, s);
    cudaEventRecord(aux->fork, s);
    out.n_faces = NF;
    out.n_face_verts = NL;
    out.n_face_tets = NF;
    if ((e = cudaMallocAsync((void**)&out.face_offsets, sizeof(int64_t) * (size_t)(NF + 1), s)) != cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_verts, sizeof(int64_t) * (size_t)(NL > 0 ? NL : 1), s)) != cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_tet_offsets, sizeof(int64_t) * (size_t)(NF + 1), s)) != cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_tets, sizeof(int64_t) * 2 * (size_t)(NF > 0 ? NF : 1), s)) !=
            cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.face_func, sizeof(int64_t) * 2 * (size_t)(NF > 0 ? NF : 1), s)) !=
            cudaSuccess)
        return e;
    if (A > 0) {
        k_mi_face_emit<<<nblk(A), kBs, 0, s>>>(C, h_emit, out.face_offsets, out.face_verts, out.face_tet_offsets,
                                             out.face_tets, out.face_func);
        note_launch();
    }
    k_mi_close<<<1, 1, 0, s>>>(out.face_offsets, out.face_tet_offsets, NF, NL);
    note_launch();
    if ((e = cudaEventSynchronize(aux->fork)) != cudaSuccess) return e;
    const int64_t n_verts = (int64_t)pin[4];
    out.n_verts = n_verts;
    if ((e = cudaMallocAsync((void**)&out.xyz, sizeof(double) * 3 * (size_t)(n_verts > 0 ? n_verts : 1), s)) !=
            cudaSuccess ||
        (e = cudaMallocAsync((void**)&out.verts, sizeof(int64_t) * 11 * (size_t)(n_verts > 0 ? n_verts : 1), s)) !=
            cudaSuccess)
        return e;
    if (NV > 0) {
        k_mi_vert_emit<<<nblk(NV), kBs, 0, s>>>(C, NV, out.verts, out.xyz);
        note_launch();
    }
    return cudaGetLastError();
}

}  // namespace ria
