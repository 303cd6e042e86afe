// Local-to-global maps of a finished mesh: the outputs of the reference's extraction variants used
// when useTopoRayShooting is off (src/implicit_arrangement.cpp:370-385):
//   global_vId_of_tet_vert  per record vertex of every active tet: its mesh vertex, or -v-1 for a tet
//                           corner (a vertex on no iso / interface face, or one lying on a tet vertex);
//   iso_fId_of_tet_face     per record face: its mesh face, or -1 (Mesh_None) for a face that is not
//   / MI_fId_of_tet_face    on the surface; a material-interface face on the tet boundary is set in
//                           both tets that share it (src/extract_mesh.cpp:1431);
// each a CRS over all tets (src/extract_mesh.cpp:268-566, 988-1443).
//
// They are computed after the extraction, from the per-tet records and the mesh:
//   * vertices: every mesh vertex that is not a tet corner is inserted in a hash under the key the
//     extraction deduplicated it by (tet edge, tet face, or (tet, local vertex) inside a tet); every
//     record vertex then looks its key up;
//   * faces: the mesh's tet-face lists name every occurrence of an implicit-arrangement face, and the
//     occurrence at which a material-interface face was made; the other occurrence of a boundary
//     material-interface face is the first record face of the same key (smallest, second smallest,
//     largest vertex id, corners as -v-1), found by atomicMin of the record-face positions.
#include "extract_common.cuh"
#include "launch.hpp"

namespace ria {

using namespace xc;

namespace {

// 128-bit key of a mesh vertex that is not a tet corner: vertex ids below 2^31 (31 bits each),
// function / material ids below 127 (7 bits each, stored + 1), the simplex size in the top bits;
// a vertex inside a tet is keyed by (tet, local vertex).
__device__ __forceinline__ void vkey(int type, const int64_t sv[4], const int fn[3], int64_t tet, int local,
                                     uint64_t& lo, uint64_t& hi) {
    if (type == 4) {
        lo = (uint64_t)tet;
        hi = (4ull << 56) | (uint64_t)local;
        return;
    }
    const uint64_t a = type >= 1 ? (uint64_t)sv[0] : 0, b = type >= 2 ? (uint64_t)sv[1] : 0,
                   c = type >= 3 ? (uint64_t)sv[2] : 0;
    lo = a | (b << 31) | ((c & 3) << 62);
    hi = (c >> 2) | ((uint64_t)(fn[0] + 1) << 29) | ((uint64_t)(fn[1] + 1) << 36) | ((uint64_t)(fn[2] + 1) << 43) |
         ((uint64_t)type << 56);
}

__device__ __forceinline__ int64_t ht_find(const HashTab& h, uint64_t k0, uint64_t k1) {
    uint64_t slot = mix64(k0 * 0x9E3779B97F4A7C15ull ^ mix64(k1)) & h.cap_mask;
    for (uint64_t probe = 0; probe <= h.cap_mask; ++probe) {
        const ulonglong2 k = h.keys[slot];
        if (k.x == k0 && k.y == k1) return (int64_t)slot;
        if (k.x == ~0ull && k.y == ~0ull) return -1;
        slot = (slot + 1) & h.cap_mask;
    }
    return -1;
}

struct MapCtx {
    bool mi;
    int64_t A;
    const uint32_t* act_tet;
    const uint64_t* act_desc;
    const uint64_t* act_mask;
    RecSrc rs;
    TetSrc ts;
    const int64_t* verts;  // mesh vertex records [n][11]
    int64_t n_verts;
    HashTab hv;            // mesh vertex keys -> owner = vertex id
    HashTab hb;            // boundary-face keys (material interface) -> first record-face position
    const uint32_t* vbase;  // per active tet: first entry in the vertex map
    const uint32_t* fbase;  // per active tet: first entry in the face map
    int64_t* tet_verts;
    int64_t* tet_faces;
    uint32_t* status;
};

__global__ void k_map_counts(MapCtx C, uint32_t* __restrict__ nv, uint32_t* __restrict__ nf) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.A) return;
    const uint8_t* b = C.rs.get(C.act_desc[a]);
    nv[a] = rd16(b + 2);
    nf[a] = rd16(b + 4);
}

// every mesh vertex that is not on a tet vertex, under its extraction key
__global__ void k_map_insert_verts(MapCtx C) {
    const int64_t g = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (g >= C.n_verts) return;
    const int64_t* r = C.verts + 11 * g;
    const int type = (int)r[2];
    if (type == 1) return;
    const int fn[3] = {(int)r[7], (int)r[8], (int)r[9]};
    uint64_t lo, hi;
    vkey(type, r + 3, fn, r[0], (int)r[1], lo, hi);
    if (ht_insert_min(C.hv, lo, hi, (uint32_t)g) < 0) raise_status(C.status, ST_HASH_FULL);
}

// the vertex map of every active tet (and, for the material interface, the boundary-face keys)
__global__ void __launch_bounds__(kBs) k_map_verts(MapCtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.A) return;
    const uint8_t* b = C.rs.get(C.act_desc[a]);
    int64_t tv[4];
    const int64_t tet = C.act_tet[a];
    C.ts.get(tet, tv);
    const uint64_t mask = C.act_mask[a];
    int64_t* out = C.tet_verts + C.vbase[a];
    if (!C.mi) {
        IAView r;
        r.init(b);
        uint64_t iso[4];
        iso_vertex_flags(r, iso);
        for (int j = 0; j < r.nv; ++j) {
            const VertKey k = ia_vertex_key(r, j, tv, mask);
            int64_t g;
            if (k.type == 1) {
                g = -k.sv[0] - 1;
            } else if (!((iso[j >> 6] >> (j & 63)) & 1)) {
                raise_status(C.status, ST_INTERNAL);  // a vertex on no iso face is a tet corner
                g = -1;
            } else {
                uint64_t lo, hi;
                vkey(k.type, k.sv, k.fn, tet, j, lo, hi);
                const int64_t s = ht_find(C.hv, lo, hi);
                if (s < 0) raise_status(C.status, ST_INTERNAL);
                g = s < 0 ? -1 : (int64_t)C.hv.owner[s];
            }
            out[j] = g;
        }
        return;
    }
    MIView r;
    r.init(b);
    uint64_t mif[4] = {0, 0, 0, 0};  // vertices of a face inside the tet
    {
        int off = 0;
        for (int f = 0; f < r.nf; ++f) {
            const int L = r.len(f);
            if (r.pos(f) > 3)
                for (int t = 0; t < L; ++t) {
                    const int v = r.loopv(off + t);
                    mif[v >> 6] |= 1ull << (v & 63);
                }
            off += L;
        }
    }
    for (int j = 0; j < r.nv; ++j) {
        const MIKey k = mi_vertex_key(r, j, tv, mask);
        int64_t g;
        if (!((mif[j >> 6] >> (j & 63)) & 1)) {
            // a vertex on no interface face is a tet vertex (src/extract_mesh.cpp:1112-1128)
            g = -tv[corner_of(r.vlab + 4 * j, 3)] - 1;
        } else if (k.type == 1) {
            g = -k.sv[0] - 1;
        } else {
            const int fn[3] = {k.mats[0], k.mats[1], k.type == 4 ? -1 : k.mats[2]};
            uint64_t lo, hi;
            vkey(k.type, k.sv, fn, tet, j, lo, hi);
            const int64_t s = ht_find(C.hv, lo, hi);
            if (s < 0) raise_status(C.status, ST_INTERNAL);
            g = s < 0 ? -1 : (int64_t)C.hv.owner[s];
        }
        out[j] = g;
    }
}

// key of a record face on the tet boundary: (smallest, second smallest, largest) entry of the
// vertex map over its loop (src/extract_mesh.h:68-92); entries are >= -2^31 and < 2^31
__device__ __forceinline__ void bface_key(const MIView& r, int loff, int L, const int64_t* vmap, uint64_t& lo,
                                          uint64_t& hi) {
    int64_t mn = 0, mx = 0;
    int mpos = 0;
    for (int t = 0; t < L; ++t) {
        const int64_t v = vmap[r.loopv(loff + t)];
        if (t == 0 || v < mn) {
            mn = v;
            mpos = t;
        }
        if (t == 0 || v > mx) mx = v;
    }
    int64_t second = mx;
    bool have = false;
    for (int t = 0; t < L; ++t) {
        const int64_t v = vmap[r.loopv(loff + t)];
        if (t != mpos && (!have || v < second)) {
            second = v;
            have = true;
        }
    }
    lo = ((uint64_t)(uint32_t)(int32_t)mn << 32) | (uint64_t)(uint32_t)(int32_t)second;
    hi = (uint64_t)(uint32_t)(int32_t)mx;
}

// material interface: every boundary record face under its key, first occurrence by position
__global__ void __launch_bounds__(kBs) k_map_bfaces(MapCtx C) {
    const int64_t a = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (a >= C.A) return;
    MIView r;
    r.init(C.rs.get(C.act_desc[a]));
    const int64_t* vmap = C.tet_verts + C.vbase[a];
    int off = 0;
    for (int f = 0; f < r.nf; ++f) {
        const int L = r.len(f);
        if (r.pos(f) <= 3) {
            uint64_t lo, hi;
            bface_key(r, off, L, vmap, lo, hi);
            if (ht_insert_min(C.hb, lo, hi, C.fbase[a] + (uint32_t)f) < 0) raise_status(C.status, ST_HASH_FULL);
        }
        off += L;
    }
}

// every occurrence the mesh lists; for a material-interface face on the tet boundary also the other
// occurrence of its key
__global__ void k_map_faces(MapCtx C, int64_t n_faces, const int64_t* __restrict__ face_tet_offsets,
                            const int64_t* __restrict__ face_tets, const int64_t* __restrict__ tet_face_offsets) {
    const int64_t f = (int64_t)blockIdx.x * kBs + threadIdx.x;
    if (f >= n_faces) return;
    for (int64_t e = face_tet_offsets[f]; e < face_tet_offsets[f + 1]; ++e) {
        const int64_t t = face_tets[2 * e], j = face_tets[2 * e + 1];
        C.tet_faces[tet_face_offsets[t] + j] = f;
        if (!C.mi) continue;
        // active index of tet t (act_tet is sorted)
        int64_t lo = 0, hi = C.A;
        while (lo < hi) {
            const int64_t mid = (lo + hi) >> 1;
            if ((int64_t)C.act_tet[mid] < t) lo = mid + 1;
            else hi = mid;
        }
        if (lo >= C.A || (int64_t)C.act_tet[lo] != t) {
            raise_status(C.status, ST_INTERNAL);
            continue;
        }
        MIView r;
        r.init(C.rs.get(C.act_desc[lo]));
        if (r.pos((int)j) > 3) continue;
        int off = 0;
        for (int x = 0; x < (int)j; ++x) off += r.len(x);
        uint64_t k0, k1;
        bface_key(r, off, r.len((int)j), C.tet_verts + C.vbase[lo], k0, k1);
        const int64_t s = ht_find(C.hb, k0, k1);
        if (s < 0) {
            raise_status(C.status, ST_INTERNAL);
            continue;
        }
        C.tet_faces[C.hb.owner[s]] = f;
    }
}

}  // namespace

cudaError_t gather_tet_maps(const TetMapArgs& m, int64_t* d_vert_offsets, int64_t* d_face_offsets,
                            int64_t** d_tet_verts, int64_t* n_tet_verts, int64_t** d_tet_faces, int64_t* n_tet_faces,
                            cudaStream_t s) {
    Pool pool{s};
    MapCtx C{};
    C.mi = m.mi;
    C.A = m.A;
    C.act_tet = m.act_tet;
    C.act_desc = m.act_desc;
    C.act_mask = m.act_mask;
    C.rs = RecSrc{m.heap, m.heap_big, m.table, m.table_off};
    C.ts = TetSrc{m.d_tets, m.res};
    C.verts = m.verts;
    C.n_verts = m.n_verts;
    C.status = pool.get<uint32_t>(1);
    uint32_t* nv = pool.get<uint32_t>(m.A);
    uint32_t* nf = pool.get<uint32_t>(m.A);
    uint32_t* vb = pool.get<uint32_t>(m.A);
    uint32_t* fb = pool.get<uint32_t>(m.A);
    if (pool.err) return pool.err;
    cudaMemsetAsync(C.status, 0, 4, s);
    if (m.A > 0) {
        k_map_counts<<<nblk(m.A), kBs, 0, s>>>(C, nv, nf);
        note_launch();
    }
    cudaError_t e;
    if ((e = exscan_u32(nv, vb, m.A, s)) != cudaSuccess) return e;
    if ((e = exscan_u32(nf, fb, m.A, s)) != cudaSuccess) return e;
    ScanTotals st;
    st.add(nv, vb, m.A);
    st.add(nf, fb, m.A);
    int64_t tots[2] = {0, 0};
    if ((e = read_totals(st, tots, pool, s)) != cudaSuccess) return e;
    *n_tet_verts = tots[0];
    *n_tet_faces = tots[1];
    if (tots[1] >= (1ll << 32) - 1) return cudaErrorInvalidValue;  // record-face positions are 32-bit
    C.vbase = vb;
    C.fbase = fb;
    if ((e = cudaMallocAsync((void**)d_tet_verts, sizeof(int64_t) * (size_t)(tots[0] > 0 ? tots[0] : 1), s)) !=
        cudaSuccess)
        return e;
    if ((e = cudaMallocAsync((void**)d_tet_faces, sizeof(int64_t) * (size_t)(tots[1] > 0 ? tots[1] : 1), s)) !=
        cudaSuccess)
        return e;
    C.tet_verts = *d_tet_verts;
    C.tet_faces = *d_tet_faces;
    cudaMemsetAsync(C.tet_faces, 0xFF, sizeof(int64_t) * (size_t)(tots[1] > 0 ? tots[1] : 1), s);
    if (m.T >= 0) {
        k_expand_offsets<<<nblk(m.T + 1), kBs, 0, s>>>(m.T, m.A, m.act_tet, vb, nv, d_vert_offsets);
        note_launch();
        k_expand_offsets<<<nblk(m.T + 1), kBs, 0, s>>>(m.T, m.A, m.act_tet, fb, nf, d_face_offsets);
        note_launch();
    }
    const uint64_t cap_v = pow2_at_least(2 * (uint64_t)m.n_verts + 1);
    C.hv = HashTab{pool.get<ulonglong2>((int64_t)cap_v), pool.get<uint32_t>((int64_t)cap_v), cap_v - 1};
    const uint64_t cap_b = m.mi ? pow2_at_least(2 * (uint64_t)tots[1] + 1) : 0;
    C.hb = m.mi ? HashTab{pool.get<ulonglong2>((int64_t)cap_b), pool.get<uint32_t>((int64_t)cap_b), cap_b - 1}
                : HashTab{nullptr, nullptr, 0};
    if (pool.err) return pool.err;
    cudaMemsetAsync(C.hv.keys, 0xFF, sizeof(ulonglong2) * cap_v, s);
    cudaMemsetAsync(C.hv.owner, 0xFF, sizeof(uint32_t) * cap_v, s);
    if (m.mi) {
        cudaMemsetAsync(C.hb.keys, 0xFF, sizeof(ulonglong2) * cap_b, s);
        cudaMemsetAsync(C.hb.owner, 0xFF, sizeof(uint32_t) * cap_b, s);
    }
    if (m.n_verts > 0) {
        k_map_insert_verts<<<nblk(m.n_verts), kBs, 0, s>>>(C);
        note_launch();
    }
    if (m.A > 0) {
        k_map_verts<<<nblk(m.A), kBs, 0, s>>>(C);
        note_launch();
        if (m.mi) {
            k_map_bfaces<<<nblk(m.A), kBs, 0, s>>>(C);
            note_launch();
        }
    }
    if (m.n_faces > 0) {
        k_map_faces<<<nblk(m.n_faces), kBs, 0, s>>>(C, m.n_faces, m.face_tet_offsets, m.face_tets, d_face_offsets);
        note_launch();
    }
    uint32_t h = 0;
    cudaMemcpyAsync(&h, C.status, 4, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
    if (h) return cudaErrorUnknown;  // an inconsistency between the records and the mesh
    return cudaGetLastError();
}

}  // namespace ria
