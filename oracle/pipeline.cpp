// CPU oracle (test infrastructure only): stages (a)-(d) of the reference's implicit-arrangement
// and material-interface paths, restated for parity checking and the CPU baseline.
//
//   grid            src/io.cpp:95-152               (generate_tet_mesh)
//   sampling        implicit_functions (absent; formulas defined in include/ria.h)
//   IA signs/filter src/implicit_arrangement.cpp:53-116
//   MI filter       src/material_interface.cpp:53-152
//   per-tet cut     cut.cpp (replaces the absent simplicial_arrangement library)
//   IA extraction   src/extract_mesh.cpp:10-265     (extract_iso_mesh)
//   MI extraction   src/extract_mesh.cpp:569-986    (extract_MI_mesh)
//   local-to-global maps of the extraction variants  src/extract_mesh.cpp:268-566, 988-1443
//   vertex xyz      src/extract_mesh.cpp:1446-1637, src/extract_mesh.h:111-159
//   edges/patches/chains  src/mesh_connectivity.cpp:10-242 (only to pin the oracle against the
//                   reference's known-answer tests)
//
// Only tests/, the smoke check and bench.py's CPU baseline load this library.
// Build with -ffp-contract=off: the sampled values and vertex coordinates must round exactly as
// the device code does.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <queue>
#include <climits>
#include <set>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "cut.hpp"

namespace oracle {
extern int g_selfcheck;
}

using namespace oracle;

namespace {

constexpr int64_t kNone = -1;

struct Func {  // mirrors ria_function in include/ria.h
    int32_t type;
    int32_t flipped;
    double p[12];
};

double sample_one(const Func& f, double x, double y, double z) {
    double v = 0.0;
    switch (f.type) {
        case 0:
            v = 0.0;
            break;
        case 1: {  // plane through point p[0..2] with normal p[3..5]
            v = (f.p[3] * (x - f.p[0]) + f.p[4] * (y - f.p[1])) + f.p[5] * (z - f.p[2]);
            break;
        }
        case 2:
        case 3: {  // sphere r - |x-c|, or r^2 - |x-c|^2 (positive inside)
            double dx = x - f.p[0], dy = y - f.p[1], dz = z - f.p[2];
            double d2 = (dx * dx + dy * dy) + dz * dz;
            v = (f.type == 2) ? f.p[3] - std::sqrt(d2) : f.p[3] * f.p[3] - d2;
            break;
        }
        case 4: {  // cylinder r - dist(x, axis): axis point p[0..2], unit axis p[3..5], radius p[6]
            double vx = x - f.p[0], vy = y - f.p[1], vz = z - f.p[2];
            double t = (vx * f.p[3] + vy * f.p[4]) + vz * f.p[5];
            double wx = vx - t * f.p[3], wy = vy - t * f.p[4], wz = vz - t * f.p[5];
            v = f.p[6] - std::sqrt((wx * wx + wy * wy) + wz * wz);
            break;
        }
        case 5: {  // torus r - dist(x, core circle): centre p[0..2], unit axis p[3..5], major p[6], minor p[7]
            double vx = x - f.p[0], vy = y - f.p[1], vz = z - f.p[2];
            double h = (vx * f.p[3] + vy * f.p[4]) + vz * f.p[5];
            double wx = vx - h * f.p[3], wy = vy - h * f.p[4], wz = vz - h * f.p[5];
            double rho = std::sqrt((wx * wx + wy * wy) + wz * wz);
            double a = rho - f.p[6];
            v = f.p[7] - std::sqrt(a * a + h * h);
            break;
        }
        default:
            v = 0.0;
    }
    return f.flipped ? -v : v;
}

template <class Fn>
void parallel_for(int64_t n, int threads, Fn fn) {
    if (threads <= 1 || n < 4096) {
        fn(0, n);
        return;
    }
    std::vector<std::thread> th;
    int64_t chunk = (n + threads - 1) / threads;
    for (int t = 0; t < threads; ++t) {
        int64_t b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([=, &fn] { fn(b, e); });
    }
    for (auto& x : th) x.join();
}

struct KeyHash {
    template <size_t N>
    size_t operator()(const std::array<int64_t, N>& a) const {
        uint64_t h = 1469598103934665603ull;
        for (auto x : a) {
            h ^= (uint64_t)x + 0x9e3779b97f4a7c15ull + (h << 6) + (h >> 2);
        }
        return h;
    }
};

struct Mesh {
    // stage b
    std::vector<int64_t> func_in_tet, start_index;
    // stage c
    std::vector<int64_t> rec_offsets;
    std::vector<uint8_t> rec_bytes;
    // stage d
    std::vector<int64_t> verts;  // N x 11: tet, local, simplex_size, sv[4], funcs[4]
    std::vector<double> xyz;
    std::vector<int64_t> face_offsets{0}, face_verts, face_tet_offsets{0}, face_tets, face_func;
    // local-to-global maps of the extraction variants (src/extract_mesh.cpp:268-566, 988-1443):
    // per record vertex its mesh vertex or -v-1, per record face its mesh face or -1; CRS over the tets
    std::vector<int64_t> tet_vert_offsets{0}, tet_verts, tet_face_offsets{0}, tet_faces;
    // downstream (KAT pinning)
    std::vector<int64_t> edges, patch_offsets{0}, patch_faces, patch_label, chain_offsets{0}, chain_edges;
    // each edge's occurrences (face, local edge) in face order, and each face corner's edge
    std::vector<int64_t> edge_face_offsets{0}, edge_faces, face_edges;
    std::vector<int64_t> nm_degree;  // per vertex: number of incident non-manifold edges
    std::vector<int64_t> stats;
    std::vector<double> timings;
};

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

void compute_iso_face_key(const std::vector<int64_t>& fv, std::array<int64_t, 3>& key) {
    int64_t mn = fv[0], mx = fv[0];
    size_t mpos = 0;
    for (size_t i = 1; i < fv.size(); ++i) {
        if (fv[i] < mn) {
            mn = fv[i];
            mpos = i;
        } else if (fv[i] > mx) {
            mx = fv[i];
        }
    }
    int64_t second = mx + 1;
    for (size_t i = 0; i < fv.size(); ++i)
        if (i != mpos && fv[i] < second) second = fv[i];
    key = {mn, second, mx};
}

// ---- decoded per-tet records (views into the serialised bytes)
struct IAView {
    int k, nv, nf, nc;
    const uint8_t* rep;
    const uint8_t* vlab;
    const uint8_t* faces;
    const uint8_t* loops;
    int face_supp(int f) const { return faces[8 * f]; }
    bool face_bnd(int f) const { return faces[8 * f + 1] & 1; }
    int face_len(int f) const { return faces[8 * f + 6] | (faces[8 * f + 7] << 8); }
};

inline int rd16(const uint8_t* p) { return p[0] | (p[1] << 8); }

IAView ia_view(const uint8_t* b) {
    IAView v;
    v.k = b[1];
    v.nv = rd16(b + 2);
    v.nf = rd16(b + 4);
    v.nc = rd16(b + 6);
    v.rep = b + 10;
    v.vlab = v.rep + v.k;
    v.faces = v.vlab + 3 * v.nv;
    v.loops = v.faces + 8 * v.nf;
    return v;
}

struct MIView {
    int k, nv, nf, nc;
    const uint8_t* rep;
    const uint8_t* vlab;
    const uint8_t* faces;
    const uint8_t* loops;
    int face_pos(int f) const { return faces[4 * f]; }
    int face_neg(int f) const { return faces[4 * f + 1]; }
    int face_len(int f) const { return rd16(faces + 4 * f + 2); }
};

MIView mi_view(const uint8_t* b) {
    MIView v;
    v.k = b[1];
    v.nv = rd16(b + 2);
    v.nf = rd16(b + 4);
    v.nc = rd16(b + 6);
    v.rep = b + 10;
    v.vlab = v.rep + v.k;
    v.faces = v.vlab + 4 * v.nv;
    v.loops = v.faces + 4 * v.nf;
    return v;
}

// ---- stage c driver: run the per-tet cut for every active tet (parallel over tets)
void run_cuts(bool mi, int64_t T, const int64_t* tets, const double* fv, int F, Mesh& M, int threads,
              int64_t* num_exact) {
    std::vector<std::vector<uint8_t>> recs(T);
    std::vector<long> exact(std::max(threads, 1), 0);
    std::vector<int> fail(std::max(threads, 1), 0);
    int nth = std::max(threads, 1);
    std::vector<std::thread> th;
    int64_t chunk = (T + nth - 1) / nth;
    auto work = [&](int t, int64_t b, int64_t e) {
        std::vector<double> rows;
        CutStats st;
        for (int64_t i = b; i < e; ++i) {
            int64_t s0 = M.start_index[i], s1 = M.start_index[i + 1];
            int k = (int)(s1 - s0);
            if (k == 0) continue;
            rows.assign(4 * k, 0.0);
            for (int j = 0; j < k; ++j) {
                int64_t f = M.func_in_tet[s0 + j];
                for (int c = 0; c < 4; ++c) rows[4 * j + c] = fv[tets[4 * i + c] * F + f];
            }
            bool ok;
            if (mi) {
                MIRecord r;
                ok = mi_cut(k, rows.data(), r, &st);
                if (ok) mi_serialize(r, recs[i]);
            } else {
                IARecord r;
                ok = ia_cut(k, rows.data(), r, &st);
                if (ok) ia_serialize(r, recs[i]);
            }
            if (!ok) fail[t] = 1;
        }
        exact[t] = st.exact_calls;
    };
    if (nth == 1 || T < 4096) {
        work(0, 0, T);
    } else {
        for (int t = 0; t < nth; ++t) {
            int64_t b = t * chunk, e = std::min(T, b + chunk);
            if (b >= e) break;
            th.emplace_back(work, t, b, e);
        }
        for (auto& x : th) x.join();
    }
    M.rec_offsets.assign(T + 1, 0);
    for (int64_t i = 0; i < T; ++i) M.rec_offsets[i + 1] = M.rec_offsets[i] + (int64_t)recs[i].size();
    M.rec_bytes.resize(M.rec_offsets[T]);
    for (int64_t i = 0; i < T; ++i)
        if (!recs[i].empty()) std::memcpy(M.rec_bytes.data() + M.rec_offsets[i], recs[i].data(), recs[i].size());
    long tot = 0;
    for (auto e : exact) tot += e;
    *num_exact = tot;
}

// ---- IA extraction (src/extract_mesh.cpp:10-265)
void extract_iso(int64_t T, const int64_t* tets, Mesh& M) {
    std::unordered_map<int64_t, int64_t> vert_on_tetVert;
    std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> vert_on_tetEdge;
    std::unordered_map<std::array<int64_t, 5>, int64_t, KeyHash> vert_on_tetFace;
    std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> face_on_tetFace;
    std::vector<std::vector<std::pair<int64_t, int64_t>>> tet_face_lists;
    std::vector<std::vector<int64_t>> face_vlists;
    std::vector<int64_t> face_func;
    std::vector<char> is_iso_vert, is_iso_face;
    std::vector<int64_t> iso_vid;
    int64_t nverts = 0;
    auto new_vert = [&](int64_t tet, int64_t local, int64_t ss, std::array<int64_t, 4> sv, std::array<int64_t, 4> fn) {
        int64_t rec[11] = {tet, local, ss, sv[0], sv[1], sv[2], sv[3], fn[0], fn[1], fn[2], fn[3]};
        M.verts.insert(M.verts.end(), rec, rec + 11);
        return nverts++;
    };
    for (int64_t i = 0; i < T; ++i) {
        if (M.rec_offsets[i + 1] == M.rec_offsets[i]) {
            M.tet_vert_offsets.push_back((int64_t)M.tet_verts.size());
            M.tet_face_offsets.push_back((int64_t)M.tet_faces.size());
            continue;
        }
        IAView r = ia_view(M.rec_bytes.data() + M.rec_offsets[i]);
        int64_t start = M.start_index[i];
        const int64_t* tet = tets + 4 * i;
        // which supporting planes carry an implicit function
        bool unique = true;
        for (int j = 0; j < r.k; ++j)
            if (r.rep[j] != 4 + j) unique = false;
        auto plane_is_iso = [&](int p) {
            if (p > 3) return true;
            if (unique) return false;
            for (int j = 0; j < r.k; ++j)
                if (r.rep[j] == p) return true;
            return false;
        };
        // function carried by a supporting plane: the plane itself, or for a tet face made
        // coplanar by an implicit plane, the smallest implicit plane of its group
        auto plane_func = [&](int p) -> int64_t {
            if (p > 3) return M.func_in_tet[p - 4 + start];
            for (int j = 0; j < r.k; ++j)
                if (r.rep[j] == p) return M.func_in_tet[j + start];
            return kNone;
        };
        is_iso_vert.assign(r.nv, 0);
        is_iso_face.assign(r.nf, 0);
        {
            int off = 0;
            for (int f = 0; f < r.nf; ++f) {
                int len = r.face_len(f);
                if (plane_is_iso(r.face_supp(f))) {
                    is_iso_face[f] = 1;
                    for (int t = 0; t < len; ++t) is_iso_vert[rd16(r.loops + 2 * (off + t))] = 1;
                }
                off += len;
            }
        }
        iso_vid.assign(r.nv, kNone);
        for (int j = 0; j < r.nv; ++j) {
            if (!is_iso_vert[j]) continue;
            const uint8_t* lab = r.vlab + 3 * j;
            int nb = 0, ni = 0;
            int bnd[3];
            int64_t impl[3] = {kNone, kNone, kNone};
            for (int t = 0; t < 3; ++t) {
                if (lab[t] > 3)
                    impl[ni++] = M.func_in_tet[lab[t] - 4 + start];
                else
                    bnd[nb++] = lab[t];
            }
            switch (nb) {
                case 2: {
                    int64_t vv[2];
                    int n = 0;
                    for (int c = 0; c < 4; ++c)
                        if (c != bnd[0] && c != bnd[1]) vv[n++] = tet[c];
                    int64_t a = std::min(vv[0], vv[1]), b = std::max(vv[0], vv[1]);
                    std::array<int64_t, 3> key{a, b, impl[0]};
                    auto it = vert_on_tetEdge.find(key);
                    if (it == vert_on_tetEdge.end()) {
                        int64_t id = new_vert(i, j, 2, {a, b, kNone, kNone}, {impl[0], kNone, kNone, kNone});
                        vert_on_tetEdge.emplace(key, id);
                        iso_vid[j] = id;
                    } else {
                        iso_vid[j] = it->second;
                    }
                    break;
                }
                case 1: {
                    int64_t vv[3];
                    int n = 0;
                    for (int c = 0; c < 4; ++c)
                        if (c != bnd[0]) vv[n++] = tet[c];
                    std::sort(vv, vv + 3);
                    std::array<int64_t, 5> key{vv[0], vv[1], vv[2], impl[0], impl[1]};
                    auto it = vert_on_tetFace.find(key);
                    if (it == vert_on_tetFace.end()) {
                        int64_t id = new_vert(i, j, 3, {vv[0], vv[1], vv[2], kNone}, {impl[0], impl[1], kNone, kNone});
                        vert_on_tetFace.emplace(key, id);
                        iso_vid[j] = id;
                    } else {
                        iso_vid[j] = it->second;
                    }
                    break;
                }
                case 0: {
                    iso_vid[j] = new_vert(i, j, 4, {tet[0], tet[1], tet[2], tet[3]}, {impl[0], impl[1], impl[2], kNone});
                    break;
                }
                case 3: {
                    int c0 = 0;
                    for (int c = 0; c < 4; ++c)
                        if (c != bnd[0] && c != bnd[1] && c != bnd[2]) {
                            c0 = c;
                            break;
                        }
                    int64_t key = tet[c0];
                    auto it = vert_on_tetVert.find(key);
                    if (it == vert_on_tetVert.end()) {
                        int64_t id = new_vert(i, j, 1, {key, kNone, kNone, kNone}, {kNone, kNone, kNone, kNone});
                        vert_on_tetVert.emplace(key, id);
                        iso_vid[j] = id;
                    } else {
                        iso_vid[j] = it->second;
                    }
                    break;
                }
            }
        }
        // vertex map: a vertex on no iso face is a tet corner (its three labels are tet faces), and an
        // iso vertex on a tet vertex is named by that vertex too (src/extract_mesh.cpp:384-403, 514-519)
        for (int j = 0; j < r.nv; ++j) {
            const uint8_t* lab = r.vlab + 3 * j;
            int nb = 0;
            bool used[4] = {false, false, false, false};
            for (int t = 0; t < 3; ++t)
                if (lab[t] <= 3) {
                    used[lab[t]] = true;
                    ++nb;
                }
            if (!is_iso_vert[j] || nb == 3) {
                if (nb != 3) {  // impossible for a vertex on no iso face: marked for the tests to see
                    M.tet_verts.push_back(INT64_MIN);
                    continue;
                }
                int c0 = 0;
                while (used[c0]) ++c0;
                M.tet_verts.push_back(-tet[c0] - 1);
            } else {
                M.tet_verts.push_back(iso_vid[j]);
            }
        }
        M.tet_vert_offsets.push_back((int64_t)M.tet_verts.size());
        const size_t fmap0 = M.tet_faces.size();
        M.tet_faces.resize(fmap0 + r.nf, kNone);
        int off = 0;
        std::vector<int64_t> fvs;
        for (int f = 0; f < r.nf; ++f) {
            int len = r.face_len(f);
            if (is_iso_face[f]) {
                fvs.clear();
                for (int t = 0; t < len; ++t) fvs.push_back(iso_vid[rd16(r.loops + 2 * (off + t))]);
                if (r.face_bnd(f)) {
                    std::array<int64_t, 3> key;
                    compute_iso_face_key(fvs, key);
                    auto it = face_on_tetFace.find(key);
                    if (it == face_on_tetFace.end()) {
                        M.tet_faces[fmap0 + f] = (int64_t)face_vlists.size();
                        face_on_tetFace.emplace(key, (int64_t)face_vlists.size());
                        face_vlists.push_back(fvs);
                        tet_face_lists.push_back({{i, f}});
                        face_func.push_back(plane_func(r.face_supp(f)));
                    } else {
                        M.tet_faces[fmap0 + f] = it->second;
                        tet_face_lists[it->second].push_back({i, f});
                    }
                } else {
                    M.tet_faces[fmap0 + f] = (int64_t)face_vlists.size();
                    face_vlists.push_back(fvs);
                    tet_face_lists.push_back({{i, f}});
                    face_func.push_back(plane_func(r.face_supp(f)));
                }
            }
            off += len;
        }
        M.tet_face_offsets.push_back((int64_t)M.tet_faces.size());
    }
    for (size_t f = 0; f < face_vlists.size(); ++f) {
        for (auto v : face_vlists[f]) M.face_verts.push_back(v);
        M.face_offsets.push_back((int64_t)M.face_verts.size());
        for (auto& tf : tet_face_lists[f]) {
            M.face_tets.push_back(tf.first);
            M.face_tets.push_back(tf.second);
        }
        M.face_tet_offsets.push_back((int64_t)M.face_tets.size() / 2);
        M.face_func.push_back(face_func[f]);
        M.face_func.push_back(kNone);
    }
}

// ---- MI extraction (src/extract_mesh.cpp:569-986)
void extract_mi(int64_t T, const int64_t* tets, Mesh& M) {
    std::unordered_map<int64_t, int64_t> vert_on_tetVert;
    std::unordered_map<std::array<int64_t, 4>, int64_t, KeyHash> vert_on_tetEdge;
    std::unordered_map<std::array<int64_t, 6>, int64_t, KeyHash> vert_on_tetFace;
    std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> material_of_bndry_face;
    std::unordered_map<std::array<int64_t, 3>, std::vector<int64_t>, KeyHash> materials_of_bndry_face;
    std::vector<std::vector<int64_t>> face_vlists;
    std::vector<std::pair<int64_t, int64_t>> face_tf;
    std::vector<std::pair<int64_t, int64_t>> face_func;
    std::vector<int64_t> simplex_size;
    std::vector<int64_t> sv0;
    int64_t nverts = 0;
    auto new_vert = [&](int64_t tet, int64_t local, int64_t ss, std::array<int64_t, 4> sv, std::array<int64_t, 4> mats) {
        int64_t rec[11] = {tet, local, ss, sv[0], sv[1], sv[2], sv[3], mats[0], mats[1], mats[2], mats[3]};
        M.verts.insert(M.verts.end(), rec, rec + 11);
        simplex_size.push_back(ss);
        sv0.push_back(sv[0]);
        return nverts++;
    };
    std::vector<char> is_mi_vert;
    std::vector<int64_t> mvid;
    // first record face of each boundary key, as a position in tet_faces (src/extract_mesh.cpp:1420-1431)
    std::unordered_map<std::array<int64_t, 3>, int64_t, KeyHash> tet_face_of_bndry_face;
    for (int64_t i = 0; i < T; ++i) {
        if (M.rec_offsets[i + 1] == M.rec_offsets[i]) {
            M.tet_vert_offsets.push_back((int64_t)M.tet_verts.size());
            M.tet_face_offsets.push_back((int64_t)M.tet_faces.size());
            continue;
        }
        MIView r = mi_view(M.rec_bytes.data() + M.rec_offsets[i]);
        int64_t start = M.start_index[i];
        const int64_t* tet = tets + 4 * i;
        bool unique = true;
        for (int j = 0; j < r.k; ++j)
            if (r.rep[j] != 4 + j) unique = false;
        is_mi_vert.assign(r.nv, 0);
        {
            int off = 0;
            for (int f = 0; f < r.nf; ++f) {
                int len = r.face_len(f);
                if (r.face_pos(f) > 3)
                    for (int t = 0; t < len; ++t) is_mi_vert[rd16(r.loops + 2 * (off + t))] = 1;
                off += len;
            }
        }
        mvid.assign(r.nv, 0);
        for (int j = 0; j < r.nv; ++j) {
            const uint8_t* lab = r.vlab + 4 * j;
            int nb = 0, nm = 0;
            int bnd[4];
            int64_t mats[4] = {kNone, kNone, kNone, kNone};
            for (int t = 0; t < 4; ++t) {
                if (lab[t] > 3)
                    mats[nm++] = M.func_in_tet[lab[t] - 4 + start];
                else
                    bnd[nb++] = lab[t];
            }
            auto corner = [&]() {
                for (int c = 0; c < 4; ++c) {
                    bool used = false;
                    for (int t = 0; t < nb; ++t) used = used || bnd[t] == c;
                    if (!used) return c;
                }
                return 0;
            };
            if (!is_mi_vert[j]) {
                mvid[j] = -tet[corner()] - 1;
                continue;
            }
            switch (nb) {
                case 2: {
                    int64_t vv[2];
                    int n = 0;
                    for (int c = 0; c < 4; ++c)
                        if (c != bnd[0] && c != bnd[1]) vv[n++] = tet[c];
                    int64_t a = std::min(vv[0], vv[1]), b = std::max(vv[0], vv[1]);
                    int64_t m1 = std::min(mats[0], mats[1]), m2 = std::max(mats[0], mats[1]);
                    std::array<int64_t, 4> key{a, b, m1, m2};
                    auto it = vert_on_tetEdge.find(key);
                    if (it == vert_on_tetEdge.end()) {
                        int64_t id = new_vert(i, j, 2, {a, b, kNone, kNone}, {m1, m2, kNone, kNone});
                        vert_on_tetEdge.emplace(key, id);
                        mvid[j] = id;
                    } else {
                        mvid[j] = it->second;
                    }
                    break;
                }
                case 1: {
                    int64_t vv[3];
                    int n = 0;
                    for (int c = 0; c < 4; ++c)
                        if (c != bnd[0]) vv[n++] = tet[c];
                    std::sort(vv, vv + 3);
                    int64_t ms[3] = {mats[0], mats[1], mats[2]};
                    std::sort(ms, ms + 3);
                    std::array<int64_t, 6> key{vv[0], vv[1], vv[2], ms[0], ms[1], ms[2]};
                    auto it = vert_on_tetFace.find(key);
                    if (it == vert_on_tetFace.end()) {
                        int64_t id = new_vert(i, j, 3, {vv[0], vv[1], vv[2], kNone}, {ms[0], ms[1], ms[2], kNone});
                        vert_on_tetFace.emplace(key, id);
                        mvid[j] = id;
                    } else {
                        mvid[j] = it->second;
                    }
                    break;
                }
                case 0:
                    mvid[j] = new_vert(i, j, 4, {tet[0], tet[1], tet[2], tet[3]}, {mats[0], mats[1], mats[2], mats[3]});
                    break;
                case 3: {
                    int64_t key = tet[corner()];
                    auto it = vert_on_tetVert.find(key);
                    if (it == vert_on_tetVert.end()) {
                        int64_t id = new_vert(i, j, 1, {key, kNone, kNone, kNone}, {kNone, kNone, kNone, kNone});
                        vert_on_tetVert.emplace(key, id);
                        mvid[j] = id;
                    } else {
                        mvid[j] = it->second;
                    }
                    break;
                }
            }
        }
        // vertex map (src/extract_mesh.cpp:1112-1128, 1240-1259): tet vertices, and interface vertices
        // on a tet vertex, as -v-1
        for (int j = 0; j < r.nv; ++j) {
            if (!is_mi_vert[j] || (mvid[j] >= 0 && simplex_size[mvid[j]] == 1))
                M.tet_verts.push_back(mvid[j] >= 0 ? -sv0[mvid[j]] - 1 : mvid[j]);
            else
                M.tet_verts.push_back(mvid[j]);
        }
        M.tet_vert_offsets.push_back((int64_t)M.tet_verts.size());
        const size_t fmap0 = M.tet_faces.size();
        M.tet_faces.resize(fmap0 + r.nf, kNone);
        int off = 0;
        std::vector<int64_t> fvs, bfv, mats_here;
        for (int f = 0; f < r.nf; ++f) {
            int len = r.face_len(f);
            const uint8_t* loop = r.loops + 2 * off;
            off += len;
            int pos = r.face_pos(f), neg = r.face_neg(f);
            if (pos > 3) {
                fvs.clear();
                for (int t = 0; t < len; ++t) fvs.push_back(mvid[rd16(loop + 2 * t)]);
                M.tet_faces[fmap0 + f] = (int64_t)face_vlists.size();
                face_vlists.push_back(fvs);
                face_tf.push_back({i, f});
                face_func.push_back({M.func_in_tet[pos - 4 + start], M.func_in_tet[neg - 4 + start]});
                continue;
            }
            bfv.clear();
            for (int t = 0; t < len; ++t) {
                int64_t id = mvid[rd16(loop + 2 * t)];
                if (id >= 0 && simplex_size[id] == 1)
                    bfv.push_back(-sv0[id] - 1);
                else
                    bfv.push_back(id);
            }
            std::array<int64_t, 3> key;
            compute_iso_face_key(bfv, key);
            const int64_t first_occ = tet_face_of_bndry_face.emplace(key, (int64_t)(fmap0 + f)).first->second;
            int64_t m = kNone;
            mats_here.clear();
            if (unique) {
                m = M.func_in_tet[neg - 4 + start];
            } else {
                int grp = 0;
                for (int j = 0; j < r.k; ++j)
                    if (r.rep[j] == neg) ++grp;
                if (grp == 1) {
                    m = M.func_in_tet[neg - 4 + start];
                } else {
                    for (int j = 0; j < r.k; ++j)
                        if (r.rep[j] == neg) mats_here.push_back(M.func_in_tet[j + start]);
                }
            }
            bool interface = false;
            int64_t m_other = kNone;  // one material of the other side (for the label pair)
            if (m != kNone) {
                auto ins = material_of_bndry_face.emplace(key, m);
                if (!ins.second) {
                    if (ins.first->second == m) {
                        material_of_bndry_face.erase(ins.first);
                    } else {
                        interface = true;
                        m_other = ins.first->second;
                    }
                } else {
                    auto it = materials_of_bndry_face.find(key);
                    if (it != materials_of_bndry_face.end()) {
                        bool has = std::find(it->second.begin(), it->second.end(), m) != it->second.end();
                        if (has) {
                            material_of_bndry_face.erase(ins.first);
                            materials_of_bndry_face.erase(it);
                        } else {
                            interface = true;
                            m_other = it->second.front();
                        }
                    }
                }
            } else {
                auto ins = materials_of_bndry_face.emplace(key, mats_here);
                if (!ins.second) {
                    bool common = false;
                    for (auto a : ins.first->second)
                        for (auto b : mats_here)
                            if (a == b) common = true;
                    if (common) {
                        materials_of_bndry_face.erase(ins.first);
                    } else {
                        interface = true;
                        m_other = ins.first->second.front();
                    }
                } else {
                    auto it = material_of_bndry_face.find(key);
                    if (it != material_of_bndry_face.end()) {
                        int64_t mo = it->second;
                        bool has = std::find(mats_here.begin(), mats_here.end(), mo) != mats_here.end();
                        if (has) {
                            material_of_bndry_face.erase(it);
                            materials_of_bndry_face.erase(ins.first);
                        } else {
                            interface = true;
                            m_other = mo;
                        }
                    }
                }
            }
            if (interface) {
                fvs.clear();
                for (int t = 0; t < len; ++t) {
                    int lv = rd16(loop + 2 * t);
                    if (bfv[t] < 0) {
                        int64_t vkey = -bfv[t] - 1;
                        auto it = vert_on_tetVert.find(vkey);
                        if (it == vert_on_tetVert.end()) {
                            int64_t id = new_vert(i, lv, 1, {vkey, kNone, kNone, kNone}, {kNone, kNone, kNone, kNone});
                            vert_on_tetVert.emplace(vkey, id);
                            fvs.push_back(id);
                        } else {
                            fvs.push_back(it->second);
                        }
                    } else {
                        fvs.push_back(mvid[lv]);
                    }
                }
                int64_t m_here = (m != kNone) ? m : mats_here.front();
                M.tet_faces[fmap0 + f] = (int64_t)face_vlists.size();
                M.tet_faces[first_occ] = (int64_t)face_vlists.size();
                face_vlists.push_back(fvs);
                face_tf.push_back({i, f});
                face_func.push_back({std::max(m_here, m_other), std::min(m_here, m_other)});
            }
        }
        M.tet_face_offsets.push_back((int64_t)M.tet_faces.size());
    }
    for (size_t f = 0; f < face_vlists.size(); ++f) {
        for (auto v : face_vlists[f]) M.face_verts.push_back(v);
        M.face_offsets.push_back((int64_t)M.face_verts.size());
        M.face_tets.push_back(face_tf[f].first);
        M.face_tets.push_back(face_tf[f].second);
        M.face_tet_offsets.push_back((int64_t)M.face_tets.size() / 2);
        M.face_func.push_back(face_func[f].first);
        M.face_func.push_back(face_func[f].second);
    }
}

// ---- vertex coordinates (src/extract_mesh.cpp:1446-1637; src/extract_mesh.h:111-159)
void bary4(const double* p1, const double* p2, const double* p3, double* b) {
    double n1 = p1[3] * (p2[2] * p3[1] - p2[1] * p3[2]) + p1[2] * (p2[1] * p3[3] - p2[3] * p3[1]) +
                p1[1] * (p2[3] * p3[2] - p2[2] * p3[3]);
    double n2 = p1[3] * (p2[0] * p3[2] - p2[2] * p3[0]) + p1[2] * (p2[3] * p3[0] - p2[0] * p3[3]) +
                p1[0] * (p2[2] * p3[3] - p2[3] * p3[2]);
    double n3 = p1[3] * (p2[1] * p3[0] - p2[0] * p3[1]) + p1[1] * (p2[0] * p3[3] - p2[3] * p3[0]) +
                p1[0] * (p2[3] * p3[1] - p2[1] * p3[3]);
    double n4 = p1[2] * (p2[0] * p3[1] - p2[1] * p3[0]) + p1[1] * (p2[2] * p3[0] - p2[0] * p3[2]) +
                p1[0] * (p2[1] * p3[2] - p2[2] * p3[1]);
    double d = n1 + n2 + n3 + n4;
    b[0] = n1 / d;
    b[1] = n2 / d;
    b[2] = n3 / d;
    b[3] = n4 / d;
}

void bary3(const double* p1, const double* p2, double* b) {
    double n1 = p1[2] * p2[1] - p1[1] * p2[2];
    double n2 = p1[0] * p2[2] - p1[2] * p2[0];
    double n3 = p1[1] * p2[0] - p1[0] * p2[1];
    double d = n1 + n2 + n3;
    b[0] = n1 / d;
    b[1] = n2 / d;
    b[2] = n3 / d;
}

void compute_xyz(bool mi, const double* pts, const double* fv, int F, Mesh& M) {
    int64_t N = (int64_t)M.verts.size() / 11;
    M.xyz.assign(3 * N, 0.0);
    for (int64_t i = 0; i < N; ++i) {
        const int64_t* r = &M.verts[11 * i];
        int64_t ss = r[2];
        const int64_t* sv = r + 3;
        const int64_t* fn = r + 7;
        double* out = &M.xyz[3 * i];
        auto val = [&](int64_t v, int a) {  // IA: f_a; MI: f_a - f_{a+1}
            if (!mi) return fv[v * F + fn[a]];
            return fv[v * F + fn[a]] - fv[v * F + fn[a + 1]];
        };
        switch (ss) {
            case 2: {
                double f1 = val(sv[0], 0), f2 = val(sv[1], 0);
                double b0 = f2 / (f2 - f1);
                double b1 = 1 - b0;
                for (int c = 0; c < 3; ++c) out[c] = b0 * pts[3 * sv[0] + c] + b1 * pts[3 * sv[1] + c];
                break;
            }
            case 3: {
                double a[3] = {val(sv[0], 0), val(sv[1], 0), val(sv[2], 0)};
                double b[3] = {val(sv[0], 1), val(sv[1], 1), val(sv[2], 1)};
                double w[3];
                bary3(a, b, w);
                for (int c = 0; c < 3; ++c)
                    out[c] = w[0] * pts[3 * sv[0] + c] + w[1] * pts[3 * sv[1] + c] + w[2] * pts[3 * sv[2] + c];
                break;
            }
            case 4: {
                double a[4], b[4], d[4], w[4];
                for (int t = 0; t < 4; ++t) {
                    a[t] = val(sv[t], 0);
                    b[t] = val(sv[t], 1);
                    d[t] = val(sv[t], 2);
                }
                bary4(a, b, d, w);
                for (int c = 0; c < 3; ++c)
                    out[c] = w[0] * pts[3 * sv[0] + c] + w[1] * pts[3 * sv[1] + c] + w[2] * pts[3 * sv[2] + c] +
                             w[3] * pts[3 * sv[3] + c];
                break;
            }
            case 1:
                for (int c = 0; c < 3; ++c) out[c] = pts[3 * sv[0] + c];
                break;
        }
    }
}

// ---- downstream connectivity (src/mesh_connectivity.cpp:10-242)
void connectivity(Mesh& M, bool mi) {
    int64_t nf = (int64_t)M.face_offsets.size() - 1;
    std::map<std::pair<int64_t, int64_t>, int64_t> eid;
    std::vector<std::vector<std::pair<int64_t, int64_t>>> efaces;
    std::vector<std::vector<int64_t>> face_edges(nf);
    for (int64_t f = 0; f < nf; ++f) {
        int64_t b = M.face_offsets[f], e = M.face_offsets[f + 1];
        int64_t n = e - b;
        for (int64_t j = 0; j < n; ++j) {
            int64_t v1 = M.face_verts[b + j], v2 = M.face_verts[b + (j + 1) % n];
            if (v1 > v2) std::swap(v1, v2);
            auto ins = eid.emplace(std::make_pair(v1, v2), (int64_t)efaces.size());
            if (ins.second) {
                efaces.push_back({});
                M.edges.push_back(v1);
                M.edges.push_back(v2);
            }
            efaces[ins.first->second].push_back({f, j});
            face_edges[f].push_back(ins.first->second);
        }
    }
    for (auto& occ : efaces) {
        for (auto& fj : occ) {
            M.edge_faces.push_back(fj.first);
            M.edge_faces.push_back(fj.second);
        }
        M.edge_face_offsets.push_back((int64_t)M.edge_faces.size() / 2);
    }
    for (auto& fe : face_edges) M.face_edges.insert(M.face_edges.end(), fe.begin(), fe.end());
    std::vector<char> seen(nf, 0);
    for (int64_t i = 0; i < nf; ++i) {
        if (seen[i]) continue;
        std::queue<int64_t> Q;
        Q.push(i);
        seen[i] = 1;
        M.patch_faces.push_back(i);
        M.patch_label.push_back(M.face_func[2 * i]);
        M.patch_label.push_back(mi ? M.face_func[2 * i + 1] : kNone);
        while (!Q.empty()) {
            int64_t f = Q.front();
            Q.pop();
            for (int64_t e : face_edges[f]) {
                if (efaces[e].size() != 2) continue;
                int64_t o = efaces[e][0].first == f ? efaces[e][1].first : efaces[e][0].first;
                if (!seen[o]) {
                    seen[o] = 1;
                    Q.push(o);
                    M.patch_faces.push_back(o);
                }
            }
        }
        M.patch_offsets.push_back((int64_t)M.patch_faces.size());
    }
    int64_t nv = (int64_t)M.verts.size() / 11;
    std::vector<std::vector<int64_t>> nm_of_vert(nv);
    int64_t ne = (int64_t)efaces.size();
    for (int64_t e = 0; e < ne; ++e)
        if (efaces[e].size() > 2) {
            nm_of_vert[M.edges[2 * e]].push_back(e);
            nm_of_vert[M.edges[2 * e + 1]].push_back(e);
        }
    M.nm_degree.resize(nv);
    for (int64_t v = 0; v < nv; ++v) M.nm_degree[v] = (int64_t)nm_of_vert[v].size();
    std::vector<char> vis(ne, 0);
    for (int64_t i = 0; i < ne; ++i) {
        if (vis[i] || efaces[i].size() <= 2) continue;
        std::queue<int64_t> Q;
        Q.push(i);
        vis[i] = 1;
        M.chain_edges.push_back(i);
        while (!Q.empty()) {
            int64_t e = Q.front();
            Q.pop();
            for (int end = 0; end < 2; ++end) {
                int64_t v = M.edges[2 * e + end];
                if (nm_of_vert[v].size() == 2) {
                    int64_t o = nm_of_vert[v][0] == e ? nm_of_vert[v][1] : nm_of_vert[v][0];
                    if (!vis[o]) {
                        vis[o] = 1;
                        Q.push(o);
                        M.chain_edges.push_back(o);
                    }
                }
            }
        }
        M.chain_offsets.push_back((int64_t)M.chain_edges.size());
    }
}

}  // namespace

extern "C" {

void oracle_set_selfcheck(int on) { g_selfcheck = on; }

int oracle_ia_cut(int k, const double* planes, uint8_t* buf, int cap) {
    IARecord r;
    try {
        if (!ia_cut(k, planes, r)) return -1;
    } catch (...) {
        return -2;
    }
    std::vector<uint8_t> b;
    ia_serialize(r, b);
    if ((int)b.size() > cap) return -3;
    std::memcpy(buf, b.data(), b.size());
    return (int)b.size();
}

int oracle_mi_cut(int k, const double* mats, uint8_t* buf, int cap) {
    MIRecord r;
    try {
        if (!mi_cut(k, mats, r)) return -1;
    } catch (...) {
        return -2;
    }
    std::vector<uint8_t> b;
    mi_serialize(r, b);
    if ((int)b.size() > cap) return -3;
    std::memcpy(buf, b.data(), b.size());
    return (int)b.size();
}

void oracle_grid(int64_t res, const double* bmin, const double* bmax, double* pts, int64_t* tets) {
    const int64_t N = res + 1;
    for (int64_t i = 0; i < N; ++i) {
        double x = (double(i) / double(N - 1)) * (bmax[0] - bmin[0]) + bmin[0];
        for (int64_t j = 0; j < N; ++j) {
            double y = (double(j) / double(N - 1)) * (bmax[1] - bmin[1]) + bmin[1];
            for (int64_t k = 0; k < N; ++k) {
                double z = (double(k) / double(N - 1)) * (bmax[2] - bmin[2]) + bmin[2];
                int64_t idx = i * N * N + j * N + k;
                pts[3 * idx] = x;
                pts[3 * idx + 1] = y;
                pts[3 * idx + 2] = z;
            }
        }
    }
    for (int64_t i = 0; i < res; ++i)
        for (int64_t j = 0; j < res; ++j)
            for (int64_t k = 0; k < res; ++k) {
                int64_t idx = (i * res * res + j * res + k) * 5;
                int64_t v0 = i * N * N + j * N + k, v1 = (i + 1) * N * N + j * N + k;
                int64_t v2 = (i + 1) * N * N + (j + 1) * N + k, v3 = i * N * N + (j + 1) * N + k;
                int64_t v4 = v0 + 1, v5 = v1 + 1, v6 = v2 + 1, v7 = v3 + 1;
                int64_t t[5][4];
                if ((i + j + k) % 2 == 0) {
                    int64_t a[5][4] = {{v4, v6, v1, v3}, {v6, v3, v4, v7}, {v1, v3, v0, v4}, {v3, v1, v2, v6}, {v4, v1, v6, v5}};
                    std::memcpy(t, a, sizeof(t));
                } else {
                    int64_t a[5][4] = {{v7, v0, v2, v5}, {v2, v3, v0, v7}, {v5, v7, v0, v4}, {v7, v2, v6, v5}, {v0, v1, v2, v5}};
                    std::memcpy(t, a, sizeof(t));
                }
                std::memcpy(tets + 4 * idx, t, sizeof(t));
            }
}

void oracle_sample(const void* funcs, int nf, const double* pts, int64_t V, double* out, int threads) {
    const Func* fs = (const Func*)funcs;
    parallel_for(V, threads, [&](int64_t b, int64_t e) {
        for (int64_t v = b; v < e; ++v)
            for (int j = 0; j < nf; ++j) out[v * nf + j] = sample_one(fs[j], pts[3 * v], pts[3 * v + 1], pts[3 * v + 2]);
    });
}

// mode 0: implicit arrangement, 1: material interface.  Returns an opaque handle.
void* oracle_run(int mode, const double* pts, int64_t V, const int64_t* tets, int64_t T, const double* fv, int F,
                 int threads, int do_connectivity) {
    Mesh* M = new Mesh();
    bool mi = mode == 1;
    double t0 = now();
    int64_t n_int = 0, n_deg = 0;
    M->start_index.assign(T + 1, 0);
    if (!mi) {
        // signs and filter (src/implicit_arrangement.cpp:53-116)
        std::vector<int8_t> sgn((size_t)V * F);
        for (int64_t v = 0; v < V; ++v)
            for (int j = 0; j < F; ++j) {
                double x = fv[v * F + j];
                int s = x > 0 ? 1 : (x < 0 ? -1 : 0);
                sgn[v * F + j] = (int8_t)s;
                if (s == 0) ++n_deg;
            }
        std::vector<std::vector<int64_t>> part(std::max(threads, 1));
        std::vector<int64_t> cnt(T, 0);
        std::vector<uint64_t> act(T * ((F + 63) / 64), 0);
        int W = (F + 63) / 64;
        parallel_for(T, threads, [&](int64_t b, int64_t e) {
            for (int64_t i = b; i < e; ++i)
                for (int j = 0; j < F; ++j) {
                    int pc = 0, nc = 0;
                    for (int c = 0; c < 4; ++c) {
                        int s = sgn[tets[4 * i + c] * F + j];
                        if (s == 1) ++pc;
                        else if (s == -1) ++nc;
                    }
                    if (pc < 4 && nc < 4) {
                        act[i * W + j / 64] |= uint64_t(1) << (j % 64);
                        ++cnt[i];
                    }
                }
        });
        for (int64_t i = 0; i < T; ++i) {
            M->start_index[i + 1] = M->start_index[i] + cnt[i];
            if (cnt[i]) ++n_int;
        }
        M->func_in_tet.resize(M->start_index[T]);
        for (int64_t i = 0; i < T; ++i) {
            int64_t o = M->start_index[i];
            for (int j = 0; j < F; ++j)
                if (act[i * W + j / 64] & (uint64_t(1) << (j % 64))) M->func_in_tet[o++] = j;
        }
    } else {
        // highest material and filter (src/material_interface.cpp:53-152)
        std::vector<int64_t> hi(V);
        std::vector<char> deg(V, 0);
        for (int64_t v = 0; v < V; ++v) {
            double mx = fv[v * F];
            int64_t id = 0, count = 1;
            for (int j = 1; j < F; ++j) {
                double x = fv[v * F + j];
                if (x > mx) {
                    mx = x;
                    id = j;
                    count = 1;
                } else if (x == mx) {
                    ++count;
                }
            }
            hi[v] = id;
            if (count > 1) {
                deg[v] = 1;
                ++n_deg;
            }
        }
        std::vector<std::vector<int64_t>> lists(T);
        parallel_for(T, threads, [&](int64_t b, int64_t e) {
            std::set<int64_t> mats;
            for (int64_t i = b; i < e; ++i) {
                const int64_t* tet = tets + 4 * i;
                mats.clear();
                for (int c = 0; c < 4; ++c) {
                    int64_t v = tet[c];
                    if (deg[v]) {
                        double mx = fv[v * F + hi[v]];
                        for (int j = 0; j < F; ++j)
                            if (fv[v * F + j] == mx) mats.insert(j);
                    } else {
                        mats.insert(hi[v]);
                    }
                }
                if (mats.size() < 2) continue;
                double min_h[4];
                for (int c = 0; c < 4; ++c) min_h[c] = 1.7976931348623157e308;
                for (int64_t m : mats)
                    for (int c = 0; c < 4; ++c) {
                        double x = fv[tet[c] * F + m];
                        if (x < min_h[c]) min_h[c] = x;
                    }
                for (int j = 0; j < F; ++j) {
                    int g = 0;
                    for (int c = 0; c < 4; ++c)
                        if (fv[tet[c] * F + j] > min_h[c]) ++g;
                    if (g > 1) mats.insert(j);
                }
                lists[i].assign(mats.begin(), mats.end());
            }
        });
        for (int64_t i = 0; i < T; ++i) {
            M->start_index[i + 1] = M->start_index[i] + (int64_t)lists[i].size();
            if (!lists[i].empty()) ++n_int;
        }
        M->func_in_tet.reserve(M->start_index[T]);
        for (int64_t i = 0; i < T; ++i) M->func_in_tet.insert(M->func_in_tet.end(), lists[i].begin(), lists[i].end());
    }
    double t1 = now();
    int64_t n_exact = 0;
    run_cuts(mi, T, tets, fv, F, *M, threads, &n_exact);
    int64_t n1 = 0, n2 = 0, n3 = 0;
    for (int64_t i = 0; i < T; ++i) {
        int64_t k = M->start_index[i + 1] - M->start_index[i];
        if (k == 0) continue;
        if (!mi) {
            if (k == 1) ++n1; else if (k == 2) ++n2; else ++n3;
        } else {
            if (k == 2) ++n1; else if (k == 3) ++n2; else ++n3;
        }
    }
    double t2 = now();
    if (!mi)
        extract_iso(T, tets, *M);
    else
        extract_mi(T, tets, *M);
    double t3 = now();
    compute_xyz(mi, pts, fv, F, *M);
    double t4 = now();
    if (do_connectivity) connectivity(*M, mi);
    double t5 = now();
    int64_t nv = (int64_t)M->verts.size() / 11, nfc = (int64_t)M->face_offsets.size() - 1;
    // num_pts, num_tets, num_degenerate_vertex, num_intersecting_tet, num_{1,2,more}_func
    // (MI: num_{2,3,more}_func), num_verts, num_faces, exact predicate calls
    M->stats = {V, T, n_deg, n_int, n1, n2, n3, nv, nfc, n_exact};
    M->timings = {t1 - t0, t2 - t1, t3 - t2, t4 - t3, t5 - t4};
    return M;
}

int64_t oracle_len(void* h, const char* name) {
    Mesh* M = (Mesh*)h;
    std::string n(name);
    if (n == "func_in_tet") return (int64_t)M->func_in_tet.size();
    if (n == "start_index") return (int64_t)M->start_index.size();
    if (n == "rec_offsets") return (int64_t)M->rec_offsets.size();
    if (n == "rec_bytes") return (int64_t)M->rec_bytes.size();
    if (n == "verts") return (int64_t)M->verts.size();
    if (n == "xyz") return (int64_t)M->xyz.size();
    if (n == "face_offsets") return (int64_t)M->face_offsets.size();
    if (n == "face_verts") return (int64_t)M->face_verts.size();
    if (n == "face_tet_offsets") return (int64_t)M->face_tet_offsets.size();
    if (n == "face_tets") return (int64_t)M->face_tets.size();
    if (n == "face_func") return (int64_t)M->face_func.size();
    if (n == "edges") return (int64_t)M->edges.size();
    if (n == "patch_offsets") return (int64_t)M->patch_offsets.size();
    if (n == "patch_faces") return (int64_t)M->patch_faces.size();
    if (n == "patch_label") return (int64_t)M->patch_label.size();
    if (n == "chain_offsets") return (int64_t)M->chain_offsets.size();
    if (n == "chain_edges") return (int64_t)M->chain_edges.size();
    if (n == "nm_degree") return (int64_t)M->nm_degree.size();
    if (n == "stats") return (int64_t)M->stats.size();
    if (n == "timings") return (int64_t)M->timings.size();
    if (n == "face_edges") return (int64_t)M->face_edges.size();
    if (n == "edge_faces") return (int64_t)M->edge_faces.size();
    if (n == "edge_face_offsets") return (int64_t)M->edge_face_offsets.size();
    if (n == "tet_faces") return (int64_t)M->tet_faces.size();
    if (n == "tet_face_offsets") return (int64_t)M->tet_face_offsets.size();
    if (n == "tet_verts") return (int64_t)M->tet_verts.size();
    if (n == "tet_vert_offsets") return (int64_t)M->tet_vert_offsets.size();
    return -1;
}

int oracle_copy(void* h, const char* name, void* dst) {
    Mesh* M = (Mesh*)h;
    std::string n(name);
    auto cp = [&](const auto& v) {
        std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
        return 0;
    };
    if (n == "func_in_tet") return cp(M->func_in_tet);
    if (n == "start_index") return cp(M->start_index);
    if (n == "rec_offsets") return cp(M->rec_offsets);
    if (n == "rec_bytes") return cp(M->rec_bytes);
    if (n == "verts") return cp(M->verts);
    if (n == "xyz") return cp(M->xyz);
    if (n == "face_offsets") return cp(M->face_offsets);
    if (n == "face_verts") return cp(M->face_verts);
    if (n == "face_tet_offsets") return cp(M->face_tet_offsets);
    if (n == "face_tets") return cp(M->face_tets);
    if (n == "face_func") return cp(M->face_func);
    if (n == "edges") return cp(M->edges);
    if (n == "patch_offsets") return cp(M->patch_offsets);
    if (n == "patch_faces") return cp(M->patch_faces);
    if (n == "patch_label") return cp(M->patch_label);
    if (n == "chain_offsets") return cp(M->chain_offsets);
    if (n == "chain_edges") return cp(M->chain_edges);
    if (n == "nm_degree") return cp(M->nm_degree);
    if (n == "stats") return cp(M->stats);
    if (n == "timings") return cp(M->timings);
    if (n == "face_edges") return cp(M->face_edges);
    if (n == "edge_faces") return cp(M->edge_faces);
    if (n == "edge_face_offsets") return cp(M->edge_face_offsets);
    if (n == "tet_faces") return cp(M->tet_faces);
    if (n == "tet_face_offsets") return cp(M->tet_face_offsets);
    if (n == "tet_verts") return cp(M->tet_verts);
    if (n == "tet_vert_offsets") return cp(M->tet_vert_offsets);
    return -1;
}

void oracle_free(void* h) { delete (Mesh*)h; }

}  // extern "C"
