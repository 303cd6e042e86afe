// GPU half of the host layer: stages a-d through the C ABI, then the CPU connectivity stages.
#include <chrono>
#include <iostream>

#include "ria_host.hpp"

namespace ria_host {

namespace {

double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

size_t none_or(int64_t x) { return x < 0 ? Mesh_None : (size_t)x; }

struct DeviceMesh {
    ria_mesh* m = nullptr;
    ~DeviceMesh() {
        if (m) ria_mesh_free(m);
    }
    std::vector<int64_t> i64(ria_mesh_field f) const {
        std::vector<int64_t> v(ria_mesh_count(m, f));
        if (!v.empty()) ria_mesh_copy(m, f, v.data());
        return v;
    }
};

void fetch_faces(const DeviceMesh& dm, std::vector<PolygonFace>& faces) {
    auto fo = dm.i64(RIA_MESH_FACE_OFFSETS), fv = dm.i64(RIA_MESH_FACE_VERTS);
    auto to = dm.i64(RIA_MESH_FACE_TET_OFFSETS), tf = dm.i64(RIA_MESH_FACE_TETS), fn = dm.i64(RIA_MESH_FACE_FUNC);
    faces.assign(fo.empty() ? 0 : fo.size() - 1, PolygonFace());
    for (size_t f = 0; f < faces.size(); ++f) {
        faces[f].vert_indices.assign(fv.begin() + fo[f], fv.begin() + fo[f + 1]);
        faces[f].tet_face_indices.reserve((size_t)(to[f + 1] - to[f]));
        for (int64_t t = to[f]; t < to[f + 1]; ++t) faces[f].tet_face_indices.emplace_back(tf[2 * t], tf[2 * t + 1]);
        faces[f].func_index = {none_or(fn[2 * f]), none_or(fn[2 * f + 1])};
    }
}

void fetch_points(const DeviceMesh& dm, std::vector<std::array<double, 3>>& pts) {
    pts.resize(ria_mesh_count(dm.m, RIA_MESH_POINTS) / 3);
    if (!pts.empty()) ria_mesh_copy(dm.m, RIA_MESH_POINTS, pts.data());
}

// shared part of the two pipelines: GPU stages a-d, then edges / patches / chains on the host
template <class Label>
bool run_pipeline(bool mi, bool robust_test, bool use_lookup, bool use_secondary_lookup,
                  const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                  const double* funcVals, size_t n_func, std::vector<std::array<double, 3>>& out_pts,
                  std::vector<PolygonFace>& faces, std::vector<std::vector<size_t>>& patches,
                  std::vector<Label>& patch_function_label, std::vector<Edge>& edges,
                  std::vector<std::vector<size_t>>& chains, std::vector<std::vector<size_t>>& nm_edges_of_vert,
                  std::vector<std::string>& timing_labels, std::vector<double>& timings,
                  std::vector<std::string>& stats_labels, std::vector<size_t>& stats,
                  std::vector<uint64_t>* face_sides = nullptr) {
    if (!use_lookup) use_secondary_lookup = false;
    ria_config cfg{use_lookup ? 1 : 0, use_secondary_lookup ? 1 : 0, 1, robust_test ? 1 : 0, 0};
    DeviceMesh dm;
    static_assert(sizeof(size_t) == sizeof(int64_t), "tet vertex ids are passed as int64");
    const double t0 = now();
    ria_status st = mi ? ria_compute_material_interface(&cfg, pts.empty() ? nullptr : pts[0].data(), pts.size(),
                                                         tets.empty() ? nullptr : (const int64_t*)tets[0].data(),
                                                         tets.size(), funcVals, (uint32_t)n_func, &dm.m)
                       : ria_compute_implicit_arrangement(&cfg, pts.empty() ? nullptr : pts[0].data(), pts.size(),
                                                          tets.empty() ? nullptr : (const int64_t*)tets[0].data(),
                                                          tets.size(), funcVals, (uint32_t)n_func, &dm.m);
    if (robust_test) {
        int64_t s[RIA_NUM_STATS] = {0};
        if (dm.m) ria_mesh_copy(dm.m, RIA_MESH_STATS, s);
        if (st != RIA_OK && !dm.m) {
            std::cout << ria_last_error() << std::endl;
            return false;
        }
        // the reference's messages, in its order of precedence (src/implicit_arrangement.cpp:329-343)
        if (s[RIA_STAT_ROBUST_TYPE2])
            std::cout << "type 2 failure (crash in the normal order)." << std::endl;
        else if (s[RIA_STAT_ROBUST_TYPE3])
            std::cout << "type 3 failure (crash in the reverse order)." << std::endl;
        else if (s[RIA_STAT_ROBUST_FAILURES])
            std::cout << "type 1 failure (inconsistency)." << std::endl;
        else if (st == RIA_OK)
            std::cout << "success." << std::endl;
        else
            std::cout << ria_last_error() << std::endl;
        return st == RIA_OK;
    }
    if (st != RIA_OK) {
        std::cout << ria_last_error() << std::endl;
        return false;
    }
    int64_t s[RIA_NUM_STATS];
    double tm[RIA_NUM_TIMINGS];
    ria_mesh_copy(dm.m, RIA_MESH_STATS, s);
    ria_mesh_copy(dm.m, RIA_MESH_TIMINGS, tm);
    fetch_points(dm, out_pts);
    fetch_faces(dm, faces);
    if (face_sides) {
        face_sides->assign(2 * faces.size(), 0);
        if (!faces.empty() && ria_mesh_face_sides(dm.m, face_sides->data()) != RIA_OK) {
            std::cout << ria_last_error() << std::endl;
            return false;
        }
    }
    const double t1 = now();
    const char* ia_names[] = {"num_pts", "num_tets", "num_degenerate_vertex", "num_intersecting_tet",
                              "num_1_func", "num_2_func", "num_more_func", "num_iso_verts", "num_iso_faces"};
    const char* mi_names[] = {"num_pts", "num_tets", "num_degenerate_vertex", "num_intersecting_tet",
                              "num_2_func", "num_3_func", "num_more_func", "num_MI_verts", "num_MI_faces"};
    for (int i = 0; i < 9; ++i) {
        stats_labels.emplace_back(mi ? mi_names[i] : ia_names[i]);
        stats.push_back((size_t)s[i]);
    }
    const char* tnames[] = {"GPU sample/upload", "GPU signs+filter", "GPU per-tet cut", "GPU extract mesh+xyz"};
    for (int i = 0; i < 4; ++i) {
        timing_labels.emplace_back(tnames[i]);
        timings.push_back(tm[i]);
    }
    timing_labels.emplace_back("device to host");
    timings.push_back(t1 - t0 - tm[RIA_TIME_TOTAL]);
    // edges, patches and chains (src/mesh_connectivity.cpp:10-242): computed on the device with the
    // reference's numbering and orders, then laid out in the reference's containers
    double h0 = now();
    auto eo = dm.i64(RIA_MESH_EDGE_FACE_OFFSETS);  // the first request builds all three on the device
    if (eo.empty()) {  // n_edges + 1 entries when it succeeded
        std::cout << ria_last_error() << std::endl;
        return false;
    }
    auto ev = dm.i64(RIA_MESH_EDGES), ef = dm.i64(RIA_MESH_EDGE_FACES);
    edges.assign(ev.size() / 2, Edge());
    parallel_ranges(edges.size(), 1 << 15, [&](size_t lo, size_t hi) {
        for (size_t e = lo; e < hi; ++e) {
            edges[e].v1 = (size_t)ev[2 * e];
            edges[e].v2 = (size_t)ev[2 * e + 1];
            auto& fe = edges[e].face_edge_indices;
            fe.reserve((size_t)(eo[e + 1] - eo[e]));
            for (int64_t o = eo[e]; o < eo[e + 1]; ++o) fe.emplace_back((size_t)ef[2 * o], (size_t)ef[2 * o + 1]);
        }
    });
    double h1 = now();
    timing_labels.emplace_back(mi ? "MIEdge-face connectivity" : "isoEdge-face connectivity");
    timings.push_back(h1 - h0);
    stats_labels.emplace_back(mi ? "num_MI_edges" : "num_iso_edges");
    stats.push_back(edges.size());
    auto lists = [](const std::vector<int64_t>& off, const std::vector<int64_t>& val,
                    std::vector<std::vector<size_t>>& out) {
        out.assign(off.empty() ? 0 : off.size() - 1, {});
        parallel_ranges(out.size(), 1 << 12, [&](size_t lo, size_t hi) {
            for (size_t i = lo; i < hi; ++i) out[i].assign(val.begin() + off[i], val.begin() + off[i + 1]);
        });
    };
    lists(dm.i64(RIA_MESH_PATCH_OFFSETS), dm.i64(RIA_MESH_PATCH_FACES), patches);
    auto pl = dm.i64(RIA_MESH_PATCH_LABELS);
    patch_function_label.clear();
    for (size_t p = 0; p < patches.size(); ++p) {
        if constexpr (std::is_same<Label, size_t>::value)
            patch_function_label.push_back(none_or(pl[2 * p]));
        else
            patch_function_label.push_back({none_or(pl[2 * p]), none_or(pl[2 * p + 1])});
    }
    double h2 = now();
    timing_labels.emplace_back("patches");
    timings.push_back(h2 - h1);
    stats_labels.emplace_back("num_patches");
    stats.push_back(patches.size());
    nm_edges_of_vert.assign(out_pts.size(), {});
    for (size_t i = 0; i < edges.size(); ++i)
        if (eo[i + 1] - eo[i] > 2) {
            nm_edges_of_vert[edges[i].v1].push_back(i);
            nm_edges_of_vert[edges[i].v2].push_back(i);
        }
    lists(dm.i64(RIA_MESH_CHAIN_OFFSETS), dm.i64(RIA_MESH_CHAIN_EDGES), chains);
    timing_labels.emplace_back("chains");
    timings.push_back(now() - h2);
    stats_labels.emplace_back("num_chains");
    stats.push_back(chains.size());
    return true;
}

}  // namespace

bool sample_functions(const std::vector<ria_function>& funcs, const std::vector<std::array<double, 3>>& pts,
                      FuncVals& fv) {
    fv.n_rows = pts.size();
    fv.n_cols = funcs.size();
    fv.v.assign(fv.n_rows * fv.n_cols, 0.0);
    ria_status st = ria_sample_functions(funcs.data(), (uint32_t)funcs.size(), pts.empty() ? nullptr : pts[0].data(),
                                         pts.size(), fv.v.data());
    if (st != RIA_OK) {
        std::cout << ria_last_error() << std::endl;
        return false;
    }
    return true;
}

bool load_functions(const std::string& filename, const std::vector<std::array<double, 3>>& pts, FuncVals& fv) {
    std::vector<ria_function> funcs;
    return load_functions(filename, funcs) && sample_functions(funcs, pts, fv);
}

bool implicit_arrangement(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool,
                          const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                          const double* funcVals, size_t n_func, std::vector<std::array<double, 3>>& iso_pts,
                          std::vector<PolygonFace>& iso_faces, std::vector<std::vector<size_t>>& patches,
                          std::vector<size_t>& patch_function_label, std::vector<Edge>& iso_edges,
                          std::vector<std::vector<size_t>>& chains,
                          std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                          std::vector<std::vector<size_t>>& shells, std::vector<std::vector<size_t>>& arrangement_cells,
                          std::vector<std::vector<bool>>& cell_function_label, std::vector<std::string>& timing_labels,
                          std::vector<double>& timings, std::vector<std::string>& stats_labels,
                          std::vector<size_t>& stats) {
    shells.clear();
    arrangement_cells.clear();
    cell_function_label.clear();
    return run_pipeline<size_t>(false, robust_test, use_lookup, use_secondary_lookup, pts, tets, funcVals, n_func, iso_pts,
                                iso_faces, patches, patch_function_label, iso_edges, chains, non_manifold_edges_of_vert,
                                timing_labels, timings, stats_labels, stats);
}

bool material_interface(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool,
                        const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                        const double* funcVals, size_t n_func, std::vector<std::array<double, 3>>& MI_pts,
                        std::vector<PolygonFace>& MI_faces, std::vector<std::vector<size_t>>& patches,
                        std::vector<std::pair<size_t, size_t>>& patch_function_label, std::vector<Edge>& MI_edges,
                        std::vector<std::vector<size_t>>& chains,
                        std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                        std::vector<std::vector<size_t>>& shells, std::vector<std::vector<size_t>>& material_cells,
                        std::vector<size_t>& cell_function_label, std::vector<std::string>& timing_labels,
                        std::vector<double>& timings, std::vector<std::string>& stats_labels, std::vector<size_t>& stats) {
    shells.clear();
    material_cells.clear();
    cell_function_label.clear();
    return run_pipeline<std::pair<size_t, size_t>>(true, robust_test, use_lookup, use_secondary_lookup, pts, tets,
                                                   funcVals, n_func, MI_pts, MI_faces, patches, patch_function_label,
                                                   MI_edges, chains, non_manifold_edges_of_vert, timing_labels, timings,
                                                   stats_labels, stats);
}

bool csg(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool, bool positive_inside,
         const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
         const double* funcVals, size_t n_func, const std::function<bool(std::vector<bool>)>& lambda,
         std::vector<std::array<double, 3>>& mesh_pts, std::vector<PolygonFace>& mesh_faces,
         std::vector<std::vector<size_t>>& patches, std::vector<size_t>& patch_function_label,
         std::vector<bool>& patch_sign_label, std::vector<Edge>& edges, std::vector<std::vector<size_t>>& chains,
         std::vector<std::vector<size_t>>& non_manifold_edges_of_vert, std::vector<std::vector<size_t>>& shells,
         std::vector<std::vector<size_t>>& cells, std::vector<std::vector<bool>>& cell_function_label,
         std::vector<std::string>& timing_labels, std::vector<double>& timings, std::vector<std::string>& stats_labels,
         std::vector<size_t>& stats) {
    shells.clear();
    cells.clear();
    cell_function_label.clear();
    std::vector<double> negated;
    if (!positive_inside) {  // src/csg.cpp:36
        negated.assign(funcVals, funcVals + pts.size() * n_func);
        for (double& x : negated) x = -x;
        funcVals = negated.data();
    }
    std::vector<uint64_t> sides;
    if (!run_pipeline<size_t>(false, robust_test, use_lookup, use_secondary_lookup, pts, tets, funcVals, n_func,
                              mesh_pts, mesh_faces, patches, patch_function_label, edges, chains,
                              non_manifold_edges_of_vert, timing_labels, timings, stats_labels, stats,
                              robust_test ? nullptr : &sides))
        return false;
    if (robust_test) return true;
    const double t0 = now();
    // src/csg.cpp:55-116 with each patch's two cells labelled from the sides of its first face
    auto labels = [&](uint64_t bits) {
        std::vector<bool> v(n_func);
        for (size_t j = 0; j < n_func; ++j) v[j] = (bits >> j) & 1;
        return v;
    };
    std::vector<std::vector<size_t>> kept;
    patch_sign_label.clear();
    std::vector<size_t> vertex_to_patch_count(mesh_pts.size(), 0);
    for (auto& patch : patches) {
        const size_t f = patch.front();
        const bool in_pos = lambda(labels(sides[2 * f])), in_neg = lambda(labels(sides[2 * f + 1]));
        if (in_pos == in_neg) continue;
        kept.push_back(patch);
        patch_sign_label.push_back(in_pos);
        for (size_t face : patch)
            for (size_t v : mesh_faces[face].vert_indices) ++vertex_to_patch_count[v];
    }
    std::vector<std::vector<size_t>> kept_chains;
    for (auto& chain : chains) {
        bool active = true;
        for (size_t e : chain)
            if (vertex_to_patch_count[edges[e].v1] < 2 || vertex_to_patch_count[edges[e].v2] < 2) {
                active = false;
                break;
            }
        if (active) kept_chains.push_back(chain);
    }
    for (size_t v = 0; v < non_manifold_edges_of_vert.size(); ++v)
        if (vertex_to_patch_count[v] <= 2) non_manifold_edges_of_vert[v].clear();
    patches.swap(kept);
    chains.swap(kept_chains);
    timing_labels.emplace_back("csg prune");
    timings.push_back(now() - t0);
    return true;
}

}  // namespace ria_host
