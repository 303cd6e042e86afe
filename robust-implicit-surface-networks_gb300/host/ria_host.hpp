// Host C++ layer with the reference's names and signatures over the C ABI (include/ria.h).
//
//   implicit_arrangement(...)   src/implicit_arrangement.h:39-62
//   material_interface(...)     src/material_interface.h:38-61
//   parse_config_file / load_tet_mesh / generate_tet_mesh / save_result* / save_timings /
//   save_statistics             src/io.h:30-92
//   compute_mesh_edges / compute_patches / compute_chains
//                               src/mesh_connectivity.h (restated host stages that consume the
//                               extracted mesh; src/mesh_connectivity.cpp:10-242)
// Stages a-d run on the GPU.  Face pairing, shells, topological ray shooting, cell grouping and
// sign propagation are not part of this build: `shells`, `arrangement_cells` and
// `cell_function_label` come back empty.
#pragma once
#include <algorithm>
#include <array>
#include <atomic>
#include <cstddef>
#include <functional>
#include <limits>
#include <string>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/ria.h"

namespace ria_host {

// Host threads for the parallel host stages, and a parallel loop over contiguous ranges.
inline size_t host_threads() {
    const unsigned hw = std::thread::hardware_concurrency();
    return std::min<size_t>(hw ? hw : 1, 32);
}

// f(lo, hi) over [0, n) in contiguous chunks (at most ceil(n / grain) of them, and at most four per
// thread), on up to host_threads() threads
template <class F>
void parallel_ranges(size_t n, size_t grain, const F& f) {
    const size_t chunks = std::min(host_threads() * 4, (n + grain - 1) / grain);
    if (chunks <= 1) {
        if (n) f(size_t(0), n);
        return;
    }
    std::atomic<size_t> next{0};
    auto work = [&] {
        for (size_t c; (c = next.fetch_add(1)) < chunks;) f(n * c / chunks, n * (c + 1) / chunks);
    };
    std::vector<std::thread> pool;
    for (size_t t = 1; t < std::min(host_threads(), chunks); ++t) pool.emplace_back(work);
    work();
    for (auto& t : pool) t.join();
}


constexpr size_t Mesh_None = std::numeric_limits<size_t>::max();

struct PolygonFace {  // src/mesh.h:15-25
    std::vector<size_t> vert_indices;
    std::vector<std::pair<size_t, size_t>> tet_face_indices;
    std::pair<size_t, size_t> func_index{Mesh_None, Mesh_None};
};

struct IsoVert {  // src/mesh.h:28-41
    size_t tet_index;
    size_t tet_vert_index;
    size_t simplex_size;
    std::array<size_t, 4> simplex_vert_indices;
    std::array<size_t, 3> func_indices = {Mesh_None, Mesh_None, Mesh_None};
};

struct MI_Vert {  // src/mesh.h:45-58
    size_t tet_index;
    size_t tet_vert_index;
    size_t simplex_size;
    std::array<size_t, 4> simplex_vert_indices;
    std::array<size_t, 4> material_indices;
};

struct Edge {  // src/mesh.h:63-72
    size_t v1, v2;
    std::vector<std::pair<size_t, size_t>> face_edge_indices;
};

struct Config {  // src/io.h:12-28; missing lookup switches default to true (README)
    std::string tet_mesh_file;
    std::string func_file;
    std::string output_dir;
    bool use_lookup = true;
    bool use_secondary_lookup = true;
    bool use_topo_ray_shooting = true;
    size_t tet_mesh_resolution = 0;
    std::array<double, 3> tet_mesh_bbox_min{-1, -1, -1};
    std::array<double, 3> tet_mesh_bbox_max{1, 1, 1};
};

// Row-major n_pts x n_func values (the reference's Eigen RowMajor funcVals)
struct FuncVals {
    size_t n_rows = 0, n_cols = 0;
    std::vector<double> v;
    size_t rows() const { return n_rows; }
    size_t cols() const { return n_cols; }
    const double* data() const { return v.data(); }
};

Config parse_config_file(const std::string& filename);
bool load_tet_mesh(const std::string& filename, std::vector<std::array<double, 3>>& pts,
                   std::vector<std::array<size_t, 4>>& tets);
bool generate_tet_mesh(size_t resolution, const std::array<double, 3>& bbox_min, const std::array<double, 3>& bbox_max,
                       std::vector<std::array<double, 3>>& pts, std::vector<std::array<size_t, 4>>& tets);
// reference function files (plane, sphere, cylinder, torus, zero); false on an unsupported type
bool load_functions(const std::string& filename, std::vector<ria_function>& funcs);
// stage a on the GPU
bool sample_functions(const std::vector<ria_function>& funcs, const std::vector<std::array<double, 3>>& pts,
                      FuncVals& funcVals);
// load + sample, the reference's load_functions(file, pts, funcVals) (src/implicit_functions.h)
bool load_functions(const std::string& filename, const std::vector<std::array<double, 3>>& pts, FuncVals& funcVals);

bool implicit_arrangement(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool use_topo_ray_shooting,
                          const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                          const double* funcVals, size_t n_func,
                          std::vector<std::array<double, 3>>& iso_pts, std::vector<PolygonFace>& iso_faces,
                          std::vector<std::vector<size_t>>& patches, std::vector<size_t>& patch_function_label,
                          std::vector<Edge>& iso_edges, std::vector<std::vector<size_t>>& chains,
                          std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                          std::vector<std::vector<size_t>>& shells, std::vector<std::vector<size_t>>& arrangement_cells,
                          std::vector<std::vector<bool>>& cell_function_label, std::vector<std::string>& timing_labels,
                          std::vector<double>& timings, std::vector<std::string>& stats_labels,
                          std::vector<size_t>& stats);

bool material_interface(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool use_topo_ray_shooting,
                        const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                        const double* funcVals, size_t n_func,
                        std::vector<std::array<double, 3>>& MI_pts, std::vector<PolygonFace>& MI_faces,
                        std::vector<std::vector<size_t>>& patches,
                        std::vector<std::pair<size_t, size_t>>& patch_function_label, std::vector<Edge>& MI_edges,
                        std::vector<std::vector<size_t>>& chains,
                        std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                        std::vector<std::vector<size_t>>& shells, std::vector<std::vector<size_t>>& material_cells,
                        std::vector<size_t>& cell_function_label, std::vector<std::string>& timing_labels,
                        std::vector<double>& timings, std::vector<std::string>& stats_labels, std::vector<size_t>& stats);

// src/csg.h:46-72: the implicit arrangement, then the patches that separate the shape's inside
// (lambda over a cell's function labels: true where the function is positive) from its outside;
// chains and corners are pruned to the kept patches.  positive_inside = false negates the functions
// first, as the reference does.  Cell labels come from the device (each face's two sides), not from
// shells and cells.
bool csg(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool use_topo_ray_shooting, bool positive_inside,
         const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
         const double* funcVals, size_t n_func, const std::function<bool(std::vector<bool>)>& lambda,
         std::vector<std::array<double, 3>>& mesh_pts, std::vector<PolygonFace>& mesh_faces,
         std::vector<std::vector<size_t>>& patches, std::vector<size_t>& patch_function_label,
         std::vector<bool>& patch_sign_label, std::vector<Edge>& edges, std::vector<std::vector<size_t>>& chains,
         std::vector<std::vector<size_t>>& non_manifold_edges_of_vert, std::vector<std::vector<size_t>>& shells,
         std::vector<std::vector<size_t>>& cells, std::vector<std::vector<bool>>& cell_function_label,
         std::vector<std::string>& timing_labels, std::vector<double>& timings, std::vector<std::string>& stats_labels,
         std::vector<size_t>& stats);
template <class M, class... Rest>
bool csg(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool use_topo_ray_shooting, bool positive_inside,
         const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets, const M& funcVals,
         const std::function<bool(std::vector<bool>)>& lambda, Rest&... rest) {
    return csg(robust_test, use_lookup, use_secondary_lookup, use_topo_ray_shooting, positive_inside, pts, tets,
               funcVals.data(), (size_t)funcVals.cols(), lambda, rest...);
}

// CSG tree files (app/csg.cpp:15-52): units {type: Intersection | Union | Negation, elements: [a, b]};
// element e > 0 is unit e (1-based), e < 0 is function -e-1; unit 1 is the root.
struct CsgUnit {
    int op;  // 0 Intersection, 1 Union, 2 Negation
    std::array<int, 2> elements;
};
bool load_csg_tree(const std::string& filename, std::vector<CsgUnit>& tree);
// membership over cell labels (true: function positive); an empty tree is the union of all functions
std::function<bool(std::vector<bool>)> csg_lambda(const std::vector<CsgUnit>& tree);

// Matrix types with data() / cols() and row-major storage (Eigen RowMajor, FuncVals)
template <class M, class... Rest>
bool implicit_arrangement(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool use_topo_ray_shooting,
                          const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                          const M& funcVals, Rest&... rest) {
    return implicit_arrangement(robust_test, use_lookup, use_secondary_lookup, use_topo_ray_shooting, pts, tets,
                                funcVals.data(), (size_t)funcVals.cols(), rest...);
}
template <class M, class... Rest>
bool material_interface(bool robust_test, bool use_lookup, bool use_secondary_lookup, bool use_topo_ray_shooting,
                        const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                        const M& funcVals, Rest&... rest) {
    return material_interface(robust_test, use_lookup, use_secondary_lookup, use_topo_ray_shooting, pts, tets,
                              funcVals.data(), (size_t)funcVals.cols(), rest...);
}

// host stages that consume the mesh (src/mesh_connectivity.cpp:10-242)
void compute_mesh_edges(const std::vector<PolygonFace>& mesh_faces, std::vector<std::vector<size_t>>& edges_of_face,
                        std::vector<Edge>& mesh_edges);
void compute_patches(const std::vector<std::vector<size_t>>& edges_of_face, const std::vector<Edge>& mesh_edges,
                     const std::vector<PolygonFace>& mesh_faces, std::vector<std::vector<size_t>>& patches,
                     std::vector<std::pair<size_t, size_t>>& patch_label);
void compute_chains(const std::vector<Edge>& mesh_edges, const std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                    std::vector<std::vector<size_t>>& chains);

// writers (src/io.cpp:154-312, 554-588): same keys and value types as the reference's files
bool save_result(const std::string& filename, const std::vector<std::array<double, 3>>& mesh_pts,
                 const std::vector<PolygonFace>& mesh_faces, const std::vector<std::vector<size_t>>& patches,
                 const std::vector<size_t>& patch_function_label, const std::vector<Edge>& edges,
                 const std::vector<std::vector<size_t>>& chains,
                 const std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                 const std::vector<std::vector<size_t>>& shells, const std::vector<std::vector<size_t>>& cells,
                 const std::vector<std::vector<bool>>& cell_function_label);
bool save_result_MI(const std::string& filename, const std::vector<std::array<double, 3>>& mesh_pts,
                    const std::vector<PolygonFace>& mesh_faces, const std::vector<std::vector<size_t>>& patches,
                    const std::vector<std::pair<size_t, size_t>>& patch_function_label, const std::vector<Edge>& edges,
                    const std::vector<std::vector<size_t>>& chains,
                    const std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                    const std::vector<std::vector<size_t>>& shells, const std::vector<std::vector<size_t>>& cells,
                    const std::vector<size_t>& cell_function_label);
bool save_result_CSG(const std::string& filename, const std::vector<std::array<double, 3>>& mesh_pts,
                     const std::vector<PolygonFace>& mesh_faces, const std::vector<std::vector<size_t>>& patches,
                     const std::vector<bool>& patch_sign_label, const std::vector<Edge>& edges,
                     const std::vector<std::vector<size_t>>& chains,
                     const std::vector<std::vector<size_t>>& non_manifold_edges_of_vert);
bool save_timings(const std::string& filename, const std::vector<std::string>& timing_labels,
                  const std::vector<double>& timings);
bool save_statistics(const std::string& filename, const std::vector<std::string>& stats_labels,
                     const std::vector<size_t>& stats);

}  // namespace ria_host
