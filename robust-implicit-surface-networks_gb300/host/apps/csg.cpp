// Command line of app/csg.cpp: `csg config_file [-T] [-R] [-P] [--tree tree.json]`.
// Writes mesh.json (the CSG layout of src/io.cpp:314-372), timings.json and stats.json into the
// config's outputDir.  Without --tree the shape is the union of all functions.
#include <cstring>
#include <iostream>

#include "../ria_host.hpp"

using namespace ria_host;

int main(int argc, const char* argv[]) {
    std::string config_file, csg_file;
    bool timing_only = false, robust_test = false, positive_inside = true;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "-T") || !std::strcmp(argv[i], "--timing-only"))
            timing_only = true;
        else if (!std::strcmp(argv[i], "-R") || !std::strcmp(argv[i], "--robust-test"))
            robust_test = true;
        else if (!std::strcmp(argv[i], "-P") || !std::strcmp(argv[i], "--positive-inside"))
            positive_inside = true;
        else if (!std::strcmp(argv[i], "--tree") && i + 1 < argc)
            csg_file = argv[++i];
        else
            config_file = argv[i];
    }
    if (config_file.empty()) {
        std::cerr << "usage: " << argv[0] << " config_file [-T] [-R] [-P] [--tree tree.json]" << std::endl;
        return 106;
    }
    Config config = parse_config_file(config_file);
    if (!config.use_lookup) config.use_secondary_lookup = false;
    std::vector<CsgUnit> tree;
    if (!csg_file.empty() && !load_csg_tree(csg_file, tree)) return -1;

    std::vector<std::array<double, 3>> pts;
    std::vector<std::array<size_t, 4>> tets;
    if (!config.tet_mesh_file.empty()) {
        std::cout << "load mesh file " << config.tet_mesh_file << std::endl;
        if (!load_tet_mesh(config.tet_mesh_file, pts, tets)) return -1;
    } else {
        std::cout << "generating mesh with resolution " << config.tet_mesh_resolution << std::endl;
        generate_tet_mesh(config.tet_mesh_resolution, config.tet_mesh_bbox_min, config.tet_mesh_bbox_max, pts, tets);
    }
    FuncVals funcVals;
    if (load_functions(config.func_file, pts, funcVals)) {
        std::cout << "function loading finished." << std::endl;
    } else {
        std::cout << "function loading failed." << std::endl;
        return -2;
    }

    std::vector<std::array<double, 3>> iso_pts;
    std::vector<PolygonFace> iso_faces;
    std::vector<std::vector<size_t>> patches;
    std::vector<size_t> patch_function_label;
    std::vector<bool> patch_sign_label;
    std::vector<Edge> iso_edges;
    std::vector<std::vector<size_t>> chains;
    std::vector<std::vector<size_t>> non_manifold_edges_of_vert;
    std::vector<std::vector<size_t>> shells;
    std::vector<std::vector<size_t>> arrangement_cells;
    std::vector<std::vector<bool>> cell_function_label;
    std::vector<std::string> timing_labels;
    std::vector<double> timings;
    std::vector<std::string> stats_labels;
    std::vector<size_t> stats;
    if (!csg(robust_test, config.use_lookup, config.use_secondary_lookup, config.use_topo_ray_shooting, positive_inside,
             pts, tets, funcVals, csg_lambda(tree), iso_pts, iso_faces, patches, patch_function_label,
             patch_sign_label, iso_edges, chains, non_manifold_edges_of_vert, shells, arrangement_cells,
             cell_function_label, timing_labels, timings, stats_labels, stats))
        return -1;
    if (robust_test) return 0;
    if (!timing_only)
        save_result_CSG(config.output_dir + "/mesh.json", iso_pts, iso_faces, patches, patch_sign_label, iso_edges,
                        chains, non_manifold_edges_of_vert);
    save_timings(config.output_dir + "/timings.json", timing_labels, timings);
    save_statistics(config.output_dir + "/stats.json", stats_labels, stats);
    return 0;
}
