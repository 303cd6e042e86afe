// Test driver for the CPU half of the C++ host layer (host/mesh_io.cpp): readers, tet grid,
// connectivity and mesh.json writers, run without a GPU.  Binary files are little-endian int64 /
// float64 arrays, each preceded by its int64 element count.
//
//   meshio_check grid RES x0 y0 z0 x1 y1 z1 OUT      -> pts, tets
//   meshio_check tetmesh FILE OUT                    -> pts, tets
//   meshio_check funcs FILE OUT                      -> raw ria_function records
//   meshio_check config FILE                         -> parsed fields, one per line
//   meshio_check mesh ia|mi IN OUT_JSON              -> mesh.json from (xyz, face offsets/verts/func)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>

#include "../../robust-implicit-surface-networks_gb300/host/ria_host.hpp"

using namespace ria_host;

static void put(FILE* f, const void* p, int64_t n, size_t elem) {
    fwrite(&n, 8, 1, f);
    if (n) fwrite(p, elem, (size_t)n, f);
}

template <class T>
static std::vector<T> get(FILE* f) {
    int64_t n = 0;
    if (fread(&n, 8, 1, f) != 1) throw std::runtime_error("short read");
    std::vector<T> v((size_t)n);
    if (n && fread(v.data(), sizeof(T), (size_t)n, f) != (size_t)n) throw std::runtime_error("short read");
    return v;
}

static int write_grid(const std::vector<std::array<double, 3>>& pts, const std::vector<std::array<size_t, 4>>& tets,
                      const char* out) {
    FILE* f = fopen(out, "wb");
    if (!f) return 2;
    put(f, pts.data(), (int64_t)pts.size() * 3, 8);
    put(f, tets.data(), (int64_t)tets.size() * 4, 8);
    fclose(f);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const std::string cmd = argv[1];
    try {
        if (cmd == "grid" && argc == 10) {
            std::array<double, 3> lo{atof(argv[3]), atof(argv[4]), atof(argv[5])};
            std::array<double, 3> hi{atof(argv[6]), atof(argv[7]), atof(argv[8])};
            std::vector<std::array<double, 3>> pts;
            std::vector<std::array<size_t, 4>> tets;
            if (!generate_tet_mesh((size_t)atol(argv[2]), lo, hi, pts, tets)) return 1;
            return write_grid(pts, tets, argv[9]);
        }
        if (cmd == "tetmesh" && argc == 4) {
            std::vector<std::array<double, 3>> pts;
            std::vector<std::array<size_t, 4>> tets;
            if (!load_tet_mesh(argv[2], pts, tets)) return 1;
            return write_grid(pts, tets, argv[3]);
        }
        if (cmd == "funcs" && argc == 4) {
            std::vector<ria_function> fs;
            if (!load_functions(argv[2], fs)) return 1;
            FILE* f = fopen(argv[3], "wb");
            if (!f) return 2;
            if (!fs.empty()) fwrite(fs.data(), sizeof(ria_function), fs.size(), f);
            fclose(f);
            return 0;
        }
        if (cmd == "config" && argc == 3) {
            Config c = parse_config_file(argv[2]);
            std::cout << "tet_mesh_file " << c.tet_mesh_file << "\nfunc_file " << c.func_file << "\noutput_dir "
                      << c.output_dir << "\nresolution " << c.tet_mesh_resolution << "\nuse_lookup " << c.use_lookup
                      << "\nuse_secondary_lookup " << c.use_secondary_lookup << "\nuse_topo_ray_shooting "
                      << c.use_topo_ray_shooting << "\nbbox";
            for (double x : c.tet_mesh_bbox_min) std::cout << ' ' << x;
            for (double x : c.tet_mesh_bbox_max) std::cout << ' ' << x;
            std::cout << std::endl;
            return 0;
        }
        if (cmd == "mesh" && argc == 5) {
            const bool mi = !strcmp(argv[2], "mi");
            FILE* f = fopen(argv[3], "rb");
            if (!f) return 2;
            auto xyz = get<double>(f);
            auto fo = get<int64_t>(f);
            auto fv = get<int64_t>(f);
            auto fn = get<int64_t>(f);
            fclose(f);
            std::vector<std::array<double, 3>> pts(xyz.size() / 3);
            for (size_t i = 0; i < pts.size(); ++i) pts[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            std::vector<PolygonFace> faces(fo.empty() ? 0 : fo.size() - 1);
            for (size_t i = 0; i < faces.size(); ++i) {
                for (int64_t j = fo[i]; j < fo[i + 1]; ++j) faces[i].vert_indices.push_back((size_t)fv[j]);
                faces[i].func_index = {fn[2 * i] < 0 ? Mesh_None : (size_t)fn[2 * i],
                                       fn[2 * i + 1] < 0 ? Mesh_None : (size_t)fn[2 * i + 1]};
            }
            std::vector<std::vector<size_t>> eof, patches, chains, shells, cells;
            std::vector<Edge> edges;
            compute_mesh_edges(faces, eof, edges);
            std::vector<std::pair<size_t, size_t>> labels;
            compute_patches(eof, edges, faces, patches, labels);
            std::vector<std::vector<size_t>> nm(pts.size());
            for (size_t i = 0; i < edges.size(); ++i)
                if (edges[i].face_edge_indices.size() > 2) {
                    nm[edges[i].v1].push_back(i);
                    nm[edges[i].v2].push_back(i);
                }
            compute_chains(edges, nm, chains);
            if (!strcmp(argv[2], "csg")) {
                // CSG writer: patch i labelled inside when i % 3 == 0
                std::vector<bool> signs(patches.size());
                for (size_t i = 0; i < signs.size(); ++i) signs[i] = i % 3 == 0;
                if (!save_result_CSG(argv[4], pts, faces, patches, signs, edges, chains, nm)) return 4;
            } else if (mi) {
                std::vector<size_t> cell_label;
                save_result_MI(argv[4], pts, faces, patches, labels, edges, chains, nm, shells, cells, cell_label);
            } else {
                std::vector<size_t> first;
                for (auto& l : labels) first.push_back(l.first);
                std::vector<std::vector<bool>> cell_label;
                save_result(argv[4], pts, faces, patches, first, edges, chains, nm, shells, cells, cell_label);
            }
            return 0;
        }
    } catch (const std::exception& e) {
        std::cerr << e.what() << std::endl;
        return 3;
    }
    return 2;
}
