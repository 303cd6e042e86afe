// CPU half of the host layer: configuration, tet-mesh and function-file readers, the tet grid,
// mesh connectivity (edges, patches, chains) and the JSON writers.  Needs no GPU.
#include <cmath>
#include <fstream>
#include <iostream>
#include <map>
#include <queue>
#include <sstream>

#include "json.hpp"
#include "ria_host.hpp"

namespace ria_host {

namespace {

std::string read_file(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

std::string dir_of(const std::string& path) {
    size_t p = path.find_last_of('/');
    return p == std::string::npos ? std::string(".") : path.substr(0, p);
}

std::string resolve(const std::string& base, const std::string& p) {
    if (!p.empty() && p[0] == '/') return p;
    return base + "/" + p;
}

std::array<double, 3> unit(const Json& a) {
    double v[3] = {a[0].as_double(), a[1].as_double(), a[2].as_double()};
    double n = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    if (n == 0.0) throw std::runtime_error("zero axis vector");
    return {v[0] / n, v[1] / n, v[2] / n};
}

template <class V>
void put_list(std::ostringstream& o, const V& v) {
    o << '[';
    for (size_t i = 0; i < v.size(); ++i) o << (i ? "," : "") << v[i];
    o << ']';
}

void put_lists(std::ostringstream& o, const std::vector<std::vector<size_t>>& v) {
    if (v.empty()) {
        o << "null";
        return;
    }
    o << '[';
    for (size_t i = 0; i < v.size(); ++i) {
        if (i) o << ',';
        put_list(o, v[i]);
    }
    o << ']';
}

// the keys of the reference's mesh.json, in its library's (sorted) key order; a list the reference
// never appends to stays null, as there
void write_mesh_json(const std::string& filename, const std::vector<std::array<double, 3>>& pts,
                     const std::vector<PolygonFace>& faces, const std::vector<std::vector<size_t>>& patches,
                     const std::string& patches_label, const std::vector<Edge>& edges,
                     const std::vector<std::vector<size_t>>& chains,
                     const std::vector<std::vector<size_t>>& nm_edges_of_vert,
                     const std::vector<std::vector<size_t>>& shells, const std::vector<std::vector<size_t>>& cells,
                     const std::string& cells_label) {
    std::ostringstream o;
    o << "{\"cells\":";
    put_lists(o, cells);
    o << ",\"cells_label\":" << cells_label << ",\"chains\":";
    put_lists(o, chains);
    std::vector<size_t> corners;
    for (size_t i = 0; i < nm_edges_of_vert.size(); ++i)
        if (nm_edges_of_vert[i].size() > 2 || nm_edges_of_vert[i].size() == 1) corners.push_back(i);
    o << ",\"corners\":";
    if (corners.empty())
        o << "null";
    else
        put_list(o, corners);
    o << ",\"edges\":";
    if (edges.empty()) {
        o << "null";
    } else {
        o << '[';
        for (size_t i = 0; i < edges.size(); ++i) o << (i ? "," : "") << '[' << edges[i].v1 << ',' << edges[i].v2 << ']';
        o << ']';
    }
    o << ",\"faces\":";
    if (faces.empty()) {
        o << "null";
    } else {
        o << '[';
        for (size_t i = 0; i < faces.size(); ++i) {
            if (i) o << ',';
            put_list(o, faces[i].vert_indices);
        }
        o << ']';
    }
    o << ",\"patches\":";
    put_lists(o, patches);
    o << ",\"patches_label\":" << patches_label << ",\"points\":";
    if (pts.empty()) {
        o << "null";
    } else {
        o << '[';
        for (size_t i = 0; i < pts.size(); ++i)
            o << (i ? "," : "") << '[' << json_double(pts[i][0]) << ',' << json_double(pts[i][1]) << ','
              << json_double(pts[i][2]) << ']';
        o << ']';
    }
    o << ",\"shells\":";
    put_lists(o, shells);
    o << "}\n";
    std::ofstream f(filename);
    f << o.str();
}

}  // namespace

Config parse_config_file(const std::string& filename) {
    std::ifstream fin(filename);
    if (!fin) throw std::runtime_error("Config file does not exist!");
    Json d = JsonParser(read_file(filename)).parse();
    Config c;
    const std::string base = dir_of(filename);
    if (d.contains("tetMeshFile")) {
        c.tet_mesh_file = resolve(base, d["tetMeshFile"].as_string());
        c.tet_mesh_resolution = 0;
    } else {
        c.tet_mesh_resolution = (size_t)d["gridResolution"].as_double();
        for (int a = 0; a < 3; ++a) {
            c.tet_mesh_bbox_min[a] = d["gridBbox"][0][a].as_double();
            c.tet_mesh_bbox_max[a] = d["gridBbox"][1][a].as_double();
        }
    }
    c.func_file = resolve(base, d["funcFile"].as_string());
    c.output_dir = resolve(base, d.contains("outputDir") ? d["outputDir"].as_string() : std::string("."));
    if (d.contains("useLookup")) c.use_lookup = d["useLookup"].as_bool();
    if (d.contains("useSecondaryLookup")) c.use_secondary_lookup = d["useSecondaryLookup"].as_bool();
    if (d.contains("useTopoRayShooting")) c.use_topo_ray_shooting = d["useTopoRayShooting"].as_bool();
    return c;
}

bool load_tet_mesh(const std::string& filename, std::vector<std::array<double, 3>>& pts,
                   std::vector<std::array<size_t, 4>>& tets) {
    std::ifstream fin(filename);
    if (!fin) {
        std::cout << "tet mesh file not exist!" << std::endl;
        return false;
    }
    Json d = JsonParser(read_file(filename)).parse();
    pts.resize(d[0].size());
    for (size_t j = 0; j < pts.size(); ++j)
        for (int k = 0; k < 3; ++k) pts[j][k] = d[0][j][k].as_double();
    tets.resize(d[1].size());
    for (size_t j = 0; j < tets.size(); ++j)
        for (int k = 0; k < 4; ++k) tets[j][k] = (size_t)d[1][j][k].as_double();
    return true;
}

bool generate_tet_mesh(size_t resolution, const std::array<double, 3>& bmin, const std::array<double, 3>& bmax,
                       std::vector<std::array<double, 3>>& pts, std::vector<std::array<size_t, 4>>& tets) {
    if (resolution == 0) return false;
    const size_t N = resolution + 1;
    pts.resize(N * N * N);
    for (size_t i = 0; i < N; ++i)
        for (size_t j = 0; j < N; ++j)
            for (size_t k = 0; k < N; ++k) {
                size_t idx[3] = {i, j, k};
                auto& p = pts[i * N * N + j * N + k];
                for (int a = 0; a < 3; ++a) p[a] = (double(idx[a]) / double(N - 1)) * (bmax[a] - bmin[a]) + bmin[a];
            }
    tets.resize(resolution * resolution * resolution * 5);
    for (size_t i = 0; i < resolution; ++i)
        for (size_t j = 0; j < resolution; ++j)
            for (size_t k = 0; k < resolution; ++k) {
                size_t idx = (i * resolution * resolution + j * resolution + k) * 5;
                size_t v0 = i * N * N + j * N + k, v1 = (i + 1) * N * N + j * N + k;
                size_t v2 = (i + 1) * N * N + (j + 1) * N + k, v3 = i * N * N + (j + 1) * N + k;
                size_t v4 = v0 + 1, v5 = v1 + 1, v6 = v2 + 1, v7 = v3 + 1;
                if ((i + j + k) % 2 == 0) {
                    tets[idx] = {{v4, v6, v1, v3}};
                    tets[idx + 1] = {{v6, v3, v4, v7}};
                    tets[idx + 2] = {{v1, v3, v0, v4}};
                    tets[idx + 3] = {{v3, v1, v2, v6}};
                    tets[idx + 4] = {{v4, v1, v6, v5}};
                } else {
                    tets[idx] = {{v7, v0, v2, v5}};
                    tets[idx + 1] = {{v2, v3, v0, v7}};
                    tets[idx + 2] = {{v5, v7, v0, v4}};
                    tets[idx + 3] = {{v7, v2, v6, v5}};
                    tets[idx + 4] = {{v0, v1, v2, v5}};
                }
            }
    return true;
}

bool load_functions(const std::string& filename, std::vector<ria_function>& funcs) {
    Json d = JsonParser(read_file(filename)).parse();
    funcs.clear();
    for (size_t i = 0; i < d.size(); ++i) {
        const Json& s = d[i];
        ria_function f{};
        const std::string& t = s["type"].as_string();
        if (t == "zero") {
            f.type = RIA_FUNC_ZERO;
        } else if (t == "plane") {
            f.type = RIA_FUNC_PLANE;
            for (int a = 0; a < 3; ++a) {
                f.p[a] = s["point"][a].as_double();
                f.p[3 + a] = s["normal"][a].as_double();
            }
        } else if (t == "sphere") {
            f.type = (s.contains("squared") && s["squared"].as_bool()) ? RIA_FUNC_SPHERE_SQUARED : RIA_FUNC_SPHERE;
            for (int a = 0; a < 3; ++a) f.p[a] = s["center"][a].as_double();
            f.p[3] = s["radius"].as_double();
        } else if (t == "cylinder") {
            f.type = RIA_FUNC_CYLINDER;
            auto u = unit(s["axis_vector"]);
            for (int a = 0; a < 3; ++a) {
                f.p[a] = s["axis_point"][a].as_double();
                f.p[3 + a] = u[a];
            }
            f.p[6] = s["radius"].as_double();
        } else if (t == "torus") {
            f.type = RIA_FUNC_TORUS;
            auto u = unit(s["axis_vector"]);
            for (int a = 0; a < 3; ++a) {
                f.p[a] = s["center"][a].as_double();
                f.p[3 + a] = u[a];
            }
            f.p[6] = s["major_radius"].as_double();
            f.p[7] = s["minor_radius"].as_double();
        } else {
            std::cout << "unsupported implicit function type: " << t << std::endl;
            return false;
        }
        f.flipped = (s.contains("is_flipped") && s["is_flipped"].as_bool()) ? 1 : 0;
        funcs.push_back(f);
    }
    return true;
}

void compute_mesh_edges(const std::vector<PolygonFace>& mesh_faces, std::vector<std::vector<size_t>>& edges_of_face,
                        std::vector<Edge>& mesh_edges) {
    std::map<std::pair<size_t, size_t>, size_t> edge_id;
    edges_of_face.assign(mesh_faces.size(), {});
    for (size_t i = 0; i < mesh_faces.size(); ++i) {
        const auto& vs = mesh_faces[i].vert_indices;
        const size_t n = vs.size();
        edges_of_face[i].resize(n);
        for (size_t j = 0; j < n; ++j) {
            size_t v1 = vs[j], v2 = vs[(j + 1) % n];
            if (v1 > v2) std::swap(v1, v2);
            auto ins = edge_id.emplace(std::make_pair(v1, v2), mesh_edges.size());
            if (ins.second) {
                mesh_edges.push_back(Edge{v1, v2, {}});
            }
            mesh_edges[ins.first->second].face_edge_indices.emplace_back(i, j);
            edges_of_face[i][j] = ins.first->second;
        }
    }
}

void compute_patches(const std::vector<std::vector<size_t>>& edges_of_face, const std::vector<Edge>& mesh_edges,
                     const std::vector<PolygonFace>& mesh_faces, std::vector<std::vector<size_t>>& patches,
                     std::vector<std::pair<size_t, size_t>>& patch_label) {
    std::vector<char> visited(edges_of_face.size(), 0);
    for (size_t i = 0; i < edges_of_face.size(); ++i) {
        if (visited[i]) continue;
        patches.emplace_back();
        auto& patch = patches.back();
        std::queue<size_t> Q;
        Q.push(i);
        patch.push_back(i);
        visited[i] = 1;
        patch_label.push_back(mesh_faces[i].func_index);
        while (!Q.empty()) {
            size_t f = Q.front();
            Q.pop();
            for (size_t e : edges_of_face[f]) {
                const auto& fe = mesh_edges[e].face_edge_indices;
                if (fe.size() != 2) continue;
                size_t o = fe[0].first == f ? fe[1].first : fe[0].first;
                if (!visited[o]) {
                    visited[o] = 1;
                    Q.push(o);
                    patch.push_back(o);
                }
            }
        }
    }
}

void compute_chains(const std::vector<Edge>& mesh_edges, const std::vector<std::vector<size_t>>& nm_edges_of_vert,
                    std::vector<std::vector<size_t>>& chains) {
    std::vector<char> visited(mesh_edges.size(), 0);
    for (size_t i = 0; i < mesh_edges.size(); ++i) {
        if (visited[i] || mesh_edges[i].face_edge_indices.size() <= 2) continue;
        chains.emplace_back();
        auto& chain = chains.back();
        std::queue<size_t> Q;
        Q.push(i);
        chain.push_back(i);
        visited[i] = 1;
        while (!Q.empty()) {
            size_t e = Q.front();
            Q.pop();
            for (size_t v : {mesh_edges[e].v1, mesh_edges[e].v2}) {
                if (nm_edges_of_vert[v].size() != 2) continue;
                size_t o = nm_edges_of_vert[v][0] == e ? nm_edges_of_vert[v][1] : nm_edges_of_vert[v][0];
                if (!visited[o]) {
                    visited[o] = 1;
                    Q.push(o);
                    chain.push_back(o);
                }
            }
        }
    }
}

bool save_result(const std::string& filename, const std::vector<std::array<double, 3>>& mesh_pts,
                 const std::vector<PolygonFace>& mesh_faces, const std::vector<std::vector<size_t>>& patches,
                 const std::vector<size_t>& patch_function_label, const std::vector<Edge>& edges,
                 const std::vector<std::vector<size_t>>& chains,
                 const std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                 const std::vector<std::vector<size_t>>& shells, const std::vector<std::vector<size_t>>& cells,
                 const std::vector<std::vector<bool>>& cell_function_label) {
    std::ostringstream pl;
    pl << '[';
    put_list(pl, patch_function_label);
    pl << ']';
    std::ostringstream cl;
    if (cell_function_label.empty()) {
        cl << "null";
    } else {
        cl << '[';
        for (size_t i = 0; i < cell_function_label.size(); ++i) {
            cl << (i ? "," : "") << '[';
            for (size_t j = 0; j < cell_function_label[i].size(); ++j)
                cl << (j ? "," : "") << (cell_function_label[i][j] ? "true" : "false");
            cl << ']';
        }
        cl << ']';
    }
    write_mesh_json(filename, mesh_pts, mesh_faces, patches, pl.str(), edges, chains, non_manifold_edges_of_vert, shells,
                    cells, cl.str());
    return true;
}

bool save_result_MI(const std::string& filename, const std::vector<std::array<double, 3>>& mesh_pts,
                    const std::vector<PolygonFace>& mesh_faces, const std::vector<std::vector<size_t>>& patches,
                    const std::vector<std::pair<size_t, size_t>>& patch_function_label, const std::vector<Edge>& edges,
                    const std::vector<std::vector<size_t>>& chains,
                    const std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                    const std::vector<std::vector<size_t>>& shells, const std::vector<std::vector<size_t>>& cells,
                    const std::vector<size_t>& cell_function_label) {
    std::ostringstream pl;
    pl << "[[";
    for (size_t i = 0; i < patch_function_label.size(); ++i)
        pl << (i ? "," : "") << '[' << patch_function_label[i].first << ',' << patch_function_label[i].second << ']';
    pl << "]]";
    std::ostringstream cl;
    cl << '[';
    put_list(cl, cell_function_label);
    cl << ']';
    write_mesh_json(filename, mesh_pts, mesh_faces, patches, pl.str(), edges, chains, non_manifold_edges_of_vert, shells,
                    cells, cl.str());
    return true;
}

bool save_timings(const std::string& filename, const std::vector<std::string>& labels, const std::vector<double>& t) {
    std::map<std::string, double> m;
    for (size_t i = 0; i < t.size() && i < labels.size(); ++i) m[labels[i]] = t[i];
    std::ofstream f(filename);
    f << '{';
    bool first = true;
    for (auto& kv : m) {
        f << (first ? "" : ",") << '"' << kv.first << "\":" << json_double(kv.second);
        first = false;
    }
    f << "}\n";
    return true;
}

bool save_statistics(const std::string& filename, const std::vector<std::string>& labels, const std::vector<size_t>& s) {
    std::map<std::string, size_t> m;
    for (size_t i = 0; i < s.size() && i < labels.size(); ++i) m[labels[i]] = s[i];
    std::ofstream f(filename);
    f << '{';
    bool first = true;
    for (auto& kv : m) {
        f << (first ? "" : ",") << '"' << kv.first << "\":" << kv.second;
        first = false;
    }
    f << "}\n";
    return true;
}

bool save_result_CSG(const std::string& filename, const std::vector<std::array<double, 3>>& pts,
                     const std::vector<PolygonFace>& faces, const std::vector<std::vector<size_t>>& patches,
                     const std::vector<bool>& patch_sign_label, const std::vector<Edge>& edges,
                     const std::vector<std::vector<size_t>>& chains,
                     const std::vector<std::vector<size_t>>& nm_edges_of_vert) {
    // src/io.cpp:314-372: no shells, cells or cell labels
    std::ostringstream o;
    o << "{\"chains\":";
    put_lists(o, chains);
    std::vector<size_t> corners;
    for (size_t i = 0; i < nm_edges_of_vert.size(); ++i)
        if (nm_edges_of_vert[i].size() > 2 || nm_edges_of_vert[i].size() == 1) corners.push_back(i);
    o << ",\"corners\":";
    if (corners.empty())
        o << "null";
    else
        put_list(o, corners);
    o << ",\"edges\":";
    if (edges.empty()) {
        o << "null";
    } else {
        o << '[';
        for (size_t i = 0; i < edges.size(); ++i) o << (i ? "," : "") << '[' << edges[i].v1 << ',' << edges[i].v2 << ']';
        o << ']';
    }
    o << ",\"faces\":";
    if (faces.empty()) {
        o << "null";
    } else {
        o << '[';
        for (size_t i = 0; i < faces.size(); ++i) {
            if (i) o << ',';
            put_list(o, faces[i].vert_indices);
        }
        o << ']';
    }
    o << ",\"patches\":";
    put_lists(o, patches);
    o << ",\"patches_label\":[[";
    for (size_t i = 0; i < patch_sign_label.size(); ++i) o << (i ? "," : "") << (patch_sign_label[i] ? "true" : "false");
    o << "]],\"points\":";
    if (pts.empty()) {
        o << "null";
    } else {
        o << '[';
        for (size_t i = 0; i < pts.size(); ++i)
            o << (i ? "," : "") << '[' << json_double(pts[i][0]) << ',' << json_double(pts[i][1]) << ','
              << json_double(pts[i][2]) << ']';
        o << ']';
    }
    o << "}\n";
    std::ofstream f(filename);
    f << o.str();
    return true;
}

bool load_csg_tree(const std::string& filename, std::vector<CsgUnit>& tree) {
    std::ifstream fin(filename);
    if (!fin) {
        std::cout << "function file not exist!" << std::endl;
        return false;
    }
    Json d = JsonParser(read_file(filename)).parse();
    tree.clear();
    for (size_t j = 0; j < d.size(); ++j) {
        const std::string& t = d[j]["type"].as_string();
        CsgUnit u;
        u.op = t == "Intersection" ? 0 : (t == "Union" ? 1 : (t == "Negation" ? 2 : -1));
        if (u.op < 0) throw std::runtime_error("not a valid CSG operation: " + t);
        for (int i = 0; i < 2; ++i) u.elements[i] = (int)d[j]["elements"][i].as_double();
        tree.push_back(u);
    }
    return true;
}

std::function<bool(std::vector<bool>)> csg_lambda(const std::vector<CsgUnit>& tree) {
    if (tree.empty())
        return [](std::vector<bool> labels) {
            for (bool b : labels)
                if (b) return true;
            return false;
        };
    return [tree](std::vector<bool> labels) {
        // app/csg.cpp:54-136: function j is [1, 2] where positive, [-1, -2] elsewhere; union is the
        // maximum, intersection the minimum, negation the mirror; inside where the root is positive
        std::function<bool(int, int)> ev = [&](int e, int depth) -> bool {
            if (depth > 1000) throw std::runtime_error("CSG tree too deep or cyclic");
            if (e < 0) return labels.at((size_t)(-e - 1));
            const CsgUnit& u = tree.at((size_t)(e - 1));
            if (u.op == 2) return !ev(u.elements[0], depth + 1);
            const bool a = ev(u.elements[0], depth + 1), b = ev(u.elements[1], depth + 1);
            return u.op == 0 ? (a && b) : (a || b);
        };
        return ev(1, 0);
    };
}

}  // namespace ria_host
