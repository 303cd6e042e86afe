// CPU half of the host layer: configuration, tet-mesh and function-file readers, the tet grid,
// mesh connectivity (edges, patches, chains) and the JSON writers.  Needs no GPU.
#include <algorithm>
#include <atomic>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <mutex>
#include <sstream>
#include <thread>

#include "json.hpp"
#include "ria_host.hpp"

namespace ria_host {

namespace {

std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    f.seekg(0, std::ios::end);
    const std::streamoff n = f.tellg();
    f.seekg(0, std::ios::beg);
    std::string s(n > 0 ? (size_t)n : 0, '\0');
    if (n > 0 && !f.read(&s[0], n)) throw std::runtime_error("cannot read " + path);
    return s;
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

// The tet-mesh file [[[x, y, z], ...], [[v0, v1, v2, v3], ...]] read straight into the outputs:
// numbers by from_chars, no document tree.  Returns false at anything else (another layout,
// malformed text), which the general parser then reads or reports.
bool read_tet_mesh_fast(const std::string& text, std::vector<std::array<double, 3>>& pts,
                        std::vector<std::array<size_t, 4>>& tets) {
    const char* p = text.data();
    const char* const end = p + text.size();
    auto ws = [&] {
        while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
    };
    auto lit = [&](char c) {
        ws();
        if (p >= end || *p != c) return false;
        ++p;
        return true;
    };
    auto num = [&](double& v) {
        ws();
        const char* q = p;
        while (q < end && ((*q >= '0' && *q <= '9') || *q == '-' || *q == '+' || *q == '.' || *q == 'e' || *q == 'E'))
            ++q;
        if (q == p || std::from_chars(p, q, v).ptr != q) return false;
        p = q;
        return true;
    };
    // a list of rows of `width` numbers; `put(row)` stores one
    auto rows = [&](int width, auto&& put) {
        if (!lit('[')) return false;
        ws();
        if (p < end && *p == ']') {
            ++p;
            return true;
        }
        for (;;) {
            double row[4];
            if (!lit('[')) return false;
            for (int k = 0; k < width; ++k)
                if ((k && !lit(',')) || !num(row[k])) return false;
            if (!lit(']')) return false;
            put(row);
            if (lit(',')) continue;
            return lit(']');
        }
    };
    std::vector<std::array<double, 3>> P;
    std::vector<std::array<size_t, 4>> T;
    P.reserve(text.size() / 64);
    T.reserve(text.size() / 64);
    const bool ok = lit('[') && rows(3, [&](const double* r) { P.push_back({r[0], r[1], r[2]}); }) && lit(',') &&
                    rows(4, [&](const double* r) {
                        T.push_back({(size_t)r[0], (size_t)r[1], (size_t)r[2], (size_t)r[3]});
                    }) &&
                    lit(']');
    ws();
    if (!ok || p != end) return false;
    pts.swap(P);
    tets.swap(T);
    return true;
}

template <class V>
void put_list(JsonBuf& o, const V& v) {
    o.c('[');
    for (size_t i = 0; i < v.size(); ++i) {
        if (i) o.c(',');
        o.u(v[i]);
    }
    o.c(']');
}

// A JSON document written in order from pieces.  The large arrays (points, faces, edges) are
// formatted in chunks by several threads, each chunk its own piece.
struct JsonDoc {
    std::vector<std::string> parts;
    JsonBuf cur;

    void flush() {
        if (!cur.s.empty()) parts.push_back(std::move(cur.s));
        cur.s = std::string();
    }
    // "null" when n is 0, else [item0,item1,...]; emit(buf, i) writes item i and may run on any thread
    template <class Emit>
    void array(size_t n, const Emit& emit) {
        if (n == 0) {
            cur.str("null");
            return;
        }
        cur.c('[');
        constexpr size_t kChunk = 1 << 15;
        if (host_threads() < 2 || n < 2 * kChunk) {
            for (size_t i = 0; i < n; ++i) {
                if (i) cur.c(',');
                emit(cur, i);
            }
        } else {
            flush();
            // one piece per range, kept in range order
            std::vector<std::pair<size_t, std::string>> out;
            std::mutex mu;
            parallel_ranges(n, kChunk, [&](size_t lo, size_t hi) {
                JsonBuf b;
                for (size_t i = lo; i < hi; ++i) {
                    if (i) b.c(',');
                    emit(b, i);
                }
                std::lock_guard<std::mutex> lk(mu);
                out.emplace_back(lo, std::move(b.s));
            });
            std::sort(out.begin(), out.end(),
                      [](const std::pair<size_t, std::string>& a, const std::pair<size_t, std::string>& b) {
                          return a.first < b.first;
                      });
            for (auto& piece : out) parts.push_back(std::move(piece.second));
        }
        cur.c(']');
    }
    bool write(const std::string& filename) {
        flush();
        FILE* f = std::fopen(filename.c_str(), "wb");
        if (!f) return false;
        bool ok = true;
        for (const auto& piece : parts) ok = ok && std::fwrite(piece.data(), 1, piece.size(), f) == piece.size();
        return std::fclose(f) == 0 && ok;
    }
};

void put_lists(JsonDoc& o, const std::vector<std::vector<size_t>>& v) {
    o.array(v.size(), [&](JsonBuf& b, size_t i) { put_list(b, v[i]); });
}

void put_corners(JsonDoc& o, const std::vector<std::vector<size_t>>& nm_edges_of_vert) {
    std::vector<size_t> corners;
    for (size_t i = 0; i < nm_edges_of_vert.size(); ++i)
        if (nm_edges_of_vert[i].size() > 2 || nm_edges_of_vert[i].size() == 1) corners.push_back(i);
    if (corners.empty())
        o.cur.str("null");
    else
        put_list(o.cur, corners);
}

void put_edges(JsonDoc& o, const std::vector<Edge>& edges) {
    o.array(edges.size(), [&](JsonBuf& b, size_t i) {
        b.c('[');
        b.u(edges[i].v1);
        b.c(',');
        b.u(edges[i].v2);
        b.c(']');
    });
}

void put_faces(JsonDoc& o, const std::vector<PolygonFace>& faces) {
    o.array(faces.size(), [&](JsonBuf& b, size_t i) { put_list(b, faces[i].vert_indices); });
}

void put_points(JsonDoc& o, const std::vector<std::array<double, 3>>& pts) {
    o.array(pts.size(), [&](JsonBuf& b, size_t i) {
        b.c('[');
        b.d(pts[i][0]);
        b.c(',');
        b.d(pts[i][1]);
        b.c(',');
        b.d(pts[i][2]);
        b.c(']');
    });
}

// the keys of the reference's mesh.json, in its library's (sorted) key order; a list the reference
// never appends to stays null, as there
bool write_mesh_json(const std::string& filename, const std::vector<std::array<double, 3>>& pts,
                     const std::vector<PolygonFace>& faces, const std::vector<std::vector<size_t>>& patches,
                     const std::string& patches_label, const std::vector<Edge>& edges,
                     const std::vector<std::vector<size_t>>& chains,
                     const std::vector<std::vector<size_t>>& nm_edges_of_vert,
                     const std::vector<std::vector<size_t>>& shells, const std::vector<std::vector<size_t>>& cells,
                     const std::string& cells_label) {
    JsonDoc o;
    o.cur.str("{\"cells\":");
    put_lists(o, cells);
    o.cur.str(",\"cells_label\":");
    o.cur.str(cells_label);
    o.cur.str(",\"chains\":");
    put_lists(o, chains);
    o.cur.str(",\"corners\":");
    put_corners(o, nm_edges_of_vert);
    o.cur.str(",\"edges\":");
    put_edges(o, edges);
    o.cur.str(",\"faces\":");
    put_faces(o, faces);
    o.cur.str(",\"patches\":");
    put_lists(o, patches);
    o.cur.str(",\"patches_label\":");
    o.cur.str(patches_label);
    o.cur.str(",\"points\":");
    put_points(o, pts);
    o.cur.str(",\"shells\":");
    put_lists(o, shells);
    o.cur.str("}\n");
    return o.write(filename);
}

// compute_mesh_edges for large meshes, on several threads, with the same result: the occurrences
// (face, local edge) are bucketed by their smaller vertex in occurrence order; within a bucket each
// occurrence finds the first one of its larger vertex; the first occurrences are numbered by one
// scan in occurrence order; each edge's occurrences, all in one bucket, are listed in that order.
void compute_mesh_edges_parallel(const std::vector<PolygonFace>& mesh_faces,
                                 std::vector<std::vector<size_t>>& edges_of_face, std::vector<Edge>& mesh_edges,
                                 size_t vmax) {
    const size_t F = mesh_faces.size();
    std::vector<size_t> foff(F + 1, 0);
    for (size_t i = 0; i < F; ++i) foff[i + 1] = foff[i] + mesh_faces[i].vert_indices.size();
    const size_t n_occ = foff[F];
    std::vector<uint32_t> lo(n_occ), hi(n_occ), face(n_occ);
    parallel_ranges(F, 4096, [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i) {
            const auto& vs = mesh_faces[i].vert_indices;
            const size_t n = vs.size();
            for (size_t j = 0; j < n; ++j) {
                const size_t v1 = vs[j], v2 = vs[(j + 1) % n];
                lo[foff[i] + j] = (uint32_t)(v1 < v2 ? v1 : v2);
                hi[foff[i] + j] = (uint32_t)(v1 < v2 ? v2 : v1);
                face[foff[i] + j] = (uint32_t)i;
            }
        }
    });
    // buckets by smaller vertex, occurrences in increasing order within each
    std::vector<uint32_t> boff(vmax + 2, 0);
    for (size_t o = 0; o < n_occ; ++o) ++boff[lo[o] + 1];
    for (size_t v = 0; v <= vmax; ++v) boff[v + 1] += boff[v];
    std::vector<uint32_t> bucket(n_occ);
    {
        std::vector<uint32_t> fill(boff.begin(), boff.end() - 1);
        for (size_t o = 0; o < n_occ; ++o) bucket[fill[lo[o]]++] = (uint32_t)o;
    }
    // first occurrence of every occurrence's edge, and how many occurrences each first one heads
    std::vector<uint32_t> first(n_occ), count(n_occ, 0);
    parallel_ranges(vmax + 1, 4096, [&](size_t a, size_t b) {
        for (size_t v = a; v < b; ++v)
            for (uint32_t x = boff[v]; x < boff[v + 1]; ++x) {
                const uint32_t o = bucket[x];
                uint32_t f = o;
                for (uint32_t y = boff[v]; y < x; ++y)
                    if (hi[bucket[y]] == hi[o]) {
                        f = first[bucket[y]];
                        break;
                    }
                first[o] = f;
                ++count[f];
            }
    });
    // edge ids of the first occurrences, in occurrence order
    const size_t base = mesh_edges.size();
    std::vector<uint32_t> eid(n_occ);
    size_t n_edges = 0;
    for (size_t o = 0; o < n_occ; ++o)
        if (first[o] == o) eid[o] = (uint32_t)n_edges++;
    mesh_edges.resize(base + n_edges);
    parallel_ranges(vmax + 1, 4096, [&](size_t a, size_t b) {
        for (size_t v = a; v < b; ++v)
            for (uint32_t x = boff[v]; x < boff[v + 1]; ++x) {
                const uint32_t o = bucket[x];
                Edge& e = mesh_edges[base + eid[first[o]]];
                if (first[o] == o) {
                    e.v1 = lo[o];
                    e.v2 = hi[o];
                    e.face_edge_indices.reserve(count[o]);
                }
                e.face_edge_indices.emplace_back(face[o], o - foff[face[o]]);
            }
    });
    edges_of_face.assign(F, {});
    parallel_ranges(F, 4096, [&](size_t a, size_t b) {
        for (size_t i = a; i < b; ++i) {
            auto& ef = edges_of_face[i];
            ef.resize(foff[i + 1] - foff[i]);
            for (size_t j = 0; j < ef.size(); ++j) ef[j] = base + eid[first[foff[i] + j]];
        }
    });
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
    const std::string text = read_file(filename);
    if (read_tet_mesh_fast(text, pts, tets)) return true;
    Json d = JsonParser(text).parse();
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

// src/mesh_connectivity.cpp:10-56: edges numbered by first occurrence in face order, each with its
// (face, local edge) occurrences in that order.  An edge is found among the edges already seen at
// its smaller vertex: those lists are laid out by vertex (counted in a first pass) and stay short,
// and vertices numbered in face order keep the accesses local.  Ids past 32 bits take an ordered map.
void compute_mesh_edges(const std::vector<PolygonFace>& mesh_faces, std::vector<std::vector<size_t>>& edges_of_face,
                        std::vector<Edge>& mesh_edges) {
    size_t n_occ = 0, vmax = 0;
    for (const auto& f : mesh_faces) {
        n_occ += f.vert_indices.size();
        for (size_t v : f.vert_indices) vmax = v > vmax ? v : vmax;
    }
    if (vmax < 0xFFFFFFFFull && n_occ >= (1u << 16) && n_occ < 0xFFFFFFFFull && host_threads() > 1) {
        compute_mesh_edges_parallel(mesh_faces, edges_of_face, mesh_edges, vmax);
        return;
    }
    edges_of_face.assign(mesh_faces.size(), {});
    mesh_edges.reserve(mesh_edges.size() + n_occ / 2 + 16);  // interior edges are shared by two faces
    auto add = [&](size_t i, size_t j, size_t v1, size_t v2, size_t id) {
        if (id == mesh_edges.size()) {
            mesh_edges.push_back(Edge{v1, v2, {}});
            mesh_edges.back().face_edge_indices.reserve(2);
        }
        mesh_edges[id].face_edge_indices.emplace_back(i, j);
        edges_of_face[i][j] = id;
    };
    if (vmax < 0xFFFFFFFFull && mesh_edges.size() + n_occ < 0xFFFFFFFFull) {
        // first[v]..first[v+1]: room for every occurrence whose smaller vertex is v
        std::vector<uint32_t> first(vmax + 2, 0), used(vmax + 1, 0);
        for (const auto& f : mesh_faces) {
            const auto& vs = f.vert_indices;
            for (size_t j = 0; j < vs.size(); ++j) {
                const size_t a = vs[j], b = vs[(j + 1) % vs.size()];
                ++first[(a < b ? a : b) + 1];
            }
        }
        for (size_t v = 0; v <= vmax; ++v) first[v + 1] += first[v];
        std::vector<uint64_t> seen(n_occ);  // (larger vertex << 32) | edge id
        for (size_t i = 0; i < mesh_faces.size(); ++i) {
            const auto& vs = mesh_faces[i].vert_indices;
            const size_t n = vs.size();
            edges_of_face[i].resize(n);
            for (size_t j = 0; j < n; ++j) {
                size_t v1 = vs[j], v2 = vs[(j + 1) % n];
                if (v1 > v2) std::swap(v1, v2);
                uint64_t* list = seen.data() + first[v1];
                const uint32_t m = used[v1];
                size_t id = mesh_edges.size();
                for (uint32_t t = 0; t < m; ++t)
                    if ((list[t] >> 32) == v2) {
                        id = (size_t)(list[t] & 0xFFFFFFFFull);
                        break;
                    }
                if (id == mesh_edges.size()) list[used[v1]++] = ((uint64_t)v2 << 32) | (uint64_t)id;
                add(i, j, v1, v2, id);
            }
        }
        return;
    }
    std::map<std::pair<size_t, size_t>, size_t> edge_id;
    for (size_t i = 0; i < mesh_faces.size(); ++i) {
        const auto& vs = mesh_faces[i].vert_indices;
        const size_t n = vs.size();
        edges_of_face[i].resize(n);
        for (size_t j = 0; j < n; ++j) {
            size_t v1 = vs[j], v2 = vs[(j + 1) % n];
            if (v1 > v2) std::swap(v1, v2);
            auto ins = edge_id.emplace(std::make_pair(v1, v2), mesh_edges.size());
            add(i, j, v1, v2, ins.first->second);
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
        patch.push_back(i);
        visited[i] = 1;
        patch_label.push_back(mesh_faces[i].func_index);
        // breadth-first: the patch lists faces in the order they are reached, which is the order
        // they are expanded, so it serves as the queue
        for (size_t q = 0; q < patch.size(); ++q) {
            const size_t f = patch[q];
            for (size_t e : edges_of_face[f]) {
                const auto& fe = mesh_edges[e].face_edge_indices;
                if (fe.size() != 2) continue;
                size_t o = fe[0].first == f ? fe[1].first : fe[0].first;
                if (!visited[o]) {
                    visited[o] = 1;
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
        chain.push_back(i);
        visited[i] = 1;
        for (size_t q = 0; q < chain.size(); ++q) {  // breadth-first, the chain as the queue
            const size_t e = chain[q];
            for (size_t v : {mesh_edges[e].v1, mesh_edges[e].v2}) {
                if (nm_edges_of_vert[v].size() != 2) continue;
                size_t o = nm_edges_of_vert[v][0] == e ? nm_edges_of_vert[v][1] : nm_edges_of_vert[v][0];
                if (!visited[o]) {
                    visited[o] = 1;
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
    JsonBuf pl;
    pl.c('[');
    put_list(pl, patch_function_label);
    pl.c(']');
    JsonBuf cl;
    if (cell_function_label.empty()) {
        cl.str("null");
    } else {
        cl.c('[');
        for (size_t i = 0; i < cell_function_label.size(); ++i) {
            if (i) cl.c(',');
            cl.c('[');
            for (size_t j = 0; j < cell_function_label[i].size(); ++j) {
                if (j) cl.c(',');
                cl.str(cell_function_label[i][j] ? "true" : "false");
            }
            cl.c(']');
        }
        cl.c(']');
    }
    return write_mesh_json(filename, mesh_pts, mesh_faces, patches, pl.s, edges, chains, non_manifold_edges_of_vert,
                           shells, cells, cl.s);
}

bool save_result_MI(const std::string& filename, const std::vector<std::array<double, 3>>& mesh_pts,
                    const std::vector<PolygonFace>& mesh_faces, const std::vector<std::vector<size_t>>& patches,
                    const std::vector<std::pair<size_t, size_t>>& patch_function_label, const std::vector<Edge>& edges,
                    const std::vector<std::vector<size_t>>& chains,
                    const std::vector<std::vector<size_t>>& non_manifold_edges_of_vert,
                    const std::vector<std::vector<size_t>>& shells, const std::vector<std::vector<size_t>>& cells,
                    const std::vector<size_t>& cell_function_label) {
    JsonBuf pl;
    pl.str("[[");
    for (size_t i = 0; i < patch_function_label.size(); ++i) {
        if (i) pl.c(',');
        pl.c('[');
        pl.u(patch_function_label[i].first);
        pl.c(',');
        pl.u(patch_function_label[i].second);
        pl.c(']');
    }
    pl.str("]]");
    JsonBuf cl;
    cl.c('[');
    put_list(cl, cell_function_label);
    cl.c(']');
    return write_mesh_json(filename, mesh_pts, mesh_faces, patches, pl.s, edges, chains, non_manifold_edges_of_vert,
                           shells, cells, cl.s);
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
    JsonDoc o;
    o.cur.str("{\"chains\":");
    put_lists(o, chains);
    o.cur.str(",\"corners\":");
    put_corners(o, nm_edges_of_vert);
    o.cur.str(",\"edges\":");
    put_edges(o, edges);
    o.cur.str(",\"faces\":");
    put_faces(o, faces);
    o.cur.str(",\"patches\":");
    put_lists(o, patches);
    o.cur.str(",\"patches_label\":[[");
    for (size_t i = 0; i < patch_sign_label.size(); ++i) {
        if (i) o.cur.c(',');
        o.cur.str(patch_sign_label[i] ? "true" : "false");
    }
    o.cur.str("]],\"points\":");
    put_points(o, pts);
    o.cur.str("}\n");
    return o.write(filename);
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
