// CPU oracle (test infrastructure only): per-tet implicit arrangement (IA) and material
// interface (MI), written from the mathematics.  See cut.hpp for the contract and the
// canonical form.  Only tests/, the smoke check and bench.py's CPU baseline use this code.
#include "cut.hpp"

#include <algorithm>
#include <cstdlib>
#include <map>
#include <stdexcept>

#include "exact.hpp"

namespace oracle {

int g_selfcheck = 0;  // when set, canonical labels are re-derived by an exact greedy search

namespace {

// Tet face b is opposite corner b.  Loops below run counter-clockwise seen from inside the tet
// (the positive side of b) in the reference frame x = (b1, b2, b3).
const int kInward[4][3] = {{1, 3, 2}, {0, 2, 3}, {0, 3, 1}, {0, 1, 2}};
const int kOutward[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};

inline uint64_t bit(int l) { return uint64_t(1) << l; }

struct Row4 {
    double v[4];
};

// ----------------------------------------------------------------------------------------------
// shared helpers

// Lexicographically smallest independent label set drawn from `mask` (greedy over a matroid).
// IA rows: boundary b -> e_b, plane l -> its 4 values (4 columns); size 3.
// MI rows: boundary b -> (e_b, 0), material l -> (values, 1) (5 columns); size 4.
std::vector<int> greedy_labels(uint64_t mask, const std::vector<Row4>& P, bool mi) {
    int want = mi ? 4 : 3;
    int ncol = mi ? 5 : 4;
    std::vector<std::array<double, 5>> rows;
    std::vector<int> out;
    for (int l = 0; l < 64 && (int)out.size() < want; ++l) {
        if (!(mask & bit(l))) continue;
        std::array<double, 5> r{};
        if (l < 4) {
            r[l] = 1.0;
        } else {
            for (int c = 0; c < 4; ++c) r[c] = P[l].v[c];
            if (mi) r[4] = 1.0;
        }
        rows.push_back(r);
        std::vector<const double*> ptr;
        for (auto& x : rows) ptr.push_back(x.data());
        if (rows_independent(ptr.data(), (int)rows.size(), ncol)) {
            out.push_back(l);
        } else {
            rows.pop_back();
        }
    }
    return out;
}

template <size_t N>
void build_cache(VCache& c, const std::array<int, N>& lab, const std::vector<Row4>& P, bool mi) {
    bool bound[4] = {false, false, false, false};
    const double* rows[4];
    int m = 0;
    for (size_t t = 0; t < N; ++t) {
        int l = lab[t];
        if (l < 4)
            bound[l] = true;
        else
            rows[m++] = P[l].v;
    }
    int S[4], s = 0;
    for (int c = 0; c < 4; ++c)
        if (!bound[c]) S[s++] = c;
    vcache_build(c, mi, s, S, m, rows);
}

// From a loop (already in the orientation wanted) and per-vertex signs, return the directed cap
// edge (wa -> wb) bounding the run of negative vertices, or false when there is none.
bool negative_run_edge(const std::vector<int>& seq, const std::vector<int>& sg, int& wa, int& wb) {
    int n = (int)seq.size();
    int j0 = -1;
    for (int j = 0; j < n; ++j) {
        int prev = seq[(j - 1 + n) % n];
        if (sg[seq[j]] < 0 && sg[prev] >= 0) {
            j0 = j;
            break;
        }
    }
    if (j0 < 0) return false;  // no negative vertex, or all negative
    int j1 = j0;
    while (sg[seq[(j1 + 1) % n]] < 0) j1 = (j1 + 1) % n;
    wa = seq[(j0 - 1 + n) % n];
    wb = seq[(j1 + 1) % n];
    return wa != wb;
}

std::vector<int> chain_loop(const std::map<int, int>& next) {
    std::vector<int> loop;
    if (next.empty()) return loop;
    int start = next.begin()->first;
    int cur = start;
    for (size_t it = 0; it <= next.size(); ++it) {
        loop.push_back(cur);
        auto f = next.find(cur);
        if (f == next.end()) throw std::runtime_error("cap loop open");
        cur = f->second;
        if (cur == start) break;
    }
    if (cur != start || loop.size() != next.size()) throw std::runtime_error("cap loop inconsistent");
    return loop;
}

void rotate_min(std::vector<int>& loop) {
    auto it = std::min_element(loop.begin(), loop.end());
    std::rotate(loop.begin(), it, loop.end());
}

// ----------------------------------------------------------------------------------------------
// implicit arrangement

struct IV {
    std::array<int, 3> lab;
    uint64_t mask;
    VCache c;
};

struct IF {
    int supp;
    int pos, neg;
    std::vector<int> loop;
};

}  // namespace

bool ia_cut(int k, const double* planes, IARecord& out, CutStats* st) {
    if (k < 0 || k > 60) return false;
    const int L = 4 + k;
    std::vector<Row4> P(L);
    for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c) P[b].v[c] = (b == c) ? 1.0 : 0.0;
    for (int i = 0; i < k; ++i)
        for (int c = 0; c < 4; ++c) P[4 + i].v[c] = planes[4 * i + c];

    // coincident planes: exact proportionality of the 4-vectors
    std::vector<uint8_t> rep(k);
    for (int i = 0; i < k; ++i) {
        const double* a = P[4 + i].v;
        int nz = 0, last = -1;
        for (int c = 0; c < 4; ++c)
            if (a[c] != 0.0) {
                ++nz;
                last = c;
            }
        if (nz == 0) {
            rep[i] = 0xFF;
            continue;
        }
        if (nz == 1) {
            rep[i] = (uint8_t)last;
            continue;
        }
        rep[i] = (uint8_t)(4 + i);
        for (int j = 0; j < i; ++j) {
            if (rep[j] != 4 + j) continue;
            const double* b = P[4 + j].v;
            bool prop = true;
            for (int x = 0; x < 4 && prop; ++x)
                for (int y = x + 1; y < 4 && prop; ++y)
                    if (!prod_eq(a[x], b[y], a[y], b[x])) prop = false;
            if (prop) {
                rep[i] = (uint8_t)(4 + j);
                break;
            }
        }
    }

    std::vector<IV> V(4);
    for (int c = 0; c < 4; ++c) {
        int t = 0;
        for (int b = 0; b < 4; ++b)
            if (b != c) V[c].lab[t++] = b;
        V[c].mask = 0xFull & ~bit(c);
        build_cache(V[c].c, V[c].lab, P, false);
    }
    std::vector<IF> F(4);
    for (int b = 0; b < 4; ++b) {
        F[b].supp = b;
        F[b].pos = 0;
        F[b].neg = -1;
        F[b].loop.assign(kInward[b], kInward[b] + 3);
    }
    std::vector<uint64_t> Csign(1, 0);

    for (int i = 0; i < k; ++i) {
        if (rep[i] != 4 + i) continue;
        const int q = 4 + i;
        std::vector<int> sg(V.size());
        for (size_t v = 0; v < V.size(); ++v) {
            sg[v] = vcache_query(V[v].c, P[q].v, st ? &st->exact_calls : nullptr);
            if (sg[v] == 0) V[v].mask |= bit(q);
        }
        const int nc = (int)Csign.size();
        std::vector<char> cpos(nc, 0), cneg(nc, 0);
        for (auto& f : F)
            for (int v : f.loop)
                for (int cid : {f.pos, f.neg}) {
                    if (cid < 0) continue;
                    if (sg[v] > 0) cpos[cid] = 1;
                    if (sg[v] < 0) cneg[cid] = 1;
                }
        std::vector<char> strad(nc, 0);
        bool any = false;
        for (int c = 0; c < nc; ++c) {
            strad[c] = cpos[c] && cneg[c];
            any = any || strad[c];
            if (!strad[c] && cpos[c]) Csign[c] |= bit(q);
        }
        if (!any) continue;

        // vertices on crossing edges
        std::map<std::pair<int, int>, int> emap;
        for (auto& f : F) {
            std::vector<int> nl;
            int n = (int)f.loop.size();
            for (int j = 0; j < n; ++j) {
                int u = f.loop[j], w = f.loop[(j + 1) % n];
                nl.push_back(u);
                if (sg[u] * sg[w] < 0) {
                    auto key = std::make_pair(std::min(u, w), std::max(u, w));
                    auto it = emap.find(key);
                    int id;
                    if (it != emap.end()) {
                        id = it->second;
                    } else {
                        uint64_t em = V[u].mask & V[w].mask;
                        int p1 = __builtin_ctzll(em);
                        int p2 = __builtin_ctzll(em & ~bit(p1));
                        IV nv;
                        nv.lab = {p1, p2, q};
                        nv.mask = em | bit(q);
                        build_cache(nv.c, nv.lab, P, false);
                        id = (int)V.size();
                        V.push_back(nv);
                        sg.push_back(0);
                        emap[key] = id;
                    }
                    nl.push_back(id);
                }
            }
            f.loop = nl;
        }

        // split faces
        const int nF0 = (int)F.size();
        std::vector<std::vector<int>> full(nF0);
        std::vector<int> fside(nF0, 0), fneg_of(nF0, -1);
        for (int f = 0; f < nF0; ++f) {
            full[f] = F[f].loop;
            bool hp = false, hn = false;
            for (int v : F[f].loop) {
                hp = hp || sg[v] > 0;
                hn = hn || sg[v] < 0;
            }
            if (hp && hn) {
                std::vector<int> lp, ln;
                for (int v : F[f].loop) {
                    if (sg[v] >= 0) lp.push_back(v);
                    if (sg[v] <= 0) ln.push_back(v);
                }
                IF g = F[f];
                g.loop = ln;
                F[f].loop = lp;
                fneg_of[f] = (int)F.size();
                F.push_back(g);
                fside[f] = 2;
            } else {
                fside[f] = hp ? 1 : -1;
            }
        }
        const int nF1 = (int)F.size();

        // split cells
        std::vector<int> cneg_of(nc, -1);
        for (int c = 0; c < nc; ++c) {
            if (!strad[c]) continue;
            cneg_of[c] = (int)Csign.size();
            Csign.push_back(Csign[c]);
            Csign[c] |= bit(q);
        }
        // cap faces
        std::vector<IF> caps;
        for (int c = 0; c < nc; ++c) {
            if (!strad[c]) continue;
            std::map<int, int> next;
            for (int f = 0; f < nF0; ++f) {
                if (F[f].pos != c && F[f].neg != c) continue;
                std::vector<int> seq = full[f];
                if (F[f].neg != c) std::reverse(seq.begin(), seq.end());  // inward -> outward
                int wa, wb;
                if (negative_run_edge(seq, sg, wa, wb)) {
                    if (next.count(wa)) throw std::runtime_error("cap edge clash");
                    next[wa] = wb;
                }
            }
            IF cap;
            cap.supp = q;
            cap.pos = c;
            cap.neg = cneg_of[c];
            cap.loop = chain_loop(next);
            if (cap.loop.size() < 3) throw std::runtime_error("degenerate cap");
            caps.push_back(cap);
        }
        // cell references of the faces on the negative side
        auto mapneg = [&](int cid) { return (cid >= 0 && cneg_of[cid] >= 0) ? cneg_of[cid] : cid; };
        for (int f = 0; f < nF0; ++f)
            if (fside[f] == -1) {
                F[f].pos = mapneg(F[f].pos);
                F[f].neg = mapneg(F[f].neg);
            }
        for (int f = nF0; f < nF1; ++f) {
            F[f].pos = mapneg(F[f].pos);
            F[f].neg = mapneg(F[f].neg);
        }
        for (auto& cp : caps) F.push_back(cp);
    }

    // ---- canonical form
    std::vector<char> live(V.size(), 0);
    for (auto& f : F)
        for (int v : f.loop) live[v] = 1;
    std::vector<int> order;
    for (size_t v = 0; v < V.size(); ++v)
        if (live[v]) order.push_back((int)v);
    for (int v : order) {
        std::sort(V[v].lab.begin(), V[v].lab.end());
        if (g_selfcheck) {
            auto g = greedy_labels(V[v].mask, P, false);
            if (g.size() != 3 || g[0] != V[v].lab[0] || g[1] != V[v].lab[1] || g[2] != V[v].lab[2])
                throw std::runtime_error("IA vertex label is not the lexicographically smallest basis");
        }
    }
    std::sort(order.begin(), order.end(), [&](int a, int b) { return V[a].lab < V[b].lab; });
    std::vector<int> vnew(V.size(), -1);
    for (size_t i = 0; i < order.size(); ++i) vnew[order[i]] = (int)i;

    std::vector<int> corder(Csign.size());
    for (size_t c = 0; c < Csign.size(); ++c) corder[c] = (int)c;
    std::sort(corder.begin(), corder.end(), [&](int a, int b) { return Csign[a] < Csign[b]; });
    std::vector<int> cnew(Csign.size());
    for (size_t i = 0; i < corder.size(); ++i) cnew[corder[i]] = (int)i;

    struct FK {
        int supp;
        std::vector<int> sorted;
        int idx;
    };
    std::vector<FK> keys;
    for (size_t f = 0; f < F.size(); ++f) {
        for (int& v : F[f].loop) v = vnew[v];
        rotate_min(F[f].loop);
        FK key{F[f].supp, F[f].loop, (int)f};
        std::sort(key.sorted.begin(), key.sorted.end());
        keys.push_back(key);
    }
    std::sort(keys.begin(), keys.end(), [](const FK& a, const FK& b) {
        if (a.supp != b.supp) return a.supp < b.supp;
        return a.sorted < b.sorted;
    });

    out = IARecord();
    out.k = k;
    out.rep = rep;
    for (int v : order) out.verts.push_back({(uint8_t)V[v].lab[0], (uint8_t)V[v].lab[1], (uint8_t)V[v].lab[2]});
    for (auto& key : keys) {
        const IF& f = F[key.idx];
        IAFaceRec r;
        r.supp = f.supp;
        r.pos = cnew[f.pos];
        r.neg = f.neg < 0 ? -1 : cnew[f.neg];
        r.loop = f.loop;
        out.faces.push_back(r);
    }
    for (int c : corder) out.cell_sign.push_back(Csign[c]);
    return true;
}

// ----------------------------------------------------------------------------------------------
// material interface

namespace {

struct MV {
    uint64_t mask;
    VCache c;
};

struct MF {
    int other;  // 0..3: tet face; >= 4: the material on the other side
    std::vector<int> loop;  // counter-clockwise seen from outside the cell
};

struct Poly {
    std::vector<MV> V;
    std::vector<MF> F;
};

}  // namespace

bool mi_cut(int k, const double* materials, MIRecord& out, CutStats* st) {
    if (k < 0 || k > 60) return false;
    const int L = 4 + k;
    std::vector<Row4> P(L);
    for (int b = 0; b < 4; ++b)
        for (int c = 0; c < 4; ++c) P[b].v[c] = (b == c) ? 1.0 : 0.0;
    for (int i = 0; i < k; ++i)
        for (int c = 0; c < 4; ++c) P[4 + i].v[c] = materials[4 * i + c];

    // identical materials share one cell
    std::vector<uint8_t> rep(k);
    std::vector<int> uniq;
    for (int i = 0; i < k; ++i) {
        rep[i] = (uint8_t)(4 + i);
        for (int j = 0; j < i; ++j) {
            if (rep[j] != 4 + j) continue;
            bool same = true;
            for (int c = 0; c < 4; ++c)
                if (P[4 + i].v[c] != P[4 + j].v[c]) same = false;
            if (same) {
                rep[i] = (uint8_t)(4 + j);
                break;
            }
        }
        if (rep[i] == 4 + i) uniq.push_back(4 + i);
    }

    std::map<int, Poly> cells;
    for (int m : uniq) {
        Poly poly;
        poly.V.resize(4);
        for (int c = 0; c < 4; ++c) {
            std::array<int, 4> lab;
            int t = 0;
            for (int b = 0; b < 4; ++b)
                if (b != c) lab[t++] = b;
            lab[3] = m;
            poly.V[c].mask = (0xFull & ~bit(c)) | bit(m);
            build_cache(poly.V[c].c, lab, P, true);
        }
        poly.F.resize(4);
        for (int b = 0; b < 4; ++b) {
            poly.F[b].other = b;
            poly.F[b].loop.assign(kOutward[b], kOutward[b] + 3);
        }
        bool empty = false;
        for (int j : uniq) {
            if (j == m) continue;
            std::vector<int> sg(poly.V.size(), 0);
            std::vector<char> live(poly.V.size(), 0);
            for (auto& f : poly.F)
                for (int v : f.loop) live[v] = 1;
            bool hp = false, hn = false;
            for (size_t v = 0; v < poly.V.size(); ++v) {
                if (!live[v]) continue;
                sg[v] = vcache_query(poly.V[v].c, P[j].v, st ? &st->exact_calls : nullptr);
                if (sg[v] == 0) poly.V[v].mask |= bit(j);
                hp = hp || sg[v] > 0;
                hn = hn || sg[v] < 0;
            }
            if (!hn) {
                empty = true;
                break;
            }
            if (!hp) continue;
            std::map<std::pair<int, int>, int> emap;
            for (auto& f : poly.F) {
                std::vector<int> nl;
                int n = (int)f.loop.size();
                for (int a = 0; a < n; ++a) {
                    int u = f.loop[a], w = f.loop[(a + 1) % n];
                    nl.push_back(u);
                    if (sg[u] * sg[w] < 0) {
                        auto key = std::make_pair(std::min(u, w), std::max(u, w));
                        auto it = emap.find(key);
                        int id;
                        if (it != emap.end()) {
                            id = it->second;
                        } else {
                            uint64_t em = poly.V[u].mask & poly.V[w].mask;
                            MV nv;
                            nv.mask = em | bit(j);
                            std::array<int, 4> lab;
                            if (__builtin_popcountll(em) == 3) {
                                int t = 0;
                                for (int l = 0; l < 64; ++l)
                                    if (nv.mask & bit(l)) lab[t++] = l;
                            } else {
                                auto g = greedy_labels(nv.mask, P, true);
                                if (g.size() != 4) throw std::runtime_error("MI vertex without a basis");
                                for (int t = 0; t < 4; ++t) lab[t] = g[t];
                            }
                            build_cache(nv.c, lab, P, true);
                            id = (int)poly.V.size();
                            poly.V.push_back(nv);
                            sg.push_back(0);
                            emap[key] = id;
                        }
                        nl.push_back(id);
                    }
                }
                f.loop = nl;
            }
            std::map<int, int> next;
            std::vector<MF> nf;
            for (auto& f : poly.F) {
                bool fp = false, fn = false;
                for (int v : f.loop) {
                    fp = fp || sg[v] > 0;
                    fn = fn || sg[v] < 0;
                }
                if (!fn) continue;  // entirely on the removed side (or a touching edge/point)
                int wa, wb;
                if (negative_run_edge(f.loop, sg, wa, wb)) {
                    if (next.count(wa)) throw std::runtime_error("MI cap edge clash");
                    next[wa] = wb;
                }
                MF g;
                g.other = f.other;
                if (fp) {
                    for (int v : f.loop)
                        if (sg[v] <= 0) g.loop.push_back(v);
                } else {
                    g.loop = f.loop;
                }
                nf.push_back(g);
            }
            MF cap;
            cap.other = j;
            cap.loop = chain_loop(next);
            if (cap.loop.size() < 3) throw std::runtime_error("MI degenerate cap");
            nf.push_back(cap);
            poly.F = nf;
        }
        if (!empty) cells[m] = std::move(poly);
    }

    // ---- canonical form
    std::map<std::array<int, 4>, int> vid;
    std::map<int, std::vector<std::array<int, 4>>> clab;  // per cell: labels of its vertices
    for (auto& [m, poly] : cells) {
        std::vector<std::array<int, 4>> labs(poly.V.size());
        std::vector<char> live(poly.V.size(), 0);
        for (auto& f : poly.F)
            for (int v : f.loop) live[v] = 1;
        for (size_t v = 0; v < poly.V.size(); ++v) {
            if (!live[v]) continue;
            std::array<int, 4> lab;
            uint64_t mk = poly.V[v].mask;
            if (__builtin_popcountll(mk) == 4) {
                int t = 0;
                for (int l = 0; l < 64; ++l)
                    if (mk & bit(l)) lab[t++] = l;
            } else {
                auto g = greedy_labels(mk, P, true);
                if (g.size() != 4) throw std::runtime_error("MI vertex without a basis");
                for (int t = 0; t < 4; ++t) lab[t] = g[t];
            }
            labs[v] = lab;
            vid[lab] = 0;
        }
        clab[m] = labs;
    }
    int nextid = 0;
    for (auto& kv : vid) kv.second = nextid++;

    out = MIRecord();
    out.k = k;
    out.rep = rep;
    for (auto& kv : vid) out.verts.push_back({(uint8_t)kv.first[0], (uint8_t)kv.first[1], (uint8_t)kv.first[2], (uint8_t)kv.first[3]});
    // Interface faces are identified by their vertex sets: the face of cell m against the material
    // j it was clipped by may border another cell when tie planes coincide (m - j parallel to
    // m - k), so the neighbouring cell is the one holding the same polygon.  Each interface is
    // emitted once, from the smaller material's cell (outward there, so toward the larger one).
    struct CF {
        int m, other;
        std::vector<int> loop, sorted;
    };
    std::vector<CF> all;
    for (auto& [m, poly] : cells) {
        const auto& labs = clab[m];
        for (auto& f : poly.F) {
            CF c{m, f.other, {}, {}};
            for (int v : f.loop) c.loop.push_back(vid[labs[v]]);
            c.sorted = c.loop;
            std::sort(c.sorted.begin(), c.sorted.end());
            all.push_back(c);
        }
    }
    std::map<std::pair<int, int>, std::vector<int>> faces;  // (pos, neg) -> loop
    for (size_t i = 0; i < all.size(); ++i) {
        CF& f = all[i];
        std::vector<int> loop = f.loop;
        if (f.other < 4) {
            rotate_min(loop);
            faces[{f.other, f.m}] = loop;
            continue;
        }
        int partner = -1;
        for (size_t j = 0; j < all.size() && partner < 0; ++j)
            if (j != i && all[j].other >= 4 && all[j].m != f.m && all[j].sorted == f.sorted) partner = (int)j;
        if (partner >= 0) {
            const int mo = all[partner].m;
            if (f.m > mo) continue;
            rotate_min(loop);
            if (g_selfcheck) {
                std::vector<int> rev = all[partner].loop;
                std::reverse(rev.begin(), rev.end());
                rotate_min(rev);
                if (rev != loop) throw std::runtime_error("MI interface seen differently from its two cells");
            }
            faces[{mo, f.m}] = loop;
        } else {
            // no cell holds the same polygon (coincident tie planes splitting the neighbour):
            // keep the clipping label, oriented toward the larger material
            if (f.m > f.other) std::reverse(loop.begin(), loop.end());
            rotate_min(loop);
            faces[{std::max(f.m, f.other), std::min(f.m, f.other)}] = loop;
        }
    }
    for (auto& kv : faces) {
        MIFaceRec r;
        r.pos_label = kv.first.first;
        r.neg_label = kv.first.second;
        r.loop = kv.second;
        out.faces.push_back(r);
    }
    for (auto& kv : cells) out.cell_label.push_back(kv.first);
    return true;
}

// ----------------------------------------------------------------------------------------------
// serialisation

namespace {
void put8(std::vector<uint8_t>& b, int v) { b.push_back((uint8_t)v); }
void put16(std::vector<uint8_t>& b, int v) {
    b.push_back((uint8_t)(v & 0xFF));
    b.push_back((uint8_t)((v >> 8) & 0xFF));
}
void put64(std::vector<uint8_t>& b, uint64_t v) {
    for (int i = 0; i < 8; ++i) b.push_back((uint8_t)((v >> (8 * i)) & 0xFF));
}
}  // namespace

void ia_serialize(const IARecord& r, std::vector<uint8_t>& b) {
    int nloop = 0;
    for (auto& f : r.faces) nloop += (int)f.loop.size();
    put8(b, 1);
    put8(b, r.k);
    put16(b, (int)r.verts.size());
    put16(b, (int)r.faces.size());
    put16(b, (int)r.cell_sign.size());
    put16(b, nloop);
    for (auto x : r.rep) put8(b, x);
    for (auto& v : r.verts)
        for (int t = 0; t < 3; ++t) put8(b, v[t]);
    for (auto& f : r.faces) {
        put8(b, f.supp);
        put8(b, f.neg < 0 ? 1 : 0);
        put16(b, f.pos);
        put16(b, f.neg < 0 ? kNone16 : f.neg);
        put16(b, (int)f.loop.size());
    }
    for (auto& f : r.faces)
        for (int v : f.loop) put16(b, v);
    for (auto s : r.cell_sign) put64(b, s);
}

void mi_serialize(const MIRecord& r, std::vector<uint8_t>& b) {
    int nloop = 0;
    for (auto& f : r.faces) nloop += (int)f.loop.size();
    put8(b, 2);
    put8(b, r.k);
    put16(b, (int)r.verts.size());
    put16(b, (int)r.faces.size());
    put16(b, (int)r.cell_label.size());
    put16(b, nloop);
    for (auto x : r.rep) put8(b, x);
    for (auto& v : r.verts)
        for (int t = 0; t < 4; ++t) put8(b, v[t]);
    for (auto& f : r.faces) {
        put8(b, f.pos_label);
        put8(b, f.neg_label);
        put16(b, (int)f.loop.size());
    }
    for (auto& f : r.faces)
        for (int v : f.loop) put16(b, v);
    for (int c : r.cell_label) put8(b, c);
}

}  // namespace oracle
