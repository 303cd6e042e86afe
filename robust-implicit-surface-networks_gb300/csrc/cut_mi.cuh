// Per-tet material interface on fixed-capacity state (one thread per tet).
//
// Replaces simplicial_arrangement::compute_material_interface (third-party, absent), called by
// the reference at src/material_interface.cpp:323,327 with the corner values of the tet's
// candidate materials (:307-316).  Labels 0..3 are the tet faces, material i is 4+i
// (src/extract_mesh.cpp:659).
//
// Algorithm: identical materials are grouped.  The cell of each material m is the tet clipped,
// in order, by the half-spaces m >= j of every other material j (a convex polytope).  A vertex
// carries the exact set of labels that are tight at it (tet faces through it, materials tied
// with the maximum); its label is the lexicographically smallest independent subset of that set.
// The record is the canonical one documented in include/ria.h: vertices sorted by label, faces
// sorted by (positive, negative) label, the positive label of an interface being the larger
// material, loops counter-clockwise seen from the positive side.
#pragma once
#include "cut_ia.cuh"

namespace ria {

struct MISummary {
    uint16_t n_mi_v;     // vertices on an interface face
    uint16_t n_mi_f;     // interface faces (positive label > 3)
    uint16_t n_mi_loop;  // their total loop length
    uint16_t n_bnd_f;    // faces on the tet boundary
    uint16_t n_bnd_loop; // their total loop length
};

RIA_HD int popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __popcll(x);
#else
    return __builtin_popcountll(x);
#endif
}

// One material's cell, exported from its clipped polytope (vertex keys: four sorted labels).
template <int V, int F, int L>
struct MICell {
    static constexpr int kV = V, kF = F, kL = L;
    uint8_t nv, nf;
    uint32_t vkey[V];
    uint8_t fother[F];
    uint8_t flen[F];
    uint8_t loops[L];
};

template <int PV, int PF, int PL, int OV, int OF, int OL, bool EXACT>
struct MICut {
    const double* mt;  // k x 4 corner values
    int k;
    uint8_t rep[64];
    // the polytope being clipped
    int nv;
    uint64_t mask[PV];
    uint8_t clab[PV][4];
    VCache vc[PV];
    int8_t sg[PV];
    int nf;
    uint8_t fother[PF];
    uint16_t foff[PF], flen[PF];
    uint8_t loops[2][PL];
    int cur;
    // accumulated output
    int onv, onf, onc, oloop;
    uint32_t okey[OV];
    uint8_t opos[OF], oneg[OF];
    uint16_t ooff[OF], olen[OF];
    uint8_t oloops[OL];
    uint8_t ocell[64];

    RIA_HD const double* row_of(int l) const { return mt + 4 * (l - 4); }

    RIA_HD bool build_cache(int v) {
        bool bound[4] = {false, false, false, false};
        const double* rows[4];
        int m = 0;
        for (int t = 0; t < 4; ++t) {
            int l = clab[v][t];
            if (l < 4)
                bound[l] = true;
            else
                rows[m++] = row_of(l);
        }
        uint8_t S[4];
        int s = 0;
        for (int c = 0; c < 4; ++c)
            if (!bound[c]) S[s++] = (uint8_t)c;
        return vcache_build(vc[v], true, s, S, m, rows, EXACT);
    }

    RIA_HD int query(int v, const double* q) const {
        const double* rows[4];
        int m = 0;
        for (int t = 0; t < 4; ++t)
            if (clab[v][t] >= 4) rows[m++] = row_of(clab[v][t]);
        return vcache_query(vc[v], q, rows, EXACT);
    }

    // lexicographically smallest independent label set of a tight mask (exact rank tests);
    // returns false if undecidable here
    RIA_HD bool greedy(uint64_t mk, uint8_t* out) const {
        if (!EXACT) return false;
        double rows[4 * 5];
        int n = 0;
        for (int l = 0; l < 64 && n < 4; ++l) {
            if (!(mk & bit64(l))) continue;
            double* r = rows + 5 * n;
            if (l < 4) {
                for (int c = 0; c < 5; ++c) r[c] = (c == l) ? 1.0 : 0.0;
            } else {
                for (int c = 0; c < 4; ++c) r[c] = row_of(l)[c];
                r[4] = 1.0;
            }
            int ind = rows_independent(rows, n + 1, 5);
            if (ind == 2) return false;
            if (ind) out[n++] = (uint8_t)l;
        }
        return n == 4;
    }

    RIA_HD bool labels_of_mask(uint64_t mk, uint8_t* out) const {
        if (popc64(mk) == 4) {
            int t = 0;
            for (int l = 0; l < 64; ++l)
                if (mk & bit64(l)) out[t++] = (uint8_t)l;
            return true;
        }
        return greedy(mk, out);
    }

    RIA_HD void group_materials() {
        for (int i = 0; i < k; ++i) {
            rep[i] = (uint8_t)(4 + i);
            for (int j = 0; j < i; ++j) {
                if (rep[j] != 4 + j) continue;
                const double* a = mt + 4 * i;
                const double* b = mt + 4 * j;
                if (a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3]) {
                    rep[i] = (uint8_t)(4 + j);
                    break;
                }
            }
        }
    }

    uint64_t no_cell, no_clip;

    // materials, grouping of identical materials, dominated materials; empty output
    RIA_HDI int prepare(const double* mats, int kk) {
        mt = mats;
        k = kk;
        if (k > 60) return CUT_FAIL;
        group_materials();
        // A material b >= a at all four corners leaves the half-space a >= b without interior in the
        // tet (values are linear), so a owns no cell; if b > a at all corners, a never reaches the
        // maximum anywhere in the tet and its half-space clips nothing.  Both are skipped; the result
        // is the same as clipping with them.
        no_cell = 0;
        no_clip = 0;
        for (int a = 0; a < k; ++a) {
            if (rep[a] != 4 + a) continue;
            const double* x = mt + 4 * a;
            for (int b = 0; b < k; ++b) {
                if (b == a || rep[b] != 4 + b) continue;
                const double* y = mt + 4 * b;
                if (y[0] >= x[0] && y[1] >= x[1] && y[2] >= x[2] && y[3] >= x[3]) {
                    no_cell |= bit64(a);
                    if (y[0] > x[0] && y[1] > x[1] && y[2] > x[2] && y[3] > x[3]) no_clip |= bit64(a);
                }
            }
        }
        onv = onf = onc = oloop = 0;
        return CUT_OK;
    }

    // does material m (label) own a cell that has to be computed?
    RIA_HD bool has_cell(int m) const { return rep[m - 4] == m && !(no_cell & bit64(m - 4)); }

    // The cell of material m: the tet clipped by m >= j for every other material j.  Leaves the
    // polytope (nv, mask, faces, loops[cur]) for export_cell; `empty` when it has no interior.
    RIA_HDI int clip(int m, bool& empty) {
        const int kBad = EXACT ? CUT_FAIL : CUT_DEFER;
        {
            // the whole tet, labelled with material m
            nv = 4;
            for (int c = 0; c < 4; ++c) {
                int t = 0;
                for (int b = 0; b < 4; ++b)
                    if (b != c) clab[c][t++] = (uint8_t)b;
                clab[c][3] = (uint8_t)m;
                mask[c] = (0xFull & ~bit64(c)) | bit64(m);
                if (!build_cache(c)) return kBad;
            }
            nf = 4;
            cur = 0;
            for (int b = 0; b < 4; ++b) {
                fother[b] = (uint8_t)b;
                foff[b] = (uint16_t)(3 * b);
                flen[b] = 3;
                for (int j = 0; j < 3; ++j) loops[0][3 * b + j] = (uint8_t)tet_face_outward(b, j);
            }
            empty = false;
            for (int j = 4; j < 4 + k; ++j) {
                if (j == m || rep[j - 4] != j || (no_clip & bit64(j - 4))) continue;
                const double* qv = row_of(j);
                uint8_t live[PV];
                for (int v = 0; v < nv; ++v) live[v] = 0;
                for (int f = 0; f < nf; ++f)
                    for (int t = 0; t < flen[f]; ++t) live[loops[cur][foff[f] + t]] = 1;
                bool hp = false, hn = false;
                for (int v = 0; v < nv; ++v) {
                    sg[v] = 0;
                    if (!live[v]) continue;
                    int s = query(v, qv);
                    if (s == 2) return kBad;
                    sg[v] = (int8_t)s;
                    if (s == 0) mask[v] |= bit64(j);
                    hp = hp || s > 0;
                    hn = hn || s < 0;
                }
                if (!hn) {
                    empty = true;
                    break;
                }
                if (!hp) continue;
                // new vertices on crossing edges
                int ne = 0;
                uint16_t ekey[PV];
                uint8_t eval[PV];
                for (int f = 0; f < nf; ++f) {
                    const int L = flen[f];
                    for (int t = 0; t < L; ++t) {
                        int u = loops[cur][foff[f] + t], w = loops[cur][foff[f] + (t + 1 == L ? 0 : t + 1)];
                        if (sg[u] * sg[w] >= 0) continue;
                        uint16_t key = (uint16_t)(u < w ? (u | (w << 8)) : (w | (u << 8)));
                        bool found = false;
                        for (int e = 0; e < ne; ++e)
                            if (ekey[e] == key) found = true;
                        if (found) continue;
                        if (nv >= PV || ne >= PV) return kBad;
                        uint64_t em = mask[u] & mask[w];
                        mask[nv] = em | bit64(j);
                        if (popc64(em) == 3) {
                            uint8_t lb[4];
                            int c = 0;
                            for (int l = 0; l < 64; ++l)
                                if (mask[nv] & bit64(l)) lb[c++] = (uint8_t)l;
                            for (int c2 = 0; c2 < 4; ++c2) clab[nv][c2] = lb[c2];
                        } else if (!greedy(mask[nv], clab[nv])) {
                            return kBad;
                        }
                        sg[nv] = 0;
                        if (!build_cache(nv)) return kBad;
                        ekey[ne] = key;
                        eval[ne] = (uint8_t)nv;
                        ++ne;
                        ++nv;
                    }
                }
                // clip the faces; collect the cap edges
                int nb = cur ^ 1, used = 0, nfn = 0;
                uint8_t et[PF], eh[PF];
                int nedge = 0;
                uint8_t nother[PF];
                uint16_t noff[PF], nlen[PF];
                for (int f = 0; f < nf; ++f) {
                    const int L = flen[f];
                    uint8_t full[PV + 8];
                    int n = 0;
                    bool fp = false, fn = false;
                    for (int t = 0; t < L; ++t) {
                        int u = loops[cur][foff[f] + t], w = loops[cur][foff[f] + (t + 1 == L ? 0 : t + 1)];
                        if (n >= PV + 8) return kBad;
                        full[n++] = (uint8_t)u;
                        fp = fp || sg[u] > 0;
                        fn = fn || sg[u] < 0;
                        if (sg[u] * sg[w] < 0) {
                            uint16_t key = (uint16_t)(u < w ? (u | (w << 8)) : (w | (u << 8)));
                            int id = -1;
                            for (int e = 0; e < ne; ++e)
                                if (ekey[e] == key) id = eval[e];
                            if (n >= PV + 8) return kBad;
                            full[n++] = (uint8_t)id;
                        }
                    }
                    if (!fn) continue;
                    int j0 = -1;
                    for (int t = 0; t < n; ++t) {
                        int prev = full[t == 0 ? n - 1 : t - 1];
                        if (sg[full[t]] < 0 && sg[prev] >= 0) {
                            j0 = t;
                            break;
                        }
                    }
                    if (j0 >= 0) {
                        int j1 = j0;
                        while (sg[full[(j1 + 1) % n]] < 0) j1 = (j1 + 1) % n;
                        int wa = full[(j0 - 1 + n) % n], wb = full[(j1 + 1) % n];
                        if (wa != wb) {
                            if (nedge >= PF) return kBad;
                            et[nedge] = (uint8_t)wa;
                            eh[nedge] = (uint8_t)wb;
                            ++nedge;
                        }
                    }
                    if (nfn >= PF) return kBad;
                    nother[nfn] = fother[f];
                    noff[nfn] = (uint16_t)used;
                    int cnt = 0;
                    for (int t = 0; t < n; ++t) {
                        if (fp && sg[full[t]] > 0) continue;
                        if (used >= PL) return kBad;
                        loops[nb][used++] = full[t];
                        ++cnt;
                    }
                    nlen[nfn] = (uint16_t)cnt;
                    ++nfn;
                }
                if (nedge < 3) return CUT_FAIL;
                if (nfn >= PF || used + nedge > PL) return kBad;
                nother[nfn] = (uint8_t)j;
                noff[nfn] = (uint16_t)used;
                nlen[nfn] = (uint16_t)nedge;
                int curv = et[0];
                for (int t = 0; t < nedge; ++t) {
                    loops[nb][used++] = (uint8_t)curv;
                    int nxt = -1;
                    for (int e = 0; e < nedge; ++e)
                        if (et[e] == curv) {
                            nxt = eh[e];
                            break;
                        }
                    if (nxt < 0) return CUT_FAIL;
                    curv = nxt;
                }
                if (curv != et[0]) return CUT_FAIL;
                ++nfn;
                nf = nfn;
                for (int f = 0; f < nf; ++f) {
                    fother[f] = nother[f];
                    foff[f] = noff[f];
                    flen[f] = nlen[f];
                }
                cur = nb;
            }
        }
        return CUT_OK;
    }

    // The clipped polytope as a self-contained cell: the keys of its live vertices (the four sorted
    // labels of each, in polytope order) and its faces with loops over those vertices.
    template <class Cell>
    RIA_HDI int export_cell(Cell& out) const {
        const int kBad = EXACT ? CUT_FAIL : CUT_DEFER;
        uint8_t id[PV];
        uint8_t live[PV];
        for (int v = 0; v < nv; ++v) live[v] = 0;
        for (int f = 0; f < nf; ++f)
            for (int t = 0; t < flen[f]; ++t) live[loops[cur][foff[f] + t]] = 1;
        int n = 0;
        for (int v = 0; v < nv; ++v) {
            if (!live[v]) continue;
            uint8_t lb[4];
            if (!labels_of_mask(mask[v], lb)) return kBad;
            if (n >= Cell::kV) return kBad;
            out.vkey[n] = ((uint32_t)lb[0] << 24) | ((uint32_t)lb[1] << 16) | ((uint32_t)lb[2] << 8) | lb[3];
            id[v] = (uint8_t)n++;
        }
        out.nv = (uint8_t)n;
        if (nf > Cell::kF) return kBad;
        int used = 0;
        for (int f = 0; f < nf; ++f) {
            if (used + flen[f] > Cell::kL) return kBad;
            out.fother[f] = fother[f];
            out.flen[f] = (uint8_t)flen[f];
            for (int t = 0; t < flen[f]; ++t) out.loops[used++] = id[loops[cur][foff[f] + t]];
        }
        out.nf = (uint8_t)nf;
        return CUT_OK;
    }

    // Appends cell m to the output: its vertices are merged with those of earlier cells by key.
    template <class Cell>
    RIA_HDI int append_cell(int m, const Cell& cell) {
        const int kBad = EXACT ? CUT_FAIL : CUT_DEFER;
        if (onc >= 64) return kBad;
        ocell[onc++] = (uint8_t)m;
        uint8_t oid[Cell::kV];
        for (int v = 0; v < cell.nv; ++v) {
            const uint32_t key = cell.vkey[v];
            int id = -1;
            for (int x = 0; x < onv; ++x)
                if (okey[x] == key) id = x;
            if (id < 0) {
                if (onv >= OV) return kBad;
                id = onv;
                okey[onv++] = key;
            }
            oid[v] = (uint8_t)id;
        }
        int used = 0;
        for (int f = 0; f < cell.nf; ++f) {
            if (onf >= OF || oloop + cell.flen[f] > OL) return kBad;
            opos[onf] = cell.fother[f];
            oneg[onf] = (uint8_t)m;
            ooff[onf] = (uint16_t)oloop;
            olen[onf] = cell.flen[f];
            for (int t = 0; t < cell.flen[f]; ++t) oloops[oloop++] = oid[cell.loops[used++]];
            ++onf;
        }
        return CUT_OK;
    }

    RIA_HDI int run(const double* mats, int kk) {
        int st = prepare(mats, kk);
        if (st != CUT_OK) return st;
        for (int m = 4; m < 4 + k; ++m) {
            if (!has_cell(m)) continue;
            bool empty = false;
            st = clip(m, empty);
            if (st != CUT_OK) return st;
            if (empty) continue;
            MICell<PV, PF, PL> cell;
            st = export_cell(cell);
            if (st != CUT_OK) return st;
            st = append_cell(m, cell);
            if (st != CUT_OK) return st;
        }
        return CUT_OK;
    }

    // Interface faces are identified by their vertex sets: when tie planes coincide the face of cell m
    // against the material it was clipped by can border another cell, which holds the same polygon.
    // Each interface is kept once, from the smaller material's cell (its loop is outward there, so
    // it turns toward the larger material), and labelled (larger, smaller).
    RIA_HD bool same_polygon(int a, int b) const {
        if (olen[a] != olen[b]) return false;
        for (int t = 0; t < olen[a]; ++t) {
            bool in = false;
            for (int u = 0; u < olen[b] && !in; ++u) in = oloops[ooff[a] + t] == oloops[ooff[b] + u];
            if (!in) return false;
        }
        return true;
    }

    RIA_HDI void pair_faces() {
        uint8_t keep[OF];
        // vertex-set signature of each face (length, smallest id, id sum): equal polygons have equal
        // signatures, so only faces with the signature of face i are compared vertex by vertex
        uint32_t sig[OF];
        for (int i = 0; i < onf; ++i) {
            uint32_t mn = 0xFF, sum = 0;
            for (int t = 0; t < olen[i]; ++t) {
                const uint32_t v = oloops[ooff[i] + t];
                mn = v < mn ? v : mn;
                sum += v;
            }
            sig[i] = ((uint32_t)olen[i] << 24) | (mn << 16) | (sum & 0xFFFFu);
        }
        for (int i = 0; i < onf; ++i) {
            keep[i] = 1;
            if (opos[i] < 4) continue;
            int partner = -1;
            for (int j = 0; j < onf && partner < 0; ++j)
                if (j != i && sig[j] == sig[i] && opos[j] >= 4 && oneg[j] != oneg[i] && same_polygon(i, j))
                    partner = j;
            if (partner >= 0) {
                if (oneg[i] > oneg[partner]) {
                    keep[i] = 0;
                } else {
                    opos[i] = oneg[partner];
                }
            } else if (oneg[i] > opos[i]) {
                // no cell holds the same polygon: keep the clipping label, toward the larger material
                uint8_t t = opos[i];
                opos[i] = oneg[i];
                oneg[i] = t;
                for (int x = 0, y = olen[i] - 1; x < y; ++x, --y) {
                    uint8_t s = oloops[ooff[i] + x];
                    oloops[ooff[i] + x] = oloops[ooff[i] + y];
                    oloops[ooff[i] + y] = s;
                }
            }
        }
        int n = 0, total = 0;
        for (int i = 0; i < onf; ++i) {
            if (!keep[i]) continue;
            opos[n] = opos[i];
            oneg[n] = oneg[i];
            ooff[n] = ooff[i];
            olen[n] = olen[i];
            total += olen[i];
            ++n;
        }
        onf = n;
        oloop = total;  // the record writes only the kept loops
    }

    // ---- canonical form
    uint8_t vorder[OV], vnew[OV];
    uint16_t forder[OF];  // face ids exceed 8 bits in the exact variant

    RIA_HDI void canonicalize() {
        pair_faces();
        for (int i = 0; i < onv; ++i) vorder[i] = (uint8_t)i;
        for (int x = 1; x < onv; ++x)
            for (int y = x; y > 0 && okey[vorder[y - 1]] > okey[vorder[y]]; --y) {
                uint8_t t = vorder[y];
                vorder[y] = vorder[y - 1];
                vorder[y - 1] = t;
            }
        for (int i = 0; i < onv; ++i) vnew[vorder[i]] = (uint8_t)i;
        for (int i = 0; i < onf; ++i) forder[i] = (uint16_t)i;
        auto fk = [&](int f) { return ((int)opos[f] << 8) | oneg[f]; };
        for (int x = 1; x < onf; ++x)
            for (int y = x; y > 0 && fk(forder[y - 1]) > fk(forder[y]); --y) {
                uint16_t t = forder[y];
                forder[y] = forder[y - 1];
                forder[y - 1] = t;
            }
    }

    RIA_HD int record_size() const { return 10 + k + 4 * onv + 4 * onf + 2 * oloop + onc; }

    RIA_HDI void emit(uint8_t* dst, MISummary& sum) const {
        int o = 0;
        auto w8 = [&](int v) { dst[o++] = (uint8_t)v; };
        auto w16 = [&](int v) {
            dst[o++] = (uint8_t)(v & 0xFF);
            dst[o++] = (uint8_t)((v >> 8) & 0xFF);
        };
        w8(2);
        w8(k);
        w16(onv);
        w16(onf);
        w16(onc);
        w16(oloop);
        for (int i = 0; i < k; ++i) w8(rep[i]);
        for (int i = 0; i < onv; ++i) {
            uint32_t key = okey[vorder[i]];
            w8((int)(key >> 24));
            w8((int)((key >> 16) & 0xFF));
            w8((int)((key >> 8) & 0xFF));
            w8((int)(key & 0xFF));
        }
        uint8_t onmi[OV];
        for (int i = 0; i < onv; ++i) onmi[i] = 0;
        int nmf = 0, nml = 0, nbf = 0, nbl = 0;
        for (int i = 0; i < onf; ++i) {
            int f = forder[i];
            w8(opos[f]);
            w8(oneg[f]);
            w16(olen[f]);
            if (opos[f] > 3) {
                ++nmf;
                nml += olen[f];
                for (int t = 0; t < olen[f]; ++t) onmi[vnew[oloops[ooff[f] + t]]] = 1;
            } else {
                ++nbf;
                nbl += olen[f];
            }
        }
        for (int i = 0; i < onf; ++i) {
            int f = forder[i];
            int L = olen[f];
            int jm = 0;
            for (int t = 1; t < L; ++t)
                if (vnew[oloops[ooff[f] + t]] < vnew[oloops[ooff[f] + jm]]) jm = t;
            for (int t = 0; t < L; ++t) w16(vnew[oloops[ooff[f] + (jm + t) % L]]);
        }
        for (int i = 0; i < onc; ++i) w8(ocell[i]);
        int nmv = 0;
        for (int i = 0; i < onv; ++i) nmv += onmi[i];
        sum.n_mi_v = (uint16_t)nmv;
        sum.n_mi_f = (uint16_t)nmf;
        sum.n_mi_loop = (uint16_t)nml;
        sum.n_bnd_f = (uint16_t)nbf;
        sum.n_bnd_loop = (uint16_t)nbl;
    }
};

}  // namespace ria
