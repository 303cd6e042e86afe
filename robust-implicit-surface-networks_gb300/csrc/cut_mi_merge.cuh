// The material interface's merge step across the lanes of a warp: the cells of one tet, clipped
// independently (one lane per material), become the tet's canonical record (the same bytes as
// MICut's serial append_cell / canonicalize / emit).
//
//   vertices  every cell vertex is an entry; an entry is the first of its key when no earlier
//             entry carries it; a vertex's id is the number of distinct keys below its own (the
//             canonical order sorts vertices by key)
//   faces     each cell face (the cell's material negative, the other side positive); an interface
//             face held by two cells (the same vertex set) is kept once, from the smaller material's
//             cell, labelled (larger, smaller); one held by a single cell is turned toward the larger
//             material.  These decisions only read the cells, so every face decides on its own lane.
//   order     kept faces sorted by (positive, negative) label, stably; loops start at their
//             smallest vertex id
//
// Capacities beyond kMergeV entries or kMergeF faces are reported, and the caller merges serially.
#pragma once
#include "cut_ia_warp.cuh"
#include "cut_mi.cuh"

namespace ria {

constexpr int kMergeV = 512;  // vertex entries (cell vertices, before deduplication)
constexpr int kMergeF = 256;  // cell faces

template <class Cell>
struct MIMerge {
    int nc;                       // cells, in ascending material order
    uint8_t cm[32];               // their material labels (4 + j)
    uint16_t voff[33], foff[33];  // prefix counts of cell vertices and faces
    uint16_t ne, nface;
    uint8_t vid[kMergeV];         // canonical vertex id of each entry
    uint8_t first[kMergeV];
    uint32_t fsig[kMergeF];
    uint8_t fpos[kMergeF], fneg[kMergeF], fkeep[kMergeF], fflip[kMergeF];
    uint16_t forder[kMergeF], floff[kMergeF], fstart[kMergeF];
    uint8_t mark[256];  // vertex on an interface face
    int onv, onf, oloop;

    RIA_HD int cell_of_entry(int e) const {
        int c = 0;
        while (c + 1 < nc && voff[c + 1] <= e) ++c;
        return c;
    }
    RIA_HD int cell_of_face(int g) const {
        int c = 0;
        while (c + 1 < nc && foff[c + 1] <= g) ++c;
        return c;
    }
    RIA_HD uint32_t key_of(const Cell* cells, int e) const {
        const int c = cell_of_entry(e);
        return cells[cm[c] - 4].vkey[e - voff[c]];
    }
    // canonical vertex id of loop position t of face g
    RIA_HD int fvert(const Cell* cells, int g, int t) const {
        const int c = cell_of_face(g);
        return vid[voff[c] + cells[cm[c] - 4].loops[fstart[g] + t]];
    }
    RIA_HD int flen(const Cell* cells, int g) const {
        const int c = cell_of_face(g);
        return cells[cm[c] - 4].flen[g - foff[c]];
    }
    RIA_HD bool same_polygon(const Cell* cells, int a, int b) const {
        const int la = flen(cells, a), lb = flen(cells, b);
        if (la != lb) return false;
        for (int t = 0; t < la; ++t) {
            const int v = fvert(cells, a, t);
            bool in = false;
            for (int u = 0; u < lb && !in; ++u) in = v == fvert(cells, b, u);
            if (!in) return false;
        }
        return true;
    }

    // `has[j]`: material 4+j has a cell in cells[j].  Returns CUT_OK or CUT_DEFER (capacity).
    RIA_HDI int run(const Lanes& L, const Cell* cells, const uint8_t* has, int k) {
        const int lane = L.lane;
        if (lane == 0) {
            nc = 0;
            int nv = 0, nf = 0;
            for (int j = 0; j < k; ++j) {
                if (!has[j]) continue;
                if (nc >= 32) break;
                cm[nc] = (uint8_t)(4 + j);
                voff[nc] = (uint16_t)nv;
                foff[nc] = (uint16_t)nf;
                nv += cells[j].nv;
                nf += cells[j].nf;
                ++nc;
            }
            voff[nc] = (uint16_t)(nv < 65535 ? nv : 65535);
            foff[nc] = (uint16_t)(nf < 65535 ? nf : 65535);
            ne = (uint16_t)(nv <= kMergeV ? nv : 0xFFFF);
            nface = (uint16_t)(nf <= kMergeF ? nf : 0xFFFF);
        }
        L.sync();
        if (ne == 0xFFFF || nface == 0xFFFF || nc > 32) return CUT_DEFER;
        const int E = ne, NF = nface;
        // vertices
        for (int e = lane; e < E; e += L.W) {
            const uint32_t key = key_of(cells, e);
            bool f = true;
            for (int x = 0; x < e && f; ++x) f = key_of(cells, x) != key;
            first[e] = f ? 1 : 0;
        }
        L.sync();
        int nd = 0;
        for (int e = lane; e < E; e += L.W) {
            const uint32_t key = key_of(cells, e);
            int r = 0;
            for (int x = 0; x < E; ++x) r += first[x] && key_of(cells, x) < key;
            if (r > 255) r = 255;  // beyond the 8-bit id range: reported below
            vid[e] = (uint8_t)r;
            nd += first[e];
        }
        nd = L.add_all(nd);
        if (nd > 255) return CUT_DEFER;
        // faces: loop starts within their cell, signatures
        for (int g = lane; g < NF; g += L.W) {
            const int c = cell_of_face(g);
            const Cell& cell = cells[cm[c] - 4];
            int s = 0;
            for (int f = 0; f < g - foff[c]; ++f) s += cell.flen[f];
            fstart[g] = (uint16_t)s;
        }
        L.sync();
        for (int g = lane; g < NF; g += L.W) {
            uint32_t mn = 0xFF, sum = 0;
            const int len = flen(cells, g);
            for (int t = 0; t < len; ++t) {
                const uint32_t v = (uint32_t)fvert(cells, g, t);
                mn = v < mn ? v : mn;
                sum += v;
            }
            fsig[g] = ((uint32_t)len << 24) | (mn << 16) | (sum & 0xFFFFu);
            const int c = cell_of_face(g);
            fpos[g] = cells[cm[c] - 4].fother[g - foff[c]];
            fneg[g] = cm[c];
        }
        L.sync();
        // pairing: every decision reads the cells' labels only
        constexpr int kPer = kMergeF / Lanes::W;  // faces per lane
        uint8_t np[kPer], nn[kPer], nk[kPer], nfl[kPer];
        int q = 0;
        for (int g = lane; g < NF; g += L.W, ++q) {
            uint8_t pos = fpos[g], neg = fneg[g], keep = 1, flip = 0;
            if (pos >= 4) {
                int partner = -1;
                for (int j = 0; j < NF && partner < 0; ++j)
                    if (j != g && fsig[j] == fsig[g] && fpos[j] >= 4 && fneg[j] != neg && same_polygon(cells, g, j))
                        partner = j;
                if (partner >= 0) {
                    if (neg > fneg[partner])
                        keep = 0;
                    else
                        pos = fneg[partner];
                } else if (neg > pos) {
                    const uint8_t t = pos;
                    pos = neg;
                    neg = t;
                    flip = 1;
                }
            }
            np[q] = pos;
            nn[q] = neg;
            nk[q] = keep;
            nfl[q] = flip;
        }
        L.sync();
        q = 0;
        for (int g = lane; g < NF; g += L.W, ++q) {
            fpos[g] = np[q];
            fneg[g] = nn[q];
            fkeep[g] = nk[q];
            fflip[g] = nfl[q];
        }
        L.sync();
        // canonical face order: kept faces by (positive, negative), ties by index
        int kept = 0, lsum = 0;
        for (int g = lane; g < NF; g += L.W) {
            if (!fkeep[g]) continue;
            const int key = ((int)fpos[g] << 8) | fneg[g];
            int r = 0;
            for (int j = 0; j < NF; ++j)
                r += fkeep[j] && ((((int)fpos[j] << 8) | fneg[j]) < key || ((((int)fpos[j] << 8) | fneg[j]) == key && j < g));
            forder[r] = (uint16_t)g;
            ++kept;
            lsum += flen(cells, g);
        }
        kept = L.add_all(kept);
        lsum = L.add_all(lsum);
        L.sync();
        int acc = 0;
        for (int base = 0; base < kept; base += L.W) {
            const int i = base + lane;
            const int len = i < kept ? flen(cells, forder[i]) : 0;
            int tot = 0;
            const int off = L.scan(len, tot);
            if (i < kept) floff[i] = (uint16_t)(acc + off);
            acc += tot;
        }
        if (lane == 0) {
            onv = nd;
            onf = kept;
            oloop = lsum;
        }
        L.sync();
        return CUT_OK;
    }

    RIA_HD int record_size(int k) const { return 10 + k + 4 * onv + 4 * onf + 2 * oloop + nc; }

    // the record: the layout of MICut::emit
    RIA_HDI void emit(const Lanes& L, const Cell* cells, int k, const uint8_t* rep, uint8_t* dst, MISummary& sum) {
        const int lane = L.lane;
        auto w16 = [&](int o, int v) {
            dst[o] = (uint8_t)(v & 0xFF);
            dst[o + 1] = (uint8_t)((v >> 8) & 0xFF);
        };
        if (lane == 0) {
            dst[0] = 2;
            dst[1] = (uint8_t)k;
            w16(2, onv);
            w16(4, onf);
            w16(6, nc);
            w16(8, oloop);
        }
        for (int i = lane; i < k; i += L.W) dst[10 + i] = rep[i];
        const int ov = 10 + k, ofc = ov + 4 * onv, olp = ofc + 4 * onf, oc = olp + 2 * oloop;
        for (int e = lane; e < ne; e += L.W) {
            if (!first[e]) continue;
            const uint32_t key = key_of(cells, e);
            const int o = ov + 4 * vid[e];
            dst[o] = (uint8_t)(key >> 24);
            dst[o + 1] = (uint8_t)((key >> 16) & 0xFF);
            dst[o + 2] = (uint8_t)((key >> 8) & 0xFF);
            dst[o + 3] = (uint8_t)(key & 0xFF);
        }
        for (int v = lane; v < 256; v += L.W) mark[v] = 0;
        L.sync();
        int nmf = 0, nml = 0, nbf = 0, nbl = 0;
        for (int i = lane; i < onf; i += L.W) {
            const int g = forder[i];
            const int len = flen(cells, g);
            const int o = ofc + 4 * i;
            dst[o] = fpos[g];
            dst[o + 1] = fneg[g];
            w16(o + 2, len);
            const bool mi = fpos[g] > 3;
            if (mi) {
                ++nmf;
                nml += len;
            } else {
                ++nbf;
                nbl += len;
            }
            // the loop, reversed for a face turned toward the larger material, from its smallest id
            int jm = 0, vm = 256;
            for (int t = 0; t < len; ++t) {
                const int v = fvert(cells, g, fflip[g] ? len - 1 - t : t);
                if (v < vm) {
                    vm = v;
                    jm = t;
                }
                if (mi) mark[v] = 1;
            }
            for (int t = 0; t < len; ++t) {
                const int tt = (jm + t) % len;
                w16(olp + 2 * (floff[i] + t), fvert(cells, g, fflip[g] ? len - 1 - tt : tt));
            }
        }
        for (int c = lane; c < nc; c += L.W) dst[oc + c] = cm[c];
        nmf = L.add_all(nmf);
        nml = L.add_all(nml);
        nbf = L.add_all(nbf);
        nbl = L.add_all(nbl);
        L.sync();
        int nmv = 0;
        for (int v = lane; v < onv; v += L.W) nmv += mark[v];
        nmv = L.add_all(nmv);
        sum.n_mi_v = (uint16_t)nmv;
        sum.n_mi_f = (uint16_t)nmf;
        sum.n_mi_loop = (uint16_t)nml;
        sum.n_bnd_f = (uint16_t)nbf;
        sum.n_bnd_loop = (uint16_t)nbl;
    }
};

}  // namespace ria
